"""Bit flags.  The first seven are the reference's (ufo/methods.py:8-14) with
the same values, so scripts that pass ``ufo.KICK | ufo.DOUBLE_PRECISION`` keep
working.  Arithmetic is FP64 whatever DOUBLE_PRECISION says; the flag only
selects the dtype of the returned arrays, as the reference's buffers would
have it.  The last two are this build's:

FMA      contract multiply-add pairs into fused multiply-adds, replace the teapot
         inner-drift division ``(px*A)/(N-1)`` by ``px*(A/(N-1))``, evaluate
         general multipole kicks as one complex Horner pass and sextupole
         slices as t(x^2 - y^2), 2t xy, and fold plain drifts into the outer
         drifts of neighbouring magnets.
         Results agree with the default mode to FP64 rounding (tested to
         1e-12 relative after 1 turn and 1e-9 after 1000 turns) but are not
         bit-identical to the reference.
YOSHIDA  4th-order Yoshida splitting of each teapot slice (no reference
         counterpart; not with EXACT, not differentiated).
"""
LINEAR = 1 << 0
FIVED = 1 << 1
EXACT = 1 << 2
KICK = 1 << 3
RADIATION = 1 << 4
DOUBLE_PRECISION = 1 << 5
ACHROMATIC = 1 << 6
YOSHIDA = 1 << 8
FMA = 1 << 9
