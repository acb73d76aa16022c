"""Lattice compiler: flattened line -> opcode table + per-seed FP64 constants.

The reference turns a line into one straight-line OpenCL C function with every
element constant pasted in as a literal (ufo/lattice.py:86-119 driving the
templates of ufo/methods.py:16-241).  Here the same arithmetic is split into
 * an opcode table shared by all particles of a launch (``Program.ops``,
   int32 ``[n_ops, 8]``), which the sm_103a kernels interpret warp-uniformly,
 * per-seed FP64 constant tables (``Program.table``, ``[n_seeds, stride]``),
   one row per distinct setting of the lattice parameters.

Bit-exactness rules (what makes the kernels reproduce the reference's FP64
results to the last bit):
 * Every constant sub-expression is folded here with IEEE double arithmetic in
   the order the reference's C expression evaluates it (C is left-associative
   and the templates paste text without parentheses, e.g. the inner teapot
   drift is ``x += px * (A) / 3.0`` = ``(px*A)/3.0``, ufo/methods.py:81-82 and
   :39-40).  Constants are folded per seed with numpy float64 arithmetic.
 * Transcendentals of literal arguments are folded correctly rounded
   (:mod:`ufo_gb300.crmath`), as GCC folds them; those of parameter-derived
   values use the C library (``math``), as the reference calls it at run time.
 * Terms whose coefficient is exactly zero in every seed ("structurally zero")
   are dropped.  For finite coordinates the result is unchanged (up to the sign
   of an exact zero); the kernels evaluate the full expression, zero terms
   included, whenever x or y is not finite, so NaN/inf propagation is also the
   reference's.

Parameter binding mirrors ufo/lattice.py:107-110 (match on ``p[0]`` against
the element label or its flat index, later entries overriding earlier ones)
and the ``x or self.x`` resolution of the element ``method()``s.
"""
import math

import numpy as np

from . import aperture as _ap
from . import cexpr as _cx
from . import crmath
from . import elements as E
from .flags import LINEAR, FIVED, EXACT, KICK, ACHROMATIC, YOSHIDA, FMA

# ---- opcodes (the same numbering as csrc/ops.cuh) ----
OP_NOP, OP_DRIFT, OP_KICK, OP_TEAPOT, OP_ALIGN, OP_EDGE, OP_THICKQ, OP_THICKB, OP_WIRE, \
    OP_APERTURE, OP_OBSERVE, OP_DYNKICK, OP_LINEAR = range(13)
OP_NAMES = ['nop', 'drift', 'kick', 'teapot', 'align', 'edge', 'thickq', 'thickb', 'wire',
            'aperture', 'observe', 'dynkick', 'linear']
# deepest expression stack of a dynamic-kick coefficient (csrc/ops.cuh: eval_prog)
DYN_STACK = 32

# drift forms: 0 -> x + px*c0 ; 1 -> x + (px*c0)*c1 ; 2 -> x + (px*c0)/c1
DF_MUL, DF_MUL2, DF_DIV = 0, 1, 2

# op flag bits
F_ACHRO = 1 << 0        # no oodppo factor (ACHROMATIC)
F_EXACT = 1 << 1        # exact drifts
F_WEAK = 1 << 2         # teapot: weak-focusing term present
F_RTPSI = 1 << 3        # edge: tan(psi) evaluated per particle
F_T1 = 1 << 4           # edge: px term present
F_T2 = 1 << 5           # edge: py term present
F_CONST = 1 << 6        # thick: transcendentals folded per seed
F_AX = 1 << 7           # align: x term present
F_AY = 1 << 8           # align: y term present
F_T1Z = 1 << 9          # edge: px term structurally zero (poison-only)
F_T2Z = 1 << 10         # edge: py term structurally zero (poison-only)
F_WEAKZ = 1 << 11       # teapot: weak term structurally zero (poison-only)
F_YOSHIDA = 1 << 12     # teapot: 4th-order Yoshida splitting instead of TEAPOT
F_CIRCLE = 1 << 13      # aperture: x*x + y*y < c (table: [c])
F_SPLITO = 1 << 14      # teapot: exit outer drift is its own constant, after the others
F_PSER = 1 << 15        # kick/teapot (FMA programs): dense power series appended last
# drift form of teapot outer/inner drifts packed in bits 16..19
SH_FOUTER, SH_FINNER = 16, 18

OP_WORDS = 8
MAX_ORDERS = 32

COORDS = ('x', 'px', 'y', 'py', 'z', 'dp')

# Yoshida 4th-order coefficients (H. Yoshida, Phys. Lett. A 150 (1990) 262):
# w1 = 1/(2 - 2^(1/3)), w0 = 1 - 2 w1; drift fractions c and kick fractions d.
_Y_W1 = 1.0 / (2.0 - 2.0 ** (1.0 / 3.0))
_Y_W0 = 1.0 - 2.0 * _Y_W1
YOSHIDA_C = (_Y_W1 / 2.0, (_Y_W0 + _Y_W1) / 2.0, (_Y_W0 + _Y_W1) / 2.0, _Y_W1 / 2.0)
YOSHIDA_D = (_Y_W1, _Y_W0, _Y_W1)


class Val:
    """A folded FP64 value over seeds: ``v`` is a numpy float64 array
    ``[n_seeds]`` or a scalar; ``lit`` tells whether the reference would have
    seen a literal (compile-time constant) rather than a parameter."""
    __slots__ = ('v', 'lit')

    def __init__(self, v, lit):
        self.v = v
        self.lit = lit

    @staticmethod
    def of(x, lit=True):
        if isinstance(x, Val):
            return x
        return Val(np.float64(x) if np.ndim(x) == 0 else np.asarray(x, np.float64), lit)

    def _bin(self, o, f):
        o = Val.of(o)
        with np.errstate(all='ignore'):
            return Val(f(np.float64(self.v) if np.ndim(self.v) == 0 else self.v,
                         np.float64(o.v) if np.ndim(o.v) == 0 else o.v), self.lit and o.lit)

    def __add__(self, o): return self._bin(o, np.add)
    def __sub__(self, o): return self._bin(o, np.subtract)
    def __mul__(self, o): return self._bin(o, np.multiply)
    def __truediv__(self, o): return self._bin(o, np.divide)
    def __radd__(self, o): return Val.of(o)._bin(self, np.add)
    def __rsub__(self, o): return Val.of(o)._bin(self, np.subtract)
    def __rmul__(self, o): return Val.of(o)._bin(self, np.multiply)
    def __rtruediv__(self, o): return Val.of(o)._bin(self, np.divide)

    def __neg__(self):
        return Val(-self.v, self.lit)

    def zero(self):
        """True when the value is +-0 in every seed (a structural zero)."""
        return bool(np.all(np.asarray(self.v) == 0.0))

    def finite_nonzero_everywhere(self):
        a = np.asarray(self.v)
        return bool(np.all(a != 0.0))


class Dyn:
    """A value that the reference computed at run time from C text reading
    the turn or the particle (a user ``method()`` override, e.g. the
    time-gated kicker of HOWTO.md:84-200): a stack program whose PUSH values
    are Vals over seeds (bound parameters resolved per seed)."""
    __slots__ = ('code', 'text')

    def __init__(self, code, text):
        self.code = code
        self.text = text


def _fn(name, a):
    """Math call on a folded value: correctly rounded for literals (GCC folds
    them), the C library otherwise (the reference calls it at run time)."""
    a = Val.of(a)
    if name in ('sqrt', 'fabs'):
        with np.errstate(all='ignore'):
            return Val(np.sqrt(a.v) if name == 'sqrt' else np.abs(a.v), a.lit)
    f = getattr(crmath, name) if a.lit else getattr(math, name)

    def safe(x):
        try:
            return f(float(x))
        except (ValueError, OverflowError):
            return math.nan if name != 'cosh' else math.inf
    if np.ndim(a.v) == 0:
        return Val(np.float64(safe(a.v)), a.lit)
    return Val(np.array([safe(x) for x in a.v]), a.lit)


class Op:
    """One opcode row plus its constants (each a Val)."""
    __slots__ = ('kind', 'flags', 'ints', 'consts', 'elem', 'flops', 'flops_fast')

    def __init__(self, kind, flags=0, ints=(), consts=(), elem=-1):
        self.kind = kind
        self.flags = flags
        self.ints = list(ints)
        self.consts = list(consts)
        self.elem = elem
        self.flops = 0
        self.flops_fast = 0


# ------------------------------------------------------------------ kicks

def _pad(m, min_order):
    """copy_multipoles_and_pad (ufo/methods.py:16-20): append max(len, min)
    literal zeros."""
    m = list(m)
    m += [Val.of(0.0)] * max(len(m), min_order)
    return m


class KickSpec:
    """Normal/skew coefficient lists of one kick, already scaled (teapot) and
    truncated (LINEAR).  Coefficient j is structurally zero if zero in every
    seed."""

    def __init__(self, knl, ksl, flags):
        self.achro = bool(flags & ACHROMATIC)
        self.norm = self._trunc(knl, flags)
        self.skew = self._trunc(ksl, flags)
        for lst in (self.norm, self.skew):
            if len(lst) > MAX_ORDERS:
                raise NotImplementedError(f'more than {MAX_ORDERS} multipole orders')

    @staticmethod
    def _trunc(lst, flags):
        # methods.kick: n = len(k); max_order = min(n, 2) if LINEAR else n
        if not lst:
            return []
        n = len(lst)
        mo = min(n, 2) if flags & LINEAR else n
        return lst[:mo]

    @staticmethod
    def mask(lst):
        m = 0
        for j, c in enumerate(lst):
            if not c.zero():
                m |= 1 << j
        return m

    def packed(self):
        """(n_norm, n_skew, mask_norm, mask_skew, consts) -- consts are the
        structurally non-zero coefficients, normal then skew, ascending j."""
        mn, ms = self.mask(self.norm), self.mask(self.skew)
        consts = [c for j, c in enumerate(self.norm) if mn >> j & 1]
        consts += [c for j, c in enumerate(self.skew) if ms >> j & 1]
        return len(self.norm), len(self.skew), mn, ms, consts

    def flops(self):
        """Strict-mode FP64 operations of one kick (reference tree minus
        structural zeros and exact identities), per kick."""
        total = 0
        for lst, skew in ((self.norm, False), (self.skew, True)):
            total += _horner_flops(lst, self.achro, skew)
        return total

    def general(self):
        """True when the kernels take the general path (not the quadrupole or
        sextupole short forms, not an empty kick)."""
        nn, ns, mn, ms, _ = self.packed()
        if ms:
            return True
        return not ((nn == 2 and mn == 2) or (nn == 3 and mn == 4) or mn == 0)

    def flops_fast(self):
        """FMA-mode FP64 flops the kernels execute per kick (an FMA counts 2).
        General kicks are one complex Horner pass over the dense power series
        prepared on the host (F_PSER): 4 FMA per order below the top one and 2
        FMA for the update, the strength factor o being the particle's own."""
        if self.general():
            _, _, mn, ms, _ = self.packed()
            top = (mn | ms).bit_length() - 1
            return 8 * top + 4
        total = 0
        for lst, skew in ((self.norm, False), (self.skew, True)):
            total += _horner_flops(lst, self.achro, skew, fast=True)
        return total


def _div_flops(order):
    return 0 if order == 1 else 1


def _horner_flops(lst, achro, skew, fast=False):
    """Count the operations of methods.kick's Horner scheme (ufo/methods.py:
    45-76) with structural zeros trimmed.  Fast mode counts an FMA as 2."""
    n = len(lst)
    if n == 0:
        return 0
    zx = lst[n - 1].zero()  # 'a' accumulator (dpx for normal, dpy for skew)
    zy = True
    f = 0
    if not zx and not achro:
        f += 1  # c * oodppo
    for order in range(n - 1, 0, -1):
        za = zx and zy
        if not zx and not zy:
            f += 3  # two products and one add/sub
            f += 3  # second pair
        elif not za:
            f += 2  # one product each
        if not za:
            f += 2 * _div_flops(order)
        zc = lst[order - 1].zero()
        if not zc:
            if not achro:
                f += 1
            if not za:
                f += 1
            zx = False
        else:
            zx = za
        zy = za
    if not zx:
        f += 1
    if not zy:
        f += 1
    return f


# ------------------------------------------------------------------ lowering

class _Lowerer:
    def __init__(self, flags, n_seeds):
        self.flags = flags
        self.S = n_seeds
        self.segments = [[]]   # list of lists of Op; dumps between segments

    def emit(self, op):
        self.segments[-1].append(op)

    def new_segment(self):
        self.segments.append([])

    # -- primitive templates (ufo/methods.py) --
    def align(self, dx, dy, elem):
        """methods.align: x -= dx; y -= dy (ufo/methods.py:22-26).  A zero
        offset is an exact identity (x - 0.0 == x, x - (-0.0) == x + 0)."""
        dx, dy = Val.of(dx), Val.of(dy)
        fl = (0 if dx.zero() else F_AX) | (0 if dy.zero() else F_AY)
        if fl:
            op = Op(OP_ALIGN, fl, consts=[dx, dy], elem=elem)
            op.flops = op.flops_fast = bool(fl & F_AX) + bool(fl & F_AY)
            self.emit(op)

    def drift(self, form, c0, c1=None, elem=-1):
        """methods.drift (ufo/methods.py:28-43) on the length text the caller
        pasted: form DF_MUL ``L``, DF_MUL2 ``L * f``, DF_DIV ``(A) / d``."""
        c0 = Val.of(c0)
        if self.flags & EXACT:
            # l = {length} / sqrt(...): the pasted length folds to one constant
            if form == DF_MUL2:
                lc = c0 * c1
            elif form == DF_DIV:
                lc = c0 / c1
            else:
                lc = c0
            op = Op(OP_DRIFT, F_EXACT, ints=[DF_MUL], consts=[lc], elem=elem)
            op.flops = op.flops_fast = 11
            self.emit(op)
            return
        form, consts = self._drift_form(form, c0, c1)
        op = Op(OP_DRIFT, 0, ints=[form], consts=consts, elem=elem)
        op.flops = {DF_MUL: 4, DF_MUL2: 6, DF_DIV: 6}[form]
        op.flops_fast = 4
        self.emit(op)

    @staticmethod
    def _drift_form(form, c0, c1):
        """Exact rewrites: (px*L)*1.0 == px*L; (px*A)/1.0 == px*A; (px*A)/2^k ==
        px*(A/2^k) (scaling by a power of two commutes with rounding)."""
        if form == DF_MUL2:
            c1 = Val.of(c1)
            if np.all(np.asarray(c1.v) == 1.0):
                return DF_MUL, [c0]
            return DF_MUL2, [c0, c1]
        if form == DF_DIV:
            c1 = Val.of(c1)
            d = np.asarray(c1.v)
            if np.all(d == d.flat[0]):
                dv = float(d.flat[0])
                m, e = math.frexp(dv)
                if dv != 0 and m == 0.5 and math.isfinite(dv):
                    return DF_MUL, [c0 / c1]
            # (px*A)/d: the kernels divide by d exactly (Markstein correction with
            # r = RN(1/d)); A/d serves the FMA mode's px*(A/d)
            return DF_DIV, [c0, c1, 1.0 / c1, c0 / c1]
        return DF_MUL, [c0]

    def kick(self, knl, ksl, elem, weak=None):
        ks = KickSpec(knl, ksl, self.flags)
        nn, nsk, mn, ms, consts = ks.packed()
        fl = F_ACHRO if self.flags & ACHROMATIC else 0
        op = Op(OP_KICK, fl, ints=[nn, nsk, mn, ms], consts=consts, elem=elem)
        op.flops = ks.flops()
        op.flops_fast = ks.flops_fast()
        self.emit(op)

    def teapot(self, length, slices, knl, ksl, angle, elem, lenf):
        """methods.teapot (ufo/methods.py:79-97).  ``length`` is the pasted
        text ``L * f``: (L, f) with f the fracture fraction."""
        L, f = length
        Lf = Val.of(L) * f
        if slices == 1:
            outer = Lf / 2.0
        else:
            outer = Lf / float(2 * (1 + slices))
        inner_a = Lf - 2.0 * outer
        inner_d = Val.of(float(slices - 1.0))
        # weak focusing: (A*f) * (A*f) * (L*f) / N / (L*f) / (L*f)
        if angle is None:
            weak = Val.of(0.0) * Lf / float(slices) / Lf / Lf
        else:
            A, fa = angle
            Af = Val.of(A) * fa
            weak = Af * Af * Lf / float(slices) / Lf / Lf
        # coefficients: ({k}*{length}/{slices}) -> ((k*L)*f)/N
        kn = [(Val.of(k) * L) * f / float(slices) for k in knl]
        ksk = [(Val.of(k) * L) * f / float(slices) for k in ksl]
        ks = KickSpec(kn, ksk, self.flags)
        nn, nsk, mn, ms, kconsts = ks.packed()

        fl = F_ACHRO if self.flags & ACHROMATIC else 0
        if self.flags & YOSHIDA:
            if self.flags & EXACT:
                raise NotImplementedError('YOSHIDA integration with EXACT drifts')
            return self._yoshida(Lf, slices, ks, weak, elem)
        exact = bool(self.flags & EXACT)
        if exact:
            fl |= F_EXACT
            fo, oc = DF_MUL, [outer]
            fi, ic = DF_MUL, [inner_a / inner_d]
        else:
            fo, oc = DF_MUL, [outer]
            fi, ic = self._drift_form(DF_DIV, inner_a, inner_d)
        if slices == 1:
            fi, ic = DF_MUL, []
        if not weak.zero():
            fl |= F_WEAK
            wc = [weak]
        else:
            fl |= F_WEAKZ
            wc = []
        fl |= fo << SH_FOUTER | fi << SH_FINNER
        op = Op(OP_TEAPOT, fl, ints=[slices, nn, nsk, mn, ms], consts=oc + ic + kconsts + wc,
                elem=elem)
        dflops_o = 11 if exact else 4
        dflops_i = 11 if exact else {DF_MUL: 4, DF_MUL2: 6, DF_DIV: 6}[fi]
        wflops = 2 if fl & F_WEAK else 0
        op.flops = 2 * dflops_o + (slices - 1) * dflops_i + slices * (ks.flops() + wflops)
        if exact:
            op.flops_fast = (slices + 1) * 11 + slices * (ks.flops_fast() + wflops)
        else:
            # what the FMA-mode kernel executes (csrc/ops.cuh: teapot_v): drifts 2
            # FMA each; the kick strength formed once per element (quadrupole
            # t = K o: 1 mul; sextupole K o and t = (K o) 0.5: 2 muls); per
            # slice the kick (quadrupole 2 FMA, sextupole 2 mul + 3 FMA, general
            # the power-series Horner) and the weak term (1 FMA)
            pat = 0 if nsk else 1 if (nn == 2 and mn == 2) else 2 if (nn == 3 and mn == 4) \
                else 3 if mn == 0 else 0
            per_elem = {0: 0, 1: 1, 2: 2, 3: 0}[pat]
            kick = {0: ks.flops_fast() if (mn | ms) else 0, 1: 4, 2: 8, 3: 0}[pat]
            op.flops_fast = 4 * (slices + 1) + per_elem + slices * (kick + wflops)
        self.emit(op)

    def _yoshida(self, Lf, slices, ks, weak, elem):
        """Build's extra integrator: each of the N slices is a 4th-order
        Yoshida drift-kick composition (3 kicks of weights d_i/N, 4 drifts of
        c_i*L/N).  No reference counterpart."""
        fl = F_YOSHIDA | (F_ACHRO if self.flags & ACHROMATIC else 0)
        # kick coefficients scaled per slice are (k*L*f)/N; Yoshida weights
        # multiply them, drifts are c_i * (L*f)/N
        nn, nsk, mn, ms, kconsts = ks.packed()
        dl = Lf / float(slices)
        drifts = [dl * c for c in YOSHIDA_C]
        wts = [Val.of(d) for d in YOSHIDA_D]
        if not weak.zero():
            fl |= F_WEAK
            wc = [weak]
        else:
            fl |= F_WEAKZ
            wc = []
        op = Op(OP_TEAPOT, fl, ints=[slices, nn, nsk, mn, ms],
                consts=drifts + wts + kconsts + wc, elem=elem)
        # executed arithmetic (no reference expression to follow): the kernel
        # forms the weighted strengths once per element (quadrupole: K*o*w_i,
        # sextupole: K*o*0.5*w_i, weak: W*w_i); per slice 4 drifts (4 flops
        # each) and 3 kicks: quadrupole 4, sextupole 10, general Horner + 4
        # (weighted accumulation), plus 2 per weak term
        pat = 0 if nsk else 1 if (nn == 2 and mn == 2) else 2 if (nn == 3 and mn == 4) else \
            3 if mn == 0 else 0
        achro = bool(self.flags & ACHROMATIC)
        per_elem = {0: 0, 1: 3 + (0 if achro else 1), 2: 4 + (0 if achro else 1), 3: 0}[pat] + \
            (3 if wc else 0)
        # general kicks: FMA programs evaluate the dense power series (plus the
        # strength factor o w), strict ones the reference's Horner + the
        # weighted accumulation
        general = ks.flops_fast() + 1 if self.flags & FMA else ks.flops() + 4
        kick = {0: general, 1: 4, 2: 10, 3: 0}[pat]
        op.flops = op.flops_fast = per_elem + slices * (16 + 3 * (kick + (2 if wc else 0)))
        self.emit(op)

    def edge(self, length, angle, e, fringe, elem):
        """methods.edge (ufo/methods.py:199-211) with the full (unfractured)
        length and angle: curvature = angle/L (* oodppo);
        psi = e - 2*curv*fringe/cos(e)*(1 + sin(e)*sin(e));
        px += x*curv*tan(e); py -= y*curv*tan(psi)."""
        achro = bool(self.flags & ACHROMATIC)
        A = Val.of(angle) / Val.of(length)
        e = Val.of(e)
        fringe = Val.of(fringe)
        cos_e = _fn('cos', e)
        sin_e = _fn('sin', e)
        onepss = 1.0 + sin_e * sin_e
        t1 = _fn('tan', e)
        fl = F_ACHRO if achro else 0
        if achro:
            psi = e - 2.0 * A * fringe / cos_e * onepss
            t2 = _fn('tan', psi)
            consts = [A, t1, t2]
        elif fringe.zero():
            # psi = e - (+-0) == e exactly for finite curvature
            t2 = t1
            consts = [A, t1, t2]
        else:
            fl |= F_RTPSI
            consts = [A, t1, e, fringe, cos_e, onepss]
        fl |= F_T1Z if t1.zero() else F_T1
        if fl & F_RTPSI:
            fl |= F_T2
        else:
            fl |= F_T2Z if consts[2].zero() else F_T2
        op = Op(OP_EDGE, fl, consts=consts, elem=elem)
        base = 0 if (achro or not fl & (F_T1 | F_T2)) else 1
        op.flops = base + (3 if fl & F_T1 else 0) + (3 if fl & F_T2 else 0) + \
            (7 if fl & F_RTPSI else 0)
        op.flops_fast = op.flops
        self.emit(op)

    def thick_quad(self, L, f, k1, elem):
        """methods.quadrupole thick branch (ufo/methods.py:99-134)."""
        achro = bool(self.flags & ACHROMATIC)
        k = Val.of(k1)
        Lf = Val.of(L) * f
        fl = F_ACHRO if achro else 0
        consts = [k, Lf]
        if achro:
            k2 = _fn('sqrt', _fn('fabs', k))
            k2l = Lf * k2
            consts += [k2, _fn('cos', k2l), _fn('sin', k2l), _fn('cosh', k2l), _fn('sinh', k2l)]
            fl |= F_CONST
        op = Op(OP_THICKQ, fl, consts=consts, elem=elem)
        op.flops = op.flops_fast = 16 + (0 if achro else 4)
        self.emit(op)

    def thick_bend(self, L, f, angle, k1, elem):
        """methods.sbend thick branch (ufo/methods.py:136-196)."""
        achro = bool(self.flags & ACHROMATIC)
        Lf = Val.of(L) * f
        Af = Val.of(angle) * f
        c0 = Af / Lf
        k1 = Val.of(k1)
        fl = F_ACHRO if achro else 0
        consts = [c0, k1, Lf]
        if achro:
            curv = c0
            kv = k1
            k2v = _fn('sqrt', _fn('fabs', kv))
            k2lv = Lf * k2v
            kx = kv + curv * curv
            k2x = _fn('sqrt', _fn('fabs', kx))
            k2lx = Lf * k2x
            consts += [kv, k2v, _fn('cos', k2lv), _fn('sin', k2lv), _fn('cosh', k2lv),
                       _fn('sinh', k2lv),
                       kx, k2x, _fn('cos', k2lx), _fn('sin', k2lx), _fn('cosh', k2lx),
                       _fn('sinh', k2lx), _fn('fabs', kx)]
            fl |= F_CONST
        op = Op(OP_THICKB, fl, consts=consts, elem=elem)
        op.flops = op.flops_fast = 30 + (6 if not achro else 0)
        self.emit(op)

    def wire(self, x, y, k, elem):
        op = Op(OP_WIRE, 0, consts=[Val.of(x), Val.of(y), Val.of(k)], elem=elem)
        op.flops = op.flops_fast = 9
        self.emit(op)

    def aperture(self, window, elem):
        code = _ap.compile_window(window)
        # `x*x + y*y < c == 0` -> lost when !((x*x + y*y) < c): evaluated in
        # registers by the kernels (same operations, same order)
        circle = [(_ap.VAR, 0.0), (_ap.VAR, 0.0), (_ap.MUL, 0.0), (_ap.VAR, 2.0), (_ap.VAR, 2.0),
                  (_ap.MUL, 0.0), (_ap.ADD, 0.0), (_ap.PUSH, None), (_ap.LT, 0.0),
                  (_ap.PUSH, 0.0), (_ap.EQ, 0.0)]
        if len(code) == len(circle) and all(
                a[0] == b[0] and (b[1] is None or a[1] == b[1]) for a, b in zip(code, circle)):
            op = Op(OP_APERTURE, F_CIRCLE, ints=[0], consts=[Val.of(code[7][1])], elem=elem)
            op.flops = op.flops_fast = 3
            self.emit(op)
            return
        consts = []
        for opc, v in code:
            consts += [Val.of(float(opc)), Val.of(float(v))]
        op = Op(OP_APERTURE, 0, ints=[len(code)], consts=consts, elem=elem)
        op.flops = op.flops_fast = sum(1 for opc, _ in code if opc in (
            _ap.ADD, _ap.SUB, _ap.MUL, _ap.DIV, _ap.SQRT))
        self.emit(op)


def _dyn_kick(lw, knl, ksl, elem):
    """A thin kick some of whose coefficients are run-time expressions: the
    reference's untrimmed Horner (methods.kick, ufo/methods.py:45-76, LINEAR
    truncation included) with each coefficient evaluated per particle and
    turn.  Table: for every coefficient, normal then skew, [n, (opcode,
    value) x n]; a plain coefficient is the one-op program PUSH c."""
    norm = KickSpec._trunc(list(knl), lw.flags)
    skew = KickSpec._trunc(list(ksl), lw.flags)
    if len(norm) > MAX_ORDERS or len(skew) > MAX_ORDERS:
        raise NotImplementedError(f'more than {MAX_ORDERS} multipole orders')
    consts = []
    flops = 0
    for c in norm + skew:
        code = c.code if isinstance(c, Dyn) else [(_cx.PUSH, Val.of(c))]
        consts.append(Val.of(float(len(code))))
        for opc, v in code:
            consts += [Val.of(float(opc)), Val.of(v)]
            flops += opc in (_cx.ADD, _cx.SUB, _cx.MUL, _cx.DIV)
    fl = F_ACHRO if lw.flags & ACHROMATIC else 0
    op = Op(OP_DYNKICK, fl, ints=[len(norm), len(skew), len(consts)], consts=consts, elem=elem)
    # the untrimmed kick: per order 4 mul + 2 add/sub + 2 div, plus the oodppo products
    n_terms = sum(max(len(lst) - 1, 0) for lst in (norm, skew))
    op.flops = op.flops_fast = flops + 8 * n_terms + (0 if fl else len(norm) + len(skew)) + \
        2 * (len(norm) > 0) + 2 * (len(skew) > 0)
    lw.emit(op)


def _to_value(v, seed_values, name, coord_cols=()):
    """One attribute value handed to a base-class method(): numbers become
    Vals; C text becomes a Val when it reads neither the turn nor the particle
    (folded per seed as the reference's compiler would compute it) and a Dyn
    otherwise."""
    if isinstance(v, (Val, Dyn)):
        return v
    if isinstance(v, str):
        code, _, top = _cx.compile_expr(v, f'{name} = {v!r}', allow_params=True)
        if top is not None:
            raise NotImplementedError(
                f'{name} = {v!r}: the reference pastes this text next to other operators, '
                f'where C precedence regroups it; wrap it in parentheses')
        if any(op == _cx.VAR and int(val) in (1, 3) for op, val in code):
            raise NotImplementedError(f'{name} = {v!r}: px and py change within the kick')
        if _cx.depth(code) > DYN_STACK:
            raise NotImplementedError(f'{name} = {v!r}: expression too deep')
        cols = [int(val) for op, val in code if op == _cx.PARAM]
        for c in cols:
            if c >= seed_values.shape[1]:
                raise IndexError(f'{name} = {v!r}: parameters[{c}] outside the parameter list')
            if c in coord_cols:
                raise NotImplementedError(f'{name} = {v!r}: parameters[{c}] is a particle '
                                          f'coordinate, not a lattice value')
        if _cx.is_constant(code):
            vals = np.array([_cx.evaluate(code, params=row, correctly_rounded=not cols)
                             for row in seed_values])
            return Val(vals if cols else np.float64(vals[0]), not cols)
        prog = [(_cx.PUSH, Val(seed_values[:, int(val)].copy(), False)) if op == _cx.PARAM
                else (op, Val.of(val)) for op, val in code]
        return Dyn(prog, v)
    if isinstance(v, (list, tuple)):
        return [_to_value(x, seed_values, f'{name}[{i}]', coord_cols) for i, x in enumerate(v)]
    return Val.of(float(v))


def _user_method(elem, idx, cols, seed_values, flags, where, coord_cols=()):
    """Run an element's own ``method()`` override the way ufo/lattice.py:107-113
    calls it (bound parameters as the text ``parameters[i]``, plus flags and
    fracture) and return the attribute values it handed to its base class."""
    tokens = {name: f'parameters[{col}]' for name, col in cols.items()}
    out = elem.method(flags=flags, fracture=list(where), **tokens)
    passes = [p for p in (out if isinstance(out, (list, tuple)) else [out])
              if isinstance(p, E.PassMethod)]
    if len(passes) != 1 or passes[0].element is not elem:
        raise NotImplementedError(
            f'{elem.label}: method() must return its base class method() result; user '
            f'OpenCL pass methods cannot run in the data-driven GPU kernels')
    prm = {}
    for name, v in passes[0].values.items():
        if name in ('flags', 'fracture') or v is None:
            continue
        prm[name] = _to_value(v, seed_values, f'{elem.label}.{name}', coord_cols)
    return prm


def reads_turn(prog):
    """True when an aperture window or a dynamic-kick coefficient of the
    compiled program reads ``turn`` (only the Track and StableAperture kernels
    of the reference define it)."""
    T = prog.table[0]
    for row in prog.ops:
        kind, fl, off = int(row[0]), int(row[1]), int(row[2])
        if kind == OP_APERTURE and not fl & F_CIRCLE:
            progs = [(off, int(row[3]))]
        elif kind == OP_DYNKICK:
            progs, q = [], off
            while q < off + int(row[5]):
                n = int(T[q])
                progs.append((q + 1, n))
                q += 1 + 2 * n
        else:
            continue
        for start, n in progs:
            codes = T[start:start + 2 * n].reshape(n, 2)
            if np.any((codes[:, 0] == _cx.VAR) & (codes[:, 1] == _cx.VARS['turn'])):
                return True
    return False


def _has_dyn(v):
    if isinstance(v, Dyn):
        return True
    if isinstance(v, list):
        return any(_has_dyn(x) for x in v)
    return False


def _mp_list(lst, name, seed_values=None):
    if isinstance(lst, str) or isinstance(lst, Val):
        raise NotImplementedError(f'{name} cannot be a parameter as a whole vector; '
                                  f'use the scalar names (e.g. dk2, k3s)')
    out = []
    for i, v in enumerate(lst):
        if isinstance(v, str):  # C text in the lattice itself, pasted by the reference
            v = _to_value(v, seed_values if seed_values is not None else np.zeros((1, 1)),
                          f'{name}[{i}]')
        out.append(v if isinstance(v, Dyn) else Val.of(v))
    return out


def _dk_from_kwargs(kwargs, dkn, dks):
    """__dk_from_kwargs__ (ufo/elements.py:14-23): dkN / dkNs overrides,
    padding the lists with zeros."""
    for prm, value in kwargs.items():
        if prm[:2] == 'dk' and prm[2:].isdigit():
            idx = int(prm[2:])
            dkn += [Val.of(0.0)] * (idx + 1 - len(dkn))
            dkn[idx] = value
        if prm[:2] == 'dk' and prm[-1:] == 's' and prm[2:-1].isdigit():
            idx = int(prm[2:-1])
            dks += [Val.of(0.0)] * (idx + 1 - len(dks))
            dks[idx] = value


def _resolve(elem, prm, name, default=None):
    """``value = value or self.value``: a bound parameter always wins."""
    if name in prm:
        return prm[name]
    return Val.of(getattr(elem, name, default) if default is None else
                  getattr(elem, name, default))


def lower_element(lw, elem, idx, prm, where, cols=None, seed_values=None, coord_cols=()):
    """Lower one flat element.  ``prm`` maps attribute name -> Val (bound
    parameters); ``where`` is its fracture list (fractions in [0, 1)).  An
    element whose class overrides ``method()`` is lowered from the values its
    override hands to the base class (``cols``: attribute -> parameter column,
    ``seed_values``: the per-seed parameter rows)."""
    flags = lw.flags
    if type(elem).method is not E.Element.method:
        if seed_values is None:
            seed_values = np.zeros((lw.S, 1))
        prm = _user_method(elem, idx, cols or {}, seed_values, flags, where, coord_cols)
    kind = elem.kind
    if kind != 'multipole' and any(_has_dyn(v) for v in prm.values()):
        raise NotImplementedError(
            f'{elem.label}: values that depend on the turn or the particle are supported for '
            f'thin multipole coefficients (knl, ksl, kN, kNs) only')
    pieces = []
    f0 = 0.0
    for f in list(where) + [1.0]:
        pieces.append(f - f0)
        f0 = f

    def chunks(emit_piece, prefix=None, suffix=None):
        for i, fr in enumerate(pieces):
            if i > 0:
                lw.new_segment()
            if i == 0 and prefix:
                prefix()
            emit_piece(fr)
            if i == len(pieces) - 1 and suffix:
                suffix()

    if kind == 'marker':
        return
    if kind == 'drift':
        # Drift.method takes no **kwargs (ufo/elements.py:98): other names raise
        extra = [k for k in prm if k != 'length']
        if extra:
            raise TypeError(f"Drift.method() got an unexpected keyword argument '{extra[0]}'")
        L = _resolve(elem, prm, 'length')
        chunks(lambda fr: lw.drift(DF_MUL2, L, fr, elem=idx))
        return
    if kind == 'multipole':
        knl = _mp_list(prm['knl'] if 'knl' in prm else elem.knl, 'knl', seed_values)
        ksl = _mp_list(prm['ksl'] if 'ksl' in prm else elem.ksl, 'ksl', seed_values)
        dx = _resolve(elem, prm, 'dx')
        dy = _resolve(elem, prm, 'dy')
        for p, v in prm.items():
            if p[:1] == 'k' and p[1:].isdigit():
                knl[int(p[1:])] = v
            if p[:1] == 'k' and p[-1:] == 's' and p[1:-1].isdigit():
                ksl[int(p[1:-1])] = v
        if _has_dyn(dx) or _has_dyn(dy):
            raise NotImplementedError(f'{elem.label}: turn-dependent offsets')
        lw.align(dx, dy, idx)
        if _has_dyn(knl) or _has_dyn(ksl):
            _dyn_kick(lw, knl, ksl, idx)
        else:
            lw.kick(knl, ksl, idx)
        lw.align(-dx, -dy, idx)
        return
    if kind == 'wire':
        lw.wire(_resolve(elem, prm, 'x'), _resolve(elem, prm, 'y'), _resolve(elem, prm, 'k'),
                idx)
        return
    if kind == 'aperture':
        lw.aperture(elem.window, idx)
        return

    slices = prm.get('slices', None)
    if slices is not None:
        raise NotImplementedError('slices cannot be a parameter')
    slices = int(elem.slices)
    L = _resolve(elem, prm, 'length')
    dx = _resolve(elem, prm, 'dx')
    dy = _resolve(elem, prm, 'dy')
    dkn = _mp_list(elem.dkn, 'dkn') if 'dkn' not in prm else _mp_list(prm['dkn'], 'dkn')
    dks = _mp_list(elem.dks, 'dks') if 'dks' not in prm else _mp_list(prm['dks'], 'dks')
    _dk_from_kwargs(prm, dkn, dks)
    align_in = lambda: lw.align(dx, dy, idx)
    align_out = lambda: lw.align(-dx, -dy, idx)

    if kind == 'quadrupole':
        k1 = _resolve(elem, prm, 'k1')
        if flags & KICK:
            knl = _pad(dkn, 2)
            knl[1] = knl[1] + k1
            chunks(lambda fr: lw.teapot((L, fr), slices, knl, dks, None, idx, fr),
                   align_in, align_out)
        else:
            chunks(lambda fr: lw.thick_quad(L, fr, k1, idx), align_in, align_out)
        return
    if kind in ('sbend', 'rbend'):
        angle = _resolve(elem, prm, 'angle')
        k1 = _resolve(elem, prm, 'k1')
        e1 = _resolve(elem, prm, 'e1')
        e2 = _resolve(elem, prm, 'e2')
        hgap = _resolve(elem, prm, 'hgap')
        fint = _resolve(elem, prm, 'fint')
        fringe = Val.of(hgap) * Val.of(fint)
        if kind == 'rbend':
            e1 = e1 + angle * 0.5
            e2 = e2 + angle * 0.5

        def pre():
            align_in()
            lw.edge(L, angle, e1, fringe, idx)

        def post():
            lw.edge(L, angle, e2, fringe, idx)
            align_out()
        if flags & KICK:
            knl = _pad(dkn, 2)
            knl[1] = knl[1] + k1
            chunks(lambda fr: lw.teapot((L, fr), slices, knl, dks, (angle, fr), idx, fr),
                   pre, post)
        else:
            chunks(lambda fr: lw.thick_bend(L, fr, angle, k1, idx), pre, post)
        return
    if kind in ('sextupole', 'octupole'):
        main = 'k2' if kind == 'sextupole' else 'k3'
        order = 3 if kind == 'sextupole' else 4
        kmain = _resolve(elem, prm, main)
        knl = _pad(dkn, order)
        knl[order - 1] = knl[order - 1] + kmain
        # the reference passes dks, not the padded skew list (methods.py:219,227),
        # so k2s / k3s never reach the kick
        chunks(lambda fr: lw.teapot((L, fr), slices, knl, dks, None, idx, fr),
               align_in, align_out)
        return
    raise NotImplementedError(f'element type {type(elem).__name__}')


# ------------------------------------------------------------------ program

class Program:
    """A compiled line.

    ops      int32 [n_ops, 8]   kind, flags, table offset, i0..i4
    table    float64 [n_seeds, stride]
    n_dumps  observation points executed per turn (D)
    count    len(where) as the reference sizes its output (>= n_dumps)
    """

    def __init__(self, segments, n_seeds, n_elements, count, dump_end):
        self.segments = segments
        self.n_seeds = n_seeds
        self.n_elements = n_elements
        self.count = count
        ops = []
        consts = []
        off = 0
        dump = 0
        self.flops = 0
        self.flops_fast = 0
        self.op_elem = []
        for si, seg in enumerate(segments):
            if si > 0:
                ops.append([OP_OBSERVE, 0, 0, dump, 0, 0, 0, 0])
                self.op_elem.append(-1)
                dump += 1
            for op in seg:
                row = [op.kind, op.flags, off] + op.ints + [0] * (5 - len(op.ints))
                ops.append(row)
                self.op_elem.append(op.elem)
                consts.extend(op.consts)
                off += len(op.consts)
                self.flops += op.flops
                self.flops_fast += op.flops_fast
        if dump_end:
            ops.append([OP_OBSERVE, 0, 0, dump, 0, 0, 0, 0])
            self.op_elem.append(-1)
            dump += 1
        self.n_dumps = dump
        self.ops = np.ascontiguousarray(np.array(ops, dtype=np.int32).reshape(-1, OP_WORDS))
        stride = max(off, 1)
        table = np.zeros((n_seeds, stride), dtype=np.float64)
        for j, c in enumerate(consts):
            table[:, j] = c.v
        self.table = np.ascontiguousarray(table)

    @property
    def n_ops(self):
        return self.ops.shape[0]

    def describe(self):
        lines = []
        for i, row in enumerate(self.ops):
            lines.append(f'{i:5d} {OP_NAMES[row[0]]:8s} flags={row[1]:#x} toff={row[2]} '
                         f'ints={list(row[3:])} elem={self.op_elem[i]}')
        return '\n'.join(lines)


def parse_parameters(parameters):
    """Split the reference's parameter list into coordinate columns and lattice
    bindings.  Returns (coord_cols {name: col}, bindings [(col, key, attr)])."""
    coord_cols = {}
    binds = []
    for i, p in enumerate(parameters):
        if isinstance(p, str) and p in COORDS:
            coord_cols[p] = i
        binds.append((i, p))
    return coord_cols, binds


def element_bindings(flat, parameters):
    """For every flat element: {attr: column}, mirroring ufo/lattice.py:109-110
    (``p[0] == label or p[0] == idx``; later columns override earlier)."""
    out = []
    for idx, elem in enumerate(flat):
        prms = {}
        for i, p in enumerate(parameters):
            try:
                key = p[0]
            except (TypeError, IndexError):
                continue
            if key == elem.label or key == idx:
                try:
                    name = p[1]
                except IndexError:
                    raise IndexError(f'parameter {p!r} matches element {elem.label!r} '
                                     f'but names no attribute')
                prms[name] = i
        out.append(prms)
    return out


def fractures(n, where):
    """Per-element fracture lists and pre-element dump flags, mirroring
    ufo/lattice.py:101-105."""
    per = []
    pre = []
    for idx in range(n):
        w = [f - idx for f in where if f != '*' and idx <= f < idx + 1]
        if 0 in w:
            w.remove(0)
            pre.append(True)
        else:
            pre.append(False)
        per.append(w)
    return per, pre


def _merge_drifts(ops):
    """FMA mode: fold each plain drift (x += px L) into the outer drift of a
    nearby non-exact TEAPOT element (x += px (L + Lo)): one op and two FMAs
    fewer per drift; the sum of lengths changes the rounding only.  A drift
    commutes with the alignment shifts between it and the teapot (they move x
    and y, not px and py), so those may lie in between; apertures, edges and
    observation points may not.  A teapot that absorbs a drift after it keeps
    its exit length as a separate constant (F_SPLITO).  The reference count
    (``flops``) keeps the merged drifts; the executed count (``flops_fast``)
    does not: their arithmetic is gone."""
    def teapot_ok(op):
        return (op.kind == OP_TEAPOT and not op.flags & (F_EXACT | F_YOSHIDA)
                and (op.flags >> SH_FOUTER) & 3 == DF_MUL)

    def drift_ok(op):
        return op.kind == OP_DRIFT and not op.flags & F_EXACT and op.ints[0] == DF_MUL

    def split(t):
        if not t.flags & F_SPLITO:  # the exit keeps the original length
            t.consts = t.consts + [t.consts[0]]
            t.flags |= F_SPLITO

    out = []
    i = 0
    n = len(ops)
    while i < n:
        op = ops[i]
        if drift_ok(op):
            k = i + 1
            while k < n and ops[k].kind == OP_ALIGN:
                k += 1
            if k < n and teapot_ok(ops[k]):  # into the entry of the next teapot
                t = ops[k]
                split(t)
                t.consts[0] = op.consts[0] + t.consts[0]
                t.flops += op.flops
                i += 1
                continue
            k = len(out) - 1
            while k >= 0 and out[k].kind == OP_ALIGN:
                k -= 1
            if k >= 0 and teapot_ok(out[k]):  # into the exit of the previous one
                t = out[k]
                split(t)
                t.consts[-1] = t.consts[-1] + op.consts[0]
                t.flops += op.flops
                i += 1
                continue
        out.append(op)
        i += 1
    return out


def _linearize(ops):
    """FMA programs: a teapot or Yoshida element with no kick coefficient (a bend
    without gradient or errors, or a zero-strength magnet) is, for finite
    coordinates, a linear map that does not depend on the particle's dp: its
    drifts and weak-focusing kicks compose on the host into one 2x2 matrix for
    (x, px) and one drift length for (y, py) (OP_LINEAR: 5 FP64 instructions
    instead of 4 per slice), and its zero-angle edges are dropped.  The composition is formed per seed in FP64, so
    results change in rounding only (tolerance parity, like the rest of FMA
    mode).  The reference count of the element is kept; the executed count is
    the op's own."""
    out = []
    for op in ops:
        if op.kind != OP_TEAPOT or op.flags & F_EXACT:
            out.append(op)
            continue
        N, nn, ns, mn, ms = op.ints[:5]
        if mn or ms:
            out.append(op)
            continue
        c = op.consts
        weak = bool(op.flags & F_WEAK)
        steps = []  # ('d', L) drift, ('k', W) weak kick px -= W x
        if op.flags & F_YOSHIDA:
            d, w = c[0:4], c[4:7]
            W = c[7] if weak else None
            for _ in range(N):
                steps.append(('d', d[0]))
                for k in range(3):
                    if weak:
                        steps.append(('k', W * w[k]))
                    steps.append(('d', d[k + 1]))
        else:
            fi = (op.flags >> SH_FINNER) & 3
            Lo = c[0]
            Li = None if N <= 1 else (c[1] if fi == DF_MUL else c[4])
            ck = 1 + (0 if N <= 1 else (4 if fi == DF_DIV else 1))
            W = c[ck] if weak else None
            Lx = c[ck + (1 if weak else 0)] if op.flags & F_SPLITO else Lo
            steps.append(('d', Lo))
            for sl in range(N):
                if weak:
                    steps.append(('k', W))
                steps.append(('d', Li if sl < N - 1 else Lx))
        m11, m12, m21, m22 = Val.of(1.0), Val.of(0.0), Val.of(0.0), Val.of(1.0)
        ly = Val.of(0.0)
        for kind, v in steps:
            if kind == 'd':   # x += px L
                m11, m12 = m11 + v * m21, m12 + v * m22
                ly = ly + v
            else:             # px -= W x
                m21, m22 = m21 - v * m11, m22 - v * m12
        lin = Op(OP_LINEAR, 0, consts=[m11, m12, m21, m22, ly], elem=op.elem)
        lin.flops = op.flops
        lin.flops_fast = 8  # x, px: a multiplication and an FMA each; y: one FMA
        out.append(lin)
    # the element's own zero edges (no face angle: their terms are structural
    # zeros, kept only to poison px, py when x, y are not finite) go with it:
    # the composed map already propagates non-finite values its own way
    linear = {op.elem for op in out if op.kind == OP_LINEAR}
    return [op for op in out if not (op.kind == OP_EDGE and op.elem in linear and
                                     not op.flags & (F_T1 | F_T2 | F_RTPSI))]


def _rcp_factorials(n):
    """1/k! for k = 0..n-1, each RN(1 / RN(k!)) with k! built by successive
    multiplication: the same doubles as the kernels' constant table
    (csrc/ufo_gb300.cu: ensure_constants)."""
    out, fact = [], 1.0
    for k in range(n):
        if k > 0:
            fact *= float(k)
        out.append(1.0 / fact)
    return out


def _append_series(ops):
    """FMA programs: a general kick (not the quadrupole or sextupole short
    form) is one complex Horner pass over S(z) = sum_n (kn_n + i ks_n) z^n / n!.
    Append to each such op, after all its other constants, the dense power
    series a_n = RN(kn_n * RN(1/n!)), b_n likewise, n = 0..top (structurally
    zero terms +0.0): the products the kernels would otherwise form at every
    order of every slice, with the same rounding, so results are unchanged
    bit for bit (F_PSER)."""
    for op in ops:
        if op.kind not in (OP_KICK, OP_TEAPOT) or op.flags & F_EXACT:
            continue
        if op.kind == OP_KICK:
            nn, ns, mn, ms = op.ints[:4]
            first = 0
        else:
            nn, ns, mn, ms = op.ints[1:5]
            if op.flags & F_YOSHIDA:
                first = 7
            else:
                fi = (op.flags >> SH_FINNER) & 3
                first = 1 + (0 if op.ints[0] <= 1 else 4 if fi == DF_DIV else 1)
        general = bool(ms) or not ((nn == 2 and mn == 2) or (nn == 3 and mn == 4) or mn == 0)
        if not general or not (mn | ms):
            continue
        M = (mn | ms).bit_length()
        rf = _rcp_factorials(M)
        cn = op.consts[first:first + bin(mn).count('1')]
        cs = op.consts[first + len(cn):first + len(cn) + bin(ms).count('1')]
        a, b = [], []
        for lst, mask, out in ((cn, mn, a), (cs, ms, b)):
            it = iter(lst)
            for j in range(M):
                out.append(next(it) * rf[j] if mask >> j & 1 else Val.of(0.0))
        op.consts = op.consts + a + b
        op.flags |= F_PSER


def compile_line(line, flags=0, parameters=(), where=(), seed_values=None, count=None,
                 dump_end=None, linearize=True):
    """Compile ``line`` for ``flags``.

    seed_values : float64 [n_seeds, len(parameters)] -- the distinct rows of
                  the parameter pool restricted to lattice columns (columns of
                  coordinate parameters are ignored).  None -> one seed with
                  every bound attribute = 0 (the value the reference's
                  zero-initialised parameter buffer holds).
    """
    flat = line.flatten() if hasattr(line, 'flatten') else list(line)
    parameters = list(parameters)
    where = list(where)
    if seed_values is None:
        seed_values = np.zeros((1, max(len(parameters), 1)))
    seed_values = np.asarray(seed_values, dtype=np.float64)
    S = seed_values.shape[0]
    lw = _Lowerer(flags, S)
    binds = element_bindings(flat, parameters)
    coord_cols = set(parse_parameters(parameters)[0].values())
    per, pre = fractures(len(flat), where)
    for idx, elem in enumerate(flat):
        if pre[idx]:
            lw.new_segment()
        prm = {name: Val(seed_values[:, col].copy(), False) for name, col in binds[idx].items()}
        lower_element(lw, elem, idx, prm, per[idx], binds[idx], seed_values, coord_cols)
    if flags & FMA:
        lw.segments = [_merge_drifts(seg) for seg in lw.segments]
        if linearize:
            lw.segments = [_linearize(seg) for seg in lw.segments]
        for seg in lw.segments:
            _append_series(seg)
    if dump_end is None:
        dump_end = -1 in where
    if count is None:
        count = len(where)
    return Program(lw.segments, S, len(flat), count, dump_end)
