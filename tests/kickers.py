"""Time-dependent user elements for the tests: the two non-linear kickers of
the reference's HOWTO.md:84-200, written the way a user of the reference
writes them (a Multipole subclass whose method() hands C text of ``turn`` to
its base class), against this library's Multipole.  The golden fixtures hold
the reference's tracks of the same subclasses (tests/golden/make_golden.py)."""
import ufo_gb300 as ufo


class NLKGate(ufo.Multipole):
    """Kick only on turn 20."""

    def method(self, k1=None, **kwargs):
        k1 = k1 or self.knl[1]
        return super().method(k1=f'((turn == 20) ? {k1} : 0.)', **kwargs)


class NLKPulse(ufo.Multipole):
    """Half-sine pulse of length ``tau`` turns fired at turn ``t0`` (a
    parameter in the trigger-time scan)."""

    def __init__(self, label, t0=0., tau=0., **kwargs):
        super().__init__(label, **kwargs)
        self.tau = tau
        self.t0 = t0
        self.parameters += ['tau', 't0']

    def method(self, k1=None, t0=None, tau=None, **kwargs):
        k1, t0, tau = k1 or self.knl[1], t0 or self.t0, tau or self.tau
        k = (f'((turn >= {t0}) && (turn < {t0} + {tau}) )? '
             f'{k1} * sin(3.1415 * ((float)turn - {t0}) / {tau}): 0.')
        return super().method(k1=f'({k})', **kwargs)


class SkewKick(ufo.Multipole):
    """A sextupole term every third turn and a skew quadrupole that flips sign
    after turn 4 (orders above 2 and the skew part of a time-dependent kick)."""

    def method(self, k2=None, k1s=None, **kwargs):
        k2, k1s = k2 or self.knl[2], k1s or self.ksl[1]
        return super().method(k2=f'((turn % 3 == 0) ? {k2} : 0.)',
                              k1s=f'((turn > 4) ? {k1s} : -{k1s})', **kwargs)
