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
