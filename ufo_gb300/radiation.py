"""Synchrotron-radiation integrals from the Twiss functions of an ``Optics``
run: the host-side consumer of the tracking library's optics output that the
reference provides in ufo/radiation.py (``emittance``, ``RadiationIntegrals``).

The integrals are those of SLAC-1193 (Helm, Lee, Morton) for a combined-
function sector dipole of length L, bending angle theta (rho = L / theta) and
focusing k = k1, evaluated from the Twiss functions (alpha, beta, D, D') at
each observation point of the ``Optics`` object that sits on a dipole:

  I1 = sum <D> L / rho                I2 = sum L / rho^2
  I4 = sum <D> (1/rho^2 + 2 k) L / rho
  I5 = sum <H> L / |rho|^3

with <D> and <H> the closed-form averages over the magnet of the dispersion
and of the curly-H function, propagated through the magnet's linear map
(cos/sin for k > 0, cosh/sinh for k < 0), as ufo/radiation.py:37-81 writes
them.  Edge focusing is ignored, as in the reference.

Deviation: where |L sqrt(k)| < 1e-2 the closed forms cancel (at k = 0 they
are 0/0 and the reference returns NaN; at |k| = 1e-6 the <H> term has lost
four digits), so there the averages are taken by 8-point Gauss-Legendre
quadrature of the same propagated D(s) and H(s), written with sin(x)/x and
sin^2(x/2) forms that stay exact as k -> 0.  Elsewhere the closed forms are
evaluated as written, so the results agree with the reference's to rounding.
"""
import numpy as np

from . import constants as _c
from .lattice import Beam


class RadiationIntegrals:
    """I1, I2, I4, I5 and the damping partition numbers Jx = 1 - I4/I2,
    Jt = 1 + I4/I2 (ufo/radiation.py:12-33).  ``U0`` (energy loss per turn,
    GeV) and ``Ex`` (equilibrium horizontal emittance, m) are for the default
    ``Beam`` (3 GeV electrons), as in the reference; ``energy_loss(beam)`` and
    ``equilibrium_emittance(beam)`` take another beam."""

    def __init__(self, I1, I2, I4, I5):
        self.I1 = I1
        self.I2 = I2
        self.I4 = I4
        self.I5 = I5
        self.Jx = 1. - I4 / I2
        self.Jt = 1. + I4 / I2

    def energy_loss(self, beam=None):
        beam = beam if beam is not None else Beam()
        return _c.radiation_loss_constant * (beam.energy * 1e-9) ** 4 * self.I2

    def equilibrium_emittance(self, beam=None):
        beam = beam if beam is not None else Beam()
        return _c.quantum_radiation_constant * beam.gamma ** 2 * self.I5 / self.I2 / self.Jx

    U0 = property(energy_loss)
    Ex = property(equilibrium_emittance)


_GL_X, _GL_W = np.polynomial.legendre.leggauss(8)


def _closed_form(L, theta, k, alpha, beta, gamma, d, dp):
    """<D> and <H> by the closed forms of ufo/radiation.py:53-79."""
    rho = L / theta
    sq = np.sqrt(np.abs(k))
    phi = L * sq
    foc = k >= 0
    C = np.where(foc, np.cos(phi), np.cosh(phi))
    S = np.where(foc, np.sin(phi), np.sinh(phi))
    mean_d = d * S / phi + dp * (1. - C) / (L * k) + (phi - S) / (rho * phi * k)
    mean_h = gamma * d * d + 2. * alpha * d * dp + beta * dp * dp
    mean_h = mean_h + 2. * theta * (-(gamma * d + alpha * dp) * (phi - S) / (sq * k * L ** 2)
                                    + (alpha * d + beta * dp) * (1. - C) / (k * L ** 2))
    mean_h = mean_h + theta * theta * (gamma * (3. * phi - 4. * S + S * C) / (2. * sq * k * k * L ** 3)
                                       - alpha * (1. - C) ** 2 / (k * k * L ** 3)
                                       + beta * (phi - C * S) / (2. * phi * k * L ** 2))
    return mean_d, mean_h


def _by_quadrature(L, theta, k, alpha, beta, gamma, d, dp):
    """<D> and <H> averaged over Gauss-Legendre nodes of the magnet, with the
    horizontal map m = [[C, S/w], [-k S/w, C]] (w = sqrt|k|; cos/sin for
    k >= 0, cosh/sinh for k < 0) written so that k -> 0 is exact:
      S/w = s sinc(w s),  (1 - C)/k = 2 (sin(w s/2)/w)^2 (sinh for k < 0)
      D(s) = C D0 + (S/w) D0' + (1 - C)/(k rho)
      D'(s) = -k (S/w) D0 + C D0' + (S/w)/rho
      H(s) = gamma(s) D^2 + 2 alpha(s) D D' + beta(s) D'^2"""
    rho = (L / theta)[:, None]
    s = L[:, None] * (_GL_X[None] + 1.) / 2.
    w = np.sqrt(np.abs(k))[:, None]
    foc = (k >= 0)[:, None]
    x = w * s
    xh = x / 2.
    safe = np.where(x == 0., 1., x)
    safe_h = np.where(xh == 0., 1., xh)
    sinc = np.where(x == 0., 1., np.where(foc, np.sin(safe), np.sinh(safe)) / safe)
    sinc_h = np.where(xh == 0., 1., np.where(foc, np.sin(safe_h), np.sinh(safe_h)) / safe_h)
    C = np.where(foc, np.cos(x), np.cosh(x))
    m12 = s * sinc                      # S / w
    omc = s * s * sinc_h * sinc_h / 2.  # (1 - C) / k
    kk = k[:, None]
    m21 = -kk * m12
    a0, b0, g0 = alpha[:, None], beta[:, None], gamma[:, None]
    D = C * d[:, None] + m12 * dp[:, None] + omc / rho
    Dp = m21 * d[:, None] + C * dp[:, None] + m12 / rho
    b = C * C * b0 - 2. * C * m12 * a0 + m12 * m12 * g0
    a = -C * m21 * b0 + (C * C + m12 * m21) * a0 - m12 * C * g0
    g = m21 * m21 * b0 - 2. * m21 * C * a0 + C * C * g0
    H = g * D * D + 2. * a * D * Dp + b * Dp * Dp
    wts = _GL_W[None] / 2.
    return np.sum(wts * D, axis=1), np.sum(wts * H, axis=1)


def _dipole_terms(L, theta, k, alpha, beta, d, dp):
    """Per-dipole rho, <D> and <H> (arrays over the dipoles)."""
    rho = L / theta
    gamma = (1. + alpha * alpha) / beta
    mean_d = np.empty_like(L)
    mean_h = np.empty_like(L)
    small = L * np.sqrt(np.abs(k)) < 1e-2
    for sel, fn in ((~small, _closed_form), (small, _by_quadrature)):
        if sel.any():
            mean_d[sel], mean_h[sel] = fn(L[sel], theta[sel], k[sel], alpha[sel], beta[sel],
                                          gamma[sel], d[sel], dp[sel])
    return rho, mean_d, mean_h


def emittance(optics):
    """Radiation integrals of the dipoles among ``optics.where`` (an ``Optics``
    run with observation points on the bends, e.g. ``where =
    ring.find(lambda e: hasattr(e, 'angle'))``), from the Twiss functions
    ``optics.ax, bx, dx, dpx`` at those points (ufo/radiation.py:35-83).
    Only elements with a non-zero ``angle`` contribute."""
    rows = [(float(getattr(e, 'length', 0.)), float(getattr(e, 'angle', 0.)),
             float(getattr(e, 'k1', 0.)), float(a), float(b), float(d), float(dp))
            for (_, e), a, b, d, dp in zip(optics.where, optics.ax, optics.bx, optics.dx,
                                            optics.dpx)
            if getattr(e, 'angle', 0.) != 0.]
    if not rows:
        return RadiationIntegrals(0., 0., 0., 0.)
    L, theta, k, alpha, beta, d, dp = (np.array(c, dtype=np.float64) for c in zip(*rows))
    rho, mean_d, mean_h = _dipole_terms(L, theta, k, alpha, beta, d, dp)
    I1 = float(np.sum(mean_d * L / rho))
    I2 = float(np.sum(L / rho ** 2))
    I4 = float(np.sum(mean_d * (1. / rho ** 2 + 2. * k) * L / rho))
    I5 = float(np.sum(mean_h * L / np.abs(rho ** 3)))
    return RadiationIntegrals(I1, I2, I4, I5)
