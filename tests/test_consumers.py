"""Host consumers of the optics output: radiation integrals
(ufo_gb300/radiation.py, the reference's ufo/radiation.py) and the analytic
chromaticity (ufo_gb300.drivers.chromaticity, the reference's ufo/chroma.py).

CPU: applied to the reference's own Optics arrays (golden fixtures) they must
give the reference's own results; the closed forms and the small-k quadrature
must agree with an independent Simpson integration of the propagated
dispersion and H function.  GPU: the whole chain (this library's Optics, then
the consumers) against the reference's chain."""
import types

import numpy as np
import pytest

import helpers as H

RAD = ('I1', 'I2', 'I4', 'I5', 'Jx', 'Jt', 'U0', 'Ex')
CASES = ['alba_radiation_fp32', 'alba_radiation_fp64', 'alba_chroma_fp32', 'alba_chroma_fp64']


def _reference_optics(name):
    """A stand-in Optics object holding the reference's Twiss arrays."""
    c = H.case(name)
    flat = H.line_of(c).flatten()
    where = list(c['where'])
    if c['periodic'] and -1 not in where:
        where.append(-1)
    o = types.SimpleNamespace(where=[(i, flat[int(i)]) for i in where])
    for k in ('ax', 'ay', 'bx', 'by', 'dx', 'dpx'):
        setattr(o, k, H.arr(name, f'out/{k}'))
    return o


@pytest.mark.parametrize('name', CASES)
def test_consumers_match_reference_on_its_optics(name):
    import ufo_gb300 as u
    from ufo_gb300 import drivers
    o = _reference_optics(name)
    r = u.emittance(o)
    for k in RAD:
        ref = float(H.arr(name, f'out/rad_{k}'))
        assert abs(getattr(r, k) - ref) <= 1e-14 * abs(ref), (k, getattr(r, k), ref)
    ch = np.array(drivers.chromaticity(o)).ravel()
    assert np.allclose(ch, H.arr(name, 'out/chroma'), rtol=1e-14, atol=0)


@pytest.mark.parametrize('name', ['alba_optics_where', 'alba_chroma_fp64', 'alba_radiation_fp64',
                                  'alba_optics_propagate'])
def test_twiss_from_reference_unit_tracks(name):
    """The host Twiss (ufo_gb300/twiss.py) applied to the reference's own
    unit-particle tracks gives the reference's Twiss functions, tunes and
    dispersion.  Tolerance: 1e-15 of each array's scale (a few ulps); the
    propagated alphas of the non-periodic case start from alpha0 ~ 1e-14, so
    they are compared in absolute terms (1e-15)."""
    from ufo_gb300 import drivers
    c = H.case(name)
    tr = H.arr(name, 'out/track')
    n = tr.shape[1]
    o = types.SimpleNamespace(track=tr, periodic=c.get('periodic', True))
    for k in ('ax', 'ay', 'bx', 'by', 'dx', 'dy', 'dpx', 'dpy', 'mux', 'muy'):
        setattr(o, k, np.empty(n))
    o.ax0 = o.bx0 = o.dx0 = o.dpx0 = o.ay0 = o.by0 = o.dy0 = o.dpy0 = 0.
    for k, v in c.get('attrs', {}).items():
        setattr(o, k, v)
    drivers.twiss(o)
    keys = ['bx', 'by', 'ax', 'ay', 'dx', 'dpx', 'mux', 'muy'] + (['qx', 'qy'] if o.periodic
                                                                 else [])
    for k in keys:
        ref = np.asarray(H.arr(name, f'out/{k}'), dtype=np.float64)
        got = np.asarray(getattr(o, k), dtype=np.float64)
        scale = np.max(np.abs(ref))
        tol = 1e-15 if (k in ('ax', 'ay') and not o.periodic) else 1e-15 * scale + 1e-300
        assert np.max(np.abs(got - ref)) <= max(tol, 4e-16 * scale), (k, got, ref)


def test_reference_consumers_against_madx():
    """What the reference's own tests pin (tests/radiation.py:5-12,
    tests/chroma.py:8-9): I2 is geometry and matches MAD-X; I5 lies within
    those tests' 1e-2 tolerance.  I1, I4 and the chromaticities of the
    reference differ from MAD-X beyond it (dipole edges are ignored, as the
    reference's docstring warns); parity here is with the reference's code."""
    madx = H.golden()[0]['madx']
    for tag in ('fp32', 'fp64'):
        name = f'alba_radiation_{tag}'
        assert abs(float(H.arr(name, 'out/rad_I2')) - madx['alba_I2']) < 1e-9
        assert abs(float(H.arr(name, 'out/rad_I5')) - madx['alba_I5']) < 1e-2
        assert 0.0 < float(H.arr(name, 'out/rad_Jx')) < 2.0


def _simpson_reference(L, theta, k, a0, b0, d0, dp0, n=20001):
    """I1, I4, I5 of one dipole by Simpson integration of D(s) and H(s)
    propagated through the horizontal map of focusing k."""
    rho = L / theta
    g0 = (1 + a0 * a0) / b0
    s = np.linspace(0, L, n)
    if k > 0:
        w = np.sqrt(k)
        C, S = np.cos(w * s), np.sin(w * s)
        m11, m12, m21 = C, S / w, -w * S
        D = C * d0 + S / w * dp0 + (1 - C) / (rho * k)
        Dp = -w * S * d0 + C * dp0 + S / (rho * w)
    elif k < 0:
        w = np.sqrt(-k)
        C, S = np.cosh(w * s), np.sinh(w * s)
        m11, m12, m21 = C, S / w, w * S
        D = C * d0 + S / w * dp0 + (1 - C) / (rho * k)
        Dp = w * S * d0 + C * dp0 + S / (rho * w)
    else:
        m11, m12, m21 = np.ones_like(s), s, 0 * s
        D = d0 + dp0 * s + s * s / (2 * rho)
        Dp = dp0 + s / rho
    m22 = m11
    b = m11 ** 2 * b0 - 2 * m11 * m12 * a0 + m12 ** 2 * g0
    a = -m11 * m21 * b0 + (m11 * m22 + m12 * m21) * a0 - m12 * m22 * g0
    g = m21 ** 2 * b0 - 2 * m21 * m22 * a0 + m22 ** 2 * g0
    Hs = g * D * D + 2 * a * D * Dp + b * Dp * Dp
    h = L / (n - 1)
    wts = np.ones(n)
    wts[1:-1:2], wts[2:-1:2] = 4, 2
    mean = lambda f: h / 3 * np.dot(wts, f) / L  # noqa: E731
    return mean(D) * L / rho, mean(D) * (1 / rho ** 2 + 2 * k) * L / rho, mean(Hs) * L / abs(rho ** 3)


@pytest.mark.parametrize('k', [0.0, 0.5, -0.5668989841, 1e-6, -1e-6, 2e-5])
def test_dipole_averages_against_quadrature(k):
    """Closed forms (|L sqrt k| >= 1e-2) and the small-k Gauss-Legendre
    branch (including the pure sector dipole, where the reference's closed
    forms are 0/0) against Simpson integration."""
    import ufo_gb300 as u
    el = u.Sbend('B', length=1.37, angle=0.19635, k1=k)
    o = types.SimpleNamespace(where=[(0, el)], ax=[0.7], bx=[3.1], dx=[0.12], dpx=[-0.05])
    r = u.emittance(o)
    ref = _simpson_reference(1.37, 0.19635, k, 0.7, 3.1, 0.12, -0.05)
    for got, want in zip((r.I1, r.I4, r.I5), ref):
        assert np.isfinite(got) and abs(got - want) <= 1e-11 * abs(want), (got, want)


def test_beam_and_constants():
    import ufo_gb300 as u
    b = u.Beam()
    assert b.energy == 3e9 and b.particle_mass == u.electron_mass
    assert b.gamma == (1. + 3e9) / u.electron_mass
    r = u.RadiationIntegrals(0.2, 0.9, -0.3, 4e-4)
    assert r.Jx == 1. + 0.3 / 0.9 and r.Jt == 1. - 0.3 / 0.9
    assert r.U0 == u.radiation_loss_constant * 3.0 ** 4 * 0.9
    assert r.energy_loss(u.Beam(energy=6e9)) == u.radiation_loss_constant * 6.0 ** 4 * 0.9


@pytest.mark.gpu
@pytest.mark.parametrize('name', CASES)
def test_gpu_optics_consumers_vs_reference(name):
    """This library's Optics on the GPU, then the consumers, against the
    reference's chain.  FP64 optics agree to 1e-10 with the reference's, so the
    integrals to 1e-9; with the reference's FP32 default its Twiss carry FP32
    rounding (ours are FP64 rounded to FP32 on output)."""
    import ufo_gb300 as u
    c = H.case(name)
    o = u.Optics(H.line_of(c), where=c['where'], flags=c['flags'])
    o.run()
    tol = 1e-9 if c['flags'] & u.DOUBLE_PRECISION else 5e-5
    r = u.emittance(o)
    for k in RAD:
        ref = float(H.arr(name, f'out/rad_{k}'))
        assert abs(getattr(r, k) - ref) <= tol * abs(ref), (k, getattr(r, k), ref)
    ch = np.array(u.chromaticity(o)).ravel()
    ref = H.arr(name, 'out/chroma')
    assert np.all(np.abs(ch - ref) <= tol * np.abs(ref)), (ch, ref)
