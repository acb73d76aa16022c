"""The differentiator's opcode list (ufo_gb300/diff.py) against the oracle, on
the CPU: a small numpy interpreter of the lowered program (the forward map of
csrc/diff.cu, one particle per row) must reproduce the oracle's one-turn map."""
import numpy as np
import pytest


def interpret(dprog, z, o, turns=1, seed=0):
    """Forward map of a DiffProgram: z [n, 4], o [n] (1/(1+dp))."""
    from ufo_gb300 import diff as D
    z = np.array(z, np.float64)
    x, px, y, py = z.T.copy()
    T = dprog.tab[seed]
    for _ in range(turns):
        for kind, _fl, off, N, M, _ps, _pm, achro in dprog.ops:
            c = T[off:]
            oo = 1.0 if achro else o
            if kind == D.D_DRIFT:
                x, y = x + px * c[0], y + py * c[0]
            elif kind == D.D_ALIGN:
                x, y = x - c[0], y - c[1]
            elif kind == D.D_EDGE:
                curv = c[0] * oo
                t2 = np.tan(c[2] - 2 * curv * c[3] / c[4] * c[5]) if _fl & D.DE_RTPSI else c[2]
                px, py = px + x * curv * c[1], py - y * curv * t2
            elif kind == D.D_THICK:
                L, k1, h = c[0], c[1], c[2]
                bend = _fl & D.DT_BEND
                Kx = oo * (k1 + h * h)
                Ky = -oo * k1
                Cx, Sx, D1x, _, _, _ = D.thick_functions(Kx, L)
                Cy, Sy, _, _, _, _ = D.thick_functions(Ky, L)
                disp = (1 / o - 1) * h * oo if bend else 0.0
                x, px = Cx * x + Sx * px + disp * D1x, -Kx * Sx * x + Cx * px + disp * Sx
                y, py = Cy * y + Sy * py, -Ky * Sy * y + Cy * py
            elif kind in (D.D_TEAPOT, D.D_KICK):
                tp = kind == D.D_TEAPOT
                n = N if tp else 1
                Lo, Li, W, Lx = c[0], c[1], c[2], c[5]
                a, b = c[D.KHDR:D.KHDR + M], c[D.KHDR + M:D.KHDR + 2 * M]
                if tp:
                    x, y = x + px * Lo, y + py * Lo
                for sl in range(n):
                    zz = x + 1j * y
                    S = np.zeros_like(zz) + (a[M - 1] + 1j * b[M - 1])
                    for k in range(M - 2, -1, -1):
                        S = S * zz + (a[k] + 1j * b[k])
                    px, py = px - oo * S.real, py + oo * S.imag
                    if tp:
                        px = px - W * x
                        L = Li if sl < n - 1 else Lx
                        x, y = x + px * L, y + py * L
    return np.stack([x, px, y, py], axis=1)


def _linear_ring():
    import ufo_gb300 as u
    from ufo_gb300 import workloads as W
    ring = W.c2_ring(u)
    return u.Line('RING', [e for e in ring.flatten() if type(e).__name__ != 'Aperture'])


def _c5():
    import ufo_gb300 as u
    from ufo_gb300 import workloads as W
    return W.c5_ring(u)


@pytest.mark.parametrize('which', ['c5_kick', 'c2_linear', 'c5_thick', 'alba_thick',
                                   'alba_thick_achromatic'])
def test_lowered_program_matches_oracle(which):
    import ufo_gb300 as u
    from ufo_gb300 import diff as D
    from oracle import oracle as O
    if which == 'c5_kick':
        ring, flags = _c5(), u.KICK
        coords = np.array([[1e-3, 1e-4, -5e-4, 2e-5, 0, 1e-3],
                           [-2e-4, 3e-5, 1e-4, -1e-5, 0, -2e-3],
                           [0, 0, 0, 0, 0, 0]])
    elif which == 'c2_linear':
        ring, flags = _linear_ring(), u.KICK | u.LINEAR
        coords = np.array([[1.0, 0, 1.0, 0, 0, 0], [0, 1.0, 0, 1.0, 0, 0],
                           [1e-3, 0, 0, 0, 0, 1e-4], [0, 0, 0, 0, 0, 0]])
    else:  # exact thick quadrupoles and sector bends (the reference's default)
        import os
        if which == 'c5_thick':
            ring, flags = _c5(), 0
        else:
            import helpers as H
            ring = u.Lattice(path=os.path.join(H.HERE, 'golden', 'madx', 'alba.mad')).RING
            flags = u.ACHROMATIC if which == 'alba_thick_achromatic' else 0
        coords = np.array([[1e-3, 1e-4, -5e-4, 2e-5, 0, 1e-3],
                           [-2e-4, 3e-5, 1e-4, -1e-5, 0, -2e-3],
                           [0, 0, 0, 0, 0, 0]])
    dp = D.DiffProgram(ring, flags, [])
    got = interpret(dp, coords[:, :4], 1 / (1 + coords[:, 5]))
    ref = O.track(ring, flags | u.DOUBLE_PRECISION, coords, 1, tracks=False)['final'][:, :4]
    scale = np.maximum(np.abs(ref).max(axis=0), 1e-300)
    assert np.all(np.abs(got - ref) <= 1e-12 * scale + 1e-18), (got - ref)


def test_thick_functions_and_their_derivatives():
    """thick_functions: the closed forms against the series across the switch
    at |K L^2| = 1, both signs of K, and the K-derivatives against central
    differences."""
    from ufo_gb300 import diff as D
    L = 0.7
    K = np.array([-30.0, -2.05, -2.0408, -0.5, -1e-9, 1e-9, 0.3, 2.0408, 2.05, 40.0])
    C, Sw, D1, dC, dSw, dD1 = D.thick_functions(K, L)
    w = np.sqrt(np.abs(K).astype(np.longdouble))
    Cr = np.where(K > 0, np.cos(w * L), np.cosh(w * L))
    Sr = np.where(K > 0, np.sin(w * L), np.sinh(w * L)) / w
    np.testing.assert_allclose(C, Cr.astype(float), rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(Sw, Sr.astype(float), rtol=1e-14)
    big = np.abs(K) > 1e-3
    np.testing.assert_allclose(D1[big], ((1 - Cr) / K)[big].astype(float), rtol=1e-12)
    for f, df in ((0, dC), (1, dSw), (2, dD1)):
        h = 1e-5 * np.maximum(np.abs(K), 1.0)
        fp = D.thick_functions(K + h, L)[f]
        fm = D.thick_functions(K - h, L)[f]
        fp2 = D.thick_functions(K + 2 * h, L)[f]
        fm2 = D.thick_functions(K - 2 * h, L)[f]
        fd = (-fp2 + 8 * fp - 8 * fm + fm2) / (12 * h)
        np.testing.assert_allclose(df, fd, rtol=1e-8, atol=1e-12)
