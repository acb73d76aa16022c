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
                px, py = px + x * curv * c[1], py - y * curv * c[2]
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


@pytest.mark.parametrize('which', ['c5_kick', 'c2_linear'])
def test_lowered_program_matches_oracle(which):
    import ufo_gb300 as u
    from ufo_gb300 import diff as D
    from oracle import oracle as O
    if which == 'c5_kick':
        ring, flags = _c5(), u.KICK
        coords = np.array([[1e-3, 1e-4, -5e-4, 2e-5, 0, 1e-3],
                           [-2e-4, 3e-5, 1e-4, -1e-5, 0, -2e-3],
                           [0, 0, 0, 0, 0, 0]])
    else:
        ring, flags = _linear_ring(), u.KICK | u.LINEAR
        coords = np.array([[1.0, 0, 1.0, 0, 0, 0], [0, 1.0, 0, 1.0, 0, 0],
                           [1e-3, 0, 0, 0, 0, 1e-4], [0, 0, 0, 0, 0, 0]])
    dp = D.DiffProgram(ring, flags, [])
    got = interpret(dp, coords[:, :4], 1 / (1 + coords[:, 5]))
    ref = O.track(ring, flags | u.DOUBLE_PRECISION, coords, 1, tracks=False)['final'][:, :4]
    scale = np.maximum(np.abs(ref).max(axis=0), 1e-300)
    assert np.all(np.abs(got - ref) <= 1e-12 * scale + 1e-18), (got - ref)
