"""Twiss functions and linear chromaticity on the host, from the tracked map.

``Optics.run`` tracks three unit particles (x = y = 1; px = py = 1; dp = 1)
once around the line with observations at ``where``.  In LINEAR | ACHROMATIC
mode the map is affine, so at observation point i the three rows of
``track[:, i, :4]`` are the columns of the partial transfer matrix R_i (the
x/y column, the px/py column and the dispersion column).  The quantities the
reference derives from them (ufo/optics.py:156-238) are computed here as array
operations over all observation points and both planes at once:

* periodic solution (last observation point = one turn): for each plane's
  2x2 block M, cos(mu) = tr(M) / 2 and the Twiss matrix
  B0 = [[beta0, -alpha0], [-alpha0, gamma0]] with M = I cos(mu) + J B0 sin(mu)
  (J the symplectic unit); the tune is mu / 2pi in [0, 1); the horizontal
  dispersion is the fixed point of the affine map, (I - M) eta0 = d;
* propagation: B_i = R_i B0 R_i^T (beta = B[0, 0], alpha = -B[0, 1]), the
  phase advance mu_i = atan2(R12, beta0 R11 - alpha0 R12), and
  eta_i = R_i eta0 + d_i.

The reference reads only the horizontal periodic dispersion; the vertical one
stays at ``dy0, dpy0`` (0 unless the caller sets them), as there.  A plane
whose one-turn block is unstable (|cos mu| > 1) gets NaN for its periodic
values and hence for its propagated ones; the reference returns at that point
and leaves its arrays unset.

``chromaticity`` integrates the same Twiss functions through each quadrupole
and sextupole in closed form (the quantities of ufo/chroma.py:11-52):
    xi = -1/(4 pi) sum_quads K int beta ds + 1/(4 pi) sum_sext k2 int eta beta ds
with beta(s) = B(s)[0, 0] carried through the quadrupole's own linear map and
eta(s) = eta0 + eta0' s, beta(s) = beta0 - 2 alpha0 s + gamma0 s^2 through the
sextupole body (a drift in the linear optics).  One sign follows the reference
rather than the integral: its eta0' term uses -gamma0 L^4/4 (see below).  In a
mirror-symmetric ring the eta0' terms cancel in pairs, so the effect is small.
"""
import numpy as np

# ---------------------------------------------------------------- Twiss


def _blocks(track):
    """Partial maps from the three unit tracks: R [n, 2 planes, 2, 2] and the
    dispersion columns d [n, 2 planes, 2]."""
    t = np.asarray(track, dtype=np.float64)[..., :4]   # [3 particles, n, 4]
    cols = t.reshape(3, t.shape[1], 2, 2)              # [particle, n, plane, (q, p)]
    R = np.stack([cols[0], cols[1]], axis=-1)          # column j = particle j
    return R, cols[2]


def periodic(M):
    """Periodic Twiss of stable 2x2 one-turn blocks M [..., 2, 2]:
    (beta0, alpha0, tune); NaN where |cos mu| > 1."""
    c = 0.5 * (M[..., 0, 0] + M[..., 1, 1])
    stable = np.abs(c) <= 1.0
    with np.errstate(invalid='ignore', divide='ignore'):
        s = np.copysign(np.sqrt(np.where(stable, 1.0 - c * c, np.nan)), M[..., 0, 1])
        beta = M[..., 0, 1] / s
        alpha = 0.5 * (M[..., 0, 0] - M[..., 1, 1]) / s
        mu = np.mod(np.arctan2(s, c), 2.0 * np.pi)
    return beta, alpha, mu / (2.0 * np.pi)


def fixed_dispersion(M, d):
    """eta0 with (I - M) eta0 = d for 2x2 blocks (det M = 1)."""
    k = 2.0 - M[..., 0, 0] - M[..., 1, 1]
    return np.stack([((1.0 - M[..., 1, 1]) * d[..., 0] + M[..., 0, 1] * d[..., 1]) / k,
                     (M[..., 1, 0] * d[..., 0] + (1.0 - M[..., 0, 0]) * d[..., 1]) / k], -1)


def propagate(R, d, beta0, alpha0, eta0):
    """Twiss at every observation point from the partial maps.
    R [n, 2, 2, 2], d [n, 2, 2]; beta0, alpha0 [2]; eta0 [2, 2].
    Returns beta, alpha, mu, eta: [n, 2] ([n, 2, 2] for eta)."""
    gamma0 = (1.0 + alpha0 * alpha0) / beta0
    B0 = np.empty((2, 2, 2))
    B0[:, 0, 0], B0[:, 0, 1], B0[:, 1, 0], B0[:, 1, 1] = beta0, -alpha0, -alpha0, gamma0
    B = np.einsum('npij,pjk,npkl->npil', R, B0, np.swapaxes(R, -1, -2))
    beta, alpha = B[..., 0, 0], -B[..., 0, 1]
    r11, r12 = R[..., 0, 0], R[..., 0, 1]
    mu = np.arctan2(r12, beta0 * r11 - alpha0 * r12)
    eta = np.einsum('npij,pj->npi', R, eta0) + d
    return beta, alpha, mu, eta


def twiss(o):
    """Fill an Optics object's periodic values (``qx, qy, bx0, ...``) and its
    per-point arrays (``bx, ax, mux, dx, dpx`` and the vertical ones) from
    ``o.track``."""
    R, d = _blocks(o.track)
    if o.periodic:
        M, dM = R[-1], d[-1]
        b0, a0, q = periodic(M)
        o.bx0, o.by0 = float(b0[0]), float(b0[1])
        o.ax0, o.ay0 = float(a0[0]), float(a0[1])
        o.qx, o.qy = float(q[0]), float(q[1])
        o.dx0, o.dpx0 = (float(v) for v in fixed_dispersion(M[0], dM[0]))
    beta0 = np.array([o.bx0, o.by0], dtype=np.float64)
    alpha0 = np.array([o.ax0, o.ay0], dtype=np.float64)
    eta0 = np.array([[o.dx0, o.dpx0], [o.dy0, o.dpy0]], dtype=np.float64)
    with np.errstate(invalid='ignore', divide='ignore'):
        beta, alpha, mu, eta = propagate(R, d, beta0, alpha0, eta0)
    o.bx[:], o.by[:] = beta[:, 0], beta[:, 1]
    o.ax[:], o.ay[:] = alpha[:, 0], alpha[:, 1]
    o.mux[:], o.muy[:] = mu[:, 0], mu[:, 1]
    o.dx[:], o.dpx[:] = eta[:, 0, 0], eta[:, 0, 1]
    o.dy[:], o.dpy[:] = eta[:, 1, 0], eta[:, 1, 1]


# --------------------------------------------------------- chromaticity


def _quad_beta_integrals(L, K):
    """(int C^2, int C S, int S^2) over [0, L] of the principal trajectories
    C, S of the equation q'' = -K q, for K != 0 (arrays)."""
    w = np.sqrt(np.abs(K))
    foc = K > 0
    sin2 = np.where(foc, np.sin(2 * w * L), np.sinh(2 * w * L)) / (4 * w)
    half = np.where(foc, np.sin(w * L), np.sinh(w * L))
    cc = 0.5 * L + sin2
    cs = half * half / (2 * K) * np.where(foc, 1.0, -1.0)
    ss = (0.5 * L - sin2) / K
    return cc, cs, ss


def _drift_moments(L):
    """int_0^L s^n ds, n = 0..3."""
    return L, L * L / 2, L ** 3 / 3, L ** 4 / 4


def chromaticity(optics):
    """Natural and total linear chromaticity from Twiss at the elements'
    entrances: ``optics.where`` pairs each observation point with its element
    (attributes ``length``, ``k1``, ``k2``), ``optics.ax, ay, bx, by, dx, dpx``
    hold the Twiss there.  Returns ((xi_x0, xi_y0), (xi_x, xi_y)), the first
    pair from quadrupoles alone."""
    names = ('ax', 'ay', 'bx', 'by', 'dx', 'dpx')
    tw = {k: np.asarray(getattr(optics, k), dtype=np.float64) for k in names}
    n = min([len(optics.where)] + [len(v) for v in tw.values()])  # pairs as zip() would
    elems = [e for _, e in optics.where[:n]]
    tw = {k: v[:n] for k, v in tw.items()}
    L = np.array([float(getattr(e, 'length', 0.0)) for e in elems])
    k1 = np.array([float(getattr(e, 'k1', 0.0)) for e in elems])
    k2 = np.array([float(getattr(e, 'k2', 0.0)) for e in elems])
    beta = np.stack([tw['bx'], tw['by']])    # [plane, n]
    alpha = np.stack([tw['ax'], tw['ay']])
    with np.errstate(divide='ignore', invalid='ignore'):
        gamma = (1.0 + alpha * alpha) / beta

    xi0 = np.zeros(2)
    q = (L != 0) & (k1 != 0)
    if q.any():
        for plane, K in ((0, k1[q]), (1, -k1[q])):  # focusing strength of the plane
            cc, cs, ss = _quad_beta_integrals(L[q], K)
            ib = beta[plane, q] * cc - 2 * alpha[plane, q] * cs + gamma[plane, q] * ss
            xi0[plane] = -np.sum(K * ib)
    xi_s = np.zeros(2)
    s = (L != 0) & (k2 != 0)
    if s.any():
        m0, m1, m2, m3 = _drift_moments(L[s])
        for plane, sign in ((0, 1.0), (1, -1.0)):
            b, a, g = beta[plane, s], alpha[plane, s], gamma[plane, s]
            # the dispersion-slope moment carries -gamma0 L^4/4 where the
            # integral of s beta(s) has +gamma0 L^4/4: the reference's sign
            # (ufo/chroma.py:46-47), mirrored like its other quirks
            ieb = (tw['dx'][s] * (b * m0 - 2 * a * m1 + g * m2) +
                   tw['dpx'][s] * (b * m1 - 2 * a * m2 - g * m3))
            xi_s[plane] = sign * np.sum(k2[s] * ieb)
    xi0 /= 4 * np.pi
    xi = xi0 + xi_s / (4 * np.pi)
    return (float(xi0[0]), float(xi0[1])), (float(xi[0]), float(xi[1]))
