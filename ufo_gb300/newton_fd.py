"""Closed orbit by Newton iteration with a finite-difference Jacobian.

F(z) = z is solved for z = (x, px, y, py) at dp = 0 (the reference's
ClosedOrbit forces dp = 0, oodppo = 1, z = 0: ufo/co.py:182-184).  Each Newton
step evaluates F at the iterate and at 8 central-difference points for every
orbit in ONE batched launch of the tracking kernel (the reference's
per-particle-parameter batching idiom), then solves (J - I) dz = z - F(z) on
the host.  The fixed point itself is exact FP64 tracking; the Jacobian only
steers the iteration.  (The differentiator, ufo_gb300/diff.py, has a Newton
iteration on the exact tangent map instead: OpticsModel.)
"""
import numpy as np

from . import capi


def closed_orbit(ctx, dprog, guess, seed=None, fma=False, max_iter=50, h=1e-7, tol=0.0):
    guess = np.asarray(guess, dtype=np.float64)
    n = guess.shape[0]
    z = guess.copy()
    flags = capi.UFO_TRACK_FMA if fma else 0
    best = np.full(n, np.inf)
    best_z = z.copy()
    seed9 = None if seed is None else np.repeat(np.asarray(seed, np.int32), 9)
    for _ in range(max(1, int(max_iter))):
        coords = np.zeros((n, 9, 6))
        coords[:, :, :4] = z[:, None, :]
        for j in range(4):
            coords[:, 1 + 2 * j, j] += h
            coords[:, 2 + 2 * j, j] -= h
        _, _, final = capi.track(ctx, dprog, coords.reshape(-1, 6), 1, capi.UFO_MODE_TRACK,
                                 flags, seed=seed9, slots=0)
        f = final.reshape(n, 9, 6)[:, :, :4]
        res = f[:, 0] - z
        nrm = np.max(np.abs(res), axis=1)
        improved = nrm < best
        best = np.where(improved, nrm, best)
        best_z[improved] = z[improved]
        if np.all(nrm <= tol) or not np.any(improved):
            break
        J = np.empty((n, 4, 4))
        for j in range(4):
            J[:, :, j] = (f[:, 1 + 2 * j] - f[:, 2 + 2 * j]) / (2 * h)
        A = J - np.eye(4)[None]
        try:
            dz = np.linalg.solve(A, -res[:, :, None])[:, :, 0]
        except np.linalg.LinAlgError:
            break
        z = z + np.where(np.isfinite(dz), dz, 0.0)
    return best_z, best
