"""Tangent map and adjoint against finite differences (FP64, central)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ring():
    """The C5 configuration: C2 ring (1024 elements) with one error seed."""
    import ufo_gb300 as u
    from ufo_gb300 import workloads as W
    return W.c5_ring(u)


def _params(ring):
    from ufo_gb300 import workloads as W
    return W.c5_parameters(ring)


def test_tangent_matches_tracking_differences():
    import ufo_gb300 as u
    from ufo_gb300 import diff as D, capi, compiler as C
    ring = _ring()
    eng = D.DiffEngine(D.DiffProgram(ring, u.KICK, []))
    z = np.array([[1e-3, 1e-4, -5e-4, 2e-5]])
    out, _ = eng.forward(z, np.array([1 / 1.001]), 3, tangent=True)
    J = out[0, 4:].reshape(4, 4)
    ctx = u.context(0)
    dp = capi.DeviceProgram(ctx, C.compile_line(ring, u.KICK, where=[-1]))
    h = 1e-7
    coords = np.zeros((8, 6))
    coords[:, :4] = z
    coords[:, 5] = 0.001
    for j in range(4):
        coords[2 * j, j] += h
        coords[2 * j + 1, j] -= h
    _, _, f = capi.track(ctx, dp, coords, 3, capi.UFO_MODE_TRACK, 0, slots=0)
    Jfd = np.array([(f[2 * j, :4] - f[2 * j + 1, :4]) / (2 * h) for j in range(4)]).T
    assert np.max(np.abs(J - Jfd)) < 1e-6 * np.max(np.abs(J))
    # the state itself agrees with the strict tracking kernel to rounding
    _, _, f0 = capi.track(ctx, dp, np.concatenate([z[0], [0, 0.001]])[None], 3,
                          capi.UFO_MODE_TRACK, 0, slots=0)
    assert np.max(np.abs(out[0, :4] - f0[0, :4])) < 1e-15


def _optics_grads(ring, params, vals, which):
    import torch
    import ufo_gb300 as u
    from ufo_gb300 import diff as D
    model = D.OpticsModel(ring, u.KICK, params, h_dp=1e-5)
    k = torch.tensor(vals, dtype=torch.float64, requires_grad=True)
    out = D.optics(k, model)
    assert np.all(np.isfinite(out.detach().numpy()))
    out[which].backward()
    return model, k.grad.numpy()


@pytest.mark.parametrize('which,h_rel,tol', [(0, 1e-7, 1e-6), (1, 1e-7, 1e-6), (4, 1e-7, 1e-6),
                                             (5, 1e-7, 1e-6), (6, 1e-4, 1e-4), (7, 1e-4, 1e-4)])
def test_optics_gradients_match_central_differences(which, h_rel, tol):
    """Adjoint gradients of x_co, px_co, Qx, Qy (FD step 1e-7 relative) and of
    the chromaticities (themselves differences in dp: step 1e-4 relative, the
    FD noise floor of a difference of differences) vs central differences.

    The bound is tol x |FD| plus the FD rounding floor eps/(2h): the outputs
    carry ~1e-14 absolute rounding (the one-turn matrix through 1024 elements
    and the Newton closed orbit), the chromaticities that divided by 2 h_dp."""
    ring = _ring()
    params, vals = _params(ring)
    model, g = _optics_grads(ring, params, vals, which)
    rng = np.random.default_rng(which)
    scale = np.max(np.abs(g))
    idx = rng.choice(len(vals), 16, replace=False)
    h = h_rel * np.abs(vals[idx])
    rows = np.repeat(vals[None], 2 * len(idx), axis=0)
    rows[0::2][np.arange(len(idx)), idx] += h
    rows[1::2][np.arange(len(idx)), idx] -= h
    f = model.evaluate_many(rows)
    fd = (f[0::2, which] - f[1::2, which]) / (2 * h)
    eps = 1e-14 if which < 6 else 1e-14 / (2 * model.h)
    for i, gi, fdi, hi in zip(idx, g[idx], fd, h):
        assert abs(gi - fdi) <= tol * max(abs(fdi), 1e-6 * scale) + eps / (2 * hi), (i, gi, fdi)


def _stencil4(model, vals, hrel, idx=None):
    """Jacobian columns by the 4-point stencil (f(k-2h) - 8 f(k-h) + 8 f(k+h)
    - f(k+2h)) / 12h at relative step ``hrel`` (truncation ~h^4, rounding noise
    ~eps/h): [8, len(idx)]."""
    idx = np.arange(len(vals)) if idx is None else np.asarray(idx)
    m = len(idx)
    h = hrel * np.abs(vals[idx])
    rows = np.repeat(vals[None], 4 * m, axis=0)
    for q, cst in enumerate((2.0, 1.0, -1.0, -2.0)):
        rows[q::4][np.arange(m), idx] += cst * h
    f = model.evaluate_many(rows)
    return ((-f[0::4] + 8 * f[1::4] - 8 * f[2::4] + f[3::4]) / (12 * h[:, None])).T


def _richardson(model, vals, hrel, idx=None):
    """Two 4-point stencils at h and 2h combined to cancel the h^4 term
    (error ~h^6); and the difference between the two stencils' estimates."""
    a = _stencil4(model, vals, hrel, idx)
    b = _stencil4(model, vals, 2 * hrel, idx)
    return (16 * a - b) / 15, a


def _normwise(J, R):
    return np.max(np.abs(J - R), axis=1) / np.max(np.abs(R), axis=1)


def test_optics_jacobian_within_1e7_of_accurate_differences():
    """The whole 8 x 512 Jacobian (closed orbit, tunes, chromaticities with
    respect to all 320 k1 and 192 k2 of the C5 ring) from one adjoint pass,
    against finite differences accurate well below 1e-7: Richardson-combined
    4-point stencils, at h = 1e-5 (relative) for orbit and tunes and h = 1e-3
    for the chromaticities.  The chromaticity is itself a central difference
    of the tunes in dp (step 1e-4, the reference's dp step in
    tests/optics3.py); its rounding noise, divided by a small k step, would
    swamp a small-step difference.  Bar: normwise relative error <= 1e-7 on
    every output row.  The differences' own error is bounded by comparing the
    Richardson estimate with the plain stencil at the smaller step."""
    import ufo_gb300 as u
    from ufo_gb300 import diff as D
    ring = _ring()
    params, vals = _params(ring)
    model = D.OpticsModel(ring, u.KICK, params, h_dp=1e-4)
    out, saved = model.evaluate(vals)
    J = model.vjp(saved, np.eye(8))
    Ro, So = _richardson(model, vals, 1e-5)
    Rx, Sx = _richardson(model, vals, 1e-3)
    R = np.concatenate([Ro[:6], Rx[6:]])
    err = _normwise(J, R)
    assert np.all(err <= 1e-7), err
    own = np.concatenate([_normwise(So, Ro)[:6], _normwise(Sx, Rx)[6:]])
    assert np.all(own <= 1e-7), own


def _thick_alba():
    import os
    import ufo_gb300 as u
    import helpers as H
    ring = u.Lattice(path=os.path.join(H.HERE, 'golden', 'madx', 'alba.mad')).RING
    flat = ring.flatten()
    params, vals = [], []
    for i, e in enumerate(flat):
        if type(e).__name__ == 'Quadrupole':
            params.append((i, 'k1'))
            vals.append(e.k1)
    return ring, params, np.array(vals)


def test_thick_alba_tune_gradients_within_1e7():
    """The reference's default model: the ALBA ring with exact thick
    quadrupoles and sector bends (no KICK; fringe-field edges whose angle
    depends on dp).  dQx/dk1, dQy/dk1 over every quadrupole, and the
    chromaticity gradients, from the adjoint against Richardson-combined
    4-point stencils: <= 1e-7 normwise."""
    from ufo_gb300 import diff as D
    ring, params, vals = _thick_alba()
    model = D.OpticsModel(ring, 0, params, h_dp=1e-4)
    out, saved = model.evaluate(vals)
    assert 0 < out[4] < 1 and 0 < out[5] < 1
    J = model.vjp(saved, np.eye(8))
    Ro, _ = _richardson(model, vals, 1e-5)
    Rx, _ = _richardson(model, vals, 1e-3)
    err = _normwise(J[4:6], Ro[4:6])
    assert np.all(err <= 1e-7), err
    errx = _normwise(J[6:8], Rx[6:8])
    assert np.all(errx <= 1e-7), errx


def test_thick_tunes_match_the_optics_driver():
    """The differentiator's thick maps give the tunes of the Optics driver
    (the reference's unit-particle method through the tracking kernels) on
    the thick ALBA ring, chromatic and achromatic."""
    import ufo_gb300 as u
    from ufo_gb300 import diff as D
    ring, params, vals = _thick_alba()
    for flags in (0, u.ACHROMATIC):
        out, _ = D.OpticsModel(ring, flags, params).evaluate(vals)
        o = u.Optics(ring, flags=u.LINEAR | flags | u.DOUBLE_PRECISION)
        o.run()
        assert abs(out[4] - o.qx) < 1e-10 and abs(out[5] - o.qy) < 1e-10, (out[4:6], o.qx, o.qy)


def test_thick_multiturn_adjoint_matches_stencil():
    """Multi-turn amplitude adjoint through thick quadrupoles and bends (C5
    ring without KICK, 256 particles x 256 turns, checkpoints every 32)
    against a 4-point stencil of the same map: <= 1e-7."""
    import torch
    import ufo_gb300 as u
    from ufo_gb300 import diff as D, workloads as W
    ring = _ring()
    params, vals = _params(ring)
    model = D.OpticsModel(ring, 0, params)
    coords = W.c2_beam(256, seed=3)
    k = torch.tensor(vals, dtype=torch.float64, requires_grad=True)
    a = D.amplitudes(k, model, coords, 256, ck=32)
    a.sum().backward()
    g = k.grad.numpy()
    idx = np.sort(np.random.default_rng(4).choice(len(vals), 8, replace=False))
    o = 1 / (1 + coords[:, 5])
    fd = []
    for hr in (1e-6, 2e-6):
        h = hr * np.abs(vals[idx])
        rows = np.repeat(vals[None], 32, axis=0)
        for q, cst in enumerate((2.0, 1.0, -1.0, -2.0)):
            rows[q::4][np.arange(8), idx] += cst * h
        eng = D.DiffEngine(D.DiffProgram(ring, 0, params, rows))
        z, _ = eng.forward(np.tile(coords[:, :4], (32, 1)), np.tile(o, 32), 256,
                           seed=np.repeat(np.arange(32, dtype=np.int32), 256))
        f = (z[:, 0] ** 2 + z[:, 2] ** 2).reshape(32, 256).sum(axis=1)
        fd.append((-f[0::4] + 8 * f[1::4] - 8 * f[2::4] + f[3::4]) / (12 * h))
    R = (16 * fd[0] - fd[1]) / 15
    err = np.max(np.abs(g[idx] - R)) / np.max(np.abs(R))
    assert err <= 1e-7, (err, g[idx], R)


def test_multiturn_1024_turns_within_1e7_of_stencil():
    """The 1,024-turn amplitude adjoint (C5 ring, 512 beam particles,
    checkpoints every 64 turns) over the regular particles (final state moves
    by less than 200x a 1e-9 m start displacement) against a 4-point stencil of
    the same map at h = 5e-7 (relative; its truncation ~h^4 and rounding
    noise ~eps/h balance there): normwise <= 1e-7 over 8 sampled strengths."""
    import ufo_gb300 as u
    from ufo_gb300 import diff as D, workloads as W
    ring = _ring()
    params, vals = _params(ring)
    model = D.OpticsModel(ring, u.KICK, params)
    Np, T = 512, 1024
    coords = W.c2_beam(Np, seed=3)
    o = 1.0 / (coords[:, 5] + 1.0)
    eng = model.engine(vals)
    pair = np.concatenate([coords[:, :4], coords[:, :4] + [1e-9, 0, 0, 0]])
    zp, _ = eng.forward(pair, np.concatenate([o, o]), T)
    growth = np.max(np.abs(zp[Np:, :4] - zp[:Np, :4]), axis=1) / 1e-9
    reg = growth < 200
    assert reg.sum() >= 0.95 * Np
    zT, st = eng.forward(coords[:, :4], o, T, ck=64)
    zbar = np.zeros((Np, 4))
    zbar[:, 0] = 2 * zT[:, 0] * reg
    zbar[:, 2] = 2 * zT[:, 2] * reg
    _, gp = eng.reverse(st, zbar)
    g = gp.sum(axis=0)
    idx = np.sort(np.random.default_rng(1).choice(len(vals), 8, replace=False))
    h = 5e-7 * np.abs(vals[idx])
    rows = np.repeat(vals[None], 32, axis=0)
    for q, cst in enumerate((2.0, 1.0, -1.0, -2.0)):
        rows[q::4][np.arange(8), idx] += cst * h
    e4 = D.DiffEngine(D.DiffProgram(ring, u.KICK, params, rows))
    z4, _ = e4.forward(np.tile(coords[:, :4], (32, 1)), np.tile(o, 32), T,
                       seed=np.repeat(np.arange(32, dtype=np.int32), Np))
    f = ((z4[:, 0] ** 2 + z4[:, 2] ** 2).reshape(32, Np) * reg[None]).sum(axis=1)
    fd = (-f[0::4] + 8 * f[1::4] - 8 * f[2::4] + f[3::4]) / (12 * h)
    err = np.max(np.abs(g[idx] - fd)) / np.max(np.abs(fd))
    assert err <= 1e-7, (err, g[idx], fd)


def test_multiturn_amplitude_adjoint_matches_differences():
    import torch
    import ufo_gb300 as u
    from ufo_gb300 import diff as D, workloads as W
    ring = _ring()
    params, vals = _params(ring)
    model = D.OpticsModel(ring, u.KICK, params)
    coords = W.c2_beam(64, seed=3)
    k = torch.tensor(vals, dtype=torch.float64, requires_grad=True)
    a = D.amplitudes(k, model, coords, 96, ck=16)
    a.sum().backward()
    g = k.grad.numpy()
    eng0 = model.engine(vals)
    rng = np.random.default_rng(1)
    for i in rng.choice(len(vals), 6, replace=False):
        h = 1e-6 * abs(vals[i])
        s = []
        for sgn in (1, -1):
            v = vals.copy()
            v[i] += sgn * h
            zT, _ = model.engine(v).forward(coords[:, :4], 1 / (1 + coords[:, 5]), 96)
            s.append(np.sum(zT[:, 0] ** 2 + zT[:, 2] ** 2))
        fd = (s[0] - s[1]) / (2 * h)
        assert np.isfinite(fd)
        assert abs(g[i] - fd) <= 1e-5 * max(abs(fd), 1e-3 * np.max(np.abs(g))), (i, g[i], fd)
    del eng0


def test_seed_rows_match_single_row_programs():
    """A multi-seed constant table gives, row by row, bit-identical results to
    one single-row program per seed (tracking, tangents and cotangents)."""
    import ufo_gb300 as u
    from ufo_gb300 import diff as D
    ring = _ring()
    params, vals = _params(ring)
    rng = np.random.default_rng(7)
    rows = vals[None] * (1 + 1e-3 * rng.standard_normal((3, len(vals))))
    multi = D.DiffEngine(D.DiffProgram(ring, u.KICK, params, rows))
    z = np.tile([[1e-4, 0.0, -1e-4, 0.0]], (6, 1))
    o = np.full(6, 1 / 1.0005)
    seed = np.array([0, 1, 2, 2, 1, 0], np.int32)
    out, st = multi.forward(z, o, 4, tangent=True, ck=2, seed=seed)
    zbar = rng.standard_normal((6, 4))
    Tbar = rng.standard_normal((6, 16))
    zb0, pb = multi.reverse(st, zbar, Tbar)
    for j, s in enumerate(seed):
        one = D.DiffEngine(D.DiffProgram(ring, u.KICK, params, rows[s]))
        o1, st1 = one.forward(z[j:j + 1], o[j:j + 1], 4, tangent=True, ck=2)
        zb1, pb1 = one.reverse(st1, zbar[j:j + 1], Tbar[j:j + 1])
        assert np.array_equal(out[j], o1[0])
        assert np.array_equal(zb0[j], zb1[0])
        assert np.array_equal(pb[j], pb1[0])


def test_batched_optics_match_single_evaluations():
    import ufo_gb300 as u
    from ufo_gb300 import diff as D
    ring = _ring()
    params, vals = _params(ring)
    model = D.OpticsModel(ring, u.KICK, params)
    rows = np.stack([vals, vals * (1 + 1e-6), vals * (1 - 1e-6)])
    many = model.evaluate_many(rows)
    for s in range(3):
        one, _ = model.evaluate(rows[s])
        assert np.array_equal(many[s], one)


def test_vjp_rows_match_single_vjps():
    """[S, R, 8] cotangent blocks (several seeds, several cotangents each) give
    the same parameter cotangents as one vjp per (seed, cotangent)."""
    import ufo_gb300 as u
    from ufo_gb300 import diff as D
    ring = _ring()
    params, vals = _params(ring)
    model = D.OpticsModel(ring, u.KICK, params)
    rng = np.random.default_rng(11)
    rows = vals[None] * (1 + 1e-3 * rng.standard_normal((2, len(vals))))
    G = rng.standard_normal((2, 3, 8))
    out, saved = model.evaluate_batch(rows)
    K = model.vjp(saved, G)
    assert K.shape == (2, 3, len(vals))
    for s in range(2):
        o1, sv1 = model.evaluate(rows[s])
        assert np.array_equal(o1, out[s])
        for r in range(3):
            k1 = model.vjp(sv1, G[s, r])
            np.testing.assert_allclose(K[s, r], k1, rtol=1e-13, atol=1e-13 * np.abs(k1).max())


def _linear_ring():
    """The C2 ring without its apertures (the reference's optics method tracks
    unit particles at 1 m amplitude)."""
    import ufo_gb300 as u
    from ufo_gb300 import workloads as W
    ring = W.c2_ring(u)
    return u.Line('RING', [e for e in ring.flatten() if type(e).__name__ != 'Aperture'])


def test_tunes_and_gradients_vs_reference_optics_method():
    """Against the reference's own machinery: the Optics driver (unit-particle
    linear-map columns, ufo/optics.py:96-103, bit-exact with the reference's
    kernel) in LINEAR mode with a DOUBLE_PRECISION parameter pool (without it
    the pool, like the reference's, is float32).  The origin is the closed
    orbit of this error-free ring, so the unit-particle columns are the map:
    tunes agree to rounding; adjoint dQ/dk1 agrees with central differences of
    the Optics tunes; the chromaticity agrees with the reference's one-sided dp
    difference (tests/optics3.py, delta 1e-4) to that method's own truncation
    and affine-offset error."""
    import torch
    import ufo_gb300 as u
    from ufo_gb300 import diff as D
    ring = _linear_ring()
    flat = ring.flatten()
    quads = [i for i, e in enumerate(flat) if type(e).__name__ == 'Quadrupole']
    params = [(i, 'k1') for i in quads]
    vals = np.array([flat[i].k1 for i in quads])
    flags = u.KICK | u.LINEAR | u.DOUBLE_PRECISION
    model = D.OpticsModel(ring, flags, params)
    k = torch.tensor(vals, dtype=torch.float64, requires_grad=True)
    out = D.optics(k, model)
    out[4].backward()
    g = k.grad.numpy()
    o = u.Optics(ring, where=[], parameters=params + ['dp'], flags=flags)

    def tunes(v, dp=0.0):
        o.parameters[0, :len(v)] = v
        o.parameters[0, -1] = dp
        o.run()
        return o.qx, o.qy

    qx, qy = tunes(vals)
    assert np.max(np.abs(out[:4].detach().numpy())) < 1e-15
    assert abs(out[4].item() - qx) < 1e-12 and abs(out[5].item() - qy) < 1e-12
    rng = np.random.default_rng(5)
    scale = np.abs(g).max()
    for i in rng.choice(len(vals), 8, replace=False):
        h = 1e-7 * abs(vals[i])
        vp, vm = vals.copy(), vals.copy()
        vp[i] += h
        vm[i] -= h
        fd = (tunes(vp)[0] - tunes(vm)[0]) / (2 * h)
        assert abs(g[i] - fd) <= 1e-6 * max(abs(fd), 1e-6 * scale) + 1e-14 / (2 * h), (i, g[i], fd)
    d = 1e-4
    q1 = tunes(vals, d)
    xi_ref = [(q1[0] - qx) / d, (q1[1] - qy) / d]
    xi = out[6:8].detach().numpy()
    assert np.all(np.abs(xi - xi_ref) <= 1e-2 * np.abs(xi)), (xi, xi_ref)


def test_segment_grouping_is_bit_identical():
    """The plain reverse pass re-tracks G checkpoint segments at once; the
    group size (set by the tape budget) must not change any result bit."""
    import ufo_gb300 as u
    from ufo_gb300 import diff as D, workloads as W
    ring = _ring()
    params, vals = _params(ring)
    coords = W.c2_beam(64, seed=3)
    o = 1 / (1 + coords[:, 5])
    out = []
    for budget in (1, 2 * 16 * 2560 * 4 * 64 * 8, 64 << 30):
        eng = D.DiffEngine(D.DiffProgram(ring, u.KICK, params, vals), tape_budget=budget)
        zT, st = eng.forward(coords[:, :4], o, 90, ck=16)
        zbar = np.zeros((64, 4))
        zbar[:, 0] = 2 * zT[:, 0]
        zbar[:, 2] = 2 * zT[:, 2]
        out.append(eng.reverse(st, zbar) + (eng.last_tape_segments,))
    assert [r[2] for r in out] == [1, 2, 6]
    for zb, pb, _ in out[1:]:
        assert np.array_equal(zb, out[0][0]) and np.array_equal(pb, out[0][1])


def test_pair_lane_forward_is_bit_identical_to_one_lane():
    """Plain mode runs each job on two lanes (x and y planes) with the same
    IEEE operations in the same order as the one-lane tangent-mode code: the
    states must agree bit for bit (checkpointed, 37 jobs so warps are ragged)."""
    import ufo_gb300 as u
    from ufo_gb300 import diff as D, workloads as W
    ring = _ring()
    params, vals = _params(ring)
    rows = vals[None] * (1 + 1e-3 * np.random.default_rng(2).standard_normal((2, len(vals))))
    eng = D.DiffEngine(D.DiffProgram(ring, u.KICK, params, rows))
    c = W.c2_beam(37, seed=8)
    o = 1 / (1 + c[:, 5])
    seed = (np.arange(37) % 2).astype(np.int32)
    plain, _ = eng.forward(c[:, :4], o, 7, ck=3, seed=seed)
    tang, _ = eng.forward(c[:, :4], o, 7, tangent=True, ck=3, seed=seed)
    assert np.array_equal(plain[:, :4], tang[:, :4])
