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
