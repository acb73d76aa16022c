"""The build's 4th-order Yoshida integrator (no reference counterpart).

CPU: compiled table layout, rejected combinations, and the order of the numpy
restatement (oracle/yoshida.py).  GPU: the library against that restatement
(strict and FMA modes, with errors and misalignments) and its convergence order
measured on the device."""
import numpy as np
import pytest


def _c1(slices=4):
    import ufo_gb300 as u
    from ufo_gb300 import workloads as W
    return W.c1_ring(u, slices=slices)


def _beam(n, seed=7):
    rng = np.random.default_rng(seed)
    c = np.zeros((n, 6))
    c[:, 0] = rng.normal(0, 1e-3, n)
    c[:, 1] = rng.normal(0, 1e-4, n)
    c[:, 2] = rng.normal(0, 1e-3, n)
    c[:, 3] = rng.normal(0, 1e-4, n)
    c[:, 5] = rng.normal(0, 1e-3, n)
    return c


def test_compiled_yoshida_table():
    import ufo_gb300 as u
    from ufo_gb300 import compiler as C
    ring = _c1()
    prog = C.compile_line(ring, u.KICK | u.YOSHIDA, [], [-1])
    flat = ring.flatten()
    seen = 0
    for r, e in zip(prog.ops, prog.op_elem):
        if int(r[0]) != C.OP_TEAPOT:
            continue
        assert int(r[1]) & C.F_YOSHIDA
        c = prog.table[0, int(r[2]):]
        h = flat[e].length / flat[e].slices
        assert abs(sum(c[:4]) - h) <= 1e-15 * h
        assert abs(sum(c[4:7]) - 1.0) <= 1e-15
        seen += 1
    assert seen > 0


def test_yoshida_rejects_exact_and_differentiation():
    import ufo_gb300 as u
    from ufo_gb300 import compiler as C, diff as D
    with pytest.raises(NotImplementedError):
        C.compile_line(_c1(), u.KICK | u.YOSHIDA | u.EXACT, [], [-1])
    with pytest.raises(NotImplementedError):
        D.DiffProgram(_c1(), u.KICK | u.YOSHIDA, [])


def _order_errors(run):
    """Errors after one turn at N = 2, 4, 8 slices against N = 64."""
    ref = run(64)
    return [np.max(np.abs(run(n) - ref)) for n in (2, 4, 8)]


def test_restatement_is_fourth_order():
    from oracle import yoshida as Y
    c = _beam(64)
    e = _order_errors(lambda n: Y.track(_c1(n), c, 1))
    assert 12 < e[0] / e[1] < 20 and 12 < e[1] / e[2] < 20, e


def _gpu_track(line, flags, coords, turns):
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C
    ctx = u.context(0)
    dp = capi.DeviceProgram(ctx, C.compile_line(line, flags, [], [-1]))
    tf = capi.UFO_TRACK_FMA if flags & u.FMA else 0
    _, _, f = capi.track(ctx, dp, coords, turns, capi.UFO_MODE_TRACK, tf, slots=0)
    return f


@pytest.mark.gpu
@pytest.mark.parametrize('ring,fma', [('c1', False), ('c1', True), ('c2', True), ('c5', False)])
def test_gpu_yoshida_matches_restatement(ring, fma):
    import ufo_gb300 as u
    from ufo_gb300 import workloads as W
    from oracle import yoshida as Y
    if ring == 'c1':
        line, c, turns = _c1(), _beam(256), 50
    elif ring == 'c2':
        line, c, turns = W.c2_ring(u), W.c2_beam(256, seed=4), 20
    else:  # misalignments, normal and skew errors: the general kick pattern
        line, c, turns = W.c5_ring(u), W.c2_beam(128, seed=5), 10
    flags = u.KICK | u.YOSHIDA | (u.FMA if fma else 0)
    got = _gpu_track(line, flags, c, turns)[:, :4]
    ref = Y.track(line, c, turns)[:, :4]
    ok = np.all(np.isfinite(ref), axis=1)
    assert ok.sum() >= 0.9 * len(c)
    scale = np.max(np.abs(ref[ok]), axis=0)
    err = np.max(np.abs(got[ok] - ref[ok]) / scale)
    assert err <= 1e-12 * turns, err
    assert np.array_equal(np.isfinite(got[:, 0]), np.isfinite(ref[:, 0]))


@pytest.mark.gpu
def test_gpu_yoshida_is_fourth_order_teapot_second():
    import ufo_gb300 as u
    c = _beam(64)
    ey = _order_errors(lambda n: _gpu_track(_c1(n), u.KICK | u.YOSHIDA, c, 1))
    et = _order_errors(lambda n: _gpu_track(_c1(n), u.KICK, c, 1))
    assert 12 < ey[0] / ey[1] < 20 and 12 < ey[1] / ey[2] < 20, ey
    # teapot is second order; N = 2 -> 4 is not yet asymptotic
    assert 3 < et[0] / et[1] < 6 and 3 < et[1] / et[2] < 5, et
