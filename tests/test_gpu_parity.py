"""GPU parity: the CUDA path (public API -> C ABI -> sm_103a kernels) against
the reference's golden outputs and the C oracle.

Bars: bit-identical coordinates and loss turns in the default (strict) mode
whenever the lattice needs no per-particle transcendental; otherwise, and in
FMA mode, agreement within 1e-12 relative per turn (1e-9 after 1000 turns).
"""
import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


def _prog(obj):
    return obj.program


@pytest.mark.parametrize('name', [c['name'] for c in H.cases('track')])
def test_tracks_vs_reference(name):
    c = H.case(name)
    t = H.gpu_case(c)
    ref = H.arr(name, 'out/tracks')
    assert t.tracks.shape == ref.shape
    if H.program_is_exact(_prog(t)):
        assert np.array_equal(t.tracks, ref, equal_nan=True), H.track_rel_err(t.tracks, ref)
    else:
        _assert_within_tolerance(c, t.tracks, ref)


def _assert_within_tolerance(c, got, ref):
    """Turn 1: every particle within 1e-12.  All turns: every regular
    particle within 1e-12 x turns (1e-9 after 1000 turns)."""
    k = H.first_turn_slots(c)
    assert H.track_rel_err(got[:, :k], ref[:, :k]) <= 1e-12
    reg = H.regular_mask(c, H.tolerance(c['turns']))
    assert reg.sum() >= 1, 'no regular particle to test'
    assert H.track_rel_err(got[reg], ref[reg]) <= H.tolerance(c['turns'])


@pytest.mark.parametrize('name', [c['name'] for c in H.cases('track')])
def test_tracks_fma_mode_within_tolerance(name):
    import ufo_gb300 as u
    c = H.case(name)
    t = H.gpu_case(c, extra_flags=u.FMA)
    ref = H.arr(name, 'out/tracks')
    _assert_within_tolerance(c, t.tracks, ref)


@pytest.mark.parametrize('name', [c['name'] for c in H.cases('sa')])
def test_loss_turns_vs_reference(name):
    c = H.case(name)
    s = H.gpu_case(c)
    ref = H.arr(name, 'out/lost')
    if H.program_is_exact(_prog(s)):
        assert np.array_equal(s.lost, ref)
    else:
        # per-particle transcendentals (wire) use CUDA's libm, which may differ
        # from the C library in the last bit.  A particle whose loss turn the
        # oracle keeps when its start moves by +-1e-15 (relative; several ulps,
        # more than a libm difference) must have the reference's loss turn;
        # only particles on a loss boundary that a last-bit change moves are
        # exempt
        o = H.oracle_case(c)['lost']
        stable = (H.oracle_case(c, perturb=1e-15)['lost'] == o) & \
            (H.oracle_case(c, perturb=-1e-15)['lost'] == o)
        assert stable.mean() >= 0.9, stable.mean()
        assert np.array_equal(s.lost[stable], ref[stable])


def test_fodo_matches_madx_golden():
    import ufo_gb300 as u
    meta, _ = H.golden()
    lat = H.line_of(H.case('fodo_fived'))
    tr = u.Track(lat, turns=10, particles=2, where=[-1], flags=u.FIVED, parameters=['x'])
    tr.parameters[:, 0] = 0.001
    tr.run(threads=1)
    x = np.array(meta['madx']['tracking_fodo_x'])
    assert tr.tracks.dtype == np.float32
    assert np.max(np.abs(tr.tracks[0][:, 0] - x)) < 1e-6
    assert np.max(np.abs(tr.tracks[1][:, 0] - x)) < 1e-6


def test_plain_and_persistent_kernels_identical():
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    ring = W.c3_ring(u)
    prog = C.compile_line(ring, u.KICK, where=[-1])
    ctx = u.context(0)
    dp = capi.DeviceProgram(ctx, prog)
    coords = W.c3_grid(24, 24)
    a = capi.track(ctx, dp, coords, 300, capi.UFO_MODE_SA, 0, slots=0)
    b = capi.track(ctx, dp, coords, 300, capi.UFO_MODE_SA, capi.UFO_TRACK_PLAIN, slots=0)
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[2], b[2], equal_nan=True)
    assert 0 < np.sum(a[1] < 300) < len(a[1])


def test_full_size_c2_subset_vs_oracle():
    """65,536 particles of the C2 ring on the GPU; a random subset re-tracked
    by the oracle must agree bit for bit (particles are independent, so this
    checks the full-size launch)."""
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    from oracle import oracle as O
    ring = W.c2_ring(u)
    beam = W.c2_beam(65536)
    turns = 20
    prog = C.compile_line(ring, u.KICK, where=[-1])
    ctx = u.context(0)
    dp = capi.DeviceProgram(ctx, prog)
    _, lost, final = capi.track(ctx, dp, beam, turns, capi.UFO_MODE_TRACK, 0, slots=0)
    idx = np.random.default_rng(0).choice(65536, 256, replace=False)
    ref = O.track(ring, u.KICK, beam[idx], turns, where=[-1], tracks=False)
    assert np.array_equal(final[idx], ref['final'], equal_nan=True)
    assert np.array_equal(lost[idx], ref['lost'])


def test_full_size_c2_fma_within_tolerance_of_strict():
    """The benchmark workload at full size: all 65,536 particles, FMA mode vs
    the strict (reference-identical) mode: <= 1e-12 relative after 1 turn,
    <= 1e-9 after 1000 turns, identical loss masks; strict mode itself
    checked against the oracle on a random subset after 1000 turns."""
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    from oracle import oracle as O
    ring = W.c2_ring(u)
    beam = W.c2_beam(65536)
    ctx = u.context(0)
    ps = capi.DeviceProgram(ctx, C.compile_line(ring, u.KICK, where=[-1]))
    pf = capi.DeviceProgram(ctx, C.compile_line(ring, u.KICK | u.FMA, where=[-1]))
    for turns, tol in ((1, 1e-12), (1000, 1e-9)):
        _, ls, fs = capi.track(ctx, ps, beam, turns, capi.UFO_MODE_TRACK, 0, slots=0)
        _, lf, ff = capi.track(ctx, pf, beam, turns, capi.UFO_MODE_TRACK, capi.UFO_TRACK_FMA,
                               slots=0)
        assert np.array_equal(ls, lf)
        scale = np.max(np.abs(fs[:, :4]), axis=0)
        err = np.max(np.abs(ff[:, :4] - fs[:, :4]) / scale)
        assert err <= tol, (turns, err)
    idx = np.random.default_rng(1).choice(65536, 64, replace=False)
    ref = O.track(ring, u.KICK, beam[idx], 1000, where=[-1], tracks=False)
    assert np.array_equal(fs[idx], ref['final'], equal_nan=True)


@pytest.mark.parametrize('which', ['c3', 'c5'])
def test_general_kicks_fma_within_tolerance_of_strict(which):
    """General multipole kicks (normal and skew errors of orders 3-6 on every
    magnet, misalignments): the FMA mode's single complex Horner pass against
    the strict mode (the reference's two real passes, bit-identical to it):
    <= 1e-12 relative after 1 turn and 1e-12 * turns after 1000 turns on every
    regular particle (strict re-tracking from a start perturbed by 1e-15 moves
    it by less than a tenth of the tolerance)."""
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    if which == 'c3':
        ring, beam = W.c3_ring(u), W.c1_beam(2048, seed=9)
    else:
        ring, beam = W.c5_ring(u), W.c2_beam(2048, seed=9)
    ctx = u.context(0)
    ps = capi.DeviceProgram(ctx, C.compile_line(ring, u.KICK, where=[-1]))
    pf = capi.DeviceProgram(ctx, C.compile_line(ring, u.KICK | u.FMA, where=[-1]))
    for turns in (1, 1000):
        tol = 1e-12 * turns
        _, ls, fs = capi.track(ctx, ps, beam, turns, capi.UFO_MODE_TRACK, 0, slots=0)
        _, _, fp = capi.track(ctx, ps, beam * (1 + 1e-15), turns, capi.UFO_MODE_TRACK, 0,
                              slots=0)
        _, lf, ff = capi.track(ctx, pf, beam, turns, capi.UFO_MODE_TRACK, capi.UFO_TRACK_FMA,
                               slots=0)
        scale = np.nanmax(np.abs(fs[:, :4]), axis=0)
        pert = np.max(np.abs(fp[:, :4] - fs[:, :4]) / scale, axis=1)
        reg = (pert <= tol / 10) & np.all(np.isfinite(fs[:, :4]), axis=1)
        assert reg.sum() >= 0.9 * len(beam), reg.sum()
        err = np.max(np.abs(ff[reg, :4] - fs[reg, :4]) / scale)
        assert err <= tol, (turns, err)
        assert np.array_equal(ls[reg], lf[reg])


def test_c3_full_grid_subset_loss_turns_vs_oracle():
    """The dynamic-aperture benchmark case at full size (C1 ring with apertures
    and errors, 2,048 turns, StableAperture test): strict-mode loss turns and
    final coordinates of a random subset of the 196,608 grid particles are the
    oracle's, bit for bit; the persistent and plain kernels agree on the whole
    grid."""
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    from oracle import oracle as O
    ring = W.c3_ring(u)
    grid = W.c3_grid()
    idx = np.random.default_rng(3).choice(len(grid), 256, replace=False)
    ctx = u.context(0)
    dp = capi.DeviceProgram(ctx, C.compile_line(ring, u.KICK, where=[-1]))
    _, lost, fin = capi.track(ctx, dp, grid[idx], 2048, capi.UFO_MODE_SA, 0, slots=0)
    ref = O.track(ring, u.KICK, grid[idx], 2048, where=[-1], mode=1, tracks=False)
    assert np.array_equal(lost, ref['lost'])
    assert np.array_equal(fin, ref['final'], equal_nan=True)
    assert 0 < np.sum(lost < 2048) < len(idx)  # survival is uneven
    _, lp, _ = capi.track(ctx, dp, grid, 2048, capi.UFO_MODE_SA, 0, slots=0)
    _, lq, _ = capi.track(ctx, dp, grid, 2048, capi.UFO_MODE_SA, capi.UFO_TRACK_PLAIN, slots=0)
    assert np.array_equal(lp, lq)


def test_stable_aperture_two_phase_is_identical():
    """StableAperture's two-phase compaction (the default: first turns/8 on
    the full grid, the survivors on a grid sized to them) and its in-kernel
    compaction (CTAs packing and exchanging particles) give the loss turns and
    coordinates of one plain persistent run, bit for bit, in strict and FMA
    modes."""
    import ufo_gb300 as u
    from ufo_gb300 import workloads as W
    ring = W.c3_ring(u)
    grid = W.c3_grid(48, 48)
    for flags in (u.KICK | u.DOUBLE_PRECISION, u.KICK | u.FMA | u.DOUBLE_PRECISION):
        out = []
        for compact in (False, 'two-phase', True):
            sa = u.StableAperture(ring, flags=flags, turns=600, particles=len(grid),
                                  parameters=['x', 'px', 'y', 'py', 'dp'])
            sa.parameters[:] = grid[:, [0, 1, 2, 3, 5]]
            sa.run(compact=compact)
            out.append((sa.lost.copy(), sa.final.copy()))
        for lost, final in out[1:]:
            assert np.array_equal(out[0][0], lost)
            assert np.array_equal(out[0][1], final, equal_nan=True)
        assert 0 < np.sum(out[0][0] < 600) < len(grid)


def test_seed_batch_equals_individual_launches():
    """One launch over many error seeds == one launch per seed, bit for bit."""
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    ring = W.c1_ring(u)
    params = W.c4_parameters(ring)
    rows = W.c4_seed_rows(ring, 6)
    ctx = u.context(0)
    prog = C.compile_line(ring, u.KICK, params, [-1], seed_values=rows)
    dp = capi.DeviceProgram(ctx, prog)
    beam = W.c1_beam(6 * 40, seed=3)
    seed = np.repeat(np.arange(6), 40).astype(np.int32)
    pturns = np.repeat(np.array([50, 80, 30, 60, 45, 70]), 40).astype(np.int32)
    _, lost, final = capi.track(ctx, dp, beam, 80, capi.UFO_MODE_TRACK, 0, seed=seed,
                                pturns=pturns, slots=0)
    for s in range(6):
        p1 = C.compile_line(ring, u.KICK, params, [-1], seed_values=rows[s:s + 1])
        d1 = capi.DeviceProgram(ctx, p1)
        sl = slice(40 * s, 40 * (s + 1))
        _, l1, f1 = capi.track(ctx, d1, beam[sl], int(pturns[40 * s]), capi.UFO_MODE_TRACK, 0,
                               slots=0)
        assert np.array_equal(f1, final[sl], equal_nan=True)
        assert np.array_equal(l1, lost[sl])


def test_seed_batch_vs_oracle_high_orders():
    """C4 errors up to index 5 (orders beyond what the reference's source
    generator handles) against the oracle."""
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    from oracle import oracle as O
    ring = W.c1_ring(u)
    params = W.c4_parameters(ring)
    rows = W.c4_seed_rows(ring, 3)
    beam = W.c1_beam(96, seed=5) * 30
    seed = np.repeat(np.arange(3), 32).astype(np.int32)
    prog = C.compile_line(ring, u.KICK, params, [-1], seed_values=rows)
    ctx = u.context(0)
    dp = capi.DeviceProgram(ctx, prog)
    _, lost, final = capi.track(ctx, dp, beam, 40, capi.UFO_MODE_TRACK, 0, seed=seed, slots=0)
    ref = O.track(ring, u.KICK, beam, 40, parameters=params, where=[-1], seed=seed,
                  seed_values=rows, tracks=False)
    assert np.array_equal(final, ref['final'], equal_nan=True)


def test_optics_tunes():
    import ufo_gb300 as u
    meta, _ = H.golden()
    c = H.case('alba_optics_fp64')
    o = u.Optics(H.line_of(c), where=[], flags=c['flags'])
    o.run()
    assert abs(o.qx - float(H.arr(c['name'], 'out/qx'))) < 1e-12
    assert abs(o.qy - float(H.arr(c['name'], 'out/qy'))) < 1e-12
    assert abs(o.qx - meta['madx']['alba_qx']) < 1e-5
    assert abs(o.qy - meta['madx']['alba_qy']) < 1e-5


def test_optics_chromaticity_fd():
    import ufo_gb300 as u
    meta, _ = H.golden()
    c0 = H.case('alba_chroma_fd_0')
    o = u.Optics(H.line_of(c0), where=[], parameters=['dp'], flags=c0['flags'])
    o.parameters[0] = 0.0
    o.run()
    qx0, qy0 = o.qx, o.qy
    o.parameters[0] = 1e-4
    o.run()
    dqx, dqy = (o.qx - qx0) / 1e-4, (o.qy - qy0) / 1e-4
    rx = (float(H.arr('alba_chroma_fd_1', 'out/qx')) - float(H.arr('alba_chroma_fd_0', 'out/qx')))
    assert abs(dqx - rx / 1e-4) < 1e-6
    assert abs(dqx - meta['madx']['alba_dqx']) < 0.1
    assert abs(dqy - meta['madx']['alba_dqy']) < 0.1


def test_thick_vs_kick_tunes():
    import ufo_gb300 as u
    c = H.case('alba_kick_16_48')
    kick = u.Optics(H.line_of(c), flags=c['flags'])
    kick.run()
    assert abs(kick.qx - float(H.arr(c['name'], 'out/qx'))) < 1e-12
    thick = u.Optics(H.line_of(H.case('alba_optics_fp64')),
                     flags=u.LINEAR | u.ACHROMATIC | u.DOUBLE_PRECISION)
    thick.run()
    assert abs(thick.qx - kick.qx) < 5e-4 and abs(thick.qy - kick.qy) < 5e-4


def test_align_dispersion():
    import ufo_gb300 as u
    fo = H.case('align_fodo')
    eq = H.case('align_equiv')
    a = u.Optics(H.line_of(fo), where=[-1], flags=fo['flags'])
    b = u.Optics(H.line_of(eq), where=[-1], flags=eq['flags'])
    a.run()
    b.run()
    assert abs(a.dx[0] - float(H.arr('align_fodo', 'out/dx')[0])) < 1e-12
    assert abs(a.dx[0] - b.dx[0]) < 1e-6


def test_optics_propagate_and_where():
    import ufo_gb300 as u
    c = H.case('alba_optics_where')
    o = u.Optics(H.line_of(c), where=c['where'], flags=c['flags'])
    o.run()
    for k in ('bx', 'by', 'ax', 'ay', 'dx', 'dpx', 'mux', 'muy'):
        assert np.allclose(getattr(o, k), H.arr(c['name'], f'out/{k}'), rtol=1e-10, atol=1e-12)
    c = H.case('alba_optics_propagate')
    p = u.Optics(H.line_of(c), where=c['where'], periodic=False, flags=c['flags'])
    for k, v in c['attrs'].items():
        setattr(p, k, v)
    p.run()
    assert np.allclose(p.bx, H.arr(c['name'], 'out/bx'), rtol=1e-10)


def test_closed_orbit_vs_reference_and_tracking():
    """The reference's Nelder-Mead search on the GPU reproduces its orbit bit
    for bit; Newton finds the exact fixed point (within the reference's 1e-8
    Nelder-Mead accuracy of it, and a fixed point of the tracking to 1e-14)."""
    import ufo_gb300 as u
    c = H.case('alba_co_qd1')
    line = H.line_of(c)
    ref = H.arr(c['name'], 'out/orbits')
    am = u.ClosedOrbit(line, particles=1, flags=c['flags'])
    am.run()
    assert np.array_equal(am.orbits, ref)
    co = u.ClosedOrbit(line, particles=1, flags=c['flags'], method='newton')
    co.run()
    assert np.max(np.abs(co.orbits - ref)) < 1e-8
    tr = u.Track(line, parameters=['x', 'px', 'y', 'py'], turns=1, particles=1, where=[-1],
                 flags=u.DOUBLE_PRECISION)
    tr.parameters[0, :4] = co.orbits[0]
    tr.run()
    assert np.max(np.abs(tr.tracks[0, 0, :4] - co.orbits[0])) < 1e-14


def test_closed_orbit_parameter_batch():
    import ufo_gb300 as u
    c = H.case('alba_co_sext_dx')
    line = H.line_of(c)
    params = H.latjson.params_load(c['parameters'])
    ref = H.arr(c['name'], 'out/orbits')
    for method in ('amoeba', 'newton'):
        co = u.ClosedOrbit(line, particles=c['particles'], flags=c['flags'], parameters=params,
                           method=method)
        co.parameters[:, :] = H.arr(c['name'], 'in/pool')
        co.run()
        if method == 'amoeba':  # one seed row per orbit, the reference's steps
            assert np.array_equal(co.orbits, ref)
        else:
            assert np.max(np.abs(co.orbits - ref)) < 1e-8


@pytest.mark.parametrize('name', ['c1_seeds_kick', 'nlk_pulse'])
def test_parameter_rerun_reuses_the_program(name):
    """The reference's workflow: one simulation object, new lattice values in
    ``.parameters`` between runs.  The second run takes the set-table path (the
    device program object is the same; only the per-seed constants are
    re-uploaded) and reproduces the reference's golden tracks.  Cases: the C1
    ring with per-particle misalignments and sextupole errors, and the HOWTO's
    pulsed kicker with a per-particle trigger turn (cases whose particles keep
    tracking, so that the first run's other values show in its tracks)."""
    c = H.case(name)
    import ufo_gb300 as u
    line = H.line_of(c)
    params = H.latjson.params_load(c['parameters'])
    pool = H.arr(name, 'in/pool')
    t = u.Track(line, flags=c['flags'], turns=c['turns'], particles=pool.shape[0],
                parameters=params, where=c['where'], dp=c.get('dp', 0.0))
    lat = [j for j, p in enumerate(params) if isinstance(p, tuple)]
    assert lat
    first = pool.copy()
    first[:, lat] *= 1.5  # other lattice values, same zero pattern
    t.parameters[:] = first
    t.run()
    dprog = t._c._dprog
    before = t.tracks.copy()
    t.parameters[:] = pool
    t.run()
    assert t._c._dprog is dprog
    ref = H.arr(name, 'out/tracks')
    assert not np.array_equal(before, ref, equal_nan=True)
    if H.program_is_exact(t.program):
        assert np.array_equal(t.tracks, ref, equal_nan=True)
    else:
        _assert_within_tolerance(c, t.tracks, ref)


def test_c3_full_grid_fma_loss_turns_equal_strict():
    """Survival masks and loss turns of the whole dynamic-aperture benchmark
    (196,608 particles x 2,048 turns, C1 ring with apertures and errors) in
    FMA mode are the strict mode's, particle for particle; strict mode is the
    reference's arithmetic (bit-exact against the oracle above).  So the FMA
    throughput figures of this scan come with the reference's loss turns."""
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    ring = W.c3_ring(u)
    grid = W.c3_grid()
    ctx = u.context(0)
    ds = capi.DeviceProgram(ctx, C.compile_line(ring, u.KICK, where=[-1]))
    df = capi.DeviceProgram(ctx, C.compile_line(ring, u.KICK | u.FMA, where=[-1]))
    _, ls, _ = capi.track(ctx, ds, grid, 2048, capi.UFO_MODE_SA, 0, slots=0)
    _, lf, _ = capi.track(ctx, df, grid, 2048, capi.UFO_MODE_SA, capi.UFO_TRACK_FMA, slots=0)
    assert 0 < np.sum(ls < 2048) < len(grid)
    assert np.array_equal(lf, ls), int(np.sum(lf != ls))


@pytest.mark.parametrize('fma', [False, True])
def test_compacting_kernel_is_bit_identical(fma):
    """The CTA-compacting persistent kernel (survivors packed into the lowest
    warps of each CTA once the work counter is exhausted) moves particle
    states between lanes only: loss turns and final coordinates equal the
    one-warp persistent kernel's and the plain kernel's bit for bit, on an
    uneven dynamic-aperture grid and on a batch of error seeds with uneven
    particle and turn counts."""
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    ctx = u.context(0)
    fl = (u.FMA if fma else 0)
    tf = capi.UFO_TRACK_FMA if fma else 0
    ring = W.c3_ring(u)
    grid = W.c3_grid(96, 96)
    dp = capi.DeviceProgram(ctx, C.compile_line(ring, u.KICK | fl, where=[-1]))
    runs = [capi.track(ctx, dp, grid, 700, capi.UFO_MODE_SA, tf | extra, slots=0)
            for extra in (0, capi.UFO_TRACK_COMPACT, capi.UFO_TRACK_PLAIN)]
    assert 0 < np.sum(runs[0][1] < 700) < len(grid)
    for _, lost, final in runs[1:]:
        assert np.array_equal(lost, runs[0][1])
        assert np.array_equal(final, runs[0][2], equal_nan=True)
    # error seeds, uneven particles and turns, fewer warps than one CTA holds
    ring1 = W.c1_ring(u)
    params = W.c4_parameters(ring1)
    rows = W.c4_seed_rows(ring1, 5)
    prog = C.compile_line(ring1, u.KICK | fl, params, [], seed_values=rows)
    dq = capi.DeviceProgram(ctx, prog)
    parts = np.array([37, 300, 5, 64, 211])
    seed = np.repeat(np.arange(5), parts).astype(np.int32)
    pturns = np.repeat(np.array([90, 7, 150, 0, 41]), parts).astype(np.int32)
    beam = W.c1_beam(int(parts.sum()), seed=12)
    out = [capi.track(ctx, dq, beam, 150, capi.UFO_MODE_TRACK, tf | extra, seed=seed,
                      pturns=pturns, slots=0) for extra in (0, capi.UFO_TRACK_COMPACT)]
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2], equal_nan=True)
    assert np.array_equal(out[0][1], pturns)  # nothing is lost in the C1 ring


@pytest.mark.parametrize('fma', [False, True])
def test_compacting_kernel_pool_exchange_is_bit_identical(fma):
    """Uneven work per CTA once the work counter runs out: the particles of
    every seventh chunk of 32 track 300 turns, the others 3.  The compacting
    kernel's CTAs then hold from none to several chunks of long-lived
    particles and even them out through the context's particle pool (CTAs
    that run empty leave).  Loss turns and final coordinates equal the
    one-warp and plain kernels' bit for bit, so every particle was finished
    exactly once and none stayed behind in the pool."""
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    ctx = u.context(0)
    tf = capi.UFO_TRACK_FMA if fma else 0
    ring = W.c1_ring(u)
    dp = capi.DeviceProgram(ctx, C.compile_line(ring, u.KICK | (u.FMA if fma else 0),
                                                where=[-1]))
    n = 152 * 8 * 32 + 17
    beam = W.c1_beam(n, seed=21)
    pturns = np.where((np.arange(n) // 32) % 7 == 0, 300, 3).astype(np.int32)
    before = ctx.warps_per_sm
    out = {}
    try:
        for name, extra, warps in (('one-warp', 0, 16), ('plain', capi.UFO_TRACK_PLAIN, 16),
                                   ('compact8', capi.UFO_TRACK_COMPACT, 8),
                                   ('compact16', capi.UFO_TRACK_COMPACT, 16)):
            ctx.set_tuning(warps)
            out[name] = capi.track(ctx, dp, beam, 300, capi.UFO_MODE_TRACK, tf | extra,
                                   pturns=pturns, slots=0)
    finally:
        ctx.set_tuning(before)
    _, lost, final = out['one-warp']
    assert np.array_equal(lost, pturns)  # nothing is lost in the C1 ring
    for name in ('plain', 'compact8', 'compact16'):
        assert np.array_equal(out[name][1], lost), name
        assert np.array_equal(out[name][2], final, equal_nan=True), name


def test_stable_aperture_with_turn_dependent_kicker_runs_in_one_phase():
    """A time-dependent element (the HOWTO's gate kicker, firing on turn 20)
    reads ``turn``: StableAperture must not restart turn numbers in a second
    phase, so a two-phase request runs the in-kernel compaction instead, and
    every variant equals the plain one-launch run."""
    import ufo_gb300 as u
    import kickers
    from ufo_gb300 import workloads as W
    ring = W.c3_ring(u)
    kick = kickers.NLKGate('nlk', knl=[0.0, 0.0, 0.0], ksl=[0.0])
    kick.knl[1] = 0.5
    line = u.Line('ring', [kick] + list(ring.flatten()))
    grid = W.c3_grid(80, 80)
    out = []
    for compact in (None, 'two-phase', False):
        sa = u.StableAperture(line, flags=u.KICK | u.DOUBLE_PRECISION, turns=520,
                              particles=len(grid), parameters=['x', 'px', 'y', 'py', 'dp'])
        assert sa._uses_turn()
        sa.parameters[:] = grid[:, [0, 1, 2, 3, 5]]
        sa.run(compact=compact)
        out.append(sa.lost.copy())
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])
    assert 0 < np.sum(out[0] < 520) < len(grid)


@pytest.mark.parametrize('yoshida', [False, True])
def test_power_series_kicks_are_bit_identical(yoshida):
    """FMA programs give general kicks a dense power series prepared on the
    host (F_PSER): the kernels load the products RN(kn * RN(1/n!)) they would
    otherwise form at every order.  The same program with the flag cleared
    takes the per-order path; both give the same bits (error seeds of orders
    3-6 on every magnet, teapot and Yoshida slices, plain thin kicks)."""
    import types
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    ctx = u.context(0)
    ring = W.c1_ring(u)
    extra = [u.Multipole('m', knl=[0.0, 0.0, 3.0, 10.0, 1e3, 1e5], ksl=[0.0, 0.1, 0.0, 5.0])]
    line = u.Line('l', list(ring.flatten()) + extra)
    params = W.c4_parameters(ring)
    rows = W.c4_seed_rows(ring, 4)
    fl = u.KICK | u.FMA | (u.YOSHIDA if yoshida else 0)
    prog = C.compile_line(line, fl, params, [], seed_values=rows)
    assert any(int(r[1]) & C.F_PSER for r in prog.ops)
    plain = types.SimpleNamespace(ops=prog.ops.copy(), table=prog.table, n_dumps=prog.n_dumps)
    plain.ops[:, 1] &= ~C.F_PSER
    beam = W.c1_beam(3000, seed=21)
    seed = (np.arange(3000) % 4).astype(np.int32)
    out = [capi.track(ctx, capi.DeviceProgram(ctx, p), beam, 60, capi.UFO_MODE_TRACK,
                      capi.UFO_TRACK_FMA, seed=seed, slots=0) for p in (prog, plain)]
    assert np.array_equal(out[0][2], out[1][2], equal_nan=True)
    assert np.array_equal(out[0][1], out[1][1])
