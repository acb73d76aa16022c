#!/usr/bin/env python
"""Benchmark: FP64 particle*element*turns/s on one GB300 (or N, weak scaling).

Headline workload (C2): 65,536 Gaussian particles through the 1024-element
synthetic light-source ring (teapot, 4 slices; see ufo_gb300/workloads.py).  A
step is one launch tracking every particle 1,000 turns, each step continuing
from the previous step's coordinates.  Element = one entry of Line.flatten().

Printed (rank 0, one JSON line):
  value      device-resident inputs, CUDA events over exactly K steps, max
             over ranks, L2 flushed (256 MiB memset) between steps
  e2e        the same K steps through the public API (Track.run with host
             numpy buffers: H2D of the coordinates, D2H of tracks/lost/final
             inside the timed region)
  roofline   FP64-pipe bound: the FP64 work the kernel executes (compiler model
             of its instruction mix, FMA = 2) over the mean launch time, against
             the DFMA peak measured live on the same GPU; beside it the
             reference expression's operation count over the same time and the
             committed ncu figures (profiles/track_kernel_c2_ncu.json)
  cpu_baseline  the reference's own generated kernel (oracle/_ref) under its
             default fast-math options, or the oracle port when that is absent,
             on a bounded sample on the host cores; cpu_baseline_strict_ieee the
             same kernel built strict (the parity build)
  strict, yoshida4  the same ring bit-identical to the reference, and with the
             4th-order Yoshida integrator of the configuration as specified
  c4, c3, c5 (one-rank runs only) the metric's other clauses: 512 batched error
             seeds against one launch per seed, the dynamic-aperture scan with
             in-kernel compaction, the adjoint against finite differences
--impl reference times the reference's CPU implementation the same way.

Other workloads (--workload) print one line each with more detail: c3 (every
kernel and particle order, the StableAperture variants), c4, c5.  --op-mix runs
one small launch per element type for an ncu instruction-mix capture.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

PARAMS = ['x', 'px', 'y', 'py', 'dp']


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--mode', default='fma', choices=['strict', 'fma'])
    ap.add_argument('--no-alt', action='store_true', help='skip the other-mode measurement')
    ap.add_argument('--no-yoshida', action='store_true',
                    help='skip the Yoshida-4 measurement of the C2 ring')
    ap.add_argument('--turns-per-step', type=int, default=1000)
    ap.add_argument('--particles', type=int, default=65536)
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--workload', default='c2', choices=['c2', 'c3', 'c4', 'c5'])
    ap.add_argument('--seeds', type=int, default=512, help='C4: number of seeds')
    ap.add_argument('--turn-div', type=int, default=1, help='C4: divide turn counts by this')
    ap.add_argument('--c5-seeds', type=int, default=256,
                    help='C5: error seeds in the GPU-filling adjoint batch')
    ap.add_argument('--c5-fd-params', type=int, default=8,
                    help='C5: parameters in the sampled multi-turn FD')
    ap.add_argument('--fp64-probe', action='store_true',
                    help='print the FP64-pipe probe table (latency, occupancy, active lanes)')
    ap.add_argument('--c5-skip-multiturn', action='store_true',
                    help='C5: optics gradients only (for profiling captures)')
    ap.add_argument('--c3-grid', type=int, default=256,
                    help='C3: radial and angular grid points (256: the benchmark grid)')
    ap.add_argument('--c3-compact-warps', type=int, default=0,
                    help='C3: resident warps per SM of the compacting kernel '
                         '(0: StableAperture.COMPACT_WARPS_PER_SM)')
    ap.add_argument('--op-mix', action='store_true',
                    help='one small launch per element type and mode (for an ncu op-mix capture)')
    ap.add_argument('--no-c4', action='store_true',
                    help='default line: skip the C4 batched-seed measurement')
    ap.add_argument('--no-c5', action='store_true',
                    help='default line: skip the C5 adjoint measurement')
    ap.add_argument('--no-c3', action='store_true',
                    help='default line: skip the C3 dynamic-aperture measurement')
    return ap.parse_args()


def dist():
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return world, rank, local


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile('w+', suffix='.csv', delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(['nvidia-smi', f'--id={self.device}',
                                       f'--query-gpu={self.Q}', '--format=csv,noheader,nounits',
                                       '-lms', '200'], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = []
        with open(self.f.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(',')]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace('.', '').isdigit()]
        reasons = set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == 'active':
                    reasons.add(name)
        load = sorted(sm)[len(sm) // 4:] if sm else []
        return {'sm_mhz': statistics.median(load) if load else None,
                'sm_max_mhz': max(mx) if mx else None, 'reasons': sorted(reasons),
                'samples': len(rows)}


def ref_runner(fast=False):
    """The reference's generated C2 kernel (oracle/_ref) when present, else
    the oracle port; bounded sample of 16,384 particles x 100 turns on all
    host cores.  ``fast``: the build under the reference's default fast-math
    options instead of the strict (parity) build.
    Returns (run, sample description, kind, particles, turns, threads)."""
    from ufo_gb300 import workloads as W
    threads = len(os.sched_getaffinity(0))
    n, turns = 16384, 100
    beam = W.c2_beam(n, seed=2)
    try:
        from oracle import ref_kernels as R
        if not R.available('c2_track'):
            raise FileNotFoundError('oracle/_ref/c2_track.c')
        k = R.RefKernel('c2_track', fast=fast)
        kind = 'reference'
        opts = ('gcc -O3 -ffast-math -ffp-contract=fast (the reference\'s default '
                '-cl-fast-relaxed-math -cl-mad-enable)' if fast else
                'gcc -O2 -ffp-contract=off (strict IEEE, the parity build)')
        desc = ('reference-generated OpenCL C of the C2 ring (its Track kernel), ' + opts +
                ', OpenMP team over its atomic work queue')
        run = lambda: k.run(beam[:, [0, 1, 2, 3, 5]], threads)  # noqa: E731
    except Exception:  # noqa: BLE001
        import ufo_gb300 as u
        from oracle import oracle as O
        ring = W.c2_ring(u)
        kind = 'port'
        desc = 'C restatement of the reference (oracle/ufo_oracle.c), OpenMP'
        run = lambda: O.track(ring, u.KICK, beam, turns, where=[-1], threads=threads,  # noqa
                              tracks=False)
    return run, f'C2 ring, {n} particles x {turns} turns per run; {desc}', kind, n, turns, threads


def cpu_baseline(ring_elems, runs=2, fast=False):
    run, desc, kind, n, turns, threads = ref_runner(fast)
    run()  # first touch
    best = min(_timed(run) for _ in range(runs))
    return {'value': n * ring_elems * turns / best, 'unit': 'particle*element*turns/s',
            'cores': threads, 'kind': kind, 'sample': desc, 'seconds': best}


def _timed(fn):
    t0 = time.perf_counter()
    fn()
    return time.perf_counter() - t0


def bench_reference(args):
    world, rank, _ = dist()
    if rank != 0:
        return
    from ufo_gb300 import workloads as W
    import ufo_gb300 as u
    ring_elems = len(W.c2_ring(u).flatten())
    # the reference's own default build options (fast math, contraction): its
    # speed as shipped; the strict build is the parity one
    run, desc, kind, n, turns, threads = ref_runner(fast=True)
    for _ in range(max(0, args.warmup)):
        run()
    sec = sum(_timed(run) for _ in range(args.steps))
    value = args.steps * n * ring_elems * turns / sec
    line = {'impl': 'reference', 'metric': 'FP64 particle*element*turns/s', 'value': value,
            'unit': 'particle*element*turns/s', 'n_gpus': args.gpus, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': 1e3 * sec / args.steps,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic',
            'config': {'workload': 'C2 light-source ring (1024 elements, teapot 4 slices, 10 mm '
                                   'aperture), Gaussian beam',
                       'sample_per_step': f'{n} particles x {turns} turns'},
            'cpu_baseline': {'value': value, 'unit': 'particle*element*turns/s',
                             'cores': threads, 'kind': kind, 'sample': desc},
            'e2e': {'value': value, 'unit': 'particle*element*turns/s',
                    'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def load_ncu(mode):
    """The committed ncu figures of the C2 kernel (profiles/track_kernel_c2_ncu.json):
    DRAM traffic per launch, FP64-pipe activity, executed flops per particle-turn."""
    p = os.path.join(HERE, 'profiles', 'track_kernel_c2_ncu.json')
    try:
        with open(p) as f:
            return json.load(f).get(mode) or {}
    except (OSError, ValueError):
        return {}


def roofline_obj(m, peak, ncu):
    """The roofline object of a tracking measurement ``m`` (timed_device):
    FP64-pipe bound.  achieved = executed FP64 flops (the compiler's model of
    the kernel's instruction mix, FMA = 2, equal to ncu's count on the C2
    kernel) x particle-turns / mean launch time.  Beside it: the same time
    against the reference expression's operation count (its arithmetic as
    written: the strength x oodppo in every slice, divisions by constants),
    and the committed ncu figures (FP64-pipe activity, DRAM traffic, executed
    flops measured)."""
    out = {'bound': 'fp64', 'achieved': m['achieved'], 'peak': peak, 'unit': 'GFLOP/s',
           'frac': m['achieved'] / peak if peak else None,
           'traffic': ncu.get('traffic_bytes_per_launch'),
           'flops_per_particle_turn': m['flops_per_particle_turn'],
           'flops_basis': 'executed FP64 work (FMA = 2), compiler model of the kernel',
           'reference_flops_per_particle_turn': m['reference_flops_per_particle_turn'],
           'frac_reference_expression': m['achieved_reference'] / peak if peak else None,
           'peak_source': 'measured live: ufo_fp64_peak (DFMA chains, 2 flop each); '
                          'MEASURED_PEAKS.json has no FP64 figure'}
    ex = ncu.get('executed_flops_per_particle_turn')
    if ex and peak:
        out['frac_executed_ncu'] = ex * m['pt_per_s'] / 1e9 / peak
    if ncu.get('fp64_pipe_active') is not None:
        out['fp64_pipe_active_ncu'] = ncu['fp64_pipe_active']
    return out


def bench_ours(args):
    import torch
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    from ufo_gb300.ranks import beam_seed, max_over_ranks
    world, rank, local = dist()
    torch.cuda.set_device(local)  # before the process group: NCCL binds the current device
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group('nccl')
    dev = torch.device('cuda', local)
    ctx = u.context(local)
    ring = W.c2_ring(u)
    n_elem = len(ring.flatten())
    n = args.particles
    T = args.turns_per_step
    beam = W.c2_beam(n, seed=beam_seed(rank))
    c0 = torch.from_numpy(beam).to(dev)
    bufs = [c0.clone(), torch.empty_like(c0)]
    lost = torch.empty(n, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    # a dedicated stream: the library launches on the stream it is given, and
    # the CUDA events below are recorded on the same stream
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    lib = capi.load()

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            import torch.distributed as tdist
            tdist.barrier()

    def timed_device(mode, steps, warmup, yoshida=False):
        """Exactly `steps` chained launches (1000 turns each) on HBM-resident
        coordinates, L2 flushed between launches; CUDA events on the stream."""
        flags = u.KICK | (u.FMA if mode == 'fma' else 0) | (u.YOSHIDA if yoshida else 0)
        tflags = capi.UFO_TRACK_FMA if mode == 'fma' else 0
        prog = C.compile_line(ring, flags, where=[-1])
        dprog = capi.DeviceProgram(ctx, prog)

        def step(i, ev=None):
            src, dst = bufs[i % 2], bufs[(i + 1) % 2]
            if ev:
                ev[0].record(stream)
            capi.check(lib.ufo_track_device(ctx.handle, dprog.handle, capi.ptr(src.data_ptr()),
                                            None, None, n, T, capi.UFO_MODE_TRACK, tflags, 0, 1,
                                            None, capi.ptr(lost.data_ptr()),
                                            capi.ptr(dst.data_ptr()),
                                            capi.ptr(stream.cuda_stream)))
            if ev:
                ev[1].record(stream)

        for i in range(warmup):
            flush.zero_()
            step(i)
        bufs[0].copy_(c0)
        barrier()
        l0 = ctx.launches()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for i in range(steps):
            flush.zero_()
            step(i, evs[i])
        t_end.record(stream)
        barrier()
        total_ms = max_over_ranks(t_start.elapsed_time(t_end), dev)
        kern_ms = [a.elapsed_time(b) for a, b in evs]
        lost_np = lost.cpu().numpy()
        # particle-turns tracked by the last launch (a lost particle stops)
        pt = np.where(lost_np < T, lost_np + 1, T).astype(np.float64).sum()
        # executed FP64 work of the kernel (FMA = 2; the compiler's model of
        # the instruction mix, equal to ncu's count on the C2 kernel) and the
        # reference expression's operation count
        fl = prog.flops_fast if mode == 'fma' else prog.flops
        sec = statistics.mean(kern_ms) / 1e3
        return {'value': world * n * n_elem * T * steps / (total_ms / 1e3),
                'ms_per_step': total_ms / steps, 'kernel_ms': kern_ms,
                'launches': ctx.launches() - l0, 'achieved': fl * pt / sec / 1e9,
                'achieved_reference': prog.flops * pt / sec / 1e9, 'pt_per_s': pt / sec,
                'flops_per_particle_turn': fl, 'reference_flops_per_particle_turn': prog.flops,
                'lost': int((lost_np < T).sum())}

    clocks = Clocks(local)
    clocks.start()
    main = timed_device(args.mode, args.steps, args.warmup)
    clk = clocks.stop()
    peak = ctypes_peak(ctx)
    other = 'strict' if args.mode == 'fma' else 'fma'
    alt = None if args.no_alt else timed_device(other, min(3, args.steps), 1)
    ysh = None if args.no_yoshida else timed_device(args.mode, min(2, args.steps), 1, True)

    e2e = None
    if not args.no_e2e:
        flags = u.KICK | (u.FMA if args.mode == 'fma' else 0)
        tr = u.Track(ring, flags=flags | u.DOUBLE_PRECISION, turns=T, particles=n,
                     parameters=PARAMS, where=[-1], every=T, context=ctx)
        host = beam[:, [0, 1, 2, 3, 5]].copy()
        for _ in range(args.warmup):
            tr.parameters[:] = host
            tr.run()
        barrier()
        t0 = time.perf_counter()
        cur = host
        for _ in range(args.steps):
            tr.parameters[:] = cur
            tr.run()
            cur = tr.final[:, [0, 1, 2, 3, 5]]
        barrier()
        e2e_s = max_over_ranks(time.perf_counter() - t0, dev)
        e2e = {'value': world * n * n_elem * T * args.steps / e2e_s,
               'unit': 'particle*element*turns/s',
               'h2d_bytes_per_step': n * 6 * 8,
               'd2h_bytes_per_step': n * (6 * 8 + 4 + 6 * 8),
               'api': 'ufo_gb300.Track(...).run() -> ufo_track (host buffers)'}
    # the other clauses of the metric, measured once on one GPU (rank 0 of a
    # one-rank run): batched vs one-launch-per-seed (C4), the dynamic-aperture
    # scan (C3) and the adjoint against finite differences (C5)
    side = {}
    if world == 1:
        if not args.no_c4:
            side['c4'] = c4_measure(ctx, stream, args.mode, seeds=512, turn_div=1, reps=2,
                                    warmup=1)
        if not args.no_c3:
            side['c3'] = c3_measure(ctx, stream, args.mode)
        if not args.no_c5:
            side['c5'] = c5_summary(c5_measure(args, ctx, stream))
    if rank != 0:
        return
    cb = None if args.no_cpu else cpu_baseline(n_elem, fast=True)
    cbs = None if args.no_cpu else cpu_baseline(n_elem, fast=False)
    line = {
        'metric': 'FP64 particle*element*turns/s', 'value': main['value'],
        'unit': 'particle*element*turns/s', 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': main['ms_per_step'], 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
        'config': {'workload': f'C2 light-source ring (1024 elements, teapot 4 slices, 10 mm '
                               f'aperture), {n} Gaussian particles, {args.steps * T} turns '
                               f'tracked ({args.steps} launches of {T} turns)',
                   'particles_per_gpu': n, 'turns_per_step': T, 'elements': n_elem,
                   'turns_tracked': args.steps * T,
                   'deviations_from_spec': [
                       'ring: 32 identical 12 m cells (384 m, 1024 elements); the specified '
                       'magnets need 9.22 m per cell, more than 268.8 m / 32',
                       'integrator: TEAPOT, 4 slices (the reference has no other); the '
                       'specified 4th-order Yoshida is the yoshida4 object of this line',
                       'reference arm and cpu_baseline: a sample of 16384 particles x 100 '
                       'turns per step of the same ring and metric'],
                   'mode': args.mode, 'l2': 'flushed (256 MiB memset) between steps',
                   'parallelism': f'weak: {n} particles per GPU, no collective'},
        'roofline': roofline_obj(main, peak, load_ncu(args.mode)),
        'gpu_launches': main['launches'],
        'kernel_ms': main['kernel_ms'],
        'lost_particles': main['lost'],
    }
    if alt:
        line[other] = {'value': alt['value'], 'ms_per_step': alt['ms_per_step'],
                       'steps': min(3, args.steps),
                       'roofline_frac': alt['achieved'] / peak if peak else None,
                       'flops_per_particle_turn': alt['flops_per_particle_turn'],
                       'note': ('bit-identical to the reference' if other == 'strict' else
                                'fused multiply-add, within 1e-9 of strict after 1000 turns')}
    if ysh:
        line['yoshida4'] = {
            'value': ysh['value'], 'ms_per_step': ysh['ms_per_step'], 'steps': min(2, args.steps),
            'roofline_frac': ysh['achieved'] / peak if peak else None,
            'flops_per_particle_turn': ysh['flops_per_particle_turn'], 'mode': args.mode,
            'note': 'the C2 configuration as specified (4th-order Yoshida, 4 slices); the '
                    'reference has only TEAPOT, so the headline and the reference arm use '
                    'TEAPOT'}
    if e2e:
        line['e2e'] = e2e
    if cb:
        line['cpu_baseline'] = {k: cb[k] for k in ('value', 'unit', 'cores', 'kind', 'sample')}
    if cbs:
        line['cpu_baseline_strict_ieee'] = {
            k: cbs[k] for k in ('value', 'unit', 'cores', 'kind', 'sample')}
    if clk:
        line['clocks'] = clk
    line.update(side)
    print(json.dumps(line), flush=True)


def c4_measure(ctx, stream, mode, seeds=512, turn_div=1, reps=2, warmup=1, plain=True):
    """Batched error seeds (C4): one autotuned persistent CUDA-graph launch over
    all seeds, timed ``reps`` times after ``warmup``; then the same seeds with
    one launch per seed (timed once), whose outputs must be identical.
    Returns a dict (the C4 object of the bench line)."""
    import torch
    import ufo_gb300 as u
    from ufo_gb300 import workloads as W
    parts, turns = W.c4_sizes(512)
    parts, turns = parts[:seeds], np.maximum(1, turns[:seeds] // turn_div)
    ring = W.c1_ring(u)
    params = W.c4_parameters(ring)
    rows = W.c4_seed_rows(ring, seeds)
    flags = u.KICK | (u.FMA if mode == 'fma' else 0)
    b = u.TrackBatch(ring, params, rows, parts, turns, flags=flags, context=ctx)
    b.coords[:] = W.c1_beam(b.n, seed=4)
    t0 = time.perf_counter()
    tuning = u.autotune(b)
    tune_s = time.perf_counter() - t0
    pet = b.particle_element_turns()

    def timed(fn, n):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    b.upload()
    b.capture()
    for _ in range(warmup):
        b.launch(stream=stream.cuda_stream)
    clocks = Clocks(ctx.device)
    clocks.start()
    l0 = ctx.launches()
    ms_batch = timed(lambda: b.launch(stream=stream.cuda_stream), reps)
    launches = ctx.launches() - l0
    clk = clocks.stop()
    fb, lb = [a.copy() for a in b.download()]
    peak = ctypes_peak(ctx)
    pt_own = np.repeat(b.turns.astype(np.int64), b.particles)
    lb64 = lb.astype(np.int64)
    tracked = float(np.where(lb64 < pt_own, lb64 + 1, pt_own).sum())
    fl = b.prog.flops_fast if mode == 'fma' else b.prog.flops
    achieved = fl * tracked / (ms_batch / 1e3) / 1e9
    out = {'value': pet / (ms_batch / 1e3), 'unit': 'particle*element*turns/s',
           'ms_per_launch': ms_batch, 'reps': reps, 'warmup': warmup,
           'seeds': seeds, 'turn_divisor': turn_div, 'particles': b.n,
           'particle_element_turns': pet, 'mode': mode, 'tuning': tuning,
           'autotune_s': tune_s,
           'workload': f'C4 batched error seeds: {seeds} seeds of the C1 ring (128 elements) with '
                       f'dx/dy ~ N(0, 50 um) and normal/skew errors of MAD orders 3-6, '
                       f'particles log-uniform 256-8192, turns U(1000, 4096)'
                       + (f' // {turn_div}' if turn_div > 1 else ''),
           'roofline': {'bound': 'fp64', 'achieved': achieved, 'peak': peak, 'unit': 'GFLOP/s',
                        'frac': achieved / peak if peak else None,
                        'flops_per_particle_turn': fl,
                        'flops_basis': 'executed FP64 work (FMA = 2), compiler model',
                        'reference_flops_per_particle_turn': b.prog.flops,
                        'frac_reference_expression':
                            achieved * b.prog.flops / fl / peak if peak else None},
           'gpu_launches': launches, 'clocks': clk}
    if plain:
        b.upload('seed')
        t0 = time.perf_counter()
        ms_plain = timed(lambda: b.plain_launches(stream=stream.cuda_stream), 1)
        fp, lp = b.download()
        identical = bool(np.array_equal(fb, fp, equal_nan=True) and np.array_equal(lb, lp))
        out['plain_one_launch_per_seed'] = {'value': pet / (ms_plain / 1e3), 'ms': ms_plain,
                                            'launches': int(np.sum(b.particles > 0)),
                                            'wall_s': time.perf_counter() - t0}
        out['speedup_batched_vs_plain'] = ms_plain / ms_batch
        out['identical_results'] = identical
    del b
    torch.cuda.empty_cache()
    return out


def bench_c4(args):
    """Batched error seeds (C4) as its own line."""
    import torch
    import ufo_gb300 as u
    torch.cuda.set_device(0)
    ctx = u.context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    r = c4_measure(ctx, stream, args.mode, seeds=args.seeds, turn_div=args.turn_div,
                   reps=args.steps, warmup=args.warmup)
    line = {'metric': 'FP64 particle*element*turns/s', 'value': r['value'],
            'unit': 'particle*element*turns/s', 'n_gpus': 1, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': r['ms_per_launch'], 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': r['workload'], 'particles': r['particles'],
                       'seeds': r['seeds'], 'mode': args.mode, 'tuning': r['tuning']},
            'roofline': dict(r['roofline'], traffic=None,
                             peak_source='measured live: ufo_fp64_peak'),
            'plain_one_launch_per_seed': r['plain_one_launch_per_seed'],
            'speedup_batched_vs_plain': r['speedup_batched_vs_plain'],
            'identical_results': r['identical_results'], 'gpu_launches': r['gpu_launches']}
    if r['clocks']:
        line['clocks'] = r['clocks']
    print(json.dumps(line), flush=True)


def bench_c3(args):
    """Dynamic-aperture scan (C3): 256 x 256 polar grid x 3 momenta = 196,608
    particles, 2,048 turns, StableAperture loss test, on the C1 ring with a 10 mm
    aperture and C4-style errors (survival very uneven).  The persistent kernel
    (lanes refilled from a work counter at turn boundaries) against the plain
    one-thread-per-particle kernel; loss turns must be identical.  Throughput
    counts the particle-turns actually tracked (a lost particle stops)."""
    import torch
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    torch.cuda.set_device(0)
    dev = torch.device('cuda', 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx = u.context(0)
    lib = capi.load()
    ring = W.c3_ring(u)
    n_elem = len(ring.flatten())
    grid = W.c3_grid(args.c3_grid, args.c3_grid)
    n, T = grid.shape[0], 2048
    flags = u.KICK | (u.FMA if args.mode == 'fma' else 0)
    tflags = capi.UFO_TRACK_FMA if args.mode == 'fma' else 0
    prog = C.compile_line(ring, flags, where=[-1])
    dprog = capi.DeviceProgram(ctx, prog)
    perms = {'shuffled': np.random.default_rng(3).permutation(n),
             # largest amplitude first: the early losses churn through the
             # refill first and the survivors follow as one block
             'amplitude': np.lexsort((-np.abs(grid[:, 5]), -np.hypot(grid[:, 0], grid[:, 2])))}
    inputs = {'sorted': torch.from_numpy(grid).to(dev)}
    for k, pm in perms.items():
        inputs[k] = torch.from_numpy(np.ascontiguousarray(grid[pm])).to(dev)
    lost = torch.empty(n, dtype=torch.int32, device=dev)
    final = torch.empty((n, 6), dtype=torch.float64, device=dev)

    kinds = {'compact': capi.UFO_TRACK_COMPACT, 'persistent': 0, 'plain': capi.UFO_TRACK_PLAIN}

    def launch(coords, kind):
        capi.check(lib.ufo_track_device(
            ctx.handle, dprog.handle, capi.ptr(coords.data_ptr()), None, None, n, T,
            capi.UFO_MODE_SA, tflags | kinds[kind], 0, 1, None,
            capi.ptr(lost.data_ptr()), capi.ptr(final.data_ptr()), capi.ptr(stream.cuda_stream)))

    def timed(order, kind, steps):
        coords = inputs[order]
        # the compacting kernel at StableAperture's resident warps per SM
        cw = args.c3_compact_warps or u.StableAperture.COMPACT_WARPS_PER_SM
        ctx.set_tuning(cw if kind == 'compact' else 16)
        for _ in range(args.warmup):
            launch(coords, kind)
        torch.cuda.synchronize()
        l0 = ctx.launches()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            launch(coords, kind)
        e1.record(stream)
        torch.cuda.synchronize()
        lo = lost.cpu().numpy().view(np.uint32).astype(np.int64)
        if order in perms:
            un = np.empty_like(lo)
            un[perms[order]] = lo
            lo = un
        return e0.elapsed_time(e1) / steps, ctx.launches() - l0, lo

    clocks = Clocks(0)
    clocks.start()
    runs = {}
    for order in ('sorted', 'shuffled', 'amplitude'):
        for kind in kinds:
            runs[(order, kind)] = timed(order, kind, args.steps)
    ctx.set_tuning(16)
    ms_p, launches, lost_p = runs[('sorted', 'compact')]
    ms_pers = runs[('sorted', 'persistent')][0]
    ms_plain = runs[('sorted', 'plain')][0]
    # the public API: StableAperture.run with two-phase compaction (default),
    # in-kernel compaction and none (host buffers in and out, wall clock)
    api = {}
    for compact in (False, 'two-phase', True):
        sa = u.StableAperture(ring, flags=flags | u.DOUBLE_PRECISION, turns=T, particles=n,
                              parameters=['x', 'px', 'y', 'py', 'dp'], context=ctx)
        sa.parameters[:] = grid[:, [0, 1, 2, 3, 5]]
        sa.run(compact=compact)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sa.run(compact=compact)
        api[compact] = (time.perf_counter() - t0, sa.lost.astype(np.int64).copy(),
                        getattr(sa, 'second_phase_warps_per_sm', None),
                        getattr(sa, 'survivors_after_first_phase', None))
    clk = clocks.stop()
    peak = ctypes_peak(ctx)
    # a particle lost at the end of turn t tracked t + 1 turns
    tracked = np.where(lost_p < T, lost_p + 1, T).sum()
    pet = float(tracked) * n_elem
    fl = prog.flops_fast if args.mode == 'fma' else prog.flops
    surv = float(np.mean(lost_p >= T))
    line = {'metric': 'FP64 particle*element*turns/s', 'value': pet / (ms_p / 1e3),
            'unit': 'particle*element*turns/s', 'n_gpus': 1, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': ms_p, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': f'C3 dynamic aperture: {args.c3_grid}x{args.c3_grid} polar '
                                   'grid (r 0-25 mm, angle 0-pi/2) x dp {-2%, 0, +2%}, 2048 '
                                   'turns, SA loss test, C1 ring with 10 mm apertures and C4 '
                                   'seed-0 errors',
                       'particles': n, 'turns': T, 'elements': n_elem, 'mode': args.mode,
                       'l2': 'inputs resident; each launch re-reads 9.4 MB of coordinates'},
            'roofline': {'bound': 'fp64', 'achieved': fl * tracked / (ms_p / 1e3) / 1e9,
                         'peak': peak, 'unit': 'GFLOP/s',
                         'frac': fl * tracked / (ms_p / 1e3) / 1e9 / peak if peak else None,
                         'traffic': None, 'flops_per_particle_turn': fl,
                         'peak_source': 'measured live: ufo_fp64_peak'},
            'survival_fraction': surv,
            'particle_turns_tracked': int(tracked),
            'kernel': 'CTA-compacting persistent kernel, one launch, '
                      f'{u.StableAperture.COMPACT_WARPS_PER_SM} warps per SM',
            'one_warp_persistent': {'value': pet / (ms_pers / 1e3), 'ms': ms_pers},
            'plain_one_thread_per_particle': {'value': pet / (ms_plain / 1e3), 'ms': ms_plain},
            'speedup_compact_vs_plain': ms_plain / ms_p,
            'speedup_compact_vs_one_warp_persistent': ms_pers / ms_p,
            'shuffled_order': {
                k: pet / (runs[('shuffled', k)][0] / 1e3) for k in kinds},
            'amplitude_order': {
                k: pet / (runs[('amplitude', k)][0] / 1e3) for k in kinds},
            'order_note': 'the same grid in a seeded random order (warps of the plain kernel '
                          'mix survivors and early losses) and largest amplitude first',
            'stable_aperture_api': {
                'one_phase_no_compaction': {'value': pet / api[False][0], 's': api[False][0]},
                'two_phase_compaction': {
                    'value': pet / api['two-phase'][0], 's': api['two-phase'][0],
                    'survivors_after_turns_div_8': api['two-phase'][3],
                    'second_phase_warps_per_sm': api['two-phase'][2]},
                'in_kernel_compaction': {'value': pet / api[True][0], 's': api[True][0]},
                'note': 'StableAperture.run end to end (host buffers); the two-phase run '
                        'tracks turns/8 on the full grid, then only the survivors on a grid '
                        'sized to them (the default); the in-kernel form packs survivors and '
                        'evens out the CTAs inside one launch'},
            'identical_loss_turns': bool(all(np.array_equal(lost_p, r[2])
                                             for r in runs.values()) and
                                         all(np.array_equal(a[1], lost_p)
                                             for a in api.values())),
            'gpu_launches': launches,
            # the second phase copies the survivors in and out once more
            'e2e': {'value': pet / api['two-phase'][0], 'unit': 'particle*element*turns/s',
                    'h2d_bytes_per_step': (n + (api['two-phase'][3] or 0)) * 6 * 8,
                    'd2h_bytes_per_step': (n + (api['two-phase'][3] or 0)) * (6 * 8 + 4),
                    'api': 'ufo_gb300.StableAperture(...).run() (two-phase compaction, the '
                           'default; host buffers)'}}
    if clk:
        line['clocks'] = clk
    print(json.dumps(line), flush=True)


def c3_measure(ctx, stream, mode, reps=2):
    """Dynamic-aperture scan (C3) for the default line: the 196,608-particle
    grid x 2,048 turns with the StableAperture loss test, in one launch of the
    CTA-compacting persistent kernel, the one-warp persistent kernel and the
    plain kernel (FMA arithmetic unless ``mode`` is strict), plus one strict
    launch whose loss turns are the reference's (bit-exact against the oracle
    in the GPU tests): every variant's loss turns must equal the strict
    ones.  ``e2e``: StableAperture.run (host buffers, two-phase compaction)."""
    import torch
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    lib = capi.load()
    dev = torch.device('cuda', ctx.device)
    ring = W.c3_ring(u)
    n_elem = len(ring.flatten())
    grid = W.c3_grid()
    n, T = grid.shape[0], 2048
    coords = torch.from_numpy(grid).to(dev)
    lost = torch.empty(n, dtype=torch.int32, device=dev)
    final = torch.empty((n, 6), dtype=torch.float64, device=dev)
    progs = {}

    def launch(m, extra):
        if m not in progs:
            progs[m] = capi.DeviceProgram(ctx, C.compile_line(
                ring, u.KICK | (u.FMA if m == 'fma' else 0), where=[-1]))
        tf = (capi.UFO_TRACK_FMA if m == 'fma' else 0) | extra
        capi.check(lib.ufo_track_device(
            ctx.handle, progs[m].handle, capi.ptr(coords.data_ptr()), None, None, n, T,
            capi.UFO_MODE_SA, tf, 0, 1, None, capi.ptr(lost.data_ptr()),
            capi.ptr(final.data_ptr()), capi.ptr(stream.cuda_stream)))

    def timed(m, extra, k):
        # the compacting kernel with StableAperture's resident warps per SM
        ctx.set_tuning(u.StableAperture.COMPACT_WARPS_PER_SM
                       if extra & capi.UFO_TRACK_COMPACT else 16)
        launch(m, extra)  # warm-up
        torch.cuda.synchronize()
        l0 = ctx.launches()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            launch(m, extra)
        e1.record(stream)
        torch.cuda.synchronize()
        return (e0.elapsed_time(e1) / k, ctx.launches() - l0,
                lost.cpu().numpy().view(np.uint32).astype(np.int64))

    ms_strict, _, lost_strict = timed('strict', capi.UFO_TRACK_COMPACT, 1)
    tracked = float(np.where(lost_strict < T, lost_strict + 1, T).sum())
    pet = tracked * n_elem
    variants = {}
    identical = True
    for name, extra in (('compact', capi.UFO_TRACK_COMPACT), ('persistent', 0),
                        ('plain', capi.UFO_TRACK_PLAIN)):
        ms, launches, lo = timed(mode, extra, reps)
        identical &= bool(np.array_equal(lo, lost_strict))
        variants[name] = {'value': pet / (ms / 1e3), 'ms': ms, 'launches': launches}
    ctx.set_tuning(16)
    sa = u.StableAperture(ring, flags=u.KICK | (u.FMA if mode == 'fma' else 0) |
                          u.DOUBLE_PRECISION, turns=T, particles=n,
                          parameters=['x', 'px', 'y', 'py', 'dp'], context=ctx)
    sa.parameters[:] = grid[:, [0, 1, 2, 3, 5]]
    sa.run()  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sa.run()
    e2e_s = time.perf_counter() - t0
    # the two-phase run copies the survivors of its first phase in and out once more
    n_io = n + (getattr(sa, 'survivors_after_first_phase', None) or 0)
    identical &= bool(np.array_equal(sa.lost.astype(np.int64), lost_strict))
    peak = ctypes_peak(ctx)
    prog = C.compile_line(ring, u.KICK | (u.FMA if mode == 'fma' else 0), where=[-1])
    fl = prog.flops_fast if mode == 'fma' else prog.flops
    best = variants['compact']
    achieved = fl * tracked / (best['ms'] / 1e3) / 1e9
    return {
        'workload': 'C3 dynamic aperture: 256x256 polar grid (r 0-25 mm, angle 0-pi/2) x dp '
                    '{-2%, 0, +2%} = 196,608 particles, 2,048 turns, SA loss test, C1 ring with '
                    '10 mm apertures and C4 seed-0 errors',
        'value': best['value'], 'unit': 'particle*element*turns/s', 'mode': mode,
        'kernel': 'CTA-compacting persistent kernel (CTAs exchange particles through a pool), '
                  f'one launch, {u.StableAperture.COMPACT_WARPS_PER_SM} warps per SM',
        'ms_per_launch': best['ms'], 'particle_turns_tracked': int(tracked),
        'survival_fraction': float(np.mean(lost_strict >= T)),
        'roofline': {'bound': 'fp64', 'achieved': achieved, 'peak': peak, 'unit': 'GFLOP/s',
                     'frac': achieved / peak if peak else None, 'flops_per_particle_turn': fl,
                     'flops_basis': 'executed FP64 work (FMA = 2), compiler model',
                     'reference_flops_per_particle_turn': prog.flops,
                     'frac_reference_expression':
                         achieved * prog.flops / fl / peak if peak else None},
        'variants': variants,
        'strict_one_launch': {'value': pet / (ms_strict / 1e3), 'ms': ms_strict},
        'loss_turns_identical_to_strict': identical,
        'loss_turns_note': 'every variant and the public API give, for all 196,608 particles, '
                           'the loss turns of the strict (bit-identical) arithmetic',
        'e2e': {'value': pet / e2e_s, 'unit': 'particle*element*turns/s', 's': e2e_s,
                'h2d_bytes_per_step': n_io * 6 * 8, 'd2h_bytes_per_step': n_io * (6 * 8 + 4),
                'api': 'ufo_gb300.StableAperture(...).run() (two-phase compaction, the default; '
                       'host buffers)'}}


def _normwise(g, fd):
    """max |g - fd| / max |fd| per output row."""
    g, fd = np.atleast_2d(g), np.atleast_2d(fd)
    return (np.max(np.abs(g - fd), axis=1) / np.max(np.abs(fd), axis=1)).tolist()


def _c5_multiturn(args, u, W, torch, ctx, stream, model, ring, params, vals, rng):
    """d/dk of the summed final amplitudes of 4,096 particles after 1,024 turns
    (checkpoints every 64) against central FD through the tracking kernel."""
    P = len(vals)
    launches = 0
    Np, T, ck = 4096, 1024, 64
    coords = W.c2_beam(Np, seed=3)
    o = 1.0 / (coords[:, 5] + 1.0)
    eng = model.engine(vals)
    # particles near a resonance have no derivative a finite difference can
    # resolve over 1,024 turns: a 1e-9 m start displacement grows far beyond
    # the regular orbits' linear growth there (median 47x, 99th percentile
    # 94x).  Particles above 200x are excluded from the objective (a fixed mask,
    # not differentiated); the comparison at looser thresholds is reported.
    pair = np.concatenate([coords[:, :4], coords[:, :4] + [1e-9, 0, 0, 0]])
    zp, _ = eng.forward(pair, np.concatenate([o, o]), T)
    growth = np.max(np.abs(zp[Np:, :4] - zp[:Np, :4]), axis=1) / 1e-9
    mask = growth < 1e4  # cotangents are computed for these; the objective uses < 200
    eng.device_ms, eng.launches = 0.0, 0
    t0 = time.perf_counter()
    zT, st = eng.forward(coords[:, :4], o, T, ck=ck)
    zbar = np.zeros((Np, 4))
    zbar[:, 0] = 2 * zT[:, 0] * mask
    zbar[:, 2] = 2 * zT[:, 2] * mask
    _, gp = eng.reverse(st, zbar)  # per particle [Np, P]
    obj = growth < 200
    g = gp[obj].sum(axis=0)
    wall_mt = time.perf_counter() - t0
    dev_mt = eng.device_ms
    launches += eng.launches
    tape_segments = eng.last_tape_segments
    del st
    torch.cuda.empty_cache()
    m = args.c5_fd_params
    idx = np.sort(rng.choice(P, m, replace=False))
    hm = 1e-7 * np.abs(vals[idx])
    rows_m = np.repeat(vals[None], 2 * m, 0)
    rows_m[0::2][np.arange(m), idx] += hm
    rows_m[1::2][np.arange(m), idx] -= hm
    b = u.TrackBatch(ring, params, rows_m, [Np] * (2 * m), [T] * (2 * m),
                     flags=u.KICK | u.FMA, context=ctx)
    b.coords[:] = np.tile(coords, (2 * m, 1))
    b.upload()
    b.capture()
    b.launch(stream=stream.cuda_stream)  # warm-up (graph upload)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ctx.launches()
    e0.record(stream)
    b.launch(stream=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    launches += ctx.launches() - l0
    dev_fdm = e0.elapsed_time(e1)
    fin, lost = b.download()
    ampp = (fin[:, 0] ** 2 + fin[:, 2] ** 2).reshape(2 * m, Np) * obj[None]
    fdp = (ampp[0::2] - ampp[1::2]) / (2 * hm[:, None])  # per particle [m, Np]
    fdm = fdp.sum(axis=1)
    rel = np.abs(g[idx] - fdm) / np.abs(fdp).sum(axis=1)
    pp = np.abs(gp[:, idx].T - fdp)[:, obj] / np.maximum(np.abs(fdp[:, obj]), 1e-300)
    fd_full = dev_fdm * P / m
    # the same differences through the differentiator's own forward map (the
    # map the adjoint differentiates; accuracy only, not timed)
    from ufo_gb300 import diff as D
    efd = D.DiffEngine(D.DiffProgram(ring, u.KICK, params, rows_m))
    zf, _ = efd.forward(np.tile(coords[:, :4], (2 * m, 1)), np.tile(o, 2 * m), T,
                        seed=np.repeat(np.arange(2 * m, dtype=np.int32), Np))
    ampp2 = (zf[:, 0] ** 2 + zf[:, 2] ** 2).reshape(2 * m, Np) * mask[None]
    fdp2 = (ampp2[0::2] - ampp2[1::2]) / (2 * hm[:, None])
    rel2 = np.abs(g[idx] - fdp2[:, obj].sum(axis=1)) / np.abs(fdp2[:, obj]).sum(axis=1)
    launches += efd.launches
    del efd, zf
    # a 4-point stencil (f(k-2h) - 8 f(k-h) + 8 f(k+h) - f(k+2h)) / 12h of the
    # same map at two steps: its truncation error falls as h^4 and its rounding
    # noise as 1/h, so at h = 1e-6..4e-6 (relative) it resolves the derivative
    # far below a central difference at h = 1e-7; the two steps' disagreement
    # is the stencil's own error estimate (accuracy only, not timed)
    steps4 = (1e-6, 4e-6)
    offs = np.array([2.0, 1.0, -1.0, -2.0])
    rows4, h4s = [], []
    for hr in steps4:
        h4 = hr * np.abs(vals[idx])
        h4s.append(h4)
        r = np.repeat(vals[None], 4 * m, 0)
        for q, c in enumerate(offs):
            r[q::4][np.arange(m), idx] += c * h4
        rows4.append(r)
    rows4 = np.concatenate(rows4)
    e4 = D.DiffEngine(D.DiffProgram(ring, u.KICK, params, rows4))
    z4, _ = e4.forward(np.tile(coords[:, :4], (len(rows4), 1)), np.tile(o, len(rows4)), T,
                       seed=np.repeat(np.arange(len(rows4), dtype=np.int32), Np))
    launches += e4.launches
    amp4 = (z4[:, 0] ** 2 + z4[:, 2] ** 2).reshape(len(steps4), m, 4, Np)
    del e4, z4
    st4 = {}
    fd4 = []
    for s, hr in enumerate(steps4):
        a4 = amp4[s]
        d = (-a4[:, 0] + 8 * a4[:, 1] - 8 * a4[:, 2] + a4[:, 3]) / (12 * h4s[s][:, None])
        fd4.append(d)
        st4[f'{hr:g}'] = float(np.max(np.abs(g[idx] - d[:, obj].sum(axis=1)) /
                                      np.abs(d[:, obj]).sum(axis=1)))
    stencil_self = float(np.max(np.abs(fd4[0][:, obj].sum(axis=1) - fd4[1][:, obj].sum(axis=1)) /
                                np.abs(fd4[0][:, obj]).sum(axis=1)))
    # the per-particle cotangents do not depend on the mask: the same
    # comparison over stricter regularity thresholds
    by_thr = {}
    for thr in (1e4, 1e3, 2e2):
        sub = growth < thr
        ga = gp[:, idx][sub].sum(axis=0)
        fs = fdp2[:, sub]
        by_thr[f'{thr:g}'] = {'particles': int(sub.sum()),
                              'max_rel_err': float(np.max(np.abs(ga - fs.sum(axis=1)) /
                                                          np.abs(fs).sum(axis=1)))}
    out = {
        'particles': Np, 'turns': T, 'checkpoint_every': ck,
        'regular_particles': int(obj.sum()),
        'regularity': 'final-state growth of a 1e-9 m start displacement < 200x',
        'tape_segments_in_parallel': tape_segments,
        'adjoint_device_ms': dev_mt, 'adjoint_wall_s': wall_mt,
        'fd_sample_params': m, 'fd_sample_device_ms': dev_fdm,
        'fd_all_params_device_ms_scaled': fd_full,
        'device_cost_ratio': fd_full / dev_mt,
        'fd_lost_particles': int(np.sum(lost < T)),
        'growth_quantiles_50_99_max': np.quantile(growth, [0.5, 0.99, 1.0]).tolist(),
        'max_rel_err_vs_central_fd_h1e-7': float(rel.max()),
        'rel_err_per_param': rel.tolist(),
        'rel_err_note': '|sum(adjoint - FD)| / sum|per-particle FD| over the regular '
                        'particles; FD through the tracking kernel (FMA mode); '
                        '_fd_same_map: through the differentiator\'s forward map; '
                        '4pt_stencil: (f(k-2h) - 8f(k-h) + 8f(k+h) - f(k+2h)) / 12h of '
                        'the same map at the relative steps named',
        'sampled_params': [params[i] for i in idx],
        'rel_err_per_param_fd_same_map': rel2.tolist(),
        'same_map_by_growth_threshold': by_thr,
        'max_rel_err_vs_4pt_stencil_same_map': st4,
        'stencil_steps_disagreement': stencil_self,
        'per_particle_median_rel_err': float(np.median(pp))}
    return out, launches


def c5_measure(args, ctx, stream):
    """Adjoint gradients (C5: the C2 ring with one error seed, 320 k1 + 192 k2)
    against central finite differences, accuracy over all 512 parameters and
    cost in device time (CUDA events around every kernel) and wall time:
      optics_one_seed    the 8 x 512 Jacobian of (closed orbit, Qx, Qy, xi_x,
                         xi_y): adjoint = Newton + one vjp launch pair for all
                         8 cotangents; FD = 1,024 perturbed rows batched into
                         one Newton job list (h = 1e-7 relative), plus a
                         4-point stencil (h = 1e-5, xi: 1e-4) as the tighter
                         check
      optics_batched     the same Jacobians for many error seeds, each method
                         batched until the GPU is full (adjoint: --c5-seeds
                         seeds; FD: 2 seeds = 2,048 rows), cost per Jacobian
      multiturn          d/dk of sum(x^2 + y^2) of 4,096 particles after 1,024
                         turns (particles on chaotic orbits masked out),
                         checkpoints every 64 turns; FD = batched
                         tracking of 2 x --c5-fd-params perturbed rings (4,096
                         particles each) through the persistent tracking
                         kernel, scaled to all 512 parameters
    """
    import torch
    import ufo_gb300 as u
    from ufo_gb300 import diff as D, workloads as W
    ring = W.c5_ring(u)
    params, vals = W.c5_parameters(ring)
    P = len(vals)
    # chromaticity = central difference of the tunes in dp at the reference's
    # dp step (1e-4, tests/optics3.py)
    model = D.OpticsModel(ring, u.KICK, params, h_dp=1e-4)
    clocks = Clocks(0)
    clocks.start()
    model.evaluate(vals)  # warm-up
    res = {}
    launches = 0

    # ---- one seed: full Jacobian
    t0 = time.perf_counter()
    out, saved = model.evaluate(vals)
    Jad = model.vjp(saved, np.eye(8))
    wall_adj = time.perf_counter() - t0
    dev_adj = saved[0].device_ms
    launches += saved[0].launches

    def fd_rows(hrel, stencil):
        h = hrel * np.abs(vals)
        rows = np.repeat(vals[None], len(stencil) * P, 0)
        for j, c in enumerate(stencil):
            rows[j::len(stencil)][np.arange(P), np.arange(P)] += c * h
        return rows, h

    rows, h = fd_rows(1e-7, (1, -1))
    t0 = time.perf_counter()
    fo, fs = model.evaluate_batch(rows)
    wall_fd = time.perf_counter() - t0
    dev_fd = fs[0].device_ms
    launches += fs[0].launches
    Jfd = ((fo[0::2] - fo[1::2]) / (2 * h[:, None])).T
    def st4(hrel):
        r, hh = fd_rows(hrel, (2, 1, -1, -2))
        f = model.evaluate_many(r)
        return ((-f[0::4] + 8 * f[1::4] - 8 * f[2::4] + f[3::4]) / (12 * hh[:, None])).T

    def richardson(hrel):  # 4-point stencils at h and 2h: the h^4 term cancels
        a, b = st4(hrel), st4(2 * hrel)
        return (16 * a - b) / 15, a

    J4, S4 = richardson(1e-5)
    J4x, S4x = richardson(1e-3)
    J4[6:8] = J4x[6:8]
    S4[6:8] = S4x[6:8]
    names = ['x_co', 'px_co', 'y_co', 'py_co', 'Qx', 'Qy', 'xi_x', 'xi_y']
    res['optics_one_seed'] = {
        'outputs': dict(zip(names, out.tolist())),
        'adjoint_device_ms': dev_adj, 'adjoint_wall_s': wall_adj,
        'fd_device_ms': dev_fd, 'fd_wall_s': wall_fd,
        'device_cost_ratio': dev_fd / dev_adj, 'wall_cost_ratio': wall_fd / wall_adj,
        'normwise_rel_err_vs_central_fd_h1e-7': dict(zip(names, _normwise(Jad, Jfd))),
        'normwise_rel_err_vs_4pt_fd': dict(zip(names, _normwise(Jad, J4))),
        'stencil': 'Richardson-combined 4-point stencils (h, 2h): h = 1e-5 relative for orbit '
                   'and tunes, 1e-3 for the chromaticities (dp difference at 1e-4)',
        'stencil_own_error_estimate': dict(zip(names, _normwise(S4, J4))),
        'note': 'one seed leaves the GPU mostly idle: the 3,072 FD Newton jobs run '
                'beside each other in the time of the 3 adjoint jobs'}

    # ---- GPU-filling batches: cost per 8 x 512 Jacobian
    rng = np.random.default_rng(55)
    Sa = args.c5_seeds
    rows_a = vals[None] * (1 + 1e-3 * rng.standard_normal((Sa, P)))
    t0 = time.perf_counter()
    oa, sa = model.evaluate_batch(rows_a)
    Ka = model.vjp(sa, np.repeat(np.eye(8)[None], Sa, 0))
    wall_a = time.perf_counter() - t0
    dev_a = sa[0].device_ms
    launches += sa[0].launches
    Sf = 2
    rows_f = np.concatenate([fd_rows(1e-7, (1, -1))[0] * (r / vals)[None]
                             for r in rows_a[:Sf]])
    t0 = time.perf_counter()
    of, sf = model.evaluate_batch(rows_f)
    wall_f = time.perf_counter() - t0
    dev_f = sf[0].device_ms
    launches += sf[0].launches
    res['optics_batched'] = {
        'adjoint_seeds': Sa, 'fd_seeds': Sf,
        'adjoint_device_ms_per_jacobian': dev_a / Sa, 'fd_device_ms_per_jacobian': dev_f / Sf,
        'adjoint_wall_ms_per_jacobian': 1e3 * wall_a / Sa,
        'fd_wall_ms_per_jacobian': 1e3 * wall_f / Sf,
        'device_cost_ratio': (dev_f / Sf) / (dev_a / Sa),
        'wall_cost_ratio': (wall_f / Sf) / (wall_a / Sa)}

    # ---- multi-turn amplitude adjoint
    if not args.c5_skip_multiturn:
        res['multiturn'], n_l = _c5_multiturn(args, u, W, torch, ctx, stream, model, ring,
                                              params, vals, rng)
        launches += n_l
    clk = clocks.stop()
    ratios = [res['optics_batched']['device_cost_ratio']]
    if res.get('multiturn'):
        ratios.append(res['multiturn']['device_cost_ratio'])
    res['device_cost_ratio_min'] = min(ratios)
    res['gpu_launches'] = launches
    res['clocks'] = clk
    return res


def bench_c5(args):
    """Adjoint gradients (C5) as its own line."""
    import torch
    import ufo_gb300 as u
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)  # every kernel below and its events on one stream
    ctx = u.context(0)
    res = c5_measure(args, ctx, stream)
    line = {'metric': 'adjoint gradient cost advantage over central finite differences '
                      '(device time, all 512 parameters)',
            'value': res.pop('device_cost_ratio_min'), 'unit': 'x', 'n_gpus': 1, 'steps': 1,
            'warmup': 1, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': C5_WORKLOAD},
            'gpu_launches': res.pop('gpu_launches'), 'clocks': res.pop('clocks')}
    line.update(res)
    print(json.dumps(line), flush=True)


def c5_summary(res):
    """The C5 object of the default line: cost ratios and accuracy over all
    512 strengths (details in ``--workload c5``)."""
    one, bat = res['optics_one_seed'], res['optics_batched']
    out = {'workload': C5_WORKLOAD,
           'value': res['device_cost_ratio_min'], 'unit': 'x (FD device time / adjoint)',
           'optics_jacobian_8x512': {
               'device_cost_ratio_batched': bat['device_cost_ratio'],
               'wall_cost_ratio_batched': bat['wall_cost_ratio'],
               'device_cost_ratio_one_seed': one['device_cost_ratio'],
               'max_normwise_rel_err_vs_stencil': max(one['normwise_rel_err_vs_4pt_fd'].values()),
               'normwise_rel_err_vs_stencil': one['normwise_rel_err_vs_4pt_fd'],
               'normwise_rel_err_vs_central_fd_h1e-7':
                   one['normwise_rel_err_vs_central_fd_h1e-7'],
               'stencil': one.get('stencil')},
           'gpu_launches': res['gpu_launches'], 'clocks': res['clocks']}
    mt = res.get('multiturn')
    if mt:
        out['multiturn_4096x1024'] = {
            k: mt[k] for k in ('device_cost_ratio', 'adjoint_device_ms',
                               'fd_all_params_device_ms_scaled', 'regular_particles',
                               'max_rel_err_vs_4pt_stencil_same_map',
                               'stencil_steps_disagreement',
                               'max_rel_err_vs_central_fd_h1e-7') if k in mt}
    return out


C5_WORKLOAD = ('C5 adjoint optics gradients: C2 ring (1024 elements) with one error seed, '
               'd/d(320 k1 + 192 k2) of closed orbit, tunes, chromaticity; 4096-particle '
               '1024-turn amplitude adjoint with checkpoints every 64 turns')


def ctypes_peak(ctx):
    import ctypes
    from ufo_gb300 import capi
    g = ctypes.c_double()
    capi.check(capi.load().ufo_fp64_peak(ctx.handle, ctypes.byref(g)))
    return g.value


def fp64_probe():
    """The FP64 pipe under controlled conditions: resident warps per SM,
    independent DFMA chains per thread, active lanes per warp."""
    import ctypes
    import ufo_gb300 as u
    from ufo_gb300 import capi
    ctx = u.context(0)
    lib = capi.load()
    rows = []
    for w, ch, lanes in ((4, 1, 32), (4, 8, 32), (16, 1, 32), (16, 8, 32), (32, 8, 32),
                         (16, 8, 16), (16, 8, 8), (16, 8, 1)):
        g = ctypes.c_double()
        capi.check(lib.ufo_fp64_probe(ctx.handle, w, ch, lanes, ctypes.byref(g)))
        rows.append({'warps_per_sm': w, 'chains_per_thread': ch, 'active_lanes': lanes,
                     'useful_gflops': g.value})
    print(json.dumps({'fp64_probe': rows, 'fp64_peak_gflops': ctypes_peak(ctx)}), flush=True)


def op_mix():
    """One small launch per element type and arithmetic mode (strict, FMA):
    64 identical elements, 4,096 particles, 10 turns each -- the command an
    ncu capture of the FP64 instruction mix per element type runs (counts per
    launch / (4,096 x 10 x 64) = per particle and element)."""
    import math
    import ufo_gb300 as u
    from ufo_gb300 import capi, compiler as C, workloads as W
    ctx = u.context(0)
    n, T = 4096, 10
    beam = W.c2_beam(n, seed=6)
    lines = {
        'drift': [u.Drift(f'd{i}', length=1.0) for i in range(64)],
        'quad': [u.Quadrupole(f'q{i}', length=0.25, k1=1.2 * (-1) ** i, slices=4)
                 for i in range(64)],
        'sext': [u.Sextupole(f's{i}', length=0.2, k2=40.0 * (-1) ** i, slices=4)
                 for i in range(64)],
        'bend': [u.Sbend(f'b{i}', length=1.38, angle=2 * math.pi / 128, slices=4)
                 for i in range(64)],
    }
    out = []
    for name, elems in lines.items():
        line = u.Line(name, elems)
        for mode in ('strict', 'fma'):
            prog = C.compile_line(line, u.KICK | (u.FMA if mode == 'fma' else 0), where=[-1])
            dp = capi.DeviceProgram(ctx, prog)
            capi.track(ctx, dp, beam, T, capi.UFO_MODE_TRACK,
                       capi.UFO_TRACK_FMA if mode == 'fma' else 0, slots=0)
            out.append({'type': name, 'mode': mode, 'elements': 64, 'particles': n, 'turns': T,
                        'ops_per_turn': len(prog.ops),
                        'reference_flops_per_element': prog.flops / 64,
                        'fma_flops_per_element': prog.flops_fast / 64})
    print(json.dumps({'op_mix_launches': out}), flush=True)


def main():
    args = parse()
    if args.fp64_probe:
        fp64_probe()
        return
    if args.op_mix:
        op_mix()
        return
    if args.impl == 'reference':
        bench_reference(args)
    elif args.workload == 'c3':
        bench_c3(args)
    elif args.workload == 'c4':
        bench_c4(args)
    elif args.workload == 'c5':
        bench_c5(args)
    else:
        bench_ours(args)


if __name__ == '__main__':
    main()
