"""Batched error seeds: many lattice variants, uneven particle and turn counts,
one persistent launch.

The reference runs lattice variants by giving every particle its own
parameter row in one NDRange (HOWTO.md:21, :522-565; ufo/track.py:96-101).
Here a seed is one row of lattice-parameter values (a per-seed constant
table); every particle carries its seed index and its own turn count, and one
launch of the persistent kernel tracks them all.  The launch (work-counter
reset + kernel) is captured once into a CUDA graph and replayed.  Particles are
ordered longest-first (LPT) so the last warps to finish hold the shortest
work; the resident-warp count and the ordering come from the autotuner
(``autotune``), which times candidates on a turn-scaled copy of the workload
and caches the winner per device and workload shape.

Device buffers are PyTorch tensors (plumbing only; the arithmetic is the
library's).  ``run_plain`` is the one-launch-per-seed path the batched launch
is compared with.
"""
import hashlib
import json
import os

import numpy as np

from . import capi
from . import compiler as C
from .flags import FMA, KICK


def _torch():
    import torch
    return torch


class TrackBatch:
    """Track ``particles[s]`` particles of seed ``s`` for ``turns[s]`` turns,
    for all seeds in one launch.

    line        the ring (its flattened elements)
    parameters  the reference-style lattice parameter list, e.g.
                [(7, 'dx'), (7, 'dk2'), ...]; ``seeds[s]`` holds their values
    seeds       float64 [S, len(parameters)]
    coords      float64 [sum(particles), 6], grouped by seed (filled by caller)
    After ``run()``: ``final`` [n, 6], ``lost`` [n] (loss turn, or the
    particle's own turn count if it survived), in the caller's order.
    """

    def __init__(self, line, parameters, seeds, particles, turns, flags=KICK, context=None,
                 mode=capi.UFO_MODE_TRACK, order='lpt'):
        from .drivers import context as _context
        self.ctx = context if context is not None else _context(0)
        self.flags = flags
        self.mode = mode
        self.order = order
        seeds = np.atleast_2d(np.asarray(seeds, dtype=np.float64))
        self.particles = np.asarray(particles, dtype=np.int64)
        self.turns = np.asarray(turns, dtype=np.int32)
        if seeds.shape[0] != len(self.particles) or len(self.turns) != len(self.particles):
            raise ValueError('seeds, particles and turns must have one entry per seed')
        self.n = int(self.particles.sum())
        self.seed = np.repeat(np.arange(len(self.particles), dtype=np.int32), self.particles)
        self.pturns = np.repeat(self.turns, self.particles).astype(np.int32)
        self.coords = np.zeros((self.n, 6))
        self.prog = C.compile_line(line, flags, list(parameters), [], seed_values=seeds)
        self.dprog = capi.DeviceProgram(self.ctx, self.prog)
        self.n_elements = self.prog.n_elements
        self._graph = None
        self._dev = None
        self.final = None
        self.lost = None

    @property
    def tflags(self):
        return capi.UFO_TRACK_FMA if self.flags & FMA else 0

    def particle_element_turns(self):
        return float(np.sum(self.particles * self.turns.astype(np.int64))) * self.n_elements

    def permutation(self, order=None):
        order = order or self.order
        if order == 'lpt':
            return np.argsort(-self.pturns, kind='stable')
        if order == 'seed':
            return np.arange(self.n)
        raise ValueError(f'unknown order {order!r}')

    # ------------------------------------------------------------ device
    def upload(self, order=None):
        """Copy coordinates, seeds and turn counts to the device in launch
        order; drops any captured graph."""
        torch = _torch()
        dev = torch.device('cuda', self.ctx.device)
        perm = self.permutation(order)
        self._perm = perm
        self._order_used = order or self.order
        self._dev = {
            'coords': torch.from_numpy(np.ascontiguousarray(self.coords[perm])).to(dev),
            'seed': torch.from_numpy(np.ascontiguousarray(self.seed[perm])).to(dev),
            'pturns': torch.from_numpy(np.ascontiguousarray(self.pturns[perm])).to(dev),
            'lost': torch.empty(self.n, dtype=torch.int32, device=dev),
            'final': torch.empty((self.n, 6), dtype=torch.float64, device=dev),
        }
        self.destroy_graph()

    def _ptrs(self):
        d = self._dev
        return (capi.ptr(d['coords'].data_ptr()), capi.ptr(d['seed'].data_ptr()),
                capi.ptr(d['pturns'].data_ptr()), capi.ptr(d['final'].data_ptr()),
                capi.ptr(d['lost'].data_ptr()))

    def capture(self):
        """Capture the batched launch into a CUDA graph (ufo_graph_create)."""
        import ctypes
        if self._dev is None:
            self.upload()
        self.destroy_graph()
        co, sd, pt, fi, lo = self._ptrs()
        g = ctypes.c_void_p()
        capi.check(capi.load().ufo_graph_create(
            self.ctx.handle, self.dprog.handle, co, sd, pt, self.n, int(self.turns.max()),
            int(self.mode), self.tflags, 0, 1, None, lo, fi, ctypes.byref(g)))
        self._graph = g

    def launch(self, stream=None, graph=True):
        """Enqueue the batched launch (graph replay, or a direct launch) on
        the CUDA stream handle ``stream`` (None or 0: the context's own
        stream, which does not synchronise with the legacy default stream)."""
        if self._dev is None:
            self.upload()
        lib = capi.load()
        st = capi.ptr(stream) if stream else None
        if graph:
            if self._graph is None:
                self.capture()
            capi.check(lib.ufo_graph_launch(self._graph, st))
        else:
            co, sd, pt, fi, lo = self._ptrs()
            capi.check(lib.ufo_track_device(self.ctx.handle, self.dprog.handle, co, sd, pt,
                                            self.n, int(self.turns.max()), int(self.mode),
                                            self.tflags, 0, 1, None, lo, fi, st))

    def plain_launches(self, stream=None):
        """One launch per seed over that seed's particles (the comparison path)."""
        if self._dev is None or self._order_used != 'seed':
            self.upload('seed')
        lib = capi.load()
        st = capi.ptr(stream) if stream else None
        d = self._dev
        start = 0
        for s, cnt in enumerate(self.particles):
            cnt = int(cnt)
            if cnt == 0:
                continue
            co = capi.ptr(d['coords'].data_ptr() + start * 48)
            sd = capi.ptr(d['seed'].data_ptr() + start * 4)
            fi = capi.ptr(d['final'].data_ptr() + start * 48)
            lo = capi.ptr(d['lost'].data_ptr() + start * 4)
            capi.check(lib.ufo_track_device(self.ctx.handle, self.dprog.handle, co, sd, None, cnt,
                                            int(self.turns[s]), int(self.mode), self.tflags, 0,
                                            1, None, lo, fi, st))
            start += cnt

    def download(self):
        torch = _torch()
        torch.cuda.synchronize()
        final = self._dev['final'].cpu().numpy()
        lost = self._dev['lost'].cpu().numpy().view(np.uint32)
        inv = np.empty_like(self._perm)
        inv[self._perm] = np.arange(self.n)
        self.final = final[inv]
        self.lost = lost[inv]
        return self.final, self.lost

    def run(self, graph=True):
        self.upload()
        self.launch(graph=graph)
        return self.download()

    def run_plain(self):
        self.upload('seed')
        self.plain_launches()
        return self.download()

    def destroy_graph(self):
        if self._graph is not None and capi.alive():
            capi._lib.ufo_graph_destroy(self._graph)
        self._graph = None

    def __del__(self):
        try:
            self.destroy_graph()
        except Exception:  # noqa: BLE001
            pass


# ------------------------------------------------------------------ autotuner

def _cache_path():
    root = os.environ.get('UFO_GB300_CACHE', os.path.join(os.path.expanduser('~'), '.cache',
                                                          'ufo_gb300'))
    return os.path.join(root, 'autotune.json')


def _key(batch):
    torch = _torch()
    h = hashlib.sha1()
    h.update(batch.prog.ops.tobytes())
    h.update(np.sort(batch.pturns).tobytes()[:4096])
    return f'{torch.cuda.get_device_name(batch.ctx.device)}|{batch.n}|{h.hexdigest()[:16]}'


def autotune(batch, warps=(6, 8, 10, 12, 16), orders=('lpt', 'seed'), scale=16, use_cache=True):
    """Choose resident warps per SM and the particle order for ``batch``.

    Candidates are timed with CUDA events on a copy of the workload whose turn
    counts are divided by ``scale``; the winner is applied to the batch's
    context and order and cached (``$UFO_GB300_CACHE/autotune.json``).
    Returns {'warps_per_sm', 'order', 'times_ms'}."""
    torch = _torch()
    key = _key(batch)
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        best = cache[key]
    else:
        saved = batch.pturns
        batch.pturns = np.maximum(1, saved // scale).astype(np.int32)
        times = {}
        # launches and their events on one stream of our own (the library
        # launches on the stream it is given)
        stream = torch.cuda.Stream(torch.device('cuda', batch.ctx.device))
        try:
            with torch.cuda.stream(stream):
                for order in orders:
                    batch.upload(order)
                    for w in warps:
                        batch.ctx.set_tuning(w)
                        batch.launch(stream=stream.cuda_stream, graph=False)  # warm
                        stream.synchronize()
                        e0 = torch.cuda.Event(enable_timing=True)
                        e1 = torch.cuda.Event(enable_timing=True)
                        e0.record(stream)
                        batch.launch(stream=stream.cuda_stream, graph=False)
                        e1.record(stream)
                        stream.synchronize()
                        times[f'{order}/{w}'] = e0.elapsed_time(e1)
        finally:
            batch.pturns = saved
            batch._dev = None
            batch.destroy_graph()
        k = min(times, key=times.get)
        order, w = k.split('/')
        best = {'warps_per_sm': int(w), 'order': order, 'times_ms': times}
        if use_cache:
            cache[key] = best
            try:
                os.makedirs(os.path.dirname(path), exist_ok=True)
                with open(path, 'w') as f:
                    json.dump(cache, f, indent=1)
            except OSError:
                pass
    batch.ctx.set_tuning(best['warps_per_sm'])
    batch.order = best['order']
    return best
