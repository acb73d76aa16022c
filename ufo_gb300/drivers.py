"""Simulation drivers with the reference's class API, running on the GPU.

``Track``, ``StableAperture``, ``ClosedOrbit`` and ``Optics`` keep the
reference's constructor signatures, attributes (``parameters``, ``tracks``,
``lost``, ``orbits``, ``track``, ``bx``...), ``run(threads)`` and error
behaviour (ufo/track.py:40-139, ufo/sa.py:37-145, ufo/co.py:146-250,
ufo/optics.py:44-238).  Instead of generating and building an OpenCL kernel
in ``__init__`` they snapshot the line (element values are frozen at
construction, as the reference's literals were) and in ``run()`` lower it
with the current parameter values and call libufo_gb300.

Arithmetic is FP64 whatever the flags say; DOUBLE_PRECISION only selects the
dtype of ``parameters`` and of the outputs, as in the reference.  ``threads``
is accepted and ignored: the kernels size their own grid.
"""
import copy

import numpy as np

from . import capi
from . import compiler as C
from . import twiss as _twiss
from .flags import FIVED, DOUBLE_PRECISION, LINEAR, ACHROMATIC, FMA, KICK

COORDS = ('x', 'px', 'y', 'py', 'z', 'dp')

_default_ctx = {}


class Context(capi.Context):
    """CUDA device handle; the reference's ``ufo.context(device)``."""


def context(device=0):
    """Return the (shared) context of ``device``."""
    if device not in _default_ctx:
        _default_ctx[device] = Context(device)
    return _default_ctx[device]


def list_devices(device=None):
    """Print the CUDA devices, or return the id of ``device`` if given."""
    import ctypes
    lib = capi.load()
    n = ctypes.c_int()
    capi.check(lib.ufo_device_count(ctypes.byref(n)))
    if device is not None:
        if not 0 <= device < n.value:
            raise ValueError(f'no CUDA device {device}')
        return device
    for i in range(n.value):
        print(f'{i}:   CUDA device {i}')
    return None


def _ufloat(flags):
    return np.float64 if flags & DOUBLE_PRECISION else np.float32


def _snapshot(line):
    """Frozen copy of the flattened line (the reference bakes element values
    into its kernel at construction time)."""
    from .lattice import Line
    flat = line.flatten() if hasattr(line, 'flatten') else list(line)
    return Line(getattr(line, 'label', 'line'), [copy.deepcopy(e) for e in flat])


def _lattice_columns(parameters):
    return [i for i, p in enumerate(parameters) if not (isinstance(p, str) and p in COORDS)]


class _Compiled:
    """Lowers the frozen line per run; re-uploads only what changed."""

    def __init__(self, line, flags, parameters, where, count=None, dump_end=None):
        self.line = line
        self.flags = flags
        self.parameters = list(parameters)
        self.where = list(where)
        self.count = count
        self.dump_end = dump_end
        self.lat_cols = _lattice_columns(self.parameters)
        self._key = None
        self._dprog = None
        self._ops = None
        self.prog = None
        # compile once with zeros so that lowering errors surface in __init__
        self.prog = C.compile_line(line, flags, self.parameters, self.where,
                                   count=count, dump_end=dump_end)

    def seeds(self, pool):
        """Distinct lattice-parameter rows -> (seed_values, seed index per row)."""
        n = pool.shape[0]
        width = max(len(self.parameters), 1)
        if not self.lat_cols:
            return np.zeros((1, width)), None
        lat = np.ascontiguousarray(pool[:, self.lat_cols], dtype=np.float64)
        uniq, inv = np.unique(lat, axis=0, return_inverse=True)
        vals = np.zeros((uniq.shape[0], width))
        vals[:, self.lat_cols] = uniq
        inv = inv.reshape(n).astype(np.int32)
        if uniq.shape[0] == 1:
            return vals, None
        return vals, inv

    def device(self, ctx, seed_values):
        key = seed_values.tobytes()
        if self._dprog is not None and key == self._key:
            return self._dprog
        prog = C.compile_line(self.line, self.flags, self.parameters, self.where, seed_values,
                              count=self.count, dump_end=self.dump_end)
        if self._dprog is not None and self._ops is not None and \
                np.array_equal(prog.ops, self._ops) and \
                prog.table.shape == (self._dprog.n_seeds, self._dprog.stride):
            self._dprog.set_table(prog.table)
        else:
            self._dprog = capi.DeviceProgram(ctx, prog)
            self._ops = prog.ops.copy()
        self.prog = prog
        self._key = key
        return self._dprog


def _no_turn(prog, what):
    """The reference's closed-orbit and optics kernels declare no ``turn``
    (ufo/co.py:146-250, ufo/optics.py:87-154): element text that reads it fails
    their OpenCL build, and fails here the same way."""
    if C.reads_turn(prog):
        raise RuntimeError(f'an aperture window or element strength reads `turn`, which the '
                           f'{what} kernel does not define')


def _coords_from_pool(pool, parameters, flags, dp):
    n = pool.shape[0]
    coords = np.zeros((n, 6))
    for j, c in enumerate(COORDS):
        if c in parameters:
            coords[:, j] = pool[:, parameters.index(c)]
    if flags & FIVED:
        coords[:, 4] = 0.0
        coords[:, 5] = dp
    return coords


def _track_flags(flags):
    f = 0
    if flags & FMA:
        f |= capi.UFO_TRACK_FMA
    if flags & FIVED:
        f |= capi.UFO_TRACK_FIVED
    return f


class Track:
    """Track a bunch through a ring, sampling coordinates at ``where`` every
    turn (ufo/track.py:19-139).  Extensions: ``every`` samples only on every
    ``every``-th turn (for long runs whose full record would not fit in host
    memory); after ``run()``, ``lost`` holds the turn at which each particle
    was lost (``turns`` if it survived) and ``final`` the last coordinates."""

    def __init__(self, line, flags=0x00, turns=1000, particles=1000, parameters=None, where=None,
                 dp=0., context=None, options=None, every=1):
        parameters = list(parameters) if parameters is not None else []
        where = where if where is not None else []
        where = where if type(where) is list else [where]
        self.turns = turns
        self.ctx = context if context is not None else globals()['context'](0)
        self.flags = flags
        self.dp = dp
        self.every = max(1, int(every))
        ufloat = _ufloat(flags)
        self.pool_idx = np.empty(1, np.int32)
        self.parameters = np.zeros([particles, len(parameters)], dtype=ufloat)
        self._names = parameters
        self.count = len(where)
        flat = line.flatten()
        self.where = [(idx, flat[int(idx)]) for idx in where]
        count = self.count * (turns // self.every)
        if count < 1:
            raise Exception("No valid observation points found in 'where'")
        self._line = _snapshot(line)
        self._c = _Compiled(self._line, flags, parameters, list(where))
        self.tracks = np.zeros([particles, count, 6], dtype=ufloat)
        self.lost = np.zeros(particles, dtype=np.uint32)
        self.final = np.zeros([particles, 6], dtype=ufloat)
        self.src = self._c.prog.describe()

    @property
    def program(self):
        return self._c.prog

    def run(self, threads=1):
        """Track (synchronous).  ``threads`` is ignored."""
        pool = np.asarray(self.parameters, dtype=np.float64)
        seed_values, seed = self._c.seeds(pool)
        dprog = self._c.device(self.ctx, seed_values)
        coords = _coords_from_pool(pool, self._names, self.flags, self.dp)
        slots = self.tracks.shape[1]
        tracks, lost, final = capi.track(self.ctx, dprog, coords, self.turns,
                                         capi.UFO_MODE_TRACK, _track_flags(self.flags),
                                         seed=seed, slots=slots, every=self.every)
        self.tracks = tracks.astype(self.tracks.dtype, copy=False)
        self.lost = lost
        self.final = final.astype(self.final.dtype, copy=False)


def _sm_count(device):
    import torch
    return torch.cuda.get_device_properties(device).multi_processor_count


class StableAperture:
    """Turns survived per particle (ufo/sa.py:18-145): lost at the end of the
    first turn with |x| > 1 or |y| > 1 or isnan(x); ``lost`` holds that turn,
    or ``turns`` for survivors."""

    def __init__(self, line, flags=0x00, turns=1000, particles=1000, parameters=None, dp=0.,
                 context=None, options=None):
        parameters = list(parameters) if parameters is not None else []
        self.turns = turns
        self.ctx = context if context is not None else globals()['context'](0)
        self.flags = flags
        self.dp = dp
        ufloat = _ufloat(flags)
        self.pool_idx = np.empty(1, np.int32)
        self.parameters = np.zeros([particles, max(1, len(parameters))], dtype=ufloat)
        self._names = parameters
        self.lost = np.empty(particles, dtype=np.uint32)
        self._line = _snapshot(line)
        self._c = _Compiled(self._line, flags, parameters, [])
        self.src = self._c.prog.describe()

    @property
    def program(self):
        return self._c.prog

    def _uses_turn(self):
        """An aperture window or a time-dependent element reads ``turn``: the
        particles' turn numbers must then not restart."""
        return C.reads_turn(self._c.prog)

    # resident warps per SM of the compacting kernel for a scan: measured
    # best on the 196,608-particle dynamic-aperture grid with the CTAs
    # exchanging particles (16: 8.1e9, 8: 7.8e9 particle*element*turns/s)
    COMPACT_WARPS_PER_SM = 16

    def run(self, threads=1, compact=None):
        """``compact='two-phase'`` (the default, ``compact=None``, for lattices
        that do not read ``turn``): track the first turns/8 with the full
        persistent grid, then relaunch only the survivors on a grid sized to
        them, whose warps run free of one another.  ``compact=True`` (the
        default for lattices that read ``turn``, which a second phase would
        renumber): one launch of the CTA-compacting persistent kernel; once
        every particle has been handed out, each CTA packs its survivors into
        its lowest warps at every turn and the CTAs even out their particle
        counts through a pool, so the long-lived particles of an uneven scan
        fill whole warps on every SM.  ``compact=False``: one launch of the
        one-warp persistent kernel.  Loss turns and coordinates are the same
        in every case."""
        pool = np.asarray(self.parameters, dtype=np.float64)
        seed_values, seed = self._c.seeds(pool)
        dprog = self._c.device(self.ctx, seed_values)
        coords = _coords_from_pool(pool, self._names, self.flags, self.dp)
        T, n = int(self.turns), coords.shape[0]
        if compact is None:
            compact = 'two-phase'
        if compact == 'two-phase' and self._uses_turn():
            compact = True
        flags = _track_flags(self.flags)
        if compact is True:
            before = self.ctx.warps_per_sm
            self.ctx.set_tuning(self.COMPACT_WARPS_PER_SM)
            try:
                _, lost, final = capi.track(self.ctx, dprog, coords, T, capi.UFO_MODE_SA,
                                            flags | capi.UFO_TRACK_COMPACT, seed=seed, slots=0)
            finally:
                self.ctx.set_tuning(before)
            self.lost = lost
            self.final = final
            return
        if not compact:
            _, lost, final = capi.track(self.ctx, dprog, coords, T, capi.UFO_MODE_SA, flags,
                                        seed=seed, slots=0)
            self.lost = lost
            self.final = final
            return
        T1 = max(1, T // 8)
        _, lost, final = capi.track(self.ctx, dprog, coords, T1, capi.UFO_MODE_SA, flags,
                                    seed=seed, slots=0)
        alive = np.nonzero(lost >= T1)[0]
        self.survivors_after_first_phase = len(alive)
        if len(alive) and T > T1:
            sms = _sm_count(self.ctx.device)
            warps = int(min(16, max(2, round(len(alive) / (0.9 * 32 * sms)))))
            self.second_phase_warps_per_sm = warps
            before = self.ctx.warps_per_sm
            self.ctx.set_tuning(warps)
            try:
                _, lost2, final2 = capi.track(
                    self.ctx, dprog, np.ascontiguousarray(final[alive]), T - T1,
                    capi.UFO_MODE_SA, flags,
                    seed=None if seed is None else np.ascontiguousarray(seed[alive]), slots=0)
            finally:
                self.ctx.set_tuning(before)
            lost = lost.copy()
            lost[alive] = T1 + lost2
            final = final.copy()
            final[alive] = final2
        self.lost = lost
        self.final = final


class ClosedOrbit:
    """Closed orbits (x, px, y, py) of the 4D one-turn map at dp = 0
    (ufo/co.py:146-250).

    method='amoeba' (default): the reference's own search, ``iterations``
    Nelder-Mead steps on the squared one-turn residual, run on the GPU in the
    reference's operation order: the orbits are the reference's, bit for bit
    (ufo_closed_orbit).  method='newton': F(z) = z solved by Newton iteration
    with the Jacobian of the tangent map, until the step stops shrinking (at
    most ``iterations`` steps): the exact fixed point, to rounding."""

    def __init__(self, line, flags=0x00, particles=1000, parameters=None, dp=0., iterations=200,
                 context=None, options=None, method='amoeba'):
        if method not in ('amoeba', 'newton'):
            raise ValueError(f'unknown closed-orbit method {method!r}')
        self.method = method
        parameters = list(parameters) if parameters is not None else []
        self.ctx = context if context is not None else globals()['context'](0)
        self.flags = flags
        self.iterations = iterations
        ufloat = _ufloat(flags)
        self.pool_idx = np.empty(1, np.int32)
        self.parameters = np.zeros([particles, max(1, len(parameters))], dtype=ufloat)
        self._names = parameters
        self.orbits = np.zeros([particles, 4], dtype=ufloat)
        self._line = _snapshot(line)
        # dp = 0, oodppo = 1, z = 0 are forced by the reference (ufo/co.py:182-184)
        self._c = _Compiled(self._line, flags & ~FIVED, parameters, [])
        _no_turn(self._c.prog, 'closed-orbit')
        self.src = self._c.prog.describe()

    def run(self, threads=1):
        from . import newton_fd
        pool = np.asarray(self.parameters, dtype=np.float64)
        seed_values, seed = self._c.seeds(pool)
        dprog = self._c.device(self.ctx, seed_values)
        guess = np.zeros((pool.shape[0], 4))
        for j, c in enumerate(COORDS[:4]):
            if c in self._names:
                guess[:, j] = pool[:, self._names.index(c)]
        if self.method == 'amoeba':
            orbits = np.empty_like(guess)
            sd = np.ascontiguousarray(seed, dtype=np.int32) if seed is not None else None
            capi.check(capi.load().ufo_closed_orbit(
                self.ctx.handle, dprog.handle, capi.ptr(np.ascontiguousarray(guess)),
                capi.ptr(sd) if sd is not None else None, guess.shape[0], int(self.iterations),
                capi.ptr(orbits)))
            self.residual = None
        else:
            orbits, self.residual = newton_fd.closed_orbit(self.ctx, dprog, guess, seed=seed,
                                                         fma=bool(self.flags & FMA),
                                                         max_iter=self.iterations)
        self.orbits = orbits.astype(self.orbits.dtype, copy=False)


class Optics:
    """Periodic (or propagated) Twiss functions from the one-turn and partial
    maps (ufo/optics.py:21-238): three unit particles (x=y=1), (px=py=1),
    (dp=1) are tracked once with observations at ``where``; with the default
    LINEAR | ACHROMATIC flags the map is linear so the tracks are the map's
    columns.  Results: ``qx, qy, bx, by, ax, ay, dx, dpx, dy, dpy, mux, muy``."""

    def __init__(self, line, where=None, periodic=True, parameters=None, flags=LINEAR | ACHROMATIC,
                 context=None, options=None):
        parameters = list(parameters) if parameters is not None else []
        where = list(where) if where is not None else []
        where = where if type(where) is list else [where]
        self.ctx = context if context is not None else globals()['context'](0)
        self.periodic = periodic
        self.flags = flags
        if periodic and -1 not in where and line[-1] not in where:
            where.append(-1)
        self.parameters = np.zeros([1, max(1, len(parameters))], dtype=_ufloat(flags))
        self._names = parameters
        self.count = len(where) - 1
        if -1 in where:
            self.count += 1
        flat = line.flatten()
        self.where = [(idx, flat[int(idx)]) for idx in where]
        if self.count < 1:
            raise Exception("No valid observation points found in 'where'")
        self._line = _snapshot(line)
        self._c = _Compiled(self._line, flags, parameters, where, count=self.count)
        _no_turn(self._c.prog, 'optics')
        self.track = np.zeros([3, self.count, 6], dtype=_ufloat(flags))
        self.src = self._c.prog.describe()
        self.ax0 = self.bx0 = self.dx0 = self.dpx0 = 0.
        self.ay0 = self.by0 = self.dy0 = self.dpy0 = 0.
        for a in ('ax', 'ay', 'bx', 'by', 'dx', 'dy', 'dpx', 'dpy', 'mux', 'muy'):
            setattr(self, a, np.empty(self.count))

    def run(self, threads=3):
        pool = np.asarray(self.parameters, dtype=np.float64)
        seed_values, _ = self._c.seeds(pool[:1])
        dprog = self._c.device(self.ctx, seed_values)
        coords = np.zeros((3, 6))
        coords[0, 0] = coords[0, 2] = 1.0
        coords[1, 1] = coords[1, 3] = 1.0
        coords[2, 5] = 1.0
        if 'dp' in self._names:
            coords[:, 5] += pool[0, self._names.index('dp')]
        tracks, _, _ = capi.track(self.ctx, dprog, coords, 1, capi.UFO_MODE_TRACK,
                                  _track_flags(self.flags & ~FIVED), slots=self.count)
        tracks[:, :, 4:] = 0.0  # the reference's optics kernel dumps only x..py
        self.track = tracks.astype(self.track.dtype, copy=False)
        twiss(self)


def twiss(o):
    """Twiss, tunes and dispersion of an Optics object from its unit tracks
    (ufo_gb300/twiss.py)."""
    _twiss.twiss(o)


def chromaticity(optics):
    """Analytic natural and total linear chromaticity from Twiss at the
    elements' entrances (the reference's ufo/chroma.py:11-52; computed in
    ufo_gb300/twiss.py).  Returns ((dqx0, dqy0), (dqx, dqy))."""
    return _twiss.chromaticity(optics)
