"""ctypes binding of libufo_gb300.so (include/ufo_gb300.h).

The library is required: there is no CPU fallback.  If it is missing or fails
to load, every GPU entry point raises ``RuntimeError``.
"""
import atexit
import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, 'lib', 'libufo_gb300.so')

UFO_MODE_TRACK, UFO_MODE_SA = 0, 1
UFO_TRACK_FMA, UFO_TRACK_FIVED, UFO_TRACK_PLAIN, UFO_TRACK_COMPACT = 1, 2, 4, 8

_lib = None
_lock = threading.Lock()
_exiting = False  # set at interpreter exit: destructors then leave teardown to the CUDA driver


def _mark_exit():
    global _exiting
    _exiting = True


atexit.register(_mark_exit)


def alive():
    """True while native handles may still be released."""
    return _lib is not None and not _exiting

P = ctypes.c_void_p
I32, I64, D = ctypes.c_int32, ctypes.c_int64, ctypes.c_double

# name -> argtypes (all return int status unless listed in _VOID)
SIGNATURES = {
    'ufo_last_error': [],
    'ufo_device_count': [P],
    'ufo_ctx_create': [ctypes.c_int, P],
    'ufo_ctx_destroy': [P],
    'ufo_prog_create': [P, P, ctypes.c_int, P, I64, ctypes.c_int, ctypes.c_int, P],
    'ufo_prog_set_table': [P, P, ctypes.c_int],
    'ufo_prog_destroy': [P],
    'ufo_track': [P, P, P, P, P, I64, ctypes.c_int, ctypes.c_int, ctypes.c_int, I64, ctypes.c_int,
                  P, P, P],
    'ufo_track_device': [P, P, P, P, P, I64, ctypes.c_int, ctypes.c_int, ctypes.c_int, I64,
                         ctypes.c_int, P, P, P, P],
    'ufo_launch_count': [P, P],
    'ufo_fp64_peak': [P, P],
    'ufo_fp64_probe': [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P],
    'ufo_ctx_set_tuning': [P, ctypes.c_int],
    'ufo_closed_orbit': [P, P, P, P, I64, ctypes.c_int, P],
    'ufo_graph_create': [P, P, P, P, P, I64, ctypes.c_int, ctypes.c_int, ctypes.c_int, I64,
                         ctypes.c_int, P, P, P, P],
    'ufo_graph_launch': [P, P],
    'ufo_graph_destroy': [P],
    'ufo_diff_forward': [P, ctypes.c_int, P, I64, P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                         P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P],
    'ufo_diff_reverse': [P, ctypes.c_int, P, I64, P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                         P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, P, ctypes.c_int,
                         P, P, P],
    'ufo_track_noalloc': [P, ctypes.c_int, P, I64, ctypes.c_int, ctypes.c_int, P, P, P, I64,
                          ctypes.c_int, ctypes.c_int, ctypes.c_int, I64, ctypes.c_int, P, P, P,
                          P],
}
_VOID = {'ufo_ctx_destroy', 'ufo_prog_destroy', 'ufo_graph_destroy'}


def load(path=None):
    """Load the library (building it first when the sources are newer)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or SO
        if not os.path.exists(path):
            try:
                from . import build
                build.build()
            except Exception as exc:  # noqa: BLE001
                raise RuntimeError(f'libufo_gb300.so is missing and could not be built: {exc}')
        lib = ctypes.CDLL(path)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            if name == 'ufo_last_error':
                fn.restype = ctypes.c_char_p
            elif name in _VOID:
                fn.restype = None
            else:
                fn.restype = ctypes.c_int
        _lib = lib
        return lib


def check(rc):
    if rc != 0:
        msg = load().ufo_last_error().decode(errors='replace')
        raise RuntimeError(f'libufo_gb300 error {rc}: {msg}')


def ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return ctypes.c_void_p(a)
    return a.ctypes.data_as(ctypes.c_void_p)


class Context:
    """A CUDA device + stream (the reference's OpenCL context and queue)."""

    def __init__(self, device=0):
        lib = load()
        h = ctypes.c_void_p()
        check(lib.ufo_ctx_create(int(device), ctypes.byref(h)))
        self.handle = h
        self.device = device

    warps_per_sm = 16  # resident warps per SM of the persistent grid (library default)

    def set_tuning(self, warps_per_sm):
        """ufo_ctx_set_tuning, remembered so that callers can restore it."""
        check(load().ufo_ctx_set_tuning(self.handle, int(warps_per_sm)))
        self.warps_per_sm = int(warps_per_sm)

    def launches(self):
        n = ctypes.c_int64()
        check(load().ufo_launch_count(self.handle, ctypes.byref(n)))
        return n.value

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h and alive():
            _lib.ufo_ctx_destroy(h)
            self.handle = None


class DeviceProgram:
    """A compiled line uploaded to the device."""

    def __init__(self, ctx, prog):
        lib = load()
        self.ctx = ctx
        ops = np.ascontiguousarray(prog.ops, dtype=np.int32)
        table = np.ascontiguousarray(prog.table, dtype=np.float64)
        h = ctypes.c_void_p()
        check(lib.ufo_prog_create(ctx.handle, ptr(ops), ops.shape[0], ptr(table), table.shape[1],
                                  table.shape[0], int(prog.n_dumps), ctypes.byref(h)))
        self.handle = h
        self.n_seeds = table.shape[0]
        self.stride = table.shape[1]

    def set_table(self, table):
        table = np.ascontiguousarray(table, dtype=np.float64)
        if table.shape[1] != self.stride:
            raise ValueError('table stride changed')
        check(load().ufo_prog_set_table(self.handle, ptr(table), table.shape[0]))

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h and alive():
            _lib.ufo_prog_destroy(h)
            self.handle = None


def track(ctx, dprog, coords, turns, mode=UFO_MODE_TRACK, flags=0, seed=None, pturns=None,
          slots=0, every=1, want_tracks=True, want_final=True):
    """Host-buffer tracking through ufo_track.  Returns (tracks, lost, final)."""
    lib = load()
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    n = coords.shape[0]
    seed = None if seed is None else np.ascontiguousarray(seed, dtype=np.int32)
    pturns = None if pturns is None else np.ascontiguousarray(pturns, dtype=np.int32)
    tracks = np.empty((n, slots, 6), dtype=np.float64) if (want_tracks and slots) else None
    lost = np.empty(n, dtype=np.uint32)
    final = np.empty((n, 6), dtype=np.float64) if want_final else None
    check(lib.ufo_track(ctx.handle, dprog.handle, ptr(coords), ptr(seed), ptr(pturns), n,
                        int(turns), int(mode), int(flags), int(slots if tracks is not None else 0),
                        int(every), ptr(tracks), ptr(lost), ptr(final)))
    return tracks, lost, final
