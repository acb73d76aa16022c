"""Stand-in for the third-party ``pyopencl`` package (unpinned in the reference's
setup.py:13, absent here): just enough of its API for the reference's drivers
(ufo/track.py, ufo/sa.py, ufo/co.py, ufo/optics.py, ufo/cl_utils.py) to run
UNMODIFIED on the host cores.

TEST INFRASTRUCTURE ONLY. Imported by the golden-vector generator and the
reference arm of the CPU baseline; the product path never imports it.

``Program(ctx, src).build()`` prepends a small prelude (``__kernel``, ``__global``,
``uint``, ``get_global_id``, ``atomic_inc``) to the OpenCL C source the
reference generated, compiles it with gcc as plain C under strict IEEE
(``-O2 -ffp-contract=off -fno-fast-math``) and loads it with ctypes.
``kernel.run(queue, (threads,), None, *buffers)`` starts ``threads`` work-items
on an OpenMP team; each work-item runs the reference's kernel body, which
pulls further particles from the shared ``pool_idx`` counter exactly as the
reference's atomic work queue does on an OpenCL device.
"""
import ctypes
import hashlib
import os
import subprocess

import numpy as np

from . import tools, array  # noqa: F401  (the reference imports both)

_HERE = os.path.dirname(os.path.abspath(__file__))
_CACHE = os.environ.get(
    "UFO_REFSHIM_CACHE",
    os.path.join(os.environ.get("TMPDIR", "/tmp"), "ufo_refshim_cache"))

_PRELUDE = r"""
#include <math.h>
#include <omp.h>
#define __kernel
#define __global
typedef unsigned int uint;
static __thread int refshim_gid;
static inline int get_global_id(int dim) { (void)dim; return refshim_gid; }
static inline int atomic_inc(volatile int *p) { return __atomic_fetch_add(p, 1, __ATOMIC_SEQ_CST); }
#line 1 "generated.cl"
"""

_EPILOGUE = r"""
void refshim_launch(int threads, int team, void *a0, void *a1, void *a2) {
    #pragma omp parallel for num_threads(team) schedule(dynamic, 1)
    for (int g = 0; g < threads; ++g) {
        refshim_gid = g;
        run(a0, a1, a2);
    }
}
"""

CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off",
          "-fno-fast-math", "-fopenmp", "-w"]


class mem_flags:
    READ_ONLY = 1
    WRITE_ONLY = 2
    READ_WRITE = 4
    COPY_HOST_PTR = 8


class Device:
    name = "host-cpu (gcc, OpenMP)"


class Platform:
    def get_devices(self):
        return [Device()]


def get_platforms():
    return [Platform()]


class Context:
    def __init__(self, devices=None):
        self.devices = devices


class CommandQueue:
    def __init__(self, ctx):
        self.ctx = ctx


class Buffer:
    def __init__(self, ctx, flags, size=None, hostbuf=None):
        if hostbuf is not None:
            self.data = np.array(hostbuf, copy=True).view(np.uint8).reshape(-1)
        else:
            self.data = np.zeros(int(size), dtype=np.uint8)

    def ptr(self):
        return self.data.ctypes.data_as(ctypes.c_void_p)


def enqueue_copy(queue, dst, src):
    if isinstance(dst, Buffer):
        raw = np.ascontiguousarray(src).view(np.uint8).reshape(-1)
        dst.data[: raw.size] = raw
    else:
        out = dst.view(np.uint8).reshape(-1)
        out[:] = src.data[: out.size]


def _team():
    env = os.environ.get("UFO_REFSHIM_THREADS")
    if env:
        return max(1, int(env))
    return len(os.sched_getaffinity(0))


class _Kernel:
    def __init__(self, lib):
        self._fn = lib.refshim_launch
        self._fn.restype = None
        self._fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                             ctypes.c_void_p, ctypes.c_void_p]

    def __call__(self, queue, global_size, local_size, *buffers):
        return self.run(queue, global_size, local_size, *buffers)

    def run(self, queue, global_size, local_size, *buffers):
        threads = int(global_size[0])
        ptrs = [b.ptr() for b in buffers] + [None] * (3 - len(buffers))
        self._fn(threads, min(threads, _team()), *ptrs)
        return None


class Program:
    def __init__(self, ctx, src):
        self.src = src

    def build(self, options=None):
        full = _PRELUDE + self.src + _EPILOGUE
        key = hashlib.sha256((" ".join(CFLAGS) + full).encode()).hexdigest()[:24]
        os.makedirs(_CACHE, exist_ok=True)
        so = os.path.join(_CACHE, f"k_{key}.so")
        if not os.path.exists(so):
            c = os.path.join(_CACHE, f"k_{key}.c")
            with open(c, "w") as f:
                f.write(full)
            tmp = so + f".{os.getpid()}.tmp"
            subprocess.run(["gcc", *CFLAGS, "-o", tmp, c, "-lm"], check=True)
            os.replace(tmp, so)
        self._lib = ctypes.CDLL(so)
        self.run = _Kernel(self._lib)
        return self
