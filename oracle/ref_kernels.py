"""The reference's own generated tracking kernels, compiled for the host CPU.

TEST INFRASTRUCTURE (CPU baseline and reference arm of bench.py).

``generate(ref_path)`` runs the reference's code generator (its Track class,
ufo/track.py:40-123, through the pyopencl stand-in in oracle/refshim) on the
benchmark lattice and writes the exact OpenCL C it produces, wrapped in the
stand-in's prelude, to ``oracle/_ref/<name>.c``.  That needs the reference's
source tree, so it runs where the reference is mounted; the generated files
are build outputs (git-ignored) that travel with the working tree.
``build_all()`` compiles them with gcc (strict IEEE, OpenMP) on any machine,
and ``RefKernel`` runs one on the host cores over the reference's own atomic
work queue (``pool_idx``), as the reference's pyopencl CPU back-end would.
"""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_ref')
CFLAGS = ['-O2', '-std=gnu11', '-fPIC', '-shared', '-ffp-contract=off', '-fno-fast-math',
          '-fopenmp', '-w']
# the reference's own default build options, -cl-fast-relaxed-math -cl-mad-enable
# (ufo/__init__.py:22), in gcc's terms: contraction and fast math allowed.  A
# speed figure only; parity is held against the strict build above.
CFLAGS_FAST = ['-O3', '-std=gnu11', '-fPIC', '-shared', '-ffast-math', '-ffp-contract=fast',
               '-fopenmp', '-w']

# benchmark samples: (name, workload, particles, turns)
SAMPLES = [('c2_track', 'c2', 16384, 100), ('c1_track', 'c1', 8192, 200)]


def generate(ref_path):
    sys.path.insert(0, HERE)  # the stand-in package oracle/refshim
    sys.path.insert(0, os.path.join(HERE, 'refshim'))
    sys.path.insert(0, ref_path)
    sys.dont_write_bytecode = True
    import ufo
    sys.path.insert(0, os.path.dirname(HERE))
    from ufo_gb300 import workloads as W
    from refshim import pyopencl as shim  # noqa: F401 (the module ufo imported)
    import pyopencl
    os.makedirs(OUT, exist_ok=True)
    for name, wl, n, turns in SAMPLES:
        ring = W.c2_ring(ufo) if wl == 'c2' else W.c1_ring(ufo)
        params = ['x', 'px', 'y', 'py', 'dp']
        tr = ufo.Track(ring, flags=ufo.KICK | ufo.DOUBLE_PRECISION, turns=turns, particles=n,
                       parameters=params, where=[-1])
        src = pyopencl._PRELUDE + tr.src + pyopencl._EPILOGUE
        with open(os.path.join(OUT, f'{name}.c'), 'w') as f:
            f.write(src)
        with open(os.path.join(OUT, f'{name}.json'), 'w') as f:
            json.dump({'workload': wl, 'particles': n, 'turns': turns, 'parameters': params,
                       'elements': len(ring.flatten()), 'count': tr.count}, f)


def _so(name, fast):
    return os.path.join(OUT, f'{name}_fast.so' if fast else f'{name}.so')


def build_all(quiet=False):
    """Compile every generated kernel twice: strict IEEE (the parity build,
    ``<name>.so``) and under the reference's default fast-math options
    (``<name>_fast.so``)."""
    if not os.path.isdir(OUT):
        raise FileNotFoundError('no generated reference kernels (oracle/_ref)')
    jobs = []
    for f in sorted(os.listdir(OUT)):
        if not f.endswith('.c'):
            continue
        src = os.path.join(OUT, f)
        for fast in (False, True):
            so = _so(f[:-2], fast)
            if os.path.exists(so) and os.path.getmtime(so) >= os.path.getmtime(src):
                continue
            tmp = so + f'.{os.getpid()}.tmp'
            cmd = ['gcc', *(CFLAGS_FAST if fast else CFLAGS), '-o', tmp, src, '-lm']
            jobs.append((subprocess.Popen(cmd), tmp, so))
    failed = []
    for proc, tmp, so in jobs:
        if proc.wait() == 0:
            os.replace(tmp, so)
        else:
            failed.append(so)
    if failed:
        raise RuntimeError(f'gcc failed for {failed}')
    built = sorted(os.path.join(OUT, f) for f in os.listdir(OUT) if f.endswith('.so'))
    if not quiet:
        print('\n'.join(built))
    return built


class RefKernel:
    """One generated reference kernel: ``run(pool, threads)`` -> tracks.
    ``fast``: the build under the reference's default fast-math options."""

    def __init__(self, name, fast=False):
        self.name = name
        self.fast = fast
        with open(os.path.join(OUT, f'{name}.json')) as f:
            self.meta = json.load(f)
        so = _so(name, fast)
        if not os.path.exists(so):
            build_all(quiet=True)
        self.lib = ctypes.CDLL(so)
        self.fn = self.lib.refshim_launch
        self.fn.restype = None
        P = ctypes.c_void_p
        self.fn.argtypes = [ctypes.c_int, ctypes.c_int, P, P, P]

    def run(self, pool, threads, work_items=None):
        n, turns, count = self.meta['particles'], self.meta['turns'], self.meta['count']
        pool = np.ascontiguousarray(pool, dtype=np.float64)
        assert pool.shape == (n, len(self.meta['parameters']))
        work_items = work_items or threads
        pool_idx = np.array([work_items], dtype=np.int32)
        tracks = np.zeros((n, count * turns, 6))
        self.fn(work_items, threads, pool.ctypes.data_as(ctypes.c_void_p),
                pool_idx.ctypes.data_as(ctypes.c_void_p), tracks.ctypes.data_as(ctypes.c_void_p))
        return tracks


def available(name):
    return os.path.exists(os.path.join(OUT, f'{name}.c'))


if __name__ == '__main__':
    generate(sys.argv[1] if len(sys.argv) > 1 else os.environ.get('UFO_REFERENCE', ''))
    build_all()
