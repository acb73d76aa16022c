"""Build libufo_gb300.so in-tree with nvcc for sm_103a (GB300).

    python -m ufo_gb300.build

The library is plain CUDA C++ behind an ``extern "C"`` ABI (include/ufo_gb300.h);
no PyTorch headers are involved, so it builds in seconds and loads with ctypes.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, 'csrc')
OUT_DIR = os.path.join(HERE, 'lib')
SO = os.path.join(OUT_DIR, 'libufo_gb300.so')
SOURCES = ['ufo_gb300.cu', 'diff.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-shared', '-Xcompiler', '-fPIC',
              '-I', os.path.join(ROOT, 'include')]


def nvcc():
    for cand in (os.environ.get('NVCC'), '/usr/local/cuda/bin/nvcc', 'nvcc'):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return 'nvcc'


def _stale():
    if not os.path.exists(SO):
        return True
    t = os.path.getmtime(SO)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)]
    deps.append(os.path.join(ROOT, 'include', 'ufo_gb300.h'))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    if not force and not _stale():
        return SO
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = SO + f'.{os.getpid()}.tmp'
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, '-o', tmp] + [os.path.join(SRC, s) for s in SOURCES]
    if verbose:
        print(' '.join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, SO)
    return SO


if __name__ == '__main__':
    build(force='--force' in sys.argv, verbose=True,
          extra=['-Xptxas', '-v'] if '--ptxas' in sys.argv else [])
    print(SO)
