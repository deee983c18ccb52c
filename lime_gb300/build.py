"""Build the in-tree CUDA library ``lime_gb300/liblime_gb300.so`` for sm_103a.

Every ``csrc/*.cu`` translation unit is compiled in parallel with nvcc to an
object file under ``lime_gb300/_build/`` and linked into one shared library
(static CUDA runtime, no torch dependency).  Rebuilds only what changed.

``build(check=True)`` builds the bounds-checked variant
``lime_gb300/liblime_gb300_check.so`` (``-DLIME_CHECK``, objects under
``lime_gb300/_build_check/``): the same kernels with index checks that raise
LIME_FLAG_BOUNDS and skip the access instead of touching memory outside a
buffer.  Load it instead of the regular library by setting
``LIME_GB300_LIBRARY`` to its path before the first call.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'liblime_gb300.so')
BUILD_CHECK = os.path.join(HERE, '_build_check')
LIB_CHECK = os.path.join(HERE, 'liblime_gb300_check.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2',
         '--expt-relaxed-constexpr', '-I' + os.path.join(ROOT, 'include')]


def nvcc() -> str:
    cand = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(cand):
        raise RuntimeError('nvcc not found; the CUDA 13 toolkit is required to build lime_gb300')
    return cand


def _deps(src):
    hdrs = glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(ROOT, 'include', '*.h'))
    return [src] + hdrs


def _compile(src, verbose=False, check=False):
    obj = os.path.join(BUILD_CHECK if check else BUILD, os.path.basename(src) + '.o')
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(p) for p in _deps(src)):
        return obj, False
    cmd = [nvcc()] + ARCH + FLAGS + (['-DLIME_CHECK'] if check else []) + ['-c', src, '-o', obj]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, r.stdout, r.stderr))
    if verbose:
        sys.stderr.write(r.stderr)
    return obj, True


def build(verbose: bool = False, force: bool = False, check: bool = False) -> str:
    bdir, lib = (BUILD_CHECK, LIB_CHECK) if check else (BUILD, LIB)
    os.makedirs(bdir, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    if force:
        for o in glob.glob(os.path.join(bdir, '*.o')):
            os.remove(o)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, check), srcs))
    objs = [o for o, _ in results]
    changed = any(c for _, c in results)
    if changed or not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        tmp = lib + '.tmp'
        cmd = [nvcc()] + ARCH + ['-shared', '-Xcompiler', '-fPIC', '-o', tmp] + objs + ['-lcuda']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('link failed:\n%s\n%s' % (r.stdout, r.stderr))
        os.replace(tmp, lib)
    return lib


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv, force='-f' in sys.argv, check='--check' in sys.argv))
