"""The bounds-checked build (liblime_gb300_check.so, compiled with
-DLIME_CHECK): the same kernels, with the tile, piece and instance offsets
of their global and operand accesses checked against the extents of their
buffers.  A failed check raises LIME_FLAG_BOUNDS and skips the access (no
trap), so a propagation that passes through it without a flag has kept
every checked access inside its buffer.

Run on small shapes that exercise padding and tile edges (tests/
bounds_cases.py) in a child process that loads the checked build; every
call must finish without a flag and give the regular build's results (to
1e-12: the Redfield observable pass and the adjoint gradients add partial
sums with atomics, in varying order).  The check itself is shown to fire by
lime_wait_selftest kind 4: a tile told that its operand is one piece short
refuses the copy and reports LIME_FLAG_BOUNDS."""
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from conftest import ROOT

pytestmark = pytest.mark.gpu
BOUNDS, TIMEOUT = 0x20, 0x4


@pytest.fixture(scope='module')
def check_lib():
    from lime_gb300 import build
    build.build()
    return build.build(check=True)


def test_checked_build_matches_regular_without_flags(check_lib, tmp_path):
    from lime_gb300 import _native
    _native.require_device()
    sys.path.insert(0, os.path.join(ROOT, 'tests'))
    import bounds_cases
    ref = bounds_cases.run_all()
    path = tmp_path / 'checked.npz'
    env = dict(os.environ, LIME_GB300_LIBRARY=check_lib)
    r = subprocess.run([sys.executable, os.path.join(ROOT, 'tests', 'bounds_cases.py'), str(path)],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]   # any LIME_FLAG_BOUNDS raises in the child
    got = np.load(path)
    for k, v in ref.items():
        for i, x in enumerate(v):
            if x is None:
                continue
            y = got['%s__%d' % (k, i)]
            scale = max(float(np.max(np.abs(x))), 1e-300) if x.size else 1.0
            assert x.shape == y.shape, k
            assert float(np.max(np.abs(x - y))) <= 1e-12 * scale, k


def test_extent_check_fires(check_lib):
    """Kind 4 in the checked build refuses the short operand copy and flags
    it; the regular build does not offer kind 4."""
    from lime_gb300 import _native
    lib = _native.require_device()
    n = int(lib.lime_wait_selftest_workspace())
    ws = torch.zeros(n, dtype=torch.uint8, device='cuda')
    ws[n - 128 * 4:].view(torch.float32).fill_(1.0)
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    assert lib.lime_wait_selftest(4, 4096, ws.data_ptr(), status.data_ptr(),
                                  torch.cuda.current_stream().cuda_stream) == -2
    code = ('import torch, ctypes, sys\n'
            'from lime_gb300 import _native as nat\n'
            'lib = nat.require_device()\n'
            'n = int(lib.lime_wait_selftest_workspace())\n'
            'ws = torch.zeros(n, dtype=torch.uint8, device="cuda")\n'
            'ws[n - 512:].view(torch.float32).fill_(1.0)\n'
            'out = []\n'
            'for kind in (4, 3):\n'
            '    st = torch.zeros(1, dtype=torch.int32, device="cuda")\n'
            '    assert lib.lime_wait_selftest(kind, 4096, ws.data_ptr(), st.data_ptr(), '
            'torch.cuda.current_stream().cuda_stream) == 0\n'
            '    torch.cuda.synchronize()\n'
            '    out.append(int(st.item()))\n'
            'print(out[0], out[1])\n')
    env = dict(os.environ, LIME_GB300_LIBRARY=check_lib)
    r = subprocess.run([sys.executable, '-c', code], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    flags4, flags3 = (int(x) for x in r.stdout.split()[-2:])
    assert flags4 & BOUNDS and flags4 & TIMEOUT
    assert flags3 == 0
