"""Failure detection of the bounded device-side waits, without a GPU fault.

Every wait of the propagator kernels polls an mbarrier a bounded number of
times; on expiry the kernel reports LIME_FLAG_TIMEOUT in its status word,
releases its tensor memory and returns.  lime_wait_selftest makes such waits
run out on purpose (a barrier that nothing completes; the streaming GEMM
tile with its operand copies withheld) next to controls in which they
complete, and the context must stay usable: a propagation afterwards still
matches the FP64 path.
"""
import numpy as np
import pytest
import torch

from lime_gb300 import chains

pytestmark = pytest.mark.gpu
TIMEOUT = 0x4


@pytest.fixture(scope='module')
def lib():
    from lime_gb300 import build, _native
    build.build()
    return _native.require_device()


def _workspace(lib):
    n = int(lib.lime_wait_selftest_workspace())
    ws = torch.zeros(n, dtype=torch.uint8, device='cuda')
    ws[n - 128 * 4:].view(torch.float32).fill_(1.0)     # the tile's 128 row scales
    return ws


@pytest.mark.parametrize('kind,expected', [(0, TIMEOUT), (1, 0), (2, TIMEOUT), (3, 0)])
def test_wait_expiry_reported(lib, kind, expected):
    ws = _workspace(lib)
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    rc = lib.lime_wait_selftest(kind, 4096, ws.data_ptr(), status.data_ptr(),
                                torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(status.item()) == expected


def test_bad_arguments_rejected(lib):
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.lime_wait_selftest(7, 100, None, status.data_ptr(), stream) < 0
    assert lib.lime_wait_selftest(0, 0, None, status.data_ptr(), stream) < 0
    assert lib.lime_wait_selftest(2, 100, None, status.data_ptr(), stream) < 0
    assert lib.lime_wait_selftest(0, 100, None, None, stream) < 0
    # kind 4 (the extent check) exists only in the bounds-checked build
    assert lib.lime_wait_selftest(4, 100, None, status.data_ptr(), stream) == -2


def test_context_usable_after_expired_waits(lib):
    """Expired waits in both forms, then the batched tensor-core kernel and
    the streaming path still agree with the FP64 path."""
    ws = _workspace(lib)
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    stream = torch.cuda.current_stream().cuda_stream
    for kind in (0, 2, 2, 0):
        assert lib.lime_wait_selftest(kind, 1024, ws.data_ptr(), status.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == TIMEOUT

    from lime_gb300 import engine
    w = chains.single_chain(n=16, n_steps=60)
    gen = engine.LindbladGenerator.build(w['H'], w['c_ops'])
    o64, _, _ = engine.propagate(gen, w['rho0'], w['dt'], w['Nt'], w['e_ops'])
    osp, _, _ = engine.propagate(gen, w['rho0'], w['dt'], w['Nt'], w['e_ops'], precision='split')
    assert np.max(np.abs(osp.cpu().numpy() - o64.cpu().numpy())) < 1e-6

    H, c_ops = chains.uneven_chain(12, np.random.default_rng(5), n_ops=2)
    gen = engine.LindbladGenerator.build(H, c_ops)
    e = chains.population_ops(12)[:2]
    o64, _, _ = engine.propagate(gen, chains.ground_dm(12), 0.05, 40, e)
    osp, _, _ = engine.propagate(gen, chains.ground_dm(12), 0.05, 40, e, precision='split')
    assert np.max(np.abs(osp.cpu().numpy() - o64.cpu().numpy())) < 1e-6
