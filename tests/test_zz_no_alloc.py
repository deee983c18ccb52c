"""The no-allocation FP64 entry point against the regular one, through the C ABI.

lime_lindblad_rk4_f64_noalloc serves callers that cannot give this library
device memory (a host framework whose pool owns the GPU, a latency-critical
loop where cudaMalloc/cudaFree would synchronise the device, a process with a
fixed device footprint).  It must give the same results as
lime_lindblad_rk4_f64 with a caller-provided workspace, also on a second call
that finds the previous call's data in the shared scratch array.  This file
is collected last so that a failure here leaves every other test already run.
"""
import numpy as np
import pytest

from lime_gb300 import chains

pytestmark = pytest.mark.gpu
RTOL = 1e-10


@pytest.fixture(scope='module')
def lib():
    from lime_gb300 import build, _native
    build.build()
    return _native.require_device()


def _case(n, batch, n_dense, seed):
    rng = np.random.default_rng(seed)
    Hs, Ls = [], []
    for _ in range(batch):
        H, L = chains.uneven_chain(n, rng, n_ops=max(n_dense, 1))
        Hs.append(H)
        Ls.append(L[:n_dense])
    c_ops = [np.stack([Ls[b][k] for b in range(batch)]) for k in range(n_dense)]
    c_ops += chains.dephasing_ops(n, 0.02)
    e = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    return np.stack(Hs), c_ops, [e + e.conj().T, chains.population_ops(n)[1]]


def _run(lib, gen, rho0, e_ops, n_steps, noalloc):
    import torch
    from lime_gb300 import _native as nat, engine
    dev = gen.heff.device
    B, n = gen.P, gen.n
    rho = engine.as_device(np.broadcast_to(rho0, (B, n, n)).copy(), dev)
    Et, n_obs, obs_diag, obs_stride = engine.prepare_obs(e_ops, n, gen.P, dev)
    obs_out = torch.zeros((B, n_steps, n_obs), dtype=torch.complex128, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    d = nat.LindbladDesc()
    d.n, d.batch, d.param_batch, d.n_steps = n, B, B, n_steps
    d.k_dense, d.n_obs, d.obs_diag, d.obs_every = gen.k_dense, n_obs, obs_diag, 1
    d.dt, d.trace_tol = 0.05, 1e-9
    d.rho = rho.data_ptr()
    d.heff, d.heff_stride = gen.heff.data_ptr(), n * n
    if gen.m is not None:
        d.m, d.m_stride = gen.m.data_ptr(), (0 if gen.m.shape[0] == 1 else n * n)
    if gen.l_dense is not None:
        d.l_dense = gen.l_dense.data_ptr()
        d.l_dense_stride = 0 if gen.l_dense.shape[0] == 1 else gen.k_dense * n * n
    d.obs_ops, d.obs_stride, d.obs_out = Et.data_ptr(), obs_stride, obs_out.data_ptr()
    d.status = status.data_ptr()
    stream = torch.cuda.current_stream().cuda_stream
    if noalloc:
        rc = lib.lime_lindblad_rk4_f64_noalloc(d, stream)
    else:
        wsb = lib.lime_lindblad_rk4_f64_workspace(n, B, gen.k_dense)
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        d.workspace, d.workspace_bytes = ws.data_ptr(), wsb
        rc = lib.lime_lindblad_rk4_f64(d, stream)
    assert rc == 0, nat.status_string(rc)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return obs_out.cpu().numpy(), rho.cpu().numpy()


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_noalloc_matches_workspace_entry_point_twice(lib):
    from lime_gb300 import engine
    # first call: dense collapse operators (uses every workspace buffer);
    # second call: another size and no dense operators, so it reads a
    # scratch array that still holds the first call's data
    for n, batch, n_dense, seed in [(12, 3, 2, 11), (20, 2, 0, 12)]:
        H, c_ops, e_ops = _case(n, batch, n_dense, seed)
        gen = engine.LindbladGenerator.build(H, c_ops)
        rho0 = chains.ground_dm(n)
        ref_obs, ref_rho = _run(lib, gen, rho0, e_ops, 30, noalloc=False)
        obs, rho = _run(lib, gen, rho0, e_ops, 30, noalloc=True)
        assert relerr(obs, ref_obs) < RTOL
        assert relerr(rho, ref_rho) < RTOL


def test_noalloc_multi_launch_call_after_a_larger_one(lib):
    """A 60-step call at n = 64 with two dense operators runs as three
    launches (about 25 steps each) whose later launches read the start trace
    the first one left in the scratch array; it follows a call with more
    instances, so every scratch buffer it uses holds stale data first."""
    from lime_gb300 import engine
    H, c_ops, e_ops = _case(64, 4, 2, 21)
    gen = engine.LindbladGenerator.build(H, c_ops)
    _run(lib, gen, chains.ground_dm(64), e_ops, 10, noalloc=True)
    H, c_ops, e_ops = _case(64, 2, 2, 22)
    gen = engine.LindbladGenerator.build(H, c_ops)
    rho0 = chains.ground_dm(64)
    ref_obs, ref_rho = _run(lib, gen, rho0, e_ops, 60, noalloc=False)
    obs, rho = _run(lib, gen, rho0, e_ops, 60, noalloc=True)
    assert relerr(obs, ref_obs) < RTOL
    assert relerr(rho, ref_rho) < RTOL


def test_noalloc_rejects_requests_beyond_the_scratch(lib):
    from lime_gb300 import _native as nat
    cap = lib.lime_noalloc_scratch_bytes()
    assert cap == 16 << 20
    n, batch = 256, 64
    assert lib.lime_lindblad_rk4_f64_workspace(n, batch, 0) > cap
    d = nat.LindbladDesc()
    d.n, d.batch, d.n_steps = n, batch, 1
    before = nat.launch_count()
    assert lib.lime_lindblad_rk4_f64_noalloc(d, None) == -6
    assert nat.launch_count() == before
    assert b'scratch' in lib.lime_status_string(-6)
