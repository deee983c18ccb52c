"""Split-precision tensor-core path vs the FP64 path and the oracle.

Tolerance (stated by the accuracy target of the split path): populations
within 1e-6 absolute of FP64, correlation functions within 1e-6 relative to
max |C_FP64|, over the full 4000-step horizon of the ensemble workload.
"""
import numpy as np
import pytest
import torch

from lime_gb300 import chains

pytestmark = pytest.mark.gpu
POP_TOL = 1e-6
COR_TOL = 1e-6


@pytest.fixture(scope='module', autouse=True)
def _lib():
    from lime_gb300 import build, _native
    build.build()
    _native.require_device()


def _ensemble(n, batch, steps, cfg=2):
    from lime_gb300.engine import DiagonalOps
    w = chains.disorder_ensemble(n=n, batch=batch, n_steps=steps, cfg=cfg)
    l = np.zeros((batch, n, n), dtype=np.complex128)
    idx = np.arange(n)
    l[:, idx, idx] = np.sqrt(w['gamma'])[:, None]
    return w, [DiagonalOps(l)]


def test_ensemble_populations_full_horizon_vs_fp64():
    from lime_gb300 import engine
    n, batch, steps = 64, 16, 4000
    w, c_ops = _ensemble(n, batch, steps)
    gen = engine.LindbladGenerator.build(w['H'], c_ops)
    pops = chains.population_ops(n)
    o64, _, r64 = engine.propagate(gen, w['rho0'], w['dt'], steps, pops, obs_every=10)
    osp, _, rsp = engine.propagate(gen, w['rho0'], w['dt'], steps, pops, obs_every=10,
                                   precision='split')
    assert osp.shape == o64.shape == (batch, steps // 10, n)
    err = (osp - o64).abs().max().item()
    assert err < POP_TOL, err
    # the final state, trace and Hermiticity
    assert (rsp - r64).abs().max().item() < POP_TOL
    # the trace sums n populations whose independent rounding walks add up
    tr = torch.diagonal(rsp, dim1=-2, dim2=-1).sum(-1)
    assert (tr - 1).abs().max().item() < 1e-5
    assert torch.equal(rsp, rsp.mH)


def test_short_run_vs_oracle():
    from oracle import lindblad as ol
    from lime_gb300 import engine
    n, batch, steps = 64, 2, 100
    w, c_ops = _ensemble(n, batch, steps)
    gen = engine.LindbladGenerator.build(w['H'], c_ops)
    pops = chains.population_ops(n)
    osp, _, _ = engine.propagate(gen, w['rho0'], w['dt'], steps, pops, precision='split')
    for b in range(batch):
        ref, _ = ol.lindblad(w['H'][b], w['rho0'], chains.dephasing_ops(n, w['gamma'][b]), pops,
                             Nt=steps, dt=w['dt'], store_states=False)
        assert np.max(np.abs(osp[b].cpu().numpy() - ref)) < POP_TOL


@pytest.mark.parametrize('n', [1, 5, 16, 33, 63])
def test_padded_sizes_vs_fp64(n):
    from lime_gb300 import engine
    w, c_ops = _ensemble(n, 3, 300)
    gen = engine.LindbladGenerator.build(w['H'], c_ops)
    pops = chains.population_ops(n)
    o64, _, r64 = engine.propagate(gen, w['rho0'], w['dt'], 300, pops)
    osp, _, rsp = engine.propagate(gen, w['rho0'], w['dt'], 300, pops, precision='split')
    assert (osp - o64).abs().max().item() < POP_TOL
    assert (rsp - r64).abs().max().item() < POP_TOL


def test_dipole_correlation_vs_fp64():
    """<mu(t) mu(0)> from rho0 = mu|g><g| (non-Hermitian: two Hermitian parts)."""
    from lime_gb300 import engine
    m = chains.absorption_chain(40, chains.rng_for(4, child=77))
    gen = engine.LindbladGenerator.build(m['H'], m['c_ops'])
    rho = m['mu'] @ chains.ground_dm(41)
    o64, _, _ = engine.propagate(gen, rho, 0.05, 2000, [m['mu']])
    osp, _, _ = engine.propagate(gen, rho, 0.05, 2000, [m['mu']], precision='split')
    c64, csp = o64[0, :, 0], osp[0, :, 0]
    rel = ((csp - c64).abs().max() / c64.abs().max()).item()
    assert rel < COR_TOL, rel


def test_public_api_split_precision():
    from lime_gb300.oqs import Lindblad_solver
    w = chains.single_chain(n=16, n_steps=500)
    r64 = Lindblad_solver(w['H'], c_ops=w['c_ops']).evolve(w['rho0'], w['dt'], 500, e_ops=w['e_ops'])
    rsp = Lindblad_solver(w['H'], c_ops=w['c_ops'], precision='split').evolve(
        w['rho0'], w['dt'], 500, e_ops=w['e_ops'], store_states=False)
    assert np.max(np.abs(rsp.observables - r64.observables)) < POP_TOL


def test_split_nonfinite_flag():
    from lime_gb300 import _native, engine
    w, c_ops = _ensemble(8, 2, 10)
    gen = engine.LindbladGenerator.build(w['H'], c_ops)
    rho = np.broadcast_to(w['rho0'], (2, 8, 8)).copy()
    rho[1, 2, 2] = np.inf
    with pytest.raises(_native.KernelFlagError) as ei:
        engine.propagate(gen, rho, 0.05, 5, precision='split')
    assert ei.value.flags & (_native.LIME_FLAG_NONFINITE | _native.LIME_FLAG_TRACE_DRIFT)


def test_device_non_hermitian_start_reruns_as_two_parts():
    """A device-tensor rho0 is checked by the kernel itself: a non-Hermitian
    start raises LIME_FLAG_NOT_HERMITIAN and runs again as its two Hermitian
    parts; the results match the FP64 path (which checks on the device)."""
    from lime_gb300 import engine
    m = chains.absorption_chain(20, chains.rng_for(4, child=5))
    gen = engine.LindbladGenerator.build(m['H'], m['c_ops'])
    rho = torch.as_tensor(m['mu'] @ chains.ground_dm(21), device='cuda')
    o64, _, r64 = engine.propagate(gen, rho, 0.05, 300, [m['mu']])
    osp, _, rsp = engine.propagate(gen, rho, 0.05, 300, [m['mu']], precision='split')
    assert ((osp - o64).abs().max() / o64.abs().max()).item() < COR_TOL
    assert (rsp - r64).abs().max().item() < POP_TOL


def test_hermiticity_flag_and_untouched_input():
    """One perturbed element makes one instance non-Hermitian: the kernel
    flags it; a Hermitian device start is propagated into a new tensor and
    the input is left as it was."""
    from lime_gb300 import _native, engine
    w, c_ops = _ensemble(12, 3, 20)
    gen = engine.LindbladGenerator.build(w['H'], c_ops)
    rho = torch.as_tensor(np.broadcast_to(w['rho0'], (3, 12, 12)).copy(), device='cuda')
    keep = rho.clone()
    o1, _, r1 = engine.propagate(gen, rho, 0.05, 20, chains.population_ops(12), precision='split')
    assert torch.equal(rho, keep) and r1.data_ptr() != rho.data_ptr()
    bad = rho.clone()
    bad[1, 3, 5] += 1e-9
    # the kernel's own verdict on the device tensor
    _, _, st = engine._run_split(gen, bad, 0.05, 20, None, 1, 1e-5, param_batch=3,
                                 rho_out=torch.empty_like(bad))
    assert int(st.item()) & _native.LIME_FLAG_NOT_HERMITIAN
    # the public call reruns the two Hermitian parts
    _, _, r2 = engine.propagate(gen, bad, 0.05, 20, precision='split')
    _, _, r64 = engine.propagate(gen, bad, 0.05, 20)
    assert (r2 - r64).abs().max().item() < POP_TOL


@pytest.mark.parametrize('entries', ['ensemble', 'wide'])
def test_prepared_operand_matches_in_kernel_split(entries):
    """The A operand prepared once per generator (integer conversions) and
    the one split inside the kernel (FP64 instructions) are the same pieces:
    bitwise identical results.  'wide': Hamiltonian entries over 30 decades,
    exact zeros among them, so that the conversions' fallback range (scaled
    entries below 2^-74) is exercised too."""
    from lime_gb300 import _native, engine
    lib = _native.require_device()
    w, c_ops = _ensemble(40, 5, 50)
    if entries == 'wide':
        rng = np.random.default_rng(5)
        a = (rng.normal(size=(5, 40, 40)) + 1j * rng.normal(size=(5, 40, 40))) * \
            10.0 ** rng.uniform(-30, 0, (5, 40, 40))
        a[rng.random((5, 40, 40)) < 0.3] = 0
        w['H'] = 0.1 * (a + np.conj(np.swapaxes(a, 1, 2)))
    gen = engine.LindbladGenerator.build(w['H'], c_ops)
    prep = engine.split_operands(gen)
    rho = torch.as_tensor(np.broadcast_to(w['rho0'], (5, 40, 40)).copy(), device='cuda')
    outs = []
    for use in (True, False):
        out = torch.empty_like(rho)
        obs = torch.empty((5, 50, 40), dtype=torch.complex128, device='cuda')
        st = torch.zeros(1, dtype=torch.int32, device='cuda')
        d = _native.SplitDesc()
        d.n, d.batch, d.param_batch, d.n_steps = 40, 5, 5, 50
        d.obs_mode, d.n_obs, d.obs_every = 1, 40, 1
        d.scale_a_log2, d.auto_scale_b = prep['scale_a'], 1
        d.dt, d.trace_tol = 0.05, 1e-5
        d.rho, d.rho_out = rho.data_ptr(), out.data_ptr()
        d.heff, d.heff_stride = gen.heff.data_ptr(), 40 * 40
        d.m_diag, d.m_stride = prep['m_diag'].data_ptr(), 40
        d.obs_out, d.status = obs.data_ptr(), st.data_ptr()
        if use:
            d.a_pieces, d.a_stride = prep['pieces'].data_ptr(), prep['stride']
        _native.check(lib.lime_lindblad_rk4_split(d, engine._stream_ptr()), 'split')
        assert int(st.item()) == 0
        outs.append((obs, out))
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize('chunk,obs_every', [(7, 3), (40, 40), (1, 1)])
def test_multi_launch_continues_the_state(chunk, obs_every):
    """A call split into several launches (chunk_steps) continues every
    launch from the state the previous one wrote to rho_out: observables
    and final states as in one launch (up to the per-launch state scale)
    and within the bar of the FP64 path.  (A long call of the full ensemble
    is split this way: 4096 realisations x 4000 steps run as 4 launches.)"""
    from lime_gb300 import engine
    n, batch, steps = 24, 6, 120
    w, c_ops = _ensemble(n, batch, steps)
    gen = engine.LindbladGenerator.build(w['H'], c_ops)
    E = chains.population_ops(n)
    o64, _, r64 = engine.propagate(gen, w['rho0'], w['dt'], steps, E, obs_every=obs_every)
    rho = torch.as_tensor(np.stack([w['rho0']] * batch if np.ndim(w['rho0']) == 2 else w['rho0']),
                          device='cuda').contiguous()
    outs = []
    for ck in (0, chunk):
        out = torch.empty_like(rho)
        o, _, status = engine._run_split(gen, rho, w['dt'], steps, E, obs_every, 1e-5, batch, rho_out=out,
                                         chunk_steps=ck)
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        outs.append((o, out))
    (o1, r1), (oc, rc) = outs
    assert (oc - o1).abs().max().item() < 1e-7
    assert (rc - r1).abs().max().item() < 1e-7
    assert (oc - o64).abs().max().item() < POP_TOL
    assert (rc - r64).abs().max().item() < POP_TOL
    # the input is not modified
    assert torch.equal(rho, torch.as_tensor(np.stack([w['rho0']] * batch if np.ndim(w['rho0']) == 2
                                                     else w['rho0']), device='cuda'))
