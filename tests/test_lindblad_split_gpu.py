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
