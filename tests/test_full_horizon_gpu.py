"""Split-precision error against FP64 over the full horizons of the
configured workloads (a few instances each; the ensemble workload's
4000-step check is in test_lindblad_split_gpu.py):

* uneven batch: one chain of every N in {8, 16, 32, 64, 128, 256} (and a
  block-diagonal pack of two N = 8 chains), 3 dense collapse operators,
  2000 steps, through the public uneven-batch call;
* differentiated absorption shape: the dipole correlation <mu(t) mu(0)> of
  two 129-dimensional chains over 4096 steps;
* dense Redfield superoperator: N = 96 (Liouville dimension 9216), two
  right-hand sides, all 96 populations over 2000 steps.

Bars (the split path's stated accuracy): populations within 1e-6 absolute,
correlations within 1e-6 of max |C| (relative).  The FP64 side is the
PyTorch FP64 RK4 of tests/fp64_torch.py (whole-GPU cuBLAS calls), anchored
here to the library's FP64 kernels on a short horizon at 1e-12.
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


def _fp64():
    import fp64_torch
    return fp64_torch


def test_uneven_batch_every_size_2000_steps():
    from lime_gb300 import engine
    sizes = (8, 8, 16, 32, 64, 128, 256)          # two N = 8 chains share a packed instance
    rng = np.random.default_rng(20261203 + 3)
    H, C, R0, E = [], [], [], []
    for n in sizes:
        h, c = chains.uneven_chain(n, rng)
        H.append(h)
        C.append(c)
        R0.append(chains.ground_dm(n))
        E.append(chains.population_ops(n)[:4])
    steps = 2000
    osp, _, rsp = engine.propagate_ragged(H, R0, 0.05, steps, C, E, precision='split')
    ref = _fp64()
    dev = torch.device('cuda')
    for i, n in enumerate(sizes):
        gen = engine.LindbladGenerator.build(H[i], C[i], device=dev)
        Et = torch.as_tensor(np.stack(E[i]), device=dev)
        r0 = torch.as_tensor(R0[i], device=dev)[None]
        o64, r64 = ref.lindblad_rk4(gen, r0, 0.05, steps, Et, hermitian=True)
        err = (osp[i] - o64[0]).abs().max().item()
        assert err < POP_TOL, (n, err)
        assert (rsp[i] - r64[0]).abs().max().item() < POP_TOL, n
    # anchor: the PyTorch FP64 reference against the library's FP64 kernel
    gen = engine.LindbladGenerator.build(H[4], C[4], device=dev)
    o_k, _, r_k = engine.propagate(gen, R0[4], 0.05, 50, E[4])
    o_t, r_t = ref.lindblad_rk4(gen, torch.as_tensor(R0[4], device=dev)[None], 0.05, 50,
                                torch.as_tensor(np.stack(E[4]), device=dev))
    assert (o_k - o_t).abs().max().item() < 1e-12
    assert (r_k - r_t).abs().max().item() < 1e-12


def test_dipole_correlation_dim129_4096_steps():
    from lime_gb300 import engine
    w = chains.absorption_ensemble(n_sites=128, batch=2, n_steps=4096)
    dev = torch.device('cuda')
    # site dephasing on the 128 sites, none on |g> (absorption_chain's operators)
    rates = np.r_[0.0, np.full(128, w['gamma'])]
    gen = engine.LindbladGenerator.build(w['H'], [engine.SiteDephasing(rates)], device=dev)
    mu = torch.as_tensor(w['mu'], device=dev)
    rho = mu @ torch.as_tensor(w['rho_g'], device=dev)
    osp, _, _ = engine.propagate(gen, rho, w['dt'], 4096, [mu], precision='split')
    o64, _ = _fp64().lindblad_rk4(gen, rho, w['dt'], 4096, mu[:, None])
    c64, csp = o64[..., 0], osp[..., 0]
    rel = ((csp - c64).abs().max() / c64.abs().max()).item()
    assert rel < COR_TOL, rel
    # anchor on a short horizon
    o_k, _, _ = engine.propagate(gen, rho, w['dt'], 20, [mu])
    o_t, _ = _fp64().lindblad_rk4(gen, rho, w['dt'], 20, mu[:, None])
    assert ((o_k - o_t).abs().max() / o_t.abs().max()).item() < 1e-12


def test_redfield_dim9216_2000_steps():
    from lime_gb300.redfield import redfield_tensor, propagate_vec, propagate_vec_split
    dev = torch.device('cuda')
    w = chains.redfield_chain(n=96, n_rhs=2, cfg=5)
    R, evecs = redfield_tensor(w['H'], w['a_ops'], w['spectra'], device=dev)
    V = torch.as_tensor(evecs, dtype=torch.complex128, device=dev)
    r0 = V.mH @ torch.as_tensor(w['rho0'], dtype=torch.complex128, device=dev) @ V
    E = torch.stack([V.mH @ torch.as_tensor(e, dtype=torch.complex128, device=dev) @ V
                     for e in chains.population_ops(96)])
    Rg = (R.R, 96)
    osp, _, rsp = propagate_vec_split(Rg, r0, 0.05, 2000, list(E), obs_every=10)
    o64, r64 = _fp64().redfield_rk4(R.R, r0, 0.05, 2000, E, obs_every=10)
    assert (osp - o64).abs().max().item() < POP_TOL
    assert (rsp - r64).abs().max().item() < POP_TOL
    # anchor: the PyTorch FP64 reference against the library's FP64 kernel
    o_k, _, r_k = propagate_vec(Rg, r0, 0.05, 3, list(E))
    o_t, r_t = _fp64().redfield_rk4(R.R, r0, 0.05, 3, E)
    assert (o_k - o_t).abs().max().item() < 1e-12
    assert (r_k - r_t).abs().max().item() < 1e-12
