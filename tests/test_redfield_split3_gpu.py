"""The 3M form of the tensor-core Redfield RK4 (lime_redfield_rk4_split3:
three real products instead of the four of the block form) against the
FP64 GPU path, Hermitian and non-Hermitian right-hand sides,
right-hand-side counts on both sides of a 128-column tile.

Bars: observables (populations and a coherence, all of magnitude <= 1)
within 1e-6 absolute of FP64, final states within 1e-6 relative to their
largest element, and within 4x the block form's error.  The observables
are read from the state's B operand (10-bit fixed point + fp16 residual,
about 2^-22 of the largest element per entry), which bounds both forms'
readout error to a few 1e-7 on these small systems (the block form 2.4e-7,
the 3M form 5.8e-7 on the 8-site chain, constant over 1..800 steps); the
propagated states themselves differ from FP64 by ~2e-8."""
import numpy as np
import pytest
import torch

from lime_gb300 import chains

pytestmark = pytest.mark.gpu
TOL = 1e-6


@pytest.fixture(scope='module', autouse=True)
def _lib():
    from lime_gb300 import build, _native
    build.build()
    _native.require_device()


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _eb(n, n_rhs, non_hermitian=False):
    from lime_gb300.redfield import redfield_tensor
    w = chains.redfield_chain(n=n, n_rhs=n_rhs, cfg=5)
    R, evecs = redfield_tensor(w['H'], w['a_ops'], w['spectra'])
    V = torch.as_tensor(evecs, dtype=torch.complex128, device='cuda')
    r0 = torch.as_tensor(np.stack(w['rho0']), dtype=torch.complex128, device='cuda')
    if non_hermitian:
        mu = torch.zeros((n, n), dtype=torch.complex128, device='cuda')
        mu[0, 1:] = mu[1:, 0] = torch.linspace(1.0, 0.5, n - 1, dtype=torch.float64, device='cuda').to(mu.dtype)
        r0 = mu @ r0
    r0 = V.mH @ r0 @ V
    ops = [torch.as_tensor(e, device='cuda') for e in chains.population_ops(n)[:4]]
    c = torch.zeros((n, n), dtype=torch.complex128, device='cuda')
    c[0, 1] = 1.0
    ops.append(c)
    E = [V.mH @ e @ V for e in ops]
    return R, r0, E


@pytest.mark.parametrize('n,n_rhs,steps,nh', [(8, 5, 200, False), (12, 130, 120, False), (10, 3, 150, True)])
def test_split3_matches_fp64(n, n_rhs, steps, nh):
    from lime_gb300.redfield import propagate_vec, propagate_vec_split
    R, r0, E = _eb(n, n_rhs, nh)
    Rg = (R.R, n)
    o64, _, p64 = propagate_vec(Rg, r0, 0.05, steps, E)
    o3, _, p3 = propagate_vec_split(Rg, r0, 0.05, steps, E, product='3m')
    o4, _, p4 = propagate_vec_split(Rg, r0, 0.05, steps, E, product='4m')
    assert o3.shape == o64.shape
    e3, e4 = (o3 - o64).abs().max().item(), (o4 - o64).abs().max().item()
    assert e3 < TOL, (e3, e4)
    assert rel(p3.cpu(), p64.cpu()) < TOL
    # and about as close as the block form
    assert e3 < 4 * max(e4, 1e-9), (e3, e4)
    assert rel(p3.cpu(), p64.cpu()) < 4 * max(rel(p4.cpu(), p64.cpu()), 1e-10)


def test_split3_obs_every_and_no_observables():
    from lime_gb300.redfield import propagate_vec, propagate_vec_split
    n = 9
    R, r0, E = _eb(n, 4)
    Rg = (R.R, n)
    o64, _, _ = propagate_vec(Rg, r0, 0.05, 30, E)
    o3, _, _ = propagate_vec_split(Rg, r0, 0.05, 30, E, obs_every=3, product='3m')
    assert o3.shape[1] == 10
    assert (o3 - o64[:, 2::3]).abs().max().item() < TOL
    _, _, p3 = propagate_vec_split(Rg, r0, 0.05, 30, None, product='3m')
    _, _, p64 = propagate_vec(Rg, r0, 0.05, 30, None)
    assert rel(p3.cpu(), p64.cpu()) < TOL
