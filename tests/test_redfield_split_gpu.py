"""Tensor-core split-precision Redfield RK4 against the FP64 GPU path
(itself pinned to the reference at 1e-10): observables and final states
within 1e-6 of the FP64 results, relative to their largest magnitude."""
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


def _coherence_ops(n):
    ops = []
    for (i, j) in [(0, 1), (1, 2), (0, n - 1)]:
        e = np.zeros((n, n), dtype=complex)
        e[i, j] = 1.0
        ops.append(e)
    return ops


@pytest.mark.parametrize('n,n_rhs,steps', [(8, 5, 200), (12, 70, 120)])
def test_split_matches_fp64(n, n_rhs, steps):
    from lime_gb300.redfield import redfield_tensor, _redfield
    w = chains.redfield_chain(n=n, n_rhs=n_rhs, cfg=5)
    R, evecs = redfield_tensor(w['H'], w['a_ops'], w['spectra'])
    e_ops = chains.population_ops(n)[:4] + _coherence_ops(n)
    ref = _redfield(R, w['rho0'], evecs=evecs, Nt=steps, dt=0.05, e_ops=e_ops, store_states=False)
    spl = _redfield(R, w['rho0'], evecs=evecs, Nt=steps, dt=0.05, e_ops=e_ops, store_states=False,
                    precision='split')
    assert spl.observables.shape == (n_rhs, steps, len(e_ops))
    assert rel(spl.observables, ref.observables) < TOL
    assert rel(np.stack(spl.rholist), np.stack(ref.rholist)) < TOL
    # trace is conserved by the generator; the split run keeps it to 1e-6
    tr = np.trace(np.stack(spl.rholist), axis1=1, axis2=2)
    assert np.max(np.abs(tr - 1.0)) < TOL


def test_split_non_hermitian_right_hand_side():
    """Correlation-function initial condition mu rho_g (not Hermitian)."""
    from lime_gb300.redfield import redfield_tensor, _redfield
    n = 10
    w = chains.redfield_chain(n=n, n_rhs=3, cfg=5)
    R, evecs = redfield_tensor(w['H'], w['a_ops'], w['spectra'])
    mu = np.zeros((n, n), dtype=complex)
    mu[0, 1:] = mu[1:, 0] = np.linspace(1.0, 0.5, n - 1)
    r0 = np.stack([mu @ w['rho0'][b] for b in range(3)])
    e_ops = [mu, _coherence_ops(n)[0]]
    ref = _redfield(R, r0, evecs=evecs, Nt=150, dt=0.05, e_ops=e_ops, store_states=False)
    spl = _redfield(R, r0, evecs=evecs, Nt=150, dt=0.05, e_ops=e_ops, store_states=False,
                    precision='split')
    assert rel(spl.observables, ref.observables) < TOL
    assert rel(np.stack(spl.rholist), np.stack(ref.rholist)) < TOL


def test_split_solver_entry_and_states():
    from lime_gb300.redfield import Redfield_solver
    n = 8
    w = chains.redfield_chain(n=n, n_rhs=1, cfg=5)
    rs = Redfield_solver(w['H'], c_ops=w['a_ops'], spectra=w['spectra'])
    e_ops = chains.population_ops(n)[:3]
    ref = rs.evolve(w['rho0'][0], dt=0.05, Nt=40, e_ops=e_ops)
    spl = rs.evolve(w['rho0'][0], dt=0.05, Nt=40, e_ops=e_ops, store_states=True, precision='split')
    assert spl.observables.shape == ref.observables.shape == (40, 3)
    assert rel(spl.observables, ref.observables) < TOL
    assert len(spl.rholist) == 40
    assert rel(np.stack(spl.rholist), np.stack(ref.rholist)) < TOL


def test_split_launches_are_counted():
    from lime_gb300 import _native
    from lime_gb300.redfield import redfield_tensor, propagate_vec_split
    n = 8
    w = chains.redfield_chain(n=n, n_rhs=2, cfg=5)
    R, evecs = redfield_tensor(w['H'], w['a_ops'], w['spectra'])
    r0 = torch.as_tensor(w['rho0'], dtype=torch.complex128, device='cuda')
    c0 = _native.launch_count()
    propagate_vec_split((R.R, n), r0, 0.05, 10)
    torch.cuda.synchronize()
    # convert + init + 4 stages per step + final state
    assert _native.launch_count() - c0 == 3 + 4 * 10


def test_split_many_observables():
    """More than one 128-row tile of observables (general complex matrices)."""
    from lime_gb300.redfield import redfield_tensor, _redfield
    n = 12
    w = chains.redfield_chain(n=n, n_rhs=3, cfg=5)
    R, evecs = redfield_tensor(w['H'], w['a_ops'], w['spectra'])
    rng = np.random.default_rng(7)
    e_ops = list(rng.normal(size=(140, n, n)) + 1j * rng.normal(size=(140, n, n)))
    ref = _redfield(R, w['rho0'], evecs=evecs, Nt=30, dt=0.05, e_ops=e_ops, store_states=False)
    spl = _redfield(R, w['rho0'], evecs=evecs, Nt=30, dt=0.05, e_ops=e_ops, store_states=False,
                    precision='split')
    assert spl.observables.shape == (3, 30, 140)
    assert rel(spl.observables, ref.observables) < TOL
