"""FP64 Redfield path vs the reference's golden vectors and the oracle (1e-10)."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from lime_gb300 import chains

pytestmark = pytest.mark.gpu
RTOL = 1e-10


@pytest.fixture(scope='module', autouse=True)
def _lib():
    from lime_gb300 import build, _native
    build.build()
    _native.require_device()


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _gauge(evecs, ref_evecs):
    """Phase matrix D with evecs D = ref_evecs (eigh phases are LAPACK's choice)."""
    ph = np.sum(evecs.conj() * ref_evecs, axis=0)
    assert np.allclose(np.abs(ph), 1.0, atol=1e-8)
    D = np.diag(ph)
    return np.kron(D.conj().T, D.T)


def test_redfield_tensor_matches_reference():
    from lime_gb300.redfield import redfield_tensor
    g = load_golden('redfield_chain8')
    w = chains.redfield_chain(n=8, n_rhs=2, cfg=5)
    R, evecs = redfield_tensor(g['H'], list(g['a_ops']), w['spectra'])
    T = _gauge(evecs, g['evecs'])
    assert rel(T @ R.toarray() @ np.linalg.inv(T), g['R']) < 1e-12


def test_redfield_evolution_matches_reference():
    from lime_gb300.redfield import Redfield_solver
    g = load_golden('redfield_chain8')
    w = chains.redfield_chain(n=8, n_rhs=2, cfg=5)
    rs = Redfield_solver(g['H'], c_ops=list(g['a_ops']), spectra=w['spectra'])
    res = rs.evolve(g['rho0'], dt=float(g['dt']), Nt=int(g['Nt']), e_ops=list(g['e_ops']))
    assert res.observables.shape == g['observables'].shape
    assert rel(res.observables, g['observables']) < RTOL
    for i, k in enumerate(g['snap']):
        assert rel(res.rholist[k], g['rho_snap'][i]) < RTOL


def test_greens_function_route_matches_reference():
    from lime_gb300.redfield import Redfield_solver, RedfieldTensor
    g = load_golden('redfield_chain8')
    rs = Redfield_solver(g['H'], c_ops=list(g['a_ops']))
    rs.R = RedfieldTensor(torch.as_tensor(g['R'], device='cuda'), 8)
    rs.evecs = g['evecs']
    U = rs.propagator(g['tau'])
    assert rel(U[:, :, :3], g['U']) < 1e-9
    assert rel(rs.expect(g['rho0'], list(g['e_ops'][:3])), g['expect']) < 1e-9
    c = rs.correlation_4op_3t(g['rho0'], [g['mu']] * 4, 'llll', g['tau'][:4])
    assert rel(c, g['c4op_3t']) < 1e-9
    # the EOM propagator is RK4 of dU/dt = R U on the same grid
    U2 = rs.propagator(g['tau'], method='EOM')
    assert rel(U2, U) < 1e-3   # RK4 at dt = 0.5 vs the exact exponential


def test_batched_right_hand_sides_vs_oracle():
    from oracle import redfield as orf
    from lime_gb300.redfield import redfield_tensor, _redfield
    w = chains.redfield_chain(n=6, n_rhs=5, cfg=5)
    R, evecs = redfield_tensor(w['H'], w['a_ops'], w['spectra'])
    e_ops = chains.population_ops(6)[:3]
    res = _redfield(R, w['rho0'], evecs=evecs, Nt=60, dt=0.05, e_ops=e_ops)
    assert res.observables.shape == (5, 60, 3)
    # the oracle propagates the GPU-built tensor with the same eigenvectors
    for b in range(5):
        ro, rl = orf.redfield(R.toarray(), w['rho0'][b], evecs=evecs, Nt=60, dt=0.05, e_ops=e_ops)
        assert rel(res.observables[b], ro) < RTOL
        assert rel(res.rholist[b][-1], rl[-1]) < RTOL
    # and the oracle's own tensor agrees with it up to the eigenvector gauge
    Rref, evref = orf.redfield_tensor(w['H'], w['a_ops'], w['spectra'])
    T = _gauge(evecs, evref)
    assert rel(T @ R.toarray() @ np.linalg.inv(T), Rref) < 1e-12


def test_non_hermitian_bath_operator_raises():
    from lime_gb300.redfield import redfield_tensor
    a = np.array([[0, 1], [0, 0]], dtype=complex)
    with pytest.raises(TypeError):
        redfield_tensor(np.eye(2), [a], [lambda x: 1.0])
