"""Uneven batches (a list of Hamiltonians of different dimensions) through
the public API: every instance against the oracle run on its own."""
import numpy as np
import pytest

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


def _uneven(sizes, seed, n_ops=2):
    rng = np.random.default_rng(seed)
    H, C, R, E = [], [], [], []
    for n in sizes:
        h, c = chains.uneven_chain(n, rng, n_ops=n_ops)
        H.append(h)
        C.append(c)
        R.append(chains.ground_dm(n))
        E.append([chains.population_ops(n)[0], (h + h.conj().T) / 2])
    return H, C, R, E


def test_uneven_batch_dense_collapse_vs_oracle():
    from oracle import lindblad as ol
    from lime_gb300.oqs import _lindblad
    sizes = [5, 3, 8, 5, 12, 3, 8]
    H, C, R, E = _uneven(sizes, 11)
    res = _lindblad(H, R, C, e_ops=E, Nt=25, dt=0.05)
    assert isinstance(res, list) and len(res) == len(sizes)
    for i, n in enumerate(sizes):
        ro, rl = ol.lindblad(H[i], R[i], C[i], E[i], Nt=25, dt=0.05)
        assert res[i].observables.shape == (25, 2)
        assert res[i].rholist[-1].shape == (n, n)
        assert rel(res[i].observables, ro) < RTOL
        assert rel(res[i].rholist[-1], rl[-1]) < RTOL


def test_uneven_batch_from_workload_generator():
    """The uneven-batch workload's own generator (sizes up to 32 here)."""
    from oracle import lindblad as ol
    from lime_gb300.oqs import Lindblad_solver
    w = chains.uneven_batch(batch=24, n_steps=10, limit_n=32)
    E = [[chains.population_ops(int(n))[0]] for n in w['ns']]
    sol = Lindblad_solver(w['H'], c_ops=w['c_ops'])
    res = sol.evolve(w['rho0'], dt=w['dt'], Nt=10, e_ops=E, store_states=False)
    assert len(res) == len(w['ns'])
    for i in range(0, len(res), 5):
        ro, _ = ol.lindblad(w['H'][i], w['rho0'][i], w['c_ops'][i], E[i], Nt=10, dt=w['dt'])
        assert rel(res[i].observables, ro) < RTOL


def test_uneven_batch_split_precision():
    """precision='split' on every size group: the dephasing groups with
    n <= 64 take the batched kernel, the 70-dim one the streaming GEMMs;
    all agree with FP64 to the split path's bar."""
    from lime_gb300 import engine
    rng = np.random.default_rng(5)
    sizes = [16, 40, 16, 70]
    H, C, R, E = [], [], [], []
    for n in sizes:
        eps = rng.normal(0, 0.05, n)
        h = chains.exciton_chain(n, eps, -0.1)
        H.append(h)
        C.append(chains.dephasing_ops(n, 0.01))
        R.append(chains.ground_dm(n))
        E.append(chains.population_ops(n)[:4])
    o64, _, r64 = engine.propagate_ragged(H, R, 0.05, 200, C, E)
    osp, _, rsp = engine.propagate_ragged(H, R, 0.05, 200, C, E, precision='split')
    for i in range(len(sizes)):
        assert np.max(np.abs((osp[i] - o64[i]).cpu().numpy())) < 1e-6
        assert np.max(np.abs((rsp[i] - r64[i]).cpu().numpy())) < 1e-6


def test_uneven_batch_argument_errors():
    from lime_gb300 import engine
    H, C, R, E = _uneven([3, 4], 2)
    with pytest.raises(ValueError):
        engine.propagate_ragged(H, R[:1], 0.05, 3, C, E)
    with pytest.raises(ValueError):
        engine.propagate_ragged(H, R, 0.05, 3, C, [E[0], E[1][:1]])


def test_packed_small_chains_split_vs_fp64():
    """Chains of n <= 32 run block-diagonally packed on the tensor-core
    paths (64 // n to an instance, the last pack partly empty): dense
    collapse operators, an odd dimension, a non-Hermitian start and
    dephasing-only chains (the batched kernel) all agree with FP64 per
    instance."""
    from lime_gb300 import engine
    rng = np.random.default_rng(17)
    sizes = [5] * 13 + [8] * 9 + [32] * 3
    H, C, R, E = _uneven(sizes, 23)
    psi = rng.normal(size=5) + 1j * rng.normal(size=5)
    phi = rng.normal(size=5) + 1j * rng.normal(size=5)
    R[1] = np.outer(psi, phi.conj()) / (np.linalg.norm(psi) * np.linalg.norm(phi))   # non-Hermitian
    o64, _, r64 = engine.propagate_ragged(H, R, 0.05, 120, C, E)
    osp, _, rsp = engine.propagate_ragged(H, R, 0.05, 120, C, E, precision='split')
    for i, n in enumerate(sizes):
        assert osp[i].shape == o64[i].shape == (120, 2)
        assert rsp[i].shape == (n, n)
        assert np.max(np.abs((osp[i] - o64[i]).cpu().numpy())) < 1e-6
        assert np.max(np.abs((rsp[i] - r64[i]).cpu().numpy())) < 1e-6

    Hd, Cd, Rd, Ed = [], [], [], []
    for n in [6] * 11 + [16] * 5:
        Hd.append(chains.exciton_chain(n, rng.normal(0, 0.05, n), -0.1))
        Cd.append(chains.dephasing_ops(n, 0.01))
        Rd.append(chains.ground_dm(n, 1))
        Ed.append(chains.population_ops(n)[:2])
    o64, _, r64 = engine.propagate_ragged(Hd, Rd, 0.05, 150, Cd, Ed)
    osp, _, rsp = engine.propagate_ragged(Hd, Rd, 0.05, 150, Cd, Ed, precision='split')
    for i in range(len(Hd)):
        assert np.max(np.abs((osp[i] - o64[i]).cpu().numpy())) < 1e-6
        assert np.max(np.abs((rsp[i] - r64[i]).cpu().numpy())) < 1e-6
