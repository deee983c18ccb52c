"""The seeded synthetic workloads (lime_gb300.chains) have the configured
shapes, value distributions and physical properties: the single dephasing
chain, the 4096-realisation disorder ensemble, the uneven batch, the
absorption ensemble of the gradient workload and the Redfield chain."""
import numpy as np

from lime_gb300 import chains


def _herm(a):
    return np.allclose(a, np.conj(np.swapaxes(a, -1, -2)))


def test_single_chain():
    w = chains.single_chain()
    H = w['H']
    assert H.shape == (16, 16) and _herm(H) and w['Nt'] == 2000 and w['dt'] == 0.05
    assert np.allclose(np.diag(H, 1), -0.1) and np.count_nonzero(np.triu(H, 2)) == 0   # open-ended chain
    assert len(w['c_ops']) == 16
    for k, L in enumerate(w['c_ops']):
        assert L[k, k] == np.sqrt(0.01) and np.count_nonzero(L) == 1
    assert w['rho0'][0, 0] == 1 and np.trace(w['rho0']) == 1


def test_disorder_ensemble_distribution_and_seed():
    w = chains.disorder_ensemble()
    H, g = w['H'], w['gamma']
    assert H.shape == (4096, 64, 64) and _herm(H[:8])
    eps = np.real(np.diagonal(H, axis1=1, axis2=2))
    assert abs(eps.std() - 0.05) < 0.002 and abs(eps.mean()) < 0.002
    assert np.allclose(np.diagonal(H, 1, axis1=1, axis2=2), -0.1)
    assert g.min() >= 0.005 and g.max() <= 0.02 and abs(g.mean() - 0.0125) < 0.0005
    w2 = chains.disorder_ensemble(batch=8)
    assert np.array_equal(w2['H'], H[:8])               # seeded: prefixes agree


def test_uneven_batch_shapes_and_operators():
    w = chains.uneven_batch(batch=96)
    ns = w['ns']
    assert set(ns) <= set(chains.UNEVEN_SIZES) and len(set(ns)) >= 5
    for H, C, r, n in zip(w['H'][:24], w['c_ops'][:24], w['rho0'][:24], ns[:24]):
        assert H.shape == (n, n) and _herm(H)
        # tridiagonal chain + 0.01-scaled GOE perturbation
        off = H - np.diag(np.diag(H)) - np.diag(np.diag(H, 1), 1) - np.diag(np.diag(H, -1), -1)
        assert 0 < np.abs(off).max() < 0.05
        assert len(C) == 3
        for L in C:
            assert np.isclose(np.linalg.norm(L, 2) ** 2, 0.01)
        assert r[0, 0] == 1
    w_again = chains.uneven_batch(batch=96)
    assert np.array_equal(w_again['ns'], ns) and np.array_equal(w_again['H'][5], w['H'][5])


def test_absorption_ensemble():
    w = chains.absorption_ensemble(batch=4)
    H, mu, d = w['H'], w['mu'], w['d']
    assert H.shape == (4, 129, 129) and _herm(H) and _herm(mu)
    assert np.all(H[:, 0, :] == 0)                       # |g> at energy 0, uncoupled
    assert np.allclose(mu[:, 0, 1:], d) and np.count_nonzero(mu[:, 1:, 1:]) == 0
    assert abs(d.mean() - 1.0) < 0.05


def test_redfield_chain():
    w = chains.redfield_chain(n=96, n_rhs=8)
    assert w['H'].shape == (96, 96) and len(w['a_ops']) == 96 and len(w['spectra']) == 96
    r = w['rho0']
    assert r.shape == (8, 96, 96)
    assert np.allclose(np.trace(r, axis1=1, axis2=2), 1) and np.allclose(r @ r, r)   # pure states
    S = w['spectra'][0]
    for om in (0.01, 0.05, 0.2):                         # detailed balance at kT = 0.025
        assert np.isclose(S(-om), np.exp(-om / 0.025) * S(om))
