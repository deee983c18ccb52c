"""Generator preparation (``lime_lindblad_prepare_f64``) with site dephasing
given by its rates, against the same operators given as dense projectors.

Bar: Heff and M agree to 1e-15 absolute (the rate r_k enters as r_k itself
instead of sqrt(r_k)^2); the propagated observables agree with the NumPy
oracle at 1e-10 relative.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def _lib():
    from lime_gb300 import build, _native
    build.build()
    _native.require_device()


def _hermitian(rng, P, n):
    a = rng.normal(size=(P, n, n)) + 1j * rng.normal(size=(P, n, n))
    return 0.05 * (a + np.conj(np.swapaxes(a, 1, 2)))


def _projectors(rates):
    """sqrt(r_k)|k><k| as dense operators: a list of n arrays ((n, n) or (P, n, n))."""
    n = rates.shape[-1]
    out = []
    for k in range(n):
        op = np.zeros(rates.shape[:-1] + (n, n), dtype=np.complex128)
        op[..., k, k] = np.sqrt(rates[..., k])
        out.append(op)
    return out


@pytest.mark.parametrize('per_instance', [True, False])
def test_rates_build_the_projectors_generator(per_instance):
    from lime_gb300 import engine
    rng = np.random.default_rng(11)
    P, n = 5, 12
    H = _hermitian(rng, P, n)
    rates = rng.uniform(0.0, 0.03, (P, n) if per_instance else (n,))
    a = engine.LindbladGenerator.build(H, [engine.SiteDephasing(rates)])
    b = engine.LindbladGenerator.build(H, _projectors(rates))
    assert a.P == b.P == P and a.m is not None and b.m is not None
    assert (a.heff - b.heff).abs().max().item() <= 1e-15
    assert (a.m - b.m).abs().max().item() <= 1e-15
    assert engine.split_supported(a) is None and engine.split_supported(b) is None


def test_rates_with_other_operators():
    """Rates of two SiteDephasing sets, a diagonal operator with several
    nonzero entries (off-diagonal M) and a dense operator, all at once."""
    from lime_gb300 import engine
    rng = np.random.default_rng(12)
    P, n = 3, 10
    H = _hermitian(rng, P, n)
    r1 = rng.uniform(0.0, 0.02, (P, n))
    r2 = rng.uniform(0.0, 0.02, n)
    spread = np.zeros((1, n), dtype=np.complex128)
    spread[0, :4] = 0.1 * (1 + 1j)
    dense = 0.05 * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    a = engine.LindbladGenerator.build(
        H, [engine.SiteDephasing(r1), engine.DiagonalOps(spread), dense, engine.SiteDephasing(r2)])
    b = engine.LindbladGenerator.build(
        H, _projectors(r1) + [np.diag(spread[0]), dense] + _projectors(r2))
    assert (a.heff - b.heff).abs().max().item() <= 1e-15
    assert (a.m - b.m).abs().max().item() <= 1e-15
    assert a.k_dense == b.k_dense == 1


def test_rates_propagate_like_the_oracle():
    from lime_gb300.oqs import Lindblad_solver, Populations, SiteDephasing
    from oracle import lindblad as ol
    rng = np.random.default_rng(13)
    P, n = 4, 8
    H = _hermitian(rng, P, n)
    rates = rng.uniform(0.005, 0.03, (P, n))
    rho0 = np.zeros((n, n), dtype=np.complex128)
    rho0[0, 0] = 1
    res = Lindblad_solver(H, c_ops=[SiteDephasing(rates)]).evolve(
        rho0, dt=0.05, Nt=15, e_ops=Populations(n), store_states=False)
    pops = [np.diag(np.eye(n)[k]).astype(complex) for k in range(n)]
    for p in range(P):
        ro, _ = ol.lindblad(H[p], rho0, _projectors(rates[p]), pops, Nt=15, dt=0.05)
        got = np.asarray(res.observables)[p]
        assert np.max(np.abs(got - ro)) / np.max(np.abs(ro)) < 1e-10
