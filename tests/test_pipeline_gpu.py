"""The pipelined host batch (``engine.propagate_host_pipelined``) against the
same batch as one launch of the batched split kernel.

Both run the same kernel on the same instances with the same A-operand
scale (the batch's max |Heff|), so the results are bitwise equal; against
the FP64 path they stay within the split path's bar (populations: 1e-6
absolute).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
POP_TOL = 1e-6


@pytest.fixture(scope='module', autouse=True)
def _lib():
    from lime_gb300 import build, _native
    build.build()
    _native.require_device()


def _slots():
    from lime_gb300 import engine
    return engine.SPLIT_CTAS_PER_SM * torch.cuda.get_device_properties(0).multi_processor_count


def _batch(P, n, seed, eps=0.02):
    """P tridiagonal chains (|J| = 0.1, site energies within eps), one
    dephasing rate per site."""
    rng = np.random.default_rng(seed)
    H = np.zeros((P, n, n), dtype=np.complex128)
    idx = np.arange(n)
    H[:, idx, idx] = rng.uniform(-eps, eps, (P, n))
    H[:, idx[:-1], idx[1:]] = -0.1
    H[:, idx[1:], idx[:-1]] = -0.1
    rates = rng.uniform(0.005, 0.02, (P, n))
    return H, rates


def _evolve(H, rho0, c_ops, e_ops, Nt, nout, pipelined, monkeypatch):
    """evolve() with the pipeline on or off; checks which path ran."""
    from lime_gb300 import engine
    from lime_gb300.oqs import Lindblad_solver
    monkeypatch.setattr(engine, 'PIPELINE_MIN_ROUNDS', 3 if pipelined else 1 << 30)
    ran, orig = [], engine.propagate_host_pipelined

    def spy(*a, **k):
        r = orig(*a, **k)
        ran.append(r is not None)
        return r

    monkeypatch.setattr(engine, 'propagate_host_pipelined', spy)
    res = Lindblad_solver(H, c_ops=c_ops, precision='split').evolve(
        rho0, dt=0.05, Nt=Nt, e_ops=e_ops, nout=nout, store_states=False)
    monkeypatch.setattr(engine, 'propagate_host_pipelined', orig)
    assert ran == [pipelined]
    return np.asarray(res.observables), np.asarray(res.rholist)


def test_pipeline_ranges_cover_the_batch_on_this_device():
    from lime_gb300 import engine
    S = _slots()
    P = 3 * S + 17
    ch = engine.pipeline_chunks(P, S)
    assert ch == [(0, 3 * S), (3 * S, P)]


@pytest.mark.parametrize('n', [16, 64])
def test_pipelined_equals_one_launch_populations(n, monkeypatch):
    from lime_gb300.engine import Populations, SiteDephasing
    P = 3 * _slots() + 17
    H, rates = _batch(P, n, seed=n)
    rho0 = np.zeros((n, n), dtype=np.complex128)
    rho0[0, 0] = 1
    args = (H, rho0, [SiteDephasing(rates)], Populations(n), 10, 2)
    o1, r1 = _evolve(*args, pipelined=False, monkeypatch=monkeypatch)
    o2, r2 = _evolve(*args, pipelined=True, monkeypatch=monkeypatch)
    assert o1.shape == o2.shape == (P, 5, n) and r1.shape == r2.shape == (P, n, n)
    assert np.array_equal(o1, o2) and np.array_equal(r1, r2)


def test_pipelined_equals_one_launch_per_instance_states_and_dense_observable(monkeypatch):
    """Per-instance rho0 and DiagonalOps, pinned host tensors, a general
    (non-population) Hermitian observable shared by every instance."""
    from lime_gb300.engine import DiagonalOps
    n = 32
    P = 4 * _slots() + 5
    H, rates = _batch(P, n, seed=7)
    rng = np.random.default_rng(8)
    psi = rng.normal(size=(P, n)) + 1j * rng.normal(size=(P, n))
    psi /= np.linalg.norm(psi, axis=1, keepdims=True)
    r = np.einsum('bi,bj->bij', psi, psi.conj())
    rho0 = torch.as_tensor((r + np.conj(np.swapaxes(r, 1, 2))) / 2).pin_memory()   # exactly Hermitian
    # n site projectors sqrt(rate_k)|k><k| (the batched kernel's diagonal M)
    l = np.zeros((P, n, n), dtype=np.complex128)
    l[:, np.arange(n), np.arange(n)] = np.sqrt(rates)
    A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    E = [(A + A.conj().T) / 2, np.diag(np.arange(n, dtype=np.complex128))]
    args = (torch.as_tensor(H).pin_memory(), rho0, [DiagonalOps(l)], E, 12, 3)
    o1, r1 = _evolve(*args, pipelined=False, monkeypatch=monkeypatch)
    o2, r2 = _evolve(*args, pipelined=True, monkeypatch=monkeypatch)
    assert o1.shape == o2.shape == (P, 4, 2)
    assert np.array_equal(o1, o2) and np.array_equal(r1, r2)


def test_pipelined_ranges_of_different_magnitude(monkeypatch):
    """The first range's Hamiltonians are 8x larger than the second's: every
    range still takes the batch's A scale, so the result is bitwise that of
    one launch, and within the split path's bar of FP64."""
    from lime_gb300 import engine
    from lime_gb300.engine import Populations, SiteDephasing
    n, S = 16, _slots()
    P = 5 * S
    assert engine.pipeline_chunks(P, S) == [(0, 4 * S), (4 * S, P)]
    H, rates = _batch(P, n, seed=3)
    H[:4 * S] *= 8
    rho0 = np.zeros((n, n), dtype=np.complex128)
    rho0[0, 0] = 1
    c_ops = [SiteDephasing(rates)]
    o1, r1 = _evolve(H, rho0, c_ops, Populations(n), 20, 1, pipelined=False, monkeypatch=monkeypatch)
    o2, r2 = _evolve(H, rho0, c_ops, Populations(n), 20, 1, pipelined=True, monkeypatch=monkeypatch)
    assert np.array_equal(o1, o2) and np.array_equal(r1, r2)
    from lime_gb300.oqs import Lindblad_solver
    ref = Lindblad_solver(H, c_ops=c_ops).evolve(rho0, dt=0.05, Nt=20, e_ops=Populations(n),
                                                 store_states=False)
    assert np.max(np.abs(o2 - np.asarray(ref.observables))) < POP_TOL
    assert np.max(np.abs(r2 - np.asarray(ref.rholist))) < POP_TOL


def test_pipeline_declines_what_it_does_not_cover():
    from lime_gb300 import engine
    from lime_gb300.engine import Populations, SiteDephasing
    n, P = 16, 3 * _slots()
    H, rates = _batch(P, n, seed=4)
    rho_nh = np.zeros((n, n), dtype=np.complex128)
    rho_nh[0, 1] = 1                                   # not Hermitian
    assert engine.propagate_host_pipelined(H, rho_nh, [SiteDephasing(rates)], Populations(n),
                                           0.05, 4) is None
    rho0 = np.eye(n, dtype=np.complex128) / n
    small = engine.propagate_host_pipelined(H[:_slots()], rho0, [SiteDephasing(rates[:_slots()])],
                                            Populations(n), 0.05, 4)
    assert small is None                               # one round: one launch
    dense = np.zeros((n, n), dtype=np.complex128)
    dense[0, 1] = dense[1, 0] = 0.1                    # not diagonal: another kernel
    assert engine.propagate_host_pipelined(H, rho0, [dense], Populations(n), 0.05, 4) is None
