"""General Lindblad generators on the tensor cores (streaming split-precision
GEMMs: dense collapse operators, any dimension) against the FP64 path, which
is itself pinned to the reference at 1e-10.  Bar: 1e-6 on populations,
observables and states (relative to their largest magnitude for
correlations)."""
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


def _both(gen, rho0, steps, e_ops, **kw):
    from lime_gb300 import engine
    o64, _, r64 = engine.propagate(gen, rho0, 0.05, steps, e_ops, **kw)
    osp, _, rsp = engine.propagate(gen, rho0, 0.05, steps, e_ops, precision='split', **kw)
    return (o64.cpu().numpy(), r64.cpu().numpy()), (osp.cpu().numpy(), rsp.cpu().numpy())


def _dev(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b)))


@pytest.mark.parametrize('n,n_ops,steps', [(8, 3, 300), (20, 2, 150), (130, 2, 25)])
def test_dense_collapse_operators(n, n_ops, steps):
    from lime_gb300 import engine
    rng = np.random.default_rng(40 + n)
    H, c_ops = chains.uneven_chain(n, rng, n_ops=n_ops)
    gen = engine.LindbladGenerator.build(H, c_ops)
    assert engine.split_supported(gen) is not None    # not the batched kernel's case
    e_ops = chains.population_ops(n)[:3] + [(H + H.conj().T) / 2]
    (o64, r64), (osp, rsp) = _both(gen, chains.ground_dm(n), steps, e_ops)
    assert osp.shape == o64.shape == (1, steps, 4)
    assert _dev(osp, o64) < TOL
    assert _dev(rsp, r64) < TOL


def test_large_dephasing_chain_no_dense_operators():
    """n = 80 > 64 with diagonal collapse operators: GEMM 1 + the M term."""
    from lime_gb300 import engine
    n = 80
    eps = np.random.default_rng(8).normal(0, 0.05, n)
    gen = engine.LindbladGenerator.build(chains.exciton_chain(n, eps, -0.1), chains.dephasing_ops(n, 0.01))
    (o64, r64), (osp, rsp) = _both(gen, chains.ground_dm(n), 300, chains.population_ops(n)[:5])
    assert _dev(osp, o64) < TOL
    assert _dev(rsp, r64) < TOL


def test_dense_and_diagonal_operators_batched():
    """Three different generators (dense + diagonal operators) in one call."""
    from lime_gb300 import engine
    rng = np.random.default_rng(12)
    n, P = 24, 3
    Hs, Ls = [], []
    for _ in range(P):
        h, c = chains.uneven_chain(n, rng, n_ops=2)
        Hs.append(h)
        Ls.append(c)
    H = np.stack(Hs)
    c_ops = [np.stack([Ls[p][k] for p in range(P)]) for k in range(2)] + chains.dephasing_ops(n, 0.02)
    gen = engine.LindbladGenerator.build(H, c_ops)
    assert gen.m is not None and gen.k_dense == 2
    rho0 = np.stack([chains.ground_dm(n, k) for k in range(P)])
    e_ops = chains.population_ops(n)[:4]
    (o64, r64), (osp, rsp) = _both(gen, rho0, 120, e_ops)
    assert osp.shape == (P, 120, 4)
    assert _dev(osp, o64) < TOL
    assert _dev(rsp, r64) < TOL


def test_shared_generator_many_states():
    from lime_gb300 import engine
    rng = np.random.default_rng(21)
    n = 16
    H, c_ops = chains.uneven_chain(n, rng, n_ops=3)
    gen = engine.LindbladGenerator.build(H, c_ops)
    psi = rng.normal(size=(5, n)) + 1j * rng.normal(size=(5, n))
    psi /= np.linalg.norm(psi, axis=1, keepdims=True)
    rho0 = np.einsum('bi,bj->bij', psi, psi.conj())
    (o64, r64), (osp, rsp) = _both(gen, rho0, 100, chains.population_ops(n)[:2])
    assert _dev(osp, o64) < TOL
    assert _dev(rsp, r64) < TOL


def test_dipole_correlation_dense_operators():
    """Non-Hermitian start mu rho_g (two Hermitian parts) through the public
    correlation call."""
    from lime_gb300.oqs import Lindblad_solver
    rng = np.random.default_rng(31)
    n = 12
    H, c_ops = chains.uneven_chain(n, rng, n_ops=2)
    mu = np.zeros((n, n), dtype=complex)
    mu[0, 1:] = mu[1:, 0] = np.linspace(1.0, 0.5, n - 1)
    rho_g = chains.ground_dm(n)
    c64 = Lindblad_solver(H, c_ops=c_ops).correlation_2op_1t(rho_g, mu, mu, 0.05, 300, output=None)
    csp = Lindblad_solver(H, c_ops=c_ops, precision='split').correlation_2op_1t(rho_g, mu, mu, 0.05, 300,
                                                                              output=None)
    assert _dev(csp, c64) / np.max(np.abs(c64)) < TOL


def test_stream_launch_count():
    from lime_gb300 import _native, engine
    rng = np.random.default_rng(2)
    H, c_ops = chains.uneven_chain(8, rng, n_ops=1)
    gen = engine.LindbladGenerator.build(H, c_ops)
    c0 = _native.launch_count()
    engine.propagate(gen, chains.ground_dm(8), 0.05, 6, [chains.population_ops(8)[0]], precision='split',
                     obs_every=2)
    torch.cuda.synchronize()
    # convert + init + 2 GEMMs per stage + an observable pass every 2 steps + final
    assert _native.launch_count() - c0 == 2 + 8 * 6 + 3 + 1


def test_multi_operator_correlations_split():
    """The reference's 3- and 4-operator one- and two-time correlations
    (golden vectors from the reference) on the tensor cores."""
    from conftest import load_golden
    from lime_gb300.oqs import Lindblad_solver
    g = load_golden('correlations_n4')
    sol = Lindblad_solver(g['H'], c_ops=list(g['c_ops']), precision='split')
    ops, rho0, dt = list(g['ops']), g['rho0'], float(g['dt'])

    def rel(a, b):
        return np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b))

    assert rel(sol.correlation_3op_1t(rho0, ops[:3], dt=dt, Nt=30), g['c3op_1t']) < TOL
    assert rel(sol.correlation_4op_1t(rho0, ops, dt, 30), g['c4op_1t']) < TOL
    assert rel(sol.correlation_3op_2t(rho0, ops[:3], dt, 12, 10), g['c3op_2t']) < TOL
    assert rel(sol.correlation_4op_2t(rho0, ops, dt, 12, 10), g['c4op_2t']) < TOL


@pytest.mark.parametrize('n', [1, 2, 3])
def test_tiny_dimensions(n):
    from lime_gb300 import engine
    rng = np.random.default_rng(60 + n)
    if n == 1:
        H, c_ops = np.array([[0.3]], dtype=complex), [np.array([[0.1 + 0.05j]])]
    else:
        H, c_ops = chains.uneven_chain(n, rng, n_ops=2)
    gen = engine.LindbladGenerator.build(H, c_ops)
    (o64, r64), (osp, rsp) = _both(gen, chains.ground_dm(n), 40, [chains.population_ops(n)[0]])
    assert _dev(osp, o64) < TOL
    assert _dev(rsp, r64) < TOL


def test_zero_steps_returns_the_input():
    from lime_gb300 import engine
    rng = np.random.default_rng(70)
    H, c_ops = chains.uneven_chain(10, rng, n_ops=2)
    gen = engine.LindbladGenerator.build(H, c_ops)
    psi = rng.normal(size=10) + 1j * rng.normal(size=10)
    rho0 = np.outer(psi, psi.conj()) / np.vdot(psi, psi).real
    obs, _, rho = engine.propagate(gen, rho0, 0.05, 0, [chains.population_ops(10)[0]], precision='split')
    assert obs.shape == (1, 0, 1)
    assert _dev(rho[0].cpu().numpy(), rho0) < 1e-7          # fp32 hi + lo round trip
