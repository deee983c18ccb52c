"""FP64 CUDA Lindblad path vs the reference's golden vectors and the oracle.

Bar: 1e-10 relative (max |x - ref| / max |ref|) for every output.
"""
import os

import numpy as np
import pytest

from conftest import load_golden
from lime_gb300 import chains

pytestmark = pytest.mark.gpu
RTOL = 1e-10


def relerr(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.fixture(scope='module', autouse=True)
def _lib():
    from lime_gb300 import build, _native
    build.build()
    _native.require_device()
    assert _native._lib._name.endswith('liblime_gb300.so')


def test_chain16_matches_reference_run():
    from lime_gb300.oqs import Lindblad_solver
    g = load_golden('lindblad_chain16')
    res = Lindblad_solver(g['H'], c_ops=list(g['c_ops'])).evolve(
        g['rho0'], dt=float(g['dt']), Nt=int(g['Nt']), e_ops=list(g['e_ops']))
    assert res.observables.shape == g['observables'].shape
    assert res.observables.dtype == np.complex128
    assert relerr(res.observables, g['observables']) < RTOL
    assert len(res.rholist) == int(g['Nt'])
    for i, k in enumerate(g['snap']):
        assert relerr(res.rholist[k], g['rho_snap'][i]) < RTOL
    assert np.allclose(res.times, np.arange(int(g['Nt'])) * float(g['dt']))


def test_file_branch_matches_reference(tmp_path, monkeypatch):
    from lime_gb300.oqs import _lindblad
    g = load_golden('lindblad_chain16_noresult')
    monkeypatch.chdir(tmp_path)
    rho = _lindblad(g['H'], g['rho0'], list(g['c_ops']), e_ops=list(g['e_ops']),
                    Nt=int(g['Nt']), dt=float(g['dt']), return_result=False)
    assert relerr(rho, g['rho_final']) < RTOL
    rows = [line.split() for line in open(tmp_path / 'obs.dat')]
    obs = np.array([[complex(x) for x in r[1:]] for r in rows])
    assert relerr(obs, g['observables']) < 1e-12
    t = np.array([float(r[0]) for r in rows])
    assert np.allclose(t, (np.arange(int(g['Nt'])) + 1) * float(g['dt']))


def test_dense_collapse_operators():
    from lime_gb300.oqs import Lindblad_solver
    g = load_golden('lindblad_dense8')
    res = Lindblad_solver(g['H'], c_ops=list(g['c_ops'])).evolve(
        g['rho0'], dt=float(g['dt']), Nt=int(g['Nt']), e_ops=list(g['e_ops']))
    assert relerr(res.observables, g['observables']) < RTOL
    for i, k in enumerate(g['snap']):
        assert relerr(res.rholist[k], g['rho_snap'][i]) < RTOL


def test_dipole_correlation(tmp_path):
    from lime_gb300.oqs import Lindblad_solver
    g = load_golden('correlation_2op_chain8')
    out = tmp_path / 'cor.dat'
    cor = Lindblad_solver(g['H'], c_ops=list(g['c_ops'])).correlation_2op_1t(
        g['rho0'], g['mu'], g['mu'], dt=float(g['dt']), Nt=int(g['Nt']), output=str(out))
    assert cor.shape == g['cor'].shape
    assert relerr(cor, g['cor']) < RTOL
    rows = [line.split() for line in open(out)]
    assert len(rows) == int(g['Nt'])
    assert relerr(np.array([complex(r[1]) for r in rows]), g['cor']) < 1e-12


def test_multi_operator_correlations():
    from lime_gb300.oqs import Lindblad_solver
    g = load_golden('correlations_n4')
    sol = Lindblad_solver(g['H'], c_ops=list(g['c_ops']))
    ops, rho0, dt = list(g['ops']), g['rho0'], float(g['dt'])
    assert relerr(sol.correlation_3op_1t(rho0, ops[:3], dt=dt, Nt=30), g['c3op_1t']) < RTOL
    assert relerr(sol.correlation_4op_1t(rho0, ops, dt, 30), g['c4op_1t']) < RTOL
    assert relerr(sol.correlation_3op_2t(rho0, ops[:3], dt, 12, 10), g['c3op_2t']) < RTOL
    assert relerr(sol.correlation_4op_2t(rho0, ops, dt, 12, 10), g['c4op_2t']) < RTOL
    with pytest.raises(ValueError):
        sol.correlation_4op_1t(rho0, ops[:3], dt, 30)


@pytest.mark.parametrize('n', [1, 2, 5, 17, 33, 65])
def test_ragged_sizes_vs_oracle(n):
    from oracle import lindblad as ol
    from lime_gb300.oqs import _lindblad
    rng = np.random.default_rng(100 + n)
    H, c_ops = chains.uneven_chain(n, rng, n_ops=2) if n > 1 else (
        np.array([[0.3]], dtype=complex), [np.array([[0.1 + 0.05j]])])
    c_ops = c_ops + chains.dephasing_ops(n, 0.02)
    rho0 = chains.ground_dm(n)
    e_ops = [chains.population_ops(n)[0], (H + H.conj().T) / 2]
    ro, rl = ol.lindblad(H, rho0, c_ops, e_ops, Nt=7, dt=0.05)
    res = _lindblad(H, rho0, c_ops, e_ops=e_ops, Nt=7, dt=0.05)
    assert relerr(res.observables, ro) < RTOL
    assert relerr(res.rholist[-1], rl[-1]) < RTOL


def test_batched_disorder_vs_oracle():
    from oracle import lindblad as ol
    from lime_gb300.oqs import _lindblad
    w = chains.disorder_ensemble(n=12, batch=5, n_steps=40)
    c_ops = [np.sqrt(w['gamma'])[:, None, None] * p[None] for p in chains.population_ops(12)]
    e_ops = chains.population_ops(12)
    res = _lindblad(w['H'], w['rho0'], c_ops, e_ops=e_ops, Nt=40, dt=w['dt'], store_states=False)
    assert res.observables.shape == (5, 40, 12)
    for b in range(5):
        ro, _ = ol.lindblad(w['H'][b], w['rho0'], chains.dephasing_ops(12, w['gamma'][b]),
                            e_ops, Nt=40, dt=w['dt'])
        assert relerr(res.observables[b], ro) < RTOL


def test_non_hermitian_start_vs_oracle():
    from oracle import lindblad as ol
    from lime_gb300.oqs import _lindblad
    rng = np.random.default_rng(7)
    H, c_ops = chains.uneven_chain(6, rng)
    rho0 = rng.normal(size=(6, 6)) + 1j * rng.normal(size=(6, 6))
    e = rng.normal(size=(6, 6)) + 1j * rng.normal(size=(6, 6))
    ro, rl = ol.lindblad(H, rho0, c_ops, [e], Nt=25, dt=0.05)
    res = _lindblad(H, rho0, c_ops, e_ops=[e], Nt=25, dt=0.05)
    assert relerr(res.observables, ro) < RTOL
    assert relerr(res.rholist[-1], rl[-1]) < RTOL


def test_zero_steps_and_no_observables():
    from lime_gb300.oqs import _lindblad
    w = chains.single_chain(n=4, n_steps=0)
    res = _lindblad(w['H'], w['rho0'], w['c_ops'], e_ops=None, Nt=0, dt=w['dt'])
    assert res.observables.shape == (0, 0)
    res = _lindblad(w['H'], w['rho0'], w['c_ops'], e_ops=None, Nt=3, dt=w['dt'])
    assert res.observables.shape == (3, 0)


def test_nonfinite_input_raises_flag():
    from lime_gb300 import _native
    from lime_gb300.oqs import _lindblad
    w = chains.single_chain(n=4)
    rho0 = w['rho0'].copy()
    rho0[1, 1] = np.nan
    with pytest.raises(_native.KernelFlagError) as ei:
        _lindblad(w['H'], rho0, w['c_ops'], e_ops=None, Nt=3, dt=w['dt'])
    assert ei.value.flags & _native.LIME_FLAG_NONFINITE


def test_trace_drift_flag_from_inconsistent_generator():
    """A generator with decay in Heff but no matching jump term loses trace."""
    import torch
    from lime_gb300 import _native, engine
    gen = engine.LindbladGenerator.build(np.eye(3) * 0.1, chains.dephasing_ops(3, 0.5))
    gen.m = None  # drop the jump term: d Tr(rho)/dt = -0.5 Tr(rho)
    with pytest.raises(_native.KernelFlagError) as ei:
        engine.propagate(gen, chains.ground_dm(3), 0.05, 10, trace_tol=1e-6)
    assert ei.value.flags & _native.LIME_FLAG_TRACE_DRIFT
    # with the check disabled the call completes and the trace decays as exp(-0.5 t)
    _, _, rho = engine.propagate(gen, chains.ground_dm(3), 0.05, 10, trace_tol=0.0)
    tr = torch.diagonal(rho[0]).sum().real.item()
    assert abs(tr - np.exp(-0.5 * 0.5)) < 1e-6


def test_bad_arguments_rejected():
    from lime_gb300 import _native, engine
    gen = engine.LindbladGenerator.build(np.eye(3), None)
    with pytest.raises(ValueError):
        engine.propagate(gen, np.eye(4) / 4, 0.05, 2)
    lib = _native.load()
    d = _native.LindbladDesc()
    d.n, d.batch, d.n_steps = 3, 1, 1
    assert lib.lime_lindblad_rk4_f64(d, None) == -1   # null rho / heff
