"""Pin the NumPy oracle against golden vectors produced by the reference.

The fixtures under tests/golden/ were written by make_golden.py running the
reference lime solvers; every tolerance here is a rounding-level bound
(different BLAS summation order), not a modelling tolerance.
"""
import numpy as np
import pytest

from oracle import lindblad as ol
from oracle import redfield as orf
from oracle import superop as osp
from oracle import spectra as ospec
from lime_gb300 import chains

from conftest import load_golden

RTOL = 1e-10


def relerr(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_chain16_full_run():
    g = load_golden('lindblad_chain16')
    obs, rholist = ol.lindblad(g['H'], g['rho0'], list(g['c_ops']), list(g['e_ops']),
                               Nt=int(g['Nt']), dt=float(g['dt']))
    assert relerr(obs, g['observables']) < RTOL
    for i, k in enumerate(g['snap']):
        assert relerr(rholist[k], g['rho_snap'][i]) < RTOL


def test_chain16_file_branch():
    g = load_golden('lindblad_chain16_noresult')
    obs, rho = ol.lindblad(g['H'], g['rho0'], list(g['c_ops']), list(g['e_ops']),
                           Nt=int(g['Nt']), dt=float(g['dt']), return_result=False)
    # obs.dat is text written with str(complex): ~17 significant digits
    assert relerr(obs, g['observables']) < 1e-12
    assert relerr(rho, g['rho_final']) < RTOL


def test_dense_collapse_ops():
    g = load_golden('lindblad_dense8')
    obs, rholist = ol.lindblad(g['H'], g['rho0'], list(g['c_ops']), list(g['e_ops']),
                               Nt=int(g['Nt']), dt=float(g['dt']))
    assert relerr(obs, g['observables']) < RTOL
    for i, k in enumerate(g['snap']):
        assert relerr(rholist[k], g['rho_snap'][i]) < RTOL


def test_dipole_correlation():
    g = load_golden('correlation_2op_chain8')
    cor = ol.correlation_2p_1t(g['H'], g['rho0'], [g['mu'], g['mu']], list(g['c_ops']),
                               float(g['dt']), int(g['Nt']))
    assert relerr(cor, g['cor']) < RTOL


def test_multi_operator_correlations():
    g = load_golden('correlations_n4')
    H, c, ops, rho0, dt = g['H'], list(g['c_ops']), list(g['ops']), g['rho0'], float(g['dt'])
    assert relerr(ol.correlation_3op_1t(H, c, rho0, ops[:3], dt, 30), g['c3op_1t']) < RTOL
    assert relerr(ol.correlation_4op_1t(H, c, rho0, ops, dt, 30), g['c4op_1t']) < RTOL
    assert relerr(ol.correlation_3op_2t(H, c, rho0, ops[:3], dt, 12, 10), g['c3op_2t']) < RTOL
    assert relerr(ol.correlation_4op_2t(H, c, rho0, ops, dt, 12, 10), g['c4op_2t']) < RTOL


def test_redfield_tensor_and_run():
    g = load_golden('redfield_chain8')
    w = chains.redfield_chain(n=8, n_rhs=2, cfg=5)
    # the spectral density the fixture was built with
    assert relerr(w['spectra'][0](g['spectrum_w']), g['spectrum_S']) < 1e-14
    R, evecs = orf.redfield_tensor(g['H'], list(g['a_ops']), w['spectra'])
    # eigenvector phases are LAPACK's choice: compare gauge-free quantities
    assert relerr(np.abs(evecs), np.abs(g['evecs'])) < 1e-9
    # with the fixture's own eigenvectors the tensor itself must agree
    phase = np.sum(evecs.conj() * g['evecs'], axis=0)
    assert np.allclose(np.abs(phase), 1.0, atol=1e-9)
    D = np.diag(phase)
    # R transforms as rho_eb -> D^dag rho_eb D under evecs -> evecs D
    T = np.kron(D.conj().T, D.T)
    assert relerr(T @ R @ np.linalg.inv(T), g['R']) < 1e-9
    obs, rholist = orf.redfield(g['R'], g['rho0'], evecs=g['evecs'], Nt=int(g['Nt']),
                                dt=float(g['dt']), e_ops=list(g['e_ops']))
    assert relerr(obs, g['observables']) < RTOL
    for i, k in enumerate(g['snap']):
        assert relerr(rholist[k], g['rho_snap'][i]) < RTOL


def test_redfield_greens_function():
    g = load_golden('redfield_chain8')
    gf = orf.GreensFunction(g['R'], g['evecs'], 8)
    U = gf.propagator(g['tau'])
    assert relerr(U[:, :, :3], g['U']) < 1e-9
    assert relerr(gf.expect(g['rho0'], list(g['e_ops'][:3])), g['expect']) < 1e-9
    # the reference reuses the propagator cached by propagator(tau) above and
    # ignores the tau passed here (lime/oqs.py:333-336)
    c = gf.correlation_4op_3t(g['rho0'], [g['mu']] * 4, 'llll', g['tau'][:4])
    assert relerr(c, g['c4op_3t']) < 1e-9


def test_superoperators_and_eigen_series():
    g = load_golden('superop_n4')
    H, c = g['H'], list(g['c_ops'])
    assert relerr(osp.liouvillian(H, c), g['L']) < 1e-14
    assert relerr(osp.op2sop(H), g['op2sop_c']) < 1e-15
    assert relerr(osp.op2sop(H, 'left'), g['op2sop_l']) < 1e-15
    assert relerr(osp.op2sop(H, 'right'), g['op2sop_r']) < 1e-15
    assert relerr(osp.op2sop(H, 'anticommutator'), g['op2sop_a']) < 1e-15
    es = osp.EigenSeries(H, c)
    assert relerr(es.evolve(chains.ground_dm(4), g['t'], list(g['e_ops'])), g['evolve']) < 1e-9
    assert relerr(es.correlation_2op_1t(chains.ground_dm(4), [g['a'], g['a']], g['t']),
                  g['cor']) < 1e-9


def test_driven():
    g = load_golden('driven_n4')
    f = lambda t: 0.1 * np.sin(t)
    obs, rholist = ol.lindblad_driven([g['H0'], [g['H1'], f]], chains.ground_dm(4),
                                      list(g['c_ops']), chains.population_ops(4),
                                      Nt=int(g['Nt']), dt=float(g['dt']))
    assert relerr(obs, g['observables']) < RTOL
    assert relerr(rholist[-1], g['rho_final']) < RTOL


def test_fft_convention():
    g = load_golden('fft')
    gg, freq = ospec.fft(g['f'], g['x'])
    assert relerr(gg, g['g']) < 1e-13
    assert relerr(freq, g['freq']) < 1e-15


def test_rk4_against_expm():
    """RK4 on the 16-site chain vs the exact propagator exp(L t) (row-major vec)."""
    import scipy.linalg
    w = chains.single_chain(n_steps=200)
    L = osp.liouvillian(w['H'], w['c_ops'])
    obs, rholist = ol.lindblad(w['H'], w['rho0'], w['c_ops'], Nt=200, dt=w['dt'])
    exact = scipy.linalg.expm(L * 200 * w['dt']) @ osp.dm2vec(w['rho0'])
    assert np.max(np.abs(rholist[-1].flatten() - exact)) < 1e-9


def test_pure_dephasing_two_level():
    """Analytic coherence decay exp(-gamma t) for H = 0 and L = sqrt(g)|0><0|, sqrt(g)|1><1|."""
    gam, dt, Nt = 0.3, 0.01, 300
    H = np.zeros((2, 2), dtype=complex)
    rho0 = np.full((2, 2), 0.5, dtype=complex)
    _, rl = ol.lindblad(H, rho0, chains.dephasing_ops(2, gam), Nt=Nt, dt=dt)
    t = Nt * dt
    assert abs(rl[-1][0, 1] - 0.5 * np.exp(-gam * t)) < 1e-10
