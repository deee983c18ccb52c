"""Driven Lindblad, spectra and the eigen-series solver vs the reference's golden vectors."""
import platform

import numpy as np
import pytest
import torch

from conftest import load_golden
from lime_gb300 import chains

RTOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.gpu
def test_fft_convention_numpy_io():
    """numpy in, numpy out (the reference's types), computed by the
    library's DFT on the device."""
    from lime_gb300.spectra import fft
    g = load_golden('fft')
    gg, freq = fft(g['f'], g['x'], device='cuda')
    assert isinstance(gg, np.ndarray) and isinstance(freq, np.ndarray)
    assert rel(gg, g['g']) < 1e-13 and rel(freq, g['freq']) < 1e-15


@pytest.fixture(scope='module')
def lib():
    from lime_gb300 import build, _native
    build.build()
    return _native.require_device()


@pytest.mark.gpu
def test_driven_matches_reference(lib):
    from lime_gb300.oqs import Lindblad_solver
    g = load_golden('driven_n4')
    f = lambda t: 0.1 * np.sin(t)
    sol = Lindblad_solver([g['H0'], [g['H1'], f]], c_ops=list(g['c_ops']))
    res = sol.evolve(chains.ground_dm(4), dt=float(g['dt']), Nt=int(g['Nt']),
                     e_ops=chains.population_ops(4))
    assert rel(res.observables, g['observables']) < RTOL
    assert rel(res.rholist[-1], g['rho_final']) < RTOL


@pytest.mark.gpu
def test_driven_split_matches_reference(lib):
    """The driven solver on the tensor cores (Heff(t) re-split every step)
    against the reference's golden run, plus a dense-operator 20-site case
    against the FP64 driven path."""
    from lime_gb300.oqs import Lindblad_solver
    g = load_golden('driven_n4')
    f = lambda t: 0.1 * np.sin(t)
    sol = Lindblad_solver([g['H0'], [g['H1'], f]], c_ops=list(g['c_ops']), precision='split')
    res = sol.evolve(chains.ground_dm(4), dt=float(g['dt']), Nt=int(g['Nt']),
                     e_ops=chains.population_ops(4), store_states=False)
    assert np.max(np.abs(res.observables - g['observables'])) < 1e-6
    assert np.max(np.abs(res.rholist[-1] - g['rho_final'])) < 1e-6
    rng = np.random.default_rng(4)
    H0, c_ops = chains.uneven_chain(20, rng, n_ops=2)
    H1 = np.diag(np.linspace(-1, 1, 20)).astype(complex)
    drive = [H0, [H1, lambda t: 0.05 * np.cos(0.3 * t)]]
    e_ops = chains.population_ops(20)[:3]
    r64 = Lindblad_solver(drive, c_ops=c_ops).evolve(chains.ground_dm(20), 0.05, 150, e_ops=e_ops)
    rsp = Lindblad_solver(drive, c_ops=c_ops, precision='split').evolve(
        chains.ground_dm(20), 0.05, 150, e_ops=e_ops, store_states=False)
    assert np.max(np.abs(rsp.observables - r64.observables)) < 1e-6
    assert np.max(np.abs(rsp.rholist[-1] - r64.rholist[-1])) < 1e-6


@pytest.mark.gpu
def test_driven_split_batched_kernel(lib):
    """Dephasing chains (n <= 64, diagonal operators) with a drive run on the
    batched tensor-core kernel, which re-splits Heff(t) = Heff - sum_d c_d
    mu_d every step: per-instance generators, two drive operators, a
    non-Hermitian start, against the FP64 driven path."""
    import torch
    from lime_gb300 import _native, engine
    rng = np.random.default_rng(33)
    n, P, steps, dt = 64, 3, 400, 0.05
    H = np.stack([chains.exciton_chain(n, rng.normal(0, 0.05, n), -0.1) for _ in range(P)])
    gen = engine.LindbladGenerator.build(H, chains.dephasing_ops(n, 0.01))
    assert engine.split_supported(gen) is None
    mu = np.zeros((n, n), dtype=complex)
    mu[0, 1:] = mu[1:, 0] = rng.normal(1.0, 0.1, n - 1)
    mod = np.diag(np.linspace(-0.5, 0.5, n)).astype(complex)
    t = dt * np.arange(1, steps + 1)
    coef = np.stack([0.02 * np.cos(0.2 * t), 0.01 * np.sin(0.05 * t)], 1)
    drive = (torch.as_tensor(np.stack([mu, mod]), device='cuda'), torch.as_tensor(coef, device='cuda'))
    psi = rng.normal(size=n) + 1j * rng.normal(size=n)
    phi = rng.normal(size=n) + 1j * rng.normal(size=n)
    rho0 = np.stack([chains.ground_dm(n), chains.ground_dm(n, 5),
                     np.outer(psi, phi.conj()) / (np.linalg.norm(psi) * np.linalg.norm(phi))])
    e_ops = [chains.population_ops(n)[0], chains.population_ops(n)[5], (mu + mu.conj().T) / 2]
    o64, _, r64 = engine.propagate(gen, rho0, dt, steps, e_ops, drive=drive)
    c0 = _native.launch_count()
    osp, _, rsp = engine.propagate(gen, rho0, dt, steps, e_ops, drive=drive, precision='split')
    torch.cuda.synchronize()
    assert _native.launch_count() - c0 <= 8          # the batched kernel, not the GEMM sequence
    assert np.max(np.abs((osp - o64).cpu().numpy())) < 1e-6
    assert np.max(np.abs((rsp - r64).cpu().numpy())) < 1e-6


@pytest.mark.gpu
def test_driven_complex_coefficients_rejected(lib):
    from lime_gb300.driven import _lindblad_driven
    H0 = np.eye(2, dtype=complex)
    with pytest.raises(ValueError):
        _lindblad_driven([H0, [np.eye(2), lambda t: 1j * t]], chains.ground_dm(2), Nt=2, dt=0.1)


@pytest.mark.gpu
def test_fft_on_device_matches_reference(lib):
    from lime_gb300.spectra import fft
    g = load_golden('fft')
    gg, freq = fft(torch.as_tensor(g['f'], device='cuda'), g['x'])
    assert rel(gg.cpu().numpy(), g['g']) < 1e-13


@pytest.mark.skipif(platform.machine() not in ('x86_64', 'AMD64'),
                    reason='the reference normalises eigenvectors with diag(vl^dag vr).real, so its '
                           'results follow the LAPACK build\'s eigenvector phases; the golden run '
                           'used the x86_64 build')
def test_eigen_series_solver_matches_reference():
    from lime_gb300.superoperator import Lindblad_solver
    g = load_golden('superop_n4')
    es = Lindblad_solver(g['H'], c_ops=list(g['c_ops']))
    es.eigenstates()
    ev = es.evolve(chains.ground_dm(4), g['t'], list(g['e_ops'])).observables
    assert rel(ev, g['evolve']) < 1e-9
    cc = es.correlation_2op_1t(chains.ground_dm(4), [g['a'], g['a']], g['t'])
    assert rel(cc, g['cor']) < 1e-9


@pytest.mark.gpu
def test_eigen_series_two_time_vs_rk4(lib):
    """The eigen-series 3op_2t agrees with the RK4 drop-in up to RK4 truncation."""
    from lime_gb300.superoperator import Lindblad_solver as ES
    from lime_gb300.oqs import Lindblad_solver
    rng = np.random.default_rng(4)
    H, c_ops = chains.uneven_chain(4, rng, n_ops=2)
    ops = [rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)) for _ in range(3)]
    dt, Nt, Ntau = 0.02, 6, 5
    rk = Lindblad_solver(H, c_ops=c_ops).correlation_3op_2t(chains.ground_dm(4), ops, dt, Nt, Ntau)
    es = ES(H, c_ops, exact_norm=True)
    es.eigenstates()
    t = dt * np.arange(1, Nt + 1)
    tau = dt * np.arange(1, Ntau + 1)
    ex = es.correlation_3op_2t(chains.ground_dm(4), ops, t, tau).T
    assert rel(rk, ex) < 1e-7


@pytest.mark.gpu
def test_spectrum_gradient_flows_through_adjoint(lib):
    from lime_gb300.adjoint import chain_observables
    from lime_gb300.spectra import correlation_spectrum
    dev = torch.device('cuda')
    ns, N = 4, 5
    eps = torch.zeros((1, ns), dtype=torch.float64, device=dev, requires_grad=True)
    bond = torch.full((1, ns - 1), -0.1, dtype=torch.float64, device=dev, requires_grad=True)
    gamma = torch.full((1, ns), 0.02, dtype=torch.float64, device=dev, requires_grad=True)
    mu = torch.zeros((N, N), dtype=torch.complex128, device=dev)
    mu[0, 1:] = 1.0
    mu[1:, 0] = 1.0
    rho0 = mu @ torch.as_tensor(chains.ground_dm(N), device=dev)
    H0 = torch.zeros((N, N), dtype=torch.complex128, device=dev)
    cor = chain_observables(H0, eps, bond, gamma, rho0, [mu], 0.05, 64, site0=1, checkpoint=16)
    spec, w = correlation_spectrum(cor[0, :, 0], 0.05)
    spec.real.max().backward()
    assert torch.isfinite(eps.grad).all() and eps.grad.abs().sum() > 0
    assert torch.isfinite(gamma.grad).all() and gamma.grad.abs().sum() > 0
