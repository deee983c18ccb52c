"""Adjoint-kernel gradients vs central finite differences and torch autograd.

Bar: gradients within 1e-5 relative (max |g - g_ref| / max |g_ref|) of
central finite differences of the FP64 forward path, and of torch autograd
through an FP64 torch restatement of the RK4 Lindblad step
(lime/phys.py:636-649, lime/oqs.py:706-723).
"""
import numpy as np
import pytest
import torch

from lime_gb300 import chains

pytestmark = pytest.mark.gpu
GTOL = 1e-5


@pytest.fixture(scope='module', autouse=True)
def _lib():
    from lime_gb300 import build, _native
    build.build()
    _native.require_device()


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def torch_reference(H0, eps, bond, gamma, rho0, E, dt, n_steps, site0):
    """Differentiable FP64 restatement: rk4 with -i[H,rho] + sum_k lindbladian."""
    from lime_gb300.adjoint import chain_hamiltonian
    B, ns = eps.shape
    N = H0.shape[-1]
    H = chain_hamiltonian(H0, eps, bond, site0)
    rho = rho0.expand(B, N, N).to(torch.complex128)
    sites = torch.arange(ns, device=eps.device) + site0

    def L(r):
        out = -1j * (H @ r - r @ H)
        d = torch.diagonal(r, dim1=-2, dim2=-1)[:, sites]          # rho_kk
        # sum_k gamma_k (P_k r P_k - 1/2 {P_k, r})
        g = torch.zeros((B, N), dtype=torch.float64, device=eps.device)
        g[:, sites] = gamma
        gc = g.to(torch.complex128)
        out = out - 0.5 * (gc[:, :, None] * r + r * gc[:, None, :])
        diag = torch.zeros((B, N), dtype=torch.complex128, device=eps.device)
        diag[:, sites] = gamma.to(torch.complex128) * d
        return out + torch.diag_embed(diag)

    obs = []
    for _ in range(n_steps):
        k1 = L(rho)
        k2 = L(rho + k1 * dt / 2)
        k3 = L(rho + k2 * dt / 2)
        k4 = L(rho + k3 * dt)
        rho = rho + (k1 + 2 * k2 + 2 * k3 + k4) / 6. * dt
        obs.append(torch.stack([torch.einsum('ji,bij->b', e, rho) for e in E], -1))
    return torch.stack(obs, 1)


def _loss(obs, w):
    return (torch.conj(w) * obs).real.sum()


def _setup_population(dev):
    n, B = 6, 2
    rng = np.random.default_rng(5)
    eps = torch.tensor(rng.normal(0, 0.05, (B, n)), device=dev)
    bond = torch.tensor(-0.1 + 0.01 * rng.normal(size=(B, n - 1)), device=dev)
    gamma = torch.tensor(rng.uniform(0.005, 0.05, (B, n)), device=dev)
    H0 = torch.zeros((n, n), dtype=torch.complex128, device=dev)
    rho0 = torch.as_tensor(chains.ground_dm(n), device=dev)
    E = [torch.as_tensor(p, device=dev) for p in chains.population_ops(n)]
    return dict(H0=H0, eps=eps, bond=bond, gamma=gamma, rho0=rho0, E=E, site0=0)


def _setup_absorption(dev):
    ns, B = 5, 2
    rng = np.random.default_rng(9)
    N = ns + 1
    eps = torch.tensor(rng.normal(0, 0.05, (B, ns)), device=dev)
    bond = torch.tensor(-0.1 + 0.01 * rng.normal(size=(B, ns - 1)), device=dev)
    gamma = torch.tensor(rng.uniform(0.005, 0.05, (B, ns)), device=dev)
    H0 = torch.zeros((N, N), dtype=torch.complex128, device=dev)
    mu = np.zeros((N, N), dtype=complex)
    mu[0, 1:] = rng.normal(1, 0.1, ns)
    mu[1:, 0] = mu[0, 1:]
    mu_t = torch.as_tensor(mu, device=dev)
    rho0 = mu_t @ torch.as_tensor(chains.ground_dm(N), device=dev)
    return dict(H0=H0, eps=eps, bond=bond, gamma=gamma, rho0=rho0, E=[mu_t], site0=1)


@pytest.mark.parametrize('case', ['population', 'absorption'])
def test_adjoint_matches_autograd_and_finite_differences(case):
    from lime_gb300.adjoint import chain_observables
    dev = torch.device('cuda')
    c = _setup_population(dev) if case == 'population' else _setup_absorption(dev)
    dt, n_steps, K = 0.05, 37, 8          # last checkpoint segment is partial
    eps = c['eps'].clone().requires_grad_(True)
    bond = c['bond'].clone().requires_grad_(True)
    gamma = c['gamma'].clone().requires_grad_(True)
    obs = chain_observables(c['H0'], eps, bond, gamma, c['rho0'], c['E'], dt, n_steps,
                            site0=c['site0'], checkpoint=K)
    g = torch.Generator(device='cpu').manual_seed(3)
    w = torch.complex(torch.randn(obs.shape, generator=g, dtype=torch.float64),
                      torch.randn(obs.shape, generator=g, dtype=torch.float64)).to(dev)
    _loss(obs, w).backward()
    grads = [eps.grad.cpu().numpy(), bond.grad.cpu().numpy(), gamma.grad.cpu().numpy()]

    # torch autograd through the FP64 restatement
    e2 = c['eps'].clone().requires_grad_(True)
    b2 = c['bond'].clone().requires_grad_(True)
    g2 = c['gamma'].clone().requires_grad_(True)
    ref_obs = torch_reference(c['H0'], e2, b2, g2, c['rho0'], c['E'], dt, n_steps, c['site0'])
    assert rel(obs.detach().cpu().numpy(), ref_obs.detach().cpu().numpy()) < 1e-10
    _loss(ref_obs, w).backward()
    refs = [e2.grad.cpu().numpy(), b2.grad.cpu().numpy(), g2.grad.cpu().numpy()]
    for got, ref in zip(grads, refs):
        assert rel(got, ref) < GTOL, (case, rel(got, ref))

    # central finite differences of the CUDA forward path, a few coordinates
    h = 1e-6
    with torch.no_grad():
        for which, (param, got) in enumerate(zip([c['eps'], c['bond'], c['gamma']], grads)):
            for (bi, k) in [(0, 0), (1, param.shape[1] - 1)]:
                vals = []
                for sgn in (+1, -1):
                    p = [c['eps'].clone(), c['bond'].clone(), c['gamma'].clone()]
                    p[which][bi, k] += sgn * h
                    o = chain_observables(c['H0'], p[0], p[1], p[2], c['rho0'], c['E'], dt, n_steps,
                                          site0=c['site0'], checkpoint=K)
                    vals.append(_loss(o, w).item())
                fd = (vals[0] - vals[1]) / (2 * h)
                assert abs(got[bi, k] - fd) <= GTOL * max(np.max(np.abs(got)), 1e-12), (case, which, got[bi, k], fd)


def test_checkpoint_interval_does_not_change_gradients():
    from lime_gb300.adjoint import chain_observables
    dev = torch.device('cuda')
    c = _setup_population(dev)
    out = []
    for K in (1, 5, 64):
        eps = c['eps'].clone().requires_grad_(True)
        obs = chain_observables(c['H0'], eps, c['bond'], c['gamma'], c['rho0'], c['E'], 0.05, 20,
                                checkpoint=K)
        obs.real.sum().backward()
        out.append(eps.grad.cpu().numpy())
    assert rel(out[0], out[2]) < 1e-12 and rel(out[1], out[2]) < 1e-12


def _grads(c, precision, dt, n_steps, K, w=None):
    from lime_gb300.adjoint import chain_observables
    eps = c['eps'].clone().requires_grad_(True)
    bond = c['bond'].clone().requires_grad_(True)
    gamma = c['gamma'].clone().requires_grad_(True)
    obs = chain_observables(c['H0'], eps, bond, gamma, c['rho0'], c['E'], dt, n_steps,
                            site0=c['site0'], checkpoint=K, precision=precision)
    if w is None:
        g = torch.Generator(device='cpu').manual_seed(7)
        w = torch.complex(torch.randn(obs.shape, generator=g, dtype=torch.float64),
                          torch.randn(obs.shape, generator=g, dtype=torch.float64)).to(obs.device)
    _loss(obs, w).backward()
    return obs.detach().cpu().numpy(), [eps.grad.cpu().numpy(), bond.grad.cpu().numpy(),
                                        gamma.grad.cpu().numpy()], w


@pytest.mark.parametrize('case', ['population', 'absorption'])
def test_split_adjoint_matches_fp64_adjoint(case):
    """Tensor-core adjoint (streaming split-precision GEMMs) against the FP64
    adjoint, which the test above pins to autograd and finite differences."""
    dev = torch.device('cuda')
    c = _setup_population(dev) if case == 'population' else _setup_absorption(dev)
    o64, g64, w = _grads(c, 'fp64', 0.05, 37, 8)
    osp, gsp, _ = _grads(c, 'split', 0.05, 37, 8, w)
    assert rel(osp, o64) < 1e-6
    for got, ref in zip(gsp, g64):
        assert rel(got, ref) < GTOL, (case, rel(got, ref))


def test_split_adjoint_source_paths_agree(monkeypatch):
    """The adjoint's observable sources from the fp32 coefficient pairs (the
    host's default) and formed in FP64 inside the kernel (no obs_coef) give
    the same gradients."""
    from lime_gb300 import adjoint
    dev = torch.device('cuda')
    c = _setup_absorption(dev)
    o1, g1, w = _grads(c, 'split', 0.05, 29, 8)
    monkeypatch.setattr(adjoint, '_source_coef', lambda Et: None)
    o2, g2, _ = _grads(c, 'split', 0.05, 29, 8, w)
    assert rel(o1, o2) < 1e-12
    for a, b in zip(g1, g2):
        assert rel(a, b) < 1e-6, rel(a, b)


def test_split_adjoint_large_chain():
    """n = 70 (> 64): the forward runs on the streaming path too."""
    dev = torch.device('cuda')
    n, B = 70, 2
    rng = np.random.default_rng(17)
    c = dict(eps=torch.tensor(rng.normal(0, 0.05, (B, n)), device=dev),
             bond=torch.tensor(-0.1 + 0.01 * rng.normal(size=(B, n - 1)), device=dev),
             gamma=torch.tensor(rng.uniform(0.005, 0.05, (B, n)), device=dev),
             H0=torch.zeros((n, n), dtype=torch.complex128, device=dev),
             rho0=torch.as_tensor(chains.ground_dm(n), device=dev),
             E=[torch.as_tensor(p, device=dev) for p in chains.population_ops(n)[:3]], site0=0)
    o64, g64, w = _grads(c, 'fp64', 0.05, 12, 4)
    osp, gsp, _ = _grads(c, 'split', 0.05, 12, 4, w)
    assert rel(osp, o64) < 1e-6
    for got, ref in zip(gsp, g64):
        assert rel(got, ref) < GTOL, rel(got, ref)


def test_split_adjoint_per_instance_dipoles():
    """The absorption workload's generator: per-realisation dipoles (batched
    observables) and the real loss sum_t Re C(t) of a spectrum."""
    from lime_gb300.adjoint import chain_observables
    dev = torch.device('cuda')
    w = chains.absorption_ensemble(n_sites=9, batch=3, n_steps=24, dt=0.05)
    N = 10
    H0 = torch.zeros((N, N), dtype=torch.complex128, device=dev)
    mu = torch.as_tensor(w['mu'], device=dev)
    rho0 = mu @ torch.as_tensor(w['rho_g'], device=dev)
    out = {}
    for precision in ('fp64', 'split'):
        eps = torch.tensor(w['eps'], device=dev).requires_grad_(True)
        bond = torch.full((3, 8), w['J'], dtype=torch.float64, device=dev).requires_grad_(True)
        gamma = torch.full((3, 9), w['gamma'], dtype=torch.float64, device=dev).requires_grad_(True)
        obs = chain_observables(H0, eps, bond, gamma, rho0, [mu], 0.05, 24, site0=1, checkpoint=8,
                                precision=precision)
        obs.real.sum().backward()
        out[precision] = [eps.grad.cpu().numpy(), bond.grad.cpu().numpy(), gamma.grad.cpu().numpy()]
    for got, ref in zip(out['split'], out['fp64']):
        assert rel(got, ref) < GTOL, rel(got, ref)
