"""Seeded synthetic workloads for the open-system propagator.

Each builder returns plain NumPy arrays (complex128) in the layout the
reference solvers take (``lime/oqs.py``: ``Lindblad_solver(H, c_ops)`` with
``H`` (N, N), ``c_ops`` a list of (N, N) arrays, ``rho0`` (N, N)).  Batched
builders stack instances on a leading axis.

Models
------
* Frenkel exciton chain: ``H = diag(eps) + J (|k><k+1| + h.c.)`` with open
  ends, ``eps ~ N(0, sigma)``.
* Pure dephasing: ``L_k = sqrt(gamma) |k><k|``.
* Uneven chains: tridiagonal chain plus ``0.01 * GOE`` with
  ``GOE = (X + X^T)/2``, ``X ~ N(0,1)/sqrt(N)``, and three complex Gaussian
  collapse operators scaled to ``||L||_2^2 = rate``.
* Linear absorption: ground state ``|g>`` (index 0, energy 0) plus an exciton
  chain, dipole ``mu = sum_k d_k (|g><k| + |k><g|)``, ``d_k ~ N(1, 0.1)``,
  ``rho(0) = mu |g><g|``.
* Redfield: exciton chain with site-projector system-bath operators and an
  Ohmic spectral density with exponential cutoff.

Seeds follow ``numpy.random.Generator(PCG64(20261203 + cfg))``.
"""
from __future__ import annotations

import numpy as np

SEED_BASE = 20261203


def rng_for(cfg: int, child: int | None = None) -> np.random.Generator:
    """Generator for workload ``cfg``; ``child`` selects an independent stream."""
    ss = np.random.SeedSequence(SEED_BASE + cfg)
    if child is not None:
        ss = ss.spawn(child + 1)[child]
    return np.random.Generator(np.random.PCG64(ss))


def exciton_chain(n: int, eps: np.ndarray, J: float = -0.1) -> np.ndarray:
    """Tight-binding chain with open ends: diag(eps) + J on the off-diagonals."""
    H = np.diag(np.asarray(eps, dtype=np.float64)).astype(np.complex128)
    idx = np.arange(n - 1)
    H[idx, idx + 1] = J
    H[idx + 1, idx] = J
    return H


def dephasing_ops(n: int, gamma: float) -> list[np.ndarray]:
    """Pure-dephasing collapse operators sqrt(gamma)|k><k|, k = 0..n-1."""
    ops = []
    for k in range(n):
        L = np.zeros((n, n), dtype=np.complex128)
        L[k, k] = np.sqrt(gamma)
        ops.append(L)
    return ops


def population_ops(n: int) -> list[np.ndarray]:
    """Site-population observables |k><k|."""
    ops = []
    for k in range(n):
        P = np.zeros((n, n), dtype=np.complex128)
        P[k, k] = 1.0
        ops.append(P)
    return ops


def ground_dm(n: int, k: int = 0) -> np.ndarray:
    rho = np.zeros((n, n), dtype=np.complex128)
    rho[k, k] = 1.0
    return rho


# ---------------------------------------------------------------- workloads

def single_chain(n: int = 16, n_steps: int = 2000, dt: float = 0.05,
                 gamma: float = 0.01, sigma: float = 0.05, J: float = -0.1,
                 cfg: int = 1) -> dict:
    """Single exciton chain with pure dephasing and population observables.

    Defaults are the 16-site, 2000-step single-instance workload.
    """
    rng = rng_for(cfg)
    eps = rng.normal(0.0, sigma, size=n)
    H = exciton_chain(n, eps, J)
    return dict(H=H, c_ops=dephasing_ops(n, gamma), rho0=ground_dm(n),
                e_ops=population_ops(n), dt=dt, Nt=n_steps)


def disorder_ensemble(n: int = 64, batch: int = 4096, n_steps: int = 4000,
                      dt: float = 0.05, sigma: float = 0.05, J: float = -0.1,
                      gamma_range=(0.005, 0.02), cfg: int = 2) -> dict:
    """Static-disorder ensemble of dephasing exciton chains.

    Returns ``H`` (B, N, N), ``gamma`` (B,) and ``rho0`` (N, N).  Realisation
    ``b`` has ``c_ops = dephasing_ops(n, gamma[b])``.
    """
    rng = rng_for(cfg)
    eps = rng.normal(0.0, sigma, size=(batch, n))
    gamma = rng.uniform(gamma_range[0], gamma_range[1], size=batch)
    H = np.zeros((batch, n, n), dtype=np.complex128)
    idx = np.arange(n)
    H[:, idx, idx] = eps
    H[:, idx[:-1], idx[:-1] + 1] = J
    H[:, idx[:-1] + 1, idx[:-1]] = J
    return dict(H=H, gamma=gamma, rho0=ground_dm(n), dt=dt, Nt=n_steps)


UNEVEN_SIZES = (8, 16, 32, 64, 128, 256)


def uneven_chain(n: int, rng: np.random.Generator, sigma: float = 0.05,
                 J: float = -0.1, goe_scale: float = 0.01, n_ops: int = 3,
                 rate: float = 0.01):
    """One chain of the uneven batch: tridiagonal + GOE, dense collapse ops."""
    eps = rng.normal(0.0, sigma, size=n)
    H = exciton_chain(n, eps, J)
    X = rng.normal(0.0, 1.0, size=(n, n)) / np.sqrt(n)
    H = H + goe_scale * (X + X.T) / 2.0
    c_ops = []
    for _ in range(n_ops):
        L = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
        L *= np.sqrt(rate) / np.linalg.norm(L, 2)
        c_ops.append(L.astype(np.complex128))
    return H.astype(np.complex128), c_ops


def uneven_batch(batch: int = 1024, sizes=UNEVEN_SIZES, n_steps: int = 2000,
                 dt: float = 0.05, cfg: int = 3, limit_n: int | None = None) -> dict:
    """Batch of chains with N drawn uniformly from ``sizes``.

    Returns lists ``H``, ``c_ops``, ``rho0`` (one entry per chain) and ``ns``.
    ``limit_n`` drops chains above that size (for small test cases).
    """
    rng = rng_for(cfg)
    ns = rng.choice(np.asarray(sizes), size=batch)
    Hs, Cs, R0 = [], [], []
    keep = []
    for b, n in enumerate(ns):
        crng = rng_for(cfg, child=b)
        H, c_ops = uneven_chain(int(n), crng)
        if limit_n is not None and n > limit_n:
            continue
        keep.append(int(n))
        Hs.append(H)
        Cs.append(c_ops)
        R0.append(ground_dm(int(n)))
    return dict(H=Hs, c_ops=Cs, rho0=R0, ns=np.asarray(keep), dt=dt, Nt=n_steps)


def absorption_chain(n_sites: int, rng: np.random.Generator, sigma: float = 0.05,
                     J: float = -0.1, gamma: float = 0.01, d_mean: float = 1.0,
                     d_sigma: float = 0.1):
    """Ground state plus an exciton chain, for the dipole correlation function.

    Index 0 is |g> (energy 0, rotating frame); indices 1..n_sites are sites.
    Returns ``H``, ``mu``, ``eps`` (site energies), ``d`` (dipoles) and the
    site-dephasing collapse operators.
    """
    dim = n_sites + 1
    eps = rng.normal(0.0, sigma, size=n_sites)
    d = rng.normal(d_mean, d_sigma, size=n_sites)
    H = np.zeros((dim, dim), dtype=np.complex128)
    H[1:, 1:] = exciton_chain(n_sites, eps, J)
    mu = np.zeros((dim, dim), dtype=np.complex128)
    mu[0, 1:] = d
    mu[1:, 0] = d
    c_ops = []
    for k in range(n_sites):
        L = np.zeros((dim, dim), dtype=np.complex128)
        L[k + 1, k + 1] = np.sqrt(gamma)
        c_ops.append(L)
    return dict(H=H, mu=mu, eps=eps, d=d, c_ops=c_ops)


def absorption_ensemble(n_sites: int = 128, batch: int = 256, n_steps: int = 4096,
                        dt: float = 0.05, gamma: float = 0.01, cfg: int = 4) -> dict:
    """Disorder ensemble for the linear absorption workload.

    Returns ``H`` (B, D, D), ``mu`` (B, D, D), ``eps`` (B, n_sites),
    ``d`` (B, n_sites), ``gamma`` and the ground-state ``rho_g``.
    """
    dim = n_sites + 1
    Hs = np.zeros((batch, dim, dim), dtype=np.complex128)
    mus = np.zeros_like(Hs)
    eps = np.zeros((batch, n_sites))
    ds = np.zeros((batch, n_sites))
    for b in range(batch):
        m = absorption_chain(n_sites, rng_for(cfg, child=b), gamma=gamma)
        Hs[b], mus[b], eps[b], ds[b] = m['H'], m['mu'], m['eps'], m['d']
    return dict(H=Hs, mu=mus, eps=eps, d=ds, gamma=gamma, rho_g=ground_dm(dim),
                dt=dt, Nt=n_steps, J=-0.1)


def ohmic_spectrum(lam: float = 0.05, omega_c: float = 0.1, kT: float = 0.025):
    """Bath correlation spectrum S(w) of an Ohmic bath with exponential cutoff.

    ``J(w) = (pi lam / omega_c) w exp(-|w|/omega_c)`` (odd in w) and
    ``S(w) = 2 J(w) / (1 - exp(-w/kT))`` (detailed balance
    ``S(-w) = exp(-w/kT) S(w)``), with the limit ``S(0) = 2 pi lam kT / omega_c``.
    The callable accepts scalars and arrays.
    """
    eta = np.pi * lam / omega_c

    def S(w):
        w = np.asarray(w, dtype=np.float64)
        small = np.abs(w) < 1e-12
        ws = np.where(small, 1.0, w)
        val = 2.0 * eta * ws * np.exp(-np.abs(ws) / omega_c) / (-np.expm1(-ws / kT))
        out = np.where(small, 2.0 * eta * kT, val)
        return out if out.ndim else float(out)

    return S


def redfield_chain(n: int = 96, n_rhs: int = 512, n_steps: int = 2000,
                   dt: float = 0.05, cfg: int = 5, lam: float = 0.05,
                   omega_c: float = 0.1, kT: float = 0.025) -> dict:
    """Exciton chain with site-projector bath couplings and an Ohmic bath.

    ``rho0`` is (n_rhs, N, N): random pure states |psi><psi| with complex
    Gaussian amplitudes.
    """
    rng = rng_for(cfg)
    eps = rng.normal(0.0, 0.05, size=n)
    H = exciton_chain(n, eps, -0.1)
    a_ops = population_ops(n)
    S = ohmic_spectrum(lam, omega_c, kT)
    psi = rng.normal(size=(n_rhs, n)) + 1j * rng.normal(size=(n_rhs, n))
    psi /= np.linalg.norm(psi, axis=1, keepdims=True)
    rho0 = np.einsum('bi,bj->bij', psi, psi.conj())
    return dict(H=H, a_ops=a_ops, spectra=[S] * n, rho0=rho0, dt=dt, Nt=n_steps)
