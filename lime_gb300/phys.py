"""Operator-algebra helpers of the propagation path, drop-in for the ones in
lime/phys.py: ``rk4`` (lime/phys.py:636-649), ``transform`` /
``basis_transform`` (706-730), ``comm`` / ``anticomm`` / ``commutator`` /
``anticommutator`` (737-754), ``dag`` / ``dagger`` (756-762) and ``obs_dm``
(837-844).

Inside the propagators these operations are fused into the kernels (the RK4
combination into every stage epilogue, observables into the epilogue or an
observable pass, the eigenbasis transforms into the Redfield set-up); these
functions serve user code built on them.  Each accepts NumPy arrays (and
scipy.sparse where the reference does) or torch tensors; torch tensors stay
on their device, so CUDA tensors are computed on the GPU.
"""
from __future__ import annotations

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def _is_torch(a) -> bool:
    return torch is not None and isinstance(a, torch.Tensor)


def _mm(a, b):
    if _is_torch(a) or _is_torch(b):
        return a @ b
    return a.dot(b)


def dag(a):
    """Hermitian conjugate."""
    if _is_torch(a):
        return a.conj().transpose(-2, -1).resolve_conj()
    return a.conjugate().transpose()


dagger = dag


def comm(A, B):
    """[A, B] = A B - B A."""
    assert A.shape == B.shape
    return _mm(A, B) - _mm(B, A)


def anticomm(A, B):
    """{A, B} = A B + B A."""
    assert A.shape == B.shape
    return _mm(A, B) + _mm(B, A)


commutator = comm
anticommutator = anticomm


def transform(A, v):
    """A in the basis of the columns of v: v^dag A v."""
    return _mm(dag(v), _mm(A, v))


def basis_transform(A, v):
    """``transform`` returned as a CSR matrix (NumPy/scipy inputs), as the
    reference does; torch tensors are returned dense."""
    out = transform(A, v)
    if _is_torch(out):
        return out
    from scipy.sparse import csr_matrix
    return csr_matrix(out)


def obs_dm(rho, d):
    """Tr(d rho)."""
    if _is_torch(rho) or _is_torch(d):
        return (d * rho.transpose(-2, -1)).sum((-2, -1))
    prod = d.dot(rho)
    return prod.diagonal().sum()


def rk4(rho, fun, dt, *args):
    """One classic RK4 step of d rho/dt = fun(rho, *args), applied to ``rho``
    in place (and returned), as the reference does."""
    dt2 = dt / 2.0
    k1 = fun(rho, *args)
    k2 = fun(rho + k1 * dt2, *args)
    k3 = fun(rho + k2 * dt2, *args)
    k4 = fun(rho + k3 * dt, *args)
    rho += (k1 + 2 * k2 + 2 * k3 + k4) / 6.0 * dt
    return rho
