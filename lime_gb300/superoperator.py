"""Liouville-space builders with the conventions of ``lime/superoperator.py``.

Row-major vectorisation (``dm2vec(rho) = rho.flatten()``,
lime/superoperator.py:131-151): ``vec(A rho B) = (A kron B^T) vec(rho)``.
These return ``scipy.sparse`` matrices exactly like the reference builders
(lime/superoperator.py:30-59, 186-271); they are set-up utilities, not part
of the propagation loop, which never forms a Lindblad superoperator.
"""
from __future__ import annotations

import numpy as np
from scipy.sparse import identity, issparse, kron


def _dense(a):
    return a.toarray() if issparse(a) else np.asarray(a)


def dm2vec(rho):
    if issparse(rho):
        n, m = rho.shape
        return rho.tolil().reshape((n * m, 1))
    return np.asarray(rho).flatten()


def operator_to_vector(rho):
    return np.asarray(_dense(rho)).flatten()


def operator_to_superoperator(a, kind='commutator'):
    N = a.shape[-1]
    idm = identity(N)
    if kind in ('commutator', 'c', '-'):
        return kron(a, idm) - kron(idm, a.T)
    if kind in ('left', 'l'):
        return kron(a, idm)
    if kind in ('right', 'r'):
        return kron(idm, a.T)
    if kind in ('anticommutator', 'a', '+'):
        return kron(a, idm) + kron(idm, a.T)
    raise ValueError('Error: superoperator {} does not exist.'.format(kind))


def op2sop(a, kind='commutator'):
    return operator_to_superoperator(a, kind=kind)


def to_super(a, kind='commutator'):
    return operator_to_superoperator(a, kind=kind)


def left(a):
    return kron(a, identity(_dense(a).shape[-1]))


def right(a):
    return kron(identity(_dense(a).shape[-1]), a.T)


def kraus(a):
    return right(_dense(a).conj().T).dot(left(a))


def lindblad_dissipator(l):
    ld = _dense(l)
    return kron(l, ld.conj()) - 0.5 * operator_to_superoperator(ld.conj().T.dot(ld), kind='anticommutator')


def liouvillian(H, c_ops):
    """-i op2sop(H) + sum_k D[L_k] (lime/superoperator.py:30-59), csr."""
    L = -1j * operator_to_superoperator(H)
    for c in (c_ops or []):
        L = L + lindblad_dissipator(c)
    return L.tocsr()


def obs(rho, a):
    return np.vdot(operator_to_vector(_dense(a).conj().T), rho)


def trace(rho):
    import math
    n = math.isqrt(len(rho))
    return np.vdot(operator_to_vector(np.identity(n)), rho)


def sort(eigvals, eigvecs):
    """Order by |eigenvalue| (lime/liouville.py:45-52)."""
    idx = np.argsort(np.abs(eigvals))
    return eigvals[idx], eigvecs[:, idx]
