"""Liouville-space restatement of lime/superoperator.py (test infrastructure).

Row-major vectorisation throughout: ``dm2vec(rho) = rho.flatten()``
(lime/superoperator.py:131-151), so ``vec(A rho B) = (A kron B^T) vec(rho)``.

* ``op2sop``             lime/superoperator.py:186-247 (commutator/left/right/anticommutator)
* ``left/right``         lime/superoperator.py:257-271
* ``lindblad_dissipator``lime/superoperator.py:250-252
* ``liouvillian``        lime/superoperator.py:30-59
* ``EigenSeries``        lime/superoperator.py:456-773 (Lindblad_solver: eig with
                         left and right vectors, closed-form exp(lambda t) sums)
* ``sort``               lime/liouville.py:45-52 (order by |eigenvalue|)
"""
from __future__ import annotations

import numpy as np
import scipy.linalg


def dm2vec(rho):
    return np.asarray(rho).flatten()


def op2sop(a, kind='commutator'):
    a = np.asarray(a)
    n = a.shape[-1]
    idm = np.identity(n)
    if kind in ('commutator', 'c', '-'):
        return np.kron(a, idm) - np.kron(idm, a.T)
    if kind in ('left', 'l'):
        return np.kron(a, idm)
    if kind in ('right', 'r'):
        return np.kron(idm, a.T)
    if kind in ('anticommutator', 'a', '+'):
        return np.kron(a, idm) + np.kron(idm, a.T)
    raise ValueError('Error: superoperator {} does not exist.'.format(kind))


def left(a):
    return op2sop(a, 'left')


def right(a):
    return op2sop(a, 'right')


def lindblad_dissipator(l):
    l = np.asarray(l)
    return np.kron(l, l.conj()) - 0.5 * op2sop(l.conj().T @ l, 'anticommutator')


def liouvillian(H, c_ops):
    """Dense -i op2sop(H) + sum_k D[L_k] (lime/superoperator.py:30-59)."""
    L = -1j * op2sop(H)
    for c in (c_ops or []):
        L = L + lindblad_dissipator(c)
    return L


def sort(eigvals, eigvecs):
    idx = np.argsort(np.abs(eigvals))
    return eigvals[idx], eigvecs[:, idx]


class EigenSeries:
    """Exact e^{Lt} through eig of the dense Liouvillian (N <~ 30)."""

    def __init__(self, H, c_ops):
        n = H.shape[-1]
        self.n = n
        self.L = liouvillian(H, c_ops)
        w, vl, vr = scipy.linalg.eig(self.L, left=True, right=True)
        self.w, self.vl, self.vr = w, vl, vr
        self.norm = np.diagonal(vl.conj().T @ vr).real
        self.idv = dm2vec(np.identity(n))

    def evolve(self, rho0, tlist, e_ops):
        coeff = (self.vl.conj().T @ dm2vec(rho0)) / self.norm
        out = np.zeros((len(tlist), len(e_ops)), dtype=np.complex128)
        for i, t in enumerate(tlist):
            rho = self.vr @ (coeff * np.exp(self.w * t))
            out[i] = [np.vdot(dm2vec(e.conj().T), rho) for e in e_ops]
        return out

    def correlation_2op_1t(self, rho0, ops, tlist):
        a, b = ops
        c1 = np.array([np.vdot(self.idv, left(a) @ self.vr[:, n])
                       for n in range(self.vr.shape[1])])
        c2 = (self.vl.conj().T @ dm2vec(b @ rho0)) / self.norm
        coeff = c1 * c2
        return np.array([np.sum(np.exp(self.w * t) * coeff) for t in tlist])
