"""Liouville-space builders with the conventions of ``lime/superoperator.py``.

Row-major vectorisation (``dm2vec(rho) = rho.flatten()``,
lime/superoperator.py:131-151): ``vec(A rho B) = (A kron B^T) vec(rho)``.
These return ``scipy.sparse`` matrices exactly like the reference builders
(lime/superoperator.py:30-59, 186-271); they are set-up utilities, not part
of the propagation loop, which never forms a Lindblad superoperator.
"""
from __future__ import annotations

import numpy as np
from scipy.sparse import coo_matrix, identity, issparse
from scipy.sparse import kron as _kron


def kron(a, b):
    """scipy.sparse.kron returning a sparse matrix for dense or sparse inputs."""
    return _kron(coo_matrix(a), b)


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


class Lindblad_solver:
    """Eigen-series Liouville-space solver (lime/superoperator.py:456-773).

    Diagonalises the dense Liouvillian (left and right eigenvectors, LAPACK
    through scipy, as the reference) and evaluates observables and
    correlation functions as closed-form sums of exp(lambda t).  O(N^6): a
    cross-check for small systems (N <~ 30), not a propagation path.

    The reference normalises with ``diag(vl^dag vr).real``
    (lime/superoperator.py:512), which drops the imaginary part of complex
    overlaps, so its results depend on LAPACK's eigenvector phases and do not
    reproduce rho0 at t = 0.  ``exact_norm=True`` keeps the complex overlap
    and gives the exact exp(L t); the default reproduces the reference.
    """

    def __init__(self, H, c_ops=None, exact_norm=False):
        self.H = H
        self.c_ops = c_ops
        self.L = None
        self.dim = H.shape[-1] ** 2
        self.idv = operator_to_vector(np.identity(H.shape[-1]))
        self.left_eigvecs = None
        self.right_eigvecs = None
        self.eigvals = None
        self.norm = None
        self.exact_norm = exact_norm

    def liouvillian(self):
        self.L = liouvillian(self.H, self.c_ops)
        return self.L

    def eigenstates(self, k=None):
        import scipy.linalg
        if self.L is None:
            self.liouvillian()
        w, vl, vr = scipy.linalg.eig(_dense(self.L), left=True, right=True)
        self.eigvals, self.left_eigvecs, self.right_eigvecs = w, vl, vr
        ov = np.diagonal(vl.conj().T @ vr)
        self.norm = ov if self.exact_norm else ov.real
        return w, vr, vl

    def _coeff_rho(self, v):
        return (self.left_eigvecs.conj().T @ v) / self.norm

    def evolve(self, rho0, tlist, e_ops):
        from .result import Result
        res = Result(times=tlist)
        U1, w = self.right_eigvecs, self.eigvals
        c = self._coeff_rho(operator_to_vector(rho0))
        out = np.zeros((len(tlist), len(e_ops)), dtype=np.complex128)
        evs = [operator_to_vector(_dense(e).conj().T) for e in e_ops]
        for i, t in enumerate(tlist):
            rho = U1 @ (c * np.exp(w * t))
            out[i, :] = [np.vdot(ev, rho) for ev in evs]
        res.observables = out
        return res

    def _left_coeff(self, a):
        la = _dense(left(a))
        return np.array([np.vdot(self.idv, la @ self.right_eigvecs[:, m])
                         for m in range(self.right_eigvecs.shape[1])])

    def correlation_2op_1t(self, rho0, ops, tlist):
        a, b = ops
        coeff = self._left_coeff(a) * self._coeff_rho(operator_to_vector(_dense(b) @ _dense(rho0)))
        return np.array([np.sum(np.exp(self.eigvals * t) * coeff) for t in tlist])

    def correlation_2op_1w(self, rho0, ops, w):
        a, b = ops
        coeff = self._left_coeff(a) * self._coeff_rho(operator_to_vector(_dense(b) @ _dense(rho0)))
        return np.array([np.sum(-1. / (self.eigvals + 1j * wi) * coeff) for wi in w])

    def correlation_3op_1t(self, rho0, ops, t):
        a, b, c = ops
        coeff = self._left_coeff(b) * self._coeff_rho(
            operator_to_vector(_dense(c) @ _dense(rho0) @ _dense(a)))
        return np.array([np.sum(np.exp(self.eigvals * ti) * coeff) for ti in t])

    def correlation_3op_1w(self, rho0, ops, w):
        a, b, c = ops
        coeff = self._left_coeff(b) * self._coeff_rho(
            operator_to_vector(_dense(c) @ _dense(rho0) @ _dense(a)))
        return np.array([np.sum(-1. / (self.eigvals + 1j * wi) * coeff) for wi in w])

    def correlation_3op_2t(self, rho0, ops, tlist, taulist, k=None):
        a, b, c = ops
        U1, U2, norm = self.right_eigvecs, self.left_eigvecs, self.norm
        r0 = operator_to_vector(_dense(rho0))
        lb = self._left_coeff(b)
        ra_lc = _dense(right(_dense(a))) @ _dense(left(_dense(c)))
        mid = (U2.conj().T @ ra_lc @ U1) / norm[:, None]
        coeff = lb[:, None] * mid * ((U2.conj().T @ r0) / norm)[None, :]
        tmp1 = np.exp(np.outer(self.eigvals, taulist))
        tmp2 = np.exp(np.outer(self.eigvals, tlist))
        return tmp1.T @ coeff @ tmp2

    def correlation_4op_2t(self, rho0, ops, tlist, taulist, k=None):
        if len(ops) != 4:
            raise ValueError('Number of operators is not 4.')
        a, b, c, d = ops
        return self.correlation_3op_2t(rho0, [a, _dense(b) @ _dense(c), d], tlist, taulist, k)
