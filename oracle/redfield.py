"""NumPy restatement of the reference Bloch-Redfield path (test infrastructure).

* ``redfield_tensor``  lime/oqs.py:528-579.  eigh(H); C_k[n,m] = S_k(-(E_n-E_m));
  A_k = V^dag a_k V; Lambda_k = C_k * A_k;
  R = sum_k op2sop(A_k) (left(Lambda_k) - right(Lambda_k^dag));
  returns ``-1j op2sop(diag E) - R`` (the generator: d vec(rho)/dt = L vec(rho))
  and the eigenvectors.  Dense here; the reference returns csr.
* ``redfield``         lime/oqs.py:373-468 (_redfield, return_result=True):
  rho0 and e_ops to the eigenbasis, row-major vec, RK4 with rhs = R.dot,
  rholist transformed back to the site basis, observables in the eigenbasis
  at t = (k+1) dt.
* ``propagator/expect/correlation_2op_1t/correlation_4op_3t`` lime/oqs.py:169-366
  (eigen-series Green's-function route).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg

from .lindblad import rk4, transform, dag, obs_dm
from .superop import op2sop, left, right, dm2vec


def is_herm(a):
    return np.allclose(a, dag(a))


def spectra_matrix(S, W):
    """C[n, m] = S(-W[n, m]) evaluated pointwise as the reference does."""
    n = W.shape[0]
    C = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            C[i, j] = S(-W[i, j])
    return C


def redfield_tensor(H, a_ops, spectra):
    for a in a_ops:
        if not is_herm(a):
            raise TypeError("Operators in a_ops must be Hermitian.")
    evals, evecs = scipy.linalg.eigh(H)
    W = np.real(evals[:, None] - evals[None, :])
    K = len(a_ops)
    cache = {}
    C = []
    for k in range(K):
        key = id(spectra[k])
        if key not in cache:
            cache[key] = spectra_matrix(spectra[k], W)
        C.append(cache[key])
    A = [transform(a, evecs) for a in a_ops]
    Lam = [C[k] * A[k] for k in range(K)]
    R = 0
    for k in range(K):
        R = R + op2sop(A[k]) @ (left(Lam[k]) - right(dag(Lam[k])))
    return -1j * op2sop(np.diag(evals)) - R, evecs


def redfield(R, rho0, evecs=None, Nt=1, dt=0.005, e_ops=None, store_states=True):
    """RK4 on vec(rho) (lime/oqs.py:373-468); returns (observables, rholist)."""
    N = rho0.shape[0]
    e_ops = [] if e_ops is None else list(e_ops)
    if evecs is not None:
        rho0 = transform(rho0, evecs)
        e_ops = [transform(e, evecs) for e in e_ops]
    rho = dm2vec(np.array(rho0, copy=True)).astype(np.complex128)
    obs = np.zeros((Nt, len(e_ops)), dtype=np.complex128)
    rholist = []
    rhs = lambda psi, L: L @ psi
    for k in range(Nt):
        rho = rk4(rho, rhs, dt, R)
        tmp = rho.reshape(N, N)
        if store_states:
            rholist.append(transform(tmp, dag(evecs)) if evecs is not None else tmp.copy())
        obs[k, :] = [obs_dm(tmp, e) for e in e_ops]
    return obs, rholist


class GreensFunction:
    """Eigen-series propagator of the Redfield generator (lime/oqs.py:169-366)."""

    def __init__(self, R, evecs, dim):
        self.R, self.evecs, self.dim = R, evecs, dim
        self.U = None
        self.G = None

    def propagator(self, t):
        evals1, U1 = scipy.linalg.eig(self.R)
        U2 = scipy.linalg.inv(U1)
        E = np.exp(evals1[:, None] * np.asarray(t)[None, :])
        self.U = np.einsum('aj,jk,jb->abk', U1, E, U2)
        self.G = -1j * self.U
        return self.U

    def expect(self, rho0, e_ops):
        rho0_eb = dm2vec(transform(rho0, self.evecs))
        e_ops = [transform(e, self.evecs) for e in e_ops]
        rho = np.tensordot(self.U, rho0_eb, axes=([1], [0]))
        out = np.zeros((self.U.shape[-1], len(e_ops)), dtype=np.complex128)
        for j, e in enumerate(e_ops):
            out[:, j] = dm2vec(e) @ rho
        return out

    def correlation_2op_1t(self, rho0, a, b, tau):
        if self.G is None:
            self.propagator(tau)
        idm = dm2vec(np.identity(self.dim))
        if rho0.ndim == 2:
            rho0 = dm2vec(rho0)
        return idm @ (a @ np.tensordot(self.G, b @ rho0, axes=([1], [0])))

    def correlation_4op_3t(self, rho0, oplist, signature, tau):
        if len(oplist) != 4:
            raise ValueError('Number of operators is not 4.')
        a, b, c, d = [op2sop(o, s) for o, s in zip(oplist, signature)]
        if self.G is None:
            self.propagator(tau)
        G = self.G
        idm = dm2vec(np.identity(self.dim))
        rho = d @ dm2vec(rho0)
        tmp = np.tensordot(G, rho, axes=((1), (0)))
        tmp = c @ tmp
        tmp = np.tensordot(G, tmp, axes=([1], [0]))
        tmp = np.tensordot(b, tmp, axes=([1], [0]))
        tmp = np.tensordot(G, tmp, axes=([1], [0]))
        return np.einsum('a,ab,bijk->ijk', idm, a, tmp)
