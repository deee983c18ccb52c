"""Complex128 contractions on the library's strided batched GEMM
(``lime_zgemm_strided_f64``): the propagator and Green's-function
contractions of the Redfield solver (lime/oqs.py:169-366) and the
eigenbasis transforms (lime/phys.py:706-718), without copies of strided
views and without torch matmul/einsum."""
from __future__ import annotations

import torch

from . import _native as nat

CDT = torch.complex128


def _view3(x: torch.Tensor):
    """(tensor without the lazy conjugate bit, conj flag) of a complex128
    3-d device view."""
    if x.dtype != CDT or x.dim() != 3 or x.device.type != 'cuda':
        raise ValueError('expected a 3-d complex128 CUDA tensor, got %s %s on %s'
                         % (tuple(x.shape), x.dtype, x.device))
    if x.is_conj():
        return x.conj(), 1
    return x, 0


def bmm(A: torch.Tensor, B: torch.Tensor, conj_a: bool = False, conj_b: bool = False,
        scale: torch.Tensor | None = None, out: torch.Tensor | None = None) -> torch.Tensor:
    """C[z] = op(A[z]) diag(scale[z]) op(B[z]).

    ``A`` (Z|1, M, K), ``B`` (Z|1, K, N), ``scale`` (Z|1, K) or None, any
    strides (a batch of 1 broadcasts); op conjugates.  ``out``: a (Z, M, N)
    view written in place (any strides), else a new contiguous tensor.
    """
    A, ca = _view3(A)
    B, cb = _view3(B)
    Z = max(A.shape[0], B.shape[0], 1 if scale is None else scale.shape[0])
    M, K = A.shape[1], A.shape[2]
    if B.shape[1] != K:
        raise ValueError('inner dimensions %d and %d differ' % (K, B.shape[1]))
    N = B.shape[2]
    for x, nm in ((A, 'A'), (B, 'B')):
        if x.shape[0] not in (1, Z):
            raise ValueError('batch of %s is %d, not 1 or %d' % (nm, x.shape[0], Z))
    if out is None:
        out = torch.empty((Z, M, N), dtype=CDT, device=A.device)
    elif tuple(out.shape) != (Z, M, N) or out.dtype != CDT or out.is_conj():
        raise ValueError('out must be a (%d, %d, %d) complex128 view' % (Z, M, N))
    if M == 0 or N == 0 or Z == 0:
        return out
    if K == 0:
        out.zero_()
        return out
    d = nat.ZgemmDesc()
    d.M, d.N, d.K, d.batch = M, N, K, Z
    d.conj_a, d.conj_b = int(bool(conj_a) ^ ca), int(bool(conj_b) ^ cb)
    d.A = A.data_ptr()
    d.a_rs, d.a_cs = A.stride(1), A.stride(2)
    d.a_bs = A.stride(0) if A.shape[0] > 1 else 0
    d.B = B.data_ptr()
    d.b_rs, d.b_cs = B.stride(1), B.stride(2)
    d.b_bs = B.stride(0) if B.shape[0] > 1 else 0
    if scale is not None:
        if scale.dtype != CDT or scale.dim() != 2 or scale.shape[1] != K or scale.shape[0] not in (1, Z):
            raise ValueError('scale must be (1|%d, %d) complex128' % (Z, K))
        if scale.is_conj():
            scale = scale.resolve_conj()
        d.scale = scale.data_ptr()
        d.s_ks = scale.stride(1)
        d.s_bs = scale.stride(0) if scale.shape[0] > 1 else 0
    d.C = out.data_ptr()
    d.c_rs, d.c_cs, d.c_bs = out.stride(1), out.stride(2), out.stride(0)
    lib = nat.require_device()
    nat.check(lib.lime_zgemm_strided_f64(d, torch.cuda.current_stream(A.device).cuda_stream),
              'lime_zgemm_strided_f64')
    return out


def mm(A: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
    """A @ B for 2-d complex128 device tensors."""
    return bmm(A.unsqueeze(0), B.unsqueeze(0))[0]


def to_basis(V: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
    """V^dag X V for X (n, n) or (B, n, n) (lime/phys.py:706-718)."""
    Xb = X.unsqueeze(0) if X.dim() == 2 else X
    Vb = V.unsqueeze(0)
    t = bmm(Vb.transpose(1, 2), Xb, conj_a=True)
    out = bmm(t, Vb)
    return out[0] if X.dim() == 2 else out


def from_basis(V: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
    """V X V^dag for X (n, n) or (B, n, n)."""
    Xb = X.unsqueeze(0) if X.dim() == 2 else X
    Vb = V.unsqueeze(0)
    t = bmm(Vb, Xb)
    out = bmm(t, Vb.transpose(1, 2), conj_b=True)
    return out[0] if X.dim() == 2 else out


def green_apply(G: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
    """Y[a, k, ...] = sum_b G[a, b, k] X[b, ...] (``tensordot(G, X,
    dims=([1], [0]))`` for a propagator G of shape (D, D, Nt))."""
    D, D2, Nt = G.shape
    rest = tuple(X.shape[1:])
    m = 1
    for r in rest:
        m *= r
    Xm = X.reshape(D2, m)
    Y = torch.empty((D, Nt) + rest, dtype=CDT, device=G.device)
    # batch over k: A = G[:, :, k] (strides of the (D, D, Nt) layout), B = X
    bmm(G.permute(2, 0, 1), Xm.unsqueeze(0), out=Y.reshape(D, Nt, m).permute(1, 0, 2))
    return Y
