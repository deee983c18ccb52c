"""The strided batched complex128 GEMM (lime_zgemm_strided_f64) behind the
Redfield Green's-function route and the eigenbasis transforms, against
torch complex128 matmul: strided and broadcast operands, conjugation, the
per-(batch, k) scale, batches above one grid's z extent, and the
Green's-function contraction over a (D, D, Nt) propagator."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
CDT = torch.complex128


@pytest.fixture(scope='module', autouse=True)
def _lib():
    from lime_gb300 import build, _native
    build.build()
    _native.require_device()


def _rand(*shape, seed=0):
    g = torch.Generator(device='cpu').manual_seed(seed)
    x = torch.randn(shape, dtype=torch.float64, generator=g) + 1j * torch.randn(shape, dtype=torch.float64,
                                                                                 generator=g)
    return x.to(CDT).cuda()


def _close(a, b, tol=1e-13):
    assert (a - b).abs().max().item() <= tol * max(1.0, b.abs().max().item())


@pytest.mark.parametrize('Z,M,N,K', [(1, 1, 1, 1), (3, 70, 65, 130), (5, 64, 128, 17), (2, 129, 3, 64)])
def test_bmm_matches_torch(Z, M, N, K):
    from lime_gb300 import zlinalg as zl
    A, B = _rand(Z, M, K, seed=1), _rand(Z, K, N, seed=2)
    _close(zl.bmm(A, B), A @ B)
    _close(zl.bmm(A, B, conj_a=True, conj_b=True), A.conj() @ B.conj())
    # strided (transposed) views, broadcast batch, lazy conjugate views
    At = _rand(Z, K, M, seed=3).transpose(1, 2)
    B1 = _rand(1, K, N, seed=4)
    _close(zl.bmm(At, B1), At @ B1)
    _close(zl.bmm(At.conj(), B1), At.conj() @ B1)
    # scale: A diag(s[z]) B
    s = _rand(Z, K, seed=5)
    _close(zl.bmm(A, B, scale=s), (A * s[:, None, :]) @ B)
    # written into a strided output view
    out = torch.zeros((M, Z, N), dtype=CDT, device='cuda')
    zl.bmm(A, B, out=out.permute(1, 0, 2))
    _close(out.permute(1, 0, 2), A @ B)


def test_bmm_batch_above_grid_limit():
    from lime_gb300 import zlinalg as zl
    A, B = _rand(70000, 2, 3, seed=6), _rand(70000, 3, 1, seed=7)
    _close(zl.bmm(A, B), A @ B)


def test_green_apply_and_transforms():
    from lime_gb300 import zlinalg as zl
    D, Nt = 36, 7
    G = _rand(D, D, Nt, seed=8)
    X = _rand(D, 5, 3, seed=9)
    _close(zl.green_apply(G, X), torch.tensordot(G, X, dims=([1], [0])))
    V, _ = torch.linalg.qr(_rand(6, 6, seed=10))
    R = _rand(4, 6, 6, seed=11)
    _close(zl.to_basis(V, R), V.mH @ R @ V)
    _close(zl.from_basis(V, R), V @ R @ V.mH)
    _close(zl.to_basis(V, R[0]), V.mH @ R[0] @ V)


def test_bad_arguments_rejected():
    from lime_gb300 import _native as nat
    lib = nat.require_device()
    d = nat.ZgemmDesc()
    assert lib.lime_zgemm_strided_f64(None, None) < 0
    assert lib.lime_zgemm_strided_f64(d, None) < 0          # zero sizes, null pointers
    x = _rand(1, 2, 2)
    d.M = d.N = d.K = d.batch = 2
    d.A = d.B = d.C = x.data_ptr()
    d.conj_a = 2
    assert lib.lime_zgemm_strided_f64(d, None) < 0
