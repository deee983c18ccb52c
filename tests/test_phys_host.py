"""The operator-algebra helpers (lime_gb300.phys) against the oracle's
restatement of lime/phys.py, on NumPy inputs and on torch tensors (CPU here;
the same code runs on CUDA tensors)."""
import numpy as np
import torch
from scipy.sparse import csr_matrix

from lime_gb300 import phys
from oracle import lindblad as ol


def _mats(n=6, seed=0):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    B = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    v, _ = np.linalg.qr(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    return A, B, v


def test_algebra_matches_oracle_numpy():
    A, B, v = _mats()
    assert np.allclose(phys.dag(A), ol.dag(A), rtol=0, atol=0)
    assert np.allclose(phys.comm(A, B), ol.comm(A, B), rtol=1e-14, atol=1e-14)
    assert np.allclose(phys.anticomm(A, B), ol.anticomm(A, B), rtol=1e-14, atol=1e-14)
    assert np.allclose(phys.transform(A, v), ol.transform(A, v), rtol=1e-14, atol=1e-14)
    assert np.allclose(phys.basis_transform(A, v).toarray(), ol.transform(A, v), rtol=1e-14, atol=1e-14)
    assert np.isclose(phys.obs_dm(A, B), ol.obs_dm(A, B), rtol=1e-14)
    # sparse operators, as the reference accepts
    assert np.isclose(phys.obs_dm(A, csr_matrix(B)), ol.obs_dm(A, B), rtol=1e-14)


def test_algebra_on_torch_tensors():
    A, B, v = _mats(seed=1)
    At, Bt, vt = (torch.as_tensor(x) for x in (A, B, v))
    assert np.allclose(phys.dag(At).numpy(), ol.dag(A))
    assert np.allclose(phys.comm(At, Bt).numpy(), ol.comm(A, B), rtol=1e-13, atol=1e-13)
    assert np.allclose(phys.anticomm(At, Bt).numpy(), ol.anticomm(A, B), rtol=1e-13, atol=1e-13)
    assert np.allclose(phys.transform(At, vt).numpy(), ol.transform(A, v), rtol=1e-13, atol=1e-13)
    assert np.isclose(complex(phys.obs_dm(At, Bt)), ol.obs_dm(A, B), rtol=1e-13)


def test_rk4_in_place_matches_oracle():
    rng = np.random.default_rng(2)
    H = rng.normal(size=(5, 5)); H = (H + H.T) / 2
    fun = lambda r, h: -1j * (h @ r - r @ h)
    r1 = np.eye(5, dtype=complex) / 5 + 0.01j * (H - H.T)
    r2 = r1.copy()
    out = phys.rk4(r1, fun, 0.05, H)
    assert out is r1                    # in place, as the reference
    ol.rk4(r2, fun, 0.05, H)
    assert np.array_equal(r1, r2)
