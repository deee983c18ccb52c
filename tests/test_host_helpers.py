"""Host-side helpers of the device paths, on the CPU: the frequency grid of
lime's fft convention, the diagonal-observable test of the streaming path,
and the validation of the strided GEMM wrapper."""
import numpy as np
import pytest
import torch


@pytest.mark.parametrize('n', [1, 2, 3, 8, 9, 100, 4096])
@pytest.mark.parametrize('dx', [0.05, 1.0, 0.3])
def test_fft_frequency_grid_matches_numpy(n, dx):
    from lime_gb300.spectra import _freq
    ref = 2 * np.pi * np.fft.fftshift(np.fft.fftfreq(n, d=dx))
    assert np.max(np.abs(_freq(n, dx) - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))


def test_diagonal_observable_detection():
    from lime_gb300.engine import _is_diag_host
    for n in (1, 2, 5):
        d = np.diag(np.arange(1, n + 1)).astype(complex)
        assert _is_diag_host(d) and _is_diag_host(np.stack([d, 2 * d]))
        for i in range(n):
            for j in range(n):
                if i != j:
                    e = d.copy()
                    e[i, j] = 1e-300
                    assert not _is_diag_host(e)
    assert not _is_diag_host(np.zeros((2, 3)))


def test_zgemm_wrapper_rejects_bad_operands():
    from lime_gb300 import zlinalg as zl
    a = torch.zeros((1, 2, 2), dtype=torch.complex128)
    with pytest.raises(ValueError):
        zl.bmm(a, a)                                   # not on a CUDA device
    with pytest.raises(ValueError):
        zl.bmm(torch.zeros((2, 2), dtype=torch.complex128), a)   # not 3-d
