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


@pytest.mark.parametrize('P', [0, 1, 151, 304, 305, 912, 929, 4096, 4100, 12345])
@pytest.mark.parametrize('slots', [1, 7, 304])
def test_pipeline_ranges(P, slots):
    """The ranges tile [0, P) in order; all but a partial last one are whole
    rounds, at most four; the number of rounds is that of one launch."""
    from lime_gb300.engine import pipeline_chunks
    ch = pipeline_chunks(P, slots)
    lo = 0
    rounds = 0
    for a, b in ch:
        assert a == lo and b > a
        size = b - a
        if b < P or P % slots == 0:
            assert size % slots == 0 and size // slots <= 4
        rounds += -(-size // slots)
        lo = b
    assert lo == P
    assert rounds == -(-P // slots)
    if P % slots:
        assert ch[-1] == (P - P % slots, P)                # the partial round alone


def test_pipeline_operand_classification():
    from lime_gb300.engine import DiagonalOps, SiteDephasing, _per_instance
    P, n = 10, 4
    assert _per_instance(np.zeros((P, n, n)), P) is True
    assert _per_instance(np.zeros((1, n, n)), P) is False
    assert _per_instance(np.zeros((n, n)), P) is False
    assert _per_instance(np.zeros((3, n, n)), P) is None
    assert _per_instance(SiteDephasing(np.ones((P, n))), P) is True
    assert _per_instance(SiteDephasing(np.ones(n)), P) is False
    assert _per_instance(DiagonalOps(np.ones((P, 2, n))), P) is True
    assert _per_instance(DiagonalOps(np.ones((2, n))), P) is False
    assert _per_instance(torch.zeros((P, n, n)), P) is True


def test_pipeline_needs_a_gpu_batch_to_engage():
    """Without a GPU (or for a device H) the pipeline declines and the caller
    takes the one-launch path."""
    from lime_gb300.engine import Populations, SiteDephasing, propagate_host_pipelined
    if torch.cuda.is_available():
        pytest.skip('checks the CPU-only answer')
    H = np.zeros((4096, 8, 8), dtype=np.complex128)
    assert propagate_host_pipelined(H, np.eye(8) / 8, [SiteDephasing(np.ones(8))], Populations(8),
                                    0.05, 4) is None


def test_pipeline_upload_slices_each_operand_form():
    """_upload (here onto the CPU device) takes instances lo:hi of a per-
    instance operand in each accepted form and converts it to the kernels'
    dtypes; a shared operand is copied whole."""
    import scipy.sparse as sp
    from lime_gb300.engine import DiagonalOps, SiteDephasing, _upload
    cpu = torch.device('cpu')
    P, n = 6, 3
    H = np.arange(P * n * n, dtype=np.float64).reshape(P, n, n)
    got = _upload(H, cpu, 2, 5)
    assert got.dtype == torch.complex128 and tuple(got.shape) == (3, n, n)
    assert np.array_equal(got.numpy().real, H[2:5])
    got = _upload(torch.as_tensor(H).to(torch.complex128), cpu, 1, 2)
    assert np.array_equal(got.numpy().real, H[1:2])
    r = _upload(SiteDephasing(np.ones((P, n)) * np.arange(P)[:, None]), cpu, 3, 6)
    assert isinstance(r, SiteDephasing) and r.rates.dtype == torch.float64
    assert np.array_equal(r.rates.numpy()[:, 0], [3, 4, 5])
    l = _upload(DiagonalOps(np.ones((P, 2, n))), cpu, 0, 4)
    assert isinstance(l, DiagonalOps) and tuple(l.l.shape) == (4, 2, n) and l.l.dtype == torch.complex128
    s = _upload(sp.csr_matrix(np.eye(n)), cpu)
    assert np.array_equal(s.numpy(), np.eye(n))
    # a non-contiguous per-instance array is sliced before it is made contiguous
    Hf = np.asfortranarray(H)
    assert np.array_equal(_upload(Hf, cpu, 4, 6).numpy().real, H[4:6])
