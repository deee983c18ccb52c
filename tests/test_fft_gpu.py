"""The library's batched FP64 DFT (lime_fft_f64) and lime's fft convention
on it (lime_gb300.spectra): against numpy.fft for power-of-two lengths
(in-shared-memory radix 2) and other lengths (Bluestein), strided rows,
both signs, the fused fftshift and phase, and the autograd adjoint against
torch autograd through torch.fft."""
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


def _rows(B, n, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(B, n)) + 1j * rng.normal(size=(B, n))


@pytest.mark.parametrize('n', [1, 2, 3, 5, 8, 12, 100, 128, 1000, 1024, 4095, 4096, 8192])
def test_dft_matches_numpy(n):
    from lime_gb300.spectra import _dft_rows
    B = 3
    x = _rows(B, n, n)
    xt = torch.as_tensor(x, device='cuda')
    y = _dft_rows(xt, False, False, None).cpu().numpy()
    ref = np.fft.fft(x, axis=-1)
    assert np.max(np.abs(y - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))
    yi = _dft_rows(xt, True, False, None).cpu().numpy()
    refi = np.fft.ifft(x, axis=-1) * n
    assert np.max(np.abs(yi - refi)) <= 1e-12 * max(1.0, np.max(np.abs(refi)))


def test_strided_rows_and_shift_with_post():
    from lime_gb300 import _native as nat
    lib = nat.require_device()
    n, B = 64, 4
    x = torch.as_tensor(_rows(n, B, 1), device='cuda')       # transform down the columns
    y = torch.zeros((n, B), dtype=CDT, device='cuda')
    post = torch.as_tensor(np.exp(1j * np.arange(n)), dtype=CDT, device='cuda')
    d = nat.FftDesc()
    d.n, d.batch, d.inverse, d.shift = n, B, 0, 1
    d.x, d.x_s, d.x_bs = x.data_ptr(), B, 1
    d.y, d.y_s, d.y_bs = y.data_ptr(), B, 1
    d.post = post.data_ptr()
    assert lib.lime_fft_f64(d, torch.cuda.current_stream().cuda_stream) == 0
    ref = np.fft.fftshift(np.fft.fft(x.cpu().numpy(), axis=0), axes=0) * post.cpu().numpy()[:, None]
    assert np.max(np.abs(y.cpu().numpy() - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_lime_fft_convention_and_gradient():
    from lime_gb300.spectra import fft
    n = 300
    t = 0.05 * np.arange(1, n + 1)
    x = torch.as_tensor(_rows(2, n, 7), device='cuda').requires_grad_(True)
    g, w = fft(x, t)
    # the convention of lime/fft.py:9-56, in numpy
    xn = x.detach().cpu().numpy()
    dx = t[1] - t[0]
    freq = 2 * np.pi * np.fft.fftshift(np.fft.fftfreq(n, d=dx))
    ref = np.fft.fftshift(np.fft.fft(xn, axis=-1), axes=(-1,)) * dx * np.exp(-1j * freq * t[0])
    assert np.max(np.abs(g.detach().cpu().numpy() - ref)) <= 1e-12 * np.max(np.abs(ref))
    assert np.max(np.abs(w.cpu().numpy() - freq)) <= 1e-12 * np.max(np.abs(freq))
    # the adjoint against autograd through torch.fft
    wts = torch.as_tensor(_rows(2, n, 8), device='cuda')
    (g * wts).real.sum().backward()
    xr = x.detach().clone().requires_grad_(True)
    post = torch.as_tensor(dx * np.exp(-1j * freq * t[0]), device='cuda')
    gr = torch.fft.fftshift(torch.fft.fft(xr, dim=-1), dim=-1) * post
    (gr * wts).real.sum().backward()
    assert (x.grad - xr.grad).abs().max().item() <= 1e-12 * xr.grad.abs().max().item()


def test_axis_and_unsupported_length():
    from lime_gb300 import _native as nat
    from lime_gb300.spectra import fft
    x = _rows(5, 16, 9)
    g0, _ = fft(x.T, axis=0)
    g1, _ = fft(x, axis=-1)
    assert np.max(np.abs(g0.T - g1)) <= 1e-13 * np.max(np.abs(g1))
    with pytest.raises(nat.LimeError):
        fft(torch.zeros(5000, dtype=CDT, device='cuda'))
