"""Spectra from propagated correlation functions.

``fft`` follows lime/fft.py:9-56: g(w) = int dt f(t) exp(-i w t), computed as
``fftshift(fft(f)) * dx * exp(-i w x[0])`` on ``w = 2 pi fftshift(fftfreq(n, dx))``.
The transform, the shift and the phase run in one call of the library's
batched FP64 DFT (``lime_fft_f64``) on the device.  Tensor inputs may
require grad: the backward pass is the adjoint map (conjugate phase,
unshift, the transform with the opposite sign), so the gradient of a
spectrum flows back through the correlation function into the adjoint
propagator (``lime_gb300.adjoint``).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _native as nat

CDT = torch.complex128


def _as_tensor(f, device):
    if isinstance(f, torch.Tensor):
        return f.to(device=device, dtype=CDT)
    return torch.as_tensor(np.asarray(f), dtype=CDT, device=device)


def _freq(nx: int, dx: float) -> np.ndarray:
    """2 pi fftshift(fftfreq(nx, dx)) (numpy's layout)."""
    k = np.arange(nx)
    f = np.where(k < (nx + 1) // 2, k, k - nx) / (nx * dx)
    return 2.0 * math.pi * np.roll(f, nx // 2)


def _dft_rows(x: torch.Tensor, inverse: bool, shift: bool, post: torch.Tensor | None) -> torch.Tensor:
    """lime_fft_f64 over the last axis of a contiguous (B, n) complex128 tensor."""
    lib = nat.require_device()
    B, n = x.shape
    y = torch.empty_like(x)
    wsb = int(lib.lime_fft_f64_workspace(n, B))
    ws = torch.empty(max(wsb, 16), dtype=torch.uint8, device=x.device)
    d = nat.FftDesc()
    d.n, d.batch, d.inverse, d.shift = n, B, int(inverse), int(shift)
    d.x, d.x_s, d.x_bs = x.data_ptr(), 1, n
    d.y, d.y_s, d.y_bs = y.data_ptr(), 1, n
    if post is not None:
        d.post = post.data_ptr()
    d.workspace, d.workspace_bytes = ws.data_ptr(), wsb
    nat.check(lib.lime_fft_f64(d, torch.cuda.current_stream(x.device).cuda_stream), 'lime_fft_f64')
    return y


class _Spectrum(torch.autograd.Function):
    """y = post * shift(DFT(x)) along the last axis of (B, n); the adjoint is
    DFT^dag(unshift(conj(post) * g)), DFT^dag the transform of opposite sign."""

    @staticmethod
    def forward(ctx, x, post):
        ctx.save_for_backward(post)
        return _dft_rows(x.contiguous(), False, True, post)

    @staticmethod
    def backward(ctx, g):
        (post,) = ctx.saved_tensors
        n = g.shape[-1]
        h = torch.roll(g * post.conj(), -(n // 2), dims=-1).contiguous()
        return _dft_rows(h, True, False, None), None


def fft(f, x=None, axis=-1, device=None):
    """Fourier transform with the reference sign and phase convention.

    Returns ``(g, freq)``; numpy arrays for numpy input, tensors for tensor input.
    """
    is_t = isinstance(f, torch.Tensor)
    dev = f.device if is_t else (device or ('cuda' if torch.cuda.is_available() else 'cpu'))
    if torch.device(dev).type != 'cuda':
        raise RuntimeError('lime_gb300.spectra.fft runs on the GPU (lime_fft_f64); no CUDA device given')
    ft = _as_tensor(f, dev)
    nx = ft.shape[axis]
    if x is None:
        x = np.arange(nx)
    x = np.asarray(x.detach().cpu() if isinstance(x, torch.Tensor) else x, dtype=np.float64)
    dx = float(x[1] - x[0])
    freq = _freq(nx, dx)
    post = torch.as_tensor(dx * np.exp(-1j * freq * float(x[0])), dtype=CDT, device=dev)
    moved = ft.movedim(axis, -1)
    lead = moved.shape[:-1]
    g = _Spectrum.apply(moved.reshape(-1, nx), post).reshape(lead + (nx,)).movedim(-1, axis)
    fr = torch.as_tensor(freq, dtype=torch.float64, device=dev)
    if is_t:
        return g, fr
    return g.detach().cpu().numpy(), freq


def correlation_spectrum(cor, dt, t0=0.0, device=None):
    """Spectrum of a correlation function recorded after each step.

    ``cor[..., k]`` is C(t0 + (k+1) dt) (the timing of
    ``Lindblad_solver.correlation_2op_1t``, lime/oqs.py:777-787); returns
    ``fft(cor, t)`` on that grid.
    """
    n = (cor.shape[-1] if isinstance(cor, torch.Tensor) else np.shape(cor)[-1])
    t = t0 + dt * np.arange(1, n + 1)
    return fft(cor, t, device=device)
