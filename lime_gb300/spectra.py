"""Spectra from propagated correlation functions.

``fft`` follows lime/fft.py:9-56: g(w) = int dt f(t) exp(-i w t), computed as
``fftshift(fft(f)) * dx * exp(-i w x[0])`` on ``w = 2 pi fftshift(fftfreq(n, dx))``.
It runs on the device (torch.fft) and accepts torch tensors that require
grad, so the gradient of a spectrum flows back through the correlation
function into the adjoint propagator (``lime_gb300.adjoint``).
"""
from __future__ import annotations

import math

import numpy as np
import torch


def _as_tensor(f, device):
    if isinstance(f, torch.Tensor):
        return f.to(device=device, dtype=torch.complex128)
    return torch.as_tensor(np.asarray(f), dtype=torch.complex128, device=device)


def fft(f, x=None, axis=-1, device=None):
    """Fourier transform with the reference sign and phase convention.

    Returns ``(g, freq)``; numpy arrays for numpy input, tensors for tensor input.
    """
    is_t = isinstance(f, torch.Tensor)
    dev = f.device if is_t else (device or ('cuda' if torch.cuda.is_available() else 'cpu'))
    ft = _as_tensor(f, dev)
    nx = ft.shape[axis]
    if x is None:
        x = np.arange(nx)
    x = np.asarray(x.detach().cpu() if isinstance(x, torch.Tensor) else x, dtype=np.float64)
    dx = float(x[1] - x[0])
    g = torch.fft.fftshift(torch.fft.fft(ft, dim=axis), dim=axis) * dx
    freq = 2. * math.pi * torch.fft.fftshift(torch.fft.fftfreq(nx, d=dx, device=dev, dtype=torch.float64))
    shape = [1] * ft.dim()
    shape[axis] = nx
    g = g * torch.exp(-1j * freq * float(x[0])).reshape(shape)
    if is_t:
        return g, freq
    return g.cpu().numpy(), freq.cpu().numpy()


def correlation_spectrum(cor, dt, t0=0.0, device=None):
    """Spectrum of a correlation function recorded after each step.

    ``cor[..., k]`` is C(t0 + (k+1) dt) (the timing of
    ``Lindblad_solver.correlation_2op_1t``, lime/oqs.py:777-787); returns
    ``fft(cor, t)`` on that grid.
    """
    n = (cor.shape[-1] if isinstance(cor, torch.Tensor) else np.shape(cor)[-1])
    t = t0 + dt * np.arange(1, n + 1)
    return fft(cor, t, device=device)
