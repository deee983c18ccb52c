"""FFT with the reference sign convention (test infrastructure).

Restates ``lime/fft.py:9-56``: g(w) = int dt f(t) exp(-i w t), computed as
``fftshift(fft(f)) * dx * exp(-i w x[0])`` on ``w = 2 pi fftshift(fftfreq(n, dx))``.
"""
import numpy as np


def fft(f, x=None, axis=-1):
    nx = np.asarray(f).shape[axis]
    if x is None:
        x = np.arange(nx)
    dx = x[1] - x[0]
    g = np.fft.fftshift(np.fft.fft(f, axis=axis), axes=(axis,)) * dx
    freq = 2. * np.pi * np.fft.fftshift(np.fft.fftfreq(nx, d=dx))
    g = g * np.exp(-1j * freq * x[0])
    return g, freq
