"""FP64 RK4 references in PyTorch (cuBLAS complex128 GEMMs) for measuring
the split-precision paths' error over the full horizons of the configured
workloads (test and bench infrastructure, not part of the library).

The library's FP64 kernels run one CTA per density matrix, which is the right
shape for ensembles but takes minutes for a handful of large instances over
thousands of steps (a 129-dimensional chain, a 256-dimensional chain with
dense collapse operators, one 9216-dimensional Redfield right-hand side).
These references apply the same equations with whole-GPU cuBLAS calls, one
RK4 step captured as a CUDA graph and replayed:

* ``lindblad_rk4``  f(rho) = -i (Heff rho - rho Heff^dag) + M o rho
                    + sum_k L_k rho L_k^dag (the generator of
                    lime/oqs.py:706-723 in the library's Heff form), RK4 of
                    lime/phys.py:636-649; observables Tr(E rho)
                    (lime/phys.py:837-844) after every obs_every-th step
* ``redfield_rk4``  d vec(rho)/dt = R vec(rho) on a block of right-hand
                    sides (lime/oqs.py:453-472)

Both agree with the library's FP64 kernels to rounding (checked in the
tests that use them).
"""
from __future__ import annotations

import torch


def _rk4_graph(f, x, dt):
    """CUDA graph of one in-place RK4 step x <- x + dt/6 (k1 + 2k2 + 2k3 + k4)
    of x' = f(x); f is captured with its closure's static tensors."""
    def step():
        k1 = f(x)
        k2 = f(x + k1 * (dt / 2))
        k3 = f(x + k2 * (dt / 2))
        k4 = f(x + k3 * dt)
        x.add_((k1 + 2 * k2 + 2 * k3 + k4) / 6. * dt)

    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(2):   # warm-up on the capture stream, as CUDA graphs require
            keep = x.clone()
            step()
            x.copy_(keep)
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        step()
    return g


def lindblad_rk4(gen, rho0: torch.Tensor, dt: float, n_steps: int, E=None, obs_every: int = 1,
                 hermitian: bool = False):
    """RK4 of (B, n, n) complex128 states under ``gen`` (an
    ``engine.LindbladGenerator``: its FP64 Heff, M and dense collapse
    operators).  Per stage three GEMMs: [Heff; L_1..L_K] rho, rho Heff^dag
    (or (Heff rho)^dag when ``hermitian``: the states stay Hermitian) and
    [L_1 rho | .. | L_K rho] [L_1^dag; ..; L_K^dag].  Returns (obs (B,
    n_steps // obs_every, n_obs), final rho)."""
    x = rho0.to(torch.complex128).contiguous().clone()
    B, n = x.shape[0], x.shape[-1]
    heff = gen.heff
    hd = heff.mH.contiguous()
    m = gen.m
    L = gen.l_dense
    K = 0 if L is None else L.shape[1]
    A = heff if L is None else torch.cat([heff.unsqueeze(1), L], 1).reshape(L.shape[0], (K + 1) * n, n)
    Ld = None if L is None else L.mH.reshape(L.shape[0], K * n, n).contiguous()

    def f(r):
        Y = A @ r                                        # (B, (K+1) n, n)
        X = Y[:, :n]
        out = -1j * (X - (X.mH if hermitian else r @ hd))
        if m is not None:
            out = out + m * r
        if K:
            Yc = Y[:, n:].reshape(B, K, n, n).permute(0, 2, 1, 3).reshape(B, n, K * n)
            out = out + Yc @ Ld
        return out

    g = _rk4_graph(f, x, float(dt))
    x.copy_(rho0)
    n_obs = 0 if E is None else E.shape[-3]
    obs = torch.zeros((B, n_steps // obs_every, n_obs), dtype=torch.complex128, device=x.device)
    for s in range(n_steps):
        g.replay()
        if n_obs and (s + 1) % obs_every == 0:
            # Tr(E rho) = sum_ij E_ji rho_ij; E is (n_obs, n, n) or (B, n_obs, n, n)
            eq = 'oji,bij->bo' if E.dim() == 3 else 'boji,bij->bo'
            obs[:, (s + 1) // obs_every - 1] = torch.einsum(eq, E, x)
    return obs, x


def redfield_rk4(R: torch.Tensor, rho0: torch.Tensor, dt: float, n_steps: int, E=None, obs_every: int = 1):
    """RK4 of eigenbasis states (B, n, n) under the dense generator R
    (D x D, row-major vec).  Returns (obs (B, n_steps // obs_every, n_obs),
    final rho (B, n, n))."""
    B, n = rho0.shape[0], rho0.shape[-1]
    D = n * n
    x = rho0.reshape(B, D).transpose(0, 1).contiguous().to(torch.complex128)   # D x B
    start = x.clone()

    def f(s):
        # one matrix-vector product per right-hand side: cuBLAS runs a
        # skinny complex128 GEMM (D x D by D x 2) about 9x slower than two
        # matrix-vector products on this part
        return torch.stack([torch.mv(R, s[:, j]) for j in range(s.shape[1])], 1)

    g = _rk4_graph(f, x, float(dt))
    x.copy_(start)
    n_obs = 0 if E is None else E.shape[0]
    Et = None if E is None else E.transpose(-2, -1).reshape(n_obs, D)   # Tr(E rho) = vec(E^T) . vec(rho)
    obs = torch.zeros((B, n_steps // obs_every, n_obs), dtype=torch.complex128, device=x.device)
    for s in range(n_steps):
        g.replay()
        if n_obs and (s + 1) % obs_every == 0:
            obs[:, (s + 1) // obs_every - 1] = (Et @ x).transpose(0, 1)
    return obs, x.transpose(0, 1).reshape(B, n, n)
