"""Gradients of Lindblad observables through the discrete RK4 adjoint.

``chain_observables`` propagates density matrices of a Frenkel-chain model

    H = H0 + sum_k eps_k |s_k><s_k| + sum_k J_k (|s_k><s_{k+1}| + h.c.)
    c_ops = { sqrt(gamma_k) |s_k><s_k| }_k          (s_k = site0 + k)

with the FP64 RK4 propagator (the time loop of ``_lindblad``,
lime/oqs.py:1590-1688) and returns the observables ``Tr(E rho(t))`` as a
differentiable torch tensor.  Its backward pass runs the hand-written
adjoint kernel (``lime_lindblad_adjoint_f64``): states are checkpointed every
``checkpoint`` steps in the forward pass and recomputed segment by segment,
and the gradients with respect to every site energy, bond coupling and
dephasing rate are accumulated in FP64 on the device.

Non-Hermitian starting states (the dipole correlation <mu(t) mu(0)> starts
from mu|g><g|) run as their two Hermitian parts rho = A + iB; for complex
observables torch's convention dL = Re sum conj(grad) d(obs) makes the
source of the B chain ``-i grad``.

``precision='split'`` runs the same computation on the tensor cores: the
forward pass segment by segment through the split-precision propagators
(keeping the checkpoints), the backward pass through
``lime_lindblad_adjoint_stream`` (the same discrete adjoint on the streaming
split-precision GEMMs).
"""
from __future__ import annotations

import math

import torch

from . import _native as nat
from . import engine

CDT = torch.complex128


def chain_hamiltonian(H0: torch.Tensor, eps: torch.Tensor, bond: torch.Tensor, site0: int) -> torch.Tensor:
    """H0 (B|1, N, N) + diag(eps) + bonds on sites site0..site0+n_sites-1."""
    B, ns = eps.shape
    N = H0.shape[-1]
    H = H0.expand(B, N, N).clone().to(CDT)
    idx = torch.arange(ns, device=H.device) + site0
    H[:, idx, idx] += eps.to(CDT)
    if ns > 1:
        H[:, idx[:-1], idx[1:]] += bond.to(CDT)
        H[:, idx[1:], idx[:-1]] += bond.to(CDT)
    return H


def dephasing_diagonals(gamma: torch.Tensor, N: int, site0: int) -> torch.Tensor:
    """l (B, n_sites, N) with l[b, k, site0+k] = sqrt(gamma[b, k])."""
    B, ns = gamma.shape
    l = torch.zeros((B, ns, N), dtype=CDT, device=gamma.device)
    k = torch.arange(ns, device=gamma.device)
    l[:, k, k + site0] = torch.sqrt(gamma).to(CDT)
    return l


def _forward_split(gen, work, dt, n_steps, E, obs_every, B, K):
    """Split-precision forward in segments of K steps: observables and the
    states at steps 0, K, 2K, ... (the checkpoints, complex128)."""
    ckpts, parts = [], []
    done = 0
    while done < n_steps:
        seg = min(K, n_steps - done)
        ckpts.append(work.clone())
        if engine.split_supported(gen) is None:
            o, _, status = engine._run_split(gen, work, dt, seg, E, obs_every, 1e-5, param_batch=B)
        else:
            o, _, status, work, _ = engine._run_stream(gen, work, dt, seg, E, obs_every, param_batch=B)
        flags = int(status.item())
        if flags:
            raise nat.KernelFlagError(flags, 'chain_observables forward (split)')
        parts.append(o)
        done += seg
    return torch.cat(parts, 1), torch.stack(ckpts, 0).contiguous()


def _pow2_scale(bound: float) -> int:
    """Largest power-of-two exponent s with 1.25 * bound * 2^s <= 2^13."""
    if not bound > 0 or not math.isfinite(bound):
        return 0
    return max(-60, min(60, int(math.floor(math.log2(8192.0 / (1.25 * bound))))))


def _source_coef(Et: torch.Tensor) -> torch.Tensor:
    """fp32 coefficient pairs of the observable sources (the kernel forms
    Re g Q.x + Im g Q.y): Et (P|1, n_obs, N, N) -> (P|1, n_obs, 2, N, N, 2),
    index [.., x, row] with A = E[x, row], B = E[row, x]."""
    A, Bt = Et, Et.transpose(-1, -2)
    re = torch.stack([(A.real + Bt.real) / 2, (A.imag + Bt.imag) / 2], -1)
    im = torch.stack([(Bt.imag - A.imag) / 2, (A.real - Bt.real) / 2], -1)
    return torch.stack([re, im], 2).to(torch.float32).contiguous()


def _backward_split(heff, m, ckpts, gsrc, Et, n_obs, dt, n_steps, obs_every, K, B, N, max_retries=2):
    """The discrete adjoint on the tensor cores (lime_lindblad_adjoint_stream)."""
    lib = nat.require_device()
    dev = heff.device
    C = gsrc.shape[0]
    heff_adj = (-heff.mH).contiguous()
    m_adj = None if m is None else m.conj().contiguous()
    # a diagonal M (pure dephasing) goes in as its real diagonal
    m_diag = None
    if m is not None and engine.is_diagonal(m):
        m_diag = torch.diagonal(m, dim1=-2, dim2=-1).real.contiguous()
    shared = heff.shape[0] == 1
    G = 1 if shared else B
    # rho is scaled by its largest element over the checkpoints (the
    # evolution contracts); the adjoint stage inputs are scaled per step on
    # the device from max |lam|
    pmax = float(torch.view_as_real(ckpts).abs().max().item())
    sb = _pow2_scale(pmax)
    qcoef = _source_coef(Et) if n_obs > 0 else None
    wsb = lib.lime_lindblad_adjoint_stream_workspace(N, C, G, K)
    ws = torch.empty(wsb + 1024, dtype=torch.uint8, device=dev)
    aligned = (ws.data_ptr() + 1023) // 1024 * 1024
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    for attempt in range(max_retries + 1):
        gd = torch.zeros((C, N), dtype=torch.float64, device=dev)
        gb = torch.zeros((C, max(N - 1, 1)), dtype=torch.float64, device=dev)
        gg = torch.zeros((C, N), dtype=torch.float64, device=dev)
        status.zero_()
        d = nat.AdjointStreamDesc()
        d.n, d.batch, d.param_batch, d.n_steps, d.seg_steps = N, C, B, n_steps, K
        d.n_obs, d.obs_every = n_obs, obs_every
        d.scale_b_log2, d.scale_l_log2 = sb, 0
        d.dt = float(dt)
        d.ckpt = ckpts.data_ptr()
        d.heff, d.heff_stride = heff.data_ptr(), (0 if shared else N * N)
        d.heff_adj, d.heff_adj_stride = heff_adj.data_ptr(), (0 if shared else N * N)
        if m_diag is not None:
            d.m_diag, d.m_diag_stride = m_diag.data_ptr(), (0 if m_diag.shape[0] == 1 else N)
        elif m is not None:
            d.m, d.m_adj = m.data_ptr(), m_adj.data_ptr()
            d.m_stride = 0 if m.shape[0] == 1 else N * N
        if n_obs > 0:
            d.obs_ops, d.obs_stride = Et.data_ptr(), (0 if Et.shape[0] == 1 else n_obs * N * N)
            d.obs_grad = gsrc.data_ptr()
            if qcoef is not None:
                d.obs_coef = qcoef.data_ptr()
        d.grad_diag, d.grad_bond, d.grad_gamma = gd.data_ptr(), gb.data_ptr(), gg.data_ptr()
        d.workspace, d.workspace_bytes = aligned, wsb
        d.status = status.data_ptr()
        nat.check(lib.lime_lindblad_adjoint_stream(d, torch.cuda.current_stream().cuda_stream),
                  'lime_lindblad_adjoint_stream')
        flags = int(status.item())
        if flags & nat.LIME_FLAG_RANGE and attempt < max_retries:
            sb -= 2
            continue
        if flags:
            raise nat.KernelFlagError(flags, 'chain_observables backward (split)')
        return gd, gb, gg


class _ChainObservables(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps, bond, gamma, H0, rho0, E, dt, n_steps, site0, obs_every, checkpoint, precision):
        dev = eps.device
        B, ns = eps.shape
        N = H0.shape[-1]
        H = chain_hamiltonian(H0, eps.detach(), bond.detach(), site0)
        l = dephasing_diagonals(gamma.detach(), N, site0)
        gen = engine.LindbladGenerator.build(H, [engine.DiagonalOps(l)], device=dev)
        rho = rho0.to(device=dev, dtype=CDT)
        if rho.dim() == 2:
            rho = rho.unsqueeze(0).expand(B, N, N)
        herm = bool(torch.equal(rho, rho.mH))
        if herm:
            work = rho.clone().contiguous()
        else:
            a, b = engine.hermitian_parts(rho)
            work = torch.cat([a, b], 0).contiguous()
        ckpt0 = work.clone()
        obs = engine.prepare_obs(list(E), N, B, dev)
        K = max(1, min(checkpoint, n_steps))
        if precision == 'split':
            if K % obs_every:
                raise ValueError('precision="split" needs checkpoint to be a multiple of obs_every')
            o, states = _forward_split(gen, work, dt, n_steps, list(E), obs_every, B, K)
            Ed = None
            if len(E):
                # dense observables, per instance (B, n_obs, N, N) when any is batched
                if any(e.dim() == 3 for e in E):
                    Ed = torch.stack([(e.expand(B, N, N) if e.dim() == 2 else e).to(CDT) for e in E], 1)
                else:
                    Ed = torch.stack([e.to(CDT) for e in E], 0).unsqueeze(0)
                Ed = Ed.contiguous()
            obs = (Ed, len(E), 0, 0)
        else:
            o, states, status = engine._run_f64(gen, work, dt, n_steps, obs, obs_every, K, 0.0,
                                                param_batch=B)
            flags = int(status.item())
            if flags:
                raise nat.KernelFlagError(flags, 'chain_observables forward')
        if not herm:
            o_out = o[:B] + 1j * o[B:]
        else:
            o_out = o
        ctx.save_for_backward(gen.heff, gen.m, ckpt0, states, obs[0])
        ctx.meta = (B, N, ns, herm, dt, n_steps, site0, obs_every, K, obs[1], obs[2], obs[3], precision)
        return o_out.clone()

    @staticmethod
    def backward(ctx, g):
        heff, m, ckpt0, states, Et = ctx.saved_tensors
        B, N, ns, herm, dt, n_steps, site0, obs_every, K, n_obs, obs_diag, obs_stride, precision = ctx.meta
        lib = nat.require_device()
        dev = heff.device
        g = g.to(CDT).contiguous()
        gsrc = g if herm else torch.cat([g, -1j * g], 0).contiguous()
        C = gsrc.shape[0]                       # number of Hermitian chains x B
        if precision == 'split':
            gd, gb, gg = _backward_split(heff, m, states, gsrc, Et, n_obs, dt, n_steps, obs_every, K, B, N)
            return _finish_grads(gd, gb, gg, herm, B, ns, site0)
        heff_adj = (-heff.mH).contiguous()
        m_adj = None if m is None else m.conj().contiguous()
        lam = torch.zeros((C, N, N), dtype=CDT, device=dev)
        gd = torch.zeros((C, N), dtype=torch.float64, device=dev)
        gb = torch.zeros((C, max(N - 1, 1)), dtype=torch.float64, device=dev)
        gg = torch.zeros((C, N), dtype=torch.float64, device=dev)
        n_seg = (n_steps + K - 1) // K
        wsb = lib.lime_lindblad_adjoint_f64_workspace(N, C, K, 0)
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        for sgi in range(n_seg - 1, -1, -1):
            s0 = sgi * K
            seg = min(K, n_steps - s0)
            ck = ckpt0 if sgi == 0 else states[:, sgi - 1].contiguous()
            d = nat.AdjointDesc()
            d.n, d.batch, d.param_batch, d.seg_steps = N, C, B, seg
            d.step0, d.total_steps = s0, n_steps
            d.k_dense, d.n_obs, d.obs_diag, d.obs_every = 0, n_obs, obs_diag, obs_every
            d.dt = float(dt)
            d.ckpt, d.lam = ck.data_ptr(), lam.data_ptr()
            d.heff, d.heff_stride = heff.data_ptr(), (0 if heff.shape[0] == 1 else N * N)
            d.heff_adj, d.heff_adj_stride = heff_adj.data_ptr(), (0 if heff.shape[0] == 1 else N * N)
            if m is not None:
                d.m, d.m_stride = m.data_ptr(), (0 if m.shape[0] == 1 else N * N)
                d.m_adj, d.m_adj_stride = m_adj.data_ptr(), (0 if m.shape[0] == 1 else N * N)
            if n_obs > 0:
                d.obs_ops, d.obs_stride = Et.data_ptr(), obs_stride
                d.obs_grad = gsrc.data_ptr()
            d.grad_diag, d.grad_bond, d.grad_gamma = gd.data_ptr(), gb.data_ptr(), gg.data_ptr()
            d.workspace, d.workspace_bytes = ws.data_ptr(), wsb
            nat.check(lib.lime_lindblad_adjoint_f64(d, torch.cuda.current_stream().cuda_stream),
                      'lime_lindblad_adjoint_f64')
        return _finish_grads(gd, gb, gg, herm, B, ns, site0)


def _finish_grads(gd, gb, gg, herm, B, ns, site0):
    if not herm:
        gd = gd[:B] + gd[B:]
        gb = gb[:B] + gb[B:]
        gg = gg[:B] + gg[B:]
    sl = slice(site0, site0 + ns)
    g_eps = gd[:, sl]
    g_bond = gb[:, site0:site0 + ns - 1] if ns > 1 else gb[:, :0]
    g_gamma = gg[:, sl]
    return g_eps, g_bond, g_gamma, None, None, None, None, None, None, None, None, None


def chain_observables(H0, eps, bond, gamma, rho0, e_ops, dt: float, n_steps: int, site0: int = 0,
                      obs_every: int = 1, checkpoint: int = 64, precision: str = 'fp64'):
    """Observables Tr(E rho) of the chain model, differentiable in eps, bond, gamma.

    ``eps`` (B, n_sites), ``bond`` (B, n_sites - 1), ``gamma`` (B, n_sites)
    are real tensors on the GPU; ``H0`` (N, N) or (B, N, N) holds the rest of
    the Hamiltonian (e.g. the ground state of an absorption model);
    ``rho0`` (N, N) or (B, N, N); ``e_ops`` a list of (N, N) observables.
    Returns (B, n_steps // obs_every, n_obs) complex128 with observable k
    recorded after step (k + 1) obs_every - 1.
    """
    if precision not in ('fp64', 'split'):
        raise ValueError("precision must be 'fp64' or 'split'")
    dev = eps.device
    H0 = engine.as_device(H0, dev)
    if H0.dim() == 2:
        H0 = H0.unsqueeze(0)
    rho0 = engine.as_device(rho0, dev)
    E = [engine.as_device(e, dev) for e in e_ops]
    return _ChainObservables.apply(eps, bond, gamma, H0, rho0, E, float(dt), int(n_steps), int(site0),
                                   int(obs_every), int(checkpoint), precision)
