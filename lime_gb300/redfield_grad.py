"""Differentiable Bloch-Redfield observables (torch.autograd) on the
library's kernels: gradients of populations (or any observables) with
respect to the site energies and couplings in H, the bath coupling
operators and the parameters of the bath spectral density.

The reference has no gradients; the forward computation is that of
``redfield_tensor`` (lime/oqs.py:528-579) followed by the RK4 loop of
``_redfield`` (lime/oqs.py:453-472):

* ``eigh(H)``, the eigenbasis transforms ``A_k = V^dag a_k V``, the spectral
  factors ``C_k = S_k(-(E_a - E_b))`` and the O(N^3 K) factors
  ``Lam_k = C_k o A_k``, ``P = sum_k A_k Lam_k``, ``Q = sum_k Lam_k^dag A_k``
  are small and stay in torch, which differentiates them;
* the O(N^4 K) assembly of the dense generator runs in
  ``lime_redfield_assemble_f64``, its closed-form adjoint in
  ``lime_redfield_assemble_adjoint_f64``;
* the RK4 time loop runs in the library's FP64 or tensor-core propagators,
  checkpointed every ``checkpoint`` steps, and its discrete adjoint in
  ``lime_redfield_adjoint_f64`` or, on the tensor cores,
  ``lime_redfield_adjoint_split`` (backward-in-time RK4 with L^dag and the
  generator gradient sum_i a_i y_i^dag).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from . import engine
from .redfield import propagate_vec, propagate_vec_split, stage_buffer_floats

CDT = torch.complex128


def ohmic_spectrum(lam, omega_c, kT):
    """Ohmic bath spectrum S(w) = 2 J(w) / (1 - exp(-w/kT)) with
    J(w) = (pi lam / omega_c) w exp(-|w|/omega_c), S(0) = 2 pi lam kT /
    omega_c (the same function as ``chains.ohmic_spectrum``), as a torch
    callable differentiable in ``lam``, ``omega_c`` and ``kT`` (floats or
    0-dim tensors)."""
    def S(w):
        eta = np.pi * lam / omega_c
        small = w.abs() < 1e-12
        ws = torch.where(small, torch.ones_like(w), w)
        val = 2.0 * eta * ws * torch.exp(-ws.abs() / omega_c) / (-torch.expm1(-ws / kT))
        return torch.where(small, 2.0 * eta * kT * torch.ones_like(w), val)
    return S


class _Assemble(torch.autograd.Function):
    """R = assemble(E, A, Lam, P, Q) (lime_redfield_assemble_f64) with the
    closed-form adjoint (lime_redfield_assemble_adjoint_f64)."""

    @staticmethod
    def forward(ctx, E, A, Lam, P, Q):
        lib = nat.require_device()
        n, K = E.shape[0], A.shape[0]
        E, A, Lam, P, Q = (x.detach().contiguous() for x in (E, A, Lam, P, Q))
        R = torch.empty((n * n, n * n), dtype=CDT, device=E.device)
        d = nat.RedfieldAssembleDesc()
        d.n, d.k = n, K
        d.evals, d.a_eig, d.lam, d.p, d.q, d.R = (E.data_ptr(), A.data_ptr(), Lam.data_ptr(), P.data_ptr(),
                                                  Q.data_ptr(), R.data_ptr())
        nat.check(lib.lime_redfield_assemble_f64(d, engine._stream_ptr()), 'lime_redfield_assemble_f64')
        ctx.save_for_backward(A, Lam)
        return R

    @staticmethod
    def backward(ctx, G):
        lib = nat.require_device()
        A, Lam = ctx.saved_tensors
        K, n = A.shape[0], A.shape[1]
        G = G.to(CDT).contiguous()
        dev = G.device
        gE = torch.empty(n, dtype=torch.float64, device=dev)
        gA = torch.empty_like(A)
        gL = torch.empty_like(Lam)
        gP = torch.empty((n, n), dtype=CDT, device=dev)
        gQ = torch.empty((n, n), dtype=CDT, device=dev)
        d = nat.RedfieldAssembleAdjointDesc()
        d.n, d.k = n, K
        d.a_eig, d.lam, d.G = A.data_ptr(), Lam.data_ptr(), G.data_ptr()
        d.grad_evals, d.grad_a, d.grad_lam, d.grad_p, d.grad_q = (gE.data_ptr(), gA.data_ptr(), gL.data_ptr(),
                                                                  gP.data_ptr(), gQ.data_ptr())
        nat.check(lib.lime_redfield_assemble_adjoint_f64(d, engine._stream_ptr()),
                  'lime_redfield_assemble_adjoint_f64')
        return gE, gA, gL, gP, gQ


def _segments(n_steps, checkpoint):
    out, s0 = [], 0
    while s0 < n_steps:
        out.append((s0, min(checkpoint, n_steps - s0)))
        s0 += checkpoint
    return out


class _Propagate(torch.autograd.Function):
    """Observables (B, n_steps // obs_every, n_obs) of the RK4 evolution of
    the eigenbasis states r0 (B, n, n) under R, checkpointed forward and the
    discrete adjoint (lime_redfield_adjoint_f64) backward."""

    @staticmethod
    def forward(ctx, R, r0, E, dt, n_steps, obs_every, checkpoint, precision, keep_bytes):
        n = r0.shape[-1]
        B = r0.shape[0]
        Rg = (R.detach(), n)
        rho = r0.detach().to(CDT).contiguous()
        E = E.detach().to(CDT).contiguous()
        segs = _segments(n_steps, checkpoint)
        # split path: the stage inputs of the last segments, as many as fit
        # keep_bytes, stay in device memory for the backward pass (which
        # then skips their recomputation)
        stages = [None] * len(segs)
        if precision == 'split' and keep_bytes:
            left = int(keep_bytes)
            for i in range(len(segs) - 1, -1, -1):
                need = stage_buffer_floats(n, B, segs[i][1]) * 4
                if need > left:
                    break
                stages[i] = torch.empty(stage_buffer_floats(n, B, segs[i][1]), dtype=torch.float32,
                                        device=rho.device)
                left -= need
        ckpts, parts = [], []
        for (s0, m), sbuf in zip(segs, stages):
            ckpts.append(rho)
            if precision == 'fp64':
                o, _, rho = propagate_vec(Rg, rho, dt, m, list(E), obs_every=obs_every)
            elif sbuf is not None:
                o, _, rho = propagate_vec_split(Rg, rho, dt, m, list(E), obs_every=obs_every, stage_out=sbuf)
            else:
                # the block form: the backward pass recomputes segments with it
                o, _, rho = propagate_vec_split(Rg, rho, dt, m, list(E), obs_every=obs_every, product='4m')
            parts.append(o)
        obs = torch.cat(parts, 1) if parts else torch.zeros((rho.shape[0], 0, E.shape[0]), dtype=CDT,
                                                           device=rho.device)
        ctx.save_for_backward(R.detach(), E, *ckpts)
        ctx.stages = stages
        ctx.cfg = (float(dt), int(n_steps), int(obs_every), int(checkpoint), precision)
        return obs

    @staticmethod
    def backward(ctx, g):
        R, E, *ckpts = ctx.saved_tensors
        if ctx.cfg[4] == 'split':
            stages, ctx.stages = ctx.stages, None
            return _backward_split(R, E, ckpts, g, *ctx.cfg[:4], stages=stages) + (None,)
        lib = nat.require_device()
        dt, n_steps, obs_every, checkpoint = ctx.cfg[:4]
        B, n = ckpts[0].shape[0], ckpts[0].shape[-1]
        D = n * n
        dev = R.device
        n_obs = E.shape[0]
        gsrc = g.to(CDT).permute(1, 0, 2).contiguous()           # [slot][rhs][obs]
        lam = torch.zeros((D, B), dtype=CDT, device=dev)
        gR = torch.zeros((D, D), dtype=CDT, device=dev)
        gE = torch.zeros((n_obs, n, n), dtype=CDT, device=dev)
        segs = _segments(n_steps, checkpoint)
        wsb = int(lib.lime_redfield_adjoint_f64_workspace(n, B, max(m for _, m in segs)))
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        for (s0, m), ck in reversed(list(zip(segs, ckpts))):
            P = ck.reshape(B, D).transpose(0, 1).contiguous()
            d = nat.RedfieldAdjointDesc()
            d.n, d.n_rhs, d.seg_steps, d.step0 = n, B, m, s0
            d.n_obs, d.obs_every, d.n_slots = n_obs, obs_every, gsrc.shape[0]
            d.dt = dt
            d.R, d.ckpt, d.lam = R.data_ptr(), P.data_ptr(), lam.data_ptr()
            if n_obs:
                d.obs_ops, d.obs_grad = E.data_ptr(), gsrc.data_ptr()
            d.grad_R, d.grad_obs = gR.data_ptr(), gE.data_ptr()
            d.workspace, d.workspace_bytes = ws.data_ptr(), wsb
            nat.check(lib.lime_redfield_adjoint_f64(d, engine._stream_ptr()), 'lime_redfield_adjoint_f64')
        g_r0 = lam.transpose(0, 1).reshape(B, n, n)
        return gR, g_r0, gE, None, None, None, None, None, None


def _backward_split(R, E, ckpts, g, dt, n_steps, obs_every, checkpoint, max_retries=3, stages=None):
    """The backward pass on the tensor cores (lime_redfield_adjoint_split),
    segment by segment from the last; a segment whose adjoint operands left
    their fixed-point range is repeated with a 4x larger margin (a smaller
    power-of-two scale of the adjoint stage inputs) or, for the recomputed
    states, a 4x smaller state scale.  ``stages[i]``: segment i's stage
    inputs kept by the forward pass (its recomputation is skipped), or
    None."""
    lib = nat.require_device()
    B, n = ckpts[0].shape[0], ckpts[0].shape[-1]
    D = n * n
    dev = R.device
    n_obs = E.shape[0]
    gsrc = g.to(CDT).permute(1, 0, 2).contiguous()           # [slot][rhs][obs]
    lam = torch.zeros((B, D), dtype=CDT, device=dev)
    gR = torch.zeros((D, D), dtype=CDT, device=dev)
    gE = torch.zeros((n_obs, n, n), dtype=CDT, device=dev)
    segs = _segments(n_steps, checkpoint)
    wsb = int(lib.lime_redfield_adjoint_split_workspace(n, B, max(m for _, m in segs), n_obs))
    ws = torch.empty(wsb + 1024, dtype=torch.uint8, device=dev)
    aligned = (ws.data_ptr() + 1023) // 1024 * 1024
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    stages = stages or [None] * len(segs)
    for (s0, m), ck, sbuf in reversed(list(zip(segs, ckpts, stages))):
        P = ck.reshape(B, D).contiguous()
        pmax = float(torch.view_as_real(P).abs().max().item())
        sb = int(np.floor(np.log2(8192.0 / (1.25 * pmax)))) if pmax > 0 else 0
        margin = 0
        for attempt in range(max_retries + 1):
            lam_t, gR_t, gE_t = lam.clone(), torch.zeros_like(gR), torch.zeros_like(gE)
            status.zero_()
            d = nat.RedfieldAdjointSplitDesc()
            d.n, d.n_rhs, d.seg_steps, d.step0 = n, B, m, s0
            d.n_obs, d.obs_every, d.n_slots = n_obs, obs_every, gsrc.shape[0]
            d.scale_b_log2, d.margin_log2 = max(-60, min(60, sb)), margin
            d.dt = dt
            d.R, d.ckpt, d.lam = R.data_ptr(), P.data_ptr(), lam_t.data_ptr()
            if n_obs:
                d.obs_ops, d.obs_grad = E.data_ptr(), gsrc.data_ptr()
            d.grad_R, d.grad_obs = gR_t.data_ptr(), gE_t.data_ptr()
            d.workspace, d.workspace_bytes = aligned, wsb
            d.status = status.data_ptr()
            if sbuf is not None:
                d.stage_in = sbuf.data_ptr()
            nat.check(lib.lime_redfield_adjoint_split(d, engine._stream_ptr()), 'lime_redfield_adjoint_split')
            flags = int(status.item())
            if flags & nat.LIME_FLAG_RANGE and attempt < max_retries:
                margin += 2
                if sbuf is None:
                    sb -= 2
                continue
            if flags:
                raise nat.KernelFlagError(flags, 'lime_redfield_adjoint_split')
            break
        lam, gR, gE = lam_t, gR + gR_t, gE + gE_t
        sbuf = None
    return gR, lam.reshape(B, n, n), gE, None, None, None, None, None


def redfield_observables(H, a_ops, spectrum, rho0, e_ops, dt: float, n_steps: int, obs_every: int = 1,
                         checkpoint: int = 64, precision: str = 'fp64', keep_stages='auto'):
    """<E_o>(t) = Tr(E_o rho(t)) of the Bloch-Redfield evolution of ``rho0``,
    differentiable (torch.autograd) in every tensor input.

    ``H`` (n, n) real or complex Hermitian; ``a_ops`` (K, n, n) Hermitian
    bath coupling operators (a list or a stacked tensor); ``spectrum`` a
    torch callable S(w) shared by all K operators, or a list of K; ``rho0``
    (n, n) or (B, n, n) and ``e_ops`` (n_obs, n, n) in the site basis.
    Returns (B, n_steps // obs_every, n_obs) complex128, observable k after
    step (k + 1) obs_every - 1 (the reference's timing, t = (k+1) dt for
    obs_every = 1).  ``precision='split'`` runs the forward and the backward
    pass on the tensor cores (lime_redfield_rk4_split,
    lime_redfield_adjoint_split).  ``checkpoint`` must be a multiple of
    ``obs_every``.  ``keep_stages`` (split path): bytes of device memory in
    which the forward pass keeps the stage inputs of its last checkpoint
    segments, so that the backward pass recomputes only the others; 'auto'
    is half the free device memory, 0 recomputes every segment (the
    gradients are the same either way).
    """
    if precision not in ('fp64', 'split'):
        raise ValueError("precision must be 'fp64' or 'split'")
    if checkpoint % obs_every:
        raise ValueError('checkpoint must be a multiple of obs_every')
    dev = H.device if isinstance(H, torch.Tensor) else engine._dev(None)
    H = torch.as_tensor(H, device=dev)
    A0 = torch.stack([torch.as_tensor(a, device=dev) for a in a_ops]) if isinstance(a_ops, (list, tuple)) \
        else torch.as_tensor(a_ops, device=dev)
    # the n x n eigendecomposition runs on the host, as in the reference
    # (scipy eigh in redfield_tensor); autograd carries the device transfer
    E, V = torch.linalg.eigh(H.cpu())
    E = E.to(device=dev, dtype=torch.float64)
    Vc = V.to(device=dev, dtype=CDT)
    A = Vc.mH @ A0.to(CDT) @ Vc                                    # (K, n, n)
    W = E[:, None] - E[None, :]
    if callable(spectrum):
        C = spectrum(-W).to(torch.float64)
    else:
        C = torch.stack([s(-W) for s in spectrum]).to(torch.float64)
    Lam = C.to(CDT) * A
    P = (A @ Lam).sum(0)
    Q = (Lam.mH @ A).sum(0)
    R = _Assemble.apply(E, A, Lam, P, Q)
    r0 = torch.as_tensor(rho0, device=dev).to(CDT)
    if r0.dim() == 2:
        r0 = r0.unsqueeze(0)
    Es = torch.stack([torch.as_tensor(e, device=dev) for e in e_ops]) if isinstance(e_ops, (list, tuple)) \
        else torch.as_tensor(e_ops, device=dev)
    r0e = Vc.mH @ r0 @ Vc
    Ee = Vc.mH @ Es.to(CDT) @ Vc
    keep = 0
    if precision == 'split':
        if keep_stages == 'auto':
            keep = torch.cuda.mem_get_info(dev)[0] // 2 if torch.is_grad_enabled() else 0
        else:
            keep = int(keep_stages)
    return _Propagate.apply(R, r0e, Ee, float(dt), int(n_steps), int(obs_every), int(checkpoint), precision,
                            keep)
