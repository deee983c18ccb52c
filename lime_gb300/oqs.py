"""Drop-in for the open-quantum-system solvers of ``lime/oqs.py``.

Same names, arguments, return values and side-effect files as the reference
(binggu56/lime), with the time loops running in the lime_gb300 CUDA kernels:

* ``_lindblad``            lime/oqs.py:1590-1688
* ``_correlation_2p_1t``   lime/oqs.py:726-800
* ``Lindblad_solver``      lime/oqs.py:1117-1331
* ``liouvillian`` / ``lindbladian`` (single RHS evaluations) lime/oqs.py:706-723

Beyond the reference: a leading batch axis on ``H`` / ``rho0`` (and on each
collapse operator) propagates many instances in one launch, and a list of
Hamiltonians of different dimensions (an uneven batch, with per-instance
lists of initial states, collapse operators and observables) propagates
every size group concurrently and returns one ``Result`` per instance.

Errors follow the reference: ValueError for wrong operator counts
(lime/oqs.py:1310,1326), TypeError for non-Hermitian bath operators.  There is
no CPU fallback: without the CUDA library or a GB300 every call raises.
"""
from __future__ import annotations

import numpy as np
import torch

from . import engine
from .engine import DiagonalOps, Populations, SiteDephasing  # noqa: F401  (public: compact operator forms)
from .result import Result


_PINNED_MIN_BYTES = 1 << 20


def _np(t):
    """Host ndarray of a result tensor.  Large device results are copied into
    page-locked memory from torch's caching host allocator (a pageable
    destination makes the driver stage the copy through a bounce buffer at a
    fraction of the link's rate); the array keeps that block alive, and the
    block returns to the cache when the array is released."""
    t = t.detach()
    if t.device.type != 'cuda' or t.numel() * t.element_size() < _PINNED_MIN_BYTES:
        return t.cpu().numpy()
    out = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    out.copy_(t.resolve_conj())
    return out.numpy()


def _squeeze_batch(x, batched):
    return x if batched else x[0]


def _is_batched(H, rho0):
    def nd(a):
        return a.dim() if isinstance(a, torch.Tensor) else np.ndim(a.toarray() if hasattr(a, 'toarray') else a)
    return nd(H) == 3 or nd(rho0) == 3


def _lindblad(H, rho0, c_ops, e_ops=None, Nt=1, dt=0.005, return_result=True,
              precision='fp64', store_states=True, nout=1):
    """Lindblad RK4 time loop (lime/oqs.py:1590-1688).

    ``return_result=True`` returns a ``Result`` with ``observables``
    (Nt, n_e) at t = (k+1) dt and ``rholist`` (the state after every step).
    ``return_result=False`` writes ``obs.dat`` (observables before each step,
    time after it) and returns the final density matrix.

    Extensions (defaults reproduce the reference): a leading batch axis on
    ``H``/``rho0``/collapse operators (``engine.DiagonalOps`` for compact
    diagonal operators), ``nout`` (record observables and states every
    ``nout`` steps), ``store_states=False`` (keep only the final state) and
    ``precision``.
    """
    if engine.is_ragged(H):
        return _lindblad_ragged(H, rho0, c_ops, e_ops, Nt, dt, precision, store_states, nout)
    if e_ops is None:
        e_ops = []
    elif not isinstance(e_ops, engine.Populations):
        e_ops = list(e_ops)
    batched = _is_batched(H, rho0) or any(
        (isinstance(c, engine.DiagonalOps) and np.ndim(c.l) == 3) or
        (isinstance(c, engine.SiteDephasing) and np.ndim(c.rates) == 2) for c in (c_ops or []))
    if return_result and precision == 'split' and not store_states:
        # a host batch: uploads, launches and copies back overlapped per instance range
        got = engine.propagate_host_pipelined(H, rho0, c_ops, e_ops, dt, Nt, obs_every=nout)
        if got is not None:
            res = Result(dt=dt, Nt=Nt, rho0=rho0, t0=0.0, nout=nout)
            res.observables = got[0].numpy()
            res.rholist = got[1].numpy()
            return res
    gen = engine.LindbladGenerator.build(H, c_ops)
    if return_result:
        obs, states, rho = engine.propagate(gen, rho0, dt, Nt, e_ops,
                                            states_every=nout if store_states else 0,
                                            precision=precision, obs_every=nout)
        res = Result(dt=dt, Nt=Nt, rho0=rho0, t0=0.0, nout=nout)
        o = _np(obs)
        res.observables = _squeeze_batch(o, batched)
        if states is not None:
            st = _np(states)
            res.rholist = list(st[0]) if not batched else st
        else:
            res.rholist = [_np(rho[0])] if not batched else _np(rho)
        return res
    obs, _, rho = engine.propagate(gen, rho0, dt, Nt, e_ops, precision=precision)
    e_ops = engine.expand_e_ops(e_ops, gen.n)
    # observables before each step: Tr(E rho0), then after steps 0..Nt-2
    r0 = engine.as_device(rho0, rho.device)
    if r0.dim() == 2:
        r0 = r0.unsqueeze(0)
    first = torch.stack([torch.einsum('ji,bij->b', engine.as_device(e, rho.device), r0)
                         for e in e_ops], -1) if e_ops else torch.zeros((r0.shape[0], 0), dtype=engine.CDT)
    before = torch.cat([first.unsqueeze(1).to(obs.device), obs[:, :-1]], 1) if Nt > 0 else obs
    ob = _np(before)[0]
    fmt = '{} ' * (len(e_ops) + 1) + '\n'
    with open('obs.dat', 'w') as f:
        t = 0.0
        for k in range(Nt):
            t += dt
            f.write(fmt.format(t, *ob[k]))
    return _squeeze_batch(_np(rho), batched)


def _lindblad_ragged(H, rho0, c_ops, e_ops, Nt, dt, precision, store_states, nout):
    """Uneven batch (a list of Hamiltonians of different dimensions): one
    ``Result`` per instance, in input order.  ``rho0``, ``c_ops`` and
    ``e_ops`` are lists with one entry per instance (``c_ops[i]`` and
    ``e_ops[i]`` lists of operators of instance i's dimension)."""
    B = len(H)
    if not isinstance(rho0, (list, tuple)) or len(rho0) != B:
        raise ValueError('an uneven batch needs one initial state per Hamiltonian')
    c_ops = [[] for _ in range(B)] if c_ops is None else c_ops
    e_ops = [[] for _ in range(B)] if e_ops is None else e_ops
    obs, states, rhos = engine.propagate_ragged(
        list(H), list(rho0), dt, Nt, c_ops_list=c_ops, e_ops_list=e_ops,
        states_every=nout if store_states else 0, precision=precision, obs_every=nout)
    out = []
    for i in range(B):
        res = Result(dt=dt, Nt=Nt, rho0=rho0[i], t0=0.0, nout=nout)
        res.observables = _np(obs[i])
        res.rholist = list(_np(states[i])) if states[i] is not None else [_np(rhos[i])]
        out.append(res)
    return out


def _correlation_2p_1t(H, rho0, ops, c_ops, dt, Nt, method='lindblad', output='cor.dat',
                       precision='fp64'):
    """<A(t) B> = Tr[A e^{Lt}(B rho0)] (lime/oqs.py:726-800).

    Returns C at t = dt..Nt dt (shape (Nt,), or (B, Nt) for batched input)
    and writes ``output`` with one ``t C`` line per step.
    """
    if method != 'lindblad':
        raise SystemExit('The method {} has not been implemented yet! Please \
                 try lindblad.'.format(method))
    A, B = ops
    batched = _is_batched(H, rho0) or np.ndim(A) == 3
    gen = engine.LindbladGenerator.build(H, c_ops)
    dev = gen.heff.device
    Bd = engine.as_device(B, dev)
    r0 = engine.as_device(rho0, dev)
    rho = Bd @ r0
    obs, _, _ = engine.propagate(gen, rho, dt, Nt, [A], precision=precision)
    cor = _np(obs[:, :, 0])
    if output is not None:
        with open(output, 'w') as f:
            t = 0.0
            c0 = cor[0]
            for k in range(Nt):
                t += dt
                f.write('{} {} \n'.format(t, c0[k]))
    return cor if batched else cor[0]


def liouvillian(rho, H, c_ops):
    """One evaluation of -i[H, rho] + sum_k D[L_k] rho (lime/oqs.py:706-713).

    A single generator application (not part of any time loop), written with
    the Heff / M / dense-L factors that the prepare kernel builds, so it
    checks the same operands the propagation kernels consume.
    """
    gen = engine.LindbladGenerator.build(H, c_ops)
    r = engine.as_device(rho, gen.heff.device)
    heff = gen.heff[0]
    out = -1j * (heff @ r - r @ heff.mH)
    if gen.m is not None:
        out = out + gen.m[0] * r
    if gen.l_dense is not None:
        for L in gen.l_dense[0]:
            out = out + L @ r @ L.mH
    return _np(out)


def lindbladian(l, rho):
    """L rho L^dag - 1/2 {L^dag L, rho} (lime/oqs.py:716-723)."""
    l = np.asarray(l)
    ld = l.conj().T
    return l @ (rho @ ld) - 0.5 * (ld @ l @ rho + rho @ (ld @ l))


class Lindblad_solver:
    """Lindblad master-equation solver (lime/oqs.py:1117-1331)."""

    def __init__(self, H=None, c_ops=None, e_ops=None, precision='fp64'):
        self.c_ops = c_ops
        self.e_ops = e_ops
        self.H = H
        self.precision = precision

    def set_c_ops(self, c_ops):
        self.c_ops = c_ops

    def set_e_ops(self, e_ops):
        self.e_ops = e_ops

    def setH(self, H):
        self.H = H

    def configure(self, c_ops, e_ops):
        self.c_ops = c_ops
        self.e_ops = e_ops

    def liouvillian(self):
        from . import superoperator
        return superoperator.liouvillian(self.H, self.c_ops)

    def steady_state(self):
        pass

    def evolve(self, rho0, dt, Nt, t0=0., e_ops=None, return_result=True, nout=1,
               store_states=True):
        if isinstance(self.H, list) and not engine.is_ragged(self.H):
            from .driven import _lindblad_driven
            return _lindblad_driven(self.H, rho0=rho0, c_ops=self.c_ops, e_ops=e_ops,
                                    Nt=Nt, dt=dt, t0=t0, return_result=return_result,
                                    precision=self.precision,
                                    store_states=store_states if self.precision == 'split' else True)
        return _lindblad(self.H, rho0, c_ops=self.c_ops, e_ops=e_ops, Nt=Nt, dt=dt,
                         return_result=return_result, precision=self.precision, nout=nout,
                         store_states=store_states)

    def correlation_2op_1t(self, rho0, a_op, b_op, dt, Nt, output='cor.dat'):
        return _correlation_2p_1t(self.H, rho0, ops=[a_op, b_op], c_ops=self.c_ops, dt=dt,
                                  Nt=Nt, output=output, precision=self.precision)

    def correlation_3op_1t(self, rho0, oplist, dt=0.005, Nt=1):
        """<A B(t) C>: propagate C rho0 A and observe B (lime/oqs.py:1227-1246)."""
        a_op, b_op, c_op = oplist
        gen = engine.LindbladGenerator.build(self.H, self.c_ops)
        dev = gen.heff.device
        r = engine.as_device(c_op, dev) @ engine.as_device(rho0, dev) @ engine.as_device(a_op, dev)
        obs, _, _ = engine.propagate(gen, r, dt, Nt, [b_op], precision=self.precision)
        out = _np(obs[:, :, 0])
        return out if out.shape[0] > 1 else out[0]

    def correlation_4op_1t(self, rho0, ops, dt, nt):
        """<A B(t) C(t) D> (lime/oqs.py:1301-1315)."""
        if len(ops) != 4:
            raise ValueError('Number of operators is not 4.')
        a, b, c, d = ops
        return self.correlation_3op_1t(rho0, [a, np.asarray(b) @ np.asarray(c), d], dt, nt)

    def correlation_3op_2t(self, rho0, ops, dt, Nt, Ntau):
        """<A(t) B(t+tau) C(t)>, shape (Nt, Ntau) (lime/oqs.py:1268-1299).

        The Nt inner propagations are independent and run as one batch (on
        the tensor cores with ``precision='split'``); the single outer
        trajectory that seeds them is stored step by step, which the FP64
        path does.
        """
        gen = engine.LindbladGenerator.build(self.H, self.c_ops)
        dev = gen.heff.device
        _, states, _ = engine.propagate(gen, rho0, dt, Nt, None, states_every=1, precision='fp64')
        a, b, c = [engine.as_device(o, dev) for o in ops]
        rho_t = states[0]  # (Nt, n, n)
        start = c @ rho_t @ a
        if gen.shared:
            obs, _, _ = engine.propagate(gen, start, dt, Ntau, [b], precision=self.precision)
        else:
            raise ValueError('correlation_3op_2t takes a single (n, n) Hamiltonian')
        return _np(obs[:, :, 0])

    def correlation_4op_2t(self, rho0, ops, dt, nt, ntau):
        """<A(t) B(t+tau) C(t+tau) D(t)> (lime/oqs.py:1317-1331)."""
        if len(ops) != 4:
            raise ValueError('Number of operators is not 4.')
        a, b, c, d = ops
        return self.correlation_3op_2t(rho0, [a, np.asarray(b) @ np.asarray(c), d], dt, nt, ntau)
