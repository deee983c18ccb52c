"""Driven (time-dependent) Lindblad solver, drop-in for ``_lindblad_driven``.

Follows lime/oqs.py:1691-1800: ``H = [H0, [H1, f1], [H2, f2], ...]`` with
``H(t) = H0 - sum_i f_i(t) H_i`` evaluated at the END of each step (the
reference advances t before building H(t)) and held constant through the
four RK4 stages.  The drive functions are Python callables evaluated on the
host on the time grid; the kernel (FP64 path) forms Heff(t) per step.

The reference builds H(t) with ``Ht = H[0]; Ht += ...``, which mutates H[0]
in place every step; this solver implements the documented formula.  The
``return_result=False`` branch writes ``obs.dat`` with the observables after
each step (unlike ``_lindblad``) and creates an empty ``den_mat.dat``, as the
reference does.
"""
from __future__ import annotations

import numpy as np
import torch

from . import engine
from .result import Result


def _lindblad_driven(H, rho0, c_ops=None, e_ops=None, Nt=1, dt=0.005, t0=0., return_result=True,
                     precision='fp64', store_states=True):
    """``precision='split'`` runs the streaming tensor-core path (Heff(t)
    re-split on the device every step); it keeps the state on the device, so
    ``rholist`` then holds the final state only (pass store_states=False)."""
    if precision == 'split' and return_result and store_states:
        raise ValueError('precision="split" keeps the state on the device: pass store_states=False '
                         '(rholist then holds the final state)')
    c_ops = [] if c_ops is None else c_ops
    e_ops = [] if e_ops is None else list(e_ops)
    H0 = H[0]
    ops = [np.asarray(h[0].toarray() if hasattr(h[0], 'toarray') else h[0], dtype=np.complex128)
           for h in H[1:]]
    fns = [h[1] for h in H[1:]]
    times = t0 + dt * np.arange(1, Nt + 1)
    coef = np.zeros((Nt, len(fns)), dtype=np.float64)
    for q, f in enumerate(fns):
        vals = np.array([f(t) for t in times])
        if np.iscomplexobj(vals) and np.any(np.abs(np.imag(vals)) > 0):
            raise ValueError('drive coefficients must be real (a complex f(t) makes H(t) '
                             'non-Hermitian)')
        coef[:, q] = np.real(vals)
    gen = engine.LindbladGenerator.build(H0, c_ops)
    dev = gen.heff.device
    drive = None
    if ops:
        drive = (torch.as_tensor(np.stack(ops), dtype=torch.complex128, device=dev).contiguous(),
                 torch.as_tensor(coef, dtype=torch.float64, device=dev).contiguous())
    obs, states, rho = engine.propagate(gen, rho0, dt, Nt, e_ops,
                                        states_every=1 if (return_result and store_states) else 0,
                                        drive=drive, precision=precision)
    if not return_result:
        open('den_mat.dat', 'w').close()
        fmt = '{} ' * (len(e_ops) + 1) + '\n'
        ob = obs[0].cpu().numpy()
        with open('obs.dat', 'w') as f:
            for k in range(Nt):
                f.write(fmt.format(times[k], *ob[k]))
        return rho[0].cpu().numpy()
    res = Result(dt=dt, Nt=Nt, rho0=rho0, t0=t0, nout=1)
    res.observables = obs[0].cpu().numpy()
    res.rholist = list(states[0].cpu().numpy()) if states is not None else [rho[0].cpu().numpy()]
    return res
