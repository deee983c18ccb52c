"""NumPy restatement of the reference Lindblad RK4 path (test infrastructure).

Follows binggu56/lime:

* ``rk4``            lime/phys.py:636-649   (classic RK4, in-place ``rho +=``)
* ``comm/anticomm``  lime/phys.py:741-748
* ``dag``            lime/phys.py:758-759
* ``transform``      lime/phys.py:706-718   (v^dag A v)
* ``obs_dm``         lime/phys.py:837-844   (Tr(d rho) via d.dot(rho).diagonal().sum())
* ``liouvillian``    lime/oqs.py:706-713    (-i[H,rho] + sum_k lindbladian)
* ``lindbladian``    lime/oqs.py:716-723    (L rho L^dag - 1/2 {L^dag L, rho})
* ``lindblad``       lime/oqs.py:1590-1688  (_lindblad, both return_result branches)
* ``lindblad_driven``lime/oqs.py:1691-1800  (H(t) = H0 - sum_i f_i(t) H_i)
* ``correlation_2p_1t`` lime/oqs.py:726-800
* ``correlation_3op_1t`` / ``_4op_1t`` / ``_3op_2t`` / ``_4op_2t``
                     lime/oqs.py:1227-1331

The arithmetic is the same sequence of dense complex128 products the
reference performs (the reference's csr products in ``_correlation_2p_1t``
are the same sums in another order).
"""
from __future__ import annotations

import numpy as np


def dag(a):
    return a.conj().T


def comm(A, B):
    return A @ B - B @ A


def anticomm(A, B):
    return A @ B + B @ A


def transform(A, v):
    """v^dag A v (lime/phys.py:706-718)."""
    return dag(v) @ (A @ v)


def obs_dm(rho, d):
    """Tr(d rho) as the reference forms it (lime/phys.py:837-844)."""
    return (d @ rho).diagonal().sum()


def rk4(rho, fun, dt, *args):
    """Classic RK4; updates ``rho`` in place and returns it (lime/phys.py:636-649)."""
    dt2 = dt / 2.0
    k1 = fun(rho, *args)
    k2 = fun(rho + k1 * dt2, *args)
    k3 = fun(rho + k2 * dt2, *args)
    k4 = fun(rho + k3 * dt, *args)
    rho += (k1 + 2 * k2 + 2 * k3 + k4) / 6. * dt
    return rho


def lindbladian(l, rho):
    """L rho L^dag - 1/2 {L^dag L, rho} (lime/oqs.py:716-723)."""
    ld = dag(l)
    return l @ (rho @ ld) - 0.5 * anticomm(ld @ l, rho)


def liouvillian(rho, H, c_ops):
    """-i[H, rho] + sum_k lindbladian(L_k, rho) (lime/oqs.py:706-713)."""
    rhs = -1j * comm(H, rho)
    for c in c_ops:
        rhs = rhs + lindbladian(c, rho)
    return rhs


def lindblad(H, rho0, c_ops, e_ops=None, Nt=1, dt=0.005, return_result=True,
             store_states=True):
    """Time loop of ``_lindblad`` (lime/oqs.py:1590-1688).

    ``return_result=True``: returns ``(observables, rholist)`` with
    ``observables[k]`` taken after step k (t = (k+1) dt).
    ``return_result=False``: returns ``(observables, rho_final)`` with
    ``observables[k]`` taken before step k (t = k dt), as the reference's
    file-writing branch records them.
    """
    rho = np.array(rho0, dtype=np.complex128, copy=True)
    e_ops = [] if e_ops is None else list(e_ops)
    obs = np.zeros((Nt, len(e_ops)), dtype=np.complex128)
    if not return_result:
        for k in range(Nt):
            obs[k, :] = [obs_dm(rho, e) for e in e_ops]
            rho = rk4(rho, liouvillian, dt, H, c_ops)
        return obs, rho
    rholist = []
    for k in range(Nt):
        rho = rk4(rho, liouvillian, dt, H, c_ops)
        if store_states:
            rholist.append(rho.copy())
        obs[k, :] = [obs_dm(rho, e) for e in e_ops]
    if not store_states:
        rholist = [rho.copy()]
    return obs, rholist


def lindblad_driven(H, rho0, c_ops=None, e_ops=None, Nt=1, dt=0.005, t0=0.0):
    """``_lindblad_driven`` (lime/oqs.py:1691-1800), return_result=True branch.

    ``H = [H0, [H1, f1], [H2, f2], ...]`` with ``H(t) = H0 - sum_i f_i(t) H_i``
    evaluated at the END of each step (t is advanced before the step).  The
    reference accumulates into ``H[0]`` in place (``Ht += ...`` aliases H0);
    this restatement builds ``H(t)`` from a fresh copy each step, which is
    the evident intent.
    """
    c_ops = [] if c_ops is None else c_ops
    e_ops = [] if e_ops is None else e_ops
    rho = np.array(rho0, dtype=np.complex128, copy=True)
    obs = np.zeros((Nt, len(e_ops)), dtype=np.complex128)
    rholist = []
    t = t0
    for k in range(Nt):
        t += dt
        Ht = np.array(H[0], dtype=np.complex128, copy=True)
        for i in range(1, len(H)):
            Ht = Ht - H[i][1](t) * H[i][0]
        rho = rk4(rho, liouvillian, dt, Ht, c_ops)
        rholist.append(rho.copy())
        obs[k, :] = [obs_dm(rho, e) for e in e_ops]
    return obs, rholist


def correlation_2p_1t(H, rho0, ops, c_ops, dt, Nt):
    """<A(t) B> = Tr[A e^{Lt}(B rho0)] (lime/oqs.py:726-800); C at t=(k+1)dt."""
    A, B = ops
    rho = np.asarray(B) @ np.asarray(rho0)
    rho = rho.astype(np.complex128)
    cor = np.zeros(Nt, dtype=np.complex128)
    for k in range(Nt):
        rho = rk4(rho, liouvillian, dt, H, c_ops)
        cor[k] = obs_dm(rho, A)
    return cor


def correlation_3op_1t(H, c_ops, rho0, oplist, dt, Nt):
    """<A B(t) C> (lime/oqs.py:1227-1246): propagate C rho0 A, observe B."""
    a, b, c = oplist
    obs, _ = lindblad(H, c @ rho0 @ a, c_ops, e_ops=[b], Nt=Nt, dt=dt,
                      store_states=False)
    return obs[:, 0]


def correlation_4op_1t(H, c_ops, rho0, oplist, dt, Nt):
    """<A B(t) C(t) D> (lime/oqs.py:1301-1315) = 3op with B@C."""
    a, b, c, d = oplist
    return correlation_3op_1t(H, c_ops, rho0, [a, b @ c, d], dt, Nt)


def correlation_3op_2t(H, c_ops, rho0, ops, dt, Nt, Ntau):
    """<A(t) B(t+tau) C(t)> (lime/oqs.py:1268-1299), shape (Nt, Ntau)."""
    _, rho_t = lindblad(H, rho0, c_ops, Nt=Nt, dt=dt)
    a, b, c = ops
    out = np.zeros((Nt, Ntau), dtype=np.complex128)
    for t_idx, rho in enumerate(rho_t):
        o, _ = lindblad(H, c @ rho @ a, c_ops, e_ops=[b], Nt=Ntau, dt=dt,
                        store_states=False)
        out[t_idx, :] = o[:, 0]
    return out


def correlation_4op_2t(H, c_ops, rho0, ops, dt, Nt, Ntau):
    """<A(t) B(t+tau) C(t+tau) D(t)> (lime/oqs.py:1317-1331)."""
    a, b, c, d = ops
    return correlation_3op_2t(H, c_ops, rho0, [a, b @ c, d], dt, Nt, Ntau)


def lindblad_step_count_flops(n, n_ops, dephasing):
    """Algorithmic real flops of one RK4 step (8 m n k per complex GEMM).

    Dephasing / diagonal collapse operators: 2 complex N^3 GEMMs per RHS
    (Heff rho and rho Heff^dag); dense: 2 + 2K per RHS.
    """
    g = 2 if dephasing else 2 + 2 * n_ops
    return 4 * g * 8 * n ** 3
