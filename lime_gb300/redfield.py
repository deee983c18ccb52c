"""Drop-in for the Bloch-Redfield solvers of ``lime/oqs.py``.

* ``redfield_tensor(H, a_ops, spectra, secular=False)``  lime/oqs.py:528-579
* ``_redfield(R, rho0, evecs, Nt, dt, t0, e_ops, return_result)``  lime/oqs.py:373-468
* ``Redfield_solver``  lime/oqs.py:40-371

As in the reference, ``eigh(H)``, the eigenbasis transforms and the user's
bath spectral callbacks run on the host; the O(N^4 K) assembly of the dense
generator (``lime_redfield_build_f64``) and the RK4 time loop over a block
of right-hand sides (``lime_redfield_rk4_f64``) run on the GPU in FP64.  The
generator is kept on the device in a ``RedfieldTensor``, which offers the
``toarray()/todense()/shape/dot`` surface of the reference's csr return
value.  A leading batch axis on ``rho0`` propagates many initial states as
one GEMM right-hand-side block.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg
import torch

from . import _native as nat
from . import engine
from . import zlinalg as zl
from .result import Result

CDT = torch.complex128


def _dense(a):
    return a.toarray() if hasattr(a, 'toarray') else np.asarray(a)


def _isherm(a):
    return np.allclose(a, a.conj().T)


class RedfieldTensor:
    """Dense Redfield generator (D x D complex128) resident on the GPU."""

    def __init__(self, R: torch.Tensor, n: int):
        self.R = R
        self.n = n
        self.shape = tuple(R.shape)

    def toarray(self):
        return self.R.cpu().numpy()

    def todense(self):
        return np.asmatrix(self.toarray())

    def dot(self, x):
        xt = torch.as_tensor(np.asarray(x), dtype=CDT, device=self.R.device)
        y = zl.mm(self.R, xt.reshape(xt.shape[0], -1))
        return y.reshape((self.R.shape[0],) + tuple(xt.shape[1:])).cpu().numpy()

    __matmul__ = dot


def _spectrum_matrix(S, W):
    """C[n, m] = S(-W[n, m]): one vectorised call when the callback accepts
    arrays, else the reference's element-by-element evaluation."""
    try:
        C = np.asarray(S(-W), dtype=np.float64)
        if C.shape == W.shape:
            return C
    except Exception:
        pass
    n = W.shape[0]
    C = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            C[i, j] = S(-W[i, j])
    return C


def redfield_tensor(H, a_ops, spectra, secular=False, device=None):
    """Bloch-Redfield generator in the eigenbasis of H (lime/oqs.py:528-579).

    Returns ``(R, evecs)`` with d vec(rho)/dt = R vec(rho) (row-major vec);
    ``secular`` is accepted and ignored, as in the reference.
    """
    for a in a_ops:
        if not _isherm(_dense(a)):
            raise TypeError("Operators in a_ops must be Hermitian.")
    lib = nat.require_device()
    dev = engine._dev(device)
    Hd = _dense(H)
    evals, evecs = scipy.linalg.eigh(Hd)
    n = len(evals)
    K = len(a_ops)
    W = np.real(evals[:, None] - evals[None, :])
    cache = {}
    Cs = []
    for k in range(K):
        key = id(spectra[k])
        if key not in cache:
            cache[key] = _spectrum_matrix(spectra[k], W)
        Cs.append(cache[key])
    shared = len(cache) == 1
    A = np.stack([evecs.conj().T @ _dense(a) @ evecs for a in a_ops]).astype(np.complex128)
    Ct = torch.as_tensor(np.stack([Cs[0]] if shared else Cs), dtype=torch.float64, device=dev).contiguous()
    At = torch.as_tensor(A, dtype=CDT, device=dev).contiguous()
    Et = torch.as_tensor(evals, dtype=torch.float64, device=dev).contiguous()
    D = n * n
    R = torch.empty((D, D), dtype=CDT, device=dev)
    wsb = lib.lime_redfield_build_f64_workspace(n, K)
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    d = nat.RedfieldBuildDesc()
    d.n, d.k = n, K
    d.evals, d.a_eig = Et.data_ptr(), At.data_ptr()
    d.spec, d.spec_stride = Ct.data_ptr(), (0 if shared else n * n)
    d.R = R.data_ptr()
    d.workspace, d.workspace_bytes = ws.data_ptr(), wsb
    nat.check(lib.lime_redfield_build_f64(d, engine._stream_ptr()), 'lime_redfield_build_f64')
    return RedfieldTensor(R, n), evecs


def _as_generator(R, device):
    if isinstance(R, RedfieldTensor):
        return R.R, R.n
    Rd = torch.as_tensor(_dense(R), dtype=CDT, device=device).contiguous()
    n = int(round(np.sqrt(Rd.shape[0])))
    return Rd, n


def propagate_vec(R, rho0_eb: torch.Tensor, dt: float, n_steps: int, e_eb=None, states_every=0,
                  obs_every=1):
    """RK4 of eigenbasis density matrices (B, n, n) under the dense generator.

    Returns (obs (B, n_steps // obs_every, n_obs), states (B, S, n, n) or None,
    final rho (B, n, n)), all in the eigenbasis.
    """
    lib = nat.require_device()
    Rd, n = R
    dev = Rd.device
    B = rho0_eb.shape[0]
    D = n * n
    # D x B, column = vec rho; always a fresh buffer (the kernel writes it
    # in place, and the input may itself be a view of an earlier result)
    P = torch.empty((D, B), dtype=CDT, device=dev)
    P.copy_(rho0_eb.reshape(B, D).transpose(0, 1))
    E = None
    n_obs = 0
    if e_eb is not None and len(e_eb):
        E = torch.stack(list(e_eb)).to(CDT).contiguous()
        n_obs = E.shape[0]
    n_slots = n_steps // obs_every
    obs = torch.zeros((max(n_slots, 1), B, max(n_obs, 1)), dtype=CDT, device=dev)
    states = None
    if states_every:
        states = torch.empty((n_steps // states_every, D, B), dtype=CDT, device=dev)
    wsb = lib.lime_redfield_rk4_f64_workspace(n, B)
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    d = nat.RedfieldRK4Desc()
    d.n, d.n_rhs, d.n_steps, d.n_obs = n, B, n_steps, n_obs
    d.obs_every, d.states_every = obs_every, states_every if states is not None else 0
    d.dt = float(dt)
    d.R, d.rho = Rd.data_ptr(), P.data_ptr()
    if E is not None:
        d.obs_ops, d.obs_out = E.data_ptr(), obs.data_ptr()
    d.states = None if states is None else states.data_ptr()
    d.workspace, d.workspace_bytes = ws.data_ptr(), wsb
    nat.check(lib.lime_redfield_rk4_f64(d, engine._stream_ptr()), 'lime_redfield_rk4_f64')
    o = obs[:n_slots, :, :n_obs].permute(1, 0, 2)
    st = None
    if states is not None:
        st = states.permute(2, 0, 1).reshape(B, -1, n, n)
    return o, st, P.transpose(0, 1).reshape(B, n, n)


def _pow2_floor(x: float) -> int:
    return int(np.floor(np.log2(x)))


# complex product of the tensor-core Redfield RK4: the block form '4m'
# (one launch of 2 Dp / 64-chunk tiles over [Yr | Yi]) or '3m' (three real
# products: 3/4 of the tensor work in 1.5x as many tiles of half the K, plus
# an elementwise stage pass).  'auto': the autotuner's cached choice for the
# shape, else the wave-quantised cost model of split_product(); 3M only from
# Liouville dimension SPLIT_3M_MIN_DIM up (below it the run time is
# negligible and the block form's observable readout is ~2x closer).
SPLIT_3M_MIN_DIM = 1024
SPLIT_PRODUCT = 'auto'


def split_cost(n: int, n_rhs: int, sms: int):
    """Model of one stage's streaming-GEMM time in chunk-iterations of the
    busiest CTA, (block form, 3M): waves of tiles x K chunks per tile, the 3M
    form with 8 % for its elementwise stage pass."""
    D = n * n
    Dp = -(-D // 128) * 128
    MT = Dp // 128
    Rp = -(-n_rhs // 64) * 64
    Rq = -(-n_rhs // 128) * 128
    t4 = -(-(MT * (2 * Rp // 128)) // sms) * (2 * Dp // 64)
    t3 = -(-(3 * MT * (Rq // 128)) // sms) * (Dp // 64) * 1.08
    return t4, t3


def split_product(n: int, n_rhs: int, device=None) -> str:
    """'3m' or '4m' for this shape: the tuning cache's choice, else the
    cost model (3M only from SPLIT_3M_MIN_DIM up and when the model gives it
    at least 3 % less)."""
    from . import tuning
    if n * n < SPLIT_3M_MIN_DIM:
        return '4m'
    dev = engine._dev(device)
    got = tuning.choose('redfield_split', split_class(n, n_rhs), 'split', {}, arch=tuning.arch_tag(dev))
    if got.get('product') in ('3m', '4m'):
        return got['product']
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    t4, t3 = split_cost(n, n_rhs, sms)
    return '3m' if t3 < 0.97 * t4 else '4m'


def split_class(n: int, n_rhs: int) -> str:
    """The autotuner's class of a Redfield split shape (padded dimensions)."""
    return 'D%d|R%d' % (-(-(n * n) // 128) * 128, -(-n_rhs // 64) * 64)


def autotune_split(R, n_rhs: int, dt: float = 0.05, steps=(2, 6), device=None, cache=None, force=False):
    """Time both complex-product forms on this generator and ``n_rhs``
    right-hand sides (GPU time of ``steps[1]`` minus ``steps[0]`` RK4
    steps, CUDA events) and cache the faster under the shape's class.
    Returns ``(choice, times)``."""
    from . import tuning
    Rd, n = R
    dev = Rd.device
    r0 = torch.zeros((n_rhs, n, n), dtype=CDT, device=dev)
    r0[:, 0, 0] = 1.0

    def measure(cand):
        def run(k):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            a.record()
            propagate_vec_split(R, r0, dt, k, None, product=cand['product'])
            b.record()
            torch.cuda.synchronize(dev)
            return a.elapsed_time(b) / 1e3
        run(1)
        return (run(steps[1]) - run(steps[0])) / (steps[1] - steps[0])

    return tuning.tune('redfield_split', split_class(n, n_rhs), 'split', [{'product': '4m'}, {'product': '3m'}],
                       measure, arch=tuning.arch_tag(dev), cache=cache, force=force)


def stage_buffer_floats(n: int, n_rhs: int, n_steps: int) -> int:
    """Floats of the stage-input buffer of ``propagate_vec_split(...,
    stage_out=...)``: [4 n_steps + 1][2 Rp][Dp], Rp = n_rhs rounded up to
    64, Dp = n^2 rounded up to 128."""
    Rp = -(-n_rhs // 64) * 64
    Dp = -(-(n * n) // 128) * 128
    return (4 * n_steps + 1) * 2 * Rp * Dp


def propagate_vec_split(R, rho0_eb: torch.Tensor, dt: float, n_steps: int, e_eb=None, obs_every=1,
                        max_retries=3, product=None, stage_out=None):
    """Tensor-core split-precision RK4 (``lime_redfield_rk4_split``) of
    eigenbasis density matrices (B, n, n) under the dense generator.
    ``product``: '4m' (the real block form of the complex product), '3m'
    (three real products, ``lime_redfield_rk4_split3``) or 'auto'
    (``split_product``); default ``SPLIT_PRODUCT``.  ``stage_out``: a float32 device tensor of
    ``stage_buffer_floats(n, B, n_steps)`` elements that receives every
    stage input (for the adjoint without recomputation; block form only).

    Same returns as ``propagate_vec`` without states.  The states are
    scaled to max |rho0| * 1.25 <= 2^13 (a power of two, so the scaling is
    exact; the kernel scales every generator and observable row itself); a
    run whose states leave the fixed-point range raises LIME_FLAG_RANGE and
    is repeated with the state scale lowered by 4x.
    """
    lib = nat.require_device()
    Rd, n = R
    dev = Rd.device
    B = rho0_eb.shape[0]
    D = n * n
    E = None
    n_obs = 0
    if e_eb is not None and len(e_eb):
        E = torch.stack(list(e_eb)).to(CDT).contiguous()
        n_obs = E.shape[0]
    n_slots = n_steps // obs_every
    pmax = float(torch.view_as_real(rho0_eb).abs().max().item()) if rho0_eb.numel() else 0.0
    sb = _pow2_floor(8192.0 / (1.25 * pmax)) if pmax > 0 else 0
    product = SPLIT_PRODUCT if product is None else product
    if product == 'auto':
        product = split_product(n, B, dev)
    if product not in ('3m', '4m'):
        raise ValueError("product must be '3m', '4m' or 'auto'")
    if stage_out is not None:
        product = '4m'
        if stage_out.dtype != torch.float32 or stage_out.numel() < stage_buffer_floats(n, B, n_steps):
            raise ValueError('stage_out needs stage_buffer_floats(n, n_rhs, n_steps) float32 elements')
    name = 'lime_redfield_rk4_split3' if product == '3m' else 'lime_redfield_rk4_split'
    run = getattr(lib, name)
    wsb = (lib.lime_redfield_split3_workspace if product == '3m' else lib.lime_redfield_split_workspace)(n, B, n_obs)
    ws = torch.empty(wsb + 1024, dtype=torch.uint8, device=dev)
    base = ws.data_ptr()
    aligned = (base + 1023) // 1024 * 1024
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    for attempt in range(max_retries + 1):
        P = rho0_eb.reshape(B, D).to(CDT).contiguous().clone()        # [R][D], row = vec rho
        obs = torch.zeros((max(n_slots, 1), B, max(n_obs, 1)), dtype=CDT, device=dev)
        status.zero_()
        d = nat.RedfieldSplitDesc()
        d.n, d.n_rhs, d.n_steps, d.n_obs, d.obs_every = n, B, n_steps, n_obs, obs_every
        d.scale_b_log2 = max(-60, min(60, sb))
        d.dt = float(dt)
        d.R, d.rho = Rd.data_ptr(), P.data_ptr()
        if E is not None:
            d.obs_ops, d.obs_out = E.data_ptr(), obs.data_ptr()
        d.workspace, d.workspace_bytes = aligned, wsb
        d.status = status.data_ptr()
        if stage_out is not None:
            d.stage_out = stage_out.data_ptr()
        nat.check(run(d, engine._stream_ptr()), name)
        flags = int(status.item())
        if flags & nat.LIME_FLAG_RANGE and attempt < max_retries:
            sb -= 2
            continue
        if flags:
            raise nat.KernelFlagError(flags, name)
        break
    o = obs[:n_slots, :, :n_obs].permute(1, 0, 2)
    return o, None, P.reshape(B, n, n)


def _propagate(Rg, r0t, dt, Nt, e_eb, states_every=0, precision='fp64'):
    if precision == 'fp64':
        return propagate_vec(Rg, r0t, dt, Nt, e_eb, states_every=states_every)
    if precision != 'split':
        raise ValueError("precision must be 'fp64' or 'split'")
    if not states_every:
        return propagate_vec_split(Rg, r0t, dt, Nt, e_eb)
    # states every `states_every` steps: segments of split runs restarted
    # from each segment's complex128 end state
    n = Rg[1]
    obs_parts, states = [], []
    rho = r0t
    done = 0
    while done < Nt:
        m = min(states_every, Nt - done)
        o, _, rho = propagate_vec_split(Rg, rho, dt, m, e_eb)
        obs_parts.append(o)
        if m == states_every:
            states.append(rho)
        done += m
    o = torch.cat(obs_parts, 1)
    st = torch.stack(states, 1) if states else None
    return o, st, rho


def _redfield(R, rho0, evecs=None, Nt=1, dt=0.005, t0=0, e_ops=None, return_result=True,
              store_states=True, precision='fp64'):
    """RK4 of the Redfield equation (lime/oqs.py:373-468).

    ``return_result=True``: a ``Result`` with ``observables`` (Nt, n_e)
    evaluated in the eigenbasis at t = (k+1) dt and ``rholist`` transformed
    back to the site basis.  ``return_result=False``: writes ``obs.dat``
    (observables before each step) and returns the final vec(rho).
    A batch of initial states (B, n, n) gives (B, Nt, n_e) observables.
    ``precision='split'`` runs the RK4 on the tensor cores
    (``propagate_vec_split``); stored states then come from restarting the
    split run every step, so pass ``store_states=False`` for long runs.
    """
    e_ops = [] if e_ops is None else list(e_ops)
    dev = engine._dev(None)
    Rg = _as_generator(R, dev)
    n = Rg[1]
    r0 = np.asarray(_dense(rho0) if np.ndim(rho0) == 2 else rho0)
    batched = r0.ndim == 3
    r0 = r0.reshape((-1, n, n)).astype(np.complex128)
    V = None if evecs is None else torch.as_tensor(np.asarray(evecs), dtype=CDT, device=dev)
    r0t = torch.as_tensor(r0, dtype=CDT, device=dev)
    if V is not None:
        r0t = zl.to_basis(V, r0t)
    e_eb = [torch.as_tensor(_dense(e), dtype=CDT, device=dev) for e in e_ops]
    if V is not None and e_eb:
        e_eb = list(zl.to_basis(V, torch.stack(e_eb)))
    if not return_result:
        o, _, rho = _propagate(Rg, r0t, dt, Nt, e_eb, precision=precision)
        # Tr(E rho0) = sum_ij E[j, i] rho0[i, j]
        first = zl.mm(r0t.reshape(r0t.shape[0], -1),
                      torch.stack([e.transpose(0, 1) for e in e_eb]).reshape(len(e_eb), -1).t()) \
            if e_eb else None
        ob = o[0].cpu().numpy()
        rows = [first[0].cpu().numpy()] + [ob[k] for k in range(Nt - 1)] if e_eb else [[]] * Nt
        fmt = '{} ' * (len(e_ops) + 1) + '\n'
        with open('obs.dat', 'w') as f:
            t = t0
            for k in range(Nt):
                t += dt
                f.write(fmt.format(t, *rows[k]))
        out = rho.reshape(rho.shape[0], -1).cpu().numpy()
        return out if batched else out[0]
    o, st, rho = _propagate(Rg, r0t, dt, Nt, e_eb, states_every=1 if store_states else 0,
                            precision=precision)
    res = Result(dt=dt, Nt=Nt, rho0=rho0, t0=t0, nout=1)
    obs_np = o.cpu().numpy()
    res.observables = obs_np if batched else obs_np[0]
    if st is not None:
        if V is not None:
            st = zl.from_basis(V, st.reshape(-1, n, n)).reshape(st.shape)
        stn = st.cpu().numpy()
        res.rholist = stn if batched else list(stn[0])
    else:
        fin = rho if V is None else zl.from_basis(V, rho)
        res.rholist = fin.cpu().numpy() if batched else [fin[0].cpu().numpy()]
    return res


class Redfield_solver:
    """Bloch-Redfield solver (lime/oqs.py:40-371)."""

    def __init__(self, H, c_ops=None, spectra=None, e_ops=None):
        self.H = H
        self.c_ops = c_ops
        self.R = None
        self.spectra = spectra
        self.evecs = None
        self.dim = H.shape[0]
        self.U = None
        self.G = None
        self.e_ops = e_ops

    def idm(self, sp=True):
        from scipy.sparse import identity
        from .superoperator import dm2vec
        return dm2vec(identity(self.dim)) if sp else dm2vec(identity(self.dim).toarray())

    def configure(self, H, c_ops, e_ops):
        self.c_ops = c_ops
        self.e_ops = e_ops
        self.H = H

    def redfield_tensor(self, secular=False):
        if self.spectra is None:
            raise TypeError('Specify the bath spectral function.')
        R, evecs = redfield_tensor(self.H, self.c_ops, self.spectra, secular)
        self.R = R
        self.evecs = evecs
        return R, evecs

    def evolve(self, rho0, dt, Nt, evecs=None, e_ops=[], store_states=False, t0=0, nout=1,
               precision='fp64'):
        if self.R is None:
            self.redfield_tensor()
        return _redfield(self.R, rho0, evecs=self.evecs, Nt=Nt, dt=dt, t0=t0, e_ops=e_ops,
                         store_states=True if precision == 'fp64' else store_states,
                         precision=precision)

    def steady_state(self):
        pass

    # ---------------- Green's-function route (lime/oqs.py:169-366)
    def propagator(self, t, method='SOS'):
        """U(t) = exp(R t) for the times t, shape (D, D, len(t)).

        ``method='SOS'``: eigen-decomposition of R (lime/oqs.py:205-216);
        ``'EOM'``: RK4 of U with the generator (lime/oqs.py:195-203, the
        reference's expm(A, t) integrates dU/dt = A U on the grid t).
        """
        if self.R is None:
            raise TypeError('Redfield tensor is not computed. Please call redfield_tensor()')
        t = np.asarray(t, dtype=np.float64)
        Rd = self.R.R
        if method in ('eseries', 'SOS'):
            # eigen-decomposition on the host, as the reference (scipy eig
            # and inv); U[:, :, k] = U1 diag(exp(w t_k)) U1^-1 for every k as
            # one strided batched GEMM on the device
            w, U1 = scipy.linalg.eig(Rd.cpu().numpy())
            U2 = scipy.linalg.inv(U1)
            Et = np.exp(w[:, np.newaxis] * t[np.newaxis, :])
            dev = Rd.device
            D = Rd.shape[0]
            U = torch.empty((D, D, len(t)), dtype=CDT, device=dev)
            zl.bmm(torch.as_tensor(U1, dtype=CDT, device=dev).unsqueeze(0),
                   torch.as_tensor(U2, dtype=CDT, device=dev).unsqueeze(0),
                   scale=torch.as_tensor(Et, dtype=CDT, device=dev).t(), out=U.permute(2, 0, 1))
        elif method == 'EOM':
            n = self.R.n
            D = n * n
            eye = torch.eye(D, dtype=CDT, device=Rd.device).reshape(D, n, n)
            dt = t[1] - t[0] if len(t) > 1 else 0.0
            Us = [torch.eye(D, dtype=CDT, device=Rd.device)]
            if len(t) > 1:
                _, st, _ = propagate_vec((Rd, n), eye, dt, len(t) - 1, None, states_every=1)
                for k in range(len(t) - 1):
                    Us.append(st[:, k].reshape(D, D).transpose(0, 1))
            U = torch.stack(Us, -1)
        else:
            raise NotImplementedError('Method of {} has not been implemented.'.format(method))
        self.U = U
        self.G = -1j * U
        return U.cpu().numpy()

    def expect(self, rho0, e_ops):
        """<E_j>(t_k) = vec(E_j)^T U(t_k) vec(rho0) in the eigenbasis
        (lime/oqs.py:218-252)."""
        U = self.U
        dev = U.device
        V = torch.as_tensor(np.asarray(self.evecs), dtype=CDT, device=dev)
        rho0_eb = zl.to_basis(V, torch.as_tensor(_dense(rho0), dtype=CDT, device=dev)).reshape(-1, 1)
        rho = zl.green_apply(U, rho0_eb)[:, :, 0]                              # (D, Nt)
        if not len(e_ops):
            return np.zeros((U.shape[-1], 0), dtype=np.complex128)
        E = zl.to_basis(V, torch.stack([torch.as_tensor(_dense(e), dtype=CDT, device=dev) for e in e_ops]))
        out = zl.mm(E.reshape(len(e_ops), -1), rho)                            # (n_e, Nt)
        return out.t().cpu().numpy()

    def correlation_2op_1t(self, rho0, a, b, tau):
        """<<I| a G(tau) b |rho0>> (lime/oqs.py:254-275) with a dense identity
        vector (the reference's sparse one cannot be contracted)."""
        if self.G is None:
            self.propagator(tau)
        G = self.G
        dev = G.device
        idm = torch.as_tensor(np.identity(self.dim).flatten(), dtype=CDT, device=dev)
        r = _dense(rho0)
        if r.ndim == 2:
            r = r.flatten()
        at = torch.as_tensor(_dense(a), dtype=CDT, device=dev)
        bt = torch.as_tensor(_dense(b), dtype=CDT, device=dev)
        x = zl.mm(bt, torch.as_tensor(r, dtype=CDT, device=dev).reshape(-1, 1))
        y = zl.green_apply(G, x)[:, :, 0]                                       # (D, Nt)
        return zl.mm(zl.mm(idm.reshape(1, -1), at), y)[0].cpu().numpy()

    def correlation_4op_3t(self, rho0, oplist, signature, tau):
        """<<I|A G(t3) B G(t2) C G(t1) D|rho0>> (lime/oqs.py:277-366)."""
        from .superoperator import operator_to_superoperator
        if len(oplist) != 4:
            raise ValueError('Number of operators is not 4.')
        if self.G is None:
            self.propagator(tau)
        G = self.G
        dev = G.device
        ops = [torch.as_tensor(operator_to_superoperator(o, s).toarray(), dtype=CDT, device=dev)
               for o, s in zip(oplist, signature)]
        a, b, c, d = ops
        idm = torch.as_tensor(np.identity(self.dim).flatten(), dtype=CDT, device=dev)
        D = G.shape[0]

        def left(op, x):          # op (D, D) applied to the first index of x
            return zl.mm(op, x.reshape(D, -1)).reshape(x.shape)

        rho = zl.mm(d, torch.as_tensor(_dense(rho0).flatten(), dtype=CDT, device=dev).reshape(-1, 1))[:, 0]
        tmp = zl.green_apply(G, rho)                 # (D, Nt)
        tmp = left(c, tmp)
        tmp = zl.green_apply(G, tmp)                 # (D, Nt, Nt)
        tmp = left(b, tmp)
        tmp = zl.green_apply(G, tmp)                 # (D, Nt, Nt, Nt)
        v = zl.mm(idm.reshape(1, -1), a)             # <<I| a
        return zl.mm(v, tmp.reshape(D, -1)).reshape(tmp.shape[1:]).cpu().numpy()
