"""Device-side orchestration of the Lindblad propagators.

``LindbladGenerator`` holds one or many Lindblad generators on the GPU
(``Heff``, ``M`` and the dense collapse operators, built by the
``lime_lindblad_prepare_f64`` kernel).  ``propagate`` runs RK4 on a batch of
density matrices through the C ABI and returns device tensors.

Array conventions: complex128, row-major, instance-major; torch tensors are
used only as device buffers whose ``data_ptr()`` is handed to the kernels.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as nat

CDT = torch.complex128


def _dev(device=None):
    if device is None:
        return torch.device('cuda', torch.cuda.current_device())
    return torch.device(device)


def _to_dense_np(a):
    if hasattr(a, 'toarray'):
        a = a.toarray()
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    return np.asarray(a)


def as_device(a, device, dtype=CDT) -> torch.Tensor:
    """Dense complex128 device tensor from ndarray / scipy.sparse / tensor."""
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(_to_dense_np(a), dtype=dtype, device=device).contiguous()


def _stream_ptr():
    return torch.cuda.current_stream().cuda_stream


def _ptr(t):
    return None if t is None else t.data_ptr()


class DiagonalOps:
    """K diagonal collapse operators given by their diagonals.

    ``l`` has shape (K, n) (shared) or (P, K, n) (one set per instance);
    operator k is ``diag(l[..., k, :])``.  Equivalent to passing the K dense
    diagonal matrices, without materialising them (a dephasing ensemble of
    4096 64-site chains is 268 MB this way instead of 17 GB).
    """

    def __init__(self, l):
        self.l = l


class SiteDephasing:
    """Pure site dephasing given by its rates: the n collapse operators
    sqrt(rates[k]) |k><k|, k = 0 .. n-1.  ``rates`` has shape (n,) (shared)
    or (P, n) (one set per instance).  Equivalent to
    ``DiagonalOps(diag_embed(sqrt(rates)))``, with n values per instance
    passed instead of n^2."""

    def __init__(self, rates):
        self.rates = rates

    def rates_on(self, device) -> torch.Tensor:
        """The rates as a float64 tensor on ``device``: (n,) or (P, n)."""
        g = self.rates
        g = g.to(device=device, dtype=torch.float64) if isinstance(g, torch.Tensor) else \
            torch.as_tensor(np.asarray(g, dtype=np.float64), device=device)
        if g.dim() not in (1, 2):
            raise ValueError('SiteDephasing rates must be (n,) or (P, n)')
        return g

    def diagonal_ops(self, device) -> DiagonalOps:
        return DiagonalOps(torch.diag_embed(torch.sqrt(self.rates_on(device))).to(CDT))


class Populations:
    """Observables given compactly: the populations rho_kk of sites
    k = 0 .. count-1, i.e. the projectors |k><k| as e_ops.  Equivalent to
    passing those dense projectors (which are recognised too), without
    building or inspecting count n x n matrices per call."""

    def __init__(self, count: int):
        self.count = int(count)

    def __len__(self):
        return self.count

    def dense(self, n: int) -> list:
        out = []
        for k in range(self.count):
            e = np.zeros((n, n), dtype=np.complex128)
            e[k, k] = 1.0
            out.append(e)
        return out


def expand_e_ops(e_ops, n: int):
    """e_ops as a list of operators (a Populations object becomes its dense
    projectors)."""
    if isinstance(e_ops, Populations):
        if e_ops.count > n:
            raise ValueError('%d populations of a %d-dimensional system' % (e_ops.count, n))
        return e_ops.dense(n)
    return e_ops


def is_diagonal(op: torch.Tensor) -> bool:
    n = op.shape[-1]
    off = op * (1 - torch.eye(n, dtype=op.dtype, device=op.device))
    return bool(torch.count_nonzero(off) == 0)


@dataclass
class LindbladGenerator:
    """``P`` Lindblad generators of dimension ``n`` resident on the device."""
    n: int
    P: int
    heff: torch.Tensor            # (P|1, n, n)
    m: torch.Tensor | None        # (P|1, n, n) or None
    l_dense: torch.Tensor | None  # (P|1, K, n, n) or None
    k_dense: int
    shared: bool                  # one generator for every instance
    # operands of the batched split kernel, built on first use (split_operands)
    split_cache: dict = field(default_factory=dict, repr=False, compare=False)

    @staticmethod
    def build(H, c_ops=None, device=None) -> 'LindbladGenerator':
        """Generators from ``H`` ((n,n) or (P,n,n)) and ``c_ops``.

        ``c_ops`` is a list of K operators, each (n,n) (shared) or (P,n,n).
        Diagonal operators enter through ``M``; the rest are kept dense.
        """
        lib = nat.require_device()
        device = _dev(device)
        Hd = as_device(H, device)
        if Hd.dim() == 2:
            Hd = Hd.unsqueeze(0)
        if Hd.dim() != 3 or Hd.shape[-1] != Hd.shape[-2]:
            raise ValueError('H must be (n, n) or (P, n, n); got %s' % (tuple(Hd.shape),))
        n = Hd.shape[-1]
        c_ops = list(c_ops or [])
        # site dephasing enters the preparation kernel as its rates
        rates = [c.rates_on(device) for c in c_ops if isinstance(c, SiteDephasing)]
        c_ops = [c for c in c_ops if not isinstance(c, SiteDephasing)]
        packed = [as_device(c.l, device) for c in c_ops if isinstance(c, DiagonalOps)]
        ops = [as_device(c, device) for c in c_ops if not isinstance(c, DiagonalOps)]
        P = Hd.shape[0]
        for r in rates:
            if r.shape[-1] != n:
                raise ValueError('SiteDephasing rates must be (%d,) or (P, %d)' % (n, n))
            if r.dim() == 2:
                if P not in (1, r.shape[0]):
                    raise ValueError('inconsistent batch sizes in H and c_ops')
                P = r.shape[0]
        for p in packed:
            if p.shape[-1] != n or p.dim() not in (2, 3):
                raise ValueError('DiagonalOps.l must be (K, %d) or (P, K, %d)' % (n, n))
            if p.dim() == 3:
                if P not in (1, p.shape[0]):
                    raise ValueError('inconsistent batch sizes in H and c_ops')
                P = p.shape[0]
        for c in ops:
            if c.shape[-2:] != (n, n):
                raise ValueError('collapse operator shape %s does not match H (%d, %d)'
                                 % (tuple(c.shape), n, n))
            if c.dim() == 3:
                if P not in (1, c.shape[0]):
                    raise ValueError('inconsistent batch sizes in H and c_ops')
                P = c.shape[0]
        shared = (P == 1)
        diag = [c for c in ops if is_diagonal(c)]
        dense = [c for c in ops if not is_diagonal(c)]

        def stack(lst, per):
            # -> (P|1, K, ...) with per-instance broadcast when mixed
            if not lst:
                return None
            if all(x.dim() == per for x in lst):
                return torch.stack(lst, 0).unsqueeze(0).contiguous()
            return torch.stack([x.expand((P,) + x.shape[-per:]) if x.dim() == per else x
                                for x in lst], 1).contiguous()

        ld = stack(dense, 2)
        lg = stack([torch.diagonal(x, dim1=-2, dim2=-1) for x in diag], 1)
        if packed:
            parts = ([] if lg is None else [lg]) + [p if p.dim() == 3 else p.unsqueeze(0) for p in packed]
            if any(x.shape[0] != 1 for x in parts):
                parts = [x.expand((P,) + x.shape[1:]) for x in parts]
            lg = parts[0].contiguous() if len(parts) == 1 else torch.cat(parts, 1).contiguous()
        rate = None
        if rates:
            rate = rates[0]
            for r in rates[1:]:
                rate = rate + r
            rate = (rate if rate.dim() == 2 else rate.unsqueeze(0)).contiguous()
        Hs = Hd.contiguous()
        heff = torch.empty((P, n, n), dtype=CDT, device=device)
        m = torch.empty((P, n, n), dtype=CDT, device=device)
        d = nat.PrepareDesc()
        d.n, d.batch = n, P
        d.k_dense = 0 if ld is None else ld.shape[1]
        d.k_diag = 0 if lg is None else lg.shape[1]
        d.h, d.h_stride = Hs.data_ptr(), (0 if Hs.shape[0] == 1 else n * n)
        if ld is not None:
            d.l_dense, d.l_dense_stride = ld.data_ptr(), (0 if ld.shape[0] == 1 else d.k_dense * n * n)
        if lg is not None:
            d.l_diag, d.l_diag_stride = lg.data_ptr(), (0 if lg.shape[0] == 1 else d.k_diag * n)
        if rate is not None:
            d.dephasing, d.dephasing_stride = rate.data_ptr(), (0 if rate.shape[0] == 1 else n)
        d.heff, d.m = heff.data_ptr(), m.data_ptr()
        nat.check(lib.lime_lindblad_prepare_f64(d, _stream_ptr()), 'lime_lindblad_prepare_f64')
        gen = LindbladGenerator(n=n, P=P, heff=heff, m=(m if lg is not None or rate is not None else None),
                                l_dense=ld, k_dense=d.k_dense, shared=shared)
        if lg is None and rate is not None:
            gen.split_cache['m_diagonal'] = True   # site dephasing alone: M = diag(rates)
        return gen


def hermitian_parts(rho: torch.Tensor):
    """rho = A + i B with A = (rho + rho^dag)/2 and B = (rho - rho^dag)/(2i), both Hermitian."""
    rh = rho.mH
    return (rho + rh) / 2, (rho - rh) / 2j


def prepare_obs(e_ops, n, P, device):
    """Stack observables: returns (tensor, n_obs, obs_diag, stride)."""
    if isinstance(e_ops, Populations):
        if e_ops.count > n:
            raise ValueError('%d populations of a %d-dimensional system' % (e_ops.count, n))
        if not e_ops.count:
            return None, 0, 0, 0
        Et = torch.zeros((1, e_ops.count, n), dtype=CDT, device=device)
        idx = torch.arange(e_ops.count, device=device)
        Et[0, idx, idx] = 1
        return Et, e_ops.count, 1, 0
    if not e_ops:
        return None, 0, 0, 0
    E = [as_device(e, device) for e in e_ops]
    per = any(e.dim() == 3 for e in E)
    if per:
        E = [e.expand(P, n, n) if e.dim() == 2 else e for e in E]
        Et = torch.stack(E, 1)  # (P, n_obs, n, n)
    else:
        Et = torch.stack(E, 0).unsqueeze(0)  # (1, n_obs, n, n)
    n_obs = Et.shape[1]
    diag = all(is_diagonal(e) for e in E)
    if diag:
        Et = torch.diagonal(Et, dim1=-2, dim2=-1).contiguous()  # (P|1, n_obs, n)
        stride = 0 if Et.shape[0] == 1 else n_obs * n
    else:
        Et = Et.contiguous()
        stride = 0 if Et.shape[0] == 1 else n_obs * n * n
    return Et, n_obs, int(diag), stride


def _run_f64(gen: LindbladGenerator, rho: torch.Tensor, dt: float, n_steps: int,
             obs, obs_every: int, states_every: int, trace_tol: float, param_batch: int,
             events=None, drive=None):
    lib = nat.require_device()
    B, n = rho.shape[0], gen.n
    Et, n_obs, obs_diag, obs_stride = obs
    obs_out = torch.zeros((B, n_steps // obs_every, max(n_obs, 1)), dtype=CDT, device=rho.device)
    states = None
    if states_every > 0:
        states = torch.empty((B, n_steps // states_every, n, n), dtype=CDT, device=rho.device)
    wsb = lib.lime_lindblad_rk4_f64_workspace(n, B, gen.k_dense)
    ws = torch.empty(wsb, dtype=torch.uint8, device=rho.device)
    status = torch.zeros(1, dtype=torch.int32, device=rho.device)
    d = nat.LindbladDesc()
    d.n, d.batch, d.param_batch, d.n_steps = n, B, param_batch, n_steps
    d.k_dense, d.n_obs, d.obs_diag, d.obs_every = gen.k_dense, n_obs, obs_diag, obs_every
    d.states_every = states_every if states is not None else 0
    d.dt, d.trace_tol = float(dt), float(trace_tol)
    d.rho = rho.data_ptr()
    d.heff, d.heff_stride = gen.heff.data_ptr(), (0 if gen.heff.shape[0] == 1 else n * n)
    if gen.m is not None:
        d.m, d.m_stride = gen.m.data_ptr(), (0 if gen.m.shape[0] == 1 else n * n)
    if gen.l_dense is not None:
        d.l_dense = gen.l_dense.data_ptr()
        d.l_dense_stride = 0 if gen.l_dense.shape[0] == 1 else gen.k_dense * n * n
    if Et is not None:
        d.obs_ops, d.obs_stride = Et.data_ptr(), obs_stride
        d.obs_out = obs_out.data_ptr()
    d.states = _ptr(states)
    d.workspace, d.workspace_bytes = ws.data_ptr(), wsb
    d.status = status.data_ptr()
    if drive is not None:
        ops, coef = drive
        d.n_drive, d.drive_ops, d.drive_coef = ops.shape[0], ops.data_ptr(), coef.data_ptr()
    if events is not None:
        events[0].record()
    nat.check(lib.lime_lindblad_rk4_f64(d, _stream_ptr()), 'lime_lindblad_rk4_f64')
    if events is not None:
        events[1].record()
    return obs_out[:, :, :n_obs], states, status


SPLIT_MAX_N = 64


def split_supported(gen: LindbladGenerator) -> str | None:
    """None if the batched tensor-core kernel handles ``gen``, else the
    reason it does not (decided once per generator)."""
    c = gen.split_cache
    if 'why' not in c:
        why = None
        if gen.n > SPLIT_MAX_N:
            why = 'dimension %d > %d' % (gen.n, SPLIT_MAX_N)
        elif gen.k_dense:
            why = 'dense (non-diagonal) collapse operators'
        elif gen.m is not None and not c.get('m_diagonal') and not is_diagonal(gen.m):
            why = 'diagonal collapse operators with a non-diagonal M = sum_k l_k l_k^dag'
        c['why'] = why
    return c['why']


def _pow2_exponent(target: float, bound: float) -> int:
    import math
    if not bound > 0 or not math.isfinite(bound):
        return 0
    return int(math.floor(math.log2(target / bound)))


def heff_amax(gen: LindbladGenerator) -> float:
    """max |Heff| over every generator (computed once per generator)."""
    c = gen.split_cache
    if 'amax' not in c:
        c['amax'] = float(gen.heff.abs().max().item())
    return c['amax']


def split_operands(gen: LindbladGenerator) -> dict:
    """Operands of the batched split kernel, built once per generator: the A
    operand (``lime_lindblad_split_prepare``: 2^a Heff in its fixed-point +
    two fp16 pieces, in the kernel's tensor-memory order), its scale exponent
    a (max |2^a Heff| in [2^12, 2^13)) and the real diagonal of M."""
    c = gen.split_cache
    if 'pieces' not in c:
        lib = nat.require_device()
        sa = _pow2_exponent(4096.0, heff_amax(gen))
        count = gen.heff.shape[0]
        nbytes = int(lib.lime_lindblad_split_prepared_bytes(gen.n, count))
        pieces = torch.empty(nbytes, dtype=torch.uint8, device=gen.heff.device)
        d = nat.SplitPrepareDesc()
        d.n, d.count, d.scale_a_log2 = gen.n, count, sa
        d.heff, d.heff_stride = gen.heff.data_ptr(), (gen.n * gen.n if count > 1 else 0)
        d.out, d.out_bytes = pieces.data_ptr(), nbytes
        nat.check(lib.lime_lindblad_split_prepare(d, _stream_ptr()), 'lime_lindblad_split_prepare')
        c['pieces'], c['stride'], c['scale_a'] = pieces, (nbytes // count if count > 1 else 0), sa
    split_operands_mdiag(gen)
    return c


def _is_diag_host(a) -> bool:
    """A host operator (or a stack of them) with no nonzero off-diagonal entry."""
    a = np.asarray(a)
    if a.ndim < 2 or a.shape[-1] != a.shape[-2]:
        return False
    n = a.shape[-1]
    m = a.reshape(-1, n, n)
    return not np.any(m[:, ~np.eye(n, dtype=bool)])


def _host_array(a):
    """NumPy view of a host operand, or None for a device tensor."""
    if isinstance(a, torch.Tensor):
        return a.detach().resolve_conj().numpy() if a.device.type == 'cpu' else None
    return _to_dense_np(a)


def _is_population(e, k, n) -> bool:
    """e == |k><k| (n x n), checked on the host."""
    if e is None or e.shape != (n, n) or e[k, k] != 1:
        return False
    return int(np.count_nonzero(e)) == 1


def _split_obs(e_ops, n, P, device):
    """(mode, n_obs, tensor, stride) for the split kernel.  Site
    populations given as host arrays are recognised on the host (no device
    round trip); device tensors are compared on the device."""
    if isinstance(e_ops, SplitObs):
        return e_ops.spec
    if isinstance(e_ops, Populations):
        if e_ops.count > n:
            raise ValueError('%d populations of a %d-dimensional system' % (e_ops.count, n))
        return (1, e_ops.count, None, 0) if e_ops.count else (0, 0, None, 0)
    if not e_ops:
        return 0, 0, None, 0
    if len(e_ops) <= n:
        host = [_host_array(e) for e in e_ops]
        if all(h is not None for h in host):
            if all(_is_population(h, k, n) for k, h in enumerate(host)):
                return 1, len(e_ops), None, 0
            E = [torch.as_tensor(h, dtype=CDT, device=device) for h in host]
        else:
            E = [as_device(e, device) for e in e_ops]
            if all(e.dim() == 2 for e in E):
                pops = torch.zeros((len(E), n, n), dtype=CDT, device=device)
                idx = torch.arange(len(E), device=device)
                pops[idx, idx, idx] = 1
                if torch.equal(torch.stack(E), pops):
                    return 1, len(E), None, 0
    else:
        E = [as_device(e, device) for e in e_ops]
    per = any(e.dim() == 3 for e in E)
    if per:
        Et = torch.stack([e.expand(P, n, n) if e.dim() == 2 else e for e in E], 1).contiguous()
        return 2, len(E), Et, len(E) * n * n
    return 2, len(E), torch.stack(E, 0).unsqueeze(0).contiguous(), 0


def _run_split(gen: LindbladGenerator, rho: torch.Tensor, dt: float, n_steps: int, e_ops,
               obs_every: int, trace_tol: float, param_batch: int, events=None,
               ctas_per_sm: int = 0, drive=None, rho_out=None, chunk_steps: int = 0):
    """The batched tensor-core kernel (n <= 64, diagonal collapse operators).
    The A operand is split once per generator (``split_operands``); each
    instance takes its state scale from its own rho(0) on the device
    (sqrt(n) ||rho(0)||_F bounds |rho_ij(t)|: the trace norm contracts) and
    the kernel picks each B row's fixed-point quantum from the previous
    stage's row bound, so nothing here waits for the GPU.  The final state
    goes to ``rho_out`` (None: over ``rho``).  ``drive`` = (ops (n_drive, n,
    n), coef (n_steps, n_drive)): Heff(t) = Heff - sum_d coef[k, d] ops[d],
    re-split on the device every step; the A scale then covers max|Heff| +
    sum_d max|coef_d| max|ops_d|."""
    lib = nat.require_device()
    why = split_supported(gen)
    if why is not None:
        raise ValueError('precision="split" does not support this generator: ' + why)
    B, n = rho.shape[0], gen.n
    mode, n_obs, Et, obs_stride = _split_obs(e_ops, n, gen.P, rho.device)
    obs_out = torch.empty((B, n_steps // obs_every, max(n_obs, 1)), dtype=CDT, device=rho.device)
    status = torch.zeros(1, dtype=torch.int32, device=rho.device)
    ws = None
    if drive is not None:
        prep = None
        m_diag = split_operands_mdiag(gen)
        dops, dcoef = drive
        if dcoef.shape[0] < n_steps:
            raise ValueError('drive coefficients cover %d steps, %d requested' % (dcoef.shape[0], n_steps))
        amax = heff_amax(gen) + float((dcoef.abs().amax(0) * dops.abs().amax((-2, -1))).sum().item())
        ws = torch.empty(int(lib.lime_lindblad_split_workspace(n, param_batch, dops.shape[0], n_steps)),
                         dtype=torch.uint8, device=rho.device)
        scale_a = _pow2_exponent(4096.0, amax)
    else:
        prep = split_operands(gen)
        m_diag = prep['m_diag']
        scale_a = prep['scale_a']
    d = nat.SplitDesc()
    d.n, d.batch, d.param_batch, d.n_steps = n, B, param_batch, n_steps
    d.obs_mode, d.n_obs, d.obs_every = mode, n_obs, obs_every
    d.scale_a_log2 = scale_a
    d.scale_b_log2 = 0
    d.auto_scale_b = 1
    if prep is not None:
        d.a_pieces, d.a_stride = prep['pieces'].data_ptr(), prep['stride']
    if rho_out is not None:
        d.rho_out = rho_out.data_ptr()
    d.ctas_per_sm = ctas_per_sm
    d.chunk_steps = chunk_steps
    d.dt, d.trace_tol = float(dt), float(trace_tol)
    d.rho = rho.data_ptr()
    d.heff, d.heff_stride = gen.heff.data_ptr(), (0 if gen.heff.shape[0] == 1 else n * n)
    if m_diag is not None:
        d.m_diag, d.m_stride = m_diag.data_ptr(), (0 if m_diag.shape[0] == 1 else n)
    if Et is not None:
        d.obs_ops, d.obs_stride = Et.data_ptr(), obs_stride
    d.obs_out = obs_out.data_ptr()
    d.status = status.data_ptr()
    if drive is not None:
        d.n_drive, d.drive_ops, d.drive_coef = dops.shape[0], dops.data_ptr(), dcoef.data_ptr()
        d.workspace, d.workspace_bytes = ws.data_ptr(), ws.numel()
    if events is not None:
        events[0].record()
    nat.check(lib.lime_lindblad_rk4_split(d, _stream_ptr()), 'lime_lindblad_rk4_split')
    if events is not None:
        events[1].record()
    return obs_out[:, :, :n_obs], None, status


def split_operands_mdiag(gen: LindbladGenerator):
    """The real diagonal of M (cached on the generator), or None."""
    c = gen.split_cache
    if 'm_diag' not in c:
        c['m_diag'] = (None if gen.m is None else
                       torch.diagonal(gen.m, dim1=-2, dim2=-1).real.contiguous())
    return c['m_diag']


def _run_stream(gen: LindbladGenerator, rho: torch.Tensor, dt: float, n_steps: int, e_ops,
                obs_every: int, param_batch: int, events=None, max_retries: int = 3, drive=None,
                defer: bool = False, sink=None):
    """Any generator on the tensor cores (``lime_lindblad_rk4_stream``):
    streaming split-precision GEMMs for Heff rho and sum_k L_k rho L_k^dag.
    State scale: max |rho0| * 1.25 <= 2^13; L_k rho scale from the largest
    absolute row sum of the collapse operators; a run whose values leave the
    fixed-point range raises LIME_FLAG_RANGE and is repeated with both
    scales lowered 4x.  Returns (obs, None, status, final rho, redo):
    ``redo()`` relaunches with 4x smaller scales and returns the new
    (obs, status, rho).  With ``defer=True`` the range check is left to the
    caller (no host synchronisation after the launch, so launches on other
    streams are enqueued without waiting); otherwise it is done here.
    ``sink``: a list that receives the descriptor (with the buffers it
    points to) instead of launching it, for one grouped launch of several
    propagations (``lime_lindblad_rk4_stream_groups``); implies defer, and
    retries relaunch the propagation on its own."""
    lib = nat.require_device()
    B, n = rho.shape[0], gen.n
    dev = rho.device
    K = gen.k_dense
    E = None
    n_obs = 0
    obs_diag = False
    if e_ops:
        # diagonal observables (populations) go in as their diagonals: the
        # readout then touches n state elements instead of n^2; decided on
        # the host for host operators
        host = [_host_array(e) for e in e_ops]
        obs_diag = all(h is not None and _is_diag_host(h) for h in host)
        Es = [as_device(e, dev) for e in e_ops]
        if any(e.dim() == 3 for e in Es):
            E = torch.stack([e.expand(gen.P, n, n) if e.dim() == 2 else e for e in Es], 1).contiguous()
        else:
            E = torch.stack(Es, 0).unsqueeze(0).contiguous()
        n_obs = E.shape[1]
        if not obs_diag and any(h is None for h in host):
            # device operators: one check per call
            obs_diag = bool(is_diagonal(E.reshape(-1, n, n)))
        if obs_diag:
            E = torch.diagonal(E, dim1=-2, dim2=-1).contiguous()
    n_slots = n_steps // obs_every
    obs_out = torch.zeros((B, max(n_slots, 1), max(n_obs, 1)), dtype=CDT, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    pmax = float(torch.view_as_real(rho).abs().max().item()) if rho.numel() else 0.0
    lrow = 0.0
    if K:
        lrow = float(gen.l_dense.abs().sum(-1).max().item())
    scales = [_pow2_exponent(8192.0 / 1.25, pmax), _pow2_exponent(8192.0 / 1.25, lrow * pmax) if K else 0]
    heff_shared = gen.heff.shape[0] == 1
    l_shared = gen.l_dense is None or gen.l_dense.shape[0] == 1
    # a diagonal M (pure dephasing) goes in as its real diagonal
    m_diag = None
    if gen.m is not None and (gen.split_cache.get('m_diagonal') or is_diagonal(gen.m)):
        m_diag = torch.diagonal(gen.m, dim1=-2, dim2=-1).real.contiguous()
    G = 1 if (heff_shared and l_shared) else param_batch
    wsb = lib.lime_lindblad_stream_workspace(n, B, G, K)
    ws = torch.empty(wsb + 1024, dtype=torch.uint8, device=dev)
    aligned = (ws.data_ptr() + 1023) // 1024 * 1024
    start = rho.contiguous()

    def launch(alone=False):
        work = start.clone()
        status.zero_()
        d = nat.LindbladStreamDesc()
        d.n, d.batch, d.param_batch, d.n_ops = n, B, param_batch, K
        d.n_steps, d.n_obs, d.obs_every = n_steps, n_obs, obs_every
        d.scale_b_log2, d.scale_y_log2 = max(-60, min(60, scales[0])), max(-60, min(60, scales[1]))
        d.dt = float(dt)
        d.rho = work.data_ptr()
        d.heff, d.heff_stride = gen.heff.data_ptr(), (0 if heff_shared else n * n)
        if m_diag is not None:
            d.m_diag, d.m_diag_stride = m_diag.data_ptr(), (0 if m_diag.shape[0] == 1 else n)
        elif gen.m is not None:
            d.m, d.m_stride = gen.m.data_ptr(), (0 if gen.m.shape[0] == 1 else n * n)
        if K:
            d.l_ops, d.l_stride = gen.l_dense.data_ptr(), (0 if l_shared else K * n * n)
        if E is not None:
            d.obs_ops, d.obs_stride = E.data_ptr(), (0 if E.shape[0] == 1 else E[0].numel())
            d.obs_out = obs_out.data_ptr()
            d.obs_diag = int(obs_diag)
        d.workspace, d.workspace_bytes = aligned, wsb
        d.status = status.data_ptr()
        if drive is not None:
            ops, coef = drive
            d.n_drive, d.drive_ops, d.drive_coef = ops.shape[0], ops.data_ptr(), coef.data_ptr()
        if sink is not None and not alone:
            sink.append((d, (work, start, ws, obs_out, status, E, m_diag, gen)))
            return work
        if events is not None:
            events[0].record()
        nat.check(lib.lime_lindblad_rk4_stream(d, _stream_ptr()), 'lime_lindblad_rk4_stream')
        if events is not None:
            events[1].record()
        return work

    def redo():
        scales[0] -= 2
        scales[1] -= 2
        return obs_out[:, :n_slots, :n_obs], status, launch(alone=True)

    work = launch()
    if not defer and sink is None:
        for _ in range(max_retries):
            if not int(status.item()) & nat.LIME_FLAG_RANGE:
                break
            _, _, work = redo()
    return obs_out[:, :n_slots, :n_obs], None, status, work, redo


def _host_hermitian(rho0):
    """Hermiticity of a host rho0 (NumPy, scipy or CPU tensor), checked on
    the host before the upload; None for a device tensor."""
    a = _host_array(rho0)
    if a is None:
        return None
    return bool(np.array_equal(a, np.conj(np.swapaxes(a, -1, -2))))


def _launch(gen: LindbladGenerator, rho0, dt: float, n_steps: int, e_ops=None,
            states_every: int = 0, precision: str = 'fp64', trace_tol: float | None = None,
            obs_every: int = 1, events=None, drive=None, defer: bool = False,
            hermitian: bool | None = None, stream_sink=None):
    """Enqueue one propagation on the current stream; returns a closure that
    checks the status word (synchronising the stream) and assembles
    ``(obs, states, rho)``.  ``defer``: nothing after the launch waits for
    the GPU (range retries of the streaming path happen in the closure).

    Every kernel acts on Hermitian states; a non-Hermitian rho0 runs as its
    two Hermitian parts.  Hermiticity is checked on the host for host
    inputs; for a device tensor the batched split kernel checks it itself
    (LIME_FLAG_NOT_HERMITIAN, after which the closure reruns the two parts),
    the other paths compare rho0 with its adjoint on the device.
    ``stream_sink``: see ``_run_stream`` (a propagation on the streaming
    path is collected there instead of launched)."""
    if obs_every < 1 or states_every < 0 or n_steps < 0:
        raise ValueError('obs_every must be >= 1, states_every >= 0, n_steps >= 0')
    device = gen.heff.device
    herm = _host_hermitian(rho0) if hermitian is None else hermitian
    rho = as_device(rho0, device)
    if rho.dim() == 2:
        rho = rho.unsqueeze(0)
    B, n = rho.shape[0], gen.n
    if rho.shape[-2:] != (n, n):
        raise ValueError('rho0 shape %s does not match the generator dimension %d'
                         % (tuple(rho.shape), n))
    if not gen.shared and B != gen.P:
        if B == 1:
            rho = rho.expand(gen.P, n, n)
            B = gen.P
        else:
            raise ValueError('rho0 batch %d does not match %d generators' % (B, gen.P))
    if precision not in ('fp64', 'split'):
        raise ValueError("unknown precision %r (use 'fp64' or 'split')" % (precision,))
    if precision == 'split' and states_every:
        raise ValueError('precision="split" keeps the state on chip; states_every is not '
                         'supported (use precision="fp64" for rholist output)')
    batched_kernel = precision == 'split' and split_supported(gen) is None
    optimistic = herm is None and batched_kernel
    if herm is None and not batched_kernel:
        herm = bool(torch.equal(rho, rho.mH))
    out = None
    if optimistic or herm:
        if batched_kernel:
            work = rho.contiguous()
            out = torch.empty((B, n, n), dtype=CDT, device=device)
        else:
            work = rho.clone().contiguous()
    else:
        a, b = hermitian_parts(rho)
        work = torch.cat([a, b], 0).contiguous()
    redo = None
    if precision == 'fp64':
        obs = prepare_obs(e_ops, n, gen.P, device)
        tol = 1e-9 if trace_tol is None else trace_tol
        o, s, status = _run_f64(gen, work, dt, n_steps, obs, obs_every, states_every, tol,
                                param_batch=B, events=events, drive=drive)
    elif batched_kernel:
        tol = 1e-5 if trace_tol is None else trace_tol
        o, s, status = _run_split(gen, work, dt, n_steps, e_ops, obs_every, tol,
                                  param_batch=B, events=events, drive=drive, rho_out=out)
        if out is not None:
            work = out
    else:
        o, s, status, work, redo = _run_stream(gen, work, dt, n_steps, expand_e_ops(e_ops, n), obs_every,
                                               param_batch=B, events=events, drive=drive,
                                               defer=defer, sink=stream_sink)

    def finish(check: bool = True):
        nonlocal o, status, work
        if optimistic and int(status.item()) & nat.LIME_FLAG_NOT_HERMITIAN:
            return _launch(gen, rho, dt, n_steps, e_ops, states_every, precision, trace_tol,
                           obs_every, None, drive, defer, hermitian=False)(check)
        if redo is not None:
            for _ in range(3):
                if not int(status.item()) & nat.LIME_FLAG_RANGE:
                    break
                o, status, work = redo()
        if check:
            flags = int(status.item())
            if flags:
                raise nat.KernelFlagError(flags, 'lindblad RK4 (%s)' % precision)
        if not (optimistic or herm):
            return (o[:B] + 1j * o[B:], None if s is None else s[:B] + 1j * s[B:],
                    work[:B] + 1j * work[B:])
        return o, s, work

    return finish


def propagate(gen: LindbladGenerator, rho0, dt: float, n_steps: int, e_ops=None,
              states_every: int = 0, precision: str = 'fp64', trace_tol: float | None = None,
              check: bool = True, obs_every: int = 1, events=None, drive=None):
    """RK4-propagate density matrices under ``gen``.

    ``rho0``: (n, n) or (B, n, n); with a non-shared generator B must equal
    ``gen.P``.  Returns ``(obs, states, rho)`` device tensors:
    ``obs`` (B, n_steps // obs_every, n_obs) = Tr(E rho) after steps
    obs_every-1, 2 obs_every-1, ..., ``states`` (B, n_steps // states_every,
    n, n) or None, ``rho`` (B, n, n) final.  ``events``: optional pair of
    CUDA events recorded on the launching stream around the kernel call.
    ``drive``: optional (ops (q, n, n), coef (n_steps, q) float64) device
    tensors for H(t) = H0 - sum_q coef[k, q] ops[q] during step k (FP64 path,
    or the streaming tensor-core path with ``precision='split'``).
    """
    return _launch(gen, rho0, dt, n_steps, e_ops, states_every, precision, trace_tol,
                   obs_every, events, drive)(check)


# A host batch for the batched split kernel runs as a pipeline of launches
# over instance ranges: the generators of the ranges are prepared while the
# later ranges upload, and the copy back of range c overlaps the kernel on
# range c + 1.  The kernel keeps SPLIT_CTAS_PER_SM CTAs per SM resident (its
# launch default) and each CTA propagates one instance at a time, so a
# "round" is 2 x SMs instances; the ranges are whole rounds (the partial
# round last), which keeps the number of rounds, and so the kernel time,
# that of a single launch.
SPLIT_CTAS_PER_SM = 2
PIPELINE_MIN_ROUNDS = 3      # host batches of fewer rounds run as one launch
PIPELINE_ROUNDS = 4          # rounds per range


class SplitObs:
    """Observables already resolved for the batched split kernel (the
    ``(mode, n_obs, tensor, stride)`` of ``_split_obs``), shared by the
    launches of a pipeline so that none of them inspects the operators."""

    def __init__(self, spec):
        self.spec = spec


def pipeline_chunks(P: int, slots: int, rounds: int = PIPELINE_ROUNDS) -> list:
    """Instance ranges [(lo, hi), ...] of a pipelined batch of P instances:
    ``rounds`` whole rounds of ``slots`` instances per range, the last whole
    rounds, then the partial last round alone (its copy back is the
    pipeline's tail)."""
    if P < 0 or slots < 1 or rounds < 1:
        raise ValueError('pipeline_chunks needs P >= 0 and positive slots / rounds')
    full, rem = divmod(P, slots)
    out = [(lo, min(lo + rounds * slots, full * slots)) for lo in range(0, full * slots, rounds * slots)]
    if rem:
        out.append((full * slots, P))
    return out


def _ndim(a) -> int:
    if isinstance(a, torch.Tensor):
        return a.dim()
    if hasattr(a, 'toarray'):
        return 2
    return int(np.ndim(a))


def _per_instance(a, P: int):
    """True if operand ``a`` (an array, SiteDephasing or DiagonalOps) has a
    leading instance axis of length P, False if it is shared, None if it is
    neither (left to the one-launch path to report)."""
    if isinstance(a, SiteDephasing):
        x, nd = a.rates, 2
    elif isinstance(a, DiagonalOps):
        x, nd = a.l, 3
    else:
        x, nd = a, 3
    d = _ndim(x)
    if d == nd - 1:
        return False
    if d != nd:
        return None
    lead = int(x.shape[0]) if hasattr(x, 'shape') else len(x)
    return True if lead == P else (False if lead == 1 else None)


def _upload(a, device, lo=None, hi=None):
    """Device copy (asynchronous on the current stream for pinned memory) of
    a host operand, instances lo:hi of it when given."""
    def dev(x, dtype):
        if hasattr(x, 'toarray'):
            x = x.toarray()
        if lo is not None:
            x = x[lo:hi]
        t = x if isinstance(x, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(x))
        return t.to(device=device, dtype=dtype, non_blocking=True)
    if isinstance(a, SiteDephasing):
        return SiteDephasing(dev(a.rates, torch.float64))
    if isinstance(a, DiagonalOps):
        return DiagonalOps(dev(a.l, CDT))
    return dev(a, CDT)


_PIPE_STREAMS = {}


def _pipeline_streams(device):
    """The pipeline's upload, preparation and copy-back streams of a device,
    created once: the caching allocator keeps freed blocks per stream, so
    fresh streams on every call would allocate every buffer anew."""
    k = device.index if device.index is not None else torch.cuda.current_device()
    if k not in _PIPE_STREAMS:
        _PIPE_STREAMS[k] = tuple(torch.cuda.Stream(device) for _ in range(3))
    return _PIPE_STREAMS[k]


def propagate_host_pipelined(H, rho0, c_ops, e_ops, dt: float, n_steps: int, obs_every: int = 1,
                             trace_tol: float | None = None, device=None):
    """A batch given in host memory on the batched split kernel, as a
    pipeline of launches over instance ranges (``pipeline_chunks``).

    Four streams: uploads of each range's operands, generator preparation,
    the kernels (the caller's current stream, in range order) and the copies
    of each range's observables and final states into page-locked host
    tensors.  The ranges' generators are prepared while the uploads land;
    the copies back overlap the propagation of the later ranges.  Returns
    ``(obs, rho)``, host tensors (P, n_steps // obs_every, n_obs) and
    (P, n, n), or None when the batch does not qualify: the kernel does not
    handle the generator, rho0 is not Hermitian, an observable is per
    instance, or the batch is shorter than PIPELINE_MIN_ROUNDS rounds.  The
    caller then runs it as one launch.

    Every range's A operand takes the power-of-two scale of the whole
    batch's max |Heff| (one read back to the host), so the results are
    bitwise those of the single launch."""
    if not torch.cuda.is_available() or n_steps < 1 or obs_every < 1:
        return None
    if not hasattr(H, 'shape') or (isinstance(H, torch.Tensor) and H.device.type != 'cpu'):
        return None
    if _ndim(H) != 3:
        return None
    P, n = int(H.shape[0]), int(H.shape[-1])
    if n > SPLIT_MAX_N or tuple(H.shape[-2:]) != (n, n):
        return None
    device = _dev(device)
    slots = SPLIT_CTAS_PER_SM * torch.cuda.get_device_properties(device).multi_processor_count
    if -(-P // slots) < PIPELINE_MIN_ROUNDS:
        return None
    c_ops = list(c_ops or [])
    per = [_per_instance(a, P) for a in c_ops]
    rho_per = _per_instance(rho0, P)
    if any(p is None for p in per) or rho_per is None:
        return None
    if not isinstance(e_ops, Populations) and e_ops and any(_ndim(e) != 2 for e in e_ops):
        return None
    if not _host_hermitian(rho0):
        return None
    nat.require_device()
    comp = torch.cuda.current_stream(device)
    up, prep, down = _pipeline_streams(device)
    spec = _split_obs(e_ops if e_ops is not None else [], n, 1, device)
    T, n_obs = n_steps // obs_every, spec[1]
    obs_h = torch.empty((P, T, n_obs), dtype=CDT, pin_memory=True)
    rho_h = torch.empty((P, n, n), dtype=CDT, pin_memory=True)
    chunks = pipeline_chunks(P, slots)
    # every upload is enqueued first, in range order: range c lands while the
    # generators of the ranges before it are prepared
    inputs = []
    with torch.cuda.stream(up):
        shared = [None if p else _upload(a, device) for a, p in zip(c_ops, per)]
        rho_shared = None if rho_per else _upload(rho0, device)
        for lo, hi in chunks:
            ev = torch.cuda.Event()
            Hc = _upload(H, device, lo, hi)
            cc = [_upload(a, device, lo, hi) if p else s for a, p, s in zip(c_ops, per, shared)]
            rc = _upload(rho0, device, lo, hi) if rho_per else rho_shared
            ev.record(up)
            inputs.append((ev, Hc, cc, rc))
    # each range's generator as soon as its upload lands, and its max |Heff|
    gens, amax = [], []
    for i, (ev_in, Hc, cc, rc) in enumerate(inputs):
        with torch.cuda.stream(prep):
            prep.wait_event(ev_in)
            gen = LindbladGenerator.build(Hc, cc, device=device)
            if split_supported(gen) is not None:
                if i:
                    raise RuntimeError('pipelined batch: range %d needs another kernel' % i)
                torch.cuda.synchronize(device)
                return None
            amax.append(gen.heff.abs().amax())
        gens.append(gen)
    # one read back for the whole batch: every range's A operand takes the
    # scale of the batch's max |Heff|, the scale of a single launch.  The A
    # operands are prepared before the first propagation: the propagation
    # kernel keeps every SM busy, so kernels queued behind it would wait
    with torch.cuda.stream(prep):
        top = float(torch.stack(amax).max().item())
        for gen in gens:
            gen.split_cache['amax'] = top
            split_operands(gen)
    comp.wait_stream(prep)               # (prep waited for every upload)
    # the propagations back to back; each range's results are copied back
    # while the next range runs
    keep, finishers = [], []
    for (lo, hi), gen, (_, _, _, rc) in zip(chunks, gens, inputs):
        ev_done = torch.cuda.Event()
        with torch.cuda.stream(comp):
            fin = _launch(gen, rc, dt, n_steps, SplitObs(spec), 0, 'split', trace_tol, obs_every,
                          hermitian=True)
            o, _, r = fin(False)
            ev_done.record(comp)
        with torch.cuda.stream(down):
            down.wait_event(ev_done)
            obs_h[lo:hi].copy_(o, non_blocking=True)
            rho_h[lo:hi].copy_(r, non_blocking=True)
        # every range's buffers live until the last copy back has finished:
        # a buffer freed early could be handed to another stream mid-use
        keep.append((o, r))
        finishers.append(fin)
    down.synchronize()
    for fin in finishers:
        fin(True)                        # raises on a kernel status flag
    del keep, inputs, gens, amax
    return obs_h, rho_h


def _dims(a):
    if isinstance(a, torch.Tensor):
        return a.dim()
    return np.ndim(a.toarray() if hasattr(a, 'toarray') else a)


def is_ragged(H) -> bool:
    """True for an uneven batch: a list/tuple of two or more 2-D Hamiltonians
    (the reference's list form [H0, [H1, f1], ...] is the driven solver)."""
    return isinstance(H, (list, tuple)) and len(H) >= 2 and all(
        not isinstance(x, (list, tuple)) and _dims(x) == 2 for x in H)


# The tensor-core paths pad a chain to dimension 64 (the batched kernel's
# fixed size, the streaming GEMMs' 64-wide K chunks).  An uneven batch packs
# up to 64 // n chains of dimension n <= 32 block-diagonally into one
# instance: the generator of a block-diagonal system (Heff, the collapse
# operators, M) is block-diagonal, a block-diagonal state stays so, and the
# zero blocks contribute exact zeros, so every chain evolves as it would
# alone (up to the summation order inside the tensor-core accumulation).
PACK_DIM = 64


def pack_count(n: int, precision: str) -> int:
    """Chains of dimension n per packed instance (1: not packed)."""
    return PACK_DIM // n if precision == 'split' and 2 * n <= PACK_DIM else 1


def _embed(blocks: torch.Tensor) -> torch.Tensor:
    """(G, p, n, n) -> (G, p n, p n) block-diagonal."""
    G, p, n, _ = blocks.shape
    out = torch.zeros(G, p, n, p, n, dtype=blocks.dtype, device=blocks.device)
    for s in range(p):
        out[:, s, :, s, :] = blocks[:, s]
    return out.reshape(G, p * n, p * n)


class RaggedGroup:
    """One batched launch of an uneven batch: instances ``idx`` (input
    order) of dimension ``n``, ``pack`` of them block-diagonally to a
    launched instance; ``gen``, ``rho``, ``e_ops`` are the launch's inputs."""

    def __init__(self, idx, n, n_obs, pack, gen, rho, e_ops):
        self.idx, self.n, self.n_obs, self.pack = idx, n, n_obs, pack
        self.gen, self.rho, self.e_ops = gen, rho, e_ops

    def unpack(self, o, s, r):
        """Per-instance (obs, states, rho) from the launch's outputs."""
        n, p, m = self.n, self.pack, self.n_obs
        out = []
        for j in range(len(self.idx)):
            if p == 1:
                out.append((o[j], None if s is None else s[j], r[j]))
            else:
                g, q = divmod(j, p)
                out.append((o[g][..., q * m:(q + 1) * m], None,
                            r[g][q * n:(q + 1) * n, q * n:(q + 1) * n]))
        return out


def ragged_groups(H_list, rho0_list, c_ops_list, e_ops_list, precision: str, device,
                  pack: bool = True) -> list:
    """Group an uneven batch by (dimension, operator count) and build each
    group's generator, states and observables on ``device`` (packed
    block-diagonally for precision='split' and n <= 32 unless ``pack`` is
    False)."""
    groups = {}
    for i in range(len(H_list)):
        h = H_list[i]
        n = int(h.shape[-1]) if hasattr(h, 'shape') else int(np.shape(h)[-1])
        groups.setdefault((n, len(c_ops_list[i])), []).append(i)
    out = []
    for (n, K), idx in sorted(groups.items()):
        m = len(e_ops_list[idx[0]])
        p = pack_count(n, precision) if pack else 1

        def stacked(get):
            x = torch.stack([as_device(get(i), device) for i in idx])
            if p == 1:
                return x
            G = -(-len(idx) // p)
            pad = torch.zeros((G * p - len(idx), n, n), dtype=x.dtype, device=device)
            return _embed(torch.cat([x, pad]).reshape(G, p, n, n))

        H = stacked(lambda i: H_list[i])
        ops = [stacked(lambda i, k=k: c_ops_list[i][k]) for k in range(K)]
        rho = stacked(lambda i: rho0_list[i])
        if p == 1:
            E = [torch.stack([as_device(e_ops_list[i][o], device) for i in idx]) for o in range(m)]
        else:
            # observable o of slot q: chain (g, q)'s operator in block q only
            G = H.shape[0]
            E = []
            zero = torch.zeros((n, n), dtype=CDT, device=device)
            for q in range(p):
                for o in range(m):
                    blocks = torch.zeros((G, p, n, n), dtype=CDT, device=device)
                    for g in range(G):
                        j = g * p + q
                        blocks[g, q] = as_device(e_ops_list[idx[j]][o], device) if j < len(idx) else zero
                    E.append(_embed(blocks))
        gen = LindbladGenerator.build(H, ops, device=device)
        out.append(RaggedGroup(idx, n, m, p, gen, rho, E))
    return out


UNEVEN_DEFAULT = {'mode': 'groups', 'order': 1, 'n_ctas': 0, 'pack': True}
UNEVEN_CANDIDATES = (
    {'mode': 'groups', 'order': 1, 'n_ctas': 0, 'pack': True},
    {'mode': 'groups', 'order': 0, 'n_ctas': 0, 'pack': True},
    {'mode': 'groups', 'order': 1, 'n_ctas': 0, 'pack': False},
    {'mode': 'streams', 'order': 1, 'n_ctas': 0, 'pack': True},
    {'mode': 'streams', 'order': 1, 'n_ctas': 0, 'pack': False},
)


def _ragged_dims(H_list, c_ops_list):
    """(dimension, operator count) -> instance count of an uneven batch."""
    cnt = {}
    for i, h in enumerate(H_list):
        n = int(h.shape[-1]) if hasattr(h, 'shape') else int(np.shape(h)[-1])
        k = (n, len(c_ops_list[i]))
        cnt[k] = cnt.get(k, 0) + 1
    return cnt


def uneven_class(H_list, c_ops_list, precision: str, pack: bool = True) -> str:
    """The autotuner's N-class of an uneven batch (``tuning.uneven_class``
    over the groups the streaming path would launch)."""
    from . import tuning
    dims, counts, ks = [], [], set()
    for (n, K), c in sorted(_ragged_dims(H_list, c_ops_list).items()):
        p = pack_count(n, precision) if pack else 1
        dims.append((n * p + 63) // 64 * 64)
        counts.append(-(-c // p))
        ks.add(K)
    return tuning.uneven_class(dims, counts, max(ks) if ks else 0)


def ragged_enqueue(groups, dt: float, n_steps: int, precision: str, schedule=None, states_every: int = 0,
                   trace_tol: float | None = None, obs_every: int = 1, device=None):
    """Enqueue the propagation of prepared uneven-batch groups
    (``ragged_groups``) on the current stream and return one finishing
    closure per group (``closure(check) -> (obs, states, rho)``).

    ``schedule['mode']``: 'groups' runs every group on the streaming
    tensor-core path in one ``lime_lindblad_rk4_stream_groups`` call (per
    stage one persistent launch for the GEMM 1 tiles of all groups and one
    for the GEMM 2 tiles; ``order`` and ``n_ctas`` as there), the other
    groups (batched kernel, FP64) one after another; 'streams' runs each
    group's launch sequence on its own CUDA stream."""
    sched = dict(UNEVEN_DEFAULT if schedule is None else schedule)
    device = _dev(device)
    main = torch.cuda.current_stream(device)
    fins = []
    if sched.get('mode') == 'groups' and precision == 'split':
        sink = []
        for grp in groups:
            fins.append(_launch(grp.gen, grp.rho, dt, n_steps, grp.e_ops, states_every=states_every,
                                precision=precision, trace_tol=trace_tol, obs_every=obs_every, defer=True,
                                stream_sink=sink))
        if sink:
            lib = nat.require_device()
            cap = int(lib.lime_lindblad_stream_max_groups())
            for c0 in range(0, len(sink), cap):
                part = sink[c0:c0 + cap]
                arr = (nat.LindbladStreamDesc * len(part))(*[d for d, _ in part])
                nat.check(lib.lime_lindblad_rk4_stream_groups(arr, len(part), int(sched.get('n_ctas', 0)),
                                                              int(sched.get('order', 1)), _stream_ptr()),
                          'lime_lindblad_rk4_stream_groups')
        return fins
    streams = []
    for grp in groups:
        st = torch.cuda.Stream(device=device)
        st.wait_stream(main)
        with torch.cuda.stream(st):
            fins.append(_launch(grp.gen, grp.rho, dt, n_steps, grp.e_ops, states_every=states_every,
                                precision=precision, trace_tol=trace_tol, obs_every=obs_every, defer=True))
        streams.append(st)
    for st in streams:
        main.wait_stream(st)
    return fins


def propagate_ragged(H_list, rho0_list, dt: float, n_steps: int, c_ops_list=None,
                     e_ops_list=None, states_every: int = 0, precision: str = 'fp64',
                     trace_tol: float | None = None, obs_every: int = 1, device=None,
                     schedule=None):
    """Uneven batch: instance i has its own Hamiltonian H_list[i] (n_i x n_i),
    collapse operators c_ops_list[i] and observables e_ops_list[i] (lists of
    n_i x n_i operators; every instance has the same number of observables).

    Instances with equal dimension and operator counts are stacked into one
    batched propagation (with precision='split', chains of dimension <= 32
    are packed block-diagonally, 64 // n to an instance).  With
    precision='split' the groups on the streaming tensor-core path run in
    lockstep, per RK4 stage one persistent launch for all groups' GEMM 1
    tiles and one for their GEMM 2 tiles (``ragged_enqueue``); the
    schedule is the autotuner's cached choice for this batch's N-class
    (``tuning``, ``autotune_ragged``) or ``UNEVEN_DEFAULT``, unless given.
    Status words are checked once everything is enqueued.  ``precision``:
    'fp64' or 'split'.  Returns three lists in input order: observables
    (n_steps // obs_every, n_obs), states or None, final rho.
    """
    B = len(H_list)
    if len(rho0_list) != B:
        raise ValueError('%d Hamiltonians but %d initial states' % (B, len(rho0_list)))
    c_ops_list = [[] for _ in range(B)] if c_ops_list is None else list(c_ops_list)
    e_ops_list = [[] for _ in range(B)] if e_ops_list is None else list(e_ops_list)
    if len(c_ops_list) != B or len(e_ops_list) != B:
        raise ValueError('c_ops_list and e_ops_list need one entry per instance')
    n_obs = {len(e) for e in e_ops_list}
    if len(n_obs) > 1:
        raise ValueError('every instance needs the same number of observables')
    device = _dev(device)
    if schedule is None:
        from . import tuning
        schedule = UNEVEN_DEFAULT
        if precision == 'split':
            schedule = tuning.choose('lindblad_uneven', uneven_class(H_list, c_ops_list, precision),
                                     precision, UNEVEN_DEFAULT, arch=tuning.arch_tag(device))
    groups = ragged_groups(H_list, rho0_list, c_ops_list, e_ops_list, precision, device,
                           pack=bool(schedule.get('pack', True)))
    fins = ragged_enqueue(groups, dt, n_steps, precision, schedule, states_every=states_every,
                          trace_tol=trace_tol, obs_every=obs_every, device=device)
    obs, states, rhos = [None] * B, [None] * B, [None] * B
    for grp, fin in zip(groups, fins):
        res = grp.unpack(*fin(True))
        for i, (o, s, r) in zip(grp.idx, res):
            obs[i], states[i], rhos[i] = o, s, r
    return obs, states, rhos


def autotune_ragged(H_list, rho0_list, dt: float, c_ops_list=None, e_ops_list=None, precision: str = 'split',
                    steps: int = 8, candidates=UNEVEN_CANDIDATES, device=None, cache=None, force: bool = False):
    """Time every candidate schedule of ``propagate_ragged`` on this batch
    (GPU time of ``steps`` RK4 steps minus that of ``steps // 2``, so the
    per-call operand conversion cancels; CUDA events) and store the fastest
    in the tuning cache under the batch's N-class.  Returns
    ``(choice, times)`` (times None when the cache already held the key)."""
    from . import tuning
    B = len(H_list)
    c_ops_list = [[] for _ in range(B)] if c_ops_list is None else list(c_ops_list)
    e_ops_list = [[] for _ in range(B)] if e_ops_list is None else list(e_ops_list)
    device = _dev(device)
    prepared = {}

    def measure(cand):
        pack = bool(cand.get('pack', True))
        if pack not in prepared:
            prepared[pack] = ragged_groups(H_list, rho0_list, c_ops_list, e_ops_list, precision, device,
                                           pack=pack)
        groups = prepared[pack]

        def run(k):
            main = torch.cuda.current_stream(device)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(device)
            a.record(main)
            fins = ragged_enqueue(groups, dt, k, precision, cand, device=device)
            b.record(main)
            torch.cuda.synchronize(device)
            for f in fins:
                f(True)
            return a.elapsed_time(b) / 1e3

        run(1)
        return (run(steps) - run(max(1, steps // 2))) / (steps - max(1, steps // 2))

    return tuning.tune('lindblad_uneven', uneven_class(H_list, c_ops_list, precision), precision, candidates,
                       measure, arch=tuning.arch_tag(device), cache=cache, force=force)
