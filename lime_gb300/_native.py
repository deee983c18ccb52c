"""ctypes binding of the C ABI declared in include/lime_gb300.h.

The library is the in-tree ``lime_gb300/liblime_gb300.so`` produced by
``lime_gb300.build``.  There is no fallback: if the library is missing or no
compute-capability-10.3 GPU is current, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# LIME_GB300_LIBRARY selects another build of the same ABI, e.g. the
# bounds-checked liblime_gb300_check.so (lime_gb300.build.build(check=True))
LIB_PATH = os.environ.get('LIME_GB300_LIBRARY') or os.path.join(HERE, 'liblime_gb300.so')

c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
c_size_t = ctypes.c_size_t

LIME_FLAG_NONFINITE = 0x1
LIME_FLAG_TRACE_DRIFT = 0x2
LIME_FLAG_TIMEOUT = 0x4
LIME_FLAG_RANGE = 0x8
LIME_FLAG_NOT_HERMITIAN = 0x10
LIME_FLAG_BOUNDS = 0x20


class LimeError(RuntimeError):
    """A lime_gb300 entry point returned a negative status."""

    def __init__(self, status, where):
        self.status = status
        super().__init__('%s failed: %s (status %d)' % (where, status_string(status), status))


class KernelFlagError(RuntimeError):
    """A kernel raised a device status flag (non-finite values, trace drift, timeout)."""

    def __init__(self, flags, where):
        self.flags = flags
        names = []
        if flags & LIME_FLAG_NONFINITE:
            names.append('non-finite values in rho')
        if flags & LIME_FLAG_TRACE_DRIFT:
            names.append('trace drift above tolerance')
        if flags & LIME_FLAG_TIMEOUT:
            names.append('device-side wait timed out')
        if flags & LIME_FLAG_RANGE:
            names.append('split-precision operand outside its fixed-point range')
        if flags & LIME_FLAG_NOT_HERMITIAN:
            names.append('rho(0) is not Hermitian')
        if flags & LIME_FLAG_BOUNDS:
            names.append('an index left its buffer (bounds-checked build)')
        super().__init__('%s: %s (flags 0x%x)' % (where, ', '.join(names) or 'unknown', flags))


class PrepareDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('batch', c_int32), ('k_dense', c_int32), ('k_diag', c_int32),
                ('h', c_void_p), ('h_stride', c_int64),
                ('l_dense', c_void_p), ('l_dense_stride', c_int64),
                ('l_diag', c_void_p), ('l_diag_stride', c_int64),
                ('heff', c_void_p), ('m', c_void_p),
                ('dephasing', c_void_p), ('dephasing_stride', c_int64)]


class LindbladDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('batch', c_int32), ('param_batch', c_int32),
                ('n_steps', c_int32), ('k_dense', c_int32),
                ('n_obs', c_int32), ('obs_diag', c_int32), ('obs_every', c_int32),
                ('states_every', c_int32),
                ('dt', c_double), ('trace_tol', c_double),
                ('rho', c_void_p),
                ('heff', c_void_p), ('heff_stride', c_int64),
                ('m', c_void_p), ('m_stride', c_int64),
                ('l_dense', c_void_p), ('l_dense_stride', c_int64),
                ('obs_ops', c_void_p), ('obs_stride', c_int64),
                ('obs_out', c_void_p), ('states', c_void_p),
                ('workspace', c_void_p), ('workspace_bytes', c_size_t),
                ('status', c_void_p),
                ('n_drive', c_int32), ('drive_ops', c_void_p), ('drive_coef', c_void_p)]


class SplitDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('batch', c_int32), ('param_batch', c_int32), ('n_steps', c_int32),
                ('obs_mode', c_int32), ('n_obs', c_int32), ('obs_every', c_int32),
                ('scale_a_log2', c_int32), ('scale_b_log2', c_int32), ('ctas_per_sm', c_int32),
                ('dt', c_double), ('trace_tol', c_double),
                ('rho', c_void_p),
                ('heff', c_void_p), ('heff_stride', c_int64),
                ('m_diag', c_void_p), ('m_stride', c_int64),
                ('obs_ops', c_void_p), ('obs_stride', c_int64),
                ('obs_out', c_void_p),
                ('status', c_void_p),
                ('n_drive', c_int32),
                ('drive_ops', c_void_p),
                ('drive_coef', c_void_p),
                ('workspace', c_void_p), ('workspace_bytes', c_size_t),
                ('a_pieces', c_void_p), ('a_stride', c_int64),
                ('rho_out', c_void_p),
                ('auto_scale_b', c_int32), ('chunk_steps', c_int32)]


class SplitPrepareDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('count', c_int32), ('scale_a_log2', c_int32),
                ('heff', c_void_p), ('heff_stride', c_int64),
                ('out', c_void_p), ('out_bytes', c_size_t)]


class AdjointDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('batch', c_int32), ('param_batch', c_int32), ('seg_steps', c_int32),
                ('step0', c_int32), ('total_steps', c_int32),
                ('k_dense', c_int32), ('n_obs', c_int32), ('obs_diag', c_int32), ('obs_every', c_int32),
                ('dt', c_double),
                ('ckpt', c_void_p), ('lam', c_void_p),
                ('heff', c_void_p), ('heff_stride', c_int64),
                ('m', c_void_p), ('m_stride', c_int64),
                ('l_dense', c_void_p), ('l_dense_stride', c_int64),
                ('heff_adj', c_void_p), ('heff_adj_stride', c_int64),
                ('m_adj', c_void_p), ('m_adj_stride', c_int64),
                ('l_dense_adj', c_void_p), ('l_dense_adj_stride', c_int64),
                ('obs_ops', c_void_p), ('obs_stride', c_int64),
                ('obs_grad', c_void_p),
                ('grad_diag', c_void_p), ('grad_bond', c_void_p), ('grad_gamma', c_void_p),
                ('workspace', c_void_p), ('workspace_bytes', c_size_t)]


class RedfieldBuildDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('k', c_int32),
                ('evals', c_void_p), ('a_eig', c_void_p),
                ('spec', c_void_p), ('spec_stride', c_int64),
                ('R', c_void_p),
                ('workspace', c_void_p), ('workspace_bytes', c_size_t)]


class RedfieldAssembleDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('k', c_int32),
                ('evals', c_void_p), ('a_eig', c_void_p), ('lam', c_void_p),
                ('p', c_void_p), ('q', c_void_p), ('R', c_void_p)]


class RedfieldAssembleAdjointDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('k', c_int32),
                ('a_eig', c_void_p), ('lam', c_void_p), ('G', c_void_p),
                ('grad_evals', c_void_p), ('grad_a', c_void_p), ('grad_lam', c_void_p),
                ('grad_p', c_void_p), ('grad_q', c_void_p)]


class RedfieldAdjointDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('n_rhs', c_int32), ('seg_steps', c_int32), ('step0', c_int32),
                ('n_obs', c_int32), ('obs_every', c_int32), ('n_slots', c_int32),
                ('dt', c_double),
                ('R', c_void_p), ('ckpt', c_void_p), ('lam', c_void_p),
                ('obs_ops', c_void_p), ('obs_grad', c_void_p),
                ('grad_R', c_void_p), ('grad_obs', c_void_p),
                ('workspace', c_void_p), ('workspace_bytes', c_size_t)]


class RedfieldAdjointSplitDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('n_rhs', c_int32), ('seg_steps', c_int32), ('step0', c_int32),
                ('n_obs', c_int32), ('obs_every', c_int32), ('n_slots', c_int32),
                ('scale_b_log2', c_int32), ('margin_log2', c_int32),
                ('dt', c_double),
                ('R', c_void_p), ('ckpt', c_void_p), ('lam', c_void_p),
                ('obs_ops', c_void_p), ('obs_grad', c_void_p),
                ('grad_R', c_void_p), ('grad_obs', c_void_p),
                ('workspace', c_void_p), ('workspace_bytes', c_size_t),
                ('status', c_void_p), ('stage_in', c_void_p)]


class RedfieldRK4Desc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('n_rhs', c_int32), ('n_steps', c_int32), ('n_obs', c_int32),
                ('obs_every', c_int32), ('states_every', c_int32),
                ('dt', c_double),
                ('R', c_void_p), ('rho', c_void_p),
                ('obs_ops', c_void_p), ('obs_out', c_void_p), ('states', c_void_p),
                ('workspace', c_void_p), ('workspace_bytes', c_size_t)]


class RedfieldSplitDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('n_rhs', c_int32), ('n_steps', c_int32), ('n_obs', c_int32),
                ('obs_every', c_int32), ('scale_b_log2', c_int32),
                ('dt', c_double),
                ('R', c_void_p), ('rho', c_void_p),
                ('obs_ops', c_void_p), ('obs_out', c_void_p),
                ('workspace', c_void_p), ('workspace_bytes', c_size_t),
                ('status', c_void_p), ('stage_out', c_void_p)]


class ZgemmDesc(ctypes.Structure):
    _fields_ = [('M', c_int32), ('N', c_int32), ('K', c_int32), ('batch', c_int32),
                ('conj_a', c_int32), ('conj_b', c_int32),
                ('A', c_void_p), ('a_rs', c_int64), ('a_cs', c_int64), ('a_bs', c_int64),
                ('B', c_void_p), ('b_rs', c_int64), ('b_cs', c_int64), ('b_bs', c_int64),
                ('scale', c_void_p), ('s_ks', c_int64), ('s_bs', c_int64),
                ('C', c_void_p), ('c_rs', c_int64), ('c_cs', c_int64), ('c_bs', c_int64)]


class FftDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('batch', c_int32), ('inverse', c_int32), ('shift', c_int32),
                ('x', c_void_p), ('x_s', c_int64), ('x_bs', c_int64),
                ('y', c_void_p), ('y_s', c_int64), ('y_bs', c_int64),
                ('post', c_void_p),
                ('workspace', c_void_p), ('workspace_bytes', c_size_t)]


class LindbladStreamDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('batch', c_int32), ('param_batch', c_int32), ('n_ops', c_int32),
                ('n_steps', c_int32), ('n_obs', c_int32), ('obs_every', c_int32),
                ('scale_b_log2', c_int32), ('scale_y_log2', c_int32),
                ('dt', c_double),
                ('rho', c_void_p),
                ('heff', c_void_p), ('heff_stride', c_int64),
                ('m', c_void_p), ('m_stride', c_int64),
                ('l_ops', c_void_p), ('l_stride', c_int64),
                ('obs_ops', c_void_p), ('obs_stride', c_int64),
                ('obs_out', c_void_p),
                ('workspace', c_void_p), ('workspace_bytes', c_size_t),
                ('status', c_void_p),
                ('n_drive', c_int32), ('drive_ops', c_void_p), ('drive_coef', c_void_p),
                ('m_diag', c_void_p), ('m_diag_stride', c_int64), ('obs_diag', c_int32)]


class AdjointStreamDesc(ctypes.Structure):
    _fields_ = [('n', c_int32), ('batch', c_int32), ('param_batch', c_int32), ('n_steps', c_int32),
                ('seg_steps', c_int32), ('n_obs', c_int32), ('obs_every', c_int32),
                ('scale_b_log2', c_int32), ('scale_l_log2', c_int32),
                ('dt', c_double),
                ('ckpt', c_void_p), ('lam', c_void_p),
                ('heff', c_void_p), ('heff_stride', c_int64),
                ('heff_adj', c_void_p), ('heff_adj_stride', c_int64),
                ('m', c_void_p), ('m_adj', c_void_p), ('m_stride', c_int64),
                ('obs_ops', c_void_p), ('obs_stride', c_int64),
                ('obs_grad', c_void_p),
                ('grad_diag', c_void_p), ('grad_bond', c_void_p), ('grad_gamma', c_void_p),
                ('workspace', c_void_p), ('workspace_bytes', c_size_t),
                ('status', c_void_p),
                ('m_diag', c_void_p), ('m_diag_stride', c_int64),
                ('obs_coef', c_void_p)]


# (name, restype, argtypes) of every exported symbol; tests check the header
# declares exactly these.
SIGNATURES = [
    ('lime_lindblad_prepare_f64', c_int32, [ctypes.POINTER(PrepareDesc), c_void_p]),
    ('lime_lindblad_rk4_f64_workspace', c_size_t, [c_int32, c_int32, c_int32]),
    ('lime_lindblad_rk4_f64', c_int32, [ctypes.POINTER(LindbladDesc), c_void_p]),
    ('lime_lindblad_adjoint_f64_workspace', c_size_t, [c_int32, c_int32, c_int32, c_int32]),
    ('lime_lindblad_adjoint_f64', c_int32, [ctypes.POINTER(AdjointDesc), c_void_p]),
    ('lime_redfield_build_f64_workspace', c_size_t, [c_int32, c_int32]),
    ('lime_redfield_build_f64', c_int32, [ctypes.POINTER(RedfieldBuildDesc), c_void_p]),
    ('lime_redfield_assemble_f64', c_int32, [ctypes.POINTER(RedfieldAssembleDesc), c_void_p]),
    ('lime_redfield_assemble_adjoint_f64', c_int32, [ctypes.POINTER(RedfieldAssembleAdjointDesc), c_void_p]),
    ('lime_redfield_adjoint_f64_workspace', c_size_t, [c_int32, c_int32, c_int32]),
    ('lime_redfield_adjoint_f64', c_int32, [ctypes.POINTER(RedfieldAdjointDesc), c_void_p]),
    ('lime_redfield_adjoint_split_workspace', c_size_t, [c_int32, c_int32, c_int32, c_int32]),
    ('lime_redfield_adjoint_split', c_int32, [ctypes.POINTER(RedfieldAdjointSplitDesc), c_void_p]),
    ('lime_redfield_rk4_f64_workspace', c_size_t, [c_int32, c_int32]),
    ('lime_redfield_rk4_f64', c_int32, [ctypes.POINTER(RedfieldRK4Desc), c_void_p]),
    ('lime_redfield_split_workspace', c_size_t, [c_int32, c_int32, c_int32]),
    ('lime_redfield_rk4_split', c_int32, [ctypes.POINTER(RedfieldSplitDesc), c_void_p]),
    ('lime_redfield_split3_workspace', c_size_t, [c_int32, c_int32, c_int32]),
    ('lime_zgemm_strided_f64', c_int32, [ctypes.POINTER(ZgemmDesc), c_void_p]),
    ('lime_fft_f64_workspace', c_size_t, [c_int32, c_int32]),
    ('lime_fft_f64', c_int32, [ctypes.POINTER(FftDesc), c_void_p]),
    ('lime_redfield_rk4_split3', c_int32, [ctypes.POINTER(RedfieldSplitDesc), c_void_p]),
    ('lime_lindblad_stream_workspace', c_size_t, [c_int32, c_int32, c_int32, c_int32]),
    ('lime_lindblad_rk4_stream', c_int32, [ctypes.POINTER(LindbladStreamDesc), c_void_p]),
    ('lime_lindblad_stream_max_groups', c_int32, []),
    ('lime_lindblad_rk4_stream_groups', c_int32, [ctypes.POINTER(LindbladStreamDesc), c_int32, c_int32, c_int32,
                                                  c_void_p]),
    ('lime_lindblad_adjoint_stream_workspace', c_size_t, [c_int32, c_int32, c_int32, c_int32]),
    ('lime_lindblad_adjoint_stream', c_int32, [ctypes.POINTER(AdjointStreamDesc), c_void_p]),
    ('lime_noalloc_scratch_bytes', c_size_t, []),
    ('lime_lindblad_rk4_f64_noalloc', c_int32, [ctypes.POINTER(LindbladDesc), c_void_p]),
    ('lime_lindblad_split_workspace', c_size_t, [c_int32, c_int32, c_int32, c_int32]),
    ('lime_lindblad_rk4_split', c_int32, [ctypes.POINTER(SplitDesc), c_void_p]),
    ('lime_lindblad_split_prepared_bytes', c_size_t, [c_int32, c_int32]),
    ('lime_lindblad_split_prepare', c_int32, [ctypes.POINTER(SplitPrepareDesc), c_void_p]),
    ('lime_wait_selftest_workspace', c_size_t, []),
    ('lime_wait_selftest', c_int32, [c_int32, ctypes.c_uint32, c_void_p, c_void_p, c_void_p]),
    ('lime_device_check', c_int32, []),
    ('lime_launch_count', c_int64, []),
    ('lime_status_string', ctypes.c_char_p, [c_int32]),
    ('lime_version', c_int32, []),
]

_lib = None


def load(path: str = LIB_PATH):
    """Load the library (without touching the GPU)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError('lime_gb300 CUDA library not found at %s; build it with '
                           '`python -m lime_gb300.build`' % path)
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def launch_count() -> int:
    return int(load().lime_launch_count())


def status_string(status: int) -> str:
    try:
        return load().lime_status_string(status).decode()
    except Exception:  # pragma: no cover
        return 'status %d' % status


def check(status: int, where: str):
    if status != 0:
        raise LimeError(status, where)


_device_ok = False


def require_device():
    """Raise unless a compute-capability-10.3 (GB300) device is current."""
    global _device_ok
    if _device_ok:
        return load()
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError('lime_gb300 needs a CUDA GPU (sm_103a); none is available')
    torch.cuda.init()
    lib = load()
    check(lib.lime_device_check(), 'lime_device_check')
    _device_ok = True
    return lib
