"""C-ABI checks that need no GPU: the library loads, exports every symbol the
header declares, and the ctypes descriptor layouts match the C compiler's."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, 'include', 'lime_gb300.h')


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(lime_\w+)\s*\(', src)))


@pytest.fixture(scope='module')
def lib():
    from lime_gb300 import build, _native
    build.build()
    return _native.load()


def test_exports_every_declared_symbol(lib):
    from lime_gb300 import _native
    declared = header_functions()
    assert declared, 'no declarations parsed'
    bound = sorted(name for name, _, _ in _native.SIGNATURES)
    assert declared == bound
    for name in declared:
        assert hasattr(lib, name), name


def test_status_strings(lib):
    assert lib.lime_status_string(0) == b'ok'
    assert b'argument' in lib.lime_status_string(-1)
    assert lib.lime_version() >= 100


def test_workspace_query(lib):
    # 4 matrices per instance (+ one trace double), 6 with dense collapse ops
    n, b = 16, 3
    assert lib.lime_lindblad_rk4_f64_workspace(n, b, 0) == b * (4 * n * n * 16 + 8)
    assert lib.lime_lindblad_rk4_f64_workspace(n, b, 2) == b * (6 * n * n * 16 + 8)
    assert lib.lime_lindblad_rk4_f64_workspace(0, b, 0) == 0


def test_null_descriptor_rejected(lib):
    # argument validation happens before any CUDA call
    assert lib.lime_lindblad_rk4_f64(None, None) == -1
    assert lib.lime_lindblad_prepare_f64(None, None) == -1
    assert lib.lime_lindblad_rk4_split(None, None) == -1
    assert lib.lime_lindblad_rk4_stream(None, None) == -1
    assert lib.lime_redfield_rk4_split(None, None) == -1
    assert lib.lime_redfield_rk4_f64(None, None) == -1
    assert lib.lime_lindblad_adjoint_f64(None, None) == -1
    assert lib.lime_redfield_assemble_f64(None, None) == -1
    assert lib.lime_redfield_assemble_adjoint_f64(None, None) == -1
    assert lib.lime_redfield_adjoint_f64(None, None) == -1
    assert lib.lime_redfield_adjoint_split(None, None) == -1


def test_stream_descriptor_validation(lib):
    """Host-side checks of the streaming entry point (no CUDA call is made
    before they pass): sizes, missing pointers, scales, workspace, alignment."""
    from lime_gb300 import _native
    d = _native.LindbladStreamDesc()
    d.n, d.batch, d.n_ops, d.n_steps, d.dt = 8, 2, 1, 3, 0.05
    assert lib.lime_lindblad_rk4_stream(ctypes.byref(d), None) == -1      # no pointers
    d.rho, d.heff, d.status, d.workspace = 0x1000, 0x2000, 0x3000, 0x410
    assert lib.lime_lindblad_rk4_stream(ctypes.byref(d), None) == -1      # l_ops missing
    d.l_ops = 0x5000
    d.scale_b_log2 = 99
    assert lib.lime_lindblad_rk4_stream(ctypes.byref(d), None) == -1      # scale out of range
    d.scale_b_log2 = 0
    d.workspace_bytes = 16
    assert lib.lime_lindblad_rk4_stream(ctypes.byref(d), None) == -5      # workspace too small
    d.workspace_bytes = lib.lime_lindblad_stream_workspace(8, 2, 2, 1)
    assert lib.lime_lindblad_rk4_stream(ctypes.byref(d), None) == -1      # workspace not 1024-aligned
    d.n = 5000
    assert lib.lime_lindblad_rk4_stream(ctypes.byref(d), None) == -2      # unsupported size


def test_stream_and_redfield_workspace_queries(lib):
    # n padded to 64: A1 pieces 3 x MT1 x KC1 x 16 KB etc.; monotone in every size
    w = lib.lime_lindblad_stream_workspace
    assert w(0, 1, 1, 0) == 0 and w(8, 0, 1, 0) == 0
    # same padded dimension: equal up to the FP64 Heff(t) buffer of driven generators
    assert w(64, 1, 1, 3) - w(8, 1, 1, 3) == (64 * 64 - 8 * 8) * 16
    assert w(65, 1, 1, 3) > w(64, 1, 1, 3)
    assert w(64, 4, 4, 3) > w(64, 4, 1, 3) > w(64, 2, 1, 3)
    r = lib.lime_redfield_split_workspace
    assert r(0, 4, 0) == 0
    assert r(8, 64, 0) == r(8, 1, 0)                # right-hand sides padded to 64
    assert r(8, 64, 200) > r(8, 64, 100) > r(8, 64, 0)


def test_split_drive_workspace_query(lib):
    # no drive: no workspace; otherwise fp32 pairs of Heff ([P][2][64][64]),
    # of the drive operators, the coefficients, their maxima and row ranges
    w = lib.lime_lindblad_split_workspace
    assert w(64, 16, 0, 100) == 0 and w(0, 1, 1, 1) == 0 and w(8, 0, 1, 1) == 0
    pair = 2 * 64 * 64 * 8
    assert w(8, 1, 1, 1) >= 2 * pair + 8 + 8 + 2 * 2 * 64 * 8
    assert w(64, 1, 1, 1) == w(8, 1, 1, 1)           # padded to 64 either way
    assert w(64, 3, 1, 10) - w(64, 2, 1, 10) >= pair
    assert w(64, 1, 2, 10) - w(64, 1, 1, 10) >= pair
    assert w(64, 1, 1, 4000) > w(64, 1, 1, 10)
    assert w(64, 1, 1, 10) % 256 == 0


def test_split_prepared_bytes(lib):
    b = lib.lime_lindblad_split_prepared_bytes
    # three fp16 pieces of the 128 x 128 real block form per generator
    assert b(64, 1) == 3 * 128 * 128 * 2 and b(8, 5) == 5 * b(8, 1)
    assert b(0, 1) == 0 and b(65, 1) == 0 and b(8, 0) == 0
    assert lib.lime_lindblad_split_prepare(None, None) == -1


def _c_layout(struct_name, fields):
    prog = ['#include <stdio.h>', '#include <stddef.h>', '#include "lime_gb300.h"', 'int main(void){',
            'printf("%zu\\n", sizeof({}));'.format(struct_name)]
    prog += ['printf("%zu\\n", offsetof({}, {}));'.format(struct_name, f) for f in fields]
    prog += ['return 0;}']
    return '\n'.join(prog)


@pytest.mark.parametrize('cname,pyname', [
    ('LimePrepareDesc', 'PrepareDesc'),
    ('LimeLindbladDesc', 'LindbladDesc'),
    ('LimeLindbladSplitDesc', 'SplitDesc'),
    ('LimeLindbladSplitPrepareDesc', 'SplitPrepareDesc'),
    ('LimeAdjointDesc', 'AdjointDesc'),
    ('LimeRedfieldBuildDesc', 'RedfieldBuildDesc'),
    ('LimeRedfieldRK4Desc', 'RedfieldRK4Desc'),
    ('LimeRedfieldAssembleDesc', 'RedfieldAssembleDesc'),
    ('LimeRedfieldAssembleAdjointDesc', 'RedfieldAssembleAdjointDesc'),
    ('LimeRedfieldAdjointDesc', 'RedfieldAdjointDesc'),
    ('LimeRedfieldAdjointSplitDesc', 'RedfieldAdjointSplitDesc'),
    ('LimeRedfieldSplitDesc', 'RedfieldSplitDesc'),
    ('LimeLindbladStreamDesc', 'LindbladStreamDesc'),
    ('LimeLindbladAdjointStreamDesc', 'AdjointStreamDesc'),
])
def test_descriptor_layout_matches_c(tmp_path, cname, pyname):
    from lime_gb300 import _native
    py = getattr(_native, pyname)
    fields = [f[0] for f in py._fields_]
    src = tmp_path / 'layout.c'
    src.write_text(_c_layout(cname, fields))
    exe = tmp_path / 'layout'
    subprocess.run(['gcc', '-I', os.path.join(ROOT, 'include'), str(src), '-o', str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(py)
    assert out[1:] == [getattr(py, f).offset for f in fields]
