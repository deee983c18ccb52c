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
    ('LimeAdjointDesc', 'AdjointDesc'),
    ('LimeRedfieldBuildDesc', 'RedfieldBuildDesc'),
    ('LimeRedfieldRK4Desc', 'RedfieldRK4Desc'),
    ('LimeRedfieldSplitDesc', 'RedfieldSplitDesc'),
    ('LimeLindbladStreamDesc', 'LindbladStreamDesc'),
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
