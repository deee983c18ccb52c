"""The FP64-free conversions of the split-precision kernels (load of FP64
states into fp32 pairs, exact widening and power-of-two scaling of the
outputs) give bit-identical results to the conversion instructions: a host
build of lime_gb300/csrc/fpconv.cuh is checked against the host's own
round-to-nearest-even conversions over 2 million random and edge values."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_fpconv_bit_identical(tmp_path):
    nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(nvcc):
        pytest.skip('nvcc not available')
    exe = tmp_path / 'fpconv_check'
    subprocess.run([nvcc, '-O2', '-std=c++17', '-I', os.path.join(ROOT, 'lime_gb300', 'csrc'),
                    os.path.join(ROOT, 'tests', 'native', 'fpconv_check.cu'), '-o', str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.startswith('ok'), out.stdout[-2000:]
