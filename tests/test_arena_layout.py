"""Host-only compile-and-run check of the device arena layouts (cf_device.cuh)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_arena_layouts(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "arena_layout_check")
    subprocess.check_call([nvcc, "-std=c++17", "-o", exe, os.path.join(HERE, "native", "arena_layout_check.cu")])
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "OK" in out.stdout
