"""The per-LP shared-memory layout, checked on the host: tests/layout_check.cu
is built with nvcc as a host program (no kernel launch, no GPU needed) from
the same header the plans and the kernel use."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


def test_norm_region_and_alignment(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not found")
    exe = tmp_path / "layout_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O1", "-o", str(exe), str(HERE / "layout_check.cu")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
