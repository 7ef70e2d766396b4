"""The reference-compatible command line (blpg_cli) and the C++ mirror of
the reference's Simplex class (include/blpg_simplex.hpp)."""
import os
import subprocess

import pytest

from simplexprojects_gb300 import build as B
from conftest import NETLIB


def test_cli_usage(built):
    r = subprocess.run([str(B.CLI)], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stdout


def test_simplex_mirror_header_compiles(built, tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text('#include "blpg_simplex.hpp"\n'
                   "int main(){ blpg::Simplex s(3); blpg::matrix<double> A(2,2); "
                   "s.setConstratint(A, {1.0, 2.0}); return s.getNo_OF_Simplx() == 3 ? 0 : 1; }\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", str(B.ROOT / "include"),
                        "-I", "/usr/local/cuda/include", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_cli_random_mode(built):
    r = subprocess.run([str(B.CLI), "40", "1", "200", "1", "2"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert "VERIFICATION FOR CORRECTNESS" in r.stdout and "status 5" in r.stdout


@pytest.mark.gpu
def test_cli_netlib_mode(built):
    """The reference's benchmark mode on SC50B (committed copy of its files)."""
    env = dict(os.environ, BLPG_BENCH_DIR=str(NETLIB))
    r = subprocess.run([str(B.CLI), "8", "1", "100", "10", "1"], capture_output=True, text=True,
                       env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "70.0000000000" in r.stdout  # SC50B's optimum (parseBenchmark.cpp:25)
