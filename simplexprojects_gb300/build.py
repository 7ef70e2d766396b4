"""Build recipe for libblpg.so (CUDA, sm_103a) and the CPU oracle.

Every translation unit is compiled in parallel with nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), then linked into
``simplexprojects_gb300/lib/libblpg.so`` with the CUDA runtime linked
statically.  The oracle (``oracle/cpu_ref.c``) is built with gcc into
``oracle/_build/libblpg_oracle.so``; it is test infrastructure, built here
only so that tests, ``smoke()`` and the bench's CPU-baseline leg can load it.

Host code is compiled with ``-ffp-contract=off`` (the workload generator must
give bit-identical data on x86 and Arm) and the solver's device code with
``--fmad=false`` (every fused multiply-add in it is an explicit ``fma``, as in
the oracle).

The size-class table tuned on GB300 (``tuning/gb300.json``, written by
``autotune.py``) is compiled into the library as its default table
(``_build/blpg_tuning_default.inc``).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libblpg.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_BUILD = ORACLE_DIR / "_build"
ORACLE_LIB = ORACLE_BUILD / "libblpg_oracle.so"
TUNING = PKG / "tuning" / "gb300.json"
TUNING_INC = BUILD / "blpg_tuning_default.inc"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: libblpg.so needs the CUDA 13 toolkit")


# (source, extra nvcc flags)
SOURCES = [
    ("blpg_api.cu", ["--fmad=false"]),
    ("blpg_part.cu", ["--fmad=false"]),
    ("blpg_peaks.cu", []),
    ("blpg_noalloc.cu", ["--fmad=false"]),
    ("blpg_mlp.cu", []),
    ("blpg_learned.cu", []),
    ("blpg_gen.cpp", []),
]


def _common(nvcc: str) -> list[str]:
    return [
        nvcc, "-std=c++17", "-O3", *ARCH, "-lineinfo",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
        "-I", str(ROOT / "include"), "-I", str(BUILD),
    ]


def _tuning_include() -> Path:
    """The compiled-in default tuning table: tuning/gb300.json as a C string
    (an empty table when the file is absent); rewritten only on change."""
    import json
    text = "{}"
    if TUNING.exists():
        table = json.loads(TUNING.read_text())
        text = json.dumps({k: v for k, v in table.items() if isinstance(v, int)})
    body = ("// generated by build.py from tuning/gb300.json\n"
            f'static const char kDefaultTuning[] = R"BLPGJSON({text})BLPGJSON";\n')
    if not TUNING_INC.exists() or TUNING_INC.read_text() != body:
        TUNING_INC.write_text(body)
    return TUNING_INC


def _compile(nvcc: str, src: str, extra: list[str]) -> Path:
    obj = BUILD / (Path(src).stem + ".o")
    srcp = CSRC / src
    deps = [srcp, *CSRC.glob("*.h"), *CSRC.glob("*.cuh"), ROOT / "include" / "blpg.h",
            TUNING_INC]
    if obj.exists() and obj.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return obj
    cmd = _common(nvcc) + extra + ["-c", str(srcp), "-o", str(obj)]
    if src.endswith(".cpp"):
        cmd[cmd.index(str(srcp))] = str(srcp)
        cmd.insert(1, "-x")
        cmd.insert(2, "c++")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build_library(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    _tuning_include()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(SOURCES), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s[0], s[1]), SOURCES))
    if LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs),
           "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


CLI = LIBDIR / "blpg_cli"


def build_cli(verbose: bool = False) -> Path:
    """The reference-compatible command line (csrc/blpg_cli.cpp), linked
    against libblpg.so with an $ORIGIN rpath."""
    nvcc = _nvcc()
    src = CSRC / "blpg_cli.cpp"
    deps = [src, ROOT / "include" / "blpg.h", ROOT / "include" / "blpg_simplex.hpp", LIB]
    if CLI.exists() and CLI.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return CLI
    tmp = CLI.with_name("blpg_cli.tmp")
    cmd = [nvcc, "-std=c++17", "-O2", "-x", "c++", str(src), "-I", str(ROOT / "include"),
           "-L", str(LIBDIR), "-lblpg", "-Xlinker", "-rpath,$ORIGIN", "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"cli build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CLI)
    if verbose:
        print(f"built {CLI}")
    return CLI


def build_oracle(verbose: bool = False) -> Path:
    ORACLE_BUILD.mkdir(exist_ok=True)
    srcs = [ORACLE_DIR / "cpu_ref.c"]
    deps = srcs + [ORACLE_DIR / "cpu_ref.h", ORACLE_DIR / "cpu_ref_impl.h"]
    if ORACLE_LIB.exists() and ORACLE_LIB.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return ORACLE_LIB
    cc = os.environ.get("CC", "gcc")
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
           "-o", str(tmp), *map(str, srcs), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, ORACLE_LIB)
    if verbose:
        print(f"built {ORACLE_LIB}")
    return ORACLE_LIB


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, verbose)
        f2 = ex.submit(build_oracle, verbose)
        f1.result()
        f2.result()
    build_cli(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
