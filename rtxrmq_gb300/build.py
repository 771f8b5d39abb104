"""Build recipe for the native parts of rtxrmq_gb300.

Produces, in-tree under ``rtxrmq_gb300/_lib/``:
  librmq.so  -- the C ABI of include/rmq.h (CUDA kernels for sm_103a + host code)
  rtxrmq     -- the command-line front end (same arguments as the reference's
                ./rtxrmq, src/main.cu + src/tools.h)

Every translation unit compiles in parallel with one ``-gencode`` for sm_103a;
a unit is rebuilt only when a source or header is newer than its object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-fopenmp,-O3", *ARCH]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp"]

LIB_CU = ["api.cu", "build.cu", "query.cu", "batch.cu", "batch_light.cu", "noalloc.cu",
          "persist.cu"]
LIB_CPP = ["gen.cpp", "power.cpp"]
CLI_CPP = ["cli.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build rtxrmq_gb300")


def _cuda_home(nvcc: str) -> Path:
    return Path(nvcc).resolve().parent.parent


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n  " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, force: bool = False, checked: bool = False) -> Path:
    """Compile librmq.so and the rtxrmq CLI; return the library path.

    checked=True builds the range-checked variant (-DRMQ_CHECKED=1: every
    global index the kernels use is checked, violations are counted and
    skipped, read back with rmq_checked_violations) into _lib/checked/."""
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    out_dir = OUT / "checked" if checked else OUT
    flags = NVCC_FLAGS + (["-DRMQ_CHECKED=1"] if checked else [])
    out_dir.mkdir(parents=True, exist_ok=True)
    obj_dir = out_dir / "obj"
    obj_dir.mkdir(exist_ok=True)
    hdrs = _headers()
    inc = [f"-I{INCLUDE}", f"-I{CSRC}", f"-I{cuda / 'include'}"]

    jobs = []
    for src in LIB_CU:
        o = obj_dir / (src + ".o")
        if force or _stale(o, [CSRC / src, *hdrs]):
            jobs.append([nvcc, *flags, *inc, "-c", str(CSRC / src), "-o", str(o)])
    for src in LIB_CPP + CLI_CPP:
        o = obj_dir / (src + ".o")
        if force or _stale(o, [CSRC / src, *hdrs]):
            jobs.append(["g++", *CXX_FLAGS, *inc, "-c", str(CSRC / src), "-o", str(o)])
    if verbose:
        for j in jobs:
            print(" ".join(j), file=sys.stderr)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))

    lib = out_dir / "librmq.so"
    lib_objs = [obj_dir / (s + ".o") for s in LIB_CU + LIB_CPP]
    if force or _stale(lib, lib_objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, lib_objs),
              "-Xcompiler", "-fopenmp", "-lgomp", "-ldl", "-lpthread"])
    cli = out_dir / "rtxrmq"
    cli_objs = [obj_dir / (s + ".o") for s in CLI_CPP]
    if force or _stale(cli, cli_objs + [lib]):
        _run(["g++", "-o", str(cli), *map(str, cli_objs), f"-L{out_dir}", "-lrmq",
              "-Wl,-rpath,$ORIGIN", f"-L{cuda / 'lib64'}", "-lcudart", "-fopenmp"])
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
