"""Build recipe for the native parts of kernels_gb300.

Outputs (all under kernels_gb300/_build/, git-ignored):
  libprk_gb300.so   the CUDA kernels and the C ABI (include/prk_gb300.h), sm_103a only
  stencil-gb300     the C++ host driver with PRK's stencil CLI, linked against the library

Every translation unit is compiled in parallel with one -gencode, so a build takes well under a
minute. `python -m kernels_gb300.build` runs it from the repository root.
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
HOST = PKG / "host"
BUILD = Path(os.environ.get("PRK_BUILD_DIR", PKG / "_build"))
LIB = BUILD / "libprk_gb300.so"
CLI = BUILD / "stencil-gb300"
# extra nvcc options (e.g. -DPRK_TILE_STAGES=2) for a variant build in PRK_BUILD_DIR
EXTRA = os.environ.get("PRK_NVCC_EXTRA", "").split()

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills",
              "--expt-relaxed-constexpr", *ARCH]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build kernels_gb300")


def _cuda_home(nvcc: str) -> Path:
    return Path(nvcc).resolve().parent.parent


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile libprk_gb300.so and the stencil-gb300 driver; return the library path."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h*"))
    objs = [BUILD / (s.stem + ".o") for s in sources]
    jobs = []
    for src, obj in zip(sources, objs):
        if force or _stale(obj, [src, *headers]):
            jobs.append([nvcc, *NVCC_FLAGS, *EXTRA, "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_run, j) for j in jobs]:
                f.result()
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    cli_src = HOST / "stencil_gb300.cc"
    if cli_src.exists() and (force or _stale(CLI, [cli_src, LIB, *headers])):
        cuda = _cuda_home(nvcc)
        _run(["g++", "-std=c++17", "-O2", "-Wall", f"-I{ROOT / 'include'}", f"-I{cuda / 'include'}", str(cli_src),
              "-o", str(CLI), f"-L{BUILD}", "-lprk_gb300", "-Wl,-rpath,$ORIGIN", f"-L{cuda / 'lib64'}", "-lcudart_static", "-ldl", "-lrt", "-lpthread"])
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(reference: str | None = None) -> None:
    """Compile the CPU oracle (oracle/Makefile). With a ParRes/Kernels checkout (`reference`, else
    $PRK_REFERENCE) also compile oracle/_ref, the reference's own drivers, dump harness and CUDA
    stencil, from the sources where they lie. Without one, say that those are skipped."""
    _run(["make", "-s", "-C", str(ROOT / "oracle"), "all"])
    ref_dir = reference or os.environ.get("PRK_REFERENCE")
    if not ref_dir:
        print("no reference checkout given (PRK_REFERENCE unset): oracle/_ref, the reference's own builds, skipped")
        return
    ref = Path(ref_dir)
    if (ref / "Cxx11" / "stencil_seq.hpp").exists():
        _run(["make", "-s", "-C", str(ROOT / "oracle"), "ref", f"REF={ref}"])
    else:
        print(f"{ref}/Cxx11/stencil_seq.hpp not found: the reference drivers and dump harness skipped")
    if (ref / "Cxx11" / "stencil-cuda.cu").exists():
        _run(["make", "-s", "-C", str(ROOT / "oracle"), "ref-cuda", f"REF={ref}"])
    else:
        print(f"{ref}/Cxx11/stencil-cuda.cu not found: the reference CUDA stencil skipped")


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    build_oracle()
