"""Build libchollagb.so (the CUDA kernels + C ABI) in-tree for sm_103a.

One nvcc process per translation unit, run in parallel, then one link.  Output:
cholla_gb300/_build/libchollagb.so (git-ignored).  Run as ``python -m cholla_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "libchollagb.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", str(HERE.parent / "include")]
# Per-file flags.  The exact FP64 kernels keep every multiply and add separately rounded so
# that they reproduce the reference's -fmad=false build bit for bit (mhd_fast.cu compiles the
# same MHD source with contraction: the fast FP64 form).
PER_FILE = {
    "hydro_exact.cu": ["-fmad=false"],
    "hydro_exact_hllc.cu": ["-fmad=false"],
    "hydro_exact_roe.cu": ["-fmad=false"],
    "hydro_exact_hll.cu": ["-fmad=false"],
    "hydro_exact_exact.cu": ["-fmad=false"],
    "hydro_2d.cu": ["-fmad=false"],
    "mhd_exact.cu": ["-fmad=false"],
}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libchollagb")
    return cand


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _compile(src: Path, verbose_ptxas: bool) -> Path:
    obj = OUT / (src.name + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *PER_FILE.get(src.name, []), "-c", str(src), "-o", str(obj)]
    if verbose_ptxas and src.suffix == ".cu":
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    deps = list(CSRC.iterdir()) + [HERE.parent / "include" / "cholla_gb300.h", Path(__file__)]
    return all(p.stat().st_mtime <= t for p in deps if p.is_file())


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
