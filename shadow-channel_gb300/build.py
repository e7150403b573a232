"""Build the product library libc_channel.so in place (sm_103a only).

    python shadow-channel_gb300/build.py [--jobs N]

Compiles each CUDA / C++ translation unit in parallel with nvcc for
compute_103a/sm_103a and links one shared library next to this file.  No
PyTorch and no CMake are involved; the result exports the plain C ABI
declared in include/c_channel.h.
"""
import argparse
import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "_build"
LIB = HERE / "libc_channel.so"
SOURCES = ["engine.cu", "phys.cu", "phys_tc.cu", "phys_tc5.cu", "recon_solve.cu", "recon_tc.cu", "adjoint_exact.cu", "misc.cu", "noalloc.cu", "lss.cu", "stats.cu", "split_variants_a.cu", "split_variants_b.cu", "setup.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def compile_one(src: str) -> Path:
    obj = OUT_DIR / (src + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
           "-I", str(ROOT / "include"), "-c", str(CSRC / src), "-o", str(obj)]
    if src.endswith(".cpp"):
        # host table construction: no FMA contraction, so the tables match the
        # reference's on every host architecture
        cmd[1:1] = ["-x", "c++"]
        cmd += ["-Xcompiler", "-ffp-contract=off"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(jobs: int = 0) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    srcs = [CSRC / s for s in SOURCES]
    deps = srcs + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "c_channel.h"]
    if LIB.exists() and LIB.stat().st_mtime > max(p.stat().st_mtime for p in deps):
        return LIB
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=0)
    args = ap.parse_args()
    print(build(args.jobs))
