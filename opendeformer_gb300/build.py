"""Build the GB300 library ``opendeformer_gb300/_lib/libodgpu.so`` (sm_103a).

Every CUDA translation unit is compiled for ``sm_103a`` only, in parallel,
then linked into one shared object exporting the C ABI of
``include/od_gb300.h``.  The host-only setup code is compiled by nvcc's host
compiler as plain C++17.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libodgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]
SOURCES = ["od_host.cpp", "od_rif.cpp", "od_ric.cpp", "od_relabel.cpp", "od_server.cpp", "od_elements.cu", "od_sparse.cu", "od_api.cu",
           "od_batch.cu", "od_noalloc.cu", "od_sweep.cu", "od_collision.cu", "od_peaks.cu", "od_mixed_ic0.cu",
           "od_modal.cu"]
# per-file flags: the collision geometry rounds every operation separately,
# as the reference's compiled code does
FILE_FLAGS = {"od_collision.cu": ["-fmad=false"]}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "od_gb300.h"))
    procs, objs = [], []
    for src in SOURCES:
        path = os.path.join(SRC, src)
        obj = os.path.join(OUT_DIR, src + ".o")
        objs.append(obj)
        if not _stale(obj, [path, *headers, __file__]):
            continue
        if src.endswith(".cpp"):
            # no contraction into FMA: the host factorisations give the same
            # bits on x86-64 and aarch64
            cmd = [cc, "-x", "c++", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                   "-c", path, "-o", obj]
        else:
            cmd = [cc, *ARCH, *NVCC_FLAGS, *FILE_FLAGS.get(src, []), *(extra or []), "-c", path, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed.append(src)
            sys.stderr.write(text)
        elif verbose and text.strip():
            print(text)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    if _stale(LIB, objs):
        subprocess.check_call([cc, *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
