"""Build libabcgpu.so for sm_103a with nvcc (no cmake, no torch extension).

Each translation unit is compiled in parallel; the FP64 units get -fmad=false
so that their results are bit-identical to the FP64 CPU oracle.  Host code is
compiled with -ffp-contract=off for the same reason.  Rebuilds are skipped
when sources and flags are unchanged.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libabcgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
          f"-I{INCLUDE}", "--expt-relaxed-constexpr"]
UNITS = {
    "abcgpu.cu": [],
    "kernels_fp64.cu": ["-fmad=false"],
    "kernels_fp32.cu": [],
    "distance_fp64.cu": ["-fmad=false"],
    "distance_fp32.cu": [],
    "distance_tc.cu": [],
    "posterior.cu": ["-fmad=false"],
    "moment.cu": ["-fmad=false"],
    "moment_fp32.cu": [],
    "datastats.cu": ["-fmad=false"],
    "noalloc.cu": [],
    "mlp.cu": [],
    "mlp_tc.cu": [],
    "surrogate.cu": [],
    "formats.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _digest(extra: list[str]) -> str:
    h = hashlib.sha256()
    for root in (CSRC, INCLUDE):
        for name in sorted(os.listdir(root)):
            if name.endswith((".cu", ".cuh", ".h")):
                with open(os.path.join(root, name), "rb") as f:
                    h.update(name.encode())
                    h.update(f.read())
    h.update(repr((ARCH, COMMON, UNITS, extra)).encode())
    return h.hexdigest()


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    stamp = os.path.join(OUT_DIR, "stamp.txt")
    dig = _digest(extra)
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == dig:
        return LIB
    cc = nvcc()
    procs = []
    objs = []
    for unit, flags in UNITS.items():
        obj = os.path.join(OUT_DIR, unit.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [cc, *ARCH, *COMMON, *flags, *extra, "-c", os.path.join(CSRC, unit), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for unit, p in procs:
        out, _ = p.communicate()
        if out and (verbose or ptxas_info or p.returncode):
            print(out, file=sys.stderr)
        if p.returncode:
            failed.append(unit)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    link = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    if verbose:
        print(" ".join(link), flush=True)
    subprocess.run(link, check=True)
    with open(stamp, "w") as f:
        f.write(dig)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv, force="-f" in sys.argv)
    print(LIB)
