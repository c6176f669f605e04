"""Build libftcrypto_gb300/libftcrypto.so: the CUDA kernels (sm_103a only) and
the C ABI of include/ftcrypto.h + include/ftcrypto_gb300.h.

The translation units compile in parallel with nvcc into _build/, then link
into one shared library with the CUDA runtime linked statically, so the .so
is a self-contained drop-in for the reference's library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libftcrypto.so")
BENCH_LIB = os.path.join(HERE, "libftbench.so")  # bench.py's integer-pipe peak probe
# (source, object, extra defines): k_ladder.cu is compiled once per block size
LADDER_BLOCKS = (128, 192, 224, 384, 448)  # > 256: tables half in TMEM
SOURCES = [(s, s.replace(".cu", ".o"), []) for s in ("ft_api.cu", "k_elem.cu", "k_smul.cu", "k_reduce.cu",
                                                     "k_noalloc.cu", "k_batch.cu", "k_elgamal.cu", "k_encrypt.cu", "serve.cu")]
SOURCES += [("k_ladder.cu", f"k_ladder_{nt}.o", [f"-DFT_LADDER_NT={nt}"]) for nt in LADDER_BLOCKS]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--extended-lambda"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libftcrypto_gb300")


def _inputs():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h", ".inc"))]
    inc = os.path.join(HERE, os.pardir, "include")
    deps += [os.path.join(inc, f) for f in os.listdir(inc)]
    return deps


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(BENCH_LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _inputs())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    procs = []
    for src, objname, defs in SOURCES:
        obj = os.path.join(BUILD, objname)
        cmd = [cc] + FLAGS + defs + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((objname, obj, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    objs = []
    failed = []
    for src, obj, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        objs.append(obj)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(f"--- {s}\n{o}" for s, o in failed))
    tmp = LIB + ".tmp"
    subprocess.check_call([cc] + ARCH + ["-shared", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    bench_src = os.path.join(CSRC, "bench_peak.cu")
    bench_deps = [bench_src] + [os.path.join(CSRC, f) for f in ("fe.cuh", "ptx.cuh")]
    if force or not os.path.exists(BENCH_LIB) or os.path.getmtime(BENCH_LIB) < max(map(os.path.getmtime, bench_deps)):
        subprocess.check_call([cc] + FLAGS + ["-shared", "-o", BENCH_LIB, bench_src])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
