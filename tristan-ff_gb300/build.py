"""Build libffe_gb300.so in-tree with nvcc for sm_103a (GB300).

    python tristan-ff_gb300/build.py [--force] [--ptxas-verbose]

Translation units (compiled in parallel, then linked):
  csrc/ffe_api.cu      C ABI, handle and step drivers
  csrc/ffe_staged.cu   one kernel per reference procedure, -fmad=false
  csrc/ffe_fused.cu    fused stage kernels (fast: contraction on)
  csrc/ffe_fused.cu    again with -DFFE_FUSED_EXACT -fmad=false (verification path)
  csrc/ffe_fused.cu    with -DFFE_BATCH_TY=8 and =16: batched (many-grid) launches
  csrc/ffe_fused.cu    with -DFFE_BATCH_TY=8 -DFFE_BATCH_SPEC: batched launches of one variant
  csrc/ffe_noalloc.cu  cleanEpar on caller-owned arrays, fixed device scratch
  csrc/ffe_output.cu   writeOutput's node datasets (interpolation + downsampling)
Output: tristan-ff_gb300/lib/libffe_gb300.so (git-ignored; rebuilt on each box).
"""
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
LIB = os.path.join(OUT, "libffe_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
BASE = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
        "-I", CSRC, "-I", INCLUDE]

UNITS = [
    ("ffe_api.cu", "ffe_api.o", []),
    ("ffe_staged.cu", "ffe_staged.o", ["-fmad=false"]),
    ("ffe_fused.cu", "ffe_fused_fast.o", []),
    ("ffe_fused.cu", "ffe_fused_exact.o", ["-fmad=false", "-DFFE_FUSED_EXACT"]),
    ("ffe_fused.cu", "ffe_batch_t8.o", ["-DFFE_BATCH_TY=8"]),
    ("ffe_fused.cu", "ffe_batch_t16.o", ["-DFFE_BATCH_TY=16"]),
    ("ffe_fused.cu", "ffe_batch_t8s.o", ["-DFFE_BATCH_TY=8", "-DFFE_BATCH_SPEC"]),
    ("ffe_noalloc.cu", "ffe_noalloc.o", ["-fmad=false"]),
    ("ffe_output.cu", "ffe_output.o", ["-fmad=false"]),
]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "ffe.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, ptxas_verbose=False, quiet=True):
    """Compile every unit for sm_103a and link the shared library; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    t0 = time.time()
    procs = []
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    for src, obj, flags in UNITS:
        cmd = [nvcc()] + ARCH + BASE + flags + extra + ["-c", os.path.join(CSRC, src),
                                                        "-o", os.path.join(OUT, obj)]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    logs = []
    for cmd, p in procs:
        out, _ = p.communicate()
        logs.append(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append((cmd, out.decode(errors="replace")))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    link = [nvcc()] + ARCH + ["-shared", "-o", LIB] + [os.path.join(OUT, o) for _, o, _ in UNITS] + ["-lcudart"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + " ".join(link) + "\n" + r.stdout.decode(errors="replace"))
    if ptxas_verbose or not quiet:
        sys.stdout.write("".join(logs))
        sys.stdout.write("built %s in %.1fs\n" % (LIB, time.time() - t0))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, ptxas_verbose="--ptxas-verbose" in sys.argv, quiet=False)
