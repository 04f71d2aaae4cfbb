"""Builds libigsolve.so in-tree for sm_103a with nvcc (no cmake, no torch
extension machinery): each .cu translation unit compiles in parallel, then one
shared link with the static CUDA runtime.

    python -m ion_gym_gb300.build          # or __graft_entry__.build()
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libigsolve.so")
ROOT = os.path.dirname(PKG)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-fno-strict-aliasing", "--expt-relaxed-constexpr"]
# per-file extra flags: the exact FP64 kernels forbid FMA contraction on top
# of their explicit round-to-nearest intrinsics
EXTRA = {"ig_f64.cu": ["--fmad=false"]}
SOURCES = ["ig_f64.cu", "ig_solvers.cu", "ig_mixed.cu",
           "ig_noalloc.cu", "ig_geometry.cu", "ig_field.cu"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"),
              "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to "
                       "build libigsolve.so")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
          if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "igsolve.h"))
    return hs


def build(force=False, verbose=False, ptxas_verbose=False):
    """Compile every translation unit present in SOURCES and link
    libigsolve.so.  Returns the library path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    hdrs = _headers()
    objs = []
    jobs = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT_DIR, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            cmd = [cc, *ARCH, *COMMON, *EXTRA.get(s, []),
                   "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
            if ptxas_verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for cmd, r in zip(jobs, ex.map(
                lambda c: subprocess.run(c, capture_output=True, text=True),
                jobs)):
            if verbose or ptxas_verbose or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-cudart", "static",
               "-Xcompiler", "-fPIC"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libigsolve.so failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                ptxas_verbose="--ptxas" in sys.argv))
