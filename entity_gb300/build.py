"""Builds libentity_pic.so in-tree for sm_103a (GB300).

Each CUDA translation unit is compiled to an object in parallel, then linked
with the host engine into entity_gb300/libentity_pic.so. Objects go to
entity_gb300/_build/ (git-ignored). Rebuilds only what changed.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libentity_pic.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: every multiply and add rounds separately, as the reference's
# source writes them; the few fused multiply-adds are explicit fma calls.
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--extended-lambda",
           "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]


def _sources():
    cu = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp"))
    return cu, cpp


def _headers():
    hs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    for d in (CSRC, HOST):
        hs += [os.path.join(d, f) for f in os.listdir(d)
               if f.endswith((".cuh", ".h", ".hpp", ".inc"))]
    return hs


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _compile(src, hdr_time, verbose):
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
        return obj
    cmd = ["nvcc", *ARCH, *NVFLAGS, "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = ["nvcc", "-x", "cu", *ARCH, *NVFLAGS, "-I", os.path.join(ROOT, "include"),
               "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose=False, jobs=None):
    os.makedirs(OUT_DIR, exist_ok=True)
    cu, cpp = _sources()
    hdr_time = _newest(_headers())
    jobs = jobs or min(len(cu) + len(cpp), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr_time, verbose), cu + cpp))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        cmd = ["nvcc", *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
