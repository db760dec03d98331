"""Builds libctdm_gb300.so in-tree with nvcc for sm_103a.

Each translation unit compiles in its own nvcc process (in parallel), then the
objects are linked into ctdm_gb300/_build/libctdm_gb300.so.  Host code is built
without floating-point contraction so the host-side FP64 geometry matches the
oracle bit for bit on both x86 and aarch64.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libctdm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["ctdm_api.cu", "k_recon.cu", "k_qpi.cu", "k_dct.cu", "k_stack.cu", "k_compat.cu", "k_fastuw.cu",
           "k_gold.cu", "k_noalloc.cu", "k_grad.cu", "batch.cu", "tune.cu", "k_loop_small.cu", "k_loop_256.cu",
           "k_loop_384.cu", "k_loop_512.cu", "k_loop_768.cu", "driver.cu", "k_pocs.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler",
                   "-fPIC,-ffp-contract=off,-fvisibility=hidden", "-I", os.path.join(ROOT, "include"),
                   "-I", CSRC, "-DCTDM_BUILD"]


def _compile(src, extra):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "ctdm.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [nvcc(), "-c", srcp, "-o", obj] + flags() + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, extra=None, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    extra = list(extra or [])
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for o, log in results:
            if log:
                print(log)
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    extra = sys.argv[1:]
    print(build(verbose=True, extra=extra))
