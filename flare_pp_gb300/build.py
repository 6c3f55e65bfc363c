"""Build libflare_pp_gb300.so in-tree with nvcc for sm_103a.

Each CUDA translation unit is compiled in parallel, then linked with cuBLAS and cuSOLVER.  Usage:

    python -m flare_pp_gb300.build        # or flare_pp_gb300.build.build()
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libflare_pp_gb300.so")
SOURCES = ["neighbors.cu", "b2_kernels.cu", "gemm_tc.cu", "kernel_form.cu",
           "capi_core.cu", "capi_predict.cu", "capi_pair.cu", "capi_solve.cu",
           "capi_noalloc.cu", "capi_struc.cu", "capi_std.cu",
           "capi_likelihood.cu", "gemm_ozaki.cu", "capi_gemm.cu", "capi_batch.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _compile(nvcc, src, obj):
    cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler",
           "-fPIC,-ffp-contract=off", "-diag-suppress", "177", "-c",
           os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force=False, verbose=False):
    """Compile every translation unit (in parallel) and link the library."""
    nvcc = _nvcc()
    home = _cuda_home(nvcc)
    os.makedirs(OBJ, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
            if f.endswith((".h", ".cuh"))]
    hdrs.append(os.path.join(HERE, "..", "include", "flare_pp_gb300.h"))
    newest_src = max(os.path.getmtime(p) for p in srcs + hdrs)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= newest_src):
        return LIB
    objs = [os.path.join(OBJ, s + ".o") for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(SOURCES))) as ex:
        futs = [ex.submit(_compile, nvcc, s, o) for s, o in zip(SOURCES, objs)]
        for f in futs:
            f.result()
    libdirs = [os.path.join(home, "lib64"), os.path.join(home, "lib64", "stubs"),
               os.path.join(home, "targets", "sbsa-linux", "lib"),
               os.path.join(home, "targets", "sbsa-linux", "lib", "stubs"),
               os.path.join(home, "targets", "x86_64-linux", "lib"),
               os.path.join(home, "targets", "x86_64-linux", "lib", "stubs")]
    link = [nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs]
    for d in libdirs:
        if os.path.isdir(d):
            link += ["-L", d]
    link += ["-lcublas", "-lcusolver"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
