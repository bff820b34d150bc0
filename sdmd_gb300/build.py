"""Build the engine's native libraries in-tree.

  sdmd_gb300/libsdmd_gpu.so   CUDA kernels + C ABI (include/sdmd_gpu.h), sm_103a only
  sdmd_gb300/libsdmd_host.so  host-side C: system builder for the reference's inputs
  sdmd_gb300/sdmd-gb300       the sDMD executable on the engine (app/sdmd_run.c)
  sdmd_gb300/sremd-gb300      the REMD launcher, all replicas in one engine batch (app/sremd_run.c)

Translation units compile in parallel; nothing here uses cmake or torch.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(HERE, "_build")

GPU_LIB = os.path.join(HERE, "libsdmd_gpu.so")
HOST_LIB = os.path.join(HERE, "libsdmd_host.so")

CUDA_SOURCES = ["api.cu", "loop_fp64.cu", "samples.cu", "remd.cu"]
# -fmad=false: no multiply-add contraction, so FP64 results are bit-identical to
# the reference's (gcc -O2 on x86-64 contracts nothing either).  Kernels that want
# FMA use fma()/__fmaf_rn explicitly.
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-fmad=false", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC]


def nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _deps():
    out = [os.path.join(INCLUDE, "sdmd_gpu.h"), os.path.abspath(__file__)]
    for d in (CSRC,):
        out += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cu", ".cuh", ".h"))]
    return out


def build_gpu(force=False, verbose=False):
    deps = _deps()
    if not force and _newer(GPU_LIB, deps):
        return GPU_LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nv, "-c", *NVCC_FLAGS, "-o", obj, os.path.join(CSRC, src)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(CUDA_SOURCES)) as ex:
        objs = list(ex.map(compile_one, CUDA_SOURCES))
    tmp = GPU_LIB + ".tmp"
    r = subprocess.run([nv, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp, *objs, "-lcudart"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, GPU_LIB)
    return GPU_LIB


def build_host(force=False):
    srcs = [os.path.join(HOST, f) for f in sorted(os.listdir(HOST)) if f.endswith(".c")] if os.path.isdir(HOST) else []
    if not srcs:
        return None
    deps = srcs + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")] + [
        os.path.join(INCLUDE, "sdmd_gpu.h"), os.path.join(INCLUDE, "sdmd_host.h")]
    if not force and _newer(HOST_LIB, deps):
        return HOST_LIB
    tmp = HOST_LIB + ".tmp"
    subprocess.check_call(["gcc", "-O2", "-std=gnu99", "-ffp-contract=off", "-fPIC", "-shared", "-Wall", "-pthread",
                           "-I" + INCLUDE, "-I" + HOST, "-o", tmp, *srcs, "-lm"])
    os.replace(tmp, HOST_LIB)
    return HOST_LIB


APP = os.path.join(HERE, "sdmd-gb300")
REMD_APP = os.path.join(HERE, "sremd-gb300")
APP_DIR = os.path.join(HERE, "app")
APP_SRC = os.path.join(APP_DIR, "sdmd_run.c")
REMD_APP_SRC = os.path.join(APP_DIR, "sremd_run.c")
APP_COMMON = [os.path.join(APP_DIR, "app_common.c"), os.path.join(APP_DIR, "app_common.h")]


def build_app(force=False):
    """The sDMD executable and the REMD launcher, linked with the two libraries beside them."""
    common = [GPU_LIB, HOST_LIB, os.path.join(INCLUDE, "sdmd_gpu.h"), os.path.join(INCLUDE, "sdmd_host.h")] + APP_COMMON
    for out, src in ((APP, APP_SRC), (REMD_APP, REMD_APP_SRC)):
        if not force and _newer(out, [src] + common):
            continue
        tmp = out + ".tmp"
        subprocess.check_call(["gcc", "-O2", "-std=gnu99", "-Wall", "-I" + INCLUDE, "-I" + APP_DIR, "-o", tmp, src,
                               APP_COMMON[0], "-L" + HERE, "-lsdmd_gpu", "-lsdmd_host", "-Wl,-rpath,$ORIGIN", "-lm"])
        os.replace(tmp, out)
    return APP


def build_all(force=False):
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        fg = ex.submit(build_gpu, force)
        fh = ex.submit(build_host, force)
        out = fg.result(), fh.result()
    build_app(force)
    return out


if __name__ == "__main__":
    print(build_all(force=True))
