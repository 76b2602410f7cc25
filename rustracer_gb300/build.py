"""Builds libgbrt.so (the CUDA library behind include/gbrt.h) in-tree.

Each .cu file under csrc/ is compiled by nvcc for sm_103a only, in parallel,
into rustracer_gb300/_build/, and linked into rustracer_gb300/libgbrt.so with
the CUDA runtime linked statically.  Host code is compiled with
-ffp-contract=off so that host-side float arithmetic (instance inverses) is
rounded like the CPU oracle's on x86_64 and aarch64 alike.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbrt.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler",
                     "-fPIC,-ffp-contract=off,-fno-fast-math", "-Xptxas", "-warn-spills"]
# Path-tracing translation units: their plain `/` and sqrtf feed shading only
# (BRDF terms, pdfs, normalisations), so they compile to the approximate
# forms.  Every result that must match the CPU bit for bit -- camera rays, ray
# setup, the triangle test, texture filtering on the any-hit path -- is written
# with the explicit IEEE intrinsics (__fdiv_rn, __fsqrt_rn), which these flags
# do not touch.
SHADING_FLAGS = ["-prec-div=false", "-prec-sqrt=false"]
SHADING_UNITS = {"wavefront.cu", "wave_multi.cu", "render.cu"}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "gbrt.h"))
    return deps


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False, ptxas_info=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    extra += os.environ.get("GBRT_NVCC_FLAGS", "").split()  # e.g. -DGBRT_TRACE_MINB=4 for tuning sweeps

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        unit = SHADING_FLAGS if os.path.basename(src) in SHADING_UNITS else []
        cmd = [nv] + NVCC_FLAGS + unit + extra + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stdout + r.stderr

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, srcs))
    if verbose or ptxas_info:
        for obj, log in results:
            if log.strip():
                print(f"--- {os.path.basename(obj)}\n{log}", file=sys.stderr)
    tmp = LIB + ".tmp"
    cmd = [nv] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
