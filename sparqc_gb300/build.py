"""Build the engine library ``sparqc_gb300/_lib/libsparqc.so`` with nvcc for sm_103a.

The translation units are compiled in parallel and linked with the static CUDA runtime. No
FMA contraction is allowed (``--fmad=false`` on the device, ``-ffp-contract=off`` on the
host): the gate arithmetic rounds every product and sum as written.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libsparqc.so")
SOURCES = ["sqc_pass.cu", "sqc_kernels.cu", "sqc_batch.cu", "sqc_measure.cu", "sqc_engine.cpp", "sqc_plan.cpp", "sqc_batch.cpp",
           "sqc_serve.cpp",
           "sqc_capi.cpp", "sqc_capi_batch.cpp", "sqc_fixed.cu", "sqc_part.cpp", "sqc_capi_part.cpp", "sqc_twoq.cpp"]
# per-file extra flags: the persistent batch kernel reads data other SMs wrote during the
# same launch, so its global loads default to L2 (L1 is not coherent across SMs)
EXTRA = {"sqc_batch.cu": ["-Xptxas", "-dlcm=cg"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-lineinfo", "-O3", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return files + [__file__]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src.replace(".", "_") + ".o")
        cmd = [cc] + _flags() + EXTRA.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc] + ARCH + ["-shared", "-o", tmp] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
