"""Build recipe for the oracle libraries -- TEST INFRASTRUCTURE ONLY.

``build_oracle()`` compiles ``sparse_oracle.c`` with gcc into ``oracle/_build/``.
``build_refemu()`` compiles the reference's own FC kernel headers for the host (see
``ref_harness.cpp``) into ``oracle/_ref/``; it needs the reference sources and is skipped
when they are absent.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# The reference checkout: $SPARQC_REFERENCE_ROOT, else a sibling directory named "reference" next
# to this repository. Without it the host build of the reference's kernels is skipped.
REFERENCE_ROOT = os.environ.get("SPARQC_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                           "reference")

ORACLE_SO = os.path.join(BUILD, "liboracle.so")
DENSE_SO = os.path.join(BUILD, "libdense.so")
REFEMU_SO = os.path.join(REF_OUT, "librefemu.so")


def _newer(out, srcs):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs)


def _build_c(src_name, out, force):
    src = os.path.join(HERE, src_name)
    if not force and _newer(out, [src, __file__]):
        return out
    os.makedirs(BUILD, exist_ok=True)
    base = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
            src, "-o", out + ".tmp", "-lm"]
    try:
        subprocess.run(base[:1] + ["-fopenmp"] + base[1:], check=True, capture_output=True, text=True)
    except subprocess.CalledProcessError:
        subprocess.run(base, check=True, capture_output=True, text=True)
    os.replace(out + ".tmp", out)
    return out


def build_oracle(force=False):
    """The sparse restatement of the reference's algorithm (also the CPU baseline)."""
    return _build_c("sparse_oracle.c", ORACLE_SO, force)


def build_dense(force=False):
    """The paged dense FP64 statevector (textbook matrices, no pruning)."""
    return _build_c("dense_oracle.c", DENSE_SO, force)


def reference_available():
    return os.path.exists(os.path.join(REFERENCE_ROOT, "emulator", "device", "device_table_FC.cuh"))


def build_refemu(force=False):
    """Compile the reference FC kernels for the host. Returns the .so path or None."""
    if not reference_available():
        return None
    src = os.path.join(HERE, "ref_harness.cpp")
    shim = os.path.join(HERE, "ref_shim")
    deps = [src, __file__] + [os.path.join(shim, f) for f in os.listdir(shim)]
    if not force and _newer(REFEMU_SO, deps):
        return REFEMU_SO
    os.makedirs(REF_OUT, exist_ok=True)
    cuda_inc = "/usr/local/cuda/include"
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-w", "-I", shim, "-I", os.path.join(REFERENCE_ROOT, "emulator", "device"),
           "-I", cuda_inc, src, "-o", REFEMU_SO + ".tmp"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    os.replace(REFEMU_SO + ".tmp", REFEMU_SO)
    return REFEMU_SO


def clean():
    for d in (BUILD, REF_OUT):
        if os.path.isdir(d):
            shutil.rmtree(d)
