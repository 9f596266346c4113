"""sparqc_gb300: a GB300-native sparse statevector gate engine.

The state is a GPU open-addressing hash table from 64-bit basis-state keys to complex
amplitudes; single-qubit and multi-controlled single-qubit gates pair each key with
k ^ (1 << q), apply the 2x2 update into a fresh table and prune negligible amplitudes.
The compute path is hand-written CUDA for sm_103a behind the C ABI in include/sparqc.h;
this package holds the kernels (csrc/), the build recipe, the ctypes binding and the
seeded workload generator.
"""
from .gates import GATE_DTYPE, gate, gate_array  # noqa: F401


def __getattr__(name):
    if name in ("State", "Circuit", "SparqcError", "load"):
        from . import engine
        return getattr(engine, name)
    raise AttributeError(name)
