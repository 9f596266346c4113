"""ctypes wrapper of the sparse CPU oracle -- TEST INFRASTRUCTURE ONLY.

``SparseOracle`` runs the C restatement in ``sparse_oracle.c`` (the reference's FC pair
rule, 2x2 formulas and branching-only pruning) over gate arrays laid out like the
engine's ``sqc_gate``: (kind u32, target u32, controls u64, theta, phi, lambda f64).
"""
import ctypes
import numpy as np

from . import build

GATE_DTYPE = np.dtype([("kind", "<u4"), ("target", "<u4"), ("controls", "<u8"),
                       ("theta", "<f8"), ("phi", "<f8"), ("lambda", "<f8")])
assert GATE_DTYPE.itemsize == 40

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build.build_oracle()
        L = ctypes.CDLL(path)
        P, U64, D, I = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, ctypes.c_int
        L.orc_create.restype = P
        L.orc_create.argtypes = [I, D]
        L.orc_destroy.argtypes = [P]
        L.orc_set_threads.argtypes = [P, I]
        L.orc_max_threads.restype = I
        L.orc_set_state.restype = I
        L.orc_set_state.argtypes = [P, P, P, P, U64]
        L.orc_apply.restype = I
        L.orc_apply.argtypes = [P, P, U64]
        L.orc_nnz.restype = U64
        L.orc_nnz.argtypes = [P]
        L.orc_amp_updates.restype = U64
        L.orc_amp_updates.argtypes = [P]
        L.orc_get_state.restype = ctypes.c_int64
        L.orc_get_state.argtypes = [P, P, P, P, U64, I]
        L.orc_norm2.restype = D
        L.orc_norm2.argtypes = [P]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class SparseOracle:
    """Sparse state on the CPU, starting from |0...0> (key 0, amplitude 1)."""

    def __init__(self, precision=64, prune_threshold=1e-14, threads=1):
        self._L = lib()
        self._h = self._L.orc_create(int(precision), float(prune_threshold))
        if not self._h:
            raise MemoryError("orc_create failed")
        self._L.orc_set_threads(self._h, int(threads))

    def close(self):
        if self._h:
            self._L.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @staticmethod
    def max_threads():
        return lib().orc_max_threads()

    def set_threads(self, n):
        self._L.orc_set_threads(self._h, int(n))

    def set_state(self, keys, re, im):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        re = np.ascontiguousarray(re, dtype=np.float64)
        im = np.ascontiguousarray(im, dtype=np.float64)
        rc = self._L.orc_set_state(self._h, _ptr(keys), _ptr(re), _ptr(im), keys.size)
        if rc:
            raise ValueError(f"orc_set_state failed ({rc})")

    def apply(self, gates):
        gates = np.ascontiguousarray(gates, dtype=GATE_DTYPE)
        rc = self._L.orc_apply(self._h, _ptr(gates), gates.size)
        if rc:
            raise ValueError(f"orc_apply failed ({rc})")

    @property
    def nnz(self):
        return int(self._L.orc_nnz(self._h))

    @property
    def amp_updates(self):
        return int(self._L.orc_amp_updates(self._h))

    def state(self, sorted=True):
        n = self.nnz
        keys = np.empty(n, np.uint64)
        re = np.empty(n, np.float64)
        im = np.empty(n, np.float64)
        got = self._L.orc_get_state(self._h, _ptr(keys), _ptr(re), _ptr(im), n, 1 if sorted else 0)
        assert got == n
        return keys, re, im

    def norm2(self):
        return float(self._L.orc_norm2(self._h))
