"""ctypes binding of the engine's C ABI (include/sparqc.h).

``State`` wraps one ``sqc_state`` handle: a sparse statevector on one GPU. ``Circuit``
mirrors the reference's ``Circuit__`` names (emulator/include/circuit.h:34-105). There is no
CPU path: loading fails with an error when the CUDA library is missing or no GPU is present.
"""
import ctypes
import os

import numpy as np

from .gates import GATE_DTYPE, X, Y, Z, H, PHASE, RZ, RX, RY, S, SDG, T, TDG, U

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libsparqc.so")

OK, ERR_ARG, ERR_OOM, ERR_TABLE_FULL, ERR_CUDA, ERR_BUDGET, ERR_CAPACITY, ERR_NO_DEVICE, ERR_STATE = range(9)
READ_SORTED, READ_DROP_NEGLIGIBLE = 1, 2
FP64, FP32 = 64, 32

EXPORTS = ("sqc_default_options", "sqc_create", "sqc_destroy", "sqc_set_zero_state", "sqc_set_state",
           "sqc_apply_gates", "sqc_x", "sqc_y", "sqc_z", "sqc_h", "sqc_phase", "sqc_rz", "sqc_rx", "sqc_ry",
           "sqc_flush", "sqc_sync", "sqc_nnz", "sqc_get_state", "sqc_norm2", "sqc_compare", "sqc_get_stats",
           "sqc_status_string", "sqc_last_error", "sqc_stream", "sqc_apply_fixed")


class HashTableParameters(ctypes.Structure):
    _fields_ = [("N_devices", ctypes.c_uint32), ("coef_gpu_memory_reserve", ctypes.c_double),
                ("N_subtables", ctypes.c_uint32), ("log2_N_bucket_spots", ctypes.c_uint32)]


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_uint32), ("prune_threshold", ctypes.c_double),
                ("load_factor", ctypes.c_double), ("initial_buckets", ctypes.c_uint64),
                ("stream", ctypes.c_void_p), ("device", ctypes.c_uint32),
                ("max_fused_gates", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 4)]


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("gates_applied", "passes", "kernel_launches", "buckets",
                                                "table_bytes", "replays", "amp_updates", "alg_bytes")]


class SparqcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


_lib = None


def load(path=LIB_PATH):
    """Load the engine library (build it first with sparqc_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"engine library missing: {path} (run sparqc_gb300.build.build())")
    L = ctypes.CDLL(path)
    P, U32, U64, D, I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double, ctypes.c_int
    L.sqc_default_options.argtypes = [ctypes.POINTER(Options)]
    L.sqc_default_options.restype = None
    L.sqc_create.argtypes = [U32, ctypes.POINTER(HashTableParameters), ctypes.POINTER(Options), ctypes.POINTER(P)]
    L.sqc_destroy.argtypes = [P]
    L.sqc_set_zero_state.argtypes = [P]
    L.sqc_set_state.argtypes = [P, P, P, P, U64]
    L.sqc_apply_gates.argtypes = [P, P, U64]
    for n in ("sqc_x", "sqc_y", "sqc_z", "sqc_h"):
        getattr(L, n).argtypes = [P, U32]
    for n in ("sqc_phase", "sqc_rz", "sqc_rx", "sqc_ry"):
        getattr(L, n).argtypes = [P, U32, D]
    L.sqc_sync.argtypes = [P]
    L.sqc_flush.argtypes = [P]
    L.sqc_nnz.argtypes = [P, ctypes.POINTER(U64)]
    L.sqc_get_state.argtypes = [P, P, P, P, U64, ctypes.POINTER(U64), U32]
    L.sqc_norm2.argtypes = [P, ctypes.POINTER(D)]
    L.sqc_compare.argtypes = [P, P, ctypes.POINTER(D), ctypes.POINTER(D)]
    L.sqc_get_stats.argtypes = [P, ctypes.POINTER(Stats)]
    L.sqc_status_string.argtypes = [I]
    L.sqc_status_string.restype = ctypes.c_char_p
    L.sqc_last_error.argtypes = [P]
    L.sqc_last_error.restype = ctypes.c_char_p
    L.sqc_stream.argtypes = [P]
    L.sqc_stream.restype = P
    for n in EXPORTS:
        f = getattr(L, n)
        if f.restype is ctypes.c_int or n in ("sqc_create", "sqc_destroy", "sqc_set_zero_state", "sqc_set_state",
                                               "sqc_apply_gates", "sqc_flush", "sqc_sync", "sqc_nnz", "sqc_get_state",
                                               "sqc_norm2", "sqc_compare", "sqc_get_stats", "sqc_x", "sqc_y",
                                               "sqc_z", "sqc_h", "sqc_phase", "sqc_rz", "sqc_rx", "sqc_ry"):
            f.restype = I
    _lib = L
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class State:
    """A sparse statevector of ``nq`` qubits on one GPU, starting in |0...0>."""

    def __init__(self, nq, precision=FP64, prune_threshold=1e-14, load_factor=0.5, initial_buckets=0,
                 stream=None, device=0, max_fused_gates=0, params=None):
        self._L = load()
        o = Options()
        self._L.sqc_default_options(ctypes.byref(o))
        o.precision = precision
        o.prune_threshold = prune_threshold
        o.load_factor = load_factor
        o.initial_buckets = initial_buckets
        o.stream = stream
        o.device = device
        o.max_fused_gates = max_fused_gates
        h = ctypes.c_void_p()
        pp = ctypes.byref(params) if params is not None else None
        rc = self._L.sqc_create(nq, pp, ctypes.byref(o), ctypes.byref(h))
        if rc != OK:
            raise SparqcError(rc, f"sqc_create: {self._L.sqc_status_string(rc).decode()}")
        self._h = h
        self.nq = nq
        self.precision = precision

    def _check(self, rc, what):
        if rc != OK:
            msg = self._L.sqc_last_error(self._h).decode() if self._h else ""
            raise SparqcError(rc, f"{what}: {self._L.sqc_status_string(rc).decode()} ({msg})")

    def close(self):
        if getattr(self, "_h", None):
            self._L.sqc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    @property
    def stream(self):
        return self._L.sqc_stream(self._h)

    def set_zero(self):
        self._check(self._L.sqc_set_zero_state(self._h), "set_zero")

    def set_state(self, keys, re, im):
        keys = np.ascontiguousarray(keys, np.uint64)
        re = np.ascontiguousarray(re, np.float64)
        im = np.ascontiguousarray(im, np.float64)
        self._check(self._L.sqc_set_state(self._h, _p(keys), _p(re), _p(im), keys.size), "set_state")

    def apply(self, gates):
        gates = np.ascontiguousarray(gates, GATE_DTYPE)
        self._check(self._L.sqc_apply_gates(self._h, _p(gates), gates.size), "apply")

    def flush(self):
        """Launch everything queued without waiting."""
        self._check(self._L.sqc_flush(self._h), "flush")

    def sync(self):
        self._check(self._L.sqc_sync(self._h), "sync")

    @property
    def nnz(self):
        n = ctypes.c_uint64()
        self._check(self._L.sqc_nnz(self._h, ctypes.byref(n)), "nnz")
        return n.value

    def state(self, sorted=True, drop_negligible=False):
        n = self.nnz
        keys = np.empty(max(n, 1), np.uint64)
        re = np.empty(max(n, 1), np.float64)
        im = np.empty(max(n, 1), np.float64)
        got = ctypes.c_uint64()
        flags = (READ_SORTED if sorted else 0) | (READ_DROP_NEGLIGIBLE if drop_negligible else 0)
        self._check(self._L.sqc_get_state(self._h, _p(keys), _p(re), _p(im), n, ctypes.byref(got), flags),
                    "get_state")
        m = got.value
        return keys[:m].copy(), re[:m].copy(), im[:m].copy()

    def norm2(self):
        v = ctypes.c_double()
        self._check(self._L.sqc_norm2(self._h, ctypes.byref(v)), "norm2")
        return v.value

    def compare(self, other):
        f, e = ctypes.c_double(), ctypes.c_double()
        self._check(self._L.sqc_compare(self._h, other._h, ctypes.byref(f), ctypes.byref(e)), "compare")
        return f.value, e.value

    def stats(self):
        s = Stats()
        self._check(self._L.sqc_get_stats(self._h, ctypes.byref(s)), "stats")
        return {n: getattr(s, n) for n, _ in Stats._fields_}

    # one-gate helpers
    def _g(self, kind, t, controls=0, theta=0.0, phi=0.0, lam=0.0):
        g = np.zeros(1, GATE_DTYPE)
        g["kind"], g["target"], g["controls"] = kind, t, controls
        g["theta"], g["phi"], g["lambda"] = theta, phi, lam
        self.apply(g)


class Circuit(State):
    """The reference's Circuit__ gate names over one GPU state (emulator/include/circuit.h:45-83)."""

    def __init__(self, nq, hp=None, **kw):
        super().__init__(nq, params=hp, **kw)

    def x(self, t): self._check(self._L.sqc_x(self._h, t), "x")
    def y(self, t): self._check(self._L.sqc_y(self._h, t), "y")
    def z(self, t): self._check(self._L.sqc_z(self._h, t), "z")
    def h(self, t): self._check(self._L.sqc_h(self._h, t), "h")
    def phase(self, t, par): self._check(self._L.sqc_phase(self._h, t, par), "phase")
    def rz(self, t, par): self._check(self._L.sqc_rz(self._h, t, par), "rz")
    def rx(self, t, par): self._check(self._L.sqc_rx(self._h, t, par), "rx")
    def ry(self, t, par): self._check(self._L.sqc_ry(self._h, t, par), "ry")
    def s(self, t, controls=0): self._g(S, t, controls)
    def sdg(self, t, controls=0): self._g(SDG, t, controls)
    def t(self, q, controls=0): self._g(T, q, controls)
    def tdg(self, q, controls=0): self._g(TDG, q, controls)
    def u(self, t, theta, phi, lam, controls=0): self._g(U, t, controls, theta, phi, lam)

    def controlled(self, kind, t, controls, theta=0.0, phi=0.0, lam=0.0):
        m = 0
        for c in controls:
            m |= 1 << int(c)
        self._g(kind, t, m, theta, phi, lam)

    def print_raw_data(self):
        k, r, i = self.state(sorted=True, drop_negligible=True)
        for kk, rr, ii in zip(k, r, i):
            print(f"{int(kk)}: \t{rr: .3e} + {ii: .3e}j")
