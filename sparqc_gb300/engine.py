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
           "sqc_status_string", "sqc_last_error", "sqc_stream", "sqc_apply_fixed",
           "sqc_get_state_where", "sqc_probability", "sqc_measure", "sqc_sample", "sqc_swap", "sqc_save",
           "sqc_load", "sqc_fp64_rate", "sqc_twoq_gates", "sqc_apply_twoq", "sqc_schedule_gates",
           "sqc_get_state_async", "sqc_readout_wait",
           "sqc_batch_default_options", "sqc_batch_create", "sqc_batch_destroy", "sqc_batch_prepare",
           "sqc_batch_run", "sqc_batch_sync", "sqc_batch_circuit_status", "sqc_batch_nnz", "sqc_batch_get_state",
           "sqc_batch_get_states",
           "sqc_batch_autotune", "sqc_batch_get_stats", "sqc_batch_compare", "sqc_batch_last_error",
           "sqc_batch_stream",
           "sqc_server_default_options", "sqc_server_create", "sqc_server_destroy", "sqc_server_submit",
           "sqc_server_step", "sqc_server_completed", "sqc_server_request_status", "sqc_server_nnz",
           "sqc_server_get_state", "sqc_server_release", "sqc_server_get_stats", "sqc_server_compare",
           "sqc_server_last_error", "sqc_server_stream",
           "sqc_part_create", "sqc_part_destroy", "sqc_part_set_zero_state", "sqc_part_apply_gates",
           "sqc_part_sync", "sqc_part_nnz", "sqc_part_get_state", "sqc_part_get_stats", "sqc_part_last_error")


class HashTableParameters(ctypes.Structure):
    _fields_ = [("N_devices", ctypes.c_uint32), ("coef_gpu_memory_reserve", ctypes.c_double),
                ("N_subtables", ctypes.c_uint32), ("log2_N_bucket_spots", ctypes.c_uint32)]


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_uint32), ("prune_threshold", ctypes.c_double),
                ("load_factor", ctypes.c_double), ("initial_buckets", ctypes.c_uint64),
                ("stream", ctypes.c_void_p), ("device", ctypes.c_uint32),
                ("max_fused_gates", ctypes.c_uint32), ("time_passes", ctypes.c_uint32),
                ("max_cross_qubits", ctypes.c_uint32), ("device_updates_only", ctypes.c_uint32),
                ("schedule_gates", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("gates_applied", "passes", "kernel_launches", "buckets",
                                                "table_bytes", "replays", "amp_updates", "alg_bytes",
                                                "alg_bytes_pair", "passes_pair", "pass_ns_pair", "pass_ns_stream")]


class CircuitDesc(ctypes.Structure):
    _fields_ = [("nq", ctypes.c_uint32), ("reserved", ctypes.c_uint32), ("gates", ctypes.c_void_p),
                ("n_gates", ctypes.c_uint64)]


class BatchOptions(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_uint32), ("device", ctypes.c_uint32), ("stream", ctypes.c_void_p),
                ("prune_threshold", ctypes.c_double), ("load_factor", ctypes.c_double),
                ("min_chunk", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_uint32),
                ("memory_budget", ctypes.c_uint64), ("use_graph", ctypes.c_uint32),
                ("idle_limit_us", ctypes.c_uint32), ("threads_per_unit", ctypes.c_uint32),
                ("schedule_gates", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 2)]


class BatchTuning(ctypes.Structure):
    _fields_ = [("load_factor", ctypes.c_double), ("min_chunk", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_uint32),
                ("best_ms", ctypes.c_double), ("default_ms", ctypes.c_double), ("candidates", ctypes.c_uint32),
                ("threads_per_unit", ctypes.c_uint32)]


class BatchStats(ctypes.Structure):
    _fields_ = [("circuits", ctypes.c_uint64), ("passes", ctypes.c_uint64), ("amp_updates", ctypes.c_uint64),
                ("alg_bytes", ctypes.c_uint64), ("table_bytes", ctypes.c_uint64),
                ("kernel_launches", ctypes.c_uint64), ("last_run_ms", ctypes.c_double)]


class ServerOptions(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_uint32), ("device", ctypes.c_uint32), ("stream", ctypes.c_void_p),
                ("prune_threshold", ctypes.c_double), ("load_factor", ctypes.c_double),
                ("memory_budget", ctypes.c_uint64), ("max_slots", ctypes.c_uint32), ("min_chunk", ctypes.c_uint32),
                ("slice_ms", ctypes.c_double), ("solo_log2_groups", ctypes.c_uint32),
                ("solo_share_pct", ctypes.c_uint32), ("inject_alloc_failures", ctypes.c_uint32),
                ("schedule_gates", ctypes.c_uint32), ("overlap_steps", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("queued", ctypes.c_uint64), ("running", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("solo_running", ctypes.c_uint64),
                ("steps", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64), ("amp_updates", ctypes.c_uint64),
                ("pool_bytes", ctypes.c_uint64), ("pool_used", ctypes.c_uint64), ("busy_ms", ctypes.c_double)]


class PartStats(ctypes.Structure):
    _fields_ = [("spilled", ctypes.c_uint32), ("partition_bits", ctypes.c_uint32)] + [
        (n, ctypes.c_uint64) for n in ("spills", "returns", "windows", "bins", "splits", "bytes_h2d", "bytes_d2h",
                                       "amp_updates", "max_bin_keys", "table_budget")]


REQ_QUEUED, REQ_RUNNING, REQ_DONE = 0, 1, 2


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
    L.sqc_get_state_where.argtypes = [P, U64, U64, P, P, P, U64, ctypes.POINTER(U64), U32]
    L.sqc_probability.argtypes = [P, U64, U64, ctypes.POINTER(D)]
    L.sqc_measure.argtypes = [P, U32, D, ctypes.POINTER(I), ctypes.POINTER(D)]
    L.sqc_sample.argtypes = [P, U64, U64, P]
    L.sqc_swap.argtypes = [P, U32, U32]
    L.sqc_save.argtypes = [P, ctypes.c_char_p]
    L.sqc_load.argtypes = [P, ctypes.c_char_p]
    for n in ("sqc_get_state_where", "sqc_probability", "sqc_measure", "sqc_sample", "sqc_swap", "sqc_save",
              "sqc_load"):
        getattr(L, n).restype = I
    L.sqc_status_string.argtypes = [I]
    L.sqc_status_string.restype = ctypes.c_char_p
    L.sqc_last_error.argtypes = [P]
    L.sqc_last_error.restype = ctypes.c_char_p
    L.sqc_stream.argtypes = [P]
    L.sqc_stream.restype = P
    L.sqc_fp64_rate.argtypes = [U32, ctypes.POINTER(D)]
    L.sqc_fp64_rate.restype = I
    L.sqc_twoq_gates.argtypes = [U32, U32, U32, U32, U64, D, D, P, P, U64, ctypes.POINTER(U64)]
    L.sqc_twoq_gates.restype = I
    L.sqc_apply_twoq.argtypes = [P, U32, U32, U32, U32, U64, D, D, P]
    L.sqc_apply_twoq.restype = I
    L.sqc_batch_default_options.argtypes = [ctypes.POINTER(BatchOptions)]
    L.sqc_batch_default_options.restype = None
    L.sqc_batch_create.argtypes = [ctypes.POINTER(BatchOptions), ctypes.POINTER(P)]
    L.sqc_batch_destroy.argtypes = [P]
    L.sqc_batch_prepare.argtypes = [P, P, U32]
    L.sqc_batch_run.argtypes = [P]
    L.sqc_batch_sync.argtypes = [P]
    L.sqc_batch_circuit_status.argtypes = [P, U32, ctypes.POINTER(I)]
    L.sqc_batch_nnz.argtypes = [P, U32, ctypes.POINTER(U64)]
    L.sqc_batch_get_state.argtypes = [P, U32, P, P, P, U64, ctypes.POINTER(U64), U32]
    L.sqc_batch_get_states.argtypes = [P, P, P, P, U64, P, ctypes.POINTER(U64), U32]
    L.sqc_batch_autotune.argtypes = [P, ctypes.POINTER(BatchTuning)]
    L.sqc_batch_get_stats.argtypes = [P, ctypes.POINTER(BatchStats)]
    L.sqc_batch_last_error.argtypes = [P]
    L.sqc_batch_last_error.restype = ctypes.c_char_p
    L.sqc_batch_stream.argtypes = [P]
    L.sqc_batch_stream.restype = P
    L.sqc_server_default_options.argtypes = [ctypes.POINTER(ServerOptions)]
    L.sqc_server_default_options.restype = None
    L.sqc_server_create.argtypes = [ctypes.POINTER(ServerOptions), ctypes.POINTER(P)]
    L.sqc_server_destroy.argtypes = [P]
    L.sqc_server_submit.argtypes = [P, ctypes.POINTER(CircuitDesc), ctypes.POINTER(U64)]
    L.sqc_server_step.argtypes = [P, ctypes.POINTER(U32)]
    L.sqc_server_completed.argtypes = [P, P, U32, ctypes.POINTER(U32)]
    L.sqc_server_request_status.argtypes = [P, U64, ctypes.POINTER(I), ctypes.POINTER(I)]
    L.sqc_server_nnz.argtypes = [P, U64, ctypes.POINTER(U64)]
    L.sqc_server_get_state.argtypes = [P, U64, P, P, P, U64, ctypes.POINTER(U64), U32]
    L.sqc_server_release.argtypes = [P, U64]
    L.sqc_server_get_stats.argtypes = [P, ctypes.POINTER(ServerStats)]
    L.sqc_batch_compare.argtypes = [P, U32, P, ctypes.POINTER(D), ctypes.POINTER(D)]
    L.sqc_server_compare.argtypes = [P, U64, P, ctypes.POINTER(D), ctypes.POINTER(D)]
    L.sqc_server_last_error.argtypes = [P]
    L.sqc_server_last_error.restype = ctypes.c_char_p
    L.sqc_server_stream.argtypes = [P]
    L.sqc_server_stream.restype = P
    L.sqc_part_create.argtypes = [U32, ctypes.POINTER(HashTableParameters), ctypes.POINTER(Options), U64,
                                  ctypes.POINTER(P)]
    L.sqc_part_destroy.argtypes = [P]
    L.sqc_part_set_zero_state.argtypes = [P]
    L.sqc_part_apply_gates.argtypes = [P, P, U64]
    L.sqc_part_sync.argtypes = [P]
    L.sqc_part_nnz.argtypes = [P, ctypes.POINTER(U64)]
    L.sqc_part_get_state.argtypes = [P, P, P, P, U64, ctypes.POINTER(U64), U32]
    L.sqc_part_get_stats.argtypes = [P, ctypes.POINTER(PartStats)]
    L.sqc_part_last_error.argtypes = [P]
    L.sqc_part_last_error.restype = ctypes.c_char_p
    for n in ("sqc_part_create", "sqc_part_destroy", "sqc_part_set_zero_state", "sqc_part_apply_gates",
              "sqc_part_sync", "sqc_part_nnz", "sqc_part_get_state", "sqc_part_get_stats"):
        getattr(L, n).restype = I
    for n in ("sqc_batch_create", "sqc_batch_destroy", "sqc_batch_prepare", "sqc_batch_run", "sqc_batch_sync",
              "sqc_batch_circuit_status", "sqc_batch_nnz", "sqc_batch_get_state", "sqc_batch_get_states",
              "sqc_batch_autotune",
              "sqc_batch_get_stats", "sqc_server_create", "sqc_server_destroy", "sqc_server_submit",
              "sqc_server_step", "sqc_server_completed", "sqc_server_request_status", "sqc_server_nnz",
              "sqc_server_get_state", "sqc_server_release", "sqc_server_get_stats", "sqc_batch_compare",
              "sqc_server_compare"):
        getattr(L, n).restype = I
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


TWOQ_UNITARY, TWOQ_RZZ, TWOQ_ISWAP, TWOQ_FSIM, TWOQ_CSWAP, TWOQ_SWAP = range(6)


def _twoq_matrix(u):
    if u is None:
        return None
    m = np.ascontiguousarray(np.asarray(u, dtype=np.complex128).reshape(4, 4)).view(np.float64)
    return m


def twoq_gates(form, a, b, c=0, controls=0, theta=0.0, phi=0.0, u=None):
    """The engine's gate sequence of one two-qubit gate (a GATE_DTYPE array), for gate arrays
    given to batches, servers or the oracle. u: the 4x4 unitary of TWOQ_UNITARY (index i_a + 2 i_b)."""
    L = load()
    m = _twoq_matrix(u)
    out = np.zeros(32, GATE_DTYPE)
    n = ctypes.c_uint64()
    rc = L.sqc_twoq_gates(form, a, b, c, controls, theta, phi, _p(m) if m is not None else None, _p(out), out.size,
                          ctypes.byref(n))
    if rc != OK:
        raise SparqcError(rc, f"sqc_twoq_gates: {L.sqc_status_string(rc).decode()}")
    return out[:n.value].copy()


def schedule_gates(nq, gates, max_cross_qubits=3):
    """The order sqc_schedule_gates gives a gate array: a permutation (uint32 indices) that moves
    gates ahead of gates they commute with, so that passes fuse more gates."""
    L = load()
    g = np.ascontiguousarray(gates, GATE_DTYPE)
    perm = np.zeros(g.size, np.uint32)
    rc = L.sqc_schedule_gates(nq, _p(g), g.size, max_cross_qubits, _p(perm))
    if rc != OK:
        raise SparqcError(rc, f"sqc_schedule_gates: {L.sqc_status_string(rc).decode()}")
    return perm


def fp64_rate(device=0):
    """Measured FP64 fused multiply-add rate of a device (lane operations per second)."""
    L = load()
    r = ctypes.c_double()
    rc = L.sqc_fp64_rate(device, ctypes.byref(r))
    if rc != OK:
        raise SparqcError(rc, f"sqc_fp64_rate: {L.sqc_status_string(rc).decode()}")
    return r.value


class State:
    """A sparse statevector of ``nq`` qubits on one GPU, starting in |0...0>."""

    def __init__(self, nq, precision=FP64, prune_threshold=1e-14, load_factor=0.5, initial_buckets=0,
                 stream=None, device=0, max_fused_gates=0, params=None, time_passes=False, max_cross_qubits=0,
                 device_updates_only=False, schedule_gates=False):
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
        o.time_passes = 1 if time_passes else 0
        o.max_cross_qubits = max_cross_qubits
        o.device_updates_only = 1 if device_updates_only else 0
        o.schedule_gates = 1 if schedule_gates else 0
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

    def state_async(self, keys, re, im, count):
        """Start an asynchronous readout into page-locked arrays (keys uint64, re/im float64 of
        equal size, count a one-element uint64 array, all page-locked); readout_wait() completes it
        and the entry count is then count[0]."""
        self._check(self._L.sqc_get_state_async(self._h, _p(keys), _p(re), _p(im), keys.size, _p(count)),
                    "get_state_async")

    def readout_wait(self):
        self._check(self._L.sqc_readout_wait(self._h), "readout_wait")

    def state_where(self, mask, value, sorted=True, drop_negligible=False):
        """Entries whose keys have (key & mask) == value."""
        n = self.nnz
        keys = np.empty(max(n, 1), np.uint64)
        re = np.empty(max(n, 1), np.float64)
        im = np.empty(max(n, 1), np.float64)
        got = ctypes.c_uint64()
        flags = (READ_SORTED if sorted else 0) | (READ_DROP_NEGLIGIBLE if drop_negligible else 0)
        self._check(self._L.sqc_get_state_where(self._h, mask, value, _p(keys), _p(re), _p(im), n,
                                                ctypes.byref(got), flags), "get_state_where")
        m = got.value
        return keys[:m].copy(), re[:m].copy(), im[:m].copy()

    def probability(self, mask, value):
        p = ctypes.c_double()
        self._check(self._L.sqc_probability(self._h, mask, value, ctypes.byref(p)), "probability")
        return p.value

    def measure(self, qubit, u):
        """Measure one qubit with the uniform number u in [0, 1): (outcome, probability of 1)."""
        o, p1 = ctypes.c_int(), ctypes.c_double()
        self._check(self._L.sqc_measure(self._h, qubit, u, ctypes.byref(o), ctypes.byref(p1)), "measure")
        return o.value, p1.value

    def sample(self, shots, seed=0):
        out = np.empty(max(shots, 1), np.uint64)
        self._check(self._L.sqc_sample(self._h, shots, seed, _p(out)), "sample")
        return out[:shots]

    def swap(self, a, b):
        self._check(self._L.sqc_swap(self._h, a, b), "swap")

    def save(self, path):
        self._check(self._L.sqc_save(self._h, os.fsencode(path)), "save")

    def load(self, path):
        self._check(self._L.sqc_load(self._h, os.fsencode(path)), "load")

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
    def apply_twoq(self, form, a, b, c=0, controls=0, theta=0.0, phi=0.0, u=None):
        """One two-qubit gate (TWOQ_* form; u: the 4x4 unitary of TWOQ_UNITARY, index i_a + 2 i_b)."""
        m = _twoq_matrix(u)
        self._check(self._L.sqc_apply_twoq(self._h, form, a, b, c, controls, theta, phi,
                                           _p(m) if m is not None else None), "apply_twoq")

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


class Batch:
    """Many independent circuits, each from |0...0>, run by one persistent kernel launch.

    ``circuits`` is a list of ``(nq, gates)`` with ``gates`` a GATE_DTYPE array. Each
    circuit's result is bit-identical to running it alone on a ``State`` (with schedule_gates,
    to running ``gates[schedule_gates(nq, gates, 2)]`` alone).
    """

    def __init__(self, precision=FP64, prune_threshold=1e-14, load_factor=0.45, min_chunk=8, blocks_per_sm=0,
                 memory_budget=0, use_graph=False, stream=None, device=0, idle_limit_us=0, threads_per_unit=0,
                 schedule_gates=False):
        self._L = load()
        o = BatchOptions()
        self._L.sqc_batch_default_options(ctypes.byref(o))
        o.precision = precision
        o.prune_threshold = prune_threshold
        o.load_factor = load_factor
        o.min_chunk = min_chunk
        o.blocks_per_sm = blocks_per_sm
        o.memory_budget = memory_budget
        o.use_graph = 1 if use_graph else 0
        o.stream = stream
        o.device = device
        o.idle_limit_us = idle_limit_us
        o.threads_per_unit = threads_per_unit
        o.schedule_gates = 1 if schedule_gates else 0
        h = ctypes.c_void_p()
        rc = self._L.sqc_batch_create(ctypes.byref(o), ctypes.byref(h))
        if rc != OK:
            raise SparqcError(rc, f"sqc_batch_create: {self._L.sqc_status_string(rc).decode()}")
        self._h = h
        self.precision = precision
        self._keep = []
        self.n = 0

    def _check(self, rc, what):
        if rc != OK:
            msg = self._L.sqc_batch_last_error(self._h).decode() if self._h else ""
            raise SparqcError(rc, f"{what}: {self._L.sqc_status_string(rc).decode()} ({msg})")

    def close(self):
        if getattr(self, "_h", None):
            self._L.sqc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self):
        return self._L.sqc_batch_stream(self._h)

    def prepare(self, circuits):
        descs = (CircuitDesc * max(len(circuits), 1))()
        keep = []
        for i, (nq, gates) in enumerate(circuits):
            g = np.ascontiguousarray(gates, GATE_DTYPE)
            keep.append(g)
            descs[i].nq = nq
            descs[i].gates = g.ctypes.data
            descs[i].n_gates = g.size
        self._check(self._L.sqc_batch_prepare(self._h, descs, len(circuits)), "batch prepare")
        self.n = len(circuits)

    def run(self):
        self._check(self._L.sqc_batch_run(self._h), "batch run")

    def sync(self):
        self._check(self._L.sqc_batch_sync(self._h), "batch sync")

    def status(self, i):
        s = ctypes.c_int()
        self._check(self._L.sqc_batch_circuit_status(self._h, i, ctypes.byref(s)), "batch status")
        return s.value

    def nnz(self, i):
        n = ctypes.c_uint64()
        self._check(self._L.sqc_batch_nnz(self._h, i, ctypes.byref(n)), "batch nnz")
        return n.value

    def state(self, i, sorted=True, drop_negligible=False):
        n = self.nnz(i)
        keys = np.empty(max(n, 1), np.uint64)
        re = np.empty(max(n, 1), np.float64)
        im = np.empty(max(n, 1), np.float64)
        got = ctypes.c_uint64()
        flags = (READ_SORTED if sorted else 0) | (READ_DROP_NEGLIGIBLE if drop_negligible else 0)
        self._check(self._L.sqc_batch_get_state(self._h, i, _p(keys), _p(re), _p(im), n, ctypes.byref(got), flags),
                    "batch get_state")
        m = got.value
        return keys[:m].copy(), re[:m].copy(), im[:m].copy()

    def states(self, sorted=False, drop_negligible=False, out=None):
        """Every circuit's state in one call: a list of (keys, re, im) views into three arrays.
        out: optional (keys, re, im) arrays to fill (e.g. page-locked), large enough for every
        circuit's keys."""
        n = int(sum(self.nnz(i) for i in range(self.n)))
        if out is None:
            out = (np.empty(max(n, 1), np.uint64), np.empty(max(n, 1), np.float64), np.empty(max(n, 1), np.float64))
        keys, re, im = out
        counts = np.zeros(max(self.n, 1), np.uint64)
        total = ctypes.c_uint64()
        flags = (READ_SORTED if sorted else 0) | (READ_DROP_NEGLIGIBLE if drop_negligible else 0)
        self._check(self._L.sqc_batch_get_states(self._h, _p(keys), _p(re), _p(im), keys.size, _p(counts),
                                                 ctypes.byref(total), flags), "batch get_states")
        res, at = [], 0
        for i in range(self.n):
            c = int(counts[i])
            res.append((keys[at:at + c], re[at:at + c], im[at:at + c]))
            at += c
        return res

    def compare(self, i, ref):
        """(fidelity, max abs error) of circuit i against a State of the same qubit count."""
        f, e = ctypes.c_double(), ctypes.c_double()
        self._check(self._L.sqc_batch_compare(self._h, i, ref.handle, ctypes.byref(f), ctypes.byref(e)),
                    "batch compare")
        return f.value, e.value

    def autotune(self):
        t = BatchTuning()
        self._check(self._L.sqc_batch_autotune(self._h, ctypes.byref(t)), "batch autotune")
        return {n: getattr(t, n) for n, _ in BatchTuning._fields_ if n != "reserved"}

    def stats(self):
        s = BatchStats()
        self._check(self._L.sqc_batch_get_stats(self._h, ctypes.byref(s)), "batch stats")
        return {n: getattr(s, n) for n, _ in BatchStats._fields_}


class Server:
    """Serving loop: circuits submitted one by one share the GPU with those already running.

    ``submit(nq, gates)`` queues a circuit and returns its request id; every ``step()`` admits
    what fits the memory budget and runs one time slice of all resident circuits; completed
    requests are listed by ``completed()`` and read with ``state(id)`` until ``release(id)``.
    """

    def __init__(self, precision=FP64, prune_threshold=1e-14, load_factor=0.45, memory_budget=0, max_slots=1024,
                 min_chunk=8, slice_ms=2.0, stream=None, device=0, solo_log2_groups=0, solo_share_pct=25,
                 inject_alloc_failures=0, schedule_gates=False, overlap_steps=False):
        self._L = load()
        o = ServerOptions()
        self._L.sqc_server_default_options(ctypes.byref(o))
        o.precision = precision
        o.prune_threshold = prune_threshold
        o.load_factor = load_factor
        o.memory_budget = memory_budget
        o.max_slots = max_slots
        o.min_chunk = min_chunk
        o.slice_ms = slice_ms
        o.solo_log2_groups = solo_log2_groups
        o.solo_share_pct = solo_share_pct
        o.inject_alloc_failures = inject_alloc_failures
        o.schedule_gates = 1 if schedule_gates else 0
        o.overlap_steps = 1 if overlap_steps else 0
        o.stream = stream
        o.device = device
        h = ctypes.c_void_p()
        rc = self._L.sqc_server_create(ctypes.byref(o), ctypes.byref(h))
        if rc != OK:
            raise SparqcError(rc, f"sqc_server_create: {self._L.sqc_status_string(rc).decode()}")
        self._h = h
        self.precision = precision

    def _check(self, rc, what):
        if rc != OK:
            msg = self._L.sqc_server_last_error(self._h).decode() if self._h else ""
            raise SparqcError(rc, f"{what}: {self._L.sqc_status_string(rc).decode()} ({msg})")

    def close(self):
        if getattr(self, "_h", None):
            self._L.sqc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self):
        return self._L.sqc_server_stream(self._h)

    def submit(self, nq, gates):
        g = np.ascontiguousarray(gates, GATE_DTYPE)
        d = CircuitDesc()
        d.nq = nq
        d.gates = g.ctypes.data
        d.n_gates = g.size
        rid = ctypes.c_uint64()
        self._check(self._L.sqc_server_submit(self._h, ctypes.byref(d), ctypes.byref(rid)), "server submit")
        return rid.value

    def step(self):
        n = ctypes.c_uint32()
        self._check(self._L.sqc_server_step(self._h, ctypes.byref(n)), "server step")
        return n.value

    def completed(self, cap=1 << 16):
        ids = np.empty(cap, np.uint64)
        n = ctypes.c_uint32()
        self._check(self._L.sqc_server_completed(self._h, _p(ids), cap, ctypes.byref(n)), "server completed")
        return [int(x) for x in ids[:n.value]]

    def status(self, rid):
        st, code = ctypes.c_int(), ctypes.c_int()
        self._check(self._L.sqc_server_request_status(self._h, rid, ctypes.byref(st), ctypes.byref(code)),
                    "server status")
        return st.value, code.value

    def nnz(self, rid):
        n = ctypes.c_uint64()
        self._check(self._L.sqc_server_nnz(self._h, rid, ctypes.byref(n)), "server nnz")
        return n.value

    def state(self, rid, sorted=True, drop_negligible=False):
        n = self.nnz(rid)
        keys = np.empty(max(n, 1), np.uint64)
        re = np.empty(max(n, 1), np.float64)
        im = np.empty(max(n, 1), np.float64)
        got = ctypes.c_uint64()
        flags = (READ_SORTED if sorted else 0) | (READ_DROP_NEGLIGIBLE if drop_negligible else 0)
        self._check(self._L.sqc_server_get_state(self._h, rid, _p(keys), _p(re), _p(im), n, ctypes.byref(got),
                                                 flags), "server get_state")
        m = got.value
        return keys[:m].copy(), re[:m].copy(), im[:m].copy()

    def compare(self, rid, ref):
        """(fidelity, max abs error) of a completed request against a State of the same qubit count."""
        f, e = ctypes.c_double(), ctypes.c_double()
        self._check(self._L.sqc_server_compare(self._h, rid, ref.handle, ctypes.byref(f), ctypes.byref(e)),
                    "server compare")
        return f.value, e.value

    def release(self, rid):
        self._check(self._L.sqc_server_release(self._h, rid), "server release")

    def stats(self):
        s = ServerStats()
        self._check(self._L.sqc_server_get_stats(self._h, ctypes.byref(s)), "server stats")
        return {n: getattr(s, n) for n, _ in ServerStats._fields_}


class PartState:
    """A state that may outgrow the device: it runs in one device table while the table fits in
    ``device_bytes`` and moves to host memory, processed partition by partition, when it does not.
    Results are bit-identical to a single table."""

    def __init__(self, nq, device_bytes=0, precision=FP64, prune_threshold=1e-14, load_factor=0.5, stream=None,
                 device=0, params=None):
        self._L = load()
        o = Options()
        self._L.sqc_default_options(ctypes.byref(o))
        o.precision = precision
        o.prune_threshold = prune_threshold
        o.load_factor = load_factor
        o.stream = stream
        o.device = device
        h = ctypes.c_void_p()
        pp = ctypes.byref(params) if params is not None else None
        rc = self._L.sqc_part_create(nq, pp, ctypes.byref(o), device_bytes, ctypes.byref(h))
        if rc != OK:
            raise SparqcError(rc, f"sqc_part_create: {self._L.sqc_status_string(rc).decode()}")
        self._h = h
        self.nq = nq
        self.precision = precision

    def _check(self, rc, what):
        if rc != OK:
            msg = self._L.sqc_part_last_error(self._h).decode() if self._h else ""
            raise SparqcError(rc, f"{what}: {self._L.sqc_status_string(rc).decode()} ({msg})")

    def close(self):
        if getattr(self, "_h", None):
            self._L.sqc_part_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_zero(self):
        self._check(self._L.sqc_part_set_zero_state(self._h), "set_zero")

    def apply(self, gates):
        gates = np.ascontiguousarray(gates, GATE_DTYPE)
        self._check(self._L.sqc_part_apply_gates(self._h, _p(gates), gates.size), "apply")

    def sync(self):
        self._check(self._L.sqc_part_sync(self._h), "sync")

    @property
    def nnz(self):
        n = ctypes.c_uint64()
        self._check(self._L.sqc_part_nnz(self._h, ctypes.byref(n)), "nnz")
        return n.value

    def state(self, sorted=True, drop_negligible=False):
        n = self.nnz
        keys = np.empty(max(n, 1), np.uint64)
        re = np.empty(max(n, 1), np.float64)
        im = np.empty(max(n, 1), np.float64)
        got = ctypes.c_uint64()
        flags = (READ_SORTED if sorted else 0) | (READ_DROP_NEGLIGIBLE if drop_negligible else 0)
        self._check(self._L.sqc_part_get_state(self._h, _p(keys), _p(re), _p(im), n, ctypes.byref(got), flags),
                    "get_state")
        m = got.value
        return keys[:m].copy(), re[:m].copy(), im[:m].copy()

    def stats(self):
        s = PartStats()
        self._check(self._L.sqc_part_get_stats(self._h, ctypes.byref(s)), "part stats")
        return {n: getattr(s, n) for n, _ in PartStats._fields_}
