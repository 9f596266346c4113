"""ctypes wrapper of the host-emulated reference kernels -- TEST INFRASTRUCTURE ONLY.

Runs the reference's own FC gate code (compiled for the host by ``build.build_refemu``)
for the eight reference gates: X, Y, Z, H, Phase, Rz, Rx, Ry, uncontrolled, on a
dense-capacity table of 2**nq slots (nq <= 22). Available only where the reference
sources are present; the emulated table is a process-wide singleton, as the reference's
``__constant__`` descriptor is (emulator/device/device_data.cuh:36).
"""
import ctypes
import numpy as np

from . import build

REF_KINDS = (0, 1, 2, 3, 4, 5, 6, 7)   # X Y Z H Phase Rz Rx Ry
_lib = None


def available():
    return build.reference_available()


def lib():
    global _lib
    if _lib is None:
        path = build.build_refemu()
        if path is None:
            raise RuntimeError("reference sources not present; reference emulation unavailable")
        L = ctypes.CDLL(path)
        L.refemu_create.restype = ctypes.c_int
        L.refemu_create.argtypes = [ctypes.c_uint32]
        L.refemu_destroy.argtypes = []
        L.refemu_gate.restype = ctypes.c_int
        L.refemu_gate.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_double]
        L.refemu_address_book_size.restype = ctypes.c_int64
        L.refemu_get_state.restype = ctypes.c_int64
        L.refemu_get_state.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_uint64]
        _lib = L
    return _lib


def run(nq, gates):
    """Run uncontrolled reference gates from |0...0>.

    Returns (keys, re, im, hazards): the key-sorted non-negligible state and the indices of
    gates that hit the reference's Rx/Ry address-book race.
    """
    L = lib()
    if L.refemu_create(nq) != 0:
        raise ValueError("refemu_create failed")
    hazards = []
    try:
        for i, g in enumerate(gates):
            kind = int(g["kind"])
            if kind not in REF_KINDS or int(g["controls"]) != 0:
                raise ValueError(f"gate {i}: not a reference gate")
            rc = L.refemu_gate(kind, int(g["target"]), float(g["theta"]))
            if rc < 0:
                raise ValueError(f"refemu_gate failed at gate {i} ({rc})")
            if rc == 1:
                hazards.append(i)
        cap = 1 << nq
        keys = np.empty(cap, np.uint64)
        re = np.empty(cap, np.float64)
        im = np.empty(cap, np.float64)
        n = L.refemu_get_state(keys.ctypes.data_as(ctypes.c_void_p), re.ctypes.data_as(ctypes.c_void_p),
                               im.ctypes.data_as(ctypes.c_void_p), cap)
        if n < 0:
            raise ValueError(f"refemu_get_state failed ({n})")
        return keys[:n].copy(), re[:n].copy(), im[:n].copy(), hazards
    finally:
        L.refemu_destroy()
