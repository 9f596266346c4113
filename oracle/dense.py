"""Dense FP64 statevector oracle -- TEST INFRASTRUCTURE ONLY.

An independent check of the gate definitions: textbook 2x2 matrices applied to a full
complex128 vector of 2**nq amplitudes (nq <= 26 here; 30 would need 16 GiB), with no
pruning. Qubit t is bit t of the basis-state index, qubit 0 the least significant bit
(the reference's ordering, emulator/src/QLib.cpp:15-28). Rz/Rx/Ry take the full angle
theta and use theta/2 inside the matrix (emulator/device/table_manager.cuh:333-336);
Phase takes theta unchanged. Controls: the gate acts iff every control bit is 1.
"""
import numpy as np

# gate kinds, same numbering as the engine's sqc_gate
X, Y, Z, H, PHASE, RZ, RX, RY, S, SDG, T, TDG, U = range(13)


def matrix(kind, theta=0.0, phi=0.0, lam=0.0):
    c2, s2 = np.cos(theta / 2), np.sin(theta / 2)
    r = 1 / np.sqrt(2)
    m = {
        X: [[0, 1], [1, 0]],
        Y: [[0, -1j], [1j, 0]],
        Z: [[1, 0], [0, -1]],
        H: [[r, r], [r, -r]],
        PHASE: [[1, 0], [0, np.exp(1j * theta)]],
        RZ: [[np.exp(-0.5j * theta), 0], [0, np.exp(0.5j * theta)]],
        RX: [[c2, -1j * s2], [-1j * s2, c2]],
        RY: [[c2, -s2], [s2, c2]],
        S: [[1, 0], [0, 1j]],
        SDG: [[1, 0], [0, -1j]],
        T: [[1, 0], [0, np.exp(0.25j * np.pi)]],
        TDG: [[1, 0], [0, np.exp(-0.25j * np.pi)]],
        U: [[c2, -np.exp(1j * lam) * s2], [np.exp(1j * phi) * s2, np.exp(1j * (phi + lam)) * c2]],
    }[kind]
    return np.asarray(m, dtype=np.complex128)


def matrix2(form, theta=0.0, phi=0.0):
    """Textbook 4x4 matrices of the named two-qubit gates over the index i_a + 2 i_b (CSWAP: the
    SWAP it applies where its control is 1). Forms numbered as the engine's SQC_2Q_*."""
    c, s = np.cos(theta), np.sin(theta)
    e = np.exp(-0.5j * theta)
    m = {
        1: np.diag([e, np.conj(e), np.conj(e), e]),                                  # RZZ
        2: [[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]],                # iSWAP
        3: [[1, 0, 0, 0], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [0, 0, 0, np.exp(-1j * phi)]],   # fSim
        4: [[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]],                  # CSWAP's SWAP
        5: [[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]],                  # SWAP
    }[form]
    return np.asarray(m, dtype=np.complex128)


class DenseOracle:
    def __init__(self, nq):
        if nq > 26:
            raise ValueError("dense oracle limited to 26 qubits here")
        self.nq = nq
        self.psi = np.zeros(1 << nq, np.complex128)
        self.psi[0] = 1.0
        self._idx = np.arange(1 << nq, dtype=np.uint64)

    def set_state(self, keys, re, im):
        self.psi[:] = 0
        self.psi[np.asarray(keys, dtype=np.int64)] = np.asarray(re) + 1j * np.asarray(im)

    def apply(self, gates):
        for g in gates:
            self.apply_one(int(g["kind"]), int(g["target"]), int(g["controls"]),
                           float(g["theta"]), float(g["phi"]), float(g["lambda"]))

    def apply_one(self, kind, t, controls, theta=0.0, phi=0.0, lam=0.0):
        m = matrix(kind, theta, phi, lam)
        bq = np.uint64(1 << t)
        idx = self._idx
        sel = ((idx & bq) == 0) & ((idx & np.uint64(controls)) == np.uint64(controls))
        i0 = idx[sel].astype(np.int64)
        i1 = i0 | (1 << t)
        a0 = self.psi[i0].copy()
        a1 = self.psi[i1].copy()
        self.psi[i0] = m[0, 0] * a0 + m[0, 1] * a1
        self.psi[i1] = m[1, 0] * a0 + m[1, 1] * a1

    def apply_matrix2(self, a, b, controls, m):
        """A 4x4 matrix m on qubits (a, b), index i_a + 2 i_b, where every control bit is 1."""
        ba, bb = np.uint64(1 << a), np.uint64(1 << b)
        idx = self._idx
        sel = ((idx & (ba | bb)) == 0) & ((idx & np.uint64(controls)) == np.uint64(controls))
        i0 = idx[sel].astype(np.int64)
        grp = [i0, i0 | (1 << a), i0 | (1 << b), i0 | (1 << a) | (1 << b)]
        v = [self.psi[g].copy() for g in grp]
        for r in range(4):
            self.psi[grp[r]] = sum(m[r, k] * v[k] for k in range(4))

    def state(self, threshold=1e-14):
        """Key-sorted entries whose amplitude is not negligible (|re|,|im| < threshold)."""
        nz = ~((np.abs(self.psi.real) < threshold) & (np.abs(self.psi.imag) < threshold))
        keys = np.nonzero(nz)[0].astype(np.uint64)
        return keys, self.psi.real[nz].copy(), self.psi.imag[nz].copy()


# ---- paged dense statevector in C (oracle/dense_oracle.c) ---------------------------------
_dlib = None


def _dense_lib():
    global _dlib
    if _dlib is None:
        import ctypes
        from . import build
        L = ctypes.CDLL(build.build_dense())
        P, U64, U32, D, I = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_double, ctypes.c_int
        L.dno_create.restype = P
        L.dno_create.argtypes = [I]
        L.dno_destroy.argtypes = [P]
        L.dno_set_threads.argtypes = [P, I]
        L.dno_max_threads.restype = I
        L.dno_set_state.restype = I
        L.dno_set_state.argtypes = [P, P, P, P, U64]
        L.dno_apply1.restype = I
        L.dno_apply1.argtypes = [P, U32, U64, P]
        L.dno_apply2.restype = I
        L.dno_apply2.argtypes = [P, U32, U32, U64, P]
        L.dno_get_state.restype = U64
        L.dno_get_state.argtypes = [P, P, P, P, U64, D]
        _dlib = L
    return _dlib


def _ptr(a):
    import ctypes
    return a.ctypes.data_as(ctypes.c_void_p)


class PagedDenseOracle:
    """Dense FP64 statevector of up to 30 qubits (and beyond, for states that reach few pages),
    starting from |0...0>: the same textbook matrices as DenseOracle, applied in C to every
    index pair of the full vector; pages that have only held zeros are not stored."""

    def __init__(self, nq, threads=None):
        if not 1 <= nq <= 40:
            raise ValueError("nq out of range")
        self.nq = nq
        self._L = _dense_lib()
        self._h = self._L.dno_create(int(nq))
        if not self._h:
            raise MemoryError("dno_create failed")
        self._L.dno_set_threads(self._h, int(threads or self._L.dno_max_threads()))

    def close(self):
        if self._h:
            self._L.dno_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_state(self, keys, re, im):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        re = np.ascontiguousarray(re, dtype=np.float64)
        im = np.ascontiguousarray(im, dtype=np.float64)
        if self._L.dno_set_state(self._h, _ptr(keys), _ptr(re), _ptr(im), keys.size):
            raise ValueError("bad key")

    def apply_matrix(self, targets, controls, m):
        """Apply a 2x2 (one target) or 4x4 (two targets, index i0 + 2*i1) complex matrix."""
        m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128)).view(np.float64)
        if len(targets) == 1:
            rc = self._L.dno_apply1(self._h, int(targets[0]), int(controls), _ptr(m))
        else:
            rc = self._L.dno_apply2(self._h, int(targets[0]), int(targets[1]), int(controls), _ptr(m))
        if rc:
            raise ValueError(f"dno_apply failed ({rc})")

    def apply(self, gates):
        for g in gates:
            self.apply_matrix([int(g["target"])], int(g["controls"]),
                              matrix(int(g["kind"]), float(g["theta"]), float(g["phi"]), float(g["lambda"])))

    def state(self, threshold=1e-14):
        """Key-sorted entries whose amplitude is not negligible (|re|,|im| < threshold)."""
        n = int(self._L.dno_get_state(self._h, None, None, None, 0, threshold))
        keys = np.empty(n, np.uint64)
        re = np.empty(n, np.float64)
        im = np.empty(n, np.float64)
        self._L.dno_get_state(self._h, _ptr(keys), _ptr(re), _ptr(im), n, threshold)
        return keys, re, im
