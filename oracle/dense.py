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

    def state(self, threshold=1e-14):
        """Key-sorted entries whose amplitude is not negligible (|re|,|im| < threshold)."""
        nz = ~((np.abs(self.psi.real) < threshold) & (np.abs(self.psi.imag) < threshold))
        keys = np.nonzero(nz)[0].astype(np.uint64)
        return keys, self.psi.real[nz].copy(), self.psi.imag[nz].copy()
