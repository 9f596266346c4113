"""Gate descriptors of the engine's C ABI (``sqc_gate`` in include/sparqc.h).

A gate is (kind, target, controls, theta, phi, lambda): a 40-byte record. ``controls`` is a
bit mask of control qubits; the gate acts on a key iff every control bit is 1. Qubit t is
bit t of the 64-bit basis-state key (qubit 0 = least significant bit), as in the reference
(emulator/src/QLib.cpp:15-28).

The eight reference gates keep the reference's argument meaning (emulator/include/circuit.h:45-83):
``phase(t, par)`` multiplies the bit-1 amplitude by e^{i par}; ``rz/rx/ry(t, par)`` are
rotations by ``par`` (the engine, like the reference, applies cos/sin of par/2,
emulator/device/table_manager.cuh:333-336). Added gates: S, Sdg, T, Tdg and the u3 gate
U(theta, phi, lambda) = [[cos(theta/2), -e^{i lambda} sin(theta/2)],
                         [e^{i phi} sin(theta/2), e^{i(phi+lambda)} cos(theta/2)]].
"""
import numpy as np

X, Y, Z, H, PHASE, RZ, RX, RY, S, SDG, T, TDG, U = range(13)
NAMES = ("x", "y", "z", "h", "phase", "rz", "rx", "ry", "s", "sdg", "t", "tdg", "u")

SWAP_KINDS = (X, Y)                       # move keys, never prune
DIAG_KINDS = (Z, PHASE, RZ, S, SDG, T, TDG)  # keep keys, never prune
BRANCH_KINDS = (H, RX, RY, U)             # may create keys, prune negligible outputs

GATE_DTYPE = np.dtype([("kind", "<u4"), ("target", "<u4"), ("controls", "<u8"),
                       ("theta", "<f8"), ("phi", "<f8"), ("lambda", "<f8")])
assert GATE_DTYPE.itemsize == 40


def mask(qubits):
    m = 0
    for q in qubits:
        m |= 1 << int(q)
    return m


def gate(kind, target, controls=(), theta=0.0, phi=0.0, lam=0.0):
    g = np.zeros((), GATE_DTYPE)
    g["kind"] = kind
    g["target"] = target
    g["controls"] = controls if isinstance(controls, (int, np.integer)) else mask(controls)
    g["theta"] = theta
    g["phi"] = phi
    g["lambda"] = lam
    return g


def gate_array(gates):
    """Stack gate records (or (kind, target, controls, theta, phi, lam) tuples) into an array."""
    out = np.zeros(len(gates), GATE_DTYPE)
    for i, g in enumerate(gates):
        if isinstance(g, np.ndarray) or isinstance(g, np.void):
            out[i] = g
        else:
            out[i] = gate(*g)
    return out
