"""Generate the golden fixtures from the reference's own gate kernels.

Run from the repository root where the reference sources are present:
    python tests/golden/make_golden.py
It compiles the reference's FC kernel headers for the host (oracle/ref_harness.cpp, built
by oracle/build.py), runs seeded circuits of the reference gate set through them, and
stores gates and the key-sorted non-negligible final state in ``reference_fc.npz``.

Circuits (all uncontrolled, the only form the reference has):
  * ``hn``   : H on every qubit, the reference's own workload (emulator/src/main.cu:142-143);
  * ``kat_*``: one gate of each of the eight reference kinds on a fixed complex 4-key
               state, on a superposed target and on an unsuperposed one;
  * ``rnd_*``: random X/Y/Z/H/Phase/Rz circuits, plus Rx/Ry gates placed only where the
               reference's Rx/Ry address-book race cannot fire (no pair on the target has
               both members present), checked by the emulation itself.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import refemu  # noqa: E402
from oracle.sparse import SparseOracle  # noqa: E402
from sparqc_gb300 import circuits, gates as G  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_fc.npz")


def both_present(keys, t):
    s = set(int(k) for k in keys)
    return any(((k >> t) & 1) and (k ^ (1 << t)) in s for k in s)


def hazard_free_circuit(nq, k, depth, seed):
    """Random reference-gate circuit whose Rx/Ry gates never meet a fully present pair."""
    rng = circuits.SplitMix64(circuits.stream_seed("golden", seed))
    orc = SparseOracle()
    out = []
    for q in range(k):
        g = G.gate(G.H, q)
        out.append(g)
        orc.apply(np.array([g]))
    while len(out) < depth:
        u = rng.uniform()
        if u < 0.3:
            kind = (G.Z, G.PHASE, G.RZ)[rng.next() % 3]
            t = rng.next() % nq
        elif u < 0.6:
            kind = (G.X, G.Y)[rng.next() % 2]
            t = rng.next() % nq
        else:
            kind = (G.H, G.RX, G.RY)[rng.next() % 3]
            t = rng.next() % nq
            if kind in (G.RX, G.RY) and both_present(orc.state()[0], t):
                continue
        theta = rng.uniform() * 2 * np.pi if kind in (G.PHASE, G.RZ, G.RX, G.RY) else 0.0
        g = G.gate(kind, t, 0, theta)
        out.append(g)
        orc.apply(np.array([g]))
    return G.gate_array(out)


def kat_circuits():
    base = [(G.H, 0), (G.H, 1), (G.RZ, 0, 0, 0.4), (G.PHASE, 1, 0, 1.1)]
    out = {}
    for kind in range(8):
        for t in (0, 1, 3):
            if kind in (G.RX, G.RY) and t in (0, 1):
                continue
            out[f"kat_{G.NAMES[kind]}_t{t}"] = (4, G.gate_array(base + [(kind, t, 0, 0.9)]))
    return out


def main():
    if not refemu.available():
        raise SystemExit("reference sources not present")
    cases = {"hn": (10, G.gate_array([(G.H, q) for q in range(10)]))}
    cases.update(kat_circuits())
    for seed in range(8):
        nq = 9 + seed % 3
        cases[f"rnd_{seed}"] = (nq, hazard_free_circuit(nq, 5 + seed % 3, 160, seed))
    data = {}
    for name, (nq, g) in cases.items():
        keys, re, im, hazards = refemu.run(nq, g)
        if hazards:
            raise SystemExit(f"{name}: reference race hit at gates {hazards}")
        data[f"{name}/nq"] = np.array(nq)
        data[f"{name}/gates"] = g
        data[f"{name}/keys"] = keys
        data[f"{name}/re"] = re
        data[f"{name}/im"] = im
        print(f"{name:16s} nq={nq:2d} gates={g.size:4d} nnz={keys.size}")
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
