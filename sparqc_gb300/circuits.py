"""Seeded synthetic circuits for the parity tests and the benchmark.

The reference ships no benchmark circuits (its only workload is H on every qubit,
emulator/src/main.cu:142-143), so the workloads are generated here from a splitmix64
stream keyed by (config, circuit index, seed):

* every circuit starts with H on qubits 0..k-1, then draws the rest of its gates with
  30% diagonal (Z, S, T, Rz, Phase), 30% permutation (X, Y) and 40% branching
  (H, Rx, Ry, U) gates, angles uniform in [0, 2*pi);
* branching gates target qubits < k; diagonal gates target any qubit; permutation gates
  target any qubit;
* controls: a uniform count in 0..max_controls of distinct qubits other than the target;
  a permutation gate whose target is >= k takes controls from qubits >= k only.

The last rule keeps every key's bits >= k identical across the state (a permutation on a
high qubit then acts on all keys or on none), so the state never holds more than 2**k
nonzeros. Without it a CNOT from a low control onto a high target followed by branching
gates would double the nonzero count per branching qubit.

Configurations (sizes from the engine's benchmark definitions):
  c1: 20 qubits, k=10, 200 gates, 0-2 controls
  c2: 40 qubits, k=20, 2000 gates, 0-3 controls
  c3: 64 qubits, k=26, 500 gates, 0-3 controls
  c4: 256 circuits, qubits ~U{16..48}, k ~U{8..18}, depth ~U{100..1000}, 0-3 controls
  c5: c4 draws plus 5% large circuits (48 qubits, k=24, depth 2000); Poisson arrivals
"""
import math

import numpy as np

from .gates import GATE_DTYPE, X, Y, Z, H, PHASE, RZ, RX, RY, S, T, U

M64 = (1 << 64) - 1
DIAG = (Z, S, T, RZ, PHASE)
PERM = (X, Y)
BRANCH = (H, RX, RY, U)
TWO_PI = 2.0 * math.pi


class SplitMix64:
    def __init__(self, seed):
        self.s = seed & M64

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        return z ^ (z >> 31)

    def uniform(self):
        return (self.next() >> 11) * (1.0 / (1 << 53))

    def randint(self, lo, hi):
        """Uniform integer in [lo, hi]."""
        return lo + self.next() % (hi - lo + 1)


def stream_seed(config, index=0, seed=0):
    h = 0x5EED
    for part in (hash_str(config), index, seed):
        h = SplitMix64(h ^ part).next()
    return h


def hash_str(s):
    h = 1469598103934665603
    for ch in str(s).encode():
        h = ((h ^ ch) * 1099511628211) & M64
    return h


def _pick_controls(rng, n, pool):
    pool = list(pool)
    out = []
    for _ in range(min(n, len(pool))):
        j = rng.next() % len(pool)
        out.append(pool.pop(j))
    m = 0
    for q in out:
        m |= 1 << q
    return m


def random_circuit(nq, k, depth, max_controls, rng, prefix_h=True, kinds=None):
    """Draw one circuit as a GATE_DTYPE array (see the module docstring for the rules).

    ``kinds`` optionally restricts the gate set, as (diag, perm, branch) kind tuples.
    """
    if not (1 <= k <= nq <= 64):
        raise ValueError("need 1 <= k <= nq <= 64")
    diag, perm, branch = kinds if kinds is not None else (DIAG, PERM, BRANCH)
    g = np.zeros(depth, GATE_DTYPE)
    i = 0
    if prefix_h:
        for q in range(min(k, depth)):
            g[i]["kind"] = H
            g[i]["target"] = q
            i += 1
    while i < depth:
        u = rng.uniform()
        if u < 0.3 and diag:
            kind = diag[rng.next() % len(diag)]
            target = rng.next() % nq
            pool = [q for q in range(nq) if q != target]
        elif u < 0.6 and perm:
            kind = perm[rng.next() % len(perm)]
            target = rng.next() % nq
            lo = k if target >= k else 0
            pool = [q for q in range(lo, nq) if q != target]
        elif branch:
            kind = branch[rng.next() % len(branch)]
            target = rng.next() % k
            pool = [q for q in range(nq) if q != target]
        else:
            continue
        nctl = rng.randint(0, max_controls) if max_controls > 0 else 0
        g[i]["kind"] = kind
        g[i]["target"] = target
        g[i]["controls"] = _pick_controls(rng, nctl, pool)
        if kind in (RZ, RX, RY, PHASE, U):
            g[i]["theta"] = rng.uniform() * TWO_PI
        if kind == U:
            g[i]["phi"] = rng.uniform() * TWO_PI
            g[i]["lambda"] = rng.uniform() * TWO_PI
        i += 1
    return g


CONFIGS = {
    "c1": dict(nq=20, k=10, depth=200, max_controls=2),
    "c2": dict(nq=40, k=20, depth=2000, max_controls=3),
    "c3": dict(nq=64, k=26, depth=500, max_controls=3),
}


def config_circuit(name, index=0, seed=0):
    """One circuit of configuration c1, c2 or c3."""
    p = CONFIGS[name]
    rng = SplitMix64(stream_seed(name, index, seed))
    return p["nq"], random_circuit(p["nq"], p["k"], p["depth"], p["max_controls"], rng)


def batch_circuits(count=256, seed=0, qrange=(16, 48), krange=(8, 18), drange=(100, 1000),
                   max_controls=3, config="c4"):
    """Circuits of the batching configuration: list of (nq, k, gates)."""
    out = []
    for i in range(count):
        rng = SplitMix64(stream_seed(config, i, seed))
        nq = rng.randint(*qrange)
        k = min(rng.randint(*krange), nq)
        depth = rng.randint(*drange)
        out.append((nq, k, random_circuit(nq, k, depth, max_controls, rng)))
    return out


def serving_stream(count, rate_hz, seed=0, large_fraction=0.05, large=(48, 24, 2000)):
    """Poisson arrivals of batching-config circuits plus a fraction of large ones.

    Returns a list of (arrival_seconds, nq, k, gates), arrivals increasing.
    """
    rng = SplitMix64(stream_seed("c5", 0, seed))
    t = 0.0
    out = []
    for i in range(count):
        t += -math.log(1.0 - rng.uniform()) / rate_hz
        crng = SplitMix64(stream_seed("c5", i + 1, seed))
        if crng.uniform() < large_fraction:
            nq, k, depth = large
        else:
            nq = crng.randint(16, 48)
            k = min(crng.randint(8, 18), nq)
            depth = crng.randint(100, 1000)
        out.append((t, nq, k, random_circuit(nq, k, depth, 3, crng)))
    return out
