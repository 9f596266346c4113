"""Two-qubit gates: the engine's gate sequences against textbook 4x4 matrices.

CPU part: the sequences (sqc_twoq_gates, host code of the library) run through the numpy dense
statevector equal the 4x4 matrix applied directly, within 1e-12, with and without controls.
GPU part: the engine applying them matches the oracle fed the same sequence bit for bit, and the
dense statevector applying the matrices within the usual tolerance.
"""
import numpy as np
import pytest

from oracle.dense import DenseOracle, PagedDenseOracle, matrix2
from oracle.sparse import SparseOracle
from sparqc_gb300 import circuits, gates as G
from sparqc_gb300.engine import (TWOQ_CSWAP, TWOQ_FSIM, TWOQ_ISWAP, TWOQ_RZZ, TWOQ_SWAP, TWOQ_UNITARY, SparqcError,
                                 State, twoq_gates)
from test_oracle import assert_close, assert_identical, drop_negligible


def random_unitary(rng):
    z = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def random_state(nq, rng):
    psi = rng.normal(size=1 << nq) + 1j * rng.normal(size=1 << nq)
    return psi / np.linalg.norm(psi)


def dense_with_state(nq, psi):
    d = DenseOracle(nq)
    d.psi[:] = psi
    return d


CASES = [(TWOQ_RZZ, 0.7, 0.0), (TWOQ_ISWAP, 0.0, 0.0), (TWOQ_FSIM, 1.1, 0.4), (TWOQ_SWAP, 0.0, 0.0)]


@pytest.mark.parametrize("a,b,controls", [(0, 1, 0), (3, 1, 0), (2, 4, 1 << 0), (5, 0, (1 << 2) | (1 << 3))])
def test_sequences_equal_their_matrices(a, b, controls):
    rng = np.random.default_rng(a * 7 + b)
    nq = 6
    for form, th, ph in CASES + [(TWOQ_UNITARY, 0.0, 0.0)] * 3:
        u = random_unitary(rng) if form == TWOQ_UNITARY else matrix2(form, th, ph)
        psi = random_state(nq, rng)
        want = dense_with_state(nq, psi)
        want.apply_matrix2(a, b, controls, u)
        got = dense_with_state(nq, psi)
        got.apply(twoq_gates(form, a, b, controls=controls, theta=th, phi=ph,
                             u=u if form == TWOQ_UNITARY else None))
        assert np.max(np.abs(got.psi - want.psi)) < 1e-12, form


def test_cswap_sequence():
    rng = np.random.default_rng(3)
    for c, a, b in ((0, 1, 2), (4, 0, 3), (2, 5, 1)):
        psi = random_state(6, rng)
        want = dense_with_state(6, psi)
        want.apply_matrix2(a, b, 1 << c, matrix2(TWOQ_CSWAP))
        got = dense_with_state(6, psi)
        got.apply(twoq_gates(TWOQ_CSWAP, a, b, c))
        assert np.max(np.abs(got.psi - want.psi)) < 1e-15


def test_bad_two_qubit_arguments():
    with pytest.raises(SparqcError):
        twoq_gates(TWOQ_RZZ, 3, 3, theta=0.1)
    with pytest.raises(SparqcError):
        twoq_gates(TWOQ_ISWAP, 1, 2, controls=1 << 2)
    with pytest.raises(SparqcError):
        twoq_gates(TWOQ_UNITARY, 0, 1, u=np.eye(4) * 2.0)


def mixed_circuit(nq, k, seed):
    """A random circuit with two-qubit gates interleaved (from their sequences), the list of
    (position, form, a, b, c, controls, theta, phi, u) of those gates, and the full gate array."""
    rng = circuits.SplitMix64(circuits.stream_seed("twoq", seed))
    npr = np.random.default_rng(seed)
    base = circuits.random_circuit(nq, k, 120, 2, rng)
    parts, twoqs = [], []
    for i in range(0, base.size, 12):
        parts.append(base[i:i + 12])
        form = [TWOQ_UNITARY, TWOQ_RZZ, TWOQ_ISWAP, TWOQ_FSIM, TWOQ_CSWAP, TWOQ_SWAP][(i // 12) % 6]
        a, b = (int(x) for x in npr.choice(k, 2, replace=False))
        c = int(npr.choice([q for q in range(nq) if q not in (a, b)]))
        others = [q for q in range(nq) if q not in (a, b, c)]
        controls = (1 << int(npr.choice(others))) if (i // 12) % 3 == 1 else 0
        th, ph = float(npr.uniform(0, 6.28)), float(npr.uniform(0, 6.28))
        u = random_unitary(npr) if form == TWOQ_UNITARY else None
        twoqs.append((sum(p.size for p in parts), form, a, b, c, controls, th, ph, u))
        parts.append(twoq_gates(form, a, b, c, controls, th, ph, u))
    return np.concatenate(parts), twoqs, base


@pytest.mark.gpu
@pytest.mark.parametrize("seed,nq,k", [(0, 12, 8), (1, 20, 10), (2, 40, 11)])
def test_engine_two_qubit_gates_against_oracles(seed, nq, k):
    gates, twoqs, _ = mixed_circuit(nq, k, seed)
    # the engine: single-qubit gates from the array, two-qubit gates through sqc_apply_twoq
    st = State(nq)
    pos = 0
    for at, form, a, b, c, controls, th, ph, u in twoqs:
        st.apply(gates[pos:at])
        st.apply_twoq(form, a, b, c, controls, th, ph, u)
        pos = at + twoq_gates(form, a, b, c, controls, th, ph, u).size
    st.apply(gates[pos:])
    got = st.state(sorted=True)
    st.close()
    o = SparseOracle()
    o.apply(gates)
    assert_identical(got, o.state(sorted=True))
    # the dense statevector applies the two-qubit gates as 4x4 matrices
    d = PagedDenseOracle(nq)
    pos = 0
    for at, form, a, b, c, controls, th, ph, u in twoqs:
        d.apply(gates[pos:at])
        m = u if form == TWOQ_UNITARY else matrix2(form, th, ph)
        d.apply_matrix([a, b], controls | ((1 << c) if form == TWOQ_CSWAP else 0), m)
        pos = at + twoq_gates(form, a, b, c, controls, th, ph, u).size
    d.apply(gates[pos:])
    assert_close(drop_negligible(got), d.state())
