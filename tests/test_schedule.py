"""Gate scheduling (sqc_schedule_gates and the schedule_gates options).

CPU part: the order is a permutation that only moves gates past gates they commute with
(neither changes a qubit the other touches), checked pair by pair from the gates themselves; the
rule itself is checked on dense matrices; the dense statevector gives the same state in both
orders; bad arguments are refused.
GPU part: a State, a Batch and a Server with schedule_gates on equal the oracle fed the same
scheduled order bit for bit (the oracle applies gates in the order given, as the reference
does), amp-update counts included.
"""
import numpy as np
import pytest

from oracle.dense import DenseOracle
from oracle.sparse import SparseOracle
from sparqc_gb300 import circuits, gates as G
from sparqc_gb300.engine import FP32, FP64, Batch, Server, SparqcError, State, schedule_gates
from test_oracle import assert_identical

DIAG = np.array(sorted(G.DIAG_KINDS), np.uint32)


def moves_commute(g, perm):
    """Every pair the order inverts commutes: neither gate changes a qubit the other touches (a
    gate touches its target and controls, and changes its target unless it is diagonal)."""
    n = g.size
    pos = np.empty(n, np.int64)
    pos[perm] = np.arange(n)
    tbit = np.uint64(1) << g["target"].astype(np.uint64)
    sup = tbit | g["controls"]
    moves = np.where(np.isin(g["kind"], DIAG), np.uint64(0), tbit)
    i, j = np.triu_indices(n, 1)
    inv = pos[j] < pos[i]   # j (later in the input) now runs before i
    i, j = i[inv], j[inv]
    ok = ((moves[i] & sup[j]) == 0) & ((moves[j] & sup[i]) == 0)
    return bool(np.all(ok)), int(inv.sum())


def test_commutation_rule_on_matrices():
    # the rule the scheduler uses, checked on dense matrices: controlled gates sharing only
    # controls commute, diagonal gates commute, a gate changing another's control does not
    rng = np.random.default_rng(0)
    nq = 4
    cases = [((G.RX, 0, 1 << 2), (G.RY, 1, 1 << 2), True),     # shared control
             ((G.RZ, 2, 0), (G.H, 0, 1 << 2), True),           # diagonal target is the other's control
             ((G.PHASE, 1, 1 << 3), (G.T, 1, 0), True),        # both diagonal
             ((G.X, 2, 0), (G.H, 0, 1 << 2), False),           # changes the other's control
             ((G.H, 1, 0), (G.RZ, 1, 0), False)]
    for a, b, commute in cases:
        ga = G.gate_array([(a[0], a[1], [q for q in range(nq) if (a[2] >> q) & 1], 0.7)])
        gb = G.gate_array([(b[0], b[1], [q for q in range(nq) if (b[2] >> q) & 1], 1.3)])
        psi = rng.normal(size=1 << nq) + 1j * rng.normal(size=1 << nq)
        x = DenseOracle(nq)
        x.psi[:] = psi
        x.apply(np.concatenate([ga, gb]))
        y = DenseOracle(nq)
        y.psi[:] = psi
        y.apply(np.concatenate([gb, ga]))
        same = np.max(np.abs(x.psi - y.psi)) < 1e-12
        assert same == commute, (a, b)
        ok, _ = moves_commute(np.concatenate([ga, gb]), np.array([1, 0]))
        assert ok == commute, (a, b)


def some_circuits():
    out = []
    for seed, (nq, k, depth, ctl) in enumerate([(8, 6, 150, 2), (20, 10, 300, 3), (40, 12, 400, 3),
                                                (64, 14, 500, 2)]):
        out.append((nq, circuits.random_circuit(nq, k, depth, ctl,
                                                circuits.SplitMix64(circuits.stream_seed("sched", seed)))))
    for name in ("c2", "c3"):
        out.append(circuits.config_circuit(name, 0))
    return out


@pytest.mark.parametrize("max_cross", [1, 2, 3])
def test_schedule_only_moves_commuting_gates(max_cross):
    moved = 0
    for nq, g in some_circuits():
        perm = schedule_gates(nq, g, max_cross)
        assert np.array_equal(np.sort(perm), np.arange(g.size))
        ok, inv = moves_commute(g, perm)
        assert ok
        moved += inv
        assert np.array_equal(perm, schedule_gates(nq, g, max_cross))   # deterministic
    assert moved > 0


def test_schedule_keeps_the_state():
    for seed in range(4):
        nq = 10
        g = circuits.random_circuit(nq, 8, 200, 3, circuits.SplitMix64(circuits.stream_seed("sched-dense", seed)))
        a = DenseOracle(nq)
        a.apply(g)
        b = DenseOracle(nq)
        b.apply(g[schedule_gates(nq, g, 2)])
        assert np.max(np.abs(a.psi - b.psi)) < 1e-12


def test_schedule_keeps_the_state_with_two_qubit_gates():
    # U gates with controls and the relabelling X gates of two-qubit sequences
    from test_twoq import mixed_circuit
    for seed in range(3):
        g, _, _ = mixed_circuit(10, 8, seed)
        a = DenseOracle(10)
        a.apply(g)
        for mx in (1, 2, 3):
            b = DenseOracle(10)
            b.apply(g[schedule_gates(10, g, mx)])
            assert np.max(np.abs(a.psi - b.psi)) < 1e-12


def test_schedule_bad_arguments():
    g = G.gate_array([(G.H, 3), (G.H, 5)])
    with pytest.raises(SparqcError):
        schedule_gates(4, g)          # target 5 on 4 qubits
    with pytest.raises(SparqcError):
        schedule_gates(8, g, 0)
    with pytest.raises(SparqcError):
        schedule_gates(8, g, 4)
    assert schedule_gates(8, g[:0]).size == 0


def oracle_state(g, precision=64):
    o = SparseOracle(precision)
    o.apply(g)
    out = o.state(sorted=True), o.amp_updates
    o.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [FP64, FP32])
@pytest.mark.parametrize("seed,nq,k", [(0, 20, 10), (1, 40, 12), (2, 64, 13)])
def test_state_with_schedule_equals_oracle_in_that_order(precision, seed, nq, k):
    g = circuits.random_circuit(nq, k, 400, 3, circuits.SplitMix64(circuits.stream_seed("sched-gpu", seed)))
    st = State(nq, precision=precision, schedule_gates=True)
    st.apply(g)
    got = st.state(sorted=True)
    upd = st.stats()["amp_updates"]
    st.close()
    want, wupd = oracle_state(g[schedule_gates(nq, g, 3 if precision == FP32 else 2)], precision)
    assert_identical(got, want)
    assert upd == wupd


@pytest.mark.gpu
def test_batch_with_schedule_equals_oracle_in_that_order():
    cs = circuits.batch_circuits(24, seed=5)
    b = Batch(precision=FP64, schedule_gates=True)
    b.prepare([(nq, g) for nq, _, g in cs])
    b.run()
    b.sync()
    for i, (nq, _, g) in enumerate(cs[:8]):
        want, _ = oracle_state(g[schedule_gates(nq, g, 2)])
        assert_identical(b.state(i), want)
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [FP64, FP32])
def test_server_with_schedule_equals_oracle_in_that_order(precision):
    # solo_log2_groups=6: circuits that can reach 2^6 groups run on the single-state engine
    # (three cross-group qubits per pass in FP32), the others in the pool (two)
    cs = circuits.batch_circuits(12, seed=9)
    sv = Server(precision=precision, memory_budget=int(4e9), solo_log2_groups=6, schedule_gates=True)
    rids = [sv.submit(nq, g) for nq, _, g in cs]
    results = {}
    while len(results) < len(rids):
        sv.step()
        for rid in sv.completed():
            assert sv.status(rid)[1] == 0
            results[rid] = sv.state(rid)
            sv.release(rid)
    sv.close()
    for rid, (nq, _, g) in zip(rids, cs):
        got = results[rid]
        ok = False
        for mx in ((3, 2) if precision == FP32 else (2,)):   # the order of whichever path ran it
            want, _ = oracle_state(g[schedule_gates(nq, g, mx)], precision)
            if got[0].size == want[0].size and all(np.array_equal(x, y) for x, y in zip(got, want)):
                ok = True
                break
        assert ok, f"request {rid}"
