"""States larger than the device budget (the reference's "PC" mode, described in
emulator/device/device_data.cuh:20-23 and never built there). GPU only.

A partitioned state with a small device budget must spill to host memory, run the rest of the
circuit partition by partition, and still give bit for bit the state that one table gives: the
oracle's in FP64, the single-table engine's in FP32.
"""
import numpy as np
import pytest

from oracle.sparse import SparseOracle
from sparqc_gb300 import circuits, gates as G
from sparqc_gb300.engine import FP32, FP64, PartState, State
from test_oracle import assert_identical

pytestmark = pytest.mark.gpu


def _circuit(nq, k, depth, seed):
    return circuits.random_circuit(nq, k, depth, 2, circuits.SplitMix64(circuits.stream_seed("part", seed)))


@pytest.mark.parametrize("precision", [FP64, FP32])
def test_spilled_state_matches_one_table(precision):
    nq, k = 30, 14
    g = _circuit(nq, k, 400, 1)
    ps = PartState(nq, device_bytes=160 << 10, precision=precision)
    ps.apply(g)
    got = ps.state(sorted=True)
    if precision == FP64:
        o = SparseOracle()
        o.apply(g)
        want = o.state(sorted=True)
    else:
        st = State(nq, precision=FP32)
        st.apply(g)
        want = st.state(sorted=True)
    assert_identical(got, want)
    s = ps.stats()
    assert s["spills"] >= 1 and s["windows"] >= 2
    assert s["max_bin_keys"] < got[0].size      # no partition held the whole state
    assert s["bytes_h2d"] > 0 and s["bytes_d2h"] > 0
    assert ps.nnz == got[0].size
    # the negligible filter and the unsorted readout agree with the sorted one
    ks, rs, is_ = ps.state(sorted=False)
    order = np.argsort(ks)
    assert_identical((ks[order], rs[order], is_[order]), got)
    kd, _, _ = ps.state(sorted=True, drop_negligible=True)
    keep = ~((np.abs(got[1]) < 1e-14) & (np.abs(got[2]) < 1e-14))
    assert np.array_equal(kd, got[0][keep])


def test_partitions_split_when_they_outgrow_the_device():
    # CX copies qubits 4..7 into 11..14, so H gates on 11..14 double the keys although those
    # qubits already vary. Rx on 8 and 9 (no growth) end the first window early, so the H gates
    # on 12..14 share a window whose partitions start small for a state that does not grow,
    # outgrow the 60 KB table inside it and are split at the pass that cannot grow.
    nq = 24
    g = G.gate_array([(G.H, q, ()) for q in range(4, 10)] + [(G.X, 7 + q, (q,)) for q in range(4, 8)] +
                     [(G.RX, 8, (), 0.3), (G.RX, 9, (), 1.1)] +
                     [(G.H, q, ()) for q in range(11, 15)] + [(G.RZ, 12, (), 0.7), (G.PHASE, 5, (11,), 0.4)])
    ps = PartState(nq, device_bytes=60 << 10)
    ps.apply(g)
    got = ps.state(sorted=True)
    o = SparseOracle()
    o.apply(g)
    assert_identical(got, o.state(sorted=True))
    assert got[0].size == 1024
    s = ps.stats()
    assert s["spills"] >= 1 and s["splits"] >= 1
    # a random circuit under the same budget
    g2 = _circuit(nq, 13, 300, 2)
    ps.set_zero()
    ps.apply(g2)
    o2 = SparseOracle()
    o2.apply(g2)
    assert_identical(ps.state(sorted=True), o2.state(sorted=True))


def test_large_budget_stays_on_the_device_and_resets():
    nq, k = 30, 12
    g = _circuit(nq, k, 300, 3)
    ps = PartState(nq)   # the HBM budget
    ps.apply(g)
    o = SparseOracle()
    o.apply(g)
    assert_identical(ps.state(sorted=True), o.state(sorted=True))
    s = ps.stats()
    assert s["spills"] == 0 and s["spilled"] == 0 and s["amp_updates"] > 0
    ps.set_zero()
    k0, r0, i0 = ps.state()
    assert k0.tolist() == [0] and r0.tolist() == [1.0] and i0.tolist() == [0.0]


def test_spilled_state_returns_to_the_device_when_it_shrinks():
    # grow past the budget, then undo the branching: the state shrinks back to one key
    nq = 20
    hs = [(G.H, q, ()) for q in range(14)]
    g = G.gate_array(hs + [(G.RZ, 7, (), 0.3)] + [(G.RZ, 7, (), -0.3)] + list(reversed(hs)))
    ps = PartState(nq, device_bytes=100 << 10)
    ps.apply(g)
    keys, re, im = ps.state(sorted=True, drop_negligible=True)
    o = SparseOracle()
    o.apply(g)
    assert_identical(ps.state(sorted=True), o.state(sorted=True))
    assert keys.tolist() == [0]
    s = ps.stats()
    assert s["spills"] >= 1 and s["returns"] >= 1 and s["spilled"] == 0
