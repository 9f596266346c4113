"""SWAP and state snapshots. GPU only.

SWAP is three controlled X gates, so it must equal those gates applied by the oracle bit for
bit. A snapshot written and loaded back must give the same state bits, and continuing a
circuit from a reloaded snapshot must give the same bits as running it straight through.
"""
import numpy as np
import pytest

from oracle.sparse import SparseOracle
from sparqc_gb300 import circuits, gates as G
from sparqc_gb300.engine import ERR_ARG, SparqcError, State
from test_oracle import assert_identical

pytestmark = pytest.mark.gpu


def _circuit(nq, k, depth, seed):
    return circuits.random_circuit(nq, k, depth, 2, circuits.SplitMix64(circuits.stream_seed("snap", seed)))


def test_swap_is_three_cnots():
    g = _circuit(24, 10, 120, 1)
    st = State(24)
    st.apply(g)
    for a, b in [(0, 9), (3, 20), (15, 2)]:
        st.swap(a, b)
    o = SparseOracle()
    o.apply(g)
    cx = []
    for a, b in [(0, 9), (3, 20), (15, 2)]:
        cx += [(G.X, b, (a,)), (G.X, a, (b,)), (G.X, b, (a,))]
    o.apply(G.gate_array(cx))
    assert_identical(st.state(sorted=True), o.state(sorted=True))
    with pytest.raises(SparqcError) as e:
        st.swap(3, 3)
    assert e.value.code == ERR_ARG


@pytest.mark.parametrize("precision", [64, 32])
def test_snapshot_round_trip_and_restart(tmp_path, precision):
    g = _circuit(40, 14, 300, 2)
    half = g.size // 2
    straight = State(40, precision=precision)
    straight.apply(g)
    want = straight.state(sorted=True)

    first = State(40, precision=precision)
    first.apply(g[:half])
    path = tmp_path / "state.sqc"
    first.save(path)
    before = first.state(sorted=True)
    second = State(40, precision=precision)
    second.load(path)
    assert_identical(second.state(sorted=True), before)
    second.apply(g[half:])
    assert_identical(second.state(sorted=True), want)

    wrong = State(20)
    with pytest.raises(SparqcError):
        wrong.load(path)
    bad = tmp_path / "bad.sqc"
    bad.write_bytes(b"not a snapshot")
    with pytest.raises(SparqcError):
        second.load(bad)
