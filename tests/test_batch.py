"""Many-circuit batch (sqc_batch_*): every circuit's result equals running it alone.

The batch plans each circuit exactly as a single state does and runs the same per-slot
code, so results are compared bit for bit (keys, real and imaginary parts, key-sorted)
against sqc_create + sqc_apply_gates on the same circuit, in FP64 and FP32, and a few
members against the CPU oracle. GPU only.
"""
import numpy as np
import pytest

from sparqc_gb300 import circuits, gates as G
from sparqc_gb300.engine import ERR_ARG, ERR_BUDGET, FP32, FP64, Batch, SparqcError, State

pytestmark = pytest.mark.gpu


def _alone(nq, gates, precision):
    st = State(nq, precision=precision)
    st.apply(gates)
    out = st.state(sorted=True)
    st.close()
    return out


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def _mixed(count, seed, qrange=(12, 40), krange=(5, 12), drange=(20, 300)):
    return [(nq, g) for nq, _, g in circuits.batch_circuits(count, seed=seed, qrange=qrange, krange=krange,
                                                              drange=drange, config="batch-test")]


@pytest.mark.parametrize("precision", [FP64, FP32])
def test_batch_matches_each_circuit_alone(precision):
    cs = _mixed(40, 1)
    b = Batch(precision=precision)
    b.prepare(cs)
    b.run()
    b.sync()
    for i, (nq, g) in enumerate(cs):
        assert _same(b.state(i), _alone(nq, g, precision)), f"circuit {i}"
    b.close()


@pytest.mark.parametrize("precision", [FP64, FP32])
def test_batch_readout_of_every_circuit_in_one_call(precision):
    cs = _mixed(30, 5)
    b = Batch(precision=precision)
    b.prepare(cs)
    b.run()
    b.sync()
    sorted_all = b.states(sorted=True)
    assert len(sorted_all) == len(cs)
    for i in range(len(cs)):
        assert _same(sorted_all[i], b.state(i)), f"circuit {i}"
    # unsorted: the same entries per circuit; dropping negligible entries as get_state does
    for i, (k, r, im) in enumerate(b.states()):
        order = np.argsort(k)
        assert _same((k[order], r[order], im[order]), b.state(i)), f"circuit {i}"
    for i, got in enumerate(b.states(sorted=True, drop_negligible=True)):
        assert _same(got, b.state(i, drop_negligible=True)), f"circuit {i}"
    b.close()


def test_batch_matches_oracle():
    from oracle.sparse import SparseOracle
    cs = _mixed(6, 2, qrange=(10, 30), krange=(4, 10), drange=(50, 150))
    b = Batch()
    b.prepare(cs)
    b.run()
    b.sync()
    for i, (nq, g) in enumerate(cs):
        o = SparseOracle()
        o.apply(g)
        want = o.state()
        assert _same(b.state(i), want), f"circuit {i}"


def test_batch_repeat_runs_and_graph_replay():
    cs = _mixed(16, 3)
    b = Batch(use_graph=True)
    b.prepare(cs)
    first = []
    for r in range(3):
        b.run()
        b.sync()
        got = [b.state(i) for i in range(len(cs))]
        if r == 0:
            first = got
        else:
            assert all(_same(x, y) for x, y in zip(got, first))
    s = b.stats()
    assert s["circuits"] == len(cs) and s["passes"] > 0 and s["amp_updates"] > 0 and s["last_run_ms"] > 0


def test_batch_c4_configuration_bit_exact():
    # the batching configuration: 256 circuits, 16-48 qubits, k 8-18, depth 100-1000
    cs = [(nq, g) for nq, _, g in circuits.batch_circuits(256, seed=0)]
    b = Batch()
    b.prepare(cs)
    b.run()
    b.sync()
    for i in (0, 1, 7, 100, 255) + tuple(range(2, 256, 23)):
        nq, g = cs[i]
        st = State(nq)
        st.apply(g)
        want = st.state(sorted=True)
        st.close()
        assert _same(b.state(i), want), f"circuit {i}"
    # the amp-update count of the whole batch equals the sum over circuits run alone
    total = 0
    for nq, g in cs[:32]:
        st = State(nq)
        st.apply(g)
        st.sync()
        total += st.stats()["amp_updates"]
        st.close()
    b32 = Batch()
    b32.prepare(cs[:32])
    b32.run()
    b32.sync()
    assert b32.stats()["amp_updates"] == total


def test_batch_autotune_keeps_results():
    cs = _mixed(12, 4)
    b = Batch()
    b.prepare(cs)
    b.run()
    b.sync()
    before = [b.state(i) for i in range(len(cs))]
    t = b.autotune()
    assert t["candidates"] > 1 and t["best_ms"] > 0 and t["best_ms"] <= t["default_ms"]
    assert t["min_chunk"] in (4, 8, 16, 32) and t["load_factor"] in (0.45, 0.25)
    assert t["threads_per_unit"] in (16, 32)
    after = [b.state(i) for i in range(len(cs))]
    assert all(_same(x, y) for x, y in zip(before, after))


@pytest.mark.parametrize("precision", [FP64, FP32])
def test_batch_threads_per_unit_keeps_results(precision):
    """Pair units on half-warps (16 threads, one qubit >= 4 per pass) and quad units on whole
    warps (32 threads, two per pass) give the same bits, and those of each circuit alone."""
    cs = _mixed(10, 7)
    out = {}
    for tpu in (16, 32):
        b = Batch(precision=precision, threads_per_unit=tpu)
        b.prepare(cs)
        b.run()
        b.sync()
        out[tpu] = ([b.state(i) for i in range(len(cs))], b.stats()["passes"])
        b.close()
    assert all(_same(x, y) for x, y in zip(out[16][0], out[32][0]))
    assert out[16][1] > out[32][1]
    for i, (nq, g) in enumerate(cs):
        assert _same(out[16][0][i], _alone(nq, g, precision))


def test_batch_edge_circuits():
    # no gates; gates the host resolves entirely (uncontrolled X relabels keys); 64 qubits;
    # a 1-qubit register
    cs = [(8, G.gate_array([])),
          (20, G.gate_array([(G.X, q) for q in (0, 5, 19)])),
          (64, G.gate_array([(G.H, 63), (G.X, 62), (G.H, 0), (G.RZ, 63, (), 0.3), (G.Y, 2, (63,))])),
          (1, G.gate_array([(G.H, 0), (G.T, 0), (G.H, 0)]))]
    b = Batch()
    b.prepare(cs)
    b.run()
    b.sync()
    for i, (nq, g) in enumerate(cs):
        assert _same(b.state(i), _alone(nq, g, FP64)), f"circuit {i}"
    k, r, _ = b.state(1)
    assert k.tolist() == [(1 << 0) | (1 << 5) | (1 << 19)] and r.tolist() == [1.0]


def test_batch_errors():
    b = Batch(memory_budget=1 << 20)
    with pytest.raises(SparqcError) as e:
        b.prepare([(40, G.gate_array([(G.H, q) for q in range(24)]))])
    assert e.value.code == ERR_BUDGET
    b2 = Batch()
    with pytest.raises(SparqcError) as e:
        b2.prepare([(4, G.gate_array([(G.H, 4)]))])
    assert e.value.code == ERR_ARG
    with pytest.raises(SparqcError):
        Batch(load_factor=0.9)
