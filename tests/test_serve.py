"""Serving loop (sqc_server_*): requests admitted while others run give the same result as
running each circuit alone.

Requests arrive between steps (so they join circuits already on the GPU), the time slice
is short (so long circuits park and resume many times) and the memory budget is small (so
admission waits for memory to free up). Every result is compared bit for bit, key-sorted,
against the circuit run alone through sqc_create + sqc_apply_gates. GPU only.
"""
import numpy as np
import pytest

from sparqc_gb300 import circuits, gates as G
from sparqc_gb300.engine import (ERR_BUDGET, FP32, FP64, OK, REQ_DONE, REQ_QUEUED, REQ_RUNNING, Server, SparqcError,
                                 State)

pytestmark = pytest.mark.gpu

MB = 1 << 20


def _alone(nq, gates, precision):
    st = State(nq, precision=precision)
    st.apply(gates)
    out = st.state(sorted=True)
    st.close()
    return out


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def _stream(count, seed):
    return [(nq, g) for nq, _, g in circuits.batch_circuits(count, seed=seed, qrange=(12, 40), krange=(5, 13),
                                                              drange=(20, 400), config="serve-test")]


def _serve(server, cs, per_step=3):
    """Submit per_step circuits before every step; run until all are done. Returns {index: state}."""
    ids = {}
    out = {}
    i = 0
    steps = 0
    while len(out) < len(cs):
        for _ in range(per_step):
            if i < len(cs):
                nq, g = cs[i]
                ids[server.submit(nq, g)] = i
                i += 1
        server.step()
        steps += 1
        assert server.stats()["pool_used"] <= server.stats()["pool_bytes"]
        for rid in server.completed():
            st, code = server.status(rid)
            assert st == REQ_DONE and code == OK
            out[ids[rid]] = server.state(rid)
            server.release(rid)
        assert steps < 100000
    return out, steps


@pytest.mark.parametrize("precision", [FP64, FP32])
def test_served_results_equal_alone(precision):
    cs = _stream(30, 1)
    sv = Server(precision=precision, memory_budget=256 * MB, slice_ms=0.05, max_slots=64)
    got, steps = _serve(sv, cs)
    assert steps > len(cs) // 3   # circuits really did park and resume across steps
    for i, (nq, g) in enumerate(cs):
        assert _same(got[i], _alone(nq, g, precision)), f"request {i}"
    s = sv.stats()
    assert s["pool_used"] == 0 and s["queued"] == 0 and s["running"] == 0 and s["completed"] == 0


def test_same_alone_and_in_the_mix():
    cs = _stream(24, 2)
    probe = cs[5]
    alone_sv = Server(memory_budget=64 * MB, slice_ms=0.05)
    rid = alone_sv.submit(*probe)
    while alone_sv.status(rid)[0] != REQ_DONE:
        alone_sv.step()
    alone = alone_sv.state(rid)
    alone_sv.close()
    mix_sv = Server(memory_budget=128 * MB, slice_ms=0.05)
    got, _ = _serve(mix_sv, cs, per_step=2)
    assert _same(got[5], alone)


def test_admission_waits_for_memory():
    # every circuit needs about 150 KB (a 256-bucket slice and 300 gate descriptors); the
    # budget admits only a few at once
    cs = [(30, circuits.random_circuit(30, 10, 300, 2, circuits.SplitMix64(100 + i))) for i in range(12)]
    sv = Server(memory_budget=512 << 10, slice_ms=0.05, max_slots=16)
    ids = [sv.submit(nq, g) for nq, g in cs]
    sv.step()
    states = [sv.status(r)[0] for r in ids]
    assert states[0] != REQ_QUEUED and states.count(REQ_QUEUED) > 0
    # first come, first served: nothing later in the queue runs before an earlier request
    first_q = states.index(REQ_QUEUED)
    assert all(s == REQ_QUEUED for s in states[first_q:])
    done = {}
    for _ in range(100000):
        if len(done) == len(ids):
            break
        sv.step()
        for rid in sv.completed():
            done[rid] = sv.state(rid)
            sv.release(rid)
    for rid, (nq, g) in zip(ids, cs):
        assert _same(done[rid], _alone(nq, g, FP64))


def test_server_rejects_what_can_never_fit():
    sv = Server(memory_budget=4 * MB)
    with pytest.raises(SparqcError) as e:
        sv.submit(40, G.gate_array([(G.H, q) for q in range(20)]))
    assert e.value.code == ERR_BUDGET
    rid = sv.submit(10, G.gate_array([(G.H, 0)]))
    with pytest.raises(SparqcError):
        sv.state(rid)   # not completed yet
    sv.step()
    assert sv.status(rid)[0] == REQ_DONE
    k, r, _ = sv.state(rid)
    assert k.tolist() == [0, 1] and np.allclose(r, [2 ** -0.5] * 2)


@pytest.mark.parametrize("precision", [FP64, FP32])
def test_large_requests_run_alone_with_the_same_result(precision):
    # circuits that can hold 2^6 groups or more run on their own engine, a slice of gates per
    # step, beside the small ones in the persistent kernel
    cs = _stream(16, 3)
    big = [(30, circuits.random_circuit(30, 16, 300, 2, circuits.SplitMix64(900 + i))) for i in range(3)]
    mix = cs[:6] + big[:1] + cs[6:12] + big[1:] + cs[12:]
    sv = Server(precision=precision, memory_budget=512 * MB, slice_ms=0.2, solo_log2_groups=6, solo_share_pct=50)
    got, steps = _serve(sv, mix, per_step=2)
    assert steps > 5
    for i, (nq, g) in enumerate(mix):
        assert _same(got[i], _alone(nq, g, precision)), f"request {i}"
    s = sv.stats()
    assert s["pool_used"] == 0 and s["solo_running"] == 0


@pytest.mark.parametrize("precision", [FP64, FP32])
def test_overlapped_steps_give_the_same_results(precision):
    # overlap_steps: a step returns with its slice in flight and the next one retires it, so the
    # submits, reads and releases between steps run while the device works; large circuits run
    # alone (and their engines are kept for the next of the same shape), small ones in the pool
    cs = _stream(16, 5)
    big = [(30, circuits.random_circuit(30, 16, 300, 2, circuits.SplitMix64(950 + i))) for i in range(3)]
    mix = cs[:5] + big[:1] + cs[5:11] + big[1:] + cs[11:]
    sv = Server(precision=precision, memory_budget=512 * MB, slice_ms=0.2, solo_log2_groups=6, solo_share_pct=50,
                overlap_steps=True)
    got, steps = _serve(sv, mix, per_step=2)
    assert steps > 5
    for i, (nq, g) in enumerate(mix):
        assert _same(got[i], _alone(nq, g, precision)), f"request {i}"
    s = sv.stats()
    assert s["pool_used"] == 0 and s["solo_running"] == 0 and s["running"] == 0
    sv.close()
