"""Failure paths, made to fire without faulting the GPU. GPU only.

* The persistent batch kernel's bounded idle wait: with a 1 us limit its idle warps give up at
  once, the run reports SQC_ERR_STATE ("found no work for too long"), and a batch with the
  default limit then gives the oracle's results.
* The probe limit of bucket claims: groups whose keys all hash to one home bucket (built with
  the inverse of the table's hash) make a claim walk past the limit; set_state reports
  SQC_ERR_TABLE_FULL, and the state then works normally.
* Allocation failures injected on the host into the serving loop's admissions (pool placement
  and a large circuit's own tables): each step that hits one reports SQC_ERR_OOM and the
  request stays queued; afterwards every request completes with its alone result and nothing
  is left held.
"""
import numpy as np
import pytest

from oracle.sparse import SparseOracle
from sparqc_gb300 import circuits
from sparqc_gb300.engine import (ERR_OOM, ERR_STATE, ERR_TABLE_FULL, Batch, Server, SparqcError, State)
from test_oracle import assert_identical

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def oracle(gates):
    o = SparseOracle()
    o.apply(gates)
    return o.state(sorted=True)


def test_batch_idle_limit_reports_timeout_and_a_new_run_recovers():
    cs = [(24, circuits.random_circuit(24, 14, 300, 2, circuits.SplitMix64(circuits.stream_seed("idle", i))))
          for i in range(2)]
    b = Batch(idle_limit_us=1)
    b.prepare(cs)
    b.run()
    with pytest.raises(SparqcError) as e:
        b.sync()
    assert e.value.code == ERR_STATE and "no work" in str(e.value)
    b.close()
    ok = Batch()
    ok.prepare(cs)
    ok.run()
    ok.sync()
    for i, (_, g) in enumerate(cs):
        assert_identical(ok.state(i), oracle(g))
    ok.close()


def _unmix64(h):
    """Inverse of the table's hash (splitmix64's finalizer)."""
    def unxorshift(x, s):
        y = x
        for _ in range(64 // s + 1):
            y = x ^ (y >> s)
        return y & M64
    x = unxorshift(h, 31)
    x = (x * pow(0x94d049bb133111eb, -1, 1 << 64)) & M64
    x = unxorshift(x, 27)
    x = (x * pow(0xbf58476d1ce4e5b9, -1, 1 << 64)) & M64
    return unxorshift(x, 30)


def _mix64(x):
    x ^= x >> 30
    x = (x * 0xbf58476d1ce4e5b9) & M64
    x ^= x >> 27
    x = (x * 0x94d049bb133111eb) & M64
    return x ^ (x >> 31)


def test_probe_limit_reports_table_full_and_the_state_recovers():
    nb = 1 << 14
    groups, r = [], 0
    while len(groups) < 4200:   # more groups on one home bucket than a claim may probe (4096)
        g = _unmix64(((r << 14) | 77) & M64)
        r += 1
        if g < 1 << 60:
            assert _mix64(g) & (nb - 1) == 77
            groups.append(g)
    keys = np.array(groups, np.uint64) << np.uint64(4)
    amp = np.full(keys.size, 1.0 / np.sqrt(keys.size))
    st = State(64, initial_buckets=nb)
    with pytest.raises(SparqcError) as e:
        st.set_state(keys, amp, np.zeros(keys.size))
    assert e.value.code == ERR_TABLE_FULL
    g = circuits.random_circuit(64, 10, 200, 3, circuits.SplitMix64(5))
    st.set_zero()
    st.apply(g)
    assert_identical(st.state(sorted=True), oracle(g))
    st.close()


@pytest.mark.parametrize("solo", [False, True])
def test_server_injected_allocation_failures_leak_nothing(solo):
    reqs = [(20, circuits.random_circuit(20, 9, 150, 2, circuits.SplitMix64(circuits.stream_seed("inj", i))))
            for i in range(4)]
    # solo: every circuit of at least 2^5 groups runs on its own engine (its tables are allocated
    # at admission); otherwise each is placed in the pool
    sv = Server(inject_alloc_failures=2, solo_log2_groups=5 if solo else 0, memory_budget=1 << 30)
    rids = [sv.submit(nq, g) for nq, g in reqs]
    failures = 0
    done = {}
    for _ in range(10000):
        if len(done) == len(reqs):
            break
        try:
            sv.step()
        except SparqcError as e:
            assert e.code == ERR_OOM and "injected" in str(e)
            failures += 1
            s = sv.stats()
            assert s["running"] == 0 and s["pool_used"] == 0 and s["solo_running"] == 0
            continue
        for rid in sv.completed():
            done[rid] = sv.state(rid)
            sv.release(rid)
    assert failures == 2 and len(done) == len(reqs)
    if solo:
        assert sv.stats()["steps"] > 0
    for rid, (nq, g) in zip(rids, reqs):
        assert_identical(done[rid], oracle(g))
    s = sv.stats()
    assert s["queued"] == 0 and s["running"] == 0 and s["completed"] == 0 and s["pool_used"] == 0
    sv.close()
