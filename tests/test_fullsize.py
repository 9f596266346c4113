"""The benchmark configurations at their full sizes, against the oracles. GPU only.

* 40-qubit configuration (2000 gates, up to 2^20 keys) and 64-qubit configuration (500 gates,
  up to 2^26 keys), FP64: the engine's key-sorted (key, re, im) arrays equal the sparse
  oracle's (the reference's FC algorithm restated on the CPU) bit for bit, and so do the
  amp-update counts.
* 64-qubit configuration, FP32: bit for bit against the oracle run in FP32, and fidelity
  |<psi64|psi32>|^2 >= 1 - 1e-6 against the FP64 run (the FP32 amplitudes' own rounding); the
  same with the gates in scheduled order (sqc_schedule_gates), the oracle fed that order.
* batching configuration (256 circuits, one persistent launch): every member of at most 30
  qubits against the dense FP64 statevector (textbook matrices, no pruning) within
  |a - b| <= 1e-12 |b| + 1e-13 over the union of keys -- the floor covers what the 1e-14 prune
  discards and gates later mix in; every FP32 member (scheduled order, as benchmarked) at
  fidelity >= 1 - 1e-6 against FP64.
* serving configuration: a Poisson stream with large circuits, served in FP32 in scheduled
  order (as benchmarked), each result at fidelity >= 1 - 1e-6 against the plain FP64
  per-circuit path.
"""
import numpy as np
import pytest

from oracle.dense import PagedDenseOracle
from oracle.sparse import SparseOracle
from sparqc_gb300 import circuits
from sparqc_gb300.engine import Batch, Server, State, schedule_gates
from test_oracle import assert_identical

pytestmark = pytest.mark.gpu

FID = 1 - 1e-6


def oracle_run(gates, precision):
    o = SparseOracle(precision, threads=SparseOracle.max_threads())
    o.apply(gates)
    out = o.state(sorted=True), o.amp_updates
    o.close()
    return out


def engine_run(nq, gates, precision, k, schedule=False):
    st = State(nq, precision=precision, initial_buckets=1 << max(6, k - 4 + 1), schedule_gates=schedule)
    st.apply(gates)
    out = st.state(sorted=True)
    stats = st.stats()
    st.close()
    return out, stats


def fidelity(a, b):
    """|<a|b>|^2 / (<a|a><b|b>) and max |a_k - b_k| over the union of keys (absent = 0), for
    key-sorted states: a binary search pairs the common keys, so no union array is built."""
    ka, kb = a[0], b[0]
    if ka.size == 0 or kb.size == 0:
        return 0.0, float(max(np.hypot(a[1], a[2]).max(initial=0.0), np.hypot(b[1], b[2]).max(initial=0.0)))
    if ka.size == kb.size and np.array_equal(ka, kb):
        ia, hit = np.arange(ka.size), np.ones(kb.size, bool)
        ar, ai, br, bi = a[1], a[2], b[1], b[2]
    else:
        ia = np.minimum(np.searchsorted(ka, kb), ka.size - 1)
        hit = ka[ia] == kb                  # b's keys that a holds, and where
        ia = ia[hit]
        ar, ai, br, bi = a[1][ia], a[2][ia], b[1][hit], b[2][hit]
    ov_r = np.dot(br, ar) + np.dot(bi, ai)  # <b|a> over the common keys
    ov_i = np.dot(br, ai) - np.dot(bi, ar)
    na = np.dot(a[1], a[1]) + np.dot(a[2], a[2])
    nb = np.dot(b[1], b[1]) + np.dot(b[2], b[2])
    err = np.hypot(ar - br, ai - bi).max(initial=0.0)
    only_a = np.ones(ka.size, bool)
    only_a[ia] = False
    err = max(err, np.hypot(a[1][only_a], a[2][only_a]).max(initial=0.0),
              np.hypot(b[1][~hit], b[2][~hit]).max(initial=0.0))
    return float((ov_r * ov_r + ov_i * ov_i) / (na * nb)), float(err)


def assert_near_dense(got, want, rel=1e-12, floor=1e-13):
    keys = np.union1d(got[0], want[0])
    va = np.zeros(keys.size, np.complex128)
    vb = np.zeros(keys.size, np.complex128)
    va[np.searchsorted(keys, got[0])] = got[1] + 1j * got[2]
    vb[np.searchsorted(keys, want[0])] = want[1] + 1j * want[2]
    err = np.abs(va - vb)
    assert np.all(err <= rel * np.abs(vb) + floor), f"max err {err.max():.3e}"


def test_config2_full_bitexact():
    nq, g = circuits.config_circuit("c2", 0)
    want, upd = oracle_run(g, 64)
    got, stats = engine_run(nq, g, 64, 20)
    assert 0 < got[0].size <= 1 << 20
    assert_identical(got, want)
    assert stats["amp_updates"] == upd


@pytest.fixture(scope="module")
def c3():
    nq, g = circuits.config_circuit("c3", 0)
    return nq, g


@pytest.fixture(scope="module")
def c3_fp64(c3):
    nq, g = c3
    return engine_run(nq, g, 64, 26)


def test_config3_full_fp64_bitexact(c3, c3_fp64):
    nq, g = c3
    want, upd = oracle_run(g, 64)
    got, stats = c3_fp64
    assert got[0].size > 1 << 24 and stats["buckets"] > 1 << 20   # the staged (large-table) passes ran
    assert_identical(got, want)
    assert stats["amp_updates"] == upd


def test_config3_full_fp32_bitexact_and_fidelity(c3, c3_fp64):
    nq, g = c3
    got, stats = engine_run(nq, g, 32, 26)
    want, upd = oracle_run(g, 32)
    assert_identical(got, want)
    assert stats["amp_updates"] == upd
    f, err = fidelity(got, c3_fp64[0])
    print(f"64-qubit configuration FP32 vs FP64: fidelity 1 - {1 - f:.3e}, max abs err {err:.3e}")
    assert f >= FID and err < 1e-5


def test_config3_scheduled_fp32_bitexact_and_fidelity(c3, c3_fp64):
    # gates in sqc_schedule_gates order (octet passes): the oracle fed that order agrees bit for
    # bit; against the FP64 run in the given order, the usual FP32 fidelity
    nq, g = c3
    got, stats = engine_run(nq, g, 32, 26, schedule=True)
    want, upd = oracle_run(g[schedule_gates(nq, g, 3)], 32)
    assert_identical(got, want)
    assert stats["amp_updates"] == upd
    f, err = fidelity(got, c3_fp64[0])
    print(f"64-qubit configuration, scheduled FP32 vs FP64 in order: fidelity 1 - {1 - f:.3e}, max abs err {err:.3e}")
    assert f >= FID and err < 1e-5


def test_config4_members_against_dense_and_fp32_fidelity():
    cs = circuits.batch_circuits(256, seed=0)
    b64 = Batch(precision=64)
    b64.prepare([(nq, g) for nq, _, g in cs])
    b64.run()
    b64.sync()
    b32 = Batch(precision=32, schedule_gates=True)   # the batching configuration as benchmarked
    b32.prepare([(nq, g) for nq, _, g in cs])
    b32.run()
    b32.sync()
    dense_checked, fids, errs = 0, [], []
    for i, (nq, k, g) in enumerate(cs):
        s64 = b64.state(i)
        if nq <= 30:
            d = PagedDenseOracle(nq)
            d.apply(g)
            assert_near_dense(s64, d.state(threshold=1e-30))
            d.close()
            dense_checked += 1
        f, e = fidelity(b32.state(i), s64)
        fids.append(f)
        errs.append(e)
    b64.close()
    b32.close()
    print(f"batch: {dense_checked} members <= 30 qubits against the dense statevector; FP32 min fidelity "
          f"1 - {1 - min(fids):.3e}, max abs err {max(errs):.3e}")
    assert dense_checked >= 100 and min(fids) >= FID


def test_config5_served_fp32_against_plain_fp64():
    reqs = circuits.serving_stream(48, 1000.0, seed=3, large_fraction=0.1)
    assert any(r[2] == 24 for r in reqs)
    sv = Server(precision=32, memory_budget=int(120e9), slice_ms=2.0, schedule_gates=True)   # as benchmarked
    rids = {sv.submit(r[1], r[3]): j for j, r in enumerate(reqs)}
    results = {}
    while len(results) < len(reqs):
        sv.step()
        for rid in sv.completed():
            assert sv.status(rid)[1] == 0
            results[rids[rid]] = sv.state(rid)
            sv.release(rid)
    sv.close()
    fids, errs = [], []
    for j, (_, nq, k, g) in enumerate(reqs):
        ref = State(nq, precision=64)
        ref.apply(g)
        f, e = fidelity(results[j], ref.state(sorted=True))
        ref.close()
        fids.append(f)
        errs.append(e)
    print(f"served FP32 vs plain FP64: {len(reqs)} circuits ({sum(1 for r in reqs if r[2] == 24)} large), "
          f"min fidelity 1 - {1 - min(fids):.3e}, max abs err {max(errs):.3e}")
    assert min(fids) >= FID
