"""The oracle itself: pinned to the reference's own kernels and to an independent dense FP64
statevector. CPU only."""
import os
import platform

import numpy as np
import pytest

from oracle import refemu
from oracle.dense import DenseOracle
from oracle.sparse import SparseOracle
from sparqc_gb300 import circuits, gates as G

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_fc.npz")
THR = 1e-14
REL = 1e-12


def drop_negligible(state, thr=THR):
    k, r, i = state
    keep = ~((np.abs(r) < thr) & (np.abs(i) < thr))
    return k[keep], r[keep], i[keep]


def assert_close(a, b, rel=REL, floor=THR):
    """Equal key sets; amplitudes |a-b| <= rel*|b| + floor (floor = the prune threshold)."""
    ka, ra, ia = a
    kb, rb, ib = b
    assert ka.shape == kb.shape and np.array_equal(ka, kb), f"key sets differ: {ka.size} vs {kb.size}"
    za, zb = ra + 1j * ia, rb + 1j * ib
    err = np.abs(za - zb)
    assert np.all(err <= rel * np.abs(zb) + floor), f"max err {err.max():.3e}"


def assert_identical(a, b):
    for x, y, name in zip(a, b, ("keys", "re", "im")):
        assert x.shape == y.shape and np.array_equal(x, y), f"{name} differ"


def golden_cases():
    d = np.load(GOLDEN)
    names = sorted({k.split("/")[0] for k in d.files})
    return d, names


def test_golden_fixtures_present():
    d, names = golden_cases()
    assert "hn" in names and any(n.startswith("kat_") for n in names) and any(n.startswith("rnd_") for n in names)


@pytest.mark.parametrize("name", golden_cases()[1])
def test_oracle_matches_reference_golden(name):
    """The restatement reproduces the reference kernels' output for every golden circuit."""
    d, _ = golden_cases()
    o = SparseOracle()
    o.apply(d[f"{name}/gates"])
    got = drop_negligible(o.state())
    want = (d[f"{name}/keys"], d[f"{name}/re"], d[f"{name}/im"])
    if platform.machine() in ("x86_64", "AMD64"):
        assert_identical(got, want)   # fixtures were made on x86-64: bit-exact
    else:
        assert_close(got, want)       # another libm may round a cos/sin differently


def test_hn_uniform():
    """H on every qubit gives the uniform state 2^(-n/2) (the reference's own workload)."""
    o = SparseOracle()
    o.apply(G.gate_array([(G.H, q) for q in range(10)]))
    k, r, i = o.state()
    assert np.array_equal(k, np.arange(1024, dtype=np.uint64))
    assert np.allclose(r, 2 ** -5, rtol=0, atol=1e-15) and np.all(i == 0)


def test_hh_cancels_and_prunes():
    o = SparseOracle()
    o.apply(G.gate_array([(G.H, 0), (G.H, 1), (G.H, 1), (G.H, 0)]))
    k, r, i = o.state()
    assert k.tolist() == [0] and r[0] == pytest.approx(1.0, abs=1e-15)


def test_rx_pi_is_minus_i_x():
    o = SparseOracle()
    o.apply(G.gate_array([(G.RX, 3, 0, np.pi)]))
    k, r, i = o.state()
    k, r, i = drop_negligible((k, r, i))
    assert k.tolist() == [8] and abs(r[0]) < 1e-15 and i[0] == pytest.approx(-1.0)


@pytest.mark.parametrize("seed", range(6))
def test_oracle_vs_dense_all_gates(seed):
    """Every gate kind, with controls, against textbook matrices on a dense vector."""
    rng = circuits.SplitMix64(circuits.stream_seed("dense", seed))
    nq, k = 12, 7
    g = circuits.random_circuit(nq, k, 200, 3, rng,
                                kinds=((G.Z, G.S, G.SDG, G.T, G.TDG, G.RZ, G.PHASE), (G.X, G.Y),
                                       (G.H, G.RX, G.RY, G.U)))
    o = SparseOracle()
    o.apply(g)
    d = DenseOracle(nq)
    d.apply(g)
    assert_close(drop_negligible(o.state()), d.state())


def test_oracle_fp32_fidelity():
    nq, g = circuits.config_circuit("c1", 0)
    a, b = SparseOracle(64), SparseOracle(32)
    a.apply(g)
    b.apply(g)
    ka, ra, ia = a.state()
    kb, rb, ib = b.state()
    za = dict(zip(ka.tolist(), ra + 1j * ia))
    zb = dict(zip(kb.tolist(), rb + 1j * ib))
    keys = set(za) | set(zb)
    ov = sum(np.conj(za.get(x, 0)) * zb.get(x, 0) for x in keys)
    fid = abs(ov) ** 2 / (sum(abs(v) ** 2 for v in za.values()) * sum(abs(v) ** 2 for v in zb.values()))
    assert fid >= 1 - 1e-6


def test_amp_updates_counts_input_nonzeros():
    o = SparseOracle()
    o.apply(G.gate_array([(G.H, 0), (G.H, 1), (G.Z, 0)]))
    assert o.amp_updates == 1 + 2 + 4


def test_empty_state_stays_empty():
    o = SparseOracle()
    o.set_state(np.zeros(0, np.uint64), np.zeros(0), np.zeros(0))
    o.apply(G.gate_array([(G.H, 0), (G.X, 5), (G.RY, 2, 0, 0.3)]))
    assert o.nnz == 0


def test_64_qubit_keys():
    o = SparseOracle()
    o.set_state(np.array([1 << 63], np.uint64), np.array([1.0]), np.array([0.0]))
    o.apply(G.gate_array([(G.H, 63), (G.X, 0, 1 << 62), (G.X, 62)]))
    k, r, i = o.state()
    assert sorted(k.tolist()) == [1 << 62, (1 << 63) | (1 << 62)]


def test_duplicate_keys_rejected():
    o = SparseOracle()
    with pytest.raises(ValueError):
        o.set_state(np.array([5, 5], np.uint64), np.ones(2), np.zeros(2))


@pytest.mark.skipif(not refemu.available(), reason="reference sources not present")
@pytest.mark.parametrize("seed", range(4))
def test_oracle_vs_reference_kernels_fresh(seed):
    """Fresh random circuits of the reference gate set (no Rx/Ry race), run through the
    reference's own kernels compiled for the host: bit-exact."""
    import sys
    sys.path.insert(0, os.path.dirname(GOLDEN))
    from make_golden import hazard_free_circuit
    nq = 8 + seed % 3
    g = hazard_free_circuit(nq, 4 + seed % 3, 120, 1000 + seed)
    rk, rr, ri, hz = refemu.run(nq, g)
    assert not hz
    o = SparseOracle()
    o.apply(g)
    assert_identical(drop_negligible(o.state()), (rk, rr, ri))


@pytest.mark.skipif(not refemu.available(), reason="reference sources not present")
def test_reference_rxry_race_breaks_its_address_book():
    """The reference's gate_sq_par writes the skip-path address-book entry for Rx/Ry too
    (emulator/device/device_table_FC.cuh:190-193), colliding with the atomic appends of
    update_ah_sup. With both pair members present, entries are lost and the state's norm
    drops below 1. The engine and the oracle follow the guarded rule gate_sq uses for H
    (device_table_FC.cuh:133-137), which keeps the norm."""
    g = G.gate_array([(G.H, q) for q in range(4)] + [(G.RX, 0, 0, 0.7), (G.RY, 2, 0, 1.1), (G.RX, 1, 0, 0.4)] * 3)
    rk, rr, ri, hz = refemu.run(6, g)
    assert hz, "expected the race to be reported"
    assert abs(np.sum(rr ** 2 + ri ** 2) - 1.0) > 0.1
    o = SparseOracle()
    o.apply(g)
    assert o.nnz == 16 and o.norm2() == pytest.approx(1.0, abs=1e-13)


ALL_KINDS = ((G.Z, G.S, G.SDG, G.T, G.TDG, G.RZ, G.PHASE), (G.X, G.Y), (G.H, G.RX, G.RY, G.U))


@pytest.mark.parametrize("seed", range(3))
def test_paged_dense_equals_numpy_dense(seed):
    """The paged C statevector applies the same textbook matrices as the numpy one."""
    from oracle.dense import PagedDenseOracle
    rng = circuits.SplitMix64(circuits.stream_seed("paged", seed))
    g = circuits.random_circuit(13, 9, 200, 3, rng, kinds=ALL_KINDS)
    a = DenseOracle(13)
    a.apply(g)
    b = PagedDenseOracle(13)
    b.apply(g)
    assert_close(b.state(), a.state(), rel=1e-13, floor=1e-15)


def test_paged_dense_30_qubits_against_sparse():
    """A 30-qubit circuit of the batching configuration's kind: the dense statevector and the
    sparse restatement agree within the tolerance (the latter prunes at 1e-14)."""
    from oracle.dense import PagedDenseOracle
    rng = circuits.SplitMix64(circuits.stream_seed("paged30"))
    g = circuits.random_circuit(30, 14, 400, 3, rng)
    d = PagedDenseOracle(30)
    d.apply(g)
    o = SparseOracle(threads=SparseOracle.max_threads())
    o.apply(g)
    assert_close(drop_negligible(o.state()), d.state())
