"""Parity of the CUDA engine with the oracle, through the C ABI. GPU only.

With equal precision the engine and the oracle execute the same roundings, so states are
compared bit for bit (keys, real and imaginary parts). Against the golden fixtures (made on
another machine's libm) and the dense statevector the tolerance is 1e-12 relative with a
1e-14 absolute floor (the prune threshold). FP32 states are checked by fidelity >= 1 - 1e-6
against FP64.
"""
import os

import numpy as np
import pytest

from oracle.dense import DenseOracle
from oracle.sparse import SparseOracle
from sparqc_gb300 import circuits, gates as G
from sparqc_gb300.engine import State, SparqcError, ERR_ARG
from test_oracle import assert_close, assert_identical, drop_negligible, golden_cases

pytestmark = pytest.mark.gpu

ALL_KINDS = ((G.Z, G.S, G.SDG, G.T, G.TDG, G.RZ, G.PHASE), (G.X, G.Y), (G.H, G.RX, G.RY, G.U))


def run_gpu(nq, gates, precision=64, initial_buckets=64, init=None, **kw):
    st = State(nq, precision=precision, initial_buckets=initial_buckets, **kw)
    if init is not None:
        st.set_state(*init)
    st.apply(gates)
    out = st.state(sorted=True)
    stats = st.stats()
    st.close()
    return out, stats


def run_oracle(gates, precision=64, init=None):
    o = SparseOracle(precision)
    if init is not None:
        o.set_state(*init)
    o.apply(gates)
    return o.state(sorted=True), o.amp_updates


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("precision", [64, 32])
def test_random_circuits_bitexact(seed, precision):
    rng = circuits.SplitMix64(circuits.stream_seed("gpu", seed))
    nq = (6, 10, 16, 24, 40, 64)[seed % 6]
    k = min(nq, 5 + seed % 7)
    g = circuits.random_circuit(nq, k, 300, 3, rng, kinds=ALL_KINDS)
    got, stats = run_gpu(nq, g, precision)
    want, upd = run_oracle(g, precision)
    assert_identical(got, want)
    assert stats["amp_updates"] == upd


STAGED_BUCKETS = 1 << 21   # tables above 2^20 buckets take the staged (cp.async pipelined) passes


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("precision", [64, 32])
def test_random_circuits_bitexact_staged_path(seed, precision):
    rng = circuits.SplitMix64(circuits.stream_seed("gpu-staged", seed))
    nq = (12, 20, 30, 44, 64, 64)[seed]
    k = min(nq, 8 + seed)
    g = circuits.random_circuit(nq, k, 250, 3, rng, kinds=ALL_KINDS)
    got, stats = run_gpu(nq, g, precision, initial_buckets=STAGED_BUCKETS)
    want, upd = run_oracle(g, precision)
    assert_identical(got, want)
    assert stats["amp_updates"] == upd


@pytest.mark.parametrize("buckets", [64, STAGED_BUCKETS])
@pytest.mark.parametrize("precision", [64, 32])
def test_pair_and_quad_passes_agree(buckets, precision):
    """Passes pairing across one, two or three high qubits give the same bits as each other and
    as the oracle, on the direct (small table) and the staged (large table) kernels."""
    rng = circuits.SplitMix64(circuits.stream_seed("quad", buckets, precision))
    g = circuits.random_circuit(36, 11, 400, 2, rng, kinds=ALL_KINDS)
    got1, s1 = run_gpu(36, g, precision, initial_buckets=buckets, max_cross_qubits=1)
    got2, s2 = run_gpu(36, g, precision, initial_buckets=buckets, max_cross_qubits=2)
    got3, s3 = run_gpu(36, g, precision, initial_buckets=buckets, max_cross_qubits=3)
    want, upd = run_oracle(g, precision)
    assert_identical(got1, want)
    assert_identical(got2, want)
    assert_identical(got3, want)
    assert s1["amp_updates"] == s2["amp_updates"] == s3["amp_updates"] == upd
    assert s3["passes"] < s2["passes"] < s1["passes"]


@pytest.mark.parametrize("buckets", [64, STAGED_BUCKETS])
@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("precision", [64, 32])
def test_octet_passes_bitexact(seed, precision, buckets):
    """Passes over three high qubits (eight groups per unit, four slots per lane) against the
    oracle, with every gate kind, controls and growth, on the direct and the staged kernels."""
    rng = circuits.SplitMix64(circuits.stream_seed("octet", seed, precision))
    nq = (14, 24, 40, 64)[seed]
    g = circuits.random_circuit(nq, min(nq, 9 + 2 * seed), 300, 3, rng, kinds=ALL_KINDS)
    got, stats = run_gpu(nq, g, precision, initial_buckets=buckets, max_cross_qubits=3)
    want, upd = run_oracle(g, precision)
    assert_identical(got, want)
    assert stats["amp_updates"] == upd


def test_growth_from_direct_into_staged_tables():
    """A state that outgrows 2^20 buckets moves from direct to staged passes mid-circuit."""
    rng = circuits.SplitMix64(circuits.stream_seed("grow-staged"))
    g = circuits.random_circuit(40, 23, 64, 2, rng, kinds=ALL_KINDS)
    got, stats = run_gpu(40, g, 64, initial_buckets=1 << 12)
    o = SparseOracle(64, threads=SparseOracle.max_threads())
    o.apply(g)
    assert_identical(got, o.state(sorted=True))
    assert stats["buckets"] > 1 << 20 and stats["replays"] > 0


@pytest.mark.parametrize("name", golden_cases()[1])
def test_golden_reference_fixtures(name):
    d, _ = golden_cases()
    g = d[f"{name}/gates"]
    got, _ = run_gpu(int(d[f"{name}/nq"]), g)
    assert_close(drop_negligible(got), (d[f"{name}/keys"], d[f"{name}/re"], d[f"{name}/im"]))
    want, _ = run_oracle(g)
    assert_identical(got, want)


@pytest.mark.parametrize("seed", range(3))
def test_against_dense_statevector(seed):
    rng = circuits.SplitMix64(circuits.stream_seed("gdense", seed))
    nq = 14
    g = circuits.random_circuit(nq, 9, 250, 3, rng, kinds=ALL_KINDS)
    got, _ = run_gpu(nq, g)
    d = DenseOracle(nq)
    d.apply(g)
    assert_close(drop_negligible(got), d.state())


def test_config1_full():
    nq, g = circuits.config_circuit("c1", 0)
    got, stats = run_gpu(nq, g)
    want, upd = run_oracle(g)
    assert_identical(got, want)
    assert got[0].size <= 1024 and stats["amp_updates"] == upd


def test_config2_prefix_against_oracle():
    """The 40-qubit configuration, first 400 gates (up to 2^20 keys) against the oracle."""
    nq, g = circuits.config_circuit("c2", 0)
    got, _ = run_gpu(nq, g[:400], initial_buckets=1 << 12)
    want, _ = run_oracle(g[:400])
    assert_identical(got, want)


def test_table_growth_and_replay():
    """Start from the smallest table: every overflow is detected, the tables grow and the
    failed passes are replayed, with the same result."""
    rng = circuits.SplitMix64(circuits.stream_seed("grow"))
    g = circuits.random_circuit(30, 14, 200, 2, rng, kinds=ALL_KINDS)
    got, stats = run_gpu(30, g, initial_buckets=64)
    want, _ = run_oracle(g)
    assert_identical(got, want)
    assert stats["replays"] > 0 and stats["buckets"] >= 256


def test_hh_cancellation_prunes_everything_but_zero():
    g = G.gate_array([(G.H, q) for q in range(12)] + [(G.H, q) for q in reversed(range(12))])
    got, _ = run_gpu(20, g)
    assert got[0].tolist() == [0] and got[1][0] == pytest.approx(1.0, abs=1e-14)


def test_set_state_sparse_64bit_keys():
    keys = np.array([0, 1 << 63, (1 << 40) | 5, 0xFFFFFFFFFFFFFFFF], np.uint64)
    re = np.array([0.5, 0.5, 0.5, 0.0])
    im = np.array([0.0, 0.0, 0.0, 0.5])
    rng = circuits.SplitMix64(7)
    g = circuits.random_circuit(64, 8, 120, 2, rng, prefix_h=False, kinds=ALL_KINDS)   # branching on q < 8
    got, _ = run_gpu(64, g, init=(keys, re, im))
    want, _ = run_oracle(g, init=(keys, re, im))
    assert_identical(got, want)


def test_empty_state():
    got, stats = run_gpu(20, G.gate_array([(G.H, 0), (G.X, 7), (G.RY, 9, 0, 0.4)]),
                         init=(np.zeros(0, np.uint64), np.zeros(0), np.zeros(0)))
    assert got[0].size == 0 and stats["amp_updates"] == 0


def test_duplicate_keys_rejected():
    st = State(10)
    with pytest.raises(SparqcError) as e:
        st.set_state(np.array([3, 3], np.uint64), np.ones(2), np.zeros(2))
    assert e.value.code == ERR_ARG
    st.close()


def test_bad_arguments_rejected():
    st = State(10)
    for bad in ([(G.H, 10)], [(G.X, 2, 1 << 2)], [(G.X, 2, 1 << 12)]):
        with pytest.raises(SparqcError):
            st.apply(G.gate_array(bad))
    st.close()


@pytest.mark.parametrize("nq", [1, 2, 3, 4, 5])
def test_tiny_registers(nq):
    rng = circuits.SplitMix64(nq)
    g = circuits.random_circuit(nq, nq, 80, nq - 1, rng, kinds=ALL_KINDS)
    got, _ = run_gpu(nq, g)
    want, _ = run_oracle(g)
    assert_identical(got, want)


def test_reference_gate_methods_and_drop_negligible():
    from sparqc_gb300.engine import Circuit
    c = Circuit(12)
    c.h(0); c.h(5); c.rx(5, 0.3); c.ry(0, 1.2); c.rz(3, 0.9); c.phase(5, 0.1); c.x(2); c.y(7); c.z(0)
    g = G.gate_array([(G.H, 0), (G.H, 5), (G.RX, 5, 0, 0.3), (G.RY, 0, 0, 1.2), (G.RZ, 3, 0, 0.9),
                      (G.PHASE, 5, 0, 0.1), (G.X, 2), (G.Y, 7), (G.Z, 0)])
    want, _ = run_oracle(g)
    assert_identical(c.state(sorted=True), want)
    assert_identical(c.state(sorted=True, drop_negligible=True), drop_negligible(want))
    assert c.norm2() == pytest.approx(1.0, abs=1e-13)
    c.close()


def test_fp32_fidelity_and_compare():
    nq, g = circuits.config_circuit("c1", 1)
    a = State(nq, precision=64)
    b = State(nq, precision=32)
    a.apply(g)
    b.apply(g)
    fid, err = b.compare(a)
    assert fid >= 1 - 1e-6 and err < 1e-5
    fid2, err2 = a.compare(a)
    assert fid2 == pytest.approx(1.0, abs=1e-12) and err2 == 0.0
    a.close()
    b.close()


def test_norm_preserved_config2_full():
    """Full 40-qubit configuration (2000 gates, up to 2^20 keys): size-independent checks."""
    nq, g = circuits.config_circuit("c2", 0)
    st = State(nq, initial_buckets=1 << 17)
    st.apply(g)
    n = st.nnz
    assert 0 < n <= 1 << 20
    assert st.norm2() == pytest.approx(1.0, abs=1e-10)
    keys, _, _ = st.state(sorted=True)
    assert np.all(np.diff(keys.astype(np.float64)) > 0)                 # distinct keys
    assert np.unique(keys >> np.uint64(20)).size == 1                     # bits >= k shared
    st.close()


def test_stream_argument():
    import torch
    s = torch.cuda.Stream()
    st = State(16, stream=s.cuda_stream)
    assert st.stream == s.cuda_stream
    st.apply(G.gate_array([(G.H, q) for q in range(16)]))
    assert st.nnz == 1 << 16
    st.close()


def test_cpp_dropin_circuit(tmp_path):
    """The reference-style C++ program, unchanged apart from the include, runs on the engine."""
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "main.cpp"
    src.write_text(r'''
#include <cstdio>
#include "sparqc_circuit.hpp"
int main() {
    hash_table_parameters hp;
    hp.N_devices = 1; hp.N_subtables = 32; hp.coef_gpu_memory_reserve = 0.01; hp.log2_N_bucket_spots = 5;
    try {
        uint32_t nq = 24;
        Circuit__ oc(nq, hp);
        for (uint32_t ii = 0; ii < nq; ii++) oc.h(ii);
        oc.rx(3, 0.5); oc.phase(7, 0.25); oc.controlled(SQC_X, 30 % nq, {1, 2});
        std::printf("nnz %llu norm %.15f\n", (unsigned long long)oc.nnz(), oc.norm2());
        std::vector<short> pattern(nq, -1);
        pattern[0] = 1; pattern[5] = 0;
        auto sel = oc.get_state_full(pattern);
        bool ordered = true, match = true;
        uint64_t prev = 0;
        for (auto& kv : sel) { ordered = ordered && (kv.first >= prev); prev = kv.first;
                               match = match && (kv.first & 1) && !((kv.first >> 5) & 1); }
        std::printf("selected %zu ordered %d match %d\n", sel.size(), (int)ordered, (int)match);
        int m = oc.measure(0, 0.25);
        std::printf("measured %d nnz %llu samples %zu\n", m, (unsigned long long)oc.nnz(), oc.sample(10, 3).size());
        try { Circuit__ bad(8, [] { hash_table_parameters p; p.N_devices = 2; return p; }()); }
        catch (const std::string& e) { std::printf("caught: %s\n", e.c_str()); }
    } catch (const std::string& e) { std::printf("error: %s\n", e.c_str()); return 1; }
    return 0;
}
''')
    exe = tmp_path / "main"
    lib = os.path.join(root, "sparqc_gb300", "_lib")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(root, "include"), str(src), "-o", str(exe),
                    "-L", lib, "-lsparqc", f"-Wl,-rpath,{lib}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    assert "nnz 16777216" in out and "caught:" in out
    # the exact sum of the 2^24 rounded |amplitude|^2, rounded once (1 - 4e-15 here)
    norm = float(out.split("norm ")[1].split()[0])
    assert abs(norm - 1.0) < 1e-12
    assert "selected 4194304 ordered 1 match 1" in out and "nnz 8388608 samples 10" in out
