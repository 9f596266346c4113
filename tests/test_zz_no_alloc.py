"""sqc_apply_fixed, the entry point for callers that cannot allocate device memory.

It must give exactly what the allocating path (sqc_create + sqc_set_state +
sqc_apply_gates + sqc_get_state) gives for the same state and gates, call after call:
both run the same FP64 arithmetic, so entries are compared bit for bit after sorting by
key. The device buffers here are allocated by the test, standing in for the caller's own.
GPU only. Named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from oracle.sparse import SparseOracle
from sparqc_gb300 import circuits, gates as G
from sparqc_gb300.engine import ERR_ARG, ERR_CAPACITY, OK, State, load

pytestmark = pytest.mark.gpu

ALL_KINDS = ((G.Z, G.S, G.SDG, G.T, G.TDG, G.RZ, G.PHASE), (G.X, G.Y), (G.H, G.RX, G.RY, G.U))


def _lib():
    L = load()
    P = ctypes.c_void_p
    L.sqc_apply_fixed.restype = ctypes.c_int
    L.sqc_apply_fixed.argtypes = [ctypes.c_uint32, P, P, P, ctypes.c_uint64, P, ctypes.c_uint64, P, P, P,
                                  ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), P]
    return L


def _fixed(nq, keys, re, im, gates, cap):
    import torch
    dev = torch.device("cuda")
    k_in = torch.from_numpy(keys.astype(np.int64)).to(dev)
    r_in = torch.from_numpy(re).to(dev)
    i_in = torch.from_numpy(im).to(dev)
    k_out = torch.zeros(cap, dtype=torch.int64, device=dev)
    r_out = torch.zeros(cap, dtype=torch.float64, device=dev)
    i_out = torch.zeros(cap, dtype=torch.float64, device=dev)
    gates = np.ascontiguousarray(gates)
    stream = torch.cuda.current_stream()
    n = ctypes.c_uint64()
    rc = _lib().sqc_apply_fixed(nq, k_in.data_ptr(), r_in.data_ptr(), i_in.data_ptr(), keys.size,
                                gates.ctypes.data_as(ctypes.c_void_p), gates.size, k_out.data_ptr(),
                                r_out.data_ptr(), i_out.data_ptr(), cap, ctypes.byref(n), stream.cuda_stream)
    torch.cuda.synchronize()
    m = n.value
    k = k_out[:m].cpu().numpy().view(np.uint64)
    order = np.argsort(k)
    return rc, k[order], r_out[:m].cpu().numpy()[order], i_out[:m].cpu().numpy()[order]


def _allocating(nq, keys, re, im, gates):
    st = State(nq)
    st.set_state(keys, re, im)
    st.apply(gates)
    out = st.state(sorted=True)
    st.close()
    return out


def _case(seed, nq, k, depth):
    rng = circuits.SplitMix64(circuits.stream_seed("fixed", seed))
    keys = np.unique(np.array([rng.next() & ((1 << nq) - 1) & ~((1 << k) - 1) for _ in range(6)], np.uint64))
    re = np.array([rng.uniform() - 0.5 for _ in keys])
    im = np.array([rng.uniform() - 0.5 for _ in keys])
    norm = np.sqrt(np.sum(re ** 2 + im ** 2))
    gates = circuits.random_circuit(nq, k, depth, 3, rng, kinds=ALL_KINDS)
    return keys, re / norm, im / norm, gates


def _oracle(keys, re, im, gates):
    o = SparseOracle()
    o.set_state(keys, re, im)
    o.apply(gates)
    return o.state(sorted=True)


def test_fixed_matches_allocating_path_call_after_call():
    # two calls in a row on the shared scratch, both within the fixed table's group limit; each
    # result also equals the oracle's (the reference's algorithm restated on the CPU)
    for seed, nq, k, depth in ((1, 40, 10, 200), (2, 64, 12, 100)):
        keys, re, im, gates = _case(seed, nq, k, depth)
        rc, fk, fr, fi = _fixed(nq, keys, re, im, gates, 1 << 18)
        assert rc == OK
        want = _allocating(nq, keys, re, im, gates)
        assert fk.size > 0
        for x, y, z in zip((fk, fr, fi), want, _oracle(keys, re, im, gates)):
            assert np.array_equal(x, y) and np.array_equal(x, z)


def test_fixed_rejects_keys_outside_the_register_and_duplicates():
    z = np.zeros(2)
    gates = G.gate_array([(G.H, 0)])
    rc, *_ = _fixed(20, np.array([3, 1 << 20], np.uint64), z + 0.5, z + 0.5, gates, 16)
    assert rc == ERR_ARG
    rc, *_ = _fixed(20, np.array([7, 7], np.uint64), z + 0.5, z + 0.5, gates, 16)
    assert rc == ERR_ARG


def test_fixed_capacity_refusal_then_a_clean_call():
    # 16000 keys in distinct 16-key groups, then H on qubit 4: the pass could need 32000 groups,
    # more than the fixed table takes, and refuses before touching anything
    keys = (np.arange(16000, dtype=np.uint64) << np.uint64(5))
    re = np.full(keys.size, 1.0 / np.sqrt(keys.size))
    rc, *_ = _fixed(30, keys, re, np.zeros(keys.size), G.gate_array([(G.H, 4)]), 1 << 16)
    assert rc == ERR_CAPACITY
    # the next call on the same scratch is unaffected
    keys, re, im, gates = _case(1, 40, 10, 200)
    rc, fk, fr, fi = _fixed(40, keys, re, im, gates, 1 << 18)
    assert rc == OK
    for x, y in zip((fk, fr, fi), _allocating(40, keys, re, im, gates)):
        assert np.array_equal(x, y)


def test_fixed_rejects_oversized_input():
    keys = np.arange(1 << 15, dtype=np.uint64)
    z = np.zeros(keys.size)
    rc, *_ = _fixed(20, keys, z + 1.0 / 181.0, z, G.gate_array([(G.H, 0)]), 16)
    assert rc == ERR_CAPACITY


def test_fixed_reports_short_output_capacity():
    keys, re, im, gates = _case(3, 30, 9, 100)
    rc, fk, _, _ = _fixed(30, keys, re, im, gates, 4)
    assert rc == ERR_CAPACITY
