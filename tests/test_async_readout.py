"""Asynchronous readout (sqc_get_state_async / sqc_readout_wait). GPU only.

The readout of one circuit travels to page-locked host arrays while the next circuit runs on
the same state; each result equals the synchronous readout of the same circuit, entry for
entry (both list the entries in the table's order, so they are compared key-sorted).
"""
import numpy as np
import pytest
import torch

from sparqc_gb300 import circuits
from sparqc_gb300.engine import ERR_ARG, ERR_CAPACITY, FP32, FP64, SparqcError, State

pytestmark = pytest.mark.gpu


def pinned(n, dtype):
    tdt = {np.uint64: torch.int64, np.float64: torch.float64}[dtype]
    return torch.empty(n, dtype=tdt, pin_memory=True).numpy().view(dtype)


def key_sorted(k, r, i):
    o = np.argsort(k, kind="stable")
    return k[o], r[o], i[o]


@pytest.mark.parametrize("precision", [FP64, FP32])
def test_async_readout_overlaps_the_next_circuit_and_equals_the_sync_one(precision):
    cs = [circuits.random_circuit(40, 12, 300, 3, circuits.SplitMix64(circuits.stream_seed("async", j)))
          for j in range(3)]
    want = []
    ref = State(40, precision=precision)
    for g in cs:
        ref.set_zero()
        ref.apply(g)
        want.append(ref.state(sorted=True))
    ref.close()
    cap = max(w[0].size for w in want)
    bufs = [(pinned(cap, np.uint64), pinned(cap, np.float64), pinned(cap, np.float64), pinned(1, np.uint64))
            for _ in cs]
    st = State(40, precision=precision)
    for j, g in enumerate(cs):
        st.set_zero()          # queued while the previous circuit's readout is still copying
        st.apply(g)
        st.state_async(*bufs[j])   # completes the previous readout, gathers this one, returns
    st.readout_wait()
    for (k, r, i, n), w in zip(bufs, want):
        m = int(n[0])
        assert m == w[0].size
        got = key_sorted(k[:m].copy(), r[:m].copy(), i[:m].copy())
        assert all(np.array_equal(x, y) for x, y in zip(got, w))
    st.close()


def test_async_readout_capacity_and_pageable_arrays():
    g = circuits.random_circuit(30, 10, 200, 2, circuits.SplitMix64(circuits.stream_seed("async-cap", 0)))
    st = State(30)
    st.apply(g)
    full = st.nnz
    k, r, i, n = pinned(full - 1, np.uint64), pinned(full - 1, np.float64), pinned(full - 1, np.float64), \
        pinned(1, np.uint64)
    st.state_async(k, r, i, n)
    with pytest.raises(SparqcError) as e:
        st.readout_wait()
    assert e.value.code == ERR_CAPACITY and int(n[0]) == full
    with pytest.raises(SparqcError) as e:   # pageable arrays cannot be written by the device
        st.state_async(np.zeros(full, np.uint64), np.zeros(full), np.zeros(full), np.zeros(1, np.uint64))
    assert e.value.code == ERR_ARG
    k, r, i = pinned(full, np.uint64), pinned(full, np.float64), pinned(full, np.float64)
    st.state_async(k, r, i, n)   # the state is unharmed
    st.readout_wait()
    want = st.state(sorted=True)
    assert all(np.array_equal(x, y) for x, y in zip(key_sorted(k.copy(), r.copy(), i.copy()), want))
    st.close()
