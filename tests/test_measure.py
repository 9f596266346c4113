"""Selection, probabilities, measurement and sampling on the device, against numpy on the
oracle's state (same circuit, same seeded inputs). GPU only.

Probability sums run on the device in FP64 with atomics (summation order varies), so they are
compared at 1e-12 relative; key sets are compared exactly.
"""
import numpy as np
import pytest

from oracle.sparse import SparseOracle
from sparqc_gb300 import circuits, gates as G
from sparqc_gb300.engine import ERR_ARG, SparqcError, State

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def _state(nq=20, k=12, depth=150, seed=1, precision=64, **kw):
    rng = circuits.SplitMix64(circuits.stream_seed("measure", seed))
    g = circuits.random_circuit(nq, k, depth, 2, rng)
    st = State(nq, precision=precision, **kw)
    st.apply(g)
    o = SparseOracle(precision)
    o.apply(g)
    return st, o.state(sorted=True), g


def test_sorted_readout_and_patterns():
    st, (ok, orr, oi), _ = _state()
    k, r, i = st.state(sorted=True)
    assert np.array_equal(k, ok) and np.array_equal(r, orr) and np.array_equal(i, oi)
    ku, ru, iu = st.state(sorted=False)
    order = np.argsort(ku)
    assert np.array_equal(ku[order], ok) and np.array_equal(ru[order], orr)
    for mask, value in [(1 << 3, 0), (1 << 3, 1 << 3), ((1 << 2) | (1 << 7), 1 << 7), (0, 0)]:
        sel = (ok & np.uint64(mask)) == np.uint64(value)
        kw, rw, iw = st.state_where(mask, value)
        assert np.array_equal(kw, ok[sel]) and np.array_equal(rw, orr[sel]) and np.array_equal(iw, oi[sel])
        p = st.probability(mask, value)
        want = float(np.sum(orr[sel] ** 2 + oi[sel] ** 2))
        assert p == pytest.approx(want, rel=1e-12, abs=1e-300)


def test_patterns_see_through_the_key_frame():
    # uncontrolled X gates only relabel keys on the host; patterns address actual keys
    st = State(30)
    st.apply(G.gate_array([(G.H, 0), (G.X, 20), (G.X, 5), (G.H, 9)]))
    k, _, _ = st.state_where(1 << 20, 1 << 20)
    assert k.size == 4 and all(int(x) >> 20 & 1 for x in k)
    assert st.probability(1 << 5, 0) == 0.0
    assert st.probability(1 << 5, 1 << 5) == pytest.approx(1.0, rel=1e-15)


@pytest.mark.parametrize("precision", [64, 32])
def test_measure_collapses_and_renormalises(precision):
    st, (ok, orr, oi), _ = _state(precision=precision)
    q = 4
    p1_want = float(np.sum((orr ** 2 + oi ** 2)[(ok >> np.uint64(q)) & np.uint64(1) == 1])) / float(
        np.sum(orr ** 2 + oi ** 2))
    out, p1 = st.measure(q, 0.37)
    tol = 1e-12 if precision == 64 else 1e-5
    assert p1 == pytest.approx(p1_want, rel=tol)
    assert out == (1 if 0.37 < p1 else 0)
    keep = ((ok >> np.uint64(q)) & np.uint64(1)) == np.uint64(out)
    kept_p = float(np.sum(orr[keep] ** 2 + oi[keep] ** 2))
    k, r, i = st.state(sorted=True)
    assert np.array_equal(k, ok[keep])
    scale = 1.0 / np.sqrt(kept_p)
    assert np.allclose(r, orr[keep] * scale, rtol=tol, atol=1e-14)
    assert np.allclose(i, oi[keep] * scale, rtol=tol, atol=1e-14)
    assert st.norm2() == pytest.approx(1.0, rel=tol)
    # the measured qubit is now known: a gate controlled on the other value does nothing
    n0 = st.nnz
    st.apply(G.gate_array([(G.H, 5, (q,) if out == 0 else ())]))
    if out == 0:
        assert st.nnz == n0
    with pytest.raises(SparqcError) as e:
        st.measure(99, 0.5)
    assert e.value.code == ERR_ARG


def _uniform(seed, s):
    def mix(x):
        x = (x + 0x9E3779B97F4A7C15) & M64
        x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
        x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
        return x ^ (x >> 31)
    return (mix(seed ^ mix(s)) >> 11) * (1.0 / 9007199254740992.0)


def test_sampling_follows_the_cumulative_distribution():
    st, (ok, orr, oi), _ = _state(nq=16, k=9, depth=120, seed=4)
    shots = 20000
    got = st.sample(shots, seed=7)
    assert np.array_equal(got, st.sample(shots, seed=7))   # same seed, same samples
    cum = np.cumsum(orr ** 2 + oi ** 2)
    total = cum[-1]
    pos = np.searchsorted(ok, got)
    assert np.array_equal(ok[pos], got)                    # every sample is a present key
    for s in range(0, shots, 97):                          # each shot lands in its key's interval
        u = _uniform(7, s) * total
        lo = cum[pos[s] - 1] if pos[s] > 0 else 0.0
        assert lo - 1e-12 <= u <= cum[pos[s]] + 1e-12
    # frequencies against probabilities (chi-square over keys with expected count >= 20)
    counts = np.bincount(pos, minlength=ok.size)
    expected = shots * (orr ** 2 + oi ** 2) / total
    sel = expected >= 20
    chi2 = np.sum((counts[sel] - expected[sel]) ** 2 / expected[sel])
    assert chi2 < 2.0 * sel.sum() + 50
