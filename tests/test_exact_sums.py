"""Norms, probabilities and state comparisons are exact sums rounded once. GPU only.

The order in which kernels meet the keys depends on how concurrent bucket claims interleaved,
so a floating-point accumulation would differ in its last bits between two runs of the same
circuit. The engine adds every product exactly into a fixed-point accumulator and rounds the
total once: the result is the correctly rounded sum of the exact products, whatever the order.
"""
from fractions import Fraction

import numpy as np
import pytest

from sparqc_gb300 import circuits
from sparqc_gb300.engine import State

pytestmark = pytest.mark.gpu


def exact_norm(state, mask=0, value=0):
    k, r, i = state
    sel = (k & np.uint64(mask)) == np.uint64(value)
    tot = Fraction(0)
    for x, y in zip(r[sel].tolist(), i[sel].tolist()):
        tot += Fraction(x) * Fraction(x) + Fraction(y) * Fraction(y)
    return float(tot)   # Fraction -> float rounds to nearest


def test_norm_and_probability_are_the_correctly_rounded_exact_sums():
    rng = circuits.SplitMix64(circuits.stream_seed("exact"))
    g = circuits.random_circuit(30, 12, 400, 2, rng)
    st = State(30)
    st.apply(g)
    s = st.state(sorted=True)
    for c in (s[1], s[2]):   # products of components >= 2^-76 keep every bit above 2^-256
        assert np.all((c == 0) | (np.abs(c) >= 2.0 ** -76))
    assert st.norm2() == exact_norm(s)
    assert st.probability(1 << 3, 1 << 3) == exact_norm(s, 1 << 3, 1 << 3)
    st.close()


def test_same_state_in_another_order_gives_the_same_bits():
    rng = circuits.SplitMix64(circuits.stream_seed("exact-order"))
    g = circuits.random_circuit(40, 14, 300, 3, rng)
    a = State(40)
    a.apply(g)
    k, r, i = a.state(sorted=True)
    perm = np.random.default_rng(1).permutation(k.size)
    b = State(40)
    b.set_state(k[perm], r[perm], i[perm])   # claims, and so the bucket list, in another order
    assert a.norm2() == b.norm2()
    assert a.probability(1 << 5, 0) == b.probability(1 << 5, 0)
    fa, ea = a.compare(b)
    fb, eb = b.compare(a)
    assert fa == fb and ea == eb == 0.0
    a.close()
    b.close()
