"""The seeded workload generator (CPU)."""
import numpy as np

from oracle.sparse import SparseOracle
from sparqc_gb300 import circuits, gates as G


def test_deterministic():
    a = circuits.config_circuit("c2", 3, seed=1)[1]
    b = circuits.config_circuit("c2", 3, seed=1)[1]
    c = circuits.config_circuit("c2", 4, seed=1)[1]
    assert np.array_equal(a, b) and not np.array_equal(a, c)


def test_config_shapes_and_rules():
    for name, p in circuits.CONFIGS.items():
        nq, g = circuits.config_circuit(name)
        assert nq == p["nq"] and g.size == p["depth"]
        k = p["k"]
        assert np.all(g["kind"][:k] == G.H) and np.array_equal(g["target"][:k], np.arange(k))
        br = np.isin(g["kind"], G.BRANCH_KINDS)
        assert np.all(g["target"][br] < k)
        for x in g[np.isin(g["kind"], G.SWAP_KINDS) & (g["target"] >= k)]:
            assert int(x["controls"]) & ((1 << k) - 1) == 0
        assert np.all((g["controls"] >> g["target"].astype(np.uint64)) & np.uint64(1) == 0)
        ncontrols = np.array([bin(int(c)).count("1") for c in g["controls"]])
        assert ncontrols.max() <= p["max_controls"]
        mix = np.bincount(np.select([np.isin(g["kind"][k:], G.DIAG_KINDS), np.isin(g["kind"][k:], G.SWAP_KINDS)],
                                    [0, 1], 2), minlength=3) / (p["depth"] - k)
        assert abs(mix[0] - 0.3) < 0.1 and abs(mix[1] - 0.3) < 0.1 and abs(mix[2] - 0.4) < 0.1


def test_config1_nonzero_bound_and_shared_high_bits():
    nq, g = circuits.config_circuit("c1", 0)
    o = SparseOracle()
    o.apply(g)
    keys = o.state()[0]
    assert 0 < keys.size <= 1024
    assert np.unique(keys >> np.uint64(10)).size == 1


def test_batch_and_serving_draws():
    b = circuits.batch_circuits(16)
    assert len(b) == 16
    for nq, k, g in b:
        assert 16 <= nq <= 48 and 8 <= k <= 18 and 100 <= g.size <= 1000
    s = circuits.serving_stream(200, 100.0)
    t = [x[0] for x in s]
    assert all(np.diff(t) > 0)
    assert any(x[1] == 48 and x[3].size == 2000 for x in s)
