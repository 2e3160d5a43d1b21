"""Cost-balanced contiguous sharding (host logic of the multi-GPU path)."""
import numpy as np

import sharding


def test_partition_covers_and_balances():
    rng = np.random.default_rng(0)
    dt = np.where(rng.uniform(size=100000) < 0.02, 1e-8, 1e-5)  # a heavy tail of tiny carried steps
    cost = sharding.cost_estimate(dt, 1e-4)
    for world in (1, 2, 4, 8):
        r = sharding.partition(cost, world)
        assert r[0][0] == 0 and r[-1][1] == cost.size
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))  # contiguous, no gaps or overlaps
        assert sharding.imbalance(cost, r) < 1.01
        equal = [(k * cost.size // world, (k + 1) * cost.size // world) for k in range(world)]
        assert sharding.imbalance(cost, r) <= sharding.imbalance(cost, equal) + 1e-12


def test_edge_cases():
    assert sharding.partition(np.array([]), 3) == [(0, 0), (0, 0), (0, 0)]
    assert sharding.partition(np.ones(2), 4)[-1] == (2, 2)
    c = sharding.cost_estimate(np.array([0.0, 1e-4, 1e-6]), 1e-4)
    assert np.allclose(c, [1.0, 1.0, 100.0])
