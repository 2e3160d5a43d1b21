"""Cost-balanced contiguous sharding (host logic of the multi-GPU path)."""
import numpy as np

import sharding
import workloads


def test_partition_covers_and_balances():
    rng = np.random.default_rng(0)
    cost = np.where(rng.uniform(size=100000) < 0.02, 1000.0, 5.0)  # heavy tail
    cost[:20000] *= 3  # a costly region
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
    assert np.allclose(sharding.cost_estimate(dt=np.array([0.0, 1e-4, 1e-6]), hydro_dt=1e-4),
                       [1.0, 1.0, 1.0 + np.log2(100.0)])
    assert np.allclose(sharding.cost_estimate(prev_iterations=[0, 3]), [1.0, 3.0])


def test_previous_iterations_balance_clustered_particles(port):
    """Two consecutive oracle burns of c2 particles ordered by temperature (hot ones
    together, as in SPH data): ranges balanced on the first burn's iteration counts are
    better balanced in the second burn than equal-count ranges."""
    w = workloads.make("c2", P=2048, seed=11)
    order = np.argsort(w["T"])
    Y, T, rho, dt = w["Y"][:, order], w["T"][order], w["rho"][order], w["dt"][order]
    Y1, T1, dt1, st1, sub1, it1 = port.burn(86, Y, T, rho, dt, w["hydro_dt"], "helmholtz", 0.0, max_iter=20000)
    Y2, T2, dt2, st2, sub2, it2 = port.burn(86, Y1, T1, rho, dt1, w["hydro_dt"], "helmholtz", 0.0, max_iter=20000)
    it2 = np.asarray(it2, dtype=np.float64)
    r = sharding.partition(sharding.cost_estimate(prev_iterations=it1), 4)
    equal = [(k * 512, (k + 1) * 512) for k in range(4)]
    assert sharding.imbalance(it2, r) < sharding.imbalance(it2, equal)
