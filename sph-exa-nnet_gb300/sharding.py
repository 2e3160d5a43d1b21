"""Cost-balanced particle sharding for several GPUs.

Particles are independent, so a multi-GPU burn needs no exchange: each rank burns its own
contiguous range of the particle arrays.  Newton-iteration counts per particle vary by more
than 100x, and in SPH data the costly (hot) particles sit together, so equal-count ranges
can leave most ranks idle while one finishes.  The best predictor of a particle's cost is
the Newton-iteration count of its previous burn (returned per particle by the library in
`nnet_burn_args.iterations`); without it, the timestep the particle carries is a weaker one
(cost ~ 1 + log2(hydro_dt / dt)).  `partition` cuts the arrays into contiguous ranges of
(nearly) equal predicted cost.

This is host logic: bench.py --strong uses it to split one particle set over torchrun ranks,
and tests/test_sharding.py checks (with the oracle, 2,048 c2 particles ordered by temperature,
two consecutive burns) that ranges balanced on the first burn's iterations balance the second
burn better than equal-count ranges; tests/test_multirank.py runs the split over two gloo
ranks."""
import numpy as np


def cost_estimate(prev_iterations=None, dt=None, hydro_dt=None):
    """Predicted relative cost per particle: the previous burn's Newton iterations when
    given (at least 1), else 1 + log2(hydro_dt / dt) from the carried timestep."""
    if prev_iterations is not None:
        return np.maximum(np.asarray(prev_iterations, dtype=np.float64), 1.0)
    dt = np.asarray(dt, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(dt > 0, hydro_dt / dt, 1.0)
    return 1.0 + np.log2(np.maximum(r, 1.0))


def partition(cost, world):
    """Contiguous ranges [(first, last)] of the particles for `world` ranks whose cost sums
    are as equal as the cut positions allow (each cut at the first particle where the
    running cost reaches k/world of the total)."""
    cost = np.asarray(cost, dtype=np.float64)
    P = cost.size
    if world < 1:
        raise ValueError("world must be >= 1")
    csum = np.cumsum(cost)
    total = csum[-1] if P else 0.0
    cuts = [0]
    for k in range(1, world):
        cuts.append(int(np.searchsorted(csum, total * k / world, side="left")) + 1 if P else 0)
    cuts.append(P)
    cuts = np.maximum.accumulate(np.minimum(np.array(cuts), P))
    return [(int(cuts[k]), int(cuts[k + 1])) for k in range(world)]


def imbalance(cost, ranges):
    """max over ranks of the range's cost divided by the mean (1.0 = perfect balance)."""
    cost = np.asarray(cost, dtype=np.float64)
    sums = np.array([cost[a:b].sum() for a, b in ranges])
    return float(sums.max() / sums.mean()) if sums.mean() > 0 else 1.0
