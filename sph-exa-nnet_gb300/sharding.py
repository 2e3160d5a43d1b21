"""Cost-balanced particle sharding for several GPUs.

Particles are independent, so a multi-GPU burn needs no exchange: each rank burns its own
contiguous range of the particle arrays.  Newton-iteration counts per particle vary by more
than 100x, so equal-count ranges leave most ranks idle while one finishes.  The timestep a
particle carries from its previous burn predicts its cost: a particle that needed small
substeps last time needs about hydro_dt / dt of them again.  `partition` cuts the arrays
into contiguous ranges of (nearly) equal predicted cost."""
import numpy as np


def cost_estimate(dt, hydro_dt, floor=1.0):
    """Predicted relative cost per particle: the number of substeps of the carried timestep
    `dt` over `hydro_dt` (at least `floor`)."""
    dt = np.asarray(dt, dtype=np.float64)
    with np.errstate(divide="ignore"):
        c = np.where(dt > 0, hydro_dt / dt, floor)
    return np.maximum(c, floor)


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
