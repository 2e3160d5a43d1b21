"""Seeded synthetic particle states for the burn workloads (no dataset is involved).

Each workload is a batch of SPH particles with abundances Y (species-major,
Y[species, particle] = X / A), temperature T, density rho, the carried nuclear
timestep dt (initial 1e-5 s, include/nnet/nuclear_net.hpp:51) and a hydro step.

  c1  net14 + ideal gas (mu = 10), 4,096 particles, X(12C) = X(16O) = 0.5,
      rho log-uniform [1e7, 1e9], T log-uniform [1e9, 4e9], hydro dt 1e-3 s, seed 1
  c2  net86 + Helmholtz, 1,048,576 particles, X(12C) = 0.3, X(16O) = 0.7, every other
      species at a 1e-10 mass-fraction floor, rho log-uniform [1e6, 5e9],
      T log-uniform [5e8, 6e9], hydro dt 1e-4 s, seed 2
  c3  2,097,152 particles, 50% net86 / 30% net87 / 20% net14 (Helmholtz), bimodal T:
      70% log-normal(ln 8e8, sigma 0.3), 30% log-normal(ln 5e9, sigma 0.2), rho and
      composition as c2, electron fraction Y_e = 0.5 for net87, seed 3
  c4  net87 + Helmholtz, 2,097,152 particles, rho log-uniform [1e7, 1e10],
      T log-uniform [1e9, 7e9], Y_e uniform [0.45, 0.5], composition as c2, seed 4
"""
import numpy as np

# species indices
NET14_C, NET14_O = 1, 2
NET86_C, NET86_O, ELECTRON = 3, 4, 86

A14 = np.array([4, 12, 16, 20, 24, 28, 32, 36, 40, 44, 48, 52, 56, 60], dtype=np.float64)
_A86 = None


def mass_numbers(net):
    global _A86
    if net == 14:
        return A14
    if _A86 is None:
        import os
        import re
        src = open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "nnet_network_tables.h")).read()
        body = re.search(r"net86_A\[87\] = \{([^}]*)\}", src).group(1)
        _A86 = np.array([float(v) for v in body.split(",")])
    return _A86[:86] if net == 86 else _A86


_BE = {}


def binding_energies(net):
    """Binding energies of a network's species (the reference's BE tables)."""
    if net not in _BE:
        import os
        import re
        src = open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "nnet_network_tables.h")).read()
        name = {14: "net14_BE", 86: "net86_BE", 87: "net87_BE"}[net]
        body = re.search(name + r"\[\d+\] = \{([^}]*)\}", src).group(1)
        _BE[net] = np.array([float(v) for v in body.split(",")])
    return _BE[net]


def composition(net, P, xc, xo, floor):
    """Y[species, P] from mass fractions X(12C)=xc, X(16O)=xo and a floor on the others."""
    A = mass_numbers(net)
    nnuc = 14 if net == 14 else 86
    X = np.full(nnuc, floor)
    if net == 14:
        X[NET14_C], X[NET14_O] = xc, xo
    else:
        X[NET86_C], X[NET86_O] = xc, xo
    Y = np.empty((net, P))
    Y[:nnuc] = (X / A[:nnuc])[:, None]
    return Y


def _logu(rng, lo, hi, n):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n))


def make(name, P=None, seed=None):
    """Return a dict describing one workload (see the module docstring)."""
    name = name.lower()
    if name == "c1":
        P = P or 4096
        rng = np.random.default_rng(1 if seed is None else seed)
        rho = _logu(rng, 1e7, 1e9, P)
        T = _logu(rng, 1e9, 4e9, P)
        return dict(name="c1", net=14, eos="ideal", mu=10.0, Y=composition(14, P, 0.5, 0.5, 0.0), T=T, rho=rho,
                    dt=np.full(P, 1e-5), hydro_dt=1e-3)
    if name == "c2":
        P = P or 1048576
        rng = np.random.default_rng(2 if seed is None else seed)
        rho = _logu(rng, 1e6, 5e9, P)
        T = _logu(rng, 5e8, 6e9, P)
        return dict(name="c2", net=86, eos="helmholtz", mu=0.0, Y=composition(86, P, 0.3, 0.7, 1e-10), T=T, rho=rho,
                    dt=np.full(P, 1e-5), hydro_dt=1e-4)
    if name == "c4":
        P = P or 2097152
        rng = np.random.default_rng(4 if seed is None else seed)
        rho = _logu(rng, 1e7, 1e10, P)
        T = _logu(rng, 1e9, 7e9, P)
        Y = composition(87, P, 0.3, 0.7, 1e-10)
        Y[ELECTRON] = rng.uniform(0.45, 0.5, P)
        return dict(name="c4", net=87, eos="helmholtz", mu=0.0, Y=Y, T=T, rho=rho, dt=np.full(P, 1e-5),
                    hydro_dt=1e-4)
    if name == "c3":
        return make_mixed(P or 2097152, 3 if seed is None else seed)
    raise ValueError(name)


def make_mixed(P, seed):
    """c3: a list of per-network sub-batches drawn from one seeded stream."""
    rng = np.random.default_rng(seed)
    which = rng.choice(np.array([86, 87, 14]), size=P, p=[0.5, 0.3, 0.2])
    hot = rng.uniform(size=P) < 0.3
    T = np.where(hot, rng.lognormal(np.log(5e9), 0.2, P), rng.lognormal(np.log(8e8), 0.3, P))
    rho = _logu(rng, 1e6, 5e9, P)
    parts = []
    for net in (86, 87, 14):
        idx = np.nonzero(which == net)[0]
        Y = composition(net, idx.size, 0.3, 0.7, 1e-10)
        if net == 87:
            Y[ELECTRON] = 0.5
        parts.append(dict(name=f"c3-net{net}", net=net, eos="helmholtz", mu=0.0, Y=Y, T=T[idx].copy(),
                          rho=rho[idx].copy(), dt=np.full(idx.size, 1e-5), hydro_dt=1e-4, index=idx))
    return parts
