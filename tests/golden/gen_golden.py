"""Generate the golden fixtures of tests/golden from the reference compiled from its own
sources (oracle/_ref/libnnet_ref.so, built by oracle/build.py where the reference tree is
present).  The reference ships no golden vectors or assertions (its tests print only), so
these fixtures are its outputs on:

  rates_kat.npz  the rate test points of test/net14_rate_test.cpp:50-79 (net14, T=2e9,
                 rho=1e9, X(12C)=X(16O)=0.5) and test/net87_rate_test.cpp:50-91 (net87 +
                 Helmholtz, T=3e9, rho=1e9, Y_e=1), plus seeded net86 points
  eos_kat.npz    the Helmholtz EOS (stand-in table) on seeded (abar, zbar, T, rho) points
  burn_*.npz     batch burns of seeded samples of the c1 / c2 / c4 workloads
  nr_net14.npz   a solveSystemNR trajectory like test/net14_test.cpp:134-187
                 (C-O burning, rho=1e9, T=1e9, ideal gas mu=10)
  burn_special.npz  single particles whose substep loop never ends in the reference (see
                 SPECIAL): one whose timestep wanders at the rejection rule's fixed point
                 (LIVELOCK once attempt-start timesteps repeat within 2^-20), one whose
                 rejections follow a chaotic timestep map and one alternating between two
                 timesteps from a wandering Newton temperature buffer (both MAXITER)

usage: python tests/golden/gen_golden.py            (all fixtures)
       python tests/golden/gen_golden.py special    (burn_special.npz only)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "sph-exa-nnet_gb300"))
sys.path.insert(0, os.path.join(REPO, "sph-exa-nnet_gb300", "data"))

import gen_helm_table  # noqa: E402
import workloads  # noqa: E402
from oracle import Oracle  # noqa: E402

BURN_CASES = {"c1": 1024, "c2": 192, "c4": 96}
# (workload, network of a c3 part or None, particle index in it, Newton-iteration budget)
SPECIAL = [("c2", None, 168389, 20000), ("c3", 86, 881263, 2000), ("c3", 14, 169533, 2000)]


def special(ref):
    """burn_special.npz: the reference's burns of the SPECIAL particles."""
    out = {}
    for k, (name, net, i, budget) in enumerate(SPECIAL):
        w = workloads.make(name)
        if net is not None:
            w = [p for p in w if p["net"] == net][0]
        Y0, T0, rho, dt0 = (np.ascontiguousarray(w[f][..., i:i + 1]) for f in ("Y", "T", "rho", "dt"))
        Y, T, dt, st, sub, it = ref.burn(w["net"], Y0, T0, rho, dt0, w["hydro_dt"], w["eos"], w["mu"],
                                         max_iter=budget)
        out.update({f"{k}_net": w["net"], f"{k}_eos": w["eos"], f"{k}_mu": w["mu"], f"{k}_hydro_dt": w["hydro_dt"],
                    f"{k}_budget": budget, f"{k}_Y0": Y0, f"{k}_T0": T0, f"{k}_rho": rho, f"{k}_dt0": dt0,
                    f"{k}_Y": Y, f"{k}_T": T, f"{k}_dt": dt, f"{k}_status": st, f"{k}_substeps": sub,
                    f"{k}_iters": it})
        print(name, net, i, "status", int(st[0]), "iterations", int(it[0]))
        del w
    np.savez_compressed(os.path.join(HERE, "burn_special.npz"), cases=len(SPECIAL), **out)


def main():
    ref = Oracle("ref")
    tab = np.stack([gen_helm_table.tables()[n] for n in gen_helm_table.NAMES]).reshape(-1)
    ref.load_helmholtz(tab)
    special(ref)
    if sys.argv[1:] == ["special"]:
        return

    # ---- rate known-answer tests
    out = {}
    Y14 = workloads.composition(14, 1, 0.5, 0.5, 0.0)[:, 0]
    BE, r, dr, _ = ref.rates(14, Y14, 2e9, 1e9, eos="ideal", mu=10.0)
    out.update(net14_Y=Y14, net14_BE=BE, net14_rates=r, net14_drates=dr)
    Y87 = workloads.composition(87, 1, 0.5, 0.5, 0.0)[:, 0]
    Y87[86] = 1.0
    BE, r, dr, e = ref.rates(87, Y87, 3e9, 1e9, eos="helmholtz")
    out.update(net87_Y=Y87, net87_BE=BE, net87_rates=r, net87_drates=dr, net87_cv=e["cv"])
    rng = np.random.default_rng(7)
    pts = np.stack([10 ** rng.uniform(8.3, 9.9, 16), 10 ** rng.uniform(5.5, 9.9, 16)], axis=1)
    Y86 = workloads.composition(86, 1, 0.3, 0.7, 1e-10)[:, 0]
    r86, dr86, be86 = [], [], []
    for T, rho in pts:
        BE, r, dr, _ = ref.rates(86, Y86, T, rho, eos="helmholtz")
        r86.append(r), dr86.append(dr), be86.append(BE)
    out.update(net86_points=pts, net86_Y=Y86, net86_rates=np.array(r86), net86_drates=np.array(dr86),
               net86_BE=np.array(be86))
    np.savez_compressed(os.path.join(HERE, "rates_kat.npz"), **out)

    # ---- Helmholtz EOS known answers
    rng = np.random.default_rng(8)
    n = 256
    abar_ = rng.uniform(0.02, 1.0, n)
    zbar_ = abar_ * rng.uniform(0.3, 10, n)
    T = 10 ** rng.uniform(7, 10, n)
    rho = 10 ** rng.uniform(2, 10, n)
    vals = np.array([[v for v in ref.helmholtz(a, z, t, d).values()] for a, z, t, d in zip(abar_, zbar_, T, rho)])
    np.savez_compressed(os.path.join(HERE, "eos_kat.npz"), abar_=abar_, zbar_=zbar_, T=T, rho=rho, out=vals)

    # ---- batch burns
    for name, P in BURN_CASES.items():
        w = workloads.make(name, P=P)
        Y, T, dt, st, sub, it = ref.burn(w["net"], w["Y"], w["T"], w["rho"], w["dt"], w["hydro_dt"], w["eos"],
                                         w["mu"], max_iter=20000)
        np.savez_compressed(os.path.join(HERE, f"burn_{name}.npz"), P=P, Y=Y, T=T, dt=dt, status=st, substeps=sub,
                            iters=it)
        print(name, np.bincount(st, minlength=5))

    # ---- single-particle Newton trajectory (net14_test)
    Y = workloads.composition(14, 1, 0.5, 0.5, 0.0)[:, 0]
    T, dt, t = 1e9, 1e-5, 0.0
    traj = []
    for _ in range(60):
        Yn, Tn, dt, ts = ref.solve_nr(14, Y, T, 1e9, dt, eos="ideal", mu=10.0)
        t += ts
        traj.append(np.concatenate([[t, dt, Tn], Yn]))
        Y, T = Yn, Tn
    np.savez_compressed(os.path.join(HERE, "nr_net14.npz"), traj=np.array(traj))
    print("fixtures written")


if __name__ == "__main__":
    main()
