"""Post-burn steps of nnet_burn on the GPU, through the C ABI: the mass normalisation and its
drift report (sum_i X_i = 1 to 1e-12), and the post-burn Helmholtz EOS (computeHelmEOS,
parallel_nuclear_net.hpp:191-261) that the batched layout evaluates as each particle retires
and the other layouts evaluate in a pass after the burn."""
import numpy as np
import pytest

import workloads
from test_gpu_parity import SUM_X_TOL, check, gpu_burn, normalize_mass

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import torch
    import nnet_gb300 as nn
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    c = nn.Context(0)
    yield c
    c.close()


def _cold(w, n):
    """Make the first n particles cold (skipped): they keep their state but still get the EOS."""
    w = dict(w)
    T = w["T"].copy()
    T[:n] = 5e7
    w["T"] = T
    return w


def _burn_post(ctx, w, solver, layout, normalize=True, eos=True):
    import torch
    dev = torch.device("cuda:0")
    ctx.set_layout(layout)
    Y, T = torch.tensor(w["Y"], device=dev), torch.tensor(w["T"], device=dev)
    rho, dt = torch.tensor(w["rho"], device=dev), torch.tensor(w["dt"], device=dev)
    P = T.numel()
    st = torch.full((P,), -1, dtype=torch.int32, device=dev)
    drift = torch.full((P,), np.nan, dtype=torch.float64, device=dev)
    outs = [torch.full((P,), np.nan, dtype=torch.float64, device=dev) for _ in range(5)] if eos else None
    ctx.burn(w["net"], Y, T, rho, dt, w["hydro_dt"], eos=w["eos"], mu=w["mu"], solver=solver, status=st,
             max_iter=20000, normalize_mass=normalize, mass_drift=drift, eos_out=outs)
    torch.cuda.synchronize()
    ctx.set_layout("auto")
    res = dict(Y=Y.cpu().numpy(), T=T.cpu().numpy(), dt=dt.cpu().numpy(), status=st.cpu().numpy(),
               drift=drift.cpu().numpy())
    if eos:
        res.update(zip(["u", "cv", "p", "c", "dpdT"], [o.cpu().numpy() for o in outs]))
    return res


@pytest.mark.parametrize("layout,solver", [("batched", "sparse"), ("batched", "mixed"), ("thread", "sparse"),
                                           ("warp", "sparse")])
def test_normalisation_and_drift(ctx, layout, solver):
    """sum_i A_i Y_i = 1 to 1e-12 after the burn; the reported drift is the one of the same burn
    without normalisation, whose abundances the normalised ones equal up to the division."""
    w = _cold(workloads.make("c2", P=300, seed=71), 4)
    a = _burn_post(ctx, w, solver, layout, normalize=True, eos=False)
    b = _burn_post(ctx, w, solver, layout, normalize=False, eos=False)
    A = np.asarray(workloads.mass_numbers(86))[:86, None]
    burned = a["status"] != 1
    assert np.array_equal(a["status"], b["status"]) and np.array_equal(a["T"], b["T"])
    assert np.abs((A * a["Y"]).sum(0)[burned] - 1).max() <= SUM_X_TOL
    # the drift is measured on the un-normalised state (identical in both runs)
    assert np.array_equal(a["drift"], b["drift"])
    s = (A * b["Y"]).sum(0)
    assert np.allclose(a["drift"], s - 1, rtol=0, atol=1e-14)
    Yn, _ = normalize_mass(86, b["Y"], b["status"])
    assert np.allclose(a["Y"], Yn, rtol=1e-14, atol=0)
    # skipped particles are untouched, their drift still reported
    assert np.array_equal(a["Y"][:, ~burned], w["Y"][:, ~burned])
    print(f"{layout}/{solver}: max |drift| {np.abs(a['drift'][burned]).max():.2e}, "
          f"max |sum X - 1| after {np.abs((A * a['Y']).sum(0)[burned] - 1).max():.2e}")


@pytest.mark.parametrize("layout,solver", [("batched", "sparse"), ("batched", "mixed"), ("thread", "sparse"),
                                           ("warp", "sparse")])
def test_post_burn_eos(ctx, port, layout, solver):
    """The post-burn EOS at each particle's final (Y, T, rho) equals the oracle's
    computeHelmholtzImpl restatement on the same state, and the stand-alone EOS entry point
    (nnet_helmholtz_eos) on the burned arrays."""
    import torch
    import nnet_gb300 as nn
    w = _cold(workloads.make("c2", P=300, seed=72), 5)
    r = _burn_post(ctx, w, solver, layout, normalize=True, eos=True)
    Z = nn.network_charges(86)
    ref = port.helm_eos_batch(Z, r["T"], w["rho"], r["Y"])
    for name in ("u", "cv", "p", "c", "dpdT"):
        rel = np.abs(r[name] - ref[name]) / np.abs(ref[name])
        assert rel.max() < 1e-9, (name, rel.max())  # as test_helmholtz_eos_batch
    dev = torch.device("cuda:0")
    Y = torch.tensor(r["Y"], device=dev)
    outs = [torch.zeros(300, dtype=torch.float64, device=dev) for _ in range(5)]
    ctx.helmholtz_eos(Z, torch.tensor(r["T"], device=dev), torch.tensor(w["rho"], device=dev), Y, *outs)
    torch.cuda.synchronize()
    for name, o in zip(["u", "cv", "p", "c", "dpdT"], outs):
        g = o.cpu().numpy()
        if layout == "batched":  # abar, zbar summed by a warp reduction instead of in species order
            assert np.allclose(r[name], g, rtol=1e-10, atol=0), name
        else:  # the same per-thread sums as the stand-alone kernel
            assert np.array_equal(r[name], g), name


def test_post_burn_steps_keep_parity(ctx, port):
    """The post-burn instantiation of the batched kernel burns exactly as the plain one: same
    statuses, temperatures and timesteps bit for bit, abundances equal up to the division."""
    w = workloads.make("c2", P=512, seed=73)
    a = gpu_burn(ctx, w, "sparse", layout="batched", normalize=True)
    b = gpu_burn(ctx, w, "sparse", layout="batched")
    for i in (1, 2, 3, 4, 5):
        assert np.array_equal(a[i], b[i])
    o = port.burn(w["net"], w["Y"], w["T"], w["rho"], w["dt"], w["hydro_dt"], w["eos"], w["mu"], max_iter=20000)
    check(w, a, o)


def test_batch_launch_post_steps(ctx):
    """nnet_burn_batch (batched and thread layouts) applies the post-burn steps per sub-batch."""
    import torch
    dev = torch.device("cuda:0")
    A = {n: np.asarray(workloads.mass_numbers(n), dtype=np.float64) for n in (14, 86, 87)}
    for layout in ("batched", "thread"):
        ctx.set_layout(layout)
        parts = workloads.make_mixed(900, 74)
        one = []
        for w in parts:
            P = w["T"].size
            one.append(dict(network=w["net"], Y=torch.tensor(w["Y"], device=dev), T=torch.tensor(w["T"], device=dev),
                            rho=torch.tensor(w["rho"], device=dev), dt=torch.tensor(w["dt"], device=dev),
                            hydro_dt=w["hydro_dt"], status=torch.zeros(P, dtype=torch.int32, device=dev),
                            mass_drift=torch.zeros(P, dtype=torch.float64, device=dev),
                            eos_out=[torch.zeros(P, dtype=torch.float64, device=dev) for _ in range(5)]))
        ctx.burn_batch(one, solver="sparse", max_iter=20000, normalize_mass=True)
        torch.cuda.synchronize()
        ctx.set_layout("auto")
        for w, b in zip(parts, one):
            Y = b["Y"].cpu().numpy()
            burned = b["status"].cpu().numpy() != 1
            s = (A[w["net"]][: Y.shape[0], None] * Y).sum(0)
            assert np.abs(s[burned] - 1).max() <= SUM_X_TOL, (layout, w["net"])
            assert np.all(np.isfinite(b["mass_drift"].cpu().numpy()))
            assert np.all(b["eos_out"][1].cpu().numpy() > 0)  # cv
