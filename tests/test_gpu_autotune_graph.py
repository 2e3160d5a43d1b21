"""Autotuner on the device, and the burn captured in a CUDA graph."""
import numpy as np
import pytest

import workloads

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


def test_autotune_choice_and_cache(ctx, port, tmp_path):
    import torch
    import autotune
    from test_gpu_parity import check, gpu_burn
    w = workloads.make("c2", P=2048, seed=12)
    dev = torch.device("cuda:0")
    Y, T = torch.tensor(w["Y"], device=dev), torch.tensor(w["T"], device=dev)
    rho, dt = torch.tensor(w["rho"], device=dev), torch.tensor(w["dt"], device=dev)
    path = str(tmp_path / "cache.json")
    c1 = autotune.tune(ctx, 86, Y, T, rho, dt, w["hydro_dt"], eos=1, solver=1, max_iter=20000, cache_path=path)
    assert (c1["layout"], c1["slots"]) in autotune.CANDIDATES and len(c1["timings"]) == len(autotune.CANDIDATES)
    assert np.array_equal(Y.cpu().numpy(), w["Y"]) and np.array_equal(T.cpu().numpy(), w["T"])  # untouched
    c2 = autotune.tune(ctx, 86, Y, T, rho, dt, w["hydro_dt"], eos=1, solver=1, max_iter=20000, cache_path=path)
    assert c2 == c1  # served from the cache
    # the tuned context burns correctly (layout as chosen)
    g = gpu_burn(ctx, w, "sparse", layout=c1["layout"])
    o = port.burn(86, w["Y"], w["T"], w["rho"], w["dt"], w["hydro_dt"], "helmholtz", 0.0, max_iter=20000)
    check(w, g, o)
    ctx.set_layout("auto")
    ctx.set_batch_slots(32)


def test_burn_in_cuda_graph(ctx):
    """State restore + burn captured once in a CUDA graph and replayed twice gives the
    eager burn's results bit for bit (the workspace is sized by an eager call first)."""
    import torch
    import nnet_gb300 as nn
    w = workloads.make("c2", P=1024, seed=13)
    dev = torch.device("cuda:0")
    Y0, T0 = torch.tensor(w["Y"], device=dev), torch.tensor(w["T"], device=dev)
    rho, dt0 = torch.tensor(w["rho"], device=dev), torch.tensor(w["dt"], device=dev)
    Y, T, dt = Y0.clone(), T0.clone(), dt0.clone()
    st = torch.zeros(1024, dtype=torch.int32, device=dev)
    kw = dict(eos=nn.EOS_HELMHOLTZ, solver=nn.SOLVER_SPARSE_FP64, status=st, max_iter=20000)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx.burn(86, Y, T, rho, dt, w["hydro_dt"], stream=s, **kw)  # eager: sizes the workspace
    torch.cuda.synchronize()
    ref = (Y.cpu().numpy(), T.cpu().numpy(), dt.cpu().numpy(), st.cpu().numpy())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        Y.copy_(Y0), T.copy_(T0), dt.copy_(dt0)
        ctx.burn(86, Y, T, rho, dt, w["hydro_dt"], stream=s, **kw)
    for _ in range(2):
        Y.zero_(), T.zero_()
        g.replay()
        torch.cuda.synchronize()
        got = (Y.cpu().numpy(), T.cpu().numpy(), dt.cpu().numpy(), st.cpu().numpy())
        for a, b in zip(ref, got):
            assert np.array_equal(a, b)


def test_cost_order_is_a_costliest_first_permutation_and_keeps_results(ctx):
    """nnet_cost_order gives a permutation in decreasing power-of-two cost classes; a burn in
    that visiting order gives the same per-particle results bit for bit."""
    import torch
    from test_gpu_parity import gpu_burn
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(3)
    cost = torch.tensor(rng.integers(0, 5000, 100003), dtype=torch.int32, device=dev)
    order = ctx.cost_order(cost).cpu().numpy()
    c = cost.cpu().numpy()
    assert np.array_equal(np.sort(order), np.arange(c.size))
    cls = np.floor(np.log2(np.maximum(c[order], 1)))
    assert np.all(np.diff(cls) <= 0)
    w = workloads.make("c2", P=2000, seed=31)
    a = gpu_burn(ctx, w, "sparse")
    o = ctx.cost_order(torch.tensor(a[5], device=dev))
    Y, T = torch.tensor(w["Y"], device=dev), torch.tensor(w["T"], device=dev)
    rho, dt = torch.tensor(w["rho"], device=dev), torch.tensor(w["dt"], device=dev)
    st = torch.zeros(2000, dtype=torch.int32, device=dev)
    ctx.burn(86, Y, T, rho, dt, w["hydro_dt"], solver="sparse", status=st, max_iter=20000, order=o)
    torch.cuda.synchronize()
    assert np.array_equal(Y.cpu().numpy(), a[0]) and np.array_equal(T.cpu().numpy(), a[1])
    assert np.array_equal(st.cpu().numpy(), a[3])
