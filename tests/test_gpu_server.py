"""Continuous-batching server: results equal an unsliced burn, and each request's result
is the same alone and in a mix of concurrently running requests of other networks."""
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


def request_arrays(w):
    # fresh copies: the server writes results into the request's host buffers
    return (np.array(w["Y"], order="C", copy=True), w["T"].copy(), w["rho"].copy(), w["dt"].copy(),
            np.zeros(w["T"].size, np.int32))


def run_server(ctx, reqs, slice_iterations=16, solver="mixed"):
    import nnet_gb300 as nn
    srv = nn.Server(ctx, solver=solver, slice_iterations=slice_iterations, max_concurrent_requests=4)
    arrays, ids = [], []
    for w in reqs:
        a = request_arrays(w)
        arrays.append(a)
        ids.append(srv.submit(w["net"], a[0], a[1], a[2], a[3], w["hydro_dt"], eos=w["eos"], mu=w["mu"],
                              status=a[4], max_iter=20000))
    lat = [srv.wait(i) for i in ids]
    st = srv.stats()
    srv.close()
    return arrays, lat, st


def unsliced(ctx, w, solver="mixed"):
    import torch
    dev = torch.device("cuda:0")
    Y = torch.tensor(w["Y"], device=dev)
    T, rho, dt = (torch.tensor(w[k], device=dev) for k in ("T", "rho", "dt"))
    st = torch.zeros(T.numel(), dtype=torch.int32, device=dev)
    ctx.burn(w["net"], Y, T, rho, dt, w["hydro_dt"], eos=w["eos"], mu=w["mu"], solver=solver, status=st,
             max_iter=20000)
    torch.cuda.synchronize()
    return Y.cpu().numpy(), T.cpu().numpy(), dt.cpu().numpy(), st.cpu().numpy()


def test_sliced_equals_unsliced(ctx):
    w = workloads.make("c2", P=2048, seed=31)
    (a,), lat, st = run_server(ctx, [w], slice_iterations=8)
    Y, T, dt, s = unsliced(ctx, w)
    assert np.array_equal(a[0], Y) and np.array_equal(a[1], T) and np.array_equal(a[3], dt)
    assert np.array_equal(a[4], s)
    assert st["slices"] > 2 and st["completed_requests"] == 1


def test_alone_equals_in_mix(ctx):
    target = workloads.make("c2", P=3000, seed=41)
    (alone,), _, _ = run_server(ctx, [target])
    mix = [workloads.make("c1", P=5000, seed=42), target, workloads.make("c4", P=1500, seed=43)]
    mix += [p for p in workloads.make_mixed(4000, 44)]
    arrays, lat, st = run_server(ctx, mix)
    inmix = arrays[1]
    for x, y in zip(alone, inmix):
        assert np.array_equal(x, y)
    assert st["completed_requests"] == len(mix)
    assert st["latency_p99"] >= st["latency_p50"] > 0
