"""Failure detection on the GPU, in forms that fault, trap or hang nothing:

* poisoned inputs (NaN or infinite temperature, NaN abundances or timestep, a zero timestep)
  end with the statuses the reference's own logic gives them: the NaN retry of
  finalizeSystemNR (nuclear_net.hpp:732-741) shrinks dt until it underflows to 0, where the
  reference throws (nuclear_net.hpp:533-549) and the library reports ZERO_DT; a NaN timestep
  repeats its attempt-start state and ends as LIVELOCK, as in the oracle;
* the launch watchdog (nnet_burn_args.time_limit_seconds): a limit that runs out makes the
  launch return promptly with every unfinished particle ABORTED, nnet_get_stats returns
  NNET_ERR_ABORTED, and the context stays usable."""
import numpy as np
import pytest

import workloads
from test_gpu_parity import gpu_burn

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


def _poisoned():
    w = workloads.make("c2", P=64, seed=3)
    Y, T, dt = w["Y"].copy(), w["T"].copy(), w["dt"].copy()
    T[0] = np.nan      # skipped (the temperature test fails)
    Y[3, 1] = np.nan   # one NaN abundance: NaN retries until dt underflows
    dt[2] = 0.0        # zero timestep
    Y[:, 3] = np.nan   # every abundance NaN
    dt[4] = np.nan     # NaN timestep: the attempt-start state repeats
    T[5] = np.inf      # infinite temperature
    w.update(Y=Y, T=T, dt=dt)
    return w


@pytest.mark.parametrize("layout,solver", [("batched", "sparse"), ("batched", "mixed"), ("warp", "sparse"),
                                           ("thread", "sparse"), ("auto", "dense")])
def test_poisoned_inputs_match_oracle(ctx, port, layout, solver):
    w = _poisoned()
    g = gpu_burn(ctx, w, solver, layout=layout)
    ctx.set_layout("auto")
    o = port.burn(w["net"], w["Y"], w["T"], w["rho"], w["dt"], w["hydro_dt"], w["eos"], w["mu"], max_iter=20000)
    ST = {"OK": 0, "SKIPPED": 1, "LIVELOCK": 2, "ZERO_DT": 4}
    assert list(o[3][:6]) == [ST["SKIPPED"], ST["ZERO_DT"], ST["ZERO_DT"], ST["ZERO_DT"], ST["LIVELOCK"],
                              ST["ZERO_DT"]]
    assert np.array_equal(g[3][:6], o[3][:6]), (g[3][:6], o[3][:6])
    assert np.array_equal(g[5][:6], o[5][:6])  # the same number of Newton iterations
    # the healthy particles of the batch are unaffected
    assert (g[3][6:] == o[3][6:]).mean() >= 0.95
    assert ctx.stats()["status"]["ZERO_DT"] == int((g[3] == ST["ZERO_DT"]).sum())


@pytest.mark.parametrize("layout,solver", [("batched", "sparse"), ("warp", "sparse"), ("thread", "mixed"),
                                           ("auto", "dense")])
def test_watchdog_ends_launch(ctx, layout, solver):
    import time
    import torch
    dev = torch.device("cuda:0")
    P = 300000  # more particles than any layout's persistent grid holds at once
    w = workloads.make("c2", P=P, seed=9)
    ctx.set_layout(layout)
    Y, T = torch.tensor(w["Y"], device=dev), torch.tensor(w["T"], device=dev)
    rho, dt = torch.tensor(w["rho"], device=dev), torch.tensor(w["dt"], device=dev)
    st = torch.full((P,), -1, dtype=torch.int32, device=dev)
    it = torch.full((P,), -1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.burn(86, Y, T, rho, dt, w["hydro_dt"], solver=solver, status=st, iterations=it, max_iter=20000,
             time_limit=2e-3)
    s = ctx.stats()  # synchronises
    el = time.perf_counter() - t0
    ctx.set_layout("auto")
    stn, itn = st.cpu().numpy(), it.cpu().numpy()
    assert s["aborted"] and s["status"]["ABORTED"] == int((stn == 5).sum()) > 0
    assert set(np.unique(stn)) <= {0, 2, 3, 4, 5}  # every particle has a status
    assert el < 5.0  # the full burn of these particles takes far longer
    # a particle aborted before it started is untouched
    fresh = (stn == 5) & (itn == 0)
    assert fresh.any()
    assert np.array_equal(T.cpu().numpy()[fresh], w["T"][fresh])
    assert np.array_equal(Y.cpu().numpy()[:, fresh], w["Y"][:, fresh])
    # a particle aborted in progress kept a finite state
    assert np.all(np.isfinite(T.cpu().numpy()))
    # the context is usable afterwards and burns as a fresh context would
    small = workloads.make("c2", P=128, seed=10)
    a = gpu_burn(ctx, small, solver, layout=layout)
    ctx.set_layout("auto")
    assert not ctx.stats()["aborted"]
    import nnet_gb300 as nn
    c2 = nn.Context(0)
    b = gpu_burn(c2, small, solver, layout=layout)
    c2.close()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
