"""The reference-shaped adaptors on the GPU, checked against the oracle.

* C++: a program compiled by nvcc holds an SPH-EXA-like `Data` whose `devData` fields are
  thrust::device_vector<double> (the layout the reference's GPU driver reads,
  parallel_nuclear_net.hpp:63-85) and calls nnet_gb300::parallel::computeNuclearReactions<true>
  and computeHelmEOS<true> (include/nnet_gb300_parallel.hpp) on a sub-range [first, last) of
  the particles, the default context loading the Helmholtz table from NNET_HELM_TABLE.
* Python: compute_nuclear_reactions / compute_helm_eos of nnet_gb300.py on a namespace of
  per-species CUDA tensors."""
import os
import subprocess
import types

import numpy as np
import pytest

import workloads
from conftest import PKG, REPO
from test_gpu_parity import check

pytestmark = pytest.mark.gpu

FIRST = 16  # particles [0, FIRST) lie outside the burned range and must stay untouched

CPP = r"""
#include <cstdio>
#include <fstream>
#include <vector>
#include <thrust/device_vector.h>
#include "nnet_gb300_parallel.hpp"

using DV = thrust::device_vector<double>;
struct DevData { std::vector<DV> Y; DV temp, rho, rho_m1, dt, u, cv, p, c, dpdT; };
struct Data { DevData devData; int numSpecies = 0; };

template<class T> void rd(std::ifstream& f, T* v, size_t n) { f.read(reinterpret_cast<char*>(v), n * sizeof(T)); }
void put(std::ofstream& f, const DV& d) { std::vector<double> h(d.size()); thrust::copy(d.begin(), d.end(), h.begin());
                                          f.write(reinterpret_cast<const char*>(h.data()), h.size() * sizeof(double)); }

int main(int argc, char** argv)
{
    // input: int32 net, int32 P, int32 first, int32 ideal, double mu, double hydro_dt,
    //        Z[net], Y[net][P], T[P], rho[P], dt[P]
    std::ifstream in(argv[1], std::ios::binary);
    int net, P, first, ideal;
    double mu, hydro_dt;
    rd(in, &net, 1), rd(in, &P, 1), rd(in, &first, 1), rd(in, &ideal, 1), rd(in, &mu, 1), rd(in, &hydro_dt, 1);
    std::vector<double> Z(net), Y((size_t)net * P), T(P), rho(P), dt(P);
    rd(in, Z.data(), net), rd(in, Y.data(), Y.size()), rd(in, T.data(), P), rd(in, rho.data(), P), rd(in, dt.data(), P);
    Data n;
    n.numSpecies = net;
    for (int j = 0; j < net; ++j) n.devData.Y.emplace_back(Y.begin() + (size_t)j * P, Y.begin() + (size_t)(j + 1) * P);
    n.devData.temp = T, n.devData.rho = rho, n.devData.dt = dt, n.devData.rho_m1 = DV(P, 0.);
    for (DV* v : {&n.devData.u, &n.devData.cv, &n.devData.p, &n.devData.c, &n.devData.dpdT}) v->assign(P, 0.);

    using namespace nnet_gb300;
    const ReactionListTag& rl = net == 14 ? net14::reactionList : net == 86 ? net86::reactionList : net87::reactionList;
    const RatesTag& rr = net == 14 ? net14::computeReactionRates : net == 86 ? net86::computeReactionRates
                                                                            : net87::computeReactionRates;
    try {
        if (ideal)
            parallel::computeNuclearReactions<true>(n, first, P, hydro_dt, hydro_dt, rl, rr, IdealGasFunctor<double>(mu), false);
        else
            parallel::computeNuclearReactions<true>(n, first, P, hydro_dt, hydro_dt, rl, rr, HelmholtzFunctor<double>{}, false);
        parallel::computeHelmEOS<true>(n, first, P, Z);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 2;
    }
    std::ofstream out(argv[2], std::ios::binary);
    for (int j = 0; j < net; ++j) put(out, n.devData.Y[j]);
    for (const DV* v : {&n.devData.temp, &n.devData.dt, &n.devData.u, &n.devData.cv, &n.devData.p, &n.devData.c,
                        &n.devData.dpdT}) put(out, *v);
    return 0;
}
"""


@pytest.fixture(scope="module")
def cpp_driver(tmp_path_factory):
    import nnet_build
    lib = nnet_build.build()
    d = tmp_path_factory.mktemp("adaptor")
    src, exe = d / "drop_in.cu", d / "drop_in"
    src.write_text(CPP)
    r = subprocess.run([nnet_build._nvcc(), *nnet_build.ARCH, "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                        str(src), lib, "-Xlinker", f"-rpath={PKG}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _run_cpp(exe, tmp_path, w, table):
    import nnet_gb300 as nn
    net, P = w["net"], w["T"].size
    Z = nn.network_charges(net)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([net, P, FIRST, int(w["eos"] == "ideal")], dtype=np.int32).tofile(f)
        np.array([w["mu"], w["hydro_dt"]], dtype=np.float64).tofile(f)
        for a in (Z, w["Y"], w["T"], w["rho"], w["dt"]):
            np.ascontiguousarray(a, dtype=np.float64).tofile(f)
    env = {k: v for k, v in os.environ.items() if k != "NNET_HELM_TABLE"}
    if table:
        env["NNET_HELM_TABLE"] = table
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True, env=env)
    if r.returncode:
        return r
    v = np.fromfile(out, dtype=np.float64)
    Y = v[: net * P].reshape(net, P)
    rest = v[net * P:].reshape(7, P)
    return dict(Y=Y, T=rest[0], dt=rest[1], u=rest[2], cv=rest[3], p=rest[4], c=rest[5], dpdT=rest[6], Z=Z)


@pytest.mark.parametrize("name,P", [("c2", 256), ("c1", 512)])
def test_cpp_drop_in_thrust_data(cpp_driver, tmp_path, port, name, P):
    import nnet_gb300 as nn
    w = workloads.make(name, P=P, seed=80 + P)
    r = _run_cpp(cpp_driver, tmp_path, w, nn.HELM_TABLE_PATH)
    assert isinstance(r, dict), r.stderr
    s = slice(FIRST, P)
    # outside [first, last): untouched
    assert np.array_equal(r["Y"][:, :FIRST], w["Y"][:, :FIRST]) and np.array_equal(r["T"][:FIRST], w["T"][:FIRST])
    o = port.burn(w["net"], w["Y"][:, s], w["T"][s], w["rho"][s], w["dt"][s], w["hydro_dt"], w["eos"], w["mu"],
                  max_iter=100000)
    sub = dict(w, Y=w["Y"][:, s], T=w["T"][s], rho=w["rho"][s], dt=w["dt"][s])
    check(sub, (r["Y"][:, s], r["T"][s], r["dt"][s], o[3]), o)  # the adaptor returns no statuses
    ref = port.helm_eos_batch(r["Z"], r["T"][s], w["rho"][s], r["Y"][:, s])
    for k in ("u", "cv", "p", "c", "dpdT"):
        assert np.max(np.abs(r[k][s] - ref[k]) / np.abs(ref[k])) < 1e-9, k


def test_cpp_drop_in_without_table_says_how(cpp_driver, tmp_path):
    w = workloads.make("c2", P=64, seed=5)
    r = _run_cpp(cpp_driver, tmp_path, w, None)
    assert not isinstance(r, dict) and r.returncode == 2
    assert "NNET_HELM_TABLE" in r.stderr and "defaultContext" in r.stderr


def test_python_adaptors(port):
    import torch
    import nnet_gb300 as nn
    dev = torch.device("cuda:0")
    w = workloads.make("c2", P=200, seed=90)
    P = w["T"].size
    n = types.SimpleNamespace(Y=[torch.tensor(w["Y"][j], device=dev) for j in range(86)],
                              temp=torch.tensor(w["T"], device=dev), rho=torch.tensor(w["rho"], device=dev),
                              rho_m1=torch.zeros(P, dtype=torch.float64, device=dev),
                              dt=torch.tensor(w["dt"], device=dev),
                              **{k: torch.zeros(P, dtype=torch.float64, device=dev) for k in ("u", "cv", "p", "c", "dpdT")})
    nn.compute_nuclear_reactions(n, FIRST, P, w["hydro_dt"], w["hydro_dt"], nn.net86_reactionList,
                                 nn.net86_computeReactionRates, nn.HelmholtzFunctor(86), use_drhodt=False)
    Z = nn.network_charges(86)
    nn.compute_helm_eos(n, FIRST, P, Z)
    torch.cuda.synchronize()
    Y = torch.stack(n.Y).cpu().numpy()
    T, dt = n.temp.cpu().numpy(), n.dt.cpu().numpy()
    s = slice(FIRST, P)
    assert np.array_equal(Y[:, :FIRST], w["Y"][:, :FIRST]) and np.array_equal(T[:FIRST], w["T"][:FIRST])
    o = port.burn(86, w["Y"][:, s], w["T"][s], w["rho"][s], w["dt"][s], w["hydro_dt"], "helmholtz", 0.0,
                  max_iter=100000)
    sub = dict(w, Y=w["Y"][:, s], T=w["T"][s], rho=w["rho"][s], dt=w["dt"][s])
    check(sub, (Y[:, s], T[s], dt[s], o[3]), o)
    ref = port.helm_eos_batch(Z, T[s], w["rho"][s], Y[:, s])
    for k in ("u", "cv", "p", "c", "dpdT"):
        g = getattr(n, k).cpu().numpy()[s]
        assert np.max(np.abs(g - ref[k]) / np.abs(ref[k])) < 1e-9, k
    with pytest.raises(nn.NnetError):  # the library has no CPU path
        nn.compute_nuclear_reactions(types.SimpleNamespace(Y=[torch.zeros(4, dtype=torch.float64)] * 86,
                                                           temp=torch.zeros(4, dtype=torch.float64),
                                                           rho=torch.zeros(4, dtype=torch.float64),
                                                           dt=torch.zeros(4, dtype=torch.float64)),
                                     0, 4, 1e-4, 1e-4, nn.net86_reactionList, nn.net86_computeReactionRates,
                                     nn.HelmholtzFunctor(86), context=nn.default_context(0))
