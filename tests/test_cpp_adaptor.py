"""The C++ drop-in header compiles against a reference-shaped Data type and links to the
library (compile/link only: no GPU compute runs here)."""
import os
import subprocess
import tempfile

from conftest import PKG, REPO

SRC = r"""
#include <vector>
#include "nnet_gb300_parallel.hpp"
struct DevData { std::vector<std::vector<double>> Y; std::vector<double> temp, rho, rho_m1, dt, u, cv, p, c, dpdT; };
struct Data { DevData devData; };
int main(int argc, char**) {
    if (argc < 2) return 0; // linked, not run: compute needs a GPU
    Data n;
    n.devData.Y.assign(86, std::vector<double>(4));
    for (auto* v : {&n.devData.temp, &n.devData.rho, &n.devData.rho_m1, &n.devData.dt}) v->resize(4);
    nnet_gb300::parallel::computeNuclearReactions<true>(n, 0, 4, 1e-4, 1e-4, nnet_gb300::net86::reactionList,
        nnet_gb300::net86::computeReactionRates, nnet_gb300::HelmholtzFunctor<double>{}, false);
    nnet_gb300::parallel::computeNuclearReactions<true>(n, 0, 4, 1e-4, 1e-4, nnet_gb300::net86::reactionList,
        nnet_gb300::net86::computeReactionRates, nnet_gb300::IdealGasFunctor<double>(10.0), true);
    std::vector<double> Z(86, 6.);
    nnet_gb300::parallel::computeHelmEOS<true>(n, 0, 4, Z);
    return 0;
}
"""


def test_adaptor_compiles_and_links():
    import nnet_build
    lib = nnet_build.build()
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        open(src, "w").write(SRC)
        exe = os.path.join(d, "t")
        r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(REPO, "include"), src, lib,
                            f"-Wl,-rpath,{PKG}", "-o", exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert subprocess.run([exe]).returncode == 0
