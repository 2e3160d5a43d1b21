"""The warp plan on the CPU, for net14, net86 and net87: the ordering's level count, fill and
multiply-adds are pinned; the level-scheduled LU (reciprocals folded into the multiplier
round, forward substitution folded into the factorisation, one-round backward levels),
executed round by round with every lane reading the round's starting values, must equal the
plain sequential elimination; and the fixed-order gathers must reproduce the reaction-list
scatters of dY/dt and of the Jacobian."""
import os
import subprocess
import tempfile

from conftest import PKG

SRC = r"""
#include "sparse_plan.hpp"
#include "nnet_network_tables.h"
#include <cmath>
#include <cstdio>
#include <random>
using namespace nnet_gb300;
int main() {
  struct { int net; const int *rb, *rs, *rc, *pb, *ps, *pc; int R, cap; } nets[3] = {
    {14, net14_reactant_begin, net14_reactant_species, net14_reactant_count, net14_product_begin,
     net14_product_species, net14_product_count, NET14_NUM_REACTIONS, kWarpNnzCap14},
    {86, net86_reactant_begin, net86_reactant_species, net86_reactant_count, net86_product_begin,
     net86_product_species, net86_product_count, NET86_NUM_REACTIONS, kWarpNnzCap86},
    {87, net87_reactant_begin, net87_reactant_species, net87_reactant_count, net87_product_begin,
     net87_product_species, net87_product_count, NET87_NUM_REACTIONS, kWarpNnzCap86}};
  int bad = 0;
  for (auto& t : nets) {
    SparsePlan P = buildSparsePlan(t.net, t.rb, t.rs, t.rc, t.pb, t.ps, t.pc, t.R);
    WarpPlan W = buildWarpPlan(P, t.rb, t.rs, t.rc, t.pb, t.ps, t.pc, t.cap);
    const int n = P.n, N = P.N;
    if (P.nnz > t.cap) { printf("net%d: factor exceeds capacity\n", t.net); return 1; }
    // the ordering's figures: minimum degree with ties broken by elimination level (with ties
    // broken by index, net86 / net87 had the same fill and multiply-adds in 38 levels)
    const int  expLevels = t.net == 14 ? 13 : 18, expNnz = t.net == 14 ? 98 : t.net == 86 ? 1044 : 1051;
    const long expFma    = t.net == 14 ? 129 : t.net == 86 ? 2745 : 2754;
    if (W.nLevels != expLevels || P.nnz != expNnz || P.factorFma != expFma) {
      printf("net%d: plan has %d levels, %d entries, %lld multiply-adds\n", t.net, W.nLevels, P.nnz, P.factorFma);
      ++bad;
    }
    std::mt19937_64 g(5); std::uniform_real_distribution<double> u(0.1, 1);
    std::vector<double> A0(P.nnz), b(n);
    for (auto& v : A0) v = u(g) * 0.01;
    for (int k = 0; k < n; ++k) A0[P.kPiv[k]] = 5 + u(g);
    for (auto& v : b) v = u(g);
    // sequential right-looking elimination and triangular solves
    std::vector<double> A = A0, ip(n), x = b;
    for (int k = 0; k < n; ++k) {
      ip[k] = 1 / A[P.kPiv[k]];
      for (int e = P.lBeg[k]; e < P.lBeg[k + 1]; ++e) {
        const double l = A[P.lPos[e]] * ip[k]; A[P.lPos[e]] = l;
        for (int q = P.uBeg[k]; q < P.uBeg[k + 1]; ++q) A[P.tPos[P.tBeg[e] + q - P.uBeg[k]]] -= l * A[P.uPos[q]];
      }
    }
    for (int k = 0; k < n; ++k) for (int e = P.lBeg[k]; e < P.lBeg[k + 1]; ++e) x[P.lRow[e]] -= A[P.lPos[e]] * x[k];
    for (int k = n - 1; k >= 0; --k) {
      double s = x[k];
      for (int q = P.uBeg[k]; q < P.uBeg[k + 1]; ++q) s -= A[P.uPos[q]] * x[P.uCol[q]];
      x[k] = s * ip[k];
    }
    // fused level schedule, each round reading the values at its start
    std::vector<double> M(t.cap + n, 0.), ipl(n, -1.);
    for (int p = 0; p < P.nnz; ++p) M[p] = A0[p];
    for (int i = 0; i < n; ++i) M[t.cap + i] = b[i];
    for (int l = 0; l < W.nLevels; ++l) {
      std::vector<double> c = M;
      for (int e = W.scBeg[l]; e < W.scBeg[l + 1]; ++e) {
        const double iv = 1 / c[P.kPiv[W.scPiv[e]]];
        if (W.scPos[e] >= 0) M[W.scPos[e]] = c[W.scPos[e]] * iv;
        ipl[W.scPiv[e]] = iv;
      }
      c = M;
      for (int r = W.tgBegA[l]; r < W.tgBegA[l + 1]; ++r) {
        double a = c[W.tgPosA[r]];
        for (int q = W.tgUpdA[r]; q < W.tgUpdA[r + 1]; ++q) a -= c[W.tuLA[q]] * c[W.tuUA[q]];
        M[W.tgPosA[r]] = a;
      }
    }
    std::vector<double> y(M.begin() + t.cap, M.end()), xo(n, 0.);
    for (int li = 0; li < W.nLevels; ++li) {
      const int l = W.nLevels - 1 - li;
      std::vector<double> c = y;
      for (int q = W.lvBeg[l]; q < W.lvBeg[l + 1]; ++q) xo[W.lvPiv[q]] = c[W.lvPiv[q]] * ipl[W.lvPiv[q]];
      for (int r = W.bwBeg[li]; r < W.bwBeg[li + 1]; ++r) {
        double a = c[W.bwRow[r]];
        for (int e = W.bwEnt[r]; e < W.bwEnt[r + 1]; ++e) a -= M[W.buPos[e]] * (c[W.buK[e]] * ipl[W.buK[e]]);
        y[W.bwRow[r]] = a;
      }
    }
    double dx = 0;
    for (int k = 0; k < n; ++k) dx = std::fmax(dx, std::fabs(x[k] - xo[k]) / std::fabs(x[k]));
    // gathers against scatters
    std::vector<double> f(t.R), ds(N, 0.), dg(N, 0.);
    for (auto& v : f) v = u(g);
    for (int r = 0; r < t.R; ++r) {
      for (int k = t.rb[r]; k < t.rb[r + 1]; ++k) ds[t.rs[k]] -= f[r] * t.rc[k];
      for (int k = t.pb[r]; k < t.pb[r + 1]; ++k) ds[t.ps[k]] += f[r] * t.pc[k];
    }
    for (int s = 0; s < N; ++s) for (int k = W.sgBeg[s]; k < W.sgBeg[s + 1]; ++k) dg[s] += W.sgCoef[k] * f[W.sgRx[k]];
    const int NE = t.rb[t.R];
    std::vector<double> tr(NE), Js(P.nnz, 0.), Jg(P.nnz, 0.);
    for (auto& v : tr) v = u(g);
    for (int e = 0; e < NE; ++e) for (int c = P.cBeg[e]; c < P.cBeg[e + 1]; ++c) Js[P.cPos[c]] += tr[e] * P.cCoef[c];
    for (size_t m = 0; m < W.jPos.size(); ++m)
      for (int k = W.jgBeg[m]; k < W.jgBeg[m + 1]; ++k) Jg[W.jPos[m]] += W.jgCoef[k] * tr[W.jgEnt[k]];
    double dsg = 0, dj = 0;
    for (int s = 0; s < N; ++s) dsg = std::fmax(dsg, std::fabs(ds[s] - dg[s]) / (std::fabs(ds[s]) + 1));
    for (int p = 0; p < P.nnz; ++p) dj = std::fmax(dj, std::fabs(Js[p] - Jg[p]) / (std::fabs(Js[p]) + 1));
    // every species and J row appears once in the lane orders
    std::vector<int> seenS(N, 0), seenR(N, 0);
    for (int s : W.sgOrder) seenS[s]++;
    for (int i : W.rjOrder) seenR[i]++;
    for (int i = 0; i < N; ++i) bad += seenS[i] != 1 || seenR[i] != 1;
    // the per-lane op streams of the fused factorisation carry, for every target of a level,
    // exactly its update list in order, on one lane, contiguously
    long opRows = 0;
    for (int l = 0; l < W.nLevels; ++l) {
      const int rows = W.foBeg[l + 1] - W.foBeg[l];
      opRows += rows;
      std::vector<int> seen(W.tgBegA[l + 1] - W.tgBegA[l], 0);
      int busiest = 0;
      for (int q = 0; q < 32; ++q) {
        int cur = -1, next = 0, used = 0;
        for (int k = 0; k < rows; ++k) {
          const unsigned long long o = W.fOps[(size_t)(W.foBeg[l] + k) * 32 + q];
          if (!(o & WarpPlan::kOpValid)) { bad += cur >= 0; cur = -2; continue; }
          bad += cur == -2;  // no op before the end of a lane's stream
          ++used;
          const int L = o & 0xffff, U = (o >> 16) & 0xffff, pos = (o >> 32) & 0xffff;
          if (o & WarpPlan::kOpFirst) {
            bad += cur >= 0;
            cur = -1;
            for (int t2 = W.tgBegA[l]; t2 < W.tgBegA[l + 1]; ++t2) if (W.tgPosA[t2] == pos) cur = t2;
            if (cur < 0) { ++bad; break; }
            seen[cur - W.tgBegA[l]]++, next = W.tgUpdA[cur];
          }
          if (cur < 0 || next >= W.tgUpdA[cur + 1] || W.tuLA[next] != L || W.tuUA[next] != U || W.tgPosA[cur] != pos) { ++bad; break; }
          ++next;
          if (o & WarpPlan::kOpLast) { bad += next != W.tgUpdA[cur + 1]; cur = -1; }
        }
        busiest = busiest > used ? busiest : used;
      }
      for (int v : seen) bad += v != 1;
      bad += busiest != rows;
    }
    printf("net%d levels %d op rows %ld solve %.2e gathers %.2e %.2e\n", t.net, W.nLevels, opRows, dx, dsg, dj);
    bad += !(dx < 1e-13 && dsg < 1e-14 && dj < 1e-14);
  }
  return bad;
}
"""


def test_level_schedule_and_gathers():
    csrc = os.path.join(PKG, "csrc")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        open(src, "w").write(SRC)
        exe = os.path.join(d, "t")
        r = subprocess.run(["g++", "-O1", "-std=c++17", "-I", csrc, "-I", os.path.join(PKG, "data"), src,
                            os.path.join(csrc, "sparse_plan.cpp"), "-o", exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout
