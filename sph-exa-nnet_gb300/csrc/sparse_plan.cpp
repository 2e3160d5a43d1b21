// Symbolic analysis for the sparse solver forms (see sparse_plan.hpp).
#include "sparse_plan.hpp"

#include <algorithm>
#include <map>
#include <set>

namespace nnet_gb300
{

SparsePlan buildSparsePlan(int net, const int* rbeg, const int* rspec, const int* rcnt, const int* pbeg,
                           const int* pspec, const int* pcnt, int R)
{
    SparsePlan P;
    const int  N = net, n = N + 1;
    P.N = N, P.n = n, P.R = R;

    // ---- structural pattern in the reference's indexing (0 = T, 1 + species)
    std::set<std::pair<int, int>> S;
    for (int i = 0; i < n; ++i)
        S.insert({0, i}), S.insert({i, 0}), S.insert({i, i});
    for (int r = 0; r < R; ++r)
        for (int e = rbeg[r]; e < rbeg[r + 1]; ++e)
        {
            const int id = rspec[e];
            for (int o = rbeg[r]; o < rbeg[r + 1]; ++o)
                S.insert({rspec[o] + 1, id + 1});
            for (int o = pbeg[r]; o < pbeg[r + 1]; ++o)
                S.insert({pspec[o] + 1, id + 1});
        }

    // ---- greedy minimum degree on the symmetrised graph.  Ties go to the node of the lowest
    //      elimination level (one more than the deepest eliminated node it depends on), then
    //      to the lowest index: the fill is that of any minimum-degree choice, but the nodes
    //      of equal degree along the alpha-chain are taken from independent parts of the graph
    //      instead of one after the other, so the level schedule of the warp kernels is short
    //      (net86: 18 levels instead of 38, same 1,044 entries and 2,745 multiply-adds).
    std::vector<std::set<int>> adj(n);
    for (auto [i, j] : S)
        if (i != j) adj[i].insert(j), adj[j].insert(i);
    std::vector<char> alive(n, 1);
    std::vector<int>  depth(n, 0);
    for (int step = 0; step < n; ++step)
    {
        int v = -1;
        for (int x = 0; x < n; ++x)
            if (alive[x] && (v < 0 || adj[x].size() < adj[v].size() ||
                             (adj[x].size() == adj[v].size() && depth[x] < depth[v])))
                v = x;
        P.perm.push_back(v);
        std::set<int> nb = adj[v];
        for (int a : nb)
        {
            for (int b : nb)
                if (b != a) adj[a].insert(b);
            adj[a].erase(v);
            depth[a] = std::max(depth[a], depth[v] + 1);
        }
        alive[v] = 0;
        adj[v].clear();
    }
    P.iperm.assign(n, 0);
    for (int k = 0; k < n; ++k)
        P.iperm[P.perm[k]] = k;

    // ---- symbolic right-looking elimination in the new order
    std::vector<std::set<int>> rows(n);
    for (auto [i, j] : S)
        rows[P.iperm[i]].insert(P.iperm[j]);
    for (int k = 0; k < n; ++k)
    {
        std::vector<int> U;
        for (int j : rows[k])
            if (j > k) U.push_back(j);
        for (int i = k + 1; i < n; ++i)
            if (rows[i].count(k))
                for (int j : U)
                    rows[i].insert(j);
    }
    std::map<std::pair<int, int>, int> pos;
    for (int i = 0; i < n; ++i)
        for (int j : rows[i])
        {
            pos[{i, j}] = (int)P.posRow.size();
            P.posRow.push_back(i), P.posCol.push_back(j);
        }
    P.nnz = (int)P.posRow.size();
    P.rowBeg.assign(n + 1, 0);
    for (int p = 0; p < P.nnz; ++p)
        P.rowBeg[P.posRow[p] + 1] = p + 1;
    for (int i = 0; i < n; ++i)
        P.rowBeg[i + 1] = std::max(P.rowBeg[i + 1], P.rowBeg[i]);

    // ---- factorisation and solve programs
    P.lBeg.push_back(0), P.uBeg.push_back(0);
    for (int k = 0; k < n; ++k)
    {
        P.kPiv.push_back(pos.at({k, k}));
        std::vector<int> U;
        for (int j : rows[k])
            if (j > k) U.push_back(j);
        for (int j : U)
            P.uPos.push_back(pos.at({k, j})), P.uCol.push_back(j);
        P.uBeg.push_back((int)P.uPos.size());
        for (int i = k + 1; i < n; ++i)
            if (rows[i].count(k))
            {
                P.lPos.push_back(pos.at({i, k})), P.lRow.push_back(i);
                P.tBeg.push_back((int)P.tPos.size());
                for (int j : U)
                    P.tPos.push_back(pos.at({i, j}));
                P.factorFma += (long long)U.size();
            }
        P.lBeg.push_back((int)P.lPos.size());
    }
    P.solveFma = (long long)P.lPos.size() + (long long)P.uPos.size();

    // ---- assembly maps
    for (int i = 0; i < N; ++i)
    {
        const int ni = P.iperm[i + 1];
        P.diagPos.push_back(pos.at({ni, ni}));
        P.col0Pos.push_back(pos.at({ni, P.iperm[0]}));
        P.row0Pos.push_back(pos.at({P.iperm[0], ni}));
    }
    P.pos00 = pos.at({P.iperm[0], P.iperm[0]});
    P.cBeg.push_back(0);
    for (int r = 0; r < R; ++r)
        for (int e = rbeg[r]; e < rbeg[r + 1]; ++e)
        {
            const int col = P.iperm[rspec[e] + 1];
            for (int o = rbeg[r]; o < rbeg[r + 1]; ++o)
            {
                P.cPos.push_back(pos.at({P.iperm[rspec[o] + 1], col}));
                P.cRow.push_back(rspec[o]);
                P.cCoef.push_back(-(double)rcnt[o]);
            }
            for (int o = pbeg[r]; o < pbeg[r + 1]; ++o)
            {
                P.cPos.push_back(pos.at({P.iperm[pspec[o] + 1], col}));
                P.cRow.push_back(pspec[o]);
                P.cCoef.push_back((double)pcnt[o]);
            }
            P.cBeg.push_back((int)P.cPos.size());
        }
    const int t = P.iperm[0];
    for (int p = 0; p < P.nnz; ++p)
        if (P.posRow[p] != t && P.posCol[p] != t)
        {
            P.sbPos.push_back(p);
            P.sbDiag.push_back(P.posRow[p] == P.posCol[p] ? 1 : 0);
        }
    return P;
}

} // namespace nnet_gb300

namespace nnet_gb300
{

namespace
{
using Lists = std::map<int, std::vector<std::pair<int, int>>>;

// A level's targets in the order the lanes take them: longest update lists first, so that
// the 32 lanes of one round carry chains of similar length (ties by position).  The order
// of the updates within a target is unchanged.
std::vector<std::pair<int, const std::vector<std::pair<int, int>>*>> longestFirst(const Lists& m)
{
    std::vector<std::pair<int, const std::vector<std::pair<int, int>>*>> v;
    for (auto& [t, lst] : m)
        v.push_back({t, &lst});
    std::stable_sort(v.begin(), v.end(), [](auto& a, auto& b) { return a.second->size() > b.second->size(); });
    return v;
}

void buildLevels(const SparsePlan& P, WarpPlan& W, int rhsBase)
{
    const int        n = P.n;
    std::vector<int> lev(n, 0);
    for (int k = 0; k < n; ++k)
    {
        int l = 0;
        for (int p = P.rowBeg[k]; p < P.rowBeg[k + 1]; ++p)
            if (P.posCol[p] < k) l = std::max(l, lev[P.posCol[p]] + 1);
        for (int p = 0; p < P.nnz; ++p)
            if (P.posCol[p] == k && P.posRow[p] < k) l = std::max(l, lev[P.posRow[p]] + 1);
        lev[k] = l;
    }
    const int nl = n ? *std::max_element(lev.begin(), lev.end()) + 1 : 0;
    W.nLevels    = nl;
    std::vector<std::vector<int>> piv(nl);
    for (int k = 0; k < n; ++k)
        piv[lev[k]].push_back(k);
    W.lvBeg = {0}, W.lsBeg = {0}, W.tgBeg = {0}, W.tgUpd = {0}, W.fwBeg = {0}, W.fwEnt = {0};
    for (int l = 0; l < nl; ++l)
    {
        std::map<int, std::vector<std::pair<int, int>>> tgt; // target -> (L pos, U pos), pivot order
        std::map<int, std::vector<std::pair<int, int>>> fw;  // row -> (L pos, pivot)
        for (int k : piv[l])
        {
            W.lvPiv.push_back(k);
            for (int e = P.lBeg[k]; e < P.lBeg[k + 1]; ++e)
            {
                W.lsPos.push_back(P.lPos[e]), W.lsPiv.push_back(k);
                fw[P.lRow[e]].push_back({P.lPos[e], k});
                for (int u = P.uBeg[k]; u < P.uBeg[k + 1]; ++u)
                    tgt[P.tPos[P.tBeg[e] + (u - P.uBeg[k])]].push_back({P.lPos[e], P.uPos[u]});
            }
        }
        for (auto& [t, lp] : longestFirst(tgt))
        {
            auto& lst = *lp;
            W.tgPos.push_back(t);
            for (auto& pr : lst)
                W.tuL.push_back(pr.first), W.tuU.push_back(pr.second);
            W.tgUpd.push_back((int)W.tuL.size());
        }
        for (auto& [r, lp] : longestFirst(fw))
        {
            auto& lst = *lp;
            W.fwRow.push_back(r);
            for (auto& pr : lst)
                W.flPos.push_back(pr.first), W.flK.push_back(pr.second);
            W.fwEnt.push_back((int)W.flPos.size());
        }
        W.lvBeg.push_back((int)W.lvPiv.size());
        W.lsBeg.push_back((int)W.lsPos.size());
        W.tgBeg.push_back((int)W.tgPos.size());
        W.fwBeg.push_back((int)W.fwRow.size());
    }
    // fused scaling and augmented factorisation
    W.rhsBase = rhsBase;
    W.scBeg = {0}, W.tgBegA = {0}, W.tgUpdA = {0};
    for (int l = 0; l < nl; ++l)
    {
        std::map<int, std::vector<std::pair<int, int>>> tgt;
        for (int k : piv[l])
        {
            if (P.lBeg[k] == P.lBeg[k + 1]) W.scPos.push_back(-1), W.scPiv.push_back(k);
            for (int e = P.lBeg[k]; e < P.lBeg[k + 1]; ++e)
            {
                W.scPos.push_back(P.lPos[e]), W.scPiv.push_back(k);
                for (int u = P.uBeg[k]; u < P.uBeg[k + 1]; ++u)
                    tgt[P.tPos[P.tBeg[e] + (u - P.uBeg[k])]].push_back({P.lPos[e], P.uPos[u]});
                tgt[rhsBase + P.lRow[e]].push_back({P.lPos[e], rhsBase + k});
            }
        }
        for (auto& [t, lp] : longestFirst(tgt))
        {
            auto& lst = *lp;
            W.tgPosA.push_back(t);
            for (auto& pr : lst)
                W.tuLA.push_back(pr.first), W.tuUA.push_back(pr.second);
            W.tgUpdA.push_back((int)W.tuLA.size());
        }
        W.scBeg.push_back((int)W.scPos.size());
        W.tgBegA.push_back((int)W.tgPosA.size());
    }
    // the same updates as one stream of ops per lane and level: the level's targets (longest
    // list first) each go to the lane with the fewest updates so far, so a level takes as many
    // rounds as its busiest lane has updates, instead of the sum over its rounds of 32 targets
    // of their longest list; a target keeps its updates in pivot order on one lane.
    W.foBeg = {0};
    for (int l = 0; l < nl; ++l)
    {
        std::vector<std::vector<unsigned long long>> lane(32);
        std::vector<int>                             load(32, 0);
        for (int t = W.tgBegA[l]; t < W.tgBegA[l + 1]; ++t)
        {
            const int q  = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            const int u0 = W.tgUpdA[t], u1 = W.tgUpdA[t + 1];
            for (int u = u0; u < u1; ++u)
                lane[q].push_back(WarpPlan::factorOp(W.tuLA[u], W.tuUA[u], W.tgPosA[t], u == u0, u == u1 - 1));
            load[q] += u1 - u0;
        }
        const int rows = *std::max_element(load.begin(), load.end());
        for (int k = 0; k < rows; ++k)
            for (int q = 0; q < 32; ++q)
                W.fOps.push_back(k < (int)lane[q].size() ? lane[q][k] : 0ull);
        W.foBeg.push_back(W.foBeg.back() + rows);
    }
    // backward: levels last to first; rows above the level's pivots, by U column
    W.bwBeg = {0}, W.bwEnt = {0};
    for (int l = nl - 1; l >= 0; --l)
    {
        std::map<int, std::vector<std::pair<int, int>>> bw; // row i -> (U pos of (i, k), k)
        for (int k : piv[l])
            for (int q = W.ucBeg[k]; q < W.ucBeg[k + 1]; ++q)
                bw[W.ucRow[q]].push_back({W.ucPos[q], k});
        for (auto& [r, lp] : longestFirst(bw))
        {
            auto& lst = *lp;
            W.bwRow.push_back(r);
            for (auto& pr : lst)
                W.buPos.push_back(pr.first), W.buK.push_back(pr.second);
            W.bwEnt.push_back((int)W.buPos.size());
        }
        W.bwBeg.push_back((int)W.bwRow.size());
    }
}
} // namespace

WarpPlan buildWarpPlan(const SparsePlan& P, const int* rbeg, const int* rspec, const int* rcnt, const int* pbeg,
                       const int* pspec, const int* pcnt, int rhsBase)
{
    WarpPlan  W;
    const int n = P.n, N = P.N, R = P.R;
    // flat factorisation updates
    W.updBeg.push_back(0);
    for (int k = 0; k < n; ++k)
    {
        const int nu = P.uBeg[k + 1] - P.uBeg[k];
        for (int e = P.lBeg[k]; e < P.lBeg[k + 1]; ++e)
            for (int u = 0; u < nu; ++u)
            {
                W.updT.push_back(P.tPos[P.tBeg[e] + u]);
                W.updL.push_back(P.lPos[e]);
                W.updU.push_back(P.uPos[P.uBeg[k] + u]);
            }
        W.updBeg.push_back((int)W.updT.size());
    }
    // U by columns
    std::vector<std::vector<std::pair<int, int>>> cols(n);
    for (int k = 0; k < n; ++k)
        for (int u = P.uBeg[k]; u < P.uBeg[k + 1]; ++u)
            cols[P.uCol[u]].push_back({P.uPos[u], k});
    W.ucBeg.push_back(0);
    for (int c = 0; c < n; ++c)
    {
        for (auto& pr : cols[c])
            W.ucPos.push_back(pr.first), W.ucRow.push_back(pr.second);
        W.ucBeg.push_back((int)W.ucPos.size());
    }
    // species gathers (reactant: -count, product: +count), in reaction order
    std::vector<std::vector<std::pair<int, double>>> sg(N);
    for (int r = 0; r < R; ++r)
    {
        for (int k = rbeg[r]; k < rbeg[r + 1]; ++k)
            sg[rspec[k]].push_back({r, -(double)rcnt[k]});
        for (int k = pbeg[r]; k < pbeg[r + 1]; ++k)
            sg[pspec[k]].push_back({r, (double)pcnt[k]});
    }
    W.sgBeg.push_back(0);
    for (int s = 0; s < N; ++s)
    {
        for (auto& pr : sg[s])
            W.sgRx.push_back(pr.first), W.sgCoef.push_back(pr.second);
        W.sgBeg.push_back((int)W.sgRx.size());
    }
    // Jacobian entries and their gathers, from the contribution list of the sparse plan
    std::vector<int> entryOf(P.nnz, -1);
    std::vector<std::vector<std::pair<int, double>>> jg;
    for (int e = 0; e < rbeg[R]; ++e)
        for (int c = P.cBeg[e]; c < P.cBeg[e + 1]; ++c)
        {
            const int pos = P.cPos[c];
            if (entryOf[pos] < 0)
            {
                entryOf[pos] = (int)W.jPos.size();
                W.jPos.push_back(pos);
                W.jRow.push_back(P.cRow[c]);
                W.jCol.push_back(rspec[e]);
                jg.emplace_back();
            }
            jg[entryOf[pos]].push_back({e, P.cCoef[c]});
        }
    // entries with the longest contribution lists first (balanced rounds of the warp)
    {
        std::vector<int> ord(jg.size());
        for (size_t m = 0; m < ord.size(); ++m)
            ord[m] = (int)m;
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return jg[a].size() > jg[b].size(); });
        std::vector<int> jp, jr, jc;
        std::vector<std::vector<std::pair<int, double>>> jgs;
        for (int m : ord)
            jp.push_back(W.jPos[m]), jr.push_back(W.jRow[m]), jc.push_back(W.jCol[m]), jgs.push_back(jg[m]);
        W.jPos = jp, W.jRow = jr, W.jCol = jc, jg = jgs;
    }
    W.jgBeg.push_back(0);
    for (auto& l : jg)
    {
        for (auto& pr : l)
            W.jgEnt.push_back(pr.first), W.jgCoef.push_back(pr.second);
        W.jgBeg.push_back((int)W.jgEnt.size());
    }
    std::vector<std::vector<int>> rows(N);
    for (int m = 0; m < (int)W.jPos.size(); ++m)
        rows[W.jRow[m]].push_back(m);
    W.rjBeg.push_back(0);
    for (int i = 0; i < N; ++i)
    {
        std::sort(rows[i].begin(), rows[i].end(), [&](int a, int b) { return W.jCol[a] < W.jCol[b]; });
        for (int m : rows[i])
            W.rjEnt.push_back(m);
        W.rjBeg.push_back((int)W.rjEnt.size());
    }
    // species and J-row gathers in the order the lanes take them: longest lists first
    for (int i = 0; i < N; ++i)
        W.sgOrder.push_back(i), W.rjOrder.push_back(i);
    std::stable_sort(W.sgOrder.begin(), W.sgOrder.end(),
                     [&](int a, int b) { return W.sgBeg[a + 1] - W.sgBeg[a] > W.sgBeg[b + 1] - W.sgBeg[b]; });
    std::stable_sort(W.rjOrder.begin(), W.rjOrder.end(),
                     [&](int a, int b) { return W.rjBeg[a + 1] - W.rjBeg[a] > W.rjBeg[b + 1] - W.rjBeg[b]; });
    W.entRx.assign(rbeg[R], 0);
    for (int r = 0; r < R; ++r)
        for (int k = rbeg[r]; k < rbeg[r + 1]; ++k)
            W.entRx[k] = r;
    for (int s = 0; s < N; ++s)
        if (W.sgBeg[s + 1] - W.sgBeg[s] > WarpPlan::kHeavy) W.sgHeavy.push_back(s);
    for (int m = 0; m + 1 < (int)W.jgBeg.size(); ++m)
        if (W.jgBeg[m + 1] - W.jgBeg[m] > WarpPlan::kHeavy) W.jgHeavy.push_back(m);
    for (int i = 0; i < N; ++i)
        if (W.rjBeg[i + 1] - W.rjBeg[i] > WarpPlan::kHeavy) W.rjHeavy.push_back(i);
    for (int i = 0; i < n; ++i)
        if (P.rowBeg[i + 1] - P.rowBeg[i] > WarpPlan::kHeavy) W.rowHeavy.push_back(i);
    buildLevels(P, W, rhsBase);
    (void)pspec, (void)pcnt, (void)rcnt;
    return W;
}

} // namespace nnet_gb300
