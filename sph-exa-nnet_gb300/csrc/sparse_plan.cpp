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

    // ---- greedy minimum degree on the symmetrised graph
    std::vector<std::set<int>> adj(n);
    for (auto [i, j] : S)
        if (i != j) adj[i].insert(j), adj[j].insert(i);
    std::vector<char> alive(n, 1);
    for (int step = 0; step < n; ++step)
    {
        int v = -1;
        for (int x = 0; x < n; ++x)
            if (alive[x] && (v < 0 || adj[x].size() < adj[v].size())) v = x;
        P.perm.push_back(v);
        std::set<int> nb = adj[v];
        for (int a : nb)
        {
            for (int b : nb)
                if (b != a) adj[a].insert(b);
            adj[a].erase(v);
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
