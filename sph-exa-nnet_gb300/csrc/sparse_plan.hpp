// Host-side symbolic analysis of a network's Newton matrix for the sparse solver forms.
//
// The (N+1) x (N+1) system of prepareSystemFromGuess (include/nnet/nuclear_net.hpp:
// 514-609; index 0 = temperature, 1..N = species) has the structure
//   row 0 and column 0 dense (energy equation, d(dY/dt)/dT),
//   species block = identity + the reaction-list Jacobian pattern (:395-438).
// A greedy minimum-degree ordering on that pattern (ties by elimination level, then index)
// and a symbolic right-looking elimination give the fill and flat "programs" the kernels execute with
// warp-uniform control flow: every particle of a network runs the same operation list
// on its own values.  For net86 this is 1,044 stored entries and 2,745 multiply-adds
// per factorisation, against 7,569 entries and about 216k for the dense elimination.
#pragma once

#include <vector>

namespace nnet_gb300
{

struct SparsePlan
{
    int n = 0, N = 0, R = 0, nnz = 0;
    std::vector<int> perm, iperm;          // new -> old, old -> new (old 0 = T)
    std::vector<int> posRow, posCol;       // position -> (row, col) in the new order
    std::vector<int> rowBeg;               // positions of row i: rowBeg[i] .. rowBeg[i+1]
    // factorisation program (right-looking, no pivoting), for pivot k:
    //   L entries lBeg[k]..lBeg[k+1]: position lPos, row lRow, and for each its targets
    //   tPos[tBeg[e] .. tBeg[e] + (uBeg[k+1] - uBeg[k])) aligned with the U entries
    //   uBeg[k]..uBeg[k+1]: position uPos, column uCol.
    std::vector<int> kPiv, lBeg, lPos, lRow, tBeg, uBeg, uPos, uCol, tPos;
    // assembly maps (species i, j in 0..N-1)
    std::vector<int> diagPos, col0Pos, row0Pos;
    int              pos00 = 0;
    // Jacobian contributions in the reference's loop order: for reactant entry e of the
    // reaction list (reactant_begin order), targets cBeg[e]..cBeg[e+1] with position,
    // species row and stoichiometric coefficient (-count for reactants, +count for products)
    std::vector<int>    cBeg, cPos, cRow;
    std::vector<double> cCoef;
    std::vector<int>    sbPos;  // every species-block position (for I - theta dt J)
    std::vector<int>    sbDiag; // 1 where sbPos is a diagonal entry
    long long           factorFma = 0, solveFma = 0;
};

// Build the plan of network `net` (14, 86, 87) from its reaction list.
SparsePlan buildSparsePlan(int net, const int* rbeg, const int* rspec, const int* rcnt, const int* pbeg,
                           const int* pspec, const int* pcnt, int R);

// Extra lists of the warp-per-particle kernels, in which the 32 lanes of a warp share one
// particle's Newton system in shared memory.  Accumulations are written as gathers (each
// target sums its own contribution list in a fixed order) so that no two lanes write the
// same word and results are deterministic; a list longer than kHeavy (the p, n, alpha rows
// and columns of net86) is summed by the whole warp with a fixed butterfly reduction.
struct WarpPlan
{
    static constexpr int kHeavy = 16;
    // factorisation updates of pivot k: updBeg[k] .. updBeg[k+1], target / L / U positions
    std::vector<int> updBeg, updT, updL, updU;
    // column k of U above the diagonal (column-oriented backward substitution)
    std::vector<int> ucBeg, ucPos, ucRow;
    // species gathers of dY/dt: species s sums coef * flux[reaction] over sgBeg[s]..sgBeg[s+1]
    std::vector<int>    sgBeg, sgRx;
    std::vector<double> sgCoef;
    // Jacobian gathers: J entry m (position jPos[m], species row jRow[m], species column
    // jCol[m]) sums coef * tr[reactant entry] over jgBeg[m]..jgBeg[m+1]
    std::vector<int>    jPos, jRow, jCol, jgBeg, jgEnt;
    std::vector<double> jgCoef;
    // J entries of species row i: rjBeg[i] .. rjBeg[i+1] (indices into the J entry list)
    std::vector<int> rjBeg, rjEnt;
    // reaction of every reactant entry
    std::vector<int> entRx;
    // species (dY/dt) and J rows (J (Yn - Y)) in the order the lanes take them
    std::vector<int> sgOrder, rjOrder;
    // targets whose lists are longer than kHeavy (summed by the whole warp)
    std::vector<int> sgHeavy, jgHeavy, rjHeavy, rowHeavy; // species, J entries, J rows, factor rows

    // Level schedule: pivot k depends on pivot j < k when (k, j) or (j, k) is stored; the
    // pivots of one level are mutually independent, so a level's reciprocals, multipliers
    // and updates run as three warp-parallel rounds.  Updates are grouped by target (each
    // target subtracts its products in pivot order), so no two lanes write one word.
    //   pivots of level l:        lvPiv[lvBeg[l] .. lvBeg[l+1])
    //   multipliers of level l:   lsPos / lsPiv over lsBeg[l] .. lsBeg[l+1] (L position, pivot)
    //   update targets of level l: tgPos over tgBeg[l] .. tgBeg[l+1]; target t subtracts
    //                              A[tuL[u]] * A[tuU[u]] for u in tgUpd[t] .. tgUpd[t+1]
    //   forward solve, level l:   rows fwRow over fwBeg[l] .. fwBeg[l+1]; row r subtracts
    //                              A[flPos[e]] * x[flK[e]] for e in fwEnt[r] .. fwEnt[r+1]
    //   backward solve, level l:  rows bwRow over bwBeg[l] .. bwBeg[l+1]; row r subtracts
    //                              A[buPos[e]] * x[buK[e]] for e in bwEnt[r] .. bwEnt[r+1]
    //                              (levels run last to first; x[k] of the level's pivots is
    //                              scaled by the pivot reciprocal first)
    int              nLevels = 0;
    std::vector<int> lvBeg, lvPiv, lsBeg, lsPos, lsPiv, tgBeg, tgPos, tgUpd, tuL, tuU;
    std::vector<int> fwBeg, fwRow, fwEnt, flPos, flK, bwBeg, bwRow, bwEnt, buPos, buK;
    // Fused forms of the same schedule:
    //   scaling with the reciprocal folded in: scPos / scPiv over scBeg[l] .. scBeg[l+1]
    //   (every L entry of the level's pivots, plus (-1, k) for a pivot without L entries);
    //   factorisation with the forward substitution folded in: the right-hand side is
    //   column `rhsBase` + row of the stored matrix (the kernels keep b right after the
    //   factor's rhsBase entries), and tgBegA / tgPosA / tgUpdA / tuLA / tuUA list the
    //   level's targets including the right-hand-side rows.
    int              rhsBase = 0;
    std::vector<int> scBeg, scPos, scPiv, tgBegA, tgPosA, tgUpdA, tuLA, tuUA;
    // The fused factorisation's updates as per-lane op streams: level l takes rows
    // foBeg[l] .. foBeg[l+1] of fOps, 32 ops per row (op k of lane q at row k, column q).  An
    // op is target -= A[L] * A[U]; it loads the target first when it is the target's first,
    // stores it when it is the last; 0 is no op (see factorOp).
    std::vector<unsigned long long> fOps;
    std::vector<int>                foBeg;
    static constexpr unsigned long long kOpFirst = 1ull << 48, kOpLast = 1ull << 49, kOpValid = 1ull << 50;
    static unsigned long long factorOp(int L, int U, int target, bool first, bool last)
    {
        return (unsigned long long)L | (unsigned long long)U << 16 | (unsigned long long)target << 32 |
               (first ? kOpFirst : 0) | (last ? kOpLast : 0) | kOpValid;
    }
};

// capacity of the factor storage of the warp-cooperative kernels (the right-hand side
// follows it in shared memory)
constexpr int kWarpNnzCap14 = 104, kWarpNnzCap86 = 1056;

WarpPlan buildWarpPlan(const SparsePlan& P, const int* rbeg, const int* rspec, const int* rcnt, const int* pbeg,
                       const int* pspec, const int* pcnt, int rhsBase);

} // namespace nnet_gb300
