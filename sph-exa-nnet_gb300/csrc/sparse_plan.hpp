// Host-side symbolic analysis of a network's Newton matrix for the sparse solver forms.
//
// The (N+1) x (N+1) system of prepareSystemFromGuess (include/nnet/nuclear_net.hpp:
// 514-609; index 0 = temperature, 1..N = species) has the structure
//   row 0 and column 0 dense (energy equation, d(dY/dt)/dT),
//   species block = identity + the reaction-list Jacobian pattern (:395-438).
// A greedy minimum-degree ordering on that pattern (ties by index) and a symbolic
// right-looking elimination give the fill and flat "programs" the kernels execute with
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

} // namespace nnet_gb300
