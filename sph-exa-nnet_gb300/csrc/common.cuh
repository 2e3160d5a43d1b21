// Shared device definitions of the GB300 burn library: solver constants, per-particle
// status codes, strided scratch access and the device-side network / table views.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/nnet_gb300.h"
#include "../data/nnet_network_tables.h"

namespace nnet_gb300
{

// θ-method Newton substep constants (include/nnet/nuclear_net.hpp:48-106)
namespace k
{
constexpr double theta         = 0.8;
constexpr double minTemp       = 1e8;
constexpr double minRho        = 1e5;
constexpr double maxDtStep     = 2;
constexpr double minDtStep     = 1e-2;
constexpr double nanDtStep     = 2e-1;
constexpr double epsilonSystem = 1e-40;
constexpr double epsilonVector = 1e-16;
constexpr double nrMaxDt       = 1e-2;
constexpr double nrDTTarget    = 1e-2;
constexpr double nrDTTol       = 4;
constexpr int    nrMinIt       = 1;
constexpr int    nrMaxIt       = 11;
constexpr double nrItTol       = 1e-7;
constexpr double substepDtTol  = 1e-6;
// livelock detection: attempt-start timesteps equal within this relative tolerance (2^-20)
constexpr double cycleDtTol    = 9.5367431640625e-07;
} // namespace k

// Element e of scratch slot s lives at base[e * stride + s]: a warp touching element e of
// 32 consecutive slots reads 256 contiguous bytes.
template<typename T>
struct Strided
{
    T*     p;
    size_t s;
    __device__ __forceinline__ T&      operator[](int e) const { return p[(size_t)e * s]; }
    __device__ __forceinline__ Strided at(int e) const { return {p + (size_t)e * s, s}; }
};

// Device view of a network's sparse-solver plan (see sparse_plan.hpp for the meaning)
struct SparseView
{
    int           n, nnz, nsb, pos00, tNew; // tNew: position of the temperature in the new order
    const int *   perm, *iperm, *rowBeg, *posRow, *posCol, *kPiv, *lBeg, *lPos, *lRow, *tBeg, *uBeg, *uPos, *uCol,
        *tPos;
    const int *   diagPos, *col0Pos, *row0Pos, *cBeg, *cPos, *cRow, *sbPos, *sbDiag;
    const double* cCoef;
};

// Device view of a network's warp-per-particle lists (see WarpPlan in sparse_plan.hpp)
struct WarpView
{
    int           nJ, nEnt, nSgHeavy, nJgHeavy, nRjHeavy, nRowHeavy;
    const int *   updBeg, *updT, *updL, *updU, *ucBeg, *ucPos, *ucRow, *sgBeg, *sgRx, *jPos, *jRow, *jCol, *jgBeg,
        *jgEnt, *rjBeg, *rjEnt, *entRx, *sgHeavy, *jgHeavy, *rjHeavy, *rowHeavy;
    const double *sgCoef, *jgCoef;
    // level schedule of the factorisation and solves (WarpPlan::nLevels and its lists)
    int        nLevels;
    const int *lvBeg, *lvPiv, *lsBeg, *lsPos, *lsPiv, *tgBeg, *tgPos, *tgUpd, *tuL, *tuU;
    const int *fwBeg, *fwRow, *fwEnt, *flPos, *flK, *bwBeg, *bwRow, *bwEnt, *buPos, *buK;
    const int *sgOrder, *rjOrder;
    // fused forms (WarpPlan::scBeg ... tuUA), and the fused factorisation's per-lane op
    // streams (WarpPlan::fOps, foBeg)
    int                       rhsBase;
    const int *               scBeg, *scPos, *scPiv, *tgBegA, *tgPosA, *tgUpdA, *tuLA, *tuUA;
    const unsigned long long* fOps;
    const int*                foBeg;
};

// Read-only device view of one network definition (reaction list in CSR form, binding
// energies, charges, fit / partition-function tables).
struct NetView
{
    int           net, nspec, nreact;
    const int *   rbeg, *rspec, *rcnt, *pbeg, *pspec, *pcnt;
    const double *BE, *Z, *z53;
    const double* A; // mass numbers (net87: the electron entry is 0)
    // per species i: sqrt(z53), sqrt(sqrt(z53)), z53^1.9885, log(z53) (fast rate forms)
    const double* zFac;
    const double *fit, *q, *choose;
    const double* part; // choose-ratio of fitted rate r in temperature range kb at [r * 24 + kb]
    const int *   mainReactant, *secondaryReactant, *mainProduct;
    const double *eLogT, *eLogRho, *eRate;
    SparseView    sp;
    WarpView      wv;
};

// Helmholtz table: one 128-byte line per grid cell (i, j) holding the 13 quantities the
// EOS outputs depend on, in the order f ft ftt fd fdd fdt fddt fdtt fddtt dpdf dpdft
// dpdfd dpdfdt (that is, the order the interpolation consumes them), padded to 16.
constexpr int HELM_IMAX = 541, HELM_JMAX = 201, HELM_CELL = 16;
struct HelmView
{
    const double* cell; // [IMAX][JMAX][16]
    const double *d, *ddSav, *dd2Sav, *ddiSav, *t, *dtSav, *dt2Sav, *dtiSav, *dt2iSav;
};

// Per-particle status codes (mirrors nnet_particle_status in the C header)
enum : int32_t
{
    ST_OK       = NNET_PARTICLE_OK,
    ST_SKIPPED  = NNET_PARTICLE_SKIPPED,
    ST_LIVELOCK = NNET_PARTICLE_LIVELOCK,
    ST_MAXITER  = NNET_PARTICLE_MAXITER,
    ST_ZERO_DT  = NNET_PARTICLE_ZERO_DT,
    ST_ABORTED  = NNET_PARTICLE_ABORTED,
    kNumStatus  = NNET_NUM_PARTICLE_STATUS,
};

// Word offsets of a launch's statistics (BurnParams::stats)
enum : int
{
    kStatIters    = 0,                        // Newton iterations
    kStatSubsteps = 1,                        // accepted substeps
    kStatStatus   = 2,                        // [kStatStatus + s]: particles ending with status s
    kStatRefine   = kStatStatus + kNumStatus, // mixed form: refinement steps
    kStatFallback = kStatRefine + 1,          // mixed form: systems re-solved in FP64
    kStatWords    = kStatFallback + 1
};

// %globaltimer (ns) of the calling thread's SM
__device__ __forceinline__ unsigned long long globalTimerNs()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Per-particle state that lets a burn pause at an attempt boundary and resume later with
// bit-identical arithmetic (continuous batching).  phase: 0 not started, 1 paused,
// 2 finished.  Y, T and dt live in the particle arrays themselves.
struct ResumeState
{
    int*                phase;
    double *            elapsed, *nextT, *drho;
    long long*          nit;
    int *               nsub, *cdPower, *cdSteps;
    unsigned long long *cdDt, *cdNt;
};

// A particle handed from one warp to another at an attempt boundary (batched layout, after
// the work queue has drained): everything the next attempt depends on besides Y, which the
// donor writes back to the particle arrays first.  seq = position + 1 once published.
struct alignas(16) MigCell
{
    unsigned long long seq, p;
    double             T, dt, elapsed, nextT, rho, drho;
    long long          nit;
    int                nsub, cdPower, cdSteps, pad;
    unsigned long long cdDt, cdNt;
};

// Batch arguments as seen by the kernels
struct BurnParams
{
    size_t         P;
    double*        Y[NNET_MAX_SPECIES];
    double*        T;
    const double*  rho;
    const double*  rhoM1;
    double*        dt;
    double         hydroDt, previousDt, mu;
    int            useDrhodt;
    long long      maxIter;
    int32_t*       status;
    int32_t*       substeps;
    int32_t*       iterations;
    unsigned long long* queue;  // work-queue head (reset to 0 before each launch)
    unsigned long long* stats;  // kStatWords counters (kStatIters ... kStatFallback)
    const uint32_t*     order;  // optional particle visiting order (nullptr: identity)
    // launch watchdog: 0, or the nanoseconds after which the launch takes no further Newton
    // iteration (running particles stop at their last accepted substep, queued ones untouched,
    // both with ST_ABORTED)
    unsigned long long  timeLimitNs;
    // post-burn steps (all optional): divide Y by sum_i A_i Y_i, report sum_i A_i Y_i - 1 of
    // the burned state, Helmholtz EOS at the final state (computeHelmEOS)
    int                 normalize;
    double*             massDrift;
    double *            eosU, *eosCv, *eosP, *eosC, *eosDpdT;
    // continuous batching (all optional): resumable state, Newton-iteration budget of this
    // launch per particle (a particle pauses at the first attempt boundary past it), and a
    // per-particle segment id whose finished-particle counter is incremented on completion
    ResumeState         rs;
    long long           sliceIters;
    const int*          segOf;
    unsigned long long* segFinished;
    int                 laneSlots; // batched layout: particles in flight per warp (0 = 32)
    // batched layout, optional: rebalancing of the running particles over the warps once the
    // queue has drained.  migCount: [0] hand-off records reserved, [1] taken, [2] particles
    // held by warps; migCells: migCap records.
    MigCell*            migCells;
    unsigned long long  migCap;
    unsigned long long* migCount;

    __host__ __device__ bool postSteps() const { return normalize || massDrift || eosU; }
};

} // namespace nnet_gb300
