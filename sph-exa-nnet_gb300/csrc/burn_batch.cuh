// Batched-warp forms of the sparse and mixed-precision burn (templates; instantiated per
// network in burn_batch14.cu, burn_batch86.cu, burn_batch87.cu and, for the multi-network
// launch, burn_batch_multi_*.cu): each warp carries 32
// particles in lockstep, one per lane, through Newton iterations.
//
// A Newton iteration has two kinds of work.  The per-particle scalar part (temperature
// checks, the Helmholtz EOS, the special CF88 rates, the Coulomb and fit-power factors,
// electron captures, timestep control) is a few thousand FP64 instructions of branchy
// scalar code; the system part (≈150 fitted rates, fluxes, Jacobian, sparse LU) is wide.
// Here the scalar part runs SIMD across the warp's 32 particles (lane l = particle l), and
// the system part runs warp-cooperatively on one particle at a time with the shared-memory
// machinery of warp_system.cuh.  Per warp iteration:
//   S1 (lanes)     pre-iteration checks; finished particles are released and replaced
//   V1 (per slot)  apply the last decision to the slot's abundances (accept / continue),
//                  write back a finished particle, load a new one, θ-blend, Σ Y and Σ Y Z
//   S2 (lanes)     EOS and every temperature/density-only rate factor into the slot table
//   V2 (per slot)  rates, fluxes, system, sparse LU solve, Newton candidate
//   S3 (lanes)     acceptance, rejection and timestep control; release / replace
// Abundances and the slot table live in per-warp global scratch (L2-resident); one Newton
// system per warp lives in shared memory.
#pragma once

#include "burn_multi.hpp"
#include "launch.hpp"
#include "warp_system.cuh"

namespace nnet_gb300
{

namespace
{

// per-slot scalars, field-major in the warp's global scratch: field f of slot l at sc[f * 32 + l]
enum SlotField : int
{
    fT, fTth, fRho, fDrho, fDt, fCv, fDpdT,
    fGam, fGs, fGq, fGp, fGl, fNakbt, fCorr,
    fT9, fT913, fT923, fT953, fT9i, fT9i2, fT9i13, fT9i23, fT9i43, fLt9,
    fVal1, fVal2, fVal3, fVal4, fTwoT, fKb,
    fSp0,             // 9 special rates (value, derivative), screened, in the network's slot order
    fEv0 = fSp0 + 18, // net87: rate 309, d/dT, rate 310, d/dT, BE shift of n and p
    kSlotFields = fEv0 + 6
};

// rate slots of the special rates, in the order they are stored
__device__ __forceinline__ int specialSlot(int net, int k)
{
    if (net == 14)
    {
        constexpr int s14[9] = {0, 1, 2, 13, 14, 15, 16, 17, 18}; // e3a ecag eoag e2c eco e2o l3a lcag loag
        return s14[k];
    }
    constexpr int s86[9] = {0, 1, 2, 3, 4, 5, 156, 157, 158}; // e2c eco e2o e3a ecag eoag l3a lcag loag
    return s86[k];
}

// an empty warp polls for hand-offs at most this often (about 20 us apart) before leaving
constexpr unsigned kIdlePolls = 1u << 22;

enum : int
{
    ACT_ACCEPT = 1,  // Y <- clipped candidate
    ACT_CONT   = 2,  // Yn <- clipped candidate
    ACT_WRITE  = 4,  // write the slot's Y back to the particle arrays (particle pw)
    ACT_LOAD   = 8,  // load a newly acquired particle's Y
    ACT_BLEND  = 16, // θ-blend for the iteration about to run
    ACT_FINAL  = 32  // the write ends particle pw's burn (not a pause): post-burn steps apply
};

template<int NET>
constexpr int padN()
{
    return (NET + 3) & ~3;
}

// take the next particle of the queue for this lane; skipped ones, and once the launch is
// past its time limit the remaining ones, are completed here by the lane alone
template<bool POST>
__device__ bool acquireLane(const BurnParams& bp, const NetView& nv, const HelmView& hv, ParticleState& s,
                            unsigned long long deadline)
{
    for (;;)
    {
        const unsigned long long q = atomicAdd(bp.queue, 1ull);
        if (q >= bp.P) return false;
        const size_t p     = bp.order ? (size_t)bp.order[q] : (size_t)q;
        const int    phase = bp.rs.phase ? bp.rs.phase[p] : 0;
        if (phase == 2) continue;
        const double rho = bp.rho[p], T = bp.T[p];
        const bool   skip = phase == 0 && !(rho > k::minRho && T > k::minTemp);
        if (skip || expired(deadline))
        {
            if constexpr (POST) postScalar(bp, nv, hv, p, !skip);
            endUntouched(bp, p, skip ? ST_SKIPPED : ST_ABORTED);
            continue;
        }
        s.p = p, s.T = T, s.dt = bp.dt[p], s.rho = rho, s.i = 1;
        if (phase == 1)
        {
            const ResumeState& r = bp.rs;
            s.elapsed = r.elapsed[p], s.nextT = r.nextT[p], s.drho = r.drho[p], s.nit = r.nit[p];
            s.nsub = r.nsub[p], s.cdDt = r.cdDt[p], s.cdNt = r.cdNt[p], s.cdPower = r.cdPower[p];
            s.cdSteps = r.cdSteps[p];
        }
        else
        {
            double drho = 0;
            if (bp.useDrhodt && bp.rhoM1 && bp.rhoM1[p] != 0) drho = (rho - bp.rhoM1[p]) / bp.previousDt;
            s.elapsed = 0, s.nextT = 0, s.drho = drho, s.nit = 0, s.nsub = 0;
            s.cycleReset();
        }
        s.nit0 = s.nit;
        if (bp.migCount) atomicAdd(bp.migCount + 2, 1ull);
        return true;
    }
}

// scalar outputs of a finished (st >= 0) or paused (kPaused) particle; Y is written in V1
__device__ void releaseLane(const BurnParams& bp, const ParticleState& s, int st)
{
    const size_t p = s.p;
    bp.T[p]        = s.T;
    bp.dt[p]       = s.dt;
    atomicAdd(bp.stats + kStatIters, (unsigned long long)(s.nit - s.nit0));
    if (bp.migCount) atomicAdd(bp.migCount + 2, (unsigned long long)-1ll);
    if (st == kPaused)
    {
        const ResumeState& r = bp.rs;
        r.elapsed[p] = s.elapsed, r.nextT[p] = s.nextT, r.drho[p] = s.drho, r.nit[p] = s.nit, r.nsub[p] = s.nsub;
        r.cdDt[p] = s.cdDt, r.cdNt[p] = s.cdNt, r.cdPower[p] = s.cdPower, r.cdSteps[p] = s.cdSteps;
        r.phase[p] = 1;
        return;
    }
    if (bp.status) bp.status[p] = st;
    if (bp.substeps) bp.substeps[p] = s.nsub;
    if (bp.iterations) bp.iterations[p] = (int32_t)s.nit;
    atomicAdd(bp.stats + kStatSubsteps, (unsigned long long)s.nsub);
    atomicAdd(bp.stats + kStatStatus + st, 1ull);
    finishSegment(bp, p);
}

// Post-burn steps of the slot's finished particle po, by the whole warp, on the abundances
// yw[t] = Y[lane + 32 t] of its last accepted substep: s = sum_i A_i Y_i (fixed reduction
// order), the drift s - 1, Y / s written back when normalising, and the sums the EOS needs
// (returned to lane l).  Same steps as postScalar.
template<int N>
__device__ void postWarp(const BurnParams& bp, const NetView& nv, const double (&yw)[(N + 31) / 32], double sx,
                         size_t po, int l, int lane, double& abW, double& zbW)
{
    sx = warpSum(sx);
    if (lane == l && bp.massDrift) bp.massDrift[po] = sx - 1.;
    const bool scale = bp.normalize && sx > 0 && sx < INFINITY;
    double     ab = 0, zb = 0;
#pragma unroll
    for (int t = 0; t < (N + 31) / 32; ++t)
    {
        const int j = lane + 32 * t;
        if (j < N)
        {
            const double y = scale ? yw[t] / sx : yw[t];
            bp.Y[j][po]    = y;
            ab += y, zb += y * __ldg(nv.Z + j);
        }
    }
    if (bp.eosU)
    {
        ab = warpSum(ab), zb = warpSum(zb);
        if (lane == l) abW = ab, zbW = zb;
    }
}

// the lowest k set bits of m
__device__ __forceinline__ unsigned lowestBits(unsigned m, int k)
{
    unsigned r = 0;
    for (; k > 0 && m; --k)
        r |= m & (0u - m), m &= m - 1;
    return r;
}

// Hand this lane's particle over (rebalancing): reserve a record, fill it (published after the
// warp has written Y back), account its iterations.  Returns the record position or -1.
__device__ long long donateLane(const BurnParams& bp, const ParticleState& s)
{
    if (*(volatile unsigned long long*)bp.migCount >= bp.migCap) return -1;
    const unsigned long long pos = atomicAdd(bp.migCount, 1ull);
    if (pos >= bp.migCap) return -1;
    MigCell& c = bp.migCells[pos];
    c.p = s.p, c.T = s.T, c.dt = s.dt, c.elapsed = s.elapsed, c.nextT = s.nextT, c.rho = s.rho, c.drho = s.drho;
    c.nit = s.nit, c.nsub = s.nsub, c.cdPower = s.cdPower, c.cdSteps = s.cdSteps, c.cdDt = s.cdDt, c.cdNt = s.cdNt;
    atomicAdd(bp.stats + kStatIters, (unsigned long long)(s.nit - s.nit0));
    atomicAdd(bp.migCount + 2, (unsigned long long)-1ll);
    return (long long)pos;
}

// Take the next published hand-off record, if any.  The particle resumes at its attempt
// boundary: Y is loaded from the particle arrays (past the L1, which may hold lines that
// predate the donor's write-back).
__device__ bool takeLane(const BurnParams& bp, ParticleState& s)
{
    const unsigned long long h   = *(volatile unsigned long long*)(bp.migCount + 1);
    const unsigned long long lim = min(*(volatile unsigned long long*)bp.migCount, bp.migCap);
    if (h >= lim) return false;
    MigCell& c = bp.migCells[h];
    if (*(volatile unsigned long long*)&c.seq != h + 1) return false; // reserved, not yet published
    if (atomicCAS(bp.migCount + 1, h, h + 1) != h) return false;
    __threadfence();
    s.p = __ldcg(&c.p), s.T = __ldcg(&c.T), s.dt = __ldcg(&c.dt), s.elapsed = __ldcg(&c.elapsed);
    s.nextT = __ldcg(&c.nextT), s.rho = __ldcg(&c.rho), s.drho = __ldcg(&c.drho), s.nit = __ldcg(&c.nit);
    s.nsub = __ldcg(&c.nsub), s.cdPower = __ldcg(&c.cdPower), s.cdSteps = __ldcg(&c.cdSteps);
    s.cdDt = __ldcg(&c.cdDt), s.cdNt = __ldcg(&c.cdNt);
    s.i = 1, s.nit0 = s.nit;
    atomicAdd(bp.migCount + 2, 1ull);
    return true;
}

// S2: everything of one Newton iteration that depends on (T, rho) of the slot only
template<int NET, int EOS>
__device__ void slotScalars(const NetView& nv, const HelmView& hv, double mu, double* sc, int lane, double T,
                            double Tth, double rhoT, double drho, double dt, double abar, double zbar, double yElec)
{
    auto put = [&](int f, double v) { sc[f * 32 + lane] = v; };
    EosResult eos;
    if constexpr (EOS == NNET_EOS_IDEAL_GAS)
        eos = idealGasEos(mu, Tth, rhoT);
    else
        eos = helmholtzEos(hv, abar, zbar, Tth, rhoT);
    put(fT, T), put(fTth, Tth), put(fRho, rhoT), put(fDrho, drho), put(fDt, dt), put(fCv, eos.cv);
    put(fDpdT, eos.dpdT);
    const CoulombFast cf(Tth, rhoT);
    put(fGam, cf.gam), put(fGs, cf.gs), put(fGq, cf.gq), put(fGp, cf.gp), put(fGl, cf.gl), put(fNakbt, cf.nakbt);
    put(fCorr, cf.corr);
    const FitT v(Tth);
    put(fT9, v.t9), put(fT913, v.t913), put(fT923, v.t923), put(fT953, v.t953), put(fT9i, v.t9i);
    put(fT9i2, v.t9i2), put(fT9i13, v.t9i13), put(fT9i23, v.t9i23), put(fT9i43, v.t9i43), put(fLt9, v.lt9);
    if constexpr (NET == 14)
    {
        const double t9 = Tth / 1.e9, t9i = 1.e0 / t9, lt9 = log(t9);
        const double val1 = 11.6045e0 * t9i;
        put(fVal1, val1), put(fVal2, 1.5e0 * lt9), put(fVal3, val1 * t9i * 1e-9), put(fVal4, 1.5e-9 * t9i);
    }
    else
    {
        const double t9 = Tth * 1e-09, t9i = 1. / t9;
        const double val1 = 11.6045 * t9i;
        put(fVal1, val1), put(fVal2, 1.5 * log(t9)), put(fVal3, val1 * t9i * 1e-9), put(fVal4, 1.5e-9 * t9i);
    }
    put(fTwoT, 2. / Tth), put(fKb, (double)temperatureRange(Tth));
    Special s;
    specialRates(Tth, s);
    auto m = [&](int i) { return (NET != 14 && i == 1) ? 0. : cf.mu(nv, i); }; // neutrons carry no screening
    if constexpr (NET == 14)
    {
        const double m0 = m(0), m1 = m(1), m2 = m(2), m3 = m(3), m4 = m(4), m5 = m(5);
        screenFast(s.e3a, s.de3a, m0 + m0 - m1 + m0, Tth);
        screenFast(s.ecag, s.decag, m1 + m0 - m2, Tth);
        screenFast(s.eoag, s.deoag, m2 + m0 - m3, Tth);
        screenFast(s.e2c, s.de2c, 2. * m1 - m3, Tth);
        screenFast(s.eco, s.deco, m1 + m2 - m4, Tth);
        screenFast(s.e2o, s.de2o, 2. * m2 - m5, Tth);
        const double o[18] = {s.e3a, s.de3a, s.ecag, s.decag, s.eoag, s.deoag, s.e2c, s.de2c, s.eco,
                              s.deco, s.e2o, s.de2o, s.l3a, s.dl3a, s.lcag, s.dlcag, s.loag, s.dloag};
        for (int k = 0; k < 18; ++k)
            put(fSp0 + k, o[k]);
    }
    else
    {
        auto dmu = [&](int i) {
            return m(__ldg(nv.mainReactant + i)) + m(__ldg(nv.secondaryReactant + i)) - m(__ldg(nv.mainProduct + i));
        };
        screenFast(s.e2c, s.de2c, dmu(0), Tth);
        screenFast(s.eco, s.deco, dmu(1), Tth);
        screenFast(s.e2o, s.de2o, dmu(2), Tth);
        screenFast(s.e3a, s.de3a, dmu(4) + m(__ldg(nv.mainReactant + 4)), Tth);
        screenFast(s.ecag, s.decag, dmu(5), Tth);
        screenFast(s.eoag, s.deoag, dmu(6), Tth);
        const double o[18] = {s.e2c, s.de2c, s.eco, s.deco, s.e2o, s.de2o, s.e3a, s.de3a, s.ecag,
                              s.decag, s.eoag, s.deoag, s.l3a, s.dl3a, s.lcag, s.dlcag, s.loag, s.dloag};
        for (int k = 0; k < 18; ++k)
            put(fSp0 + k, o[k]);
        if constexpr (NET == 87)
        {
            // electron captures (net87.hpp:117-175)
            const double rhoElec = yElec * rhoT;
            double       ev[12];
            electronRates(nv, Tth, rhoElec, ev);
            put(fEv0 + 0, rhoElec == 0 ? 0 : ev[0] / rhoElec), put(fEv0 + 1, rhoElec == 0 ? 0 : ev[1] / rhoElec);
            put(fEv0 + 2, rhoElec == 0 ? 0 : ev[6] / rhoElec), put(fEv0 + 3, rhoElec == 0 ? 0 : ev[7] / rhoElec);
            put(fEv0 + 4, -ev[3]), put(fEv0 + 5, -ev[9]);
        }
    }
}

// V2 rates of slot l from its table entries (same arithmetic as warpRates)
template<int NET, bool MIXED>
__device__ void slotRates(const NetView& nv, WarpSmem<NET, MIXED>& S, const double* c, int lane)
{
    auto g = [&](int f) { return c[f * 32]; };
    CoulombFast cf;
    cf.gam = g(fGam), cf.gs = g(fGs), cf.gq = g(fGq), cf.gp = g(fGp), cf.gl = g(fGl), cf.nakbt = g(fNakbt);
    cf.corr = g(fCorr);
    constexpr int NS = NET == 14 ? 14 : 86;
    for (int i = lane; i < NS; i += 32)
    {
        double be, mu;
        cf.beMu(nv, i, be, mu);
        S.BE[i] = be;
        S.mu[i] = (NET != 14 && i == 1) ? 0. : mu; // neutrons carry no screening
    }
    __syncwarp();
    FitT v;
    v.t9 = g(fT9), v.t913 = g(fT913), v.t923 = g(fT923), v.t953 = g(fT953), v.t9i = g(fT9i), v.t9i2 = g(fT9i2);
    v.t9i13 = g(fT9i13), v.t9i23 = g(fT9i23), v.t9i43 = g(fT9i43), v.lt9 = g(fLt9);
    const double val1 = g(fVal1), val2 = g(fVal2), val3 = g(fVal3), val4 = g(fVal4), twoT = g(fTwoT);
    const int    kb = (int)g(fKb);
    if constexpr (NET == 14)
    {
        for (int i = 4 + lane; i < 14; i += 32)
        {
            const double* f  = nv.fit + (i - 4) * 8;
            const double  f0 = __ldg(f), f1 = __ldg(f + 1), f2 = __ldg(f + 2), f3 = __ldg(f + 3),
                         f4 = __ldg(f + 4), f5 = __ldg(f + 5), f6 = __ldg(f + 6), f7 = __ldg(f + 7);
            const double coef  = f1 * v.t9i + f2 * v.t9i13 + f3 * v.t913 + f4 * v.t9 + f5 * v.t953 + f6 * v.lt9;
            const double dcoef = (-f1 * v.t9i2 + (-f2 * v.t9i43 + f3 * v.t9i23 + 5 * f5 * v.t923) * (1. / 3.) + f4 +
                                  f6 * v.t9i) *
                                 1e-9;
            const double q   = __ldg(nv.q + i - 4);
            const double dmu = S.mu[i - 1] + S.mu[0] - S.mu[i];
            const double e = exp(f0 + coef + dmu), de = e * (dcoef - dmu * twoT);
            const double l = __ldg(nv.part + (i - 4) * 24 + kb) * exp(coef + f7 - q * val1 + val2);
            S.f[i - 1] = e, S.df[i - 1] = de;
            S.f[16 + i - 1] = l, S.df[16 + i - 1] = l * (dcoef + q * val3 + val4);
        }
    }
    else
    {
        for (int i = 7 + lane; i < 157; i += 32)
        {
            const double* f  = nv.fit + (i - 7) * 8;
            const double  f0 = __ldg(f), f1 = __ldg(f + 1), f2 = __ldg(f + 2), f3 = __ldg(f + 3),
                         f4 = __ldg(f + 4), f5 = __ldg(f + 5), f6 = __ldg(f + 6), f7 = __ldg(f + 7);
            const double coef  = f1 * v.t9i + f2 * v.t9i13 + f3 * v.t913 + f4 * v.t9 + f5 * v.t953 + f6 * v.lt9;
            const double dcoef = (-f1 * v.t9i2 + (-f2 * v.t9i43 + f3 * v.t9i23 + 5 * f5 * v.t923) * (1. / 3.) + f4 +
                                  f6 * v.t9i) *
                                 1e-9;
            const int    mr = __ldg(nv.mainReactant + i), sr = __ldg(nv.secondaryReactant + i),
                      mp = __ldg(nv.mainProduct + i);
            const double part = __ldg(nv.part + (i - 7) * 24 + kb);
            const double q    = __ldg(nv.q + i - 7);
            const double dmu  = S.mu[mr] + S.mu[sr] - S.mu[mp];
            const double sdmu = i >= 137 ? dmu : 0.;
            const double xr   = f7 + coef - val1 * q + (i < 137 ? val2 : 0.);
            const double dr   = dcoef + val3 * q + (i < 137 ? val4 : 0.);
            double       e, de, l, dl;
            if ((i >= 137 && i < 154) || i == 156)
            {
                e = part * exp(xr + dmu), de = e * (dr - dmu * twoT);
                l = exp(f0 + coef + sdmu), dl = l * (dcoef - sdmu * twoT);
            }
            else
            {
                e = exp(f0 + coef + dmu), de = e * (dcoef - dmu * twoT);
                l = part * exp(xr + sdmu), dl = l * (dr - sdmu * twoT);
            }
            S.f[fwdSlot86(i)] = e, S.df[fwdSlot86(i)] = de;
            S.f[revSlot86(i)] = l, S.df[revSlot86(i)] = dl;
        }
    }
    if (lane < 9)
    {
        const int q = specialSlot(NET, lane);
        S.f[q] = g(fSp0 + 2 * lane), S.df[q] = g(fSp0 + 2 * lane + 1);
    }
    if constexpr (NET == 87)
    {
        if (lane == 0)
        {
            S.BE[86] = __ldg(nv.BE + 86) + -1.5 * cf.nakbt;
            S.BE[0]  = S.BE[0] + g(fEv0 + 4);
            S.BE[1]  = S.BE[1] + g(fEv0 + 5);
            S.f[309] = g(fEv0 + 0), S.df[309] = g(fEv0 + 1);
            S.f[310] = g(fEv0 + 2), S.df[310] = g(fEv0 + 3);
        }
    }
    __syncwarp();
}

} // namespace

template<int NET, bool MIXED>
constexpr int perWarpDoubles()
{
    return WarpSmem<NET, MIXED>::doubles;
}

// The whole burn of one network's particles by the calling warp.  wb: this warp's shared
// memory (perWarpDoubles<NET, MIXED>() or more); VS: abundance doubles per slot (at least
// 2 * padN<NET>()).  Global warp gw owns scratch + gw * 32 * (VS + kSlotFields): its 32 slots'
// abundances (slot l at l * VS: Y then Yn), then its slot table (32 * kSlotFields).
template<int NET, int EOS, bool MIXED, bool POST>
__device__ void batchLoop(const BurnParams& bp, const NetView& nv, const HelmView& hv, double* scratch, int VS,
                          double* wb)
{
    using D                 = WDims<NET>;
    constexpr int NP        = padN<NET>();
    const int             lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpSmem<NET, MIXED>  S(wb);
    const size_t          gw   = (size_t)blockIdx.x * (blockDim.x >> 5) + warp;
    double*               vec0 = scratch + gw * 32 * (size_t)(VS + kSlotFields); // slot l at vec0 + l * VS
    double*               sc   = vec0 + 32 * VS;
    const SparseView&     sp   = nv.sp;

    // spread a small batch over every warp of the grid before filling warps
    const size_t  warps  = (size_t)gridDim.x * (blockDim.x >> 5);
    const size_t  first  = (bp.P + warps - 1) / warps;
    // particles in flight per warp (fewer shorten each particle's iteration latency)
    const size_t  spw    = bp.laneSlots > 0 && bp.laneSlots < 32 ? (size_t)bp.laneSlots : 32;
    const unsigned long long deadline = launchDeadline(bp);
    ParticleState s;
    bool has = (size_t)lane < (first < spw ? first : spw) && acquireLane<POST>(bp, nv, hv, s, deadline);
    int           act = has ? ACT_LOAD : 0;
    size_t        pw  = 0;
    double        Tth = 0, rhoT = 0, used = 0, abar = 0, zbar = 0, yElec = 0, xT = 0;
    bool          nanF = false;

    const int    gridWarps = (int)warps;
    unsigned int idle      = 0; // consecutive iterations without a particle (rebalancing wait)
    for (;;)
    {
        // ---- rebalancing: once the queue has drained, a warp holding more than its share of
        //      the running particles hands the extras over at their attempt boundaries, and a
        //      warp holding fewer takes them; the heaviest particles thus end up spread over the
        //      grid instead of queueing behind each other in a few warps.  The share is
        //      ceil(running / warps), at most the warp's slots.
        long long pubPos = -1;
        if (bp.migCells)
        {
            const unsigned hasM = __ballot_sync(kFull, has);
            unsigned long long q = 0, enq = 0, deq = 0, run = 0;
            if (lane == 0)
            {
                q   = *(volatile unsigned long long*)bp.queue;
                enq = *(volatile unsigned long long*)bp.migCount;
                deq = *(volatile unsigned long long*)(bp.migCount + 1);
                run = *(volatile unsigned long long*)(bp.migCount + 2);
            }
            q = __shfl_sync(kFull, q, 0);
            if (q >= bp.P)
            {
                enq = __shfl_sync(kFull, enq, 0), deq = __shfl_sync(kFull, deq, 0), run = __shfl_sync(kFull, run, 0);
                const long long total  = (long long)run + (long long)(enq > deq ? enq - deq : 0);
                const int       share  = (int)min((long long)spw, max(1ll, (total + gridWarps - 1) / gridWarps));
                const int       n      = __popc(hasM);
                if (n > share)
                {
                    const unsigned cand = __ballot_sync(kFull, has && s.i == 1 && !(act & ACT_LOAD));
                    if (lowestBits(cand, n - share) >> lane & 1)
                    {
                        pubPos = donateLane(bp, s);
                        if (pubPos >= 0) has = false, act |= ACT_WRITE, pw = s.p; // Y written back in V1
                    }
                }
                else if (n < share && deq < enq)
                {
                    const unsigned freeM = ~hasM & (spw >= 32 ? kFull : ((1u << spw) - 1));
                    for (unsigned m = lowestBits(freeM, share - n); m; m &= m - 1)
                    {
                        if (lane == __ffs(m) - 1 && takeLane(bp, s)) has = true, act |= ACT_LOAD;
                        __syncwarp();
                    }
                }
            }
        }

        // ---- S1: pre-iteration checks (newtonIteration prologue); finished ones are replaced
        bool cont = false;
        while (has)
        {
            int          st    = -1;
            const double dtTot = bp.hydroDt;
            if (s.nit >= bp.maxIter)
                st = ST_MAXITER;
            else if (bp.sliceIters > 0 && s.i == 1 && s.nit - s.nit0 >= bp.sliceIters)
                st = kPaused;
            else if (expired(deadline))
                st = ST_ABORTED;
            else
            {
                rhoT = s.rho - s.drho * (dtTot - s.elapsed);
                used = s.dt;
                if (dtTot - s.elapsed < s.dt) used = dtTot - s.elapsed;
                if (used == 0) st = ST_ZERO_DT;
            }
            if (st == -1)
            {
                ++s.nit;
                const double guessT = s.i <= 1 ? s.T : s.nextT;
                Tth                 = (1 - k::theta) * s.T + k::theta * guessT;
                cont                = true;
                break;
            }
            releaseLane(bp, s, st);
            if (act & ACT_LOAD)
            {
                act &= ~ACT_LOAD; // never loaded: the particle arrays still hold its state
                if constexpr (POST)
                    if (st >= 0) postScalar(bp, nv, hv, s.p, true);
            }
            else
                act = (act & ~ACT_FINAL) | ACT_WRITE | (st >= 0 ? ACT_FINAL : 0), pw = s.p;
            has = acquireLane<POST>(bp, nv, hv, s, deadline);
            if (has) act |= ACT_LOAD;
        }

        // ---- V1: per slot, pending updates, write-back / load, θ-blend
        constexpr int JN  = (D::N + 31) / 32;
        const int     a0  = act | (cont ? ACT_BLEND : 0);
        double        abW = 0, zbW = 0; // post-burn EOS sums of this lane's finished particle
        for (unsigned m = __ballot_sync(kFull, a0 != 0); m; m &= m - 1)
        {
            const int    l    = __ffs(m) - 1;
            const int    a    = __shfl_sync(kFull, a0, l);
            const size_t po   = __shfl_sync(kFull, (unsigned long long)pw, l);
            const size_t pn   = __shfl_sync(kFull, (unsigned long long)s.p, l);
            const int    il   = __shfl_sync(kFull, s.i, l);
            double*      v    = vec0 + l * VS;
            double*      vn   = v + NP;
            const bool   post = POST && (a & ACT_FINAL);
            double       ab = 0, zb = 0, ynLast = 0, sx = 0;
            double       yw[JN];
#pragma unroll
            for (int t = 0; t < JN; ++t)
            {
                const int j = lane + 32 * t;
                if (j >= D::N) break;
                double y = v[j], yn = vn[j];
                if (a & ACT_ACCEPT) y = yn <= k::epsilonVector ? 0. : yn;
                if (a & ACT_CONT) yn = yn <= k::epsilonVector ? 0. : yn;
                if (a & ACT_WRITE)
                {
                    if (post)
                        yw[t] = y, sx += y * __ldg(nv.A + j);
                    else
                        bp.Y[j][po] = y;
                }
                if (a & ACT_LOAD) y = __ldcg(&bp.Y[j][pn]);
                if (a & ACT_BLEND)
                {
                    yn = (1 - k::theta) * y + k::theta * (il <= 1 ? y : yn);
                    ab += yn, zb += yn * __ldg(nv.Z + j);
                }
                v[j] = y, vn[j] = yn, ynLast = yn;
            }
            if constexpr (POST)
                if (post) postWarp<D::N>(bp, nv, yw, sx, po, l, lane, abW, zbW);
            if (a & ACT_BLEND)
            {
                ab = warpSum(ab), zb = warpSum(zb);
                // net87: the blended electron abundance Y[86], last element of lane 86 % 32
                const double ye = __shfl_sync(kFull, ynLast, 86 % 32);
                if (lane == l) abar = ab, zbar = zb, yElec = NET == 87 ? ye : 0.;
            }
        }
        // publish the hand-off records of this iteration, now that Y is written back
        if (__any_sync(kFull, pubPos >= 0))
        {
            __threadfence();
            __syncwarp();
            if (pubPos >= 0)
            {
                __threadfence();
                atomicExch(&bp.migCells[pubPos].seq, (unsigned long long)pubPos + 1);
            }
        }
        // post-burn EOS of the particles finished by this lane (lane-parallel)
        if constexpr (POST)
            if (bp.eosU && (a0 & ACT_FINAL)) postEos(bp, hv, pw, abW, zbW);
        act = 0;

        // ---- S2: EOS and the (T, rho)-only rate factors of every running slot
        if (cont) slotScalars<NET, EOS>(nv, hv, bp.mu, sc, lane, s.T, Tth, rhoT, s.drho, used, abar, zbar, yElec);
        __syncwarp();

        // ---- V2: per running slot, rates, system, solve, candidate
        for (unsigned m = __ballot_sync(kFull, cont); m; m &= m - 1)
        {
            const int     l  = __ffs(m) - 1;
            const double* c  = sc + l;
            double*       v  = vec0 + l * VS;
            double*       vn = v + NP;
            for (int j = lane; j < D::N; j += 32)
                S.Y[j] = v[j], S.Yn[j] = vn[j];
            __syncwarp();
            slotRates<NET, MIXED>(nv, S, c, lane);
            warpAssemble<NET, MIXED>(nv, S, c[fT * 32], c[fTth * 32], c[fRho * 32], c[fDrho * 32], c[fCv * 32],
                                     c[fDpdT * 32], c[fDt * 32], lane);
            if constexpr (MIXED)
            {
                const int steps = warpSolveMixed<NET>(nv, S, c[fT * 32], lane, S.scale);
                if (steps < 0)
                {
                    warpSolve64<NET, MIXED>(nv, S, lane); // not settled: this system is solved in FP64
                    if (lane == 0) atomicAdd(bp.stats + kStatFallback, 1ull);
                }
                else if (steps && lane == 0)
                    atomicAdd(bp.stats + kStatRefine, (unsigned long long)steps);
            }
            else
                warpSolve64<NET, MIXED>(nv, S, lane);
            bool nanl = false;
            for (int j = lane; j < D::N; j += 32)
            {
                const double y = S.Y[j] + S.x[__ldg(sp.iperm + j + 1)];
                vn[j]          = y;
                nanl |= isnan(y);
            }
            const bool nan = __any_sync(kFull, nanl);
            if (lane == l) nanF = nan, xT = S.x[sp.tNew];
            __syncwarp();
        }

        // ---- S3: finalizeSystemSubstep / finalizeSystemNR (nuclear_net.hpp:724-782, :887-922)
        if (cont)
        {
            const double dtTot  = bp.hydroDt;
            double       usedDt = s.dt;
            if (dtTot - s.elapsed < s.dt) usedDt = dtTot - s.elapsed;
            const double lastT = s.nextT, T = s.T;
            s.nextT            = T + xT;
            int    iNext       = s.i;
            bool   conv        = false;
            double timestep    = 0;
            if (nanF || isnan(s.nextT) || s.nextT < 0)
            {
                usedDt *= k::nanDtStep;
                iNext = 0;
            }
            else
            {
                const double dT_T = fabs((s.nextT - T) / s.nextT);
                if (s.i >= k::nrMinIt && dT_T > k::nrDTTarget * k::nrDTTol)
                {
                    usedDt *= k::nrDTTol / dT_T;
                    iNext   = 0;
                    s.nextT = T; // the candidate abundances are dropped (Y is kept)
                }
                else
                {
                    act                     = ACT_CONT; // clip the candidate
                    const double correction = fabs((s.nextT - lastT) / s.nextT);
                    if ((s.i >= k::nrMinIt && correction < k::nrItTol) || s.i >= k::nrMaxIt)
                    {
                        const double dTT = fabs((s.nextT - T) / s.nextT);
                        timestep         = usedDt;
                        usedDt           = (dTT == 0 ? k::maxDtStep : k::nrDTTarget / dTT) * timestep;
                        usedDt           = fmin(usedDt, timestep * k::maxDtStep);
                        usedDt           = fmax(usedDt, timestep * k::minDtStep);
                        usedDt           = fmin(usedDt, k::nrMaxDt);
                        conv             = true;
                        act              = ACT_ACCEPT;
                    }
                }
            }
            if (dtTot - s.elapsed < s.dt)
            {
                if (usedDt < dtTot - s.elapsed) s.dt = usedDt;
            }
            else
                s.dt = usedDt;
            int st = -1;
            if (conv)
            {
                s.T = s.nextT;
                s.elapsed += timestep;
                ++s.nsub;
                s.i = 1;
                if ((dtTot - s.elapsed) / dtTot < k::substepDtTol)
                    st = ST_OK;
                else
                    s.cycleReset();
            }
            else if (iNext == 0)
            {
                if (s.cycleRejected())
                    st = ST_LIVELOCK;
                else
                    s.i = 1;
            }
            else
                s.i = iNext + 1;
            if (st >= 0)
            {
                releaseLane(bp, s, st);
                act |= ACT_WRITE | ACT_FINAL, pw = s.p;
                has = acquireLane<POST>(bp, nv, hv, s, deadline);
                if (has) act |= ACT_LOAD;
            }
        }
        if (!__any_sync(kFull, has || act != 0))
        {
            // rebalancing: an empty warp stays available while particles are still running, so
            // that hand-offs find a taker; it waits between polls and gives up after a bound
            if (!bp.migCells) break;
            unsigned long long run = 0, pend = 0;
            if (lane == 0)
            {
                run  = *(volatile unsigned long long*)(bp.migCount + 2);
                pend = *(volatile unsigned long long*)bp.migCount - *(volatile unsigned long long*)(bp.migCount + 1);
            }
            run = __shfl_sync(kFull, run, 0), pend = __shfl_sync(kFull, pend, 0);
            if ((run == 0 && pend == 0) || ++idle > kIdlePolls) break;
            __nanosleep(pend ? 1000 : 20000);
            continue;
        }
        idle = 0;
    }
}

template<int NET, int EOS, bool MIXED, bool POST>
__global__ void __launch_bounds__(32, 9) burnBatchKernel(BurnParams bp, NetView nv, HelmView hv, double* scratch,
                                                      size_t /*unused*/)
{
    extern __shared__ __align__(16) double smem[];
    double* wb = smem + (size_t)(threadIdx.x >> 5) * perWarpDoubles<NET, MIXED>();
    batchLoop<NET, EOS, MIXED, POST>(bp, nv, hv, scratch, 2 * padN<NET>(), wb);
}

// One launch over sub-batches of different networks (the uneven mixed workload): every warp
// drains the net86 queue, then net87, then net14, so the expensive particles start first and
// the cheap ones fill the tail.  A warp changes network once all its lanes are idle.
template<int EOS, bool MIXED, bool POST>
__global__ void __launch_bounds__(32, 9) burnBatchMultiKernel(MultiParams mp, HelmView hv, double* scratch,
                                                           size_t /*unused*/)
{
    extern __shared__ __align__(16) double smem[];
    double*       wb = smem + (size_t)(threadIdx.x >> 5) * perWarpDoubles<87, MIXED>();
    constexpr int VS = 2 * padN<87>();
    if (mp.active[1]) batchLoop<86, EOS, MIXED, POST>(mp.bp[1], mp.nv[1], hv, scratch, VS, wb);
    if (mp.active[2]) batchLoop<87, EOS, MIXED, POST>(mp.bp[2], mp.nv[2], hv, scratch, VS, wb);
    if (mp.active[0]) batchLoop<14, EOS, MIXED, POST>(mp.bp[0], mp.nv[0], hv, scratch, VS, wb);
}

// Registry entries: slot scratch per thread, shared memory per one-warp block.  `post`
// selects the instantiation that applies the post-burn steps as particles retire.
template<int NET, int EOS, bool MIXED, bool POST>
KernelInfo batchInfo()
{
    // lanesPerParticle = 32: a small batch is spread one particle per warp over the grid
    return {(const void*)burnBatchKernel<NET, EOS, MIXED, POST>, (size_t)2 * padN<NET>() + kSlotFields, 32,
            WDims<NET>::NNZ, perWarpDoubles<NET, MIXED>() * sizeof(double), 32, true};
}

template<int NET>
KernelInfo pickBatchNet(int eos, int mixed, bool post)
{
    if (eos)
    {
        if (mixed) return post ? batchInfo<NET, 1, true, true>() : batchInfo<NET, 1, true, false>();
        return post ? batchInfo<NET, 1, false, true>() : batchInfo<NET, 1, false, false>();
    }
    if (mixed) return post ? batchInfo<NET, 0, true, true>() : batchInfo<NET, 0, true, false>();
    return post ? batchInfo<NET, 0, false, true>() : batchInfo<NET, 0, false, false>();
}

template<int EOS, bool MIXED, bool POST>
KernelInfo batchMultiInfo()
{
    static_assert(perWarpDoubles<87, MIXED>() >= perWarpDoubles<86, MIXED>() &&
                      perWarpDoubles<87, MIXED>() >= perWarpDoubles<14, MIXED>(),
                  "net87 has the largest warp layout");
    return {(const void*)burnBatchMultiKernel<EOS, MIXED, POST>, (size_t)2 * padN<87>() + kSlotFields, 32,
            WDims<87>::NNZ, perWarpDoubles<87, MIXED>() * sizeof(double), 32, true};
}

template<int EOS>
KernelInfo pickBatchMulti(int mixed, bool post)
{
    if (mixed) return post ? batchMultiInfo<EOS, true, true>() : batchMultiInfo<EOS, true, false>();
    return post ? batchMultiInfo<EOS, false, true>() : batchMultiInfo<EOS, false, false>();
}

// per-slot doubles of the batched layout's scratch (the largest network's)
constexpr size_t kBatchSlotDoubles = (size_t)2 * padN<87>() + kSlotFields;
static_assert(kBatchSlotDoubles <= kNoallocSlotDoubles, "nnet_burn_noalloc's fixed slots are too small");

} // namespace nnet_gb300

