// Warp-per-particle forms of the sparse and mixed-precision burn.
//
// The thread-per-particle kernels keep each particle's Newton system in per-slot global
// scratch (about 25 KB per net86 particle), so every update of the matrix is a dependent
// round trip to L2/HBM and the kernel is latency-bound.  Here one warp owns one particle at
// a time and the whole system lives in shared memory (about 23 KB per warp for net86):
//   * species-, reaction- and matrix-entry-parallel phases are spread over the 32 lanes;
//   * accumulations are gathers in a fixed order (WarpPlan), and the few long lists (the
//     p, n, alpha rows and columns) are split across the warp and summed with a fixed
//     butterfly, so no two lanes write one word and results are deterministic;
//   * the right-looking LU runs by levels of mutually independent pivots: reciprocals,
//     multipliers, then every target's updates in parallel; the solves follow the levels;
//   * scalar work (EOS, special rates, Newton control) is evaluated identically by every
//     lane, so control flow is warp-uniform.
// The mixed form factors in FP32 (cheap reciprocals, FP32 pipe) with FP64 residuals; the
// FP64 pipe, which bounds GB300 here, then only sees rates, assembly and residuals.
#include "launch.hpp"
#include "warp_system.cuh"

namespace nnet_gb300
{

// ------------------------------------------------------------------ rates (warp)
template<int NET, bool MIXED>
__device__ void warpRates(const NetView& nv, WarpSmem<NET, MIXED>& S, double T, double rho, int lane)
{
    const CoulombFast cf(T, rho);
    constexpr int     NS = NET == 14 ? 14 : 86;
    for (int i = lane; i < NS; i += 32)
    {
        double be, mu;
        cf.beMu(nv, i, be, mu);
        S.BE[i] = be;
        S.mu[i] = (NET != 14 && i == 1) ? 0. : mu; // neutrons carry no screening // neutrons carry no screening
    }
    __syncwarp();
    const FitT   v(T);
    const double twoT = 2. / T;
    const int    kb   = temperatureRange(T);
    Special      s;
    if constexpr (NET == 14)
    {
        const double t9 = T / 1.e9, t9i = 1.e0 / t9, lt9 = log(t9);
        const double val1 = 11.6045e0 * t9i, val2 = 1.5e0 * lt9, val3 = val1 * t9i * 1e-9, val4 = 1.5e-9 * t9i;
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
        specialRates(T, s);
        const double* m = S.mu;
        screenFast(s.e3a, s.de3a, m[0] + m[0] - m[1] + m[0], T);
        screenFast(s.ecag, s.decag, m[1] + m[0] - m[2], T);
        screenFast(s.eoag, s.deoag, m[2] + m[0] - m[3], T);
        screenFast(s.e2c, s.de2c, 2. * m[1] - m[3], T);
        screenFast(s.eco, s.deco, m[1] + m[2] - m[4], T);
        screenFast(s.e2o, s.de2o, 2. * m[2] - m[5], T);
        if (lane == 0)
        {
            S.f[0] = s.e3a, S.df[0] = s.de3a, S.f[1] = s.ecag, S.df[1] = s.decag;
            S.f[2] = s.eoag, S.df[2] = s.deoag, S.f[13] = s.e2c, S.df[13] = s.de2c;
            S.f[14] = s.eco, S.df[14] = s.deco, S.f[15] = s.e2o, S.df[15] = s.de2o;
            S.f[16] = s.l3a, S.df[16] = s.dl3a, S.f[17] = s.lcag, S.df[17] = s.dlcag;
            S.f[18] = s.loag, S.df[18] = s.dloag;
        }
    }
    else
    {
        const double t9 = T * 1e-09, t9i = 1. / t9;
        const double val1 = 11.6045 * t9i, val2 = 1.5 * log(t9), val3 = val1 * t9i * 1e-9, val4 = 1.5e-9 * t9i;
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
        specialRates(T, s);
        auto dmu = [&](int i) {
            return S.mu[__ldg(nv.mainReactant + i)] + S.mu[__ldg(nv.secondaryReactant + i)] -
                   S.mu[__ldg(nv.mainProduct + i)];
        };
        screenFast(s.e2c, s.de2c, dmu(0), T);
        screenFast(s.eco, s.deco, dmu(1), T);
        screenFast(s.e2o, s.de2o, dmu(2), T);
        screenFast(s.e3a, s.de3a, dmu(4) + S.mu[__ldg(nv.mainReactant + 4)], T);
        screenFast(s.ecag, s.decag, dmu(5), T);
        screenFast(s.eoag, s.deoag, dmu(6), T);
        if (lane == 0)
        {
            S.f[0] = s.e2c, S.df[0] = s.de2c, S.f[1] = s.eco, S.df[1] = s.deco;
            S.f[2] = s.e2o, S.df[2] = s.de2o, S.f[3] = s.e3a, S.df[3] = s.de3a;
            S.f[4] = s.ecag, S.df[4] = s.decag, S.f[5] = s.eoag, S.df[5] = s.deoag;
            S.f[revSlot86(4)] = s.l3a, S.df[revSlot86(4)] = s.dl3a;
            S.f[revSlot86(5)] = s.lcag, S.df[revSlot86(5)] = s.dlcag;
            S.f[revSlot86(6)] = s.loag, S.df[revSlot86(6)] = s.dloag;
        }
        if constexpr (NET == 87)
        {
            // electron captures (net87.hpp:117-175)
            const double rhoElec = S.Yn[86] * rho;
            double       ev[12];
            electronRates(nv, T, rhoElec, ev);
            const double kbt = NNET_KB * T, nakbt = NNET_NA * kbt;
            if (lane == 0)
            {
                S.BE[86] = __ldg(nv.BE + 86) + -1.5 * nakbt;
                S.BE[0]  = S.BE[0] + -ev[3];
                S.BE[1]  = S.BE[1] + -ev[9];
                S.f[309] = rhoElec == 0 ? 0 : ev[0] / rhoElec, S.df[309] = rhoElec == 0 ? 0 : ev[1] / rhoElec;
                S.f[310] = rhoElec == 0 ? 0 : ev[6] / rhoElec, S.df[310] = rhoElec == 0 ? 0 : ev[7] / rhoElec;
            }
        }
    }
    __syncwarp();
}

// ------------------------------------------------------------------ driver (warp)
template<int NET, int EOS, bool MIXED>
__global__ void __launch_bounds__(128) burnWarpKernel(BurnParams bp, NetView nv, HelmView hv, double* /*unused*/,
                                                      size_t /*unused*/)
{
    using D = WDims<NET>;
    extern __shared__ __align__(16) double smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double*   base = smem + (size_t)warp * WarpSmem<NET, MIXED>::doubles;
    WarpSmem<NET, MIXED> S(base);
    const SparseView& sp = nv.sp;

    const unsigned long long deadline = launchDeadline(bp);
    ParticleState            s;
    for (;;)
    {
        // ---- acquire (lane 0 takes the queue index; every lane then reads the same words)
        unsigned long long q = 0;
        if (lane == 0) q = atomicAdd(bp.queue, 1ull);
        q = __shfl_sync(kFull, q, 0);
        if (q >= bp.P) break;
        const size_t p     = bp.order ? (size_t)bp.order[q] : (size_t)q;
        const int    phase = bp.rs.phase ? bp.rs.phase[p] : 0;
        if (phase == 2) continue;
        const double rho0 = bp.rho[p], T0 = bp.T[p];
        const bool skip = phase == 0 && !(rho0 > k::minRho && T0 > k::minTemp);
        const bool late = __shfl_sync(kFull, (int)expired(deadline), 0) != 0;
        if (skip || late)
        {
            if (lane == 0) endUntouched(bp, p, skip ? ST_SKIPPED : ST_ABORTED);
            continue;
        }
        for (int j = lane; j < D::N; j += 32)
            S.Y[j] = bp.Y[j][p];
        s.p = p, s.T = T0, s.dt = bp.dt[p], s.rho = rho0, s.i = 1;
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
            if (bp.useDrhodt && bp.rhoM1 && bp.rhoM1[p] != 0) drho = (rho0 - bp.rhoM1[p]) / bp.previousDt;
            s.elapsed = 0, s.nextT = 0, s.drho = drho, s.nit = 0, s.nsub = 0;
            s.cycleReset();
        }
        s.nit0 = s.nit;
        __syncwarp();

        // ---- Newton iterations of this particle
        int st;
        for (;;)
        {
            if (s.nit >= bp.maxIter)
            {
                st = ST_MAXITER;
                break;
            }
            if (bp.sliceIters > 0 && s.i == 1 && s.nit - s.nit0 >= bp.sliceIters)
            {
                st = kPaused;
                break;
            }
            if (deadline && __shfl_sync(kFull, (int)expired(deadline), 0))
            {
                st = ST_ABORTED;
                break;
            }
            const double dtTot = bp.hydroDt;
            const double rhoT  = s.rho - s.drho * (dtTot - s.elapsed);
            double       used  = s.dt;
            if (dtTot - s.elapsed < s.dt) used = dtTot - s.elapsed;
            if (used == 0)
            {
                st = ST_ZERO_DT;
                break;
            }
            ++s.nit;
            const double guessT = s.i <= 1 ? s.T : s.nextT;
            const double Ttheta = (1 - k::theta) * s.T + k::theta * guessT;
            double       ab = 0, zb = 0;
            for (int j = lane; j < D::N; j += 32)
            {
                const double y  = S.Y[j];
                const double yn = (1 - k::theta) * y + k::theta * (s.i <= 1 ? y : S.Yn[j]);
                S.Yn[j]         = yn;
                ab += yn, zb += yn * __ldg(nv.Z + j);
            }
            __syncwarp();
            EosResult eos;
            if constexpr (EOS == NNET_EOS_IDEAL_GAS)
                eos = idealGasEos(bp.mu, Ttheta, rhoT);
            else
                eos = helmholtzEos(hv, warpSum(ab), warpSum(zb), Ttheta, rhoT);

            warpRates<NET, MIXED>(nv, S, Ttheta, rhoT, lane);
            warpAssemble<NET, MIXED>(nv, S, s.T, Ttheta, rhoT, s.drho, eos.cv, eos.dpdT, used, lane);
            if constexpr (MIXED)
            {
                const int steps = warpSolveMixed<NET>(nv, S, s.T, lane, S.scale);
                if (steps < 0)
                {
                    // not settled: re-solve this system in FP64 (A and b are intact)
                    warpSolve64<NET, MIXED>(nv, S, lane);
                    if (lane == 0) atomicAdd(bp.stats + kStatFallback, 1ull);
                }
                else if (steps && lane == 0)
                    atomicAdd(bp.stats + kStatRefine, (unsigned long long)steps);
            }
            else
                warpSolve64<NET, MIXED>(nv, S, lane);

            // ---- finalizeSystemSubstep / finalizeSystemNR (nuclear_net.hpp:724-782, :887-922)
            double usedDt = s.dt;
            if (dtTot - s.elapsed < s.dt) usedDt = dtTot - s.elapsed;
            const double lastT = s.nextT, T = s.T;
            bool         nanl  = false;
            for (int j = lane; j < D::N; j += 32)
            {
                const double v = S.Y[j] + S.x[__ldg(sp.iperm + j + 1)];
                S.Yn[j]        = v;
                nanl |= isnan(v);
            }
            const bool nan = __any_sync(kFull, nanl);
            s.nextT        = T + S.x[sp.tNew];
            __syncwarp();
            int    iNext    = s.i;
            bool   conv     = false;
            double timestep = 0;
            if (nan || isnan(s.nextT) || s.nextT < 0)
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
                    iNext = 0;
                    for (int j = lane; j < D::N; j += 32)
                        S.Yn[j] = S.Y[j];
                    s.nextT = T;
                }
                else
                {
                    for (int j = lane; j < D::N; j += 32)
                        if (S.Yn[j] <= k::epsilonVector) S.Yn[j] = 0;
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
                    }
                }
            }
            if (dtTot - s.elapsed < s.dt)
            {
                if (usedDt < dtTot - s.elapsed) s.dt = usedDt;
            }
            else
                s.dt = usedDt;
            __syncwarp();
            if (conv)
            {
                for (int j = lane; j < D::N; j += 32)
                    S.Y[j] = S.Yn[j];
                __syncwarp();
                s.T = s.nextT;
                s.elapsed += timestep;
                ++s.nsub;
                s.i = 1;
                if ((dtTot - s.elapsed) / dtTot < k::substepDtTol)
                {
                    st = ST_OK;
                    break;
                }
                s.cycleReset();
                continue;
            }
            if (iNext == 0)
            {
                if (s.cycleRejected())
                {
                    st = ST_LIVELOCK;
                    break;
                }
                s.i = 1;
                continue;
            }
            s.i = iNext + 1;
        }

        // ---- write back (pause or finish)
        for (int j = lane; j < D::N; j += 32)
            bp.Y[j][p] = S.Y[j];
        __syncwarp();
        if (lane == 0)
        {
            bp.T[p]  = s.T;
            bp.dt[p] = s.dt;
            atomicAdd(bp.stats + kStatIters, (unsigned long long)(s.nit - s.nit0));
            if (st == kPaused)
            {
                const ResumeState& r = bp.rs;
                r.elapsed[p] = s.elapsed, r.nextT[p] = s.nextT, r.drho[p] = s.drho, r.nit[p] = s.nit;
                r.nsub[p] = s.nsub, r.cdDt[p] = s.cdDt, r.cdNt[p] = s.cdNt, r.cdPower[p] = s.cdPower;
                r.cdSteps[p] = s.cdSteps, r.phase[p] = 1;
            }
            else
            {
                if (bp.status) bp.status[p] = st;
                if (bp.substeps) bp.substeps[p] = s.nsub;
                if (bp.iterations) bp.iterations[p] = (int32_t)s.nit;
                atomicAdd(bp.stats + kStatSubsteps, (unsigned long long)s.nsub);
                atomicAdd(bp.stats + kStatStatus + st, 1ull);
                finishSegment(bp, p);
            }
        }
        __syncwarp();
    }
}

template<int NET, int EOS, bool MIXED>
static KernelInfo warpInfo()
{
    return {(const void*)burnWarpKernel<NET, EOS, MIXED>, 0, 128, WDims<NET>::NNZ,
            4 * WarpSmem<NET, MIXED>::doubles * sizeof(double), 32};
}

template<bool MIXED>
static KernelInfo pickWarp(int net, int eos)
{
    if (net == 14) return eos ? warpInfo<14, 1, MIXED>() : warpInfo<14, 0, MIXED>();
    if (net == 86) return eos ? warpInfo<86, 1, MIXED>() : warpInfo<86, 0, MIXED>();
    return eos ? warpInfo<87, 1, MIXED>() : warpInfo<87, 0, MIXED>();
}

KernelInfo warpKernel(int net, int eos, int mixed) { return mixed ? pickWarp<true>(net, eos) : pickWarp<false>(net, eos); }

} // namespace nnet_gb300
