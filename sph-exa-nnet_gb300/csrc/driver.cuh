// Persistent burn kernel: one thread per particle, a device work queue, and the θ-method
// Newton substep state machine of the reference (include/nnet/nuclear_net.hpp:850-959)
// unrolled into one Newton iteration per loop trip, so that every thread of a warp runs
// the same iteration code whatever substep or attempt its particle is in.  When a
// particle finishes (accepted to hydro_dt, fixed point, budget, zero dt) the thread writes
// it back and pulls the next index from the queue; uneven substep counts therefore never
// idle a lane while work remains.
//
// A solver policy supplies the per-slot scratch views (Y, Yn, DY) and `assembleSolve`,
// which builds the Newton system around the guess and leaves the solution in DY.
#pragma once

#include "physics.cuh"

namespace nnet_gb300
{

template<int NET>
struct NetDims
{
    static constexpr int N = NET;
    static constexpr int n = NET + 1;
    static constexpr int R = NET == 14 ? NET14_NUM_REACTIONS : NET == 86 ? NET86_NUM_REACTIONS : NET87_NUM_REACTIONS;
};

struct ParticleState
{
    size_t             p;
    double             T, dt, elapsed, nextT, rho, drho;
    long long          nit, nit0; // Newton iterations so far / at the start of this launch
    int                i, nsub;
    unsigned long long cdDt, cdNt; // cycle detection: saved attempt-start state (bits)
    int                cdPower, cdSteps;

    // Between accepted substeps an attempt is fully determined by (dt, Newton temperature
    // buffer).  The reference's rejection rule (nuclear_net.hpp:745-748 with :899-904) can
    // return to a pair it has seen, or let dt settle on the value it maps to itself
    // (dt <- dt 4 / |dT/T| is stationary where |dT/T| = 4, far above the 0.04 acceptance
    // bound) and wander there within rounding noise; either way it retries forever.
    // Brent's algorithm on the pair: the temperature compared bitwise, dt within a relative
    // kCycleDtTol (a bitwise dt test catches the wandering case only when the noise happens
    // to repeat a value, after any number of attempts).
    __device__ __forceinline__ void cycleReset()
    {
        cdDt = __double_as_longlong(dt), cdNt = __double_as_longlong(nextT), cdPower = 1, cdSteps = 0;
    }
    __device__ __forceinline__ bool cycleRejected()
    {
        const unsigned long long a = __double_as_longlong(dt), b = __double_as_longlong(nextT);
        if (b == cdNt && (a == cdDt || fabs(dt - __longlong_as_double(cdDt)) <= k::cycleDtTol * dt)) return true;
        if (++cdSteps == cdPower) cdDt = a, cdNt = b, cdPower <<= 1, cdSteps = 0;
        return false;
    }
};

template<int NET, int EOS>
__device__ __forceinline__ EosResult evalEos(const NetView& nv, const HelmView& hv, double mu, Strided<double> Yn,
                                             double T, double rho)
{
    if constexpr (EOS == NNET_EOS_IDEAL_GAS) { return idealGasEos(mu, T, rho); }
    else
    {
        // HelmholtzFunctor: abar_ = sum Y, zbar_ = sum Y Z over the network's species
        // (helmholtz.hpp:217-225; net87 includes the electron entry, Z = -1)
        double abar = 0, zbar = 0;
        for (int j = 0; j < NET; ++j)
            abar = abar + Yn[j];
        for (int j = 0; j < NET; ++j)
            zbar += Yn[j] * __ldg(nv.Z + j);
        return helmholtzEos(hv, abar, zbar, T, rho);
    }
}

template<int NET>
__device__ __forceinline__ void networkRates(const NetView& nv, Strided<double> Yg, double T, double rho,
                                             Strided<double> BE, Strided<double> rates, Strided<double> drates)
{
    if constexpr (NET == 14)
        net14Rates(nv, T, rho, BE, rates, drates);
    else if constexpr (NET == 86)
        net86Rates(nv, T, rho, BE, rates, drates);
    else
        net87Rates(nv, Yg[86], T, rho, BE, rates, drates);
}

// Helmholtz EOS of the post-burn step, written to particle p's outputs (out of line: it runs
// once per particle, and inlining it would add its registers to the burn loop's)
static __device__ __noinline__ void postEos(const BurnParams& bp, const HelmView& hv, size_t p, double abar,
                                            double zbar)
{
    const EosResult e = helmholtzEos(hv, abar, zbar, bp.T[p], bp.rho[p]);
    bp.eosU[p] = e.u, bp.eosCv[p] = e.cv, bp.eosP[p] = e.p, bp.eosC[p] = e.c, bp.eosDpdT[p] = e.dpdT;
}

// Post-burn steps of particle p by one thread, on the state in the particle arrays:
// s = sum_i A_i Y_i, reported as s - 1; Y_i <- Y_i / s when `normalize` (and s is positive
// and finite); then the Helmholtz EOS at the final state over the network's charges
// (computeHelmEOS, parallel_nuclear_net.hpp:191-261 with cudaKernelComputeHelmholtz,
// CUDA/parallel_nuclear_net.cu:184-210).
static __device__ __noinline__ void postScalar(const BurnParams& bp, const NetView& nv, const HelmView& hv, size_t p,
                                               bool normalize)
{
    const int N  = nv.nspec;
    double    sx = 0;
    for (int j = 0; j < N; ++j)
        sx += bp.Y[j][p] * __ldg(nv.A + j);
    if (bp.massDrift) bp.massDrift[p] = sx - 1.;
    const bool scale = normalize && bp.normalize && sx > 0 && sx < INFINITY;
    double     ab = 0, zb = 0;
    for (int j = 0; j < N; ++j)
    {
        double y = bp.Y[j][p];
        if (scale)
        {
            y          = y / sx;
            bp.Y[j][p] = y;
        }
        ab += y, zb += y * __ldg(nv.Z + j);
    }
    if (bp.eosU) postEos(bp, hv, p, ab, zb);
}

// launch watchdog: true once the launch has run past its time limit (deadline 0: no limit)
__device__ __forceinline__ bool expired(unsigned long long deadline)
{
    return deadline != 0 && globalTimerNs() > deadline;
}
__device__ __forceinline__ unsigned long long launchDeadline(const BurnParams& bp)
{
    return bp.timeLimitNs ? globalTimerNs() + bp.timeLimitNs : 0;
}

// Fetch the next burnable particle; skipped ones (rho <= 1e5 or T <= 1e8,
// parallel_nuclear_net_impl.cpp:83) are written back immediately.
__device__ __forceinline__ void finishSegment(const BurnParams& bp, size_t p)
{
    if (bp.rs.phase) bp.rs.phase[p] = 2;
    if (bp.segFinished) atomicAdd(bp.segFinished + (bp.segOf ? bp.segOf[p] : 0), 1ull);
}

// A particle that ends without a Newton iteration: skipped (cold) or, once the launch is past
// its time limit, aborted before it started; its state stays as it is.
__device__ __forceinline__ void endUntouched(const BurnParams& bp, size_t p, int st)
{
    if (bp.status) bp.status[p] = st;
    if (bp.substeps) bp.substeps[p] = 0;
    if (bp.iterations) bp.iterations[p] = 0;
    atomicAdd(bp.stats + kStatStatus + st, 1ull);
    finishSegment(bp, p);
}

template<int NET, class Policy>
__device__ bool acquire(const BurnParams& bp, Policy& pol, ParticleState& s, unsigned long long deadline)
{
    for (;;)
    {
        unsigned long long q = atomicAdd(bp.queue, 1ull);
        if (q >= bp.P) return false;
        const size_t p     = bp.order ? (size_t)bp.order[q] : (size_t)q;
        const int    phase = bp.rs.phase ? bp.rs.phase[p] : 0;
        if (phase == 2) continue; // finished in an earlier launch
        const double rho = bp.rho[p], T = bp.T[p];
        if (phase == 0 && !(rho > k::minRho && T > k::minTemp))
        {
            endUntouched(bp, p, ST_SKIPPED);
            continue;
        }
        if (expired(deadline))
        {
            endUntouched(bp, p, ST_ABORTED);
            continue;
        }
        for (int j = 0; j < NET; ++j)
            pol.Y[j] = bp.Y[j][p];
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
        return true;
    }
}

template<int NET, class Policy>
__device__ void writeState(const BurnParams& bp, Policy& pol, const ParticleState& s)
{
    for (int j = 0; j < NET; ++j)
        bp.Y[j][s.p] = pol.Y[j];
    bp.T[s.p]  = s.T;
    bp.dt[s.p] = s.dt;
}

template<int NET, class Policy>
__device__ void release(const BurnParams& bp, Policy& pol, const ParticleState& s, int status)
{
    writeState<NET>(bp, pol, s);
    if (bp.status) bp.status[s.p] = status;
    if (bp.substeps) bp.substeps[s.p] = s.nsub;
    if (bp.iterations) bp.iterations[s.p] = (int32_t)s.nit;
    atomicAdd(bp.stats + kStatIters, (unsigned long long)(s.nit - s.nit0));
    atomicAdd(bp.stats + kStatSubsteps, (unsigned long long)s.nsub);
    atomicAdd(bp.stats + kStatStatus + status, 1ull);
    finishSegment(bp, s.p);
}

// pause at an attempt boundary: everything the next attempt depends on is saved
template<int NET, class Policy>
__device__ void pause(const BurnParams& bp, Policy& pol, const ParticleState& s)
{
    writeState<NET>(bp, pol, s);
    const ResumeState& r = bp.rs;
    const size_t       p = s.p;
    r.elapsed[p] = s.elapsed, r.nextT[p] = s.nextT, r.drho[p] = s.drho, r.nit[p] = s.nit, r.nsub[p] = s.nsub;
    r.cdDt[p] = s.cdDt, r.cdNt[p] = s.cdNt, r.cdPower[p] = s.cdPower, r.cdSteps[p] = s.cdSteps;
    r.phase[p] = 1;
    atomicAdd(bp.stats + kStatIters, (unsigned long long)(s.nit - s.nit0));
}

constexpr int kPaused = -2;

// One Newton iteration of the substep loop.  Returns -1 to continue, or the particle's
// final status.
template<int NET, int EOS, class Policy>
__device__ int newtonIteration(const BurnParams& bp, const NetView& nv, const HelmView& hv, Policy& pol,
                               ParticleState& s, unsigned long long deadline)
{
    if (s.nit >= bp.maxIter) return ST_MAXITER;
    if (expired(deadline)) return ST_ABORTED;
    if (bp.sliceIters > 0 && s.i == 1 && s.nit - s.nit0 >= bp.sliceIters) return kPaused;

    // prepareSystemSubstep (nuclear_net.hpp:858-879)
    const double dtTot = bp.hydroDt;
    const double rhoT  = s.rho - s.drho * (dtTot - s.elapsed);
    double       used  = s.dt;
    if (dtTot - s.elapsed < s.dt) used = dtTot - s.elapsed;
    if (used == 0) return ST_ZERO_DT;
    ++s.nit;

    // prepareSystemNR (nuclear_net.hpp:698-716): θ-blend of the guess
    double guessT = s.nextT;
    if (s.i <= 1)
    {
        for (int j = 0; j < NET; ++j)
            pol.Yn[j] = pol.Y[j];
        guessT = s.T;
    }
    const double Ttheta = (1 - k::theta) * s.T + k::theta * guessT;
    for (int j = 0; j < NET; ++j)
        pol.Yn[j] = (1 - k::theta) * pol.Y[j] + k::theta * pol.Yn[j];
    const EosResult eos = evalEos<NET, EOS>(nv, hv, bp.mu, pol.Yn, Ttheta, rhoT);

    pol.assembleSolve(nv, s.T, Ttheta, rhoT, s.drho, eos.cv, eos.dpdT, used);

    // finalizeSystemSubstep (nuclear_net.hpp:891-921) with finalizeSystemNR (:724-782)
    double usedDt = s.dt;
    if (dtTot - s.elapsed < s.dt) usedDt = dtTot - s.elapsed;
    const double lastT = s.nextT;
    bool         nan   = false;
    for (int j = 0; j < NET; ++j)
    {
        const double v = pol.Y[j] + pol.dy(nv.sp, j + 1);
        pol.Yn[j]      = v;
        nan |= isnan(v);
    }
    const double T = s.T;
    s.nextT        = T + pol.dy(nv.sp, 0);
    int  iNext     = s.i;
    bool conv      = false;
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
            for (int j = 0; j < NET; ++j)
                pol.Yn[j] = pol.Y[j];
            s.nextT = T;
        }
        else
        {
            for (int j = 0; j < NET; ++j)
                if (pol.Yn[j] <= k::epsilonVector) pol.Yn[j] = 0;
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

    if (conv)
    {
        for (int j = 0; j < NET; ++j)
            pol.Y[j] = pol.Yn[j];
        s.T = s.nextT;
        s.elapsed += timestep;
        ++s.nsub;
        s.i = 1;
        if ((dtTot - s.elapsed) / dtTot < k::substepDtTol) return ST_OK;
        s.cycleReset();
        return -1;
    }
    if (iNext == 0)
    {
        // rejected attempt: a repeated attempt-start state means the loop never ends
        if (s.cycleRejected()) return ST_LIVELOCK;
        s.i = 1;
        return -1;
    }
    s.i = iNext + 1;
    return -1;
}

template<int NET, int EOS, class Policy>
__device__ __forceinline__ void burnLoop(const BurnParams& bp, const NetView& nv, const HelmView& hv, Policy& pol)
{
    const unsigned long long deadline = launchDeadline(bp);
    ParticleState            s;
    bool                     have = acquire<NET>(bp, pol, s, deadline);
    while (have)
    {
        const int st = newtonIteration<NET, EOS>(bp, nv, hv, pol, s, deadline);
        if (st >= 0)
        {
            release<NET>(bp, pol, s, st);
            have = acquire<NET>(bp, pol, s, deadline);
        }
        else if (st == kPaused)
        {
            pause<NET>(bp, pol, s);
            have = acquire<NET>(bp, pol, s, deadline);
        }
    }
}

} // namespace nnet_gb300
