// Test infrastructure, not product code: a C driver around the reference's own
// burn-path sources, compiled (by build_ref() in oracle/build.py) together with
//   include/nnet/parameterization/net14/net14.cpp
//   include/nnet/parameterization/net86/net86.cpp
//   include/nnet/parameterization/net87/net87.cpp
//   include/nnet/parameterization/eos/helmholtz.cpp
// into oracle/_ref/libnnet_ref.so.  It is used only to pin the oracle restatement
// (oracle/nnet_oracle.cpp) and to generate the golden fixtures under tests/golden.
//
// The per-particle loop calls the reference's step functions in the order of
// solveSystemSubstep (include/nnet/nuclear_net.hpp:944-958): prepareSystemSubstep,
// eigen::solve, finalizeSystemSubstep.  Compared with the reference's batch driver
// (include/nnet/parallel/implementation/parallel_nuclear_net_impl.cpp:63-103) it adds
// a per-particle Newton-iteration budget, a status code and detection of the exact
// fixed point the substep loop can enter (a rejected attempt that leaves dt
// unchanged replays bit for bit forever, nuclear_net.hpp:745-748 with :899-904).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <omp.h>

#include "nnet/nuclear_net.hpp"
#include "nnet/parameterization/net14/net14.hpp"
#include "nnet/parameterization/net86/net86.hpp"
#include "nnet/parameterization/net87/net87.hpp"
#include "nnet/parameterization/eos/helmholtz.hpp"
#include "nnet/parameterization/eos/ideal_gas.hpp"
#include "nnet_util/algorithm.hpp"

namespace nnet::eos::helmholtz::constants
{
extern double f[IMAX][JMAX], fd[IMAX][JMAX], ft[IMAX][JMAX], fdd[IMAX][JMAX], ftt[IMAX][JMAX], fdt[IMAX][JMAX],
    fddt[IMAX][JMAX], fdtt[IMAX][JMAX], fddtt[IMAX][JMAX], dpdf[IMAX][JMAX], dpdfd[IMAX][JMAX], dpdft[IMAX][JMAX],
    dpdfdt[IMAX][JMAX], ef[IMAX][JMAX], efd[IMAX][JMAX], eft[IMAX][JMAX], efdt[IMAX][JMAX], xf[IMAX][JMAX],
    xfd[IMAX][JMAX], xft[IMAX][JMAX], xfdt[IMAX][JMAX];
}

namespace
{
// Detection of endless retries on the state an attempt starts from.  Between accepted
// substeps Y, T and the elapsed time do not change, so an attempt is fully determined by
// (dt, Newton temperature buffer); once that pair repeats, or dt settles (within rounding
// noise) on the value the rejection rule maps to itself, the reference's substep loop
// replays rejected attempts forever.  Brent's algorithm, the temperature compared bitwise,
// dt within a relative 2^-20 (the rule of oracle/nnet_oracle.cpp and of the GPU kernels).
struct CycleDetector
{
    unsigned long long sdt = 0, snt = 0;
    long               power = 1, steps = 0;
    static unsigned long long bits(double v)
    {
        unsigned long long b;
        std::memcpy(&b, &v, sizeof b);
        return b;
    }
    void reset(double dt, double nt) { sdt = bits(dt), snt = bits(nt), power = 1, steps = 0; }
    bool rejected(double dt, double nt)
    {
        if (bits(nt) == snt)
        {
            double saved;
            std::memcpy(&saved, &sdt, sizeof saved);
            if (bits(dt) == sdt || std::fabs(dt - saved) <= 9.5367431640625e-07 * dt) return true;
        }
        if (++steps == power) sdt = bits(dt), snt = bits(nt), power <<= 1, steps = 0;
        return false;
    }
};

enum Status
{
    ST_OK       = 0,
    ST_SKIPPED  = 1,
    ST_LIVELOCK = 2,
    ST_MAXITER  = 3,
    ST_ZERO_DT  = 4,
};

struct Net
{
    int                                              dim;
    const nnet::ReactionList*                        list;
    const nnet::ComputeReactionRatesFunctor<double>* rates;
    const double*                                    Z;
};

bool getNet(int net, Net& out)
{
    switch (net)
    {
        case 14:
            out = {14, &nnet::net14::reactionList, &nnet::net14::computeReactionRates,
                   nnet::net14::constants::Z.data()};
            return true;
        case 86:
            out = {86, &nnet::net86::reactionList, &nnet::net86::computeReactionRates,
                   nnet::net86::constants::Z.data()};
            return true;
        case 87:
            out = {87, &nnet::net87::reactionList, &nnet::net87::computeReactionRates,
                   nnet::net87::constants::Z.data()};
            return true;
    }
    return false;
}
} // namespace

extern "C"
{

// Copy a stand-in table (21 x IMAX x JMAX doubles, order f fd ft fdd ftt fdt fddt fdtt
// fddtt dpdf dpdfd dpdft dpdfdt ef efd eft efdt xf xfd xft xfdt) into the
// reference's arrays.  Grid and spacing arrays were filled by readCPUTable.
int ref_load_helmholtz(const double* tab)
{
    namespace c              = nnet::eos::helmholtz::constants;
    double (*dst[21])[JMAX] = {c::f,    c::fd,    c::ft,    c::fdd,  c::ftt, c::fdt, c::fddt,
                               c::fdtt, c::fddtt, c::dpdf,  c::dpdfd, c::dpdft, c::dpdfdt, c::ef,
                               c::efd,  c::eft,   c::efdt,  c::xf,   c::xfd, c::xft, c::xfdt};
    for (int k = 0; k < 21; ++k)
        std::memcpy(dst[k], tab + (size_t)k * IMAX * JMAX, sizeof(double) * IMAX * JMAX);
    return 0;
}

// Helmholtz EOS for given abar_ = sum(Y), zbar_ = sum(Y Z) (helmholtz.cpp:341-965).
// out = {cv, dpdT, p, cp, c, u, dse, dpe, dsp, cv_gaz, cp_gaz, c_gaz, dudYe}
int ref_helmholtz(double abar_, double zbar_, double T, double rho, double* out)
{
    auto r = nnet::eos::helmholtz::helmholtzEos<double>(abar_, zbar_, T, rho);
    double v[13] = {r.cv, r.dpdT, r.p, r.cp, r.c, r.u, r.dse, r.dpe, r.dsp, r.cv_gaz, r.cp_gaz, r.c_gaz, r.dudYe};
    std::memcpy(out, v, sizeof v);
    return 0;
}

// Rates, rate derivatives and corrected binding energies of one network at (Y, T, rho).
// eos_kind 0: ideal gas(mu), 1: Helmholtz over the network's Z.  eos_out receives the
// EOS struct passed to the rate functor (same 13 fields as ref_helmholtz).
int ref_rates(int net, const double* Y, double T, double rho, int eos_kind, double mu, double* BE, double* rates,
              double* drates, double* eos_out)
{
    Net n;
    if (!getNet(net, n)) return -1;
    nnet::eos_struct<double> es;
    if (eos_kind == 0)
        es = nnet::eos::IdealGasFunctor<double>(mu)(Y, T, rho);
    else
        es = nnet::eos::HelmholtzFunctor<double>(n.Z, n.dim)(Y, T, rho);
    (*n.rates)(Y, T, rho, es, BE, rates, drates);
    if (eos_out)
    {
        double v[13] = {es.cv, es.dpdT, es.p, es.cp, es.c, es.u, es.dse, es.dpe, es.dsp, es.cv_gaz, es.cp_gaz, es.c_gaz,
                        es.dudYe};
        std::memcpy(eos_out, v, sizeof v);
    }
    return 0;
}

// Batch burn over P particles.  Y is SoA, species-major: Y[j*P + i].  T and dt are
// updated in place (Y too); drhodt_mode 0 follows the CPU driver (drho/dt always 0,
// parallel_nuclear_net_impl.cpp:89-92), 1 follows the CUDA kernel
// (drho/dt = (rho - rho_m1)/previous_dt when rho_m1 != 0, parallel_nuclear_net.cu:80-82).
// status/substeps/iters are per-particle outputs (may be null).
int ref_burn(int net, int eos_kind, double mu, size_t P, double* Y, double* T, const double* rho,
             const double* rho_m1, double* dt, double hydro_dt, double previous_dt, int drhodt_mode, long max_iter,
             int* status, int* substeps, int* iters, int nthreads)
{
    Net n;
    if (!getNet(net, n)) return -1;
    const int dim = n.dim;
    nnet::eos::IdealGasFunctor<double> ideal(mu);
    nnet::eos::HelmholtzFunctor<double> helm(n.Z, dim);
    const nnet::EosFunctor<double>&    eos = eos_kind == 0 ? (const nnet::EosFunctor<double>&)ideal
                                                           : (const nnet::EosFunctor<double>&)helm;
    const nnet::PtrReactionList        reactions(*n.list);
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    const int batch = ::util::dynamicBatchSize(P, nthreads);

#pragma omp parallel num_threads(nthreads)
    {
        std::vector<double> Mp((dim + 1) * (dim + 1)), RHS(dim + 1), DY_T(dim + 1), Ybuf(dim), Yp(dim),
            rates(n.list->size());
#pragma omp for schedule(dynamic, batch)
        for (size_t p = 0; p < P; ++p)
        {
            int  st = ST_OK, nsub = 0;
            long nit = 0;
            if (!(rho[p] > nnet::constants::minRho && T[p] > nnet::constants::minTemp))
                st = ST_SKIPPED;
            else
            {
                for (int j = 0; j < dim; ++j)
                    Yp[j] = Y[(size_t)j * P + p];
                double drho_dt = 0;
                if (drhodt_mode == 1 && rho_m1 && rho_m1[p] != 0) drho_dt = (rho[p] - rho_m1[p]) / previous_dt;

                double        final_T = T[p], next_T = 0, elapsed = 0, pdt = dt[p];
                CycleDetector cd;
                cd.reset(pdt, next_T);
                for (int i = 1;; ++i)
                {
                    if (nit >= max_iter)
                    {
                        st = ST_MAXITER;
                        break;
                    }
                    double used = pdt;
                    if (hydro_dt - elapsed < pdt) used = hydro_dt - elapsed;
                    if (used == 0)
                    {
                        st = ST_ZERO_DT;
                        break;
                    }
                    ++nit;
                    nnet::prepareSystemSubstep(dim, Mp.data(), RHS.data(), rates.data(), reactions, *n.rates, eos,
                                               Yp.data(), final_T, Ybuf.data(), next_T, rho[p], drho_dt, hydro_dt,
                                               elapsed, pdt, i);
                    eigen::solve(Mp.data(), RHS.data(), DY_T.data(), dim + 1, nnet::constants::epsilonSystem);
                    const double elapsed0 = elapsed;
                    if (nnet::finalizeSystemSubstep(dim, Yp.data(), final_T, Ybuf.data(), next_T, DY_T.data(), hydro_dt,
                                                    elapsed, pdt, i))
                    {
                        ++nsub;
                        break;
                    }
                    if (i == 0)
                    {
                        if (elapsed != elapsed0)
                        {
                            ++nsub; // accepted substep
                            cd.reset(pdt, next_T);
                        }
                        else if (cd.rejected(pdt, next_T))
                        {
                            st = ST_LIVELOCK; // the rejected attempts cycle: the reference loops forever
                            break;
                        }
                    }
                }
                for (int j = 0; j < dim; ++j)
                    Y[(size_t)j * P + p] = Yp[j];
                T[p]  = final_T;
                dt[p] = pdt;
            }
            if (status) status[p] = st;
            if (substeps) substeps[p] = nsub;
            if (iters) iters[p] = (int)nit;
        }
    }
    return 0;
}

// Single-particle Newton solve without substepping (solveSystemNR,
// include/nnet/nuclear_net.hpp:791-818), as driven by test/net14_test.cpp:134-187.
// Returns the accepted timestep; Y_out/T_out receive the new state, dt is updated.
double ref_solve_nr(int net, int eos_kind, double mu, const double* Y, double T, double* Y_out, double* T_out,
                    double rho, double drho_dt, double* dt)
{
    Net n;
    if (!getNet(net, n)) return -1;
    nnet::eos::IdealGasFunctor<double>  ideal(mu);
    nnet::eos::HelmholtzFunctor<double> helm(n.Z, n.dim);
    const nnet::EosFunctor<double>&     eos = eos_kind == 0 ? (const nnet::EosFunctor<double>&)ideal
                                                            : (const nnet::EosFunctor<double>&)helm;
    double Tn = T;
    double r = nnet::solveSystemNR(n.dim, *n.list, *n.rates, eos, Y, T, Y_out, Tn, rho, drho_dt, *dt);
    *T_out   = Tn;
    return r;
}
}
