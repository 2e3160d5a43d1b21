// Reduced-transcendental rate evaluation for the sparse and mixed-precision solver forms.
//
// Same physics as physics.cuh (net14.cpp:40-660, net86.cpp:41-686, net87.hpp:117-175) with
// two exact algebraic rewrites that cut the FP64 transcendental count of a net86 evaluation
// from about 680 to about 350 (GB300's FP64 pipe bounds these kernels):
//  * Coulomb plasma parameters: gamma_i = gam * Z_i^(5/3), so sqrt(gamma_i),
//    gamma_i^(1/4), gamma_i^1.9885 and log(gamma_i) are one per-particle value of gam
//    times (plus, for the log) a per-species constant computed once on the host;
//  * screening: eff * exp(dmu) = exp(f0 + coef + dmu), and
//    d/dT [eff exp(dmu)] as used by the reference = eff_s (dcoef - 2 dmu / T), so screened
//    fitted rates cost one exponential instead of two.
// The two computations of the ion-sphere radius (BE correction and screening) are the same
// quantity, evaluated once.  Results differ from the plain form at rounding level only.
#pragma once

#include "physics.cuh"

namespace nnet_gb300
{

struct CoulombFast
{
    double gam, gs, gq, gp, gl, nakbt, corr;
    CoulombFast() = default; // fields filled by the caller (values computed elsewhere)
    __device__ CoulombFast(double T, double rho)
    {
        const double kbt = NNET_KB * T;
        nakbt            = NNET_NA * kbt;
        corr             = -1.5 * nakbt;
        const double ne  = rho * NNET_NA / 2.;
        const double ae  = cbrt((3. / 4.) / (NNET_PI * ne));
        gam              = NNET_E2 / (kbt * ae);
        gs               = sqrt(gam);
        gq               = sqrt(gs);
        gp               = pow(gam, 1.9885);
        gl               = log(gam);
    }
    // corrected binding energy of species i (ggt1 / glt1, net14_tables.hpp:47-69)
    __device__ __forceinline__ double be(const NetView& nv, int i) const
    {
        const double z = __ldg(nv.z53 + i), g = gam * z;
        const double* f = nv.zFac + 4 * i;
        double        fn;
        if (g > 1)
        {
            const double s = gq * __ldg(f + 1);
            fn             = -.898004 * g + .96786 * s + .220703 / s + -.86097;
        }
        else
            fn = -.5 * 1.7320508075688772 * g * (gs * __ldg(f)) + .29561 * (gp * __ldg(f + 2));
        return __ldg(nv.BE + i) + corr - nakbt * fn;
    }
    // screening potential mu/kT of species i (net86.cpp:577-596)
    __device__ __forceinline__ double mu(const NetView& nv, int i) const
    {
        const double  g = gam * __ldg(nv.z53 + i);
        const double* f = nv.zFac + 4 * i;
        if (g <= 1) return -(1. / 1.7320508075688772) * g * (gs * __ldg(f)) + (gp * __ldg(f + 2)) * .29561 / 1.9885;
        const double s2 = gq * __ldg(f + 1);
        return -.898004 * g + 4. * (.96786 * s2 - .220703 / s2) + -.86097 * (gl + __ldg(f + 3)) - 2.520058332;
    }
    // be(nv, i) and mu(nv, i) together: the same values, with the shared loads and quotient once
    __device__ __forceinline__ void beMu(const NetView& nv, int i, double& beOut, double& muOut) const
    {
        const double  g = gam * __ldg(nv.z53 + i);
        const double* f = nv.zFac + 4 * i;
        double        fn;
        if (g > 1)
        {
            const double s = gq * __ldg(f + 1), q = .220703 / s;
            fn             = -.898004 * g + .96786 * s + q + -.86097;
            muOut          = -.898004 * g + 4. * (.96786 * s - q) + -.86097 * (gl + __ldg(f + 3)) - 2.520058332;
        }
        else
        {
            const double a = gs * __ldg(f), b = gp * __ldg(f + 2);
            fn             = -.5 * 1.7320508075688772 * g * a + .29561 * b;
            muOut          = -(1. / 1.7320508075688772) * g * a + b * .29561 / 1.9885;
        }
        beOut = __ldg(nv.BE + i) + corr - nakbt * fn;
    }
};

__device__ __forceinline__ void screenFast(double& e, double& de, double dmu, double T)
{
    const double EF = exp(dmu);
    e               = e * EF;
    de              = de * EF - 2. * e * dmu / T;
}

// net86 (and the net86 part of net87), slots as net86Rates in physics.cuh
static __device__ void net86RatesFast(const NetView& nv, double T, double rho, Strided<double> BE,
                                      Strided<double> rates, Strided<double> drates)
{
    const CoulombFast cf(T, rho);
    double            mukbt[86];
#pragma unroll 2
    for (int i = 0; i < 86; ++i)
    {
        BE[i]    = cf.be(nv, i);
        mukbt[i] = cf.mu(nv, i);
    }
    mukbt[1] = 0; // neutrons
    const FitT   v(T);
    const double t9 = T * 1e-09, t9i = 1. / t9;
    const double val1 = 11.6045 * t9i, val2 = 1.5 * log(t9), val3 = val1 * t9i * 1e-9, val4 = 1.5e-9 * t9i;
    const int    kb   = temperatureRange(T);
    const double twoT = 2. / T;
#pragma unroll 1
    for (int i = 7; i < 157; ++i)
    {
        const double* f  = nv.fit + (i - 7) * 8;
        const double  f0 = __ldg(f), f1 = __ldg(f + 1), f2 = __ldg(f + 2), f3 = __ldg(f + 3), f4 = __ldg(f + 4),
                     f5 = __ldg(f + 5), f6 = __ldg(f + 6), f7 = __ldg(f + 7);
        const double coef  = f1 * v.t9i + f2 * v.t9i13 + f3 * v.t913 + f4 * v.t9 + f5 * v.t953 + f6 * v.lt9;
        const double dcoef = (-f1 * v.t9i2 + (-f2 * v.t9i43 + f3 * v.t9i23 + 5 * f5 * v.t923) * (1. / 3.) + f4 +
                              f6 * v.t9i) *
                             1e-9;
        const int    mr = __ldg(nv.mainReactant + i), sr = __ldg(nv.secondaryReactant + i),
                  mp = __ldg(nv.mainProduct + i);
        const double part = __ldg(nv.choose + (mr - 5) * 24 + kb) / __ldg(nv.choose + (mp - 5) * 24 + kb);
        const double q    = __ldg(nv.q + i - 7);
        const double dmu  = mukbt[mr] + mukbt[sr] - mukbt[mp];
        const double sdmu = i >= 137 ? dmu : 0.;          // reverse slot screened only for i >= 137
        const double xr   = f7 + coef - val1 * q + (i < 137 ? val2 : 0.);
        const double dr   = dcoef + val3 * q + (i < 137 ? val4 : 0.);
        double       e, de, l, dl;
        if ((i >= 137 && i < 154) || i == 156)
        {
            // (a,p) / (a,n): the tabulated reverse is the network's forward (net86.cpp:561-567)
            e = part * exp(xr + dmu), de = e * (dr - dmu * twoT);
            l = exp(f0 + coef + sdmu), dl = l * (dcoef - sdmu * twoT);
        }
        else
        {
            e = exp(f0 + coef + dmu), de = e * (dcoef - dmu * twoT);
            l = part * exp(xr + sdmu), dl = l * (dr - sdmu * twoT);
        }
        rates[fwdSlot86(i)] = e, drates[fwdSlot86(i)] = de;
        rates[revSlot86(i)] = l, drates[revSlot86(i)] = dl;
    }
    Special s;
    specialRates(T, s);
    auto dmu = [&](int i) {
        return mukbt[__ldg(nv.mainReactant + i)] + mukbt[__ldg(nv.secondaryReactant + i)] -
               mukbt[__ldg(nv.mainProduct + i)];
    };
    screenFast(s.e2c, s.de2c, dmu(0), T);
    screenFast(s.eco, s.deco, dmu(1), T);
    screenFast(s.e2o, s.de2o, dmu(2), T);
    screenFast(s.e3a, s.de3a, dmu(4) + mukbt[__ldg(nv.mainReactant + 4)], T);
    screenFast(s.ecag, s.decag, dmu(5), T);
    screenFast(s.eoag, s.deoag, dmu(6), T);
    rates[0] = s.e2c, drates[0] = s.de2c, rates[1] = s.eco, drates[1] = s.deco;
    rates[2] = s.e2o, drates[2] = s.de2o, rates[3] = s.e3a, drates[3] = s.de3a;
    rates[4] = s.ecag, drates[4] = s.decag, rates[5] = s.eoag, drates[5] = s.deoag;
    rates[revSlot86(4)] = s.l3a, drates[revSlot86(4)] = s.dl3a;
    rates[revSlot86(5)] = s.lcag, drates[revSlot86(5)] = s.dlcag;
    rates[revSlot86(6)] = s.loag, drates[revSlot86(6)] = s.dloag;
}

// net14, slots as net14Rates in physics.cuh
static __device__ void net14RatesFast(const NetView& nv, double T, double rho, Strided<double> BE,
                                      Strided<double> rates, Strided<double> drates)
{
    const CoulombFast cf(T, rho);
    double            mukbt[14];
#pragma unroll
    for (int i = 0; i < 14; ++i)
    {
        BE[i]    = cf.be(nv, i);
        mukbt[i] = cf.mu(nv, i);
    }
    const FitT   v(T);
    const double t9 = T / 1.e9, t9i = 1.e0 / t9, lt9 = log(t9);
    const double val1 = 11.6045e0 * t9i, val2 = 1.5e0 * lt9, val3 = val1 * t9i * 1e-9, val4 = 1.5e-9 * t9i;
    const int    kb   = temperatureRange(T);
    const double twoT = 2. / T;
#pragma unroll 1
    for (int i = 4; i < 14; ++i)
    {
        const double* f = nv.fit + (i - 4) * 8;
        const double  f0 = __ldg(f), f1 = __ldg(f + 1), f2 = __ldg(f + 2), f3 = __ldg(f + 3), f4 = __ldg(f + 4),
                     f5 = __ldg(f + 5), f6 = __ldg(f + 6), f7 = __ldg(f + 7);
        const double coef  = f1 * v.t9i + f2 * v.t9i13 + f3 * v.t913 + f4 * v.t9 + f5 * v.t953 + f6 * v.lt9;
        const double dcoef = (-f1 * v.t9i2 + (-f2 * v.t9i43 + f3 * v.t9i23 + 5 * f5 * v.t923) * (1. / 3.) + f4 +
                              f6 * v.t9i) *
                             1e-9;
        const double q   = __ldg(nv.q + i - 4);
        const double dmu = mukbt[i - 1] + mukbt[0] - mukbt[i];
        const double e = exp(f0 + coef + dmu), de = e * (dcoef - dmu * twoT);
        const double l = __ldg(nv.choose + (i - 4) * 24 + kb) / __ldg(nv.choose + (i + 1 - 4) * 24 + kb) *
                         exp(coef + f7 - q * val1 + val2);
        rates[i - 1] = e, drates[i - 1] = de;
        rates[16 + i - 1] = l, drates[16 + i - 1] = l * (dcoef + q * val3 + val4);
    }
    Special s;
    specialRates(T, s);
    screenFast(s.e3a, s.de3a, mukbt[0] + mukbt[0] - mukbt[1] + mukbt[0], T);
    screenFast(s.ecag, s.decag, mukbt[1] + mukbt[0] - mukbt[2], T);
    screenFast(s.eoag, s.deoag, mukbt[2] + mukbt[0] - mukbt[3], T);
    screenFast(s.e2c, s.de2c, 2. * mukbt[1] - mukbt[3], T);
    screenFast(s.eco, s.deco, mukbt[1] + mukbt[2] - mukbt[4], T);
    screenFast(s.e2o, s.de2o, 2. * mukbt[2] - mukbt[5], T);
    rates[0] = s.e3a, drates[0] = s.de3a, rates[1] = s.ecag, drates[1] = s.decag;
    rates[2] = s.eoag, drates[2] = s.deoag, rates[13] = s.e2c, drates[13] = s.de2c;
    rates[14] = s.eco, drates[14] = s.deco, rates[15] = s.e2o, drates[15] = s.de2o;
    rates[16] = s.l3a, drates[16] = s.dl3a, rates[17] = s.lcag, drates[17] = s.dlcag;
    rates[18] = s.loag, drates[18] = s.dloag;
}

template<int NET>
__device__ __forceinline__ void networkRatesFast(const NetView& nv, Strided<double> Yg, double T, double rho,
                                                 Strided<double> BE, Strided<double> rates, Strided<double> drates)
{
    if constexpr (NET == 14)
        net14RatesFast(nv, T, rho, BE, rates, drates);
    else if constexpr (NET == 86)
        net86RatesFast(nv, T, rho, BE, rates, drates);
    else
    {
        // net87 = net86 + electron captures (net87.hpp:117-175)
        const double rhoElec = Yg[86] * rho;
        double       ev[12];
        electronRates(nv, T, rhoElec, ev);
        net86RatesFast(nv, T, rho, BE, rates, drates);
        const double kbt = NNET_KB * T, nakbt = NNET_NA * kbt;
        BE[86]     = __ldg(nv.BE + 86) + -1.5 * nakbt;
        BE[0]      = BE[0] + -ev[3];
        BE[1]      = BE[1] + -ev[9];
        rates[309] = rhoElec == 0 ? 0 : ev[0] / rhoElec, drates[309] = rhoElec == 0 ? 0 : ev[1] / rhoElec;
        rates[310] = rhoElec == 0 ? 0 : ev[6] / rhoElec, drates[310] = rhoElec == 0 ? 0 : ev[7] / rhoElec;
    }
}

} // namespace nnet_gb300
