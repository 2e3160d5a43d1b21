// Device physics of the burn path: ideal-gas and Helmholtz EOS, net14 / net86 / net87
// reaction rates with temperature derivatives and Coulomb-corrected binding energies.
//
// Each value is evaluated with the same formula and floating-point association as the
// reference (citations below), so results track the reference's FP64 CPU path to
// rounding level.  The structure is GPU-first: one thread evaluates one particle, the
// network tables are read with warp-uniform addresses (L1 broadcast), and rates are
// streamed straight into the caller's strided scratch instead of per-thread arrays.
#pragma once

#include "common.cuh"

namespace nnet_gb300
{

struct EosResult
{
    double cv, dpdT, p, u, c;
};

// ------------------------------------------------------------------ ideal gas
// include/nnet/parameterization/eos/ideal_gas.hpp:69-82
__device__ __forceinline__ EosResult idealGasEos(double mu, double T, double rho)
{
    EosResult    r;
    const double dmy = 8.317e7 / mu;
    r.cv             = 1.5 * dmy;
    r.u              = T * r.cv;
    r.p              = rho * T * dmy;
    r.c              = sqrt(r.p / rho);
    r.dpdT           = rho * dmy;
    return r;
}

// ------------------------------------------------------------------ Helmholtz EOS
namespace helm
{
constexpr double tlo = 3., thi = 13., dlo = -12., dhi = 15.;
constexpr double tstpi = 1. / ((thi - tlo) / (double)(HELM_JMAX - 1));
constexpr double dstpi = 1. / ((dhi - dlo) / (double)(HELM_IMAX - 1));
constexpr double pi      = 3.14159265358979323846264338327950288;
constexpr double h       = 6.6260689633e-27;
constexpr double qe      = 4.8032042712e-10;
constexpr double avo     = 6.0221417930e23;
constexpr double clight  = 2.99792458e10;
constexpr double kerg    = 1.380650424e-16;
constexpr double amu     = 1.66053878283e-24;
constexpr double ssol    = 5.6704e-5;
constexpr double a1 = -0.898004, b1 = 0.96786, c1 = 0.220703, d1 = -0.86097, e1 = 2.5269;
constexpr double a2 = 0.29561, b2 = 1.9885, c2 = 0.288675;

// Quintic / cubic Hermite basis functions (helmholtz.cpp:222-311)
__device__ __forceinline__ double psi0(double z) { return z * z * z * (z * (-6. * z + 15.) - 10.) + 1.; }
__device__ __forceinline__ double dpsi0(double z) { return z * z * (z * (-30. * z + 60.) - 30.); }
__device__ __forceinline__ double ddpsi0(double z) { return z * (z * (-120. * z + 180.) - 60.); }
__device__ __forceinline__ double psi1(double z) { return z * (z * z * (z * (-3. * z + 8.) - 6.) + 1.); }
__device__ __forceinline__ double dpsi1(double z) { return z * z * (z * (-15. * z + 32.) - 18.) + 1.; }
__device__ __forceinline__ double ddpsi1(double z) { return z * (z * (-60. * z + 96.) - 36.); }
__device__ __forceinline__ double psi2(double z) { return 0.5 * z * z * (z * (z * (-z + 3.) - 3.) + 1.); }
__device__ __forceinline__ double dpsi2(double z) { return 0.5 * z * (z * (z * (-5. * z + 12.) - 9.) + 2.); }
__device__ __forceinline__ double ddpsi2(double z) { return 0.5 * (z * (z * (-20. * z + 36.) - 18.) + 2.); }
__device__ __forceinline__ double xpsi0(double z) { return z * z * (2. * z - 3.) + 1.; }
__device__ __forceinline__ double xdpsi0(double z) { return z * (6. * z - 6.); }
__device__ __forceinline__ double xpsi1(double z) { return z * (z * (z - 2.) + 1.); }
__device__ __forceinline__ double xdpsi1(double z) { return z * (3. * z - 4.) + 1.; }

// Biquintic interpolant over the 36 stencil coefficients, terms summed in the order of
// helmholtz.cpp:273-286.  fi layout: [q][corner] with q = f ft ftt fd fdd fdt fddt fdtt
// fddtt and corner = (i,j) (i+1,j) (i,j+1) (i+1,j+1).
struct W6
{
    double t0, t1, t2, mt0, mt1, mt2, d0, d1, d2, md0, md1, md2;
};
__device__ __forceinline__ double h5(const double* fi, const W6& w)
{
    return fi[0] * w.d0 * w.t0 + fi[1] * w.md0 * w.t0 + fi[2] * w.d0 * w.mt0 + fi[3] * w.md0 * w.mt0 +
           fi[4] * w.d0 * w.t1 + fi[5] * w.md0 * w.t1 + fi[6] * w.d0 * w.mt1 + fi[7] * w.md0 * w.mt1 +
           fi[8] * w.d0 * w.t2 + fi[9] * w.md0 * w.t2 + fi[10] * w.d0 * w.mt2 + fi[11] * w.md0 * w.mt2 +
           fi[12] * w.d1 * w.t0 + fi[13] * w.md1 * w.t0 + fi[14] * w.d1 * w.mt0 + fi[15] * w.md1 * w.mt0 +
           fi[16] * w.d2 * w.t0 + fi[17] * w.md2 * w.t0 + fi[18] * w.d2 * w.mt0 + fi[19] * w.md2 * w.mt0 +
           fi[20] * w.d1 * w.t1 + fi[21] * w.md1 * w.t1 + fi[22] * w.d1 * w.mt1 + fi[23] * w.md1 * w.mt1 +
           fi[24] * w.d2 * w.t1 + fi[25] * w.md2 * w.t1 + fi[26] * w.d2 * w.mt1 + fi[27] * w.md2 * w.mt1 +
           fi[28] * w.d1 * w.t2 + fi[29] * w.md1 * w.t2 + fi[30] * w.d1 * w.mt2 + fi[31] * w.md1 * w.mt2 +
           fi[32] * w.d2 * w.t2 + fi[33] * w.md2 * w.t2 + fi[34] * w.d2 * w.mt2 + fi[35] * w.md2 * w.mt2;
}
// bicubic interpolant (helmholtz.cpp:315-322)
__device__ __forceinline__ double h3(const double* fi, double w0t, double w1t, double w0mt, double w1mt, double w0d,
                                     double w1d, double w0md, double w1md)
{
    return fi[0] * w0d * w0t + fi[1] * w0md * w0t + fi[2] * w0d * w0mt + fi[3] * w0md * w0mt + fi[4] * w0d * w1t +
           fi[5] * w0md * w1t + fi[6] * w0d * w1mt + fi[7] * w0md * w1mt + fi[8] * w1d * w0t + fi[9] * w1md * w0t +
           fi[10] * w1d * w0mt + fi[11] * w1md * w0mt + fi[12] * w1d * w1t + fi[13] * w1md * w1t +
           fi[14] * w1d * w1mt + fi[15] * w1md * w1mt;
}
} // namespace helm

// Helmholtz EOS for abar_ = sum Y, zbar_ = sum Y Z (helmholtz.cpp:341-965).  Computes the
// outputs the burn and the post-burn EOS consume (cv, dpdT, p, u, c) with the reference's
// expressions; the chemical-potential and number-density interpolations, which feed no
// output, are not evaluated.
static __device__ EosResult helmholtzEos(const HelmView& hv, double abar_, double zbar_, double temp, double rho)
{
    using namespace helm;
    const double abar = 1 / abar_;
    const double zbar = zbar_ / abar_;
    const double ye   = fmax((double)1e-16, zbar / abar);
    const double din  = ye * rho;

    int jat = int((log10(temp) - tlo) * tstpi);
    jat     = max(1, min(jat, HELM_JMAX - 2));
    int iat = int((log10(din) - dlo) * dstpi);
    iat     = max(1, min(iat, HELM_IMAX - 2));

    // gather the 2x2 stencil: 4 cache lines of the cell-interleaved table
    double fi[52];
    {
        const double2* c00 = reinterpret_cast<const double2*>(hv.cell + ((size_t)iat * HELM_JMAX + jat) * HELM_CELL);
        const double2* c01 = c00 + HELM_CELL / 2;                          // (i, j+1)
        const double2* c10 = c00 + (size_t)HELM_JMAX * HELM_CELL / 2;      // (i+1, j)
        const double2* c11 = c10 + HELM_CELL / 2;                          // (i+1, j+1)
        double         v00[14], v10[14], v01[14], v11[14];
#pragma unroll
        for (int q = 0; q < 7; ++q)
        {
            double2 a = __ldg(c00 + q), b = __ldg(c10 + q), c = __ldg(c01 + q), d = __ldg(c11 + q);
            v00[2 * q] = a.x, v00[2 * q + 1] = a.y, v10[2 * q] = b.x, v10[2 * q + 1] = b.y;
            v01[2 * q] = c.x, v01[2 * q + 1] = c.y, v11[2 * q] = d.x, v11[2 * q + 1] = d.y;
        }
#pragma unroll
        for (int q = 0; q < 13; ++q)
            fi[4 * q] = v00[q], fi[4 * q + 1] = v10[q], fi[4 * q + 2] = v01[q], fi[4 * q + 3] = v11[q];
    }

    const double ytot1 = 1 / abar;
    const double rhoi = 1. / rho, tempi = 1. / temp, kt = kerg * temp, ktinv = 1. / kt;
    const double asol = 4.0 * ssol / clight, kergavo = kerg * avo, esqu = qe * qe;

    const double prad    = asol * temp * temp * temp * temp / 3;
    const double dpraddt = 4. * prad * tempi;
    const double erad = 3. * prad * rhoi, deraddt = 3. * dpraddt * rhoi;
    (void)kergavo;

    const double xni = avo * ytot1 * rho, dxnidd = avo * ytot1, dxnida = -xni * ytot1;
    const double pion = xni * kt, dpiondd = dxnidd * kt, dpiondt = xni * kerg;
    const double eion = 1.5 * pion * rhoi, deiondt = 1.5 * dpiondt * rhoi;
    (void)dxnida;

    // electron-positron: biquintic of the free energy (helmholtz.cpp:468-557)
    const double dti = hv.dtiSav[jat], dts = hv.dtSav[jat], dt2s = hv.dt2Sav[jat], dt2i = hv.dt2iSav[jat];
    const double ddi = hv.ddiSav[iat], dds = hv.ddSav[iat], dd2s = hv.dd2Sav[iat];
    const double xt = fmax((temp - hv.t[jat]) * dti, 0.), xd = fmax((din - hv.d[iat]) * ddi, 0.);
    const double mxt = 1. - xt, mxd = 1. - xd;

    W6 w;
    w.t0 = psi0(xt), w.t1 = psi1(xt) * dts, w.t2 = psi2(xt) * dt2s;
    w.mt0 = psi0(mxt), w.mt1 = -psi1(mxt) * dts, w.mt2 = psi2(mxt) * dt2s;
    w.d0 = psi0(xd), w.d1 = psi1(xd) * dds, w.d2 = psi2(xd) * dd2s;
    w.md0 = psi0(mxd), w.md1 = -psi1(mxd) * dds, w.md2 = psi2(mxd) * dd2s;
    const double free = h5(fi, w);

    W6 wd = w; // density derivative weights
    wd.d0 = dpsi0(xd) * ddi, wd.d1 = dpsi1(xd), wd.d2 = dpsi2(xd) * dds;
    wd.md0 = -dpsi0(mxd) * ddi, wd.md1 = dpsi1(mxd), wd.md2 = -dpsi2(mxd) * dds;
    const double df_d = h5(fi, wd);

    W6 wt = w; // temperature derivative weights
    wt.t0 = dpsi0(xt) * dti, wt.t1 = dpsi1(xt), wt.t2 = dpsi2(xt) * dts;
    wt.mt0 = -dpsi0(mxt) * dti, wt.mt1 = dpsi1(mxt), wt.mt2 = -dpsi2(mxt) * dts;
    const double df_t = h5(fi, wt);

    W6 wtt = w;
    wtt.t0 = ddpsi0(xt) * dt2i, wtt.t1 = ddpsi1(xt) * dti, wtt.t2 = ddpsi2(xt);
    wtt.mt0 = ddpsi0(mxt) * dt2i, wtt.mt1 = -ddpsi1(mxt) * dti, wtt.mt2 = ddpsi2(mxt);
    const double df_tt = h5(fi, wtt);

    W6 wdt = wt;
    wdt.d0 = wd.d0, wdt.d1 = wd.d1, wdt.d2 = wd.d2, wdt.md0 = wd.md0, wdt.md1 = wd.md1, wdt.md2 = wd.md2;
    const double df_dt = h5(fi, wdt);

    // bicubic of dP/dden (helmholtz.cpp:562-606)
    const double s0t = xpsi0(xt), s1t = xpsi1(xt) * dts, s0mt = xpsi0(mxt), s1mt = -xpsi1(mxt) * dts;
    const double s0d = xpsi0(xd), s1d = xpsi1(xd) * dds, s0md = xpsi0(mxd), s1md = -xpsi1(mxd) * dds;
    double       dpepdd = h3(fi + 36, s0t, s1t, s0mt, s1mt, s0d, s1d, s0md, s1md);
    dpepdd              = fmax(ye * dpepdd, (double)1.e-30);

    // electron-positron thermodynamics (helmholtz.cpp:679-703)
    double       x      = din * din;
    const double pele   = x * df_d;
    const double dpepdt = x * df_dt;
    x                   = ye * ye;
    const double sele   = -df_t * ye;
    const double dsepdt = -df_tt * ye;
    const double eele   = ye * free + temp * sele;
    const double deepdt = temp * dsepdt;
    const double deepdd = x * df_d + temp * (-df_dt * x);

    // Coulomb (helmholtz.cpp:719-824)
    double       z      = pi * 4. / 3.;
    double       s      = z * xni;
    const double dsdd   = z * dxnidd;
    const double lami   = pow((double)1. / s, (double)1. / 3.), inv_lami = 1. / lami;
    z                   = -lami / 3;
    const double lamidd = z * dsdd / s;
    const double plasg  = zbar * zbar * esqu * ktinv * inv_lami;
    z                   = -plasg * inv_lami;
    const double plasgdd = z * lamidd;
    const double plasgdt = -plasg * ktinv * kerg;

    double ecoul = 0, pcoul = 0, decouldd = 0, decouldt = 0, dpcouldd = 0, dpcouldt = 0;
    if (plasg >= 1.)
    {
        x           = pow(plasg, (double)0.25);
        double y    = avo * ytot1 * kerg;
        ecoul       = y * temp * (a1 * plasg + b1 * x + c1 / x + d1);
        pcoul       = rho * ecoul / 3.;
        y           = avo * ytot1 * kt * (a1 + 0.25 / plasg * (b1 * x - c1 / x));
        decouldd    = y * plasgdd;
        decouldt    = y * plasgdt + ecoul / temp;
        y           = rho / 3.;
        dpcouldd    = ecoul + y * decouldd / 3.;
        dpcouldt    = y * decouldt;
    }
    else if (plasg < 1.)
    {
        x        = plasg * sqrt(plasg);
        double y = pow(plasg, (double)b2);
        z        = c2 * x - a2 * y / 3.;
        pcoul    = -pion * z;
        ecoul    = 3.0 * pcoul / rho;
        s        = 1.5 * c2 * x / plasg - a2 * b2 * y / plasg / 3.;
        dpcouldd = -dpiondd * z - pion * s * plasgdd;
        dpcouldt = -dpiondt * z - pion * s * plasgdt;
        s        = 3.0 / rho;
        decouldd = s * dpcouldd - ecoul / rho;
        decouldt = s * dpcouldt;
    }

    x = prad + pion + pele + pcoul;
    double y = erad + eion + eele + ecoul;
    if (x <= 0. || y <= 0.)
    {
        pcoul = dpcouldd = dpcouldt = 0.;
        ecoul = decouldd = decouldt = 0.;
    }

    const double dpiondd_ = dpiondd;
    const double pgas = pion + pele + pcoul, egas = eion + eele + ecoul;
    const double dpgasdd = dpiondd_ + dpepdd + dpcouldd, dpgasdt = dpiondt + dpepdt + dpcouldt;
    const double degasdt = deiondt + deepdt + decouldt;
    (void)deepdd, (void)decouldd;

    EosResult r;
    const double pres = prad + pgas, ener = erad + egas;
    const double dpresdd = 0. + dpgasdd, dpresdt = dpraddt + dpgasdt;
    r.cv              = deraddt + degasdt;
    const double zz   = pres * rhoi, zzi = rho / pres;
    const double chit = temp / pres * dpresdt, chid = dpresdd * zzi;
    x                 = zz * chit / (temp * r.cv);
    const double gam1 = chit * x + chid;
    z                 = 1. + (ener + clight * clight) * zzi;
    r.c               = clight * sqrt(gam1 / z);
    r.dpdT            = dpresdt;
    r.p               = pres;
    r.u               = ener;
    return r;
}

// ------------------------------------------------------------------ rate helpers
// temperature bin of the partition-function tables (net14_tables.hpp:71-101)
__device__ __forceinline__ int temperatureRange(double T)
{
    if (T < 1.5e8) return 0;
    if (T < 1e9) return T < 2e8 ? 1 : T < 3e8 ? 2 : T < 4e8 ? 3 : T < 5e8 ? 4 : T < 6e8 ? 5 : T < 7e8 ? 6 : T < 8e8 ? 7 : T < 9e8 ? 8 : 9;
    if (T < 5e9) return T < 1.5e9 ? 10 : T < 2e9 ? 11 : T < 2.5e9 ? 12 : T < 3e9 ? 13 : T < 3.5e9 ? 14 : T < 4e9 ? 15 : T < 4.5e9 ? 16 : 17;
    return T < 6e9 ? 18 : T < 7e9 ? 19 : T < 8e9 ? 20 : T < 9e9 ? 21 : T < 1e10 ? 22 : 23;
}

// Coulomb correction functions (net14_tables.hpp:47-69)
__device__ __forceinline__ double ggt1(double x)
{
    const double s = sqrt(sqrt(x));
    return -.898004 * x + .96786 * s + .220703 / s + -.86097;
}
__device__ __forceinline__ double glt1(double x)
{
    const double a1 = -.5 * 1.7320508075688772; // -.5 * sqrt(3.)
    return a1 * x * sqrt(x) + .29561 * pow(x, 1.9885);
}

// binding energies with ideal-gas and Coulomb corrections (net14.cpp:46-75, net86.cpp:47-74)
template<int N>
__device__ __forceinline__ void correctedBE(const NetView& nv, double T, double rho, Strided<double> out)
{
    const double kbt = NNET_KB * T, nakbt = NNET_NA * kbt, corr = -1.5 * nakbt;
    const double ne  = rho * NNET_NA / 2.;
    const double ae  = pow((3. / 4.) / (NNET_PI * ne), 1. / 3.);
    const double gam = NNET_E2 / (kbt * ae);
    for (int i = 0; i < N; ++i)
    {
        double       v     = __ldg(nv.BE + i) + corr;
        const double gamma = gam * __ldg(nv.z53 + i);
        v -= nakbt * (gamma > 1 ? ggt1(gamma) : glt1(gamma));
        out[i] = v;
    }
}

// screening potential mu/kT of species i (net14.cpp:597-616, net86.cpp:577-596)
__device__ __forceinline__ double screeningMu(double gam, double z53)
{
    const double gamp = gam * z53, sg = sqrt(gamp), s2 = sqrt(sg);
    if (gamp <= 1) return -(1. / 1.7320508075688772) * gamp * sg + pow(gamp, 1.9885) * .29561 / 1.9885;
    return -.898004 * gamp + 4. * (.96786 * s2 - .220703 / s2) + -.86097 * log(gamp) - 2.520058332;
}
__device__ __forceinline__ double screeningGamma(double T, double rho)
{
    const double ne  = rho * NNET_NA / 2.;
    const double kbt = T * NNET_KB;
    const double ae  = pow(3. / (4. * NNET_PI * ne), 1. / 3.);
    return NNET_E2 / (kbt * ae);
}

// REACLIB-style fitted rate (net14.cpp:104-131)
struct FitT
{
    double t9, t913, t923, t953, t9i, t9i2, t9i13, t9i23, t9i43, lt9;
    FitT() = default; // fields filled by the caller (values computed elsewhere)
    __device__ explicit FitT(double T)
    {
        t9 = T / 1.e9, t913 = pow(t9, 1. / 3.), t923 = t913 * t913, t953 = pow(t9, 5. / 3.);
        t9i = 1.e0 / t9, t9i2 = t9i * t9i, t9i13 = 1.e0 / t913, t9i23 = t9i13 * t9i13, t9i43 = t9i23 * t9i23;
        lt9 = log(t9);
    }
};
__device__ __forceinline__ void fitRate(const double* f, const FitT& v, double& coef, double& dcoef, double& eff,
                                        double& deff)
{
    const double f0 = __ldg(f), f1 = __ldg(f + 1), f2 = __ldg(f + 2), f3 = __ldg(f + 3), f4 = __ldg(f + 4),
                 f5 = __ldg(f + 5), f6 = __ldg(f + 6);
    coef  = f1 * v.t9i + f2 * v.t9i13 + f3 * v.t913 + f4 * v.t9 + f5 * v.t953 + f6 * v.lt9;
    dcoef = (-f1 * v.t9i2 + (-f2 * v.t9i43 + f3 * v.t9i23 + 5 * f5 * v.t923) * (1. / 3.) + f4 + f6 * v.t9i) * 1e-9;
    eff   = exp(f0 + coef);
    deff  = eff * dcoef;
}

// The seven CF88-type special rates shared by net14 and net86 (net14.cpp:153-561,
// net86.cpp:135-505): triple-alpha (+ reverse), 12C+12C, 12C+16O, 16O+16O,
// 12C(a,g) (+ reverse), 16O(a,g) (+ reverse).
struct Special
{
    double e3a, de3a, l3a, dl3a, e2c, de2c, eco, deco, e2o, de2o, ecag, decag, lcag, dlcag, eoag, deoag, loag, dloag;
};
static __device__ __noinline__ void specialRates(double T, Special& s)
{
    {
        const double t9r = T * 1.0e-09, t9 = fmin((double)10., t9r);
        const double t92 = t9 * t9, t93 = t92 * t9, t95 = t92 * t93, t912 = sqrt(t9);
        const double t913 = pow(t9, 1. / 3.), t923 = t913 * t913, t932 = t9 * t912, t943 = t9 * t913,
                     t953 = t9 * t923;
        const double t9i = 1. / t9, t9i13 = 1. / t913, t9i23 = 1. / t923, t9i32 = 1. / t932, t9rm1 = 1. / t9r,
                     t9r32 = t9 * sqrt(t9r);
        const double r2abe = (7.40e+05 * t9i32) * exp(-1.0663 * t9i) +
                             4.164e+09 * t9i23 * exp(-13.49 * t9i13 - t92 / 0.009604) *
                                 (1. + 0.031 * t913 + 8.009 * t923 + 1.732 * t9 + 49.883 * t943 + 27.426 * t953);
        const double rbeac = (130. * t9i32) * exp(-3.3364 * t9i) +
                             2.510e+07 * t9i23 * exp(-23.57 * t9i13 - t92 / 0.055225) *
                                 (1. + 0.018 * t913 + 5.249 * t923 + 0.650 * t9 + 19.176 * t943 + 6.034 * t953);
        if (T > 8e7)
            s.e3a = 2.90e-16 * (r2abe * rbeac) + 0.1 * 1.35e-07 * t9i32 * exp(-24.811 * t9i);
        else
            s.e3a = 2.90e-16 * (r2abe * rbeac) *
                        (0.01 + 0.2 * (1. + 4. * exp(-pow(0.025 * t9i, 3.263))) / (1. + 4. * exp(-pow(t9 / 0.025, 9.227)))) +
                    0.1 * 1.35e-07 * t9i32 * exp(-24.811 * t9i);
        s.l3a = s.e3a * (2.e20 * exp(-84.419412e0 * t9i)) * t93;

        {
            const double t9a = t9 / (1. + 0.0396 * t9), t9a13 = pow(t9a, 1. / 3.), t9a56 = pow(t9a, 5. / 6.);
            s.e2c = 4.27e+26 * t9a56 * t9i32 * exp(-84.165 / t9a13 - 2.12e-03 * t93);
        }
        s.eco = 0;
        if (T >= 5e8)
        {
            const double t9ap = t9 / (1. + 0.055 * t9), t9a2p = t9ap * t9ap, t9a13p = pow(t9ap, 1. / 3.),
                         t9a23p = t9a13p * t9a13p, t9a56ap = pow(t9ap, 5. / 6.);
            s.eco = 1.72e+31 * t9a56ap * t9i32 * exp(-106.594 / t9a13p) /
                    (exp(-0.18 * t9a2p) + 1.06e-03 * exp(2.562 * t9a23p));
        }
        s.e2o  = 7.10e+36 * t9i23 * exp(-135.93 * t9i13 - 0.629 * t923 - 0.445 * t943 + 0.0103 * t92);
        s.ecag = 1.04e+08 / (t92 * pow(1. + 0.0489 * t9i23, 2.)) * exp(-32.120 * t9i13 - t92 / 12.222016) +
                 1.76e+08 / (t92 * pow(1. + 0.2654 * t9i23, 2.)) * exp(-32.120 * t9i13) +
                 1.25e+03 * t9i32 * exp(-27.499 * t9i) + 1.43e-02 * t95 * exp(-15.541 * t9i);
        s.lcag = s.ecag * 5.13e+10 * t9r32 * exp(-83.108047 * t9rm1);
        s.eoag = (9.37e+09 * t9i23 * exp(-39.757 * t9i13 - t92 / 2.515396) + 62.1 * t9i32 * exp(-10.297 * t9i) +
                  538. * t9i32 * exp(-12.226 * t9i) + 13. * t92 * exp(-20.093 * t9i));
        s.loag = s.eoag * 5.65e+10 * t9r32 * exp(-54.93807 * t9rm1);
    }
    {
        // temperature derivatives, unclamped t9 (net14.cpp:357-561)
        const double t9 = T * 1.0e-09, t92 = t9 * t9, t93 = t92 * t9, t94 = t93 * t9, t95 = t94 * t9;
        const double t912 = sqrt(t9), t913 = pow(t9, 1. / 3.), t923 = t913 * t913, t932 = t9 * t912,
                     t943 = t9 * t913, t952 = t9 * t932, t953 = t9 * t923;
        const double t9i = 1. / t9, t9i2 = t9i * t9i, t9i13 = 1. / t913, t9i23 = 1. / t923, t9i32 = 1. / t932,
                     t9i43 = 1. / t943, t9i52 = 1. / t952, t9i53 = 1. / t953;
        {
            const double vA  = -24.811 * t9i;
            const double vB  = -1.0663 * t9i;
            const double vC  = -13.49 * t9i13 - t92 * 104.123282;
            const double vD  = 1. + .031 * t913 + 8.009 * t923 + 1.732 * t9 + 49.883 * t943 + 27.426 * t953;
            const double vE  = -3.3364 * t9i;
            const double vF  = -23.57 * t9i13 - 18.10774106 * t92;
            const double vG  = 1. + .018 * t913 + 5.249 * t923 + .650 * t9 + 19.176 * t943 + 6.034 * t953;
            const double dvA = 24.811 * t9i2, dvB = 1.0663 * t9i2;
            const double dvC = t9i43 * 13.49 / 3. - 208.246564 * t9;
            const double dvD = (t9i23 * .031 + t9i13 * 16.018 + 5.196 + t913 * 199.532 + t923 * 137.13) / 3.;
            const double dvE = 3.3364 * t9i2;
            const double dvF = t9i43 * 23.57 / 3. - 36.21548212 * t9;
            const double dvG = (t9i23 * .018 + t9i13 * 10.498 + 1.950 + t913 * 76.704 + t923 * 30.17) / 3.;
            const double eB = exp(vB), eC = exp(vC), eE = exp(vE), eF = exp(vF);
            const double r2abe  = 7.4e5 * t9i32 * eB + 4.164e9 * t9i23 * vD * eC;
            const double rbeac  = 130. * t9i32 * eE + 2.510e7 * t9i23 * vG * eF;
            const double dr2abe = eB * (-1.11e6 * t9i52 + 7.4e5 * t9i32 * dvB) +
                                  4.164e9 * eC * (-t9i53 * vD * 2. / 3. + t9i23 * dvC * vD + t9i23 * dvD);
            const double drbeac = eE * (-195. * t9i52 + 130. * t9i32 * dvE) +
                                  2.510e7 * eF * (-2. * t9i53 * vG / 3. + t9i23 * dvF * vG + t9i23 * dvG);
            s.de3a = (2.90e-16 * (dr2abe * rbeac + r2abe * drbeac) + 1.35e-8 * exp(vA) * (-1.5 * t9i52 + t9i32 * dvA)) *
                     1.e-9;
        }
        {
            const double vA = -84.419412 * t9i, dvA = 84.419412 * t9i2;
            s.dl3a          = 2.00e20 * exp(vA) * t93 * (dvA * s.e3a + 3. * t9i * s.e3a + s.de3a) * 1.e-9;
        }
        {
            const double vA = t9 / (1. + .0396 * t9), vA56 = pow(vA, 5. / 6.);
            const double vB = -84.165 * pow(vA, -1. / 3.) - 2.12e-3 * t93;
            const double dvA = vA * vA * t9i2, dvB = 28.055 * dvA * pow(vA, -4. / 3.) - 6.36e-3 * t92;
            s.de2c = 4.27e26 * t9i32 * exp(vB) * (pow(vA, -1. / 6.) * dvA * 5. / 6. - 1.5 * vA56 * t9i + vA56 * dvB) *
                     1.e-9;
        }
        s.deco = 0;
        if (t9 > .5)
        {
            const double vA = t9 / (1. + .055 * t9), vA56 = pow(vA, 5. / 6.);
            const double vB = -106.594 * pow(vA, -1. / 3.), vC = -.18 * vA * vA, vD = 2.562 * pow(vA, 2. / 3.);
            const double val = exp(vC) + 1.06e-3 * exp(vD);
            const double dvA = vA * vA * t9i2, dvB = 106.594 * pow(vA, -4. / 3.) * dvA / 3.;
            const double dvC = -.36 * vA * dvA, dvD = 1.708 * dvA * pow(vA, -1. / 3.);
            const double dval = dvC * exp(vC) + 1.06e-3 * dvD * exp(vD);
            s.deco = 1.72e31 * t9i32 * (pow(vA, -1. / 6.) * dvA * 5. / 6. - 1.5 * vA56 * t9i + vA56 * (dvB - dval / val)) *
                     exp(vB) / val * 1.e-9;
        }
        {
            const double vA  = -135.93e0 * t9i13 - .629 * t923 - .445 * t943 + .0103 * t92;
            const double dvA = 45.31 * t9i43 - .629 * t9i13 * 2. / 3. - .445 * t913 * 4. / 3. + .0206 * t9;
            s.de2o           = 7.10e36 * exp(vA) * t9i23 * (-t9i * 2. / 3. + dvA) * 1.e-9;
        }
        {
            const double vB = pow(1. + .0489 * t9i23, 2), vC = -32.120 * t9i13 - pow(t9 / 3.496, 2.);
            const double vD = pow(1. + .2654 * t9i23, 2), vE = -32.120 * t9i13, vF = -27.499 * t9i, vG = -15.541 * t9i;
            const double dvB = -(2. + .0978 * t9i23) * (.0326 * t9i53);
            const double dvC = 32.120 * t9i43 / 3. - 2. * t9 / pow(3.496, 2.);
            const double dvD = -(2. + .5308 * t9i23) * (.5308 * t9i53 / 3.);
            const double dvE = 32.120 * t9i43 / 3., dvF = 27.499 * t9i2, dvG = 15.541 * t9i2;
            s.decag = (1.04e8 * exp(vC) * t9i2 * (-2. * t9i + dvC - dvB / vB) / vB +
                       1.76e8 * exp(vE) * t9i2 * (-2. * t9i + dvE - dvD / vD) / vD +
                       1.25e3 * exp(vF) * (-1.5 * t9i52 + dvF * t9i32) + 1.43e-2 * exp(vG) * (5. * t94 + dvG * t95)) *
                      1.e-9;
        }
        {
            const double vA = -83.108047 * t9i, vB = -39.757 * t9i13 - pow(t9 / 1.586, 2.);
            const double vC = -10.297 * t9i, vD = -12.226 * t9i, vE = -20.093 * t9i;
            const double dvA = 83.108047 * t9i2, dvB = 39.757 * t9i43 / 3. - 2. * t9 / pow(1.586, 2.);
            const double dvC = 10.297 * t9i2, dvD = 12.226 * t9i2, dvE = 20.093 * t9i2;
            s.dlcag = 5.13e10 * exp(vA) * (s.decag * t932 + s.ecag * 1.5 * t912 + s.ecag * t932 * dvA) * 1.e-9;
            s.deoag = (9.37e9 * exp(vB) * (-t9i53 * 2. / 3. + t9i23 * dvB) + 62.1 * exp(vC) * (-1.5 * t9i52 + t9i32 * dvC) +
                       538. * exp(vD) * (-1.5 * t9i52 + t9i32 * dvD) + 13. * exp(vE) * (2. * t9 + t92 * dvE)) *
                      1.e-9;
        }
        {
            const double vA = -54.903255 * t9i, dvA = 54.903255 * t9i2;
            s.dloag         = 5.65e10 * exp(vA) * (s.deoag * t932 + 1.5 * s.eoag * t912 + s.eoag * t932 * dvA) * 1.e-9;
        }
    }
}

// apply a screening factor exp(dmu) to a forward rate (net86.cpp:645-652)
__device__ __forceinline__ void screen(double& e, double& de, double dmu, double T)
{
    const double EF = exp(dmu);
    e               = e * EF;
    de              = de * EF - 2. * e * dmu / T;
}

// ------------------------------------------------------------------ net14
// include/nnet/parameterization/net14/net14.cpp:40-660; rate slots: forward e -> e
// (0..15), reverse l -> 16 + l (0..12).
static __device__ void net14Rates(const NetView& nv, double T, double rho, Strided<double> BE, Strided<double> rates,
                           Strided<double> drates)
{
    correctedBE<14>(nv, T, rho, BE);
    double mukbt[14];
    {
        const double gam = screeningGamma(T, rho);
#pragma unroll
        for (int i = 0; i < 14; ++i)
            mukbt[i] = screeningMu(gam, __ldg(nv.z53 + i));
    }
    {
        const FitT   v(T);
        const double t9 = T / 1.e9, t9i = 1.e0 / t9, lt9 = log(t9);
        const double val1 = 11.6045e0 * t9i, val2 = 1.5e0 * lt9, val3 = val1 * t9i * 1e-9, val4 = 1.5e-9 * t9i;
        const int    kb   = temperatureRange(T);
#pragma unroll 1
        for (int i = 4; i < 14; ++i)
        {
            const double* f = nv.fit + (i - 4) * 8;
            double        coef, dcoef, e, de;
            fitRate(f, v, coef, dcoef, e, de);
            const double q = __ldg(nv.q + i - 4);
            const double l = __ldg(nv.choose + (i - 4) * 24 + kb) / __ldg(nv.choose + (i + 1 - 4) * 24 + kb) *
                             exp(coef + __ldg(f + 7) - q * val1 + val2);
            const double dl = l * (dcoef + q * val3 + val4);
            // screening of forward slot e = i-1: mu_{i-1} + mu_0 - mu_i
            screen(e, de, mukbt[i - 1] + mukbt[0] - mukbt[i], T);
            rates[i - 1] = e, drates[i - 1] = de;
            rates[16 + i - 1] = l, drates[16 + i - 1] = dl;
        }
    }
    Special s;
    specialRates(T, s);
    screen(s.e3a, s.de3a, mukbt[0] + mukbt[0] - mukbt[1] + mukbt[0], T);
    screen(s.ecag, s.decag, mukbt[1] + mukbt[0] - mukbt[2], T);
    screen(s.eoag, s.deoag, mukbt[2] + mukbt[0] - mukbt[3], T);
    screen(s.e2c, s.de2c, 2. * mukbt[1] - mukbt[3], T);
    screen(s.eco, s.deco, mukbt[1] + mukbt[2] - mukbt[4], T);
    screen(s.e2o, s.de2o, 2. * mukbt[2] - mukbt[5], T);
    rates[0] = s.e3a, drates[0] = s.de3a, rates[1] = s.ecag, drates[1] = s.decag;
    rates[2] = s.eoag, drates[2] = s.deoag, rates[13] = s.e2c, drates[13] = s.de2c;
    rates[14] = s.eco, drates[14] = s.deco, rates[15] = s.e2o, drates[15] = s.de2o;
    rates[16] = s.l3a, drates[16] = s.dl3a, rates[17] = s.lcag, drates[17] = s.dlcag;
    rates[18] = s.loag, drates[18] = s.dloag;
}

// ------------------------------------------------------------------ net86
// include/nnet/parameterization/net86/net86.cpp:41-686.  Table reaction i (0..156) has
// forward slot i (i < 3) or i-1 (i > 3) and reverse slot 152 + i (i >= 4).
__device__ __forceinline__ int fwdSlot86(int i) { return i < 3 ? i : i - 1; }
__device__ __forceinline__ int revSlot86(int i) { return 152 + i; }

static __device__ void net86Rates(const NetView& nv, double T, double rho, Strided<double> BE, Strided<double> rates,
                           Strided<double> drates)
{
    correctedBE<86>(nv, T, rho, BE);
    double mukbt[86];
    {
        const double gam = screeningGamma(T, rho);
#pragma unroll 2
        for (int i = 0; i < 86; ++i)
            mukbt[i] = screeningMu(gam, __ldg(nv.z53 + i));
        mukbt[1] = 0; // neutrons
    }
    {
        const FitT   v(T);
        const double t9 = T * 1e-09, t9i = 1. / t9;
        const double val1 = 11.6045 * t9i, val2 = 1.5 * log(t9), val3 = val1 * t9i * 1e-9, val4 = 1.5e-9 * t9i;
        const int    kb   = temperatureRange(T);
#pragma unroll 1
        for (int i = 7; i < 157; ++i)
        {
            const double* f = nv.fit + (i - 7) * 8;
            double        coef, dcoef, e, de;
            fitRate(f, v, coef, dcoef, e, de);
            const int    mr = __ldg(nv.mainReactant + i), sr = __ldg(nv.secondaryReactant + i),
                      mp = __ldg(nv.mainProduct + i);
            const double part = __ldg(nv.choose + (mr - 5) * 24 + kb) / __ldg(nv.choose + (mp - 5) * 24 + kb);
            const double q    = __ldg(nv.q + i - 7);
            double       l, dl;
            if (i < 137)
            {
                l  = part * exp(__ldg(f + 7) + coef - val1 * q + val2);
                dl = l * (dcoef + val3 * q + val4);
            }
            else
            {
                l  = part * exp(__ldg(f + 7) + coef - val1 * q);
                dl = l * (dcoef + val3 * q);
            }
            // (a,p) / (a,n): tabulated direction is the network's reverse (net86.cpp:561-567)
            if ((i >= 137 && i < 154) || i == 156)
            {
                double t = e;
                e = l, l = t, t = de, de = dl, dl = t;
            }
            const double dmu = mukbt[mr] + mukbt[sr] - mukbt[mp];
            const double EF  = exp(dmu);
            e                = e * EF;
            de               = de * EF - 2. * e * dmu / T;
            if (i >= 137)
            {
                l  = l * EF;
                dl = dl * EF - 2. * l * dmu / T;
            }
            rates[fwdSlot86(i)] = e, drates[fwdSlot86(i)] = de;
            rates[revSlot86(i)] = l, drates[revSlot86(i)] = dl;
        }
    }
    Special s;
    specialRates(T, s);
    auto dmu = [&](int i) {
        return mukbt[__ldg(nv.mainReactant + i)] + mukbt[__ldg(nv.secondaryReactant + i)] -
               mukbt[__ldg(nv.mainProduct + i)];
    };
    screen(s.e2c, s.de2c, dmu(0), T);
    screen(s.eco, s.deco, dmu(1), T);
    screen(s.e2o, s.de2o, dmu(2), T);
    screen(s.e3a, s.de3a, dmu(4) + mukbt[__ldg(nv.mainReactant + 4)], T);
    screen(s.ecag, s.decag, dmu(5), T);
    screen(s.eoag, s.deoag, dmu(6), T);
    rates[0] = s.e2c, drates[0] = s.de2c, rates[1] = s.eco, drates[1] = s.deco;
    rates[2] = s.e2o, drates[2] = s.de2o, rates[3] = s.e3a, drates[3] = s.de3a;
    rates[4] = s.ecag, drates[4] = s.decag, rates[5] = s.eoag, drates[5] = s.deoag;
    rates[revSlot86(4)] = s.l3a, drates[revSlot86(4)] = s.dl3a;
    rates[revSlot86(5)] = s.lcag, drates[revSlot86(5)] = s.dlcag;
    rates[revSlot86(6)] = s.loag, drates[revSlot86(6)] = s.dloag;
}

// ------------------------------------------------------------------ net87
// electron-capture table, bilinear in (log10 T, log10 rho Ye) (net87.cpp:102-141)
static __device__ void electronRates(const NetView& nv, double temp, double rhoElec, double ev[12])
{
    constexpr int NT = 41, NR = 51, NC = 12;
    int           ts = 0;
    const double  lT = log10(temp);
    while (ts < NT && __ldg(nv.eLogT + ts) < lT)
        ++ts;
    int          rs = 0;
    const double lR = log10(rhoElec);
    while (rs < NR && __ldg(nv.eLogRho + rs) < lR)
        ++rs;
    const int ti = max(0, ts - 1), ri = max(0, rs - 1);
    ts = min(NT - 1, ts), rs = min(NR - 1, rs);
    const double x2x = __ldg(nv.eLogT + ts) - lT, xx1 = -__ldg(nv.eLogT + ti) + lT;
    const double y2y = __ldg(nv.eLogRho + rs) - lR, yy1 = -__ldg(nv.eLogRho + ri) + lR;
    double       x2x1 = __ldg(nv.eLogT + ts) - __ldg(nv.eLogT + ti);
    x2x1              = x2x1 == 0 ? 2 : x2x1;
    double y2y1       = __ldg(nv.eLogRho + rs) - __ldg(nv.eLogRho + ri);
    y2y1              = y2y1 == 0 ? 2 : y2y1;
    const double* e   = nv.eRate;
#pragma unroll
    for (int i = 0; i < NC; ++i)
        ev[i] = (__ldg(e + (ti * NR + ri) * NC + i) * x2x * y2y + __ldg(e + (ts * NR + ri) * NC + i) * xx1 * y2y +
                 __ldg(e + (ti * NR + rs) * NC + i) * x2x * yy1 + __ldg(e + (ts * NR + rs) * NC + i) * xx1 * yy1) /
                (x2x1 * y2y1);
}

// net87 functor (net87.hpp:117-175): net86 rates plus p(e,nu)n and n(e+,nu)p
static __device__ void net87Rates(const NetView& nv, double Yelec, double T, double rho, Strided<double> BE,
                           Strided<double> rates, Strided<double> drates)
{
    const double rhoElec = Yelec * rho;
    double       ev[12];
    electronRates(nv, T, rhoElec, ev);
    net86Rates(nv, T, rho, BE, rates, drates);
    const double kbt = NNET_KB * T, nakbt = NNET_NA * kbt;
    BE[86] = __ldg(nv.BE + 86) + -1.5 * nakbt;
    BE[0]  = BE[0] + -ev[3];
    BE[1]  = BE[1] + -ev[9];
    rates[309] = rhoElec == 0 ? 0 : ev[0] / rhoElec, drates[309] = rhoElec == 0 ? 0 : ev[1] / rhoElec;
    rates[310] = rhoElec == 0 ? 0 : ev[6] / rhoElec, drates[310] = rhoElec == 0 ? 0 : ev[7] / rhoElec;
}

} // namespace nnet_gb300
