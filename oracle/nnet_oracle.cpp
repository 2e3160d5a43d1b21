// ORACLE — test infrastructure only.  A scalar CPU restatement of SPH-EXA-nnet's
// per-particle burn path, used by tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg as the checker.  Nothing in the product links or calls it.
//
// Every function follows the reference line by line, in the same floating-point
// evaluation order, so that, built with -ffp-contract=off, it reproduces the
// reference compiled from its own sources (oracle/_ref) bit for bit on the same
// machine.  Citations are file:line in the reference tree.
//
// Additions over the reference (identical in the GPU product):
//  * a per-particle Newton-iteration budget -> status MAXITER;
//  * detection of the substep loop's endless retries: between accepted substeps an
//    attempt is determined by (dt, Newton temperature buffer) alone, and the rejection
//    rule (nuclear_net.hpp:745-748 together with :899-904) can return to a state it has
//    seen (period 1 or 2 in practice), or settle on the timestep it maps to itself
//    (dt <- dt 4 / |dT/T| keeps dt where |dT/T| = 4, far above the 0.04 acceptance bound)
//    and wander there within rounding noise; either way the reference retries forever.
//    Brent's algorithm on that pair: the Newton temperature compared bitwise, dt equal
//    within a relative kCycleDtTol -> status LIVELOCK (same rule as the GPU kernels);
//  * dt == 0 at system build (the reference throws, nuclear_net.hpp:533-549) -> ZERO_DT;
//  * the Newton temperature buffer starts at 0 (uninitialised in the reference,
//    nuclear_net.hpp:943 and parallel_nuclear_net.cu:65).
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>
#include <omp.h>

#include "nnet_network_tables.h"

namespace
{
// ---------------------------------------------------------------- constants
// include/nnet/nuclear_net.hpp:48-106
const double kTheta          = 0.8;
const double kMinTemp        = 1e8;
const double kMinRho         = 1e5;
const double kMaxDtStep      = 2;
const double kMinDtStep      = 1e-2;
const double kNanDtStep      = 2e-1;
const double kEpsilonSystem  = 1e-40;
const double kEpsilonVector  = 1e-16;
// relative dt tolerance of the livelock detection (2^-20)
const double kCycleDtTol     = 9.5367431640625e-07;
const double kNRMaxDt        = 1e-2;
const double kNRDTTarget     = 1e-2;
const double kNRDTTol        = 4;
const int    kNRMinIt        = 1;
const int    kNRMaxIt        = 11;
const double kNRItTol        = 1e-7;
const double kSubstepDtTol   = 1e-6;

enum Status
{
    ST_OK       = 0,
    ST_SKIPPED  = 1,
    ST_LIVELOCK = 2,
    ST_MAXITER  = 3,
    ST_ZERO_DT  = 4,
};

// ---------------------------------------------------------------- networks
struct Network
{
    int           nspec, nreact;
    const int *   rbeg, *rspec, *rcnt, *pbeg, *pspec, *pcnt;
    const double* Z; // charges used by the Helmholtz functor over `nspec` entries
};

bool getNetwork(int net, Network& n)
{
    switch (net)
    {
        case 14:
            n = {14, NET14_NUM_REACTIONS, net14_reactant_begin, net14_reactant_species, net14_reactant_count,
                 net14_product_begin, net14_product_species, net14_product_count, net14_Z};
            return true;
        case 86:
            n = {86, NET86_NUM_REACTIONS, net86_reactant_begin, net86_reactant_species, net86_reactant_count,
                 net86_product_begin, net86_product_species, net86_product_count, net86_Z};
            return true;
        case 87:
            n = {87, NET87_NUM_REACTIONS, net87_reactant_begin, net87_reactant_species, net87_reactant_count,
                 net87_product_begin, net87_product_species, net87_product_count, net86_Z};
            return true;
    }
    return false;
}

// EOS output, include/nnet/nuclear_net.hpp:446-459
struct Eos
{
    double cv = 0, dpdT = 0, p = 0, cp = 0, c = 0, u = 0, dse = 0, dpe = 0, dsp = 0, cv_gaz = 0, cp_gaz = 0,
           c_gaz = 0, dudYe = 0;
};

// ---------------------------------------------------------------- ideal gas EOS
// include/nnet/parameterization/eos/ideal_gas.hpp:69-82
Eos idealGas(double mu, double T, double rho)
{
    Eos          r;
    const double R   = 8.317e7;
    const double dmy = R / mu;
    r.cv             = 1.5 * dmy;
    r.u              = T * r.cv;
    r.p              = rho * T * dmy;
    r.c              = std::sqrt(r.p / rho);
    r.dpdT           = rho * dmy;
    return r;
}

// ---------------------------------------------------------------- Helmholtz EOS
// include/nnet/parameterization/eos/helmholtz.hpp:77-126 and helmholtz.cpp:50-965
namespace helm
{
const int    IMAX = 541, JMAX = 201;
const double tlo = 3., thi = 13., tstp = (thi - tlo) / (double)(JMAX - 1), tstpi = 1. / tstp;
const double dlo = -12., dhi = 15., dstp = (dhi - dlo) / (double)(IMAX - 1), dstpi = 1. / dstp;

const double pi      = 3.14159265358979323846264338327950288;
const double h       = 6.6260689633e-27;
const double qe      = 4.8032042712e-10;
const double avo     = 6.0221417930e23;
const double clight  = 2.99792458e10;
const double kerg    = 1.380650424e-16;
const double amu     = 1.66053878283e-24;
const double ssol    = 5.6704e-5;
const double asol    = 4.0 * ssol / clight;
const double kergavo = kerg * avo;
const double sioncon = (2.0 * pi * amu * kerg) / (h * h);
const double a1 = -0.898004, b1 = 0.96786, c1 = 0.220703, d1 = -0.86097, e1 = 2.5269;
const double a2 = 0.29561, b2 = 1.9885, c2 = 0.288675;
const double esqu = qe * qe;

// 21 tables [IMAX][JMAX] in the order f fd ft fdd ftt fdt fddt fdtt fddtt dpdf dpdfd
// dpdft dpdfdt ef efd eft efdt xf xfd xft xfdt
std::vector<double> tab;
double d[IMAX], dd_sav[IMAX - 1], dd2_sav[IMAX - 1], ddi_sav[IMAX - 1], dd2i_sav[IMAX - 1], dd3i_sav[IMAX - 1];
double t_[JMAX], dt_sav[JMAX - 1], dt2_sav[JMAX - 1], dti_sav[JMAX - 1], dt2i_sav[JMAX - 1], dt3i_sav[JMAX - 1];

enum
{
    F, FD, FT, FDD, FTT, FDT, FDDT, FDTT, FDDTT, DPDF, DPDFD, DPDFT, DPDFDT, EF, EFD, EFT, EFDT, XF, XFD, XFT, XFDT
};
inline double at(int k, int i, int j) { return tab[((size_t)k * IMAX + i) * JMAX + j]; }

// grid and spacing arrays, helmholtz.cpp:101-110 and :139-169
void load(const double* src)
{
    tab.assign(src, src + (size_t)21 * IMAX * JMAX);
    for (int i = 0; i < IMAX; ++i)
        d[i] = std::pow((double)10., dlo + i * dstp);
    for (int j = 0; j < JMAX; ++j)
        t_[j] = std::pow((double)10., tlo + j * tstp);
    for (int j = 0; j < JMAX - 1; ++j)
    {
        const double dth = t_[j + 1] - t_[j], dt2 = dth * dth, dti = 1. / dth, dt2i = 1. / dt2;
        dt_sav[j] = dth, dt2_sav[j] = dt2, dti_sav[j] = dti, dt2i_sav[j] = dt2i, dt3i_sav[j] = dt2i * dti;
    }
    for (int i = 0; i < IMAX - 1; ++i)
    {
        const double dd = d[i + 1] - d[i], dd2 = dd * dd, ddi = 1. / dd, dd2i = 1. / dd2;
        dd_sav[i] = dd, dd2_sav[i] = dd2, ddi_sav[i] = ddi, dd2i_sav[i] = dd2i, dd3i_sav[i] = dd2i * ddi;
    }
}

// quintic / cubic Hermite basis, helmholtz.cpp:222-311
inline double psi0(double z) { return z * z * z * (z * (-6. * z + 15.) - 10.) + 1.; }
inline double dpsi0(double z) { return z * z * (z * (-30. * z + 60.) - 30.); }
inline double ddpsi0(double z) { return z * (z * (-120. * z + 180.) - 60.); }
inline double psi1(double z) { return z * (z * z * (z * (-3. * z + 8.) - 6.) + 1.); }
inline double dpsi1(double z) { return z * z * (z * (-15. * z + 32.) - 18.) + 1.; }
inline double ddpsi1(double z) { return z * (z * (-60. * z + 96.) - 36.); }
inline double psi2(double z) { return 0.5 * z * z * (z * (z * (-z + 3.) - 3.) + 1.); }
inline double dpsi2(double z) { return 0.5 * z * (z * (z * (-5. * z + 12.) - 9.) + 2.); }
inline double ddpsi2(double z) { return 0.5 * (z * (z * (-20. * z + 36.) - 18.) + 2.); }
inline double xpsi0(double z) { return z * z * (2. * z - 3.) + 1.; }
inline double xdpsi0(double z) { return z * (6. * z - 6.); }
inline double xpsi1(double z) { return z * (z * (z - 2.) + 1.); }
inline double xdpsi1(double z) { return z * (3. * z - 4.) + 1.; }

// biquintic over the 36 coefficients (helmholtz.cpp:273-286); the sum runs in the
// reference's term order: (w0t,w0mt,w1t,w1mt,w2t,w2mt) x (w0d,w0md) first, then w1d,w1md
// and w2d,w2md blocks as written there.
inline double h5(const double* fi, double w0t, double w1t, double w2t, double w0mt, double w1mt, double w2mt,
                 double w0d, double w1d, double w2d, double w0md, double w1md, double w2md)
{
    return fi[0] * w0d * w0t + fi[1] * w0md * w0t + fi[2] * w0d * w0mt + fi[3] * w0md * w0mt + fi[4] * w0d * w1t +
           fi[5] * w0md * w1t + fi[6] * w0d * w1mt + fi[7] * w0md * w1mt + fi[8] * w0d * w2t + fi[9] * w0md * w2t +
           fi[10] * w0d * w2mt + fi[11] * w0md * w2mt + fi[12] * w1d * w0t + fi[13] * w1md * w0t +
           fi[14] * w1d * w0mt + fi[15] * w1md * w0mt + fi[16] * w2d * w0t + fi[17] * w2md * w0t +
           fi[18] * w2d * w0mt + fi[19] * w2md * w0mt + fi[20] * w1d * w1t + fi[21] * w1md * w1t +
           fi[22] * w1d * w1mt + fi[23] * w1md * w1mt + fi[24] * w2d * w1t + fi[25] * w2md * w1t +
           fi[26] * w2d * w1mt + fi[27] * w2md * w1mt + fi[28] * w1d * w2t + fi[29] * w1md * w2t +
           fi[30] * w1d * w2mt + fi[31] * w1md * w2mt + fi[32] * w2d * w2t + fi[33] * w2md * w2t +
           fi[34] * w2d * w2mt + fi[35] * w2md * w2mt;
}

// bicubic over 16 coefficients (helmholtz.cpp:315-322)
inline double h3(const double* fi, double w0t, double w1t, double w0mt, double w1mt, double w0d, double w1d,
                 double w0md, double w1md)
{
    return fi[0] * w0d * w0t + fi[1] * w0md * w0t + fi[2] * w0d * w0mt + fi[3] * w0md * w0mt + fi[4] * w0d * w1t +
           fi[5] * w0md * w1t + fi[6] * w0d * w1mt + fi[7] * w0md * w1mt + fi[8] * w1d * w0t + fi[9] * w1md * w0t +
           fi[10] * w1d * w0mt + fi[11] * w1md * w0mt + fi[12] * w1d * w1t + fi[13] * w1md * w1t +
           fi[14] * w1d * w1mt + fi[15] * w1md * w1mt;
}

// 2x2 stencil of table k into fi[o..o+3] in the order (i,j) (i+1,j) (i,j+1) (i+1,j+1)
inline void stencil(double* fi, int o, int k, int iat, int jat)
{
    fi[o + 0] = at(k, iat, jat), fi[o + 1] = at(k, iat + 1, jat);
    fi[o + 2] = at(k, iat, jat + 1), fi[o + 3] = at(k, iat + 1, jat + 1);
}

// helmholtz.cpp:341-965
Eos eos(double abar_, double zbar_, double temp, double rho)
{
    double       fi[36];
    const double abar = 1 / abar_;
    const double zbar = zbar_ / abar_;

    // table indices, helmholtz.cpp:325-337
    int iat, jat;
    {
        const double ye  = std::max((double)1e-16, zbar / abar);
        const double din = ye * rho;
        jat              = int((std::log10(temp) - tlo) * tstpi);
        jat              = std::max<int>(1, std::min<int>(jat, JMAX - 2));
        iat              = int((std::log10(din) - dlo) * dstpi);
        iat              = std::max<int>(1, std::min<int>(iat, IMAX - 2));
    }

    const double ytot1 = 1 / abar;
    const double ye    = std::max<double>((double)1e-16, zbar / abar);
    const double din   = ye * rho;
    const double rhoi = 1. / rho, tempi = 1. / temp, kt = kerg * temp, ktinv = 1. / kt;

    // radiation
    const double prad = asol * temp * temp * temp * temp / 3;
    const double dpraddd = 0., dpraddt = 4. * prad * tempi;
    const double erad = 3. * prad * rhoi, deraddd = -erad * rhoi, deraddt = 3. * dpraddt * rhoi;
    const double srad    = (prad * rhoi + erad) * tempi;
    const double dsraddd = (dpraddd * rhoi - prad * rhoi * rhoi + deraddd) * tempi;
    const double dsraddt = (dpraddt * rhoi + deraddt - srad) * tempi;

    // ions
    const double xni = avo * ytot1 * rho, dxnidd = avo * ytot1, dxnida = -xni * ytot1;
    const double pion = xni * kt, dpiondd = dxnidd * kt, dpiondt = xni * kerg, dpionda = dxnida * kt, dpiondz = 0.;
    const double eion = 1.5 * pion * rhoi, deiondd = (1.5 * dpiondd - eion) * rhoi, deiondt = 1.5 * dpiondt * rhoi,
                 deionda = 1.5 * dpionda * rhoi;
    double       x = abar * abar * std::sqrt(abar) * rhoi / avo;
    double       s = sioncon * temp;
    double       z = x * s * std::sqrt(s);
    double       y = std::log(z);
    const double sion    = (pion * rhoi + eion) * tempi + kergavo * ytot1 * y;
    const double dsiondd = (dpiondd * rhoi - pion * rhoi * rhoi + deiondd) * tempi - kergavo * rhoi * ytot1;
    const double dsiondt = (dpiondt * rhoi + deiondt) * tempi - (pion * rhoi + eion) * tempi * tempi +
                           1.5 * kergavo * tempi * ytot1;
    x                    = avo * kerg / abar;
    const double dsionda = (dpionda * rhoi + deionda) * tempi + kergavo * ytot1 * ytot1 * (2.5 - y);

    // electron-positron: biquintic in the free energy
    stencil(fi, 0, F, iat, jat), stencil(fi, 4, FT, iat, jat), stencil(fi, 8, FTT, iat, jat);
    stencil(fi, 12, FD, iat, jat), stencil(fi, 16, FDD, iat, jat), stencil(fi, 20, FDT, iat, jat);
    stencil(fi, 24, FDDT, iat, jat), stencil(fi, 28, FDTT, iat, jat), stencil(fi, 32, FDDTT, iat, jat);

    double xt  = std::max<double>((temp - t_[jat]) * dti_sav[jat], 0.);
    double xd  = std::max<double>((din - d[iat]) * ddi_sav[iat], 0.);
    double mxt = 1. - xt, mxd = 1. - xd;

    double si0t = psi0(xt), si1t = psi1(xt) * dt_sav[jat], si2t = psi2(xt) * dt2_sav[jat];
    double si0mt = psi0(mxt), si1mt = -psi1(mxt) * dt_sav[jat], si2mt = psi2(mxt) * dt2_sav[jat];
    double si0d = psi0(xd), si1d = psi1(xd) * dd_sav[iat], si2d = psi2(xd) * dd2_sav[iat];
    double si0md = psi0(mxd), si1md = -psi1(mxd) * dd_sav[iat], si2md = psi2(mxd) * dd2_sav[iat];

    double dsi0t = dpsi0(xt) * dti_sav[jat], dsi1t = dpsi1(xt), dsi2t = dpsi2(xt) * dt_sav[jat];
    double dsi0mt = -dpsi0(mxt) * dti_sav[jat], dsi1mt = dpsi1(mxt), dsi2mt = -dpsi2(mxt) * dt_sav[jat];
    double dsi0d = dpsi0(xd) * ddi_sav[iat], dsi1d = dpsi1(xd), dsi2d = dpsi2(xd) * dd_sav[iat];
    double dsi0md = -dpsi0(mxd) * ddi_sav[iat], dsi1md = dpsi1(mxd), dsi2md = -dpsi2(mxd) * dd_sav[iat];

    double ddsi0t = ddpsi0(xt) * dt2i_sav[jat], ddsi1t = ddpsi1(xt) * dti_sav[jat], ddsi2t = ddpsi2(xt);
    double ddsi0mt = ddpsi0(mxt) * dt2i_sav[jat], ddsi1mt = -ddpsi1(mxt) * dti_sav[jat], ddsi2mt = ddpsi2(mxt);

    const double free = h5(fi, si0t, si1t, si2t, si0mt, si1mt, si2mt, si0d, si1d, si2d, si0md, si1md, si2md);
    const double df_d = h5(fi, si0t, si1t, si2t, si0mt, si1mt, si2mt, dsi0d, dsi1d, dsi2d, dsi0md, dsi1md, dsi2md);
    const double df_t = h5(fi, dsi0t, dsi1t, dsi2t, dsi0mt, dsi1mt, dsi2mt, si0d, si1d, si2d, si0md, si1md, si2md);
    const double df_tt =
        h5(fi, ddsi0t, ddsi1t, ddsi2t, ddsi0mt, ddsi1mt, ddsi2mt, si0d, si1d, si2d, si0md, si1md, si2md);
    const double df_dt =
        h5(fi, dsi0t, dsi1t, dsi2t, dsi0mt, dsi1mt, dsi2mt, dsi0d, dsi1d, dsi2d, dsi0md, dsi1md, dsi2md);

    // bicubic weights, helmholtz.cpp:562-585
    si0t = xpsi0(xt), si1t = xpsi1(xt) * dt_sav[jat];
    si0mt = xpsi0(mxt), si1mt = -xpsi1(mxt) * dt_sav[jat];
    si0d = xpsi0(xd), si1d = xpsi1(xd) * dd_sav[iat];
    si0md = xpsi0(mxd), si1md = -xpsi1(mxd) * dd_sav[iat];
    dsi0t = xdpsi0(xt) * dti_sav[jat], dsi1t = xdpsi1(xt);
    dsi0mt = -xdpsi0(mxt) * dti_sav[jat], dsi1mt = xdpsi1(mxt);
    dsi0d = xdpsi0(xd) * ddi_sav[iat], dsi1d = xdpsi1(xd);
    dsi0md = -xdpsi0(mxd) * ddi_sav[iat], dsi1md = xdpsi1(mxd);

    stencil(fi, 0, DPDF, iat, jat), stencil(fi, 4, DPDFT, iat, jat);
    stencil(fi, 8, DPDFD, iat, jat), stencil(fi, 12, DPDFDT, iat, jat);
    double dpepdd = h3(fi, si0t, si1t, si0mt, si1mt, si0d, si1d, si0md, si1md);
    dpepdd        = std::max<double>(ye * dpepdd, (double)1.e-30);

    stencil(fi, 0, EF, iat, jat), stencil(fi, 4, EFT, iat, jat);
    stencil(fi, 8, EFD, iat, jat), stencil(fi, 12, EFDT, iat, jat);
    // chemical potential and its derivatives are computed by the reference but do not
    // enter any output field (helmholtz.cpp:627-638)

    stencil(fi, 0, XF, iat, jat), stencil(fi, 4, XFT, iat, jat);
    stencil(fi, 8, XFD, iat, jat), stencil(fi, 12, XFDT, iat, jat);
    // number densities likewise (helmholtz.cpp:659-671)

    // electron-positron thermodynamics, helmholtz.cpp:679-703
    x                   = din * din;
    const double pele   = x * df_d;
    const double dpepdt = x * df_dt;
    s                   = dpepdd / ye - 2.0 * din * df_d;
    const double dpepda = -ytot1 * (2.0 * pele + s * din);
    const double dpepdz = rho * ytot1 * (2.0 * din * df_d + s);

    x                   = ye * ye;
    const double sele   = -df_t * ye;
    const double dsepdt = -df_tt * ye;
    const double dsepdd = -df_dt * x;
    const double dsepda = ytot1 * (ye * df_dt * din - sele);
    const double dsepdz = -ytot1 * (ye * df_dt * rho + df_t);

    const double eele   = ye * free + temp * sele;
    const double deepdt = temp * dsepdt;
    const double deepdd = x * df_d + temp * dsepdd;
    const double deepda = -ye * ytot1 * (free + df_d * din) + temp * dsepda;
    const double deepdz = ytot1 * (free + ye * df_d * rho) + temp * dsepdz;

    // Coulomb corrections (Yakovlev & Shalybkov 1989), helmholtz.cpp:719-824
    z                 = pi * 4. / 3.;
    s                 = z * xni;
    const double dsdd = z * dxnidd;
    const double dsda = z * dxnida;

    const double lami = std::pow((double)1. / s, (double)1. / 3.), inv_lami = 1. / lami;
    z                   = -lami / 3;
    const double lamidd = z * dsdd / s, lamida = z * dsda / s;

    const double plasg = zbar * zbar * esqu * ktinv * inv_lami;
    z                  = -plasg * inv_lami;
    const double plasgdd = z * lamidd, plasgda = z * lamida;
    const double plasgdt = -plasg * ktinv * kerg;
    const double plasgdz = 2.0 * plasg / zbar;

    double ecoul = 0, pcoul = 0, scoul = 0, decouldd = 0, decouldt = 0, decoulda = 0, decouldz = 0, dpcouldd = 0,
           dpcouldt = 0, dpcoulda = 0, dpcouldz = 0, dscouldd = 0, dscouldt = 0, dscoulda = 0, dscouldz = 0;
    if (plasg >= 1.)
    {
        x     = std::pow(plasg, (double)0.25);
        y     = avo * ytot1 * kerg;
        ecoul = y * temp * (a1 * plasg + b1 * x + c1 / x + d1);
        pcoul = rho * ecoul / 3.;
        scoul = -y * (3.0 * b1 * x - 5.0 * c1 / x + d1 * (std::log(plasg) - 1.) - e1);

        y        = avo * ytot1 * kt * (a1 + 0.25 / plasg * (b1 * x - c1 / x));
        decouldd = y * plasgdd;
        decouldt = y * plasgdt + ecoul / temp;
        decoulda = y * plasgda - ecoul / abar;
        decouldz = y * plasgdz;

        y        = rho / 3.;
        dpcouldd = ecoul + y * decouldd / 3.;
        dpcouldt = y * decouldt;
        dpcoulda = y * decoulda;
        dpcouldz = y * decouldz;

        y        = -avo * kerg / (abar * plasg) * (0.75 * b1 * x + 1.25 * c1 / x + d1);
        dscouldd = y * plasgdd;
        dscouldt = y * plasgdt;
        dscoulda = y * plasgda - scoul / abar;
        dscouldz = y * plasgdz;
    }
    else if (plasg < 1.)
    {
        x     = plasg * std::sqrt(plasg);
        y     = std::pow(plasg, (double)b2);
        z     = c2 * x - a2 * y / 3.;
        pcoul = -pion * z;
        ecoul = 3.0 * pcoul / rho;
        scoul = -avo / abar * kerg * (c2 * x - a2 * (b2 - 1.) / b2 * y);

        s        = 1.5 * c2 * x / plasg - a2 * b2 * y / plasg / 3.;
        dpcouldd = -dpiondd * z - pion * s * plasgdd;
        dpcouldt = -dpiondt * z - pion * s * plasgdt;
        dpcoulda = -dpionda * z - pion * s * plasgda;
        dpcouldz = -dpiondz * z - pion * s * plasgdz;

        s        = 3.0 / rho;
        decouldd = s * dpcouldd - ecoul / rho;
        decouldt = s * dpcouldt;
        decoulda = s * dpcoulda;
        decouldz = s * dpcouldz;

        s        = -avo * kerg / (abar * plasg) * (1.5 * c2 * x - a2 * (b2 - 1.) * y);
        dscouldd = s * plasgdd;
        dscouldt = s * plasgdt;
        dscoulda = s * plasgda - scoul / abar;
        dscouldz = s * plasgdz;
    }

    x = prad + pion + pele + pcoul;
    y = erad + eion + eele + ecoul;
    z = srad + sion + sele + scoul;
    if (x <= 0. || y <= 0.)
    {
        pcoul = dpcouldd = dpcouldt = dpcoulda = dpcouldz = 0.;
        ecoul = decouldd = decouldt = decoulda = decouldz = 0.;
        scoul = dscouldd = dscouldt = dscoulda = dscouldz = 0.;
    }

    const double pgas = pion + pele + pcoul, egas = eion + eele + ecoul;
    const double dpgasdd = dpiondd + dpepdd + dpcouldd, dpgasdt = dpiondt + dpepdt + dpcouldt;
    const double degasdt = deiondt + deepdt + decouldt, degasdz = 0. + deepdz + decouldz;
    const double degasdd = deiondd + deepdd + decouldd;
    const double dsgasdd = dsiondd + dsepdd + dscouldd, dsgasdt = dsiondt + dsepdt + dscouldt;
    (void)dsionda, (void)deepda, (void)dpepda, (void)dsepda, (void)dpepdz, (void)dsepdz, (void)decoulda,
        (void)dpcoulda, (void)dscoulda, (void)dscouldz;

    const double pres = prad + pgas, ener = erad + egas;
    const double dpresdd = dpraddd + dpgasdd, dpresdt = dpraddt + dpgasdt;
    const double rhoerdd = deraddd + degasdd, rhoerdt = deraddt + degasdt;
    const double rhotrdd = dsraddd + dsgasdd, rhotrdt = dsraddt + dsgasdt;

    Eos          r;
    double       zz = pgas * rhoi, zzi = rho / pgas;
    const double chit_gas = temp / pgas * dpgasdt, chid_gas = dpgasdd * zzi;
    r.cv_gaz              = degasdt;
    x                     = zz * chit_gas / (temp * r.cv_gaz);
    const double gam1_gas = chit_gas * x + chid_gas;
    r.cp_gaz              = r.cv_gaz * gam1_gas / chid_gas;
    z                     = 1. + (egas + clight * clight) * zzi;
    r.c_gaz               = clight * std::sqrt(gam1_gas / z);

    zz                = pres * rhoi;
    zzi               = rho / pres;
    const double chit = temp / pres * dpresdt, chid = dpresdd * zzi;
    r.cv              = rhoerdt;
    x                 = zz * chit / (temp * r.cv);
    const double gam1 = chit * x + chid;
    r.cp              = r.cv * gam1 / chid;
    z                 = 1. + (ener + clight * clight) * zzi;
    r.c               = clight * std::sqrt(gam1 / z);

    x       = rho * rho;
    r.dse   = temp * rhotrdt / rhoerdt - 1.;
    r.dpe   = (rhoerdd * x + temp * dpresdt) / pres - 1.;
    r.dsp   = -rhotrdd * x / dpresdt - 1.;
    r.dpdT  = dpresdt;
    r.dudYe = degasdz * abar;
    r.p     = pres;
    r.u     = ener;
    return r;
}
} // namespace helm

// Helmholtz functor: abar_ = sum Y, zbar_ = sum Y Z (helmholtz.hpp:217-225,
// nnet_util/eigen.hpp:133-142)
Eos helmFunctor(const double* Y, const double* Z, int n, double T, double rho)
{
    double abar = 0, zbar = 0;
    for (int i = 0; i < n; ++i)
        abar = abar + Y[i];
    for (int i = 0; i < n; ++i)
        zbar += Y[i] * Z[i];
    return helm::eos(abar, zbar, T, rho);
}

// ---------------------------------------------------------------- rates: shared pieces
// temperature-bin of the partition-function tables, net14_tables.hpp:71-101 (identical
// in net86_tables.hpp:46-76)
int temperatureRange(double T)
{
    static const double edges[23] = {1.5e8, 2e8,   3e8,   4e8, 5e8, 6e8, 7e8, 8e8, 9e8, 1e9, 1.5e9, 2e9,
                                     2.5e9, 3e9,   3.5e9, 4e9, 4.5e9, 5e9, 6e9, 7e9, 8e9, 9e9, 1e10};
    for (int k = 0; k < 23; ++k)
        if (T < edges[k]) return k;
    return 23;
}

// Coulomb correction functions, net14_tables.hpp:47-69 (= net86_constants.hpp)
double ggt1(double x)
{
    const double a1 = -.898004, b1 = .96786, c1 = .220703, d1 = -.86097;
    const double s  = std::sqrt(std::sqrt(x));
    return a1 * x + b1 * s + c1 / s + d1;
}
double glt1(double x)
{
    const double a1 = -.5 * std::sqrt(3.), b1 = .29561, c1 = 1.9885;
    return a1 * x * std::sqrt(x) + b1 * std::pow(x, c1);
}

// binding energies with ideal-gas and Coulomb corrections (net14.cpp:46-75, net86.cpp:47-74)
void correctedBE(const double* BE, const double* Z, int n, double T, double rho, double* out)
{
    const double kbt = NNET_KB * T, nakbt = NNET_NA * kbt, correction = -1.5 * nakbt;
    for (int i = 0; i < n; ++i)
        out[i] = BE[i] + correction;
    const double ne  = rho * NNET_NA / 2.;
    const double ae  = std::pow((3. / 4.) / (NNET_PI * ne), 1. / 3.);
    const double gam = NNET_E2 / (kbt * ae);
    for (int i = 0; i < n; ++i)
    {
        const double gamma   = gam * std::pow(Z[i], 5. / 3.);
        const double funcion = gamma > 1 ? ggt1(gamma) : glt1(gamma);
        out[i] -= nakbt * funcion;
    }
}

// screening chemical potentials mu/kT per species (net14.cpp:597-616, net86.cpp:577-596)
void screeningMu(const double* Z, int n, double T, double rho, double* mukbt)
{
    const double ne  = rho * NNET_NA / 2.;
    const double kbt = T * NNET_KB;
    const double ae  = std::pow(3. / (4. * NNET_PI * ne), 1. / 3.);
    const double gam = NNET_E2 / (kbt * ae);
    const double a1 = -.898004, b1 = .96786, c1 = .220703, d1 = -.86097, e1 = 2.520058332;
    for (int i = 0; i < n; ++i)
    {
        const double gamp = gam * std::pow(Z[i], 5. / 3.), sg = std::sqrt(gamp), s2 = std::sqrt(sg);
        if (gamp <= 1)
            mukbt[i] = -(1. / std::sqrt(3.)) * gamp * sg + std::pow(gamp, 1.9885) * .29561 / 1.9885;
        else
            mukbt[i] = a1 * gamp + 4. * (b1 * s2 - c1 / s2) + d1 * std::log(gamp) - e1;
    }
}

// fitted forward rate of fit row `f` (net14.cpp:104-131, net86.cpp:107-130)
struct FitT
{
    double t9, t913, t923, t953, t9i, t9i2, t9i13, t9i23, t9i43, lt9;
    explicit FitT(double T)
    {
        t9 = T / 1.e9, t913 = std::pow(t9, 1. / 3.), t923 = t913 * t913, t953 = std::pow(t9, 5. / 3.);
        t9i = 1.e0 / t9, t9i2 = t9i * t9i, t9i13 = 1.e0 / t913, t9i23 = t9i13 * t9i13, t9i43 = t9i23 * t9i23;
        lt9 = std::log(t9);
    }
};
inline void fitRate(const double* f, const FitT& v, double& coef, double& dcoef, double& eff, double& deff)
{
    coef  = f[1] * v.t9i + f[2] * v.t9i13 + f[3] * v.t913 + f[4] * v.t9 + f[5] * v.t953 + f[6] * v.lt9;
    dcoef = (-f[1] * v.t9i2 + (-f[2] * v.t9i43 + f[3] * v.t9i23 + 5 * f[5] * v.t923) * (1. / 3.) + f[4] +
             f[6] * v.t9i) *
            1e-9;
    eff  = std::exp(f[0] + coef);
    deff = eff * dcoef;
}

// Rates of the seven special (non-fitted) reactions of net14 / net86
// (net14.cpp:153-561, net86.cpp:135-505).  Output in a "special" index space:
// s3a=0, s2c=1, sco=2, s2o=3, scag=4, soag=5.  eff/deff forward, l/dl reverse
// (only 3a, cag, oag have reverses).
struct Special
{
    double eff[6], deff[6], l[6], dl[6];
};
enum
{
    S3A = 0,
    S2C,
    SCO,
    S2O,
    SCAG,
    SOAG
};

void specialRates(double T, Special& s)
{
    std::fill(s.l, s.l + 6, 0.), std::fill(s.dl, s.dl + 6, 0.);
    {
        const double t9r = T * 1.0e-09, t9 = std::min((double)10., t9r);
        const double t92 = t9 * t9, t93 = t92 * t9, t95 = t92 * t93, t912 = std::sqrt(t9);
        const double t913 = std::pow(t9, 1. / 3.), t923 = t913 * t913, t932 = t9 * t912, t943 = t9 * t913,
                     t953 = t9 * t923;
        const double t9i = 1. / t9, t9i13 = 1. / t913, t9i23 = 1. / t923, t9i32 = 1. / t932, t9rm1 = 1. / t9r,
                     t9r32 = t9 * std::sqrt(t9r);
        {
            const double r2abe = (7.40e+05 * t9i32) * std::exp(-1.0663 * t9i) +
                                 4.164e+09 * t9i23 * std::exp(-13.49 * t9i13 - t92 / 0.009604) *
                                     (1. + 0.031 * t913 + 8.009 * t923 + 1.732 * t9 + 49.883 * t943 + 27.426 * t953);
            const double rbeac = (130. * t9i32) * std::exp(-3.3364 * t9i) +
                                 2.510e+07 * t9i23 * std::exp(-23.57 * t9i13 - t92 / 0.055225) *
                                     (1. + 0.018 * t913 + 5.249 * t923 + 0.650 * t9 + 19.176 * t943 + 6.034 * t953);
            if (T > 8e7)
                s.eff[S3A] = 2.90e-16 * (r2abe * rbeac) + 0.1 * 1.35e-07 * t9i32 * std::exp(-24.811 * t9i);
            else
                s.eff[S3A] = 2.90e-16 * (r2abe * rbeac) *
                                 (0.01 + 0.2 * (1. + 4. * std::exp(-std::pow(0.025 * t9i, 3.263))) /
                                             (1. + 4. * std::exp(-std::pow(t9 / 0.025, 9.227)))) +
                             0.1 * 1.35e-07 * t9i32 * std::exp(-24.811 * t9i);
            const double rev = 2.e20 * std::exp(-84.419412e0 * t9i);
            s.l[S3A]         = s.eff[S3A] * rev * t93;
        }
        {
            const double t9a = t9 / (1. + 0.0396 * t9), t9a13 = std::pow(t9a, 1. / 3.),
                         t9a56 = std::pow(t9a, 5. / 6.);
            s.eff[S2C]         = 4.27e+26 * t9a56 * t9i32 * std::exp(-84.165 / t9a13 - 2.12e-03 * t93);
        }
        {
            s.eff[SCO] = 0;
            if (T >= 5e8)
            {
                const double t9ap = t9 / (1. + 0.055 * t9), t9a2p = t9ap * t9ap, t9a13p = std::pow(t9ap, 1. / 3.),
                             t9a23p = t9a13p * t9a13p, t9a56ap = std::pow(t9ap, 5. / 6.);
                s.eff[SCO] = 1.72e+31 * t9a56ap * t9i32 * std::exp(-106.594 / t9a13p) /
                             (std::exp(-0.18 * t9a2p) + 1.06e-03 * std::exp(2.562 * t9a23p));
            }
        }
        s.eff[S2O] = 7.10e+36 * t9i23 * std::exp(-135.93 * t9i13 - 0.629 * t923 - 0.445 * t943 + 0.0103 * t92);
        {
            s.eff[SCAG] =
                1.04e+08 / (t92 * std::pow(1. + 0.0489 * t9i23, 2.)) * std::exp(-32.120 * t9i13 - t92 / 12.222016) +
                1.76e+08 / (t92 * std::pow(1. + 0.2654 * t9i23, 2.)) * std::exp(-32.120 * t9i13) +
                1.25e+03 * t9i32 * std::exp(-27.499 * t9i) + 1.43e-02 * t95 * std::exp(-15.541 * t9i);
            s.l[SCAG] = s.eff[SCAG] * 5.13e+10 * t9r32 * std::exp(-83.108047 * t9rm1);
        }
        {
            s.eff[SOAG] = (9.37e+09 * t9i23 * std::exp(-39.757 * t9i13 - t92 / 2.515396) +
                           62.1 * t9i32 * std::exp(-10.297 * t9i) + 538. * t9i32 * std::exp(-12.226 * t9i) +
                           13. * t92 * std::exp(-20.093 * t9i));
            s.l[SOAG] = s.eff[SOAG] * 5.65e+10 * t9r32 * std::exp(-54.93807 * t9rm1);
        }
    }
    {
        // temperature derivatives (unclamped t9)
        const double t9 = T * 1.0e-09, t92 = t9 * t9, t93 = t92 * t9, t94 = t93 * t9, t95 = t94 * t9;
        const double t912 = std::sqrt(t9), t913 = std::pow(t9, 1. / 3.), t923 = t913 * t913, t932 = t9 * t912,
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
            const double dvA = 24.811 * t9i2;
            const double dvB = 1.0663 * t9i2;
            const double dvC = t9i43 * 13.49 / 3. - 208.246564 * t9;
            const double dvD = (t9i23 * .031 + t9i13 * 16.018 + 5.196 + t913 * 199.532 + t923 * 137.13) / 3.;
            const double dvE = 3.3364 * t9i2;
            const double dvF = t9i43 * 23.57 / 3. - 36.21548212 * t9;
            const double dvG = (t9i23 * .018 + t9i13 * 10.498 + 1.950 + t913 * 76.704 + t923 * 30.17) / 3.;

            const double r2abe  = 7.4e5 * t9i32 * std::exp(vB) + 4.164e9 * t9i23 * vD * std::exp(vC);
            const double rbeac  = 130. * t9i32 * std::exp(vE) + 2.510e7 * t9i23 * vG * std::exp(vF);
            const double dr2abe = std::exp(vB) * (-1.11e6 * t9i52 + 7.4e5 * t9i32 * dvB) +
                                  4.164e9 * std::exp(vC) * (-t9i53 * vD * 2. / 3. + t9i23 * dvC * vD + t9i23 * dvD);
            const double drbeac = std::exp(vE) * (-195. * t9i52 + 130. * t9i32 * dvE) +
                                  2.510e7 * std::exp(vF) * (-2. * t9i53 * vG / 3. + t9i23 * dvF * vG + t9i23 * dvG);
            s.deff[S3A] =
                (2.90e-16 * (dr2abe * rbeac + r2abe * drbeac) + 1.35e-8 * std::exp(vA) * (-1.5 * t9i52 + t9i32 * dvA)) *
                1.e-9;
        }
        {
            const double vA = -84.419412 * t9i, dvA = 84.419412 * t9i2;
            s.dl[S3A] = 2.00e20 * std::exp(vA) * t93 * (dvA * s.eff[S3A] + 3. * t9i * s.eff[S3A] + s.deff[S3A]) * 1.e-9;
        }
        {
            const double vA   = t9 / (1. + .0396 * t9);
            const double vA56 = std::pow(vA, 5. / 6.);
            const double vB   = -84.165 * std::pow(vA, -1. / 3.) - 2.12e-3 * t93;
            const double dvA  = vA * vA * t9i2;
            const double dvB  = 28.055 * dvA * std::pow(vA, -4. / 3.) - 6.36e-3 * t92;
            s.deff[S2C]       = 4.27e26 * t9i32 * std::exp(vB) *
                          (std::pow(vA, -1. / 6.) * dvA * 5. / 6. - 1.5 * vA56 * t9i + vA56 * dvB) * 1.e-9;
        }
        {
            s.deff[SCO] = 0;
            if (t9 > .5)
            {
                const double vA   = t9 / (1. + .055 * t9);
                const double vA56 = std::pow(vA, 5. / 6.);
                const double vB   = -106.594 * std::pow(vA, -1. / 3.);
                const double vC   = -.18 * vA * vA;
                const double vD   = 2.562 * std::pow(vA, 2. / 3.);
                const double val  = std::exp(vC) + 1.06e-3 * std::exp(vD);
                const double dvA  = vA * vA * t9i2;
                const double dvB  = 106.594 * std::pow(vA, -4. / 3.) * dvA / 3.;
                const double dvC  = -.36 * vA * dvA;
                const double dvD  = 1.708 * dvA * std::pow(vA, -1. / 3.);
                const double dval = dvC * std::exp(vC) + 1.06e-3 * dvD * std::exp(vD);
                s.deff[SCO]       = 1.72e31 * t9i32 *
                              (std::pow(vA, -1. / 6.) * dvA * 5. / 6. - 1.5 * vA56 * t9i + vA56 * (dvB - dval / val)) *
                              std::exp(vB) / val * 1.e-9;
            }
        }
        {
            const double vA  = -135.93e0 * t9i13 - .629 * t923 - .445 * t943 + .0103 * t92;
            const double dvA = 45.31 * t9i43 - .629 * t9i13 * 2. / 3. - .445 * t913 * 4. / 3. + .0206 * t9;
            s.deff[S2O]      = 7.10e36 * std::exp(vA) * t9i23 * (-t9i * 2. / 3. + dvA) * 1.e-9;
        }
        {
            const double vB  = std::pow(1. + .0489 * t9i23, 2);
            const double vC  = -32.120 * t9i13 - std::pow(t9 / 3.496, 2.);
            const double vD  = std::pow(1. + .2654 * t9i23, 2);
            const double vE  = -32.120 * t9i13;
            const double vF  = -27.499 * t9i;
            const double vG  = -15.541 * t9i;
            const double dvB = -(2. + .0978 * t9i23) * (.0326 * t9i53);
            const double dvC = 32.120 * t9i43 / 3. - 2. * t9 / std::pow(3.496, 2.);
            const double dvD = -(2. + .5308 * t9i23) * (.5308 * t9i53 / 3.);
            const double dvE = 32.120 * t9i43 / 3.;
            const double dvF = 27.499 * t9i2;
            const double dvG = 15.541 * t9i2;
            s.deff[SCAG]     = (1.04e8 * std::exp(vC) * t9i2 * (-2. * t9i + dvC - dvB / vB) / vB +
                            1.76e8 * std::exp(vE) * t9i2 * (-2. * t9i + dvE - dvD / vD) / vD +
                            1.25e3 * std::exp(vF) * (-1.5 * t9i52 + dvF * t9i32) +
                            1.43e-2 * std::exp(vG) * (5. * t94 + dvG * t95)) *
                           1.e-9;
        }
        {
            const double vA  = -83.108047 * t9i;
            const double vB  = -39.757 * t9i13 - std::pow(t9 / 1.586, 2.);
            const double vC  = -10.297 * t9i;
            const double vD  = -12.226 * t9i;
            const double vE  = -20.093 * t9i;
            const double dvA = 83.108047 * t9i2;
            const double dvB = 39.757 * t9i43 / 3. - 2. * t9 / std::pow(1.586, 2.);
            const double dvC = 10.297 * t9i2;
            const double dvD = 12.226 * t9i2;
            const double dvE = 20.093 * t9i2;
            s.dl[SCAG] = 5.13e10 * std::exp(vA) *
                         (s.deff[SCAG] * t932 + s.eff[SCAG] * 1.5 * t912 + s.eff[SCAG] * t932 * dvA) * 1.e-9;
            s.deff[SOAG] = (9.37e9 * std::exp(vB) * (-t9i53 * 2. / 3. + t9i23 * dvB) +
                            62.1 * std::exp(vC) * (-1.5 * t9i52 + t9i32 * dvC) +
                            538. * std::exp(vD) * (-1.5 * t9i52 + t9i32 * dvD) +
                            13. * std::exp(vE) * (2. * t9 + t92 * dvE)) *
                           1.e-9;
        }
        {
            const double vA = -54.903255 * t9i, dvA = 54.903255 * t9i2;
            s.dl[SOAG] = 5.65e10 * std::exp(vA) *
                         (s.deff[SOAG] * t932 + 1.5 * s.eff[SOAG] * t912 + s.eff[SOAG] * t932 * dvA) * 1.e-9;
        }
    }
}

// ---------------------------------------------------------------- net14 rates
// include/nnet/parameterization/net14/net14.cpp:40-660
void net14Rates(double T, double rho, double* BE, double* rates, double* drates)
{
    correctedBE(net14_BE, net14_Z, 14, T, rho, BE);

    double coefs[10], dcoefs[10], eff[16] = {0.}, deff[16] = {0.}, l[16] = {0.}, dl[16] = {0.}, mukbt[16] = {0.},
                                  deltamukbt[16] = {0.};
    {
        const FitT v(T);
        for (int i = 4; i < 14; ++i)
            fitRate(net14_fit + (i - 4) * 8, v, coefs[i - 4], dcoefs[i - 4], eff[i - 1], deff[i - 1]);
    }
    {
        const double t9 = T / 1.e9, t9i = 1.e0 / t9, lt9 = std::log(t9);
        const double val1 = 11.6045e0 * t9i, val2 = 1.5e0 * lt9, val3 = val1 * t9i * 1e-9, val4 = 1.5e-9 * t9i;
        const int    k    = temperatureRange(T);
        for (int i = 4; i < 14; ++i)
        {
            const double* f = net14_fit + (i - 4) * 8;
            l[i - 1] = net14_choose[(i - 4) * 24 + k] / net14_choose[(i + 1 - 4) * 24 + k] *
                       std::exp(coefs[i - 4] + f[7] - net14_q[i - 4] * val1 + val2);
            dl[i - 1] = l[i - 1] * (dcoefs[i - 4] + net14_q[i - 4] * val3 + val4);
        }
    }
    {
        Special s;
        specialRates(T, s);
        // net14 slots: 3a=0, cag=1, oag=2, 2C=13, C+O=14, 2O=15 (net14.cpp:197-352)
        eff[0] = s.eff[S3A], l[0] = s.l[S3A], eff[13] = s.eff[S2C], eff[14] = s.eff[SCO], eff[15] = s.eff[S2O];
        eff[1] = s.eff[SCAG], l[1] = s.l[SCAG], eff[2] = s.eff[SOAG], l[2] = s.l[SOAG];
        deff[0] = s.deff[S3A], dl[0] = s.dl[S3A], deff[13] = s.deff[S2C], deff[14] = s.deff[SCO],
        deff[15] = s.deff[S2O], deff[1] = s.deff[SCAG], dl[1] = s.dl[SCAG], deff[2] = s.deff[SOAG],
        dl[2] = s.dl[SOAG];
    }
    {
        // screening, net14.cpp:590-643
        screeningMu(net14_Z, 14, T, rho, mukbt);
        for (int i = 0; i < 14; ++i)
            deltamukbt[i] = mukbt[i] + mukbt[0] - mukbt[i + 1];
        deltamukbt[0] += mukbt[0];
        deltamukbt[13] = 2. * mukbt[1] - mukbt[3];
        deltamukbt[14] = mukbt[1] + mukbt[2] - mukbt[4];
        deltamukbt[15] = 2. * mukbt[2] - mukbt[5];
        for (int i = 0; i < 16; ++i)
        {
            const double EF = std::exp(deltamukbt[i]);
            eff[i]          = eff[i] * EF;
            deff[i]         = deff[i] * EF - 2. * eff[i] * deltamukbt[i] / T;
        }
    }
    int idx = 0;
    for (int i = 0; i < 16; ++i, ++idx)
        rates[idx] = eff[i], drates[idx] = deff[i];
    for (int i = 0; i < 13; ++i, ++idx)
        rates[idx] = l[i], drates[idx] = dl[i];
}

// ---------------------------------------------------------------- net86 rates
// include/nnet/parameterization/net86/net86.cpp:41-686
void net86Rates(double T, double rho, double* BE, double* rates, double* drates)
{
    correctedBE(net86_BE, net86_Z, 86, T, rho, BE);

    double coefs[150], dcoefs[150], eff[157] = {0.}, deff[157] = {0.}, l[157] = {0.}, dl[157] = {0.},
                                     mukbt[86] = {0.}, deltamukbt[157] = {0.};
    {
        const FitT v(T);
        for (int i = 7; i < 157; ++i)
            fitRate(net86_fit + (i - 7) * 8, v, coefs[i - 7], dcoefs[i - 7], eff[i], deff[i]);
    }
    {
        Special s;
        specialRates(T, s);
        // net86 slots: 2C=0, C+O=1, 2O=2, 3a=4, cag=5, oag=6 (net86.cpp:135-505)
        eff[4] = s.eff[S3A], l[4] = s.l[S3A], eff[0] = s.eff[S2C], eff[1] = s.eff[SCO], eff[2] = s.eff[S2O];
        eff[5] = s.eff[SCAG], l[5] = s.l[SCAG], eff[6] = s.eff[SOAG], l[6] = s.l[SOAG];
        deff[4] = s.deff[S3A], dl[4] = s.dl[S3A], deff[0] = s.deff[S2C], deff[1] = s.deff[SCO],
        deff[2] = s.deff[S2O], deff[5] = s.deff[SCAG], dl[5] = s.dl[SCAG], deff[6] = s.deff[SOAG],
        dl[6] = s.dl[SOAG];
    }
    {
        // reverse rates by detailed balance, net86.cpp:510-554
        const double t9 = T * 1e-09, t9i = 1. / t9;
        const double val1 = 11.6045 * t9i, val2 = 1.5 * std::log(t9), val3 = val1 * t9i * 1e-9, val4 = 1.5e-9 * t9i;
        const int    k    = temperatureRange(T);
        for (int i = 7; i < 157; ++i)
        {
            const double part = net86_choose[(net86_main_reactant[i] - 5) * 24 + k] /
                                net86_choose[(net86_main_product[i] - 5) * 24 + k];
            const double* f = net86_fit + (i - 7) * 8;
            if (i < 137)
            {
                l[i]  = part * std::exp(f[7] + coefs[i - 7] - val1 * net86_q[i - 7] + val2);
                dl[i] = l[i] * (dcoefs[i - 7] + val3 * net86_q[i - 7] + val4);
            }
            else
            {
                l[i]  = part * std::exp(f[7] + coefs[i - 7] - val1 * net86_q[i - 7]);
                dl[i] = l[i] * (dcoefs[i - 7] + val3 * net86_q[i - 7]);
            }
        }
    }
    // (a,p) and (a,n): the tabulated direction is the network's inverse (net86.cpp:561-567)
    for (int i = 137; i < 154; ++i)
        std::swap(eff[i], l[i]), std::swap(deff[i], dl[i]);
    std::swap(eff[156], l[156]), std::swap(deff[156], dl[156]);
    {
        // screening, net86.cpp:569-659
        screeningMu(net86_Z, 86, T, rho, mukbt);
        mukbt[1] = 0;
        for (int i = 0; i < 157; ++i)
            deltamukbt[i] =
                mukbt[net86_main_reactant[i]] + mukbt[net86_secondary_reactant[i]] - mukbt[net86_main_product[i]];
        deltamukbt[4] += mukbt[net86_main_reactant[4]];
        for (int i = 0; i < 157; ++i)
        {
            const double EF = std::exp(deltamukbt[i]);
            eff[i]          = eff[i] * EF;
            deff[i]         = deff[i] * EF - 2. * eff[i] * deltamukbt[i] / T;
        }
        for (int i = 137; i < 157; ++i)
        {
            const double EF = std::exp(deltamukbt[i]);
            l[i]            = l[i] * EF;
            dl[i]           = dl[i] * EF - 2. * l[i] * deltamukbt[i] / T;
        }
    }
    int idx = 0;
    for (int i = 0; i < 157; ++i)
        if (i != 3) rates[idx] = eff[i], drates[idx] = deff[i], ++idx;
    for (int i = 4; i < 157; ++i, ++idx)
        rates[idx] = l[i], drates[idx] = dl[i];
}

// ---------------------------------------------------------------- net87 rates
// electron-capture table, bilinear in (log10 T, log10 rho Ye): net87.cpp:102-141
void electronInterpolate(double temp, double rhoElec, double* rate)
{
    const int     NT = NET87_ELECTRON_NTEMP, NR = NET87_ELECTRON_NRHO, NC = NET87_ELECTRON_NC;
    const double* lt = net87_electron_log_temp;
    const double* lr = net87_electron_log_rho;
    int           ts = 0;
    const double  log_temp = std::log10(temp);
    while (ts < NT && lt[ts] < log_temp)
        ++ts;
    int          rs      = 0;
    const double log_rho = std::log10(rhoElec);
    while (rs < NR && lr[rs] < log_rho)
        ++rs;
    const int ti = std::max(0, ts - 1), ri = std::max(0, rs - 1);
    ts = std::min(NT - 1, ts), rs = std::min(NR - 1, rs);
    const double x2x = lt[ts] - log_temp, xx1 = -lt[ti] + log_temp;
    const double y2y = lr[rs] - log_rho, yy1 = -lr[ri] + log_rho;
    double       x2x1 = lt[ts] - lt[ti];
    x2x1              = x2x1 == 0 ? 2 : x2x1;
    double y2y1       = lr[rs] - lr[ri];
    y2y1              = y2y1 == 0 ? 2 : y2y1;
    const double* e   = net87_electron_rate;
    for (int i = 0; i < NC; ++i)
        rate[i] = (e[(ti * NR + ri) * NC + i] * x2x * y2y + e[(ts * NR + ri) * NC + i] * xx1 * y2y +
                   e[(ti * NR + rs) * NC + i] * x2x * yy1 + e[(ts * NR + rs) * NC + i] * xx1 * yy1) /
                  (x2x1 * y2y1);
}

// net87 functor, net87.hpp:117-175
void net87Rates(const double* Y, double T, double rho, double* BE, double* rates, double* drates)
{
    const double Yelec = Y[86], rhoElec = Yelec * rho;
    double       ev[NET87_ELECTRON_NC];
    electronInterpolate(T, rhoElec, ev);
    net86Rates(T, rho, BE, rates, drates);
    const double kbt = NNET_KB * T, nakbt = NNET_NA * kbt, correction = -1.5 * nakbt;
    BE[86] = net87_BE[86] + correction;
    BE[0] += -ev[3];
    BE[1] += -ev[9];
    rates[309]  = rhoElec == 0 ? 0 : ev[0] / rhoElec;
    drates[309] = rhoElec == 0 ? 0 : ev[1] / rhoElec;
    rates[310]  = rhoElec == 0 ? 0 : ev[6] / rhoElec;
    drates[310] = rhoElec == 0 ? 0 : ev[7] / rhoElec;
}

void networkRates(int net, const double* Y, double T, double rho, double* BE, double* rates, double* drates)
{
    if (net == 14)
        net14Rates(T, rho, BE, rates, drates);
    else if (net == 86)
        net86Rates(T, rho, BE, rates, drates);
    else
        net87Rates(Y, T, rho, BE, rates, drates);
}

// ---------------------------------------------------------------- solver core
struct Ctx
{
    int     net, dim, eos_kind;
    double  mu;
    Network n;
};

Eos computeEos(const Ctx& c, const double* Y, double T, double rho)
{
    if (c.eos_kind == 0) return idealGas(c.mu, T, rho);
    return helmFunctor(Y, c.n.Z, c.dim, T, rho);
}

// dY/dt from the reaction list (nuclear_net.hpp:347-381); dY has stride 1
void derivatives(const Network& n, const double* rates, double rho, const double* Y, double* dY, int dim)
{
    for (int i = 0; i < dim; ++i)
        dY[i] = 0.;
    for (int r = 0; r < n.nreact; ++r)
    {
        double rate = rates[r];
        for (int k = n.rbeg[r]; k < n.rbeg[r + 1]; ++k)
        {
            const int cnt = n.rcnt[k];
            if (cnt != 1) rate /= std::tgamma(cnt + 1);
            rate *= std::pow(Y[n.rspec[k]] * rho, cnt);
        }
        rate /= rho;
        for (int k = n.rbeg[r]; k < n.rbeg[r + 1]; ++k)
            dY[n.rspec[k]] -= rate * n.rcnt[k];
        for (int k = n.pbeg[r]; k < n.pbeg[r + 1]; ++k)
            dY[n.pspec[k]] += rate * n.pcnt[k];
    }
}

// species-block Jacobian into Mp (nuclear_net.hpp:395-438)
void jacobian(const Network& n, const double* rates, double rho, const double* Y, double* M, int dim)
{
    const int ld = dim + 1;
    for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j)
            M[(i + 1) + ld * (j + 1)] = 0.;
    for (int r = 0; r < n.nreact; ++r)
    {
        double rate = rates[r];
        for (int k = n.rbeg[r]; k < n.rbeg[r + 1]; ++k)
        {
            const int cnt = n.rcnt[k];
            if (cnt != 1) rate /= std::tgamma(cnt + 1);
            rate *= std::pow(Y[n.rspec[k]] * rho, cnt - 1);
        }
        if (rate > kEpsilonSystem)
            for (int k = n.rbeg[r]; k < n.rbeg[r + 1]; ++k)
            {
                const int id        = n.rspec[k];
                double    this_rate = rate;
                for (int o = n.rbeg[r]; o < n.rbeg[r + 1]; ++o)
                    if (n.rspec[o] != id) this_rate *= Y[n.rspec[o]] * rho;
                for (int o = n.rbeg[r]; o < n.rbeg[r + 1]; ++o)
                    M[(n.rspec[o] + 1) + ld * (id + 1)] -= this_rate * n.rcnt[o];
                for (int o = n.pbeg[r]; o < n.pbeg[r + 1]; ++o)
                    M[(n.pspec[o] + 1) + ld * (id + 1)] += this_rate * n.pcnt[o];
            }
    }
}

// system around the guess (nuclear_net.hpp:514-609); dt != 0 is checked by the caller
void prepareFromGuess(const Ctx& c, double* Mp, double* RHS, double* rates, const double* Y, double T,
                      const double* Yg, double Tg, double rho, double drho_dt, const Eos& e, double dt)
{
    const int dim = c.dim, ld = dim + 1;
    double*   BE  = RHS + 1;
    double*   drT = Mp + dim + 1;
    networkRates(c.net, Yg, Tg, rho, BE, rates, drT);
    derivatives(c.n, drT, rho, Yg, &Mp[1], dim);
    for (int i = 0; i < dim; ++i)
        Mp[0 + ld * (i + 1)] = -BE[i] / e.cv;
    derivatives(c.n, rates, rho, Yg, &RHS[1], dim);
    for (int i = 0; i < dim; ++i)
        RHS[i + 1] *= dt;
    for (int i = 0; i < dim; ++i)
    {
        RHS[i + 1] += -kTheta * dt * Mp[(i + 1) + 0] * (Tg - T);
        Mp[(i + 1) + 0] *= -kTheta * dt;
    }
    jacobian(c.n, rates, rho, Yg, Mp, dim);
    for (int i = 0; i < dim; ++i)
    {
        double corr = 0;
        for (int j = 0; j < dim; ++j)
            corr += Mp[(i + 1) + ld * (j + 1)] * (Yg[j] - Y[j]);
        RHS[i + 1] += -kTheta * dt * corr;
    }
    for (int i = 0; i < dim; ++i)
    {
        Mp[(i + 1) + ld * (i + 1)] = 1. - kTheta * dt * Mp[(i + 1) + ld * (i + 1)];
        for (int j = 0; j < dim; ++j)
            if (i != j) Mp[(i + 1) + ld * (j + 1)] = -kTheta * dt * Mp[(i + 1) + ld * (j + 1)];
    }
    const double drho = drho_dt * dt, value_1 = e.dpdT * drho / (rho * rho);
    RHS[0] = T * value_1 / e.cv;
    Mp[0]  = 1 - kTheta * value_1 / e.cv;
}

// dense Gaussian elimination without pivoting (nnet_util/eigen.hpp:178-223)
void denseSolve(double* M, double* RHS, double* X, int n, double eps)
{
    for (int i = 0; i < n; ++i)
    {
        for (int j = 0; j < i; ++j)
        {
            const double w = M[i + n * j];
            M[i + n * j]   = 0;
            if (std::abs(w) > eps)
            {
                RHS[i] -= w * RHS[j];
                for (int k = j + 1; k < n; ++k)
                    M[i + n * k] -= w * M[j + n * k];
            }
        }
        const double diag = M[i + n * i];
        M[i + n * i]      = 1;
        RHS[i] /= diag;
        for (int j = i + 1; j < n; ++j)
            M[i + n * j] /= diag;
    }
    for (int i = n - 1; i >= 0; --i)
    {
        double res = RHS[i];
        for (int j = i + 1; j < n; ++j)
            res -= M[i + n * j] * X[j];
        X[i] = res;
    }
}

// Brent cycle detection on the attempt-start state (dt, Newton temperature buffer)
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
            if (bits(dt) == sdt || std::fabs(dt - saved) <= kCycleDtTol * dt) return true;
        }
        if (++steps == power) sdt = bits(dt), snt = bits(nt), power <<= 1, steps = 0;
        return false;
    }
};

struct Work
{
    std::vector<double> Mp, RHS, DY, Ybuf, Y, rates;
    explicit Work(int dim, int nreact)
        : Mp((dim + 1) * (dim + 1)), RHS(dim + 1), DY(dim + 1), Ybuf(dim), Y(dim), rates(nreact)
    {
    }
};

// Newton acceptance, rejection and timestep control (nuclear_net.hpp:724-782).
// `nextT` is the caller's Newton temperature buffer, `dt` the step used, `timestep`
// receives the accepted step.
bool finalizeNR(int dim, const double* Y, double T, double* nextY, double& nextT, const double* DY, double& dt,
                double& timestep, int& i)
{
    const double last_T = nextT;
    for (int j = 0; j < dim; ++j)
        nextY[j] = Y[j] + DY[j + 1];
    nextT = T + DY[0];

    bool nan = std::isnan(nextT);
    for (int j = 0; j < dim && !nan; ++j)
        nan = std::isnan(nextY[j]);
    if (nan || nextT < 0)
    {
        dt *= kNanDtStep;
        i        = 0;
        timestep = 0.;
        return false;
    }
    const double dT_T = std::abs((nextT - T) / nextT);
    if (i >= kNRMinIt && dT_T > kNRDTTarget * kNRDTTol)
    {
        dt *= kNRDTTol / dT_T;
        i        = 0;
        timestep = 0.;
        for (int j = 0; j < dim; ++j)
            nextY[j] = Y[j];
        nextT = T;
        return false;
    }
    for (int j = 0; j < dim; ++j)
        if (nextY[j] <= kEpsilonVector) nextY[j] = 0;
    const double correction = std::abs((nextT - last_T) / nextT);
    if ((i >= kNRMinIt && correction < kNRItTol) || i >= kNRMaxIt)
    {
        const double dTT = std::abs((nextT - T) / nextT);
        timestep         = dt;
        dt               = (dTT == 0 ? kMaxDtStep : kNRDTTarget / dTT) * timestep;
        dt               = std::min(dt, timestep * kMaxDtStep);
        dt               = std::max(dt, timestep * kMinDtStep);
        dt               = std::min(dt, kNRMaxDt);
        return true;
    }
    timestep = 0.;
    return false;
}

// one burn; returns status.  Follows solveSystemSubstep (nuclear_net.hpp:931-959) with
// prepareSystemSubstep (:850-880) / prepareSystemNR (:692-717) inlined.
int burnOne(const Ctx& c, Work& w, double* Y, double& T, double rho, double drho_dt, double dt_tot, double& dt,
            long max_iter, int& nsub, long& nit)
{
    const int dim = c.dim;
    double        nextT = 0, elapsed = 0;
    double*       nextY = w.Ybuf.data();
    CycleDetector cd;
    cd.reset(dt, nextT);
    nsub = 0, nit = 0;
    for (int i = 1;; ++i)
    {
        if (nit >= max_iter) return ST_MAXITER;
        // prepareSystemSubstep
        const double rho_t = rho - drho_dt * (dt_tot - elapsed);
        double       used  = dt;
        if (dt_tot - elapsed < dt) used = dt_tot - elapsed;
        if (used == 0) return ST_ZERO_DT;
        ++nit;
        // prepareSystemNR: the guess temperature is a by-value copy in the reference
        double guessT = nextT;
        if (i <= 1)
        {
            for (int j = 0; j < dim; ++j)
                nextY[j] = Y[j];
            guessT = T;
        }
        const double T_theta = (1 - kTheta) * T + kTheta * guessT;
        for (int j = 0; j < dim; ++j)
            nextY[j] = (1 - kTheta) * Y[j] + kTheta * nextY[j];
        const Eos e = computeEos(c, nextY, T_theta, rho_t);
        prepareFromGuess(c, w.Mp.data(), w.RHS.data(), w.rates.data(), Y, T, nextY, T_theta, rho_t, drho_dt, e, used);
        denseSolve(w.Mp.data(), w.RHS.data(), w.DY.data(), dim + 1, kEpsilonSystem);

        // finalizeSystemSubstep (nuclear_net.hpp:887-922)
        double used_dt = dt, timestep;
        if (dt_tot - elapsed < dt) used_dt = dt_tot - elapsed;
        const bool conv = finalizeNR(dim, Y, T, nextY, nextT, w.DY.data(), used_dt, timestep, i);
        if (dt_tot - elapsed < dt)
        {
            if (used_dt < dt_tot - elapsed) dt = used_dt;
        }
        else
            dt = used_dt;
        if (conv)
        {
            for (int j = 0; j < dim; ++j)
                Y[j] = nextY[j];
            T = nextT;
            i = 0;
            elapsed += timestep;
            ++nsub;
            if ((dt_tot - elapsed) / dt_tot < kSubstepDtTol) return ST_OK;
            cd.reset(dt, nextT);
        }
        else if (i == 0 && cd.rejected(dt, nextT))
            return ST_LIVELOCK;
    }
}
} // namespace

extern "C"
{

int oracle_load_helmholtz(const double* tab)
{
    helm::load(tab);
    return 0;
}

int oracle_helmholtz(double abar_, double zbar_, double T, double rho, double* out)
{
    Eos    r    = helm::eos(abar_, zbar_, T, rho);
    double v[13] = {r.cv, r.dpdT, r.p, r.cp, r.c, r.u, r.dse, r.dpe, r.dsp, r.cv_gaz, r.cp_gaz, r.c_gaz, r.dudYe};
    std::memcpy(out, v, sizeof v);
    return 0;
}

int oracle_rates(int net, const double* Y, double T, double rho, int eos_kind, double mu, double* BE, double* rates,
                 double* drates, double* eos_out)
{
    Ctx c{net, 0, eos_kind, mu, {}};
    if (!getNetwork(net, c.n)) return -1;
    c.dim     = c.n.nspec;
    const Eos e = computeEos(c, Y, T, rho);
    networkRates(net, Y, T, rho, BE, rates, drates);
    if (eos_out)
    {
        double v[13] = {e.cv, e.dpdT, e.p, e.cp, e.c, e.u, e.dse, e.dpe, e.dsp, e.cv_gaz, e.cp_gaz, e.c_gaz, e.dudYe};
        std::memcpy(eos_out, v, sizeof v);
    }
    return 0;
}

// Batch burn (parallel_nuclear_net_impl.cpp:63-103), Y species-major Y[j*P+i]; see
// ref_burn in ref_driver.cpp for the argument meaning.
int oracle_burn(int net, int eos_kind, double mu, size_t P, double* Y, double* T, const double* rho,
                const double* rho_m1, double* dt, double hydro_dt, double previous_dt, int drhodt_mode, long max_iter,
                int* status, int* substeps, int* iters, int nthreads)
{
    Ctx c{net, 0, eos_kind, mu, {}};
    if (!getNetwork(net, c.n)) return -1;
    c.dim = c.n.nspec;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    // scheduling batch of parallel_nuclear_net_impl.cpp:79 (nnet_util/algorithm.hpp:79-88)
    int batch;
    {
        const float phi = 1.61803398875;
        int         f   = (int)std::floor(std::log2((float)P / (float)nthreads) / phi);
        int         pw  = 1 << std::max(f, 0);
        batch           = std::max(1, (int)std::floor((float)P / ((float)pw * 2.0 * (float)nthreads)));
    }
#pragma omp parallel num_threads(nthreads)
    {
        Work w(c.dim, c.n.nreact);
#pragma omp for schedule(dynamic, batch)
        for (size_t p = 0; p < P; ++p)
        {
            int  st = ST_SKIPPED, nsub = 0;
            long nit = 0;
            if (rho[p] > kMinRho && T[p] > kMinTemp)
            {
                for (int j = 0; j < c.dim; ++j)
                    w.Y[j] = Y[(size_t)j * P + p];
                double drho_dt = 0;
                if (drhodt_mode == 1 && rho_m1 && rho_m1[p] != 0) drho_dt = (rho[p] - rho_m1[p]) / previous_dt;
                double Tp = T[p], dtp = dt[p];
                st        = burnOne(c, w, w.Y.data(), Tp, rho[p], drho_dt, hydro_dt, dtp, max_iter, nsub, nit);
                for (int j = 0; j < c.dim; ++j)
                    Y[(size_t)j * P + p] = w.Y[j];
                T[p] = Tp, dt[p] = dtp;
            }
            if (status) status[p] = st;
            if (substeps) substeps[p] = nsub;
            if (iters) iters[p] = (int)nit;
        }
    }
    return 0;
}

// Post-burn EOS over a batch (parallel_nuclear_net_impl.cpp:116-141): u, cv, p, c, dpdT
int oracle_helm_eos_batch(size_t P, int dim, const double* Z, const double* T, const double* rho, const double* Y,
                          double* u, double* cv, double* p, double* c, double* dpdT, int nthreads)
{
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (size_t i = 0; i < P; ++i)
    {
        double abar = 0, zbar = 0;
        for (int j = 0; j < dim; ++j)
            abar = abar + Y[(size_t)j * P + i];
        for (int j = 0; j < dim; ++j)
            zbar += Y[(size_t)j * P + i] * Z[j];
        Eos e   = helm::eos(abar, zbar, T[i], rho[i]);
        u[i]    = e.u;
        cv[i]   = e.cv;
        p[i]    = e.p;
        c[i]    = e.c;
        dpdT[i] = e.dpdT;
    }
    return 0;
}

// The Newton system of the first iteration of a substep from state (Y, T) with step dt, as
// M (column-major: M[i + (N+1) j] is element (i, j); index 0 = temperature) and RHS;
// for analysis of the linear solves.
int oracle_newton_system(int net, int eos_kind, double mu, const double* Y, double T, double rho, double drho_dt,
                         double dt, double* M, double* RHS)
{
    Ctx c{net, 0, eos_kind, mu, {}};
    if (!getNetwork(net, c.n)) return -1;
    c.dim = c.n.nspec;
    Work               w(c.dim, c.n.nreact);
    std::vector<double> Yg(Y, Y + c.dim);
    const Eos          e = computeEos(c, Yg.data(), T, rho);
    prepareFromGuess(c, w.Mp.data(), w.RHS.data(), w.rates.data(), Y, T, Yg.data(), T, rho, drho_dt, e, dt);
    const int ld = c.dim + 1;
    for (int i = 0; i < ld * ld; ++i)
        M[i] = w.Mp[i];
    for (int i = 0; i < ld; ++i)
        RHS[i] = w.RHS[i];
    return 0;
}

// Single-particle Newton solve without substepping (nuclear_net.hpp:791-818)
double oracle_solve_nr(int net, int eos_kind, double mu, const double* Y, double T, double* Y_out, double* T_out,
                       double rho, double drho_dt, double* dt)
{
    Ctx c{net, 0, eos_kind, mu, {}};
    if (!getNetwork(net, c.n)) return -1;
    c.dim = c.n.nspec;
    if (rho < kMinRho || T < kMinTemp)
    {
        *dt = kNRMaxDt;
        return *dt;
    }
    Work    w(c.dim, c.n.nreact);
    double  timestep = 0, nextT = T;
    double* nextY = Y_out;
    for (int i = 1;; ++i)
    {
        double guessT = nextT;
        if (i <= 1)
        {
            for (int j = 0; j < c.dim; ++j)
                nextY[j] = Y[j];
            guessT = T;
        }
        const double T_theta = (1 - kTheta) * T + kTheta * guessT;
        for (int j = 0; j < c.dim; ++j)
            nextY[j] = (1 - kTheta) * Y[j] + kTheta * nextY[j];
        const Eos e = computeEos(c, nextY, T_theta, rho);
        prepareFromGuess(c, w.Mp.data(), w.RHS.data(), w.rates.data(), Y, T, nextY, T_theta, rho, drho_dt, e, *dt);
        denseSolve(w.Mp.data(), w.RHS.data(), w.DY.data(), c.dim + 1, kEpsilonSystem);
        if (finalizeNR(c.dim, Y, T, nextY, nextT, w.DY.data(), *dt, timestep, i))
        {
            *T_out = nextT;
            return timestep;
        }
    }
}
}
