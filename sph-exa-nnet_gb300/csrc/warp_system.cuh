// Shared pieces of the kernels in which a warp cooperates on one particle's Newton system
// held in shared memory: the per-warp layout, warp reductions, assembly of the system from
// per-reaction rates, and the level-scheduled sparse LU solves (FP64 and mixed precision).
#pragma once

#include "burn_policies.cuh"
#include "sparse_plan.hpp"

namespace nnet_gb300
{
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double warpSum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// at most this many long (warp-split) lists per gather kind; checked when a network is uploaded
constexpr int kMaxHeavy = 8;

// warpSum of v[0..n) with the butterflies of the different sums interleaved (same order of
// additions per sum as warpSum)
__device__ __forceinline__ void warpSumMany(double (&v)[kMaxHeavy], int n)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int h = 0; h < kMaxHeavy; ++h)
            if (h < n) v[h] += __shfl_xor_sync(kFull, v[h], o);
}

template<int NET>
struct WDims
{
    static constexpr int N   = NET, n = NET + 1;
    static constexpr int R   = NetDims<NET>::R;
    static constexpr int NE  = NET == 14 ? 42 : NET == 86 ? 482 : 486; // reactant entries
    static constexpr int NNZ = NET == 14 ? kWarpNnzCap14 : kWarpNnzCap86; // factor capacity (checked on host)
};

// Shared-memory layout of one warp (doubles).  Only what the assembly and the solve need at
// the same time has its own storage: abundances, fluxes and their temperature derivatives,
// the factor (the right-hand side right after it), and the Jacobian bases `tr`.  The
// screening potentials and binding energies of the rate evaluation live at the start of the
// `tr` region (the temperature row takes the binding energies before the fluxes overwrite
// it); dY/dt, d(dY/dt)/dT and J (Yn - Y) go straight into the right-hand side and the
// temperature column as they are gathered; the float factor of the mixed form overlaps `tr`,
// consumed before the solve; the solve vectors reuse the flux storage.  The smaller the
// system, the more warps an SM holds, and this latency-bound kernel runs faster with each.
template<int NET, bool MIXED>
struct WarpSmem
{
    using D = WDims<NET>;
    static constexpr int kFlux = 2 * D::R > 4 * D::n ? 2 * D::R : 4 * D::n; // f, df; x, r, ipiv, scale
    static constexpr int oY = 0, oYn = oY + D::N, oF = oYn + D::N, oDF = oF + D::R, oA = oF + kFlux,
                         oB = oA + D::NNZ, oTr = oB + D::n;
    static constexpr int floatsD = (D::NNZ + 3 * D::n + 1) / 2;
    static constexpr int trD     = D::NE > 2 * D::N ? D::NE : 2 * D::N; // tr; mu and BE before it
    static constexpr int doubles = oTr + (MIXED && floatsD > trD ? floatsD : trD);

    double *Y, *Yn, *f, *df, *BE, *A, *b, *mu, *tr, *x, *r, *ipiv, *scale;
    float * LU, *d, *ipiv32, *x32;

    __device__ explicit WarpSmem(double* s)
    {
        Y = s + oY, Yn = s + oYn, f = s + oF, df = s + oDF, A = s + oA, b = s + oB, tr = s + oTr;
        mu = tr, BE = tr + D::N; // rate evaluation only: dead once the fluxes are formed
        x = f, r = f + D::n, ipiv = f + 2 * D::n, scale = f + 3 * D::n;
        LU = reinterpret_cast<float*>(tr), d = LU + D::NNZ, ipiv32 = d + D::n, x32 = ipiv32 + D::n;
    }
};

// ------------------------------------------------------------------ assembly (warp)
template<int NET, bool MIXED>
__device__ void warpAssemble(const NetView& nv, WarpSmem<NET, MIXED>& S, double T, double Tg, double rho,
                             double drho_dt, double cv, double dpdT, double dt, int lane)
{
    // one reciprocal each instead of a division per reaction / species (the quotients
    // differ from the reference's by at most one rounding)
    const double rinv = 1. / rho, cvinv = 1. / cv;
    using D                = WDims<NET>;
    const SparseView& sp   = nv.sp;
    const WarpView&   wv   = nv.wv;
    const double      mtd  = -k::theta * dt;
    // the factor starts from zero; the temperature row takes -BE / cv (prepareSystemFromGuess,
    // nuclear_net.hpp:553-556) while the binding energies are still in the `tr` region
    for (int p = lane; p < sp.nnz; p += 32)
        S.A[p] = 0.;
    __syncwarp();
    for (int i = lane; i < D::N; i += 32)
        S.A[__ldg(sp.row0Pos + i)] = -S.BE[i] * cvinv;
    __syncwarp();
    // per-reaction fluxes (dY/dt terms, nuclear_net.hpp:347-381) and Jacobian bases
    // (:395-438), in place of the rates
    for (int q = lane; q < D::R; q += 32)
    {
        const int rb = __ldg(nv.rbeg + q), re = __ldg(nv.rbeg + q + 1);
        double    f = S.f[q], df = S.df[q], base = f;
        for (int k = rb; k < re; ++k)
        {
            const int    cnt = __ldg(nv.rcnt + k);
            const double yr  = S.Yn[__ldg(nv.rspec + k)] * rho;
            if (cnt == 2)
                f *= 0.5, df *= 0.5, base *= 0.5; // exact: the same value as a division by 2
            else if (cnt != 1)
                f /= 6., df /= 6., base /= 6.;
            const double pw = ipowS(yr, cnt);
            f *= pw, df *= pw, base *= ipowS(yr, cnt - 1);
        }
        S.f[q] = f * rinv, S.df[q] = df * rinv;
        for (int k = rb; k < re; ++k)
        {
            const int id = __ldg(nv.rspec + k);
            double    tr = base;
            for (int o = rb; o < re; ++o)
            {
                const int os = __ldg(nv.rspec + o);
                if (os != id) tr *= S.Yn[os] * rho;
            }
            S.tr[k] = base > k::epsilonSystem ? tr : 0.;
        }
    }
    __syncwarp();
    // dY/dt and d(dY/dt)/dT per species, straight into the right-hand side (dt dY/dt - theta dt
    // (Tg - T) d(dY/dt)/dT; the J (Yn - Y) term follows below) and the temperature column
    // (nuclear_net.hpp:559-579)
    auto rowT = [&](int s, double dydt, double c0) {
        double rh = dydt * dt;
        rh        = rh + mtd * c0 * (Tg - T);
        S.b[__ldg(sp.iperm + s + 1)] = rh;
        S.A[__ldg(sp.col0Pos + s)]   = c0 * mtd;
    };
    for (int t = lane; t < D::N; t += 32)
    {
        const int s = __ldg(wv.sgOrder + t), b0 = __ldg(wv.sgBeg + s), b1 = __ldg(wv.sgBeg + s + 1);
        if (b1 - b0 > WarpPlan::kHeavy) continue;
        double a = 0, c = 0;
        // unrolled gathers (here and below) issue the index and value loads of four entries
        // before their products are summed, in the same order: latency hidden, same bits
#pragma unroll 4
        for (int k = b0; k < b1; ++k)
        {
            const double w = __ldg(wv.sgCoef + k);
            const int    r = __ldg(wv.sgRx + k);
            a += w * S.f[r], c += w * S.df[r];
        }
        rowT(s, a, c);
    }
    {
        // the long lists: partial sums of all of them first, then their butterflies interleaved
        double ha[kMaxHeavy], hc[kMaxHeavy];
#pragma unroll
        for (int h = 0; h < kMaxHeavy; ++h)
        {
            ha[h] = 0, hc[h] = 0;
            if (h >= wv.nSgHeavy) continue;
            const int s = __ldg(wv.sgHeavy + h), b0 = __ldg(wv.sgBeg + s), b1 = __ldg(wv.sgBeg + s + 1);
            for (int k = b0 + lane; k < b1; k += 32)
            {
                const double w = __ldg(wv.sgCoef + k);
                const int    r = __ldg(wv.sgRx + k);
                ha[h] += w * S.f[r], hc[h] += w * S.df[r];
            }
        }
        warpSumMany(ha, wv.nSgHeavy), warpSumMany(hc, wv.nSgHeavy);
        if (lane == 0)
#pragma unroll
            for (int h = 0; h < kMaxHeavy; ++h)
                if (h < wv.nSgHeavy) rowT(__ldg(wv.sgHeavy + h), ha[h], hc[h]);
    }
    // Jacobian entries
    for (int m = lane; m < wv.nJ; m += 32)
    {
        const int b0 = __ldg(wv.jgBeg + m), b1 = __ldg(wv.jgBeg + m + 1);
        if (b1 - b0 > WarpPlan::kHeavy) continue;
        double a = 0;
#pragma unroll 4
        for (int k = b0; k < b1; ++k)
            a += __ldg(wv.jgCoef + k) * S.tr[__ldg(wv.jgEnt + k)];
        S.A[__ldg(wv.jPos + m)] = a;
    }
    {
        double ha[kMaxHeavy];
#pragma unroll
        for (int h = 0; h < kMaxHeavy; ++h)
        {
            ha[h] = 0;
            if (h >= wv.nJgHeavy) continue;
            const int m = __ldg(wv.jgHeavy + h), b0 = __ldg(wv.jgBeg + m), b1 = __ldg(wv.jgBeg + m + 1);
            for (int k = b0 + lane; k < b1; k += 32)
                ha[h] += __ldg(wv.jgCoef + k) * S.tr[__ldg(wv.jgEnt + k)];
        }
        warpSumMany(ha, wv.nJgHeavy);
        if (lane == 0)
#pragma unroll
            for (int h = 0; h < kMaxHeavy; ++h)
                if (h < wv.nJgHeavy) S.A[__ldg(wv.jPos + __ldg(wv.jgHeavy + h))] = ha[h];
    }
    __syncwarp();
    // J (Yg - Y) per species row, added to the right-hand side (nuclear_net.hpp:580-589)
    auto addJdy = [&](int i, double jdy) {
        double& rh = S.b[__ldg(sp.iperm + i + 1)];
        rh         = rh + mtd * jdy;
    };
    for (int t = lane; t < D::N; t += 32)
    {
        const int i = __ldg(wv.rjOrder + t), b0 = __ldg(wv.rjBeg + i), b1 = __ldg(wv.rjBeg + i + 1);
        if (b1 - b0 > WarpPlan::kHeavy) continue;
        double a = 0;
#pragma unroll 4
        for (int k = b0; k < b1; ++k)
        {
            const int m = __ldg(wv.rjEnt + k), j = __ldg(wv.jCol + m);
            a += S.A[__ldg(wv.jPos + m)] * (S.Yn[j] - S.Y[j]);
        }
        addJdy(i, a);
    }
    {
        double ha[kMaxHeavy];
#pragma unroll
        for (int h = 0; h < kMaxHeavy; ++h)
        {
            ha[h] = 0;
            if (h >= wv.nRjHeavy) continue;
            const int i = __ldg(wv.rjHeavy + h), b0 = __ldg(wv.rjBeg + i), b1 = __ldg(wv.rjBeg + i + 1);
            for (int k = b0 + lane; k < b1; k += 32)
            {
                const int m = __ldg(wv.rjEnt + k), j = __ldg(wv.jCol + m);
                ha[h] += S.A[__ldg(wv.jPos + m)] * (S.Yn[j] - S.Y[j]);
            }
        }
        warpSumMany(ha, wv.nRjHeavy);
        if (lane == 0)
#pragma unroll
            for (int h = 0; h < kMaxHeavy; ++h)
                if (h < wv.nRjHeavy) addJdy(__ldg(wv.rjHeavy + h), ha[h]);
    }
    __syncwarp();
    // I - theta dt J and the temperature entries (:590-608)
    for (int e = lane; e < sp.nsb; e += 32)
    {
        const int p = __ldg(sp.sbPos + e);
        S.A[p]      = __ldg(sp.sbDiag + e) ? 1. - k::theta * dt * S.A[p] : mtd * S.A[p];
    }
    if (lane == 0)
    {
        const double drho = drho_dt * dt, value1 = dpdT * drho / (rho * rho);
        S.b[sp.tNew]  = T * value1 / cv;
        S.A[sp.pos00] = 1 - k::theta * value1 / cv;
    }
    __syncwarp();
}

// ------------------------------------------------------------------ solves (warp)
// pivot reciprocals, rounded to nearest
__device__ __forceinline__ double recip(double a) { return __drcp_rn(a); }
__device__ __forceinline__ float  recip(float a) { return __frcp_rn(a); }

// Level-scheduled right-looking LU without pivoting, in place (FP64 or FP32).  Per level:
// the multipliers (each lane forms its pivot's reciprocal itself, so no separate round is
// needed), then every target's updates in pivot order.  AUG: the right-hand side, stored
// right after the factor's rhsBase entries, is a column of the matrix, so the forward
// substitution happens in the same rounds; the updates then run as per-lane op streams
// (WarpPlan::fOps), the other form as rounds of 32 targets.
template<typename F, bool AUG>
__device__ void levelFactor(const SparseView& sp, const WarpView& wv, F* A, F* ipiv, int lane)
{
    const int* tgBeg = AUG ? wv.tgBegA : wv.tgBeg;
    const int* tgPos = AUG ? wv.tgPosA : wv.tgPos;
    const int* tgUpd = AUG ? wv.tgUpdA : wv.tgUpd;
    const int* tuL   = AUG ? wv.tuLA : wv.tuL;
    const int* tuU   = AUG ? wv.tuUA : wv.tuU;
    for (int l = 0; l < wv.nLevels; ++l)
    {
        for (int e = __ldg(wv.scBeg + l) + lane; e < __ldg(wv.scBeg + l + 1); e += 32)
        {
            const int k = __ldg(wv.scPiv + e), pos = __ldg(wv.scPos + e);
            const F   ip = recip(A[__ldg(sp.kPiv + k)]);
            if (pos >= 0) A[pos] *= ip;
            ipiv[k] = ip; // lanes of one pivot write the same value
        }
        __syncwarp();
        if constexpr (AUG)
        {
            // the level's updates as this lane's op stream (WarpPlan::fOps): the same products
            // per target in the same order as the target lists below, packed onto the lanes
            const int                 r0 = __ldg(wv.foBeg + l), nr = __ldg(wv.foBeg + l + 1) - r0;
            const unsigned long long* op = wv.fOps + (size_t)r0 * 32 + lane;
            F                         a  = 0;
#pragma unroll 4
            for (int k = 0; k < nr; ++k)
            {
                const unsigned long long o = __ldg(op + (size_t)k * 32);
                if (o & WarpPlan::kOpValid)
                {
                    const int pos = (int)(o >> 32) & 0xffff;
                    if (o & WarpPlan::kOpFirst) a = A[pos];
                    a = a - A[(int)o & 0xffff] * A[(int)(o >> 16) & 0xffff];
                    if (o & WarpPlan::kOpLast) A[pos] = a;
                }
            }
        }
        else
            for (int t = __ldg(tgBeg + l) + lane; t < __ldg(tgBeg + l + 1); t += 32)
            {
                const int pos = __ldg(tgPos + t);
                F         a   = A[pos];
#pragma unroll 4
                for (int u = __ldg(tgUpd + t), ue = __ldg(tgUpd + t + 1); u < ue; ++u)
                    a = a - A[__ldg(tuL + u)] * A[__ldg(tuU + u)];
                A[pos] = a;
            }
        __syncwarp();
    }
}

// y <- L^-1 y with the factor of levelFactor (unit lower triangle)
template<typename F>
__device__ void levelForward(const WarpView& wv, const F* A, F* y, int lane)
{
    for (int l = 0; l < wv.nLevels; ++l)
    {
        for (int r = __ldg(wv.fwBeg + l) + lane; r < __ldg(wv.fwBeg + l + 1); r += 32)
        {
            const int row = __ldg(wv.fwRow + r);
            F         a   = y[row];
#pragma unroll 4
            for (int e = __ldg(wv.fwEnt + r), ee = __ldg(wv.fwEnt + r + 1); e < ee; ++e)
                a = a - A[__ldg(wv.flPos + e)] * y[__ldg(wv.flK + e)];
            y[row] = a;
        }
        __syncwarp();
    }
}

// x <- U^-1 y (y is consumed): one round per level, last level first; each lane either
// finishes one of the level's pivots (x_k = y_k / u_kk) or updates one row above them
// with the same products.
template<typename F>
__device__ void levelBackward(const WarpView& wv, const F* A, const F* ipiv, F* y, F* x, int lane)
{
    for (int li = 0; li < wv.nLevels; ++li)
    {
        const int l = wv.nLevels - 1 - li;
        const int p0 = __ldg(wv.lvBeg + l), nP = __ldg(wv.lvBeg + l + 1) - p0;
        const int r0 = __ldg(wv.bwBeg + li), nR = __ldg(wv.bwBeg + li + 1) - r0;
        for (int t = lane; t < nP + nR; t += 32)
        {
            if (t < nP)
            {
                const int k = __ldg(wv.lvPiv + p0 + t);
                x[k]        = y[k] * ipiv[k];
            }
            else
            {
                const int r = r0 + t - nP, row = __ldg(wv.bwRow + r);
                F         a = y[row];
#pragma unroll 4
                for (int e = __ldg(wv.bwEnt + r), ee = __ldg(wv.bwEnt + r + 1); e < ee; ++e)
                {
                    const int k = __ldg(wv.buK + e);
                    a           = a - A[__ldg(wv.buPos + e)] * (y[k] * ipiv[k]);
                }
                y[row] = a;
            }
        }
        __syncwarp();
    }
}

// FP64: factor A in place with b as an extra column, then x = U^-1 (L^-1 b); b is consumed
template<int NET, bool MIXED>
__device__ void warpSolve64(const NetView& nv, WarpSmem<NET, MIXED>& S, int lane)
{
    levelFactor<double, true>(nv.sp, nv.wv, S.A, S.ipiv, lane);
    levelBackward<double>(nv.wv, S.A, S.ipiv, S.b, S.x, lane);
}

// rows scaled by powers of two, FP32 factorisation, FP64 residual refinement; returns
// the refinement steps, or -1 if the corrections did not settle (caller re-solves in FP64)
template<int NET>
__device__ int warpSolveMixed(const NetView& nv, WarpSmem<NET, true>& S, double T, int lane, double* scale)
{
    using D              = WDims<NET>;
    const SparseView& sp = nv.sp;
    const WarpView&   wv = nv.wv;
    // row scales from the exponent bits (integer work), then the FP32 copy
    for (int i = lane; i < D::n; i += 32)
    {
        int e = 0;
        for (int p = __ldg(sp.rowBeg + i), pe = __ldg(sp.rowBeg + i + 1); p < pe; ++p)
            e = max(e, (int)((__double_as_longlong(S.A[p]) >> 52) & 0x7ff));
        scale[i] = e == 0 ? 1. : ldexp(1., 1023 - e); // 2^-ilogb(max |a_ij|)
    }
    __syncwarp();
    for (int p = lane; p < sp.nnz; p += 32)
        S.LU[p] = (float)(S.A[p] * scale[__ldg(sp.posRow + p)]);
    __syncwarp();
    levelFactor<float, false>(sp, wv, S.LU, S.ipiv32, lane);
    for (int i = lane; i < D::n; i += 32)
        S.x[i] = 0., S.r[i] = S.b[i];
    __syncwarp();
    for (int steps = 0;; ++steps)
    {
        for (int i = lane; i < D::n; i += 32)
            S.d[i] = (float)(S.r[i] * scale[i]);
        __syncwarp();
        levelForward<float>(wv, S.LU, S.d, lane);
        levelBackward<float>(wv, S.LU, S.ipiv32, S.d, S.x32, lane);
        bool conv = true;
        for (int i = lane; i < D::n; i += 32)
        {
            const double di = (double)S.x32[i], xi = S.x[i] + di;
            const int    o  = __ldg(sp.perm + i);
            const double sc = o == 0 ? T : fabs(S.Y[o - 1]);
            conv &= fabs(di) <= kRefineTol * (fabs(xi) + sc) && isfinite(xi); // an FP32 overflow is not convergence
            S.x[i] = xi;
        }
        conv = __all_sync(kFull, conv);
        __syncwarp();
        if (conv) return steps;
        if (steps == kMaxRefine) return -1;
        // r = b - A x (FP64, rows over lanes; the long rows split across the warp)
        for (int i = lane; i < D::n; i += 32)
        {
            const int p0 = __ldg(sp.rowBeg + i), p1 = __ldg(sp.rowBeg + i + 1);
            if (p1 - p0 > WarpPlan::kHeavy) continue;
            double s = S.b[i];
            for (int p = p0; p < p1; ++p)
                s -= S.A[p] * S.x[__ldg(sp.posCol + p)];
            S.r[i] = s;
        }
        for (int h = 0; h < wv.nRowHeavy; ++h)
        {
            const int i = __ldg(wv.rowHeavy + h), p0 = __ldg(sp.rowBeg + i), p1 = __ldg(sp.rowBeg + i + 1);
            double    s = 0;
            for (int p = p0 + lane; p < p1; p += 32)
                s += S.A[p] * S.x[__ldg(sp.posCol + p)];
            s = warpSum(s);
            if (lane == 0) S.r[i] = S.b[i] - s;
        }
        __syncwarp();
    }
}

} // namespace nnet_gb300
