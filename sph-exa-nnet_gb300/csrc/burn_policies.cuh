// Solver policies of the burn kernels: per-slot scratch views plus `assembleSolve`, which
// builds the Newton system of prepareSystemFromGuess (include/nnet/nuclear_net.hpp:514-609)
// around the guess and solves it.
//
// Plain FP64 form of the burn: the Newton system is assembled densely and solved by
// Gaussian elimination without pivoting, in the reference's operation order
// (include/nnet/nuclear_net.hpp:347-438 and :514-609, include/nnet_util/eigen.hpp:178-223).
// One thread per particle; the (N+1)^2 matrix and the vectors live in per-slot scratch,
// interleaved across slots so that every access of a warp is one coalesced 256-byte line.
//
// Sparse forms of the burn.  The Newton system of prepareSystemFromGuess
// (include/nnet/nuclear_net.hpp:514-609) is assembled directly into the fill pattern of a
// minimum-degree ordering (sparse_plan.hpp) and solved with a right-looking LU without
// pivoting, executed as a flat operation list that is identical for every particle of a
// network (warp-uniform, coalesced per-slot scratch).
//
//  NNET_SOLVER_SPARSE_FP64: factorisation and triangular solves in FP64.
//  NNET_SOLVER_MIXED:       rows scaled by powers of two, factorisation and correction
//                           solves in FP32, residual r = b - A x and update in FP64,
//                           up to kMaxRefine refinement steps; a system whose correction
//                           has not converged componentwise is re-solved in FP64.
// Rates, EOS, assembly, the Newton test and the timestep control stay FP64.
#pragma once

#include "driver.cuh"
#include "physics_fast.cuh"

namespace nnet_gb300
{


// x^cnt and the stoichiometric factorial of the reference's reaction terms
// (pow(Y rho, n) / tgamma(n + 1), nuclear_net.hpp:364-367)
__device__ __forceinline__ double ipow(double x, int cnt)
{
    if (cnt == 0) return 1.;
    if (cnt == 1) return x;
    if (cnt == 2) return x * x;
    // correctly-rounded-ish cube: x^2 = hi + lo exactly, then (hi + lo) x
    const double hi = x * x, lo = fma(x, x, -hi);
    return fma(hi, x, lo * x);
}
__device__ __forceinline__ double factorial(int cnt) { return cnt == 2 ? 2. : 6.; }

template<int NET>
struct DensePolicy
{
    using D = NetDims<NET>;
    Strided<double> M, RHS, DY, Y, Yn, rates;

    static constexpr size_t perSlot() { return (size_t)D::n * D::n + 2 * D::n + 2 * D::N + D::R; }

    __device__ DensePolicy(double* scratch, size_t stride, size_t slot)
    {
        M     = {scratch + slot, stride};
        RHS   = M.at(D::n * D::n);
        DY    = RHS.at(D::n);
        Y     = DY.at(D::n);
        Yn    = Y.at(D::N);
        rates = Yn.at(D::N);
    }

    // dY/dt from the reaction list (nuclear_net.hpp:347-381)
    __device__ void derivatives(const NetView& nv, Strided<double> r, double rho, Strided<double> dY)
    {
        for (int i = 0; i < D::N; ++i)
            dY[i] = 0.;
        for (int q = 0; q < D::R; ++q)
        {
            double    rate = r[q];
            const int rb = __ldg(nv.rbeg + q), re = __ldg(nv.rbeg + q + 1);
            for (int k = rb; k < re; ++k)
            {
                const int cnt = __ldg(nv.rcnt + k);
                if (cnt != 1) rate /= factorial(cnt);
                rate *= ipow(Yn[__ldg(nv.rspec + k)] * rho, cnt);
            }
            rate /= rho;
            for (int k = rb; k < re; ++k)
            {
                const int s = __ldg(nv.rspec + k);
                dY[s]       = dY[s] - rate * __ldg(nv.rcnt + k);
            }
            const int pb = __ldg(nv.pbeg + q), pe = __ldg(nv.pbeg + q + 1);
            for (int k = pb; k < pe; ++k)
            {
                const int s = __ldg(nv.pspec + k);
                dY[s]       = dY[s] + rate * __ldg(nv.pcnt + k);
            }
        }
    }

    // species-block Jacobian (nuclear_net.hpp:395-438)
    __device__ void jacobian(const NetView& nv, double rho)
    {
        constexpr int n = D::n;
        for (int j = 0; j < D::N; ++j)
            for (int i = 0; i < D::N; ++i)
                M[(i + 1) + n * (j + 1)] = 0.;
        for (int q = 0; q < D::R; ++q)
        {
            double    rate = rates[q];
            const int rb = __ldg(nv.rbeg + q), re = __ldg(nv.rbeg + q + 1);
            for (int k = rb; k < re; ++k)
            {
                const int cnt = __ldg(nv.rcnt + k);
                if (cnt != 1) rate /= factorial(cnt);
                rate *= ipow(Yn[__ldg(nv.rspec + k)] * rho, cnt - 1);
            }
            if (rate > k::epsilonSystem)
            {
                const int pb = __ldg(nv.pbeg + q), pe = __ldg(nv.pbeg + q + 1);
                for (int k = rb; k < re; ++k)
                {
                    const int id = __ldg(nv.rspec + k);
                    double    tr = rate;
                    for (int o = rb; o < re; ++o)
                    {
                        const int os = __ldg(nv.rspec + o);
                        if (os != id) tr *= Yn[os] * rho;
                    }
                    for (int o = rb; o < re; ++o)
                    {
                        const int idx = (__ldg(nv.rspec + o) + 1) + n * (id + 1);
                        M[idx]        = M[idx] - tr * __ldg(nv.rcnt + o);
                    }
                    for (int o = pb; o < pe; ++o)
                    {
                        const int idx = (__ldg(nv.pspec + o) + 1) + n * (id + 1);
                        M[idx]        = M[idx] + tr * __ldg(nv.pcnt + o);
                    }
                }
            }
        }
    }

    // prepareSystemFromGuess (nuclear_net.hpp:514-609) then eigen::solve
    __device__ void assembleSolve(const NetView& nv, double T, double Tg, double rho, double drho_dt, double cv,
                                  double dpdT, double dt)
    {
        constexpr int n = D::n, N = D::N;
        Strided<double> BE = RHS.at(1), drT = M.at(N + 1);
        networkRates<NET>(nv, Yn, Tg, rho, BE, rates, drT);
        derivatives(nv, drT, rho, M.at(1));
        for (int i = 0; i < N; ++i)
            M[0 + n * (i + 1)] = -BE[i] / cv;
        derivatives(nv, rates, rho, RHS.at(1));
        for (int i = 0; i < N; ++i)
            RHS[i + 1] = RHS[i + 1] * dt;
        for (int i = 0; i < N; ++i)
        {
            const double m = M[i + 1];
            RHS[i + 1]     = RHS[i + 1] + -k::theta * dt * m * (Tg - T);
            M[i + 1]       = m * (-k::theta * dt);
        }
        jacobian(nv, rho);
        for (int i = 0; i < N; ++i)
        {
            double corr = 0;
            for (int j = 0; j < N; ++j)
                corr += M[(i + 1) + n * (j + 1)] * (Yn[j] - Y[j]);
            RHS[i + 1] = RHS[i + 1] + -k::theta * dt * corr;
        }
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i)
            {
                const int idx = (i + 1) + n * (j + 1);
                M[idx]        = i == j ? 1. - k::theta * dt * M[idx] : -k::theta * dt * M[idx];
            }
        const double drho = drho_dt * dt, value1 = dpdT * drho / (rho * rho);
        RHS[0] = T * value1 / cv;
        M[0]   = 1 - k::theta * value1 / cv;

        // Gaussian elimination without pivoting, zero multipliers skipped (eigen.hpp:178-223)
        for (int i = 0; i < n; ++i)
        {
            for (int j = 0; j < i; ++j)
            {
                const double w = M[i + n * j];
                M[i + n * j]   = 0;
                if (fabs(w) > k::epsilonSystem)
                {
                    RHS[i] = RHS[i] - w * RHS[j];
                    for (int c = j + 1; c < n; ++c)
                        M[i + n * c] = M[i + n * c] - w * M[j + n * c];
                }
            }
            const double diag = M[i + n * i];
            M[i + n * i]      = 1;
            RHS[i]            = RHS[i] / diag;
            for (int c = i + 1; c < n; ++c)
                M[i + n * c] = M[i + n * c] / diag;
        }
        for (int i = n - 1; i >= 0; --i)
        {
            double res = RHS[i];
            for (int c = i + 1; c < n; ++c)
                res -= M[i + n * c] * DY[c];
            DY[i] = res;
        }
    }

    __device__ __forceinline__ double dy(const SparseView&, int i) const { return DY[i]; }
};



constexpr int    kMaxRefine = 3;
// refinement ends when every correction is below kRefineTol of the component plus the
// state it updates (|Y_j| for a species row, T for the temperature row), i.e. at FP64
// rounding level of the quantities the Newton iteration produces
constexpr double kRefineTol = 8.881784197001252e-16; // 2^-50

__device__ __forceinline__ double ipowS(double x, int cnt)
{
    if (cnt == 0) return 1.;
    if (cnt == 1) return x;
    if (cnt == 2) return x * x;
    const double hi = x * x, lo = fma(x, x, -hi);
    return fma(hi, x, lo * x);
}

template<int NET, bool MIXED>
struct SparsePolicy
{
    using D = NetDims<NET>;
    static constexpr int MAXNNZ = NET == 14 ? 128 : 1100; // checked against the plan on the host
    Strided<double> A, b, x, r, Y, Yn, rates, drates, BE, dYdt, dYdT, jdy, ipiv, scale;
    Strided<float>  LU, d32;

    // per-slot doubles: the FP64 vectors, then (mixed form) the FP32 factor and correction
    static constexpr size_t doubleElems() { return (size_t)MAXNNZ + 5 * D::n + 2 * D::N + 2 * D::R + 4 * D::N; }
    static constexpr size_t floatElems() { return MIXED ? (MAXNNZ + D::n + 1) / 2 + 1 : 0; }
    static constexpr size_t perSlot() { return doubleElems() + floatElems(); }

    // floatBase: element index (in doubles) where the FP32 region of every slot starts.  The
    // FP32 rows interleave across slots at half the FP64 row width, so row e of slot s lands in
    // the FP64 row floatBase + (e * stride + s) / (2 * stride): another slot's column.  Every
    // slot of a launch must therefore use the same floatBase, at or above the FP64 rows of every
    // network that any slot of the launch runs (a multi-network launch passes the maximum).
    __device__ SparsePolicy(double* scratch, size_t stride, size_t slot, size_t floatBase = doubleElems())
    {
        A      = {scratch + slot, stride};
        b      = A.at(MAXNNZ);
        x      = b.at(D::n);
        r      = x.at(D::n);
        ipiv   = r.at(D::n);
        scale  = ipiv.at(D::n);
        Y      = scale.at(D::n);
        Yn     = Y.at(D::N);
        rates  = Yn.at(D::N);
        drates = rates.at(D::R);
        BE     = drates.at(D::R);
        dYdt   = BE.at(D::N);
        dYdT   = dYdt.at(D::N);
        jdy    = dYdT.at(D::N);
        // float region: element e of slot s at f0[e * stride + s], f0 = the float view of
        // FP64 row floatBase (2 floats per double row)
        LU  = {reinterpret_cast<float*>(scratch + floatBase * stride) + slot, stride};
        d32 = LU.at(MAXNNZ);
    }

    // ---- assembly of A (FP64, fill positions zero) and b
    __device__ void assemble(const NetView& nv, double T, double Tg, double rho, double drho_dt, double cv,
                             double dpdT, double dt)
    {
        const SparseView& sp = nv.sp;
        networkRatesFast<NET>(nv, Yn, Tg, rho, BE, rates, drates);
        for (int p = 0; p < sp.nnz; ++p)
            A[p] = 0.;
        for (int i = 0; i < D::N; ++i)
            dYdt[i] = 0., dYdT[i] = 0., jdy[i] = 0.;
        for (int q = 0; q < D::R; ++q)
        {
            const int rb = __ldg(nv.rbeg + q), re = __ldg(nv.rbeg + q + 1);
            const int pb = __ldg(nv.pbeg + q), pe = __ldg(nv.pbeg + q + 1);
            double    f = rates[q], df = drates[q], base = rates[q];
            for (int k = rb; k < re; ++k)
            {
                const int    cnt = __ldg(nv.rcnt + k);
                const double yr  = Yn[__ldg(nv.rspec + k)] * rho;
                if (cnt != 1)
                {
                    const double fac = cnt == 2 ? 2. : 6.;
                    f /= fac, df /= fac, base /= fac;
                }
                const double pw = ipowS(yr, cnt);
                f *= pw, df *= pw, base *= ipowS(yr, cnt - 1);
            }
            f /= rho, df /= rho;
            // dY/dt and d(dY/dt)/dT (nuclear_net.hpp:347-381)
            for (int k = rb; k < re; ++k)
            {
                const int s = __ldg(nv.rspec + k), c = __ldg(nv.rcnt + k);
                dYdt[s]     = dYdt[s] - f * c;
                dYdT[s]     = dYdT[s] - df * c;
            }
            for (int k = pb; k < pe; ++k)
            {
                const int s = __ldg(nv.pspec + k), c = __ldg(nv.pcnt + k);
                dYdt[s]     = dYdt[s] + f * c;
                dYdT[s]     = dYdT[s] + df * c;
            }
            // Jacobian into the fill pattern, with J (Yg - Y) accumulated on the way
            // (nuclear_net.hpp:395-438 and :580-589)
            if (base > k::epsilonSystem)
                for (int k = rb; k < re; ++k)
                {
                    const int id = __ldg(nv.rspec + k);
                    double    tr = base;
                    for (int o = rb; o < re; ++o)
                    {
                        const int os = __ldg(nv.rspec + o);
                        if (os != id) tr *= Yn[os] * rho;
                    }
                    const double dy = Yn[id] - Y[id];
                    const int    cb = __ldg(sp.cBeg + k), ce = __ldg(sp.cBeg + k + 1);
                    for (int c = cb; c < ce; ++c)
                    {
                        const double v   = tr * __ldg(sp.cCoef + c);
                        const int    pos = __ldg(sp.cPos + c), row = __ldg(sp.cRow + c);
                        A[pos]           = A[pos] + v;
                        jdy[row]         = jdy[row] + v * dy;
                    }
                }
        }
        const double mtd = -k::theta * dt;
        for (int e = 0; e < sp.nsb; ++e)
        {
            const int p = __ldg(sp.sbPos + e);
            A[p]        = __ldg(sp.sbDiag + e) ? 1. - k::theta * dt * A[p] : mtd * A[p];
        }
        for (int i = 0; i < D::N; ++i)
        {
            const double c0 = dYdT[i];
            double       rh = dYdt[i] * dt;
            rh              = rh + mtd * c0 * (Tg - T);
            rh              = rh + mtd * jdy[i];
            b[__ldg(sp.iperm + i + 1)] = rh;
            A[__ldg(sp.col0Pos + i)]   = c0 * mtd;
            A[__ldg(sp.row0Pos + i)]   = -BE[i] / cv;
        }
        const double drho = drho_dt * dt, value1 = dpdT * drho / (rho * rho);
        b[sp.tNew]   = T * value1 / cv;
        A[sp.pos00]  = 1 - k::theta * value1 / cv;
    }

    // ---- FP64 right-looking LU in place, then solve into x
    __device__ void factorSolve64(const SparseView& sp)
    {
        for (int kk = 0; kk < D::n; ++kk)
        {
            const double ip = 1. / A[__ldg(sp.kPiv + kk)];
            ipiv[kk]        = ip;
            const int ub = __ldg(sp.uBeg + kk), ue = __ldg(sp.uBeg + kk + 1);
            for (int e = __ldg(sp.lBeg + kk), ee = __ldg(sp.lBeg + kk + 1); e < ee; ++e)
            {
                const int    lp = __ldg(sp.lPos + e);
                const double l  = A[lp] * ip;
                A[lp]           = l;
                const int*   tp = sp.tPos + __ldg(sp.tBeg + e);
                for (int u = ub; u < ue; ++u)
                {
                    const int t = __ldg(tp + (u - ub));
                    A[t]        = A[t] - l * A[__ldg(sp.uPos + u)];
                }
            }
        }
        for (int kk = 0; kk < D::n; ++kk)
            x[kk] = b[kk];
        for (int kk = 0; kk < D::n; ++kk)
        {
            const double bk = x[kk];
            for (int e = __ldg(sp.lBeg + kk), ee = __ldg(sp.lBeg + kk + 1); e < ee; ++e)
            {
                const int i = __ldg(sp.lRow + e);
                x[i]        = x[i] - A[__ldg(sp.lPos + e)] * bk;
            }
        }
        for (int kk = D::n - 1; kk >= 0; --kk)
        {
            double s = x[kk];
            for (int u = __ldg(sp.uBeg + kk), ue = __ldg(sp.uBeg + kk + 1); u < ue; ++u)
                s -= A[__ldg(sp.uPos + u)] * x[__ldg(sp.uCol + u)];
            x[kk] = s * ipiv[kk];
        }
    }

    // FP32 triangular solves of LU d = rhs (rhs in d32, result in d32)
    __device__ void solve32(const SparseView& sp)
    {
        for (int kk = 0; kk < D::n; ++kk)
        {
            const float bk = d32[kk];
            for (int e = __ldg(sp.lBeg + kk), ee = __ldg(sp.lBeg + kk + 1); e < ee; ++e)
            {
                const int i = __ldg(sp.lRow + e);
                d32[i]      = d32[i] - LU[__ldg(sp.lPos + e)] * bk;
            }
        }
        for (int kk = D::n - 1; kk >= 0; --kk)
        {
            float s = d32[kk];
            for (int u = __ldg(sp.uBeg + kk), ue = __ldg(sp.uBeg + kk + 1); u < ue; ++u)
                s -= LU[__ldg(sp.uPos + u)] * d32[__ldg(sp.uCol + u)];
            d32[kk] = s * (float)ipiv[kk];
        }
    }

    // mixed precision: FP32 factorisation of the row-scaled matrix, FP64 refinement
    __device__ int mixedSolve(const SparseView& sp, double T)
    {
        for (int i = 0; i < D::n; ++i)
        {
            double m = 0;
            for (int p = __ldg(sp.rowBeg + i), pe = __ldg(sp.rowBeg + i + 1); p < pe; ++p)
                m = fmax(m, fabs(A[p]));
            const double s = m > 0 ? exp2(-(double)ilogb(m)) : 1.;
            scale[i]       = s;
            for (int p = __ldg(sp.rowBeg + i), pe = __ldg(sp.rowBeg + i + 1); p < pe; ++p)
                LU[p] = (float)(A[p] * s);
        }
        for (int kk = 0; kk < D::n; ++kk)
        {
            const float ip = 1.f / LU[__ldg(sp.kPiv + kk)];
            ipiv[kk]       = ip;
            const int ub = __ldg(sp.uBeg + kk), ue = __ldg(sp.uBeg + kk + 1);
            for (int e = __ldg(sp.lBeg + kk), ee = __ldg(sp.lBeg + kk + 1); e < ee; ++e)
            {
                const int   lp = __ldg(sp.lPos + e);
                const float l  = LU[lp] * ip;
                LU[lp]         = l;
                const int*  tp = sp.tPos + __ldg(sp.tBeg + e);
                for (int u = ub; u < ue; ++u)
                {
                    const int t = __ldg(tp + (u - ub));
                    LU[t]       = LU[t] - l * LU[__ldg(sp.uPos + u)];
                }
            }
        }
        for (int i = 0; i < D::n; ++i)
            x[i] = 0., r[i] = b[i];
        int steps = 0;
        for (;;)
        {
            for (int i = 0; i < D::n; ++i)
                d32[i] = (float)(r[i] * scale[i]);
            solve32(sp);
            bool conv = true;
            for (int i = 0; i < D::n; ++i)
            {
                const double di = (double)d32[i], xi = x[i] + di;
                const int    o  = __ldg(sp.perm + i); // reference index: 0 = T, 1.. = species
                const double sc = o == 0 ? T : fabs(Y[o - 1]);
                conv &= fabs(di) <= kRefineTol * (fabs(xi) + sc) && isfinite(xi); // an FP32 overflow is not convergence
                x[i] = xi;
            }
            if (conv) return steps;
            if (steps == kMaxRefine) return -1;
            ++steps;
            // r = b - A x in FP64 (A still holds the unscaled FP64 matrix)
            for (int i = 0; i < D::n; ++i)
            {
                double s = b[i];
                for (int p = __ldg(sp.rowBeg + i), pe = __ldg(sp.rowBeg + i + 1); p < pe; ++p)
                    s -= A[p] * x[__ldg(sp.posCol + p)];
                r[i] = s;
            }
        }
    }

    unsigned long long* refineStats = nullptr;

    __device__ void assembleSolve(const NetView& nv, double T, double Tg, double rho, double drho_dt, double cv,
                                  double dpdT, double dt)
    {
        assemble(nv, T, Tg, rho, drho_dt, cv, dpdT, dt);
        if constexpr (MIXED)
        {
            const int steps = mixedSolve(nv.sp, T);
            if (steps < 0)
            {
                factorSolve64(nv.sp); // not converged: this system is solved in FP64
                if (refineStats) atomicAdd(refineStats + 1, 1ull);
            }
            else if (refineStats && steps)
                atomicAdd(refineStats, (unsigned long long)steps);
        }
        else
            factorSolve64(nv.sp);
    }

    // solution in the reference's indexing (0 = T, 1.. = species)
    __device__ __forceinline__ double dy(const SparseView& sp, int oldIndex) const
    {
        return x[__ldg(sp.iperm + oldIndex)];
    }
};


// policy type of network NET for solver form FORM (nnet_solver)
template<int NET, int FORM>
struct PolicyOf
{
    using type = typename std::conditional<FORM == NNET_SOLVER_DENSE_FP64, DensePolicy<NET>,
                                           SparsePolicy<NET, FORM == NNET_SOLVER_MIXED>>::type;
    static constexpr int maxNnz = FORM == NNET_SOLVER_DENSE_FP64 ? 0 : SparsePolicy<NET, false>::MAXNNZ;
};

} // namespace nnet_gb300
