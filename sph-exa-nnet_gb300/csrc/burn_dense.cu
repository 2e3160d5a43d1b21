// Plain FP64 form of the burn: the Newton system is assembled densely and solved by
// Gaussian elimination without pivoting, in the reference's operation order
// (include/nnet/nuclear_net.hpp:347-438 and :514-609, include/nnet_util/eigen.hpp:155-198).
// One thread per particle; the (N+1)^2 matrix and the vectors live in per-slot scratch,
// interleaved across slots so that every access of a warp is one coalesced 256-byte line.
#include "driver.cuh"
#include "launch.hpp"

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

        // Gaussian elimination without pivoting, zero multipliers skipped (eigen.hpp:155-198)
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

template<int NET, int EOS>
__global__ void __launch_bounds__(128) burnDenseKernel(BurnParams bp, NetView nv, HelmView hv, double* scratch,
                                                       size_t stride)
{
    const size_t      slot = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    DensePolicy<NET> pol(scratch, stride, slot);
    burnLoop<NET, EOS>(bp, nv, hv, pol);
}

template<int NET, int EOS>
static KernelInfo denseInfo()
{
    return {(const void*)burnDenseKernel<NET, EOS>, DensePolicy<NET>::perSlot(), 128, 0};
}

KernelInfo denseKernel(int net, int eos)
{
    if (net == 14) return eos ? denseInfo<14, 1>() : denseInfo<14, 0>();
    if (net == 86) return eos ? denseInfo<86, 1>() : denseInfo<86, 0>();
    return eos ? denseInfo<87, 1>() : denseInfo<87, 0>();
}

} // namespace nnet_gb300
