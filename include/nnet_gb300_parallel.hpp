// C++ drop-in for SPH-EXA-nnet's GPU batch drivers, over the C ABI of nnet_gb300.h.
//
// Same call shape as the reference:
//   nnet::parallel::computeNuclearReactions<use_gpu, Data, Float>(n, firstIndex, lastIndex,
//       hydro_dt, previous_dt, reactions, construct_rates_BE, eos, use_drhodt)
//                                     include/nnet/parallel/parallel_nuclear_net.hpp:86-90
//   nnet::parallel::computeHelmEOS<use_gpu, Data, Vector>(n, firstIndex, lastIndex, Z)
//                                     include/nnet/parallel/parallel_nuclear_net.hpp:190-191
// with the networks and EOSes passed as tag objects instead of polymorphic functors
// copied to the device (which the reference's CUDA driver does at
// parallel_nuclear_net.cu:127-134).  `Data` needs the fields the reference documents
// (parallel_nuclear_net.hpp:63-85) on `n.devData`: Y (one device vector per species),
// temp, rho, rho_m1, dt, and u, cv, p, c, dpdT for the EOS; thrust::device_vector and
// any vector whose data() yields a raw device pointer are accepted.
#pragma once

#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "nnet_gb300.h"

#if __has_include(<thrust/device_vector.h>) && defined(__CUDACC__)
#include <thrust/device_vector.h>
#define NNET_GB300_HAVE_THRUST 1
#endif

namespace nnet_gb300
{

struct ReactionListTag
{
    int network;
};
struct RatesTag
{
    int network;
};
template<typename Float>
struct IdealGasFunctor
{
    double mu;
    explicit IdealGasFunctor(double mu_)
        : mu(mu_)
    {
    }
};
template<typename Float>
struct HelmholtzFunctor
{
};

namespace net14
{
inline const ReactionListTag reactionList{NNET_NET14};
inline const RatesTag        computeReactionRates{NNET_NET14};
} // namespace net14
namespace net86
{
inline const ReactionListTag reactionList{NNET_NET86};
inline const RatesTag        computeReactionRates{NNET_NET86};
} // namespace net86
namespace net87
{
inline const ReactionListTag reactionList{NNET_NET87};
inline const RatesTag        computeReactionRates{NNET_NET87};
} // namespace net87

namespace detail
{
template<class V>
double* raw(V& v, size_t offset)
{
#ifdef NNET_GB300_HAVE_THRUST
    return thrust::raw_pointer_cast(v.data()) + offset;
#else
    return reinterpret_cast<double*>(&*v.data()) + offset;
#endif
}
inline void check(int rc)
{
    if (rc != NNET_SUCCESS) throw std::runtime_error(std::string("nnet_gb300: ") + nnet_last_error_message());
}
template<class E>
void eosArgs(const E&, nnet_burn_args& a)
{
    a.eos = NNET_EOS_HELMHOLTZ;
}
template<typename Float>
void eosArgs(const IdealGasFunctor<Float>& e, nnet_burn_args& a)
{
    a.eos          = NNET_EOS_IDEAL_GAS;
    a.ideal_gas_mu = e.mu;
}
} // namespace detail

// Process-wide context (tables loaded once, as the reference's static-initialisation table
// reads, helmholtz.cpp:89-218).  The Helmholtz table comes from, in order: `helmTable`, the
// compile-time path NNET_GB300_HELM_TABLE (the reference compiles its table path in the same
// way, HELM_TABLE_PATH), or the environment variable NNET_HELM_TABLE; either file layout of
// nnet_load_helmholtz_table_file.  Without one, burns with HelmholtzFunctor throw, naming
// these three ways.  The first call fixes the device and the table.
inline nnet_handle defaultContext(int device = 0, const char* helmTable = nullptr)
{
    static nnet_handle h = nullptr;
    if (!h)
    {
        detail::check(nnet_create(device, &h));
#ifdef NNET_GB300_HELM_TABLE
        if (!helmTable) helmTable = NNET_GB300_HELM_TABLE;
#endif
        if (!helmTable) helmTable = std::getenv("NNET_HELM_TABLE");
        if (helmTable) detail::check(nnet_load_helmholtz_table_file(h, helmTable));
    }
    return h;
}

namespace detail
{
inline void checkBurn(int rc)
{
    if (rc == NNET_ERR_NO_TABLE)
        throw std::runtime_error("nnet_gb300: the Helmholtz EOS needs a table: pass its path to "
                                 "nnet_gb300::defaultContext(device, path) before the first burn, compile with "
                                 "-DNNET_GB300_HELM_TABLE=\"path\", or set NNET_HELM_TABLE");
    check(rc);
}
} // namespace detail

namespace parallel
{

// Burn particles [firstIndex, lastIndex) of n over hydro_dt on the default stream and wait,
// as the reference's GPU driver does (parallel_nuclear_net.cu:156-157).
template<bool use_gpu, class Data, typename Float, class Eos>
void computeNuclearReactions(Data& n, size_t firstIndex, size_t lastIndex, const Float hydro_dt,
                             const Float previous_dt, const ReactionListTag& reactions,
                             const RatesTag& construct_rates_BE, const Eos& eos, bool use_drhodt,
                             int solver = NNET_SOLVER_SPARSE_FP64, nnet_handle h = nullptr)
{
    static_assert(use_gpu, "nnet_gb300 has no CPU path");
    if (reactions.network != construct_rates_BE.network)
        throw std::invalid_argument("reaction list and rate functor belong to different networks");
    auto&                d = n.devData;
    std::vector<double*> Y(reactions.network);
    for (int j = 0; j < reactions.network; ++j)
        Y[j] = detail::raw(d.Y[j], firstIndex);
    nnet_burn_args a{};
    a.network = reactions.network;
    detail::eosArgs(eos, a);
    a.solver        = solver;
    a.num_particles = lastIndex - firstIndex;
    a.Y             = Y.data();
    a.T             = detail::raw(d.temp, firstIndex);
    a.rho           = detail::raw(d.rho, firstIndex);
    a.rho_m1        = use_drhodt ? detail::raw(d.rho_m1, firstIndex) : nullptr;
    a.dt            = detail::raw(d.dt, firstIndex);
    a.hydro_dt      = hydro_dt;
    a.previous_dt   = previous_dt;
    a.use_drhodt    = use_drhodt;
    nnet_handle ctx = h ? h : defaultContext();
    detail::checkBurn(nnet_burn(ctx, &a, nullptr));
    nnet_stats st;
    detail::check(nnet_get_stats(ctx, &st)); // synchronises, as the reference's blocking call
}

// Post-burn Helmholtz EOS into n.devData.{u, cv, p, c, dpdT} for [firstIndex, lastIndex).
template<bool use_gpu, class Data, class Vector>
void computeHelmEOS(Data& n, size_t firstIndex, size_t lastIndex, const Vector& Z, nnet_handle h = nullptr)
{
    static_assert(use_gpu, "nnet_gb300 has no CPU path");
    auto&                d = n.devData;
    const int            dim = (int)Z.size();
    std::vector<double*> Y(dim);
    for (int j = 0; j < dim; ++j)
        Y[j] = detail::raw(d.Y[j], firstIndex);
    nnet_handle ctx = h ? h : defaultContext();
    detail::checkBurn(nnet_helmholtz_eos(ctx, lastIndex - firstIndex, dim, Z.data(), detail::raw(d.temp, firstIndex),
                                     detail::raw(d.rho, firstIndex), Y.data(), detail::raw(d.u, firstIndex),
                                     detail::raw(d.cv, firstIndex), detail::raw(d.p, firstIndex),
                                     detail::raw(d.c, firstIndex), detail::raw(d.dpdT, firstIndex), nullptr));
}

} // namespace parallel
} // namespace nnet_gb300
