// Table generator: prints the reference's network definitions (reaction lists,
// charges, masses, binding energies, REACLIB-style fit coefficients, partition
// function tables and the net87 electron-capture table) as a plain C header.
//
// It is compiled against the reference's own headers so that every constant is
// the exact double the reference computes (same parsing, same MevToErg
// products).  Run by gen_tables.py; its output (nnet_network_tables.h) is
// committed, so nothing at run time needs the reference sources.
//
// Data sources in the reference:
//   net14 reaction list        include/nnet/parameterization/net14/net14.hpp:69-134
//   net14 Z, A                 include/nnet/parameterization/net14/net14_constants.hpp:52-62
//   net14 BE                   include/nnet/parameterization/net14/net14.hpp:45-50,66
//   net14 q, fit, choose       include/nnet/parameterization/net14/net14_tables.hpp:103-133
//   net86 reaction list        include/nnet/parameterization/net86/net86.hpp:95-192
//   net86 Z, A, indices        include/nnet/parameterization/net86/net86_constants.hpp
//   net86 BE                   include/nnet/parameterization/net86/net86.hpp:47-76,92
//   net86 q, fit, choose       include/nnet/parameterization/net86/net86_tables.hpp:78-384
//   net87 reaction list, BE    include/nnet/parameterization/net87/net87.hpp:85-98
//   electron table             include/nnet/parameterization/net87/net87.cpp:65-87
#include <cstdio>
#include <vector>
#include <string>

#include "nnet/parameterization/net14/net14.hpp"
#include "nnet/parameterization/net14/net14_tables.hpp"
#include "nnet/parameterization/net86/net86.hpp"
#include "nnet/parameterization/net86/net86_tables.hpp"
#include "nnet/parameterization/net87/net87.hpp"

namespace nnet::net87::electrons::constants
{
extern double log_temp_ref[N_TEMP];
extern double log_rho_ref[N_RHO];
extern double electron_rate[N_TEMP][N_RHO][N_C];
} // namespace nnet::net87::electrons::constants

static void arr(const char* type, const char* name, const double* v, size_t n)
{
    std::printf("static const %s %s[%zu] = {", type, name, n);
    for (size_t i = 0; i < n; ++i)
        std::printf("%s%.17g%s", (i % 4 == 0) ? "\n    " : " ", v[i], i + 1 < n ? "," : "");
    std::printf("\n};\n");
}

static void iarr(const char* name, const std::vector<int>& v)
{
    std::printf("static const int %s[%zu] = {", name, v.size());
    for (size_t i = 0; i < v.size(); ++i)
        std::printf("%s%d%s", (i % 16 == 0) ? "\n    " : " ", v[i], i + 1 < v.size() ? "," : "");
    std::printf("\n};\n");
}

// Reaction list in CSR form: begin[r]..begin[r+1] indexes reactant entries,
// pbegin[r]..pbegin[r+1] product entries.
static void reactions(const char* prefix, const nnet::ReactionList& list)
{
    std::vector<int> rbeg{0}, rspec, rnum, pbeg{0}, pspec, pnum;
    for (size_t r = 0; r < list.size(); ++r)
    {
        auto ref = list[r];
        for (auto it = ref.reactants.begin(); it != ref.reactants.end(); ++it)
            rspec.push_back(it->speciesId), rnum.push_back(it->numConsumed);
        for (auto it = ref.products.begin(); it != ref.products.end(); ++it)
            pspec.push_back(it->speciesId), pnum.push_back(it->numConsumed);
        rbeg.push_back((int)rspec.size());
        pbeg.push_back((int)pspec.size());
    }
    std::printf("#define %s_NUM_REACTIONS %zu\n", prefix, list.size());
    std::string p(prefix);
    for (auto& c : p) c = (char)std::tolower(c);
    iarr((p + "_reactant_begin").c_str(), rbeg);
    iarr((p + "_reactant_species").c_str(), rspec);
    iarr((p + "_reactant_count").c_str(), rnum);
    iarr((p + "_product_begin").c_str(), pbeg);
    iarr((p + "_product_species").c_str(), pspec);
    iarr((p + "_product_count").c_str(), pnum);
}

int main()
{
    std::printf("/* Generated by dump_reference_tables.cpp (gen_tables.py): network definitions\n"
                " * of the net14 / net86 / net87 nuclear networks and the net87 electron-capture\n"
                " * table, printed with 17 significant digits (exact double round trip).\n"
                " * Do not edit. */\n#pragma once\n\n");

    // physical constants shared by the networks (net14_constants.hpp:46-50)
    std::printf("#define NNET_KB %.17g\n#define NNET_NA %.17g\n#define NNET_E2 %.17g\n#define NNET_MEV_TO_ERG %.17g\n",
                nnet::net14::constants::Kb, nnet::net14::constants::Na, nnet::net14::constants::e2,
                nnet::net14::constants::MevToErg);
    std::printf("#define NNET_PI %.17g\n\n", nnet::net14::constants::pi);

    // ---------------- net14 ----------------
    std::printf("#define NET14_NUM_SPECIES 14\n");
    reactions("NET14", nnet::net14::reactionList);
    arr("double", "net14_Z", nnet::net14::constants::Z.data(), 14);
    arr("double", "net14_A", nnet::net14::constants::A.data(), 14);
    arr("double", "net14_BE", nnet::net14::BE.data(), 14);
    arr("double", "net14_q", nnet::net14::constants::fits::q, 10);
    arr("double", "net14_fit", &nnet::net14::constants::fits::fit[0][0], 10 * 8);
    arr("double", "net14_choose", &nnet::net14::constants::fits::choose[0][0], 11 * 24);

    // ---------------- net86 ----------------
    std::printf("\n#define NET86_NUM_SPECIES 86\n");
    reactions("NET86", nnet::net86::reactionList);
    arr("double", "net86_Z", nnet::net86::constants::Z.data(), 87);
    arr("double", "net86_A", nnet::net86::constants::A.data(), 87);
    arr("double", "net86_BE", nnet::net86::BE.data(), 86);
    {
        std::vector<int> mr(157), sr(157), mp(157);
        for (int i = 0; i < 157; ++i)
            mr[i] = nnet::net86::constants::main_reactant[i], sr[i] = nnet::net86::constants::secondary_reactant[i],
            mp[i] = nnet::net86::constants::main_product[i];
        iarr("net86_main_reactant", mr);
        iarr("net86_secondary_reactant", sr);
        iarr("net86_main_product", mp);
    }
    arr("double", "net86_q", nnet::net86::constants::fits::q, 150);
    arr("double", "net86_fit", &nnet::net86::constants::fits::fit[0][0], 150 * 8);
    arr("double", "net86_choose", &nnet::net86::constants::fits::choose[0][0], 81 * 24);

    // ---------------- net87 ----------------
    std::printf("\n#define NET87_NUM_SPECIES 87\n");
    reactions("NET87", nnet::net87::reactionList);
    arr("double", "net87_BE", nnet::net87::BE.data(), 87);

    namespace ec = nnet::net87::electrons::constants;
    std::printf("\n#define NET87_ELECTRON_NTEMP %d\n#define NET87_ELECTRON_NRHO %d\n#define NET87_ELECTRON_NC %d\n",
                N_TEMP, N_RHO, N_C);
    arr("double", "net87_electron_log_temp", ec::log_temp_ref, N_TEMP);
    arr("double", "net87_electron_log_rho", ec::log_rho_ref, N_RHO);
    arr("double", "net87_electron_rate", &ec::electron_rate[0][0][0], (size_t)N_TEMP * N_RHO * N_C);
    return 0;
}
