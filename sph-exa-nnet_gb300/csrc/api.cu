// C ABI of the GB300 burn library (include/nnet_gb300.h): context, table upload, burn
// dispatch and the post-burn Helmholtz EOS.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "driver.cuh"
#include "launch.hpp"
#include "sparse_plan.hpp"
#include "context.hpp"
#include "burn_multi.hpp"

using namespace nnet_gb300;

namespace
{
thread_local std::string g_lastError;

int fail(int code, const std::string& msg)
{
    g_lastError = msg;
    return code;
}

#define NNET_CUDA(call)                                                                                               \
    do                                                                                                                \
    {                                                                                                                 \
        cudaError_t e_ = (call);                                                                                      \
        if (e_ != cudaSuccess)                                                                                        \
            return fail(NNET_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));                           \
    } while (0)

int uploadNetwork(int net, NetBuffer& b)
{
    const int N = net, R = net == 14 ? NET14_NUM_REACTIONS : net == 86 ? NET86_NUM_REACTIONS : NET87_NUM_REACTIONS;
    const int *rbeg, *rspec, *rcnt, *pbeg, *pspec, *pcnt;
    const double *BE, *Z, *fit, *q, *choose;
    int nfit, nq, nchoose;
    if (net == 14)
    {
        rbeg = net14_reactant_begin, rspec = net14_reactant_species, rcnt = net14_reactant_count;
        pbeg = net14_product_begin, pspec = net14_product_species, pcnt = net14_product_count;
        BE = net14_BE, Z = net14_Z, fit = net14_fit, q = net14_q, choose = net14_choose;
        nfit = 80, nq = 10, nchoose = 264;
    }
    else
    {
        if (net == 86)
        {
            rbeg = net86_reactant_begin, rspec = net86_reactant_species, rcnt = net86_reactant_count;
            pbeg = net86_product_begin, pspec = net86_product_species, pcnt = net86_product_count;
            BE = net86_BE;
        }
        else
        {
            rbeg = net87_reactant_begin, rspec = net87_reactant_species, rcnt = net87_reactant_count;
            pbeg = net87_product_begin, pspec = net87_product_species, pcnt = net87_product_count;
            BE = net87_BE;
        }
        Z = net86_Z, fit = net86_fit, q = net86_q, choose = net86_choose;
        nfit = 1200, nq = 150, nchoose = 1944;
    }
    const int nr = rbeg[R], np = pbeg[R];
    // doubles: BE, Z, z53 (N each, Z padded to 87), fit, q, choose, electron tables
    std::vector<double> d;
    auto putd = [&](const double* src, size_t n) {
        size_t o = d.size();
        d.insert(d.end(), src, src + n);
        return o;
    };
    std::vector<double> z53(N, 0.);
    for (int i = 0; i < N && i < (net == 14 ? 14 : 86); ++i)
        z53[i] = std::pow(Z[i], 5. / 3.); // host libm, as the reference's per-call pow(Z, 5/3)
    std::vector<double> zf(4 * N, 0.);
    for (int i = 0; i < N; ++i)
    {
        const double z = z53[i];
        zf[4 * i + 0] = std::sqrt(z), zf[4 * i + 1] = std::sqrt(std::sqrt(z));
        zf[4 * i + 2] = std::pow(z, 1.9885), zf[4 * i + 3] = z > 0 ? std::log(z) : 0.;
    }
    const double* Am  = net == 14 ? net14_A : net86_A; // net86_A[86] = 0 is the net87 electron entry
    const size_t oBE = putd(BE, N), oZ = putd(Z, net == 14 ? 14 : 87), oZ53 = putd(z53.data(), N);
    const size_t oA  = putd(Am, net == 14 ? 14 : 87);
    const size_t oZf = putd(zf.data(), zf.size());
    const size_t oFit = putd(fit, nfit), oQ = putd(q, nq), oCh = putd(choose, nchoose);
    // partition-function ratio of every fitted rate per temperature range (the same IEEE
    // quotient the rate evaluation forms, computed once): net14 [10][24], net86 [150][24]
    std::vector<double> part;
    if (net == 14)
        for (int i = 4; i < 14; ++i)
            for (int kb = 0; kb < 24; ++kb)
                part.push_back(choose[(i - 4) * 24 + kb] / choose[(i + 1 - 4) * 24 + kb]);
    else
        for (int i = 7; i < 157; ++i)
            for (int kb = 0; kb < 24; ++kb)
                part.push_back(choose[(net86_main_reactant[i] - 5) * 24 + kb] /
                               choose[(net86_main_product[i] - 5) * 24 + kb]);
    const size_t oPart = putd(part.data(), part.size());
    const size_t oLT = putd(net87_electron_log_temp, NET87_ELECTRON_NTEMP);
    const size_t oLR = putd(net87_electron_log_rho, NET87_ELECTRON_NRHO);
    const size_t oER = putd(net87_electron_rate, (size_t)NET87_ELECTRON_NTEMP * NET87_ELECTRON_NRHO * NET87_ELECTRON_NC);
    std::vector<int> ii;
    auto puti = [&](const int* src, size_t n) {
        size_t o = ii.size();
        ii.insert(ii.end(), src, src + n);
        return o;
    };
    const size_t oRb = puti(rbeg, R + 1), oRs = puti(rspec, nr), oRc = puti(rcnt, nr);
    const size_t oPb = puti(pbeg, R + 1), oPs = puti(pspec, np), oPc = puti(pcnt, np);
    const size_t oMr = puti(net86_main_reactant, 157), oSr = puti(net86_secondary_reactant, 157),
                 oMp = puti(net86_main_product, 157);
    // sparse-solver plan (symbolic analysis of this network's Newton matrix)
    const SparsePlan sp = buildSparsePlan(net, rbeg, rspec, rcnt, pbeg, pspec, pcnt, R);
    b.plan              = sp;
    const size_t oCoef  = putd(sp.cCoef.data(), sp.cCoef.size());
    auto         putv   = [&](const std::vector<int>& v) { return puti(v.data(), v.size()); };
    const size_t oPerm = putv(sp.perm), oIperm = putv(sp.iperm), oRowBeg = putv(sp.rowBeg), oPosRow = putv(sp.posRow),
                 oPosCol = putv(sp.posCol), oKPiv = putv(sp.kPiv), oLBeg = putv(sp.lBeg), oLPos = putv(sp.lPos),
                 oLRow = putv(sp.lRow), oTBeg = putv(sp.tBeg), oUBeg = putv(sp.uBeg), oUPos = putv(sp.uPos),
                 oUCol = putv(sp.uCol), oTPos = putv(sp.tPos), oDiag = putv(sp.diagPos), oCol0 = putv(sp.col0Pos),
                 oRow0 = putv(sp.row0Pos), oCBeg = putv(sp.cBeg), oCPos = putv(sp.cPos), oCRow = putv(sp.cRow),
                 oSb = putv(sp.sbPos), oSbD = putv(sp.sbDiag);
    // warp-per-particle lists
    const WarpPlan wp = buildWarpPlan(sp, rbeg, rspec, rcnt, pbeg, pspec, pcnt, net == 14 ? kWarpNnzCap14 : kWarpNnzCap86);
    if (wp.sgHeavy.size() > 8 || wp.jgHeavy.size() > 8 || wp.rjHeavy.size() > 8 || wp.rowHeavy.size() > 8)
        return fail(NNET_ERR_TOO_LARGE, "network has more long gather lists than the warp kernels unroll");
    if (wp.rhsBase + sp.n > 0xffff)
        return fail(NNET_ERR_TOO_LARGE, "factor positions exceed the 16-bit fields of the factorisation ops");
    const size_t oSgC = putd(wp.sgCoef.data(), wp.sgCoef.size()), oJgC = putd(wp.jgCoef.data(), wp.jgCoef.size());
    const size_t oUpdB = putv(wp.updBeg), oUpdT = putv(wp.updT), oUpdL = putv(wp.updL), oUpdU = putv(wp.updU),
                 oUcB = putv(wp.ucBeg), oUcP = putv(wp.ucPos), oUcR = putv(wp.ucRow), oSgB = putv(wp.sgBeg),
                 oSgR = putv(wp.sgRx), oJP = putv(wp.jPos), oJR = putv(wp.jRow), oJC = putv(wp.jCol),
                 oJgB = putv(wp.jgBeg), oJgE = putv(wp.jgEnt), oRjB = putv(wp.rjBeg), oRjE = putv(wp.rjEnt),
                 oERx = putv(wp.entRx), oSgH = putv(wp.sgHeavy), oJgH = putv(wp.jgHeavy), oRjH = putv(wp.rjHeavy),
                 oRowH = putv(wp.rowHeavy);
    const size_t oLvB = putv(wp.lvBeg), oLvP = putv(wp.lvPiv), oLsB = putv(wp.lsBeg), oLsP = putv(wp.lsPos),
                 oLsK = putv(wp.lsPiv), oTgB = putv(wp.tgBeg), oTgP = putv(wp.tgPos), oTgU = putv(wp.tgUpd),
                 oTuL = putv(wp.tuL), oTuU = putv(wp.tuU), oFwB = putv(wp.fwBeg), oFwR = putv(wp.fwRow),
                 oFwE = putv(wp.fwEnt), oFlP = putv(wp.flPos), oFlK = putv(wp.flK), oBwB = putv(wp.bwBeg),
                 oBwR = putv(wp.bwRow), oBwE = putv(wp.bwEnt), oBuP = putv(wp.buPos), oBuK = putv(wp.buK);
    const size_t oSgO = putv(wp.sgOrder), oRjO = putv(wp.rjOrder);
    const size_t oScB = putv(wp.scBeg), oScP = putv(wp.scPos), oScK = putv(wp.scPiv), oTgBA = putv(wp.tgBegA),
                 oTgPA = putv(wp.tgPosA), oTgUA = putv(wp.tgUpdA), oTuLA = putv(wp.tuLA), oTuUA = putv(wp.tuUA);
    const size_t oFoB = putv(wp.foBeg);
    if (ii.size() % 2) ii.push_back(0); // the 64-bit ops start on an 8-byte boundary
    const size_t oFOp = ii.size();
    for (unsigned long long op : wp.fOps)
        ii.push_back((int)(unsigned)op), ii.push_back((int)(unsigned)(op >> 32)); // little-endian halves
    const size_t bytesD = d.size() * sizeof(double), bytes = bytesD + ii.size() * sizeof(int);
    NNET_CUDA(cudaMalloc(&b.mem, bytes));
    NNET_CUDA(cudaMemcpy(b.mem, d.data(), bytesD, cudaMemcpyHostToDevice));
    NNET_CUDA(cudaMemcpy((char*)b.mem + bytesD, ii.data(), ii.size() * sizeof(int), cudaMemcpyHostToDevice));
    const double* D = (const double*)b.mem;
    const int*    I = (const int*)((const char*)b.mem + bytesD);
    NetView&      v = b.view;
    v.net = net, v.nspec = N, v.nreact = R;
    v.rbeg = I + oRb, v.rspec = I + oRs, v.rcnt = I + oRc, v.pbeg = I + oPb, v.pspec = I + oPs, v.pcnt = I + oPc;
    v.BE = D + oBE, v.Z = D + oZ, v.z53 = D + oZ53, v.fit = D + oFit, v.q = D + oQ, v.choose = D + oCh;
    v.A = D + oA;
    v.zFac = D + oZf, v.part = D + oPart;
    v.mainReactant = I + oMr, v.secondaryReactant = I + oSr, v.mainProduct = I + oMp;
    v.eLogT = D + oLT, v.eLogRho = D + oLR, v.eRate = D + oER;
    SparseView& w = v.sp;
    w.n = sp.n, w.nnz = sp.nnz, w.nsb = (int)sp.sbPos.size(), w.pos00 = sp.pos00, w.tNew = sp.iperm[0];
    w.perm = I + oPerm, w.iperm = I + oIperm, w.rowBeg = I + oRowBeg, w.posRow = I + oPosRow, w.posCol = I + oPosCol;
    w.kPiv = I + oKPiv, w.lBeg = I + oLBeg, w.lPos = I + oLPos, w.lRow = I + oLRow, w.tBeg = I + oTBeg;
    w.uBeg = I + oUBeg, w.uPos = I + oUPos, w.uCol = I + oUCol, w.tPos = I + oTPos;
    w.diagPos = I + oDiag, w.col0Pos = I + oCol0, w.row0Pos = I + oRow0, w.cBeg = I + oCBeg, w.cPos = I + oCPos;
    w.cRow = I + oCRow, w.sbPos = I + oSb, w.sbDiag = I + oSbD, w.cCoef = D + oCoef;
    WarpView& x = v.wv;
    x.nJ = (int)wp.jPos.size(), x.nEnt = (int)wp.entRx.size(), x.nSgHeavy = (int)wp.sgHeavy.size();
    x.nJgHeavy = (int)wp.jgHeavy.size(), x.nRjHeavy = (int)wp.rjHeavy.size(), x.nRowHeavy = (int)wp.rowHeavy.size();
    x.updBeg = I + oUpdB, x.updT = I + oUpdT, x.updL = I + oUpdL, x.updU = I + oUpdU, x.ucBeg = I + oUcB;
    x.ucPos = I + oUcP, x.ucRow = I + oUcR, x.sgBeg = I + oSgB, x.sgRx = I + oSgR, x.jPos = I + oJP, x.jRow = I + oJR;
    x.jCol = I + oJC, x.jgBeg = I + oJgB, x.jgEnt = I + oJgE, x.rjBeg = I + oRjB, x.rjEnt = I + oRjE;
    x.entRx = I + oERx, x.sgHeavy = I + oSgH, x.jgHeavy = I + oJgH, x.rjHeavy = I + oRjH, x.rowHeavy = I + oRowH;
    x.sgCoef = D + oSgC, x.jgCoef = D + oJgC;
    x.nLevels = wp.nLevels;
    x.lvBeg = I + oLvB, x.lvPiv = I + oLvP, x.lsBeg = I + oLsB, x.lsPos = I + oLsP, x.lsPiv = I + oLsK;
    x.tgBeg = I + oTgB, x.tgPos = I + oTgP, x.tgUpd = I + oTgU, x.tuL = I + oTuL, x.tuU = I + oTuU;
    x.fwBeg = I + oFwB, x.fwRow = I + oFwR, x.fwEnt = I + oFwE, x.flPos = I + oFlP, x.flK = I + oFlK;
    x.bwBeg = I + oBwB, x.bwRow = I + oBwR, x.bwEnt = I + oBwE, x.buPos = I + oBuP, x.buK = I + oBuK;
    x.sgOrder = I + oSgO, x.rjOrder = I + oRjO;
    x.rhsBase = wp.rhsBase;
    x.scBeg = I + oScB, x.scPos = I + oScP, x.scPiv = I + oScK, x.tgBegA = I + oTgBA, x.tgPosA = I + oTgPA;
    x.tgUpdA = I + oTgUA, x.tuLA = I + oTuLA, x.tuUA = I + oTuUA;
    x.fOps = reinterpret_cast<const unsigned long long*>(I + oFOp), x.foBeg = I + oFoB;
    return NNET_SUCCESS;
}

constexpr int kNetCounters = 16;             // queue head + stats of one launch
static_assert(1 + kStatWords <= kNetCounters, "counter region too small");
constexpr int kMigCounterWord = 1 + kStatWords; // the rebalancing counters follow the statistics
static_assert(kMigCounterWord + 3 <= kNetCounters, "counter region too small");
constexpr size_t kMigRecordsPerSlot = 4;        // hand-off records reserved per slot of the grid
constexpr int kCounters    = 4 * kNetCounters; // single launch uses [0, 16); a batch one region per network

int netIndex(int net) { return net == 14 ? 0 : net == 86 ? 1 : net == 87 ? 2 : -1; }

// post-burn EOS: one thread per particle (parallel_nuclear_net.cu:184-210)
struct EosParams
{
    size_t        P;
    int           dim;
    double        Z[NNET_MAX_SPECIES];
    const double* Y[NNET_MAX_SPECIES];
    const double *T, *rho;
    double *      u, *cv, *p, *c, *dpdT;
};

// post-burn steps of launches whose kernel does not fuse them (one thread per particle)
__global__ void postBurnKernel(BurnParams bp, NetView nv, HelmView hv)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < bp.P; i += (size_t)gridDim.x * blockDim.x)
        postScalar(bp, nv, hv, i, bp.status[i] != ST_SKIPPED);
}

__global__ void helmholtzEosKernel(EosParams ep, HelmView hv)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < ep.P; i += (size_t)gridDim.x * blockDim.x)
    {
        double abar = 0, zbar = 0;
        for (int j = 0; j < ep.dim; ++j)
        {
            const double y = ep.Y[j][i];
            abar += y;
            zbar += y * ep.Z[j];
        }
        const EosResult r = helmholtzEos(hv, abar, zbar, ep.T[i], ep.rho[i]);
        ep.u[i] = r.u, ep.cv[i] = r.cv, ep.p[i] = r.p, ep.c[i] = r.c, ep.dpdT[i] = r.dpdT;
    }
}
} // namespace

extern "C" {

const char* nnet_last_error_message(void) { return g_lastError.c_str(); }

int nnet_network_info(int network, int* num_species, int* num_reactions)
{
    if (netIndex(network) < 0) return fail(NNET_ERR_INVALID, "unknown network");
    if (num_species) *num_species = network;
    if (num_reactions)
        *num_reactions = network == 14 ? NET14_NUM_REACTIONS : network == 86 ? NET86_NUM_REACTIONS : NET87_NUM_REACTIONS;
    return NNET_SUCCESS;
}

int nnet_solver_info(int network, int solver, long long* factor_fma, long long* solve_fma, int* factor_entries)
{
    const int R = network == 14 ? NET14_NUM_REACTIONS : network == 86 ? NET86_NUM_REACTIONS : NET87_NUM_REACTIONS;
    if (netIndex(network) < 0) return fail(NNET_ERR_INVALID, "unknown network");
    const int n = network + 1;
    if (solver == NNET_SOLVER_DENSE_FP64)
    {
        // eigen::solve with complete fill (eigen.hpp:178-223): elimination of row i by rows
        // j < i costs 1 + (n - 1 - j) multiply-adds, back substitution n(n-1)/2
        long long f = 0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < i; ++j)
                f += 1 + (n - 1 - j);
        if (factor_fma) *factor_fma = f;
        if (solve_fma) *solve_fma = (long long)n * (n - 1) / 2;
        if (factor_entries) *factor_entries = n * n;
        return NNET_SUCCESS;
    }
    const int *rbeg, *rspec, *rcnt, *pbeg, *pspec, *pcnt;
    if (network == 14)
        rbeg = net14_reactant_begin, rspec = net14_reactant_species, rcnt = net14_reactant_count,
        pbeg = net14_product_begin, pspec = net14_product_species, pcnt = net14_product_count;
    else if (network == 86)
        rbeg = net86_reactant_begin, rspec = net86_reactant_species, rcnt = net86_reactant_count,
        pbeg = net86_product_begin, pspec = net86_product_species, pcnt = net86_product_count;
    else
        rbeg = net87_reactant_begin, rspec = net87_reactant_species, rcnt = net87_reactant_count,
        pbeg = net87_product_begin, pspec = net87_product_species, pcnt = net87_product_count;
    const SparsePlan p = buildSparsePlan(network, rbeg, rspec, rcnt, pbeg, pspec, pcnt, R);
    if (factor_fma) *factor_fma = p.factorFma;
    if (solve_fma) *solve_fma = p.solveFma;
    if (factor_entries) *factor_entries = p.nnz;
    return NNET_SUCCESS;
}

int nnet_create(int device, nnet_handle* out)
{
    if (!out) return fail(NNET_ERR_INVALID, "null handle pointer");
    NNET_CUDA(cudaSetDevice(device));
    nnet_context* h = new nnet_context;
    h->device       = device;
    cudaDeviceGetAttribute(&h->numSMs, cudaDevAttrMultiProcessorCount, device);
    const int nets[3] = {14, 86, 87};
    for (int k = 0; k < 3; ++k)
    {
        int rc = uploadNetwork(nets[k], h->nets[k]);
        if (rc)
        {
            nnet_destroy(h);
            return rc;
        }
    }
    if (int rc = h->ws.ensure(0, nullptr))
    {
        nnet_destroy(h);
        return rc;
    }
    *out = h;
    return NNET_SUCCESS;
}

int nnet_destroy(nnet_handle h)
{
    if (!h) return NNET_SUCCESS;
    cudaSetDevice(h->device);
    cudaDeviceSynchronize();
    for (auto& n : h->nets)
        if (n.mem) cudaFree(n.mem);
    if (h->helmMem) cudaFree(h->helmMem);
    if (h->orderCounters) cudaFree(h->orderCounters);
    h->ws.release();
    delete h;
    return NNET_SUCCESS;
}

int nnet_load_helmholtz_table(nnet_handle h, const double* table)
{
    if (!h || !table) return fail(NNET_ERR_INVALID, "null argument");
    NNET_CUDA(cudaSetDevice(h->device));
    constexpr int I = HELM_IMAX, J = HELM_JMAX, C = HELM_CELL;
    // cell layout: f ft ftt fd fdd fdt fddt fdtt fddtt dpdf dpdft dpdfd dpdfdt (reference
    // table indices 0 2 4 1 3 5 6 7 8 9 11 10 12)
    static const int src[13] = {0, 2, 4, 1, 3, 5, 6, 7, 8, 9, 11, 10, 12};
    const size_t     ncell   = (size_t)I * J * C;
    std::vector<double> host(ncell + 9 * (size_t)I, 0.);
    for (int i = 0; i < I; ++i)
        for (int j = 0; j < J; ++j)
            for (int q = 0; q < 13; ++q)
                host[((size_t)i * J + j) * C + q] = table[((size_t)src[q] * I + i) * J + j];
    // grid and spacing arrays exactly as the reference computes them (helmholtz.cpp:101-169)
    const double tlo = 3., thi = 13., tstp = (thi - tlo) / (double)(J - 1);
    const double dlo = -12., dhi = 15., dstp = (dhi - dlo) / (double)(I - 1);
    double*      g = host.data() + ncell; // 9 arrays of I doubles
    double *d = g, *ddS = g + I, *dd2S = g + 2 * I, *ddiS = g + 3 * I, *t = g + 4 * I, *dtS = g + 5 * I,
           *dt2S = g + 6 * I, *dtiS = g + 7 * I, *dt2iS = g + 8 * I;
    for (int i = 0; i < I; ++i)
        d[i] = std::pow((double)10., dlo + i * dstp);
    for (int j = 0; j < J; ++j)
        t[j] = std::pow((double)10., tlo + j * tstp);
    for (int j = 0; j < J - 1; ++j)
    {
        const double dth = t[j + 1] - t[j], dt2 = dth * dth, dti = 1. / dth;
        dtS[j] = dth, dt2S[j] = dt2, dtiS[j] = dti, dt2iS[j] = 1. / dt2;
    }
    for (int i = 0; i < I - 1; ++i)
    {
        const double dd = d[i + 1] - d[i], dd2 = dd * dd;
        ddS[i] = dd, dd2S[i] = dd2, ddiS[i] = 1. / dd;
    }
    if (!h->helmMem) NNET_CUDA(cudaMalloc(&h->helmMem, host.size() * sizeof(double)));
    NNET_CUDA(cudaMemcpy(h->helmMem, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice));
    const double* D = (const double*)h->helmMem;
    const double* G = D + ncell;
    h->helm         = {D, G, G + I, G + 2 * I, G + 3 * I, G + 4 * I, G + 5 * I, G + 6 * I, G + 7 * I, G + 8 * I};
    h->helmLoaded   = true;
    return NNET_SUCCESS;
}

int nnet_load_helmholtz_table_file(nnet_handle h, const char* path)
{
    if (!h || !path) return fail(NNET_ERR_INVALID, "null argument");
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(NNET_ERR_FILE, std::string("cannot open ") + path);
    std::stringstream ss;
    ss << f.rdbuf();
    std::string s = ss.str();
    constexpr size_t kBinaryBytes = (size_t)21 * HELM_IMAX * HELM_JMAX * sizeof(double);
    if (s.size() == kBinaryBytes && s.find("STR(") == std::string::npos)
    {
        // the binary layout of nnet_load_helmholtz_table (little-endian doubles)
        std::vector<double> tab(kBinaryBytes / sizeof(double));
        std::memcpy(tab.data(), s.data(), kBinaryBytes);
        return nnet_load_helmholtz_table(h, tab.data());
    }
    // accept the STR( ... ) wrapper the reference #includes (helmholtz.cpp:92-94)
    size_t a = s.find("STR(");
    if (a != std::string::npos)
    {
        s        = s.substr(a + 4);
        size_t b = s.rfind(')');
        if (b != std::string::npos) s = s.substr(0, b);
    }
    constexpr int       I = HELM_IMAX, J = HELM_JMAX;
    std::vector<double> tab((size_t)21 * I * J);
    const char*         c   = s.c_str();
    char*               end = nullptr;
    auto                next = [&](double& v) {
        v = std::strtod(c, &end);
        if (end == c) return false;
        c = end;
        return true;
    };
    auto at = [&](int k, int i, int j) -> double& { return tab[((size_t)k * I + i) * J + j]; };
    // f-block: 9 quantities per (j, i); then three 4-quantity blocks (helmholtz.cpp:106-137)
    for (int j = 0; j < J; ++j)
        for (int i = 0; i < I; ++i)
            for (int k = 0; k < 9; ++k)
                if (!next(at(k, i, j))) return fail(NNET_ERR_FILE, "truncated Helmholtz table");
    for (int blk = 0; blk < 3; ++blk)
        for (int j = 0; j < J; ++j)
            for (int i = 0; i < I; ++i)
                for (int k = 0; k < 4; ++k)
                    if (!next(at(9 + 4 * blk + k, i, j))) return fail(NNET_ERR_FILE, "truncated Helmholtz table");
    return nnet_load_helmholtz_table(h, tab.data());
}

int nnet_burn(nnet_handle h, const nnet_burn_args* a, void* stream)
{
    if (!h) return fail(NNET_ERR_INVALID, "null argument");
    const int rc = nnet_gb300::launchBurn(h, a, h->ws, (cudaStream_t)stream, nullptr, 0, nullptr);
    if (rc == NNET_SUCCESS) h->lastStream = (cudaStream_t)stream, h->lastMulti = false;
    return rc;
}

} // extern "C"

int nnet_gb300::Workspace::ensure(size_t need, cudaStream_t st)
{
    if (!counters)
    {
        NNET_CUDA(cudaMalloc(&counters, kCounters * sizeof(unsigned long long)));
        NNET_CUDA(cudaMemset(counters, 0, kCounters * sizeof(unsigned long long)));
    }
    if (need > doubles)
    {
        // grown, never shrunk (as the reference's devData.buffer, parallel_nuclear_net.cu:148)
        NNET_CUDA(cudaStreamSynchronize(st));
        if (scratch) cudaFree(scratch);
        scratch = nullptr, doubles = 0;
        NNET_CUDA(cudaMalloc(&scratch, need * sizeof(double)));
        doubles = need;
    }
    return NNET_SUCCESS;
}

int nnet_gb300::Workspace::ensureStatus(size_t P, cudaStream_t st)
{
    if (P > statusCap)
    {
        NNET_CUDA(cudaStreamSynchronize(st));
        if (status) cudaFree(status);
        status = nullptr, statusCap = 0;
        NNET_CUDA(cudaMalloc(&status, P * sizeof(int32_t)));
        statusCap = P;
    }
    return NNET_SUCCESS;
}

int nnet_gb300::Workspace::ensureMig(size_t cells, cudaStream_t st)
{
    if (cells > migCap)
    {
        NNET_CUDA(cudaStreamSynchronize(st));
        if (mig) cudaFree(mig);
        mig = nullptr, migCap = 0;
        NNET_CUDA(cudaMalloc(&mig, cells * sizeof(MigCell)));
        migCap = cells;
    }
    return NNET_SUCCESS;
}

void nnet_gb300::Workspace::release()
{
    if (scratch) cudaFree(scratch);
    if (counters) cudaFree(counters);
    if (status) cudaFree(status);
    if (mig) cudaFree(mig);
    scratch = nullptr, counters = nullptr, doubles = 0, status = nullptr, statusCap = 0, mig = nullptr, migCap = 0;
}

int nnet_gb300::launchPostBurn(const BurnParams& bp, const NetView& nv, const HelmView& hv, int numSMs,
                               cudaStream_t st)
{
    if (!bp.postSteps() || bp.P == 0) return NNET_SUCCESS;
    const int    block  = 128;
    const size_t blocks = std::min<size_t>((bp.P + block - 1) / block, (size_t)numSMs * 16);
    postBurnKernel<<<(unsigned)blocks, block, 0, st>>>(bp, nv, hv);
    NNET_CUDA(cudaGetLastError());
    return NNET_SUCCESS;
}

int nnet_gb300::occupancy(const KernelInfo& ki, int& perSM)
{
    if (ki.smem > 48 * 1024)
        NNET_CUDA(cudaFuncSetAttribute(ki.func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ki.smem));
    NNET_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, ki.func, ki.block, ki.smem));
    return NNET_SUCCESS;
}

KernelInfo nnet_gb300::burnKernel(nnet_context* h, int net, int eos, int solver, bool post)
{
    if (solver == NNET_SOLVER_DENSE_FP64) return denseKernel(net, eos);
    const int mixed = solver == NNET_SOLVER_MIXED;
    if (h->layout == NNET_LAYOUT_THREAD) return sparseKernel(net, eos, mixed);
    if (h->layout == NNET_LAYOUT_WARP) return warpKernel(net, eos, mixed);
    return batchKernel(net, eos, mixed, post);
}

size_t nnet_gb300::maxScratchDoubles(nnet_context* h, int solver)
{
    size_t m = 0;
    for (int net : {14, 86, 87})
        for (int eos : {0, 1})
        {
            const KernelInfo ki = burnKernel(h, net, eos, solver);
            if (!ki.perSlot) continue;
            int perSM = 0;
            if (occupancy(ki, perSM) != NNET_SUCCESS) perSM = 1;
            m = std::max(m, (size_t)h->numSMs * std::max(perSM, 1) * ki.block * ki.perSlot);
        }
    return m;
}

namespace
{
int validate(nnet_context* h, const nnet_burn_args* a)
{
    if (!h || !a) return fail(NNET_ERR_INVALID, "null argument");
    if (netIndex(a->network) < 0) return fail(NNET_ERR_INVALID, "unknown network");
    if (a->eos != NNET_EOS_IDEAL_GAS && a->eos != NNET_EOS_HELMHOLTZ) return fail(NNET_ERR_INVALID, "unknown eos");
    if (a->eos == NNET_EOS_HELMHOLTZ && !h->helmLoaded)
        return fail(NNET_ERR_NO_TABLE, "Helmholtz EOS requested before nnet_load_helmholtz_table");
    if (a->eos == NNET_EOS_IDEAL_GAS && !(a->ideal_gas_mu > 0)) return fail(NNET_ERR_INVALID, "ideal_gas_mu must be > 0");
    if (a->solver < NNET_SOLVER_DENSE_FP64 || a->solver > NNET_SOLVER_MIXED) return fail(NNET_ERR_INVALID, "unknown solver");
    if (a->num_particles == 0) return NNET_SUCCESS;
    if (!a->Y || !a->T || !a->rho || !a->dt) return fail(NNET_ERR_INVALID, "null particle array");
    for (int j = 0; j < a->network; ++j)
        if (!a->Y[j]) return fail(NNET_ERR_INVALID, "null species pointer");
    if (!(a->hydro_dt > 0)) return fail(NNET_ERR_INVALID, "hydro_dt must be > 0");
    if (a->use_drhodt && !(a->previous_dt != 0)) return fail(NNET_ERR_INVALID, "use_drhodt needs previous_dt != 0");
    const int eosOut = !!a->u + !!a->cv + !!a->p + !!a->c + !!a->dpdT;
    if (eosOut != 0 && eosOut != 5) return fail(NNET_ERR_INVALID, "post-burn EOS needs all of u, cv, p, c, dpdT");
    if (eosOut && !h->helmLoaded) return fail(NNET_ERR_NO_TABLE, "post-burn EOS requested before a Helmholtz table");
    if (!(a->time_limit_seconds <= 0) && !(a->time_limit_seconds < 1e9))
        return fail(NNET_ERR_INVALID, "time_limit_seconds must be finite");
    if (a->num_particles > 0xffffffffull && a->order)
        return fail(NNET_ERR_TOO_LARGE, "a visiting order holds 32-bit indices");
    return NNET_SUCCESS;
}

void fillParams(const nnet_burn_args* a, unsigned long long* counters, BurnParams& bp)
{
    bp   = BurnParams{};
    bp.P = a->num_particles;
    for (int j = 0; j < a->network; ++j)
        bp.Y[j] = a->Y[j];
    bp.T = a->T, bp.rho = a->rho, bp.rhoM1 = a->rho_m1, bp.dt = a->dt;
    bp.hydroDt = a->hydro_dt, bp.previousDt = a->previous_dt, bp.mu = a->ideal_gas_mu;
    bp.useDrhodt = a->use_drhodt && a->rho_m1;
    bp.maxIter   = a->max_newton_iterations > 0 ? a->max_newton_iterations : 100000;
    bp.status = a->status, bp.substeps = a->substeps, bp.iterations = a->iterations;
    bp.queue = counters, bp.stats = counters + 1, bp.order = a->order;
    bp.timeLimitNs = a->time_limit_seconds > 0 ? std::max(1ull, (unsigned long long)(a->time_limit_seconds * 1e9)) : 0;
    bp.normalize = a->normalize_mass != 0, bp.massDrift = a->mass_drift;
    bp.eosU = a->u, bp.eosCv = a->cv, bp.eosP = a->p, bp.eosC = a->c, bp.eosDpdT = a->dpdT;
}

// persistent grid of `ki` for P particles: (blocks, slots)
int gridFor(nnet_context* h, const KernelInfo& ki, size_t P, size_t& blocks, size_t& slots)
{
    int perSM = 0;
    if (int rc = occupancy(ki, perSM)) return rc;
    if (perSM < 1) return fail(NNET_ERR_TOO_LARGE, "burn kernel does not fit on an SM");
    const size_t maxBlocks = (size_t)h->numSMs * perSM;
    const size_t perBlock  = ki.block / ki.lanesPerParticle; // particles in flight per block
    const size_t need      = (P + perBlock - 1) / perBlock;
    blocks                 = need < maxBlocks ? need : maxBlocks;
    slots                  = blocks * ki.block;
    return NNET_SUCCESS;
}
} // namespace

int nnet_gb300::launchBurn(nnet_context* h, const nnet_burn_args* a, Workspace& ws, cudaStream_t st,
                           const ResumeState* rs, long long sliceIters, unsigned long long* segFinished)
{
    if (int rc = validate(h, a)) return rc;
    if (a->num_particles == 0) return NNET_SUCCESS;
    NNET_CUDA(cudaSetDevice(h->device));
    const int  ni = netIndex(a->network);
    const bool post = a->normalize_mass || a->mass_drift || a->u;
    const KernelInfo ki = burnKernel(h, a->network, a->eos, a->solver, post);
    if (ki.maxNnz && h->nets[ni].plan.nnz > ki.maxNnz)
        return fail(NNET_ERR_TOO_LARGE, "sparse factor does not fit the kernel's storage");
    size_t blocks, slots;
    if (int rc = gridFor(h, ki, a->num_particles, blocks, slots)) return rc;
    if (int rc = ws.ensure(slots * ki.perSlot, st)) return rc;

    BurnParams bp;
    fillParams(a, ws.counters, bp);
    if (rs) bp.rs = *rs;
    bp.sliceIters = sliceIters, bp.segOf = nullptr, bp.segFinished = segFinished;
    bp.laneSlots  = h->laneSlots;
    if (sliceIters > 0 && bp.postSteps())
        return fail(NNET_ERR_INVALID, "post-burn steps are not available for sliced (served) launches");
    const bool postPass = bp.postSteps() && !ki.fusedPost;
    if (postPass && !bp.status)
    {
        if (int rc = ws.ensureStatus(a->num_particles, st)) return rc;
        bp.status = ws.status;
    }

    // batched layout: rebalancing of the running particles over the warps once the queue has
    // drained (not for the server's resumable slices, which rebalance at every slice)
    if (ki.fusedPost && !rs && sliceIters <= 0 && h->rebalance)
    {
        const size_t cells = kMigRecordsPerSlot * slots;
        if (int rc = ws.ensureMig(cells, st)) return rc;
        NNET_CUDA(cudaMemsetAsync(ws.mig, 0, cells * sizeof(MigCell), st));
        bp.migCells = ws.mig, bp.migCap = cells, bp.migCount = ws.counters + kMigCounterWord;
    }
    NNET_CUDA(cudaMemsetAsync(ws.counters, 0, kCounters * sizeof(unsigned long long), st));
    NetView  nv     = h->nets[ni].view;
    HelmView hv     = h->helm;
    double*  sc     = ws.scratch;
    size_t   stride = slots;
    void*    args[] = {&bp, &nv, &hv, &sc, &stride};
    NNET_CUDA(cudaLaunchKernel(ki.func, dim3((unsigned)blocks), dim3(ki.block), args, ki.smem, st));
    if (postPass) return launchPostBurn(bp, nv, hv, h->numSMs, st);
    return NNET_SUCCESS;
}

extern "C" int nnet_set_rebalance(nnet_handle h, int on)
{
    if (!h) return fail(NNET_ERR_INVALID, "null handle");
    h->rebalance = on != 0;
    return NNET_SUCCESS;
}

extern "C" int nnet_set_batch_slots(nnet_handle h, int slots)
{
    if (!h) return fail(NNET_ERR_INVALID, "null handle");
    if (slots < 1 || slots > 32) return fail(NNET_ERR_INVALID, "slots per warp must be in 1..32");
    h->laneSlots = slots;
    return NNET_SUCCESS;
}

// shared with the other translation units of the C ABI
int nnet_gb300::validateBurn(nnet_context* h, const nnet_burn_args* a) { return validate(h, a); }
void nnet_gb300::fillBurnParams(const nnet_burn_args* a, unsigned long long* counters, BurnParams& bp)
{
    fillParams(a, counters, bp);
}
int nnet_gb300::setError(int code, const char* msg) { return fail(code, msg); }

extern "C" int nnet_set_layout(nnet_handle h, int layout)
{
    if (!h) return fail(NNET_ERR_INVALID, "null handle");
    if (layout < NNET_LAYOUT_AUTO || layout > NNET_LAYOUT_BATCHED) return fail(NNET_ERR_INVALID, "unknown layout");
    h->layout = layout;
    return NNET_SUCCESS;
}

extern "C" int nnet_burn_batch(nnet_handle h, const nnet_burn_args* batches, int count, void* stream)
{
    if (!h || !batches || count < 1 || count > 3) return fail(NNET_ERR_INVALID, "need 1 to 3 sub-batches");
    MultiParams mp{};
    size_t      total = 0;
    for (int k = 0; k < count; ++k)
    {
        const nnet_burn_args* a = batches + k;
        if (int rc = validate(h, a)) return rc;
        if (a->eos != batches[0].eos || a->solver != batches[0].solver)
            return fail(NNET_ERR_INVALID, "sub-batches must share the EOS and the solver");
        const int ni = netIndex(a->network);
        if (mp.active[ni]) return fail(NNET_ERR_INVALID, "at most one sub-batch per network");
        mp.active[ni] = a->num_particles > 0;
        mp.nv[ni]     = h->nets[ni].view;
        total += a->num_particles;
    }
    if (total == 0) return NNET_SUCCESS;
    NNET_CUDA(cudaSetDevice(h->device));
    cudaStream_t st   = (cudaStream_t)stream;
    bool         post = false;
    for (int k = 0; k < count; ++k)
        post |= batches[k].num_particles > 0 && (batches[k].normalize_mass || batches[k].mass_drift || batches[k].u);
    const bool tpp = batches[0].solver == NNET_SOLVER_DENSE_FP64 || h->layout == NNET_LAYOUT_THREAD;
    KernelInfo ki  = tpp ? multiKernel(batches[0].eos, batches[0].solver)
                         : batchMultiKernel(batches[0].eos, batches[0].solver == NNET_SOLVER_MIXED, post);
    for (int ni = 0; ni < 3; ++ni)
        if (mp.active[ni] && ki.maxNnz && h->nets[ni].plan.nnz > ki.maxNnz)
            return fail(NNET_ERR_TOO_LARGE, "sparse factor does not fit the kernel's storage");
    size_t blocks, slots;
    if (int rc = gridFor(h, ki, total, blocks, slots)) return rc;
    if (int rc = h->ws.ensure(slots * ki.perSlot, st)) return rc;
    const bool postPass = post && !ki.fusedPost;
    if (postPass)
        if (int rc = h->ws.ensureStatus(total, st)) return rc;
    size_t statusOff = 0;
    for (int k = 0; k < count; ++k)
    {
        const int ni = netIndex(batches[k].network);
        fillParams(batches + k, h->ws.counters + kNetCounters * (ni + 1), mp.bp[ni]);
        mp.bp[ni].laneSlots = h->laneSlots;
        if (postPass && mp.bp[ni].postSteps() && !mp.bp[ni].status)
            mp.bp[ni].status = h->ws.status + statusOff, statusOff += batches[k].num_particles;
    }
    NNET_CUDA(cudaMemsetAsync(h->ws.counters, 0, kCounters * sizeof(unsigned long long), st));
    HelmView hv     = h->helm;
    double*  sc     = h->ws.scratch;
    size_t   stride = slots;
    void*    args[] = {&mp, &hv, &sc, &stride};
    NNET_CUDA(cudaLaunchKernel(ki.func, dim3((unsigned)blocks), dim3(ki.block), args, ki.smem, st));
    h->lastStream = st;
    h->lastMulti  = true;
    if (postPass)
        for (int ni = 0; ni < 3; ++ni)
            if (mp.active[ni])
                if (int rc = launchPostBurn(mp.bp[ni], mp.nv[ni], hv, h->numSMs, st)) return rc;
    return NNET_SUCCESS;
}

extern "C" {

int nnet_get_stats(nnet_handle h, nnet_stats* out)
{
    if (!h || !out) return fail(NNET_ERR_INVALID, "null argument");
    NNET_CUDA(cudaSetDevice(h->device));
    NNET_CUDA(cudaStreamSynchronize(h->lastStream));
    unsigned long long all[kCounters], v[kNetCounters] = {};
    NNET_CUDA(cudaMemcpy(all, h->ws.counters, sizeof all, cudaMemcpyDeviceToHost));
    for (int r = h->lastMulti ? 1 : 0; r < (h->lastMulti ? 4 : 1); ++r)
        for (int k = 0; k < kNetCounters; ++k)
            v[k] += all[r * kNetCounters + k];
    const unsigned long long* w = v + 1; // [0] is the queue head
    out->newton_iterations = w[kStatIters];
    out->substeps          = w[kStatSubsteps];
    for (int s = 0; s < kNumStatus; ++s)
        out->status_count[s] = w[kStatStatus + s];
    out->refinement_steps = w[kStatRefine];
    out->fp64_fallbacks   = w[kStatFallback];
    if (out->status_count[ST_ABORTED])
        return fail(NNET_ERR_ABORTED, "the last launch stopped at its time limit (time_limit_seconds)");
    return NNET_SUCCESS;
}

int nnet_helmholtz_eos(nnet_handle h, size_t num_particles, int num_species, const double* Z, const double* T,
                       const double* rho, double* const* Y, double* u, double* cv, double* p, double* c, double* dpdT,
                       void* stream)
{
    if (!h || !Z || !T || !rho || !Y || !u || !cv || !p || !c || !dpdT) return fail(NNET_ERR_INVALID, "null argument");
    if (num_species < 1 || num_species > NNET_MAX_SPECIES) return fail(NNET_ERR_INVALID, "bad species count");
    if (!h->helmLoaded) return fail(NNET_ERR_NO_TABLE, "no Helmholtz table loaded");
    if (num_particles == 0) return NNET_SUCCESS;
    NNET_CUDA(cudaSetDevice(h->device));
    EosParams ep{};
    ep.P = num_particles, ep.dim = num_species, ep.T = T, ep.rho = rho;
    for (int j = 0; j < num_species; ++j)
        ep.Z[j] = Z[j], ep.Y[j] = Y[j];
    ep.u = u, ep.cv = cv, ep.p = p, ep.c = c, ep.dpdT = dpdT;
    const int    block  = 128;
    const size_t blocks = std::min<size_t>((num_particles + block - 1) / block, (size_t)h->numSMs * 16);
    helmholtzEosKernel<<<(unsigned)blocks, block, 0, (cudaStream_t)stream>>>(ep, h->helm);
    NNET_CUDA(cudaGetLastError());
    return NNET_SUCCESS;
}

} // extern "C"
