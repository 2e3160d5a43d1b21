// Burn server: continuous batching of burn requests on one GPU.
//
// A request (network, EOS, a batch of particles in host memory) is admitted when its
// device footprint fits the HBM budget and a workspace is free; its abundances,
// temperature, density, timestep and substep state then stay resident on the device until
// it completes.  Every admitted request runs as a sequence of slices on its own stream: one
// persistent-kernel launch in which each particle performs at most `slice_iterations`
// Newton iterations and pauses at the next attempt boundary (the pause saves everything
// the next attempt depends on, so results are bit-identical to an unsliced burn).  Slices
// of different requests overlap on the device; a request that arrives while others run is
// admitted at the next scheduling pass, as soon as memory and a workspace free up, instead
// of waiting for the running ones to finish.  Completion = results copied back into the
// caller's host buffers; latency = completion time - submission time.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "context.hpp"

using namespace nnet_gb300;

namespace
{
using Clock = std::chrono::steady_clock;

struct Request
{
    uint64_t     id = 0;
    nnet_request r{};
    size_t       P = 0, bytes = 0;
    int          N = 0;
    enum State
    {
        PENDING,
        RUNNING,
        COPYING,
        DONE,
        FAILED
    } state = PENDING;
    // device
    char*               mem = nullptr;
    double *            Y = nullptr, *T = nullptr, *rho = nullptr, *dt = nullptr;
    int32_t*            status = nullptr;
    ResumeState         rs{};
    int                 ws = -1;
    cudaStream_t        stream = nullptr;
    cudaEvent_t         ev = nullptr;
    unsigned long long* finished    = nullptr; // pinned host copy of the counter below
    unsigned long long* finishedDev = nullptr; // device counter of finished particles
    Clock::time_point   tSubmit, tDone;
    int                 slices = 0;
    std::string         error;
};

size_t requestBytes(int N, size_t P)
{
    // Y, T, rho, dt, elapsed, nextT, drho, nit, cdDt, cdNt (8 B) + status, phase, nsub,
    // cdPower, cdSteps (4 B)
    return P * ((size_t)(N + 10) * 8 + 5 * 4) + 8192;
}
} // namespace

struct nnet_server_s
{
    nnet_context*                  h = nullptr;
    nnet_server_config             cfg{};
    std::vector<Workspace>         ws;
    std::vector<char>              wsBusy;
    std::mutex                     mu;
    std::condition_variable        cv;
    std::deque<Request*>           pending;
    std::vector<Request*>          active;
    std::unordered_map<uint64_t, Request*> all;
    std::vector<double>            latencies;
    uint64_t                       nextId = 1;
    size_t                         bytesInUse = 0;
    bool                           stop = false;
    std::thread                    thread;
    double                         particlesDone = 0;
    Clock::time_point              tFirst, tLast;
    bool                           anyDone = false;
    unsigned long long             slices = 0;
    unsigned long long*            pinned = nullptr; // completion-counter copies, one per workspace

    int  admit(Request* q);
    void launchSlice(Request* q);
    void finish(Request* q);
    void loop();
};

int nnet_server_s::admit(Request* q)
{
    cudaSetDevice(h->device);
    q->bytes = requestBytes(q->N, q->P);
    if (cudaStreamCreateWithFlags(&q->stream, cudaStreamNonBlocking) != cudaSuccess) return -1;
    if (cudaEventCreateWithFlags(&q->ev, cudaEventDisableTiming) != cudaSuccess) return -1;
    if (cudaMallocAsync((void**)&q->mem, q->bytes, q->stream) != cudaSuccess) return -1;
    q->finished  = pinned + q->ws; // one pinned slot per workspace (no allocation per request)
    *q->finished = 0;
    const size_t P = q->P;
    char*        m = q->mem;
    auto         take = [&](size_t bytes) {
        char* p = m;
        m += (bytes + 255) / 256 * 256;
        return p;
    };
    q->Y          = (double*)take(sizeof(double) * P * q->N);
    q->T          = (double*)take(sizeof(double) * P);
    q->rho        = (double*)take(sizeof(double) * P);
    q->dt         = (double*)take(sizeof(double) * P);
    q->rs.elapsed = (double*)take(sizeof(double) * P);
    q->rs.nextT   = (double*)take(sizeof(double) * P);
    q->rs.drho    = (double*)take(sizeof(double) * P);
    q->rs.nit     = (long long*)take(sizeof(long long) * P);
    q->rs.cdDt    = (unsigned long long*)take(8 * P);
    q->rs.cdNt    = (unsigned long long*)take(8 * P);
    q->status     = (int32_t*)take(4 * P);
    q->rs.phase   = (int*)take(4 * P);
    q->rs.nsub    = (int*)take(4 * P);
    q->rs.cdPower = (int*)take(4 * P);
    q->rs.cdSteps = (int*)take(4 * P);
    q->finishedDev = (unsigned long long*)take(sizeof(unsigned long long));
    cudaMemsetAsync(q->finishedDev, 0, sizeof(unsigned long long), q->stream);
    cudaMemcpyAsync(q->Y, q->r.Y, sizeof(double) * P * q->N, cudaMemcpyHostToDevice, q->stream);
    cudaMemcpyAsync(q->T, q->r.T, sizeof(double) * P, cudaMemcpyHostToDevice, q->stream);
    cudaMemcpyAsync(q->rho, q->r.rho, sizeof(double) * P, cudaMemcpyHostToDevice, q->stream);
    cudaMemcpyAsync(q->dt, q->r.dt, sizeof(double) * P, cudaMemcpyHostToDevice, q->stream);
    cudaMemsetAsync(q->rs.phase, 0, 4 * P, q->stream);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

void nnet_server_s::launchSlice(Request* q)
{
    std::vector<double*> Yp(q->N);
    for (int j = 0; j < q->N; ++j)
        Yp[j] = q->Y + (size_t)j * q->P;
    nnet_burn_args a{};
    a.network = q->r.network, a.eos = q->r.eos, a.ideal_gas_mu = q->r.ideal_gas_mu, a.solver = cfg.solver;
    a.num_particles = q->P, a.Y = Yp.data(), a.T = q->T, a.rho = q->rho, a.dt = q->dt;
    a.hydro_dt = q->r.hydro_dt, a.max_newton_iterations = q->r.max_newton_iterations, a.status = q->status;
    const int rc = launchBurn(h, &a, ws[q->ws], q->stream, &q->rs, cfg.slice_iterations, q->finishedDev);
    if (rc != NNET_SUCCESS)
    {
        q->state = Request::FAILED;
        q->error = nnet_last_error_message();
        return;
    }
    cudaMemcpyAsync(q->finished, q->finishedDev, sizeof(unsigned long long), cudaMemcpyDeviceToHost, q->stream);
    cudaEventRecord(q->ev, q->stream);
    ++q->slices, ++slices;
    q->state = Request::RUNNING;
}

void nnet_server_s::finish(Request* q)
{
    const size_t P = q->P;
    cudaMemcpyAsync(q->r.Y, q->Y, sizeof(double) * P * q->N, cudaMemcpyDeviceToHost, q->stream);
    cudaMemcpyAsync(q->r.T, q->T, sizeof(double) * P, cudaMemcpyDeviceToHost, q->stream);
    cudaMemcpyAsync(q->r.dt, q->dt, sizeof(double) * P, cudaMemcpyDeviceToHost, q->stream);
    if (q->r.status) cudaMemcpyAsync(q->r.status, q->status, 4 * P, cudaMemcpyDeviceToHost, q->stream);
    cudaEventRecord(q->ev, q->stream);
    q->state = Request::COPYING;
}

void nnet_server_s::loop()
{
    cudaSetDevice(h->device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;)
    {
        // admission: FIFO, by HBM budget and free workspace
        while (!pending.empty())
        {
            Request* q    = pending.front();
            const size_t b = requestBytes(q->N, q->P);
            int          w = -1;
            for (size_t k = 0; k < ws.size(); ++k)
                if (!wsBusy[k])
                {
                    w = (int)k;
                    break;
                }
            if (w < 0 || (bytesInUse + b > (size_t)cfg.hbm_budget_bytes && !active.empty())) break;
            pending.pop_front();
            wsBusy[w] = 1, q->ws = w;
            bytesInUse += b;
            if (admit(q) != 0)
            {
                q->state = Request::FAILED, q->error = "admission failed (device allocation)";
                wsBusy[w] = 0, bytesInUse -= b;
                cv.notify_all();
                continue;
            }
            active.push_back(q);
            lk.unlock();
            launchSlice(q);
            lk.lock();
        }
        if (active.empty())
        {
            if (stop && pending.empty()) return;
            cv.wait_for(lk, std::chrono::milliseconds(1));
            continue;
        }
        lk.unlock();
        bool progressed = false;
        for (Request* q : active)
        {
            if (q->state == Request::FAILED || q->state == Request::DONE) continue;
            if (cudaEventQuery(q->ev) != cudaSuccess) continue;
            progressed = true;
            if (q->state == Request::RUNNING)
            {
                if (*(volatile unsigned long long*)q->finished >= q->P)
                    finish(q);
                else
                    launchSlice(q);
            }
            else if (q->state == Request::COPYING)
            {
                q->tDone = Clock::now();
                q->state = Request::DONE;
            }
        }
        lk.lock();
        // retire completed / failed requests
        for (size_t k = 0; k < active.size();)
        {
            Request* q = active[k];
            if (q->state == Request::DONE || q->state == Request::FAILED)
            {
                cudaFreeAsync(q->mem, q->stream);
                cudaStreamSynchronize(q->stream);
                cudaEventDestroy(q->ev);
                cudaStreamDestroy(q->stream);
                q->mem = nullptr, q->finished = nullptr;
                wsBusy[q->ws] = 0;
                bytesInUse -= requestBytes(q->N, q->P);
                if (q->state == Request::DONE)
                {
                    latencies.push_back(std::chrono::duration<double>(q->tDone - q->tSubmit).count());
                    particlesDone += (double)q->P;
                    if (!anyDone) tFirst = q->tSubmit, anyDone = true;
                    tLast = q->tDone;
                }
                active[k] = active.back();
                active.pop_back();
                cv.notify_all();
            }
            else
                ++k;
        }
        if (!progressed)
        {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(50));
            lk.lock();
        }
    }
}

extern "C" {

int nnet_server_create(nnet_handle h, const nnet_server_config* cfg, nnet_server* out)
{
    if (!h || !cfg || !out) return NNET_ERR_INVALID;
    if (cfg->max_concurrent_requests < 1 || cfg->max_concurrent_requests > 64) return NNET_ERR_INVALID;
    nnet_server_s* s = new nnet_server_s;
    s->h             = h;
    s->cfg           = *cfg;
    if (s->cfg.slice_iterations <= 0) s->cfg.slice_iterations = 64;
    if (s->cfg.hbm_budget_bytes <= 0) s->cfg.hbm_budget_bytes = 150e9;
    s->ws.resize(cfg->max_concurrent_requests);
    s->wsBusy.assign(cfg->max_concurrent_requests, 0);
    cudaSetDevice(h->device);
    if (cudaMallocHost((void**)&s->pinned, sizeof(unsigned long long) * cfg->max_concurrent_requests) != cudaSuccess)
    {
        delete s;
        return NNET_ERR_CUDA;
    }
    const size_t scratch = maxScratchDoubles(h, cfg->solver);
    for (auto& w : s->ws)
        if (w.ensure(scratch, nullptr) != NNET_SUCCESS)
        {
            for (auto& x : s->ws)
                x.release();
            cudaFreeHost(s->pinned);
            delete s;
            return NNET_ERR_CUDA;
        }
    s->thread = std::thread([s] { s->loop(); });
    *out      = s;
    return NNET_SUCCESS;
}

int nnet_server_submit(nnet_server s, const nnet_request* r, uint64_t* id)
{
    if (!s || !r || !id) return NNET_ERR_INVALID;
    if (r->network != 14 && r->network != 86 && r->network != 87) return NNET_ERR_INVALID;
    if (!r->Y || !r->T || !r->rho || !r->dt || r->num_particles == 0 || !(r->hydro_dt > 0)) return NNET_ERR_INVALID;
    Request* q = new Request;
    q->r       = *r;
    q->P       = r->num_particles;
    q->N       = r->network;
    q->tSubmit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    q->id = s->nextId++;
    s->all[q->id] = q;
    s->pending.push_back(q);
    s->cv.notify_all();
    *id = q->id;
    return NNET_SUCCESS;
}

int nnet_server_query(nnet_server s, uint64_t id, int* done)
{
    if (!s || !done) return NNET_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return NNET_ERR_INVALID;
    *done = it->second->state == Request::DONE ? 1 : it->second->state == Request::FAILED ? -1 : 0;
    return NNET_SUCCESS;
}

int nnet_server_wait(nnet_server s, uint64_t id, double* latency_seconds)
{
    if (!s) return NNET_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return NNET_ERR_INVALID;
    Request* q = it->second;
    s->cv.wait(lk, [&] {
        return (q->state == Request::DONE || q->state == Request::FAILED) &&
               std::find(s->active.begin(), s->active.end(), q) == s->active.end();
    });
    if (latency_seconds) *latency_seconds = std::chrono::duration<double>(q->tDone - q->tSubmit).count();
    const bool ok = q->state == Request::DONE;
    s->all.erase(it);
    delete q;
    return ok ? NNET_SUCCESS : NNET_ERR_CUDA;
}

int nnet_server_get_stats(nnet_server s, nnet_server_stats* out)
{
    if (!s || !out) return NNET_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) { return l.empty() ? 0. : l[std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5))]; };
    out->completed_requests = l.size();
    out->completed_particles = s->particlesDone;
    out->span_seconds = s->anyDone ? std::chrono::duration<double>(s->tLast - s->tFirst).count() : 0.;
    out->latency_p50 = pct(0.50), out->latency_p95 = pct(0.95), out->latency_p99 = pct(0.99);
    out->latency_max = l.empty() ? 0. : l.back();
    out->slices = s->slices;
    return NNET_SUCCESS;
}

int nnet_server_destroy(nnet_server s)
{
    if (!s) return NNET_SUCCESS;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    s->thread.join();
    cudaSetDevice(s->h->device);
    for (auto& w : s->ws)
        w.release();
    cudaFreeHost(s->pinned);
    for (auto& kv : s->all)
        delete kv.second;
    delete s;
    return NNET_SUCCESS;
}

} // extern "C"
