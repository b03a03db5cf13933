// One-GPU integral-build server: continuous batching of cutc_int requests.
//
// No counterpart in the reference (CuTC serves one synchronous call at a
// time).  Requests of any molecule, basis and grid size are submitted from
// any thread and complete asynchronously:
//   * n_slots workers each own an execution context (stream,
//     events, workspace); a free worker takes the first queued request whose
//     device footprint fits the memory budget, so later small requests are
//     admitted while an earlier large one waits for memory, and requests in
//     flight on different streams overlap on the GPU;
//   * the molecule arrays (grids, weights, nuclei, AO values) of requests that
//     carry a molecule key stay resident in a byte-budgeted LRU cache, so a
//     request that repeats a molecule with new Jastrow parameters copies only
//     those parameters to the device;
//   * every request records submit / start / end times; the server reports
//     p50 / p99 latency and throughput.
// Results do not depend on the mix: each request runs the same kernels on the
// same data in its own context.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "aos.cuh"
#include "common.cuh"
#include "engine.cuh"

namespace cutc {

using Clock = std::chrono::steady_clock;

struct MolEntry {
    uint64_t key = 0;
    int n1 = 0, n2 = 0, nA = 0, nN = 0;
    double *buf = nullptr;  // r1 | wr1 | r2 | wr2 | rn | aos1 (4 comps) | aos2 value comp
    size_t bytes = 0;
    int refs = 0;
    bool ready = false;   // upload finished (successfully or not)
    bool failed = false;  // upload failed: the entry holds no data
    double *r1, *wr1, *r2, *wr2, *rn, *aos1, *aos2v;
};

struct Job {
    uint64_t ticket = 0;
    cutc_request req{};
    size_t footprint = 0;
    int status = 1;  // 1 = pending
    Clock::time_point t_submit, t_start, t_end;
    bool cache_hit = false;
    std::string message;  // the worker's error message when status is non-zero
};

struct Server {
    int device = 0;
    cutc_server_config cfg{};
    std::vector<Engine *> slots;
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job *> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs;
    uint64_t next_ticket = 1;
    bool stopping = false;
    size_t reserved = 0;  // footprints of requests in flight
    int in_flight = 0, peak_in_flight = 0;
    // molecule cache (LRU by list order, front = most recent)
    std::list<MolEntry *> lru;
    std::unordered_map<uint64_t, MolEntry *> mols;
    size_t cache_bytes = 0;
    long cache_hits = 0, cache_misses = 0;
    // completed-request statistics
    std::vector<double> latencies_ms;
    Clock::time_point t_first_submit, t_last_end;
    bool any_submit = false;
    long completed = 0, failed = 0;
};

static size_t mol_bytes(int n1, int n2, int nA, int nN)
{
    return ((size_t)4 * n1 + 4 * (size_t)n2 + 3 * (size_t)nN + 4 * (size_t)n1 * nA +
            (size_t)n2 * nA) * sizeof(double);
}

// Drops unreferenced molecules, least recently used first, until `need` more
// bytes fit in the cache budget; their device buffers go to `to_free`, which the
// caller frees after releasing the lock (cudaFree waits for the device, and the
// other workers must not wait for it too).  Called with the lock held.
static void evict_for(Server *S, size_t need, std::vector<void *> &to_free)
{
    for (auto it = S->lru.end(); it != S->lru.begin() && S->cache_bytes + need > S->cfg.cache_budget_bytes;) {
        --it;
        MolEntry *m = *it;
        if (m->refs == 0) {
            to_free.push_back(m->buf);
            S->cache_bytes -= m->bytes;
            S->mols.erase(m->key);
            it = S->lru.erase(it);
            delete m;
        }
    }
}

// Returns a referenced cache entry holding the molecule of the request, with
// its arrays on the device (uploaded on the worker's stream if new).
static int acquire_molecule(Server *S, Engine *E, const cutc_request &q, MolEntry **out, bool *hit)
{
    MolEntry *m = nullptr;
    bool upload = false;
    std::vector<void *> to_free;  // evicted buffers, freed once the lock is released
    {
        std::unique_lock<std::mutex> lk(S->mu);
        auto it = S->mols.find(q.molecule_key);
        if (it != S->mols.end() && it->second->n1 == q.n_grid1 && it->second->n2 == q.n_grid2 &&
            it->second->nA == q.n_ao && it->second->nN == q.n_nuc) {
            m = it->second;
            m->refs++;
            S->lru.remove(m);
            S->lru.push_front(m);
            S->cache_hits++;
            *hit = true;
            // another worker may still be uploading it
            S->cv_done.wait(lk, [&] { return m->ready; });
            if (m->failed) {
                m->refs--;
                cutc_set_error(CUTC_ERR_NO_MEMORY, "molecule upload failed in another request");
                return CUTC_ERR_NO_MEMORY;
            }
        } else {
            const size_t bytes = mol_bytes(q.n_grid1, q.n_grid2, q.n_ao, q.n_nuc);
            evict_for(S, bytes, to_free);
            m = new MolEntry();
            m->key = q.molecule_key;
            m->n1 = q.n_grid1; m->n2 = q.n_grid2; m->nA = q.n_ao; m->nN = q.n_nuc;
            m->bytes = bytes;
            m->refs = 1;
            if (it != S->mols.end()) {  // same key, different shape: replace when unreferenced
                MolEntry *old = it->second;
                S->mols.erase(it);
                if (old->refs == 0) {
                    S->lru.remove(old);
                    S->cache_bytes -= old->bytes;
                    to_free.push_back(old->buf);
                    delete old;
                }
            }
            S->mols[m->key] = m;
            S->lru.push_front(m);
            S->cache_bytes += bytes;
            S->cache_misses++;
            *hit = false;
            upload = true;
        }
    }
    for (void *p : to_free)
        cudaFree(p);
    if (upload) {
        auto finish = [&](int status) {
            std::lock_guard<std::mutex> lk(S->mu);
            m->ready = true;
            if (status != CUTC_OK) {
                m->failed = true;
                m->refs--;
            }
            S->cv_done.notify_all();
            return status;
        };
        cudaError_t e = cudaMalloc(&m->buf, m->bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            m->buf = nullptr;
            cutc_set_error(CUTC_ERR_NO_MEMORY, "molecule cache allocation of %zu bytes", m->bytes);
            return finish(CUTC_ERR_NO_MEMORY);
        }
        double *b = m->buf;
        const size_t n1 = q.n_grid1, n2 = q.n_grid2, nA = q.n_ao, nN = q.n_nuc;
        m->r1 = b; b += 3 * n1;
        m->wr1 = b; b += n1;
        m->r2 = b; b += 3 * n2;
        m->wr2 = b; b += n2;
        m->rn = b; b += 3 * nN;
        m->aos1 = b; b += 4 * n1 * nA;
        m->aos2v = b;
        cudaStream_t st = E->stream;
        struct { double *dst; const double *src; size_t n; } cp[] = {
            {m->r1, q.r1, 3 * n1}, {m->wr1, q.wr1, n1}, {m->r2, q.r2, 3 * n2}, {m->wr2, q.wr2, n2},
            {m->rn, q.rn, 3 * nN}, {m->aos1, q.aos_data1, 4 * n1 * nA}, {m->aos2v, q.aos_data2, n2 * nA}};
        for (auto &c : cp)
            if (e == cudaSuccess && c.src)  // AO arrays may come from the basis
                e = cudaMemcpyAsync(c.dst, c.src, c.n * sizeof(double), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            cutc_set_error(CUTC_ERR_CUDA, "molecule upload: %s", cudaGetErrorString(e));
            return finish(CUTC_ERR_CUDA);
        }
        if (!q.aos_data1 || !q.aos_data2) {
            BasisDev B;
            int s = upload_basis(E->ws, 170, st, q.options.basis, &B);
            if (s == CUTC_OK && !q.aos_data1)
                s = launch_eval_aos(st, B, q.n_grid1, m->r1, 4, m->aos1, q.n_grid1);
            if (s == CUTC_OK && !q.aos_data2)
                s = launch_eval_aos(st, B, q.n_grid2, m->r2, 1, m->aos2v, q.n_grid2);
            if (s != CUTC_OK)
                return finish(s);
        }
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            cutc_set_error(CUTC_ERR_CUDA, "molecule upload: %s", cudaGetErrorString(e));
            return finish(CUTC_ERR_CUDA);
        }
        finish(CUTC_OK);
    }
    *out = m;
    return CUTC_OK;
}

static void release_molecule(Server *S, MolEntry *m)
{
    void *to_free = nullptr;  // freed after the lock is released
    {
        std::lock_guard<std::mutex> lk(S->mu);
        m->refs--;
        auto it = S->mols.find(m->key);
        if (it == S->mols.end() || it->second != m) {
            if (m->refs == 0) {  // replaced while in use
                S->lru.remove(m);
                S->cache_bytes -= m->bytes;
                to_free = m->buf;
                delete m;
            }
        }
    }
    if (to_free)
        cudaFree(to_free);
}

static Request to_request(const cutc_request &q)
{
    Request R;
    const cutc_options &o = q.options;
    R.precision = o.precision;
    R.n_slices = o.n_slices;
    R.a_en = o.a_en;
    R.a_ee = o.a_ee;
    R.x_components = o.x_components;
    R.pair_fp64 = o.pair_fp64;
    R.k_split = o.k_split;
    R.int2e_layout = o.int2e_layout;
    R.basis = o.basis;
    R.n1 = q.n_grid1; R.n2 = q.n_grid2; R.nA = q.n_ao; R.nN = q.n_nuc; R.nB = q.size_bh;
    R.r1 = q.r1; R.wr1 = q.wr1; R.r2 = q.r2; R.wr2 = q.wr2; R.rn = q.rn;
    R.aos1 = q.aos_data1; R.aos2 = q.aos_data2;
    R.c_bh = q.c_bh; R.m_bh = q.m_bh; R.n_bh = q.n_bh; R.o_bh = q.o_bh;
    R.X = q.int2_grad1_u12_ao; R.I = q.int_2e_ao;
    return R;
}

static void worker(Server *S, int slot)
{
    cudaSetDevice(S->device);
    Engine *E = S->slots[slot];
    for (;;) {
        Job *job = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            for (;;) {
                if (S->stopping && S->queue.empty())
                    return;
                // first queued request that fits next to the ones in flight
                for (auto it = S->queue.begin(); it != S->queue.end(); ++it) {
                    if (S->reserved + (*it)->footprint <= S->cfg.device_budget_bytes ||
                        S->in_flight == 0) {
                        job = *it;
                        S->queue.erase(it);
                        break;
                    }
                }
                if (job)
                    break;
                S->cv_work.wait(lk);
            }
            S->reserved += job->footprint;
            S->in_flight++;
            S->peak_in_flight = std::max(S->peak_in_flight, S->in_flight);
            job->t_start = Clock::now();
        }
        Request R = to_request(job->req);
        R.max_work_bytes = S->cfg.tile_budget_bytes;
        int status = CUTC_OK;
        MolEntry *m = nullptr;
        if (job->req.molecule_key != 0) {
            bool hit = false;
            status = acquire_molecule(S, E, job->req, &m, &hit);
            job->cache_hit = hit;
            if (status != CUTC_OK)
                m = nullptr;  // no reference is held
            if (status == CUTC_OK) {
                R.r1 = m->r1; R.wr1 = m->wr1; R.r2 = m->r2; R.wr2 = m->wr2; R.rn = m->rn;
                R.aos1 = m->aos1; R.aos2 = m->aos2v;
                R.in_device = 1;
            }
        }
        if (status == CUTC_OK)
            status = run_build(E, R, nullptr);
        std::string message;
        if (status != CUTC_OK) {
            message = cutc_last_error();  // this worker thread's message, for the waiter
            cudaStreamSynchronize(E->stream);
        }
        if (m)
            release_molecule(S, m);
        bool release = false;
        const size_t footprint = job->footprint;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            job->t_end = Clock::now();
            job->message = message;
            job->status = status;  // job may be freed by its waiter from here on
            if (status == CUTC_OK) {
                S->completed++;
                S->latencies_ms.push_back(
                    std::chrono::duration<double, std::milli>(job->t_end - job->t_submit).count());
            } else {
                S->failed++;
            }
            S->t_last_end = job->t_end;
            // an idle context keeps no memory while others wait for it
            release = !S->queue.empty() &&
                      S->reserved - footprint + S->queue.front()->footprint > S->cfg.device_budget_bytes;
        }
        S->cv_done.notify_all();  // the result is ready
        if (release) {
            // cudaFree waits for the whole device: done outside the lock, while this
            // request's reservation still covers the memory being freed
            E->ws.release();
            E->tag_x = E->tag_i = 0;
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->reserved -= footprint;
            S->in_flight--;
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
}

}  // namespace cutc

using namespace cutc;

extern "C" void cutc_server_default_config(cutc_server_config *cfg)
{
    memset(cfg, 0, sizeof(*cfg));
    cfg->n_slots = 4;
    cfg->device_budget_bytes = 0;      // 0: 3/4 of free memory at creation
    cfg->cache_budget_bytes = 0;       // 0: 1/4 of the device budget
    cfg->tile_budget_bytes = (size_t)8 << 30;
}

extern "C" int cutc_server_create(const cutc_server_config *cfg_in, cutc_server **out)
{
    if (!out) {
        cutc_set_error(CUTC_ERR_INVALID, "NULL server handle");
        return CUTC_ERR_INVALID;
    }
    cutc_server_config cfg;
    if (cfg_in)
        cfg = *cfg_in;
    else
        cutc_server_default_config(&cfg);
    if (cfg.n_slots < 1 || cfg.n_slots > 64) {
        cutc_set_error(CUTC_ERR_INVALID, "n_slots must be in [1, 64]");
        return CUTC_ERR_INVALID;
    }
    Engine *E0 = nullptr;
    CUTC_TRY(get_engine(&E0));  // checks the device
    size_t free_b = 0, total_b = 0;
    CUTC_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    if (cfg.device_budget_bytes == 0)
        cfg.device_budget_bytes = free_b / 4 * 3;
    if (cfg.cache_budget_bytes == 0)
        cfg.cache_budget_bytes = cfg.device_budget_bytes / 4;
    if (cfg.tile_budget_bytes == 0)
        cfg.tile_budget_bytes = (size_t)8 << 30;
    Server *S = new Server();
    S->device = E0->device;
    S->cfg = cfg;
    for (int i = 0; i < cfg.n_slots; i++) {
        Engine *E = nullptr;
        int s = make_engine(S->device, &E);
        if (s != CUTC_OK) {
            for (auto e : S->slots)
                destroy_engine(e);
            delete S;
            return s;
        }
        S->slots.push_back(E);
    }
    for (int i = 0; i < cfg.n_slots; i++)
        S->threads.emplace_back(worker, S, i);
    *out = reinterpret_cast<cutc_server *>(S);
    return CUTC_OK;
}

extern "C" int cutc_server_submit(cutc_server *h, const cutc_request *req, unsigned long long *ticket)
{
    Server *S = reinterpret_cast<Server *>(h);
    if (!S || !req || !ticket) {
        cutc_set_error(CUTC_ERR_INVALID, "NULL argument");
        return CUTC_ERR_INVALID;
    }
    if ((!req->aos_data1 || !req->aos_data2))
        CUTC_TRY(validate_basis(req->options.basis, req->n_ao));
    if (req->options.r1_begin != 0 || req->options.r1_end != 0) {
        cutc_set_error(CUTC_ERR_INVALID, "the server builds whole r1 grids (no r1 window)");
        return CUTC_ERR_INVALID;
    }
    auto job = std::make_unique<Job>();
    job->req = *req;
    Request R = to_request(*req);
    R.in_device = req->molecule_key != 0;
    job->footprint = build_footprint(R, S->cfg.tile_budget_bytes);
    job->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stopping) {
        cutc_set_error(CUTC_ERR_INVALID, "server is shutting down");
        return CUTC_ERR_INVALID;
    }
    if (!S->any_submit) {
        S->any_submit = true;
        S->t_first_submit = job->t_submit;
    }
    job->ticket = S->next_ticket++;
    *ticket = job->ticket;
    S->queue.push_back(job.get());
    S->jobs[job->ticket] = std::move(job);
    S->cv_work.notify_one();
    return CUTC_OK;
}

extern "C" int cutc_server_wait(cutc_server *h, unsigned long long ticket, double *latency_ms)
{
    Server *S = reinterpret_cast<Server *>(h);
    if (!S) {
        cutc_set_error(CUTC_ERR_INVALID, "NULL server");
        return CUTC_ERR_INVALID;
    }
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->jobs.find(ticket);
    if (it == S->jobs.end()) {
        cutc_set_error(CUTC_ERR_INVALID, "unknown ticket %llu", ticket);
        return CUTC_ERR_INVALID;
    }
    Job *job = it->second.get();
    S->cv_done.wait(lk, [&] { return job->status != 1; });
    const int st = job->status;
    if (latency_ms)
        *latency_ms = std::chrono::duration<double, std::milli>(job->t_end - job->t_submit).count();
    if (st != CUTC_OK)  // the cause, recorded by the worker, becomes this thread's message
        cutc_set_error(st, "request %llu: %s", ticket, job->message.c_str());
    S->jobs.erase(it);
    return st;
}

extern "C" int cutc_server_get_stats(cutc_server *h, cutc_server_stats *out)
{
    Server *S = reinterpret_cast<Server *>(h);
    if (!S || !out) {
        cutc_set_error(CUTC_ERR_INVALID, "NULL argument");
        return CUTC_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    memset(out, 0, sizeof(*out));
    out->completed = S->completed;
    out->failed = S->failed;
    out->queued = (long)S->queue.size();
    out->in_flight = S->in_flight;
    out->peak_in_flight = S->peak_in_flight;
    out->cache_hits = S->cache_hits;
    out->cache_misses = S->cache_misses;
    out->cache_bytes = S->cache_bytes;
    std::vector<double> v = S->latencies_ms;
    if (!v.empty()) {
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) {
            size_t i = (size_t)std::min<double>(v.size() - 1, std::ceil(p * v.size()) - 1);
            return v[i];
        };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->max_ms = v.back();
        const double span = std::chrono::duration<double>(S->t_last_end - S->t_first_submit).count();
        out->builds_per_s = span > 0 ? S->completed / span : 0.0;
    }
    return CUTC_OK;
}

extern "C" void cutc_server_destroy(cutc_server *h)
{
    Server *S = reinterpret_cast<Server *>(h);
    if (!S)
        return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stopping = true;
    }
    S->cv_work.notify_all();
    for (auto &t : S->threads)
        t.join();
    for (auto e : S->slots)
        destroy_engine(e);
    for (auto m : S->lru) {
        cudaFree(m->buf);
        delete m;
    }
    delete S;
}
