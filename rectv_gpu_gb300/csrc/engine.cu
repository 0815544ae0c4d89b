// Multi-problem engine: the batched form (many slice chunks of uneven size
// solved together) and the serving loop (requests admitted by device memory,
// state resident between iterations, continuous batching), plus the launch-
// shape autotuner.
//
// A job is one reconstruction problem with its own n, ntheta, m, nz, nzp and
// the arguments of rectv::run (src/cuda/rectv.cu:102-252).  The reference
// solves one problem per call and re-zeroes f, fn, psi and mu at the start of
// every run (rectv.cu:119-122); here each admitted job owns a Handle whose
// u, psi, mu, w and rho stay resident in HBM, with its geometry and its
// captured outer-iteration graphs, from admission until its last iteration.
//
// Scheduling.  Jobs are admitted in order of arrival (the batched form:
// largest first; serving may take, among the jobs that have arrived, the one
// with the least work first) when their estimated device memory fits the
// budget and fewer than max_resident jobs are running.  On admission the job's data is
// uploaded and all its outer iterations are queued on the handle's own
// stream as graph launches; the GPU interleaves the kernels of every running
// job, so the iterations of different problems overlap on the device.  The
// host loop polls completion events: a finished job's result is already in
// the caller's buffer (queued copy), its handle goes to an idle pool (reused
// by a later job of the same dimensions, or freed when memory is needed) and
// waiting jobs are admitted at once.  Buffers are stream-ordered allocations
// (cudaMallocAsync / cudaFreeAsync), so jobs come and go without
// synchronising the device.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "handle.cuh"

namespace rectv {
namespace {

using Clock = std::chrono::steady_clock;

// ---------------------------------------------------------------------------
// Launch-shape autotuner
// ---------------------------------------------------------------------------
// Launch shapes that do not change results: slices per block of the
// tensor-core gather (k_gather_tc) and the number of persistent blocks of the
// tensor-core scatter (k_scatter_tc).  Chosen per (device, n, ntheta, m,
// slices per launch) by timing the candidates on a set-up handle, cached for
// the process.
using TuneKey = std::tuple<int, int, int, int, int, int>;  // device, n, ntheta, m, zb, direction path
std::mutex g_tune_mu;
std::map<TuneKey, Tune> g_tune_cache;

int sm_count(int dev) {
    int nsm = 0;
    CUDA_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    return nsm;
}

// Average time of `reps` launches of kernel `which` on the handle's buffers.
double time_kernel(Handle &h, int which, int reps) {
    cudaEvent_t a, b;
    CUDA_CHECK(cudaEventCreate(&a));
    CUDA_CHECK(cudaEventCreate(&b));
    float ms = 0.f;
    try {
        h.launch_kernel(which, 1);  // warm
        CUDA_CHECK(cudaEventRecord(a, h.stream));
        h.launch_kernel(which, reps);
        CUDA_CHECK(cudaEventRecord(b, h.stream));
        CUDA_CHECK(cudaEventSynchronize(b));
        CUDA_CHECK(cudaEventElapsedTime(&ms, a, b));
    } catch (...) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        throw;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return (double)ms / reps;
}

}  // namespace

// Picks the launch shapes for a handle with a set-up session (its geometry
// decides which tensor-core kernels run), applies them (dropping captured
// graphs) and returns them.  Cached per (device, n, ntheta, m, zb).
Tune autotune(Handle &h, bool force) {
    const TuneKey key{h.device, h.n, h.ntheta, h.m, h.zb, h.gd.dirs ? 1 : 0};
    if (!force) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            h.ug.zper = it->second.zper;
            h.ug.sc_grid = it->second.sc_grid;
            h.drop_graphs();
            return it->second;
        }
    }
    Tune best;
    const int reps = 2;
    if (h.gd.n_fwd_tc_items > 0 || h.gd.n_dfwd_items > 0) {  // slices per block of either gather
        double tbest = 1e30;
        for (int zper : {64, 32, 16, 8}) {
            if (zper > 8 && zper >= 2 * h.zb) continue;  // one block covers the batch already
            h.ug.zper = zper;
            const double t = time_kernel(h, 0, reps);
            if (t < tbest * 0.99) {
                tbest = t;
                best.zper = zper;
            }
        }
        best.gather_ms = tbest;
        h.ug.zper = best.zper;
    }
    if (h.gd.tc_scatter) {
        const int nsm = sm_count(h.device);
        double tbest = 1e30;
        // persistent blocks: nsm * frac / 4 (tensor-core scatter, one block per
        // SM at most), nsm * frac / 2 (direction scatter, two per SM at most)
        const int per = h.gd.dirs ? 2 : 4;
        for (int frac : {4, 3, 2}) {
            h.ug.sc_grid = nsm * frac / per;
            const double t = time_kernel(h, 1, reps);
            if (t < tbest * 0.99) {
                tbest = t;
                best.sc_grid = h.ug.sc_grid;
            }
        }
        best.scatter_ms = tbest;
        if (best.sc_grid == nsm * 4 / per) best.sc_grid = 0;
        h.ug.sc_grid = best.sc_grid;
    }
    h.drop_graphs();
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = best;
    return best;
}

namespace {

// ---------------------------------------------------------------------------
// Jobs and the engine
// ---------------------------------------------------------------------------
enum JobState { kWaiting = 0, kRunning = 1, kDone = 2, kFailed = 3 };

struct Job {
    int id = 0;
    int n = 0, ntheta = 0, m = 0, nz = 0, nzp = 0, niter = 0, titer = 0;
    float center = 0, lambda0 = 0, lambda1 = 0;
    const float *g = nullptr, *theta = nullptr, *phi = nullptr;
    float *fres = nullptr;
    double arrival = 0, admitted = -1, done = -1;
    double est_bytes = 0, bytes = 0;
    int state = kWaiting;
    std::string error;
    std::unique_ptr<Handle> h;
    cudaEvent_t ev = nullptr;
    cudaStream_t stream = nullptr;  // the job's stream (priority by age) while it runs
    int priority = 0;
    double acct = 0;                // bytes counted against the budget while it runs
    double rho_final = 0, rdiff_final = 0;
    Tune tune;
};

}  // namespace

struct Engine {
    double budget;
    int max_resident;
    bool reuse;
    bool tune;
    bool largest_first = false;
    bool shortest_first = false;
    bool age_priority = false;
    int prio_least = 0, prio_greatest = 0;  // stream priority range (numerically lower = higher)
    int device = 0;
    std::vector<std::unique_ptr<Job>> jobs;
    std::vector<std::pair<double, std::unique_ptr<Handle>>> idle;  // (time returned, handle)
    double used = 0, peak = 0;
    int running = 0, peak_running = 0;
    double makespan = 0;
    Clock::time_point t0;

    Engine(double budget_, int max_resident_, int flags) {
        CUDA_CHECK(cudaGetDevice(&device));
        if (budget_ <= 0) {
            size_t fr = 0, tot = 0;
            CUDA_CHECK(cudaMemGetInfo(&fr, &tot));
            budget_ = (double)fr - 4.0 * (1ull << 30);
        }
        if (budget_ <= 0) throw Error(RECTV_ERR_NOMEM, "rectv_engine: no device memory for a budget");
        budget = budget_;
        max_resident = max_resident_ > 0 ? max_resident_ : 1 << 30;
        reuse = !(flags & RECTV_ENGINE_NO_REUSE);
        tune = (flags & RECTV_ENGINE_AUTOTUNE) != 0;
        largest_first = (flags & RECTV_ENGINE_LARGEST_FIRST) != 0;
        shortest_first = (flags & RECTV_ENGINE_SHORTEST_FIRST) != 0;
        age_priority = (flags & RECTV_ENGINE_AGE_PRIORITY) != 0;
        CUDA_CHECK(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
    }

    // Stream priority of a newly admitted job: with age priority, below every
    // running job (the oldest runs first, newer jobs fill the SMs it leaves
    // idle), down to the least priority; else the default.
    int next_priority(const std::vector<Job *> &active) const {
        if (!age_priority) return prio_least;
        int p = prio_greatest - 1;
        for (const Job *a : active) p = std::max(p, a->priority);
        return std::min(prio_least, p + 1);
    }

    ~Engine() {
        for (auto &j : jobs)
            if (j->ev) cudaEventDestroy(j->ev);
    }

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

    int submit(int n, int ntheta, int m, int nz, int nzp, const float *g, const float *theta, const float *phi,
               float center, float lambda0, float lambda1, int niter, int titer, double arrival, float *fres) {
        if (!g || !theta || !phi || !fres) throw Error(RECTV_ERR_ARG, "rectv_engine_submit: null pointer");
        if (n < 2 || ntheta < 1 || m < 1 || nz < 1 || nzp < 1 || nzp > nz || niter < 0 || titer < 0)
            throw Error(RECTV_ERR_ARG, "rectv_engine_submit: invalid dimensions or iteration counts");
        if (arrival < 0) throw Error(RECTV_ERR_ARG, "rectv_engine_submit: arrival must be >= 0");
        float mu_us = 0;
        if (detail::usfft_radius(n, &mu_us) != kR) throw Error(RECTV_ERR_ARG, "rectv_engine_submit: USFFT radius != 4");
        auto j = std::make_unique<Job>();
        j->id = (int)jobs.size();
        j->n = n, j->ntheta = ntheta, j->m = m, j->nz = nz, j->nzp = nzp, j->niter = niter, j->titer = titer;
        j->center = center, j->lambda0 = lambda0, j->lambda1 = lambda1;
        j->g = g, j->theta = theta, j->phi = phi, j->fres = fres, j->arrival = arrival;
        j->est_bytes = make_layout(n, ntheta, m, nz, nzp, -1).bytes;
        jobs.push_back(std::move(j));
        return jobs.back()->id;
    }

    static bool same_dims(const Handle &h, const Job &j) {
        return h.n == j.n && h.ntheta == j.ntheta && h.m == j.m && h.nz == j.nz && h.nzp == j.nzp;
    }

    void evict_one() {
        // least recently returned idle handle
        size_t k = 0;
        for (size_t i = 1; i < idle.size(); ++i)
            if (idle[i].first < idle[k].first) k = i;
        used -= (double)idle[k].second->device_bytes();
        idle.erase(idle.begin() + (long)k);  // Handle destructor: stream-ordered frees
    }

    // Admits job j if it fits; false when it has to wait.  Throws on errors
    // that make the job fail.
    bool admit(Job &j, const std::vector<Job *> &active) {
        std::unique_ptr<Handle> h;
        bool fresh = false;
        for (size_t i = 0; i < idle.size(); ++i)
            if (same_dims(*idle[i].second, j)) {
                h = std::move(idle[i].second);
                idle.erase(idle.begin() + (long)i);
                used -= (double)h->device_bytes();
                break;
            }
        if (!h) {
            while (used + j.est_bytes > budget && !idle.empty()) evict_one();
            if (used + j.est_bytes > budget) {
                if (running == 0)
                    throw Error(RECTV_ERR_NOMEM, "rectv_engine: job needs about " + std::to_string(j.est_bytes) +
                                                     " bytes, more than the budget of " + std::to_string(budget));
                return false;
            }
            try {
                h = std::make_unique<Handle>(j.n, j.ntheta, j.m, j.nz, j.nzp, 1);
            } catch (const Error &e) {
                if (e.code == RECTV_ERR_NOMEM && running > 0) return false;  // retry after a completion
                throw;
            }
            fresh = true;
        }
        h->verbose = false;
        // the job's own stream; the handle's earlier work has finished (fresh,
        // or idle after its previous job's completion event)
        const int prio = next_priority(active);
        cudaStream_t st = nullptr;
        CUDA_CHECK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio));
        struct Unbind {  // on any early exit: back to the handle's stream, drop st
            Handle *h;
            cudaStream_t st;
            ~Unbind() {
                if (h) {
                    cudaStreamSynchronize(st);
                    h->bind_stream(nullptr);
                }
                if (st) cudaStreamDestroy(st);
            }
        } guard{h.get(), st};
        h->bind_stream(st);
        const size_t gbytes = sizeof(float) * (size_t)j.nz * j.ntheta * j.n;
        CUDA_CHECK(cudaMemcpyAsync(h->gdata, j.g, gbytes, cudaMemcpyHostToDevice, h->stream));
        h->setup(j.theta, j.phi, j.center, j.lambda0, j.lambda1, j.titer);
        if (fresh && running > 0 && used + (double)h->device_bytes() > budget) {
            // the estimate was short: remember the real size and wait for memory
            j.est_bytes = std::max(j.est_bytes, (double)h->device_bytes());
            return false;
        }
        if (tune) j.tune = autotune(*h, false);
        h->enqueue_iterations(j.niter);
        const size_t nf = (size_t)h->nzc * h->slab;
        CUDA_CHECK(cudaMemcpyAsync(j.fres, h->U[h->cur], sizeof(float) * nf, cudaMemcpyDeviceToHost, h->stream));
        if (!j.ev) CUDA_CHECK(cudaEventCreateWithFlags(&j.ev, cudaEventDisableTiming));
        CUDA_CHECK(cudaEventRecord(j.ev, h->stream));
        guard.h = nullptr;  // the job keeps st until it finishes
        guard.st = nullptr;
        j.stream = st;
        j.priority = prio;
        j.bytes = (double)h->device_bytes();
        j.acct = j.bytes;
        used += j.acct;
        peak = std::max(peak, used);
        j.h = std::move(h);
        j.state = kRunning;
        j.admitted = now();
        ++running;
        peak_running = std::max(peak_running, running);
        return true;
    }

    void release_stream(Job &j) {
        if (!j.stream) return;
        if (j.h) {
            cudaStreamSynchronize(j.stream);
            j.h->bind_stream(nullptr);
        }
        cudaStreamDestroy(j.stream);
        j.stream = nullptr;
    }

    void finish(Job &j) {
        Handle &h = *j.h;
        h.collect_history();
        release_stream(j);
        const size_t nf = (size_t)h.nzc * h.slab, total = (size_t)j.nz * h.slab;
        if (total > nf) std::memset(j.fres + nf, 0, sizeof(float) * (total - nf));
        if (!h.h_rho.empty()) {
            j.rho_final = h.h_rho.back();
            j.rdiff_final = h.h_rdiff.back();
        }
        used -= j.acct;
        j.done = now();
        j.state = kDone;
        --running;
        if (reuse) {
            used += (double)h.device_bytes();
            idle.emplace_back(j.done, std::move(j.h));
        } else {
            j.h.reset();
        }
    }

    void fail(Job &j, const std::string &msg) {
        if (j.state == kRunning) {
            used -= j.acct;
            --running;
        }
        release_stream(j);
        j.h.reset();
        j.state = kFailed;
        j.error = msg;
        j.done = now();
    }

    // Processes every submitted job that has not finished; returns when all
    // are done or failed.  Arrival times count from the start of this call.
    void run() {
        t0 = Clock::now();
        std::vector<Job *> order;
        for (auto &j : jobs)
            if (j->state == kWaiting) order.push_back(j.get());
        std::stable_sort(order.begin(), order.end(), [&](const Job *a, const Job *b) {
            if (a->arrival != b->arrival) return a->arrival < b->arrival;
            if (largest_first) return a->est_bytes * a->niter > b->est_bytes * b->niter;
            return false;
        });
        std::vector<Job *> active, pool;
        size_t next = 0;
        while (next < order.size() || !pool.empty() || !active.empty()) {
            bool progress = false;
            for (size_t i = 0; i < active.size();) {
                Job &j = *active[i];
                const cudaError_t q = cudaEventQuery(j.ev);
                if (q == cudaErrorNotReady) {
                    ++i;
                    continue;
                }
                try {
                    if (q != cudaSuccess) CUDA_CHECK(q);
                    finish(j);
                } catch (const std::exception &e) {
                    fail(j, e.what());
                }
                active.erase(active.begin() + (long)i);
                progress = true;
            }
            const double t = now();
            // jobs that have arrived, in arrival order
            while (next < order.size() && order[next]->arrival <= t) pool.push_back(order[next++]);
            while (!pool.empty() && running < max_resident) {
                // the first in line, or the arrived job with the least work
                size_t pick = 0;
                if (shortest_first)
                    for (size_t i = 1; i < pool.size(); ++i)
                        if (pool[i]->est_bytes * pool[i]->niter < pool[pick]->est_bytes * pool[pick]->niter) pick = i;
                Job &j = *pool[pick];
                bool ok = false;
                try {
                    ok = admit(j, active);
                } catch (const std::exception &e) {
                    fail(j, e.what());
                    pool.erase(pool.begin() + (long)pick);
                    progress = true;
                    continue;
                }
                if (!ok) break;  // the chosen job waits for memory
                active.push_back(&j);
                pool.erase(pool.begin() + (long)pick);
                progress = true;
            }
            if (!progress) {
                double wait = 100e-6;
                if (active.empty() && next < order.size()) wait = std::max(0.0, order[next]->arrival - now());
                std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
            }
        }
        makespan = now();
    }
};

}  // namespace rectv

// ===========================================================================
// C ABI
// ===========================================================================
struct rectv_engine {
    rectv::Engine *e;
};

namespace {
rectv::Engine *live_engine(rectv_engine *e) {
    if (!e || !e->e) throw rectv::Error(RECTV_ERR_ARG, "rectv_engine: null engine");
    return e->e;
}
}  // namespace

extern "C" {

int rectv_engine_create(double hbm_budget_bytes, int max_resident, int flags, rectv_engine **out) {
    return rectv::guarded([&] {
        if (!out) throw rectv::Error(RECTV_ERR_ARG, "rectv_engine_create: null output");
        *out = nullptr;
        auto *e = new rectv::Engine(hbm_budget_bytes, max_resident, flags);
        *out = new rectv_engine{e};
    });
}

int rectv_engine_submit(rectv_engine *e, int n, int ntheta, int m, int nz, int nzp, const float *g,
                        const float *theta, const float *phi, float center, float lambda0, float lambda1, int niter,
                        int titer, double arrival_s, float *fres, int *job_id) {
    return rectv::guarded([&] {
        const int id = live_engine(e)->submit(n, ntheta, m, nz, nzp, g, theta, phi, center, lambda0, lambda1, niter,
                                              titer, arrival_s, fres);
        if (job_id) *job_id = id;
    });
}

int rectv_engine_run(rectv_engine *e) {
    return rectv::guarded([&] { live_engine(e)->run(); });
}

int rectv_engine_job_info(rectv_engine *e, int job_id, double *times, double *bytes, double *rho_rdiff,
                          int *tune, int *status) {
    return rectv::guarded([&] {
        rectv::Engine *E = live_engine(e);
        if (job_id < 0 || job_id >= (int)E->jobs.size()) throw rectv::Error(RECTV_ERR_ARG, "rectv_engine: bad job id");
        const auto &j = *E->jobs[job_id];
        if (times) {
            times[0] = j.arrival;
            times[1] = j.admitted;
            times[2] = j.done;
        }
        if (bytes) {
            bytes[0] = j.est_bytes;
            bytes[1] = j.bytes;
        }
        if (rho_rdiff) {
            rho_rdiff[0] = j.rho_final;
            rho_rdiff[1] = j.rdiff_final;
        }
        if (tune) {
            tune[0] = j.tune.zper;
            tune[1] = j.tune.sc_grid;
        }
        if (status) *status = j.state;
        if (j.state == rectv::kFailed) rectv::last_error() = j.error;
    });
}

int rectv_engine_stats(rectv_engine *e, double *stats) {
    return rectv::guarded([&] {
        rectv::Engine *E = live_engine(e);
        if (!stats) throw rectv::Error(RECTV_ERR_ARG, "rectv_engine_stats: null output");
        stats[0] = E->makespan;
        stats[1] = E->peak;
        stats[2] = E->budget;
        stats[3] = E->peak_running;
    });
}

int rectv_engine_job_error(rectv_engine *e, int job_id, char *buf, int len) {
    return rectv::guarded([&] {
        rectv::Engine *E = live_engine(e);
        if (job_id < 0 || job_id >= (int)E->jobs.size()) throw rectv::Error(RECTV_ERR_ARG, "rectv_engine: bad job id");
        if (!buf || len < 1) throw rectv::Error(RECTV_ERR_ARG, "rectv_engine_job_error: null buffer");
        std::strncpy(buf, E->jobs[job_id]->error.c_str(), (size_t)len - 1);
        buf[len - 1] = 0;
    });
}

void rectv_engine_destroy(rectv_engine *e) {
    if (!e) return;
    delete e->e;
    delete e;
}

int rectv_estimate_bytes(int n, int ntheta, int m, int nz, int nzp, double *bytes) {
    return rectv::guarded([&] {
        if (!bytes) throw rectv::Error(RECTV_ERR_ARG, "rectv_estimate_bytes: null output");
        if (n < 2 || ntheta < 1 || m < 1 || nz < 1 || nzp < 1 || nzp > nz)
            throw rectv::Error(RECTV_ERR_ARG, "rectv_estimate_bytes: invalid dimensions");
        *bytes = rectv::make_layout(n, ntheta, m, nz, nzp, -1).bytes;
    });
}

}  // extern "C"
