// Serving loop: independent PCA jobs of uneven size on one GPU (dpca_serve_* in dpca.h).
//
// The reference solves one PCA per MPI job (src/distpca.cpp:83-405).  Here one server owns
// `slots` host workers, each with its own non-blocking CUDA stream.  Jobs wait in a queue; a
// worker that becomes free takes the oldest job whose device footprint fits the memory budget
// beside the jobs in flight (a job may be passed by later, smaller ones at most 2*slots times,
// after which admission waits for it).  The worker then runs the whole job on its stream:
// stream-ordered allocation of a resident handle, upload (or on-device synthesis) of the packed
// rows with their per-SNP statistics, the start block, the solve, and stream-ordered release.
// Jobs in flight overlap on the device kernel by kernel; no job's allocation or release waits for
// another job's work, because every device buffer comes from the server's own memory pool on the
// job's own stream and the pool may not make one stream wait for another to reuse memory.  The
// pool belongs to the server (created with it, destroyed at shutdown), so the device's default
// pool, which other code in the process may use, keeps its settings and its memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "dpca_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
    int64_t id = 0;
    dpca_job spec{};
    dpca_job_info info{};
    size_t need = 0;  // device bytes admitted against the budget
    int passed = 0;   // times a later job was admitted ahead of this one
    bool done = false;
};

}  // namespace

struct dpca_server {
    int device = 0, slots = 4;
    size_t budget = 0, in_use = 0, peak = 0;
    int in_flight = 0, max_in_flight = 0;
    int64_t next_id = 1, done_count = 0;
    bool stop = false;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job *> pending;
    std::unordered_map<int64_t, Job *> jobs;
    std::vector<std::thread> workers;
    std::vector<cudaStream_t> streams;
    cudaMemPool_t pool = nullptr;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace dpca {
namespace {

// Device bytes a job holds at its peak: the resident handle, the upload's two staging buffers
// (host rows not at the device pitch) or the synthesis tables, and allocation rounding.
size_t job_need(const dpca_job &j, int sm_count) {
    size_t b = handle_footprint(j.n_ind, j.n_snp, j.cfg.nrhs, j.cfg.precision, sm_count);
    const int64_t pitch = ((int64_t)(j.n_ind + 3) / 4 + 127) / 128 * 128;
    if (j.packed) {
        if (j.row_stride != pitch) {
            const int64_t stride = std::max<int64_t>(1, j.row_stride);
            int64_t rows = std::max<int64_t>(512, ((int64_t)(256 << 20) / stride) / 512 * 512);
            rows = std::min<int64_t>(rows, ((int64_t)j.n_snp + 511) / 512 * 512);
            b += 2 * (size_t)rows * (size_t)stride;
        }
    } else {
        b += (size_t)j.n_ind * 5 + (size_t)j.n_snp * std::max(1, j.synth_n_pop) * 4;
    }
    return b + ((size_t)48 << 20);
}

dpca_status check_job(const dpca_job &j) {
    if (j.n_ind <= 0 || j.n_snp <= 0 || j.cfg.nrhs <= 0 || j.cfg.nsv <= 0 || j.cfg.nsv > j.cfg.nrhs) {
        set_error("dpca_serve_submit: need n_ind, n_snp > 0 and 0 < nsv <= nrhs");
        return DPCA_ERR_INVALID;
    }
    if (j.cfg.power < 1 || j.cfg.miter < 1) {
        set_error("dpca_serve_submit: power and miter must be >= 1");
        return DPCA_ERR_INVALID;
    }
    if (!j.sigma) {
        set_error("dpca_serve_submit: sigma output array is required");
        return DPCA_ERR_INVALID;
    }
    if (j.packed) {
        if (j.row_stride < (int64_t)(j.n_ind + 3) / 4) {
            set_error("dpca_serve_submit: row_stride below ceil(n_ind/4)");
            return DPCA_ERR_INVALID;
        }
    } else if (!j.synth_pop || !j.synth_miss_thr || !j.synth_snp_thr || j.synth_n_pop <= 0) {
        set_error("dpca_serve_submit: packed rows or the synthesis tables are required");
        return DPCA_ERR_INVALID;
    }
    return DPCA_OK;
}

// The whole job on one stream; returns its status (the error text stays on this thread).
dpca_status run_job(dpca_server *s, Job *j, cudaStream_t stream) {
    const dpca_job &q = j->spec;
    DPCA_CUDA(cudaSetDevice(s->device));
    dpca_handle *hh = nullptr;
    dpca_status st =
        create_serving_handle(&hh, q.n_ind, q.n_snp, q.cfg.nrhs, q.cfg.precision, s->device, stream, s->pool);
    if (st == DPCA_OK) {
        if (q.packed)
            st = dpca_upload(hh, q.packed, q.row_stride);
        else
            st = dpca_synth_fill(hh, q.synth_key, q.synth_pop, q.synth_miss_thr, q.synth_snp_thr, q.synth_n_pop);
    }
    std::vector<double> omega;
    if (st == DPCA_OK) {
        omega.resize((size_t)q.n_ind * q.cfg.nrhs);
        if (q.omega)
            std::memcpy(omega.data(), q.omega, omega.size() * sizeof(double));
        else
            st = dpca_start_block(q.n_ind, q.cfg.nrhs, omega.data());
    }
    if (st == DPCA_OK) {
        dpca_result res{};
        res.sigma = q.sigma;
        res.u = q.u;
        st = dpca_solve(hh, &q.cfg, omega.data(), &res);
        j->info.total_its = res.total_its;
        j->info.passes = res.passes;
    }
    if (hh) dpca_destroy(hh);  // waits for the job's own stream only; the frees are stream-ordered
    return st;
}

// Under s->mu: the job a free worker takes next, or nullptr.
Job *pick_locked(dpca_server *s) {
    if (s->pending.empty()) return nullptr;
    Job *head = s->pending.front();
    if (s->in_use + head->need <= s->budget) {
        s->pending.pop_front();
        return head;
    }
    if (head->passed >= 2 * s->slots) return nullptr;  // wait for memory to free up for the head
    for (auto it = s->pending.begin() + 1; it != s->pending.end(); ++it)
        if (s->in_use + (*it)->need <= s->budget) {
            Job *j = *it;
            s->pending.erase(it);
            head->passed++;
            return j;
        }
    return nullptr;
}

void worker_main(dpca_server *s, int w) {
    cudaSetDevice(s->device);
    for (;;) {
        Job *j = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] {
                j = pick_locked(s);
                return j != nullptr || (s->stop && s->pending.empty());
            });
            if (!j) return;
            s->in_use += j->need;
            s->peak = std::max(s->peak, s->in_use);
            s->in_flight++;
            s->max_in_flight = std::max(s->max_in_flight, s->in_flight);
            j->info.t_start = s->now();
        }
        clear_error();
        dpca_status st = run_job(s, j, s->streams[w]);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            j->info.status = st;
            if (st != DPCA_OK) snprintf(j->info.error, sizeof(j->info.error), "%s", dpca_last_error());
            j->info.t_done = s->now();
            j->done = true;
            s->in_use -= j->need;
            s->in_flight--;
            s->done_count++;
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

}  // namespace
}  // namespace dpca

using namespace dpca;

extern "C" {

dpca_status dpca_serve_create(dpca_server **out, const dpca_serve_config *cfg) {
    clear_error();
    if (!out || !cfg) return DPCA_ERR_INVALID;
    *out = nullptr;
    const int slots = cfg->slots == 0 ? 4 : cfg->slots;
    if (slots < 1 || slots > 64) {
        set_error("dpca_serve_create: slots must be in [1, 64]");
        return DPCA_ERR_INVALID;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device available (libdpca has no CPU fallback)");
        return DPCA_ERR_CUDA;
    }
    if (cfg->device < 0 || cfg->device >= ndev) {
        set_error("device %d out of range (%d devices)", cfg->device, ndev);
        return DPCA_ERR_INVALID;
    }
    DPCA_CUDA(cudaSetDevice(cfg->device));
    size_t free_b = 0, total_b = 0;
    DPCA_CUDA(cudaMemGetInfo(&free_b, &total_b));
    // The server's own pool serves every job: it keeps freed memory (no release to the driver at
    // synchronisations) and never lets one stream wait for another's frees.
    cudaMemPool_t pool = nullptr;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = cfg->device;
    DPCA_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t keep = UINT64_MAX;
    int no = 0;
    if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess ||
        cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no) != cudaSuccess) {
        cudaGetLastError();
        cudaMemPoolDestroy(pool);
        set_error("dpca_serve_create: memory pool attributes refused");
        return DPCA_ERR_CUDA;
    }
    dpca_server *s = new (std::nothrow) dpca_server();
    if (!s) {
        cudaMemPoolDestroy(pool);
        return DPCA_ERR_NOMEM;
    }
    s->pool = pool;
    s->device = cfg->device;
    s->slots = slots;
    s->budget = cfg->hbm_budget_gb > 0 ? (size_t)(cfg->hbm_budget_gb * 1e9) : (size_t)(0.85 * (double)free_b);
    s->t0 = Clock::now();
    for (int w = 0; w < slots; ++w) {
        cudaStream_t st = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
            cudaMemPoolDestroy(s->pool);
            delete s;
            set_error("dpca_serve_create: stream creation failed");
            return DPCA_ERR_CUDA;
        }
        s->streams.push_back(st);
    }
    for (int w = 0; w < slots; ++w) s->workers.emplace_back(worker_main, s, w);
    *out = s;
    return DPCA_OK;
}

dpca_status dpca_serve_submit(dpca_server *s, const dpca_job *job, int64_t *job_id) {
    clear_error();
    if (!s || !job || !job_id) return DPCA_ERR_INVALID;
    DPCA_TRY(check_job(*job));
    int sm = 0;
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, s->device);
    Job *j = new (std::nothrow) Job();
    if (!j) return DPCA_ERR_NOMEM;
    j->spec = *job;
    j->need = job_need(*job, std::max(sm, 1));
    j->info.device_gb = (double)j->need * 1e-9;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            delete j;
            set_error("dpca_serve_submit: the server is shutting down");
            return DPCA_ERR_INVALID;
        }
        j->id = s->next_id++;
        j->info.t_submit = s->now();
        s->jobs[j->id] = j;
        if (j->need > s->budget) {
            j->info.status = DPCA_ERR_NOMEM;
            snprintf(j->info.error, sizeof(j->info.error), "job needs %.3f GB of device memory, budget %.3f GB",
                     (double)j->need * 1e-9, (double)s->budget * 1e-9);
            j->info.t_start = j->info.t_done = j->info.t_submit;
            j->done = true;
            s->done_count++;
        } else {
            s->pending.push_back(j);
        }
        *job_id = j->id;
    }
    s->cv_work.notify_one();
    s->cv_done.notify_all();
    return DPCA_OK;
}

dpca_status dpca_serve_poll(dpca_server *s, int64_t job_id, int *done, dpca_job_info *info) {
    if (!s || !done) return DPCA_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) {
        set_error("unknown job id %lld", (long long)job_id);
        return DPCA_ERR_INVALID;
    }
    *done = it->second->done ? 1 : 0;
    if (*done && info) *info = it->second->info;
    return DPCA_OK;
}

dpca_status dpca_serve_wait(dpca_server *s, int64_t job_id, double timeout_s, dpca_job_info *info) {
    if (!s) return DPCA_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) {
        set_error("unknown job id %lld", (long long)job_id);
        return DPCA_ERR_INVALID;
    }
    Job *j = it->second;
    if (timeout_s < 0) {
        s->cv_done.wait(lk, [&] { return j->done; });
    } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return j->done; })) {
        set_error("job %lld not finished after %.3f s", (long long)job_id, timeout_s);
        return DPCA_ERR_TIMEOUT;
    }
    if (info) *info = j->info;
    return DPCA_OK;
}

dpca_status dpca_serve_stats(dpca_server *s, int64_t *done, int *max_in_flight, double *peak_gb, double *budget_gb) {
    if (!s) return DPCA_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    if (done) *done = s->done_count;
    if (max_in_flight) *max_in_flight = s->max_in_flight;
    if (peak_gb) *peak_gb = (double)s->peak * 1e-9;
    if (budget_gb) *budget_gb = (double)s->budget * 1e-9;
    return DPCA_OK;
}

dpca_status dpca_serve_shutdown(dpca_server *s) {
    if (!s) return DPCA_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (std::thread &t : s->workers) t.join();
    cudaSetDevice(s->device);
    for (cudaStream_t st : s->streams) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    // every job's buffers went back to the pool on its (now idle) stream: destroying the pool
    // returns its memory to the driver
    if (s->pool) cudaMemPoolDestroy(s->pool);
    for (auto &kv : s->jobs) delete kv.second;
    delete s;
    return DPCA_OK;
}

}  // extern "C"
