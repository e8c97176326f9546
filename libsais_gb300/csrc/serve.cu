// serve.cu -- request loop for SA+BWT jobs with continuous batching.
//
// Jobs (text in host memory, outputs SA/U in host memory) are queued as they
// arrive.  `workers` host threads each own a context (CUDA stream + device
// arena), so jobs taken by different workers run concurrently on the GPU.
// When a worker becomes free it takes the oldest queued job; if that job is
// small (n <= small_job_symbols, 8-bit), it also takes the queued small 8-bit
// jobs behind it (up to max_batch jobs) and sorts them together with the
// batched path (one set of launches per doubling round for all of them).
// Admission is against an HBM budget: every worker may hold at most
// budget / workers bytes of device memory, and a job (or batch) is admitted
// to a worker only if its footprint -- kFootprintPerSymbol bytes per symbol
// (sort workspace + text + outputs) -- fits that share.  A job larger than a
// worker's share is rejected with -2 (the reference would fail allocation
// with -2 as well, src/libsais.c:6930-6932).
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gsais.h"
#include "libsais_gb300.h"

namespace {

// device bytes per text symbol: workspace (~68.5) + text + SA + BWT + slack
constexpr double kFootprintPerSymbol = 80.0;

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Job {
    int64_t id;
    const void *T;
    int symbytes;
    int64_t n;
    int32_t *SA;
    void *U;
    double t_submit = 0, t_start = 0, t_done = 0;
    int64_t result = 0;
    bool done = false;
    int batched = 0;   // number of jobs in the batch it ran in
};

struct Server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job *> queue;
    std::unordered_map<int64_t, Job *> jobs;
    std::vector<std::thread> threads;
    std::vector<gsais_ctx *> ctxs;
    size_t budget = 0, share = 0;
    int64_t small_limit = 0;
    int max_batch = 1;
    bool stopping = false;
    int64_t next_id = 1;
    // statistics
    int64_t submitted = 0, completed = 0, rejected = 0, batches = 0, batched_jobs = 0;
    int64_t symbols_done = 0;
    std::atomic<int64_t> in_flight_bytes{0}, hwm_bytes{0};
    double first_submit = 0, last_done = 0;
};

size_t footprint(int64_t n) { return (size_t)(kFootprintPerSymbol * (double)n) + ((size_t)8 << 20); }

void note_bytes(Server *s, int64_t delta)
{
    const int64_t v = s->in_flight_bytes.fetch_add(delta) + delta;
    int64_t h = s->hwm_bytes.load();
    while (v > h && !s->hwm_bytes.compare_exchange_weak(h, v)) {
    }
}

void run_single(gsais_ctx *c, Job *j)
{
    j->result = gsais_run_bwt(c, j->T, j->symbytes, j->n, j->U, nullptr, 4, 0, nullptr, 4, j->SA, 4);
}

void run_batch(gsais_ctx *c, std::vector<Job *> &b)
{
    const int count = (int)b.size();
    std::vector<int64_t> offs(count + 1, 0);
    for (int k = 0; k < count; ++k) offs[k + 1] = offs[k] + b[k]->n;
    const int64_t n = offs[count];
    std::vector<uint8_t> T((size_t)n), U((size_t)n);
    std::vector<int32_t> SA((size_t)n), prim(count);
    for (int k = 0; k < count; ++k) std::memcpy(T.data() + offs[k], b[k]->T, (size_t)b[k]->n);
    const int64_t rc = gsais_batch_sa_bwt(c, T.data(), offs.data(), count, SA.data(), U.data(), prim.data());
    for (int k = 0; k < count; ++k) {
        Job *j = b[k];
        if (rc == 0) {
            std::memcpy(j->SA, SA.data() + offs[k], (size_t)j->n * 4);
            std::memcpy(j->U, U.data() + offs[k], (size_t)j->n);
            j->result = prim[k];
        } else {
            j->result = rc;
        }
    }
}

void worker(Server *s, int w)
{
    gsais_ctx *c = s->ctxs[w];
    for (;;) {
        std::vector<Job *> batch;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stopping || !s->queue.empty(); });
            if (s->queue.empty()) return;   // stopping and drained
            Job *first = s->queue.front();
            s->queue.pop_front();
            batch.push_back(first);
            size_t bytes = footprint(first->n);
            if (first->symbytes == 1 && first->n <= s->small_limit) {
                // coalesce the queued small 8-bit jobs behind it
                for (auto it = s->queue.begin(); it != s->queue.end() && (int)batch.size() < s->max_batch;) {
                    Job *j = *it;
                    if (j->symbytes == 1 && j->n <= s->small_limit && bytes + footprint(j->n) <= s->share) {
                        bytes += footprint(j->n);
                        batch.push_back(j);
                        it = s->queue.erase(it);
                    } else {
                        ++it;
                    }
                }
            }
        }
        const double t0 = now_s();
        size_t bytes = 0;
        for (Job *j : batch) {
            j->t_start = t0;
            bytes += footprint(j->n);
        }
        note_bytes(s, (int64_t)bytes);
        if (batch.size() == 1) run_single(c, batch[0]);
        else run_batch(c, batch);
        note_bytes(s, -(int64_t)bytes);
        const double t1 = now_s();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (Job *j : batch) {
                j->t_done = t1;
                j->done = true;
                j->batched = (int)batch.size();
                ++s->completed;
                s->symbols_done += j->n;
            }
            if (batch.size() > 1) {
                ++s->batches;
                s->batched_jobs += (int64_t)batch.size();
            }
            s->last_done = t1;
        }
        s->cv_done.notify_all();
    }
}

}  // namespace

extern "C" {

void *gsais_server_create(int64_t hbm_budget_bytes, int32_t workers, int64_t small_job_symbols, int32_t max_batch)
{
    if (hbm_budget_bytes <= 0 || workers <= 0 || max_batch <= 0) return nullptr;
    Server *s = new (std::nothrow) Server();
    if (!s) return nullptr;
    s->budget = (size_t)hbm_budget_bytes;
    s->share = s->budget / (size_t)workers;
    s->small_limit = small_job_symbols;
    s->max_batch = max_batch;
    for (int w = 0; w < workers; ++w) {
        gsais_ctx *c = gsais_ctx_create();
        if (!c) break;
        s->ctxs.push_back(c);
    }
    if ((int)s->ctxs.size() != workers) {
        for (auto *c : s->ctxs) gsais_ctx_destroy(c);
        delete s;
        return nullptr;
    }
    for (int w = 0; w < workers; ++w) s->threads.emplace_back(worker, s, w);
    return s;
}

int64_t gsais_server_submit(void *srv, const void *T, int32_t symbytes, int64_t n, int32_t *SA, void *U)
{
    Server *s = static_cast<Server *>(srv);
    if (!s || !T || !SA || !U || n < 2 || (symbytes != 1 && symbytes != 2)) return -1;
    Job *j = new (std::nothrow) Job();
    if (!j) return -2;
    j->T = T;
    j->symbytes = symbytes;
    j->n = n;
    j->SA = SA;
    j->U = U;
    j->t_submit = now_s();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stopping) {
            delete j;
            return -1;
        }
        j->id = s->next_id++;
        s->jobs[j->id] = j;
        ++s->submitted;
        if (s->first_submit == 0) s->first_submit = j->t_submit;
        if (footprint(n) > s->share) {
            // does not fit a worker's share of the HBM budget
            j->result = -2;
            j->done = true;
            j->t_done = j->t_submit;
            ++s->rejected;
            ++s->completed;
            s->cv_done.notify_all();
            return j->id;
        }
        s->queue.push_back(j);
    }
    s->cv_work.notify_one();
    return j->id;
}

// Waits for a job; returns 0 and its result (primary index or -1/-2) and
// latencies (seconds: queued, total), or -1 for an unknown id.
int32_t gsais_server_wait(void *srv, int64_t id, int64_t *result, double *queued_s, double *total_s,
                          int32_t *batched)
{
    Server *s = static_cast<Server *>(srv);
    if (!s) return -1;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return -1;
    Job *j = it->second;
    s->cv_done.wait(lk, [&] { return j->done; });
    if (result) *result = j->result;
    if (queued_s) *queued_s = j->t_start > 0 ? j->t_start - j->t_submit : 0;
    if (total_s) *total_s = j->t_done - j->t_submit;
    if (batched) *batched = j->batched;
    s->jobs.erase(it);
    delete j;
    return 0;
}

int32_t gsais_server_get_stats(void *srv, gsais_server_stats *out)
{
    Server *s = static_cast<Server *>(srv);
    if (!s || !out) return -1;
    std::lock_guard<std::mutex> lk(s->mu);
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->rejected = s->rejected;
    out->batches = s->batches;
    out->batched_jobs = s->batched_jobs;
    out->symbols_done = s->symbols_done;
    out->hbm_high_water_bytes = s->hwm_bytes.load();
    out->hbm_budget_bytes = (int64_t)s->budget;
    out->busy_seconds = s->last_done > s->first_submit ? s->last_done - s->first_submit : 0;
    out->footprint_bytes_per_symbol = kFootprintPerSymbol;
    return 0;
}

void gsais_server_destroy(void *srv)
{
    Server *s = static_cast<Server *>(srv);
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->threads) t.join();
    for (auto &kv : s->jobs) delete kv.second;
    for (auto *c : s->ctxs) gsais_ctx_destroy(c);
    delete s;
}

}  // extern "C"
