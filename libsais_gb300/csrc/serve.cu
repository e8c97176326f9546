// serve.cu -- request loop for SA+BWT jobs with continuous batching.
//
// Jobs (text in host memory, outputs SA/U in host memory) are queued as they
// arrive.  `workers` host threads each own a context (CUDA stream + device
// arena) and run one job or one coalesced batch at a time, so up to `workers`
// batches overlap on the GPU; a job that arrives while others run is admitted
// as soon as a worker and HBM are free.  Every copy goes straight between the
// job's own buffers and the device (DMA when the caller's buffers are pinned;
// the driver stages pageable ones), one copy per job and direction.
//
// Admission is against one HBM pool of `budget` bytes shared by all workers.
// A worker's reservation is the larger of the arena it holds and the
// footprint of the work it runs -- kFootprintPerSymbol bytes per symbol (sort
// workspace + text + outputs).  The oldest queued job is admitted when its
// reservation fits the pool; when it does not, idle workers give their arenas
// back first, and otherwise the job waits for running work to finish.  A job
// whose footprint exceeds the whole budget is rejected with -2 (the reference
// fails an allocation with -2 as well, src/libsais.c:6930-6932).
//
// Coalescing: when the admitted job is small (n <= small_job_symbols), the
// queued small jobs of the same symbol width behind it (up to max_batch) are
// sorted together with it in one batched sort -- one set of launches per
// doubling round for all of them -- for 8- and 16-bit texts alike.
#include <algorithm>
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

// device bytes per text symbol: workspace (~70) + text + SA + BWT + slack
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

struct WorkerState {
    bool busy = false;
    size_t held = 0;       // arena its context holds
    size_t reserved = 0;   // its share of the pool: max(held, footprint of its running work)
};

struct Server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job *> queue;
    std::unordered_map<int64_t, Job *> jobs;
    std::vector<std::thread> threads;
    std::vector<gsais_ctx *> ctxs;
    std::vector<WorkerState> ws;
    size_t budget = 0, reserved_total = 0, reserved_hwm = 0;
    int64_t small_limit = 0;
    int max_batch = 1;
    bool stopping = false;
    int64_t next_id = 1;
    // statistics
    int64_t submitted = 0, completed = 0, rejected = 0, batches = 0, batched_jobs = 0, releases = 0;
    int64_t symbols_done = 0;
    double first_submit = 0, last_done = 0;
};

size_t footprint(int64_t n) { return (size_t)(kFootprintPerSymbol * (double)n) + ((size_t)8 << 20); }

void run_single(gsais_ctx *c, Job *j)
{
    j->result = gsais_run_bwt(c, j->T, j->symbytes, j->n, j->U, nullptr, 4, 0, nullptr, 4, j->SA, 4);
}

void run_batch(gsais_ctx *c, std::vector<Job *> &b)
{
    const int count = (int)b.size();
    std::vector<const void *> T(count);
    std::vector<int64_t> n(count), res(count, 0);
    std::vector<int32_t *> SA(count);
    std::vector<void *> U(count);
    for (int k = 0; k < count; ++k) {
        T[k] = b[k]->T;
        n[k] = b[k]->n;
        SA[k] = b[k]->SA;
        U[k] = b[k]->U;
    }
    const int64_t rc = gsais_batch_jobs(c, b[0]->symbytes, count, T.data(), n.data(), SA.data(), U.data(), res.data());
    for (int k = 0; k < count; ++k) b[k]->result = rc == 0 ? res[k] : rc;
}

// Under s->mu: the jobs worker w takes next (oldest first, then the small jobs
// of the same width behind it), if their reservation fits the pool, after
// idle workers have given their arenas back if needed.  Empty: wait.
std::vector<Job *> admit(Server *s, int w)
{
    std::vector<Job *> batch;
    if (s->queue.empty()) return batch;
    Job *first = s->queue.front();
    WorkerState &me = s->ws[w];
    const size_t others = s->reserved_total - me.reserved;   // reserved by the other workers
    const size_t avail = s->budget > others ? s->budget - others : 0;
    size_t need = footprint(first->n);
    std::vector<Job *> picks;   // small jobs of the same width behind the first, in queue order
    size_t scanned = 1;
    if (first->n <= s->small_limit) {
        const size_t depth = std::min(s->queue.size(), (size_t)s->max_batch * 4);   // bounded look-ahead
        for (; scanned < depth && (int)picks.size() + 1 < s->max_batch; ++scanned) {
            Job *j = s->queue[scanned];
            if (j->symbytes == first->symbytes && j->n <= s->small_limit && need + footprint(j->n) <= avail) {
                need += footprint(j->n);
                picks.push_back(j);
            }
        }
    }
    size_t want = std::max(me.held, need);
    // give back idle workers' arenas (largest first) while the pool is short
    while (s->reserved_total - me.reserved + want > s->budget) {
        int victim = -1;
        for (int o = 0; o < (int)s->ws.size(); ++o)
            if (o != w && !s->ws[o].busy && s->ws[o].held > 0 && (victim < 0 || s->ws[o].held > s->ws[victim].held))
                victim = o;
        if (victim < 0) break;
        gsais_release_workspace(s->ctxs[victim]);   // idle: its context runs nothing
        s->reserved_total -= s->ws[victim].reserved;
        s->ws[victim].held = s->ws[victim].reserved = 0;
        ++s->releases;
    }
    if (s->reserved_total - me.reserved + want > s->budget && me.held > need) {
        // this worker's own arena is what is too large: give it back too
        gsais_release_workspace(s->ctxs[w]);
        s->reserved_total -= me.reserved;
        me.held = me.reserved = 0;
        ++s->releases;
        want = need;
    }
    if (s->reserved_total - me.reserved + want > s->budget) return batch;   // wait for running work
    batch.push_back(first);
    batch.insert(batch.end(), picks.begin(), picks.end());
    // drop the taken jobs from the scanned front of the queue (one pass, order kept)
    for (Job *j : batch) j->batched = -1;   // mark
    auto head_end = s->queue.begin() + (std::ptrdiff_t)scanned;
    auto kept_end = std::remove_if(s->queue.begin(), head_end, [](Job *j) { return j->batched == -1; });
    s->queue.erase(kept_end, head_end);
    for (Job *j : batch) j->batched = 0;
    s->reserved_total += want - me.reserved;
    me.reserved = want;
    me.busy = true;
    s->reserved_hwm = std::max(s->reserved_hwm, s->reserved_total);
    return batch;
}

void worker(Server *s, int w)
{
    gsais_ctx *c = s->ctxs[w];
    for (;;) {
        std::vector<Job *> batch;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            for (;;) {
                if (s->stopping && s->queue.empty()) return;   // stopping and drained
                batch = admit(s, w);
                if (!batch.empty()) break;
                s->cv_work.wait(lk);
            }
        }
        const double t0 = now_s();
        for (Job *j : batch) j->t_start = t0;
        if (batch.size() == 1) run_single(c, batch[0]);
        else run_batch(c, batch);
        const size_t held = (size_t)gsais_ctx_workspace_bytes(c);
        const double t1 = now_s();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            WorkerState &me = s->ws[w];
            s->reserved_total -= me.reserved;
            me.held = me.reserved = held;
            s->reserved_total += held;
            me.busy = false;
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
        s->cv_work.notify_all();   // the pool has room again
    }
}

}  // namespace

extern "C" {

void *gsais_server_create(int64_t hbm_budget_bytes, int32_t workers, int64_t small_job_symbols, int32_t max_batch)
{
    if (hbm_budget_bytes <= 0 || workers <= 0 || max_batch <= 0 || max_batch > 32000) return nullptr;
    Server *s = new (std::nothrow) Server();
    if (!s) return nullptr;
    s->budget = (size_t)hbm_budget_bytes;
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
    s->ws.resize(workers);
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
        if (footprint(n) > s->budget) {
            // larger than the whole HBM budget
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
    s->cv_work.notify_all();
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
    out->hbm_high_water_bytes = (int64_t)s->reserved_hwm;
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
