// serve.cu -- the request loop: continuous batching of reconstruction jobs.
//
// Requests (job descriptor + tilt series) arrive from any host thread.  One
// worker thread owns the device: it admits queued requests while their
// device-memory footprint fits the budget, runs each admitted job's setup on
// the job's own stream, then queues outer iterations round-robin over all
// admitted jobs -- at most two in flight per job, so a new arrival joins the
// rotation within two rounds -- and, when a job's last iteration has run,
// copies its volume to the host, records arrival-to-result latency and frees
// its memory for the next admission.  A mixed job whose next iteration waits
// on its periodic FP64 residual check is passed over until the check's
// result has reached the host, so a check never stalls the other jobs or
// admission.  Every CUDA status the loop sees other than "not ready" ends
// the request with NUDIM_ECUDA and its message.  Jobs run on separate streams, so their
// kernels overlap on the device; results do not depend on the mix (every
// kernel is deterministic and a job's work stays on its stream).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.cuh"

namespace nudim {
const char *last_error();
}
using namespace nudim;

namespace {

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

enum ReqState { R_QUEUED = 0, R_ACTIVE = 1, R_DONE = 2 };

struct Request {
    long long id = 0;
    nudim_job_desc d{};
    std::vector<double> proj;
    double t_arrival = 0, t_done = 0;
    size_t footprint = 0;
    int state = R_QUEUED;
    int rc = NUDIM_OK;
    std::string err;
    nudim_job *job = nullptr;
    int enqueued = 0;            // iterations queued so far
    cudaEvent_t ev[2] = {nullptr, nullptr};
    std::vector<double> vol;     // full volume on completion
};

}  // namespace

struct nudim_server {
    nudim_ctx *ctx = nullptr;
    size_t budget = 0, in_use = 0;
    int max_active = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> queue;
    std::vector<Request *> active;
    std::map<long long, std::unique_ptr<Request>> all;
    long long next_id = 1;
    bool stop = false;
    std::thread worker;
    std::vector<double> latencies;
    double t_first = -1, t_last = 0;
};

namespace {

// A request whose work failed: keep the first status and its message (the
// worker thread's error text is overwritten by later calls).
void fail(Request *r, int rc)
{
    if (r->rc != NUDIM_OK) return;
    r->rc = rc;
    r->err = last_error();
    r->enqueued = r->d.nhio + r->d.ner;
}

void finish(nudim_server *s, Request *r, int rc)
{
    if (r->job) {
        if (!rc) {
            size_t V = (size_t)r->d.nz * r->d.np * r->d.np;
            r->vol.resize(V);
            rc = nudim_job_get_volume(r->job, r->vol.data(), V, 0);
            if (rc) r->err = last_error();
        }
        nudim_job_destroy(r->job);
        r->job = nullptr;
    }
    for (cudaEvent_t &e : r->ev)
        if (e) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    std::lock_guard<std::mutex> lk(s->mu);
    r->rc = rc;
    r->t_done = now_s();
    r->state = R_DONE;
    r->proj.clear();
    r->proj.shrink_to_fit();
    s->in_use -= r->footprint;
    if (!rc) {
        s->latencies.push_back(r->t_done - r->t_arrival);
        s->t_last = std::max(s->t_last, r->t_done);
    }
    s->cv_done.notify_all();
}

int admit(nudim_server *s, Request *r)
{
    int rc = nudim_job_create(s->ctx, &r->d, &r->job);
    if (!rc) rc = nudim_job_set_projections(r->job, r->proj.data(), r->proj.size());
    for (cudaEvent_t &e : r->ev)
        if (!rc) {
            cudaError_t ce = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
            if (ce != cudaSuccess) rc = cuda_fail(ce, "serving: cudaEventCreate", __FILE__, __LINE__);
        }
    if (rc) r->err = last_error();
    return rc;
}

void worker_main(nudim_server *s)
{
    cudaSetDevice(s->ctx->device);
    for (;;) {
        // ---- admission by footprint
        std::vector<Request *> admitted;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->queue.empty() && s->active.empty()) {
                if (s->stop) return;
                s->cv_work.wait(lk);
                continue;
            }
            while (!s->queue.empty() && (int)s->active.size() + (int)admitted.size() <
                                            s->max_active) {
                Request *r = s->queue.front();
                bool idle = s->active.empty() && admitted.empty();
                if (!idle && s->in_use + r->footprint > s->budget) break;
                s->queue.pop_front();
                s->in_use += r->footprint;
                r->state = R_ACTIVE;
                admitted.push_back(r);
            }
        }
        for (Request *r : admitted) {
            int rc = admit(s, r);
            if (rc) {
                finish(s, r, rc);
                continue;
            }
            std::lock_guard<std::mutex> lk(s->mu);
            s->active.push_back(r);
        }
        // ---- one round: queue the next iteration of every active job
        std::vector<Request *> act;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            act = s->active;
        }
        bool progress = !admitted.empty();
        for (Request *r : act) {
            int total = r->d.nhio + r->d.ner;
            if (r->enqueued >= total) continue;
            cudaEvent_t &slot = r->ev[r->enqueued & 1];
            // at most two iterations in flight per job
            if (r->enqueued >= 2) {
                cudaError_t q = cudaEventQuery(slot);
                if (q == cudaErrorNotReady) continue;
                if (q != cudaSuccess) {
                    fail(r, cuda_fail(q, "serving: iteration event", __FILE__, __LINE__));
                    continue;
                }
            }
            bool issued = false;
            int rc = job_try_step(r->job, &issued);
            if (rc) {
                fail(r, rc);
                continue;
            }
            if (!issued) continue;  // waits on its residual check
            cudaError_t e = cudaEventRecord(slot, (cudaStream_t)nudim_job_stream(r->job));
            if (e != cudaSuccess) {
                fail(r, cuda_fail(e, "serving: cudaEventRecord", __FILE__, __LINE__));
                continue;
            }
            r->enqueued++;
            progress = true;
        }
        // ---- completions
        for (Request *r : act) {
            int total = r->d.nhio + r->d.ner;
            bool done = r->rc != NUDIM_OK || total == 0;
            if (!done && r->enqueued >= total) {
                cudaError_t q = cudaEventQuery(r->ev[(r->enqueued - 1) & 1]);
                if (q == cudaSuccess) done = true;
                else if (q != cudaErrorNotReady) {
                    fail(r, cuda_fail(q, "serving: iteration event", __FILE__, __LINE__));
                    done = true;
                }
            }
            if (!done) continue;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                s->active.erase(std::find(s->active.begin(), s->active.end(), r));
            }
            finish(s, r, r->rc);
            progress = true;
        }
        if (!progress) {
            // everything queued is still running: wait briefly for the device
            // or for a new arrival
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait_for(lk, std::chrono::microseconds(200));
        }
    }
}

double percentile(std::vector<double> v, double q)
{
    if (v.empty()) return 0;
    std::sort(v.begin(), v.end());
    double pos = q * (v.size() - 1);
    size_t i = (size_t)pos;
    double f = pos - i;
    return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

int nudim_server_create(nudim_ctx *ctx, size_t mem_budget, int max_active, nudim_server **out)
{
    if (!ctx || !out || max_active <= 0) {
        set_error("invalid nudim_server_create arguments");
        return NUDIM_EINVAL;
    }
    auto *s = new nudim_server();
    s->ctx = ctx;
    s->budget = mem_budget;
    s->max_active = max_active;
    s->worker = std::thread(worker_main, s);
    *out = s;
    return NUDIM_OK;
}

int nudim_server_submit(nudim_server *s, const nudim_job_desc *d, const double *proj, size_t n,
                        long long *ticket)
{
    if (!s || !d || (!proj && n) || !ticket) return NUDIM_EINVAL;
    size_t fp = 0;
    NUDIM_TRY(nudim_job_footprint(d, &fp));
    auto r = std::make_unique<Request>();
    r->d = *d;
    r->proj.assign(proj, proj + n);
    r->footprint = fp + ((size_t)128 << 20);  // + NFFT workspace and plans
    r->t_arrival = now_s();
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return NUDIM_ESTATE;
    r->id = s->next_id++;
    *ticket = r->id;
    if (s->t_first < 0) s->t_first = r->t_arrival;
    s->queue.push_back(r.get());
    s->all[r->id] = std::move(r);
    s->cv_work.notify_one();
    return NUDIM_OK;
}

int nudim_server_wait(nudim_server *s, long long ticket, double *vol, size_t n, int crop,
                      double *latency_s)
{
    if (!s) return NUDIM_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) {
        set_error("unknown ticket %lld", ticket);
        return NUDIM_EINVAL;
    }
    Request *r = it->second.get();
    s->cv_done.wait(lk, [&] { return r->state == R_DONE; });
    if (r->rc) {
        set_error("%s", r->err.c_str());
        return r->rc;
    }
    if (latency_s) *latency_s = r->t_done - r->t_arrival;
    if (vol) {
        const nudim_job_desc &d = r->d;
        if (crop) {
            size_t need = (size_t)d.nz * d.nx * d.nx;
            if (n != need) return NUDIM_EINVAL;
            int lo = (d.np - d.nx) / 2, hi = (d.np + d.nx) / 2;
            size_t q = 0;
            for (int i = 0; i < d.nz; i++)
                for (int j = lo; j < hi; j++)
                    for (int k = lo; k < hi; k++)
                        vol[q++] = r->vol[((size_t)i * d.np + j) * d.np + k];
        } else {
            if (n != r->vol.size()) return NUDIM_EINVAL;
            std::copy(r->vol.begin(), r->vol.end(), vol);
        }
    }
    return NUDIM_OK;
}

int nudim_server_stats(nudim_server *s, long long *completed, double *p50_s, double *p99_s,
                       double *jobs_per_s)
{
    if (!s) return NUDIM_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    if (completed) *completed = (long long)s->latencies.size();
    if (p50_s) *p50_s = percentile(s->latencies, 0.50);
    if (p99_s) *p99_s = percentile(s->latencies, 0.99);
    if (jobs_per_s) {
        double span = s->t_last - s->t_first;
        *jobs_per_s = span > 0 ? s->latencies.size() / span : 0;
    }
    return NUDIM_OK;
}

int nudim_server_destroy(nudim_server *s)
{
    if (!s) return NUDIM_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    delete s;
    return NUDIM_OK;
}

}  // extern "C"
