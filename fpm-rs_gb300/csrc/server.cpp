// Serving loop: continuous batching of reconstruction requests on one
// context, the request loop that serves run_algorithm
// (python/src/reconstruction.rs:1107-1141) to many callers.
//
// Callers submit requests (model, measurements, algorithm parameters, result
// arrays) and return at once. A dispatcher thread admits waiting requests in
// arrival order while their estimated device footprint fits the HBM budget
// beside the work already in flight; requests with equal parameters that
// arrive within the batching window go out as one submitted batch (one job,
// one frame-engine launch per tile size); and as jobs finish, their memory is
// released and the next requests are admitted, so new work overlaps the
// work already on the GPU. A request's state (measurements, object, pupil,
// mPIE momentum) lives on the device from admission to completion. The
// server is built on the public entry points only (problems and submitted
// jobs), so each request's result is bit-identical to a run of that request
// alone.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "fpm_gpu.h"
#include "kernels.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t id = 0;
    fpm_model_desc model{};
    fpm_measurement_desc meas{};
    fpm_algorithm_params params{};
    fpm_result_desc* result = nullptr;
    int64_t footprint = 0;
    fpm_request_info info{};
    fpm_problem* problem = nullptr;
    bool done = false;
};

struct Flight {
    fpm_job* job = nullptr;
    std::vector<std::shared_ptr<Request>> requests;
    std::vector<fpm_result_desc> results;  // the job writes here; copied to the callers' descriptors
    int64_t footprint = 0;
};

// Device bytes a request holds while admitted: float32 measurements (with
// masks and background when present), the FP64 staging of its upload, the
// complex64 object (with mPIE velocity and anchor, the mini-batch GD
// gradient), the FP64 grid scratch, pupils and per-frame constants.
int64_t request_footprint(const fpm_model_desc& m, const fpm_measurement_desc& ms, const fpm_algorithm_params& a) {
    const int64_t n2 = (int64_t)m.image_height * m.image_width;
    const int64_t frames = ms.frames;
    const int64_t grid = (int64_t)m.recon_height * (m.recon_width + (m.recon_width & 1));
    int64_t bytes = frames * n2 * 4 + frames * n2 * 8;
    if (ms.masks) bytes += frames * n2;
    if (m.background) bytes += (int64_t)m.background_len * 4;
    int64_t grids = 1;
    if (a.algorithm == FPM_ALG_MPIE) grids += 2;
    if (a.algorithm == FPM_ALG_GD && a.batch_size > 1) grids += 1;
    bytes += grids * grid * 8 + (int64_t)m.recon_height * m.recon_width * 16;
    bytes += n2 * (8 + 8 + 16 + 1) + frames * 64 + (4 << 10);
    return bytes;
}

// The error text of a refused call, under the context's lock like every
// other entry point's.
int32_t refuse(fpm_context* ctx, int32_t code, const char* message) {
    if (ctx) {
        std::lock_guard<std::mutex> lock(fpm::context_mutex(ctx));
        fpm::set_context_error(ctx, message);
    } else {
        fpm::set_context_error(nullptr, message);
    }
    return code;
}

double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

}  // namespace

struct fpm_server {
    fpm_context* ctx = nullptr;
    fpm_server_config cfg{};
    Clock::time_point t0 = Clock::now();
    std::mutex mu;
    std::condition_variable wake;      // new work or shutdown, for the dispatcher
    std::condition_variable finished;  // a request completed, for waiters
    std::deque<std::shared_ptr<Request>> queue;
    std::map<uint64_t, std::shared_ptr<Request>> requests;
    std::vector<Flight> flights;
    int64_t in_use = 0;
    uint64_t next_id = 1;
    bool stopping = false;
    std::thread worker;
    fpm_server_stats stats{};

    void run();
    void complete(Flight& f, int32_t status, const std::string& message);
};

void fpm_server::complete(Flight& f, int32_t status, const std::string& message) {
    const double now = ms_since(t0);
    for (size_t i = 0; i < f.requests.size(); ++i) {
        Request& r = *f.requests[i];
        if (status == FPM_OK && r.result) {
            r.result->completed_iterations = f.results[i].completed_iterations;
        }
        if (r.problem) fpm_problem_destroy(r.problem);
        r.problem = nullptr;
        r.info.done_ms = now;
        r.info.status = status;
        std::snprintf(r.info.message, sizeof r.info.message, "%s", message.c_str());
        r.done = true;
    }
}

void fpm_server::run() {
    std::unique_lock<std::mutex> lock(mu);
    for (;;) {
        // Finished jobs: release their memory and their requests.
        for (size_t k = 0; k < flights.size();) {
            Flight& f = flights[k];
            int32_t done = 0;
            lock.unlock();
            const int32_t st = fpm_job_poll(f.job, &done);
            std::string message;
            if (done && st != FPM_OK) {
                char buf[sizeof(fpm_request_info::message)];
                fpm_last_error(ctx, buf, sizeof buf);
                message = buf;
            }
            lock.lock();
            if (!done) {
                ++k;
                continue;
            }
            lock.unlock();
            fpm_job_destroy(f.job);
            lock.lock();
            complete(f, st, message);
            in_use -= f.footprint;
            stats.completed += (int64_t)f.requests.size();
            flights.erase(flights.begin() + (long)k);
            finished.notify_all();
        }
        if (stopping && queue.empty() && flights.empty()) break;
        // Admission: the oldest waiting request and the later ones with the
        // same parameters, in arrival order, while they fit the budget.
        bool dispatched = false;
        if (!queue.empty()) {
            std::shared_ptr<Request> head = queue.front();
            const double waited = ms_since(t0) - head->info.submit_ms;
            std::vector<std::shared_ptr<Request>> batch;
            int64_t need = 0;
            for (const auto& r : queue) {
                if ((int)batch.size() >= cfg.max_batch) break;
                if (std::memcmp(&r->params, &head->params, sizeof(fpm_algorithm_params)) != 0) continue;
                if (cfg.hbm_budget_bytes > 0 && in_use + need + r->footprint > cfg.hbm_budget_bytes) break;
                batch.push_back(r);
                need += r->footprint;
            }
            const bool full = (int)batch.size() >= cfg.max_batch;
            const bool window_over = waited >= cfg.batch_window_ms || stopping;
            if (!batch.empty() && (full || window_over)) {
                for (const auto& r : batch) queue.erase(std::find(queue.begin(), queue.end(), r));
                const double admit = ms_since(t0);
                for (const auto& r : batch) r->info.admit_ms = admit;
                in_use += need;
                Flight f;
                f.requests = batch;
                f.footprint = need;
                stats.admitted += (int64_t)batch.size();
                stats.batches += 1;
                stats.peak_bytes = std::max(stats.peak_bytes, in_use);
                lock.unlock();
                // Device problems for each request (one failing request does
                // not fail the others), then one submitted batch.
                std::vector<fpm_problem*> problems;
                std::vector<std::shared_ptr<Request>> ok;
                for (const auto& r : batch) {
                    fpm_problem* p = nullptr;
                    const int32_t st = fpm_problem_create(ctx, &r->model, &r->meas, &p);
                    if (st != FPM_OK) {
                        char buf[sizeof(fpm_request_info::message)];
                        fpm_last_error(ctx, buf, sizeof buf);
                        Flight single;
                        single.requests = {r};
                        lock.lock();
                        complete(single, st, buf);
                        in_use -= r->footprint;
                        f.footprint -= r->footprint;
                        stats.completed += 1;
                        finished.notify_all();
                        lock.unlock();
                        continue;
                    }
                    r->problem = p;
                    problems.push_back(p);
                    ok.push_back(r);
                }
                f.requests = ok;
                f.results.resize(ok.size());
                for (size_t i = 0; i < ok.size(); ++i) f.results[i] = *ok[i]->result;
                int32_t st = FPM_OK;
                if (!ok.empty())
                    st = fpm_run_batch_submit(ctx, (int32_t)problems.size(), problems.data(), &head->params,
                                              f.results.data(), &f.job);
                lock.lock();
                const double start = ms_since(t0);
                for (const auto& r : ok) r->info.start_ms = start;
                if (ok.empty()) {
                    // Every request of the batch failed at creation.
                } else if (st != FPM_OK) {
                    char buf[sizeof(fpm_request_info::message)];
                    fpm_last_error(ctx, buf, sizeof buf);
                    complete(f, st, buf);
                    in_use -= f.footprint;
                    stats.completed += (int64_t)ok.size();
                    finished.notify_all();
                } else {
                    flights.push_back(std::move(f));
                }
                dispatched = true;
            }
        }
        if (dispatched) continue;
        // Idle: sleep until new work arrives, or briefly while jobs run or a
        // batching window is open.
        const bool busy = !flights.empty() || !queue.empty();
        if (busy) wake.wait_for(lock, std::chrono::microseconds(200));
        else wake.wait(lock);
    }
}

extern "C" {

int32_t fpm_server_create(fpm_context* ctx, const fpm_server_config* config, fpm_server** out) {
    if (!ctx || !config || !out)
        return refuse(ctx, FPM_ERR_INVALID_PARAMETER, "fpm_server_create: null argument");
    if (config->max_batch < 1 || !(config->batch_window_ms >= 0.0) || config->hbm_budget_bytes < 0 ||
        config->max_queue < 0)
        return refuse(ctx, FPM_ERR_INVALID_PARAMETER,
                      "fpm_server_create: max_batch must be at least 1 and the window, budget and queue "
                      "limit non-negative");
    auto s = std::make_unique<fpm_server>();
    s->ctx = ctx;
    s->cfg = *config;
    s->worker = std::thread([srv = s.get()] { srv->run(); });
    *out = s.release();
    return FPM_OK;
}

int32_t fpm_server_submit(fpm_server* s, const fpm_model_desc* model, const fpm_measurement_desc* measurements,
                          const fpm_algorithm_params* params, fpm_result_desc* result, uint64_t* request) {
    if (!s || !model || !measurements || !params || !result || !request)
        return refuse(s ? s->ctx : nullptr, FPM_ERR_INVALID_PARAMETER, "fpm_server_submit: null argument");
    auto r = std::make_shared<Request>();
    r->model = *model;
    r->meas = *measurements;
    r->params = *params;
    r->result = result;
    r->footprint = request_footprint(*model, *measurements, *params);
    std::unique_lock<std::mutex> lock(s->mu);
    if (s->stopping) {
        lock.unlock();
        return refuse(s->ctx, FPM_ERR_INVALID_PARAMETER, "fpm_server_submit: the server is stopping");
    }
    if (s->cfg.hbm_budget_bytes > 0 && r->footprint > s->cfg.hbm_budget_bytes) {
        char text[256];
        std::snprintf(text, sizeof text,
                      "fpm_server_submit: the request needs %lld device bytes, more than the server's whole HBM "
                      "budget of %lld", (long long)r->footprint, (long long)s->cfg.hbm_budget_bytes);
        lock.unlock();
        return refuse(s->ctx, FPM_ERR_INVALID_PARAMETER, text);
    }
    if (s->cfg.max_queue > 0 && (int64_t)s->queue.size() >= s->cfg.max_queue) {
        s->stats.rejected += 1;
        lock.unlock();
        return refuse(s->ctx, FPM_ERR_QUEUE_FULL, "fpm_server_submit: the queue is full");
    }
    r->id = s->next_id++;
    r->info.submit_ms = ms_since(s->t0);
    r->info.footprint_bytes = r->footprint;
    r->info.status = -1;
    s->queue.push_back(r);
    s->requests[r->id] = r;
    s->stats.submitted += 1;
    *request = r->id;
    s->wake.notify_one();
    return FPM_OK;
}

int32_t fpm_server_poll(fpm_server* s, uint64_t request, int32_t* done) {
    if (!s || !done) return refuse(s ? s->ctx : nullptr, FPM_ERR_INVALID_PARAMETER, "fpm_server_poll: null argument");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->requests.find(request);
    if (it == s->requests.end()) {
        lock.unlock();
        return refuse(s->ctx, FPM_ERR_INVALID_PARAMETER, "fpm_server_poll: unknown request");
    }
    *done = it->second->done ? 1 : 0;
    return FPM_OK;
}

int32_t fpm_server_wait(fpm_server* s, uint64_t request, fpm_request_info* info) {
    if (!s) return refuse(nullptr, FPM_ERR_INVALID_PARAMETER, "fpm_server_wait: null server");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->requests.find(request);
    if (it == s->requests.end()) {
        lock.unlock();
        return refuse(s->ctx, FPM_ERR_INVALID_PARAMETER, "fpm_server_wait: unknown request");
    }
    std::shared_ptr<Request> r = it->second;
    s->finished.wait(lock, [&] { return r->done; });
    if (info) *info = r->info;
    s->requests.erase(r->id);
    lock.unlock();
    if (r->info.status != FPM_OK) return refuse(s->ctx, r->info.status, r->info.message);
    return FPM_OK;
}

int32_t fpm_server_stats_get(fpm_server* s, fpm_server_stats* stats) {
    if (!s || !stats) return refuse(s ? s->ctx : nullptr, FPM_ERR_INVALID_PARAMETER, "fpm_server_stats_get: null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    *stats = s->stats;
    stats->in_use_bytes = s->in_use;
    stats->waiting = (int64_t)s->queue.size();
    stats->in_flight_batches = (int64_t)s->flights.size();
    return FPM_OK;
}

int32_t fpm_server_destroy(fpm_server* s) {
    if (!s) return FPM_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stopping = true;
    }
    s->wake.notify_one();
    if (s->worker.joinable()) s->worker.join();
    delete s;
    return FPM_OK;
}

}  // extern "C"
