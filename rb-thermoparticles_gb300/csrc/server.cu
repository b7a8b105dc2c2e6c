// server.cu — continuous-batching solve server over the batch engine (include/rbtp.h, rbtp_server_*).
//
// Requests (a case configuration, a horizon in steps and a Nu sampling cadence) are submitted from
// any thread.  Each rbtp_server_tick:
//   1. admits queued requests in arrival order while their device footprint (rbtp_footprint) fits
//      the HBM budget and the active-slot limit: a handle is created, initialised (fresh start of
//      initial.cu:319-331), and joins the resident batch;
//   2. advances the batch by as many steps as no active request needs to stop for — up to the
//      tick size, the next Nu sample of any request, or the end of any request's horizon — so
//      every request runs exactly its horizon and is sampled exactly on its cadence;
//   3. appends a Nu row (output_statis.cu:111-223) to every request that reached a sample step,
//      and retires finished requests, freeing their memory for the queue.
// Work of requests admitted at different times overlaps on the device in the same batched launches;
// state stays resident between ticks.  Each request's result does not depend on what else is in
// the batch (the batched kernels compute every cavity independently).
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "handle.cuh"

namespace {

enum ReqState { REQ_QUEUED = 0, REQ_ACTIVE = 1, REQ_DONE = 2, REQ_FAILED = 3 };

struct ServeReq {
    int id = 0;
    rbtp_config cfg;
    int horizon = 0, every = 0;
    int state = REQ_QUEUED, status = RBTP_OK;
    rbtp_handle *h = nullptr;
    size_t bytes = 0;
    double t_submit = 0, t_admit = -1, t_done = -1;
    int steps_done = 0;
    std::vector<rbtp_nu_row> series;
};

}  // namespace

struct rbtp_server {
    int storage = RBTP_STORE_F32;
    size_t budget = 0, used = 0;
    int max_active = 0;
    rbtp_batch *batch = nullptr;
    std::deque<int> queue;
    std::map<int, ServeReq> reqs;
    std::vector<int> active;
    std::mutex mtx;
    int next_id = 1;
    std::chrono::steady_clock::time_point t0;
    double node_updates = 0.0, steps = 0.0;
    std::string err;
};

namespace {

// Requests are never erased from the map, so a pointer taken under the lock stays valid.
ServeReq *req(rbtp_server *s, int id)
{
    std::lock_guard<std::mutex> lock(s->mtx);
    auto it = s->reqs.find(id);
    return it == s->reqs.end() ? nullptr : &it->second;
}

double now(const rbtp_server *s)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - s->t0).count();
}

void retire(rbtp_server *s, ServeReq &r, int state, int status)
{
    if (r.h) {
        rbtp_batch_remove(s->batch, r.h);
        rbtp_destroy(r.h);
        r.h = nullptr;
    }
    s->used -= std::min(s->used, r.bytes);
    r.state = state;
    r.status = status;
    r.t_done = now(s);
    s->active.erase(std::remove(s->active.begin(), s->active.end(), r.id), s->active.end());
}

// Admission in arrival order (no reordering: a large request at the head waits for memory).
void admit(rbtp_server *s)
{
    for (;;) {
        int id;
        {
            std::lock_guard<std::mutex> lock(s->mtx);
            if (s->queue.empty()) return;
            id = s->queue.front();
            ServeReq &r = s->reqs.find(id)->second;
            if (s->max_active > 0 && (int)s->active.size() >= s->max_active) return;
            if (s->used + r.bytes > s->budget) {
                if (!s->active.empty()) return;   // wait for memory to free up
                s->queue.pop_front();              // cannot fit even alone
                r.state = REQ_FAILED;
                r.status = RBTP_ERR_OOM;
                r.t_done = now(s);
                continue;
            }
            s->queue.pop_front();
            s->used += r.bytes;
        }
        ServeReq &r = *req(s, id);
        int st = rbtp_create(&r.cfg, &r.h);
        if (st == RBTP_OK) st = rbtp_init_fresh(r.h);
        if (st == RBTP_OK) st = rbtp_batch_add(s->batch, r.h);
        if (st == RBTP_OK) st = rbtp_batch_set_sampling(s->batch, r.h, r.every);
        r.t_admit = now(s);
        if (st != RBTP_OK) {
            if (r.h && r.h->batch) rbtp_batch_remove(s->batch, r.h);
            if (r.h) rbtp_destroy(r.h);
            r.h = nullptr;
            s->used -= std::min(s->used, r.bytes);
            r.state = REQ_FAILED;
            r.status = st;
            r.t_done = now(s);
            continue;
        }
        r.state = REQ_ACTIVE;
        s->active.push_back(id);
    }
}

}  // namespace

extern "C" {

int rbtp_server_create(int storage, double hbm_budget_bytes, int max_active, rbtp_server **out)
{
    if (!out || hbm_budget_bytes <= 0) return RBTP_ERR_ARG;
    *out = nullptr;
    rbtp_server *s = new rbtp_server();
    s->storage = storage;
    s->budget = (size_t)hbm_budget_bytes;
    s->max_active = max_active;
    s->t0 = std::chrono::steady_clock::now();
    int st = rbtp_batch_create(storage, &s->batch);
    if (st != RBTP_OK) {
        delete s;
        return st;
    }
    *out = s;
    return RBTP_OK;
}

int rbtp_server_destroy(rbtp_server *s)
{
    if (!s) return RBTP_OK;
    for (int id : std::vector<int>(s->active)) retire(s, *req(s, id), REQ_FAILED, RBTP_ERR_STATE);
    rbtp_batch_destroy(s->batch);
    delete s;
    return RBTP_OK;
}

int rbtp_server_submit(rbtp_server *s, const rbtp_config *cfg, int horizon, int sample_every, int *id)
{
    if (!s || !cfg || !id || horizon <= 0 || sample_every < 0) return RBTP_ERR_ARG;
    ServeReq r;
    r.cfg = *cfg;
    r.cfg.storage = s->storage;
    r.cfg.continuous_steps = 0;
    r.cfg.nend = horizon;           // the final step materialises the fields of the last Nu row
    r.cfg.nflowout = 0;
    r.horizon = horizon;
    r.every = sample_every;
    int st = rbtp_footprint(&r.cfg, &r.bytes);
    if (st != RBTP_OK) return st;
    std::lock_guard<std::mutex> lock(s->mtx);
    r.id = s->next_id++;
    r.t_submit = now(s);
    *id = r.id;
    s->queue.push_back(r.id);
    s->reqs[r.id] = std::move(r);
    return RBTP_OK;
}

int rbtp_server_tick(rbtp_server *s, int max_steps, int *nactive, int *nqueued)
{
    if (!s || max_steps <= 0) return RBTP_ERR_ARG;
    admit(s);
    if (!s->active.empty()) {
        int k = max_steps;
        for (int id : s->active) {
            const ServeReq &r = *req(s, id);
            k = std::min(k, r.horizon - r.steps_done);
            if (r.every > 0) k = std::min(k, r.every - r.steps_done % r.every);
        }
        k = std::max(k, 1);
        int st = rbtp_batch_step(s->batch, k);
        if (st != RBTP_OK) {
            // fail the members whose status is bad; the rest keep their state (rbtp_batch_step
            // synchronised every member before returning)
            for (int id : std::vector<int>(s->active)) {
                ServeReq &r = *req(s, id);
                const DevStatus &ds = *r.h->status_host;
                if (ds.nonfinite || ds.link_overflow || ds.nf_overflow || ds.contact_overflow)
                    retire(s, r, REQ_FAILED, ds.nonfinite ? RBTP_ERR_NONFINITE : RBTP_ERR_CAPACITY);
            }
            if (st != RBTP_ERR_NONFINITE && st != RBTP_ERR_CAPACITY) {
                s->err = "batch step failed";
                return st;
            }
        } else {
            double nodes = 0.0;
            for (int id : s->active) nodes += (double)req(s, id)->h->geo.L;
            s->node_updates += nodes * k;
            s->steps += k;
        }
        for (int id : std::vector<int>(s->active)) {
            ServeReq &r = *req(s, id);
            if (r.state != REQ_ACTIVE) continue;
            r.steps_done += k;
            const bool sample = (r.every > 0 && r.steps_done % r.every == 0) || r.steps_done == r.horizon;
            if (sample) {
                rbtp_nu_row row;
                const int ns = rbtp_nu(r.h, r.steps_done, &row);
                if (ns != RBTP_OK) {
                    retire(s, r, REQ_FAILED, ns);
                    continue;
                }
                std::lock_guard<std::mutex> lock(s->mtx);
                r.series.push_back(row);
            }
            if (r.steps_done >= r.horizon) retire(s, r, REQ_DONE, RBTP_OK);
        }
    }
    std::lock_guard<std::mutex> lock(s->mtx);
    if (nactive) *nactive = (int)s->active.size();
    if (nqueued) *nqueued = (int)s->queue.size();
    return RBTP_OK;
}

int rbtp_server_poll(rbtp_server *s, int id, int *state, int *steps_done, rbtp_nu_row *rows, int cap,
                     int *nrows)
{
    if (!s) return RBTP_ERR_ARG;
    std::lock_guard<std::mutex> lock(s->mtx);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return RBTP_ERR_ARG;
    const ServeReq &r = it->second;
    if (state) *state = r.state;
    if (steps_done) *steps_done = r.steps_done;
    const int n = (int)r.series.size();
    if (nrows) *nrows = n;
    if (rows) std::memcpy(rows, r.series.data(), (size_t)std::min(n, std::max(cap, 0)) * sizeof(rbtp_nu_row));
    return r.status;
}

int rbtp_server_request_times(rbtp_server *s, int id, double *t_submit, double *t_admit, double *t_done)
{
    if (!s) return RBTP_ERR_ARG;
    std::lock_guard<std::mutex> lock(s->mtx);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return RBTP_ERR_ARG;
    if (t_submit) *t_submit = it->second.t_submit;
    if (t_admit) *t_admit = it->second.t_admit;
    if (t_done) *t_done = it->second.t_done;
    return RBTP_OK;
}

int rbtp_server_stats(rbtp_server *s, double *node_updates, double *steps, double *used_bytes, double *clock)
{
    if (!s) return RBTP_ERR_ARG;
    std::lock_guard<std::mutex> lock(s->mtx);
    if (node_updates) *node_updates = s->node_updates;
    if (steps) *steps = s->steps;
    if (used_bytes) *used_bytes = (double)s->used;
    if (clock) *clock = now(s);
    return RBTP_OK;
}

}  // extern "C"
