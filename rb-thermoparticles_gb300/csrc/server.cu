// server.cu — continuous-batching solve server over the batch engine (include/rbtp.h, rbtp_server_*).
//
// Requests (a case configuration, a horizon in steps and a Nu sampling cadence) are submitted from
// any thread.  Each rbtp_server_tick:
//   1. launches the tick's steps of the resident batch (rbtp_batch_launch).  Every request stops on
//      the device at its own horizon (rbtp_batch_set_stop) and samples on its own cadence into its
//      sample ring (rbtp_batch_set_sampling), so the tick length does not depend on any request's
//      horizon or sample steps: it is the tick size, capped by the longest remaining horizon and by
//      the sample-ring capacity;
//   2. while those steps run, prepares queued requests in arrival order while their device
//      footprint (rbtp_footprint) fits the HBM budget and the active-slot limit: a handle is
//      created and initialised (fresh start of initial.cu:319-331) on its own stream;
//   3. waits for the steps, turns each request's new samples into Nu rows (output_statis.cu:111-223),
//      retires finished requests (freeing their memory for the queue) and lets the prepared
//      requests join the batch for the next tick.
// Work of requests admitted at different times overlaps on the device in the same batched launches;
// state stays resident between ticks.  Each request's result does not depend on what else is in
// the batch (the batched kernels compute every cavity independently).
#include <algorithm>
#include <chrono>
#include <cstdio>
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
    std::vector<int> prepared;   // created and initialised, joining the batch after this tick
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
// Runs while the batch's steps are in flight: handle creation and the fresh start use the
// request's own stream.
void prepare(rbtp_server *s)
{
    for (;;) {
        int id;
        {
            std::lock_guard<std::mutex> lock(s->mtx);
            if (s->queue.empty()) return;
            id = s->queue.front();
            ServeReq &r = s->reqs.find(id)->second;
            if (s->max_active > 0 && (int)(s->active.size() + s->prepared.size()) >= s->max_active) return;
            if (s->used + r.bytes > s->budget) {
                if (!s->active.empty() || !s->prepared.empty()) return;   // wait for memory to free up
                s->queue.pop_front();                                      // cannot fit even alone
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
        r.t_admit = now(s);
        if (st != RBTP_OK) {
            if (r.h) rbtp_destroy(r.h);
            r.h = nullptr;
            s->used -= std::min(s->used, r.bytes);
            r.state = REQ_FAILED;
            r.status = st;
            r.t_done = now(s);
            continue;
        }
        r.state = REQ_ACTIVE;
        s->prepared.push_back(id);
    }
}

// Prepared requests join the batch (after the tick's steps have ended).
void join(rbtp_server *s)
{
    for (int id : s->prepared) {
        ServeReq &r = *req(s, id);
        int st = rbtp_batch_add(s->batch, r.h);
        if (st == RBTP_OK) st = rbtp_batch_set_sampling(s->batch, r.h, r.every);
        if (st == RBTP_OK) st = rbtp_batch_set_stop(s->batch, r.h, r.horizon);
        if (st != RBTP_OK) {
            retire(s, r, REQ_FAILED, st);
            continue;
        }
        s->active.push_back(id);
    }
    s->prepared.clear();
}

// New samples of an active request become Nu rows of its series.
int drain(rbtp_server *s, ServeReq &r)
{
    rbtp_nu_row rows[64];
    for (;;) {
        int n = 0;
        const int st = rbtp_batch_samples(s->batch, r.h, rows, 64, &n);
        if (n > 0) {
            std::lock_guard<std::mutex> lock(s->mtx);
            r.series.insert(r.series.end(), rows, rows + n);
        }
        if (st != RBTP_OK) return st;
        if (n < 64) return RBTP_OK;
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
    rbtp_batch_wait(s->batch);
    for (int id : std::vector<int>(s->active)) retire(s, *req(s, id), REQ_FAILED, RBTP_ERR_STATE);
    for (int id : std::vector<int>(s->prepared)) retire(s, *req(s, id), REQ_FAILED, RBTP_ERR_STATE);
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
    int k = 0;
    if (!s->active.empty()) {
        int remaining = 1;
        for (int id : s->active) {
            const ServeReq &r = *req(s, id);
            remaining = std::max(remaining, r.horizon - r.steps_done);
            if (r.every > 0) k = k > 0 ? std::min(k, 63 * r.every) : 63 * r.every;   // ring: 64 slots
        }
        k = std::min(k > 0 ? k : max_steps, std::min(max_steps, remaining));
        const int st = rbtp_batch_launch(s->batch, k);
        if (st != RBTP_OK) {
            s->err = "batch launch failed";
            return st;
        }
    }
    prepare(s);   // overlaps the steps in flight
    if (k > 0) {
        const int st = rbtp_batch_wait(s->batch);
        if (st != RBTP_OK) {
            // fail the members whose status is bad; the rest keep their state (the wait
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
        }
        double updates = 0.0;
        for (int id : std::vector<int>(s->active)) {
            ServeReq &r = *req(s, id);
            if (r.state != REQ_ACTIVE) continue;
            const int taken = r.h->istep - r.steps_done;
            updates += (double)r.h->geo.L * taken;
            r.steps_done = r.h->istep;
            const int ds = drain(s, r);
            if (ds != RBTP_OK) {
                retire(s, r, REQ_FAILED, ds);
                continue;
            }
            if (r.steps_done >= r.horizon) retire(s, r, REQ_DONE, RBTP_OK);
        }
        std::lock_guard<std::mutex> lock(s->mtx);
        s->node_updates += updates;
        s->steps += k;
    }
    join(s);
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

// Checkpoint between ticks: server.bin (every request's record: configuration, horizon, cadence,
// state, status, steps, times, Nu series) plus one exact handle checkpoint per active request
// (rbtp_checkpoint_write).  Restore rebuilds the records, re-queues queued requests in their
// order, resumes active requests from their checkpoints in the batch, and continues the clock.
namespace {
constexpr char SRV_MAGIC[9] = "RBTPSRV1";
struct SrvRecord {
    int id, state, status, horizon, every, steps_done, nseries, pad;
    double t_submit, t_admit, t_done;
    size_t bytes;
};
std::string ckp_path(const char *dir, int id)
{
    return std::string(dir) + "/req_" + std::to_string(id) + ".ckp";
}
}  // namespace

int rbtp_server_checkpoint(rbtp_server *s, const char *dir)
{
    if (!s || !dir) return RBTP_ERR_ARG;
    if (!s->prepared.empty()) return RBTP_ERR_STATE;   // only between ticks
    for (int id : s->active) {
        const int st = rbtp_checkpoint_write(req(s, id)->h, ckp_path(dir, id).c_str());
        if (st) return st;
    }
    std::lock_guard<std::mutex> lock(s->mtx);
    const std::string path = std::string(dir) + "/server.bin";
    FILE *fp = std::fopen(path.c_str(), "wb");
    if (!fp) return RBTP_ERR_IO;
    const int n = (int)s->reqs.size();
    const double clock = now(s);
    bool ok = std::fwrite(SRV_MAGIC, 1, 8, fp) == 8 && std::fwrite(&n, sizeof(int), 1, fp) == 1 &&
              std::fwrite(&s->next_id, sizeof(int), 1, fp) == 1 && std::fwrite(&clock, sizeof(double), 1, fp) == 1 &&
              std::fwrite(&s->node_updates, sizeof(double), 1, fp) == 1 &&
              std::fwrite(&s->steps, sizeof(double), 1, fp) == 1;
    for (const auto &kv : s->reqs) {
        const ServeReq &r = kv.second;
        SrvRecord rec{r.id, r.state, r.status, r.horizon, r.every, r.steps_done, (int)r.series.size(), 0,
                      r.t_submit, r.t_admit, r.t_done, r.bytes};
        ok = ok && std::fwrite(&rec, sizeof(rec), 1, fp) == 1 && std::fwrite(&r.cfg, sizeof(rbtp_config), 1, fp) == 1 &&
             std::fwrite(r.series.data(), sizeof(rbtp_nu_row), r.series.size(), fp) == r.series.size();
    }
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? RBTP_OK : RBTP_ERR_IO;
}

int rbtp_server_restore(rbtp_server *s, const char *dir)
{
    if (!s || !dir) return RBTP_ERR_ARG;
    if (!s->reqs.empty()) return RBTP_ERR_STATE;        // into a fresh server only
    const std::string path = std::string(dir) + "/server.bin";
    FILE *fp = std::fopen(path.c_str(), "rb");
    if (!fp) return RBTP_ERR_IO;
    char magic[8];
    int n = 0, next_id = 1;
    double clock = 0.0, updates = 0.0, steps = 0.0;
    bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, SRV_MAGIC, 8) == 0 &&
              std::fread(&n, sizeof(int), 1, fp) == 1 && std::fread(&next_id, sizeof(int), 1, fp) == 1 &&
              std::fread(&clock, sizeof(double), 1, fp) == 1 && std::fread(&updates, sizeof(double), 1, fp) == 1 &&
              std::fread(&steps, sizeof(double), 1, fp) == 1 && n >= 0;
    std::vector<ServeReq> recs;
    for (int k = 0; ok && k < n; ++k) {
        SrvRecord rec;
        ServeReq r;
        ok = std::fread(&rec, sizeof(rec), 1, fp) == 1 && std::fread(&r.cfg, sizeof(rbtp_config), 1, fp) == 1 &&
             rec.nseries >= 0;
        if (!ok) break;
        r.series.resize(rec.nseries);
        ok = std::fread(r.series.data(), sizeof(rbtp_nu_row), rec.nseries, fp) == (size_t)rec.nseries;
        r.id = rec.id; r.state = rec.state; r.status = rec.status; r.horizon = rec.horizon; r.every = rec.every;
        r.steps_done = rec.steps_done; r.t_submit = rec.t_submit; r.t_admit = rec.t_admit; r.t_done = rec.t_done;
        r.bytes = rec.bytes;
        recs.push_back(std::move(r));
    }
    std::fclose(fp);
    if (!ok) return RBTP_ERR_IO;
    s->t0 = std::chrono::steady_clock::now() -
            std::chrono::duration_cast<std::chrono::steady_clock::duration>(std::chrono::duration<double>(clock));
    s->next_id = next_id;
    s->node_updates = updates;
    s->steps = steps;
    for (ServeReq &r : recs) {
        const int id = r.id;
        const int state = r.state;
        {
            std::lock_guard<std::mutex> lock(s->mtx);
            s->reqs[id] = std::move(r);
            if (state == REQ_QUEUED) s->queue.push_back(id);   // ids ascend in arrival order
        }
        if (state != REQ_ACTIVE) continue;
        ServeReq &q = *req(s, id);
        int st = rbtp_create(&q.cfg, &q.h);
        if (st == RBTP_OK) st = rbtp_checkpoint_read(q.h, ckp_path(dir, id).c_str());
        if (st != RBTP_OK) {
            if (q.h) rbtp_destroy(q.h);
            q.h = nullptr;
            q.state = REQ_FAILED;
            q.status = st;
            q.t_done = now(s);
            continue;
        }
        s->used += q.bytes;
        s->prepared.push_back(id);
    }
    join(s);
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
