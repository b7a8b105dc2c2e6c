// batch.cu — host side of batched execution (include/rbtp.h, rbtp_batch_*).
//
// A batch advances many independent cavities in lockstep.  Per step it enqueues: a plan kernel
// (each cavity's output mode for the step, from its cadence), ONE persistent launch of the fused
// step over the packed tile table of all cavities, the particle pipeline as one launch per kernel
// over the packed (cavity, particle) map, and an advance kernel (owner parity, AA phase, step
// counter).  Every piece of per-step state lives in the device descriptors, so the sequence is
// captured once into a CUDA graph and replayed for every step.  The autotuner times the candidate
// (tile shape, persistent grid) pairs on the first steps of the batch — all candidates compute the
// same values, so tuning steps are ordinary steps — and keeps the fastest.
//
// For continuous batching each member may carry a stop step (it goes idle there while the others
// keep going: no batch call has to end on any member's horizon) and a sample ring (the step ends
// with an on-device plane-sum reduction on the member's sampling cadence, so no batch call has to
// end on a sample step either; the host turns ring slots into Nu rows later).  rbtp_batch_launch
// returns with the steps in flight so the caller can prepare the next members meanwhile.
#include <algorithm>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "handle.cuh"

struct rbtp_batch {
    int mode = RBTP_STORE_F32;
    int device = 0;
    int sms = 1;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    // side branch of each step (the contact kernels beside IBB) and its fork/join events
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::vector<rbtp_handle *> members;
    CavDesc *d_desc = nullptr, *h_desc = nullptr;
    int desc_cap = 0;
    int4 *d_tiles[BATCH_SHAPES] = {nullptr, nullptr};
    int ntiles[BATCH_SHAPES] = {0, 0};
    int2 *d_pmap = nullptr;
    int total_np = 0;
    int2 *d_cmap = nullptr;    // (particle map entry, IBB link chunk) of every IBB CTA
    int ncmap = 0;
    int *d_pmem = nullptr;
    int npmem = 0;
    bool dirty = true;
    // launch configuration (grid_factor: persistent blocks per SM, 0 = one block per tile)
    int shape = 0, grid = 0, grid_factor = 8;
    bool tuned = false, forced = false;
    std::vector<std::pair<int, int>> cand;  // (shape, grid)
    std::vector<float> cand_ms;
    // graph
    cudaGraphExec_t gexec = nullptr;
    bool graph_valid = false;
    double last_ms = 0.0;
    double nodes = 0.0;
    // asynchronous launch
    bool inflight = false;
    int inflight_steps = 0;
    bool inflight_timed = false;
    std::string err;
};

// Slots of a member's sample ring.
constexpr int RING_SLOTS = 64;

namespace {

int bfail(rbtp_batch *b, int code, const std::string &m)
{
    if (b) b->err = m;
    return code;
}

#define BCK(call)                                                                                     \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return bfail(b, e_ == cudaErrorMemoryAllocation ? RBTP_ERR_OOM : RBTP_ERR_CUDA, \
                                            std::string(#call) + ": " + cudaGetErrorString(e_));      \
    } while (0)

void drop_graph(rbtp_batch *b)
{
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
    b->graph_valid = false;
}

template <class T>
int upload(rbtp_batch *b, T **dptr, const std::vector<T> &v)
{
    if (*dptr) cudaFree(*dptr);
    *dptr = nullptr;
    BCK(cudaMalloc(reinterpret_cast<void **>(dptr), std::max<size_t>(v.size(), 1) * sizeof(T)));
    if (!v.empty()) BCK(cudaMemcpy(*dptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return RBTP_OK;
}

// Tile tables (both shapes), the particle map and the list of cavities with particles.
int rebuild(rbtp_batch *b)
{
    drop_graph(b);
    const int n = (int)b->members.size();
    const int tx[BATCH_SHAPES] = {32, 64}, ty[BATCH_SHAPES] = {4, 2};
    for (int s = 0; s < BATCH_SHAPES; ++s) {
        std::vector<int4> t;
        for (int m = 0; m < n; ++m) {
            const Geo &g = b->members[m]->geo;
            const int nx = (g.lx + tx[s] - 1) / tx[s], ny = (g.ly + ty[s] - 1) / ty[s];
            for (int z = 0; z < g.lz; z += BATCH_TILE_Z)
                for (int y = 0; y < ny; ++y)
                    for (int x = 0; x < nx; ++x) t.push_back(make_int4(m, x, y, z));
        }
        b->ntiles[s] = (int)t.size();
        int st = upload(b, &b->d_tiles[s], t);
        if (st) return st;
    }
    std::vector<int2> pmap, cmap;
    std::vector<int> pmem;
    b->nodes = 0.0;
    for (int m = 0; m < n; ++m) {
        const rbtp_handle *h = b->members[m];
        b->nodes += (double)h->geo.L;
        if (h->pb.np > 0) {
            pmem.push_back(m);
            for (int p = 0; p < h->pb.np; ++p) {
                for (int c = 0; c < h->pb.ibb_chunks; ++c) cmap.push_back(make_int2((int)pmap.size(), c));
                pmap.push_back(make_int2(m, p));
            }
        }
    }
    b->total_np = (int)pmap.size();
    b->npmem = (int)pmem.size();
    int st = upload(b, &b->d_pmap, pmap);
    if (st) return st;
    b->ncmap = (int)cmap.size();
    st = upload(b, &b->d_cmap, cmap);
    if (st) return st;
    st = upload(b, &b->d_pmem, pmem);
    if (st) return st;
    if (n > b->desc_cap) {
        if (b->d_desc) cudaFree(b->d_desc);
        if (b->h_desc) cudaFreeHost(b->h_desc);
        b->d_desc = nullptr;
        b->h_desc = nullptr;
        BCK(cudaMalloc(reinterpret_cast<void **>(&b->d_desc), (size_t)n * sizeof(CavDesc)));
        BCK(cudaMallocHost(reinterpret_cast<void **>(&b->h_desc), (size_t)n * sizeof(CavDesc)));
        b->desc_cap = n;
    }
    // autotuner candidates: tile shape x persistent grid (multiples of the SM count) and a full grid
    b->cand.clear();
    b->cand_ms.clear();
    for (int s = 0; s < BATCH_SHAPES; ++s) {
        for (int f : {4, 8, 16}) b->cand.push_back({s, f});
        b->cand.push_back({s, 0});
    }
    // a tuned choice survives membership changes (a serving loop changes them constantly)
    if (!b->forced) b->grid = b->grid_factor > 0 ? std::min(b->ntiles[b->shape], b->grid_factor * b->sms)
                                                 : b->ntiles[b->shape];
    b->dirty = false;
    return RBTP_OK;
}

// Host handle state -> device descriptors (every batch call: single-cavity calls may have changed
// a member in between).
int refresh(rbtp_batch *b)
{
    const int n = (int)b->members.size();
    for (int m = 0; m < n; ++m) {
        rbtp_handle *h = b->members[m];
        CavDesc &d = b->h_desc[m];
        std::memset(&d, 0, sizeof(d));
        d.geo = h->geo;
        d.ph = h->ph;
        d.aoff = make_aa_off(h->geo);
        d.f = h->f;
        d.g = h->g;
        for (int k = 0; k < 2; ++k) d.owner[k] = h->owner[k];
        d.faux = h->faux; d.rho_wall = h->rho_wall;
        d.rho = h->rho; d.ux = h->ux; d.uy = h->uy; d.uz = h->uz; d.phi = h->phi;
        d.status = h->status;
        d.pb = h->pb;
        d.ocur = h->ocur; d.phase = h->phase; d.istep = h->istep;
        d.ndiag = h->cfg.ndiag; d.nnuout = h->cfg.nnuout; d.nflowout = h->cfg.nflowout; d.nend = h->cfg.nend;
        d.every = h->sample_every;
        d.mode = h->mode;
        d.last_out = h->macros_valid ? OUT_MACROS : OUT_NONE;
        d.stop_at = h->stop_at;
        d.samp_now = 0;
        d.samp = h->ring;
        d.samp_cap = h->ring_cap;
        d.nchunks = h->nchunks;
        d.partials = h->partials;
        BCK(cudaStreamSynchronize(h->stream));
    }
    BCK(cudaMemcpyAsync(b->d_desc, b->h_desc, (size_t)n * sizeof(CavDesc), cudaMemcpyHostToDevice, b->stream));
    return RBTP_OK;
}

cudaError_t enqueue_step(rbtp_batch *b, int shape, int grid)
{
    const int n = (int)b->members.size();
    cudaError_t e;
    if ((e = launch_batch_plan(b->d_desc, n, b->stream))) return e;
    if ((e = launch_step_batched(b->mode, shape, b->d_desc, b->d_tiles[shape], b->ntiles[shape], grid, b->stream)))
        return e;
    if ((e = launch_particles_batched(b->mode, b->d_desc, b->d_pmap, b->total_np, b->d_cmap, b->ncmap, b->d_pmem,
                                        b->npmem, b->stream, b->side, b->ev_fork, b->ev_join)))
        return e;
    if ((e = launch_batch_advance(b->d_desc, n, b->stream))) return e;
    return launch_batch_sample(b->d_desc, n, b->stream);
}

int capture(rbtp_batch *b)
{
    drop_graph(b);
    cudaGraph_t g = nullptr;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_step(b, b->shape, b->grid);
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bfail(b, RBTP_ERR_CUDA, std::string("graph capture failed: ") + cudaGetErrorString(e ? e : e2));
    }
    e = cudaGraphInstantiate(&b->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(b, RBTP_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    b->graph_valid = true;
    return RBTP_OK;
}

// Device step state -> host handles; member status words.
int sync_back(rbtp_batch *b)
{
    const int n = (int)b->members.size();
    BCK(cudaMemcpyAsync(b->h_desc, b->d_desc, (size_t)n * sizeof(CavDesc), cudaMemcpyDeviceToHost, b->stream));
    for (int m = 0; m < n; ++m)
        BCK(cudaMemcpyAsync(b->members[m]->status_host, b->members[m]->status, sizeof(DevStatus),
                            cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    int first = RBTP_OK;
    for (int m = 0; m < n; ++m) {
        rbtp_handle *h = b->members[m];
        const CavDesc &d = b->h_desc[m];
        h->ocur = d.ocur;
        h->phase = d.phase == PHASE_SWAPPED ? PHASE_SWAPPED : PHASE_HOME;
        h->istep = d.istep;
        h->macros_valid = d.last_out == OUT_MACROS;
        h->dissip_valid = false;
        h->plane_valid = false;
        const DevStatus &s = *h->status_host;
        int code = RBTP_OK;
        if (s.link_overflow || s.nf_overflow || s.contact_overflow) { code = RBTP_ERR_CAPACITY; h->err = "device list capacity exceeded in batch step"; }
        else if (s.nonfinite) { code = RBTP_ERR_NONFINITE; h->err = "non-finite density or temperature in the lattice"; }
        if (code && first == RBTP_OK) {
            first = code;
            b->err = "member " + std::to_string(m) + ": " + h->err;
        }
    }
    return first;
}

}  // namespace

void rbtp_batch_detach(rbtp_handle *h);

extern "C" {

int rbtp_batch_create(int storage, rbtp_batch **out)
{
    if (!out) return RBTP_ERR_ARG;
    *out = nullptr;
    if (storage != RBTP_STORE_F64 && storage != RBTP_STORE_F32 && storage != RBTP_STORE_F16S) return RBTP_ERR_CONFIG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return RBTP_ERR_NODEVICE;
    }
    rbtp_batch *b = new rbtp_batch();
    b->mode = storage;
    cudaGetDevice(&b->device);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        rbtp_batch_destroy(b);
        return RBTP_ERR_CUDA;
    }
    *out = b;
    return RBTP_OK;
}

int rbtp_batch_destroy(rbtp_batch *b)
{
    if (!b) return RBTP_OK;
    if (b->inflight) rbtp_batch_wait(b);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (rbtp_handle *h : b->members) h->batch = nullptr;
    drop_graph(b);
    for (int s = 0; s < BATCH_SHAPES; ++s) cudaFree(b->d_tiles[s]);
    cudaFree(b->d_pmap);
    cudaFree(b->d_cmap);
    cudaFree(b->d_pmem);
    cudaFree(b->d_desc);
    if (b->h_desc) cudaFreeHost(b->h_desc);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return RBTP_OK;
}

int rbtp_batch_add(rbtp_batch *b, rbtp_handle *h)
{
    if (!b || !h) return RBTP_ERR_ARG;
    if (b->inflight) return bfail(b, RBTP_ERR_STATE, "a batch launch is in flight");
    if (!h->initialised) return bfail(b, RBTP_ERR_STATE, "member not initialised");
    if (h->batch) return bfail(b, RBTP_ERR_STATE, "handle already belongs to a batch");
    if (h->mode != b->mode) return bfail(b, RBTP_ERR_CONFIG, "storage mode differs from the batch's");
    if (h->device != b->device) return bfail(b, RBTP_ERR_CONFIG, "handle lives on another device");
    b->members.push_back(h);
    h->batch = b;
    b->dirty = true;
    return RBTP_OK;
}

int rbtp_batch_remove(rbtp_batch *b, rbtp_handle *h)
{
    if (!b || !h) return RBTP_ERR_ARG;
    auto it = std::find(b->members.begin(), b->members.end(), h);
    if (it == b->members.end()) return bfail(b, RBTP_ERR_ARG, "handle is not a member");
    if (b->inflight) rbtp_batch_wait(b);   // a member leaving (e.g. destroyed) ends the launch first
    cudaStreamSynchronize(b->stream);
    b->members.erase(it);
    h->batch = nullptr;
    h->sample_every = 0;
    h->stop_at = 0;
    b->dirty = true;
    return RBTP_OK;
}

int rbtp_batch_set_sampling(rbtp_batch *b, rbtp_handle *h, int every)
{
    if (!b || !h || h->batch != b || every < 0) return RBTP_ERR_ARG;
    if (b->inflight) return bfail(b, RBTP_ERR_STATE, "a batch launch is in flight");
    h->sample_every = every;
    if (!h->ring) {
        const size_t stride = 1 + (size_t)NPLANEQ * h->geo.lx;
        BCK(cudaMalloc(reinterpret_cast<void **>(&h->ring), RING_SLOTS * stride * sizeof(double)));
        h->ring_cap = RING_SLOTS;
        BCK(cudaStreamSynchronize(h->stream));
        BCK(cudaMemcpy(h->status_host, h->status, sizeof(DevStatus), cudaMemcpyDeviceToHost));
        h->ring_drained = h->status_host->nsamp;
    }
    return RBTP_OK;
}

int rbtp_batch_set_launch(rbtp_batch *b, int shape, int grid)
{
    if (!b) return RBTP_ERR_ARG;
    if (b->inflight) return bfail(b, RBTP_ERR_STATE, "a batch launch is in flight");
    if (shape < 0) {
        b->forced = false;
        b->tuned = false;
        b->cand_ms.clear();
        drop_graph(b);
        return RBTP_OK;
    }
    if (shape >= BATCH_SHAPES || grid <= 0) return RBTP_ERR_ARG;
    b->forced = true;
    b->tuned = true;
    b->shape = shape;
    b->grid = grid;
    b->grid_factor = -1;
    drop_graph(b);
    return RBTP_OK;
}

int rbtp_batch_launch(rbtp_batch *b, int nsteps)
{
    if (!b || nsteps < 0) return RBTP_ERR_ARG;
    if (b->inflight) return bfail(b, RBTP_ERR_STATE, "a batch launch is already in flight");
    if (b->members.empty() || nsteps == 0) return RBTP_OK;
    if (b->members.size() > 65535) return bfail(b, RBTP_ERR_CONFIG, "more than 65535 members");
    int st;
    if (b->dirty && (st = rebuild(b))) return st;
    if ((st = refresh(b))) return st;
    int done = 0;
    // autotuning: each candidate runs one warm step and one timed step
    while (!b->tuned && done < nsteps) {
        const size_t k = b->cand_ms.size();
        const int cs = b->cand[k].first, cf = b->cand[k].second;
        const int cg = cf > 0 ? std::min(b->ntiles[cs], cf * b->sms) : b->ntiles[cs];
        BCK(enqueue_step(b, cs, cg));
        ++done;
        if (done >= nsteps) break;
        BCK(cudaEventRecord(b->e0, b->stream));
        BCK(enqueue_step(b, cs, cg));
        BCK(cudaEventRecord(b->e1, b->stream));
        BCK(cudaEventSynchronize(b->e1));
        float ms = 0.f;
        BCK(cudaEventElapsedTime(&ms, b->e0, b->e1));
        b->cand_ms.push_back(ms);
        ++done;
        if (b->cand_ms.size() == b->cand.size()) {
            const size_t best = std::min_element(b->cand_ms.begin(), b->cand_ms.end()) - b->cand_ms.begin();
            b->shape = b->cand[best].first;
            b->grid_factor = b->cand[best].second;
            b->grid = b->grid_factor > 0 ? std::min(b->ntiles[b->shape], b->grid_factor * b->sms)
                                         : b->ntiles[b->shape];
            b->tuned = true;
            drop_graph(b);
        }
    }
    b->inflight = true;
    b->inflight_steps = nsteps - done;
    b->inflight_timed = done < nsteps;
    if (done < nsteps) {
        if (!b->graph_valid && (st = capture(b))) {
            b->inflight = false;
            return st;
        }
        BCK(cudaEventRecord(b->e0, b->stream));
        for (int k = done; k < nsteps; ++k) BCK(cudaGraphLaunch(b->gexec, b->stream));
        BCK(cudaEventRecord(b->e1, b->stream));
    }
    return RBTP_OK;
}

int rbtp_batch_wait(rbtp_batch *b)
{
    if (!b) return RBTP_ERR_ARG;
    if (!b->inflight) return RBTP_OK;
    b->inflight = false;
    if (b->inflight_timed) {
        BCK(cudaEventSynchronize(b->e1));
        float ms = 0.f;
        BCK(cudaEventElapsedTime(&ms, b->e0, b->e1));
        b->last_ms = ms / b->inflight_steps;
    }
    return sync_back(b);
}

int rbtp_batch_step(rbtp_batch *b, int nsteps)
{
    int st = rbtp_batch_launch(b, nsteps);
    if (st) return st;
    return rbtp_batch_wait(b);
}

int rbtp_batch_set_stop(rbtp_batch *b, rbtp_handle *h, int stop_step)
{
    if (!b || !h || h->batch != b) return RBTP_ERR_ARG;
    if (b->inflight) return bfail(b, RBTP_ERR_STATE, "a batch launch is in flight");
    h->stop_at = stop_step;
    return RBTP_OK;
}

int rbtp_batch_samples(rbtp_batch *b, rbtp_handle *h, rbtp_nu_row *rows, int cap, int *nrows)
{
    if (!b || !h || h->batch != b || (!rows && cap > 0) || cap < 0) return RBTP_ERR_ARG;
    if (b->inflight) return bfail(b, RBTP_ERR_STATE, "a batch launch is in flight");
    if (nrows) *nrows = 0;
    if (!h->ring) return RBTP_OK;
    const int total = h->status_host->nsamp;   // current after the last batch step
    int status = RBTP_OK;
    if (total - h->ring_drained > h->ring_cap) {  // the ring wrapped: the oldest samples are gone
        h->ring_drained = total - h->ring_cap;
        status = RBTP_ERR_CAPACITY;
        b->err = "sample ring overrun: samples lost (drain more often or sample less often)";
    }
    const int n = std::min(total - h->ring_drained, cap);
    if (n <= 0) return status;
    const size_t stride = 1 + (size_t)NPLANEQ * h->geo.lx;
    std::vector<double> buf((size_t)n * stride);
    const int s0 = h->ring_drained % h->ring_cap;
    const int first = std::min(n, h->ring_cap - s0);
    BCK(cudaMemcpy(buf.data(), h->ring + (size_t)s0 * stride, (size_t)first * stride * sizeof(double),
                   cudaMemcpyDeviceToHost));
    if (n > first)
        BCK(cudaMemcpy(buf.data() + (size_t)first * stride, h->ring, (size_t)(n - first) * stride * sizeof(double),
                       cudaMemcpyDeviceToHost));
    for (int k = 0; k < n; ++k) {
        const double *slot = buf.data() + (size_t)k * stride;
        const int st = nu_from_planes(h, slot + 1, (int)slot[0], &rows[k]);
        if (st && status == RBTP_OK) status = st;
    }
    h->ring_drained += n;
    if (nrows) *nrows = n;
    return status;
}

int rbtp_batch_stats_get(rbtp_batch *b, rbtp_batch_stats *o)
{
    if (!b || !o) return RBTP_ERR_ARG;
    std::memset(o, 0, sizeof(*o));
    if (b->dirty && !b->members.empty()) {
        int st = rebuild(b);
        if (st) return st;
    }
    o->members = (int)b->members.size();
    o->tiles = b->ntiles[b->shape];
    o->total_particles = b->total_np;
    o->tile_shape = b->shape;
    o->grid = b->grid;
    o->graph = b->graph_valid ? 1 : 0;
    o->tuned = b->tuned ? 1 : 0;
    o->last_step_ms = b->last_ms;
    o->nodes = b->nodes;
    return RBTP_OK;
}

}  // extern "C"

// Called by rbtp_destroy: a destroyed handle leaves its batch first.
void rbtp_batch_detach(rbtp_handle *h)
{
    if (h && h->batch) rbtp_batch_remove(h->batch, h);
}

// A member's buffers are in use by a batch launch in flight.
bool rbtp_batch_busy(const rbtp_handle *h)
{
    return h && h->batch && h->batch->inflight;
}
