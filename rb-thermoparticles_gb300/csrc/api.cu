// api.cu — the C ABI of librbtp (include/rbtp.h): handle lifetime, stepping, state import/export,
// diagnostics and the reference's file formats.
//
// Host-side replacement of main.cu:12-118, src_lbm/initial.cu, src_part/pinit.cu and the
// output/*.cu writers.  All device work of a step is enqueued on the handle's stream without host
// synchronisation; rbtp_step synchronises once at the end to read the device status word
// (non-finite watchdog, list-capacity guards).
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <numeric>
#include <string>
#include <sys/stat.h>
#include <sys/types.h>
#include <vector>

#include "handle.cuh"


using namespace rbtp;
constexpr int NP_COLS = RBTP_PARTICLE_COLS;
constexpr char POS_MAGIC[9] = "RBTPPOS1";   // exact particle sidecar pos_%09d.bin

namespace {

int fail(rbtp_handle *h, int code, const std::string &msg)
{
    if (h) h->err = msg;
    return code;
}

int cuda_fail(rbtp_handle *h, cudaError_t e, const char *where)
{
    std::string m = std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return fail(h, RBTP_ERR_OOM, m);
    return fail(h, RBTP_ERR_CUDA, m);
}

#define CK(call)                                                       \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, #call);         \
    } while (0)

template <class T>
cudaError_t dalloc(T **p, size_t n)
{
    return cudaMalloc(reinterpret_cast<void **>(p), (n ? n : 1) * sizeof(T));
}

// Lattice-node count of the spherical shell r0 < d <= r1 around any centre: every such node's unit
// cube lies inside the shell widened by half a cell diagonal, so the widened volume bounds it.
long long shell_bound(double r0, double r1)
{
    const double h = 0.5 * std::sqrt(3.0);
    const double a = std::max(0.0, r0 - h), b = r1 + h;
    const double pi = 3.14159265358979323846;
    return (long long)std::ceil(4.0 / 3.0 * pi * (b * b * b - a * a * a)) + 1;
}

bool cadence(int istep, int every) { return every > 0 && istep % every == 0; }

int ensure_scratch(rbtp_handle *h)
{
    if (h->fcol) return RBTP_OK;
    const size_t n = (size_t)27 * (size_t)h->geo.L;
    CK(dalloc(&h->fcol, n));
    CK(dalloc(&h->gcol, n));
    return RBTP_OK;
}

int read_status(rbtp_handle *h)
{
    CK(cudaMemcpyAsync(h->status_host, h->status, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    const DevStatus &s = *h->status_host;
    if (s.link_overflow) return fail(h, RBTP_ERR_CAPACITY, "IBB link slab overflow");
    if (s.nf_overflow) return fail(h, RBTP_ERR_CAPACITY, "new-fluid list overflow");
    if (s.contact_overflow) return fail(h, RBTP_ERR_CAPACITY, "contact candidate overflow");
    if (s.nonfinite) return fail(h, RBTP_ERR_NONFINITE, "non-finite density or temperature in the lattice");
    return RBTP_OK;
}

// The F_x auxiliary to and from host FP64 (it is FP32 on the device in the float storage modes,
// where the step computes F_x in FP32, so both directions are exact).  Synchronous.
cudaError_t aux_to_host(const rbtp_handle *h, double *dst)
{
    const size_t L = (size_t)h->geo.L;
    if (h->mode == RBTP_STORE_F64) return cudaMemcpy(dst, h->faux, L * sizeof(double), cudaMemcpyDeviceToHost);
    std::vector<float> tmp(L);
    const cudaError_t e = cudaMemcpy(tmp.data(), h->faux, L * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    for (size_t k = 0; k < L; ++k) dst[k] = (double)tmp[k];
    return cudaSuccess;
}

cudaError_t aux_from_host(rbtp_handle *h, const double *src)
{
    const size_t L = (size_t)h->geo.L;
    if (h->mode == RBTP_STORE_F64) return cudaMemcpy(h->faux, src, L * sizeof(double), cudaMemcpyHostToDevice);
    std::vector<float> tmp(L);
    for (size_t k = 0; k < L; ++k) tmp[k] = (float)src[k];
    return cudaMemcpy(h->faux, tmp.data(), L * sizeof(float), cudaMemcpyHostToDevice);
}

// Build the current solid flags and the IBB link slabs from the current particle positions
// (build_links, links.cu:143-256).
int build_links(rbtp_handle *h, int *owner, bool pgeo_fresh = false)
{
    CK(launch_mark(h->geo, h->ph, h->pb, owner, h->stream, !pgeo_fresh));
    CK(launch_link_fill(h->mode, h->geo, h->ph, h->pb, owner, h->status, h->stream));
    return RBTP_OK;
}

int upload_particles(rbtp_handle *h, const double *rows)
{
    const int np = h->pb.np;
    std::vector<double> col((size_t)np * NP_COLS);
    for (int p = 0; p < np; ++p)
        for (int c = 0; c < NP_COLS; ++c) col[(size_t)c * np + p] = rows[(size_t)p * NP_COLS + c];
    CK(cudaMemcpyAsync(h->pb.state, col.data(), col.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return RBTP_OK;
}

int check_ready(rbtp_handle *h)
{
    if (!h) return RBTP_ERR_ARG;
    if (rbtp_batch_busy(h)) return fail(h, RBTP_ERR_STATE, "the handle's batch has steps in flight (rbtp_batch_wait)");
    if (!h->initialised) return fail(h, RBTP_ERR_STATE, "state not initialised (call rbtp_init_fresh or rbtp_load_state)");
    return RBTP_OK;
}

int plane_sums(rbtp_handle *h)
{
    if (h->plane_valid) return RBTP_OK;
    const bool parts = h->pb.np > 0;
    CK(launch_plane_sums(h->geo, h->ph, h->ux, h->uy, h->uz, h->phi, parts ? h->owner[h->ocur] : nullptr,
                         h->pb.state, h->pb.np, h->partials, h->nchunks, h->plane, h->stream));
    h->plane_host.resize((size_t)NPLANEQ * h->geo.lx);
    CK(cudaMemcpyAsync(h->plane_host.data(), h->plane, h->plane_host.size() * sizeof(double),
                       cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->plane_valid = true;
    return RBTP_OK;
}

// The device address under which the kernels can read `bytes` of a caller's buffer directly:
// the buffer itself for device or managed memory of this device, the device alias of page-locked
// (cudaHostAlloc'd or registered) host memory when the whole range lies in one such allocation;
// nullptr when the buffer has to be copied (ordinary pageable host memory).
const void *device_view(const rbtp_handle *h, const void *p, size_t bytes)
{
    cudaPointerAttributes a{}, b{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if ((a.type == cudaMemoryTypeDevice && a.device == h->device) || a.type == cudaMemoryTypeManaged) return p;
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    const char *last = static_cast<const char *>(p) + bytes - 1;
    if (cudaPointerGetAttributes(&b, last) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (b.type != cudaMemoryTypeHost ||
        static_cast<const char *>(b.devicePointer) - static_cast<const char *>(a.devicePointer) != (ptrdiff_t)(bytes - 1))
        return nullptr;
    return a.devicePointer;
}

// Restart import (initial.cu:194-236, array form) of f, g (27 L doubles each) and the optional
// seven flow fields (7 L doubles): one pass of k_import_nodes writes the storage slots, the flow
// fields (or the moments of f and g) and the buoyancy auxiliary.  Sources the device can read are
// read in place; pageable host buffers are copied in chunks of nodes (one strided 2D copy per
// array and chunk) into two staging slots, alternating so that the import of one chunk overlaps
// the copy of the next.  No full-size FP64 scratch is allocated.
int import_state(rbtp_handle *h, const double *f, const double *g, const double *flow7)
{
    const long long L = h->geo.L;
    const size_t P = 27 * (size_t)L * sizeof(double), F7 = 7 * (size_t)L * sizeof(double);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    void *fs = h->f, *gs = h->g;
    const double *df = static_cast<const double *>(device_view(h, f, P));
    const double *dg = static_cast<const double *>(device_view(h, g, P));
    const double *d7 = flow7 ? static_cast<const double *>(device_view(h, flow7, F7)) : nullptr;
    if (df && dg && (!flow7 || d7)) {
        CK(launch_import_nodes(h->mode, h->geo, h->ph, 0, L, df, dg, L, d7, L, fs, gs, h->faux,
                               h->rho, h->ux, h->uy, h->uz, h->phi, h->ted, h->ked, sms, h->stream));
        return RBTP_OK;
    }
    // staged: chunks of C nodes, slot = f[27][C], g[27][C], flow7[7][C]
    const long long C = std::min<long long>(L, 1LL << 20);
    const size_t slot = (size_t)(27 + 27 + 7) * (size_t)C;
    int maxpitch = 0;
    cudaDeviceGetAttribute(&maxpitch, cudaDevAttrMaxPitch, h->device);
    double *stage = nullptr;
    CK(dalloc(&stage, 2 * slot));
    cudaStream_t cs = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};   // copied[2], imported[2]
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
    // the copy stream starts after the work already queued on the handle's stream
    if (e == cudaSuccess) e = cudaEventRecord(ev[2], h->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev[3], h->stream);
    for (long long n0 = 0, c = 0; n0 < L && e == cudaSuccess; n0 += C, ++c) {
        const int b = (int)(c & 1);
        const long long cnt = std::min<long long>(C, L - n0);
        double *sf = stage + b * slot, *sg = sf + 27 * C, *s7 = sg + 27 * C;
        const size_t w = (size_t)cnt * sizeof(double), spitch = (size_t)L * sizeof(double),
                     dpitch = (size_t)C * sizeof(double);
        // rows of one array: a 2D copy, or one copy per row where the source pitch exceeds the
        // largest pitch a 2D copy takes
        auto rows = [&](double *dst, const double *src, int nrow) {
            if (spitch <= (size_t)maxpitch)
                return cudaMemcpy2DAsync(dst, dpitch, src, spitch, w, nrow, cudaMemcpyDefault, cs);
            cudaError_t r = cudaSuccess;
            for (int k = 0; k < nrow && r == cudaSuccess; ++k)
                r = cudaMemcpyAsync(dst + (size_t)k * C, src + (size_t)k * L, w, cudaMemcpyDefault, cs);
            return r;
        };
        e = cudaStreamWaitEvent(cs, ev[2 + b], 0);          // slot b no longer read by its last import
        if (e == cudaSuccess) e = rows(sf, f + n0, 27);
        if (e == cudaSuccess) e = rows(sg, g + n0, 27);
        if (e == cudaSuccess && flow7) e = rows(s7, flow7 + n0, 7);
        if (e == cudaSuccess) e = cudaEventRecord(ev[b], cs);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, ev[b], 0);
        if (e == cudaSuccess)
            e = launch_import_nodes(h->mode, h->geo, h->ph, n0, cnt, sf, sg, C, flow7 ? s7 : nullptr, C, fs, gs,
                                    h->faux, h->rho, h->ux, h->uy, h->uz, h->phi, h->ted, h->ked, sms, h->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ev[2 + b], h->stream);
    }
    // the staging slots are released only once every import has run
    const cudaError_t es = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess) e = es;
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    if (cs) cudaStreamDestroy(cs);
    cudaFree(stage);
    CK(e);
    return RBTP_OK;
}

}  // namespace

void rbtp_batch_detach(rbtp_handle *h);  // batch.cu

// =================================================================================================
extern "C" {

void rbtp_config_default(rbtp_config *cfg)
{
    if (cfg) rbtp_config_fill_defaults(cfg);
}

const char *rbtp_version(void) { return "rbtp-gb300 0.1 (sm_103a)"; }

const char *rbtp_status_string(int s)
{
    switch (s) {
    case RBTP_OK: return "ok";
    case RBTP_ERR_CUDA: return "CUDA error";
    case RBTP_ERR_CONFIG: return "invalid configuration";
    case RBTP_ERR_OOM: return "out of device memory";
    case RBTP_ERR_NONFINITE: return "non-finite value detected";
    case RBTP_ERR_TIMEOUT: return "device wait timed out";
    case RBTP_ERR_IO: return "file missing, short or malformed";
    case RBTP_ERR_STATE: return "call-order violation";
    case RBTP_ERR_CAPACITY: return "device list capacity exceeded";
    case RBTP_ERR_ARG: return "bad argument";
    case RBTP_ERR_PLACEMENT: return "particles could not be placed";
    case RBTP_ERR_NODEVICE: return "no CUDA device";
    }
    return "unknown status";
}

// globals.cu:18-33, 126-169
int rbtp_derive(const rbtp_config *c, rbtp_derived *d)
{
    if (!c || !d) return RBTP_ERR_ARG;
    std::memset(d, 0, sizeof(*d));
    const double dT = c->t_hot - c->t_cold;
    const double LX = (double)c->lx;
    d->grav0 = (c->beta != 0.0 && dT != 0.0)
                   ? c->rayleigh * c->visc * c->visc / (c->beta * dT * LX * LX * LX * c->prandtl)
                   : 0.0;
    d->tau = 3.0 * c->visc + 0.5;
    d->u0 = std::sqrt(std::fabs(d->grav0 * c->beta * dT * LX));
    d->diff = c->visc / c->prandtl;
    d->tauc = 3.0 * d->diff + 0.5;
    const double pi = 3.14159265358979323846;
    const double radius = 0.5 * c->particle_diam_frac * LX;
    const double volume = 4.0 * pi * radius * radius * radius / 3.0;
    d->particle_radius = radius;
    d->particle_volume = volume;
    d->particle_mass = c->rho0 * c->rho_particle_ratio * volume;
    d->particle_inertia = 0.4 * d->particle_mass * radius * radius;
    d->particle_heat_capacity = d->particle_mass * c->cp_particle_ratio * c->cp_fluid;
    d->npart = 0;
    if (c->activate_particles && c->particle_fraction > 0.0 && volume > 0.0) {
        const double lxyz = (double)((long long)c->lx * c->ly * c->lz);
        const double raw = lxyz * c->particle_fraction / volume;
        d->npart = (int)std::floor(raw < 0.0 ? 0.0 : raw);
    }
    return RBTP_OK;
}

const char *rbtp_last_error(const rbtp_handle *h) { return h ? h->err.c_str() : "null handle"; }

// Device bytes rbtp_create allocates for a config (the same sizes as below; the FP64 export scratch
// that rbtp_get_fg / flow-output steps add on demand is not included).
int rbtp_footprint(const rbtp_config *cfg, size_t *bytes)
{
    if (!cfg || !bytes) return RBTP_ERR_ARG;
    rbtp_derived d;
    rbtp_derive(cfg, &d);
    const size_t L = (size_t)cfg->lx * cfg->ly * cfg->lz;
    const size_t P = 27 * L;
    const size_t sb = store_bytes(cfg->storage);
    size_t b = 2 * P * sb;                                   // f, g in place (AA storage)
    b += 8 * L * sizeof(double);                             // faux, rho, ux, uy, uz, phi, ted, ked
    b += 2 * (size_t)cfg->ly * cfg->lz * sizeof(double);     // rho_wall
    const size_t rows = (size_t)cfg->ly * cfg->lz;
    b += (std::min<size_t>(rows, 512) * NPLANEQ + NPLANEQ) * cfg->lx * sizeof(double);
    const int np = cfg->activate_particles ? d.npart : 0;
    if (np > 0) {
        const double r = d.particle_radius;
        b += (size_t)np * (NP_COLS + 7 * IBB_CHUNKS + 3) * sizeof(double);   // state, IBB partials, cF
        b += (size_t)np * sizeof(PGeo);
        b += 2 * L * sizeof(int);                             // owner maps
        const size_t lcap = (size_t)std::min<long long>(26 * shell_bound(r, r + std::sqrt(3.0)), 1LL << 30);
        b += (size_t)np * lcap * (2 * sizeof(int) + sizeof(double)) + np * sizeof(int);
        const long long nf_bound = (long long)np * shell_bound(r, r + 1.7606816861659007);
        const size_t nfc = (size_t)std::min<long long>(nf_bound, 1LL << 28);
        b += nfc * (2 * sizeof(int) + 59 * sizeof(double));
        const double cs = 2.0 * r + std::max(cfg->rep_min_gap, 0.0) + 1e-9;
        size_t nc = 1;
        for (int a : {cfg->lx, cfg->ly, cfg->lz}) nc *= (size_t)std::max(1, (int)std::floor(a / cs));
        b += 3 * nc * sizeof(int) + np * sizeof(int) + 2 * (size_t)np * 32 * sizeof(int);
    }
    *bytes = b;
    return RBTP_OK;
}

int rbtp_create(const rbtp_config *cfg, rbtp_handle **out)
{
    if (!cfg || !out) return RBTP_ERR_ARG;
    *out = nullptr;
    if (cfg->lx < 3 || cfg->ly < 3 || cfg->lz < 3) return RBTP_ERR_CONFIG;
    const long long L = (long long)cfg->lx * cfg->ly * cfg->lz;
    if (L > (1LL << 31) - 1) return RBTP_ERR_CONFIG;  // node indices are stored as int32
    if (cfg->storage != RBTP_STORE_F64 && cfg->storage != RBTP_STORE_F32 && cfg->storage != RBTP_STORE_F16S)
        return RBTP_ERR_CONFIG;
    if (!(cfg->visc > 0.0) || !(cfg->prandtl > 0.0)) return RBTP_ERR_CONFIG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return RBTP_ERR_NODEVICE;
    }
    rbtp_handle *h = new rbtp_handle();
    h->cfg = *cfg;
    rbtp_derive(cfg, &h->der);
    h->mode = cfg->storage;
    cudaGetDevice(&h->device);
    h->geo.lx = cfg->lx; h->geo.ly = cfg->ly; h->geo.lz = cfg->lz;
    h->geo.lxy = (long long)cfg->lx * cfg->ly;
    h->geo.L = L;
    Phys &ph = h->ph;
    ph.tau = h->der.tau; ph.tauc = h->der.tauc; ph.grav0 = h->der.grav0; ph.beta = cfg->beta;
    ph.thot = cfg->t_hot; ph.tcold = cfg->t_cold; ph.t0 = cfg->t_ref; ph.diff = h->der.diff;
    ph.tlb = -(cfg->t_hot - cfg->t_cold) / (double)cfg->lx;   // conduction profile, node centres
    ph.tla = cfg->t_hot + 0.5 * ph.tlb;
    ph.visc = cfg->visc; ph.rho0 = cfg->rho0;
    ph.radius = h->der.particle_radius; ph.mass = h->der.particle_mass;
    ph.inertia = h->der.particle_inertia; ph.heat_cap = h->der.particle_heat_capacity;
    ph.rho_ratio = cfg->rho_particle_ratio;
    ph.rep_coeff = h->der.particle_mass * cfg->repforce_scale;
    ph.min_gap = cfg->rep_min_gap; ph.min_gap_w = cfg->rep_min_gap_w;
    ph.stf0 = cfg->rep_stf0; ph.stf1 = cfg->rep_stf1; ph.stf0_w = cfg->rep_stf0_w; ph.stf1_w = cfg->rep_stf1_w;
    ph.cp_ratio = cfg->cp_particle_ratio; ph.vol_fraction = cfg->particle_fraction;
    ph.kd = make_step_consts<double>(ph);
    ph.kf = make_step_consts<float>(ph);

    auto cleanup_fail = [&](int code) { rbtp_destroy(h); return code; };
#define CKC(call)                                                                    \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) { int c_ = cuda_fail(h, e_, #call); (void)c_;         \
            return cleanup_fail(e_ == cudaErrorMemoryAllocation ? RBTP_ERR_OOM : RBTP_ERR_CUDA); } \
    } while (0)

    CKC(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    {
        CKC(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
        CKC(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
        CKC(cudaEventCreateWithFlags(&h->ev_side, cudaEventDisableTiming));
    }
    const size_t sb = store_bytes(h->mode);
    const size_t P = (size_t)27 * (size_t)L;
    // one population array, updated in place (AA storage, rbtp_internal.cuh)
    if (h->mode == RBTP_STORE_F64) {
        CKC(cudaMalloc(&h->f, P * sb));
        CKC(cudaMalloc(&h->g, P * sb));
    } else {
        // paired (f_i, g_i) slots: f and g are the same allocation
        CKC(cudaMalloc(&h->f, 2 * P * sb));
        h->g = h->f;
    }
    CKC(dalloc(&h->faux, L));
    CKC(dalloc(&h->rho_wall, 2 * (size_t)cfg->ly * cfg->lz));
    CKC(dalloc(&h->rho, L)); CKC(dalloc(&h->ux, L)); CKC(dalloc(&h->uy, L)); CKC(dalloc(&h->uz, L));
    CKC(dalloc(&h->phi, L)); CKC(dalloc(&h->ted, L)); CKC(dalloc(&h->ked, L));
    CKC(cudaMemsetAsync(h->rho_wall, 0, 2 * (size_t)cfg->ly * cfg->lz * sizeof(double), h->stream));
    CKC(cudaMemsetAsync(h->ted, 0, L * sizeof(double), h->stream));
    CKC(cudaMemsetAsync(h->ked, 0, L * sizeof(double), h->stream));
    CKC(dalloc(&h->status, 1));
    CKC(cudaMemsetAsync(h->status, 0, sizeof(DevStatus), h->stream));
    CKC(cudaMallocHost(reinterpret_cast<void **>(&h->status_host), sizeof(DevStatus)));
    const long long rows = (long long)cfg->ly * cfg->lz;
    h->nchunks = (int)std::min<long long>(rows, 512);
    CKC(dalloc(&h->partials, (size_t)h->nchunks * NPLANEQ * cfg->lx));
    CKC(dalloc(&h->plane, (size_t)NPLANEQ * cfg->lx));

    // particles
    PartBuffers &pb = h->pb;
    pb.np = (cfg->activate_particles ? h->der.npart : 0);
    const int np = pb.np;
    if (np > 0) {
        const double r = h->der.particle_radius;
        CKC(dalloc(&pb.state, (size_t)np * NP_COLS));
        CKC(cudaMemsetAsync(pb.state, 0, (size_t)np * NP_COLS * sizeof(double), h->stream));
        CKC(dalloc(&pb.hpart, (size_t)IBB_CHUNKS * 7 * np)); CKC(dalloc(&pb.cF, 3 * (size_t)np));
        CKC(dalloc(&pb.pgeo, (size_t)np));
        CKC(dalloc(&h->owner[0], L)); CKC(dalloc(&h->owner[1], L));
        CKC(cudaMemsetAsync(h->owner[0], 0xFF, L * sizeof(int), h->stream));
        CKC(cudaMemsetAsync(h->owner[1], 0xFF, L * sizeof(int), h->stream));
        // links of one particle: fluid nodes within r + sqrt(3) of its centre, 26 directions each
        const long long lcap = 26 * shell_bound(r, r + std::sqrt(3.0));
        pb.link_cap = (int)std::min<long long>(lcap, 1LL << 30);
        pb.ibb_chunks = ibb_chunks_for(pb.link_cap);
        const size_t ltot = (size_t)np * pb.link_cap;
        CKC(dalloc(&pb.link_node, ltot)); CKC(dalloc(&pb.link_dir, ltot)); CKC(dalloc(&pb.link_q, ltot));
        CKC(dalloc(&pb.link_cnt, (size_t)np));
        CKC(cudaMemsetAsync(pb.link_cnt, 0, (size_t)np * sizeof(int), h->stream));
        const long long nf_bound = (long long)np * shell_bound(r, r + 1.7606816861659007);
        // a sphere uncovers a few nodes per step; 128 per sphere per step (or the shell bound) is
        // far beyond any stable LBM velocity, and an overflow is reported, not written past
        // the proven bound (every node within 1.76 of a sphere's surface becoming fluid at once):
        // fast spheres (the reference's density ratio 1.5 at LX = 320 reaches several lattice
        // units per step) refill hundreds of nodes per sphere and step
        pb.nf_cap = (int)std::min<long long>(nf_bound, 1LL << 28);
        CKC(dalloc(&pb.nf_node, (size_t)pb.nf_cap)); CKC(dalloc(&pb.nf_pid, (size_t)pb.nf_cap));
        CKC(dalloc(&pb.nf_val, (size_t)pb.nf_cap * 54)); CKC(dalloc(&pb.nf_mac, (size_t)pb.nf_cap * 5));
        // contact cell list: cells no narrower than the interaction range 2r + REP_MIN_GAP
        pb.cell_size = 2.0 * r + std::max(cfg->rep_min_gap, 0.0) + 1e-9;
        const int dims[3] = {cfg->lx, cfg->ly, cfg->lz};
        for (int a = 0; a < 3; ++a) pb.ncell[a] = std::max(1, (int)std::floor(dims[a] / pb.cell_size));
        while ((long long)pb.ncell[0] * pb.ncell[1] * pb.ncell[2] > (1 << 20)) {
            pb.cell_size *= 2.0;
            for (int a = 0; a < 3; ++a) pb.ncell[a] = std::max(1, (int)std::floor(dims[a] / pb.cell_size));
        }
        const int ncells = pb.ncell[0] * pb.ncell[1] * pb.ncell[2];
        CKC(dalloc(&pb.cell_count, (size_t)ncells)); CKC(dalloc(&pb.cell_start, (size_t)ncells));
        CKC(dalloc(&pb.cell_fill, (size_t)ncells)); CKC(dalloc(&pb.cell_items, (size_t)np));
        pb.pair_cap = np * 32;
        CKC(dalloc(&pb.pair_p, (size_t)pb.pair_cap)); CKC(dalloc(&pb.pair_q, (size_t)pb.pair_cap));
    }
#undef CKC
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return cleanup_fail(RBTP_ERR_CUDA);
    *out = h;
    return RBTP_OK;
}

int rbtp_destroy(rbtp_handle *h)
{
    if (!h) return RBTP_OK;
    rbtp_batch_detach(h);
    if (h->side) cudaStreamSynchronize(h->side);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->g != h->f) cudaFree(h->g);
    cudaFree(h->f);
    for (int k = 0; k < 2; ++k) cudaFree(h->owner[k]);
    cudaFree(h->faux); cudaFree(h->rho_wall);
    cudaFree(h->rho); cudaFree(h->ux); cudaFree(h->uy); cudaFree(h->uz); cudaFree(h->phi);
    cudaFree(h->ted); cudaFree(h->ked); cudaFree(h->fcol); cudaFree(h->gcol);
    cudaFree(h->status); if (h->status_host) cudaFreeHost(h->status_host);
    cudaFree(h->partials); cudaFree(h->plane); cudaFree(h->ring);
    PartBuffers &pb = h->pb;
    cudaFree(pb.state); cudaFree(pb.hpart); cudaFree(pb.cF); cudaFree(pb.pgeo);
    cudaFree(pb.link_node); cudaFree(pb.link_dir); cudaFree(pb.link_q); cudaFree(pb.link_cnt);
    cudaFree(pb.nf_node); cudaFree(pb.nf_pid); cudaFree(pb.nf_val); cudaFree(pb.nf_mac);
    cudaFree(pb.cell_count); cudaFree(pb.cell_start); cudaFree(pb.cell_fill); cudaFree(pb.cell_items);
    cudaFree(pb.pair_p); cudaFree(pb.pair_q);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_side) cudaEventDestroy(h->ev_side);
    if (h->side) cudaStreamDestroy(h->side);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return RBTP_OK;
}

int rbtp_npart(const rbtp_handle *h, int *np)
{
    if (!h || !np) return RBTP_ERR_ARG;
    *np = h->pb.np;
    return RBTP_OK;
}

int rbtp_get_stream(rbtp_handle *h, void **stream)
{
    if (!h || !stream) return RBTP_ERR_ARG;
    *stream = (void *)h->stream;
    return RBTP_OK;
}

int rbtp_synchronize(rbtp_handle *h)
{
    if (!h) return RBTP_ERR_ARG;
    CK(cudaStreamSynchronize(h->stream));
    return RBTP_OK;
}

int rbtp_current_step(const rbtp_handle *h, int *istep)
{
    if (!h || !istep) return RBTP_ERR_ARG;
    *istep = h->istep;
    return RBTP_OK;
}

// initial.cu:240-333 (fresh branch), pinit.cu:97-295
int rbtp_init_fresh(rbtp_handle *h)
{
    if (!h) return RBTP_ERR_ARG;
    const int np = h->pb.np;
    if (np > 0) {
        // pinit.cu:97-144: glibc srand/rand rejection sampling with a gap of r/3
        const double r = h->der.particle_radius;
        std::vector<double> rows((size_t)np * NP_COLS, 0.0);
        std::srand((unsigned)h->cfg.particle_rand_seed);
        const double mnx = 1.5 * r, mny = 1.5 * r, mnz = 1.5 * r;
        const double spx = (double)h->cfg.lx - 3.0 * r, spy = (double)h->cfg.ly - 3.0 * r,
                     spz = (double)h->cfg.lz - 3.0 * r;
        long counter = 0;
        for (int p = 0; p < np; ++p) {
            for (;;) {
                const double rx = (double)std::rand() / (double)RAND_MAX;
                const double ry = (double)std::rand() / (double)RAND_MAX;
                const double rz = (double)std::rand() / (double)RAND_MAX;
                const double x = mnx + rx * spx, y = mny + ry * spy, z = mnz + rz * spz;
                bool ok = true;
                for (int q = 0; q < p; ++q) {
                    const double dx = x - rows[(size_t)q * NP_COLS + 0];
                    const double dy = y - rows[(size_t)q * NP_COLS + 1];
                    const double dz = z - rows[(size_t)q * NP_COLS + 2];
                    const double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
                    if (dist - 2.0 * r < r / 3.0) {
                        if (++counter > 1000000) return fail(h, RBTP_ERR_PLACEMENT, "cannot distribute the particles (iteration limit 1000000)");
                        ok = false;
                        break;
                    }
                }
                if (ok) {
                    rows[(size_t)p * NP_COLS + 0] = x;
                    rows[(size_t)p * NP_COLS + 1] = y;
                    rows[(size_t)p * NP_COLS + 2] = z;
                    break;
                }
            }
            rows[(size_t)p * NP_COLS + 30] = h->cfg.particle_init_temp;
        }
        int s = upload_particles(h, rows.data());
        if (s) return s;
    }
    CK(launch_fresh_init(h->mode, h->geo, h->ph, h->f, h->g, h->faux, h->rho, h->ux, h->uy,
                         h->uz, h->phi, h->stream));
    CK(cudaMemsetAsync(h->ted, 0, h->geo.L * sizeof(double), h->stream));
    h->phase = PHASE_HOME;
    h->ocur = 0;
    CK(cudaMemsetAsync(h->status, 0, sizeof(DevStatus), h->stream));
    h->ring_drained = 0;
    if (np > 0) {
        int s = build_links(h, h->owner[0]);  // initial flags == flags of build_links
        if (s) return s;
    }
    h->istep = h->cfg.continuous_steps > 0 ? h->cfg.continuous_steps : 0;
    h->initialised = true;
    h->macros_valid = true;
    h->dissip_valid = false;
    h->plane_valid = false;
    return read_status(h);
}

int rbtp_load_state(rbtp_handle *h, const double *f, const double *g, const double *flow7,
                    const double *particles)
{
    if (!h || !f || !g) return RBTP_ERR_ARG;
    const int np = h->pb.np;
    if (np > 0 && !particles) return fail(h, RBTP_ERR_ARG, "particle state required");
    int s = import_state(h, f, g, flow7);
    if (s) return s;
    h->phase = PHASE_HOME;
    h->ocur = 0;
    CK(cudaMemsetAsync(h->status, 0, sizeof(DevStatus), h->stream));
    h->ring_drained = 0;
    if (np > 0) {
        s = upload_particles(h, particles);
        if (s) return s;
        s = build_links(h, h->owner[0]);
        if (s) return s;
    }
    h->istep = h->cfg.continuous_steps > 0 ? h->cfg.continuous_steps : 0;
    h->initialised = true;
    h->macros_valid = true;
    h->dissip_valid = flow7 != nullptr;
    h->plane_valid = false;
    return read_status(h);
}

int rbtp_step_ex(rbtp_handle *h, int nsteps, unsigned flags)
{
    int s = check_ready(h);
    if (s) return s;
    if (nsteps < 0) return fail(h, RBTP_ERR_ARG, "nsteps < 0");
    if (nsteps == 0) return RBTP_OK;
    const bool parts = h->pb.np > 0;
    const rbtp_config &c = h->cfg;
    for (int k = 1; k <= nsteps; ++k) {
        const int istep = h->istep + 1;
        const bool last = k == nsteps;
        const bool flow = cadence(istep, c.nflowout) || istep == c.nend || (last && (flags & RBTP_STEP_FLOW_LAST));
        const bool macro = flow || cadence(istep, c.ndiag) || cadence(istep, c.nnuout) ||
                           (last && (flags & RBTP_STEP_MACROS_LAST));
        int out = OUT_NONE;
        if (flow) out = OUT_MACROS_COL;
        else if (macro) out = OUT_MACROS;
        else if (parts) out = OUT_RHO;
        if (out == OUT_MACROS_COL) {
            s = ensure_scratch(h);
            if (s) return s;
        }
        // AA storage: the step after a load or an odd step is even, the step after an even one odd
        const bool odd = h->phase == PHASE_SWAPPED;
        StepBuffers b;
        b.f = h->f; b.g = h->g;
        b.faux = h->faux; b.rho_wall = h->rho_wall;
        b.rho = h->rho; b.ux = h->ux; b.uy = h->uy; b.uz = h->uz; b.phi = h->phi;
        b.fcol = h->fcol; b.gcol = h->gcol; b.status = h->status;
        CK(launch_step(h->mode, odd, out, h->geo, h->ph, b, h->stream));
        if (parts) {
            // Stream order: the contacts (positions only) run on the side stream beside IBB (both
            // latency-bound, few CTAs); the integrator waits for the contact forces.  The link
            // slabs stay on the main stream: beside the HBM-bound bulk kernel their CTAs would take
            // its SM slots (measured slower).  The particle kernels use ordinary launches:
            // programmatic dependent launch, which lets each one's blocks become resident while
            // its predecessor finishes, made the 1000-sphere step 0.3 % (FP32) and 0.6 % (FP64)
            // slower.
            int *oc = h->owner[h->ocur], *on = h->owner[1 - h->ocur];
            CK(cudaEventRecord(h->ev_fork, h->stream));
            CK(cudaStreamWaitEvent(h->side, h->ev_fork, 0));
            CK(launch_contacts(h->geo, h->ph, h->pb, h->status, h->side));
            CK(cudaEventRecord(h->ev_side, h->side));
            CK(launch_links_ibb(h->mode, h->geo, h->ph, h->pb, h->f, h->g, h->rho, odd, h->stream));
            CK(cudaStreamWaitEvent(h->stream, h->ev_side, 0));
            CK(launch_update(h->geo, h->ph, h->pb, h->stream));   // also refreshes the geometry cache
            s = build_links(h, on, true);
            if (s) return s;
            CK(launch_refill(h->mode, h->geo, h->ph, h->pb, oc, on, h->f, h->g, h->faux, h->rho_wall, macro,
                             h->rho, h->ux, h->uy, h->uz, h->phi, h->status, odd, h->stream));
            h->ocur = 1 - h->ocur;
        }
        h->phase = odd ? PHASE_HOME : PHASE_SWAPPED;
        h->istep = istep;
        h->plane_valid = false;
        h->macros_valid = macro;
        if (flow) {
            CK(launch_dissipation(h->mode, h->geo, h->ph, h->fcol, h->gcol, h->rho, h->ux, h->uy, h->uz, h->phi,
                                  h->faux, parts ? h->owner[h->ocur] : nullptr, h->ted, h->ked, h->stream));
            h->dissip_valid = true;
        } else {
            h->dissip_valid = false;
        }
    }
    return read_status(h);
}

int rbtp_step(rbtp_handle *h, int nsteps) { return rbtp_step_ex(h, nsteps, 0u); }

int rbtp_get_fg(rbtp_handle *h, double *f, double *g)
{
    int s = check_ready(h);
    if (s) return s;
    s = ensure_scratch(h);
    if (s) return s;
    if (h->phase == PHASE_SWAPPED)
        CK(launch_stream_export(h->mode, h->geo, h->ph, h->f, h->g, h->rho_wall, h->fcol, h->gcol, h->stream));
    else
        CK(launch_home_export(h->mode, h->geo, h->ph, h->f, h->g, h->fcol, h->gcol, h->stream));
    const size_t P = (size_t)27 * (size_t)h->geo.L;
    if (f) CK(cudaMemcpyAsync(f, h->fcol, P * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (g) CK(cudaMemcpyAsync(g, h->gcol, P * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    // the scratch no longer holds a collided copy
    return RBTP_OK;
}

int rbtp_get_macros(rbtp_handle *h, double *rho, double *ux, double *uy, double *uz, double *phi,
                    double *force_x)
{
    int s = check_ready(h);
    if (s) return s;
    if (!h->macros_valid && (rho || ux || uy || uz || phi))
        return fail(h, RBTP_ERR_STATE, "macroscopic fields were not materialised on the last step");
    const size_t n = (size_t)h->geo.L * sizeof(double);
    if (rho) CK(cudaMemcpyAsync(rho, h->rho, n, cudaMemcpyDeviceToHost, h->stream));
    if (ux) CK(cudaMemcpyAsync(ux, h->ux, n, cudaMemcpyDeviceToHost, h->stream));
    if (uy) CK(cudaMemcpyAsync(uy, h->uy, n, cudaMemcpyDeviceToHost, h->stream));
    if (uz) CK(cudaMemcpyAsync(uz, h->uz, n, cudaMemcpyDeviceToHost, h->stream));
    if (phi) CK(cudaMemcpyAsync(phi, h->phi, n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (force_x) CK(aux_to_host(h, force_x));
    return RBTP_OK;
}

int rbtp_get_particles(rbtp_handle *h, double *rows)
{
    if (!h) return RBTP_ERR_ARG;
    const int np = h->pb.np;
    if (np == 0) return RBTP_OK;
    if (!rows) return RBTP_ERR_ARG;
    std::vector<double> col((size_t)np * NP_COLS);
    CK(cudaMemcpyAsync(col.data(), h->pb.state, col.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int p = 0; p < np; ++p)
        for (int c = 0; c < NP_COLS; ++c) rows[(size_t)p * NP_COLS + c] = col[(size_t)c * np + p];
    return RBTP_OK;
}

int rbtp_get_flags(rbtp_handle *h, int *owner, int *owner_prev)
{
    if (!h) return RBTP_ERR_ARG;
    const size_t n = (size_t)h->geo.L;
    if (h->pb.np == 0) {
        if (owner) std::fill(owner, owner + n, -1);
        if (owner_prev) std::fill(owner_prev, owner_prev + n, -1);
        return RBTP_OK;
    }
    // After a step the previous flags equal the current ones (refill.cu:327-328).
    if (owner) CK(cudaMemcpyAsync(owner, h->owner[h->ocur], n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (owner_prev) CK(cudaMemcpyAsync(owner_prev, h->owner[h->ocur], n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return RBTP_OK;
}

int rbtp_get_links(rbtp_handle *h, int *n, int *node, int *dir, int *pid, double *q, int cap)
{
    if (!h || !n) return RBTP_ERR_ARG;
    const int np = h->pb.np;
    *n = 0;
    if (np == 0) return RBTP_OK;
    std::vector<int> cnt(np);
    CK(cudaMemcpyAsync(cnt.data(), h->pb.link_cnt, np * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    long long total = 0;
    for (int p = 0; p < np; ++p) total += std::min(cnt[p], h->pb.link_cap);
    *n = (int)total;
    if (!node && !dir && !pid && !q) return RBTP_OK;
    if (cap < total) return fail(h, RBTP_ERR_ARG, "link buffer too small");
    const size_t slab = (size_t)h->pb.link_cap;
    std::vector<int> hn, hd;
    std::vector<double> hq;
    struct Lk { int node, dir, pid; double q; };
    std::vector<Lk> all;
    all.reserve((size_t)total);
    for (int p = 0; p < np; ++p) {
        const int c = std::min(cnt[p], h->pb.link_cap);
        if (!c) continue;
        hn.resize(c); hd.resize(c); hq.resize(c);
        CK(cudaMemcpy(hn.data(), h->pb.link_node + p * slab, c * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hd.data(), h->pb.link_dir + p * slab, c * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hq.data(), h->pb.link_q + p * slab, c * sizeof(double), cudaMemcpyDeviceToHost));
        for (int k = 0; k < c; ++k) all.push_back({hn[k], hd[k] & LINK_DIR_MASK, p, hq[k]});
    }
    std::sort(all.begin(), all.end(), [](const Lk &a, const Lk &b) {
        return a.node != b.node ? a.node < b.node : a.dir < b.dir;
    });
    for (size_t k = 0; k < all.size(); ++k) {
        if (node) node[k] = all[k].node;
        if (dir) dir[k] = all[k].dir;
        if (pid) pid[k] = all[k].pid;
        if (q) q[k] = all[k].q;
    }
    *n = (int)all.size();
    return RBTP_OK;
}

int rbtp_get_new_fluid(rbtp_handle *h, int *n, int *node, int *pid, int cap)
{
    if (!h || !n) return RBTP_ERR_ARG;
    *n = 0;
    if (h->pb.np == 0) return RBTP_OK;
    CK(cudaMemcpyAsync(h->status_host, h->status, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    const int c = std::min(h->status_host->nf_count, h->pb.nf_cap);
    *n = c;
    if (!node && !pid) return RBTP_OK;
    if (cap < c) return fail(h, RBTP_ERR_ARG, "new-fluid buffer too small");
    std::vector<int> a(c), b(c);
    if (c) {
        CK(cudaMemcpy(a.data(), h->pb.nf_node, c * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(b.data(), h->pb.nf_pid, c * sizeof(int), cudaMemcpyDeviceToHost));
    }
    std::vector<int> ord(c);
    std::iota(ord.begin(), ord.end(), 0);
    std::sort(ord.begin(), ord.end(), [&](int x, int y) { return a[x] < a[y]; });
    for (int k = 0; k < c; ++k) {
        if (node) node[k] = a[ord[k]];
        if (pid) pid[k] = b[ord[k]];
    }
    return RBTP_OK;
}

int rbtp_get_contacts(rbtp_handle *h, int *n, int *p, int *q, int cap)
{
    if (!h || !n) return RBTP_ERR_ARG;
    *n = 0;
    if (h->pb.np == 0) return RBTP_OK;
    CK(cudaMemcpyAsync(h->status_host, h->status, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    const int c = std::min(h->status_host->ncontacts, h->pb.pair_cap);
    *n = c;
    if (!p && !q) return RBTP_OK;
    if (cap < c) return fail(h, RBTP_ERR_ARG, "contact buffer too small");
    std::vector<int> a(c), b(c);
    if (c) {
        CK(cudaMemcpy(a.data(), h->pb.pair_p, c * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(b.data(), h->pb.pair_q, c * sizeof(int), cudaMemcpyDeviceToHost));
    }
    std::vector<int> ord(c);
    std::iota(ord.begin(), ord.end(), 0);
    std::sort(ord.begin(), ord.end(), [&](int x, int y) { return a[x] != a[y] ? a[x] < a[y] : b[x] < b[y]; });
    for (int k = 0; k < c; ++k) {
        if (p) p[k] = a[ord[k]];
        if (q) q[k] = b[ord[k]];
    }
    return RBTP_OK;
}

// output_statis.cu:111-223 applied to the on-device plane sums
int rbtp_nu(rbtp_handle *h, int istep, rbtp_nu_row *row)
{
    int s = check_ready(h);
    if (s) return s;
    if (!row) return RBTP_ERR_ARG;
    if (!h->macros_valid) return fail(h, RBTP_ERR_STATE, "macroscopic fields were not materialised on the last step");
    s = plane_sums(h);
    if (s) return s;
    return nu_from_planes(h, h->plane_host.data(), istep, row);
}

}  // extern "C"

// output_statis.cu:111-223
int rbtp::nu_from_planes(rbtp_handle *h, const double *pl, int istep, rbtp_nu_row *row)
{
    const int lx = h->geo.lx;
    const double vf = h->cfg.particle_fraction;
    const double ff = std::fmax(0.0, 1.0 - vf);
    double avg_f = 0.0, avg_p = 0.0, bottom = 0.0, top = 0.0, bc = 0.0, tc = 0.0;
    for (int ix = 0; ix < lx; ++ix) {
        const double sf = pl[0 * lx + ix], nf = pl[1 * lx + ix], sp = pl[2 * lx + ix], npp = pl[3 * lx + ix];
        if (nf > 0) avg_f += sf / nf;
        if (npp > 0) avg_p += sp / npp;
    }
    bottom = pl[4 * lx + 0]; bc = pl[5 * lx + 0];
    top = pl[4 * lx + lx - 1]; tc = pl[5 * lx + lx - 1];
    avg_f /= (double)lx;
    avg_p /= (double)lx;
    const double thot = h->cfg.t_hot, tcold = h->cfg.t_cold;
    const double cond = h->der.diff * (thot - tcold) / (double)lx;
    double nbf = ff, nbp = 0.0;
    if (cond != 0.0) {
        nbf += ff * (avg_f / cond);
        nbp = vf * h->cfg.cp_particle_ratio * (avg_p / cond);
    }
    const double area = (double)h->geo.ly * (double)h->geo.lz;
    const double scale = (double)lx / (thot - tcold);
    row->step = (double)istep;
    row->volume_fraction = vf;
    row->nu_bulk = nbf + nbp;
    row->nu_top = tc > 0 ? (top / area) * scale : 0.0;
    row->nu_bottom = bc > 0 ? (bottom / area) * scale : 0.0;
    row->nu_bulk_fluid = nbf;
    row->nu_bulk_part = nbp;
    if (!std::isfinite(row->nu_bulk) || !std::isfinite(row->nu_top) || !std::isfinite(row->nu_bottom))
        return fail(h, RBTP_ERR_NONFINITE, "non-finite Nusselt number");
    return RBTP_OK;
}

extern "C" {

// output_statis.cu:64-109
int rbtp_means(rbtp_handle *h, double means[4])
{
    int s = check_ready(h);
    if (s) return s;
    if (!means) return RBTP_ERR_ARG;
    if (!h->macros_valid) return fail(h, RBTP_ERR_STATE, "macroscopic fields were not materialised on the last step");
    s = plane_sums(h);
    if (s) return s;
    const int lx = h->geo.lx;
    const double *pl = h->plane_host.data();
    for (int k = 0; k < 4; ++k) {
        double a = 0.0;
        for (int ix = 0; ix < lx; ++ix) a += pl[(6 + k) * lx + ix];
        means[k] = a / (double)h->geo.L;
    }
    for (int k = 0; k < 4; ++k)
        if (!std::isfinite(means[k])) return fail(h, RBTP_ERR_NONFINITE, "non-finite mean field");
    return RBTP_OK;
}

// output_statis.cu:225-285
int rbtp_profile(rbtp_handle *h, double *out)
{
    int s = check_ready(h);
    if (s) return s;
    if (!out) return RBTP_ERR_ARG;
    if (!h->macros_valid) return fail(h, RBTP_ERR_STATE, "macroscopic fields were not materialised on the last step");
    s = plane_sums(h);
    if (s) return s;
    const int lx = h->geo.lx;
    const double *pl = h->plane_host.data();
    const double cnt = (double)h->geo.ly * (double)h->geo.lz;
    const double inv = cnt > 0 ? 1.0 / cnt : 0.0;
    for (int ix = 0; ix < lx; ++ix)
        for (int k = 0; k < 4; ++k) out[4 * ix + k] = pl[(6 + k) * lx + ix] * inv;
    return RBTP_OK;
}

int rbtp_dissipation(rbtp_handle *h, double *ted, double *ked)
{
    int s = check_ready(h);
    if (s) return s;
    if (!h->dissip_valid) return fail(h, RBTP_ERR_STATE, "dissipation fields are computed on flow-output steps only");
    const size_t n = (size_t)h->geo.L * sizeof(double);
    if (ted) CK(cudaMemcpyAsync(ted, h->ted, n, cudaMemcpyDeviceToHost, h->stream));
    if (ked) CK(cudaMemcpyAsync(ked, h->ked, n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return RBTP_OK;
}

}  // extern "C"

// =================================================================================================
// Reference file formats (output/output_*.cu, src_lbm/initial.cu:7-192)
// =================================================================================================
namespace {

int ensure_dir(const std::string &d)
{
    struct stat st;
    if (stat(d.c_str(), &st) == -1) {
        if (mkdir(d.c_str(), 0700) != 0 && errno != EEXIST) return RBTP_ERR_IO;
    }
    return RBTP_OK;
}

std::string out_dir(const rbtp_handle *h, const char *dir)
{
    if (dir && dir[0]) return dir;
    char buf[256];
    std::snprintf(buf, sizeof(buf), "Ra%.1ePr%.2f", h->cfg.rayleigh, h->cfg.prandtl);
    return buf;
}

// overwrite_particle_nodes (output_statis.cu:5-60) on host copies
void overwrite_solid(const rbtp_handle *h, const std::vector<int> &owner, const std::vector<double> &prow,
                     double *rho, double *ux, double *uy, double *uz, double *phi, double *ted, double *ked)
{
    const int np = h->pb.np;
    if (np == 0) return;
    const long long lxy = h->geo.lxy;
    for (long long idx = 0; idx < h->geo.L; ++idx) {
        const int pid = owner[idx];
        if (pid < 0 || pid >= np) continue;
        const int iz = (int)(idx / lxy);
        const int iy = (int)((idx - iz * lxy) / h->geo.lx);
        const int ix = (int)(idx - iz * lxy - (long long)iy * h->geo.lx);
        const double *c = &prow[(size_t)pid * NP_COLS];
        const double relx = ((double)ix + 0.5) - c[0], rely = ((double)iy + 0.5) - c[1], relz = ((double)iz + 0.5) - c[2];
        if (rho) rho[idx] = h->cfg.rho0;
        if (ux) ux[idx] = c[3] + (relz * c[19] - rely * c[20]);
        if (uy) uy[idx] = c[4] + (relx * c[20] - relz * c[18]);
        if (uz) uz[idx] = c[5] + (rely * c[18] - relx * c[19]);
        if (phi) phi[idx] = c[30];
        if (ted) ted[idx] = 0.0;
        if (ked) ked[idx] = 0.0;
    }
}

}  // namespace

extern "C" {

int rbtp_output_dirname(const rbtp_handle *h, char *buf, size_t len)
{
    if (!h || !buf || len < 2) return RBTP_ERR_ARG;
    std::snprintf(buf, len, "Ra%.1ePr%.2f", h->cfg.rayleigh, h->cfg.prandtl);
    return RBTP_OK;
}

int rbtp_write_statistics(rbtp_handle *h, const char *dir, int istep)
{
    double m[4];
    int s = rbtp_means(h, m);
    if (s) return s;
    const std::string d = out_dir(h, dir);
    if (ensure_dir(d)) return fail(h, RBTP_ERR_IO, "cannot create " + d);
    std::printf("Step %-7d umean = %14.6e, vmean = %14.6e, wmean = %14.6e, tmean = %14.6e\n", istep, m[0], m[1], m[2], m[3]);
    std::fflush(stdout);
    FILE *fp = std::fopen((d + "/statistics.dat").c_str(), "a");
    if (!fp) return fail(h, RBTP_ERR_IO, "cannot open statistics.dat");
    std::fprintf(fp, "%-7d %14.6e %14.6e %14.6e %14.6e\n", istep, m[0], m[1], m[2], m[3]);
    std::fclose(fp);
    return RBTP_OK;
}

int rbtp_write_nu(rbtp_handle *h, const char *dir, int istep)
{
    rbtp_nu_row r;
    int s = rbtp_nu(h, istep, &r);
    if (s) return s;
    const std::string d = out_dir(h, dir);
    if (ensure_dir(d)) return fail(h, RBTP_ERR_IO, "cannot create " + d);
    char name[512];
    std::snprintf(name, sizeof(name), "%s/Nu_%.2e.txt", d.c_str(), h->cfg.rayleigh);
    FILE *fp = std::fopen(name, "a");
    if (!fp) return fail(h, RBTP_ERR_IO, std::string("cannot open ") + name);
    std::fprintf(fp, "%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E\n", r.step, r.volume_fraction, r.nu_bulk,
                 r.nu_top, r.nu_bottom, r.nu_bulk_fluid, r.nu_bulk_part);
    std::fclose(fp);
    return RBTP_OK;
}

int rbtp_write_profile(rbtp_handle *h, const char *dir, int istep)
{
    std::vector<double> prof((size_t)4 * h->geo.lx);
    int s = rbtp_profile(h, prof.data());
    if (s) return s;
    const std::string d = out_dir(h, dir);
    if (ensure_dir(d)) return fail(h, RBTP_ERR_IO, "cannot create " + d);
    char name[512];
    std::snprintf(name, sizeof(name), "%s/Profile_%.2e.txt", d.c_str(), h->cfg.rayleigh);
    FILE *fp = std::fopen(name, "a");
    if (!fp) return fail(h, RBTP_ERR_IO, std::string("cannot open ") + name);
    std::fprintf(fp, "%d\n", istep);
    for (int ix = 0; ix < h->geo.lx; ++ix)
        std::fprintf(fp, "%14.6e %14.6e %14.6e %14.6e\n", prof[4 * ix], prof[4 * ix + 1], prof[4 * ix + 2], prof[4 * ix + 3]);
    std::fclose(fp);
    return RBTP_OK;
}

int rbtp_write_flow(rbtp_handle *h, const char *dir, int istep)
{
    int s = check_ready(h);
    if (s) return s;
    const size_t L = (size_t)h->geo.L;
    std::vector<double> f7(7 * L);
    s = rbtp_get_macros(h, &f7[0], &f7[L], &f7[2 * L], &f7[3 * L], &f7[4 * L], nullptr);
    if (s) return s;
    s = rbtp_dissipation(h, &f7[5 * L], &f7[6 * L]);
    if (s) return s;
    if (h->pb.np > 0) {
        std::vector<int> owner(L);
        std::vector<double> prow((size_t)h->pb.np * NP_COLS);
        if ((s = rbtp_get_flags(h, owner.data(), nullptr))) return s;
        if ((s = rbtp_get_particles(h, prow.data()))) return s;
        overwrite_solid(h, owner, prow, &f7[0], &f7[L], &f7[2 * L], &f7[3 * L], &f7[4 * L], &f7[5 * L], &f7[6 * L]);
    }
    const std::string d = out_dir(h, dir);
    if (ensure_dir(d)) return fail(h, RBTP_ERR_IO, "cannot create " + d);
    char name[512];
    std::snprintf(name, sizeof(name), "%s/%09d.dat", d.c_str(), istep);
    FILE *fp = std::fopen(name, "wb");
    if (!fp) return fail(h, RBTP_ERR_IO, std::string("cannot open ") + name);
    const size_t w = std::fwrite(f7.data(), sizeof(double), f7.size(), fp);
    std::fclose(fp);
    return w == f7.size() ? RBTP_OK : fail(h, RBTP_ERR_IO, "short write");
}

int rbtp_write_fg(rbtp_handle *h, const char *dir, int istep)
{
    int s = check_ready(h);
    if (s) return s;
    const size_t P = (size_t)27 * h->geo.L;
    std::vector<double> fg(2 * P);
    if ((s = rbtp_get_fg(h, &fg[0], &fg[P]))) return s;
    const std::string d = out_dir(h, dir);
    if (ensure_dir(d)) return fail(h, RBTP_ERR_IO, "cannot create " + d);
    char name[512];
    std::snprintf(name, sizeof(name), "%s/fg%09d.dat", d.c_str(), istep);
    FILE *fp = std::fopen(name, "wb");
    if (!fp) return fail(h, RBTP_ERR_IO, std::string("cannot open ") + name);
    const size_t w = std::fwrite(fg.data(), sizeof(double), fg.size(), fp);
    std::fclose(fp);
    return w == fg.size() ? RBTP_OK : fail(h, RBTP_ERR_IO, "short write");
}

int rbtp_write_particles(rbtp_handle *h, const char *dir, int istep)
{
    if (!h) return RBTP_ERR_ARG;
    const int np = h->pb.np;
    if (np == 0) return RBTP_OK;
    std::vector<double> prow((size_t)np * NP_COLS);
    int s = rbtp_get_particles(h, prow.data());
    if (s) return s;
    const std::string d = out_dir(h, dir);
    if (ensure_dir(d) || ensure_dir(d + "/pos")) return fail(h, RBTP_ERR_IO, "cannot create " + d + "/pos");
    char name[1024];
    std::snprintf(name, sizeof(name), "%s/pos/pos_%09d.txt", d.c_str(), istep);
    FILE *fp = std::fopen(name, "w");
    if (!fp) return fail(h, RBTP_ERR_IO, std::string("cannot open ") + name);
    for (int p = 0; p < np; ++p) {
        std::fprintf(fp, "%d ", p);
        const double *c = &prow[(size_t)p * NP_COLS];
        for (int k = 0; k < NP_COLS; ++k) std::fprintf(fp, k + 1 < NP_COLS ? "%14.6e " : "%14.6e\n", c[k]);
    }
    std::fclose(fp);
    // Exact sidecar (no counterpart in the reference, whose %14.6e text keeps 7 digits): the same
    // rows as raw doubles, preferred by rbtp_load_restart so that a restart continues bit for bit.
    std::snprintf(name, sizeof(name), "%s/pos/pos_%09d.bin", d.c_str(), istep);
    fp = std::fopen(name, "wb");
    if (!fp) return fail(h, RBTP_ERR_IO, std::string("cannot open ") + name);
    const int hdr[2] = {np, NP_COLS};
    const bool ok = std::fwrite(POS_MAGIC, 1, 8, fp) == 8 && std::fwrite(hdr, sizeof(int), 2, fp) == 2 &&
                    std::fwrite(prow.data(), sizeof(double), prow.size(), fp) == prow.size();
    std::fclose(fp);
    return ok ? RBTP_OK : fail(h, RBTP_ERR_IO, std::string("short write: ") + name);
}

// load_restart_state (initial.cu:194-236) from the reference's files
int rbtp_load_restart(rbtp_handle *h, const char *dir, int step)
{
    if (!h) return RBTP_ERR_ARG;
    const std::string d = out_dir(h, dir);
    const size_t L = (size_t)h->geo.L, P = 27 * L;
    char name[1024];
    std::snprintf(name, sizeof(name), "%s/fg%09d.dat", d.c_str(), step);
    FILE *fp = std::fopen(name, "rb");
    if (!fp) return fail(h, RBTP_ERR_IO, std::string("cannot open restart distribution file ") + name);
    std::vector<double> fg(2 * P);
    const size_t rf = std::fread(fg.data(), sizeof(double), 2 * P, fp);
    std::fclose(fp);
    if (rf != 2 * P) return fail(h, RBTP_ERR_IO, std::string("restart distribution file is corrupted: ") + name);
    std::snprintf(name, sizeof(name), "%s/%09d.dat", d.c_str(), step);
    fp = std::fopen(name, "rb");
    if (!fp) return fail(h, RBTP_ERR_IO, std::string("cannot open flow restart file ") + name);
    std::vector<double> f7(7 * L);
    const size_t r7 = std::fread(f7.data(), sizeof(double), 7 * L, fp);
    std::fclose(fp);
    if (r7 != 7 * L) return fail(h, RBTP_ERR_IO, std::string("flow restart file is short: ") + name);
    std::vector<double> prow;
    const int np = h->pb.np;
    bool exact = false;
    if (np > 0) {
        std::snprintf(name, sizeof(name), "%s/pos/pos_%09d.bin", d.c_str(), step);
        if (FILE *bf = std::fopen(name, "rb")) {
            char magic[8];
            int hdr[2] = {0, 0};
            prow.assign((size_t)np * NP_COLS, 0.0);
            exact = std::fread(magic, 1, 8, bf) == 8 && std::memcmp(magic, POS_MAGIC, 8) == 0 &&
                    std::fread(hdr, sizeof(int), 2, bf) == 2 && hdr[0] == np && hdr[1] == NP_COLS &&
                    std::fread(prow.data(), sizeof(double), prow.size(), bf) == prow.size();
            std::fclose(bf);
            if (!exact) return fail(h, RBTP_ERR_IO, std::string("particle sidecar is corrupted or for another case: ") + name);
        }
    }
    if (np > 0 && !exact) {
        std::snprintf(name, sizeof(name), "%s/pos/pos_%09d.txt", d.c_str(), step);
        std::ifstream in(name);
        if (!in) return fail(h, RBTP_ERR_IO, std::string("cannot open restart particle file ") + name);
        prow.assign((size_t)np * NP_COLS, 0.0);
        for (int line = 0; line < np; ++line) {
            int pid = -1;
            double v[NP_COLS];
            if (!(in >> pid)) return fail(h, RBTP_ERR_IO, std::string("failed to read particle restart data from ") + name);
            for (int k = 0; k < NP_COLS; ++k)
                if (!(in >> v[k])) return fail(h, RBTP_ERR_IO, std::string("failed to read particle restart data from ") + name);
            if (pid < 0 || pid >= np) return fail(h, RBTP_ERR_IO, "particle id out of range in restart file");
            std::memcpy(&prow[(size_t)pid * NP_COLS], v, sizeof(v));
        }
    }
    const int saved = h->cfg.continuous_steps;
    h->cfg.continuous_steps = step;
    int s = rbtp_load_state(h, &fg[0], &fg[P], f7.data(), np > 0 ? prow.data() : nullptr);
    h->cfg.continuous_steps = saved;
    if (s == RBTP_OK) h->istep = step;
    return s;
}

// Exact checkpoint of a handle's whole step state in its storage precision: the population array as
// it sits (post-streaming in the natural slots, or post-collision swapped with the IBB/refill
// fix-ups, with the phase that says which), the F_x auxiliary, the wall densities of the Dirichlet image, the macroscopic fields when
// they are current, and the 33 particle columns.  Solid flags and link slabs are rebuilt from the
// positions on load (deterministically, as at the end of every step), so a run resumed from a
// checkpoint continues bit for bit.  No counterpart in the reference.
namespace {
constexpr char CKP_MAGIC[9] = "RBTPCKP1";
constexpr int CKP_VERSION = 2;   // 2: in-place AA population array
struct CkpHeader {
    int version, mode, lx, ly, lz, np, phase, istep, macros_valid, pad;
};
size_t elem_bytes(int mode) { return mode == RBTP_STORE_F64 ? 8 : (mode == RBTP_STORE_F32 ? 4 : 2); }
}  // namespace

int rbtp_checkpoint_write(rbtp_handle *h, const char *path)
{
    int s = check_ready(h);
    if (s) return s;
    if (!path) return fail(h, RBTP_ERR_ARG, "path is null");
    const size_t L = (size_t)h->geo.L, P = 27 * L * elem_bytes(h->mode), W = 2 * (size_t)h->geo.ly * h->geo.lz;
    const int np = h->pb.np;
    CkpHeader hd{CKP_VERSION, h->mode, h->geo.lx, h->geo.ly, h->geo.lz, np, h->phase, h->istep,
                 h->macros_valid ? 1 : 0, 0};
    std::vector<char> pop(P);
    std::vector<double> aux(L), wall(W), mac(h->macros_valid ? 5 * L : 0), prow((size_t)np * NP_COLS);
    CK(cudaStreamSynchronize(h->stream));
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return fail(h, RBTP_ERR_IO, std::string("cannot open ") + path);
    bool ok = std::fwrite(CKP_MAGIC, 1, 8, fp) == 8 && std::fwrite(&hd, sizeof(hd), 1, fp) == 1 &&
              std::fwrite(&h->cfg, sizeof(rbtp_config), 1, fp) == 1;
    // 2P bytes of populations: f then g (FP64), or the paired (f_i, g_i) slots (float modes)
    const bool paired = h->g == h->f;
    for (int k = 0; ok && k < 2; ++k) {
        const char *src = paired ? static_cast<const char *>(h->f) + k * P
                                 : static_cast<const char *>(k == 0 ? h->f : h->g);
        if (cudaMemcpy(pop.data(), src, P, cudaMemcpyDeviceToHost) != cudaSuccess) {
            std::fclose(fp);
            return fail(h, RBTP_ERR_CUDA, "checkpoint read-back failed");
        }
        ok = std::fwrite(pop.data(), 1, P, fp) == P;
    }
    if (aux_to_host(h, aux.data()) != cudaSuccess ||
        cudaMemcpy(wall.data(), h->rho_wall, W * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
        std::fclose(fp);
        return fail(h, RBTP_ERR_CUDA, "checkpoint read-back failed");
    }
    if (h->macros_valid) {
        const double *srcs[5] = {h->rho, h->ux, h->uy, h->uz, h->phi};
        for (int k = 0; k < 5; ++k)
            if (cudaMemcpy(&mac[k * L], srcs[k], L * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
                std::fclose(fp);
                return fail(h, RBTP_ERR_CUDA, "checkpoint read-back failed");
            }
    }
    if (np > 0 && (s = rbtp_get_particles(h, prow.data()))) {
        std::fclose(fp);
        return s;
    }
    ok = ok && std::fwrite(aux.data(), sizeof(double), L, fp) == L &&
         std::fwrite(wall.data(), sizeof(double), W, fp) == W &&
         std::fwrite(mac.data(), sizeof(double), mac.size(), fp) == mac.size() &&
         std::fwrite(prow.data(), sizeof(double), prow.size(), fp) == prow.size();
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? RBTP_OK : fail(h, RBTP_ERR_IO, std::string("short write: ") + path);
}

int rbtp_checkpoint_read(rbtp_handle *h, const char *path)
{
    if (!h || !path) return RBTP_ERR_ARG;
    if (rbtp_batch_busy(h)) return fail(h, RBTP_ERR_STATE, "the handle's batch has steps in flight (rbtp_batch_wait)");
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return fail(h, RBTP_ERR_IO, std::string("cannot open checkpoint ") + path);
    char magic[8];
    CkpHeader hd{};
    rbtp_config saved;
    const bool head = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, CKP_MAGIC, 8) == 0 &&
                      std::fread(&hd, sizeof(hd), 1, fp) == 1 && std::fread(&saved, sizeof(saved), 1, fp) == 1;
    if (!head) {
        std::fclose(fp);
        return fail(h, RBTP_ERR_IO, std::string("not a checkpoint file: ") + path);
    }
    if (hd.version != CKP_VERSION) {
        std::fclose(fp);
        return fail(h, RBTP_ERR_IO, std::string("checkpoint format version ") + std::to_string(hd.version) +
                                        " (this library reads version " + std::to_string(CKP_VERSION) + "): " + path);
    }
    if (hd.mode != h->mode || hd.lx != h->geo.lx || hd.ly != h->geo.ly || hd.lz != h->geo.lz || hd.np != h->pb.np) {
        std::fclose(fp);
        return fail(h, RBTP_ERR_CONFIG, "checkpoint was written for another grid, storage mode or particle count");
    }
    const size_t L = (size_t)h->geo.L, P = 27 * L * elem_bytes(h->mode), W = 2 * (size_t)h->geo.ly * h->geo.lz;
    const int np = h->pb.np;
    std::vector<char> f(P), g(P);
    std::vector<double> aux(L), wall(W), mac(hd.macros_valid ? 5 * L : 0), prow((size_t)np * NP_COLS);
    const bool body = std::fread(f.data(), 1, P, fp) == P && std::fread(g.data(), 1, P, fp) == P &&
                      std::fread(aux.data(), sizeof(double), L, fp) == L &&
                      std::fread(wall.data(), sizeof(double), W, fp) == W &&
                      std::fread(mac.data(), sizeof(double), mac.size(), fp) == mac.size() &&
                      std::fread(prow.data(), sizeof(double), prow.size(), fp) == prow.size();
    std::fclose(fp);
    if (!body) return fail(h, RBTP_ERR_IO, std::string("checkpoint is truncated: ") + path);
    if (h->g == h->f) {   // paired (f_i, g_i) slots: the 2P bytes in file order
        CK(cudaMemcpyAsync(h->f, f.data(), P, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(static_cast<char *>(h->f) + P, g.data(), P, cudaMemcpyHostToDevice, h->stream));
    } else {
        CK(cudaMemcpyAsync(h->f, f.data(), P, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->g, g.data(), P, cudaMemcpyHostToDevice, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    CK(aux_from_host(h, aux.data()));
    CK(cudaMemcpyAsync(h->rho_wall, wall.data(), W * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (hd.macros_valid) {
        double *dst[5] = {h->rho, h->ux, h->uy, h->uz, h->phi};
        for (int k = 0; k < 5; ++k)
            CK(cudaMemcpyAsync(dst[k], &mac[k * L], L * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    }
    h->phase = hd.phase == PHASE_SWAPPED ? PHASE_SWAPPED : PHASE_HOME;
    h->ocur = 0;
    CK(cudaMemsetAsync(h->status, 0, sizeof(DevStatus), h->stream));
    h->ring_drained = 0;
    if (np > 0) {
        int s = upload_particles(h, prow.data());
        if (s) return s;
        s = build_links(h, h->owner[0]);
        if (s) return s;
    }
    CK(cudaStreamSynchronize(h->stream));   // host staging buffers go out of scope
    h->istep = hd.istep;
    h->initialised = true;
    h->macros_valid = hd.macros_valid != 0;
    h->dissip_valid = false;
    h->plane_valid = false;
    return read_status(h);
}

}  // extern "C"
