// rbtp_internal.cuh — shared device/host definitions of librbtp (GB300, sm_103a).
//
// Lattice: D3Q27 in the reference's direction order (src_lbm/initial.cu:276-286) so that every
// exported array has the reference layout.  The tables are compile-time constants: kernels unroll
// over directions with std::integer_sequence so each direction's velocity, weight and opposite fold
// into the instruction stream instead of being read from constant memory.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <string>
#include <utility>
#include <vector>

#include "../../include/rbtp.h"

namespace rbtp {

// Programmatic dependent launch (batched step sequence).  A kernel launched by pdl_launch may be
// scheduled while its stream predecessor is still running; it calls pdl_wait() before anything
// else (which returns once the predecessor has completed and its writes are visible) and then
// pdl_trigger() so that its own successor can be scheduled early.  Every such kernel waits first
// and unconditionally, so completion of a kernel implies completion of all earlier ones.
#ifndef RBTP_USE_PDL
#define RBTP_USE_PDL 1
#endif
__device__ __forceinline__ void pdl_wait()
{
#if RBTP_USE_PDL
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}
__device__ __forceinline__ void pdl_trigger()
{
#if RBTP_USE_PDL
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}
template <typename... KArgs, typename... Args>
cudaError_t pdl_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = RBTP_USE_PDL;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// ------------------------------------------------------------------------------------------------
// D3Q27 tables (initial.cu:276-286)
// ------------------------------------------------------------------------------------------------
__host__ __device__ constexpr int dcx(int i)
{
    constexpr int t[27] = {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1, 0, 1, 0, -1, 0, 1, -1, -1, 1, 1, -1, -1, 1};
    return t[i];
}
__host__ __device__ constexpr int dcy(int i)
{
    constexpr int t[27] = {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0, -1, 0, 1, 0, -1, 1, 1, -1, -1, 1, 1, -1, -1};
    return t[i];
}
__host__ __device__ constexpr int dcz(int i)
{
    constexpr int t[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
    return t[i];
}
__host__ __device__ constexpr int dopp(int i)
{
    constexpr int t[27] = {0, 3, 4, 1, 2, 6, 5, 9, 10, 7, 8, 17, 18, 15, 16, 13, 14, 11, 12, 25, 26, 23, 24, 21, 22, 19, 20};
    return t[i];
}
// weight class: 0 rest, 1 face (2/27), 2 edge (1/54), 3 corner (1/216)
__host__ __device__ constexpr int dclass(int i) { return i == 0 ? 0 : (i <= 6 ? 1 : (i <= 18 ? 2 : 3)); }
__host__ __device__ constexpr double dweight(int i)
{
    return i == 0 ? 8.0 / 27.0 : (i <= 6 ? 2.0 / 27.0 : (i <= 18 ? 1.0 / 54.0 : 1.0 / 216.0));
}
// the 13 direction pairs (i, opp(i)) with i < opp(i)
__host__ __device__ constexpr int dpair(int k)
{
    constexpr int t[13] = {1, 2, 5, 7, 8, 11, 12, 13, 14, 19, 20, 21, 22};
    return t[k];
}

// Runtime-indexed copies of the tables for loops that are not unrolled (sparse particle work).
static __constant__ int c_cx[27] = {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1, 0, 1, 0, -1, 0, 1, -1, -1, 1, 1, -1, -1, 1};
static __constant__ int c_cy[27] = {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0, -1, 0, 1, 0, -1, 1, 1, -1, -1, 1, 1, -1, -1};
static __constant__ int c_cz[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
static __constant__ int c_opp[27] = {0, 3, 4, 1, 2, 6, 5, 9, 10, 7, 8, 17, 18, 15, 16, 13, 14, 11, 12, 25, 26, 23, 24, 21, 22, 19, 20};
__device__ __forceinline__ int dcx_rt(int i) { return c_cx[i]; }
__device__ __forceinline__ int dcy_rt(int i) { return c_cy[i]; }
__device__ __forceinline__ int dcz_rt(int i) { return c_cz[i]; }
__device__ __forceinline__ int dopp_rt(int i) { return c_opp[i]; }
__device__ __forceinline__ double dweight_rt(int i)
{
    return i == 0 ? 8.0 / 27.0 : (i <= 6 ? 2.0 / 27.0 : (i <= 18 ? 1.0 / 54.0 : 1.0 / 216.0));
}
// the same weights and their inverses rounded to float (the float storage modes' factors)
__device__ __forceinline__ float fweight_rt(int i)
{
    return i == 0 ? (float)(8.0 / 27.0) : (i <= 6 ? (float)(2.0 / 27.0) : (i <= 18 ? (float)(1.0 / 54.0) : (float)(1.0 / 216.0)));
}
__device__ __forceinline__ float finvweight_rt(int i)
{
    return i == 0 ? (float)(27.0 / 8.0) : (i <= 6 ? (float)(27.0 / 2.0) : (i <= 18 ? 54.0f : 216.0f));
}

template <class F, int... Is>
__host__ __device__ __forceinline__ void unroll_impl(F &&f, std::integer_sequence<int, Is...>)
{
    (f(std::integral_constant<int, Is>()), ...);
}
template <int N, class F>
__host__ __device__ __forceinline__ void unroll(F &&f)
{
    unroll_impl(f, std::make_integer_sequence<int, N>());
}

// ------------------------------------------------------------------------------------------------
// Population storage modes.  R is the arithmetic type of the collision, S the storage type.
// FP16 mode stores (pop / w_i) for f (the deviation-form f needs no shift) and (g / w_i - T0) for g.
// ------------------------------------------------------------------------------------------------
// Population storage.  FP64 keeps f and g in two arrays of 27 L doubles ([ip][z][y][x], the
// reference layout).  The FP32 and shifted-FP16 modes pair the two distributions per slot: one
// array of 27 L (f_i, g_i) pairs (float2 / __half2, [ip][z][y][x]), so that a gather or a store
// of both populations of a direction is one 8- or 4-byte access; the f and g buffer pointers of
// such a handle are the same allocation, and ld_f/ld_g/st_f/st_g address the halves of a slot.
template <int MODE> struct Store;
// A: type of the per-node F_x auxiliary (the step stores the F_x it computed in its working
// precision R, so the stored value is exact in every mode).
template <> struct Store<RBTP_STORE_F64> {
    using S = double;
    using R = double;
    using A = double;
    static constexpr bool PAIRED = false;
    static __device__ __forceinline__ R ld_f(const S *p, double, double) { return *p; }
    static __device__ __forceinline__ R ld_g(const S *p, double, double) { return *p; }
    static __device__ __forceinline__ void st_f(S *p, R v, double, double) { *p = v; }
    static __device__ __forceinline__ void st_g(S *p, R v, double, double) { *p = v; }
};
template <> struct Store<RBTP_STORE_F32> {
    using S = float2;   // (f_i, g_i)
    using R = float;
    using A = float;
    static constexpr bool PAIRED = true;
    static __device__ __forceinline__ R ld_f(const S *p, double, double) { return p->x; }
    static __device__ __forceinline__ R ld_g(const S *p, double, double) { return p->y; }
    static __device__ __forceinline__ void st_f(S *p, R v, double, double) { p->x = v; }
    static __device__ __forceinline__ void st_g(S *p, R v, double, double) { p->y = v; }
};
// Shifted FP16: f_i / w_i (f is already the deviation from rest) and g_i / w_i - T_c(x), T_c the
// conduction profile (the thermal rest state) at the x of the slot's home node, so that FP16 holds
// only the departure from conduction.  `shift` below is T_c(x_home) (gshift), ignored elsewhere.
template <> struct Store<RBTP_STORE_F16S> {
    using S = __half2;  // (f_i / w_i, g_i / w_i - T_c(x))
    using R = float;
    using A = float;
    static constexpr bool PAIRED = true;
    // w: lattice weight of the slot's direction
    static __device__ __forceinline__ R ld_f(const S *p, double w, double) { return __low2float(*p) * (float)w; }
    static __device__ __forceinline__ R ld_g(const S *p, double w, double shift)
    {
        return (__high2float(*p) + (float)shift) * (float)w;
    }
    static __device__ __forceinline__ void st_f(S *p, R v, double w, double)
    {
        reinterpret_cast<__half *>(p)[0] = __float2half_rn(v * (float)(1.0 / w));
    }
    static __device__ __forceinline__ void st_g(S *p, R v, double w, double shift)
    {
        reinterpret_cast<__half *>(p)[1] = __float2half_rn(v * (float)(1.0 / w) - (float)shift);
    }
};

// Dirichlet anti-bounce-back image of streaming.cu:55-60, g_i = -g_opp + 2 w_i T_wall (1 + rho),
// rounded the same way (one fused multiply-add) in every kernel that applies or inverts it.
__device__ __forceinline__ double wall_image(double g, double w, double t_wall, double rho)
{
    return __fma_rn(__dmul_rn(2.0 * w, t_wall), __dadd_rn(1.0, rho), -g);
}
__device__ __forceinline__ float wall_image(float g, double w, float t_wall, float rho)
{
    return __fmaf_rn(__fmul_rn((float)(2.0 * w), t_wall), __fadd_rn(1.0f, rho), -g);
}


inline size_t store_bytes(int mode)
{
    return mode == RBTP_STORE_F64 ? 8 : (mode == RBTP_STORE_F32 ? 4 : 2);
}

// ------------------------------------------------------------------------------------------------
// Geometry and constants passed by value to kernels.
// ------------------------------------------------------------------------------------------------
struct Geo {
    int lx, ly, lz;
    long long lxy, L;
};

// Slot offsets of the odd (swapped -> natural) step relative to a node's own slot of direction 0,
// in elements: the gather of direction i reads slot (opp i, x - c_i) at g[i] = opp(i) L - off_i,
// and the scatter of direction i writes slot (i, x + c_i) at i L + off_i = g[opp i]
// (off_i = c_ix + c_iy LX + c_iz LX LY).  Built once per launch on the host, so the kernel takes
// each offset from its parameters instead of forming it in every warp.
struct AAOff {
    long long g[27];
};
inline AAOff make_aa_off(const Geo &geo)
{
    AAOff a;
    for (int i = 0; i < 27; ++i)
        a.g[i] = (long long)dopp(i) * geo.L - ((long long)dcx(i) + (long long)dcy(i) * geo.lx + (long long)dcz(i) * geo.lxy);
    return a;
}

// Relaxation and forcing constants of the step kernel, precomputed on the host in the kernel's
// arithmetic type (per-thread double divisions would occupy GB300's narrow FP64 pipe).
template <class R>
struct StepK {
    R tinv, om;        // 1/tau, 1 - 1/tau                    (collision.cu:17-18,27)
    R Gc;              // 3 (1 - 1/(2 tau)): Guo force factor  (collision.cu:18,28-30)
    R tcinv, omc;      // 1/tauc, 1 - 1/tauc                  (collision.cu:85-86)
    R gd0, Rc;         // 2 tauc / 3, 1 - 1/(2 tauc)          (collision.cu:72-73)
    R g0b, t0;         // grav0 * beta, T_REF                 (macrovar.cu:45)
    R thot, tcold;     // wall temperatures                   (streaming.cu:55-58)
    R tla, tlb;        // conduction profile T_c(x) = tla + tlb x (shifted-FP16 g storage)
};

struct Phys {
    double tau, tauc, grav0, beta, thot, tcold, t0, diff, visc, rho0;
    double tla, tlb;   // conduction profile at node x: T_c(x) = tla + tlb x
    StepK<double> kd;
    StepK<float> kf;
    double radius, mass, inertia, heat_cap, rho_ratio;
    double rep_coeff, min_gap, min_gap_w, stf0, stf1, stf0_w, stf1_w;
    double cp_ratio, vol_fraction;
};

// Shift of the shifted-FP16 g storage for a slot whose home node has x-index ix.
__host__ __device__ __forceinline__ double gshift(const Phys &ph, int ix) { return ph.tla + ph.tlb * (double)ix; }

template <class R>
__host__ __device__ __forceinline__ const StepK<R> &step_consts(const Phys &ph)
{
    if constexpr (sizeof(R) == 8) return ph.kd;
    else return ph.kf;
}

template <class R>
inline StepK<R> make_step_consts(const Phys &ph)
{
    StepK<R> k;
    k.tinv = (R)(1.0 / ph.tau);
    k.om = (R)(1.0 - 1.0 / ph.tau);
    k.Gc = (R)(3.0 * (1.0 - 0.5 / ph.tau));
    k.tcinv = (R)(1.0 / ph.tauc);
    k.omc = (R)(1.0 - 1.0 / ph.tauc);
    k.gd0 = (R)(2.0 * ph.tauc / 3.0);
    k.Rc = (R)(1.0 - 1.0 / (2.0 * ph.tauc));
    k.g0b = (R)(ph.grav0 * ph.beta);
    k.t0 = (R)ph.t0;
    k.thot = (R)ph.thot;
    k.tcold = (R)ph.tcold;
    k.tla = (R)ph.tla;
    k.tlb = (R)ph.tlb;
    return k;
}

// Device status word, read once per rbtp_step call.
struct DevStatus {
    int nonfinite;         // non-finite density seen by the step kernel
    int link_overflow;     // a particle's link slab overflowed (bound violated)
    int nf_overflow;       // new-fluid list overflowed
    int contact_overflow;  // contact candidate list overflowed
    int nf_count;          // new-fluid nodes of the last refill
    int ncontacts;         // contact pairs of the last contact pass
    int nsamp;             // plane-sum samples written to the batch sample ring (batched runs)
    int pad;
};

// Output selection of the step kernel.
// OUT_IDLE (batched runs only): the cavity has reached its stop step and does not advance.
enum StepOut { OUT_NONE = 0, OUT_RHO = 1, OUT_MACROS = 2, OUT_MACROS_COL = 3, OUT_IDLE = 4 };

// ------------------------------------------------------------------------------------------------
// Kernel launch wrappers (defined in the .cu files).
// ------------------------------------------------------------------------------------------------
// In-place AA storage.  One array holds every population slot (i, x) (direction-major, [ip][z][y][x]);
// steps alternate between two kinds, so that each slot is read and written by the same thread:
//   even step (natural -> swapped): node x reads its post-streaming f_i(x) from slot (i, x) and
//     writes its post-collision f*_i(x) to slot (opp(i), x);
//   odd step (swapped -> natural): node x gathers f_i(x) = f*_i(x - c_i) from slot
//     (opp(i), x - c_i), or, where x - c_i is outside the box, the wall's image of f*_opp(i)(x)
//     from slot (i, x); it writes f*_i(x) to slot (i, x + c_i), or, where x + c_i is outside, the
//     wall-processed population f_opp(i)(x) of the next step to slot (opp(i), x).
// Node x of an odd step reads exactly the slots it writes, so one array serves both halves.  The
// streaming of an even step's output happens in the next odd step's gather (which applies the walls
// with the even step's wall densities, rho_wall); the streaming of an odd step's output happens in
// its own scatter (walls applied with the node's own density).  After an odd step the natural slots
// hold post-streaming populations (PHASE_HOME), after an even step the post-collision populations
// of every node sit swapped in its own slots (PHASE_SWAPPED).  Shifted-FP16 storage keeps each slot
// relative to the conduction profile at the slot's own node.
constexpr int PHASE_HOME = 0;      // natural slots hold post-streaming populations: the next step is even
constexpr int PHASE_SWAPPED = 1;   // post-collision populations (+ IBB/refill fix-ups) stored swapped:
                                   // the next step is odd
struct StepBuffers {
    void *f, *g;        // the population array (g == f in the paired float modes), read and written
    void *faux;         // F_x of the previous step in, F_x of this step out (L of Store<MODE>::A)
    double *rho_wall;   // density deviation at the x = 0 and x = LX-1 planes (2*LY*LZ)
    double *rho, *ux, *uy, *uz, *phi;   // macro outputs (L each), may be null
    double *fcol, *gcol;                // FP64 copy of the post-collision populations, may be null
    DevStatus *status;
};

cudaError_t launch_step(int mode, bool odd, int out, const Geo &geo, const Phys &ph,
                        const StepBuffers &b, cudaStream_t st);
// Post-streaming populations f(n) (the reference's d_f / d_g after a step) from an array in
// PHASE_SWAPPED, as FP64 home layout: the odd step's gather, walls included, without collision.
cudaError_t launch_stream_export(int mode, const Geo &geo, const Phys &ph, const void *fin,
                                 const void *gin, const double *rho_wall, double *fout,
                                 double *gout, cudaStream_t st);
cudaError_t launch_home_export(int mode, const Geo &geo, const Phys &ph, const void *fin,
                               const void *gin, double *fout, double *gout, cudaStream_t st);
cudaError_t launch_home_import(int mode, const Geo &geo, const Phys &ph, const double *fin,
                               const double *gin, void *fout, void *gout, cudaStream_t st);
// One-pass restart import of nodes n0 .. n0 + count - 1 (populations, flow fields or moments,
// buoyancy auxiliary); sources in device memory or device-visible page-locked host memory.
cudaError_t launch_import_nodes(int mode, const Geo &geo, const Phys &ph, long long n0, long long count,
                                const double *f, const double *g, long long pstride, const double *f7,
                                long long fstride, void *fout, void *gout, void *faux, double *rho,
                                double *ux, double *uy, double *uz, double *phi, double *ted, double *ked,
                                int sms, cudaStream_t st);
cudaError_t launch_fresh_init(int mode, const Geo &geo, const Phys &ph, void *f, void *g,
                              void *faux, double *rho, double *ux, double *uy, double *uz,
                              double *phi, cudaStream_t st);
cudaError_t launch_macros_from_home(const Geo &geo, const double *f, const double *g, double *rho,
                                    double *ux, double *uy, double *uz, double *phi,
                                    cudaStream_t st);
cudaError_t launch_forcing(int mode, const Geo &geo, const Phys &ph, const double *phi, void *faux,
                           cudaStream_t st);

// Particle pipeline ------------------------------------------------------------------------------
// Link chunks of a particle's IBB pass: CTA c of particle p takes links c*128 + k*nc*128 + t, with
// nc = PartBuffers::ibb_chunks (fixed per cavity by its sphere size, at most IBB_CHUNKS); the
// chunk partial sums are added in chunk order by the integrator (deterministic, and the same in
// single-cavity and batched runs).
constexpr int IBB_CHUNKS = 8;
// Bit of a link's direction word that marks an in-domain fluid upstream node x - c_ip (the
// interpolating branch of the IBB); the direction is the word's low five bits.
constexpr int LINK_UP = 5, LINK_DIR_MASK = 31;
constexpr int ibb_chunks_for(long long link_cap)
{
    return link_cap <= 2048 ? 1 : (link_cap >= 2048LL * IBB_CHUNKS ? IBB_CHUNKS : (int)((link_cap + 2047) / 2048));
}

// Per-particle geometry derived once per link build from the FP64 position (one thread per
// particle), so that the per-particle CTAs spend no FP64 work on their setup: the integer boxes of
// marking (radius r), link fill (r, padded by 1) and new-fluid detection (r + 1.76..., padded by 1),
// the integer part of the centre and 1/2 minus its fraction (exact float node offsets), the centre
// in float, the float constants of the marking band, and the rigid-body velocity, spin and
// temperature in float for the next IBB pass (they change only in the integrator, before the build).
struct PGeo {
    int mbox[6], lbox[6], nbox[6];   // x0, x1, y0, y1, z0, z1
    int ic[3];
    float h[3], c[3];
    float rf2, band;
    float v[3], w[3], T, momk;       // velocity, spin, temperature; 2 rho0 / c_s^2
};

struct PartBuffers {
    int np;
    double *state;          // 33 columns x np, column-major (col c at state + c*np)
    double *hpart;          // IBB partial sums: np x IBB_CHUNKS x 7 (force, torque, heat)
    int ibb_chunks;         // link chunks (CTAs) per particle, 1..IBB_CHUNKS, from the link capacity
    PGeo *pgeo;             // np entries, refreshed before every marking pass
    double *cF;             // contact force (3*np)
    int link_cap;           // links per particle slab
    int *link_node, *link_cnt;
    int *link_dir;          // direction ip in bits 0-4, LINK_UP set when x - c_ip is in-domain fluid
    double *link_q;
    int nf_cap;
    int *nf_node, *nf_pid;
    double *nf_val;         // nf_cap * 54 refill values (27 f then 27 g)
    double *nf_mac;         // nf_cap * 5 refill macros (rho, ux, uy, uz, phi)
    // contacts
    int ncell[3];
    double cell_size;
    int *cell_count, *cell_start, *cell_fill, *cell_items;
    int cand_cap;
    int pair_cap;
    int *pair_p, *pair_q;
    int box_half_mark, box_half_link, box_half_nf;
};

// IBB after a step of the given parity (odd: the step just taken was odd; slots as StepBuffers
// describes).
cudaError_t launch_links_ibb(int mode, const Geo &geo, const Phys &ph, const PartBuffers &pb,
                             void *f, void *g, const double *rho, bool odd, cudaStream_t st);
cudaError_t launch_contacts(const Geo &geo, const Phys &ph, const PartBuffers &pb,
                            DevStatus *status, cudaStream_t st);
// The integrator also refreshes the particles' geometry cache (PGeo) for their new positions.
cudaError_t launch_update(const Geo &geo, const Phys &ph, const PartBuffers &pb, cudaStream_t st);
// pgeo: refresh the geometry cache first (false right after launch_update, which did it)
cudaError_t launch_mark(const Geo &geo, const Phys &ph, const PartBuffers &pb, int *owner_out,
                        cudaStream_t st, bool pgeo = true);
cudaError_t launch_link_fill(int mode, const Geo &geo, const Phys &ph, const PartBuffers &pb,
                             const int *owner, DevStatus *status, cudaStream_t st);
cudaError_t launch_refill(int mode, const Geo &geo, const Phys &ph, const PartBuffers &pb,
                          const int *owner_prev, const int *owner_cur, void *f, void *g,
                          void *faux, const double *rho_wall, bool macros, double *rho,
                          double *ux, double *uy, double *uz, double *phi, DevStatus *status,
                          bool odd, cudaStream_t st);

// ------------------------------------------------------------------------------------------------
// Batched execution: one descriptor per cavity in device memory.  The step state (buffer parity,
// owner parity, phase, step counter, this step's output mode) lives on the device and is advanced by
// the batch kernels themselves, so a captured CUDA graph can be replayed step after step.
// ------------------------------------------------------------------------------------------------
struct CavDesc {
    Geo geo;
    Phys ph;
    AAOff aoff;                         // odd-step slot offsets of this member's lattice
    void *f, *g;                        // the population array (in-place AA storage)
    void *faux;                         // F_x auxiliary (Store<MODE>::A)
    double *rho_wall, *rho, *ux, *uy, *uz, *phi;
    DevStatus *status;
    PartBuffers pb;
    int *owner[2];
    int ocur, phase, istep;             // advanced on the device (phase: PHASE_HOME / PHASE_SWAPPED)
    int ndiag, nnuout, nflowout, nend;  // output cadence (<= 0: never)
    int every;                          // extra macro cadence (sampling), <= 0: never
    int out;                            // this step's output mode (written by the plan kernel)
    int last_out;                       // output mode of the last step actually taken
    int stop_at;                        // step at which the cavity stops advancing, <= 0: never
    int samp_now;                       // this step ends with a plane-sum sample (plan kernel)
    int mode;
    // sample ring: samp_cap slots of (1 + NPLANEQ * lx) doubles (step, plane sums); null: none
    double *samp;
    int samp_cap;
    int nchunks;                        // row chunks of the plane reduction (partials buffer)
    double *partials;
};

constexpr int BATCH_SHAPES = 2;  // tile shapes of the batched step: 0 = 32x4, 1 = 64x2
// z-planes per tile of the batched step: a block stages its member's constants once and steps
// BATCH_TILE_Z planes of its (x, y) tile
#ifndef RBTP_BATCH_TILE_Z
#define RBTP_BATCH_TILE_Z 4
#endif
constexpr int BATCH_TILE_Z = RBTP_BATCH_TILE_Z;
cudaError_t launch_batch_plan(CavDesc *desc, int n, cudaStream_t st);
cudaError_t launch_batch_advance(CavDesc *desc, int n, cudaStream_t st);
cudaError_t launch_step_batched(int mode, int shape, const CavDesc *desc, const int4 *tiles,
                                int ntiles, int grid, cudaStream_t st);
// The contact kernels (positions only) run on `side` beside IBB: forked after `ev_fork` is recorded
// on st, joined through `ev_join` before the integrator.
cudaError_t launch_particles_batched(int mode, const CavDesc *desc, const int2 *pmap, int total_np,
                                     const int2 *cmap, int ncmap, const int *pmem, int npmem, cudaStream_t st,
                                     cudaStream_t side, cudaEvent_t ev_fork, cudaEvent_t ev_join);

// Diagnostics ------------------------------------------------------------------------------------
// Per-x-plane sums: 10 quantities x lx, see diagnostics.cu.
constexpr int NPLANEQ = 10;
cudaError_t launch_plane_sums(const Geo &geo, const Phys &ph, const double *ux, const double *uy,
                              const double *uz, const double *phi, const int *owner,
                              const double *pstate, int np, double *partials, int nchunks,
                              double *plane, cudaStream_t st);
// Batched sampling: plane sums of every cavity whose samp_now is set, into its sample ring.
cudaError_t launch_batch_sample(const CavDesc *desc, int n, cudaStream_t st);
cudaError_t launch_dissipation(int mode, const Geo &geo, const Phys &ph, const double *fcol,
                               const double *gcol, const double *rho, const double *ux,
                               const double *uy, const double *uz, const double *phi,
                               const void *faux, const int *owner, double *ted, double *ked,
                               cudaStream_t st);

}  // namespace rbtp
