// lbm_step.cu — fused D3Q27 f+g stream/collide kernel (in-place AA storage) for sm_103a.
//
// One thread per lattice node.  The kernel replaces the reference's per-step sequence
//   macrovar (macrovar.cu:3-34) -> forcing (macrovar.cu:36-47) -> collision_BGK (collision.cu:3-33)
//   -> f_collide copy -> streaming (streaming.cu:3-23) -> collision_BGK_scalar (collision.cu:35-89)
//   -> g_collide copy -> streaming_scalar (streaming.cu:25-63)
// with a single read and a single write of every population, in place: one population array in the
// AA pattern (slots described in rbtp_internal.cuh).  Even steps read a node's post-streaming
// populations from its natural slots and write the post-collision ones swapped into the same
// node's slots; odd steps gather the swapped populations of the neighbours (streaming the even
// step's output, with the wall bounce-back/Dirichlet image where x - c_i is outside the box) and
// scatter their own output to the neighbours' natural slots (streaming it, walls applied at the
// scatter).  Sparse particle corrections (IBB, refill) are written by their own kernels into exactly
// the slots the next step reads, so the bulk kernel never branches on solid flags.
//
// The collision is the reference's BGK algebra regrouped by direction pairs (i, opp(i)): with
// A = 4.5 (c.u)^2 - 1.5 u^2 (even in c) and B = 3 c.u (odd in c), both f and g post-collision
// values split into a pair-symmetric and a pair-antisymmetric part.  The g source term of
// collision.cu:57-88 reduces to w_i c_i.V with one per-node vector V because it is linear in c_i;
// its first pass (the non-equilibrium first moment) is sum_i c_i g_i - phi u exactly.
#include <algorithm>

#include "step_node.cuh"

namespace rbtp {

namespace {

template <int MODE, bool ODD, int OUT>
__global__ void __launch_bounds__(128, RBTP_STEP_MINB(MODE))
    k_step(const Geo geo, const Phys ph, const StepBuffers b, const AAOff ao)
{
    pdl_wait();
    pdl_trigger();
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    const int iz = blockIdx.z;
    if (ix >= geo.lx || iy >= geo.ly) return;
    step_node<MODE, ODD, OUT>(geo, ph, b, ao, ix, iy, iz);
}

// Stream-only export: the post-streaming populations f(n) of the reference (its d_f / d_g after a
// step) reconstructed from an array whose post-collision populations sit swapped (after an even
// step): the odd step's gather without the collision, as FP64 home layout.
template <int MODE>
__global__ void __launch_bounds__(128) k_stream_export(const Geo geo, const Phys ph, const void *fin_,
                                                       const void *gin_, const double *rho_wall,
                                                       double *fout, double *gout)
{
    using ST = Store<MODE>;
    using S = typename ST::S;
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y * blockDim.y + threadIdx.y;
    const int iz = blockIdx.z;
    if (ix >= geo.lx || iy >= geo.ly) return;
    const long long L = geo.L;
    const long long node = (long long)iz * geo.lxy + (long long)iy * geo.lx + ix;
    const S *fin = static_cast<const S *>(fin_);
    const S *gin = static_cast<const S *>(gin_);
    const bool xlo = ix == 0, xhi = ix == geo.lx - 1;
    const bool ylo = iy == 0, yhi = iy == geo.ly - 1;
    const bool zlo = iz == 0, zhi = iz == geo.lz - 1;
    const long long wall_slot = (long long)iz * geo.ly + iy;
    double rw = 0.0;
    if (xlo || xhi) rw = rho_wall[(xhi ? (long long)geo.lz * geo.ly : 0) + wall_slot];
    unroll<27>([&](auto I) {
        constexpr int i = decltype(I)::value;
        constexpr int cx = dcx(i), cy = dcy(i), cz = dcz(i), o = dopp(i);
        constexpr double w = dweight(i);
        const bool ox = (cx == 1 && xlo) || (cx == -1 && xhi);
        const bool oy = (cy == 1 && ylo) || (cy == -1 && yhi);
        const bool oz = (cz == 1 && zlo) || (cz == -1 && zhi);
        const bool out = ox || oy || oz;
        const long long off = (long long)cx + (long long)cy * geo.lx + (long long)cz * geo.lxy;
        // f*_i(x - c_i) in slot (opp(i), x - c_i); outside the box f*_opp(i)(x) in slot (i, x)
        const long long src = out ? ((long long)i * L + node) : ((long long)o * L + node - off);
        fout[(long long)i * L + node] = (double)ST::ld_f(fin + src, w, ph.t0);
        double gr = (double)ST::ld_g(gin + src, w, gshift(ph, out ? ix : ix - cx));
        if (ox && !oy && !oz) {
            const double tw = (cx == 1) ? ph.thot : ph.tcold;
            gr = wall_image(gr, w, tw, rw);
        }
        gout[(long long)i * L + node] = gr;
    });
}

template <int MODE>
__global__ void k_home_export(const Geo geo, const Phys ph, const void *fin_, const void *gin_,
                              double *fout, double *gout)
{
    using ST = Store<MODE>;
    using S = typename ST::S;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= geo.L) return;
    const S *fin = static_cast<const S *>(fin_);
    const S *gin = static_cast<const S *>(gin_);
    const double sh = gshift(ph, (int)(n % geo.lx));
    unroll<27>([&](auto I) {
        constexpr int i = decltype(I)::value;
        constexpr double w = dweight(i);
        fout[(long long)i * geo.L + n] = (double)ST::ld_f(fin + (long long)i * geo.L + n, w, ph.t0);
        gout[(long long)i * geo.L + n] = (double)ST::ld_g(gin + (long long)i * geo.L + n, w, sh);
    });
}

template <int MODE>
__global__ void k_home_import(const Geo geo, const Phys ph, const double *fin, const double *gin,
                              void *fout_, void *gout_)
{
    using ST = Store<MODE>;
    using S = typename ST::S;
    using R = typename ST::R;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= geo.L) return;
    S *fout = static_cast<S *>(fout_);
    S *gout = static_cast<S *>(gout_);
    const double sh = gshift(ph, (int)(n % geo.lx));
    unroll<27>([&](auto I) {
        constexpr int i = decltype(I)::value;
        constexpr double w = dweight(i);
        ST::st_f(fout + (long long)i * geo.L + n, (R)fin[(long long)i * geo.L + n], w, ph.t0);
        ST::st_g(gout + (long long)i * geo.L + n, (R)gin[(long long)i * geo.L + n], w, sh);
    });
}

// Restart import of the nodes n0 .. n0 + count - 1 in one pass (the array form of
// load_restart_state, initial.cu:194-236): the FP64 home-layout populations f_i, g_i (node n0 + k
// of direction i at f[i * pstride + k]) into the storage slots (i, n); the seven flow fields rho,
// ux, uy, uz, phi, ted, ked (field j at f7[j * fstride + k]) into the device fields, or, with f7
// null, macrovar's moments of the imported populations with zero force (macrovar.cu:3-34) and
// ted = ked = 0; and forcing()'s buoyancy F_x = g0 beta (phi - T0) (macrovar.cu:45) from phi.
// The sources are device memory or page-locked host memory read directly through its device
// alias; every source element is read once, in coalesced rows of one direction.
template <int MODE>
__global__ void __launch_bounds__(256) k_import_nodes(const Geo geo, const Phys ph, long long n0, long long count,
                                                      const double *__restrict__ f, const double *__restrict__ g,
                                                      long long pstride, const double *__restrict__ f7,
                                                      long long fstride, void *fout_, void *gout_, void *faux_,
                                                      double *rho, double *ux, double *uy, double *uz,
                                                      double *phi, double *ted, double *ked)
{
    using ST = Store<MODE>;
    using S = typename ST::S;
    using R = typename ST::R;
    S *fout = static_cast<S *>(fout_);
    S *gout = static_cast<S *>(gout_);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride) {
        const long long n = n0 + k;
        const double sh = gshift(ph, (int)(n % geo.lx));
        double r = 0, jx = 0, jy = 0, jz = 0, p = 0;
        unroll<27>([&](auto I) {
            constexpr int i = decltype(I)::value;
            constexpr double w = dweight(i);
            const double fv = f[(long long)i * pstride + k];
            const double gv = g[(long long)i * pstride + k];
            const long long slot = (long long)i * geo.L + n;
            if constexpr (ST::PAIRED) {
                S v;   // both halves of the (f_i, g_i) slot, stored at once
                ST::st_f(&v, (R)fv, w, ph.t0);
                ST::st_g(&v, (R)gv, w, sh);
                fout[slot] = v;
            } else {
                ST::st_f(fout + slot, (R)fv, w, ph.t0);
                ST::st_g(gout + slot, (R)gv, w, sh);
            }
            r += fv;
            jx += dcx(i) * fv;
            jy += dcy(i) * fv;
            jz += dcz(i) * fv;
            p += gv;
        });
        double phv;
        if (f7) {
            rho[n] = f7[k];
            ux[n] = f7[fstride + k];
            uy[n] = f7[2 * fstride + k];
            uz[n] = f7[3 * fstride + k];
            phv = f7[4 * fstride + k];
            ted[n] = f7[5 * fstride + k];
            ked[n] = f7[6 * fstride + k];
        } else {
            rho[n] = r; ux[n] = jx; uy[n] = jy; uz[n] = jz;
            phv = p;
            ted[n] = 0.0;
            ked[n] = 0.0;
        }
        phi[n] = phv;
        static_cast<typename ST::A *>(faux_)[n] = (typename ST::A)(ph.grav0 * ph.beta * (phv - ph.t0));
    }
}

// init_f / init_g (initial.cu:335-397): deviation-form rest f = 0; g from the equilibrium at
// T = T_REF with the rho field that init_f set to RHO0.
template <int MODE>
__global__ void k_fresh_init(const Geo geo, const Phys ph, void *f_, void *g_, void *faux_,
                             double *rho, double *ux, double *uy, double *uz, double *phi)
{
    using ST = Store<MODE>;
    using S = typename ST::S;
    using R = typename ST::R;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= geo.L) return;
    S *f = static_cast<S *>(f_);
    S *g = static_cast<S *>(g_);
    const double r = ph.rho0;
    const double tT = ph.t0;
    const double lambda0 = 1.0 - dweight(0);
    rho[n] = ph.rho0;
    ux[n] = 0.0; uy[n] = 0.0; uz[n] = 0.0;
    phi[n] = tT;
    static_cast<typename ST::A *>(faux_)[n] = (typename ST::A)(ph.grav0 * ph.beta * (tT - ph.t0));
    unroll<27>([&](auto I) {
        constexpr int i = decltype(I)::value;
        constexpr double w = dweight(i);
        double geq = w * tT * (1.0 + 0.0 + 0.5 * (0.0 - 0.0));
        if (i == 0) geq -= lambda0 * tT * r;
        else geq += w * tT * r;
        ST::st_f(f + (long long)i * geo.L + n, (R)(w * (0.0 + 0.0 + 0.5 * (0.0 - 0.0))), w, ph.t0);
        ST::st_g(g + (long long)i * geo.L + n, (R)geq, w, gshift(ph, (int)(n % geo.lx)));
    });
}

// macrovar (macrovar.cu:3-34) on FP64 home-layout arrays with zero force (restart without the
// %09d.dat fields).
__global__ void k_macros_from_home(const Geo geo, const double *f, const double *g, double *rho,
                                   double *ux, double *uy, double *uz, double *phi)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= geo.L) return;
    double r = 0, jx = 0, jy = 0, jz = 0, p = 0;
    unroll<27>([&](auto I) {
        constexpr int i = decltype(I)::value;
        const double fv = f[(long long)i * geo.L + n];
        r += fv;
        jx += dcx(i) * fv;
        jy += dcy(i) * fv;
        jz += dcz(i) * fv;
        p += g[(long long)i * geo.L + n];
    });
    rho[n] = r; ux[n] = jx; uy[n] = jy; uz[n] = jz; phi[n] = p;
}

template <int MODE>
__global__ void k_forcing(const Geo geo, const Phys ph, const double *phi, void *faux)
{
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= geo.L) return;
    using A = typename Store<MODE>::A;
    static_cast<A *>(faux)[n] = (A)(ph.grav0 * ph.beta * (phi[n] - ph.t0));
}

inline dim3 node_grid(const Geo &g, dim3 blk)
{
    return dim3((g.lx + blk.x - 1) / blk.x, (g.ly + blk.y - 1) / blk.y, g.lz);
}
inline unsigned lin_blocks(long long n, int t) { return (unsigned)((n + t - 1) / t); }

template <int MODE>
cudaError_t launch_step_mode(bool odd, int out, const Geo &geo, const Phys &ph,
                             const StepBuffers &b, cudaStream_t st)
{
    // Warps of 32 x-nodes in one row (FP64, FP32: 16-wide blocks cost 3 % at 320x320x160, wider
    // ones nothing).  Shifted FP16 is issue-bound: its odd steps use 16 x 2 warps, so that half as
    // many warps hold an x-face node and take the face-tested gather and scatter (0.683 against
    // 0.695 ms for 32-wide rows at 320x320x160); its even steps, which touch no neighbour, run
    // best in 64-node rows (0.583 against 0.596 ms for 32-wide rows).
    dim3 blk(32, 4, 1);
    if (MODE == RBTP_STORE_F16S) blk = odd ? dim3(16, 8, 1) : (geo.lx % 64 == 0 ? dim3(64, 2, 1) : dim3(32, 4, 1));
    const dim3 grd = node_grid(geo, blk);
    const AAOff ao = make_aa_off(geo);
#define RBTP_STEP_CASE(P, O)                                                       \
    if (odd == P && out == O) return pdl_launch(k_step<MODE, P, O>, grd, blk, st, geo, ph, b, ao);
    RBTP_STEP_CASE(true, OUT_NONE)
    RBTP_STEP_CASE(true, OUT_RHO)
    RBTP_STEP_CASE(true, OUT_MACROS)
    RBTP_STEP_CASE(true, OUT_MACROS_COL)
    RBTP_STEP_CASE(false, OUT_NONE)
    RBTP_STEP_CASE(false, OUT_RHO)
    RBTP_STEP_CASE(false, OUT_MACROS)
    RBTP_STEP_CASE(false, OUT_MACROS_COL)
#undef RBTP_STEP_CASE
    return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_step(int mode, bool odd, int out, const Geo &geo, const Phys &ph,
                        const StepBuffers &b, cudaStream_t st)
{
    switch (mode) {
    case RBTP_STORE_F64: return launch_step_mode<RBTP_STORE_F64>(odd, out, geo, ph, b, st);
    case RBTP_STORE_F32: return launch_step_mode<RBTP_STORE_F32>(odd, out, geo, ph, b, st);
    case RBTP_STORE_F16S: return launch_step_mode<RBTP_STORE_F16S>(odd, out, geo, ph, b, st);
    }
    return cudaErrorInvalidValue;
}

#define RBTP_MODE_DISPATCH(mode, CALL)                                  \
    switch (mode) {                                                     \
    case RBTP_STORE_F64: { constexpr int M = RBTP_STORE_F64; CALL; break; } \
    case RBTP_STORE_F32: { constexpr int M = RBTP_STORE_F32; CALL; break; } \
    case RBTP_STORE_F16S: { constexpr int M = RBTP_STORE_F16S; CALL; break; } \
    default: return cudaErrorInvalidValue;                              \
    }

cudaError_t launch_stream_export(int mode, const Geo &geo, const Phys &ph, const void *fin,
                                 const void *gin, const double *rho_wall, double *fout,
                                 double *gout, cudaStream_t st)
{
    const dim3 blk(32, 4, 1);
    const dim3 grd = node_grid(geo, blk);
    RBTP_MODE_DISPATCH(mode, (k_stream_export<M><<<grd, blk, 0, st>>>(geo, ph, fin, gin, rho_wall, fout, gout)));
    return cudaGetLastError();
}

cudaError_t launch_home_export(int mode, const Geo &geo, const Phys &ph, const void *fin,
                               const void *gin, double *fout, double *gout, cudaStream_t st)
{
    RBTP_MODE_DISPATCH(mode, (k_home_export<M><<<lin_blocks(geo.L, 256), 256, 0, st>>>(geo, ph, fin, gin, fout, gout)));
    return cudaGetLastError();
}

cudaError_t launch_home_import(int mode, const Geo &geo, const Phys &ph, const double *fin,
                               const double *gin, void *fout, void *gout, cudaStream_t st)
{
    RBTP_MODE_DISPATCH(mode, (k_home_import<M><<<lin_blocks(geo.L, 256), 256, 0, st>>>(geo, ph, fin, gin, fout, gout)));
    return cudaGetLastError();
}

cudaError_t launch_import_nodes(int mode, const Geo &geo, const Phys &ph, long long n0, long long count,
                                const double *f, const double *g, long long pstride, const double *f7,
                                long long fstride, void *fout, void *gout, void *faux, double *rho,
                                double *ux, double *uy, double *uz, double *phi, double *ted, double *ked,
                                int sms, cudaStream_t st)
{
    if (count <= 0) return cudaSuccess;
    // a grid of a few blocks per SM keeps many independent row loads in flight (host-memory
    // sources answer with a long latency) without one block per node
    const long long want = (count + 255) / 256;
    const unsigned blocks = (unsigned)std::min<long long>(want, 8LL * std::max(sms, 1));
    RBTP_MODE_DISPATCH(mode, (k_import_nodes<M><<<blocks, 256, 0, st>>>(geo, ph, n0, count, f, g, pstride, f7, fstride,
                                                                      fout, gout, faux, rho, ux, uy, uz, phi, ted, ked)));
    return cudaGetLastError();
}

cudaError_t launch_fresh_init(int mode, const Geo &geo, const Phys &ph, void *f, void *g,
                              void *faux, double *rho, double *ux, double *uy, double *uz,
                              double *phi, cudaStream_t st)
{
    RBTP_MODE_DISPATCH(mode, (k_fresh_init<M><<<lin_blocks(geo.L, 256), 256, 0, st>>>(geo, ph, f, g, faux, rho, ux, uy, uz, phi)));
    return cudaGetLastError();
}

cudaError_t launch_macros_from_home(const Geo &geo, const double *f, const double *g, double *rho,
                                    double *ux, double *uy, double *uz, double *phi,
                                    cudaStream_t st)
{
    k_macros_from_home<<<lin_blocks(geo.L, 256), 256, 0, st>>>(geo, f, g, rho, ux, uy, uz, phi);
    return cudaGetLastError();
}

cudaError_t launch_forcing(int mode, const Geo &geo, const Phys &ph, const double *phi, void *faux,
                           cudaStream_t st)
{
    RBTP_MODE_DISPATCH(mode, (k_forcing<M><<<lin_blocks(geo.L, 256), 256, 0, st>>>(geo, ph, phi, faux)));
    return cudaGetLastError();
}

}  // namespace rbtp
