// particles.cu — particle coupling kernels for sm_103a.
//
// Replaces src_part/{links,ibb,pforces,move,refill}.cu.  Design:
//   * solid marking: one launch over all particles' bounding boxes; the lowest pid that contains a
//     node owns it (atomicMin), which is the reference's "first serialized launch wins" rule
//     (links.cu:45, 160-188) without N serialized launches or host round trips;
//   * IBB links: a fixed-capacity slab per particle, filled by one CTA per particle in
//     (node, direction) order, so the list is compact per particle and needs no global scan or
//     host-side count (links.cu:50-139, 196-250);
//   * IBB f/g, momentum exchange and heat flux: one CTA per particle walks its slab, writes the
//     bounce-back values straight into the slots the next step reads, and reduces force,
//     torque and heat with a fixed-order tree — deterministic, no floating-point atomics
//     (ibb.cu:5-205);
//   * contacts: a cell list; each particle sums its partners in ascending pid order, the order the
//     reference's pair loop produces (pforces.cu:6-76);
//   * integration, history shift, new-fluid detection and two-phase refill (move.cu:5-103,
//     pforces.cu:80-116, refill.cu:8-240).
// Geometric predicates use explicitly rounded double operations (__dmul_rn/__dadd_rn) so they
// evaluate exactly like a non-contracted C implementation of the reference formulas.
#include "rbtp_internal.cuh"

namespace rbtp {

namespace {

constexpr double NEW_FLUID_THRESH = 1.7606816861659007;  // refill.cu:39,70

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

__device__ __forceinline__ double sq3(double dx, double dy, double dz)
{
    return dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
}

// links.cu:7-23 with explicit rounding.  The lattice direction has components in {-1, 0, 1}, so the
// products c.d are exact and are formed by sign selection, |c|^2 is an exact small integer, and the
// final division by 2|c|^2 is an exact scaling for |c|^2 = 1, 2; results are bit-identical to the
// rounded double formula.
__device__ __forceinline__ double csel(int c, double d) { return c == 0 ? 0.0 : (c > 0 ? d : -d); }

__device__ __forceinline__ bool link_q(int cxi, int cyi, int czi, double x0, double y0, double z0,
                                       double px, double py, double pz, double rsq, double &q)
{
    const double dx = dsub(x0, px), dy = dsub(y0, py), dz = dsub(z0, pz);
    const int a = cxi * cxi + cyi * cyi + czi * czi;
    const double b = dmul(2.0, dadd(dadd(csel(cxi, dx), csel(cyi, dy)), csel(czi, dz)));
    const double c = dsub(sq3(dx, dy, dz), rsq);
    const double disc = dsub(dmul(b, b), dmul((double)(4 * a), c));
    if (disc <= 0.0) return false;
    const double num = dsub(-b, __dsqrt_rn(disc));
    q = (a == 3) ? __ddiv_rn(num, 6.0) : dmul(num, a == 1 ? 0.5 : 0.25);
    return (q >= 0.0 && q <= 1.0);
}

// Single-precision ray-sphere q for the FP32/FP16 storage modes (same formula, float arithmetic).
// Returns 1 (link, q set) or -1 when the float result is too close to a decision edge (grazing
// ray, q near 0 or 1); the caller then takes the exact FP64 test, so the set of links is the FP64
// one in every storage mode and only the q values carry float rounding.
__device__ __forceinline__ int link_q_f32(int cxi, int cyi, int czi, float dx, float dy, float dz,
                                          float rsq, double &q)
{
    const int a = cxi * cxi + cyi * cyi + czi * czi;
    const float b = 2.0f * ((cxi * dx + cyi * dy) + czi * dz);
    const float c = (dx * dx + dy * dy + dz * dz) - rsq;
    const float disc = b * b - (float)(4 * a) * c;
    if (!(disc > 1.0e-3f * rsq)) return -1;
    const float qf = (-b - sqrtf(disc)) * (1.0f / (float)(2 * a));
    if (!(qf > 1.0e-3f && qf < 0.999f)) return -1;
    q = (double)qf;
    return 1;
}

// floor to int with the argument clamped first, so non-finite or far-away particle coordinates give
// empty (clipped) boxes instead of overflowing integer arithmetic; NaN maps to -1e9.
__device__ __forceinline__ int ifloor(double v)
{
    v = fmin(fmax(v, -1.0e9), 1.0e9);
    return (int)floor(v);
}

#define PCOL(st, np, c, p) (st)[(long long)(c) * (np) + (p)]

// Bounding box of links.cu:160-172: floor(p -/+ r - 0.5), clipped to the box.
struct Box { int x0, x1, y0, y1, z0, z1; };

__device__ __forceinline__ Box sphere_box(const Geo &geo, double px, double py, double pz,
                                          double r, int pad)
{
    Box b;
    b.x0 = ifloor(dsub(dsub(px, r), 0.5)) - pad;
    b.x1 = ifloor(dsub(dadd(px, r), 0.5)) + pad;
    b.y0 = ifloor(dsub(dsub(py, r), 0.5)) - pad;
    b.y1 = ifloor(dsub(dadd(py, r), 0.5)) + pad;
    b.z0 = ifloor(dsub(dsub(pz, r), 0.5)) - pad;
    b.z1 = ifloor(dsub(dadd(pz, r), 0.5)) + pad;
    if (b.x0 < 0) b.x0 = 0;
    if (b.y0 < 0) b.y0 = 0;
    if (b.z0 < 0) b.z0 = 0;
    if (b.x1 > geo.lx - 1) b.x1 = geo.lx - 1;
    if (b.y1 > geo.ly - 1) b.y1 = geo.ly - 1;
    if (b.z1 > geo.lz - 1) b.z1 = geo.lz - 1;
    return b;
}

// Per-particle geometry (PGeo) of the current position; one thread per particle.
__device__ __forceinline__ void pgeo_body(const Geo &geo, const Phys &ph, const PartBuffers &pb, int p)
{
    const double *st = pb.state;
    const double px = PCOL(st, pb.np, 0, p), py = PCOL(st, pb.np, 1, p), pz = PCOL(st, pb.np, 2, p);
    const double r = ph.radius;
    PGeo g;
    const Box m = sphere_box(geo, px, py, pz, r, 0);
    const Box l = sphere_box(geo, px, py, pz, r, 1);
    const Box n = sphere_box(geo, px, py, pz, dadd(r, NEW_FLUID_THRESH), 1);
    const Box *bs[3] = {&m, &l, &n};
    int *outs[3] = {g.mbox, g.lbox, g.nbox};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        outs[k][0] = bs[k]->x0; outs[k][1] = bs[k]->x1; outs[k][2] = bs[k]->y0;
        outs[k][3] = bs[k]->y1; outs[k][4] = bs[k]->z0; outs[k][5] = bs[k]->z1;
    }
    const double c[3] = {px, py, pz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        g.ic[a] = ifloor(c[a]);
        g.h[a] = 0.5f - (float)(c[a] - (double)g.ic[a]);
        g.c[a] = (float)c[a];
    }
    // marking band: bounds the float error of |x - X|^2 (coordinate rounding ~6e-8 |X| per
    // component, arithmetic rounding ~1e-7 relative)
    g.rf2 = (float)dmul(r, r);
    const float amax = fmaxf(fabsf(g.c[0]), fmaxf(fabsf(g.c[1]), fabsf(g.c[2])));
    g.band = 1.0e-3f * g.rf2 + 1.0e-5f * (amax + 1.0f) * ((float)r + 2.0f) + 1.0e-3f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        g.v[a] = (float)PCOL(st, pb.np, 3 + a, p);
        g.w[a] = (float)PCOL(st, pb.np, 18 + a, p);
    }
    g.T = (float)PCOL(st, pb.np, 30, p);
    g.momk = (float)(2.0 * ph.rho0 * 3.0);
    pb.pgeo[p] = g;
}

__device__ __forceinline__ Box pgeo_box(const int (&b)[6]) { return Box{b[0], b[1], b[2], b[3], b[4], b[5]}; }

// ------------------------------------------------------------------------------------------------
// Block reduction of NQ doubles in a fixed tree order (deterministic for a fixed block size).
// ------------------------------------------------------------------------------------------------
template <int NQ, int NT>
__device__ __forceinline__ void block_reduce_fixed(double (&v)[NQ], double *sh /* NQ*NT */)
{
    const int t = threadIdx.x;
#pragma unroll
    for (int q = 0; q < NQ; ++q) sh[q * NT + t] = v[q];
    __syncthreads();
#pragma unroll
    for (int s = NT / 2; s > 0; s >>= 1) {
        if (t < s) {
#pragma unroll
            for (int q = 0; q < NQ; ++q) sh[q * NT + t] += sh[q * NT + t + s];
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) v[q] = sh[q * NT];
}

// Double-float (hi + lo, two FP32 words, ~48-bit significand) sums for the FP32/FP16 storage modes:
// error-free TwoSum additions on the FP32 pipe instead of FP64 additions (GB300's FP64 rate is 1/64
// of FP32).  df_add is the standard double-float addition (Knuth TwoSum of the high words, the low
// words added into the error term, renormalised with Fast2Sum).
struct df {
    float hi, lo;
};
__device__ __forceinline__ df df_add(df a, df b)
{
    const float s = a.hi + b.hi;
    const float v = s - a.hi;
    float e = (a.hi - (s - v)) + (b.hi - v);
    e += a.lo + b.lo;
    const float hi = s + e;
    return {hi, e - (hi - s)};
}

// Block reduction of NQ double-float values in a fixed order (warp shuffles, then the warps' sums
// in warp order); the result, valid in thread 0, is returned as FP64.
template <int NQ, int NT>
__device__ __forceinline__ void block_reduce_df(df (&v)[NQ], double (&out)[NQ], float *sh /* 2*NQ*NT/32 */)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const df o{__shfl_down_sync(0xffffffffu, v[q].hi, off), __shfl_down_sync(0xffffffffu, v[q].lo, off)};
            v[q] = df_add(v[q], o);
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            sh[(2 * q) * (NT / 32) + warp] = v[q].hi;
            sh[(2 * q + 1) * (NT / 32) + warp] = v[q].lo;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            df a{sh[(2 * q) * (NT / 32)], sh[(2 * q + 1) * (NT / 32)]};
            for (int w = 1; w < NT / 32; ++w) a = df_add(a, df{sh[(2 * q) * (NT / 32) + w], sh[(2 * q + 1) * (NT / 32) + w]});
            out[q] = (double)a.hi + (double)a.lo;
        }
    }
}

// ------------------------------------------------------------------------------------------------
// Block-wide exclusive scan (NT threads) and the spherical-shell row table of a particle box.
// ------------------------------------------------------------------------------------------------
template <int NT>
__device__ __forceinline__ int block_exclusive_scan(int v, int *wsum, int &total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += t;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    int wbase = 0, tot = 0;
#pragma unroll
    for (int k = 0; k < NT / 32; ++k) {
        const int s = wsum[k];
        if (k < warp) wbase += s;
        tot += s;
    }
    __syncthreads();
    total = tot;
    return wbase + incl - v;
}

// Per-particle CTAs enumerate only the nodes of a spherical shell r_in <= |x + 1/2 - X| <= r_out
// of their box: per (y, z) row, at most two x-intervals (the caller's radii carry float margins so
// that every node its exact test could accept is enumerated).  Rows are numbered by a block scan
// and flat indices map back to nodes by a binary search, in ascending node index order.
template <int NT>
struct ShellRows {
    static constexpr int ROWS = NT >= 512 ? 2048 : 1024;
    int wsum[NT / 32];
    int start[ROWS];   // first flat index of each row
    int xa[ROWS];      // first interval: start and length
    int na[ROWS];
    int xb[ROWS];      // second interval: start
};

// Number of enumerated nodes, or -1 when the box has more rows than the table holds (the caller
// then walks the whole box).  Called by all threads of the CTA; ends with a barrier.
template <int NT>
__device__ __forceinline__ int shell_rows_build(ShellRows<NT> &sr, const Box &b, float pxf, float pyf, float pzf,
                                                float r_in, float r_out)
{
    const int ny = b.y1 - b.y0 + 1, nz = b.z1 - b.z0 + 1, rows = ny * nz;
    if (rows > ShellRows<NT>::ROWS) return -1;
    int carry = 0;
    for (int r0 = 0; r0 < rows; r0 += NT) {
        const int row = r0 + threadIdx.x;
        int cnt = 0;
        if (row < rows) {
            const int ly = row % ny, lz = row / ny;
            const float dy = ((float)(b.y0 + ly) + 0.5f) - pyf, dz = ((float)(b.z0 + lz) + 0.5f) - pzf;
            const float s2 = dy * dy + dz * dz;
            int xa = 0, na = 0, xb = 0, nb = 0;
            if (s2 <= r_out * r_out) {
                const float ho = sqrtf(r_out * r_out - s2);
                const int xl = max(b.x0, (int)ceilf(pxf - 0.5f - ho));
                const int xr = min(b.x1, (int)floorf(pxf - 0.5f + ho));
                xa = xl;
                if (s2 < r_in * r_in) {
                    const float hi = sqrtf(r_in * r_in - s2);
                    const int xle = (int)floorf(pxf - 0.5f - hi), xrs = (int)ceilf(pxf - 0.5f + hi);
                    na = max(0, min(xr, xle) - xl + 1);
                    xb = max(max(xl, xrs), xle + 1);   // never re-enter the first interval
                    nb = max(0, xr - xb + 1);
                } else {
                    na = max(0, xr - xl + 1);
                }
            }
            cnt = na + nb;
            sr.xa[row] = xa;
            sr.na[row] = na;
            sr.xb[row] = xb;
        }
        int tot;
        const int off = block_exclusive_scan<NT>(cnt, sr.wsum, tot);
        if (row < rows) sr.start[row] = carry + off;
        carry += tot;
    }
    __syncthreads();
    return carry;
}

template <int NT>
__device__ __forceinline__ void shell_rows_node(const ShellRows<NT> &sr, const Box &b, int t, int &ix, int &iy,
                                                int &iz)
{
    const int ny = b.y1 - b.y0 + 1, rows = ny * (b.z1 - b.z0 + 1);
    int lo = 0, hi = rows - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sr.start[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    const int o = t - sr.start[lo];
    ix = o < sr.na[lo] ? sr.xa[lo] + o : sr.xb[lo] + (o - sr.na[lo]);
    iy = b.y0 + lo % ny;
    iz = b.z0 + lo / ny;
}

// Calls body(ix, iy, iz) for every node of the shell (or of the whole box when the table is too
// small), each node once, spread over the CTA.
template <int NT, class F>
__device__ __forceinline__ void for_shell_nodes(ShellRows<NT> &sr, const Box &b, float pxf, float pyf, float pzf,
                                                float r_in, float r_out, F &&body)
{
    const int total = shell_rows_build<NT>(sr, b, pxf, pyf, pzf, r_in, r_out);
    if (total >= 0) {
        for (int t = threadIdx.x; t < total; t += NT) {
            int ix, iy, iz;
            shell_rows_node<NT>(sr, b, t, ix, iy, iz);
            body(ix, iy, iz);
        }
    } else {
        const int nx = b.x1 - b.x0 + 1, ny = b.y1 - b.y0 + 1, nz = b.z1 - b.z0 + 1;
        for (int t = threadIdx.x; t < nx * ny * nz; t += NT) {
            const int lz = t / (nx * ny);
            const int rem = t - lz * nx * ny;
            const int ly = rem / nx;
            body(b.x0 + (rem - ly * nx), b.y0 + ly, b.z0 + lz);
        }
    }
}

// ------------------------------------------------------------------------------------------------
// IBB for f and g plus momentum exchange and heat flux, one CTA per particle.
// ------------------------------------------------------------------------------------------------
constexpr int IBB_THREADS = 128;

// Slots of one link (x, ip) in the in-place AA storage after a step of the given parity: where the
// post-collision populations f*_ip(x), f*_ip(x - c_ip) and f*_opp(x) sit, and the slot the next
// step reads as f_opp(x), the population entering x from the solid node x + c_ip.  Even parity
// (post-collision populations swapped into their own node's slots): (opp, x), (opp, x - c),
// (ip, x) and (ip, x + c); odd parity (streamed to the neighbours' natural slots): (ip, x + c),
// (ip, x), (opp, x - c) and (opp, x).  xs_* are the x-indices of the slots' nodes (the shift of
// shifted-FP16 storage).  Reads touch only slots of fluid nodes and, in odd parity, the slot
// (ip, x + c) of the solid node, which no link writes; writes touch slots of solid nodes (even)
// or of fluid nodes that no link reads (odd), so reads and writes never alias.
struct LinkSlots {
    long long here, up, opp, out;
    int xs_here, xs_up, xs_opp, xs_out;
};
__device__ __forceinline__ LinkSlots link_slots(bool odd, long long L, int ip, int o, long long x, long long x1,
                                                long long solid, int ix, int cx)
{
    LinkSlots s;
    if (odd) {
        s.here = (long long)ip * L + solid; s.xs_here = ix + cx;
        s.up = (long long)ip * L + x;       s.xs_up = ix;
        s.opp = (long long)o * L + x1;      s.xs_opp = ix - cx;
        s.out = (long long)o * L + x;       s.xs_out = ix;
    } else {
        s.here = (long long)o * L + x;      s.xs_here = ix;
        s.up = (long long)o * L + x1;       s.xs_up = ix - cx;
        s.opp = (long long)ip * L + x;      s.xs_opp = ix;
        s.out = (long long)ip * L + solid;  s.xs_out = ix + cx;
    }
    return s;
}

template <int MODE>
__device__ __forceinline__ void links_ibb_body(const Geo &geo, const Phys &ph, const PartBuffers &pb,
                                               void *f_, void *g_, const double *rho, bool odd, int p,
                                               int chunk, double *sh)
{
    using ST = Store<MODE>;
    using S = typename ST::S;
    const int np = pb.np;
    S *fB = static_cast<S *>(f_);
    S *gB = static_cast<S *>(g_);
    const long long L = geo.L;
    const double *st = pb.state;
    const double px = PCOL(st, np, 0, p), py = PCOL(st, np, 1, p), pz = PCOL(st, np, 2, p);
    const double vx = PCOL(st, np, 3, p), vy = PCOL(st, np, 4, p), vz = PCOL(st, np, 5, p);
    const double wx = PCOL(st, np, 18, p), wy = PCOL(st, np, 19, p), wz = PCOL(st, np, 20, p);
    const double Tp = PCOL(st, np, 30, p);
    const int n = min(pb.link_cnt[p], pb.link_cap);
    const long long base = (long long)p * pb.link_cap;
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    if constexpr (MODE == RBTP_STORE_F64) {
        for (int t = chunk * IBB_THREADS + threadIdx.x; t < n; t += pb.ibb_chunks * IBB_THREADS) {
            const int x = pb.link_node[base + t];
            const int dw = pb.link_dir[base + t];
            const int ip = dw & LINK_DIR_MASK;
            const double q = pb.link_q[base + t];
            const int iz = x / (int)geo.lxy;
            const int rem = x - iz * (int)geo.lxy;
            const int iy = rem / geo.lx;
            const int ix = rem - iy * geo.lx;
            const int cxi = dcx_rt(ip), cyi = dcy_rt(ip), czi = dcz_rt(ip);
            const int o = dopp_rt(ip);
            const double w = dweight_rt(ip);
            // moving wall velocity at the intersection point (ibb.cu:33-46)
            const double relx = ((double)ix + 0.5 + q * cxi) - px;
            const double rely = ((double)iy + 0.5 + q * cyi) - py;
            const double relz = ((double)iz + 0.5 + q * czi) - pz;
            const double uwx = vx + (relz * wy - rely * wz);
            const double uwy = vy + (relx * wz - relz * wx);
            const double uwz = vz + (rely * wx - relx * wy);
            const double evel = (double)cxi * uwx + (double)cyi * uwy + (double)czi * uwz;
            const double mom = 2.0 * w * ph.rho0 * evel * 3.0;
            const double inv_2q = (q >= 0.5) ? 0.5 / q : 0.0;

            // upstream node x - c_ip, in-domain fluid (flag from the link build's owner reads)
            const bool fluid1 = (dw >> LINK_UP) & 1;
            const long long x1 = (long long)x - cxi - (long long)cyi * geo.lx - (long long)czi * geo.lxy;
            const long long solid = (long long)x + cxi + (long long)cyi * geo.lx + (long long)czi * geo.lxy;
            const LinkSlots sl = link_slots(odd, L, ip, o, x, x1, solid, ix, cxi);

            const double f_here = fB[sl.here];
            const double g_here = gB[sl.here];
            double fval, gval;
            // ibb.cu:52-73 (f: q < 0.5), ibb.cu:114-128 (g: q <= 0.5)
            if (fluid1) {
                if (q < 0.5) {
                    const double f_up = fB[sl.up];
                    fval = 2.0 * q * f_here + (1.0 - 2.0 * q) * f_up - mom;
                } else {
                    const double f_oc = fB[sl.opp];
                    fval = (f_here - mom) * inv_2q + (2.0 * q - 1.0) * inv_2q * f_oc;
                }
            } else {
                fval = f_here - mom;
            }
            const double amp = 2.0 * w * Tp * (1.0 + rho[x]);
            if (fluid1) {
                if (q <= 0.5) {
                    const double gu = gB[sl.up];
                    gval = -(2.0 * q * g_here + (1.0 - 2.0 * q) * gu) + amp;
                } else {
                    const double go = gB[sl.opp];
                    gval = -g_here * inv_2q + amp * inv_2q + (2.0 * q - 1.0) * inv_2q * go;
                }
            } else {
                gval = -g_here + amp;
            }
            // the population that streams into x along opp from the solid node x + c_ip: the slot
            // the next step reads as f_opp(x)
            fB[sl.out] = fval;
            gB[sl.out] = gval;
            // ibb.cu:160-187 (force, torque about the same intersection point) and 202-204 (heat)
            const double Fx = (cxi - uwx) * f_here - (-cxi - uwx) * fval;
            const double Fy = (cyi - uwy) * f_here - (-cyi - uwy) * fval;
            const double Fz = (czi - uwz) * f_here - (-czi - uwz) * fval;
            acc[0] += Fx;
            acc[1] += Fy;
            acc[2] += Fz;
            acc[3] += rely * Fz - relz * Fy;
            acc[4] += relz * Fx - relx * Fz;
            acc[5] += relx * Fy - rely * Fx;
            acc[6] += g_here - gval;
        }
    } else {
        // FP32 / shifted-FP16 storage: the per-link arithmetic runs in FP32 (GB300's FP64 rate is
        // 1/64 of FP32).  Node-centre offsets are formed exactly from the integer part of the
        // centre and its FP64 fraction.  Force, torque and heat are accumulated in double-float
        // (two FP32 words, error-free additions) per thread and over the block, and leave the
        // block as FP64 values.
        const PGeo &pg = pb.pgeo[p];   // from the link build of these positions
        const int ipx = pg.ic[0], ipy = pg.ic[1], ipz = pg.ic[2];
        const float hx = pg.h[0], hy = pg.h[1], hz = pg.h[2];
        const float vxf = pg.v[0], vyf = pg.v[1], vzf = pg.v[2];
        const float wxf = pg.w[0], wyf = pg.w[1], wzf = pg.w[2];
        const float mom_k = pg.momk;   // 2 rho0 / c_s^2
        const float Tpf = pg.T;
        const float tla = ph.kf.tla, tlb = ph.kf.tlb;   // conduction profile (shifted FP16 g)
        df sum[7];
#pragma unroll
        for (int k = 0; k < 7; ++k) sum[k] = df{0.0f, 0.0f};
        auto add = [&](int k, float v) { sum[k] = df_add(sum[k], df{v, 0.0f}); };
        // (f_i, g_i) slots of the paired layout: both populations of a slot in one access;
        // shifted-FP16 g holds g / w - T_c(x_home), the slot's home node x-index gives the shift
        // (read-only path: a link reads only slots of fluid nodes, which no link writes)
        auto ld2 = [&](const S *ptr, int ixh, float wr, float &fv, float &gv) {
            const S v = __ldg(ptr);
            if constexpr (MODE == RBTP_STORE_F16S) {
                fv = __low2float(v) * wr;
                gv = (__high2float(v) + (tla + tlb * (float)ixh)) * wr;
            } else {
                fv = v.x;
                gv = v.y;
            }
        };
        // Gathered inputs of one link.  A link reads slots of fluid nodes only (x and, when it
        // interpolates, x - c_ip) and writes the slot of a solid node (x + c_ip), so the gathers of
        // later links may be issued before the stores of earlier ones: two links are gathered per
        // iteration to keep twice the loads in flight.  Each thread still sums its links in
        // ascending order.
        struct LinkIn {
            int x, ip;
            float q, f_here, g_here, f_2, g_2, rho;
            bool fluid1;
        };
        auto slots_of = [&](int x, int ip) {
            const int cxi = dcx_rt(ip), cyi = dcy_rt(ip), czi = dcz_rt(ip);
            const long long off = (long long)cxi + (long long)cyi * geo.lx + (long long)czi * geo.lxy;
            return link_slots(odd, L, ip, dopp_rt(ip), x, (long long)x - off, (long long)x + off, x % geo.lx, cxi);
        };
        auto gather = [&](int t, LinkIn &a) {
            a.x = __ldg(pb.link_node + base + t);
            const int dw = __ldg(pb.link_dir + base + t);
            a.ip = dw & LINK_DIR_MASK;
            a.q = (float)__ldg(pb.link_q + base + t);
            a.fluid1 = (dw >> LINK_UP) & 1;   // upstream node x - c_ip is in-domain fluid
            const float wr = fweight_rt(a.ip);
            const LinkSlots sl = slots_of(a.x, a.ip);
            ld2(fB + sl.here, sl.xs_here, wr, a.f_here, a.g_here);
            // ibb.cu:52-73 (f: q < 0.5) and ibb.cu:114-128 (g: q <= 0.5) interpolate with the
            // upstream population f*_ip(x - c_ip) below q = 1/2 and with the opposite f*_opp(x)
            // above; at q = 1/2 f takes the opposite one and g the upstream one (both are loaded)
            a.f_2 = a.g_2 = 0.0f;
            if (a.fluid1) {
                float fu, gu, fo, go;
                if (a.q <= 0.5f) {
                    ld2(fB + sl.up, sl.xs_up, wr, fu, gu);
                    a.f_2 = fu;
                    a.g_2 = gu;
                }
                if (a.q >= 0.5f) {
                    ld2(fB + sl.opp, sl.xs_opp, wr, fo, go);
                    a.f_2 = fo;
                    if (a.q > 0.5f) a.g_2 = go;
                }
            }
            a.rho = (float)__ldg(rho + a.x);
        };
        auto finish = [&](const LinkIn &a) {
            const int x = a.x, ip = a.ip;
            const float q = a.q, f_here = a.f_here, g_here = a.g_here;
            const int iz = x / (int)geo.lxy;
            const int rem = x - iz * (int)geo.lxy;
            const int iy = rem / geo.lx;
            const int ix = rem - iy * geo.lx;
            const int cxi = dcx_rt(ip), cyi = dcy_rt(ip), czi = dcz_rt(ip);
            const float wr = fweight_rt(ip), winv = finvweight_rt(ip);   // w_opp = w_ip
            // moving wall velocity at the intersection point (ibb.cu:33-46)
            const float relx = ((float)(ix - ipx) + hx) + q * (float)cxi;
            const float rely = ((float)(iy - ipy) + hy) + q * (float)cyi;
            const float relz = ((float)(iz - ipz) + hz) + q * (float)czi;
            const float uwx = vxf + (relz * wyf - rely * wzf);
            const float uwy = vyf + (relx * wzf - relz * wxf);
            const float uwz = vzf + (rely * wxf - relx * wyf);
            const float evel = (float)cxi * uwx + (float)cyi * uwy + (float)czi * uwz;
            const float mom = wr * mom_k * evel;
            const float inv_2q = (q >= 0.5f) ? 0.5f / q : 0.0f;
            float fval, gval;
            if (a.fluid1) {
                if (q < 0.5f) fval = 2.0f * q * f_here + (1.0f - 2.0f * q) * a.f_2 - mom;
                else fval = (f_here - mom) * inv_2q + (2.0f * q - 1.0f) * inv_2q * a.f_2;
            } else {
                fval = f_here - mom;
            }
            const float amp = 2.0f * wr * Tpf * (1.0f + a.rho);
            if (a.fluid1) {
                if (q <= 0.5f) gval = -(2.0f * q * g_here + (1.0f - 2.0f * q) * a.g_2) + amp;
                else gval = -g_here * inv_2q + amp * inv_2q + (2.0f * q - 1.0f) * inv_2q * a.g_2;
            } else {
                gval = -g_here + amp;
            }
            // the population that streams into x along opp from the solid node x + c_ip, in the slot
            // the next step reads as f_opp(x); one slot holds both populations (f and g buffers
            // are the same allocation)
            const LinkSlots sl = slots_of(x, ip);
            S *fs = fB + sl.out;
            float f_out = fval, g_out = gval;
            if constexpr (MODE == RBTP_STORE_F16S) {
                // the value the reference would read back is the rounded one
                const int ixs = sl.xs_out;   // the node of the written slot
                const __half2 hv = __floats2half2_rn(fval * winv, gval * winv - (tla + tlb * (float)ixs));
                *fs = hv;
                f_out = __low2float(hv) * wr;
                g_out = (__high2float(hv) + (tla + tlb * (float)ixs)) * wr;
            } else {
                *fs = make_float2(fval, gval);
            }
            // ibb.cu:160-187 (force, torque about the same intersection point) and 202-204 (heat)
            const float Fx = ((float)cxi - uwx) * f_here - ((float)-cxi - uwx) * f_out;
            const float Fy = ((float)cyi - uwy) * f_here - ((float)-cyi - uwy) * f_out;
            const float Fz = ((float)czi - uwz) * f_here - ((float)-czi - uwz) * f_out;
            add(0, Fx);
            add(1, Fy);
            add(2, Fz);
            add(3, rely * Fz - relz * Fy);
            add(4, relz * Fx - relx * Fz);
            add(5, relx * Fy - rely * Fx);
            add(6, g_here - g_out);
        };
        const int stride = pb.ibb_chunks * IBB_THREADS;
        int t = chunk * IBB_THREADS + threadIdx.x;
        for (; t + stride < n; t += 2 * stride) {
            LinkIn a, b;
            gather(t, a);
            gather(t + stride, b);
            finish(a);
            finish(b);
        }
        if (t < n) {
            LinkIn a;
            gather(t, a);
            finish(a);
        }
        // double-float block sum (FP32 pipe), one FP64 value per quantity
        block_reduce_df<7, IBB_THREADS>(sum, acc, reinterpret_cast<float *>(sh));
        if (threadIdx.x == 0) {
            double *out = pb.hpart + ((long long)p * IBB_CHUNKS + chunk) * 7;
#pragma unroll
            for (int q = 0; q < 7; ++q) out[q] = acc[q];
        }
        return;
    }
    block_reduce_fixed<7, IBB_THREADS>(acc, sh);
    if (threadIdx.x == 0) {
        double *out = pb.hpart + ((long long)p * IBB_CHUNKS + chunk) * 7;
#pragma unroll
        for (int q = 0; q < 7; ++q) out[q] = acc[q];
    }
}

template <int MODE>
__global__ void __launch_bounds__(IBB_THREADS, MODE == RBTP_STORE_F64 ? 4 : 6) k_links_ibb(const Geo geo, const Phys ph,
                                                           const PartBuffers pb, void *f_,
                                                           void *g_, const double *rho, bool odd)
{
    __shared__ double sh[7 * IBB_THREADS];
    links_ibb_body<MODE>(geo, ph, pb, f_, g_, rho, odd, blockIdx.x, blockIdx.y, sh);
}

// ------------------------------------------------------------------------------------------------
// Contacts: cell list, ascending-partner sums (pforces.cu:6-76).
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ int cell_of(double v, double cs, int n)
{
    int c = ifloor(v / cs);
    if (c < 0) c = 0;
    if (c > n - 1) c = n - 1;
    return c;
}

__device__ __forceinline__ void cell_count_body(const PartBuffers &pb, int p)
{
    const double *st = pb.state;
    const int cx = cell_of(PCOL(st, pb.np, 0, p), pb.cell_size, pb.ncell[0]);
    const int cy = cell_of(PCOL(st, pb.np, 1, p), pb.cell_size, pb.ncell[1]);
    const int cz = cell_of(PCOL(st, pb.np, 2, p), pb.cell_size, pb.ncell[2]);
    atomicAdd(&pb.cell_count[(cz * pb.ncell[1] + cy) * pb.ncell[0] + cx], 1);
}

__global__ void k_cell_count(const PartBuffers pb)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < pb.np) cell_count_body(pb, p);
}

// one block of up to 1024 threads; sequential chunks with a block scan
__device__ __forceinline__ void cell_scan_body(const PartBuffers &pb, int ncells, int *sh, int &carry)
{
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b = 0; b < ncells; b += blockDim.x) {
        const int i = b + threadIdx.x;
        const int v = i < ncells ? pb.cell_count[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < (int)blockDim.x; off <<= 1) {
            const int add = threadIdx.x >= (unsigned)off ? sh[threadIdx.x - off] : 0;
            __syncthreads();
            sh[threadIdx.x] += add;
            __syncthreads();
        }
        if (i < ncells) pb.cell_start[i] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += sh[threadIdx.x];
        __syncthreads();
    }
}

__global__ void k_cell_scan(const PartBuffers pb, int ncells)
{
    __shared__ int sh[1024];
    __shared__ int carry;
    cell_scan_body(pb, ncells, sh, carry);
}

__device__ __forceinline__ void cell_fill_body(const PartBuffers &pb, int p)
{
    const double *st = pb.state;
    const int cx = cell_of(PCOL(st, pb.np, 0, p), pb.cell_size, pb.ncell[0]);
    const int cy = cell_of(PCOL(st, pb.np, 1, p), pb.cell_size, pb.ncell[1]);
    const int cz = cell_of(PCOL(st, pb.np, 2, p), pb.cell_size, pb.ncell[2]);
    const int c = (cz * pb.ncell[1] + cy) * pb.ncell[0] + cx;
    const int slot = atomicAdd(&pb.cell_fill[c], 1);
    pb.cell_items[pb.cell_start[c] + slot] = p;
}

__global__ void k_cell_fill(const PartBuffers pb)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < pb.np) cell_fill_body(pb, p);
}

constexpr int MAX_CAND = 256;   // contact partners of one sphere (33 fit without overlap at r = 8)
// Per-particle CTAs (marking, link fill, new-fluid detection) are LINK_WIDE threads while fewer
// particles than this are in flight (4 CTAs per SM of a 152-SM GB300) and LINK_NARROW beyond; the
// results do not depend on the width.
constexpr int PARTICLES_WIDE = 4 * 152;

constexpr int CONTACT_WARPS = 4;   // particles per 128-thread CTA, one warp each

// One warp per particle: lane k < 27 scans neighbour cell k of the particle's cell, accepted
// partners are collected in shared memory, and lane 0 sorts them and adds the pair forces in
// ascending partner order (the order pforces.cu's pair loop adds them to p), then the walls.
__device__ __forceinline__ void contact_force_body(const Geo &geo, const Phys &ph,
                                                   const PartBuffers &pb, DevStatus *status, int p,
                                                   int *cand /* MAX_CAND */, int &ncand)
{
    const int lane = threadIdx.x & 31;
    const int np = pb.np;
    const double *st = pb.state;
    const double x = PCOL(st, np, 0, p), y = PCOL(st, np, 1, p), z = PCOL(st, np, 2, p);
    const double radius = ph.radius, coeff = ph.rep_coeff, min_gap = ph.min_gap;
    if (lane == 0) ncand = 0;
    __syncwarp();
    if (np > 1 && lane < 27) {
        const int cx = cell_of(x, pb.cell_size, pb.ncell[0]);
        const int cy = cell_of(y, pb.cell_size, pb.ncell[1]);
        const int cz = cell_of(z, pb.cell_size, pb.ncell[2]);
        const int kx = cx + lane % 3 - 1, ky = cy + (lane / 3) % 3 - 1, kz = cz + lane / 9 - 1;
        if (kx >= 0 && kx < pb.ncell[0] && ky >= 0 && ky < pb.ncell[1] && kz >= 0 && kz < pb.ncell[2]) {
            const int c = (kz * pb.ncell[1] + ky) * pb.ncell[0] + kx;
            const int s0 = pb.cell_start[c], s1 = s0 + pb.cell_count[c];
            for (int s = s0; s < s1; ++s) {
                const int q = pb.cell_items[s];
                if (q == p) continue;
                const double dx = dsub(x, PCOL(st, np, 0, q));
                const double dy = dsub(y, PCOL(st, np, 1, q));
                const double dz = dsub(z, PCOL(st, np, 2, q));
                const double dsq = sq3(dx, dy, dz);
                if (dsq <= 1.0e-12) continue;
                const double hgap = dsub(__dsqrt_rn(dsq), dmul(2.0, radius));
                if (hgap >= min_gap) continue;
                const int slot = atomicAdd(&ncand, 1);
                if (slot < MAX_CAND) cand[slot] = q;
            }
        }
    }
    __syncwarp();
    if (lane != 0) return;
    int nc = ncand;
    if (nc > MAX_CAND) {
        atomicOr(&status->contact_overflow, 1);
        nc = MAX_CAND;
    }
    for (int i = 1; i < nc; ++i) {
        const int v = cand[i];
        int j = i - 1;
        while (j >= 0 && cand[j] > v) { cand[j + 1] = cand[j]; --j; }
        cand[j + 1] = v;
    }
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int i = 0; i < nc; ++i) {
        const int q = cand[i];
        const double dx = dsub(x, PCOL(st, np, 0, q));
        const double dy = dsub(y, PCOL(st, np, 1, q));
        const double dz = dsub(z, PCOL(st, np, 2, q));
        const double dist = __dsqrt_rn(sq3(dx, dy, dz));
        const double hgap = dsub(dist, dmul(2.0, radius));
        const double overlap = (hgap < 0.0) ? -hgap : 0.0;
        const double factor = __ddiv_rn(dsub(min_gap, hgap), min_gap);
        const double lub = dmul(coeff, dadd(__ddiv_rn(dmul(factor, factor), ph.stf0),
                                            __ddiv_rn(overlap, dmul(min_gap, ph.stf1))));
        fx = dadd(fx, dmul(lub, __ddiv_rn(dx, dist)));
        fy = dadd(fy, dmul(lub, __ddiv_rn(dy, dist)));
        fz = dadd(fz, dmul(lub, __ddiv_rn(dz, dist)));
        if (q > p) {
            const int slot = atomicAdd(&status->ncontacts, 1);
            if (slot < pb.pair_cap) { pb.pair_p[slot] = p; pb.pair_q[slot] = q; }
        }
    }
    // walls (pforces.cu:40-76)
    double wfx = 0.0, wfy = 0.0, wfz = 0.0;
    const double gaps[6] = {dsub(x, radius), dsub(dsub((double)geo.lx, x), radius),
                            dsub(y, radius), dsub(dsub((double)geo.ly, y), radius),
                            dsub(z, radius), dsub(dsub((double)geo.lz, z), radius)};
    const double mgw = ph.min_gap_w;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const double gap = gaps[k];
        if (gap >= mgw) continue;
        const double overlap = (gap < 0.0) ? -gap : 0.0;
        const double factor = __ddiv_rn(dsub(mgw, gap), mgw);
        const double lub = dmul(coeff, dadd(__ddiv_rn(dmul(factor, factor), ph.stf0_w),
                                            __ddiv_rn(overlap, dmul(mgw, ph.stf1_w))));
        // wall normals +x, -x, +y, -y, +z, -z; the zero components add +0.0 and are skipped
        const double sgn = (k & 1) ? -1.0 : 1.0;
        if (k < 2) wfx = dadd(wfx, dmul(lub, sgn));
        else if (k < 4) wfy = dadd(wfy, dmul(lub, sgn));
        else wfz = dadd(wfz, dmul(lub, sgn));
    }
    pb.cF[p] = dadd(fx, wfx);
    pb.cF[np + p] = dadd(fy, wfy);
    pb.cF[2 * np + p] = dadd(fz, wfz);
}

__global__ void __launch_bounds__(32 * CONTACT_WARPS) k_contact_force(const Geo geo, const Phys ph,
                                                                     const PartBuffers pb, DevStatus *status)
{
    __shared__ int cand[CONTACT_WARPS][MAX_CAND];
    __shared__ int ncand[CONTACT_WARPS];
    const int w = threadIdx.x >> 5;
    const int p = blockIdx.x * CONTACT_WARPS + w;
    if (p < pb.np) contact_force_body(geo, ph, pb, status, p, cand[w], ncand[w]);
}

// ------------------------------------------------------------------------------------------------
// History shift + Newton-Euler + temperature (pforces.cu:80-116, ibb.cu:258-262, move.cu:5-103).
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ void update_body(const Phys &ph, const PartBuffers &pb, int p)
{
    const int np = pb.np;
    double *st = pb.state;
    const double dt = 1.0;
    const double buoyancy = (1.0 - 1.0 / ph.rho_ratio) * ph.grav0;
    // this step's hydrodynamic force, torque and heat: the link-chunk partial sums in chunk order
    double h[7] = {0, 0, 0, 0, 0, 0, 0};
    const double *part = pb.hpart + (long long)p * IBB_CHUNKS * 7;
    for (int c = 0; c < pb.ibb_chunks; ++c)
#pragma unroll
        for (int q = 0; q < 7; ++q) h[q] += part[c * 7 + q];
    // every column is read before any is written (the loads need not wait on the stores)
    double col[33];
#pragma unroll
    for (int c = 0; c < 33; ++c) col[c] = PCOL(st, np, c, p);
    double cf[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) cf[a] = pb.cF[a * np + p];
    double out[33];
#pragma unroll
    for (int c = 0; c < 33; ++c) out[c] = col[c];
    double vn[3], on[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // force / torque histories: prev2 <- prev, prev <- accum, accum <- this step's sums
        const double f_prev = col[6 + a], f_prev2 = col[9 + a];
        const double t_prev = col[21 + a], t_prev2 = col[24 + a];
        const double f_now = cf[a] + h[a];
        const double t_now = h[3 + a];
        out[12 + a] = f_prev2;
        out[9 + a] = f_prev;
        out[6 + a] = f_now;
        out[27 + a] = t_prev2;
        out[24 + a] = t_prev;
        out[21 + a] = t_now;
        const double combo_f = 0.5 * f_now + f_prev + 0.5 * f_prev2;
        const double combo_t = 0.5 * t_now + t_prev + 0.5 * t_prev2;
        vn[a] = col[3 + a] + 0.5 * dt * combo_f / ph.mass;
        if (a == 0) vn[a] += dt * buoyancy;
        on[a] = col[18 + a] + 0.5 * dt * combo_t / ph.inertia;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        out[a] = col[a] + 0.5 * dt * (vn[a] + col[3 + a]);
        out[15 + a] = col[15 + a] + 0.5 * dt * (on[a] + col[18 + a]);
        out[3 + a] = vn[a];
        out[18 + a] = on[a];
    }
    const double heat_prev = col[31];
    const double heat = h[6];
    out[32] = heat_prev;
    out[31] = heat;
    out[30] = col[30] + 0.5 * dt * (heat + heat_prev) / ph.heat_cap;
#pragma unroll
    for (int c = 0; c < 33; ++c) PCOL(st, np, c, p) = out[c];
}

// The integrator, followed by the geometry cache of the new position (same thread, same particle),
// so the link build that follows needs no separate k_pgeo launch.
__global__ void k_update(const Geo geo, const Phys ph, const PartBuffers pb)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < pb.np) {
        update_body(ph, pb, p);
        pgeo_body(geo, ph, pb, p);
    }
}

// ------------------------------------------------------------------------------------------------
// Solid marking over all particles (links.cu:25-48, 160-188).
// ------------------------------------------------------------------------------------------------
template <int NT>
__device__ __forceinline__ void mark_body(const Geo &geo, const Phys &ph, const PartBuffers &pb, int *owner, int p,
                                          ShellRows<NT> &sr)
{
    const PGeo &pg = pb.pgeo[p];
    const Box b = pgeo_box(pg.mbox);
    if (b.x0 > b.x1 || b.y0 > b.y1 || b.z0 > b.z1) return;
    // Single-precision classification away from the surface, the exact FP64 predicate in a band
    // around it (PGeo::band bounds the float error), so every node is classified exactly as the
    // FP64 test classifies it.
    const float pxf = pg.c[0], pyf = pg.c[1], pzf = pg.c[2], rf2 = pg.rf2, band = pg.band;
    // the ball |x - X|^2 <= r^2 + band (plus a margin for the row arithmetic)
    for_shell_nodes<NT>(sr, b, pxf, pyf, pzf, 0.0f, sqrtf(rf2 + band) + 0.01f, [&](int ix, int iy, int iz) {
        const float fx = ((float)ix + 0.5f) - pxf, fy = ((float)iy + 0.5f) - pyf, fz = ((float)iz + 0.5f) - pzf;
        const float d2 = fx * fx + fy * fy + fz * fz;
        if (d2 > rf2 + band) return;
        if (d2 >= rf2 - band) {
            const double *st = pb.state;
            const double px = PCOL(st, pb.np, 0, p), py = PCOL(st, pb.np, 1, p), pz = PCOL(st, pb.np, 2, p);
            const double dx = dsub((double)ix + 0.5, px);
            const double dy = dsub((double)iy + 0.5, py);
            const double dz = dsub((double)iz + 0.5, pz);
            if (sq3(dx, dy, dz) > dmul(ph.radius, ph.radius)) return;
        }
        const long long idx = (long long)iz * geo.lxy + (long long)iy * geo.lx + ix;
        atomicMin(reinterpret_cast<unsigned int *>(owner) + idx, (unsigned int)p);
    });
}

__global__ void k_pgeo(const Geo geo, const Phys ph, const PartBuffers pb)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < pb.np) pgeo_body(geo, ph, pb, p);
}

template <int NT>
__global__ void __launch_bounds__(NT) k_mark(const Geo geo, const Phys ph, const PartBuffers pb, int *owner)
{
    __shared__ ShellRows<NT> sr;
    mark_body<NT>(geo, ph, pb, owner, blockIdx.x, sr);
}

// ------------------------------------------------------------------------------------------------
// Link slabs (links.cu:50-139): CTA per particle, ordered compaction over its padded box.
// Phase 1 (integer work only): every fluid node of the box within r + 2 of the centre reads the
// owners of its 26 neighbours and marks the directions whose neighbour this particle owns (a 27-bit
// mask per node); an exclusive scan of the mask popcounts numbers the candidates (node, direction)
// in node-then-direction order.  Phase 2: candidate k is located by a binary search over the scan
// and a bit select in its node's mask, the ray-sphere q of links.cu:7-23 runs with all lanes busy,
// and candidate k goes to slab entry base + k, so the slab holds the links in the reference's
// (idx, ip) order (links.cu:221-250).  A candidate whose ray-sphere test fails (a grazing ray
// rounded off the sphere) is rare; one block vote per chunk finds the chunks that hold one, and
// only those are redone with an order-preserving compaction (block scans).  Only the spherical shell that can hold link nodes is
// enumerated: per (y, z) row of the box, the x-intervals between an inner radius (nodes inside it
// are certainly solid) and the outer reach r + 2, with float margins so that every possible link
// node is kept; rows are numbered by a block scan and flat indices are mapped back by a binary
// search, so nodes are visited in ascending index order.  The same owner reads give, per link,
// whether the upstream node x - c_ip is an in-domain fluid node (the interpolating branch of
// ibb.cu:52-73 / 114-128); it is stored in bit LINK_UP of the direction word so that the IBB pass
// needs no flag gather.
// ------------------------------------------------------------------------------------------------
// CTA size: 512 threads when few particles are in flight (the per-particle chain is the latency),
// 128 when many are (more particles per SM); the links are identical either way.
constexpr int LINK_WIDE = 512, LINK_NARROW = 128;

// Shared scratch of one link-fill CTA.
template <int NT>
struct LinkShared {
    ShellRows<NT> rows;       // shell table (its wsum also serves the chunk scans)
    unsigned mask[NT];        // candidate directions of each chunk node (bit ip)
    unsigned up[NT];          // directions whose neighbour is in-domain fluid (bit ip)
    int scan[NT];             // exclusive prefix of the popcounts
    int node[NT];             // lattice index of each chunk node
};

template <bool F32Q, int NT>
__device__ __forceinline__ void link_fill_body(const Geo &geo, const Phys &ph, const PartBuffers &pb,
                                               const int *owner, DevStatus *status, int p, LinkShared<NT> &sm)
{
    const PGeo &pg = pb.pgeo[p];
    const float r = (float)ph.radius;
    const Box b = pgeo_box(pg.lbox);
    const long long slab = (long long)p * pb.link_cap;
    if (b.x0 > b.x1 || b.y0 > b.y1 || b.z0 > b.z1) {
        if (threadIdx.x == 0) pb.link_cnt[p] = 0;
        return;
    }
    const int nx = b.x1 - b.x0 + 1, ny = b.y1 - b.y0 + 1, nz = b.z1 - b.z0 + 1;
    // conservative single-precision shell test: a link needs |x - X| <= r + sqrt(3)
    const float reach = r + 2.0f;
    const float reach2 = reach * reach;
    const float pxf = pg.c[0], pyf = pg.c[1], pzf = pg.c[2];
    // exact node-centre offsets for the float q: integer part of the centre and its fraction
    const int ipx = pg.ic[0], ipy = pg.ic[1], ipz = pg.ic[2];
    const float hx = pg.h[0], hy = pg.h[1], hz = pg.h[2];
    const int lx = geo.lx, lxy = (int)geo.lxy;
    // shell |x - X| in [r_in, r_out]: nodes closer than r_in are inside the sphere (solid)
    int total = shell_rows_build<NT>(sm.rows, b, pxf, pyf, pzf, fmaxf(r - 0.05f, 0.0f), reach + 0.01f);
    const bool use_rows = total >= 0;
    if (!use_rows) total = nx * ny * nz;
    int base = 0;
    for (int c0 = 0; c0 < total; c0 += NT) {
        const int t = c0 + threadIdx.x;
        unsigned mask = 0, up = 0;
        int my_node = 0;
        if (t < total) {
            int ix, iy, iz;
            if (use_rows) {
                shell_rows_node<NT>(sm.rows, b, t, ix, iy, iz);
            } else {
                const int lz = t / (nx * ny);
                const int rem = t - lz * nx * ny;
                const int ly = rem / nx;
                ix = b.x0 + (rem - ly * nx);
                iy = b.y0 + ly;
                iz = b.z0 + lz;
            }
            const float ddx = ((float)ix + 0.5f) - pxf, ddy = ((float)iy + 0.5f) - pyf,
                        ddz = ((float)iz + 0.5f) - pzf;
            const long long idx = (long long)iz * geo.lxy + (long long)iy * geo.lx + ix;
            const int *on = owner + idx;
            if (ddx * ddx + ddy * ddy + ddz * ddz <= reach2 && __ldg(on) < 0) {
                if (ix > 0 && ix < geo.lx - 1 && iy > 0 && iy < geo.ly - 1 && iz > 0 && iz < geo.lz - 1) {
                    // interior node: all 26 neighbours are in the domain
                    unroll<26>([&](auto K) {
                        constexpr int ip = decltype(K)::value + 1;
                        const int o = __ldg(on + (dcx(ip) + dcy(ip) * lx + dcz(ip) * lxy));
                        if (o == p) mask |= 1u << ip;
                        if (o < 0) up |= 1u << ip;
                    });
                } else {
                    unroll<26>([&](auto K) {
                        constexpr int ip = decltype(K)::value + 1;
                        constexpr int cx = dcx(ip), cy = dcy(ip), cz = dcz(ip);
                        const int xn = ix + cx, yn = iy + cy, zn = iz + cz;
                        if (xn >= 0 && xn < geo.lx && yn >= 0 && yn < geo.ly && zn >= 0 && zn < geo.lz) {
                            const int o = __ldg(on + (cx + cy * lx + cz * lxy));
                            if (o == p) mask |= 1u << ip;
                            if (o < 0) up |= 1u << ip;
                        }
                    });
                }
            }
            my_node = (int)idx;
        }
        int ccount;
        const int pos = block_exclusive_scan<NT>(__popc(mask), sm.rows.wsum, ccount);
        sm.mask[threadIdx.x] = mask;
        sm.up[threadIdx.x] = up;
        sm.scan[threadIdx.x] = pos;
        sm.node[threadIdx.x] = my_node;
        __syncthreads();
        // phase 2: q for the numbered candidates.  Candidate k is written to slab entry base + k;
        // a chunk holding a ray that failed the ray-sphere test (rare: a grazing ray rounded off
        // the surface) is redone with an order-preserving compaction.
        auto candidate = [&](int k, int &node, int &dw, double &q) -> bool {
            // the chunk thread j holding candidate k: the last j with scan[j] <= k
            int lo = 0, hi = NT - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (sm.scan[mid] <= k) lo = mid;
                else hi = mid - 1;
            }
            const int ip = (int)__fns(sm.mask[lo], 0u, k - sm.scan[lo] + 1);
            node = sm.node[lo];
            dw = ip | (int)(((sm.up[lo] >> dopp_rt(ip)) & 1u) << LINK_UP);
            const int iz = node / lxy;
            const int iy = (node - iz * lxy) / lx;
            const int ix = node - iz * lxy - iy * lx;
            int r32 = -1;
            if constexpr (F32Q)
                r32 = link_q_f32(dcx_rt(ip), dcy_rt(ip), dcz_rt(ip), (float)(ix - ipx) + hx,
                                 (float)(iy - ipy) + hy, (float)(iz - ipz) + hz, pg.rf2, q);
            if (r32 > 0) return true;
            const double *st = pb.state;
            return link_q(dcx_rt(ip), dcy_rt(ip), dcz_rt(ip), (double)ix + 0.5, (double)iy + 0.5,
                          (double)iz + 0.5, PCOL(st, pb.np, 0, p), PCOL(st, pb.np, 1, p),
                          PCOL(st, pb.np, 2, p), dmul(ph.radius, ph.radius), q);
        };
        auto put = [&](int pos, int node, int dw, double q) {
            if (pos < pb.link_cap) {
                pb.link_node[slab + pos] = node;
                pb.link_dir[slab + pos] = dw;
                pb.link_q[slab + pos] = q;
            }
        };
        int rejected = 0;
        for (int k = threadIdx.x; k < ccount; k += NT) {
            int node, dw;
            double q = 0.0;
            if (candidate(k, node, dw, q)) put(base + k, node, dw, q);
            else rejected = 1;
        }
        if (__syncthreads_or(rejected)) {
            for (int k0 = 0; k0 < ccount; k0 += NT) {
                const int k = k0 + threadIdx.x;
                int node = 0, dw = 0, ok = 0;
                double q = 0.0;
                if (k < ccount) ok = candidate(k, node, dw, q) ? 1 : 0;
                int ltotal;
                const int lpos = base + block_exclusive_scan<NT>(ok, sm.rows.wsum, ltotal);
                if (ok) put(lpos, node, dw, q);
                base += ltotal;
            }
        } else {
            base += ccount;
        }
        if (base > pb.link_cap && threadIdx.x == 0) atomicOr(&status->link_overflow, 1);
        __syncthreads();
    }
    if (threadIdx.x == 0) pb.link_cnt[p] = base;
}

template <bool F32Q, int NT>
__global__ void __launch_bounds__(NT) k_link_fill(const Geo geo, const Phys ph, const PartBuffers pb,
                                                  const int *owner, DevStatus *status)
{
    __shared__ LinkShared<NT> sm;
    link_fill_body<F32Q, NT>(geo, ph, pb, owner, status, blockIdx.x, sm);
}

// ------------------------------------------------------------------------------------------------
// New-fluid detection (refill.cu:8-76), per particle around its new position.
// ------------------------------------------------------------------------------------------------
template <int NT>
__device__ __forceinline__ void new_fluid_body(const Geo &geo, const Phys &ph, const PartBuffers &pb,
                                               const int *owner_prev, const int *owner_cur,
                                               DevStatus *status, int p, ShellRows<NT> &sr)
{
    const PGeo &pg = pb.pgeo[p];
    const Box b = pgeo_box(pg.nbox);
    if (b.x0 > b.x1 || b.y0 > b.y1 || b.z0 > b.z1) return;
    const float rf = (float)ph.radius;
    // candidates are fluid now (outside the sphere: nodes closer than r - 0.05 are solid) and
    // within NEW_FLUID_THRESH of its surface
    for_shell_nodes<NT>(sr, b, pg.c[0], pg.c[1], pg.c[2], fmaxf(rf - 0.05f, 0.0f),
                        rf + (float)NEW_FLUID_THRESH + 0.01f, [&](int ix, int iy, int iz) {
        const long long idx = (long long)iz * geo.lxy + (long long)iy * geo.lx + ix;
        if (owner_prev[idx] != p || owner_cur[idx] >= 0) return;
        const double *st = pb.state;
        const double px = PCOL(st, pb.np, 0, p), py = PCOL(st, pb.np, 1, p), pz = PCOL(st, pb.np, 2, p);
        const double r = ph.radius;
        const double dx = dsub((double)ix + 0.5, px);
        const double dy = dsub((double)iy + 0.5, py);
        const double dz = dsub((double)iz + 0.5, pz);
        const double dist = __dsqrt_rn(sq3(dx, dy, dz));
        if (dsub(dist, r) > NEW_FLUID_THRESH) return;
        const int slot = atomicAdd(&status->nf_count, 1);
        if (slot < pb.nf_cap) { pb.nf_node[slot] = (int)idx; pb.nf_pid[slot] = p; }
        else atomicOr(&status->nf_overflow, 1);
    });
}

template <int NT>
__global__ void __launch_bounds__(NT) k_new_fluid(const Geo geo, const Phys ph, const PartBuffers pb,
                                                  const int *owner_prev, const int *owner_cur, DevStatus *status)
{
    __shared__ ShellRows<NT> sr;
    new_fluid_body<NT>(geo, ph, pb, owner_prev, owner_cur, status, blockIdx.x, sr);
}

// Refill values (refill.cu:78-240): one warp per new-fluid node, lane ip computes population ip
// from the post-collision populations f*_ip of previous-step fluid neighbours, as the step of the
// given parity left them in the AA storage: after an even step in slot (opp(ip), n); after an odd
// step in slot (ip, n + c_ip), or, where n + c_ip is outside the box, as the wall-processed
// population in slot (opp(ip), n) (bounce-back: f*_ip itself; the Dirichlet image of g*_ip at a pure
// x exit is inverted with the step's density at n, which the step kernel wrote to rho).
template <int MODE>
__device__ __forceinline__ void refill_compute_body(const Geo &geo, const Phys &ph, const PartBuffers &pb,
                                                    const int *owner_prev, const void *f_, const void *g_,
                                                    const double *rho, bool odd, const DevStatus *status,
                                                    int warp0, int nwarps)
{
    using ST = Store<MODE>;
    using S = typename ST::S;
    const S *fB = static_cast<const S *>(f_);
    const S *gB = static_cast<const S *>(g_);
    const int lane = threadIdx.x & 31;
    const int count = min(status->nf_count, pb.nf_cap);
    const long long L = geo.L;
    const double RT = 1.0 / 3.0;
    const double lambda0 = 1.0 - dweight(0);
    for (int n = warp0; n < count; n += nwarps) {
        const int idx = pb.nf_node[n];
        const int iz = idx / (int)geo.lxy;
        const int iy = (idx - iz * (int)geo.lxy) / geo.lx;
        const int ix = idx - iz * (int)geo.lxy - iy * geo.lx;
        int pid = pb.nf_pid[n];
        if (pid < 0) {
            const int pp = owner_prev[idx];
            if (pp >= 0) pid = pp;
        }
        double fv = 0.0, gv = 0.0;
        if (lane < 27) {
            const int ip = lane;
            const double w = dweight_rt(ip);
            const int cxp = dcx_rt(ip), cyp = dcy_rt(ip), czp = dcz_rt(ip), op = dopp_rt(ip);
            // f*_ip and g*_ip of the previous-step fluid node n = (xn, yn, zn)
            auto collided = [&](long long n, int xn, int yn, int zn, double &fo, double &go) {
                if (!odd) {
                    const long long sl = (long long)op * L + n;
                    fo = (double)ST::ld_f(fB + sl, w, ph.t0);
                    go = (double)ST::ld_g(gB + sl, w, gshift(ph, xn));
                    return;
                }
                const int xd = xn + cxp, yd = yn + cyp, zd = zn + czp;
                if (xd >= 0 && xd < geo.lx && yd >= 0 && yd < geo.ly && zd >= 0 && zd < geo.lz) {
                    const long long sl = (long long)ip * L + (long long)zd * geo.lxy + (long long)yd * geo.lx + xd;
                    fo = (double)ST::ld_f(fB + sl, w, ph.t0);
                    go = (double)ST::ld_g(gB + sl, w, gshift(ph, xd));
                    return;
                }
                const long long sl = (long long)op * L + n;
                fo = (double)ST::ld_f(fB + sl, w, ph.t0);
                go = (double)ST::ld_g(gB + sl, w, gshift(ph, xn));
                const bool ox = xd < 0 || xd >= geo.lx, oyz = yd < 0 || yd >= geo.ly || zd < 0 || zd >= geo.lz;
                if (ox && !oyz) go = wall_image(go, w, xd < 0 ? ph.thot : ph.tcold, rho[n]);
            };
            double tf = 0.0, tg = 0.0;
            int sc = 0;
            for (int ip2 = 1; ip2 < 27; ++ip2) {
                const int cx2 = dcx_rt(ip2), cy2 = dcy_rt(ip2), cz2 = dcz_rt(ip2);
                const int x1 = ix + cx2, y1 = iy + cy2, z1 = iz + cz2;
                if (x1 < 0 || x1 >= geo.lx || y1 < 0 || y1 >= geo.ly || z1 < 0 || z1 >= geo.lz) continue;
                const long long i1 = (long long)z1 * geo.lxy + (long long)y1 * geo.lx + x1;
                if (owner_prev[i1] >= 0) continue;
                const int x2 = ix + 2 * cx2, y2 = iy + 2 * cy2, z2 = iz + 2 * cz2;
                const bool in2 = x2 >= 0 && x2 < geo.lx && y2 >= 0 && y2 < geo.ly && z2 >= 0 && z2 < geo.lz;
                double f1, g1;
                collided(i1, x1, y1, z1, f1, g1);
                if (in2) {
                    const long long i2 = (long long)z2 * geo.lxy + (long long)y2 * geo.lx + x2;
                    if (owner_prev[i2] < 0) {
                        double f2, g2;
                        collided(i2, x2, y2, z2, f2, g2);
                        tf += 2.0 * f1 - f2;
                        tg += 2.0 * g1 - g2;
                        ++sc;
                        continue;
                    }
                }
                tf += f1;
                tg += g1;
                ++sc;
            }
            if (sc == 0) {
                double px = 0, py = 0, pz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
                double tT = ph.t0;
                const double *st = pb.state;
                if (pid >= 0) {
                    px = PCOL(st, pb.np, 0, pid); py = PCOL(st, pb.np, 1, pid); pz = PCOL(st, pb.np, 2, pid);
                    vx = PCOL(st, pb.np, 3, pid); vy = PCOL(st, pb.np, 4, pid); vz = PCOL(st, pb.np, 5, pid);
                    wx = PCOL(st, pb.np, 18, pid); wy = PCOL(st, pb.np, 19, pid); wz = PCOL(st, pb.np, 20, pid);
                    tT = PCOL(st, pb.np, 30, pid);
                }
                const double relx = ((double)ix + 0.5) - px;
                const double rely = ((double)iy + 0.5) - py;
                const double relz = ((double)iz + 0.5) - pz;
                double u = vx + (relz * wy - rely * wz);
                double v = vy + (relx * wz - relz * wx);
                double ww = vz + (rely * wx - relx * wy);
                if (pid < 0) { u = 0.0; v = 0.0; ww = 0.0; }
                const double r = ph.rho0;
                // refill.cu:196-201: eu is c.u without the 1/RT factor
                const double eu = dcx_rt(ip) * u + dcy_rt(ip) * v + dcz_rt(ip) * ww;
                const double uv = (u * u + v * v + ww * ww) / RT;
                tf = w * (r + eu + 0.5 * (eu * eu - uv));
                tg = w * tT * (1.0 + eu + 0.5 * (eu * eu - uv));
                if (ip == 0) tg -= lambda0 * tT * r;
                else tg += w * tT * r;
                sc = 1;
            }
            const double inv = 1.0 / (double)sc;
            fv = tf * inv;
            gv = tg * inv;
            pb.nf_val[(long long)n * 54 + ip] = fv;
            pb.nf_val[(long long)n * 54 + 27 + ip] = gv;
        }
        // node macros in population order (refill.cu:226-239), lane 0
        double rho_loc = 0, mx = 0, my = 0, mz = 0, phi_loc = 0;
        for (int ip = 0; ip < 27; ++ip) {
            const double a = __shfl_sync(0xffffffffu, fv, ip);
            const double c = __shfl_sync(0xffffffffu, gv, ip);
            rho_loc += a;
            mx += dcx_rt(ip) * a;
            my += dcy_rt(ip) * a;
            mz += dcz_rt(ip) * a;
            phi_loc += c;
        }
        if (lane == 0) {
            double *m = pb.nf_mac + (long long)n * 5;
            m[0] = rho_loc;
            if (rho_loc > 1e-12) {
                const double inv_rho = 1.0 / rho_loc;
                m[1] = mx * inv_rho; m[2] = my * inv_rho; m[3] = mz * inv_rho;
            } else {
                m[1] = 0.0; m[2] = 0.0; m[3] = 0.0;
            }
            m[4] = phi_loc;
        }
    }
}

template <int MODE>
__global__ void k_refill_compute(const Geo geo, const Phys ph, const PartBuffers pb,
                                 const int *owner_prev, const void *f_, const void *g_, const double *rho,
                                 bool odd, const DevStatus *status)
{
    refill_compute_body<MODE>(geo, ph, pb, owner_prev, f_, g_, rho, odd, status,
                              (blockIdx.x * blockDim.x + threadIdx.x) >> 5, (gridDim.x * blockDim.x) >> 5);
}

// Scatter the refill values, the post-streaming populations of each new-fluid node, into the
// slots the next step reads: after an odd step the node's natural slots (the next, even, step reads
// them as they are); after an even step the slots the next (odd) step gathers, (opp(ip), v - c_ip),
// or, where v - c_ip is outside the box, (ip, v) holding the preimage of the wall rule the gather
// applies.
template <int MODE>
__device__ __forceinline__ void refill_scatter_body(const Geo &geo, const Phys &ph, const PartBuffers &pb,
                                                    void *f_, void *g_, void *faux,
                                                    const double *rho_wall, bool macros, double *rho,
                                                    double *ux, double *uy, double *uz, double *phi,
                                                    const DevStatus *status, bool odd, long long t0,
                                                    long long stride)
{
    using ST = Store<MODE>;
    using S = typename ST::S;
    using R = typename ST::R;
    S *fB = static_cast<S *>(f_);
    S *gB = static_cast<S *>(g_);
    const int count = min(status->nf_count, pb.nf_cap);
    const long long L = geo.L;
    const long long total = (long long)count * 27;
    for (long long t = t0; t < total; t += stride) {
        const int n = (int)(t / 27);
        const int ip = (int)(t - (long long)n * 27);
        const int idx = pb.nf_node[n];
        const int iz = idx / (int)geo.lxy;
        const int iy = (idx - iz * (int)geo.lxy) / geo.lx;
        const int ix = idx - iz * (int)geo.lxy - iy * geo.lx;
        const int cx = dcx_rt(ip), cy = dcy_rt(ip), cz = dcz_rt(ip), o = dopp_rt(ip);
        const double w = dweight_rt(ip);
        const double fv = pb.nf_val[(long long)n * 54 + ip];
        const double gv = pb.nf_val[(long long)n * 54 + 27 + ip];
        const bool ox = (cx == 1 && ix == 0) || (cx == -1 && ix == geo.lx - 1);
        const bool oy = (cy == 1 && iy == 0) || (cy == -1 && iy == geo.ly - 1);
        const bool oz = (cz == 1 && iz == 0) || (cz == -1 && iz == geo.lz - 1);
        if (odd) {
            ST::st_f(fB + (long long)ip * L + idx, (R)fv, w, ph.t0);
            ST::st_g(gB + (long long)ip * L + idx, (R)gv, w, gshift(ph, ix));
        } else if (!(ox || oy || oz)) {
            const long long src = (long long)idx - cx - (long long)cy * geo.lx - (long long)cz * geo.lxy;
            ST::st_f(fB + (long long)o * L + src, (R)fv, w, ph.t0);
            ST::st_g(gB + (long long)o * L + src, (R)gv, w, gshift(ph, ix - cx));
        } else {
            ST::st_f(fB + (long long)ip * L + idx, (R)fv, w, ph.t0);
            double gs = gv;
            if (ox && !oy && !oz) {
                // the gather applies g <- -stored + 2 w T_wall (1 + rho_wall); store its preimage
                const double tw = (cx == 1) ? ph.thot : ph.tcold;
                const long long ws = (long long)iz * geo.ly + iy + (cx == 1 ? 0 : (long long)geo.lz * geo.ly);
                gs = wall_image(gv, w, tw, rho_wall[ws]);
            }
            ST::st_g(gB + (long long)ip * L + idx, (R)gs, w, gshift(ph, ix));
        }
        if (ip == 0) {
            static_cast<typename Store<MODE>::A *>(faux)[idx] = 0;
            if (macros) {
                const double *m = pb.nf_mac + (long long)n * 5;
                rho[idx] = m[0]; ux[idx] = m[1]; uy[idx] = m[2]; uz[idx] = m[3]; phi[idx] = m[4];
            }
        }
    }
}

template <int MODE>
__global__ void k_refill_scatter(const Geo geo, const Phys ph, const PartBuffers pb, void *f_,
                                 void *g_, void *faux, const double *rho_wall, bool macros,
                                 double *rho, double *ux, double *uy, double *uz, double *phi,
                                 const DevStatus *status, bool odd)
{
    refill_scatter_body<MODE>(geo, ph, pb, f_, g_, faux, rho_wall, macros, rho, ux, uy, uz, phi, status, odd,
                              (long long)blockIdx.x * blockDim.x + threadIdx.x,
                              (long long)gridDim.x * blockDim.x);
}

}  // namespace

#define RBTP_MODE_DISPATCH(mode, CALL)                                      \
    switch (mode) {                                                         \
    case RBTP_STORE_F64: { constexpr int M = RBTP_STORE_F64; CALL; break; }  \
    case RBTP_STORE_F32: { constexpr int M = RBTP_STORE_F32; CALL; break; }  \
    case RBTP_STORE_F16S: { constexpr int M = RBTP_STORE_F16S; CALL; break; } \
    default: return cudaErrorInvalidValue;                                  \
    }

cudaError_t launch_links_ibb(int mode, const Geo &geo, const Phys &ph, const PartBuffers &pb,
                             void *f, void *g, const double *rho, bool odd, cudaStream_t st)
{
    if (pb.np <= 0) return cudaSuccess;
    RBTP_MODE_DISPATCH(mode, (k_links_ibb<M><<<dim3(pb.np, pb.ibb_chunks), IBB_THREADS, 0, st>>>(geo, ph, pb, f, g, rho, odd)));
    return cudaGetLastError();
}

cudaError_t launch_contacts(const Geo &geo, const Phys &ph, const PartBuffers &pb,
                            DevStatus *status, cudaStream_t st)
{
    if (pb.np <= 0) return cudaSuccess;
    const int ncells = pb.ncell[0] * pb.ncell[1] * pb.ncell[2];
    cudaError_t e;
    if ((e = cudaMemsetAsync(pb.cell_count, 0, sizeof(int) * ncells, st))) return e;
    if ((e = cudaMemsetAsync(pb.cell_fill, 0, sizeof(int) * ncells, st))) return e;
    if ((e = cudaMemsetAsync(&status->ncontacts, 0, sizeof(int), st))) return e;
    const int t = 128, bl = (pb.np + t - 1) / t;
    k_cell_count<<<bl, t, 0, st>>>(pb);
    k_cell_scan<<<1, 1024, 0, st>>>(pb, ncells);
    k_cell_fill<<<bl, t, 0, st>>>(pb);
    k_contact_force<<<(pb.np + CONTACT_WARPS - 1) / CONTACT_WARPS, 32 * CONTACT_WARPS, 0, st>>>(geo, ph, pb, status);
    return cudaGetLastError();
}

cudaError_t launch_update(const Geo &geo, const Phys &ph, const PartBuffers &pb, cudaStream_t st)
{
    if (pb.np <= 0) return cudaSuccess;
    k_update<<<(pb.np + 127) / 128, 128, 0, st>>>(geo, ph, pb);
    return cudaGetLastError();
}

cudaError_t launch_mark(const Geo &geo, const Phys &ph, const PartBuffers &pb, int *owner_out,
                        cudaStream_t st, bool pgeo)
{
    cudaError_t e = cudaMemsetAsync(owner_out, 0xFF, sizeof(int) * (size_t)geo.L, st);
    if (e) return e;
    if (pb.np <= 0) return cudaSuccess;
    if (pgeo) k_pgeo<<<(pb.np + 127) / 128, 128, 0, st>>>(geo, ph, pb);
    if (pb.np < PARTICLES_WIDE) k_mark<LINK_WIDE><<<pb.np, LINK_WIDE, 0, st>>>(geo, ph, pb, owner_out);
    else k_mark<LINK_NARROW><<<pb.np, LINK_NARROW, 0, st>>>(geo, ph, pb, owner_out);
    return cudaGetLastError();
}

cudaError_t launch_link_fill(int mode, const Geo &geo, const Phys &ph, const PartBuffers &pb,
                             const int *owner, DevStatus *status, cudaStream_t st)
{
    if (pb.np <= 0) return cudaSuccess;
    const bool wide = pb.np < PARTICLES_WIDE;
    if (mode == RBTP_STORE_F64) {
        if (wide) k_link_fill<false, LINK_WIDE><<<pb.np, LINK_WIDE, 0, st>>>(geo, ph, pb, owner, status);
        else k_link_fill<false, LINK_NARROW><<<pb.np, LINK_NARROW, 0, st>>>(geo, ph, pb, owner, status);
    } else {
        if (wide) k_link_fill<true, LINK_WIDE><<<pb.np, LINK_WIDE, 0, st>>>(geo, ph, pb, owner, status);
        else k_link_fill<true, LINK_NARROW><<<pb.np, LINK_NARROW, 0, st>>>(geo, ph, pb, owner, status);
    }
    return cudaGetLastError();
}

cudaError_t launch_refill(int mode, const Geo &geo, const Phys &ph, const PartBuffers &pb,
                          const int *owner_prev, const int *owner_cur, void *f, void *g,
                          void *faux, const double *rho_wall, bool macros, double *rho,
                          double *ux, double *uy, double *uz, double *phi, DevStatus *status,
                          bool odd, cudaStream_t st)
{
    if (pb.np <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(&status->nf_count, 0, sizeof(int), st);
    if (e) return e;
    if (pb.np < PARTICLES_WIDE)
        k_new_fluid<LINK_WIDE><<<pb.np, LINK_WIDE, 0, st>>>(geo, ph, pb, owner_prev, owner_cur, status);
    else
        k_new_fluid<LINK_NARROW><<<pb.np, LINK_NARROW, 0, st>>>(geo, ph, pb, owner_prev, owner_cur, status);
    RBTP_MODE_DISPATCH(mode, (k_refill_compute<M><<<152, 256, 0, st>>>(geo, ph, pb, owner_prev, f, g, rho, odd, status)));
    RBTP_MODE_DISPATCH(mode, (k_refill_scatter<M><<<152, 256, 0, st>>>(geo, ph, pb, f, g, faux, rho_wall, macros, rho, ux, uy, uz, phi, status, odd)));
    return cudaGetLastError();
}

// =================================================================================================
// Batched particle pipeline: the same per-particle bodies, with (cavity, particle) taken from a
// packed particle map and each cavity's buffers and step state from its device descriptor.  They
// run after the step kernel and before the advance kernel: the parity of the step just taken is
// the descriptor's phase (PHASE_SWAPPED: odd), the solid flags of the previous build are in
// owner[ocur] and the new ones go to owner[ocur ^ 1].
// =================================================================================================
namespace {

template <int MODE>
__global__ void __launch_bounds__(IBB_THREADS, MODE == RBTP_STORE_F64 ? 4 : 6) k_links_ibb_b(const CavDesc *desc, const int2 *pmap, const int2 *cmap)
{
    pdl_wait();
    pdl_trigger();
    __shared__ double sh[7 * IBB_THREADS];
    const int2 cm = cmap[blockIdx.x];   // (particle map entry, link chunk)
    const int2 mp = pmap[cm.x];
    const CavDesc &d = desc[mp.x];
    if (d.out == OUT_IDLE) return;
    links_ibb_body<MODE>(d.geo, d.ph, d.pb, d.f, d.g, d.rho, d.phase == PHASE_SWAPPED, mp.y, cm.y, sh);
}

__global__ void k_cells_zero_b(const CavDesc *desc, const int *pmem)
{
    pdl_wait();
    pdl_trigger();
    const CavDesc &d = desc[pmem[blockIdx.y]];
    if (d.out == OUT_IDLE) return;
    const int n = d.pb.ncell[0] * d.pb.ncell[1] * d.pb.ncell[2];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        d.pb.cell_count[c] = 0;
        d.pb.cell_fill[c] = 0;
    }
}

__global__ void k_cell_count_b(const CavDesc *desc, const int2 *pmap, int total)
{
    pdl_wait();
    pdl_trigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const int2 mp = pmap[g];
    if (desc[mp.x].out == OUT_IDLE) return;
    cell_count_body(desc[mp.x].pb, mp.y);
}

__global__ void k_cell_scan_b(const CavDesc *desc, const int *pmem)
{
    pdl_wait();
    pdl_trigger();
    __shared__ int sh[1024];
    __shared__ int carry;
    const CavDesc &d = desc[pmem[blockIdx.x]];
    if (d.out == OUT_IDLE) return;
    cell_scan_body(d.pb, d.pb.ncell[0] * d.pb.ncell[1] * d.pb.ncell[2], sh, carry);
}

__global__ void k_cell_fill_b(const CavDesc *desc, const int2 *pmap, int total)
{
    pdl_wait();
    pdl_trigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const int2 mp = pmap[g];
    if (desc[mp.x].out == OUT_IDLE) return;
    cell_fill_body(desc[mp.x].pb, mp.y);
}

__global__ void __launch_bounds__(32 * CONTACT_WARPS) k_contact_force_b(const CavDesc *desc, const int2 *pmap,
                                                                       int total)
{
    pdl_wait();
    pdl_trigger();
    __shared__ int cand[CONTACT_WARPS][MAX_CAND];
    __shared__ int ncand[CONTACT_WARPS];
    const int w = threadIdx.x >> 5;
    const int g = blockIdx.x * CONTACT_WARPS + w;
    if (g >= total) return;
    const int2 mp = pmap[g];
    const CavDesc &d = desc[mp.x];
    if (d.out == OUT_IDLE) return;
    contact_force_body(d.geo, d.ph, d.pb, d.status, mp.y, cand[w], ncand[w]);
}

__global__ void k_update_b(const CavDesc *desc, const int2 *pmap, int total)
{
    pdl_wait();
    pdl_trigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const int2 mp = pmap[g];
    const CavDesc &d = desc[mp.x];
    if (d.out == OUT_IDLE) return;
    update_body(d.ph, d.pb, mp.y);
    pgeo_body(d.geo, d.ph, d.pb, mp.y);   // geometry cache of the new position
}

__global__ void k_owner_fill_b(const CavDesc *desc, const int *pmem)
{
    pdl_wait();
    pdl_trigger();
    const CavDesc &d = desc[pmem[blockIdx.y]];
    if (d.out == OUT_IDLE) return;
    int *o = d.owner[d.ocur ^ 1];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < d.geo.L;
         i += (long long)gridDim.x * blockDim.x)
        o[i] = -1;
}

template <int NT>
__global__ void __launch_bounds__(NT) k_mark_b(const CavDesc *desc, const int2 *pmap)
{
    pdl_wait();
    pdl_trigger();
    __shared__ ShellRows<NT> sr;
    const int2 mp = pmap[blockIdx.x];
    const CavDesc &d = desc[mp.x];
    if (d.out == OUT_IDLE) return;
    mark_body<NT>(d.geo, d.ph, d.pb, d.owner[d.ocur ^ 1], mp.y, sr);
}

template <bool F32Q, int NT>
// 128-thread CTAs are held to 48 registers (10 resident per SM): the descriptor fields the batched
// body reads cost registers the single-cavity kernel takes from its parameters, and at 72 registers
// only 7 CTAs fit (the 256-cavity ensemble step is 1 % faster with the small spill this leaves)
__global__ void __launch_bounds__(NT, NT == LINK_NARROW ? 10 : 1) k_link_fill_b(const CavDesc *desc, const int2 *pmap)
{
    pdl_wait();
    pdl_trigger();
    __shared__ LinkShared<NT> sm;
    const int2 mp = pmap[blockIdx.x];
    const CavDesc &d = desc[mp.x];
    if (d.out == OUT_IDLE) return;
    link_fill_body<F32Q, NT>(d.geo, d.ph, d.pb, d.owner[d.ocur ^ 1], d.status, mp.y, sm);
}

template <int NT>
__global__ void __launch_bounds__(NT) k_new_fluid_b(const CavDesc *desc, const int2 *pmap)
{
    pdl_wait();
    pdl_trigger();
    __shared__ ShellRows<NT> sr;
    const int2 mp = pmap[blockIdx.x];
    const CavDesc &d = desc[mp.x];
    if (d.out == OUT_IDLE) return;
    new_fluid_body<NT>(d.geo, d.ph, d.pb, d.owner[d.ocur], d.owner[d.ocur ^ 1], d.status, mp.y, sr);
}

template <int MODE>
__global__ void k_refill_compute_b(const CavDesc *desc, const int *pmem)
{
    pdl_wait();
    pdl_trigger();
    const CavDesc &d = desc[pmem[blockIdx.y]];
    if (d.out == OUT_IDLE) return;
    refill_compute_body<MODE>(d.geo, d.ph, d.pb, d.owner[d.ocur], d.f, d.g, d.rho, d.phase == PHASE_SWAPPED,
                              d.status, (blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                              (gridDim.x * blockDim.x) >> 5);
}

template <int MODE>
__global__ void k_refill_scatter_b(const CavDesc *desc, const int *pmem)
{
    pdl_wait();
    pdl_trigger();
    const CavDesc &d = desc[pmem[blockIdx.y]];
    if (d.out == OUT_IDLE) return;
    refill_scatter_body<MODE>(d.geo, d.ph, d.pb, d.f, d.g, d.faux, d.rho_wall, d.out == OUT_MACROS,
                              d.rho, d.ux, d.uy, d.uz, d.phi, d.status, d.phase == PHASE_SWAPPED,
                              (long long)blockIdx.x * blockDim.x + threadIdx.x,
                              (long long)gridDim.x * blockDim.x);
}

template <int MODE>
cudaError_t particles_batched_mode(const CavDesc *desc, const int2 *pmap, int total, const int2 *cmap,
                                   int ncmap, const int *pmem, int npmem, cudaStream_t st, cudaStream_t side,
                                   cudaEvent_t ev_fork, cudaEvent_t ev_join)
{
    const int t = 128, bl = (total + t - 1) / t;
    cudaError_t e;
#define RBTP_PDL(...)                                                       \
    do {                                                                    \
        if ((e = pdl_launch(__VA_ARGS__)) != cudaSuccess) return e;         \
    } while (0)
    // contacts (cell list and pair forces of the current positions) beside IBB
    if ((e = cudaEventRecord(ev_fork, st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(side, ev_fork, 0)) != cudaSuccess) return e;
    RBTP_PDL(k_cells_zero_b, dim3(4, npmem), dim3(256), side, desc, pmem);
    RBTP_PDL(k_cell_count_b, dim3(bl), dim3(t), side, desc, pmap, total);
    RBTP_PDL(k_cell_scan_b, dim3(npmem), dim3(1024), side, desc, pmem);
    RBTP_PDL(k_cell_fill_b, dim3(bl), dim3(t), side, desc, pmap, total);
    RBTP_PDL(k_contact_force_b, dim3((total + CONTACT_WARPS - 1) / CONTACT_WARPS), dim3(32 * CONTACT_WARPS), side,
             desc, pmap, total);
    if ((e = cudaEventRecord(ev_join, side)) != cudaSuccess) return e;
    RBTP_PDL(k_links_ibb_b<MODE>, dim3(ncmap), dim3(IBB_THREADS), st, desc, pmap, cmap);
    if ((e = cudaStreamWaitEvent(st, ev_join, 0)) != cudaSuccess) return e;
    RBTP_PDL(k_update_b, dim3(bl), dim3(t), st, desc, pmap, total);
    RBTP_PDL(k_owner_fill_b, dim3(64, npmem), dim3(256), st, desc, pmem);
    if (total < PARTICLES_WIDE) {
        RBTP_PDL(k_mark_b<LINK_WIDE>, dim3(total), dim3(LINK_WIDE), st, desc, pmap);
        RBTP_PDL(k_link_fill_b<MODE != RBTP_STORE_F64, LINK_WIDE>, dim3(total), dim3(LINK_WIDE), st, desc, pmap);
        RBTP_PDL(k_new_fluid_b<LINK_WIDE>, dim3(total), dim3(LINK_WIDE), st, desc, pmap);
    } else {
        RBTP_PDL(k_mark_b<LINK_NARROW>, dim3(total), dim3(LINK_NARROW), st, desc, pmap);
        RBTP_PDL(k_link_fill_b<MODE != RBTP_STORE_F64, LINK_NARROW>, dim3(total), dim3(LINK_NARROW), st, desc, pmap);
        RBTP_PDL(k_new_fluid_b<LINK_NARROW>, dim3(total), dim3(LINK_NARROW), st, desc, pmap);
    }
    RBTP_PDL(k_refill_compute_b<MODE>, dim3(8, npmem), dim3(256), st, desc, pmem);
    RBTP_PDL(k_refill_scatter_b<MODE>, dim3(8, npmem), dim3(256), st, desc, pmem);
#undef RBTP_PDL
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_particles_batched(int mode, const CavDesc *desc, const int2 *pmap, int total_np,
                                     const int2 *cmap, int ncmap, const int *pmem, int npmem, cudaStream_t st,
                                     cudaStream_t side, cudaEvent_t ev_fork, cudaEvent_t ev_join)
{
    if (total_np <= 0 || npmem <= 0) return cudaSuccess;
    switch (mode) {
    case RBTP_STORE_F64:
        return particles_batched_mode<RBTP_STORE_F64>(desc, pmap, total_np, cmap, ncmap, pmem, npmem, st, side, ev_fork, ev_join);
    case RBTP_STORE_F32:
        return particles_batched_mode<RBTP_STORE_F32>(desc, pmap, total_np, cmap, ncmap, pmem, npmem, st, side, ev_fork, ev_join);
    case RBTP_STORE_F16S:
        return particles_batched_mode<RBTP_STORE_F16S>(desc, pmap, total_np, cmap, ncmap, pmem, npmem, st, side, ev_fork, ev_join);
    }
    return cudaErrorInvalidValue;
}

}  // namespace rbtp
