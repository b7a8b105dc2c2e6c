// step_node.cuh — the per-node body of the fused stream/collide step on the in-place AA storage
// (see lbm_step.cu for the algorithm and its reference mapping, rbtp_internal.cuh for the slots).  Included by lbm_step.cu (single cavity) and batch_step.cu
// (many cavities over a packed tile table), which instantiate it for their launch shapes.
#pragma once

#include <type_traits>

#include "rbtp_internal.cuh"

// Resident 128-thread blocks per SM requested from the register allocator (FP64 is bound by the
// FP64 pipe, FP32 storage by HBM bandwidth, shifted-FP16 storage by instruction issue).  Best of
// 4/5/6 sweeps of both step parities at 320x320x160 on GB300: 5 (<= 96 registers) for FP32 and
// shifted FP16.  At 6 (<= 80 registers) the FP32 steps are 5 % slower and the shifted-FP16 even
// step, spilling, takes twice as long.
#ifndef RBTP_STEP_MINB_F64
#define RBTP_STEP_MINB_F64 1
#endif
#ifndef RBTP_STEP_MINB_F32
#define RBTP_STEP_MINB_F32 5
#endif
#ifndef RBTP_STEP_MINB_F16S
#define RBTP_STEP_MINB_F16S 5
#endif
#define RBTP_STEP_MINB(MODE)                                                 \
    ((MODE) == RBTP_STORE_F64 ? RBTP_STEP_MINB_F64                           \
                              : ((MODE) == RBTP_STORE_F32 ? RBTP_STEP_MINB_F32 : RBTP_STEP_MINB_F16S))

namespace rbtp {

// Bit i set for the directions whose component along an axis has the given sign: a node on the
// low face of that axis has its upstream neighbour x - c_i outside the box exactly for those i.
__host__ __device__ constexpr unsigned dir_mask(int axis, int sign)
{
    unsigned m = 0;
    for (int i = 0; i < 27; ++i) {
        const int c = axis == 0 ? dcx(i) : (axis == 1 ? dcy(i) : dcz(i));
        if (c == sign) m |= 1u << i;
    }
    return m;
}

// (f_i, g_i) of one direction held as one value.  The moments and both collisions apply the same
// operation to f and to g, pair by pair, so in the float modes the pair is a float2 and sm_100's
// packed FP32x2 instructions (FADD2, FMUL2, FFMA2: IEEE single operations on both halves, round
// to nearest) advance both halves in one issue slot.  FP64 keeps two scalar operations.
template <typename R>
struct PairOps;
template <>
struct PairOps<float> {
    using T = float2;
    static __device__ __forceinline__ T mk(float a, float b) { return make_float2(a, b); }
    static __device__ __forceinline__ T add(T a, T b) { return __fadd2_rn(a, b); }
    static __device__ __forceinline__ T sub(T a, T b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
    static __device__ __forceinline__ T mul(T a, T b) { return __fmul2_rn(a, b); }
    static __device__ __forceinline__ T fma(T a, T b, T c) { return __ffma2_rn(a, b, c); }
};
template <>
struct PairOps<double> {
    using T = double2;
    static __device__ __forceinline__ T mk(double a, double b) { return make_double2(a, b); }
    static __device__ __forceinline__ T add(T a, T b) { return make_double2(a.x + b.x, a.y + b.y); }
    static __device__ __forceinline__ T sub(T a, T b) { return make_double2(a.x - b.x, a.y - b.y); }
    static __device__ __forceinline__ T mul(T a, T b) { return make_double2(a.x * b.x, a.y * b.y); }
    static __device__ __forceinline__ T fma(T a, T b, T c)
    {
        return make_double2(__fma_rn(a.x, b.x, c.x), __fma_rn(a.y, b.y, c.y));
    }
};

// One node of the fused step in the in-place AA storage (StepBuffers describes the slots); shared
// by the single-cavity kernel (lbm_step.cu) and the batched kernel (batch_step.cu).  (ix, iy, iz)
// must lie inside the lattice.  ODD selects the odd step (gather from swapped neighbour slots,
// scatter to natural neighbour slots, walls at both ends); the even step reads and writes the
// node's own slots only.  INTERIOR_PATH adds, for odd steps, a second copy of the gather and the
// scatter without the box-face tests, taken by warps none of whose nodes touches a face.  It pays
// only where the step is issue-bound (shifted-FP16 storage: odd step 0.683 against 0.84 ms without
// it at 320x320x160); FP32 is HBM-bound (measured the same with it), FP64 FP64-pipe-bound, and
// the batched kernel (six step variants in one kernel at 128 registers) ran 0.7 % slower with it
// (9,010 against 9,073 MLUPS for the 256-cavity ensemble), so they leave it out.
//
// FRESH_SCATTER: the scatter addresses its slots from an opaque copy of the node index.  A node
// writes exactly the slots it read (both parities), so otherwise the compiler keeps the gather's
// addresses (two registers each) live across the collision rather than recompute them.  The
// batched kernel, whose lattice sizes are per-thread values (staged in shared memory), spills
// 460-550 bytes per thread at 128 registers without it and none with it (+7 % ensemble
// throughput).  The single-cavity kernel, addressing from its launch parameters, gains nothing
// (FP32, shifted FP16) or loses half its speed (FP64), so it leaves it out.
//
// The odd-step slot offsets come from an AAOff table: the launch parameters of the single-cavity
// kernel, a copy staged in shared memory per member in the batched kernel.
//
// FACE_MASK: the per-direction box-face tests read bits of two per-node masks built once from the
// six face flags, instead of evaluating the flags' disjunction per direction.  Measured at
// 320x320x160: FP64 odd step 13.24 against 13.41 ms, batched ensemble +0.5 % (with the staged
// offset table); the single-cavity FP32 and shifted-FP16 odd steps run 1-2 % slower with it, so
// they keep the flag expressions.
template <int MODE, bool ODD, int OUT, bool INTERIOR_PATH = MODE == RBTP_STORE_F16S, bool FRESH_SCATTER = false,
          bool FACE_MASK = MODE == RBTP_STORE_F64>
__device__ __forceinline__ void step_node(const Geo &geo, const Phys &ph, const StepBuffers &b, const AAOff &ao,
                                          int ix, int iy, int iz)
{
    using ST = Store<MODE>;
    using S = typename ST::S;
    using R = typename ST::R;
    const long long L = geo.L;
    const long long node = (long long)iz * geo.lxy + (long long)iy * geo.lx + ix;
    // read and written in place: no restrict (the paired float modes alias f and g)
    S *const fA = static_cast<S *>(b.f);
    S *const gA = static_cast<S *>(b.g);
    // Every slot a node touches is its own slot of direction 0 plus a kernel-uniform offset: i L
    // (its own slot i), o L - off_i (odd gather), i L + off_i (odd scatter).  Addressed as one
    // per-thread base pointer plus that offset, the offset stays in the load or store instruction;
    // written as (o L + node) - off_i, each access cost two 64-bit integer additions (odd steps ran
    // 1.6-2x the even steps' instructions).
    const S *const fN = fA + node;
    const S *const gN = gA + node;
    // the odd step's gather offset of direction I (AAOff)
    auto aa_gather = [&](auto I) -> long long { return ao.g[decltype(I)::value]; };
    const double t0 = ph.t0;
    const bool xlo = ix == 0, xhi = ix == geo.lx - 1;
    const bool ylo = iy == 0, yhi = iy == geo.ly - 1;
    const bool zlo = iz == 0, zhi = iz == geo.lz - 1;
    const long long wall_slot = (long long)iz * geo.ly + iy;
    const StepK<R> &K = step_consts<R>(ph);
    // Bit i of out_x / out_yz: x - c_i lies outside the box through an x face / a y or z face
    // (FACE_MASK); the scatter's neighbour x + c_i = x - c_opp(i) is tested as direction opp(i).
    unsigned out_x = 0u, out_yz = 0u;
    if constexpr (FACE_MASK) {
        out_x = (xlo ? dir_mask(0, 1) : 0u) | (xhi ? dir_mask(0, -1) : 0u);
        out_yz = (ylo ? dir_mask(1, 1) : 0u) | (yhi ? dir_mask(1, -1) : 0u) | (zlo ? dir_mask(2, 1) : 0u) |
                 (zhi ? dir_mask(2, -1) : 0u);
    }
    const unsigned out_any = out_x | out_yz;
    auto bit = [](unsigned m, int i) { return ((m >> i) & 1u) != 0u; };

    // Shifted-FP16 storage works in its scaled variables throughout: F_i = f_i / w_i and
    // G_i = g_i / w_i - T_c(x_slot) are what the memory holds (T_c the conduction profile at the
    // slot's own node), the moments take the weights once per lattice-weight class, and the
    // collision constants are divided by w_i (no per-population scaling on load or store).  A
    // gathered G_i is relative to s_i = T_c(x - c_ix) = Tc - tlb c_ix, a linear function of c_ix, so
    // its moment and collision corrections are closed-form.  The other modes work on f_i and g_i.
    constexpr bool SC = MODE == RBTP_STORE_F16S;
    const R Tc = SC ? K.tla + K.tlb * (R)ix : (R)0;   // T_c at this node
    // (f_i, g_i) of one direction as one pair value (PairOps): a float2 in the float modes
    using PO = PairOps<R>;
    using V = typename PO::T;
    constexpr R NZ = -(R)0;
    constexpr V NZ2 = V{NZ, NZ};
    // both populations of a slot (one access in the paired layouts of the float modes)
    auto ldfg = [&](const S *pf, const S *pg, double w) -> V {
        if constexpr (SC) {
            return __half22float2(*pf);
        } else if constexpr (ST::PAIRED) {
            return *pf;
        } else {
            return PO::mk(ST::ld_f(pf, w, t0), ST::ld_g(pg, w, t0));
        }
    };
    // F_x of the previous step, read ahead of the population gather
    using A = typename ST::A;
    const A fold_in = __ldg(static_cast<const A *>(b.faux) + node);
    V fg[27];
    // INTERIOR: no neighbour of this warp's nodes leaves the box, so every odd-step gather is the
    // plain f*_i(x - c_i) and every scatter the plain slot (i, x + c_i) (the face tests and the
    // wall selects drop out)
    auto gather = [&](auto INT) {
        constexpr bool INTERIOR = decltype(INT)::value;
        unroll<27>([&](auto I) {
            constexpr int i = decltype(I)::value;
            constexpr int cx = dcx(i), cy = dcy(i), cz = dcz(i), o = dopp(i);
            constexpr double w = dweight(i);
            if constexpr (!ODD || i == 0) {
                // even step: the post-streaming f_i(x) in the natural slot (i, x)
                fg[i] = ldfg(fN + (long long)i * L, gN + (long long)i * L, w);
            } else {
                // odd step: f_i(x) = f*_i(x - c_i), swapped into slot (opp(i), x - c_i); a
                // neighbour outside the box returns f*_opp(i)(x), swapped into slot (i, x)
                long long src = aa_gather(I);
                if constexpr (!INTERIOR) {
                    const bool out = FACE_MASK ? bit(out_any, i)
                                               : ((cx == 1 && xlo) || (cx == -1 && xhi) || (cy == 1 && ylo) ||
                                                  (cy == -1 && yhi) || (cz == 1 && zlo) || (cz == -1 && zhi));
                    if constexpr (SC) {
                        if (out) src = (long long)i * L;
                    } else {
                        src = out ? (long long)i * L : src;
                    }
                }
                fg[i] = ldfg(fN + src, gN + src, w);
            }
        });
    };
    const bool face = xlo || xhi || ylo || yhi || zlo || zhi;
    const bool interior = INTERIOR_PATH && ODD && !__any_sync(__activemask(), face);
    if (interior) gather(std::true_type{});
    else gather(std::false_type{});
    if constexpr (!ODD && SC) {
        // natural slots: every G_i is relative to T_c(x), not s_i
        unroll<27>([&](auto I) {
            constexpr int i = decltype(I)::value;
            constexpr int cx = dcx(i);
            if constexpr (cx != 0) fg[i].y += K.tlb * (R)cx;
        });
    }
    if constexpr (ODD && SC) {
        // a bounce-back slot belongs to this node: re-express its G relative to s_i (one branch
        // around the whole correction, taken only by box-surface nodes)
        if (xlo || xhi || ylo || yhi || zlo || zhi) {
            unroll<27>([&](auto I) {
                constexpr int i = decltype(I)::value;
                constexpr int cx = dcx(i), cy = dcy(i), cz = dcz(i);
                if constexpr (i != 0 && cx != 0) {
                    const bool out = FACE_MASK ? bit(out_any, i)
                                               : ((cx == 1 && xlo) || (cx == -1 && xhi) || (cy == 1 && ylo) ||
                                                  (cy == -1 && yhi) || (cz == 1 && zlo) || (cz == -1 && zhi));
                    if (out) fg[i].y += K.tlb * (R)cx;
                }
            });
        }
    }
    if constexpr (ODD) {
        // streaming.cu:45-61 for the even step's output: at the x walls a direction that leaves
        // only through x takes the Dirichlet anti-bounce-back with the node's density deviation of
        // the (even) step that produced it; y/z exits stay adiabatic.  Only warps holding x-wall
        // nodes enter this branch.
        if (xlo || xhi) {
            const R rw = (R)b.rho_wall[(xhi ? (long long)geo.lz * geo.ly : 0) + wall_slot];
            const R tw = xlo ? K.thot : K.tcold;
            unroll<27>([&](auto I) {
                constexpr int i = decltype(I)::value;
                constexpr int cx = dcx(i), cy = dcy(i), cz = dcz(i);
                if constexpr (cx != 0) {
                    const bool ox = FACE_MASK ? bit(out_x, i) : ((cx == 1) ? xlo : xhi);
                    const bool oyz = FACE_MASK ? bit(out_yz, i)
                                               : ((cy == 1 && ylo) || (cy == -1 && yhi) || (cz == 1 && zlo) ||
                                                  (cz == -1 && zhi));
                    if (ox && !oyz) {
                        if constexpr (SC) {
                            const R wi = (R)dweight(i);
                            const R si = Tc - K.tlb * (R)cx;
                            fg[i].y = wall_image(wi * (fg[i].y + si), dweight(i), tw, rw) * (R)(1.0 / dweight(i)) - si;
                        } else {
                            fg[i].y = wall_image(fg[i].y, dweight(i), tw, rw);
                        }
                    }
                }
            });
        }
    }

    // ---- moments (macrovar.cu:3-34), pairwise, f and g together ----
    // m0 = (rho, phi), mx = (j_x, k_x) = (sum_i c_ix f_i, sum_i c_ix g_i), my, mz likewise.  Sums
    // start from -0.0: -0.0 + x == x for every x, so the compiler drops the first addition (it
    // may not fold +0.0 + x, which differs for x = -0.0); only the sign of an exact zero can
    // differ from a +0.0 start.
    V m0 = fg[0], mx = NZ2, my = NZ2, mz = NZ2;
    auto pair_moments = [&](auto Kp, V &s0, V &sx, V &sy, V &sz) {
        constexpr int i = dpair(decltype(Kp)::value);
        constexpr int o = dopp(i);
        constexpr int cx = dcx(i), cy = dcy(i), cz = dcz(i);
        const V sum = PO::add(fg[i], fg[o]), dif = PO::sub(fg[i], fg[o]);
        s0 = PO::add(s0, sum);
        if constexpr (cx == 1) sx = PO::add(sx, dif);
        if constexpr (cx == -1) sx = PO::sub(sx, dif);
        if constexpr (cy == 1) sy = PO::add(sy, dif);
        if constexpr (cy == -1) sy = PO::sub(sy, dif);
        if constexpr (cz == 1) sz = PO::add(sz, dif);
        if constexpr (cz == -1) sz = PO::sub(sz, dif);
    };
    if constexpr (SC) {
        // per weight class: sums of the scaled variables, then one multiply by the class weight;
        // rho = w_0 F_0 + ..., phi = w_0 G_0 + T_c + ... (sum_i w_i s_i = T_c), and
        // k_x starts at sum_i c_ix w_i s_i = -tlb sum_i w_i c_ix^2 = -tlb / 3
        m0 = PO::fma(PO::mk((R)dweight(0), (R)dweight(0)), fg[0], PO::mk(NZ, Tc));
        mx = PO::mk(NZ, -K.tlb * (R)(1.0 / 3.0));
        unroll<3>([&](auto C) {
            constexpr int c = decltype(C)::value + 1;
            V s0 = NZ2, sx = NZ2, sy = NZ2, sz = NZ2;
            unroll<13>([&](auto Kp) {
                if constexpr (dclass(dpair(decltype(Kp)::value)) == c) pair_moments(Kp, s0, sx, sy, sz);
            });
            constexpr R w = (R)(c == 1 ? 2.0 / 27.0 : (c == 2 ? 1.0 / 54.0 : 1.0 / 216.0));
            const V W = PO::mk(w, w);
            m0 = PO::fma(W, s0, m0);
            mx = PO::fma(W, sx, mx);
            my = PO::fma(W, sy, my);
            mz = PO::fma(W, sz, mz);
        });
    } else {
        unroll<13>([&](auto Kp) { pair_moments(Kp, m0, mx, my, mz); });
    }
    const R rho = m0.x, phi = m0.y;
    const R jx = mx.x, jy = my.x, jz = mz.x;
    const R kx = mx.y, ky = my.y, kz = mz.y;
    if (!(fabs(rho) < (R)1e30) || !(fabs(phi) < (R)1e30)) atomicOr(&b.status->nonfinite, 1);

    const R fold = (R)fold_in;
    const R ux = jx + (R)0.5 * fold, uy = jy, uz = jz;
    // forcing (macrovar.cu:45): F_x = g0 beta (phi - T0); F_y = F_z = 0 always
    const R Fx = K.g0b * (phi - K.t0);
    static_cast<A *>(b.faux)[node] = (A)Fx;

    if constexpr (OUT >= OUT_MACROS) {
        b.rho[node] = (double)rho;
        b.ux[node] = (double)ux;
        b.uy[node] = (double)uy;
        b.uz[node] = (double)uz;
        b.phi[node] = (double)phi;
    } else if constexpr (OUT == OUT_RHO) {
        b.rho[node] = (double)rho;
    }
    if constexpr (!ODD) {
        // the wall densities the next (odd) step's gather and the stream export apply
        if (xlo) b.rho_wall[wall_slot] = (double)rho;
        if (xhi) b.rho_wall[(long long)geo.lz * geo.ly + wall_slot] = (double)rho;
    }

    // ---- f collision (collision.cu:3-33) ----
    // f*_i = om f_i + w_i [ (rho + P_i)/tau + G (c_ix - u_x)(1 + P_i) ],  P_i = A_i + B_i,
    // A = 4.5 (c.u)^2 - 1.5 u^2, B = 3 c.u, G = 3 (1 - 1/(2 tau)) F_x.
    const R G = K.Gc * Fx;
    const R Gux = G * ux;
    const R h = (R)1.5 * (ux * ux + uy * uy + uz * uz);
    const R k1 = K.tinv - Gux;
    const R k0 = rho * K.tinv - Gux;
    // ---- g collision (collision.cu:35-89) ----
    // g*_i = omc g_i + geqnew_i / tauc + w_i c_i.V, with the source vector
    // V = Rc [ -2 rho/gd (sum_i c_i g_i - phi u) + x F_x phi (3 - rho/gd) ],  gd = rho/3 + 2 tauc/3.
    const R gd = rho * (R)(1.0 / 3.0) + K.gd0;
    const R rgd = rho / gd;
    const R c2 = (R)(-2) * rgd * K.Rc;
    const R Vx = c2 * (kx - phi * ux) + K.Rc * Fx * phi * ((R)3 - rgd);
    const R Vy = c2 * (ky - phi * uy);
    const R Vz = c2 * (kz - phi * uz);
    const R pt = phi * K.tcinv;
    const R ptb = pt * ((R)1 + rho);

    // scaled g at home: G* = g*/w - T_c = omc G + (g* - omc g)/w + (omc - 1) T_c - omc tlb c_ix
    const R gshift = SC ? (K.omc - (R)1) * Tc : (R)0;
    const R gtilt = SC ? -K.omc * K.tlb : (R)0;
    const V OM = PO::mk(K.om, K.omc);
    {
        constexpr R w0 = (R)dweight(0);
        if constexpr (SC) {
            fg[0] = PO::fma(OM, fg[0], PO::mk(k0 - h * k1, (ptb - pt * h) - pt * rho * (R)(1.0 / dweight(0)) + gshift));
        } else {
            fg[0] = PO::fma(OM, fg[0], PO::mk(w0 * (k0 - h * k1), w0 * (ptb - pt * h) - pt * rho));
        }
    }
    // Pairs grouped by weight class (face, edge, corner); the class constants fold w_i into the
    // per-node coefficients and live only while their class is processed.  Per direction pair
    // (i, opp i):
    //   S = (w (A k1 + k0) + w cx G B,  w pt (1 + rho + A))        the parts even in c
    //   D = (w B k1 + w cx G (1 + A),   w pt B + w c.V)            the parts odd in c
    //   (f*, g*)_i = (om, omc) (f, g)_i + S + D,  (f*, g*)_opp = (om, omc) (f, g)_opp + S - D.
    unroll<3>([&](auto C) {
        constexpr int c = decltype(C)::value + 1;
        // class weight; 1 in the scaled variables of shifted-FP16 storage (w_i divided out)
        constexpr R w = SC ? (R)1 : (R)(c == 1 ? 2.0 / 27.0 : (c == 2 ? 1.0 / 54.0 : 1.0 / 216.0));
        const R wk1 = w * k1;
        const R wG = w * G;
        const R wpt = w * pt;
        R gb = w * ptb - h * wpt;
        if constexpr (SC) gb += gshift;
        if constexpr (sizeof(R) == 4 && !SC) {
            // Packed: S and D as (f, g) pairs.  i is the member of the pair whose first nonzero
            // component is +1 (S is even and D odd in c, so the choice is free), so the sums of
            // the (u_k, u_k) and (., v_k) pairs start without a negation and the cx terms carry
            // no sign.
            const V UX = PO::mk(ux, ux), UY = PO::mk(uy, uy), UZ = PO::mk(uz, uz);
            const V CA = PO::mk((R)4.5 * wk1, (R)4.5 * wpt);         // A coefficients
            const V CB = PO::mk(w * k0 - h * wk1, gb);                // constant parts
            const V C3 = PO::mk((R)3 * wk1, (R)3 * wpt);              // B coefficients
            const V CE = PO::mk((R)4.5 * wG, (R)0);                   // f: cx G A
            const V CG = PO::mk((R)3 * wG, (R)0);                     // f: cx G B
            // (cx G (1 - 1.5 u^2), w c.V) from per-component pairs; the shifted-FP16 tilt
            // -omc tlb c_ix rides on the x component of V
            const V ZX = PO::mk(wG - h * wG, SC ? w * Vx + gtilt : w * Vx);
            const V ZY = PO::mk(NZ, w * Vy), ZZ = PO::mk(NZ, w * Vz);
            unroll<13>([&](auto Kp) {
                constexpr int i0 = dpair(decltype(Kp)::value);
                if constexpr (dclass(i0) == c) {
                    constexpr int lead = dcx(i0) != 0 ? dcx(i0) : (dcy(i0) != 0 ? dcy(i0) : dcz(i0));
                    constexpr int i = lead > 0 ? i0 : dopp(i0);
                    constexpr int o = dopp(i);
                    constexpr int cx = dcx(i), cy = dcy(i), cz = dcz(i);
                    // sum_k c_k P_k over the nonzero components, the first one +1
                    auto csum = [&](const V &px, const V &py, const V &pz) {
                        V r;
                        if constexpr (cx != 0) r = px;
                        else if constexpr (cy != 0) r = py;
                        else r = pz;
                        if constexpr (cx != 0 && cy == 1) r = PO::add(r, py);
                        if constexpr (cx != 0 && cy == -1) r = PO::sub(r, py);
                        if constexpr ((cx != 0 || cy != 0) && cz == 1) r = PO::add(r, pz);
                        if constexpr ((cx != 0 || cy != 0) && cz == -1) r = PO::sub(r, pz);
                        return r;
                    };
                    const V CU = csum(UX, UY, UZ);                     // (c.u, c.u)
                    const V QQ = PO::mul(CU, CU);                      // ((c.u)^2, (c.u)^2)
                    V Sv = PO::fma(QQ, CA, CB);
                    V Z = csum(ZX, ZY, ZZ);
                    if constexpr (cx != 0) {                           // cx = +1 here
                        Sv = PO::fma(CU, CG, Sv);
                        Z = PO::fma(QQ, CE, Z);
                    }
                    const V Dv = PO::fma(CU, C3, Z);
                    fg[i] = PO::fma(OM, fg[i], PO::add(Sv, Dv));
                    fg[o] = PO::fma(OM, fg[o], PO::sub(Sv, Dv));
                }
            });
        } else {
            // Scalar operations: FP64 (the pair form would spend FP64 instructions on its
            // duplicated and zero lanes) and shifted FP16 (whose step, issue-bound at 96
            // registers, ran 0.768 against 0.692 ms per odd step at 320x320x160 with the
            // constant pairs)
            const R ca = (R)4.5 * wk1, cb = w * k0 - h * wk1, c3 = (R)3 * wk1;
            const R ce = (R)4.5 * wG, cd = wG - h * wG, cg = (R)3 * wG;
            const R ga = (R)4.5 * wpt, gc = (R)3 * wpt;
            const R vx = w * Vx, vy = w * Vy, vz = w * Vz;
            unroll<13>([&](auto Kp) {
                constexpr int i = dpair(decltype(Kp)::value);
                if constexpr (dclass(i) == c) {
                    constexpr int o = dopp(i);
                    constexpr int cx = dcx(i), cy = dcy(i), cz = dcz(i);
                    R cu = NZ, cV = NZ;
                    if constexpr (cx != 0) { cu += (R)cx * ux; cV += (R)cx * vx; }
                    if constexpr (cy != 0) { cu += (R)cy * uy; cV += (R)cy * vy; }
                    if constexpr (cz != 0) { cu += (R)cz * uz; cV += (R)cz * vz; }
                    const R q = cu * cu;
                    R wS = q * ca + cb;                 // w (A k1 + k0)
                    R wD = cu * c3;                     // w B k1
                    if constexpr (cx != 0) {
                        wS += (R)cx * (cu * cg);        // w cx G B
                        wD += (R)cx * (q * ce + cd);    // w cx G (1 + A)
                    }
                    const R gS = q * ga + gb;           // w pt (1 + rho + A)
                    R gD = cu * gc + cV;                // w pt B + w c.V
                    if constexpr (SC && cx != 0) gD += (R)cx * gtilt;
                    fg[i] = PO::fma(OM, fg[i], PO::mk(wS + wD, gS + gD));
                    fg[o] = PO::fma(OM, fg[o], PO::mk(wS - wD, gS - gD));
                }
            });
        }
    });

    // the node index the scatter addresses from (an opaque copy with FRESH_SCATTER)
    long long snode = node;
    if constexpr (FRESH_SCATTER) asm("" : "+l"(snode));
    S *const fS = fA + snode;
    S *const gS = gA + snode;
    // store the slot at offset rel from this node's slot of direction 0: (f, g) in the working
    // variables (shifted FP16: g relative to T_c of the slot's own node)
    auto put = [&](long long rel, const V &v, double w) {
        if constexpr (SC) {
            fS[rel] = __float22half2_rn(v);
        } else if constexpr (ST::PAIRED) {
            fS[rel] = v;
        } else {
            ST::st_f(fS + rel, v.x, w, t0);
            ST::st_g(gS + rel, v.y, w, t0);
        }
    };
    auto scatter = [&](auto INT) {
        constexpr bool INTERIOR = decltype(INT)::value;
        unroll<27>([&](auto I) {
            constexpr int i = decltype(I)::value;
            constexpr int cx = dcx(i), cy = dcy(i), cz = dcz(i), o = dopp(i);
            constexpr double w = dweight(i);
            if constexpr (!ODD || i == 0) {
                // even step: f*_i(x) swapped into the node's own slot (opp(i), x)
                put((long long)o * L, fg[i], w);
            } else {
                // odd step: f*_i(x) streams to slot (i, x + c_i); a population leaving the box
                // becomes the next step's f_opp(i)(x) in slot (opp(i), x): bounce-back for f, and
                // for g adiabatic at y/z exits or the Dirichlet image -g* + 2 w T_wall (1 + rho)
                // with this node's density at a pure x exit (streaming.cu:3-63)
                bool out = false;
                if constexpr (!INTERIOR)
                    out = FACE_MASK ? bit(out_any, o)
                                    : ((cx == 1 && xhi) || (cx == -1 && xlo) || (cy == 1 && yhi) || (cy == -1 && ylo) ||
                                       (cz == 1 && zhi) || (cz == -1 && zlo));
                if (!out) {
                    // shifted FP16: relative to T_c(x + c_i) = T_c(x) + tlb c_ix
                    put(aa_gather(std::integral_constant<int, o>{}), SC && cx != 0 ? PO::mk(fg[i].x, fg[i].y - K.tlb * (R)cx) : fg[i], w);
                } else {
                    V v = fg[i];
                    if constexpr (cx != 0) {
                        const bool ox = FACE_MASK ? bit(out_x, o) : ((cx == 1) ? xhi : xlo);
                        const bool oyz = FACE_MASK ? bit(out_yz, o)
                                                   : ((cy == 1 && yhi) || (cy == -1 && ylo) || (cz == 1 && zhi) ||
                                                      (cz == -1 && zlo));
                        if (ox && !oyz) {
                            const R tw = (cx == -1) ? K.thot : K.tcold;
                            if constexpr (SC) {
                                const R wi = (R)w;
                                v.y = wall_image(wi * (v.y + Tc), w, tw, rho) * (R)(1.0 / w) - Tc;
                            } else {
                                v.y = wall_image(v.y, w, tw, rho);
                            }
                        }
                    }
                    put((long long)o * L, v, w);
                }
            }
            if constexpr (OUT == OUT_MACROS_COL) {
                if constexpr (SC) {
                    b.fcol[(long long)i * L + node] = (double)((R)w * fg[i].x);
                    b.gcol[(long long)i * L + node] = (double)((R)w * (fg[i].y + Tc));
                } else {
                    b.fcol[(long long)i * L + node] = (double)fg[i].x;
                    b.gcol[(long long)i * L + node] = (double)fg[i].y;
                }
            }
        });
    };
    if (interior) scatter(std::true_type{});
    else scatter(std::false_type{});
}

}  // namespace rbtp
