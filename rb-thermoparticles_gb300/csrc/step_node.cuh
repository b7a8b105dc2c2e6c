// step_node.cuh — the per-node body of the fused stream/collide step on the in-place AA storage
// (see lbm_step.cu for the algorithm and its reference mapping, rbtp_internal.cuh for the slots).  Included by lbm_step.cu (single cavity) and batch_step.cu
// (many cavities over a packed tile table), which instantiate it for their launch shapes.
#pragma once

#include <type_traits>

#include "rbtp_internal.cuh"

// Resident 128-thread blocks per SM requested from the register allocator (FP64 is bound by the
// FP64 pipe, the FP32/FP16 storage modes by HBM bandwidth).
#ifndef RBTP_STEP_MINB_F64
#define RBTP_STEP_MINB_F64 1
#endif
#ifndef RBTP_STEP_MINB_LOW
#define RBTP_STEP_MINB_LOW 6  // 6 x 128 threads (<= 80 registers): best of a 1/5/6/8 sweep on GB300
#endif

namespace rbtp {

// One node of the fused step in the in-place AA storage (StepBuffers describes the slots); shared
// by the single-cavity kernel (lbm_step.cu) and the batched kernel (batch_step.cu).  (ix, iy, iz)
// must lie inside the lattice.  ODD selects the odd step (gather from swapped neighbour slots,
// scatter to natural neighbour slots, walls at both ends); the even step reads and writes the
// node's own slots only.  INTERIOR_PATH adds, for odd steps, a second copy of the gather and the
// scatter without the box-face tests, taken by warps none of whose nodes touches a face.  It pays
// only where the step is issue-bound (shifted-FP16 storage: -11 % instructions at 320x320x160);
// FP32 is HBM-bound and FP64 FP64-pipe-bound, and the batched kernel (six step variants in one
// kernel, small cavities whose warps nearly all touch an x face) leaves it out.
template <int MODE, bool ODD, int OUT, bool INTERIOR_PATH = true>
__device__ __forceinline__ void step_node(const Geo &geo, const Phys &ph, const StepBuffers &b, int ix,
                                          int iy, int iz)
{
    using ST = Store<MODE>;
    using S = typename ST::S;
    using R = typename ST::R;
    const long long L = geo.L;
    const long long node = (long long)iz * geo.lxy + (long long)iy * geo.lx + ix;
    // read and written in place: no restrict (the paired float modes alias f and g)
    S *fA = static_cast<S *>(b.f);
    S *gA = static_cast<S *>(b.g);
    const double t0 = ph.t0;
    const bool xlo = ix == 0, xhi = ix == geo.lx - 1;
    const bool ylo = iy == 0, yhi = iy == geo.ly - 1;
    const bool zlo = iz == 0, zhi = iz == geo.lz - 1;
    const long long wall_slot = (long long)iz * geo.ly + iy;
    const StepK<R> &K = step_consts<R>(ph);

    // Shifted-FP16 storage works in its scaled variables throughout: F_i = f_i / w_i and
    // G_i = g_i / w_i - T_c(x_slot) are what the memory holds (T_c the conduction profile at the
    // slot's own node), the moments take the weights once per lattice-weight class, and the
    // collision constants are divided by w_i (no per-population scaling on load or store).  A
    // gathered G_i is relative to s_i = T_c(x - c_ix) = Tc - tlb c_ix, a linear function of c_ix, so
    // its moment and collision corrections are closed-form.  The other modes work on f_i and g_i.
    constexpr bool SC = MODE == RBTP_STORE_F16S;
    const R Tc = SC ? K.tla + K.tlb * (R)ix : (R)0;   // T_c at this node
    // both populations of a slot (one access in the paired layouts of the float modes)
    auto ldfg = [&](const S *p, double w, R &fv, R &gv) {
        if constexpr (SC) {
            const __half2 v = *p;
            fv = __low2float(v);
            gv = __high2float(v);
        } else if constexpr (ST::PAIRED) {
            const float2 v = *p;
            fv = v.x;
            gv = v.y;
        }
    };
    // F_x of the previous step, read ahead of the population gather
    using A = typename ST::A;
    const A fold_in = __ldg(static_cast<const A *>(b.faux) + node);
    R f[27], g[27];
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
                if constexpr (ST::PAIRED) {
                    ldfg(fA + (long long)i * L + node, w, f[i], g[i]);
                } else {
                    f[i] = ST::ld_f(fA + (long long)i * L + node, w, t0);
                    g[i] = ST::ld_g(gA + (long long)i * L + node, w, t0);
                }
            } else {
                // odd step: f_i(x) = f*_i(x - c_i), swapped into slot (opp(i), x - c_i); a
                // neighbour outside the box returns f*_opp(i)(x), swapped into slot (i, x)
                const long long off = (long long)cx + (long long)cy * geo.lx + (long long)cz * geo.lxy;
                long long src = (long long)o * L + node - off;
                if constexpr (!INTERIOR) {
                    const bool out = (cx == 1 && xlo) || (cx == -1 && xhi) || (cy == 1 && ylo) ||
                                     (cy == -1 && yhi) || (cz == 1 && zlo) || (cz == -1 && zhi);
                    if constexpr (SC) {
                        if (out) src = (long long)i * L + node;
                    } else {
                        src = out ? ((long long)i * L + node) : src;
                    }
                }
                if constexpr (ST::PAIRED) {
                    ldfg(fA + src, w, f[i], g[i]);
                } else {
                    f[i] = ST::ld_f(fA + src, w, t0);
                    g[i] = ST::ld_g(gA + src, w, t0);
                }
            }
        });
    };
    const bool face = xlo || xhi || ylo || yhi || zlo || zhi;
    const bool interior = INTERIOR_PATH && SC && ODD && !__any_sync(__activemask(), face);
    if (interior) gather(std::true_type{});
    else gather(std::false_type{});
    if constexpr (!ODD && SC) {
        // natural slots: every G_i is relative to T_c(x), not s_i
        unroll<27>([&](auto I) {
            constexpr int i = decltype(I)::value;
            constexpr int cx = dcx(i);
            if constexpr (cx != 0) g[i] += K.tlb * (R)cx;
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
                    const bool out = (cx == 1 && xlo) || (cx == -1 && xhi) || (cy == 1 && ylo) ||
                                     (cy == -1 && yhi) || (cz == 1 && zlo) || (cz == -1 && zhi);
                    if (out) g[i] += K.tlb * (R)cx;
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
                    const bool ox = (cx == 1) ? xlo : xhi;
                    const bool oyz = (cy == 1 && ylo) || (cy == -1 && yhi) || (cz == 1 && zlo) || (cz == -1 && zhi);
                    if (ox && !oyz) {
                        if constexpr (SC) {
                            const R wi = (R)dweight(i);
                            const R si = Tc - K.tlb * (R)cx;
                            g[i] = wall_image(wi * (g[i] + si), dweight(i), tw, rw) * (R)(1.0 / dweight(i)) - si;
                        } else {
                            g[i] = wall_image(g[i], dweight(i), tw, rw);
                        }
                    }
                }
            });
        }
    }

    // ---- moments (macrovar.cu:3-34), pairwise ----
    // Sums start from -0.0: -0.0 + x == x for every x, so the compiler drops the first addition
    // (it may not fold +0.0 + x, which differs for x = -0.0); only the sign of an exact zero can
    // differ from a +0.0 start.
    constexpr R NZ = -(R)0;
    R rho = f[0], jx = NZ, jy = NZ, jz = NZ;
    R phi = g[0], kx = NZ, ky = NZ, kz = NZ;
    if constexpr (SC) {
        // per weight class: sums of the scaled variables, then one multiply by the class weight
        rho = (R)dweight(0) * f[0];
        phi = (R)dweight(0) * g[0] + Tc;     // sum_i w_i (G_i + s_i), sum_i w_i s_i = T_c
        kx = -K.tlb * (R)(1.0 / 3.0);        // sum_i c_i w_i s_i = -tlb sum_i w_i c_i c_ix
        unroll<3>([&](auto C) {
            constexpr int c = decltype(C)::value + 1;
            R r_ = NZ, p_ = NZ, ax = NZ, ay = NZ, az = NZ, bx = NZ, by = NZ, bz = NZ;
            unroll<13>([&](auto Kp) {
                constexpr int i = dpair(decltype(Kp)::value);
                if constexpr (dclass(i) == c) {
                    constexpr int o = dopp(i);
                    constexpr int cx = dcx(i), cy = dcy(i), cz = dcz(i);
                    const R sf = f[i] + f[o], df = f[i] - f[o];
                    const R sg = g[i] + g[o], dg = g[i] - g[o];
                    r_ += sf;
                    p_ += sg;
                    if constexpr (cx == 1) { ax += df; bx += dg; }
                    if constexpr (cx == -1) { ax -= df; bx -= dg; }
                    if constexpr (cy == 1) { ay += df; by += dg; }
                    if constexpr (cy == -1) { ay -= df; by -= dg; }
                    if constexpr (cz == 1) { az += df; bz += dg; }
                    if constexpr (cz == -1) { az -= df; bz -= dg; }
                }
            });
            constexpr R w = (R)(c == 1 ? 2.0 / 27.0 : (c == 2 ? 1.0 / 54.0 : 1.0 / 216.0));
            rho += w * r_;
            phi += w * p_;
            jx += w * ax; jy += w * ay; jz += w * az;
            kx += w * bx; ky += w * by; kz += w * bz;
        });
    } else {
        unroll<13>([&](auto Kp) {
            constexpr int i = dpair(decltype(Kp)::value);
            constexpr int o = dopp(i);
            constexpr int cx = dcx(i), cy = dcy(i), cz = dcz(i);
            const R sf = f[i] + f[o], df = f[i] - f[o];
            const R sg = g[i] + g[o], dg = g[i] - g[o];
            rho += sf;
            phi += sg;
            if constexpr (cx == 1) { jx += df; kx += dg; }
            if constexpr (cx == -1) { jx -= df; kx -= dg; }
            if constexpr (cy == 1) { jy += df; ky += dg; }
            if constexpr (cy == -1) { jy -= df; ky -= dg; }
            if constexpr (cz == 1) { jz += df; kz += dg; }
            if constexpr (cz == -1) { jz -= df; kz -= dg; }
        });
    }
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
    {
        constexpr R w0 = (R)dweight(0);
        if constexpr (SC) {
            f[0] = K.om * f[0] + (k0 - h * k1);
            g[0] = K.omc * g[0] + ((ptb - pt * h) - pt * rho * (R)(1.0 / dweight(0)) + gshift);
        } else {
            f[0] = K.om * f[0] + w0 * (k0 - h * k1);
            g[0] = K.omc * g[0] + (w0 * (ptb - pt * h) - pt * rho);
        }
    }
    // Pairs grouped by weight class (face, edge, corner); the class constants fold w_i into the
    // per-node coefficients and live only while their class is processed.
    unroll<3>([&](auto C) {
        constexpr int c = decltype(C)::value + 1;
        // class weight; 1 in the scaled variables of shifted-FP16 storage (w_i divided out)
        constexpr R w = SC ? (R)1 : (R)(c == 1 ? 2.0 / 27.0 : (c == 2 ? 1.0 / 54.0 : 1.0 / 216.0));
        const R wk1 = w * k1;
        const R ca = (R)4.5 * wk1, cb = w * k0 - h * wk1, c3 = (R)3 * wk1;
        const R wG = w * G;
        const R ce = (R)4.5 * wG, cd = wG - h * wG, cg = (R)3 * wG;
        const R wpt = w * pt;
        const R ga = (R)4.5 * wpt, gc = (R)3 * wpt;
        R gb = w * ptb - h * wpt;
        if constexpr (SC) gb += gshift;
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
                const R fi = f[i], fo = f[o], gi = g[i], go = g[o];
                f[i] = K.om * fi + (wS + wD);
                f[o] = K.om * fo + (wS - wD);
                g[i] = K.omc * gi + (gS + gD);
                g[o] = K.omc * go + (gS - gD);
            }
        });
    });

    // store one slot: fv, gv in the working variables (shifted FP16: gv relative to T_c of the
    // slot's own node)
    auto put = [&](long long slot, R fv, R gv, double w) {
        if constexpr (SC) {
            fA[slot] = __floats2half2_rn(fv, gv);
        } else if constexpr (ST::PAIRED) {
            fA[slot] = make_float2(fv, gv);
        } else {
            ST::st_f(fA + slot, fv, w, t0);
            ST::st_g(gA + slot, gv, w, t0);
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
                put((long long)o * L + node, f[i], g[i], w);
            } else {
                // odd step: f*_i(x) streams to slot (i, x + c_i); a population leaving the box
                // becomes the next step's f_opp(i)(x) in slot (opp(i), x): bounce-back for f, and
                // for g adiabatic at y/z exits or the Dirichlet image -g* + 2 w T_wall (1 + rho)
                // with this node's density at a pure x exit (streaming.cu:3-63)
                bool out = false;
                if constexpr (!INTERIOR)
                    out = (cx == 1 && xhi) || (cx == -1 && xlo) || (cy == 1 && yhi) || (cy == -1 && ylo) ||
                          (cz == 1 && zhi) || (cz == -1 && zlo);
                if (!out) {
                    const long long off = (long long)cx + (long long)cy * geo.lx + (long long)cz * geo.lxy;
                    // shifted FP16: relative to T_c(x + c_i) = T_c(x) + tlb c_ix
                    put((long long)i * L + node + off, f[i], SC ? g[i] - K.tlb * (R)cx : g[i], w);
                } else {
                    R gv = g[i];
                    if constexpr (cx != 0) {
                        const bool ox = (cx == 1) ? xhi : xlo;
                        const bool oyz = (cy == 1 && yhi) || (cy == -1 && ylo) || (cz == 1 && zhi) || (cz == -1 && zlo);
                        if (ox && !oyz) {
                            const R tw = (cx == -1) ? K.thot : K.tcold;
                            if constexpr (SC) {
                                const R wi = (R)w;
                                gv = wall_image(wi * (g[i] + Tc), w, tw, rho) * (R)(1.0 / w) - Tc;
                            } else {
                                gv = wall_image(g[i], w, tw, rho);
                            }
                        }
                    }
                    put((long long)o * L + node, f[i], gv, w);
                }
            }
            if constexpr (OUT == OUT_MACROS_COL) {
                if constexpr (SC) {
                    b.fcol[(long long)i * L + node] = (double)((R)w * f[i]);
                    b.gcol[(long long)i * L + node] = (double)((R)w * (g[i] + Tc));
                } else {
                    b.fcol[(long long)i * L + node] = (double)f[i];
                    b.gcol[(long long)i * L + node] = (double)g[i];
                }
            }
        });
    };
    if (interior) scatter(std::true_type{});
    else scatter(std::false_type{});
}

}  // namespace rbtp
