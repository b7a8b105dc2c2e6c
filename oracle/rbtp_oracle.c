/*
 * rbtp_oracle.c — CPU oracle (TEST INFRASTRUCTURE ONLY) for the RB-ThermoParticles per-step
 * algorithm.  FP64, OpenMP over lattice nodes, sequential over particles and links.
 *
 * Each routine restates one reference routine and cites it (paths relative to the reference
 * project root).  Arithmetic is written in the reference's operation order so that, compiled with
 * -ffp-contract=off, the oracle's integer results (flags, owners, links, new-fluid lists, contact
 * pairs) are reproducible bit for bit on x86-64 and aarch64.
 *
 * Differences from the reference that do not change results:
 *   - the reference's f -> f_collide and f_temp -> f device copies (main.cu:45,48,61,64) are
 *     replaced by pointer swaps; f_col/g_col alias the post-collision buffers of the step;
 *   - double atomicAdd accumulations (ibb.cu:182-187,204; pforces.cu:32-37) run sequentially in
 *     link / pair order, which is one of the orders the reference's atomics may produce;
 *   - the CUB exclusive scans (links.cu:202,226; refill.cu:256,272) are serial integer scans.
 */
#include "rbtp_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* D3Q27 velocity set and opposite table (src_lbm/initial.cu:276-279), weights (initial.cu:281-286). */
static const int CX[27] = {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1, 0, 1, 0, -1, 0, 1, -1, -1, 1, 1, -1, -1, 1};
static const int CY[27] = {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0, -1, 0, 1, 0, -1, 1, 1, -1, -1, 1, 1, -1, -1};
static const int CZ[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
static const int OPP[27] = {0, 3, 4, 1, 2, 6, 5, 9, 10, 7, 8, 17, 18, 15, 16, 13, 14, 11, 12, 25, 26, 23, 24, 21, 22, 19, 20};

/* refill.cu:39,70 */
#define NEW_FLUID_THRESH 1.7606816861659007

typedef struct { double x, y, z; } v3;

struct orc_sim {
    rbtp_config cfg;
    int lx, ly, lz;
    long lxy, L;
    double w[27];
    /* globals.cu:18-33 */
    double tau, tauc, grav0, u0, diff, beta, thot, tcold, t0, visc, rho0, rayl, prand;
    /* populations; f_col/g_col alias the post-collision buffer of the current step */
    double *f, *g, *f_tmp, *g_tmp, *f_col, *g_col;
    double *rho, *ux, *uy, *uz, *phi, *fx, *fy, *fz, *ted, *ked;
    /* particles (globals.cu:52-124) */
    int np;
    double radius, volume, mass, inertia, heat_cap;
    double *pos[3], *vel[3], *omg[3], *th[3];
    double *facc[3], *fprev[3], *fprev2[3], *tacc[3], *tprev[3], *tprev2[3];
    double *temp, *heat, *heat_prev;
    int *ibnode, *owner, *ibnode_prev, *owner_prev;
    /* ParticleLink list (particle.h:19-29) in SoA form */
    int nlinks, lcap;
    int *lk_i, *lk_j, *lk_k, *lk_dir, *lk_pid;
    double *lk_q, *lk_rx, *lk_ry, *lk_rz;
    int nnf, nfcap;
    int *nf_node, *nf_pid;
    int *cnt, *off;
    /* contact pairs of the last apply_repulsive_forces() (test hook) */
    int ncp, cpcap;
    int *cp_p, *cp_q;
    int initialised;
};

static inline long IDX(const orc_sim *s, int ix, int iy, int iz)
{
    return (long)iz * s->lxy + (long)iy * s->lx + ix;
}

int orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

int orc_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* globals.cu:18-33 (fluid constants), 126-148 (particle constants), 150-169 (particle count). */
int orc_derive(const rbtp_config *c, rbtp_derived *d)
{
    if (!c || !d) return RBTP_ERR_ARG;
    memset(d, 0, sizeof(*d));
    const double dT = c->t_hot - c->t_cold;
    const double LX = (double)c->lx;
    d->grav0 = (c->beta != 0.0 && dT != 0.0)
                   ? c->rayleigh * c->visc * c->visc / (c->beta * dT * LX * LX * LX * c->prandtl)
                   : 0.0;
    d->tau = 3.0 * c->visc + 0.5;
    d->u0 = sqrt(fabs(d->grav0 * c->beta * dT * LX));
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
        const double lxyz = (double)((long)c->lx * c->ly * c->lz);
        const double raw = lxyz * c->particle_fraction / volume;
        d->npart = (int)floor(raw < 0.0 ? 0.0 : raw);
    }
    return RBTP_OK;
}

static void *xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

int orc_create(const rbtp_config *cfg, orc_sim **out)
{
    if (!cfg || !out) return RBTP_ERR_ARG;
    *out = NULL;
    if (cfg->lx < 3 || cfg->ly < 3 || cfg->lz < 3) return RBTP_ERR_CONFIG;
    orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
    if (!s) return RBTP_ERR_OOM;
    s->cfg = *cfg;
    s->lx = cfg->lx; s->ly = cfg->ly; s->lz = cfg->lz;
    s->lxy = (long)s->lx * s->ly;
    s->L = s->lxy * s->lz;
    for (int i = 0; i < 27; ++i)
        s->w[i] = (i == 0) ? 8.0 / 27.0 : (i <= 6) ? 2.0 / 27.0 : (i <= 18) ? 1.0 / 54.0 : 1.0 / 216.0;
    rbtp_derived d;
    orc_derive(cfg, &d);
    s->tau = d.tau; s->tauc = d.tauc; s->grav0 = d.grav0; s->u0 = d.u0; s->diff = d.diff;
    s->beta = cfg->beta; s->thot = cfg->t_hot; s->tcold = cfg->t_cold; s->t0 = cfg->t_ref;
    s->visc = cfg->visc; s->rho0 = cfg->rho0; s->rayl = cfg->rayleigh; s->prand = cfg->prandtl;
    s->np = d.npart;
    s->radius = d.particle_radius; s->volume = d.particle_volume; s->mass = d.particle_mass;
    s->inertia = d.particle_inertia; s->heat_cap = d.particle_heat_capacity;

    const size_t L = (size_t)s->L, P = 27 * L;
    s->f = xcalloc(P, 8); s->g = xcalloc(P, 8); s->f_tmp = xcalloc(P, 8); s->g_tmp = xcalloc(P, 8);
    s->rho = xcalloc(L, 8); s->ux = xcalloc(L, 8); s->uy = xcalloc(L, 8); s->uz = xcalloc(L, 8);
    s->phi = xcalloc(L, 8); s->fx = xcalloc(L, 8); s->fy = xcalloc(L, 8); s->fz = xcalloc(L, 8);
    s->ted = xcalloc(L, 8); s->ked = xcalloc(L, 8);
    s->ibnode = xcalloc(L, 4); s->owner = xcalloc(L, 4);
    s->ibnode_prev = xcalloc(L, 4); s->owner_prev = xcalloc(L, 4);
    s->cnt = xcalloc(L, 4); s->off = xcalloc(L, 4);
    const size_t np = (size_t)s->np;
    for (int a = 0; a < 3; ++a) {
        s->pos[a] = xcalloc(np, 8); s->vel[a] = xcalloc(np, 8); s->omg[a] = xcalloc(np, 8);
        s->th[a] = xcalloc(np, 8);
        s->facc[a] = xcalloc(np, 8); s->fprev[a] = xcalloc(np, 8); s->fprev2[a] = xcalloc(np, 8);
        s->tacc[a] = xcalloc(np, 8); s->tprev[a] = xcalloc(np, 8); s->tprev2[a] = xcalloc(np, 8);
    }
    s->temp = xcalloc(np, 8); s->heat = xcalloc(np, 8); s->heat_prev = xcalloc(np, 8);
    if (!s->f || !s->g || !s->f_tmp || !s->g_tmp || !s->rho || !s->ux || !s->uy || !s->uz ||
        !s->phi || !s->fx || !s->fy || !s->fz || !s->ted || !s->ked || !s->ibnode || !s->owner ||
        !s->ibnode_prev || !s->owner_prev || !s->cnt || !s->off || !s->temp || !s->heat ||
        !s->heat_prev) {
        orc_destroy(s);
        return RBTP_ERR_OOM;
    }
    for (long i = 0; i < s->L; ++i) { s->owner[i] = -1; s->owner_prev[i] = -1; }
    s->f_col = s->f_tmp;
    s->g_col = s->g_tmp;
    *out = s;
    return RBTP_OK;
}

void orc_destroy(orc_sim *s)
{
    if (!s) return;
    free(s->f); free(s->g); free(s->f_tmp); free(s->g_tmp);
    free(s->rho); free(s->ux); free(s->uy); free(s->uz); free(s->phi);
    free(s->fx); free(s->fy); free(s->fz); free(s->ted); free(s->ked);
    free(s->ibnode); free(s->owner); free(s->ibnode_prev); free(s->owner_prev);
    free(s->cnt); free(s->off);
    for (int a = 0; a < 3; ++a) {
        free(s->pos[a]); free(s->vel[a]); free(s->omg[a]); free(s->th[a]);
        free(s->facc[a]); free(s->fprev[a]); free(s->fprev2[a]);
        free(s->tacc[a]); free(s->tprev[a]); free(s->tprev2[a]);
    }
    free(s->temp); free(s->heat); free(s->heat_prev);
    free(s->lk_i); free(s->lk_j); free(s->lk_k); free(s->lk_dir); free(s->lk_pid);
    free(s->lk_q); free(s->lk_rx); free(s->lk_ry); free(s->lk_rz);
    free(s->nf_node); free(s->nf_pid); free(s->cp_p); free(s->cp_q);
    free(s);
}

int orc_npart(const orc_sim *s) { return s ? s->np : 0; }

/* ============================== lattice kernels ============================== */

/* macrovar.cu:3-34 */
static void o_macrovar(orc_sim *s)
{
    const long L = s->L;
    const double *f = s->f, *g = s->g;
#pragma omp parallel for schedule(static)
    for (long idx = 0; idx < L; ++idx) {
        double r = 0.0, jx = 0.0, jy = 0.0, jz = 0.0, ph = 0.0;
        for (int ip = 0; ip < 27; ++ip) {
            const double fv = f[ip * L + idx];
            const double gv = g[ip * L + idx];
            r += fv;
            jx += CX[ip] * fv;
            jy += CY[ip] * fv;
            jz += CZ[ip] * fv;
            ph += gv;
        }
        s->rho[idx] = r;
        s->ux[idx] = jx + 0.5 * s->fx[idx];
        s->uy[idx] = jy + 0.5 * s->fy[idx];
        s->uz[idx] = jz + 0.5 * s->fz[idx];
        s->phi[idx] = ph;
    }
}

/* macrovar.cu:36-47 */
static void o_forcing(orc_sim *s)
{
    const long L = s->L;
#pragma omp parallel for schedule(static)
    for (long idx = 0; idx < L; ++idx) {
        s->fx[idx] = s->grav0 * s->beta * (s->phi[idx] - s->t0);
        s->fy[idx] = 0.0;
        s->fz[idx] = 0.0;
    }
}

/* collision.cu:3-33 */
static void o_collision_f(orc_sim *s)
{
    const long L = s->L;
    const double tau = s->tau;
    double *f = s->f;
#pragma omp parallel for schedule(static)
    for (long idx = 0; idx < L; ++idx) {
        const double fxl = s->fx[idx];
        const double r = s->rho[idx];
        const double u = s->ux[idx], v = s->uy[idx], w = s->uz[idx];
        const double RT = 1.0 / 3.0;
        const double force_coeff = (1.0 - 0.5 / tau);
        const double u2 = u * u + v * v + w * w;
        const double uv = u2 / RT;
        for (int ip = 0; ip < 27; ++ip) {
            const double eu = (CX[ip] * u + CY[ip] * v + CZ[ip] * w) / RT;
            const double feq = s->w[ip] * (r + eu + 0.5 * (eu * eu - uv));
            const double fpop = f[ip * L + idx];
            double fchange = -(fpop - feq) / tau;
            const double feq_rho0 = s->w[ip] * (1.0 + eu + 0.5 * (eu * eu - uv));
            const double cuF = (CX[ip] - u) * fxl;
            fchange += force_coeff * cuF / RT * feq_rho0;
            f[ip * L + idx] = fpop + fchange;
        }
    }
}

/* collision.cu:35-89 */
static void o_collision_g(orc_sim *s)
{
    const long L = s->L;
    const double tauc = s->tauc;
    double *g = s->g;
#pragma omp parallel for schedule(static)
    for (long idx = 0; idx < L; ++idx) {
        const double fxl = s->fx[idx], fyl = s->fy[idx], fzl = s->fz[idx];
        const double r = s->rho[idx];
        const double ph = s->phi[idx];
        const double u = s->ux[idx], v = s->uy[idx], w = s->uz[idx];
        const double RT = 1.0 / 3.0;
        const double u2 = u * u + v * v + w * w;
        const double uv = u2 / RT;
        const double lambda0 = 1.0 - s->w[0];
        double gnx = 0.0, gny = 0.0, gnz = 0.0;
        for (int ip = 0; ip < 27; ++ip) {
            const double eu = (CX[ip] * u + CY[ip] * v + CZ[ip] * w) / RT;
            const double geq = s->w[ip] * ph * (1.0 + eu + 0.5 * (eu * eu - uv));
            const double geqnew = (ip == 0) ? (geq - lambda0 * ph * r) : (geq + s->w[ip] * ph * r);
            const double dif = g[ip * L + idx] - geqnew;
            gnx += CX[ip] * dif;
            gny += CY[ip] * dif;
            gnz += CZ[ip] * dif;
        }
        const double Ralph_coeff = (1.0 - 1.0 / (2.0 * tauc));
        const double grad_denom = r / 3.0 + 2.0 * tauc / 3.0;
        for (int ip = 0; ip < 27; ++ip) {
            const double eb = CX[ip] * fxl + CY[ip] * fyl + CZ[ip] * fzl;
            const double gneq = CX[ip] * gnx + CY[ip] * gny + CZ[ip] * gnz;
            const double gradt = -(2.0 * gneq + eb * ph) / grad_denom;
            const double Ralph = s->w[ip] * Ralph_coeff * (gradt * r + 3.0 * ph * eb);
            const double eu = (CX[ip] * u + CY[ip] * v + CZ[ip] * w) / RT;
            const double geq = s->w[ip] * ph * (1.0 + eu + 0.5 * (eu * eu - uv));
            const double geqnew = (ip == 0) ? (geq - lambda0 * ph * r) : (geq + s->w[ip] * ph * r);
            const double gpop = g[ip * L + idx];
            const double gchange = -(gpop - geqnew) / tauc + Ralph;
            g[ip * L + idx] = gpop + gchange;
        }
    }
}

/* streaming.cu:3-23: pull with half-way bounce-back at all six walls.  Reads f (post-collision),
 * writes f_tmp; the caller swaps. */
static void o_streaming_f(orc_sim *s)
{
    const long L = s->L;
    const double *f = s->f;
    double *ft = s->f_tmp;
#pragma omp parallel for collapse(2) schedule(static)
    for (int iz = 0; iz < s->lz; ++iz)
        for (int iy = 0; iy < s->ly; ++iy)
            for (int ix = 0; ix < s->lx; ++ix) {
                const long idx = IDX(s, ix, iy, iz);
                for (int ip = 0; ip < 27; ++ip) {
                    const int sx = ix - CX[ip], sy = iy - CY[ip], sz = iz - CZ[ip];
                    if (sx >= 0 && sx < s->lx && sy >= 0 && sy < s->ly && sz >= 0 && sz < s->lz)
                        ft[ip * L + idx] = f[ip * L + IDX(s, sx, sy, sz)];
                    else
                        ft[ip * L + idx] = f[OPP[ip] * L + idx];
                }
            }
}

/* streaming.cu:25-63: adiabatic z/y walls take priority, then Dirichlet x walls. */
static void o_streaming_g(orc_sim *s)
{
    const long L = s->L;
    const double *g = s->g;
    double *gt = s->g_tmp;
#pragma omp parallel for collapse(2) schedule(static)
    for (int iz = 0; iz < s->lz; ++iz)
        for (int iy = 0; iy < s->ly; ++iy)
            for (int ix = 0; ix < s->lx; ++ix) {
                const long idx = IDX(s, ix, iy, iz);
                const double density = s->rho[idx];
                for (int ip = 0; ip < 27; ++ip) {
                    const int sx = ix - CX[ip], sy = iy - CY[ip], sz = iz - CZ[ip];
                    if (sx >= 0 && sx < s->lx && sy >= 0 && sy < s->ly && sz >= 0 && sz < s->lz) {
                        gt[ip * L + idx] = g[ip * L + IDX(s, sx, sy, sz)];
                        continue;
                    }
                    const int o = OPP[ip];
                    if (sz < 0 && CZ[ip] > 0)
                        gt[ip * L + idx] = g[o * L + idx];
                    else if (sz >= s->lz && CZ[ip] < 0)
                        gt[ip * L + idx] = g[o * L + idx];
                    else if (sy < 0 && CY[ip] > 0)
                        gt[ip * L + idx] = g[o * L + idx];
                    else if (sy >= s->ly && CY[ip] < 0)
                        gt[ip * L + idx] = g[o * L + idx];
                    else if (sx < 0 && CX[ip] > 0)
                        gt[ip * L + idx] = -g[o * L + idx] + 2.0 * s->w[ip] * s->thot * (1.0 + density);
                    else if (sx >= s->lx && CX[ip] < 0)
                        gt[ip * L + idx] = -g[o * L + idx] + 2.0 * s->w[ip] * s->tcold * (1.0 + density);
                    else
                        gt[ip * L + idx] = g[o * L + idx];
                }
            }
}

static void swap_ptr(double **a, double **b) { double *t = *a; *a = *b; *b = t; }

/* ============================== particles ============================== */

/* links.cu:7-23 (smaller root of |x0 + t c - X|^2 = r^2, accepted when 0 <= t <= 1). */
int orc_link_q(int ip, double x0, double y0, double z0, double px, double py, double pz,
               double radius_sq, double *q)
{
    const double cxd = (double)CX[ip], cyd = (double)CY[ip], czd = (double)CZ[ip];
    const double dx = x0 - px, dy = y0 - py, dz = z0 - pz;
    const double a = cxd * cxd + cyd * cyd + czd * czd;
    const double b = 2.0 * (cxd * dx + cyd * dy + czd * dz);
    const double c = dx * dx + dy * dy + dz * dz - radius_sq;
    const double disc = b * b - 4.0 * a * c;
    if (disc <= 0.0) return 0;
    *q = (-b - sqrt(disc)) / (2.0 * a);
    return (*q >= 0.0 && *q <= 1.0);
}

static int ensure_links(orc_sim *s, int n)
{
    if (n <= s->lcap) return 0;
    int cap = n + n / 4 + 64;
#define GROW(p, T) do { T *t_ = (T *)realloc(p, (size_t)cap * sizeof(T)); if (!t_) return -1; p = t_; } while (0)
    GROW(s->lk_i, int); GROW(s->lk_j, int); GROW(s->lk_k, int); GROW(s->lk_dir, int); GROW(s->lk_pid, int);
    GROW(s->lk_q, double); GROW(s->lk_rx, double); GROW(s->lk_ry, double); GROW(s->lk_rz, double);
#undef GROW
    s->lcap = cap;
    return 0;
}

/* links.cu:143-256 (build_links): per-particle marking in pid order, where the first marker of a
 * node keeps it (links.cu:45), then link count, exclusive scan and fill in node order. */
static int o_build_links(orc_sim *s)
{
    const long L = s->L;
    for (long i = 0; i < L; ++i) { s->ibnode[i] = 0; s->owner[i] = -1; }
    const double r = s->radius;
    const double rsq = r * r;
    for (int p = 0; p < s->np; ++p) {
        const double px = s->pos[0][p], py = s->pos[1][p], pz = s->pos[2][p];
        int ix0 = (int)floor(px - r - 0.5), ix1 = (int)floor(px + r - 0.5);
        int iy0 = (int)floor(py - r - 0.5), iy1 = (int)floor(py + r - 0.5);
        int iz0 = (int)floor(pz - r - 0.5), iz1 = (int)floor(pz + r - 0.5);
        if (ix0 < 0) ix0 = 0;
        if (iy0 < 0) iy0 = 0;
        if (iz0 < 0) iz0 = 0;
        if (ix1 > s->lx - 1) ix1 = s->lx - 1;
        if (iy1 > s->ly - 1) iy1 = s->ly - 1;
        if (iz1 > s->lz - 1) iz1 = s->lz - 1;
        if (ix0 > ix1 || iy0 > iy1 || iz0 > iz1) continue;
        /* links.cu:25-48 */
        for (int iz = iz0; iz <= iz1; ++iz)
            for (int iy = iy0; iy <= iy1; ++iy)
                for (int ix = ix0; ix <= ix1; ++ix) {
                    const double dx = ((double)ix + 0.5) - px;
                    const double dy = ((double)iy + 0.5) - py;
                    const double dz = ((double)iz + 0.5) - pz;
                    if (dx * dx + dy * dy + dz * dz > rsq) continue;
                    const long idx = IDX(s, ix, iy, iz);
                    if (s->owner[idx] != -1) continue;
                    s->owner[idx] = p;
                    s->ibnode[idx] = 1;
                }
    }
    /* links.cu:50-87 */
#pragma omp parallel for collapse(2) schedule(static)
    for (int iz = 0; iz < s->lz; ++iz)
        for (int iy = 0; iy < s->ly; ++iy)
            for (int ix = 0; ix < s->lx; ++ix) {
                const long idx = IDX(s, ix, iy, iz);
                if (s->ibnode[idx] == 1) { s->cnt[idx] = 0; continue; }
                const double x0 = (double)ix + 0.5, y0 = (double)iy + 0.5, z0 = (double)iz + 0.5;
                int c = 0;
                for (int ip = 1; ip < 27; ++ip) {
                    const int nx = ix + CX[ip], ny = iy + CY[ip], nz = iz + CZ[ip];
                    if (nx < 0 || nx >= s->lx || ny < 0 || ny >= s->ly || nz < 0 || nz >= s->lz) continue;
                    const int pid = s->owner[IDX(s, nx, ny, nz)];
                    if (pid < 0) continue;
                    double q = 0.0;
                    if (orc_link_q(ip, x0, y0, z0, s->pos[0][pid], s->pos[1][pid], s->pos[2][pid], rsq, &q)) ++c;
                }
                s->cnt[idx] = c;
            }
    long total = 0;
    for (long i = 0; i < L; ++i) { s->off[i] = (int)total; total += s->cnt[i]; }
    if (total > 0x7fffffffL || ensure_links(s, (int)total)) return RBTP_ERR_OOM;
    s->nlinks = (int)total;
    /* links.cu:89-139 */
#pragma omp parallel for collapse(2) schedule(static)
    for (int iz = 0; iz < s->lz; ++iz)
        for (int iy = 0; iy < s->ly; ++iy)
            for (int ix = 0; ix < s->lx; ++ix) {
                const long idx = IDX(s, ix, iy, iz);
                if (s->cnt[idx] == 0 || s->ibnode[idx] == 1) continue;
                const double x0 = (double)ix + 0.5, y0 = (double)iy + 0.5, z0 = (double)iz + 0.5;
                int wi = s->off[idx];
                for (int ip = 1; ip < 27; ++ip) {
                    const int nx = ix + CX[ip], ny = iy + CY[ip], nz = iz + CZ[ip];
                    if (nx < 0 || nx >= s->lx || ny < 0 || ny >= s->ly || nz < 0 || nz >= s->lz) continue;
                    const int pid = s->owner[IDX(s, nx, ny, nz)];
                    if (pid < 0) continue;
                    double q = 0.0;
                    if (!orc_link_q(ip, x0, y0, z0, s->pos[0][pid], s->pos[1][pid], s->pos[2][pid], rsq, &q)) continue;
                    s->lk_i[wi] = ix; s->lk_j[wi] = iy; s->lk_k[wi] = iz;
                    s->lk_dir[wi] = ip; s->lk_pid[wi] = pid; s->lk_q[wi] = q;
                    s->lk_rx[wi] = q * (double)CX[ip];
                    s->lk_ry[wi] = q * (double)CY[ip];
                    s->lk_rz[wi] = q * (double)CZ[ip];
                    ++wi;
                }
            }
    return RBTP_OK;
}

/* ibb.cu:5-82: Bouzidi linear IBB for f with the moving-wall term. */
static void o_ibb_f(orc_sim *s)
{
    const long L = s->L;
    for (int t = 0; t < s->nlinks; ++t) {
        const int ip = s->lk_dir[t], o = OPP[ip];
        const int ix = s->lk_i[t], iy = s->lk_j[t], iz = s->lk_k[t];
        const long idx = IDX(s, ix, iy, iz);
        const int pid = s->lk_pid[t];
        const double q = s->lk_q[t];
        const int ix1 = ix - CX[ip], iy1 = iy - CY[ip], iz1 = iz - CZ[ip];
        const double cx = (double)ix + 0.5 + q * CX[ip];
        const double cy = (double)iy + 0.5 + q * CY[ip];
        const double cz = (double)iz + 0.5 + q * CZ[ip];
        const double relx = cx - s->pos[0][pid], rely = cy - s->pos[1][pid], relz = cz - s->pos[2][pid];
        const double uwx = s->vel[0][pid] + (relz * s->omg[1][pid] - rely * s->omg[2][pid]);
        const double uwy = s->vel[1][pid] + (relx * s->omg[2][pid] - relz * s->omg[0][pid]);
        const double uwz = s->vel[2][pid] + (rely * s->omg[0][pid] - relx * s->omg[1][pid]);
        const double evel = CX[ip] * uwx + CY[ip] * uwy + CZ[ip] * uwz;
        const double RT = 1.0 / 3.0;
        const double mom = 2.0 * s->w[ip] * s->rho0 * evel / RT;
        int handled = 0;
        if (ix1 >= 0 && ix1 < s->lx && iy1 >= 0 && iy1 < s->ly && iz1 >= 0 && iz1 < s->lz) {
            const long idx1 = IDX(s, ix1, iy1, iz1);
            if (s->ibnode[idx1] == 0) {
                const double f_here = s->f_col[ip * L + idx];
                if (q < 0.5) {
                    const double f_up = s->f_col[ip * L + idx1];
                    s->f[o * L + idx] = 2.0 * q * f_here + (1.0 - 2.0 * q) * f_up - mom;
                } else {
                    const double f_oc = s->f_col[o * L + idx];
                    const double inv_2q = 0.5 / q;
                    s->f[o * L + idx] = (f_here - mom) * inv_2q + (2.0 * q - 1.0) * inv_2q * f_oc;
                }
                handled = 1;
            }
        }
        if (!handled && s->ibnode[idx] == 0) {
            s->f[o * L + idx] = s->f_col[ip * L + idx] - mom;
            handled = 1;
        }
        if (!handled) s->f[o * L + idx] = s->f_col[ip * L + idx];
    }
}

/* ibb.cu:84-136: Dirichlet IBB for g at the particle temperature. */
static void o_ibb_g(orc_sim *s)
{
    const long L = s->L;
    for (int t = 0; t < s->nlinks; ++t) {
        const int ip = s->lk_dir[t], o = OPP[ip];
        const int ix = s->lk_i[t], iy = s->lk_j[t], iz = s->lk_k[t];
        const long idx = IDX(s, ix, iy, iz);
        const int pid = s->lk_pid[t];
        const double q = s->lk_q[t];
        const int ix1 = ix - CX[ip], iy1 = iy - CY[ip], iz1 = iz - CZ[ip];
        const double density = s->rho[idx];
        const double Tp = s->temp[pid];
        const double amp = 2.0 * s->w[ip] * Tp * (1.0 + density);
        double value;
        if (ix1 >= 0 && ix1 < s->lx && iy1 >= 0 && iy1 < s->ly && iz1 >= 0 && iz1 < s->lz &&
            s->ibnode_prev[IDX(s, ix1, iy1, iz1)] == 0) {
            const long idx1 = IDX(s, ix1, iy1, iz1);
            if (q <= 0.5) {
                const double gh = s->g_col[ip * L + idx], gu = s->g_col[ip * L + idx1];
                value = -(2.0 * q * gh + (1.0 - 2.0 * q) * gu) + amp;
            } else {
                const double gh = s->g_col[ip * L + idx], go = s->g_col[o * L + idx];
                const double inv_2q = 0.5 / q;
                value = -gh * inv_2q + amp * inv_2q + (2.0 * q - 1.0) * inv_2q * go;
            }
        } else if (s->ibnode[idx] == 0) {
            value = -s->g_col[ip * L + idx] + amp;
        } else {
            continue; /* ibb.cu:129-132 reports and skips */
        }
        s->g[o * L + idx] = value;
    }
}

/* pforces.cu:80-116 */
static void o_prepare_forces(orc_sim *s)
{
    for (int a = 0; a < 3; ++a)
        for (int p = 0; p < s->np; ++p) {
            s->fprev2[a][p] = s->fprev[a][p];
            s->tprev2[a][p] = s->tprev[a][p];
            s->fprev[a][p] = s->facc[a][p];
            s->tprev[a][p] = s->tacc[a][p];
            s->facc[a][p] = 0.0;
            s->tacc[a][p] = 0.0;
        }
}

static int push_contact(orc_sim *s, int p, int q)
{
    if (s->ncp >= s->cpcap) {
        int cap = s->cpcap * 2 + 64;
        int *a = (int *)realloc(s->cp_p, (size_t)cap * sizeof(int));
        if (!a) return -1;
        s->cp_p = a;
        int *b = (int *)realloc(s->cp_q, (size_t)cap * sizeof(int));
        if (!b) return -1;
        s->cp_q = b;
        s->cpcap = cap;
    }
    s->cp_p[s->ncp] = p;
    s->cp_q[s->ncp] = q;
    s->ncp++;
    return 0;
}

/* pforces.cu:6-38 (pairs), 40-76 (walls), 118-148 (driver). */
static void o_repulsive(orc_sim *s)
{
    const int np = s->np;
    const double radius = s->radius;
    const double coeff = s->mass * s->cfg.repforce_scale;
    const double min_gap = s->cfg.rep_min_gap, min_gap_w = s->cfg.rep_min_gap_w;
    s->ncp = 0;
    if (np > 1) {
        for (int p = 0; p < np; ++p)
            for (int q = p + 1; q < np; ++q) {
                const double dx = s->pos[0][p] - s->pos[0][q];
                const double dy = s->pos[1][p] - s->pos[1][q];
                const double dz = s->pos[2][p] - s->pos[2][q];
                const double dsq = dx * dx + dy * dy + dz * dz;
                if (dsq <= 1.0e-12) continue;
                const double dist = sqrt(dsq);
                const double hgap = dist - 2.0 * radius;
                if (hgap >= min_gap) continue;
                push_contact(s, p, q);
                const double overlap = (hgap < 0.0) ? -hgap : 0.0;
                const double factor = (min_gap - hgap) / min_gap;
                const double lub = coeff * (factor * factor / s->cfg.rep_stf0 + overlap / (min_gap * s->cfg.rep_stf1));
                const double nx = dx / dist, ny = dy / dist, nz = dz / dist;
                s->facc[0][p] += lub * nx;
                s->facc[1][p] += lub * ny;
                s->facc[2][p] += lub * nz;
                s->facc[0][q] += -lub * nx;
                s->facc[1][q] += -lub * ny;
                s->facc[2][q] += -lub * nz;
            }
    }
    const double LXd = (double)s->lx, LYd = (double)s->ly, LZd = (double)s->lz;
    for (int p = 0; p < np; ++p) {
        double fx = 0.0, fy = 0.0, fz = 0.0;
        const double x = s->pos[0][p], y = s->pos[1][p], z = s->pos[2][p];
        const double gaps[6] = {x - radius, (LXd - x) - radius, y - radius, (LYd - y) - radius,
                                z - radius, (LZd - z) - radius};
        const double nrm[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        for (int k = 0; k < 6; ++k) {
            const double gap = gaps[k];
            if (gap >= min_gap_w) continue;
            const double overlap = (gap < 0.0) ? -gap : 0.0;
            const double factor = (min_gap_w - gap) / min_gap_w;
            const double lub = coeff * (factor * factor / s->cfg.rep_stf0_w + overlap / (min_gap_w * s->cfg.rep_stf1_w));
            fx += lub * nrm[k][0];
            fy += lub * nrm[k][1];
            fz += lub * nrm[k][2];
        }
        s->facc[0][p] += fx;
        s->facc[1][p] += fy;
        s->facc[2][p] += fz;
    }
}

/* ibb.cu:138-188 (Galilean-invariant momentum exchange), applied in link order. */
static void o_particle_forces(orc_sim *s)
{
    const long L = s->L;
    for (int t = 0; t < s->nlinks; ++t) {
        const int ip = s->lk_dir[t], o = OPP[ip];
        const long idx = IDX(s, s->lk_i[t], s->lk_j[t], s->lk_k[t]);
        const int pid = s->lk_pid[t];
        const double cxp = s->lk_i[t] + 0.5 + s->lk_rx[t];
        const double cyp = s->lk_j[t] + 0.5 + s->lk_ry[t];
        const double czp = s->lk_k[t] + 0.5 + s->lk_rz[t];
        const double relx = cxp - s->pos[0][pid], rely = cyp - s->pos[1][pid], relz = czp - s->pos[2][pid];
        const double uwx = s->vel[0][pid] + (relz * s->omg[1][pid] - rely * s->omg[2][pid]);
        const double uwy = s->vel[1][pid] + (relx * s->omg[2][pid] - relz * s->omg[0][pid]);
        const double uwz = s->vel[2][pid] + (rely * s->omg[0][pid] - relx * s->omg[1][pid]);
        const double f_in = s->f_col[ip * L + idx];
        const double f_out = s->f[o * L + idx];
        const double Fx = (CX[ip] - uwx) * f_in - (CX[o] - uwx) * f_out;
        const double Fy = (CY[ip] - uwy) * f_in - (CY[o] - uwy) * f_out;
        const double Fz = (CZ[ip] - uwz) * f_in - (CZ[o] - uwz) * f_out;
        s->facc[0][pid] += Fx;
        s->facc[1][pid] += Fy;
        s->facc[2][pid] += Fz;
        s->tacc[0][pid] += rely * Fz - relz * Fy;
        s->tacc[1][pid] += relz * Fx - relx * Fz;
        s->tacc[2][pid] += relx * Fy - rely * Fx;
    }
}

/* ibb.cu:190-205, 258-271 */
static void o_particle_heat(orc_sim *s)
{
    const long L = s->L;
    for (int p = 0; p < s->np; ++p) { s->heat_prev[p] = s->heat[p]; s->heat[p] = 0.0; }
    for (int t = 0; t < s->nlinks; ++t) {
        const int ip = s->lk_dir[t], o = OPP[ip];
        const long idx = IDX(s, s->lk_i[t], s->lk_j[t], s->lk_k[t]);
        s->heat[s->lk_pid[t]] += s->g_col[ip * L + idx] - s->g[o * L + idx];
    }
}

/* move.cu:5-103 */
static void o_update_particles(orc_sim *s)
{
    const double dt = 1.0;
    const double mass = s->mass, inertia = s->inertia, hc = s->heat_cap;
    const double buoyancy = (1.0 - 1.0 / s->cfg.rho_particle_ratio) * s->grav0;
    for (int p = 0; p < s->np; ++p) {
        double vn[3], on[3];
        for (int a = 0; a < 3; ++a) {
            const double combo_f = 0.5 * s->facc[a][p] + s->fprev[a][p] + 0.5 * s->fprev2[a][p];
            const double combo_t = 0.5 * s->tacc[a][p] + s->tprev[a][p] + 0.5 * s->tprev2[a][p];
            vn[a] = s->vel[a][p] + 0.5 * dt * combo_f / mass;
            if (a == 0) vn[a] += dt * buoyancy;
            on[a] = s->omg[a][p] + 0.5 * dt * combo_t / inertia;
        }
        for (int a = 0; a < 3; ++a) {
            const double xo = s->pos[a][p];
            s->pos[a][p] = xo + 0.5 * dt * (vn[a] + s->vel[a][p]);
            s->th[a][p] += 0.5 * dt * (on[a] + s->omg[a][p]);
        }
        for (int a = 0; a < 3; ++a) { s->vel[a][p] = vn[a]; s->omg[a][p] = on[a]; }
        s->temp[p] += 0.5 * dt * (s->heat[p] + s->heat_prev[p]) / hc;
    }
}

static int ensure_nf(orc_sim *s, int n)
{
    if (n <= s->nfcap) return 0;
    int cap = n + 64;
    int *a = (int *)realloc(s->nf_node, (size_t)cap * sizeof(int));
    if (!a) return -1;
    s->nf_node = a;
    int *b = (int *)realloc(s->nf_pid, (size_t)cap * sizeof(int));
    if (!b) return -1;
    s->nf_pid = b;
    s->nfcap = cap;
    return 0;
}

/* refill.cu:244-329 (driver), 8-76 (detection), 78-240 (refill). */
static int o_refill(orc_sim *s)
{
    const long L = s->L;
    const double rad = s->radius;
    /* refill.cu:8-41 and 43-76 in node order */
    int n = 0;
    for (long idx = 0; idx < L; ++idx) {
        s->cnt[idx] = 0;
        if (s->ibnode_prev[idx] != 1 || s->ibnode[idx] == 1) continue;
        const int pid = s->owner_prev[idx];
        if (pid < 0 || pid >= s->np) continue;
        const int iz = (int)(idx / s->lxy);
        const long rem = idx - (long)iz * s->lxy;
        const int iy = (int)(rem / s->lx);
        const int ix = (int)(rem - (long)iy * s->lx);
        const double dx = ((double)ix + 0.5) - s->pos[0][pid];
        const double dy = ((double)iy + 0.5) - s->pos[1][pid];
        const double dz = ((double)iz + 0.5) - s->pos[2][pid];
        const double dist = sqrt(dx * dx + dy * dy + dz * dz);
        if (dist - rad <= NEW_FLUID_THRESH) { s->cnt[idx] = 1; ++n; }
    }
    if (ensure_nf(s, n)) return RBTP_ERR_OOM;
    s->nnf = 0;
    for (long idx = 0; idx < L; ++idx)
        if (s->cnt[idx]) { s->nf_node[s->nnf] = (int)idx; s->nf_pid[s->nnf] = s->owner_prev[idx]; s->nnf++; }

    const double lambda0 = 1.0 - s->w[0];
    const double RT = 1.0 / 3.0;
    for (int t = 0; t < s->nnf; ++t) {
        const long idx = s->nf_node[t];
        const int iz = (int)(idx / s->lxy);
        const int iy = (int)((idx - (long)iz * s->lxy) / s->lx);
        const int ix = (int)(idx - (long)iz * s->lxy - (long)iy * s->lx);
        int pid = s->nf_pid[t];
        if (pid < 0) {
            const int pp = s->owner_prev[idx];
            if (pp >= 0) pid = pp;
        }
        double rho_loc = 0.0, mx = 0.0, my = 0.0, mz = 0.0, phi_loc = 0.0;
        for (int ip = 0; ip < 27; ++ip) {
            double tf = 0.0, tg = 0.0;
            int sc = 0;
            for (int ip2 = 1; ip2 < 27; ++ip2) {
                const int x1 = ix + CX[ip2], y1 = iy + CY[ip2], z1 = iz + CZ[ip2];
                if (x1 < 0 || x1 >= s->lx || y1 < 0 || y1 >= s->ly || z1 < 0 || z1 >= s->lz) continue;
                const long i1 = IDX(s, x1, y1, z1);
                if (s->ibnode_prev[i1] != 0) continue;
                const int x2 = ix + 2 * CX[ip2], y2 = iy + 2 * CY[ip2], z2 = iz + 2 * CZ[ip2];
                const int in2 = (x2 >= 0 && x2 < s->lx && y2 >= 0 && y2 < s->ly && z2 >= 0 && z2 < s->lz);
                if (in2) {
                    const long i2 = IDX(s, x2, y2, z2);
                    if (s->ibnode_prev[i2] == 0) {
                        tf += 2.0 * s->f_col[ip * L + i1] - s->f_col[ip * L + i2];
                        tg += 2.0 * s->g_col[ip * L + i1] - s->g_col[ip * L + i2];
                        ++sc;
                        continue;
                    }
                }
                tf += s->f_col[ip * L + i1];
                tg += s->g_col[ip * L + i1];
                ++sc;
            }
            if (sc == 0) {
                double px = 0, py = 0, pz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
                double tT = s->t0;
                if (pid >= 0) {
                    px = s->pos[0][pid]; py = s->pos[1][pid]; pz = s->pos[2][pid];
                    vx = s->vel[0][pid]; vy = s->vel[1][pid]; vz = s->vel[2][pid];
                    wx = s->omg[0][pid]; wy = s->omg[1][pid]; wz = s->omg[2][pid];
                    tT = s->temp[pid];
                }
                const double relx = ((double)ix + 0.5) - px;
                const double rely = ((double)iy + 0.5) - py;
                const double relz = ((double)iz + 0.5) - pz;
                double u = vx + (relz * wy - rely * wz);
                double v = vy + (relx * wz - relz * wx);
                double w = vz + (rely * wx - relx * wy);
                if (pid < 0) { u = 0.0; v = 0.0; w = 0.0; }
                const double r = s->rho0;
                const double eu = CX[ip] * u + CY[ip] * v + CZ[ip] * w;
                const double uv = (u * u + v * v + w * w) / RT;
                tf = s->w[ip] * (r + eu + 0.5 * (eu * eu - uv));
                tg = s->w[ip] * tT * (1.0 + eu + 0.5 * (eu * eu - uv));
                if (ip == 0) tg -= lambda0 * tT * r;
                else tg += s->w[ip] * tT * r;
                sc = 1;
            }
            const double inv = 1.0 / (double)sc;
            const double fv = tf * inv, gv = tg * inv;
            s->f[ip * L + idx] = fv;
            s->g[ip * L + idx] = gv;
            rho_loc += fv;
            mx += CX[ip] * fv;
            my += CY[ip] * fv;
            mz += CZ[ip] * fv;
            phi_loc += gv;
        }
        s->rho[idx] = rho_loc;
        if (rho_loc > 1e-12) {
            const double inv_rho = 1.0 / rho_loc;
            s->ux[idx] = mx * inv_rho;
            s->uy[idx] = my * inv_rho;
            s->uz[idx] = mz * inv_rho;
        } else {
            s->ux[idx] = 0.0; s->uy[idx] = 0.0; s->uz[idx] = 0.0;
        }
        s->phi[idx] = phi_loc;
        s->fx[idx] = 0.0; s->fy[idx] = 0.0; s->fz[idx] = 0.0;
    }
    memcpy(s->ibnode_prev, s->ibnode, (size_t)L * sizeof(int));
    memcpy(s->owner_prev, s->owner, (size_t)L * sizeof(int));
    return RBTP_OK;
}

/* ============================== init / restart ============================== */

/* pinit.cu:97-144 (glibc srand/rand rejection sampling, minimum gap r/3). */
static int o_generate_positions(orc_sim *s)
{
    const double r = s->radius;
    srand((unsigned)s->cfg.particle_rand_seed);
    const double mnx = 1.5 * r, mny = 1.5 * r, mnz = 1.5 * r;
    const double spx = (double)s->lx - 3.0 * r, spy = (double)s->ly - 3.0 * r, spz = (double)s->lz - 3.0 * r;
    long counter = 0;
    for (int p = 0; p < s->np; ++p) {
        for (;;) {
            const double rx = (double)rand() / (double)RAND_MAX;
            const double ry = (double)rand() / (double)RAND_MAX;
            const double rz = (double)rand() / (double)RAND_MAX;
            const double x = mnx + rx * spx, y = mny + ry * spy, z = mnz + rz * spz;
            int ok = 1;
            for (int q = 0; q < p; ++q) {
                const double dx = x - s->pos[0][q], dy = y - s->pos[1][q], dz = z - s->pos[2][q];
                const double dist = sqrt(dx * dx + dy * dy + dz * dz);
                if (dist - 2.0 * r < r / 3.0) {
                    counter++;
                    if (counter > 1000000) return RBTP_ERR_PLACEMENT;
                    ok = 0;
                    break;
                }
            }
            if (ok) { s->pos[0][p] = x; s->pos[1][p] = y; s->pos[2][p] = z; break; }
        }
    }
    return RBTP_OK;
}

/* pinit.cu:146-179: node inside the lowest-pid sphere (<= r^2), no bounding box. */
static void o_initial_ibnode(orc_sim *s)
{
    const double rsq = s->radius * s->radius;
#pragma omp parallel for collapse(2) schedule(static)
    for (int iz = 0; iz < s->lz; ++iz)
        for (int iy = 0; iy < s->ly; ++iy)
            for (int ix = 0; ix < s->lx; ++ix) {
                const long idx = IDX(s, ix, iy, iz);
                int own = -1;
                for (int p = 0; p < s->np; ++p) {
                    const double dx = ((double)ix + 0.5) - s->pos[0][p];
                    const double dy = ((double)iy + 0.5) - s->pos[1][p];
                    const double dz = ((double)iz + 0.5) - s->pos[2][p];
                    if (dx * dx + dy * dy + dz * dz <= rsq) { own = p; break; }
                }
                s->owner[idx] = own;
                s->ibnode[idx] = own >= 0;
            }
    memcpy(s->ibnode_prev, s->ibnode, (size_t)s->L * sizeof(int));
    memcpy(s->owner_prev, s->owner, (size_t)s->L * sizeof(int));
}

/* initial.cu:240-333 fresh branch with init_f/init_g (initial.cu:335-397). */
int orc_init_fresh(orc_sim *s)
{
    if (!s) return RBTP_ERR_ARG;
    const long L = s->L;
    if (s->np > 0) {
        for (int a = 0; a < 3; ++a)
            for (int p = 0; p < s->np; ++p) {
                s->vel[a][p] = s->omg[a][p] = s->th[a][p] = 0.0;
                s->facc[a][p] = s->fprev[a][p] = s->fprev2[a][p] = 0.0;
                s->tacc[a][p] = s->tprev[a][p] = s->tprev2[a][p] = 0.0;
            }
        for (int p = 0; p < s->np; ++p) { s->heat[p] = s->heat_prev[p] = 0.0; }
        int st = o_generate_positions(s);
        if (st) return st;
        for (int p = 0; p < s->np; ++p) s->temp[p] = s->cfg.particle_init_temp;
        o_initial_ibnode(s);
    }
    const double RT = 1.0 / 3.0;
    const double lambda0 = 1.0 - s->w[0];
#pragma omp parallel for schedule(static)
    for (long idx = 0; idx < L; ++idx) {
        /* init_f: zero velocity, deviation density 0, rho field set to RHO0 */
        const double r0 = 0.0, u = 0.0, v = 0.0, w = 0.0;
        const double uv = (u * u + v * v + w * w) / RT;
        s->rho[idx] = s->rho0;
        s->ux[idx] = u; s->uy[idx] = v; s->uz[idx] = w;
        for (int ip = 0; ip < 27; ++ip) {
            const double eu = (CX[ip] * u + CY[ip] * v + CZ[ip] * w) / RT;
            s->f[ip * L + idx] = s->w[ip] * (r0 + eu + 0.5 * (eu * eu - uv));
        }
        /* init_g: uses rho[idx] (= RHO0) written by init_f */
        const double r = s->rho[idx];
        const double tT = s->t0;
        s->phi[idx] = tT;
        s->fx[idx] = s->grav0 * s->beta * (tT - s->t0);
        s->fy[idx] = 0.0; s->fz[idx] = 0.0;
        s->ted[idx] = 0.0;
        for (int ip = 0; ip < 27; ++ip) {
            const double eu = (CX[ip] * u + CY[ip] * v + CZ[ip] * w) / RT;
            double geq = s->w[ip] * tT * (1.0 + eu + 0.5 * (eu * eu - uv));
            if (ip == 0) geq -= lambda0 * tT * r;
            else geq += s->w[ip] * tT * r;
            s->g[ip * L + idx] = geq;
        }
    }
    memcpy(s->f_tmp, s->f, (size_t)(27 * L) * sizeof(double));
    memcpy(s->g_tmp, s->g, (size_t)(27 * L) * sizeof(double));
    s->f_col = s->f_tmp; s->g_col = s->g_tmp;
    if (s->np > 0) {
        int st = o_build_links(s);
        if (st) return st;
    }
    s->nnf = 0;
    s->initialised = 1;
    return RBTP_OK;
}

/* Array form of load_restart_state (initial.cu:194-236). */
int orc_load_state(orc_sim *s, const double *f, const double *g, const double *flow7,
                   const double *particles)
{
    if (!s || !f || !g) return RBTP_ERR_ARG;
    if (s->np > 0 && !particles) return RBTP_ERR_ARG;
    const long L = s->L;
    memcpy(s->f, f, (size_t)(27 * L) * sizeof(double));
    memcpy(s->g, g, (size_t)(27 * L) * sizeof(double));
    if (s->np > 0) {
        /* initial.cu:74-170 (column order of output_part.cu:91-115) */
        for (int p = 0; p < s->np; ++p) {
            const double *c = particles + (size_t)p * RBTP_PARTICLE_COLS;
            for (int a = 0; a < 3; ++a) {
                s->pos[a][p] = c[0 + a];
                s->vel[a][p] = c[3 + a];
                s->facc[a][p] = c[6 + a];
                s->fprev[a][p] = c[9 + a];
                s->fprev2[a][p] = c[12 + a];
                s->th[a][p] = c[15 + a];
                s->omg[a][p] = c[18 + a];
                s->tacc[a][p] = c[21 + a];
                s->tprev[a][p] = c[24 + a];
                s->tprev2[a][p] = c[27 + a];
            }
            s->temp[p] = c[30];
            s->heat[p] = c[31];
            s->heat_prev[p] = c[32];
        }
        int st = o_build_links(s);
        if (st) return st;
    }
    memcpy(s->f_tmp, s->f, (size_t)(27 * L) * sizeof(double));
    memcpy(s->g_tmp, s->g, (size_t)(27 * L) * sizeof(double));
    s->f_col = s->f_tmp; s->g_col = s->g_tmp;
    if (flow7) {
        memcpy(s->rho, flow7 + 0 * L, (size_t)L * 8);
        memcpy(s->ux, flow7 + 1 * L, (size_t)L * 8);
        memcpy(s->uy, flow7 + 2 * L, (size_t)L * 8);
        memcpy(s->uz, flow7 + 3 * L, (size_t)L * 8);
        memcpy(s->phi, flow7 + 4 * L, (size_t)L * 8);
        memcpy(s->ted, flow7 + 5 * L, (size_t)L * 8);
        memcpy(s->ked, flow7 + 6 * L, (size_t)L * 8);
    } else {
        for (long i = 0; i < L; ++i) s->fx[i] = s->fy[i] = s->fz[i] = 0.0;
        o_macrovar(s);
        memset(s->ted, 0, (size_t)L * 8);
        memset(s->ked, 0, (size_t)L * 8);
    }
    o_forcing(s);
    if (s->np > 0) {
        memcpy(s->ibnode_prev, s->ibnode, (size_t)L * sizeof(int));
        memcpy(s->owner_prev, s->owner, (size_t)L * sizeof(int));
    }
    s->nnf = 0;
    s->initialised = 1;
    return RBTP_OK;
}

/* main.cu:32-85: one full step per iteration. */
int orc_step(orc_sim *s, int nsteps)
{
    if (!s) return RBTP_ERR_ARG;
    if (!s->initialised) return RBTP_ERR_STATE;
    const int parts = s->cfg.activate_particles && s->np > 0;
    for (int it = 0; it < nsteps; ++it) {
        o_macrovar(s);
        o_forcing(s);
        o_collision_f(s);
        o_streaming_f(s);
        swap_ptr(&s->f, &s->f_tmp);
        s->f_col = s->f_tmp;
        if (parts) o_ibb_f(s);
        o_collision_g(s);
        o_streaming_g(s);
        swap_ptr(&s->g, &s->g_tmp);
        s->g_col = s->g_tmp;
        if (parts) {
            o_ibb_g(s);
            o_prepare_forces(s);
            o_repulsive(s);
            o_particle_forces(s);
            o_particle_heat(s);
            o_update_particles(s);
            int st = o_build_links(s);
            if (st) return st;
            st = o_refill(s);
            if (st) return st;
        }
    }
    return RBTP_OK;
}

/* ============================== export ============================== */

int orc_get_fg(const orc_sim *s, double *f, double *g)
{
    if (!s) return RBTP_ERR_ARG;
    const size_t n = (size_t)(27 * s->L) * sizeof(double);
    if (f) memcpy(f, s->f, n);
    if (g) memcpy(g, s->g, n);
    return RBTP_OK;
}

int orc_get_macros(const orc_sim *s, double *rho, double *ux, double *uy, double *uz, double *phi,
                   double *force_x)
{
    if (!s) return RBTP_ERR_ARG;
    const size_t n = (size_t)s->L * sizeof(double);
    if (rho) memcpy(rho, s->rho, n);
    if (ux) memcpy(ux, s->ux, n);
    if (uy) memcpy(uy, s->uy, n);
    if (uz) memcpy(uz, s->uz, n);
    if (phi) memcpy(phi, s->phi, n);
    if (force_x) memcpy(force_x, s->fx, n);
    return RBTP_OK;
}

int orc_get_particles(const orc_sim *s, double *out)
{
    if (!s || (!out && s->np)) return RBTP_ERR_ARG;
    for (int p = 0; p < s->np; ++p) {
        double *c = out + (size_t)p * RBTP_PARTICLE_COLS;
        for (int a = 0; a < 3; ++a) {
            c[0 + a] = s->pos[a][p]; c[3 + a] = s->vel[a][p]; c[6 + a] = s->facc[a][p];
            c[9 + a] = s->fprev[a][p]; c[12 + a] = s->fprev2[a][p]; c[15 + a] = s->th[a][p];
            c[18 + a] = s->omg[a][p]; c[21 + a] = s->tacc[a][p]; c[24 + a] = s->tprev[a][p];
            c[27 + a] = s->tprev2[a][p];
        }
        c[30] = s->temp[p]; c[31] = s->heat[p]; c[32] = s->heat_prev[p];
    }
    return RBTP_OK;
}

int orc_get_flags(const orc_sim *s, int *owner, int *owner_prev)
{
    if (!s) return RBTP_ERR_ARG;
    if (owner) memcpy(owner, s->owner, (size_t)s->L * sizeof(int));
    if (owner_prev) memcpy(owner_prev, s->owner_prev, (size_t)s->L * sizeof(int));
    return RBTP_OK;
}

int orc_get_links(const orc_sim *s, int *n, int *node, int *dir, int *pid, double *q, int cap)
{
    if (!s || !n) return RBTP_ERR_ARG;
    *n = s->nlinks;
    if (!node && !dir && !pid && !q) return RBTP_OK;
    if (cap < s->nlinks) return RBTP_ERR_ARG;
    for (int t = 0; t < s->nlinks; ++t) {
        if (node) node[t] = (int)IDX(s, s->lk_i[t], s->lk_j[t], s->lk_k[t]);
        if (dir) dir[t] = s->lk_dir[t];
        if (pid) pid[t] = s->lk_pid[t];
        if (q) q[t] = s->lk_q[t];
    }
    return RBTP_OK;
}

int orc_get_new_fluid(const orc_sim *s, int *n, int *node, int *pid, int cap)
{
    if (!s || !n) return RBTP_ERR_ARG;
    *n = s->nnf;
    if (!node && !pid) return RBTP_OK;
    if (cap < s->nnf) return RBTP_ERR_ARG;
    for (int t = 0; t < s->nnf; ++t) {
        if (node) node[t] = s->nf_node[t];
        if (pid) pid[t] = s->nf_pid[t];
    }
    return RBTP_OK;
}

int orc_get_contacts(const orc_sim *s, int *n, int *p, int *q, int cap)
{
    if (!s || !n) return RBTP_ERR_ARG;
    *n = s->ncp;
    if (!p && !q) return RBTP_OK;
    if (cap < s->ncp) return RBTP_ERR_ARG;
    for (int t = 0; t < s->ncp; ++t) {
        if (p) p[t] = s->cp_p[t];
        if (q) q[t] = s->cp_q[t];
    }
    return RBTP_OK;
}

int orc_set_positions_and_build(orc_sim *s, const double *pos)
{
    if (!s || (!pos && s->np)) return RBTP_ERR_ARG;
    for (int p = 0; p < s->np; ++p)
        for (int a = 0; a < 3; ++a) s->pos[a][p] = pos[3 * p + a];
    return o_build_links(s);
}

/* ============================== diagnostics ============================== */

/* output_statis.cu:5-60: solid nodes report the rigid-body velocity and the particle temperature. */
static void o_overwrite(const orc_sim *s, double *rho, double *ux, double *uy, double *uz,
                        double *phi, double *ted, double *ked)
{
    if (!(s->cfg.activate_particles && s->np > 0)) return;
    for (long idx = 0; idx < s->L; ++idx) {
        if (s->ibnode[idx] == 0) continue;
        const int pid = s->owner[idx];
        if (pid < 0 || pid >= s->np) continue;
        const int iz = (int)(idx / s->lxy);
        const int iy = (int)((idx - (long)iz * s->lxy) / s->lx);
        const int ix = (int)(idx - (long)iz * s->lxy - (long)iy * s->lx);
        const double relx = ((double)ix + 0.5) - s->pos[0][pid];
        const double rely = ((double)iy + 0.5) - s->pos[1][pid];
        const double relz = ((double)iz + 0.5) - s->pos[2][pid];
        const double vx = s->vel[0][pid] + (relz * s->omg[1][pid] - rely * s->omg[2][pid]);
        const double vy = s->vel[1][pid] + (relx * s->omg[2][pid] - relz * s->omg[0][pid]);
        const double vz = s->vel[2][pid] + (rely * s->omg[0][pid] - relx * s->omg[1][pid]);
        if (rho) rho[idx] = s->rho0;
        if (ux) ux[idx] = vx;
        if (uy) uy[idx] = vy;
        if (uz) uz[idx] = vz;
        if (phi) phi[idx] = s->temp[pid];
        if (ted) ted[idx] = 0.0;
        if (ked) ked[idx] = 0.0;
    }
}

/* output_statis.cu:64-109 */
int orc_means(orc_sim *s, double out[4])
{
    if (!s || !out) return RBTP_ERR_ARG;
    const long L = s->L;
    double *ux = malloc((size_t)L * 8), *uy = malloc((size_t)L * 8), *uz = malloc((size_t)L * 8),
           *ph = malloc((size_t)L * 8);
    if (!ux || !uy || !uz || !ph) { free(ux); free(uy); free(uz); free(ph); return RBTP_ERR_OOM; }
    memcpy(ux, s->ux, (size_t)L * 8); memcpy(uy, s->uy, (size_t)L * 8);
    memcpy(uz, s->uz, (size_t)L * 8); memcpy(ph, s->phi, (size_t)L * 8);
    o_overwrite(s, NULL, ux, uy, uz, ph, NULL, NULL);
    double a = 0, b = 0, c = 0, d = 0;
    for (long i = 0; i < L; ++i) { a += ux[i]; b += uy[i]; c += uz[i]; d += ph[i]; }
    out[0] = a / L; out[1] = b / L; out[2] = c / L; out[3] = d / L;
    free(ux); free(uy); free(uz); free(ph);
    return RBTP_OK;
}

/* output_statis.cu:111-223 */
int orc_nu(orc_sim *s, int istep, rbtp_nu_row *row)
{
    if (!s || !row) return RBTP_ERR_ARG;
    const int parts = s->cfg.activate_particles && s->np > 0;
    const double vf = s->cfg.particle_fraction;
    const double ff = fmax(0.0, 1.0 - vf);
    double avg_f = 0.0, avg_p = 0.0;
    for (int ix = 0; ix < s->lx; ++ix) {
        double sf = 0.0, sp = 0.0;
        int nf = 0, np = 0;
        for (int iz = 0; iz < s->lz; ++iz)
            for (int iy = 0; iy < s->ly; ++iy) {
                const long idx = IDX(s, ix, iy, iz);
                const int fluid = parts ? (s->ibnode[idx] == 0) : 1;
                if (fluid) { sf += s->ux[idx] * s->phi[idx]; nf++; }
                else { sp += s->ux[idx] * s->phi[idx]; np++; }
            }
        if (nf > 0) avg_f += sf / (double)nf;
        if (np > 0) avg_p += sp / (double)np;
    }
    avg_f /= (double)s->lx;
    avg_p /= (double)s->lx;
    const double cond = s->diff * (s->thot - s->tcold) / (double)s->lx;
    double nbf = ff, nbp = 0.0;
    if (cond != 0.0) {
        nbf += ff * (avg_f / cond);
        nbp = vf * s->cfg.cp_particle_ratio * (avg_p / cond);
    }
    double bottom = 0.0, top = 0.0;
    int bc = 0, tc = 0;
    for (int iz = 0; iz < s->lz; ++iz)
        for (int iy = 0; iy < s->ly; ++iy) {
            const long ib = IDX(s, 0, iy, iz);
            if (parts ? (s->ibnode[ib] == 0) : 1) { bottom += (s->thot - s->phi[ib]) / 0.5; bc++; }
            const long it = IDX(s, s->lx - 1, iy, iz);
            if (parts ? (s->ibnode[it] == 0) : 1) { top += (s->phi[it] - s->tcold) / 0.5; tc++; }
        }
    const double area = (double)s->ly * (double)s->lz;
    const double scale = (double)s->lx / (s->thot - s->tcold);
    row->step = (double)istep;
    row->volume_fraction = vf;
    row->nu_bulk = nbf + nbp;
    row->nu_top = tc > 0 ? (top / area) * scale : 0.0;
    row->nu_bottom = bc > 0 ? (bottom / area) * scale : 0.0;
    row->nu_bulk_fluid = nbf;
    row->nu_bulk_part = nbp;
    return RBTP_OK;
}

/* output_statis.cu:225-285 */
int orc_profile(orc_sim *s, double *out)
{
    if (!s || !out) return RBTP_ERR_ARG;
    const long L = s->L;
    double *ux = malloc((size_t)L * 8), *uy = malloc((size_t)L * 8), *uz = malloc((size_t)L * 8),
           *ph = malloc((size_t)L * 8);
    if (!ux || !uy || !uz || !ph) { free(ux); free(uy); free(uz); free(ph); return RBTP_ERR_OOM; }
    memcpy(ux, s->ux, (size_t)L * 8); memcpy(uy, s->uy, (size_t)L * 8);
    memcpy(uz, s->uz, (size_t)L * 8); memcpy(ph, s->phi, (size_t)L * 8);
    o_overwrite(s, NULL, ux, uy, uz, ph, NULL, NULL);
    for (int ix = 0; ix < s->lx; ++ix) {
        double a = 0, b = 0, c = 0, d = 0;
        int cnt = 0;
        for (int iz = 0; iz < s->lz; ++iz)
            for (int iy = 0; iy < s->ly; ++iy) {
                const long idx = IDX(s, ix, iy, iz);
                a += ux[idx]; b += uy[idx]; c += uz[idx]; d += ph[idx];
                cnt++;
            }
        const double inv = cnt > 0 ? 1.0 / (double)cnt : 0.0;
        out[4 * ix + 0] = a * inv; out[4 * ix + 1] = b * inv;
        out[4 * ix + 2] = c * inv; out[4 * ix + 3] = d * inv;
    }
    free(ux); free(uy); free(uz); free(ph);
    return RBTP_OK;
}

/* collision.cu:91-152 (Ked) and 154-198 (ted) on the step's post-collision populations, then
 * output_flow's solid-node overwrite (output_flow.cu:95). */
int orc_dissipation(orc_sim *s, double *ted, double *ked)
{
    if (!s) return RBTP_ERR_ARG;
    const long L = s->L;
    const double tau = s->tau, tauc = s->tauc, visc = s->visc, diff = s->diff;
#pragma omp parallel for schedule(static)
    for (long idx = 0; idx < L; ++idx) {
        const double fxl = s->fx[idx], fyl = s->fy[idx], fzl = s->fz[idx];
        const double r = s->rho[idx], ph = s->phi[idx];
        const double u = s->ux[idx], v = s->uy[idx], w = s->uz[idx];
        const double RT = 1.0 / 3.0;
        const double u2 = u * u + v * v + w * w;
        const double uv = u2 / RT;
        const double bu = fxl * u + fyl * v + fzl * w;
        double txx = 0, txy = 0, txz = 0, tyy = 0, tyz = 0, tzz = 0;
        for (int ip = 0; ip < 27; ++ip) {
            const double eu = (CX[ip] * u + CY[ip] * v + CZ[ip] * w) / RT;
            const double feq = s->w[ip] * (r + eu + 0.5 * (eu * eu - uv));
            const double fneq = s->f_col[ip * L + idx] - feq;
            const double cidotF = CX[ip] * fxl + CY[ip] * fyl + CZ[ip] * fzl;
            const double feq_term = 0.5 * (cidotF - bu) * feq / RT;
            txx += CX[ip] * CX[ip] * (fneq + feq_term);
            txy += CX[ip] * CY[ip] * (fneq + feq_term);
            txz += CX[ip] * CZ[ip] * (fneq + feq_term);
            tyy += CY[ip] * CY[ip] * (fneq + feq_term);
            tyz += CY[ip] * CZ[ip] * (fneq + feq_term);
            tzz += CZ[ip] * CZ[ip] * (fneq + feq_term);
        }
        const double coeff = -(1.0 - 0.5 / tau);
        txx *= coeff; txy *= coeff; txz *= coeff; tyy *= coeff; tyz *= coeff; tzz *= coeff;
        const double Sxx = txx / (2.0 * visc), Sxy = txy / (2.0 * visc), Sxz = txz / (2.0 * visc);
        const double Syy = tyy / (2.0 * visc), Syz = tyz / (2.0 * visc), Szz = tzz / (2.0 * visc);
        s->ked[idx] = 0.5 * visc * (4.0 * (Sxx * Sxx + Syy * Syy + Szz * Szz) +
                                    8.0 * (Sxy * Sxy + Sxz * Sxz + Syz * Syz));
        const double lambda0 = 1.0 - s->w[0];
        double gnx = 0.0, gny = 0.0, gnz = 0.0;
        for (int ip = 0; ip < 27; ++ip) {
            const double eu = (CX[ip] * u + CY[ip] * v + CZ[ip] * w) / RT;
            const double geq = s->w[ip] * ph * (1.0 + eu + 0.5 * (eu * eu - uv));
            const double geqnew = (ip == 0) ? (geq - lambda0 * ph * r) : (geq + s->w[ip] * ph * r);
            const double dif = s->g_col[ip * L + idx] - geqnew;
            gnx += CX[ip] * dif;
            gny += CY[ip] * dif;
            gnz += CZ[ip] * dif;
        }
        const double p = r * RT;
        const double den = 2.0 * tauc * RT + p;
        const double tx = -(2.0 * gnx + ph * fxl) / den;
        const double ty = -(2.0 * gny + ph * fyl) / den;
        const double tz = -(2.0 * gnz + ph * fzl) / den;
        s->ted[idx] = (diff > 0.0) ? diff * (tx * tx + ty * ty + tz * tz) : 0.0;
    }
    if (ted) memcpy(ted, s->ted, (size_t)L * 8);
    if (ked) memcpy(ked, s->ked, (size_t)L * 8);
    if (ted || ked) o_overwrite(s, NULL, NULL, NULL, NULL, NULL, ted, ked);
    return RBTP_OK;
}
