/*
 * rbtp.h — C ABI of librbtp, the GB300 (sm_103a) implementation of the RB-ThermoParticles
 * per-timestep hot path: D3Q27 double-distribution BGK lattice Boltzmann (f = flow, g =
 * temperature) for Rayleigh–Bénard convection with buoyancy along x, plus finite-size thermal
 * spheres coupled by interpolated bounce-back (IBB), new-fluid refill and soft-sphere contacts.
 *
 * The reference has no FFI layer: its boundary is a set of `void f(void)` host entry points over
 * global device state (include/lbm.h:52-84, include/particle.h:110-122) driven by main.cu:32-118,
 * with compile-time case macros (parameters.h:1-55).  Each entry point below names the reference
 * code it replaces.  Every function returns an int status (RBTP_OK == 0, negative on error) and
 * never exits the process (the reference calls exit() from CHECK_CUDA_ERROR, include/lbm.h:87-95).
 *
 * Ownership: the handle owns all device memory and one CUDA stream; host buffers passed in are
 * only read/written during the call.  Handles are not thread-safe; use one handle per thread.
 * Arrays use the reference layout: populations SoA [ip][z][y][x] (index ip*L + z*LX*LY + y*LX + x),
 * scalar fields [z][y][x], all FP64 on the host side regardless of the device storage mode.
 */
#ifndef RBTP_H
#define RBTP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------ */
#define RBTP_OK              0
#define RBTP_ERR_CUDA       -1  /* a CUDA runtime call failed (message via rbtp_last_error)     */
#define RBTP_ERR_CONFIG     -2  /* invalid configuration                                        */
#define RBTP_ERR_OOM        -3  /* device allocation failed                                     */
#define RBTP_ERR_NONFINITE  -4  /* NaN/Inf detected by the on-device watchdog                   */
#define RBTP_ERR_TIMEOUT    -5  /* a bounded device wait gave up                                */
#define RBTP_ERR_IO         -6  /* restart/output file missing, short or malformed              */
#define RBTP_ERR_STATE      -7  /* call-order violation (e.g. step before init)                 */
#define RBTP_ERR_CAPACITY   -8  /* a device list exceeded its proven bound (should not happen)  */
#define RBTP_ERR_ARG        -9  /* bad argument (null pointer, short buffer)                    */
#define RBTP_ERR_PLACEMENT -10  /* particles could not be placed (pinit.cu:129-134 limit)       */
#define RBTP_ERR_NODEVICE  -11  /* no CUDA device visible                                       */

/* ---- device storage of the populations ---------------------------------------------------- */
#define RBTP_STORE_F64   0  /* FP64 storage + FP64 arithmetic: the parity path                */
#define RBTP_STORE_F32   1  /* FP32 storage + FP32 arithmetic                                 */
#define RBTP_STORE_F16S  2  /* FP16 storage of w_i-scaled, T0-shifted populations, FP32 math  */

/* Runtime mirror of every parameters.h macro (parameters.h:4-53).  BLOCK_X/Y/Z are replaced by
 * the library's own launch shapes; NPOP is fixed at 27. */
typedef struct rbtp_config {
    int lx, ly, lz;                         /* LX LY LZ                                   */
    int continuous_steps;                   /* CONTINUOUS_STEPS (restart step)            */
    int nend, ndiag, nflowout, nnuout, nout_p;
    double rayleigh, prandtl;               /* RAYLEIGH PRANDTL                           */
    double t_hot, t_cold, t_ref;            /* T_HOT T_COLD T_REF                         */
    double beta, visc, rho0;                /* BETA VISC RHO0                             */
    int activate_particles;                 /* ACTIVATE_PARTICLES                         */
    int particle_rand_seed;                 /* PARTICLE_RAND_SEED                         */
    double particle_fraction;               /* PARTICLE_FRACTION                          */
    double particle_diam_frac;              /* PARTICLE_DIAM_FRAC                         */
    double cp_particle_ratio, cp_fluid;     /* CP_PARTICLE_RATIO CP_FLUID                 */
    double rho_particle_ratio;              /* RHO_PARTICLE_RATIO                         */
    double repforce_scale;                  /* REPFORCE_SCALE                             */
    double particle_init_temp;              /* PARTICLE_INIT_TEMP                         */
    double rep_min_gap, rep_min_gap_w;      /* REP_MIN_GAP REP_MIN_GAP_W                  */
    double rep_stf0, rep_stf1;              /* REP_STF0 REP_STF1                          */
    double rep_stf0_w, rep_stf1_w;          /* REP_STF0_W REP_STF1_W                      */
    int storage;                            /* RBTP_STORE_*                               */
    int reserved[7];
} rbtp_config;

/* Constants derived from a config exactly as src_lbm/globals.cu:18-33,126-169 derive them. */
typedef struct rbtp_derived {
    double tau, tauc, grav0, u0, diff;
    double particle_radius, particle_volume, particle_mass, particle_inertia, particle_heat_capacity;
    int npart;
    int reserved;
} rbtp_derived;

/* One row of Nu_%.2e.txt (output/output_statis.cu:217-219), in file column order. */
typedef struct rbtp_nu_row {
    double step, volume_fraction, nu_bulk, nu_top, nu_bottom, nu_bulk_fluid, nu_bulk_part;
} rbtp_nu_row;

/* Number of doubles per particle in the particle-state exchange format: the 33 numeric columns of
 * pos/pos_%09d.txt after the pid (output/output_part.cu:91-115), same order:
 *   pos xyz, vel xyz, force xyz, force_prev xyz, force_prev2 xyz, theta xyz, omega xyz,
 *   torque xyz, torque_prev xyz, torque_prev2 xyz, temp, heat, heat_prev. */
#define RBTP_PARTICLE_COLS 33

typedef struct rbtp_handle rbtp_handle;

/* Fill a config with the reference defaults (parameters.h:4-53). */
static inline void rbtp_config_fill_defaults(rbtp_config *c)
{
    c->lx = 320; c->ly = 320; c->lz = 160;
    c->continuous_steps = 0;
    c->nend = 1000000; c->ndiag = 125; c->nflowout = 25000; c->nnuout = 125; c->nout_p = 125;
    c->rayleigh = 1.0e7; c->prandtl = 0.71;
    c->t_hot = 1.0; c->t_cold = 0.0; c->t_ref = 0.5;
    c->beta = 0.0000625; c->visc = 0.01206; c->rho0 = 1.0;
    c->activate_particles = 1; c->particle_rand_seed = 86143;
    c->particle_fraction = 0.05; c->particle_diam_frac = 1.0 / 20.0;
    c->cp_particle_ratio = 10.0; c->cp_fluid = 1.0; c->rho_particle_ratio = 1.0;
    c->repforce_scale = 2.0e-4; c->particle_init_temp = (0.0 + 1.0) / 2;
    c->rep_min_gap = 2.0; c->rep_min_gap_w = 2.0;
    c->rep_stf0 = 0.025; c->rep_stf1 = 0.002; c->rep_stf0_w = 0.025; c->rep_stf1_w = 0.002;
    c->storage = RBTP_STORE_F64;
    for (int i = 0; i < 7; ++i) c->reserved[i] = 0;
}

/* ---- configuration ------------------------------------------------------------------------ */
void rbtp_config_default(rbtp_config *cfg);                    /* parameters.h:4-53              */
int  rbtp_derive(const rbtp_config *cfg, rbtp_derived *out);   /* globals.cu:18-33,126-169       */
const char *rbtp_status_string(int status);
const char *rbtp_version(void);

/* ---- lifetime ------------------------------------------------------------------------------ */
/* Allocates the device state of one cavity (replaces the allocation half of initialize(),
 * src_lbm/initial.cu:240-275, and of init_particles(), src_part/pinit.cu:8-95).  The lattice
 * tables and derived constants are fixed at creation (initial.cu:276-303). */
int  rbtp_create(const rbtp_config *cfg, rbtp_handle **out);
/* Frees everything the handle owns (replaces main.cu:141-268). */
int  rbtp_destroy(rbtp_handle *h);
const char *rbtp_last_error(const rbtp_handle *h);

/* Fresh start (initial.cu:319-331): rest equilibrium with T = T_REF (init_f/init_g,
 * initial.cu:335-397), particles placed by pinit.cu:97-144 from PARTICLE_RAND_SEED, initial
 * solid flags (pinit.cu:146-179), then build_links(). */
int  rbtp_init_fresh(rbtp_handle *h);

/* Restart from host arrays (the array form of load_restart_state, initial.cu:194-236):
 *   f, g       : NPOP*L each, the post-streaming populations (layout of fg%09d.dat);
 *   flow7      : 7*L (rho,ux,uy,uz,phi,ted,Ked, layout of %09d.dat) or NULL; the buoyancy
 *                force is rebuilt from its phi as forcing() does (initial.cu:230);  NULL means
 *                phi = sum_i g_i;
 *   particles  : npart*RBTP_PARTICLE_COLS (pos file columns) or NULL when npart == 0.
 * Then build_links() and flags_prev = flags (initial.cu:231-235).
 * The arrays are read once, by one import kernel that writes the storage format, the flow fields
 * and the buoyancy force in the same pass.  Page-locked host memory (cudaHostAlloc'd or
 * registered) and device memory are read in place, the former over the host link; ordinary
 * pageable host memory is copied in chunks of 2^20 nodes through two temporary device staging
 * slots (about 1 GB, freed before the call returns), each chunk's import overlapping the next
 * chunk's copy.  The call returns once the import has completed. */
int  rbtp_load_state(rbtp_handle *h, const double *f, const double *g, const double *flow7,
                     const double *particles);
/* Restart from the reference's files in dir: fg%09d.dat, %09d.dat, pos/pos_%09d.txt. */
int  rbtp_load_restart(rbtp_handle *h, const char *dir, int step);

/* ---- time stepping ------------------------------------------------------------------------- */
/* Advance nsteps full steps in main.cu:35-84 order (macrovar → forcing → collide/stream f →
 * IBB f → collide/stream g → IBB g → contacts → forces/heat → move → links → refill), fused into
 * one stream/collide kernel per step on one in-place population array (AA pattern: even and odd
 * steps alternate) plus the particle kernels.  Macroscopic fields are
 * materialised on steps that hit the config's
 * output cadence (NDIAG, NNUOUT, NFLOWOUT, NEND) and, with RBTP_STEP_MACROS_LAST, on the last
 * step of the call.  The dissipation fields ted/Ked of output_flow (compute_Ked/compute_ted,
 * collision.cu:91-198) are produced on flow-output steps (NFLOWOUT, NEND) and, with
 * RBTP_STEP_FLOW_LAST, on the last step of the call; they need an FP64 copy of the step's
 * post-collision populations (2 x 27 L doubles, allocated on first use and kept). */
#define RBTP_STEP_MACROS_LAST 1u
#define RBTP_STEP_FLOW_LAST   2u
int  rbtp_step(rbtp_handle *h, int nsteps);
int  rbtp_step_ex(rbtp_handle *h, int nsteps, unsigned flags);
int  rbtp_current_step(const rbtp_handle *h, int *istep);
int  rbtp_synchronize(rbtp_handle *h);
/* The handle's CUDA stream (cudaStream_t) for callers that order their own work against it. */
int  rbtp_get_stream(rbtp_handle *h, void **stream);

/* ---- state export ---------------------------------------------------------------------------- */
int  rbtp_get_fg(rbtp_handle *h, double *f, double *g);        /* d_f/d_g, as output_fg writes  */
/* Macroscopic fields of the last macro-materialising step: d_rho (density deviation), d_ux..,
 * d_phi and d_force_realx, as they stand after that step (main.cu:98-114 reads them).  Any output
 * pointer may be NULL. */
int  rbtp_get_macros(rbtp_handle *h, double *rho, double *ux, double *uy, double *uz, double *phi,
                     double *force_x);
int  rbtp_get_particles(rbtp_handle *h, double *particles);    /* npart*RBTP_PARTICLE_COLS     */
int  rbtp_npart(const rbtp_handle *h, int *npart);
/* Solid-node owner maps (-1 = fluid): current (d_ibnode_owner) and previous (d_ibnode_owner_prev).
 * ibnode == (owner >= 0).  Either pointer may be NULL. */
int  rbtp_get_flags(rbtp_handle *h, int *owner, int *owner_prev);
/* IBB link list (test hook): node index, direction, particle and q of each link, sorted by
 * (node, dir) like the reference's scan order (links.cu:221-250).  *n receives the count; arrays
 * may be NULL to query the count. */
int  rbtp_get_links(rbtp_handle *h, int *n, int *node, int *dir, int *pid, double *q, int cap);
/* New-fluid nodes detected by the last step's refill (refill.cu:8-76), sorted by node. */
int  rbtp_get_new_fluid(rbtp_handle *h, int *n, int *node, int *pid, int cap);
/* Contact pairs (p < q) whose gap is below REP_MIN_GAP at the last step's start positions
 * (pforces.cu:6-38), sorted by (p, q). */
int  rbtp_get_contacts(rbtp_handle *h, int *n, int *p, int *q, int cap);

/* ---- on-device diagnostics (output/output_statis.cu) ------------------------------------------ */
/* Nu row of output_nu (output_statis.cu:111-223) for the last macro step; step stored as given. */
int  rbtp_nu(rbtp_handle *h, int istep, rbtp_nu_row *row);
/* Volume means umean, vmean, wmean, tmean of diag_flow (output_statis.cu:64-109). */
int  rbtp_means(rbtp_handle *h, double means[4]);
/* Per-x-plane means ux, uy, uz, phi of output_profile (output_statis.cu:225-285): lx*4 doubles. */
int  rbtp_profile(rbtp_handle *h, double *profile);
/* Thermal and viscous dissipation fields ted, Ked (collision.cu:91-198) of the last macro step,
 * with solid nodes zeroed as output_flow does (output_flow.cu:81-95). */
int  rbtp_dissipation(rbtp_handle *h, double *ted, double *ked);

/* ---- reference file writers (byte-compatible layouts) ------------------------------------------ */
/* Output directory name "Ra%.1ePr%.2f" (output_statis.cu:66).  buf >= 64 bytes. */
int  rbtp_output_dirname(const rbtp_handle *h, char *buf, size_t len);
int  rbtp_write_statistics(rbtp_handle *h, const char *dir, int istep);  /* diag_flow     */
int  rbtp_write_nu(rbtp_handle *h, const char *dir, int istep);          /* output_nu     */
int  rbtp_write_profile(rbtp_handle *h, const char *dir, int istep);     /* output_profile*/
int  rbtp_write_flow(rbtp_handle *h, const char *dir, int istep);        /* output_flow   */
int  rbtp_write_fg(rbtp_handle *h, const char *dir, int istep);          /* output_fg     */
int  rbtp_write_particles(rbtp_handle *h, const char *dir, int istep);   /* output_particles */

/* Exact checkpoint of the whole step state in the handle's storage precision (populations of the
 * current buffer, F_x auxiliary, wall densities, current macroscopic fields, particle columns);
 * rbtp_checkpoint_read into a handle created from the same configuration resumes the run bit for
 * bit.  No counterpart in the reference (its restart files, rbtp_load_restart, hold the exported
 * FP64 populations and %14.6e particle text). */
int  rbtp_checkpoint_write(rbtp_handle *h, const char *path);
int  rbtp_checkpoint_read(rbtp_handle *h, const char *path);

/* ---- batched execution (beyond the reference: many cavities, one persistent launch) -------- */
/* A batch advances many independent cavities (own sizes, Ra, Pr, particle counts; one storage
 * mode) in lockstep: per step ONE persistent launch of the fused step over a packed tile table of all
 * cavities, one launch per particle kernel for all spheres of all cavities, the whole step captured
 * once in a CUDA graph and replayed.  Members are ordinary handles (initialised before rbtp_batch_add);
 * between batch steps every single-cavity call (exports, Nu, writers) works on them as usual.  The
 * tile shape and persistent grid are chosen by an autotuner that times the candidates on the first
 * steps of a batch (all candidates compute identical results).  Flow-output (dissipation) steps
 * are not produced in batch mode; macroscopic fields are materialised on each member's NDIAG,
 * NNUOUT, NFLOWOUT, NEND cadence and on its sampling cadence. */
typedef struct rbtp_batch rbtp_batch;
typedef struct rbtp_batch_stats {
    int members, tiles, total_particles, tile_shape;   /* tile_shape: 0 = 32x4, 1 = 64x2 */
    int grid, graph;                                    /* persistent blocks; 1 if replaying a graph */
    int tuned, reserved;
    double last_step_ms;                                /* device time of the last step (events) */
    double nodes;                                       /* lattice nodes over all members */
} rbtp_batch_stats;
int  rbtp_batch_create(int storage, rbtp_batch **out);
int  rbtp_batch_destroy(rbtp_batch *b);
int  rbtp_batch_add(rbtp_batch *b, rbtp_handle *h);
int  rbtp_batch_remove(rbtp_batch *b, rbtp_handle *h);
/* Sample h every `every` steps (0 = only at its stop step): the step materialises the macroscopic
 * fields and ends with an on-device plane-sum reduction written into h's sample ring (64 slots), so
 * batch calls need not end on sample steps.  rbtp_batch_samples turns ring slots into Nu rows. */
int  rbtp_batch_set_sampling(rbtp_batch *b, rbtp_handle *h, int every);
/* h stops advancing once its step counter reaches stop_step (<= 0: never); the other members keep
 * going, so batch calls need not end on any member's horizon. */
int  rbtp_batch_set_stop(rbtp_batch *b, rbtp_handle *h, int stop_step);
/* The Nu rows (output_nu's formulas, rbtp_nu_row; step = the member's step of the sample) of up to
 * cap samples taken since the last call, oldest first.  RBTP_ERR_CAPACITY if more than 64 samples
 * were taken between two calls (the oldest are lost). */
int  rbtp_batch_samples(rbtp_batch *b, rbtp_handle *h, rbtp_nu_row *rows, int cap, int *nrows);
int  rbtp_batch_step(rbtp_batch *b, int nsteps);
/* rbtp_batch_step in two halves: launch returns with the steps in flight (the batch stream works
 * while the caller prepares new members); wait ends them and updates every member.  In between,
 * calls on the batch or its members return RBTP_ERR_STATE (rbtp_batch_remove and rbtp_destroy
 * wait first). */
int  rbtp_batch_launch(rbtp_batch *b, int nsteps);
int  rbtp_batch_wait(rbtp_batch *b);
int  rbtp_batch_stats_get(rbtp_batch *b, rbtp_batch_stats *out);
/* Force a tile shape (0/1) and persistent grid (blocks), or re-enable the autotuner with shape -1. */
int  rbtp_batch_set_launch(rbtp_batch *b, int shape, int grid);

/* Device bytes rbtp_create allocates for cfg (the admission currency of the server below). */
int  rbtp_footprint(const rbtp_config *cfg, size_t *bytes);

/* ---- continuous-batching solve server (beyond the reference) ----------------------------------- */
/* Requests (case, horizon in steps, Nu sampling cadence) are queued from any thread.  Each tick
 * launches max_steps steps of the batch of active requests (bounded by the longest remaining
 * horizon and the sample-ring capacity; each request stops on the device at its own horizon and
 * samples on its own cadence), and while they run prepares queued requests in arrival order whose
 * footprint fits the HBM budget (and the active-slot limit, 0 = none): allocation and fresh start.
 * After the steps it appends the Nu rows (rbtp_nu_row, step = the request's own step) of each
 * request's samples and of its last step, retires finished requests and lets the prepared ones
 * join.  State stays resident between ticks; results do not depend on the other requests. */
typedef struct rbtp_server rbtp_server;
#define RBTP_REQ_QUEUED 0
#define RBTP_REQ_ACTIVE 1
#define RBTP_REQ_DONE   2
#define RBTP_REQ_FAILED 3
int  rbtp_server_create(int storage, double hbm_budget_bytes, int max_active, rbtp_server **out);
int  rbtp_server_destroy(rbtp_server *s);
int  rbtp_server_submit(rbtp_server *s, const rbtp_config *cfg, int horizon, int sample_every, int *id);
int  rbtp_server_tick(rbtp_server *s, int max_steps, int *nactive, int *nqueued);
/* Copies up to cap Nu rows produced so far (the series streams while the request runs); returns the
 * request's status (RBTP_OK unless it failed). */
int  rbtp_server_poll(rbtp_server *s, int id, int *state, int *steps_done, rbtp_nu_row *rows, int cap,
                      int *nrows);
/* Server-clock seconds of submission, admission and completion (-1 if not reached yet). */
int  rbtp_server_request_times(rbtp_server *s, int id, double *t_submit, double *t_admit, double *t_done);
int  rbtp_server_stats(rbtp_server *s, double *node_updates, double *steps, double *used_bytes,
                       double *clock);
/* Checkpoint between ticks into an existing directory (server.bin + req_<id>.ckp per active
 * request, exact), and restore into a freshly created server: queued requests are re-queued in
 * order, active requests resume from their checkpoints bit for bit, finished ones keep their
 * series, and the server clock continues.  No counterpart in the reference. */
int  rbtp_server_checkpoint(rbtp_server *s, const char *dir);
int  rbtp_server_restore(rbtp_server *s, const char *dir);

/* ---- calibration -------------------------------------------------------------------------------- */
/* The FP64 fused multiply-add rate of the current device in flop/s (2 per FMA), measured by a
 * microkernel with independent chains on every SM and timed with CUDA events (best of four runs
 * after a warm-up): the compute roofline of the FP64 storage mode, whose step is bound by the FP64
 * pipe rather than by HBM.  No counterpart in the reference. */
int  rbtp_fp64_fma_rate(double *flops_per_s);

/* ---- allocation-free diagnostic sums ----------------------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device memory — code hosted in
 * a framework that owns the whole device memory pool, or a loop that cannot afford the implicit
 * device synchronisation of cudaMalloc/cudaFree.  Computes, on the caller's stream, the ten per-x-
 * plane sums behind rbtp_nu / rbtp_means / rbtp_profile (layout [10][lx]: fluid sum of ux*phi,
 * fluid count, solid sum of ux*phi, solid count, wall-Nusselt sum, wall count, then the sums of
 * ux, uy, uz, phi with solid nodes taken at the rigid-body velocity and particle temperature) from
 * device arrays the caller owns: ux, uy, uz, phi (L doubles each), owner (L ints, -1 = fluid; NULL
 * = no particles), particle_state (npart x RBTP_PARTICLE_COLS doubles, column-major: column c at
 * particle_state + c*npart), plane_sums (10*lx doubles, written).  It calls no allocator: its
 * partial sums live in one fixed device array of RBTP_NOALLOC_MAX_LX planes (2.6 MB per GPU, kept
 * until the process exits) whose address is looked up on the first call on each device, so make
 * that first call before any stream capture; the address is kept for the device's primary context
 * (the one the CUDA runtime uses), so it is stale after cudaDeviceReset.  Calls share that array:
 * calls that overlap on the GPU race.  lx, ly, lz must be at least 3 (as rbtp_create requires;
 * RBTP_ERR_ARG otherwise); lx > RBTP_NOALLOC_MAX_LX returns RBTP_ERR_CAPACITY. */
#define RBTP_NOALLOC_MAX_LX 1024
int  rbtp_plane_sums_noalloc(const double *ux, const double *uy, const double *uz, const double *phi,
                             const int *owner, const double *particle_state, int npart, int lx,
                             int ly, int lz, double t_hot, double t_cold, double *plane_sums,
                             void *stream);

#ifdef __cplusplus
}
#endif

#endif /* RBTP_H */
