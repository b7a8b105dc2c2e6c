/*
 * rbtp_oracle.h — CPU oracle for the RB-ThermoParticles per-timestep path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C (OpenMP, FP64) restatement of the reference
 * algorithm, kept step-for-step with the reference's kernels so that the GPU library can be
 * checked against it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it; the product library never links or calls it.
 *
 * Pinning: the reference ships no tests, fixtures or golden vectors.  The oracle is pinned by the
 * analytic invariants in tests/test_oracle_*.py (lattice symmetries, exact mass conservation
 * under wall bounce-back, quiescent rest, conduction profile, closed-form ray-sphere q) and by the
 * committed fixtures in tests/golden/.  Parity against the reference's own build: see
 * oracle/ref_pin/.
 */
#ifndef RBTP_ORACLE_H
#define RBTP_ORACLE_H

#include "../include/rbtp.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

int  orc_create(const rbtp_config *cfg, orc_sim **out);
void orc_destroy(orc_sim *s);
int  orc_set_threads(int nthreads);
int  orc_get_threads(void);

int  orc_init_fresh(orc_sim *s);
int  orc_load_state(orc_sim *s, const double *f, const double *g, const double *flow7,
                    const double *particles);
int  orc_step(orc_sim *s, int nsteps);

int  orc_npart(const orc_sim *s);
int  orc_derive(const rbtp_config *cfg, rbtp_derived *out);
int  orc_get_fg(const orc_sim *s, double *f, double *g);
int  orc_get_macros(const orc_sim *s, double *rho, double *ux, double *uy, double *uz,
                    double *phi, double *force_x);
int  orc_get_particles(const orc_sim *s, double *particles);
int  orc_get_flags(const orc_sim *s, int *owner, int *owner_prev);
int  orc_get_links(const orc_sim *s, int *n, int *node, int *dir, int *pid, double *q, int cap);
int  orc_get_new_fluid(const orc_sim *s, int *n, int *node, int *pid, int cap);
int  orc_get_contacts(const orc_sim *s, int *n, int *p, int *q, int cap);
int  orc_nu(orc_sim *s, int istep, rbtp_nu_row *row);
int  orc_means(orc_sim *s, double means[4]);
int  orc_profile(orc_sim *s, double *profile);
int  orc_dissipation(orc_sim *s, double *ted, double *ked);

/* The reference's output writers (rbtp_oracle_io.c), fed with the values to write. */
int  orc_output_dirname(double rayleigh, double prandtl, char *buf, size_t len);
int  orc_write_statistics(const char *dir, int istep, const double means[4]);
int  orc_write_nu(const char *dir, double rayleigh, const rbtp_nu_row *row);
int  orc_write_profile(const char *dir, double rayleigh, int istep, int lx, const double *profile);
int  orc_write_flow(const char *dir, int istep, int lx, int ly, int lz, double rho0, const double *fields,
                    const int *owner, const double *rows, int np);
int  orc_write_fg(const char *dir, int istep, long L, const double *f, const double *g);
int  orc_write_particles(const char *dir, int istep, int np, const double *rows);

/* Stand-alone pieces for unit tests. */
int  orc_link_q(int ip, double x0, double y0, double z0, double px, double py, double pz,
                double radius_sq, double *q);
/* Rebuild flags/links from externally set particle positions (test hook for bit-exact link
 * comparison at identical particle states). */
int  orc_set_positions_and_build(orc_sim *s, const double *pos_xyz);

#ifdef __cplusplus
}
#endif

#endif
