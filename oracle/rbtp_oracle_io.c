/*
 * rbtp_oracle_io.c — the reference's output writers restated in C, for byte-for-byte checks of the
 * files librbtp and its drop-in host write.
 *
 * TEST INFRASTRUCTURE ONLY (part of the oracle library; the product never links it).  Each writer
 * takes the values to write as arguments (arrays in the reference layout [z][y][x], particle rows of
 * the 33 pos-file columns) and produces the file exactly as the reference's host code does:
 *   output directory "Ra%.1ePr%.2f"                       output_statis.cu:66, output_flow.cu:66
 *   statistics.dat   "%-7d %14.6e %14.6e %14.6e %14.6e\n", appended        output_statis.cu:102-106
 *   Nu_%.2e.txt      7 x "%15.6E" then "\n", appended                     output_statis.cu:123,216-219
 *   Profile_%.2e.txt "%d\n", then LX lines "%14.6e %14.6e %14.6e %14.6e\n" output_statis.cu:238-282
 *   %09d.dat         rho, ux, uy, uz, phi, ted, Ked as raw doubles, solid nodes overwritten by
 *                    overwrite_particle_nodes (rho0, rigid-body velocity, particle temperature,
 *                    zero dissipation)                                     output_flow.cu:5-110
 *   fg%09d.dat       f then g as raw doubles                               output_flow.cu:112-127
 *   pos/pos_%09d.txt "%d " then 33 x "%14.6e" separated by one space, "\n" output_part.cu:91-115
 * Directories are created with mode 0700 when missing, as the reference does.
 */
#include <errno.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

#include "rbtp_oracle.h"

static int ensure_dir(const char *d)
{
    struct stat st;
    if (stat(d, &st) == 0) return RBTP_OK;
    if (mkdir(d, 0700) != 0 && errno != EEXIST) return RBTP_ERR_IO;
    return RBTP_OK;
}

int orc_output_dirname(double rayleigh, double prandtl, char *buf, size_t len)
{
    if (!buf || len < 2) return RBTP_ERR_ARG;
    const int n = snprintf(buf, len, "Ra%.1ePr%.2f", rayleigh, prandtl);
    return (n < 0 || (size_t)n >= len) ? RBTP_ERR_ARG : RBTP_OK;
}

int orc_write_statistics(const char *dir, int istep, const double means[4])
{
    char name[2048];
    if (ensure_dir(dir)) return RBTP_ERR_IO;
    snprintf(name, sizeof(name), "%s/statistics.dat", dir);
    FILE *fp = fopen(name, "a");
    if (!fp) return RBTP_ERR_IO;
    fprintf(fp, "%-7d %14.6e %14.6e %14.6e %14.6e\n", istep, means[0], means[1], means[2], means[3]);
    fclose(fp);
    return RBTP_OK;
}

int orc_write_nu(const char *dir, double rayleigh, const rbtp_nu_row *r)
{
    char name[2048];
    if (ensure_dir(dir)) return RBTP_ERR_IO;
    snprintf(name, sizeof(name), "%s/Nu_%.2e.txt", dir, rayleigh);
    FILE *fp = fopen(name, "a");
    if (!fp) return RBTP_ERR_IO;
    fprintf(fp, "%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E%15.6E\n", r->step, r->volume_fraction, r->nu_bulk,
            r->nu_top, r->nu_bottom, r->nu_bulk_fluid, r->nu_bulk_part);
    fclose(fp);
    return RBTP_OK;
}

int orc_write_profile(const char *dir, double rayleigh, int istep, int lx, const double *profile)
{
    char name[2048];
    if (ensure_dir(dir)) return RBTP_ERR_IO;
    snprintf(name, sizeof(name), "%s/Profile_%.2e.txt", dir, rayleigh);
    FILE *fp = fopen(name, "a");
    if (!fp) return RBTP_ERR_IO;
    fprintf(fp, "%d\n", istep);
    for (int ix = 0; ix < lx; ++ix)
        fprintf(fp, "%14.6e %14.6e %14.6e %14.6e\n", profile[4 * ix], profile[4 * ix + 1], profile[4 * ix + 2],
                profile[4 * ix + 3]);
    fclose(fp);
    return RBTP_OK;
}

/* output_flow.cu:5-110.  fields: 7 arrays of L doubles (rho, ux, uy, uz, phi, ted, ked), copied and
 * then overwritten at solid nodes (owner >= 0) from the owning particle's row. */
int orc_write_flow(const char *dir, int istep, int lx, int ly, int lz, double rho0, const double *fields,
                   const int *owner, const double *rows, int np)
{
    char name[2048];
    if (ensure_dir(dir)) return RBTP_ERR_IO;
    snprintf(name, sizeof(name), "%s/%09d.dat", dir, istep);
    FILE *fp = fopen(name, "wb");
    if (!fp) return RBTP_ERR_IO;
    const long lxy = (long)lx * ly, L = lxy * lz;
    int ok = 1;
    for (int k = 0; k < 7 && ok; ++k) {
        const double *src = fields + (long)k * L;
        for (long idx = 0; idx < L && ok; ++idx) {
            double v = src[idx];
            const int pid = owner ? owner[idx] : -1;
            if (pid >= 0 && pid < np) {
                const double *p = rows + (long)pid * RBTP_PARTICLE_COLS;
                const int iz = (int)(idx / lxy);
                const int iy = (int)((idx - (long)iz * lxy) / lx);
                const int ix = (int)(idx - (long)iz * lxy - (long)iy * lx);
                const double relx = ((double)ix + 0.5) - p[0];
                const double rely = ((double)iy + 0.5) - p[1];
                const double relz = ((double)iz + 0.5) - p[2];
                /* columns: pos 0-2, vel 3-5, omega 18-20, temperature 30 */
                switch (k) {
                case 0: v = rho0; break;
                case 1: v = p[3] + (relz * p[19] - rely * p[20]); break;
                case 2: v = p[4] + (relx * p[20] - relz * p[18]); break;
                case 3: v = p[5] + (rely * p[18] - relx * p[19]); break;
                case 4: v = p[30]; break;
                default: v = 0.0; break;
                }
            }
            ok = fwrite(&v, sizeof(double), 1, fp) == 1;
        }
    }
    fclose(fp);
    return ok ? RBTP_OK : RBTP_ERR_IO;
}

int orc_write_fg(const char *dir, int istep, long L, const double *f, const double *g)
{
    char name[2048];
    if (ensure_dir(dir)) return RBTP_ERR_IO;
    snprintf(name, sizeof(name), "%s/fg%09d.dat", dir, istep);
    FILE *fp = fopen(name, "wb");
    if (!fp) return RBTP_ERR_IO;
    const size_t n = (size_t)27 * (size_t)L;
    const int ok = fwrite(f, sizeof(double), n, fp) == n && fwrite(g, sizeof(double), n, fp) == n;
    fclose(fp);
    return ok ? RBTP_OK : RBTP_ERR_IO;
}

int orc_write_particles(const char *dir, int istep, int np, const double *rows)
{
    char name[2048];
    if (np <= 0) return RBTP_OK;
    if (ensure_dir(dir)) return RBTP_ERR_IO;
    snprintf(name, sizeof(name), "%s/pos", dir);
    if (ensure_dir(name)) return RBTP_ERR_IO;
    snprintf(name, sizeof(name), "%s/pos/pos_%09d.txt", dir, istep);
    FILE *fp = fopen(name, "w");
    if (!fp) return RBTP_ERR_IO;
    for (int p = 0; p < np; ++p) {
        const double *r = rows + (long)p * RBTP_PARTICLE_COLS;
        fprintf(fp, "%d ", p);
        for (int c = 0; c < RBTP_PARTICLE_COLS; ++c)
            fprintf(fp, c + 1 < RBTP_PARTICLE_COLS ? "%14.6e " : "%14.6e\n", r[c]);
    }
    fclose(fp);
    return RBTP_OK;
}
