// rb3d — drop-in host for the RB-ThermoParticles case macros, driving librbtp through its C ABI.
//
// Keeps the reference driver's surface (main.cu:1-271): parameters.h macros, fresh start or restart
// from CONTINUOUS_STEPS, the output cadence and order of main.cu:98-114, the output directory
// Ra%.1ePr%.2f and every file layout, and the timing summary of main.cu:120-136.  Steps between two
// output events are advanced in one rbtp_step call, so the device runs without host round trips.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <sys/time.h>

#include "parameters.h"
#include "rbtp.h"

static void die(rbtp_handle *h, int st, const char *what)
{
    std::fprintf(stderr, "rb3d: %s failed: %s (%s)\n", what, rbtp_status_string(st), h ? rbtp_last_error(h) : "");
    std::exit(EXIT_FAILURE);
}

#define CALL(h, x)                       \
    do {                                 \
        int st_ = (x);                   \
        if (st_ != RBTP_OK) die(h, st_, #x); \
    } while (0)

static int next_event(int istep, int final_step)
{
    int n = final_step;
    const int every[4] = {NDIAG, NFLOWOUT, NOUT_P, NNUOUT};
    for (int k = 0; k < 4; ++k)
        if (every[k] > 0) n = std::min(n, (istep / every[k] + 1) * every[k]);
    return n;
}

int main()
{
    struct timeval t_begin, t_end;
    gettimeofday(&t_begin, nullptr);
    rbtp_config c;
    rbtp_config_default(&c);
    c.lx = LX; c.ly = LY; c.lz = LZ;
    c.continuous_steps = CONTINUOUS_STEPS;
    c.nend = NEND; c.ndiag = NDIAG; c.nflowout = NFLOWOUT; c.nnuout = NNUOUT; c.nout_p = NOUT_P;
    c.rayleigh = RAYLEIGH; c.prandtl = PRANDTL;
    c.t_hot = T_HOT; c.t_cold = T_COLD; c.t_ref = T_REF;
    c.beta = BETA; c.visc = VISC; c.rho0 = RHO0;
    c.activate_particles = ACTIVATE_PARTICLES; c.particle_rand_seed = PARTICLE_RAND_SEED;
    c.particle_fraction = PARTICLE_FRACTION; c.particle_diam_frac = PARTICLE_DIAM_FRAC;
    c.cp_particle_ratio = CP_PARTICLE_RATIO; c.cp_fluid = CP_FLUID;
    c.rho_particle_ratio = RHO_PARTICLE_RATIO; c.repforce_scale = REPFORCE_SCALE;
    c.particle_init_temp = PARTICLE_INIT_TEMP;
    c.rep_min_gap = REP_MIN_GAP; c.rep_min_gap_w = REP_MIN_GAP_W;
    c.rep_stf0 = REP_STF0; c.rep_stf1 = REP_STF1; c.rep_stf0_w = REP_STF0_W; c.rep_stf1_w = REP_STF1_W;
    c.storage = RBTP_STORAGE;

    rbtp_handle *h = nullptr;
    CALL(h, rbtp_create(&c, &h));
    const int start_step = CONTINUOUS_STEPS;
    const int final_step = NEND;
    if (start_step > 0) CALL(h, rbtp_load_restart(h, nullptr, start_step));
    else CALL(h, rbtp_init_fresh(h));
    int npart = 0;
    rbtp_npart(h, &npart);
    if (ACTIVATE_PARTICLES && npart > 0 && start_step == 0) CALL(h, rbtp_write_particles(h, nullptr, 0));

    double gpu_time = 0.0, cpu_time = 0.0;
    int istep = start_step;
    while (istep < final_step) {
        const int target = next_event(istep, final_step);
        struct timeval a, b;
        gettimeofday(&a, nullptr);
        CALL(h, rbtp_step(h, target - istep));
        gettimeofday(&b, nullptr);
        gpu_time += (b.tv_sec - a.tv_sec) + (b.tv_usec - a.tv_usec) * 1e-6;
        istep = target;
        clock_t c0 = clock();
        if (NDIAG > 0 && istep % NDIAG == 0) CALL(h, rbtp_write_statistics(h, nullptr, istep));
        if ((NFLOWOUT > 0 && istep % NFLOWOUT == 0) || istep == final_step) CALL(h, rbtp_write_flow(h, nullptr, istep));
        if (NOUT_P > 0 && istep % NOUT_P == 0) CALL(h, rbtp_write_particles(h, nullptr, istep));
        if (NNUOUT > 0 && istep % NNUOUT == 0) {
            CALL(h, rbtp_write_nu(h, nullptr, istep));
            CALL(h, rbtp_write_profile(h, nullptr, istep));
        }
        if (istep == final_step) {
            CALL(h, rbtp_write_fg(h, nullptr, istep));
            CALL(h, rbtp_write_particles(h, nullptr, istep));
        }
        cpu_time += (double)(clock() - c0) / CLOCKS_PER_SEC;
    }
    gettimeofday(&t_end, nullptr);
    const double total = (t_end.tv_sec - t_begin.tv_sec) + (t_end.tv_usec - t_begin.tv_usec) / 1e6;
    std::printf("Simulation completed.\n");
    std::printf("Rayleigh number: %.2e\n", c.rayleigh);
    std::printf("Prandtl number: %.2f\n", c.prandtl);
    std::printf("Total iterations: %d\n", NEND);
    if (start_step > 0) std::printf("Restarted from step: %d, final step: %d\n", start_step, final_step);
    else std::printf("Final step: %d\n", final_step);
    std::printf("CPU computation time: %.2f seconds\n", cpu_time);
    std::printf("GPU computation time: %.2f seconds\n", gpu_time);
    std::printf("Total computation time: %.2f seconds\n", total);
    rbtp_destroy(h);
    return 0;
}
