// ref_driver.cpp — runs the reference's own CUDA kernels (compiled from its sources into
// oracle/_ref/<case>.cubin by build_ref.py) under a restatement of its host code, to pin the oracle
// and librbtp against the reference's device arithmetic on the same GPU.
//
// TEST INFRASTRUCTURE ONLY.  The host sequence follows main.cu:32-85 and the wrappers
// build_links (links.cu:143-256), bounce_back_* / compute_particle_* (ibb.cu:209-271),
// prepare_particle_forces_step / apply_repulsive_forces (pforces.cu:80-148),
// update_particles (move.cu:107-142), refill_nodes (refill.cu:244-329) and the restart load of
// initial.cu:194-236.  CUB's device scans are replaced by host integer scans (same results).
//
// usage: ref_driver <cubin> <in_dir> <nsteps> <out_dir>
//   in_dir:  cfg.txt (key value lines), f.bin, g.bin, flow7.bin, particles.bin (np x 33, optional)
//   out_dir: links0.bin owner0.bin (loaded state), f.bin g.bin macros.bin particles.bin owner.bin
//            links.bin newfluid.bin (after nsteps)
//
//   With "sample_stride k" (k > 1) in cfg.txt, f.bin, g.bin and macros.bin hold every k-th node only
//   (node indices 0, k, 2k, ...; each direction or field in turn) and fgnorm.bin holds, per direction,
//   sum f_i, sum f_i^2, sum g_i, sum g_i^2 over all nodes: full-size cases without 7 GB dumps.
//
// Nu series: ref_driver <cubin> <in_dir> nu <nsteps> <every> <out_file>
//   Runs nsteps steps and after every `every`-th step appends the Nu row of output_nu
//   (output_statis.cu:111-223: step, volume fraction, Nu_bulk, Nu_top, Nu_bottom, Nu_bulk_fluid,
//   Nu_bulk_part; 7 doubles) computed on the host from the reference kernels' d_ux, d_phi and
//   d_ibnode of that step.
//
// timing: ref_driver <cubin> <in_dir> time <warmup> <steps>
//   Times the reference's per-step sequence (kernels and device-to-device copies exactly as its host
//   loop issues them) on the seeded synthetic start that cfg.txt describes ("synthetic 1": f = 0,
//   g = w_i T with T the linear profile plus the SplitMix64 perturbation of rbtp/workloads.py) and
//   prints one line "ref_time ms_per_step <t> ms_per_step_with_host_scans <t2> ...".  The two
//   prefix sums that the reference runs with CUB are host scans here; their time is excluded from
//   the first figure (it counts only the reference's own device work and host loop).
#include <cuda.h>

#include <chrono>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#define CU(x)                                                                      \
    do {                                                                           \
        CUresult r_ = (x);                                                         \
        if (r_ != CUDA_SUCCESS) {                                                  \
            const char *s_ = nullptr;                                              \
            cuGetErrorString(r_, &s_);                                             \
            std::fprintf(stderr, "%s:%d %s -> %s\n", __FILE__, __LINE__, #x, s_);  \
            std::exit(2);                                                          \
        }                                                                          \
    } while (0)

namespace {

// ParticleLink of include/particle.h:19-29 (same member order, natural alignment: 56 bytes)
struct Link {
    int ci, cj, ck, dir, pid;
    double q, rx, ry, rz;
};
static_assert(sizeof(Link) == 56, "ParticleLink layout");

std::map<std::string, double> cfg;
int LX, LY, LZ, NP;
long long L;
CUmodule mod;
std::map<std::string, CUfunction> fn;

std::vector<char> slurp(const std::string &p)
{
    std::ifstream in(p, std::ios::binary);
    if (!in) { std::fprintf(stderr, "cannot open %s\n", p.c_str()); std::exit(2); }
    return std::vector<char>((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
}

void dump(const std::string &p, const void *d, size_t n)
{
    FILE *fp = std::fopen(p.c_str(), "wb");
    if (!fp || std::fwrite(d, 1, n, fp) != n) { std::fprintf(stderr, "cannot write %s\n", p.c_str()); std::exit(2); }
    std::fclose(fp);
}

// Kernels are found by their Itanium-mangled identifier "<length><name>", which also matches the
// anonymous-namespace kernels of the particle files.
CUfunction kernel(const std::string &name)
{
    auto it = fn.find(name);
    if (it != fn.end()) return it->second;
    unsigned n = 0;
    CU(cuModuleGetFunctionCount(&n, mod));
    std::vector<CUfunction> all(n);
    CU(cuModuleEnumerateFunctions(all.data(), n, mod));
    const std::string key = std::to_string(name.size()) + name;
    for (CUfunction f : all) {
        const char *nm = nullptr;
        CU(cuFuncGetName(&nm, f));
        std::string s(nm);
        // the length prefix delimits the identifier ("9streaming" is not inside "16streaming_scalar")
        if (s.find(key) == std::string::npos) continue;
        fn[name] = f;
        return f;
    }
    std::fprintf(stderr, "kernel %s not found\n", name.c_str());
    std::exit(2);
}

template <class T>
void set_const(const char *name, const T *v, size_t n)
{
    CUdeviceptr p;
    size_t bytes;
    CU(cuModuleGetGlobal(&p, &bytes, mod, name));
    if (bytes != n * sizeof(T)) { std::fprintf(stderr, "symbol %s size %zu\n", name, bytes); std::exit(2); }
    CU(cuMemcpyHtoD(p, v, bytes));
}

CUdeviceptr dalloc(size_t bytes)
{
    CUdeviceptr p;
    CU(cuMemAlloc(&p, bytes ? bytes : 8));
    CU(cuMemsetD8(p, 0, bytes ? bytes : 8));
    return p;
}

struct Launch {
    std::vector<void *> args;
    template <class T>
    Launch &a(T &v) { args.push_back((void *)&v); return *this; }
    void run(const char *name, unsigned gx, unsigned gy, unsigned gz, unsigned bx, unsigned by, unsigned bz)
    {
        if (gx == 0 || gy == 0 || gz == 0) return;
        CU(cuLaunchKernel(kernel(name), gx, gy, gz, bx, by, bz, 0, 0, args.data(), nullptr));
    }
};

// device state (names of include/lbm.h:38-49, include/particle.h:47-107)
CUdeviceptr d_f, d_g, d_f_temp, d_f_collide, d_g_temp, d_g_collide;
CUdeviceptr d_rho, d_ux, d_uy, d_uz, d_phi, d_fx, d_fy, d_fz, d_ted, d_Ked;
CUdeviceptr d_pos[3], d_vel[3], d_omg[3], d_th[3], d_facc[3], d_fprev[3], d_fprev2[3];
CUdeviceptr d_tacc[3], d_tprev[3], d_tprev2[3], d_ptemp, d_pheat, d_pheat_prev;
CUdeviceptr d_ibnode, d_ibnode_prev, d_owner, d_owner_prev, d_count, d_offset;
CUdeviceptr d_links = 0, d_nf_nodes = 0, d_nf_pids = 0;
int num_links = 0, link_cap = 0, num_nf = 0, nf_cap = 0;

void memcpy_dd(CUdeviceptr dst, CUdeviceptr src, size_t b) { CU(cuMemcpyDtoD(dst, src, b)); }

double g_scan_seconds = 0.0;   // wall time spent in the host stand-ins for the CUB scans

void host_scan(int n_total_last, int &total)
{
    CU(cuCtxSynchronize());
    const auto t0 = std::chrono::steady_clock::now();
    struct Clock {
        std::chrono::steady_clock::time_point t0;
        ~Clock() { g_scan_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
    } clk{t0};
    std::vector<int> cnt(L), off(L);
    CU(cuMemcpyDtoH(cnt.data(), d_count, L * sizeof(int)));
    long long run = 0;
    for (long long i = 0; i < L; ++i) { off[i] = (int)run; run += cnt[i]; }
    CU(cuMemcpyHtoD(d_offset, off.data(), L * sizeof(int)));
    total = (int)run;
    (void)n_total_last;
}

// links.cu:143-256
void build_links()
{
    std::vector<double> px(NP), py(NP), pz(NP);
    CU(cuMemcpyDtoH(px.data(), d_pos[0], NP * 8));
    CU(cuMemcpyDtoH(py.data(), d_pos[1], NP * 8));
    CU(cuMemcpyDtoH(pz.data(), d_pos[2], NP * 8));
    CU(cuMemsetD32(d_ibnode, 0, L));
    CU(cuMemsetD8(d_owner, 0xFF, L * 4));
    const double r = cfg["radius"];
    double rsq = r * r;
    for (int p = 0; p < NP; ++p) {
        int ix0 = (int)std::floor(px[p] - r - 0.5), ix1 = (int)std::floor(px[p] + r - 0.5);
        int iy0 = (int)std::floor(py[p] - r - 0.5), iy1 = (int)std::floor(py[p] + r - 0.5);
        int iz0 = (int)std::floor(pz[p] - r - 0.5), iz1 = (int)std::floor(pz[p] + r - 0.5);
        if (ix0 < 0) ix0 = 0;
        if (iy0 < 0) iy0 = 0;
        if (iz0 < 0) iz0 = 0;
        if (ix1 > LX - 1) ix1 = LX - 1;
        if (iy1 > LY - 1) iy1 = LY - 1;
        if (iz1 > LZ - 1) iz1 = LZ - 1;
        if (ix0 > ix1 || iy0 > iy1 || iz0 > iz1) continue;
        int pid = p;
        double x = px[p], y = py[p], z = pz[p];
        Launch().a(pid).a(ix0).a(iy0).a(iz0).a(ix1).a(iy1).a(iz1).a(x).a(y).a(z).a(rsq).a(d_ibnode).a(d_owner)
            .run("mark_ibnode_kernel", (ix1 - ix0 + 8) / 8, (iy1 - iy0 + 8) / 8, (iz1 - iz0 + 8) / 8, 8, 8, 8);
    }
    const unsigned blocks = (unsigned)((L + 255) / 256);
    Launch().a(d_count).a(d_ibnode).a(d_owner).a(d_pos[0]).a(d_pos[1]).a(d_pos[2])
        .run("link_count_kernel", blocks, 1, 1, 256, 1, 1);
    host_scan(0, num_links);
    if (num_links > link_cap) {
        if (d_links) CU(cuMemFree(d_links));
        d_links = dalloc((size_t)num_links * sizeof(Link));
        link_cap = num_links;
    }
    if (num_links > 0)
        Launch().a(d_count).a(d_offset).a(d_ibnode).a(d_owner).a(d_pos[0]).a(d_pos[1]).a(d_pos[2]).a(d_links)
            .run("link_fill_kernel", blocks, 1, 1, 256, 1, 1);
    CU(cuCtxSynchronize());
}

// refill.cu:244-329
void refill_nodes()
{
    const unsigned blocks = (unsigned)((L + 255) / 256);
    Launch().a(d_count).a(d_ibnode_prev).a(d_ibnode).a(d_owner_prev).a(d_pos[0]).a(d_pos[1]).a(d_pos[2])
        .run("new_fluid_count_kernel", blocks, 1, 1, 256, 1, 1);
    host_scan(0, num_nf);
    if (num_nf > nf_cap) {
        if (d_nf_nodes) CU(cuMemFree(d_nf_nodes));
        if (d_nf_pids) CU(cuMemFree(d_nf_pids));
        d_nf_nodes = dalloc((size_t)num_nf * 4);
        d_nf_pids = dalloc((size_t)num_nf * 4);
        nf_cap = num_nf;
    }
    if (num_nf > 0) {
        Launch().a(d_count).a(d_offset).a(d_ibnode_prev).a(d_ibnode).a(d_owner_prev).a(d_pos[0]).a(d_pos[1])
            .a(d_pos[2]).a(d_nf_nodes).a(d_nf_pids).run("new_fluid_fill_kernel", blocks, 1, 1, 256, 1, 1);
        int n = num_nf;
        Launch().a(d_nf_nodes).a(d_nf_pids).a(n).a(d_f).a(d_g).a(d_f_collide).a(d_g_collide).a(d_ibnode_prev)
            .a(d_owner_prev).a(d_pos[0]).a(d_pos[1]).a(d_pos[2]).a(d_vel[0]).a(d_vel[1]).a(d_vel[2])
            .a(d_omg[0]).a(d_omg[1]).a(d_omg[2]).a(d_ptemp).a(d_rho).a(d_ux).a(d_uy).a(d_uz).a(d_phi)
            .a(d_fx).a(d_fy).a(d_fz).run("refill_new_fluid_kernel", (n + 127) / 128, 1, 1, 128, 1, 1);
    }
    memcpy_dd(d_ibnode_prev, d_ibnode, L * 4);
    memcpy_dd(d_owner_prev, d_owner, L * 4);
    CU(cuCtxSynchronize());
}

void step()
{
    unsigned gx = (LX + 7) / 8, gy = (LY + 7) / 8, gz = (LZ + 3) / 4;
    const size_t P = 27 * (size_t)L * 8;
    Launch().a(d_f).a(d_g).a(d_fx).a(d_fy).a(d_fz).a(d_rho).a(d_ux).a(d_uy).a(d_uz).a(d_phi)
        .run("macrovar", gx, gy, gz, 8, 8, 4);
    Launch().a(d_fx).a(d_fy).a(d_fz).a(d_phi).run("forcing", gx, gy, gz, 8, 8, 4);
    Launch().a(d_f).a(d_fx).a(d_fy).a(d_fz).a(d_rho).a(d_ux).a(d_uy).a(d_uz).run("collision_BGK", gx, gy, gz, 8, 8, 4);
    memcpy_dd(d_f_collide, d_f, P);
    Launch().a(d_f).a(d_f_temp).run("streaming", gx, gy, gz, 8, 8, 4);
    memcpy_dd(d_f, d_f_temp, P);
    const bool parts = NP > 0;
    const unsigned lb = (unsigned)((num_links + 127) / 128);
    int nl = num_links;
    if (parts && nl > 0)
        Launch().a(d_links).a(nl).a(d_f).a(d_f_collide).a(d_ibnode).a(d_pos[0]).a(d_pos[1]).a(d_pos[2])
            .a(d_vel[0]).a(d_vel[1]).a(d_vel[2]).a(d_omg[0]).a(d_omg[1]).a(d_omg[2])
            .run("bounce_back_particles_kernel", lb, 1, 1, 128, 1, 1);
    Launch().a(d_g).a(d_fx).a(d_fy).a(d_fz).a(d_rho).a(d_ux).a(d_uy).a(d_uz).a(d_phi)
        .run("collision_BGK_scalar", gx, gy, gz, 8, 8, 4);
    memcpy_dd(d_g_collide, d_g, P);
    Launch().a(d_g).a(d_g_temp).a(d_rho).run("streaming_scalar", gx, gy, gz, 8, 8, 4);
    memcpy_dd(d_g, d_g_temp, P);
    if (!parts) { CU(cuCtxSynchronize()); return; }
    if (nl > 0)
        Launch().a(d_links).a(nl).a(d_g).a(d_g_collide).a(d_ibnode_prev).a(d_ibnode).a(d_rho).a(d_ptemp)
            .run("bounce_back_thermal_kernel", lb, 1, 1, 128, 1, 1);
    // prepare_particle_forces_step (pforces.cu:80-116)
    for (int a = 0; a < 3; ++a) {
        memcpy_dd(d_fprev2[a], d_fprev[a], NP * 8);
        memcpy_dd(d_tprev2[a], d_tprev[a], NP * 8);
    }
    for (int a = 0; a < 3; ++a) {
        memcpy_dd(d_fprev[a], d_facc[a], NP * 8);
        memcpy_dd(d_tprev[a], d_tacc[a], NP * 8);
    }
    for (int a = 0; a < 3; ++a) {
        CU(cuMemsetD8(d_facc[a], 0, NP * 8));
        CU(cuMemsetD8(d_tacc[a], 0, NP * 8));
    }
    // apply_repulsive_forces (pforces.cu:118-148)
    double radius = cfg["radius"], coeff = cfg["mass"] * cfg["repforce_scale"];
    double mg = cfg["rep_min_gap"], mgw = cfg["rep_min_gap_w"];
    int np = NP;
    if (np > 1)
        Launch().a(d_pos[0]).a(d_pos[1]).a(d_pos[2]).a(d_facc[0]).a(d_facc[1]).a(d_facc[2]).a(np).a(radius)
            .a(coeff).a(mg).run("repulsive_pair_kernel", (np + 15) / 16, (np + 15) / 16, 1, 16, 16, 1);
    Launch().a(d_pos[0]).a(d_pos[1]).a(d_pos[2]).a(d_facc[0]).a(d_facc[1]).a(d_facc[2]).a(np).a(radius)
        .a(coeff).a(mgw).run("repulsive_wall_kernel", (np + 127) / 128, 1, 1, 128, 1, 1);
    // compute_particle_forces / compute_particle_heat (ibb.cu:237-271)
    if (nl > 0)
        Launch().a(d_links).a(nl).a(d_f).a(d_f_collide).a(d_pos[0]).a(d_pos[1]).a(d_pos[2]).a(d_vel[0])
            .a(d_vel[1]).a(d_vel[2]).a(d_omg[0]).a(d_omg[1]).a(d_omg[2]).a(d_facc[0]).a(d_facc[1])
            .a(d_facc[2]).a(d_tacc[0]).a(d_tacc[1]).a(d_tacc[2])
            .run("compute_particle_forces_kernel", lb, 1, 1, 128, 1, 1);
    memcpy_dd(d_pheat_prev, d_pheat, NP * 8);
    CU(cuMemsetD8(d_pheat, 0, NP * 8));
    if (nl > 0)
        Launch().a(d_links).a(nl).a(d_g).a(d_g_collide).a(d_pheat).run("compute_particle_heat_kernel", lb, 1, 1, 128, 1, 1);
    // update_particles (move.cu:107-142)
    double mass = cfg["mass"], inertia = cfg["inertia"], hc = cfg["heat_capacity"], rr = cfg["rho_particle_ratio"];
    Launch().a(d_pos[0]).a(d_pos[1]).a(d_pos[2]).a(d_vel[0]).a(d_vel[1]).a(d_vel[2]).a(d_omg[0]).a(d_omg[1])
        .a(d_omg[2]).a(d_th[0]).a(d_th[1]).a(d_th[2]).a(d_facc[0]).a(d_facc[1]).a(d_facc[2]).a(d_tacc[0])
        .a(d_tacc[1]).a(d_tacc[2]).a(d_fprev[0]).a(d_fprev[1]).a(d_fprev[2]).a(d_fprev2[0]).a(d_fprev2[1])
        .a(d_fprev2[2]).a(d_tprev[0]).a(d_tprev[1]).a(d_tprev[2]).a(d_tprev2[0]).a(d_tprev2[1]).a(d_tprev2[2])
        .a(d_ptemp).a(d_pheat).a(d_pheat_prev).a(radius).a(mass).a(inertia).a(hc).a(rr)
        .run("update_particles_kernel", (np + 127) / 128, 1, 1, 128, 1, 1);
    CU(cuCtxSynchronize());
    build_links();
    refill_nodes();
}

// SplitMix64 output k (k = 1..n) of the stream with the given seed, as doubles in [0, 1)
// (rbtp/workloads.py splitmix64_uniform).
double splitmix_uniform(unsigned long long seed, unsigned long long k)
{
    unsigned long long z = seed + k * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// f = 0, g_i = w_i T, flow7 = (0, 0, 0, 0, T, 0, 0) with T the seeded linear-conduction start.
void synthetic_state(std::vector<char> &f, std::vector<char> &g, std::vector<char> &f7)
{
    const size_t P = 27 * (size_t)L * 8, S = (size_t)L * 8;
    f.assign(P, 0);
    g.assign(P, 0);
    f7.assign(7 * S, 0);
    double *gp = (double *)g.data(), *tp7 = (double *)f7.data() + 4 * L;
    const double th = cfg["t_hot"], tc = cfg["t_cold"], amp = cfg.count("amp") ? cfg["amp"] : 1e-3;
    const unsigned long long seed = (unsigned long long)cfg["seed"];
    const double w[4] = {8.0 / 27.0, 2.0 / 27.0, 1.0 / 54.0, 1.0 / 216.0};
    for (long long n = 0; n < L; ++n) {
        const int x = (int)(n % LX);
        double T = th - (x + 0.5) / LX * (th - tc);
        T = T + amp * (2.0 * splitmix_uniform(seed, (unsigned long long)n + 1) - 1.0);
        tp7[n] = T;
        for (int i = 0; i < 27; ++i) gp[(size_t)i * L + n] = w[i == 0 ? 0 : (i <= 6 ? 1 : (i <= 18 ? 2 : 3))] * T;
    }
}

// The Nu row of output_nu (output_statis.cu:111-223) from the device's d_ux, d_phi and (with
// particles) d_ibnode as they stand after a step: plane-averaged u_x T over fluid and solid nodes,
// and the wall gradients (T_hot - T(x = 1/2)) / (1/2) and (T(LX - 1/2) - T_cold) / (1/2) over fluid
// wall nodes, scaled as that function scales them.
void nu_row(int istep, double *row)
{
    std::vector<double> ux(L), phi(L);
    std::vector<int> ib(NP > 0 ? L : 0);
    CU(cuMemcpyDtoH(ux.data(), d_ux, L * sizeof(double)));
    CU(cuMemcpyDtoH(phi.data(), d_phi, L * sizeof(double)));
    if (NP > 0) CU(cuMemcpyDtoH(ib.data(), d_ibnode, L * sizeof(int)));
    const double th = cfg["t_hot"], tc = cfg["t_cold"], diff = cfg["diff"];
    const double vf = cfg.count("particle_fraction") ? cfg["particle_fraction"] : 0.0;
    const double cp = cfg.count("cp_particle_ratio") ? cfg["cp_particle_ratio"] : 0.0;
    const double fluid_frac = std::fmax(0.0, 1.0 - vf);
    const long long lxy = (long long)LX * LY;
    auto solid = [&](long long n) { return NP > 0 && ib[n] != 0; };
    double avg_f = 0.0, avg_p = 0.0;
    for (int ix = 0; ix < LX; ++ix) {
        double sf = 0.0, sp = 0.0;
        long long nf = 0, npart = 0;
        for (int iz = 0; iz < LZ; ++iz)
            for (int iy = 0; iy < LY; ++iy) {
                const long long n = iz * lxy + (long long)iy * LX + ix;
                if (solid(n)) { sp += ux[n] * phi[n]; ++npart; }
                else { sf += ux[n] * phi[n]; ++nf; }
            }
        if (nf > 0) avg_f += sf / (double)nf;
        if (npart > 0) avg_p += sp / (double)npart;
    }
    avg_f /= (double)LX;
    avg_p /= (double)LX;
    const double cond = diff * (th - tc) / (double)LX;
    double nb_fluid = fluid_frac, nb_part = 0.0;
    if (cond != 0.0) {
        nb_fluid += fluid_frac * (avg_f / cond);
        nb_part = vf * cp * (avg_p / cond);
    }
    double bot = 0.0, top = 0.0;
    long long nb = 0, nt = 0;
    for (int iz = 0; iz < LZ; ++iz)
        for (int iy = 0; iy < LY; ++iy) {
            const long long n0 = iz * lxy + (long long)iy * LX, n1 = n0 + LX - 1;
            if (!solid(n0)) { bot += (th - phi[n0]) / 0.5; ++nb; }
            if (!solid(n1)) { top += (phi[n1] - tc) / 0.5; ++nt; }
        }
    const double area = (double)LY * (double)LZ, scale = (double)LX / (th - tc);
    row[0] = (double)istep;
    row[1] = vf;
    row[2] = nb_fluid + nb_part;
    row[3] = nt > 0 ? (top / area) * scale : 0.0;
    row[4] = nb > 0 ? (bot / area) * scale : 0.0;
    row[5] = nb_fluid;
    row[6] = nb_part;
}

// Every stride-th node of a device array of n fields of L doubles, field after field.
std::vector<double> sampled(CUdeviceptr d, int nfield, long long stride)
{
    std::vector<double> plane(L), out;
    for (int k = 0; k < nfield; ++k) {
        CU(cuMemcpyDtoH(plane.data(), d + (size_t)k * L * 8, L * 8));
        for (long long n = 0; n < L; n += stride) out.push_back(plane[n]);
    }
    return out;
}

int run(int argc, char **argv)
{
    const bool timing = argc == 6 && std::string(argv[3]) == "time";
    const bool nu_mode = argc == 7 && std::string(argv[3]) == "nu";
    if (argc != 5 && !timing && !nu_mode) {
        std::fprintf(stderr, "usage: ref_driver <cubin> <in_dir> <nsteps> <out_dir>\n"
                             "       ref_driver <cubin> <in_dir> nu <nsteps> <every> <out_file>\n"
                             "       ref_driver <cubin> <in_dir> time <warmup> <steps>\n");
        return 2;
    }
    const std::string in = argv[2], out = (timing || nu_mode) ? std::string() : std::string(argv[4]);
    const int nsteps = timing ? 0 : std::atoi(argv[nu_mode ? 4 : 3]);
    {
        std::ifstream cf(in + "/cfg.txt");
        std::string k;
        double v;
        while (cf >> k >> v) cfg[k] = v;
    }
    LX = (int)cfg["lx"]; LY = (int)cfg["ly"]; LZ = (int)cfg["lz"]; NP = (int)cfg["npart"];
    L = (long long)LX * LY * LZ;
    CU(cuInit(0));
    CUdevice dev;
    CU(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CU(cuDevicePrimaryCtxRetain(&ctx, dev));
    CU(cuCtxSetCurrent(ctx));
    CU(cuModuleLoad(&mod, argv[1]));

    // constants (initial.cu:276-303, globals.cu:142-148, 150-169)
    const int cix[27] = {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1, 0, 1, 0, -1, 0, 1, -1, -1, 1, 1, -1, -1, 1};
    const int ciy[27] = {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0, -1, 0, 1, 0, -1, 1, 1, -1, -1, 1, 1, -1, -1};
    const int ciz[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
    const int opp[27] = {0, 3, 4, 1, 2, 6, 5, 9, 10, 7, 8, 17, 18, 15, 16, 13, 14, 11, 12, 25, 26, 23, 24, 21, 22, 19, 20};
    double tp[27];
    for (int i = 0; i < 27; ++i) tp[i] = i == 0 ? 8.0 / 27.0 : (i <= 6 ? 2.0 / 27.0 : (i <= 18 ? 1.0 / 54.0 : 1.0 / 216.0));
    set_const("d_cix", cix, 27); set_const("d_ciy", ciy, 27); set_const("d_ciz", ciz, 27);
    set_const("d_opp", opp, 27); set_const("d_tp", tp, 27);
    const char *dn[] = {"d_tau", "d_tauc", "d_grav0", "d_beta", "d_tHot", "d_tCold", "d_t0", "d_diff", "d_visc",
                        "d_particle_radius", "d_particle_mass", "d_particle_inertia", "d_particle_heat_capacity",
                        "d_particle_cp_fluid", "d_particle_rho_ratio"};
    const char *kn[] = {"tau", "tauc", "grav0", "beta", "t_hot", "t_cold", "t_ref", "diff", "visc", "radius",
                        "mass", "inertia", "heat_capacity", "cp_fluid", "rho_particle_ratio"};
    for (int k = 0; k < 15; ++k) { double v = cfg[kn[k]]; set_const(dn[k], &v, 1); }
    set_const("d_npart", &NP, 1);

    const size_t P = 27 * (size_t)L * 8, S = (size_t)L * 8;
    d_f = dalloc(P); d_g = dalloc(P); d_f_temp = dalloc(P); d_f_collide = dalloc(P); d_g_temp = dalloc(P); d_g_collide = dalloc(P);
    d_rho = dalloc(S); d_ux = dalloc(S); d_uy = dalloc(S); d_uz = dalloc(S); d_phi = dalloc(S);
    d_fx = dalloc(S); d_fy = dalloc(S); d_fz = dalloc(S); d_ted = dalloc(S); d_Ked = dalloc(S);
    d_ibnode = dalloc(L * 4); d_ibnode_prev = dalloc(L * 4); d_owner = dalloc(L * 4); d_owner_prev = dalloc(L * 4);
    d_count = dalloc(L * 4); d_offset = dalloc(L * 4);
    CU(cuMemsetD8(d_owner, 0xFF, L * 4));
    CU(cuMemsetD8(d_owner_prev, 0xFF, L * 4));
    const size_t PB = (size_t)(NP > 0 ? NP : 1) * 8;
    for (int a = 0; a < 3; ++a) {
        d_pos[a] = dalloc(PB); d_vel[a] = dalloc(PB); d_omg[a] = dalloc(PB); d_th[a] = dalloc(PB);
        d_facc[a] = dalloc(PB); d_fprev[a] = dalloc(PB); d_fprev2[a] = dalloc(PB);
        d_tacc[a] = dalloc(PB); d_tprev[a] = dalloc(PB); d_tprev2[a] = dalloc(PB);
    }
    d_ptemp = dalloc(PB); d_pheat = dalloc(PB); d_pheat_prev = dalloc(PB);

    // load_restart_state (initial.cu:194-236)
    std::vector<char> f, g, f7;
    if (cfg.count("synthetic") && cfg["synthetic"] != 0.0) synthetic_state(f, g, f7);
    else { f = slurp(in + "/f.bin"); g = slurp(in + "/g.bin"); f7 = slurp(in + "/flow7.bin"); }
    if (f.size() != P || g.size() != P || f7.size() != 7 * S) { std::fprintf(stderr, "bad input sizes\n"); return 2; }
    CU(cuMemcpyHtoD(d_f, f.data(), P));
    CU(cuMemcpyHtoD(d_g, g.data(), P));
    if (NP > 0) {
        auto pr = slurp(in + "/particles.bin");
        if (pr.size() != (size_t)NP * 33 * 8) { std::fprintf(stderr, "bad particle file\n"); return 2; }
        const double *rows = (const double *)pr.data();
        std::vector<double> col(NP);
        CUdeviceptr *dst[11] = {d_pos, d_vel, d_facc, d_fprev, d_fprev2, d_th, d_omg, d_tacc, d_tprev, d_tprev2, nullptr};
        for (int blk = 0; blk < 10; ++blk)
            for (int a = 0; a < 3; ++a) {
                for (int p = 0; p < NP; ++p) col[p] = rows[p * 33 + 3 * blk + a];
                CU(cuMemcpyHtoD(dst[blk][a], col.data(), NP * 8));
            }
        CUdeviceptr last[3] = {d_ptemp, d_pheat, d_pheat_prev};
        for (int k = 0; k < 3; ++k) {
            for (int p = 0; p < NP; ++p) col[p] = rows[p * 33 + 30 + k];
            CU(cuMemcpyHtoD(last[k], col.data(), NP * 8));
        }
        build_links();
    }
    memcpy_dd(d_f_collide, d_f, P);
    memcpy_dd(d_g_collide, d_g, P);
    CUdeviceptr fl[7] = {d_rho, d_ux, d_uy, d_uz, d_phi, d_ted, d_Ked};
    for (int k = 0; k < 7; ++k) CU(cuMemcpyHtoD(fl[k], f7.data() + k * S, S));
    Launch().a(d_fx).a(d_fy).a(d_fz).a(d_phi).run("forcing", (LX + 7) / 8, (LY + 7) / 8, (LZ + 3) / 4, 8, 8, 4);
    if (NP > 0) {
        memcpy_dd(d_ibnode_prev, d_ibnode, L * 4);
        memcpy_dd(d_owner_prev, d_owner, L * 4);
    }
    CU(cuCtxSynchronize());
    if (nu_mode) {
        f.clear(); f.shrink_to_fit(); g.clear(); g.shrink_to_fit();
        const int every = std::atoi(argv[5]);
        if (every <= 0) { std::fprintf(stderr, "every must be positive\n"); return 2; }
        std::vector<double> rows;
        double row[7];
        for (int s = 1; s <= nsteps; ++s) {
            step();
            if (s % every == 0) {
                CU(cuCtxSynchronize());
                nu_row(s, row);
                rows.insert(rows.end(), row, row + 7);
            }
        }
        dump(argv[6], rows.data(), rows.size() * 8);
        CU(cuModuleUnload(mod));
        CU(cuDevicePrimaryCtxRelease(dev));
        std::printf("ref_driver: %d steps, %zu Nu rows\n", nsteps, rows.size() / 7);
        return 0;
    }
    if (timing) {
        f.clear(); f.shrink_to_fit(); g.clear(); g.shrink_to_fit();
        const int warm = std::atoi(argv[4]), steps = std::atoi(argv[5]);
        for (int s = 0; s < warm; ++s) step();
        CU(cuCtxSynchronize());
        g_scan_seconds = 0.0;
        const auto t0 = std::chrono::steady_clock::now();
        for (int s = 0; s < steps; ++s) step();
        CU(cuCtxSynchronize());
        const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        // state check: non-finite temperatures after the run
        std::vector<double> phi(L);
        CU(cuMemcpyDtoH(phi.data(), d_phi, L * sizeof(double)));
        long long bad = 0;
        for (long long n = 0; n < L; ++n) bad += std::isfinite(phi[n]) ? 0 : 1;
        std::printf("ref_time ms_per_step %.6f ms_per_step_with_host_scans %.6f steps %d warmup %d nodes %lld "
                    "npart %d links %d nonfinite %lld\n", 1e3 * (sec - g_scan_seconds) / steps, 1e3 * sec / steps,
                    steps, warm, L, NP, num_links, bad);
        CU(cuModuleUnload(mod));
        CU(cuDevicePrimaryCtxRelease(dev));
        return 0;
    }
    // the link set of the loaded state
    {
        std::vector<Link> lk(num_links);
        if (num_links) CU(cuMemcpyDtoH(lk.data(), d_links, num_links * sizeof(Link)));
        std::vector<double> rec;
        for (auto &l : lk) { rec.push_back(((double)l.ck * LY + l.cj) * LX + l.ci); rec.push_back(l.dir); rec.push_back(l.pid); rec.push_back(l.q); }
        dump(out + "/links0.bin", rec.data(), rec.size() * 8);
        std::vector<int> own(L);
        CU(cuMemcpyDtoH(own.data(), d_owner, L * 4));
        dump(out + "/owner0.bin", own.data(), L * 4);
    }

    for (int s = 0; s < nsteps; ++s) step();

    const long long stride = cfg.count("sample_stride") ? (long long)cfg["sample_stride"] : 1;
    CUdeviceptr mp[6] = {d_rho, d_ux, d_uy, d_uz, d_phi, d_fx};
    if (stride > 1) {
        f.clear(); f.shrink_to_fit(); g.clear(); g.shrink_to_fit();
        auto fs = sampled(d_f, 27, stride), gs = sampled(d_g, 27, stride);
        dump(out + "/f.bin", fs.data(), fs.size() * 8);
        dump(out + "/g.bin", gs.data(), gs.size() * 8);
        std::vector<double> mac;
        for (int k = 0; k < 6; ++k) {
            auto m = sampled(mp[k], 1, stride);
            mac.insert(mac.end(), m.begin(), m.end());
        }
        dump(out + "/macros.bin", mac.data(), mac.size() * 8);
        std::vector<double> plane(L), norms;
        for (CUdeviceptr d : {d_f, d_g}) {
            for (int i = 0; i < 27; ++i) {
                CU(cuMemcpyDtoH(plane.data(), d + (size_t)i * L * 8, L * 8));
                // compensated (Neumaier) sums: accurate to a few units in the last place, so the
                // comparison measures the fields and not this summation order
                double s1 = 0.0, c1 = 0.0, s2 = 0.0, c2 = 0.0;
                auto add = [](double &sum, double &comp, double v) {
                    const double t = sum + v;
                    comp += std::fabs(sum) >= std::fabs(v) ? (sum - t) + v : (v - t) + sum;
                    sum = t;
                };
                for (long long n = 0; n < L; ++n) { add(s1, c1, plane[n]); add(s2, c2, plane[n] * plane[n]); }
                norms.push_back(s1 + c1);
                norms.push_back(s2 + c2);
            }
        }
        // [f or g][direction][sum, sum of squares] reordered to [direction][f sum, f sq, g sum, g sq]
        std::vector<double> fgn(27 * 4);
        for (int i = 0; i < 27; ++i) {
            fgn[4 * i + 0] = norms[2 * i]; fgn[4 * i + 1] = norms[2 * i + 1];
            fgn[4 * i + 2] = norms[54 + 2 * i]; fgn[4 * i + 3] = norms[54 + 2 * i + 1];
        }
        dump(out + "/fgnorm.bin", fgn.data(), fgn.size() * 8);
    } else {
        std::vector<char> buf(P);
        CU(cuMemcpyDtoH(buf.data(), d_f, P)); dump(out + "/f.bin", buf.data(), P);
        CU(cuMemcpyDtoH(buf.data(), d_g, P)); dump(out + "/g.bin", buf.data(), P);
        std::vector<double> mac(6 * (size_t)L);
        for (int k = 0; k < 6; ++k) CU(cuMemcpyDtoH(mac.data() + k * L, mp[k], S));
        dump(out + "/macros.bin", mac.data(), mac.size() * 8);
    }
    if (NP > 0) {
        std::vector<double> rows((size_t)NP * 33), col(NP);
        CUdeviceptr *src[10] = {d_pos, d_vel, d_facc, d_fprev, d_fprev2, d_th, d_omg, d_tacc, d_tprev, d_tprev2};
        for (int blk = 0; blk < 10; ++blk)
            for (int a = 0; a < 3; ++a) {
                CU(cuMemcpyDtoH(col.data(), src[blk][a], NP * 8));
                for (int p = 0; p < NP; ++p) rows[p * 33 + 3 * blk + a] = col[p];
            }
        CUdeviceptr last[3] = {d_ptemp, d_pheat, d_pheat_prev};
        for (int k = 0; k < 3; ++k) {
            CU(cuMemcpyDtoH(col.data(), last[k], NP * 8));
            for (int p = 0; p < NP; ++p) rows[p * 33 + 30 + k] = col[p];
        }
        dump(out + "/particles.bin", rows.data(), rows.size() * 8);
        std::vector<int> own(L);
        CU(cuMemcpyDtoH(own.data(), d_owner, L * 4));
        dump(out + "/owner.bin", own.data(), L * 4);
        std::vector<Link> lk(num_links);
        if (num_links) CU(cuMemcpyDtoH(lk.data(), d_links, num_links * sizeof(Link)));
        std::vector<double> rec;
        for (auto &l : lk) { rec.push_back(((double)l.ck * LY + l.cj) * LX + l.ci); rec.push_back(l.dir); rec.push_back(l.pid); rec.push_back(l.q); }
        dump(out + "/links.bin", rec.data(), rec.size() * 8);
        std::vector<int> nn(num_nf), npd(num_nf);
        if (num_nf) {
            CU(cuMemcpyDtoH(nn.data(), d_nf_nodes, num_nf * 4));
            CU(cuMemcpyDtoH(npd.data(), d_nf_pids, num_nf * 4));
        }
        std::vector<int> nf;
        for (int k = 0; k < num_nf; ++k) { nf.push_back(nn[k]); nf.push_back(npd[k]); }
        dump(out + "/newfluid.bin", nf.data(), nf.size() * 4);
    }
    CU(cuModuleUnload(mod));
    CU(cuDevicePrimaryCtxRelease(dev));
    std::printf("ref_driver: %d steps, %d links, %d new-fluid nodes\n", nsteps, num_links, num_nf);
    return 0;
}

}  // namespace

int main(int argc, char **argv) { return run(argc, argv); }
