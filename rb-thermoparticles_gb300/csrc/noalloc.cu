// noalloc.cu — an allocation-free variant of the per-plane diagnostic sums.
//
// rbtp_nu / rbtp_means / rbtp_profile reduce the macroscopic fields through a partial-sum scratch
// buffer that the handle allocates with cudaMalloc.  Some callers cannot allocate device memory:
// code hosted inside a framework that owns the whole device memory pool and hands out no raw
// allocations, or a latency-critical loop where the implicit device synchronisation of cudaMalloc
// and cudaFree is not acceptable.  rbtp_plane_sums_noalloc serves them: the caller passes device
// pointers to the fields and to the output, and the partial sums live in a fixed file-scope
// device array (g_plane_scratch below, NOALLOC_CHUNKS x 10 x RBTP_NOALLOC_MAX_LX doubles =
// 2.6 MB), which every GPU that loads this library holds until the process exits.
//
// The per-device address of that array is obtained once per device, on that device's first call,
// with cudaGetSymbolAddress (host code cannot use the array's name as a device address).  Make the
// first call on each device before any stream capture.  Every call shares the array: calls that
// overlap on the GPU (different streams, or several host threads without ordering) race on it.
// Each call writes every scratch element it later reads, so nothing needs clearing between calls.
#include <mutex>

#include "rbtp_internal.cuh"

namespace rbtp {
namespace {

constexpr int NOALLOC_CHUNKS = 32;
constexpr int NOALLOC_TX = 128;

static __device__ __align__(256) double g_plane_scratch[NOALLOC_CHUNKS * NPLANEQ * RBTP_NOALLOC_MAX_LX];

std::mutex g_scratch_mutex;
double *g_scratch_ptr[256] = {};  // per device ordinal

// Same ten per-plane quantities as the handle's reduction (diagnostics.cu).
__global__ void __launch_bounds__(NOALLOC_TX) k_noalloc_partial(
    int lx, int ly, int lz, double thot, double tcold, const double *ux, const double *uy,
    const double *uz, const double *phi, const int *owner, const double *pst, int np,
    double *scratch)
{
    const int ix = blockIdx.x * NOALLOC_TX + threadIdx.x;
    const int chunk = blockIdx.y;
    if (ix >= lx) return;
    const long long lxy = (long long)lx * ly;
    const long long rows = (long long)ly * lz;
    const long long r0 = rows * chunk / NOALLOC_CHUNKS, r1 = rows * (chunk + 1) / NOALLOC_CHUNKS;
    double q[NPLANEQ];
#pragma unroll
    for (int k = 0; k < NPLANEQ; ++k) q[k] = 0.0;
    for (long long r = r0; r < r1; ++r) {
        const int iz = (int)(r / ly);
        const int iy = (int)(r - (long long)iz * ly);
        const long long idx = (long long)iz * lxy + (long long)iy * lx + ix;
        const double u = ux[idx], v = uy[idx], w = uz[idx], T = phi[idx];
        const int own = owner ? owner[idx] : -1;
        if (own < 0) {
            q[0] += u * T;
            q[1] += 1.0;
            if (ix == 0) { q[4] += (thot - T) / 0.5; q[5] += 1.0; }
            else if (ix == lx - 1) { q[4] += (T - tcold) / 0.5; q[5] += 1.0; }
            q[6] += u; q[7] += v; q[8] += w; q[9] += T;
        } else {
            q[2] += u * T;
            q[3] += 1.0;
            if (own < np) {
                const long long n = np;
                const double relx = ((double)ix + 0.5) - pst[0 * n + own];
                const double rely = ((double)iy + 0.5) - pst[1 * n + own];
                const double relz = ((double)iz + 0.5) - pst[2 * n + own];
                const double wx = pst[18 * n + own], wy = pst[19 * n + own], wz = pst[20 * n + own];
                q[6] += pst[3 * n + own] + (relz * wy - rely * wz);
                q[7] += pst[4 * n + own] + (relx * wz - relz * wx);
                q[8] += pst[5 * n + own] + (rely * wx - relx * wy);
                q[9] += pst[30 * n + own];
            } else {
                q[6] += u; q[7] += v; q[8] += w; q[9] += T;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < NPLANEQ; ++k) scratch[((long long)chunk * NPLANEQ + k) * lx + ix] = q[k];
}

__global__ void k_noalloc_final(int lx, const double *scratch, double *plane)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= NPLANEQ * lx) return;
    const int k = t / lx, ix = t - k * lx;
    double s = 0.0;
    for (int c = 0; c < NOALLOC_CHUNKS; ++c) s += scratch[((long long)c * NPLANEQ + k) * lx + ix];
    plane[t] = s;
}

}  // namespace
}  // namespace rbtp

extern "C" int rbtp_plane_sums_noalloc(const double *ux, const double *uy, const double *uz,
                                       const double *phi, const int *owner,
                                       const double *particle_state, int npart, int lx, int ly,
                                       int lz, double t_hot, double t_cold, double *plane_sums,
                                       void *stream)
{
    using namespace rbtp;
    if (!ux || !uy || !uz || !phi || !plane_sums) return RBTP_ERR_ARG;
    if (lx < 1 || ly < 1 || lz < 1 || npart < 0) return RBTP_ERR_ARG;
    if (lx > RBTP_NOALLOC_MAX_LX) return RBTP_ERR_CAPACITY;  // the scratch holds at most this many planes
    if (owner && npart > 0 && !particle_state) return RBTP_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) {
        cudaGetLastError();
        return RBTP_ERR_CUDA;
    }
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_ptr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_plane_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return RBTP_ERR_CUDA;
            }
            g_scratch_ptr[dev] = static_cast<double *>(p);
        }
        scratch = g_scratch_ptr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const dim3 grd((lx + NOALLOC_TX - 1) / NOALLOC_TX, NOALLOC_CHUNKS, 1);
    k_noalloc_partial<<<grd, NOALLOC_TX, 0, st>>>(lx, ly, lz, t_hot, t_cold, ux, uy, uz, phi,
                                                  owner, particle_state, npart, scratch);
    const int n = NPLANEQ * lx;
    k_noalloc_final<<<(n + 255) / 256, 256, 0, st>>>(lx, scratch, plane_sums);
    return cudaGetLastError() == cudaSuccess ? RBTP_OK : RBTP_ERR_CUDA;
}
