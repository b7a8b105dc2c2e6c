// noalloc.cu — an allocation-free variant of the per-plane diagnostic sums.
//
// rbtp_nu / rbtp_means / rbtp_profile reduce the macroscopic fields through a partial-sum scratch
// buffer that the handle allocates with cudaMalloc.  Some callers cannot allocate device memory:
// code hosted inside a framework that owns the whole device memory pool and hands out no raw
// allocations, or a latency-critical loop where the implicit device synchronisation of cudaMalloc
// and cudaFree is not acceptable.  rbtp_plane_sums_noalloc serves them: the caller passes device
// pointers to the fields and to the output, and the partial sums live in a fixed file-scope
// device array (g_plane_scratch below, NOALLOC_SLOTS x 10 doubles = 2.6 MB), which every GPU that
// loads this library holds until the process exits.  The reduction itself is the handle's
// (launch_plane_sums in diagnostics.cu, the same kernels), run with the fixed array as its
// partial-sum buffer and as many row chunks as the array holds for the lattice's lx (at most the
// handle's 512).
//
// The per-device address of that array is obtained once per device, on that device's first call,
// with cudaGetSymbolAddress (host code cannot use the array's name as a device address).  Make the
// first call on each device before any stream capture.  The cached address belongs to the device's
// primary context as the CUDA runtime sets it up: after cudaDeviceReset, or with another driver
// context current, it is stale.  Every call shares the array: calls that overlap on the GPU
// (different streams, or several host threads without ordering) race on it.  Each call writes every
// scratch element it later reads, so nothing needs clearing between calls.
#include <algorithm>
#include <mutex>

#include "rbtp_internal.cuh"

namespace rbtp {
namespace {

// (row chunk, plane) slots of ten partial sums each: 32 chunks of RBTP_NOALLOC_MAX_LX planes
constexpr long long NOALLOC_SLOTS = 32LL * RBTP_NOALLOC_MAX_LX;
constexpr int HANDLE_CHUNKS = 512;   // the handle's chunk count (rbtp_create)

static __device__ __align__(256) double g_plane_scratch[NOALLOC_SLOTS * NPLANEQ];

std::mutex g_scratch_mutex;
double *g_scratch_ptr[256] = {};  // per device ordinal

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
    // the lattice sizes rbtp_create accepts (x = 0 and x = LX - 1 are distinct wall planes)
    if (lx < 3 || ly < 3 || lz < 3 || npart < 0) return RBTP_ERR_ARG;
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
    Geo geo{};
    geo.lx = lx; geo.ly = ly; geo.lz = lz;
    geo.lxy = (long long)lx * ly;
    geo.L = geo.lxy * lz;
    Phys ph{};            // the plane sums read only the wall temperatures
    ph.thot = t_hot;
    ph.tcold = t_cold;
    const long long rows = (long long)ly * lz;
    const int nchunks = (int)std::min<long long>({rows, (long long)HANDLE_CHUNKS, NOALLOC_SLOTS / lx});
    const cudaError_t e = launch_plane_sums(geo, ph, ux, uy, uz, phi, owner, particle_state, npart, scratch,
                                            nchunks, plane_sums, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return RBTP_ERR_CUDA;
    }
    return RBTP_OK;
}
