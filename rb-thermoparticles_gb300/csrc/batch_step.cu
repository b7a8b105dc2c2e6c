// batch_step.cu — device side of batched execution: many independent cavities (any sizes, Ra, Pr,
// particle counts, one storage mode) advanced by ONE persistent launch of the fused step over a
// packed tile table, plus the small plan/advance kernels that keep each cavity's step state on the
// device so that the whole step can be captured once in a CUDA graph and replayed.
//
// Tile table: int4 (cavity, tile_x, tile_y, z) for every TX x TY tile of every cavity, packed
// cavity after cavity.  The persistent grid (chosen by the host autotuner, a multiple of the SM
// count) walks the table with a grid stride, so small and large cavities share the machine without
// per-cavity launches.
#include "step_node.cuh"

namespace rbtp {

namespace {

__device__ __forceinline__ bool hits(int istep, int every) { return every > 0 && istep % every == 0; }

// Decide every cavity's output mode for the coming step (the cadence logic of main.cu:98-114 plus
// the batch's sampling cadence and stop step) and reset the per-step particle counters.  A cavity
// at its stop step is idle: every batched kernel skips it and its state stays as it is.
__global__ void k_batch_plan(CavDesc *desc, int n)
{
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
        CavDesc &d = desc[m];
        if (d.stop_at > 0 && d.istep >= d.stop_at) {
            d.out = OUT_IDLE;
            d.samp_now = 0;
            continue;
        }
        const int istep = d.istep + 1;
        const bool samp = d.samp != nullptr && (hits(istep, d.every) || istep == d.stop_at);
        const bool macro = hits(istep, d.ndiag) || hits(istep, d.nnuout) || hits(istep, d.nflowout) ||
                           istep == d.nend || hits(istep, d.every) || samp;
        d.samp_now = samp ? 1 : 0;
        d.out = macro ? OUT_MACROS : (d.pb.np > 0 ? OUT_RHO : OUT_NONE);
        if (d.pb.np > 0) {
            d.status->nf_count = 0;
            d.status->ncontacts = 0;
        }
    }
}

__global__ void k_batch_advance(CavDesc *desc, int n)
{
    pdl_wait();
    pdl_trigger();
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
        CavDesc &d = desc[m];
        if (d.out == OUT_IDLE) continue;
        d.last_out = d.out;
        if (d.pb.np > 0) d.ocur ^= 1;
        d.phase = d.phase == PHASE_SWAPPED ? PHASE_HOME : PHASE_SWAPPED;   // AA: even and odd alternate
        d.istep += 1;
    }
}

template <int MODE, bool ODD>
__device__ __forceinline__ void step_out(const Geo &geo, const Phys &ph, const AAOff &ao, const StepBuffers &b,
                                         int out, int ix, int iy, int iz)
{
    if (out == OUT_NONE) step_node<MODE, ODD, OUT_NONE, false, MODE != RBTP_STORE_F64, true>(geo, ph, b, ao, ix, iy, iz);
    else if (out == OUT_RHO) step_node<MODE, ODD, OUT_RHO, false, MODE != RBTP_STORE_F64, true>(geo, ph, b, ao, ix, iy, iz);
    else step_node<MODE, ODD, OUT_MACROS, false, MODE != RBTP_STORE_F64, true>(geo, ph, b, ao, ix, iy, iz);
}

// The batched kernel carries all phase/output variants of the step body behind block-uniform
// branches; it is given more registers than the single-cavity kernel (4 resident blocks of 128)
// to keep them in registers.  Its step body takes the scatter index from an opaque copy
// (FRESH_SCATTER), the odd-step offsets from the member's AAOff staged in shared memory, and the
// face tests from per-node masks (FACE_MASK); see step_node.cuh for what each is worth.
#ifndef RBTP_BATCH_MINB_LOW
#define RBTP_BATCH_MINB_LOW 4
#endif

template <int MODE, int TX, int TY>
__global__ void __launch_bounds__(TX * TY, MODE == RBTP_STORE_F64 ? RBTP_STEP_MINB_F64 : RBTP_BATCH_MINB_LOW)
    k_step_batched(const CavDesc *__restrict__ desc, const int4 *__restrict__ tiles, int ntiles)
{
    pdl_wait();
    pdl_trigger();
    // the member's lattice and relaxation constants, staged per tile in shared memory (the step body
    // reads them many times; the single-cavity kernel has them as launch parameters)
    __shared__ Geo sgeo;
    __shared__ Phys sph;
    __shared__ AAOff soff;
    constexpr int GW = sizeof(Geo) / 4, PW = sizeof(Phys) / 4, OW = sizeof(AAOff) / 4;
    const int tid = threadIdx.y * TX + threadIdx.x;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int4 tl = tiles[t];
        const CavDesc &d = desc[tl.x];
        __syncthreads();   // the previous tile's readers are done
        for (int k = tid; k < GW + PW + OW; k += TX * TY) {
            if (k < GW) reinterpret_cast<int *>(&sgeo)[k] = reinterpret_cast<const int *>(&d.geo)[k];
            else if (k < GW + PW) reinterpret_cast<int *>(&sph)[k - GW] = reinterpret_cast<const int *>(&d.ph)[k - GW];
            else reinterpret_cast<int *>(&soff)[k - GW - PW] = reinterpret_cast<const int *>(&d.aoff)[k - GW - PW];
        }
        __syncthreads();
        // tile (member, x, y, z0): BATCH_TILE_Z planes from z0
        const int ix = tl.y * TX + threadIdx.x, iy = tl.z * TY + threadIdx.y, z0 = tl.w;
        if (d.out == OUT_IDLE || ix >= sgeo.lx || iy >= sgeo.ly) continue;
        StepBuffers b;
        b.f = d.f;
        b.g = d.g;
        b.faux = d.faux;
        b.rho_wall = d.rho_wall;
        b.rho = d.rho; b.ux = d.ux; b.uy = d.uy; b.uz = d.uz; b.phi = d.phi;
        b.fcol = nullptr; b.gcol = nullptr;
        b.status = d.status;
        const int z1 = min(z0 + BATCH_TILE_Z, sgeo.lz);
        if (d.phase == PHASE_SWAPPED) {
            for (int iz = z0; iz < z1; ++iz) step_out<MODE, true>(sgeo, sph, soff, b, d.out, ix, iy, iz);
        } else {
            for (int iz = z0; iz < z1; ++iz) step_out<MODE, false>(sgeo, sph, soff, b, d.out, ix, iy, iz);
        }
    }
}

template <int MODE>
cudaError_t launch_mode(int shape, const CavDesc *desc, const int4 *tiles, int ntiles, int grid, cudaStream_t st)
{
    if (ntiles <= 0) return cudaSuccess;
    if (shape == 0) return pdl_launch(k_step_batched<MODE, 32, 4>, dim3(grid), dim3(32, 4, 1), st, desc, tiles, ntiles);
    return pdl_launch(k_step_batched<MODE, 64, 2>, dim3(grid), dim3(64, 2, 1), st, desc, tiles, ntiles);
}

}  // namespace

cudaError_t launch_batch_plan(CavDesc *desc, int n, cudaStream_t st)
{
    k_batch_plan<<<(n + 127) / 128, 128, 0, st>>>(desc, n);
    return cudaGetLastError();
}

cudaError_t launch_batch_advance(CavDesc *desc, int n, cudaStream_t st)
{
    return pdl_launch(k_batch_advance, dim3((n + 127) / 128), dim3(128), st, desc, n);
}

cudaError_t launch_step_batched(int mode, int shape, const CavDesc *desc, const int4 *tiles, int ntiles,
                                int grid, cudaStream_t st)
{
    switch (mode) {
    case RBTP_STORE_F64: return launch_mode<RBTP_STORE_F64>(shape, desc, tiles, ntiles, grid, st);
    case RBTP_STORE_F32: return launch_mode<RBTP_STORE_F32>(shape, desc, tiles, ntiles, grid, st);
    case RBTP_STORE_F16S: return launch_mode<RBTP_STORE_F16S>(shape, desc, tiles, ntiles, grid, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace rbtp
