// diagnostics.cu — on-device reductions for the reference's statistics and Nusselt outputs.
//
// output/output_statis.cu copies whole fields to the host every NDIAG/NNUOUT steps and loops over
// them serially.  Here one coalesced pass produces, for every x plane, the ten sums the three
// diagnostics need; the host then applies the reference's formulas to lx*10 numbers.  Partial sums
// are combined in a fixed order, so results are deterministic run to run.
//   q0  sum over fluid nodes of ux*phi           (output_nu, output_statis.cu:128-153)
//   q1  number of fluid nodes
//   q2  sum over solid nodes of ux*phi
//   q3  number of solid nodes
//   q4  wall sum: (T_HOT - phi)/0.5 at x = 0, (phi - T_COLD)/0.5 at x = LX-1, fluid nodes only
//   q5  wall count
//   q6..q9  sums of ux, uy, uz, phi with solid nodes replaced by the rigid-body velocity and the
//           particle temperature (overwrite_particle_nodes, output_statis.cu:5-60)
#include "rbtp_internal.cuh"

namespace rbtp {

namespace {

constexpr int PLANE_TX = 128;

// Sums of plane ix over row chunk `chunk` of nchunks (rows = (y, z) pairs in z-major order).
__device__ __forceinline__ void plane_partial_body(const Geo &geo, const Phys &ph, const double *ux,
                                                   const double *uy, const double *uz, const double *phi,
                                                   const int *owner, const double *pst, int np,
                                                   double *partials, int nchunks, int ix, int chunk)
{
    const long long rows = (long long)geo.ly * geo.lz;
    const long long r0 = rows * chunk / nchunks, r1 = rows * (chunk + 1) / nchunks;
    double q[NPLANEQ];
#pragma unroll
    for (int k = 0; k < NPLANEQ; ++k) q[k] = 0.0;
    for (long long r = r0; r < r1; ++r) {
        const int iz = (int)(r / geo.ly);
        const int iy = (int)(r - (long long)iz * geo.ly);
        const long long idx = (long long)iz * geo.lxy + (long long)iy * geo.lx + ix;
        const double u = ux[idx], v = uy[idx], w = uz[idx], T = phi[idx];
        const int own = owner ? owner[idx] : -1;
        if (own < 0) {
            q[0] += u * T;
            q[1] += 1.0;
            if (ix == 0) { q[4] += (ph.thot - T) / 0.5; q[5] += 1.0; }
            else if (ix == geo.lx - 1) { q[4] += (T - ph.tcold) / 0.5; q[5] += 1.0; }
            q[6] += u; q[7] += v; q[8] += w; q[9] += T;
        } else {
            q[2] += u * T;
            q[3] += 1.0;
            if (own < np) {
                const double relx = ((double)ix + 0.5) - pst[0 * (long long)np + own];
                const double rely = ((double)iy + 0.5) - pst[1 * (long long)np + own];
                const double relz = ((double)iz + 0.5) - pst[2 * (long long)np + own];
                const double wx = pst[18 * (long long)np + own], wy = pst[19 * (long long)np + own],
                             wz = pst[20 * (long long)np + own];
                q[6] += pst[3 * (long long)np + own] + (relz * wy - rely * wz);
                q[7] += pst[4 * (long long)np + own] + (relx * wz - relz * wx);
                q[8] += pst[5 * (long long)np + own] + (rely * wx - relx * wy);
                q[9] += pst[30 * (long long)np + own];
            } else {
                q[6] += u; q[7] += v; q[8] += w; q[9] += T;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < NPLANEQ; ++k) partials[((long long)chunk * NPLANEQ + k) * geo.lx + ix] = q[k];
}

__global__ void __launch_bounds__(PLANE_TX) k_plane_partial(const Geo geo, const Phys ph,
                                                            const double *ux, const double *uy,
                                                            const double *uz, const double *phi,
                                                            const int *owner, const double *pst,
                                                            int np, double *partials, int nchunks)
{
    const int ix = blockIdx.x * PLANE_TX + threadIdx.x;
    if (ix >= geo.lx) return;
    plane_partial_body(geo, ph, ux, uy, uz, phi, owner, pst, np, partials, nchunks, ix, blockIdx.y);
}

// Chunks are combined in ascending order: the plane sums are deterministic and identical in the
// single-cavity and the batched reductions.
__device__ __forceinline__ double plane_final_body(const double *partials, int nchunks, int lx, int t)
{
    const int k = t / lx, ix = t - k * lx;
    double s = 0.0;
    for (int c = 0; c < nchunks; ++c) s += partials[((long long)c * NPLANEQ + k) * lx + ix];
    return s;
}

__global__ void k_plane_final(const Geo geo, const double *partials, int nchunks, double *plane)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= NPLANEQ * geo.lx) return;
    plane[t] = plane_final_body(partials, nchunks, geo.lx, t);
}

// Batched sampling, after the step's advance: cavities with samp_now set reduce their current
// macroscopic fields (owners of the new solid flags, particle state after the update) exactly as
// the single-cavity reduction does, and the final pass writes (step, plane sums) into the next slot
// of the cavity's sample ring and bumps its sample counter.
__global__ void __launch_bounds__(PLANE_TX) k_batch_sample_partial(const CavDesc *desc)
{
    pdl_wait();
    pdl_trigger();
    const CavDesc &d = desc[blockIdx.y];
    if (!d.samp_now) return;
    const int *owner = d.pb.np > 0 ? d.owner[d.ocur] : nullptr;
    for (int chunk = blockIdx.x; chunk < d.nchunks; chunk += gridDim.x)
        for (int ix = threadIdx.x; ix < d.geo.lx; ix += PLANE_TX)
            plane_partial_body(d.geo, d.ph, d.ux, d.uy, d.uz, d.phi, owner, d.pb.state, d.pb.np, d.partials,
                               d.nchunks, ix, chunk);
}

__global__ void k_batch_sample_final(const CavDesc *desc)
{
    pdl_wait();
    pdl_trigger();
    const CavDesc &d = desc[blockIdx.x];
    if (!d.samp_now) return;
    const int lx = d.geo.lx;
    const int slot = d.status->nsamp % d.samp_cap;
    double *dst = d.samp + (long long)slot * (1 + NPLANEQ * lx);
    for (int t = threadIdx.x; t < NPLANEQ * lx; t += blockDim.x)
        dst[1 + t] = plane_final_body(d.partials, d.nchunks, lx, t);
    if (threadIdx.x == 0) dst[0] = (double)d.istep;
    __syncthreads();
    if (threadIdx.x == 0) d.status->nsamp += 1;
}

// compute_Ked (collision.cu:91-152) and compute_ted (collision.cu:154-198) on the FP64 copy of
// the step's post-collision populations; solid nodes are then zeroed as output_flow does.
__global__ void k_dissipation(const Geo geo, const Phys ph, const double *fcol, const double *gcol,
                              const double *rho, const double *ux, const double *uy,
                              const double *uz, const double *phi, const void *faux, bool aux32,
                              const int *owner, double *ted, double *ked)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= geo.L) return;
    const long long L = geo.L;
    const double fx = aux32 ? (double)static_cast<const float *>(faux)[idx] : static_cast<const double *>(faux)[idx];
    const double fy = 0.0, fz = 0.0;
    const double r = rho[idx], ph_ = phi[idx];
    const double u = ux[idx], v = uy[idx], w = uz[idx];
    const double RT = 1.0 / 3.0;
    const double u2 = u * u + v * v + w * w;
    const double uv = u2 / RT;
    const double bu = fx * u + fy * v + fz * w;
    double txx = 0, txy = 0, txz = 0, tyy = 0, tyz = 0, tzz = 0;
    double gnx = 0, gny = 0, gnz = 0;
    const double lambda0 = 1.0 - dweight(0);
    unroll<27>([&](auto I) {
        constexpr int i = decltype(I)::value;
        constexpr int cx = dcx(i), cy = dcy(i), cz = dcz(i);
        constexpr double wi = dweight(i);
        const double eu = (cx * u + cy * v + cz * w) / RT;
        const double feq = wi * (r + eu + 0.5 * (eu * eu - uv));
        const double fneq = fcol[(long long)i * L + idx] - feq;
        const double cidotF = cx * fx + cy * fy + cz * fz;
        const double feq_term = 0.5 * (cidotF - bu) * feq / RT;
        const double s = fneq + feq_term;
        txx += cx * cx * s; txy += cx * cy * s; txz += cx * cz * s;
        tyy += cy * cy * s; tyz += cy * cz * s; tzz += cz * cz * s;
        const double geq = wi * ph_ * (1.0 + eu + 0.5 * (eu * eu - uv));
        const double geqnew = (i == 0) ? (geq - lambda0 * ph_ * r) : (geq + wi * ph_ * r);
        const double dif = gcol[(long long)i * L + idx] - geqnew;
        gnx += cx * dif; gny += cy * dif; gnz += cz * dif;
    });
    const double coeff = -(1.0 - 0.5 / ph.tau);
    txx *= coeff; txy *= coeff; txz *= coeff; tyy *= coeff; tyz *= coeff; tzz *= coeff;
    const double v2 = 2.0 * ph.visc;
    const double Sxx = txx / v2, Sxy = txy / v2, Sxz = txz / v2;
    const double Syy = tyy / v2, Syz = tyz / v2, Szz = tzz / v2;
    double kv = 0.5 * ph.visc * (4.0 * (Sxx * Sxx + Syy * Syy + Szz * Szz) + 8.0 * (Sxy * Sxy + Sxz * Sxz + Syz * Syz));
    const double p = r * RT;
    const double den = 2.0 * ph.tauc * RT + p;
    const double tx = -(2.0 * gnx + ph_ * fx) / den;
    const double ty = -(2.0 * gny + ph_ * fy) / den;
    const double tz = -(2.0 * gnz + ph_ * fz) / den;
    double tv = (ph.diff > 0.0) ? ph.diff * (tx * tx + ty * ty + tz * tz) : 0.0;
    if (owner && owner[idx] >= 0) { kv = 0.0; tv = 0.0; }
    ked[idx] = kv;
    ted[idx] = tv;
}

}  // namespace

cudaError_t launch_batch_sample(const CavDesc *desc, int n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    cudaError_t e = pdl_launch(k_batch_sample_partial, dim3(64, n), dim3(PLANE_TX), st, desc);
    if (e != cudaSuccess) return e;
    return pdl_launch(k_batch_sample_final, dim3(n), dim3(256), st, desc);
}

cudaError_t launch_plane_sums(const Geo &geo, const Phys &ph, const double *ux, const double *uy,
                              const double *uz, const double *phi, const int *owner,
                              const double *pstate, int np, double *partials, int nchunks,
                              double *plane, cudaStream_t st)
{
    const dim3 grd((geo.lx + PLANE_TX - 1) / PLANE_TX, nchunks, 1);
    k_plane_partial<<<grd, PLANE_TX, 0, st>>>(geo, ph, ux, uy, uz, phi, owner, pstate, np, partials, nchunks);
    const int n = NPLANEQ * geo.lx;
    k_plane_final<<<(n + 255) / 256, 256, 0, st>>>(geo, partials, nchunks, plane);
    return cudaGetLastError();
}

cudaError_t launch_dissipation(int mode, const Geo &geo, const Phys &ph, const double *fcol,
                               const double *gcol, const double *rho, const double *ux,
                               const double *uy, const double *uz, const double *phi,
                               const void *faux, const int *owner, double *ted, double *ked,
                               cudaStream_t st)
{
    k_dissipation<<<(unsigned)((geo.L + 127) / 128), 128, 0, st>>>(geo, ph, fcol, gcol, rho, ux, uy, uz, phi, faux,
                                                                   mode != RBTP_STORE_F64, owner, ted, ked);
    return cudaGetLastError();
}

}  // namespace rbtp
