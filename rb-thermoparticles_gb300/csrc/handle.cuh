// handle.cuh — the host-side state of one cavity (rbtp_handle), shared by the single-cavity C ABI
// (api.cu) and batched execution (batch.cu).
#pragma once

#include <string>
#include <vector>

#include "rbtp_internal.cuh"

using namespace rbtp;

struct rbtp_handle {
    // batch membership (batch.cu)
    struct rbtp_batch *batch = nullptr;
    int sample_every = 0;
    int stop_at = 0;                 // batched runs: step at which the cavity stops (<= 0: never)
    double *ring = nullptr;          // batched runs: device sample ring (step + plane sums per slot)
    int ring_cap = 0;
    int ring_drained = 0;            // samples already turned into Nu rows
    rbtp_config cfg;
    rbtp_derived der;
    Geo geo;
    Phys ph;
    int mode = RBTP_STORE_F64;
    int device = 0;
    cudaStream_t stream = nullptr;
    // particle steps: side stream for the contacts, which run beside IBB, with its fork/join events
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_side = nullptr;
    void *f = nullptr, *g = nullptr;    // the population array (g == f in the paired float modes)
    int phase = PHASE_HOME;
    double *faux = nullptr, *rho_wall = nullptr;
    double *rho = nullptr, *ux = nullptr, *uy = nullptr, *uz = nullptr, *phi = nullptr;
    double *ted = nullptr, *ked = nullptr;
    double *fcol = nullptr, *gcol = nullptr;  // FP64 scratch (collided copy / export / import)
    DevStatus *status = nullptr;
    DevStatus *status_host = nullptr;
    // particles
    PartBuffers pb{};
    int *owner[2] = {nullptr, nullptr};
    int ocur = 0;
    // diagnostics
    double *partials = nullptr, *plane = nullptr;
    int nchunks = 1;
    std::vector<double> plane_host;
    bool plane_valid = false;
    // bookkeeping
    int istep = 0;
    bool initialised = false;
    bool macros_valid = false;
    bool dissip_valid = false;
    std::string err;
};

bool rbtp_batch_busy(const rbtp_handle *h);  // batch.cu

namespace rbtp {
// The Nu row of output_nu (output_statis.cu:111-223) from the ten plane sums of a state.
int nu_from_planes(rbtp_handle *h, const double *planes, int istep, rbtp_nu_row *row);
}  // namespace rbtp

