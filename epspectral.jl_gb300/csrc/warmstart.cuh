// warmstart.cuh -- the hook through which the scGD0 iteration applies the learned warm start.
#pragma once
#include "common.cuh"

struct epsp_warmstart;

namespace epsp {

// Σ_T [nω, ni] (column-major, the iteration's current self-energy of one temperature) += the
// network's correction, computed from Σ_T itself (the G0D0 self-energy when called after the first
// iteration), T, μ, the coupling scale and ε_i (device array [ni]); all on ctx's stream. Fails with
// EPSP_EINVAL when the network's widths are not [2 nω + 4, ..., 2 nω], when it has no feature
// scaling, or when it lives on another context. With tc_err (a device flag the caller reads back),
// the network runs on the tensor cores and its bounded waits report there; without, on the SIMT
// kernels of the training.
void warmstart_correct(epsp_warmstart* w, Ctx* ctx, double2* S_T, long nw, long ni, const double* d_eps_i, double T,
                       double mu, double scale, int* tc_err = nullptr);

}  // namespace epsp
