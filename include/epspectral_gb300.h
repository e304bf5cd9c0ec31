/*
 * epspectral_gb300.h -- C ABI of the GB300 scGD0 / ladder library (libepspectral_gb300.so).
 *
 * The library replaces the bodies of the two iteration loops of EPSpectral.jl:
 *   _loop_scgd0(setup, occ; eta_min, eta_init, maxiter, tol, backend, gpu_tile, Sigma_init,
 *               fix_mu, omega_acoustic, verbosity)                 src/scgd0.jl:189-346
 *   _loop_ladder(ladder, Sigma, mu, Tlist, Omegas; solver, rtol, maxiter, store_vertex,
 *                backend, gpu_tile, omega_acoustic, verbosity)     src/ladder.jl:303-379
 * and the single operator application apply_ladder_kernel! (src/ladder.jl:245-296) that the
 * reference's tests drive on its own.
 *
 * Conventions (every entry point):
 *  - Arrays are column-major in the reference's index order (the first index varies fastest), so a
 *    Julia caller passes pointer(A) with no copy. Complex arrays are interleaved (re, im) doubles,
 *    the memory layout of Julia's ComplexF64.
 *  - Index arrays (iq_kk, iks_i, iks_f, f_to_i, multiplet lists) are int32 and 0-based.
 *  - Inputs are caller-owned and read only during the call; outputs are caller-allocated. A plan
 *    owns all device memory it uses. No C++ exception crosses the ABI.
 *  - A context is bound to one CUDA device and one stream; it is not thread-safe. Every call is
 *    synchronous on return.
 *  - Every call returns an epsp_status; on failure epsp_last_error(ctx) holds a message.
 */
#ifndef EPSPECTRAL_GB300_H
#define EPSPECTRAL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EPSP_ABI_VERSION 1

/* Status codes. The Julia shim maps EINVAL and ENOROOT_MU to ArgumentError, as the reference
 * throws (src/scgd0.jl:81-113, src/scgd0.jl:316-322, src/ladder.jl:71-80). */
typedef enum epsp_status {
  EPSP_OK = 0,
  EPSP_EINVAL = 1,            /* an argument is out of range */
  EPSP_ENOMEM = 2,            /* a device or host allocation failed */
  EPSP_ENOROOT_MU = 3,        /* no chemical potential in the bracket (src/scgd0.jl:316-322) */
  EPSP_ENOTCONV = 4,          /* reserved: non-convergence is reported through flags, not status */
  EPSP_EDEVICE_TIMEOUT = 5,   /* a bounded device-side wait ran out */
  EPSP_ECUDA = 6,             /* a CUDA runtime call failed */
  EPSP_EUNSUPPORTED = 7       /* the requested path does not apply to these inputs */
} epsp_status;

/* Storage type of g2 (the reference's g2 is Array{FT,3}; the benchmark configurations store it as
 * FP32 or BF16). */
enum { EPSP_F64 = 0, EPSP_F32 = 1, EPSP_BF16 = 2 };

/* occ.type of ElectronOccupationParams (src/scgd0.jl:85-86, 312). */
enum { EPSP_METAL = 0, EPSP_SEMICONDUCTOR = 1 };

/* Computation path of a plan.
 *  DIRECT_FP64 : the reference's element sum, term by term in FP64 (src/scgd0_kernel.jl:27-86) and
 *                the shift-grid coupling of the ladder (src/ladder_kernel.jl:195-288); any phonon
 *                dispersion. This is the parity path.
 *  GEMM_FP64   : dispersionless modes only: the Fan-Migdal sum recast as a kernel tensor times a
 *                coupling matrix, the ladder's shift sums regrouped per mode; FP64 arithmetic.
 *  GEMM_BF16X3 : as GEMM_FP64, with the contractions on the tcgen05 tensor cores in BF16 hi/lo
 *                split precision (three products, FP32 accumulation); the chemical-potential
 *                bisection, the carrier integral and the GMRES orthogonalisation stay FP64.
 *  GEMM_TF32   : ladder plans only: as GEMM_BF16X3, with the ladder contraction as one TF32 product
 *                (operands rounded to TF32, FP32 accumulation): two thirds of the BF16X3 tensor
 *                time, ~2^-11 relative rounding per operand element. scGD0 plans refuse it
 *                (EPSP_EUNSUPPORTED). */
enum { EPSP_PATH_DIRECT_FP64 = 0, EPSP_PATH_GEMM_FP64 = 1, EPSP_PATH_GEMM_BF16 = 2, EPSP_PATH_GEMM_TF32 = 3 };

/* Ladder solver (src/ladder.jl:340-369). */
enum { EPSP_SOLVER_GMRES = 0, EPSP_SOLVER_FIXED_POINT = 1 };

/* A FrequencyGrid (src/frequency_grids.jl:119-133): nodes origin + offsets[j] * unit, offsets
 * strictly increasing, n >= 2. */
typedef struct epsp_grid {
  double origin;
  double unit;
  const int64_t* offsets;  /* [n] */
  int64_t n;
} epsp_grid;

/* The iteration-invariant inputs: the fields of the reference's `setup` NamedTuple
 * (src/scgd0.jl:173-183) plus the ladder's additions (src/ladder.jl:153-157). */
typedef struct epsp_model {
  int64_t nm, ni, nf;        /* modes, outer (irreducible) states, inner (full-BZ) states */
  int32_t g2_dtype;          /* EPSP_F64 / EPSP_F32 / EPSP_BF16 */
  int32_t reserved0;
  const void* g2;            /* [nm, ni, nf] */
  int64_t nq;
  const double* omega_ph;    /* [nm, nq] phonon frequencies */
  int64_t nk_i, nk_f;
  const int32_t* iq_kk;      /* [nk_i, nk_f] q index of a (k_i, k_f) pair */
  const int32_t* iks_i;      /* [ni] k index of each outer state */
  const int32_t* iks_f;      /* [nf] k index of each inner state */
  const double* eps_i;       /* [ni] */
  const double* w_i;         /* [ni] state weights */
  const double* eps_f;       /* [nf] */
  const double* w_f;         /* [nf] */
  const int32_t* f_to_i;     /* [nf] IBZ representative of each inner state */
  int64_t nmult;             /* degenerate multiplets, CSR: members of multiplet m are */
  const int32_t* mult_ptr;   /*   mult_idx[mult_ptr[m] .. mult_ptr[m+1]-1]   ([nmult+1]) */
  const int32_t* mult_idx;
  epsp_grid omegas;          /* output grid ωs */
  epsp_grid omegas_spectral; /* spectral grid ωs_spectral */
  double W;                  /* sum(w_i) */
  double nstates_base;
  const double* R;           /* [3, 3, nf] vertex rotation of each inner state (ladder only) */
  const double* v;           /* [3, ni] band velocities (ladder only) */
} epsp_model;

/* Plan options: the keywords of the reference loops that shape the setup. */
typedef struct epsp_options {
  int32_t path;              /* EPSP_PATH_* */
  int32_t verbosity;
  int64_t gpu_tile;          /* 0 = `nothing`; > 0 = inner states per chunk, g2 streamed */
  double omega_acoustic;     /* modes below it are skipped */
} epsp_options;

/* ElectronOccupationParams fields the loop reads. */
typedef struct epsp_occ {
  int64_t nT;
  const double* Tlist;       /* [nT] */
  const double* nlist;       /* [nT] doping */
  double nelec;
  double spin_degeneracy;
  int32_t type;              /* EPSP_METAL / EPSP_SEMICONDUCTOR */
  int32_t reserved0;
} epsp_occ;

/* `history` of SCGD0Result (src/scgd0.jl:21-23): arrays [nT, maxiter] column-major; entries of
 * iterations a temperature did not run are NaN. niter is the number of iterations run. */
typedef struct epsp_scgd0_history {
  double* err;
  double* mu;
  double* min_spectral_weight;
  double* wall;              /* [maxiter] seconds */
  int32_t* iter_frozen;      /* [nT] iteration at which T converged, 0 if it did not */
  int32_t niter;
  int32_t reserved0;
} epsp_scgd0_history;

/* Ladder history (src/ladder.jl:20-23): GMRES residual norms per (Ω, T), at most maxiter + 1 each,
 * in norms[(maxiter+1) * (iΩ + nΩ iT) + k], their counts in nnorms; fixed-point σ after each
 * iteration in sigma_iter[9 * (maxiter * (iΩ + nΩ iT) + k) + (a + 3b)], their counts in nsigma. */
typedef struct epsp_ladder_history {
  double* norms;
  int32_t* nnorms;
  double* sigma_iter;
  int32_t* nsigma;
} epsp_ladder_history;

typedef struct epsp_ctx epsp_ctx;
typedef struct epsp_scgd0_plan epsp_scgd0_plan;
typedef struct epsp_ladder_plan epsp_ladder_plan;
typedef struct epsp_warmstart epsp_warmstart;

/* ---- context ---- */

/* Binds a context to CUDA device `device`, with its own stream. Replaces the reference's backend
 * object (ElectronPhonon gpu_backend(), used at src/scgd0.jl:189 and src/ladder.jl:303). */
epsp_status epsp_create(epsp_ctx** ctx, int32_t device);
void epsp_destroy(epsp_ctx* ctx);
/* The message of the last failed call on ctx ("" if none). Valid until the next call. */
const char* epsp_last_error(const epsp_ctx* ctx);
/* Number of kernels this context launched since creation (for launch accounting). */
int64_t epsp_kernel_launches(const epsp_ctx* ctx);

/* Library utilities with no counterpart in the reference (benchmarks and tests):
 *  - epsp_profile_kernel brackets every launch of the kernel family `name` ("tc_ladder",
 *    "tc_fm", "kbuild", "jmat", "zgather", "mu", ...) with CUDA events on the context's stream
 *    until the next call (NULL or "" switches it off); epsp_profile_read returns their summed
 *    milliseconds and count;
 *  - epsp_timer_begin / epsp_timer_end time the context's stream between two calls;
 *  - epsp_ctx_keep_g2 (on = 1) makes the context keep on the device the last g2 a plan set-up
 *    streamed, in that set-up's member order; a later set-up whose model points at the same g2 array
 *    (address, size, element type) in the same order reads it instead of streaming g2 again (an
 *    scGD0 plan and a ladder plan of one model). The caller must not change the array in between;
 *    on = 0 (the default) switches it off and frees the copy;
 *  - epsp_test_fail_alloc makes the next device allocation of at least `bytes` bytes fail with
 *    EPSP_ENOMEM (0 switches it off), to test the error path without exhausting a device;
 *  - epsp_test_gemm_stall makes the one-CTA tensor-core GEMM kernel's producer skip K block
 *    `skip_kblock` of every tile (-1 switches it off) and that kernel's pipeline waits give up after
 *    `wait_limit` tries (0: the default, about 2^26), so that a call returns EPSP_EDEVICE_TIMEOUT
 *    from a bounded device wait (the kernel frees its tensor memory and returns; the context and
 *    the plan stay usable);
 *  - epsp_test_g2_host_gather(ctx, 1) makes the set-ups' g2 stream gather g2 on the host into
 *    page-locked staging and copy it even when g2 is registered page-locked memory (0, the
 *    default, gathers such a g2 on the device). */
epsp_status epsp_profile_kernel(epsp_ctx* ctx, const char* name);
epsp_status epsp_profile_read(epsp_ctx* ctx, double* total_ms, int64_t* count);
epsp_status epsp_timer_begin(epsp_ctx* ctx);
epsp_status epsp_timer_end(epsp_ctx* ctx, double* ms);
epsp_status epsp_ctx_keep_g2(epsp_ctx* ctx, int32_t on);

/* Page-locks the host memory [ptr, ptr + bytes) and maps it for the device (cudaHostRegister);
 * epsp_host_unregister(ctx, ptr) undoes it and must be called before the memory is freed. A plan
 * set-up whose g2 of at most 1 GiB lies in registered (or cudaHostAlloc'd) memory gathers it in
 * star order with a kernel that reads it in place, with no host-side gather or staging copy; a
 * larger g2, or one in pageable memory, is gathered on the host over up to 16 threads into
 * page-locked staging and copied (on a GB300 node the in-place reads of an 8.6 GB g2 ran several
 * times slower than that). Registering pins every page (0.7-2 ms for 365 MB there).
 * EPSP_EINVAL if the range is already (or, for unregister, not) registered. No counterpart in the
 * reference (CUDA.jl's pinning of host arrays plays the same role there). */
epsp_status epsp_host_register(epsp_ctx* ctx, void* ptr, uint64_t bytes);
epsp_status epsp_host_unregister(epsp_ctx* ctx, void* ptr);
epsp_status epsp_test_fail_alloc(epsp_ctx* ctx, uint64_t bytes);
epsp_status epsp_test_gemm_stall(epsp_ctx* ctx, int32_t skip_kblock, uint32_t wait_limit);
epsp_status epsp_test_g2_host_gather(epsp_ctx* ctx, int32_t on);

/* ---- scGD0 ---- */

/* Uploads the iteration-invariant tables of `model` (the `setup` of src/scgd0.jl:127-184 and the
 * buffers of src/scgd0.jl:199-245). Replaces the setup half of _loop_scgd0. */
epsp_status epsp_scgd0_setup(epsp_ctx* ctx, const epsp_model* model, const epsp_options* opts,
                             epsp_scgd0_plan** plan);
void epsp_scgd0_plan_destroy(epsp_scgd0_plan* plan);

/* The scGD0 iteration: the body of _loop_scgd0 (src/scgd0.jl:246-346). sigma_init is NULL for
 * the start -i*eta_init, else [nω, ni, nT] complex. mu_start [nT] is the starting μ (occ.μlist or
 * the bare-band μ). Outputs: sigma_out [nω, ni, nT] complex, mu_out [nT], converged [nT], hist. */
epsp_status epsp_scgd0_run(epsp_scgd0_plan* plan, const epsp_occ* occ, const double* eta_min,
                           double eta_init, int32_t maxiter, double tol, int32_t fix_mu,
                           const double* mu_start, const double* sigma_init, double* sigma_out,
                           double* mu_out, uint8_t* converged, epsp_scgd0_history* hist);

/* The self-energy of the plan's last run, on the device: Σ [nω, ni, nT] complex FP64, column-major
 * like sigma_out (nT of that run, may be NULL), valid until the next run or the plan's destruction
 * (no counterpart in the reference). epsp_scgd0_run takes sigma_out = NULL to leave Σ there only;
 * epsp_ladder_run and epsp_ladder_run_batched accept this pointer as their sigma. EPSP_EINVAL before
 * the first run. */
epsp_status epsp_scgd0_sigma_device(const epsp_scgd0_plan* plan, const double** sigma_dev, int64_t* nT);

/* One Fan-Migdal sum at one temperature: imsigma [nω, ni] += Σ_{νf} term, with sigma_in [nω, ni]
 * complex the clamped input self-energy. add_fan_migdal_imsigma! (src/scgd0_kernel.jl:59-72). */
epsp_status epsp_scgd0_imsigma(epsp_scgd0_plan* plan, const double* sigma_in, double mu, double T,
                               double* imsigma);

/* The Fan-Migdal sum for callers that cannot allocate device memory (this entry point has no
 * counterpart in the reference). A host whose own allocator holds the device budget -- a Julia
 * CUDA.jl pool, the ElectronPhonon backend's buffers -- or code running where a cudaMalloc is not
 * allowed passes every array as a device pointer it already owns, in the layouts of epsp_model
 * (g2 [nm, ni, nf] as FP64 here), sigma_in [nω, ni] complex and imsigma [nω, ni] (accumulated into,
 * as epsp_scgd0_imsigma). The library allocates nothing: the grid nodes and the cell-search table
 * live in a fixed static device array of 4.5 MiB (65536 nodes x 8 bytes + 2^20 table entries x 4
 * bytes; larger grids are rejected with EPSP_EINVAL), which every device that loads the library
 * keeps until the process exits. The first call on a device looks up that array's address (set-up
 * once per device). The kernel runs on the
 * context's own stream, which is not ordered after the caller's streams: the caller's device inputs
 * must be complete before the call (synchronise the stream that wrote them). The call is
 * synchronous: it returns after the kernel has finished, so imsigma is ready on return. Calls share
 * the array; calls that overlap on the GPU (other threads, other contexts on the same device) race
 * on it. Index arrays must hold valid indices, as the reference's @inbounds reads. */
epsp_status epsp_scgd0_imsigma_noalloc(epsp_ctx* ctx, int64_t nm, int64_t ni, int64_t nf, const double* g2,
                                       int64_t nq, const double* omega_ph, int64_t nk_i, int64_t nk_f,
                                       const int32_t* iq_kk, const int32_t* iks_i, const int32_t* iks_f,
                                       const double* eps_f, const double* w_f, const int32_t* f_to_i,
                                       const epsp_grid* omegas, double omega_acoustic, const double* sigma_in,
                                       double mu, double T, double* imsigma);

/* ---- ladder ---- */

/* Uploads the ladder tables: the scGD0 tables plus R, v, the stars of f_to_i, the hat-basis shift
 * tables and the trapezoid weights of ωs (_setup_ladder, src/ladder.jl:112-158, and
 * _ladder_workspace, src/ladder.jl:174-233). */
epsp_status epsp_ladder_setup(epsp_ctx* ctx, const epsp_model* model, const epsp_options* opts,
                              epsp_ladder_plan** plan);
void epsp_ladder_plan_destroy(epsp_ladder_plan* plan);

/* The (T, Ω) loops of _loop_ladder (src/ladder.jl:327-375). sigma [nω, ni, nT] complex in host or
 * device memory (unified addressing; e.g. epsp_scgd0_sigma_device's pointer), mu [nT],
 * Tlist [nT], Omegas [nΩ]. Outputs (unsymmetrized, without spin_degeneracy / volume):
 * sigma_bubble, sigma_ladder [3, 3, nΩ, nT]; converged [nΩ, nT]; niter [nΩ, nT]; hist (may be
 * NULL); J_out [nω, 4, 3, 2, ni, nΩ, nT] complex or NULL (store_vertex = false). */
epsp_status epsp_ladder_run(epsp_ladder_plan* plan, const double* sigma, const double* mu,
                            const double* Tlist, int64_t nT, const double* Omegas, int64_t nOmega,
                            int32_t solver, double rtol, int32_t maxiter, double* sigma_bubble,
                            double* sigma_ladder, uint8_t* converged, int32_t* niter,
                            epsp_ladder_history* hist, double* J_out);

/* The (T, Ω) loops of _loop_ladder with the pairs solved together as right-hand sides of GMRES:
 * up to max_rhs pairs (in the order idx = iΩ + nΩ iT) share every operator application -- their
 * shifted-vertex operands are stacked into one tensor-core GEMM and one Kramers-Kronig GEMM -- and
 * run their Arnoldi steps in lockstep, each stopping on its own test (atol = rtol ‖J0‖). Every pair
 * starts from x0 = 0 (the reference warm-starts each Ω from the previous one, src/ladder.jl:340-353):
 * σ agrees with epsp_ladder_run to the solver tolerance, niter and the residual history may differ.
 * GMRES only; tensor-core plans only (GEMM_BF16, GEMM_TF32; EPSP_EUNSUPPORTED otherwise). Outputs as
 * epsp_ladder_run. */
epsp_status epsp_ladder_run_batched(epsp_ladder_plan* plan, const double* sigma, const double* mu,
                                    const double* Tlist, int64_t nT, const double* Omegas, int64_t nOmega,
                                    double rtol, int32_t maxiter, int32_t max_rhs, double* sigma_bubble,
                                    double* sigma_ladder, uint8_t* converged, int32_t* niter,
                                    epsp_ladder_history* hist, double* J_out);

/* The tile shape the autotuner picked at setup for the ladder's tensor-core contraction (GEMM_BF16
 * and GEMM_TF32 plans; no counterpart in the reference): tile width bn (128 or 256), split count,
 * K block bk (64 or 32 on GEMM_BF16, 32 on GEMM_TF32; may be NULL), and the timed milliseconds per
 * launch of the choice and of the fixed heuristic's shape (0 when not a tensor-core plan). The
 * kernel choice comes from epsp_ladder_gemm_persistent and _pair. */
epsp_status epsp_ladder_gemm_config(const epsp_ladder_plan* plan, int32_t* bn, int32_t* splits, int32_t* bk,
                                    double* ms_chosen, double* ms_heuristic);
/* Overrides the autotuner's choice: GEMM_BF16: tile width bn (128 or 256) with K blocks bk = 64
 * (128-byte swizzle; two or three pipeline stages), or bn 256 with bk = 32 (64-byte swizzle, four
 * stages); GEMM_TF32: bn 128 or 256 with bk = 32 (128-byte swizzle); splits within what the plan's
 * partial buffer holds. The one-CTA kernel is selected: persistent and pair settings are reset
 * (set them after). */
epsp_status epsp_ladder_set_gemm_config(epsp_ladder_plan* plan, int32_t bn, int32_t splits, int32_t bk);
/* Whether the contraction runs as the persistent kernel (one CTA per SM over all tiles, two TMEM
 * accumulators so that a tile's epilogue overlaps the next tile's products; GEMM_BF16: bn 256 with
 * bk 32 only; GEMM_TF32: either bn): read, and set (on = 0 or 1; EPSP_EINVAL for another tile
 * shape). Same results bitwise. */
epsp_status epsp_ladder_gemm_persistent(const epsp_ladder_plan* plan, int32_t* on);
epsp_status epsp_ladder_set_gemm_persistent(epsp_ladder_plan* plan, int32_t on);
/* Whether the contraction runs on CTA pairs (tcgen05 cta_group::2: two CTAs of a cluster compute a
 * 256-row tile, each holding its 128 A rows and half of the B tile; bn 256 with bk 32): read, and
 * set (on = 0 or 1). With the persistent setting also on, the persistent CTA-pair kernel (one
 * cluster per two SMs over all tiles, two TMEM accumulators per CTA). Same results bitwise. */
epsp_status epsp_ladder_gemm_pair(const epsp_ladder_plan* plan, int32_t* on);
epsp_status epsp_ladder_set_gemm_pair(epsp_ladder_plan* plan, int32_t on);

/* One application LJ = L(J) of the ladder kernel at temperature T, chemical potential mu and
 * probe frequency Omega, with sigma_T [nω, ni] complex the self-energy of that temperature:
 * apply_ladder_kernel! (src/ladder.jl:245-296) with the propagators of contour_greens!
 * (src/ladder_kernel.jl:51-57). J, LJ: [nω, 4, 3, 2, ni] complex. */
epsp_status epsp_ladder_apply(epsp_ladder_plan* plan, const double* sigma_T, double mu, double T,
                              double Omega, const double* J, double* LJ);

/* ---- learned warm start (no counterpart in the reference) ----
 *
 * A multilayer perceptron that proposes Σ_init for epsp_scgd0_run (the `Σ_init` keyword of
 * run_scgd0, src/scgd0.jl:66 and 204-212); the iteration's own tol check judges the start, so the
 * converged result does not depend on it. Layers d_0 -> d_1 -> ... -> d_L, fully connected, SiLU
 * between layers, linear output; weights used in BF16 with FP32 accumulation, FP32 master copy
 * and Adam moments on the device. Parameters as one flat FP32 vector: per layer W [d_{l+1}][d_l]
 * row-major, then b [d_{l+1}]. X [n][d_0] and Y [n][d_L] are row-major host arrays. */
epsp_status epsp_warmstart_create(epsp_ctx* ctx, int32_t nlayers, const int32_t* dims, epsp_warmstart** net);
void epsp_warmstart_destroy(epsp_warmstart* net);
int64_t epsp_warmstart_nparams(const epsp_warmstart* net);
/* Device milliseconds of the epochs of the last epsp_warmstart_train (CUDA events around each
 * epoch's graph replay; data uploads and graph capture not included). */
double epsp_warmstart_train_ms(const epsp_warmstart* net);
/* Setting the parameters resets the optimiser state. */
epsp_status epsp_warmstart_set_params(epsp_warmstart* net, const float* params);
epsp_status epsp_warmstart_get_params(epsp_warmstart* net, float* params);
epsp_status epsp_warmstart_predict(epsp_warmstart* net, const float* X, int64_t n, float* Y);
/* Mean squared error over the batch and all outputs, and its gradient (flat, as the parameters). */
epsp_status epsp_warmstart_grad(epsp_warmstart* net, const float* X, const float* Y, int64_t n, double* loss,
                                float* grad);
/* Standardisation for the in-iteration use: network inputs (x - x_mean) / x_std [d_0], outputs
 * y * y_scale + y_mean [d_L]. */
epsp_status epsp_warmstart_set_scaling(epsp_warmstart* net, const float* x_mean, const float* x_std,
                                       const float* y_mean, float y_scale);
/* `epochs` passes of Adam (lr, beta 0.9 / 0.999, eps 1e-8) over minibatches of `batch` rows taken in
 * the order perm [epochs][n] (NULL: identity); loss_history [epochs] (may be NULL) gets each
 * epoch's mean training loss. */
epsp_status epsp_warmstart_train(epsp_warmstart* net, const float* X, const float* Y, int64_t n, int32_t epochs,
                                 int32_t batch, float lr, const int64_t* perm, double* loss_history);

/* epsp_scgd0_run started from the network's Σ_init, with the reference's plain start as fallback.
 * Iteration 1 runs from -i*eta_init (the G0D0 self-energy); the network (widths [2 nω + 4, ...,
 * 2 nω], standardisation set) then maps, per outer state i and temperature, the features
 * [Re Σ(ω_j), Im Σ(ω_j) for all ωs; T, μ, coupling_scale[iT], ε_i - μ] to a correction added to Σ
 * on the device, and the iteration continues from there with the reference's own tol check. If a
 * temperature has not converged after maxiter iterations in all, the plain run from -i*eta_init
 * (epsp_scgd0_run without sigma_init) is made and its outputs returned, with *fallback = 1.
 * *iters_total counts every iteration made. Other arguments and outputs as epsp_scgd0_run. */
epsp_status epsp_scgd0_run_warm(epsp_scgd0_plan* plan, epsp_warmstart* net, const double* coupling_scale,
                                const epsp_occ* occ, const double* eta_min, double eta_init, int32_t maxiter,
                                double tol, int32_t fix_mu, const double* mu_start, double* sigma_out,
                                double* mu_out, uint8_t* converged, epsp_scgd0_history* hist,
                                int32_t* iters_total, int32_t* fallback);

#ifdef __cplusplus
}
#endif

#endif /* EPSPECTRAL_GB300_H */
