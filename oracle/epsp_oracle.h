/*
 * epsp_oracle.h -- CPU FP64 restatement of EPSpectral.jl's scGD0 and ladder hot path.
 *
 * TEST INFRASTRUCTURE. This is the oracle the GPU library is checked against, and the timed CPU
 * baseline of the benchmark. Only the tests, the smoke check and the benchmark's CPU-baseline leg
 * load it; the product library never links or calls it.
 *
 * Every function restates the reference file:line given beside it, in the same order of
 * operations where the reference fixes one (element functions, per-column sums, the bisection over
 * floating-point values), with FP contraction disabled (the reference's Julia does not fuse a*b+c).
 * Parity of the restatement is pinned by the reference's own known-answer tests, ported under
 * tests/ (closed forms, naive loops, the Holstein run record).
 *
 * Layouts and conventions are those of include/epspectral_gb300.h.
 */
#ifndef EPSP_ORACLE_H
#define EPSP_ORACLE_H

#include "../include/epspectral_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Scalars: occ_fermion / occ_boson, src/utils.jl:14-38. */
double epsp_oracle_occ_fermion(double e, double T);
double epsp_oracle_occ_boson(double e, double T);

/* Grid maps, src/frequency_grids.jl. */
void epsp_oracle_grid_nodes(const epsp_grid* g, double* nodes);                       /* :140-141 */
void epsp_oracle_trapezoid_weights(const double* ws, int64_t n, double* W);             /* :53-54 */
void epsp_oracle_kk_matrix(const double* ws, int64_t n, double* K);                     /* :30-44 */
void epsp_oracle_interp_table(const double* ws, int64_t n, const double* xs, int64_t nx,
                              int32_t* j, double* t);                                   /* :65-84 */
/* _interp_linear_grid with cell_search_table (:184-219): column `col` of the complex ys[n, ncol]
 * at the points xs -> out (complex). Returns nonzero (message in msg) if the table is refused. */
int epsp_oracle_interp_grid(const epsp_grid* g, const double* ys, int64_t col, const double* xs,
                            int64_t nx, double* out, char* msg, int32_t msglen);

/* compute_ncarrier_spectral, src/scgd0.jl:361-366. */
double epsp_oracle_ncarrier_spectral(double mu, double T, const double* wa, const double* D,
                                     int64_t n, double W, int32_t count_holes, double nstates_base,
                                     double spin_degeneracy);

/* add_fan_migdal_imsigma! on the model's tables at one temperature, src/scgd0_kernel.jl:59-86,
 * with the chunking of src/scgd0.jl:201-202 (opts->gpu_tile). imsigma [nω, ni] is accumulated
 * into; sigma_in [nω, ni] complex is the clamped input. */
int epsp_oracle_imsigma(const epsp_model* m, const epsp_options* opts, const double* sigma_in,
                        double mu, double T, double* imsigma, char* msg, int32_t msglen);

/* _loop_scgd0, src/scgd0.jl:189-346 (same arguments as epsp_scgd0_run). */
int epsp_oracle_scgd0_run(const epsp_model* m, const epsp_options* opts, const epsp_occ* occ,
                          const double* eta_min, double eta_init, int32_t maxiter, double tol,
                          int32_t fix_mu, const double* mu_start, const double* sigma_init,
                          double* sigma_out, double* mu_out, uint8_t* converged,
                          epsp_scgd0_history* hist, char* msg, int32_t msglen);

/* Ladder pieces, src/ladder_kernel.jl. */
void epsp_oracle_contour_green(double w, double eps, double s_re, double s_im, double mu, double T,
                               int32_t c12, double* out);                               /* :27-40 */
void epsp_oracle_shift_tables(const epsp_grid* g, int64_t nshift, int32_t* klo, double* wlo,
                              double* whi);                                             /* :158-176 */
int64_t epsp_oracle_nshift(const epsp_model* m);                      /* src/ladder.jl:151 */
/* bin_coupling_on_shift_grid! for all inner states in star order as one chunk (:195-236):
 * B [nshift, nf, ni, 2], inner state at chunk position f is fidx[f] (star order). */
void epsp_oracle_bin_coupling(const epsp_model* m, double omega_acoustic, double T, double* B);
/* conductivity_from_vertex (:116-122): sigma [3, 3]. */
void epsp_oracle_conductivity(const double* J, const double* v, const double* w_i,
                              const double* Ww, int64_t nw, int64_t ni, double Omega, double T,
                              double* sigma);

/* apply_ladder_kernel! (src/ladder.jl:245-296) with the propagators of contour_greens! at
 * (T, mu, Omega) from the self-energy sigma_T [nω, ni] (src/ladder.jl:321-334). */
int epsp_oracle_ladder_apply(const epsp_model* m, const epsp_options* opts, const double* sigma_T,
                             double mu, double T, double Omega, const double* J, double* LJ,
                             char* msg, int32_t msglen);

/* _loop_ladder, src/ladder.jl:303-379 (same arguments as epsp_ladder_run). */
int epsp_oracle_ladder_run(const epsp_model* m, const epsp_options* opts, const double* sigma,
                           const double* mu, const double* Tlist, int64_t nT, const double* Omegas,
                           int64_t nOmega, int32_t solver, double rtol, int32_t maxiter,
                           double* sigma_bubble, double* sigma_ladder, uint8_t* converged,
                           int32_t* niter, epsp_ladder_history* hist, double* J_out, char* msg,
                           int32_t msglen);

/* Bounded samples of the two dominant CPU costs, for the benchmark's CPU baseline and the parity
 * tests at full size: the Fan-Migdal sum of the outer states [i0, i1) only (imsigma [nω, ni], those
 * columns accumulated); one ladder application for the output states [i0, i1) only (LJ [nω, 4, 3, 2,
 * i1 - i0], bitwise the full application's slice); the chunks of apply_ladder_kernel!
 * (src/ladder.jl:180-202: count, outer-state ranges [i_lo, i_hi) of the first cap chunks, nshift);
 * and one chunk's operands of C± += X± B̃ (src/ladder.jl:254-290): X± [16 nω, nk] and B̃ [nk, 6 ni],
 * nk = nshift·3·(i_hi - i_lo), so that the product can be timed as a BLAS DGEMM, as the reference's
 * mul! runs it. */
int epsp_oracle_imsigma_sample(const epsp_model* m, const epsp_options* opts, const double* sigma_in, double mu,
                               double T, int64_t i0, int64_t i1, double* imsigma, char* msg, int32_t msglen);
int epsp_oracle_ladder_apply_sample(const epsp_model* m, const epsp_options* opts, const double* sigma_T, double mu,
                                    double T, double Omega, const double* J, int64_t i0, int64_t i1, double* LJ,
                                    char* msg, int32_t msglen);
int epsp_oracle_ladder_chunks(const epsp_model* m, const epsp_options* opts, int64_t* n_chunks, int64_t* i_lo,
                              int64_t* i_hi, int64_t cap, int64_t* nshift, char* msg, int32_t msglen);
int epsp_oracle_ladder_chunk_operands(const epsp_model* m, const epsp_options* opts, double T, const double* J,
                                      int64_t chunk, double* Xp, double* Xm, double* Bt, char* msg, int32_t msglen);

/* Threads used by the OpenMP loops (0 = the OpenMP default). */
void epsp_oracle_set_threads(int32_t n);
int32_t epsp_oracle_get_threads(void);

#ifdef __cplusplus
}
#endif

#endif
