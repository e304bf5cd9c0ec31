// scgd0.cuh -- the scGD0 plan object shared by scgd0.cu and the tensor-core path (scgd0_tc.cu).
#pragma once

#include "common.cuh"

#include <memory>

namespace epsp {

// Per-temperature parameters of one iteration, on the device (indexed by temperature).
struct TParams {
  double T, mu, eta_min, n_target;
  int holes, pad;
};

struct Scgd0Plan {
  Ctx* ctx = nullptr;
  int path = EPSP_PATH_DIRECT_FP64;
  int verbosity = 0;
  double w_ac = 0;
  int64_t gpu_tile = 0;
  long nm = 0, ni = 0, nf = 0, nw = 0, nwa = 0;
  double W = 0, nstates_base = 0;
  GridHost ws, wsa;
  // grid tables
  DBuf<int32_t> d_jtab, d_jsp;
  DBuf<double> d_ws, d_wsa, d_tsp, d_Wa, d_eps_i, d_w_i, d_KK;
  // FP32 copies for the tensor-core path's spectral functions: ωa - ω_j(a), t(a), Wa, w_i
  DBuf<float> d_dspf, d_tspf, d_Waf, d_w_if;
  CellTableDev ct{};
  long nmult = 0;
  DBuf<int32_t> d_mptr, d_midx;
  // every state in one group: the multiplets, then the states in none (CSR, members in order)
  long ngroups = 0;
  DBuf<int32_t> d_gptr, d_gidx;
  // DIRECT_FP64
  int64_t nf_chunk = 1;
  DBuf<double> d_g2t, d_wqt, d_eps_f, d_w_f;
  DBuf<int32_t> d_f_to_i;
  // GEMM paths
  bool star_reduced = false;
  long nc = 0;
  DBuf<double> d_wnu, d_epsc, d_G, d_Fa, d_Fe, d_Kt;
  DBuf<int32_t> d_colc;
  // GEMM_BF16 with dispersive modes: the Fan-Migdal sum term by term in FP32 (fm_disp_f32_kernel):
  // w_f g2 [ν f, i] (FP32), ωph, the pair table and its indices, ε_f, f_to_i, the nodes
  // as float pairs with their neighbouring cells' inverse widths, the bucket table's origin and scale
  bool disp = false;
  long nk_i = 0, ntab = 0;
  float x0f = 0.f, inv_hf = 0.f;
  DBuf<float> d_gwf;
  DBuf<double> d_wph;
  DBuf<int32_t> d_iq, d_iksi, d_iksf, d_fti;
  DBuf<double> d_epsf;
  DBuf<float4> d_wtab;
  // cells of ω ± ω_ν for every (ω, ν): [2][nω·nm] lower node, weight and point (absorption, emission)
  DBuf<int32_t> d_cell_j;
  DBuf<double> d_cell_t, d_cell_x;
  // tensor-core path state (scgd0_tc.cu)
  struct Tc;
  std::unique_ptr<Tc, void (*)(Tc*)> tc{nullptr, [](Tc*) {}};
  // iteration buffers
  DBuf<double2> d_Sin;
  DBuf<double> d_ImS, d_ReS, d_A, d_colsum, d_D;
  // work buffers of scgd0_run, kept across runs (grown when a run needs more temperatures)
  DBuf<double2> w_S, w_Snew, w_Sin;
  int64_t sigma_nT = 0;  // temperatures of the last run's Σ in w_S (0: no run yet)
  DBuf<double> w_A, w_colsum, w_D, w_pack;
  // μ solve tables (E, first-round terms) and the FP32 spectral path's per-node Σ terms and partials
  DBuf<double> w_E, w_R1;
  DBuf<float4> w_Pf;
  DBuf<float> w_Dpart, w_Cpart;
  DBuf<int> w_slots;
  DBuf<TParams> w_tp;
  long w_gen = 0;  // bumped whenever one of them is reallocated
  HostPinned h_pin;  // the per-iteration readback and the slot list
  // the captured iteration of the last run, reused while its key matches
  cudaGraphExec_t graph = nullptr;
  long graph_key[6] = {-1, -1, -1, -1, -1, -1};
  long graph_launches = 0;
  ~Scgd0Plan() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

// Tensor-core pieces of the GEMM_BF16 path, in scgd0_tc.cu.
void tc_setup(Scgd0Plan* P);
// The FP32 term-by-term Fan-Migdal sum's tables for a model with dispersive modes (before tc_setup).
void tc_setup_dispersive(Scgd0Plan* P, const epsp_model* m);
void tc_imsigma(Scgd0Plan* P, const double2* d_Sin, double* d_ImS);
void tc_imsigma_disp(Scgd0Plan* P, const double2* d_Sin, double mu, double T, double* d_ImS);
// The g2 upload of the term-by-term sums: g2 [nm, ni, nf] of any dtype to [nm nf, ni] FP64 (scgd0.cu).
void upload_g2_permuted(Ctx* ctx, const epsp_model* m, DBuf<double>& g2t);
void tc_kk_assemble(Scgd0Plan* P, double2* d_Snew);
// Buffers and tensor maps for up to nT temperatures in one iteration.
void tc_reserve(Scgd0Plan* P, long nT);
// The temperatures tc_reserve's buffers hold now.
long tc_capacity(Scgd0Plan* P);
// One iteration of nA active temperatures at once, up to the spectral functions: slot a reads the
// clamped Σ_in + a nω ni; per-temperature T and μ from tp (device). With d_Sin_b null, the slots'
// clamped Σ are already in the FP32 buffer tc_sigma_f32 returns. The Kramers-Kronig product's
// epilogue writes Σ_new (multiplet-averaged) into S_all + slots_h[a] nω ni (temperature index),
// max |Σ_new - Σ| into d_errbits[temperature] (bit patterns, atomic maximum), the spectral
// functions' per-node terms into d_P + a nω ni, and +inf into d_minA[temperature].
void tc_iterate(Scgd0Plan* P, int nA, const int* d_slots, const int* slots_h, const TParams* d_tp,
                const double2* d_Sin_b, double2* d_S_all, float4* d_P, unsigned long long* d_errbits, double* d_minA);
// The FP32 form of the clamped Σ of every reserved temperature ({Re hi, Re lo, Im, 0}, slot-major).
float4* tc_sigma_f32(Scgd0Plan* P);
// Fails with EPSP_EDEVICE_TIMEOUT if a tensor-core GEMM's bounded wait ran out (synchronises).
void tc_check(Scgd0Plan* P);
// The device flag the tensor-core GEMMs set when a bounded wait runs out.
int* tc_err_ptr(Scgd0Plan* P);

}  // namespace epsp
