// scgd0.cu -- the scGD0 plan: setup (src/scgd0.jl:127-245) and the iteration (src/scgd0.jl:246-346)
// on one GPU.
//
// HBM layout of a plan (column-major, reference index order):
//   Σ, Σ_new       [nω, ni, nT] double2        Σ_in [nω, ni] double2 (clamped, one T at a time)
//   ImΣ, ReΣ       [nω, ni] double             KK [nω, nω] double
//   DIRECT_FP64 :  g2_t, ωq_t [nm·nf, ni] double (the (ν f, i) layout of src/scgd0.jl:275-278)
//   GEMM paths  :  G [nc·nm, ni] coupling summed over each column set (a star, or one inner state)
//                  K_t [nω, nc·nm] the kernel tensor of one iteration and temperature
//   spectral    :  A [nωa, ni] double, D [nωa], column sums [ni]
#include "common.cuh"
#include "fp_pair.cuh"
#include "g2stream.cuh"
#include "gemm_f64.cuh"
#include "scgd0.cuh"
#include "warmstart.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <array>
#include <chrono>
#include <limits>

namespace epsp {

// ---------------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------------

// kramers_kronig_matrix (src/frequency_grids.jl:5-44) on the padded nodes xs[0..n+1].
__device__ __forceinline__ double xlogx_d(double x) { return x == 0 ? 0.0 : x * log(fabs(x)); }

__global__ void kk_build_kernel(const double* __restrict__ xs, int n, double* __restrict__ K) {
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= long(n) * n) return;
  int i = int(idx % n), j = int(idx / n);
  double x = xs[i + 1], x1 = xs[j], x2 = xs[j + 1], x3 = xs[j + 2];
  double v = xlogx_d(x1 - x) / (x2 - x1) - xlogx_d(x2 - x) * (x3 - x1) / (x2 - x1) / (x3 - x2) + xlogx_d(x3 - x) / (x3 - x2);
  K[idx] = v / 3.14159265358979323846;
}

void kk_matrix_to_device(Ctx* ctx, const std::vector<double>& w, DBuf<double>& K) {
  const long n = long(w.size());
  if (n < 2) fail(EPSP_EINVAL, "the Kramers-Kronig matrix needs at least two nodes");
  std::vector<double> xs(size_t(n + 2));
  xs[0] = w[0] - (w[1] - w[0]);
  for (long j = 0; j < n; ++j) xs[size_t(j + 1)] = w[size_t(j)];
  xs[size_t(n + 1)] = w[size_t(n - 1)] + (w[size_t(n - 1)] - w[size_t(n - 2)]);
  auto d_xs = to_device(ctx, xs);
  K.alloc(ctx, size_t(n * n));
  kk_build_kernel<<<div_up(size_t(n * n), 256), 256, 0, ctx->stream>>>(d_xs.p, int(n), K.p);
  EPSP_LAUNCHED(ctx);
  EPSP_CUDA(cudaStreamSynchronize(ctx->stream));
}

// g2 [nm, ni, nf] (any storage type) -> g2_t [nm, nf, ni] double (src/scgd0.jl:275-278), and
// ωq_t[ν, f, i] = ωph[ν, iq_kk[iks_i[i], iks_f[f]]] (gather_pair_table!, src/scgd0.jl:270).

template <class T>
__global__ void permute_g2_kernel(const T* __restrict__ g2, int nm, int ni, long nf, long f0, long nfc,
                                  double* __restrict__ g2t) {
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  long total = long(nm) * nfc * ni;
  if (idx >= total) return;
  int nu = int(idx % nm);
  long f = (idx / nm) % nfc;
  int i = int(idx / (long(nm) * nfc));
  g2t[nu + nm * (f + nf * long(i))] = load_g2(g2, nu + nm * (long(i) + ni * (f0 + f)));
  (void)f0;
}

__global__ void gather_wq_kernel(const double* __restrict__ wph, const int32_t* __restrict__ iq_kk,
                                 const int32_t* __restrict__ iks_i, const int32_t* __restrict__ iks_f, int nm, int ni,
                                 long nf, long nk_i, double* __restrict__ wqt) {
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  long total = long(nm) * nf * ni;
  if (idx >= total) return;
  int nu = int(idx % nm);
  long f = (idx / nm) % nf;
  int i = int(idx / (long(nm) * nf));
  long q = iq_kk[iks_i[i] + nk_i * long(iks_f[f])];
  wqt[idx] = wph[nu + long(nm) * q];
}

// Σ = Σ_new = -i η_init everywhere (the start without Σ_init, src/scgd0.jl:226).
__global__ void fill_start_kernel(double2* __restrict__ S, double2* __restrict__ Snew, long n, double eta_init) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  S[k] = Snew[k] = make_double2(0.0, -eta_init);
}

// Σ_in = Re Σ + i min(Im Σ, -η_min) (src/scgd0.jl:256-260), for the active temperatures: slot a
// (blockIdx.y) reads Σ of temperature slots[a] and writes Sin + a n.
__global__ void clamp_kernel(const double2* __restrict__ S, double2* __restrict__ Sin, long n,
                             const int* __restrict__ slots, const TParams* __restrict__ tp) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int a = blockIdx.y, t = slots[a];
  double2 z = S[long(t) * n + k];
  Sin[long(a) * n + k] = make_double2(z.x, fmin(z.y, -tp[t].eta_min));
}

// The same clamp for the tensor-core path, written straight into its FP32 form {Re Σ as a float
// pair, Im Σ, 0} (slot a at Sf + a n).
__global__ void clamp_f32_kernel(const double2* __restrict__ S, float4* __restrict__ Sf, long n,
                                 const int* __restrict__ slots, const TParams* __restrict__ tp) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int a = blockIdx.y, t = slots[a];
  const double2 z = S[long(t) * n + k];
  const float2 r = split_df(z.x);
  Sf[long(a) * n + k] = make_float4(r.x, r.y, float(fmin(z.y, -tp[t].eta_min)), 0.f);
}

// The reference's Fan-Migdal sum, term by term in FP64: for each (ω, i), the sum over νf of
// _fan_migdal_imsigma_term (src/scgd0_kernel.jl:27-39) in ascending νf, added to ImΣ
// (src/scgd0_kernel.jl:74-86). One thread per (ω, i); the block's νf tile (g2, ωq, n_B(ωq) and the
// per-state ε, w, i_f) is staged in shared memory. n_B is evaluated once per (νf, i), the same
// function on the same argument as the reference's per-term call.
constexpr int kFmTile = 128;

__global__ void __launch_bounds__(kFmTile) fm_direct_kernel(
    const double* __restrict__ ws, int nw, CellTableDev ct, const double2* __restrict__ Sin,
    const double* __restrict__ g2t, const double* __restrict__ wqt, long nvf, const double* __restrict__ eps_f,
    const double* __restrict__ w_f, const int32_t* __restrict__ f_to_i, int nm, long vf0, long vf1, double mu,
    double T, double w_ac, double* __restrict__ imsigma) {
  __shared__ double s_g2[kFmTile], s_wq[kFmTile], s_nq[kFmTile], s_eps[kFmTile], s_wf[kFmTile];
  __shared__ int s_col[kFmTile];
  const int i = blockIdx.y;
  const int iw = blockIdx.x * kFmTile + threadIdx.x;
  const double w = iw < nw ? ws[iw] : 0.0;
  double acc = 0.0;
  for (long t0 = vf0; t0 < vf1; t0 += kFmTile) {
    long vf = t0 + threadIdx.x;
    if (vf < vf1) {
      double wq = wqt[vf + nvf * i];
      long f = vf / nm;
      s_g2[threadIdx.x] = g2t[vf + nvf * i];
      s_wq[threadIdx.x] = wq;
      s_nq[threadIdx.x] = wq < w_ac ? 0.0 : occ_boson_d(wq, T);
      s_eps[threadIdx.x] = eps_f[f];
      s_wf[threadIdx.x] = w_f[f];
      s_col[threadIdx.x] = f_to_i[f];
    }
    __syncthreads();
    int nt = int(min(long(kFmTile), vf1 - t0));
    if (iw < nw) {
      for (int k = 0; k < nt; ++k) {
        double wq = s_wq[k];
        if (wq < w_ac) continue;
        const double2* col = Sin + long(nw) * s_col[k];
        double xa = w + wq, xe = w - wq;
        double2 sa = interp_grid_d(col, ct, xa);
        double2 se = interp_grid_d(col, ct, xe);
        double zar = xa - s_eps[k] - sa.x, zai = -sa.y;
        double zer = xe - s_eps[k] - se.x, zei = -se.y;
        double ga = -zai / (zar * zar + zai * zai);
        double ge = -zei / (zer * zer + zei * zei);
        double nq = s_nq[k];
        acc += s_wf[k] * s_g2[k] * (ga * (nq + occ_fermion_d(xa - mu, T)) + ge * (nq + 1 - occ_fermion_d(xe - mu, T)));
      }
    }
    __syncthreads();
  }
  if (iw < nw) imsigma[iw + long(nw) * i] += acc;
}

// The occupation factors of the recast sum, per (ω, ν): F_abs = n_ν + f(ω + ω_ν - μ) and
// F_emi = n_ν + 1 - f(ω - ω_ν - μ) (the two brackets of src/scgd0_kernel.jl:37-38); 0 for a mode
// below ω_acoustic.
__global__ void occ_table_kernel(const double* __restrict__ ws, int nw, const double* __restrict__ wnu, int nm,
                                 double mu, double T, double w_ac, double* __restrict__ Fa, double* __restrict__ Fe) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nw * nm) return;
  int iw = k % nw, nu = k / nw;
  double q = wnu[nu], w = ws[iw];
  if (q < w_ac) {
    Fa[k] = 0;
    Fe[k] = 0;
    return;
  }
  double nq = occ_boson_d(q, T);
  Fa[k] = nq + occ_fermion_d(w + q - mu, T);
  Fe[k] = nq + 1 - occ_fermion_d(w - q - mu, T);
}

// The kernel tensor of the recast sum (dispersionless modes): K_t[ω, (ν, c)] =
// Im G_c(ω + ω_ν) F_abs[ω, ν] + Im G_c(ω - ω_ν) F_emi[ω, ν], with Im G_c(x) = Im 1/(x - ε_c -
// Σ_in,col(c)(x)), for the column set c (a star of inner states sharing ε and the representative's
// Σ, or one inner state).
__global__ void kbuild_f64_kernel(const double* __restrict__ ws, int nw, CellTableDev ct, const double2* __restrict__ Sin,
                                  const double* __restrict__ wnu, int nm, const double* __restrict__ eps_c,
                                  const int32_t* __restrict__ col_c, long nc, const double* __restrict__ Fa,
                                  const double* __restrict__ Fe, double w_ac, double* __restrict__ Kt) {
  const int iw = blockIdx.x * blockDim.x + threadIdx.x;
  const long kc = blockIdx.y;  // (ν, c) with ν fastest
  if (iw >= nw) return;
  const int nu = int(kc % nm);
  const long c = kc / nm;
  double q = wnu[nu];
  double out = 0.0;
  if (!(q < w_ac)) {
    const double2* col = Sin + long(nw) * col_c[c];
    double w = ws[iw], e = eps_c[c];
    double xa = w + q, xe = w - q;
    double2 sa = interp_grid_d(col, ct, xa);
    double2 se = interp_grid_d(col, ct, xe);
    double zar = xa - e - sa.x, zai = -sa.y;
    double zer = xe - e - se.x, zei = -se.y;
    double ga = -zai / (zar * zar + zai * zai);
    double ge = -zei / (zer * zer + zei * zei);
    out = ga * Fa[iw + long(nw) * nu] + ge * Fe[iw + long(nw) * nu];
  }
  Kt[iw + long(nw) * kc] = out;
}

// G[(ν, c), i] = Σ_{f in c} w_f g2[ν, i, f] over the inner states of column set c in star order,
// for the column sets [c0, c1) of one streamed chunk: g2c [nm, ni, p - p0] holds their members p.
// Rows of modes below ω_acoustic are 0 (they are skipped before g2 is read in the reference).
// Thread (ν, i) of column sets c0 + blockIdx.y, c0 + blockIdx.y + gridDim.y, ...: each set's sum is
// its own, so the sets run side by side.
template <class T>
__global__ void coupling_sum_chunk_kernel(const T* __restrict__ g2c, int nm, int ni, const int32_t* __restrict__ cptr,
                                          long c0, long c1, long p0, const int32_t* __restrict__ members, long nc,
                                          const double* __restrict__ w_f, const double* __restrict__ wnu, double w_ac,
                                          double* __restrict__ G) {
  const long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= long(nm) * ni) return;
  const int nu = int(idx % nm), i = int(idx / nm);
  const bool skip = wnu[nu] < w_ac;
  for (long c = c0 + blockIdx.y; c < c1; c += gridDim.y) {
    double s = 0.0;
    if (!skip)
      for (int p = cptr[c]; p < cptr[c + 1]; ++p) {
        const long f = members[p];
        s += w_f[f] * load_g2(g2c, nu + long(nm) * (i + long(ni) * (p - p0)));
      }
    G[(nu + nm * c) + long(nm) * nc * i] = s;
  }
}

// Σ_new = ReΣ + i ImΣ (src/scgd0.jl:290-291).
__global__ void assemble_kernel(const double* __restrict__ re, const double* __restrict__ im, double2* __restrict__ out,
                                long n) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) out[k] = make_double2(re[k], im[k]);
}

__global__ void assemble_f32_kernel(const float* __restrict__ re, const float* __restrict__ im, double2* __restrict__ out,
                                    long n) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) out[k] = make_double2(double(re[k]), double(im[k]));
}

// Average over degenerate multiplets (src/scgd0.jl:293-301): thread per (ω, multiplet), the sum
// over members in order divided by the count.
__global__ void multiplet_kernel(double2* __restrict__ Sall, int nw, long slab, const int* __restrict__ slots,
                                 const int32_t* __restrict__ mptr, const int32_t* __restrict__ midx, long nmult) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= long(nw) * nmult) return;
  double2* S = Sall + slab * slots[blockIdx.y];
  int iw = int(k % nw);
  long g = k / nw;
  int p0 = mptr[g], p1 = mptr[g + 1];
  double sr = 0, si = 0;
  for (int p = p0; p < p1; ++p) {
    double2 z = S[iw + long(nw) * midx[p]];
    sr += z.x;
    si += z.y;
  }
  double len = double(p1 - p0);
  for (int p = p0; p < p1; ++p) S[iw + long(nw) * midx[p]] = make_double2(sr / len, si / len);
}

// Imaginary part of Julia's inv(z) (Smith's algorithm), as in `inv.(…)` of src/scgd0.jl:305.
__device__ __forceinline__ double imag_inv_d(double c, double d) {
  if (fabs(d) <= fabs(c)) {
    double r = d / c;
    double t = 1.0 / (c + d * r);
    return -r * t;
  }
  double r = c / d;
  double t = 1.0 / (d + c * r);
  return -t;
}

// Spectral functions on ωs_spectral (src/scgd0.jl:303-305): A[a, i] = -Im(1/(ωa - ε_i -
// Σ(ωa)))/π with Σ read by the table (j_sp, t_sp) (apply_interpolation_table!).

// FP64 paths (the tensor-core path has its own FP32 kernels below).
__global__ void spectral_A_kernel(const double2* __restrict__ Sall, int nw, long slab, const int* __restrict__ slots,
                                  const double* __restrict__ wsa, int nwa, const int32_t* __restrict__ jsp,
                                  const double* __restrict__ tsp, const double* __restrict__ eps_i,
                                  double* __restrict__ Aall, int ni) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y;
  if (a >= nwa) return;
  const double2* S = Sall + slab * slots[blockIdx.z];
  double* A = Aall + long(nwa) * ni * blockIdx.z;
  int j = jsp[a];
  double t = tsp[a];
  const double2* col = S + long(nw) * i;
  double2 lo = col[j], hi = col[j + 1];
  double sr = (1 - t) * lo.x + t * hi.x;
  double si = (1 - t) * lo.y + t * hi.y;
  const double c = wsa[a] - eps_i[i] - sr;
  A[a + long(nwa) * i] = -imag_inv_d(c, -si) / 3.14159265358979323846;
}

// Fixed-order block reduction helpers (deterministic for a fixed block size).
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
#pragma unroll
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

// colsum[i] = Σ_a A[a, i] Wa[a] (the ∫A_i of min_spectral_weight, src/scgd0.jl:308).
__global__ void __launch_bounds__(256) spectral_colsum_kernel(const double* __restrict__ Aall, int nwa, int ni,
                                                              const double* __restrict__ Wa, double* __restrict__ colsum_all) {
  __shared__ double sh[256];
  int i = blockIdx.x;
  const double* A = Aall + long(nwa) * ni * blockIdx.y;
  double* colsum = colsum_all + long(ni) * blockIdx.y;
  double s = 0;
  for (int a = threadIdx.x; a < nwa; a += 256) s += A[a + long(nwa) * i] * Wa[a];
  double r = block_sum<256>(s, sh);
  if (threadIdx.x == 0) colsum[i] = r;
}

// D[a] = (Σ_i A[a, i] w_i) Wa[a] (src/scgd0.jl:306-307). A block of 256 threads covers 32 nodes a
// (the lanes) and splits i over its 8 warps (i ≡ warp mod 8, ascending); the 8 partial sums are
// added in warp order, so the result is deterministic.
__global__ void __launch_bounds__(256) spectral_D_kernel(const double* __restrict__ Aall, int nwa, int ni,
                                                         const double* __restrict__ w_i, const double* __restrict__ Wa,
                                                         double* __restrict__ Dall) {
  __shared__ double sh[8][32];
  const double* A = Aall + long(nwa) * ni * blockIdx.y;
  double* D = Dall + long(nwa) * blockIdx.y;
  const int lane = threadIdx.x % 32, g = threadIdx.x / 32;
  const int a = blockIdx.x * 32 + lane;
  double s = 0;
  if (a < nwa)
    for (int i = g; i < ni; i += 8) s += A[a + long(nwa) * i] * w_i[i];
  sh[g][lane] = s;
  __syncthreads();
  if (g == 0 && a < nwa) {
    double t = sh[0][lane];
#pragma unroll
    for (int k = 1; k < 8; ++k) t += sh[k][lane];
    D[a] = t * Wa[a];
  }
}

// The tensor-core path's spectral functions, in FP32 without FP64 arithmetic per (a, i) element.
// With ωa = ω_j + d_a (j = j_sp(a), t = t_sp(a)), the denominator's real part is
//   ωa - ε_i - [(1 - t) ReΣ_j + t ReΣ_{j+1}] = d_a - v_j - t δ_j,
//   v_j = ε_i - ω_j + ReΣ_j,  δ_j = ReΣ_{j+1} - ReΣ_j,
// where v_j and δ_j are formed in FP64 once per grid node (nω ni, not nωa ni) and rounded to FP32.
// Near a pole all three terms are of the size of the grid spacing, so the FP32 difference keeps an
// absolute error ~1e-7 h (~1e-10 eV). (Interpolating Σ in FP32 and subtracting it from ωa - ε_i
// instead leaves ~1e-8 eV, which near a pole puts ~1e-5 into A and, through μ, a floor of ~1e-7 eV
// under the iteration's convergence.)
// spectral_prep: P[i][j] = (v_j, δ_j, ImΣ_j, ImΣ_{j+1}) of slot blockIdx.z. Grid (nω / 256, ni, slots).
__global__ void spectral_prep_f32_kernel(const double2* __restrict__ Sall, int nw, long slab, const int* __restrict__ slots,
                                         const double* __restrict__ ws, const double* __restrict__ eps_i,
                                         float4* __restrict__ Pall, double* __restrict__ minA_all) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0)  // the minimum of spectral_fin starts at +inf
    minA_all[slots[blockIdx.z]] = INFINITY;
  if (j >= nw) return;
  const int i = blockIdx.y;
  const double2* col = Sall + slab * slots[blockIdx.z] + long(nw) * i;
  const double2 lo = col[j];
  const double2 hi = j + 1 < nw ? col[j + 1] : lo;
  Pall[slab * blockIdx.z + long(nw) * i + j] =
      make_float4(float(eps_i[i] - ws[j] + lo.x), float(hi.x - lo.x), float(lo.y), float(hi.y));
}

// A[a, i] = -Im(1/(d_a - v_j - t δ_j + i((1-t) ImΣ_j + t ImΣ_{j+1})))/π, never stored: a block of
// 256 nodes a and one chunk of states i accumulates Σ_i A w_i per node (Dpart[slot][chunk][a]) and
// Σ_a A Wa per state (Cpart[slot][i][a-block], summed over the block's warps in warp order), both in
// FP32 over at most ichunk resp. 256 terms. Grid (nωa / 256, ni / ichunk, slots).
constexpr int kSpecChunk = 32;
__global__ void __launch_bounds__(256) spectral_ad_f32_kernel(const float4* __restrict__ Pall, int nw, long slab,
                                                              const int32_t* __restrict__ jsp, const float* __restrict__ dsp,
                                                              const float* __restrict__ tsp, const float* __restrict__ Waf,
                                                              const float* __restrict__ w_if, int nwa, int ni,
                                                              float* __restrict__ Dpart, float* __restrict__ Cpart) {
  __shared__ float sh[8][kSpecChunk];
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
  const int i0 = blockIdx.y * kSpecChunk, i1 = min(ni, i0 + kSpecChunk);
  const int nab = gridDim.x, nch = gridDim.y;
  const bool ok = a < nwa;
  const int j = ok ? jsp[a] : 0;
  const float d = ok ? dsp[a] : 0.f, t = ok ? tsp[a] : 0.f, wa = ok ? Waf[a] : 0.f;
  const float4* P = Pall + slab * blockIdx.z + j;
  float dsum = 0.f;
  for (int i = i0; i < i1; ++i) {
    float A = 0.f;
    if (ok) {
      const float4 p = P[long(nw) * i];
      const float c = d - p.x - t * p.y;
      const float si = (1.f - t) * p.z + t * p.w;
      // -Im(1/(c - i si))/π = -si/(π (c² + si²)); Smith's form only where the square underflows
      const float den = fmaf(c, c, si * si);
      A = (den > 1e-30f ? __fdividef(-si, den) : -imag_inv_f(c, -si)) * 0.318309886183790671538f;
    }
    dsum += A * w_if[i];
    float cs = A * wa;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cs += __shfl_xor_sync(0xffffffffu, cs, o);
    if (lane == 0) sh[wid][i - i0] = cs;
  }
  if (ok) Dpart[(long(blockIdx.z) * nch + blockIdx.y) * nwa + a] = dsum;
  __syncthreads();
  if (threadIdx.x < i1 - i0) {
    float c = 0.f;
#pragma unroll
    for (int w = 0; w < 8; ++w) c += sh[w][threadIdx.x];
    Cpart[(long(blockIdx.z) * ni + i0 + threadIdx.x) * nab + blockIdx.x] = c;
  }
}

// D[a] = Wa[a] Σ_chunk Dpart (FP64, chunk order) for blocks x < nab; the blocks after them give one
// warp to each state i: ∫A_i = Σ Cpart over the node blocks (FP64: lanes in strides of 32, then a
// shuffle tree), whose minimum over i goes to minA[slots[z]] by an atomic minimum of the bit
// patterns (∫A_i >= 0, so they order as the values; spectral_prep_f32_kernel sets +inf first).
// Grid (nab + ni / 8, slots).
__global__ void __launch_bounds__(256) spectral_fin_f32_kernel(const float* __restrict__ Dpart, const float* __restrict__ Cpart,
                                                               int nch, int nab, const double* __restrict__ Wa, int nwa, int ni,
                                                               const int* __restrict__ slots, double* __restrict__ Dall,
                                                               double* __restrict__ minA_all) {
  const long z = blockIdx.y;
  if (int(blockIdx.x) < nab) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nwa) return;
    double s = 0;
    for (int c = 0; c < nch; ++c) s += double(Dpart[(z * nch + c) * nwa + a]);
    Dall[z * nwa + a] = s * Wa[a];
    return;
  }
  const int i = (int(blockIdx.x) - nab) * 8 + int(threadIdx.x) / 32, lane = threadIdx.x % 32;
  if (i >= ni) return;
  const float* c = Cpart + (z * ni + i) * nab;
  double s = 0;
  for (int b = lane; b < nab; b += 32) s += double(c[b]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) atomicMin(reinterpret_cast<unsigned long long*>(minA_all + slots[z]), (unsigned long long)__double_as_longlong(s));
}

__global__ void __launch_bounds__(256) min_kernel(const double* __restrict__ xall, int n, const int* __restrict__ slots,
                                                  double* __restrict__ out_all) {
  __shared__ double sh[256];
  const double* x = xall + long(n) * blockIdx.x;
  double* out = out_all + slots[blockIdx.x];
  double m = INFINITY;
  for (int k = threadIdx.x; k < n; k += 256) m = fmin(m, x[k]);
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmin(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// Roots.jl's Bisection midpoint over floating-point values (Roots._middle).
__device__ __forceinline__ double float_middle_d(double x, double y) {
  if (!isfinite(x) || !isfinite(y)) return x + y;
  if (x != 0 && y != 0 && (signbit(x) != signbit(y))) return 0.0;
  bool negate = (x < 0) || (y < 0);
  unsigned long long ux = __double_as_longlong(fabs(x)), uy = __double_as_longlong(fabs(y));
  double m = __longlong_as_double((long long)((ux + uy) >> 1));
  return negate ? -m : m;
}

// The μ solve of one temperature (src/scgd0.jl:309-324): the root of n(μ) - n_target on the bracket,
// n(μ) = compute_ncarrier_spectral (src/scgd0.jl:361-366), FP64 throughout. The reference
// bisects to adjacent floats (Roots.find_zero on a bracket, ~64 evaluations); here a safeguarded
// Newton iteration on the same bracket finds the same root (n is increasing in μ, with
// dn/dμ = g Σ_a D_a f(1 - f)/T), falling back to Roots' floating-point midpoint whenever the
// Newton step leaves the bracket, and stops at a step below 2^-46 max(|μ|, 1) (the rounding noise of
// n(μ) moves the root by ~1e-15) or at adjacent floats.
// One cluster of kMuCluster CTAs per temperature: each CTA sums a slice of ωs_spectral in fixed
// order, the partials are combined through distributed shared memory in rank order, so every
// thread of the cluster holds the same totals and takes the same branches.
// The per-node work of the first round runs beforehand across the whole GPU (mu_prep_kernel): the
// terms D_a f(ωa; a), D_a f(ωa; b), D_a f0, D_a f0 (1 - f0) at both bracket ends and at the start x0,
// and E_a = exp((ωa - x0)/T), so that near x0 a later round's occupations cost one product and one
// reciprocal: exp((ωa - μ)/T) = E_a exp((x0 - μ)/T) (used while |μ - x0| <= 30 T; farther out, and at
// T ~ 0, exp is evaluated directly). The cluster then only sums.
// status: 0 ok, 1 no sign change on the bracket.
constexpr int kMuCluster = 8;
constexpr int kMuThreads = 512;
constexpr int kMuWarps = kMuThreads / 32;
constexpr int kMuPrepThreads = 64;
constexpr int kMuTerms = 6;              // first-round terms per node
constexpr double kMuProbe = 8.0;         // the probes x0 -+ 8 T
constexpr double kMuProbeExp = 2980.957987041728;  // e^8

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// 1/x for x >= 1 to within an ulp or two of FP64 division: an FP32 reciprocal refined by two
// Newton-Raphson steps r <- r (2 - x r) (each squares the relative error: 6e-8 -> 4e-15 -> FP64
// rounding), on the FMA units instead of FP64 division; x beyond the FP32 range gives 0 (1/x is
// then below 3e-39).
__device__ __forceinline__ double recip_ge1(double x) {
  const float xf = float(x);
  if (isinf(xf)) return 0.0;
  double r = double(__frcp_rn(xf));
  r = fma(r, fma(-x, r, 1.0), r);
  r = fma(r, fma(-x, r, 1.0), r);
  return r;
}

// Shared by mu_prep_kernel and mu_solve_kernel: the start x0 of slot's temperature on the bracket.
__device__ __forceinline__ double mu_start(double guess, double a, double b) {
  return (guess > a && guess < b) ? guess : float_middle_d(a, b);
}

// Occupation from y = exp((ωa - μ)/T) (electrons: 1/(1 + y); holes: y/(1 + y)).
__device__ __forceinline__ double occ_from_y(double y, int holes) {
  const double r = recip_ge1(1.0 + y);
  if (holes) return isinf(y) ? 1.0 : y * r;
  return r;
}

// Grid (nωa / kMuPrepThreads, slots): E[slot][a] and R1[slot][q][a], q: the first round's terms at
// the bracket ends, f0 and f0 (1 - f0) at x0, and the occupations at x0 -+ kMuProbe T (which narrow
// the bracket before the first Newton step).
__global__ void __launch_bounds__(kMuPrepThreads)
    mu_prep_kernel(const double* __restrict__ Dall, const double* __restrict__ wsa, int nwa, const int* __restrict__ slots,
                   const TParams* __restrict__ tp, double br0, double br1, double* __restrict__ E_all,
                   double* __restrict__ R1_all) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nwa) return;
  const long slot = blockIdx.y;
  const int t = slots[slot];
  const double T = tp[t].T;
  const int holes = tp[t].holes;
  const double x0 = mu_start(tp[t].mu, br0, br1);
  const bool warm = T > 1.4901161193847656e-08;
  auto occ = [&](double wa, double mu) { return occ_fermion_d(holes ? mu - wa : wa - mu, T); };
  const double wa = wsa[k], d = Dall[slot * nwa + k];
  auto from_E = [&](double y) { return holes ? (isinf(y) ? 1.0 : y / (1.0 + y)) : 1.0 / (y + 1.0); };
  double f0, fl, fr, E = 0;
  if (warm) {
    E = exp((wa - x0) / T);
    f0 = from_E(E);
    fl = from_E(E * kMuProbeExp);  // at x0 - kMuProbe T: exp((ωa - x0)/T + kMuProbe)
    fr = from_E(E / kMuProbeExp);
  } else {
    f0 = occ(wa, x0);
    fl = fr = f0;
  }
  E_all[slot * nwa + k] = E;
  double* R1 = R1_all + slot * kMuTerms * nwa;
  R1[k] = d * occ(wa, br0);
  R1[nwa + k] = d * occ(wa, br1);
  R1[2 * nwa + k] = d * f0;
  R1[3 * nwa + k] = d * (f0 * (1 - f0));
  R1[4 * nwa + k] = d * fl;
  R1[5 * nwa + k] = d * fr;
}

__global__ void __cluster_dims__(kMuCluster, 1, 1) __launch_bounds__(kMuThreads)
    mu_solve_kernel(const double* __restrict__ Dall, const double* __restrict__ wsa, int nwa, const int* __restrict__ slots,
                    TParams* __restrict__ tp, double W, double base, double gs, double br0, double br1,
                    const double* __restrict__ E_all, const double* __restrict__ R1_all, double* __restrict__ mu_all,
                    int* __restrict__ status_all, int* __restrict__ evals_all) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = cluster.block_rank();
  // one cluster per active temperature
  const int slot = blockIdx.x / kMuCluster, t = slots[slot];
  const double* D = Dall + long(nwa) * slot;
  const double* E = E_all + long(nwa) * slot;
  const double* R1 = R1_all + long(kMuTerms) * nwa * slot;
  const double T = tp[t].T, n_target = tp[t].n_target, guess = tp[t].mu;
  const int holes = tp[t].holes;
  double* mu_out = mu_all + t;
  int* status = status_all + t;
  __shared__ double sv[kMuTerms][kMuThreads];
  __shared__ double part[2][kMuTerms];
  __shared__ double tot[kMuTerms];
  const int chunk = (nwa + kMuCluster - 1) / kMuCluster;
  const int a0 = int(rank) * chunk, a1 = min(nwa, a0 + chunk);
  const bool warm = T > 1.4901161193847656e-08;
  const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
  // Fixed-order totals of up to kMuTerms per-thread sums over the cluster: warp q adds the CTA's
  // per-thread values of sum q (lanes in strides of 32, then a shuffle tree), so the FP64 adds run in
  // nv warps rather than in all of them; the CTA partials alternate between two buffers, so one
  // cluster barrier per round suffices (a CTA can only overwrite a buffer after the next round's
  // barrier, when every CTA has read it). One thread per total reads the remote partials (not every
  // thread: that serialises on the owners' shared memory).
  int round = 0;
  auto reduce = [&](double* v, int nv) {
    for (int q = 0; q < nv; ++q) sv[q][threadIdx.x] = v[q];
    __syncthreads();
    double* pb = part[round & 1];
    if (wid < nv) {
      double t = 0;
      for (int k = lane; k < kMuThreads; k += 32) t += sv[wid][k];
      t = warp_sum_d(t);
      if (lane == 0) pb[wid] = t;
    }
    cluster.sync();
    if (threadIdx.x < nv) {
      double t = 0;
      for (unsigned r = 0; r < kMuCluster; ++r) t += cluster.map_shared_rank(pb, r)[threadIdx.x];
      tot[threadIdx.x] = t;
    }
    __syncthreads();
    for (int q = 0; q < nv; ++q) v[q] = tot[q];
    ++round;
  };
  auto occ = [&](double wa, double mu) { return occ_fermion_d(holes ? mu - wa : wa - mu, T); };
  auto total = [&](double t1) { return (holes ? (W - t1 + base) * gs : (t1 + base) * gs) - n_target; };
  // The bracket and the Newton step are scalar work: thread 0 of every CTA does it (each holds the
  // same totals, so all CTAs take the same steps) and publishes the next point through shared
  // memory, instead of every thread repeating it on the FP64 units.
  __shared__ double s_x, s_scale;
  __shared__ int s_fact, s_stop;
  double a = br0, b = br1, fa = 0, fb = 0, x = mu_start(guess, br0, br1), result = x;
  const double x0 = x;
  int it = 0;
  bool failed = false;
  auto newton = [&](double F, double dF) -> int {  // 1: done (result set)
    result = x;
    if (F == 0) return 1;
    if (signbit(F) == signbit(fa)) {
      a = x;
      fa = F;
    } else {
      b = x;
      fb = F;
    }
    double xn = x - F / dF;
    // a converged Newton step ends the solve even when it rounds onto the end the bracket update
    // just moved to x (otherwise the safeguard below would bisect down to adjacent floats)
    if (dF > 0 && fabs(xn - x) <= 0x1p-46 * fmax(fabs(x), 1.0)) {
      result = xn;
      return 1;
    }
    if (!(dF > 0) || !(xn > a && xn < b)) xn = float_middle_d(a, b);
    if (xn == a || xn == b) {
      result = fabs(fa) <= fabs(fb) ? a : b;
      return 1;
    }
    x = xn;
    return ++it >= 400 ? 1 : 0;
  };
  auto publish = [&](int stop) {
    const double sx = (x0 - x) / T;
    const bool fact = warm && fabs(sx) <= 30.0;
    s_x = x;
    s_scale = fact ? exp(sx) : 0.0;
    s_fact = fact ? 1 : 0;
    s_stop = stop;
  };
  // round 1: n(a), n(b), n(x0), n'(x0) and n(x0 -+ 8T) from the prepared terms
  {
    double v[kMuTerms] = {0, 0, 0, 0, 0, 0};
    for (int k = a0 + int(threadIdx.x); k < a1; k += kMuThreads)
#pragma unroll
      for (int q = 0; q < kMuTerms; ++q) v[q] += R1[q * nwa + k];
    reduce(v, kMuTerms);
    if (threadIdx.x == 0) {
      fa = total(v[0]);
      fb = total(v[1]);
      int stop = 1;
      if (fa * fb > 0) {
        failed = true;
      } else if (fa == 0) {
        result = a;
      } else if (fb == 0) {
        result = b;
      } else {
        // the probes narrow the bracket to the side (or the 16 T window) that holds the sign change
        const double xl = x0 - kMuProbe * T, xr = x0 + kMuProbe * T;
        const double fl = total(v[4]), fr = total(v[5]);
        const double F0 = total(v[2]), dF0 = warm ? gs * v[3] / T : 0.0;
        if (warm && xl > a && xr < b && fl != 0 && fr != 0 && signbit(fl) == signbit(fr)) {
          // x0 lies outside the narrowed bracket: its Newton step (or the midpoint) starts round 2
          if (signbit(fl) != signbit(fa)) {
            b = xl;
            fb = fl;
          } else {
            a = xr;
            fa = fr;
          }
          double xn = x0 - F0 / dF0;
          if (!(dF0 > 0) || !(xn > a && xn < b)) xn = float_middle_d(a, b);
          x = xn;
          stop = 0;
        } else {
          if (warm && xl > a && xr < b && fl != 0 && fr != 0) {
            a = xl;
            fa = fl;
            b = xr;
            fb = fr;
          }
          stop = newton(F0, dF0);
        }
      }
      publish(stop);
    }
    __syncthreads();
  }
  while (!s_stop) {
    const double xr = s_x, scale = s_scale;
    const bool fact = s_fact != 0;
    double v[2] = {0, 0};
    for (int k = a0 + int(threadIdx.x); k < a1; k += kMuThreads) {
      const double f = fact ? occ_from_y(E[k] * scale, holes) : occ(wsa[k], xr);
      v[0] += D[k] * f;
      v[1] += D[k] * (f * (1 - f));
    }
    reduce(v, 2);
    if (threadIdx.x == 0) publish(newton(total(v[0]), warm ? gs * v[1] / T : 0.0));
    __syncthreads();
  }
  // no CTA leaves while another may still read its partials
  cluster.sync();
  if (rank == 0 && threadIdx.x == 0) {
    evals_all[t] = round;
    if (failed) {
      *status = 1;
    } else {
      *mu_out = result;
      tp[t].mu = result;  // the next iteration's μ, without a round trip to the host
      *status = 0;
    }
  }
}

// err = max |Σ_new - Σ| over one temperature, and Σ ← Σ_new (src/scgd0.jl:326-328). The maximum of
// non-negative doubles is taken on their bit patterns, which order the same way; NaN wins, as in
// Julia's maximum.
// F32 (tensor-core path): the differences in FP64, their magnitude in FP32.
template <bool F32>
__global__ void err_copy_kernel(const double2* __restrict__ Snew_all, double2* __restrict__ S_all, long n,
                                const int* __restrict__ slots, unsigned long long* __restrict__ errbits_all) {
  __shared__ unsigned long long sh[256];
  const int t = slots[blockIdx.y];
  const double2* Snew = Snew_all + long(t) * n;
  double2* S = S_all + long(t) * n;
  unsigned long long* errbits = errbits_all + t;
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  unsigned long long e = 0;
  if (k < n) {
    double2 a = Snew[k], b = S[k];
    double d;
    if constexpr (F32)
      d = double(hypotf(float(a.x - b.x), float(a.y - b.y)));
    else
      d = hypot(a.x - b.x, a.y - b.y);
    e = (unsigned long long)__double_as_longlong(d);
    S[k] = a;
  }
  sh[threadIdx.x] = e;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = max(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(errbits, sh[0]);
}

// ---------------------------------------------------------------------------------------------
// setup
// ---------------------------------------------------------------------------------------------

static void check_model_common(const epsp_model* m) {
  if (!m) fail(EPSP_EINVAL, "model is NULL");
  if (m->nm < 1 || m->ni < 1 || m->nf < 1) fail(EPSP_EINVAL, "nm, ni and nf must be positive");
  if (!m->g2 || !m->omega_ph || !m->iq_kk || !m->iks_i || !m->iks_f || !m->eps_i || !m->w_i || !m->eps_f ||
      !m->w_f || !m->f_to_i)
    fail(EPSP_EINVAL, "a required model array is NULL");
  if (m->g2_dtype != EPSP_F64 && m->g2_dtype != EPSP_F32 && m->g2_dtype != EPSP_BF16)
    fail(EPSP_EINVAL, "g2_dtype must be EPSP_F64, EPSP_F32 or EPSP_BF16");
  if (m->nm > 1024) fail(EPSP_EINVAL, "at most 1024 modes");
  for (int64_t f = 0; f < m->nf; ++f) {
    if (m->f_to_i[f] < 0 || m->f_to_i[f] >= m->ni) fail(EPSP_EINVAL, "f_to_i out of range");
    if (m->iks_f[f] < 0 || m->iks_f[f] >= m->nk_f) fail(EPSP_EINVAL, "iks_f out of range");
  }
  for (int64_t i = 0; i < m->ni; ++i)
    if (m->iks_i[i] < 0 || m->iks_i[i] >= m->nk_i) fail(EPSP_EINVAL, "iks_i out of range");
  for (int64_t k = 0; k < m->nk_i * m->nk_f; ++k)
    if (m->iq_kk[k] < 0 || m->iq_kk[k] >= m->nq) fail(EPSP_EINVAL, "iq_kk out of range");
  if (m->nmult < 0 || (m->nmult > 0 && (!m->mult_ptr || !m->mult_idx))) fail(EPSP_EINVAL, "bad multiplet lists");
  std::vector<char> seen(size_t(m->ni), 0);
  for (int64_t g = 0; g < m->nmult; ++g) {
    if (m->mult_ptr[g + 1] < m->mult_ptr[g]) fail(EPSP_EINVAL, "multiplet pointers must not decrease");
    for (int32_t p = m->mult_ptr[g]; p < m->mult_ptr[g + 1]; ++p) {
      if (m->mult_idx[p] < 0 || m->mult_idx[p] >= m->ni) fail(EPSP_EINVAL, "multiplet member out of range");
      if (seen[size_t(m->mult_idx[p])]++) fail(EPSP_EINVAL, "a state belongs to two multiplets");
    }
  }
}

// Modes are dispersionless when every row of ωph is constant; then ωq[ν, f, i] = ω_ν for every pair.
static bool dispersionless(const epsp_model* m, std::vector<double>& wnu) {
  wnu.assign(size_t(m->nm), 0.0);
  for (int64_t nu = 0; nu < m->nm; ++nu) {
    double w0 = m->omega_ph[nu];
    for (int64_t q = 1; q < m->nq; ++q)
      if (!(m->omega_ph[nu + m->nm * q] == w0)) return false;
    wnu[size_t(nu)] = w0;
  }
  return true;
}

void upload_g2_permuted(Ctx* ctx, const epsp_model* m, DBuf<double>& g2t) {
  const size_t elem = m->g2_dtype == EPSP_F64 ? 8 : (m->g2_dtype == EPSP_F32 ? 4 : 2);
  const long nm = m->nm, ni = m->ni, nf = m->nf;
  g2t.alloc(ctx, size_t(nm * nf * ni));
  // Stage by slabs of inner states so the raw staging buffer stays bounded (~256 MB).
  long per_f = nm * ni;
  long fchunk = std::max<long>(1, long((size_t(256) << 20) / (elem * size_t(per_f))));
  DBuf<uint8_t> stage;
  stage.alloc(ctx, size_t(std::min(fchunk, nf) * per_f) * elem);
  for (long f0 = 0; f0 < nf; f0 += fchunk) {
    long nfc = std::min(fchunk, nf - f0);
    const uint8_t* src = static_cast<const uint8_t*>(m->g2) + size_t(f0 * per_f) * elem;
    EPSP_CUDA(cudaMemcpyAsync(stage.p, src, size_t(nfc * per_f) * elem, cudaMemcpyHostToDevice, ctx->stream));
    long total = nm * nfc * ni;
    unsigned grid = div_up(size_t(total), 256);
    // permute_g2_kernel reads slab-relative inner states and writes at absolute f0 + f.
    double* dst = g2t.p + nm * f0;
    if (m->g2_dtype == EPSP_F64)
      permute_g2_kernel<double><<<grid, 256, 0, ctx->stream>>>(reinterpret_cast<const double*>(stage.p), int(nm), int(ni), nf, 0, nfc, dst);
    else if (m->g2_dtype == EPSP_F32)
      permute_g2_kernel<float><<<grid, 256, 0, ctx->stream>>>(reinterpret_cast<const float*>(stage.p), int(nm), int(ni), nf, 0, nfc, dst);
    else
      permute_g2_kernel<uint16_t><<<grid, 256, 0, ctx->stream>>>(reinterpret_cast<const uint16_t*>(stage.p), int(nm), int(ni), nf, 0, nfc, dst);
    EPSP_LAUNCHED(ctx);
  }
  EPSP_CUDA(cudaStreamSynchronize(ctx->stream));
}

Scgd0Plan* scgd0_setup(Ctx* ctx, const epsp_model* m, const epsp_options* opts) {
  check_model_common(m);
  if (!opts) fail(EPSP_EINVAL, "options are NULL");
  if (opts->gpu_tile < 0) fail(EPSP_EINVAL, "gpu_tile must be nothing or a positive number of inner states");
  auto* P = new Scgd0Plan;
  std::unique_ptr<Scgd0Plan> guard(P);
  P->ctx = ctx;
  P->path = opts->path;
  if (P->path == EPSP_PATH_GEMM_TF32)
    fail(EPSP_EUNSUPPORTED, "GEMM_TF32 is a ladder path; scGD0 plans take DIRECT_FP64, GEMM_FP64 or GEMM_BF16");
  P->w_ac = opts->omega_acoustic;
  P->verbosity = opts->verbosity;
  P->nm = m->nm;
  P->ni = m->ni;
  P->nf = m->nf;
  P->ws = make_grid(m->omegas, "omegas");
  P->wsa = make_grid(m->omegas_spectral, "omegas_spectral");
  P->nw = P->ws.n;
  P->nwa = P->wsa.n;
  P->W = m->W;
  P->nstates_base = m->nstates_base;
  P->gpu_tile = opts->gpu_tile;
  PhaseLog plog(ctx, "scgd0", P->verbosity);
  cudaStream_t s = ctx->stream;
  // grid tables
  CellTableHost ct = make_cell_table(P->ws);
  P->d_jtab = to_device(ctx, ct.jtab);
  P->d_ws = to_device(ctx, P->ws.nodes);
  P->ct = CellTableDev{P->d_jtab.p, P->d_ws.p, ct.x0, ct.inv_h, int(P->nw)};
  P->d_wsa = to_device(ctx, P->wsa.nodes);
  std::vector<int32_t> jsp;
  std::vector<double> tsp;
  interp_table(P->ws.nodes, P->wsa.nodes, jsp, tsp);  // src/scgd0.jl:163
  P->d_jsp = to_device(ctx, jsp);
  P->d_tsp = to_device(ctx, tsp);
  P->d_Wa = to_device(ctx, trapezoid_weights(P->wsa.nodes));
  P->d_eps_i = to_device(ctx, m->eps_i, size_t(m->ni));
  P->d_w_i = to_device(ctx, m->w_i, size_t(m->ni));
  {
    std::vector<float> dspf(jsp.size()), tspf(jsp.size()), Waf(jsp.size()), w_if(static_cast<size_t>(m->ni));
    const std::vector<double> Wa = trapezoid_weights(P->wsa.nodes);
    for (size_t a = 0; a < jsp.size(); ++a) {
      dspf[a] = float(P->wsa.nodes[a] - P->ws.nodes[size_t(jsp[a])]);
      tspf[a] = float(tsp[a]);
      Waf[a] = float(Wa[a]);
    }
    for (size_t i = 0; i < w_if.size(); ++i) w_if[i] = float(m->w_i[i]);
    P->d_dspf = to_device(ctx, dspf);
    P->d_tspf = to_device(ctx, tspf);
    P->d_Waf = to_device(ctx, Waf);
    P->d_w_if = to_device(ctx, w_if);
  }
  if (m->nmult > 0) {
    P->nmult = m->nmult;
    P->d_mptr = to_device(ctx, m->mult_ptr, size_t(m->nmult + 1));
    P->d_midx = to_device(ctx, m->mult_idx, size_t(m->mult_ptr[m->nmult]));
  }
  {  // state groups of the tensor-core epilogue: the multiplets, then every state in none
    std::vector<int32_t> gptr{0}, gidx;
    std::vector<char> in_mult(size_t(m->ni), 0);
    for (int64_t g = 0; g < m->nmult; ++g) {
      for (int64_t p = m->mult_ptr[g]; p < m->mult_ptr[g + 1]; ++p) {
        gidx.push_back(int32_t(m->mult_idx[p]));
        in_mult[size_t(m->mult_idx[p])] = 1;
      }
      gptr.push_back(int32_t(gidx.size()));
    }
    for (int64_t i = 0; i < m->ni; ++i)
      if (!in_mult[size_t(i)]) {
        gidx.push_back(int32_t(i));
        gptr.push_back(int32_t(gidx.size()));
      }
    P->ngroups = long(gptr.size()) - 1;
    if (P->ngroups > 65535) fail(EPSP_EUNSUPPORTED, "at most 65535 state groups (multiplets and single states)");
    P->d_gptr = to_device(ctx, gptr);
    P->d_gidx = to_device(ctx, gidx);
  }
  plog.mark("grid tables");
  kk_matrix_to_device(ctx, P->ws.nodes, P->d_KK);
  const long nm = m->nm, ni = m->ni, nf = m->nf;
  if (P->path == EPSP_PATH_DIRECT_FP64) {
    // nf_chunk of src/scgd0.jl:201-202; the chunks fix the order of the f sum.
    const int64_t chunk_bytes = int64_t(1) << 30;
    P->nf_chunk = opts->gpu_tile <= 0 ? std::clamp<int64_t>(chunk_bytes / (8 * nm * ni), 1, nf) : std::min<int64_t>(opts->gpu_tile, nf);
    upload_g2_permuted(ctx, m, P->d_g2t);
    auto d_wph = to_device(ctx, m->omega_ph, size_t(nm * m->nq));
    auto d_iq = to_device(ctx, m->iq_kk, size_t(m->nk_i * m->nk_f));
    auto d_iksi = to_device(ctx, m->iks_i, size_t(ni));
    auto d_iksf = to_device(ctx, m->iks_f, size_t(nf));
    P->d_wqt.alloc(ctx, size_t(nm * nf * ni));
    gather_wq_kernel<<<div_up(size_t(nm * nf * ni), 256), 256, 0, s>>>(d_wph.p, d_iq.p, d_iksi.p, d_iksf.p, int(nm), int(ni), nf,
                                                                      m->nk_i, P->d_wqt.p);
    EPSP_LAUNCHED(ctx);
    P->d_eps_f = to_device(ctx, m->eps_f, size_t(nf));
    P->d_w_f = to_device(ctx, m->w_f, size_t(nf));
    P->d_f_to_i = to_device(ctx, m->f_to_i, size_t(nf));
    EPSP_CUDA(cudaStreamSynchronize(s));
  } else if (P->path == EPSP_PATH_GEMM_BF16 && [&] {
               std::vector<double> w;
               return !dispersionless(m, w);
             }()) {
    // dispersive modes on the tensor-core path: the Fan-Migdal sum term by term in FP32, the rest of
    // the iteration (Kramers-Kronig product and its epilogue, spectral functions, μ) as below
    tc_setup_dispersive(P, m);
    tc_setup(P);
    EPSP_CUDA(cudaStreamSynchronize(s));
  } else if (P->path == EPSP_PATH_GEMM_FP64 || P->path == EPSP_PATH_GEMM_BF16) {
    std::vector<double> wnu;
    if (!dispersionless(m, wnu))
      fail(EPSP_EUNSUPPORTED, "the GEMM paths need dispersionless modes (every row of omega_ph constant); use EPSP_PATH_DIRECT_FP64");
    // Column sets: the stars of the representatives when every inner state of a star has the same
    // energy (then the f sum of one star is one column); one inner state per column otherwise.
    std::vector<int32_t> order(static_cast<size_t>(nf));
    for (long f = 0; f < nf; ++f) order[size_t(f)] = int32_t(f);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return m->f_to_i[a] < m->f_to_i[b]; });
    std::vector<int32_t> sptr(size_t(ni + 1), 0);
    for (long f = 0; f < nf; ++f) sptr[size_t(m->f_to_i[f] + 1)]++;
    for (long i = 0; i < ni; ++i) sptr[size_t(i + 1)] += sptr[size_t(i)];
    bool uniform = true;
    std::vector<double> eps_star(static_cast<size_t>(ni), 0.0);
    for (long i = 0; i < ni && uniform; ++i) {
      if (sptr[size_t(i + 1)] == sptr[size_t(i)]) continue;
      double e0 = m->eps_f[order[size_t(sptr[size_t(i)])]];
      eps_star[size_t(i)] = e0;
      for (int32_t p = sptr[size_t(i)]; p < sptr[size_t(i + 1)]; ++p)
        if (!(m->eps_f[order[size_t(p)]] == e0)) uniform = false;
    }
    std::vector<int32_t> cptr, members, colc;
    std::vector<double> epsc;
    if (uniform) {
      for (long i = 0; i < ni; ++i)
        if (sptr[size_t(i + 1)] > sptr[size_t(i)]) {
          cptr.push_back(sptr[size_t(i)]);
          colc.push_back(int32_t(i));
          epsc.push_back(eps_star[size_t(i)]);
        }
      cptr.push_back(int32_t(nf));
      members = order;
    } else {
      for (long f = 0; f < nf; ++f) {
        cptr.push_back(int32_t(f));
        members.push_back(int32_t(f));
        colc.push_back(m->f_to_i[f]);
        epsc.push_back(m->eps_f[f]);
      }
      cptr.push_back(int32_t(nf));
    }
    P->star_reduced = uniform;
    P->nc = long(colc.size());
    P->d_wnu = to_device(ctx, wnu);
    P->d_colc = to_device(ctx, colc);
    P->d_epsc = to_device(ctx, epsc);
    auto d_cptr = to_device(ctx, cptr);
    auto d_mem = to_device(ctx, members);
    auto d_wf = to_device(ctx, m->w_f, size_t(nf));
    plog.mark("KK matrix, column sets");
    // The coupling sums need g2 once: it streams through the device in star order, gpu_tile inner
    // states per chunk (or about 64 MiB of g2 per chunk), copies overlapped with the sums; g2
    // stays in the caller's host memory.
    P->d_G.alloc(ctx, size_t(nm * P->nc * ni));
    const size_t member_bytes = size_t(nm * ni) * g2_elem_bytes(m->g2_dtype);
    const long chunk_f = opts->gpu_tile > 0 ? long(opts->gpu_tile) : std::max<long>(1, long((size_t(64) << 20) / member_bytes));
    const unsigned grid = div_up(size_t(nm * ni), 128);
    stream_g2_by_columns(ctx, m, members, cptr, chunk_f, [&](const void* g2c, long c0, long c1, long p0) {
      if (m->g2_dtype == EPSP_F64)
        coupling_sum_chunk_kernel<double><<<dim3(grid, unsigned(std::min<long>(c1 - c0, 65535))), 128, 0, s>>>(static_cast<const double*>(g2c), int(nm), int(ni), d_cptr.p, c0,
                                                              c1, p0, d_mem.p, P->nc, d_wf.p, P->d_wnu.p, P->w_ac, P->d_G.p);
      else if (m->g2_dtype == EPSP_F32)
        coupling_sum_chunk_kernel<float><<<dim3(grid, unsigned(std::min<long>(c1 - c0, 65535))), 128, 0, s>>>(static_cast<const float*>(g2c), int(nm), int(ni), d_cptr.p, c0,
                                                             c1, p0, d_mem.p, P->nc, d_wf.p, P->d_wnu.p, P->w_ac, P->d_G.p);
      else
        coupling_sum_chunk_kernel<uint16_t><<<dim3(grid, unsigned(std::min<long>(c1 - c0, 65535))), 128, 0, s>>>(static_cast<const uint16_t*>(g2c), int(nm), int(ni), d_cptr.p,
                                                                c0, c1, p0, d_mem.p, P->nc, d_wf.p, P->d_wnu.p, P->w_ac,
                                                                P->d_G.p);
      EPSP_LAUNCHED(ctx);
    });
    plog.mark("g2 streamed, coupling sums");
    // The cells of ω ± ω_ν, by the lookup of _interp_linear_grid (src/frequency_grids.jl:207-219):
    // the value there is (1 - t) Σ[j] + t Σ[j + 1], which is Σ[0] below the grid (t = 0) and Σ[end]
    // above it (t = 1).
    {
      const auto& w = P->ws.nodes;
      const long n = P->nw;
      std::vector<int32_t> cj(size_t(2 * n * nm));
      std::vector<double> ctt(cj.size()), cx(cj.size());
      for (long side = 0; side < 2; ++side)
        for (long nu = 0; nu < nm; ++nu)
          for (long iw = 0; iw < n; ++iw) {
            const double x = side == 0 ? w[size_t(iw)] + wnu[size_t(nu)] : w[size_t(iw)] - wnu[size_t(nu)];
            const size_t k = size_t(iw + n * (nu + nm * side));
            cx[k] = x;
            if (!(x > w[0])) {
              cj[k] = 0;
              ctt[k] = 0.0;
            } else if (x >= w[size_t(n - 1)]) {
              cj[k] = int32_t(n - 2);
              ctt[k] = 1.0;
            } else {
              const int32_t c = ct.jtab[size_t(int64_t((x - ct.x0) * ct.inv_h))];
              const int32_t j = c - 1 + (w[size_t(c)] <= x ? 1 : 0);
              cj[k] = j;
              ctt[k] = (x - w[size_t(j)]) / (w[size_t(j + 1)] - w[size_t(j)]);
            }
          }
      P->d_cell_j = to_device(ctx, cj);
      P->d_cell_t = to_device(ctx, ctt);
      P->d_cell_x = to_device(ctx, cx);
    }
    P->d_Fa.alloc(ctx, size_t(P->nw * nm));
    P->d_Fe.alloc(ctx, size_t(P->nw * nm));
    if (P->path == EPSP_PATH_GEMM_FP64) {
      P->d_Kt.alloc(ctx, size_t(P->nw * nm * P->nc));
    } else {
      tc_setup(P);
    }
    EPSP_CUDA(cudaStreamSynchronize(s));
  } else {
    fail(EPSP_EINVAL, "unknown path");
  }
  plog.mark("cells, tensor-core operands");
  // iteration buffers
  P->d_Sin.alloc(ctx, size_t(P->nw * ni));
  P->d_ImS.alloc(ctx, size_t(P->nw * ni));
  P->d_ReS.alloc(ctx, size_t(P->nw * ni));
  P->d_A.alloc(ctx, size_t(P->nwa * ni));
  P->d_colsum.alloc(ctx, size_t(ni));
  P->d_D.alloc(ctx, size_t(P->nwa));
  plog.mark("iteration buffers");
  return guard.release();
}

// ---------------------------------------------------------------------------------------------
// one Fan-Migdal sum at one temperature: ImΣ += Σ (src/scgd0_kernel.jl:59-86)
// ---------------------------------------------------------------------------------------------

void scgd0_imsigma(Scgd0Plan* P, const double2* d_Sin, double mu, double T, double* d_ImS) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  const long nm = P->nm, ni = P->ni, nf = P->nf, nw = P->nw;
  if (P->path == EPSP_PATH_DIRECT_FP64) {
    const long nvf = nm * nf;
    dim3 grid(div_up(size_t(nw), kFmTile), unsigned(ni));
    for (long f0 = 0; f0 < nf; f0 += P->nf_chunk) {
      long f1 = std::min(nf, f0 + P->nf_chunk);
      long pi = prof_begin(ctx, "fan_migdal");
      fm_direct_kernel<<<grid, kFmTile, 0, s>>>(P->d_ws.p, int(nw), P->ct, d_Sin, P->d_g2t.p, P->d_wqt.p, nvf,
                                                P->d_eps_f.p, P->d_w_f.p, P->d_f_to_i.p, int(nm), nm * f0, nm * f1, mu, T,
                                                P->w_ac, d_ImS);
      EPSP_LAUNCHED(ctx);
      prof_end(ctx, pi);
    }
    return;
  }
  if (P->disp) {
    tc_imsigma_disp(P, d_Sin, mu, T, d_ImS);
    return;
  }
  occ_table_kernel<<<div_up(size_t(nw * nm), 256), 256, 0, s>>>(P->d_ws.p, int(nw), P->d_wnu.p, int(nm), mu, T, P->w_ac,
                                                                 P->d_Fa.p, P->d_Fe.p);
  EPSP_LAUNCHED(ctx);
  const long nk = nm * P->nc;
  if (P->path == EPSP_PATH_GEMM_FP64) {
    long pk = prof_begin(ctx, "kbuild");
    kbuild_f64_kernel<<<dim3(div_up(size_t(nw), 128), unsigned(nk)), 128, 0, s>>>(
        P->d_ws.p, int(nw), P->ct, d_Sin, P->d_wnu.p, int(nm), P->d_epsc.p, P->d_colc.p, P->nc, P->d_Fa.p, P->d_Fe.p,
        P->w_ac, P->d_Kt.p);
    EPSP_LAUNCHED(ctx);
    prof_end(ctx, pk);
    long pg = prof_begin(ctx, "fm_gemm");
    // ImΣ[ω, i] += Σ_k K_t[ω, k] G[k, i]
    gemm_f64(ctx, false, int(nw), int(ni), int(nk), 1.0, P->d_Kt.p, nw, P->d_G.p, nk, 1.0, d_ImS, nw);
    prof_end(ctx, pg);
    return;
  }
  tc_imsigma(P, d_Sin, d_ImS);
}

// ---------------------------------------------------------------------------------------------
// the iteration (src/scgd0.jl:246-346)
// ---------------------------------------------------------------------------------------------

// The iteration. With `warm`, the network corrects Σ of every still-active temperature after the
// first iteration (the G0D0 one), with coupling scale warm_scale[iT]; the iterations that follow
// compare against the corrected Σ, as a run started from Σ_init = G0D0 + correction would.
void scgd0_run(Scgd0Plan* P, const epsp_occ* occ, const double* eta_min, double eta_init, int32_t maxiter, double tol,
               int32_t fix_mu, const double* mu_start, const double* sigma_init, double* sigma_out, double* mu_out,
               uint8_t* converged, epsp_scgd0_history* hist, epsp_warmstart* warm = nullptr,
               const double* warm_scale = nullptr) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  if (!occ || !occ->Tlist || (!occ->nlist && !fix_mu)) fail(EPSP_EINVAL, "occ is incomplete");
  if (maxiter < 1) fail(EPSP_EINVAL, "maxiter must be at least 1, got " + std::to_string(maxiter));
  const int64_t nT = occ->nT;
  if (nT < 1) fail(EPSP_EINVAL, "at least one temperature");
  // sigma_out may be NULL: Σ then stays on the device (epsp_scgd0_sigma_device)
  if (!eta_min || !mu_start || !mu_out || !converged || !hist || !hist->err || !hist->mu ||
      !hist->min_spectral_weight || !hist->wall || !hist->iter_frozen)
    fail(EPSP_EINVAL, "an output or input array is NULL");
  for (int64_t iT = 0; iT < nT; ++iT)
    if (!(occ->Tlist[iT] >= 0)) fail(EPSP_EINVAL, "Temperature must be positive");
  const long nw = P->nw, ni = P->ni, nwa = P->nwa;
  const long slab = nw * ni;
  DBuf<double2>& S = P->w_S;
  DBuf<double2>& Snew = P->w_Snew;
  if (ensure(S, ctx, size_t(slab * nT))) ++P->w_gen;
  if (ensure(Snew, ctx, size_t(slab * nT))) ++P->w_gen;
  if (sigma_init) {
    for (long k = 0; k < 2 * slab * nT; ++k)
      if (!std::isfinite(sigma_init[k])) fail(EPSP_EINVAL, "Sigma_init must be finite");
    long pu = prof_begin(ctx, "scgd0_io");
    S.upload(reinterpret_cast<const double2*>(sigma_init), size_t(slab * nT), s);
    prof_end(ctx, pu);
    EPSP_CUDA(cudaMemcpyAsync(Snew.p, S.p, size_t(slab * nT) * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  } else {
    fill_start_kernel<<<div_up(size_t(slab * nT), 256), 256, 0, s>>>(S.p, Snew.p, slab * nT, eta_init);
    EPSP_LAUNCHED(ctx);
  }
  std::vector<double> mu(mu_start, mu_start + nT);
  std::vector<char> active(static_cast<size_t>(nT), 1);
  const double nan = std::numeric_limits<double>::quiet_NaN();
  for (int64_t k = 0; k < nT * maxiter; ++k) hist->err[k] = hist->mu[k] = hist->min_spectral_weight[k] = nan;
  for (int32_t k = 0; k < maxiter; ++k) hist->wall[k] = 0;
  for (int64_t k = 0; k < nT; ++k) hist->iter_frozen[k] = 0;
  const double br0 = P->wsa.nodes.front() - 0.1, br1 = P->wsa.nodes.back() + 0.1;  // src/scgd0.jl:197
  // the per-iteration results in one buffer (one copy back per iteration): err bits [nT], μ [nT],
  // min ∫A [nT], μ status [nT] and evaluations [nT] (ints, in nT doubles), the tensor-core wait flag
  const size_t npack = size_t(4 * nT + 1);
  DBuf<double>& d_pack = P->w_pack;
  if (ensure(d_pack, ctx, npack)) ++P->w_gen;
  d_pack.zero(s);
  auto* d_err = reinterpret_cast<unsigned long long*>(d_pack.p);
  double* d_mu = d_pack.p + nT;
  double* d_minA = d_pack.p + 2 * nT;
  int* d_status = reinterpret_cast<int*>(d_pack.p + 3 * nT);
  int* d_evals = d_status + nT;
  int* d_tcerr = reinterpret_cast<int*>(d_pack.p + 4 * nT);
  // host side of the readback and of the slot list: pinned
  P->h_pin.ensure(npack * sizeof(double) + size_t(nT) * sizeof(int));
  double* h_pack = static_cast<double*>(P->h_pin.p);
  int* h_slots = reinterpret_cast<int*>(h_pack + npack);
  std::vector<int> up_slots;  // the slot list on the device (uploaded when it changes)
  int32_t niter = 0;
  const unsigned eb = div_up(size_t(slab), 256);
  // Every active temperature of an iteration is processed by the same launches (slot a ->
  // temperature slots[a]); per-temperature T, μ, η_min, target and branch live on the device.
  DBuf<int>& d_slots = P->w_slots;
  DBuf<TParams>& d_tp = P->w_tp;
  DBuf<double2>& Sin_b = P->w_Sin;
  DBuf<double>& A_b = P->w_A;
  DBuf<double>& colsum_b = P->w_colsum;
  DBuf<double>& D_b = P->w_D;
  bool grown = false;
  grown |= ensure(d_slots, ctx, size_t(nT));
  grown |= ensure(d_tp, ctx, size_t(nT));
  if (P->path != EPSP_PATH_GEMM_BF16) grown |= ensure(Sin_b, ctx, size_t(slab * nT));  // the tensor-core path clamps into FP32
  const bool f32_spec = P->path == EPSP_PATH_GEMM_BF16;
  const int spec_nab = int(div_up(size_t(nwa), 256)), spec_nch = int(div_up(size_t(ni), size_t(kSpecChunk)));
  if (f32_spec) {
    grown |= ensure(P->w_Pf, ctx, size_t(slab * nT));
    grown |= ensure(P->w_Dpart, ctx, size_t(long(spec_nch) * nwa * nT));
    grown |= ensure(P->w_Cpart, ctx, size_t(long(spec_nab) * ni * nT));
  } else {
    grown |= ensure(A_b, ctx, size_t(nwa * ni * nT));
    grown |= ensure(colsum_b, ctx, size_t(ni * nT));
  }
  grown |= ensure(D_b, ctx, size_t(nwa * nT));
  grown |= ensure(P->w_E, ctx, size_t(nwa * nT));
  grown |= ensure(P->w_R1, ctx, size_t(kMuTerms * nwa * nT));
  if (P->path == EPSP_PATH_GEMM_BF16) {
    const long cap0 = tc_capacity(P);
    tc_reserve(P, nT);
    grown |= tc_capacity(P) != cap0;
  }
  if (grown) ++P->w_gen;
  std::vector<TParams> h_tp(static_cast<size_t>(nT));
  std::vector<int> slots;
  // CUDA graph of the iteration body (tensor-core path; not while one of its kernels is profiled)
  static const char* kBodyProfiles[] = {"kprep", "kbuild", "tc_fm", "tc_kk", "finalize", "spectral", "mu"};
  bool use_graph = P->path == EPSP_PATH_GEMM_BF16;
  for (const char* nm : kBodyProfiles)
    if (ctx->prof_name == nm) use_graph = false;
  // a replayed graph bakes in the buffers, nT, fix_mu, the spin degeneracy and the active count
  auto graph_key = [&](int nA) {
    return std::array<long, 6>{long(nA), long(nT), long(fix_mu), P->w_gen,
                               long(std::llround(occ->spin_degeneracy * 1e6)), long(P->path)};
  };
  for (int32_t iter = 1; iter <= maxiter; ++iter) {
    auto t0 = std::chrono::steady_clock::now();
    slots.clear();
    for (int64_t iT = 0; iT < nT; ++iT) {
      if (!active[size_t(iT)]) continue;
      slots.push_back(int(iT));
      TParams& q = h_tp[size_t(iT)];
      q.T = occ->Tlist[iT];
      q.mu = mu[size_t(iT)];
      q.eta_min = eta_min[iT];
      q.holes = (!fix_mu && occ->type == EPSP_SEMICONDUCTOR && occ->nlist[iT] < 0) ? 1 : 0;
      q.n_target = fix_mu ? 0.0 : occ->nlist[iT] + occ->nelec;
      q.pad = 0;
    }
    const int nA = int(slots.size());
    if (slots != up_slots) {
      std::copy(slots.begin(), slots.end(), h_slots);
      EPSP_CUDA(cudaMemcpyAsync(d_slots.p, h_slots, slots.size() * sizeof(int), cudaMemcpyHostToDevice, s));
      up_slots = slots;
    }
    // T, η_min, target and branch are fixed for the run; μ is written on the device by the μ solve
    if (iter == 1) d_tp.upload(h_tp.data(), h_tp.size(), s);
    // the launches of one iteration; on the tensor-core path they are captured once per active set
    // into a CUDA graph and replayed (μ, T come from the device, so a replay sees the current ones)
    auto body = [&] {
      EPSP_CUDA(cudaMemsetAsync(d_err, 0, size_t(nT) * 8, s));
      EPSP_CUDA(cudaMemsetAsync(d_status, 0, size_t(2 * nT) * sizeof(int), s));
      if (P->path == EPSP_PATH_GEMM_BF16)
        clamp_f32_kernel<<<dim3(eb, unsigned(nA)), 256, 0, s>>>(S.p, tc_sigma_f32(P), slab, d_slots.p, d_tp.p);
      else
        clamp_kernel<<<dim3(eb, unsigned(nA)), 256, 0, s>>>(S.p, Sin_b.p, slab, d_slots.p, d_tp.p);
      EPSP_LAUNCHED(ctx);
      if (P->path == EPSP_PATH_GEMM_BF16) {
        // Σ_new, its multiplet average, max|ΔΣ|, Σ ← Σ_new and the spectral terms from the
        // Kramers-Kronig product's epilogue (so no multiplet, spectral-prep or err/copy pass below)
        tc_iterate(P, nA, d_slots.p, slots.data(), d_tp.p, nullptr, S.p, P->w_Pf.p, d_err, d_minA);
        EPSP_CUDA(cudaMemcpyAsync(d_tcerr, tc_err_ptr(P), sizeof(int), cudaMemcpyDeviceToDevice, s));
      } else {
        for (int a = 0; a < nA; ++a) {
          const int64_t iT = slots[size_t(a)];
          P->d_ImS.zero(s);
          scgd0_imsigma(P, Sin_b.p + slab * a, mu[size_t(iT)], occ->Tlist[iT], P->d_ImS.p);
          long pk = prof_begin(ctx, "kk");
          gemm_f64(ctx, false, int(nw), int(ni), int(nw), 1.0, P->d_KK.p, nw, P->d_ImS.p, nw, 0.0, P->d_ReS.p, nw);
          assemble_kernel<<<eb, 256, 0, s>>>(P->d_ReS.p, P->d_ImS.p, Snew.p + slab * iT, slab);
          EPSP_LAUNCHED(ctx);
          prof_end(ctx, pk);
        }
      }
      if (P->nmult > 0 && !f32_spec) {
        multiplet_kernel<<<dim3(div_up(size_t(nw * P->nmult), 256), unsigned(nA)), 256, 0, s>>>(
            Snew.p, int(nw), slab, d_slots.p, P->d_mptr.p, P->d_midx.p, P->nmult);
        EPSP_LAUNCHED(ctx);
      }
      long psp = prof_begin(ctx, "spectral");
      if (f32_spec) {  // the per-node terms came from the Kramers-Kronig epilogue
        spectral_ad_f32_kernel<<<dim3(unsigned(spec_nab), unsigned(spec_nch), unsigned(nA)), 256, 0, s>>>(
            P->w_Pf.p, int(nw), slab, P->d_jsp.p, P->d_dspf.p, P->d_tspf.p, P->d_Waf.p, P->d_w_if.p, int(nwa), int(ni),
            P->w_Dpart.p, P->w_Cpart.p);
        EPSP_LAUNCHED(ctx);
        spectral_fin_f32_kernel<<<dim3(unsigned(spec_nab + div_up(size_t(ni), 8)), unsigned(nA)), 256, 0, s>>>(
            P->w_Dpart.p, P->w_Cpart.p, spec_nch, spec_nab, P->d_Wa.p, int(nwa), int(ni), d_slots.p, D_b.p, d_minA);
        EPSP_LAUNCHED(ctx);
      } else {
        spectral_A_kernel<<<dim3(div_up(size_t(nwa), 256), unsigned(ni), unsigned(nA)), 256, 0, s>>>(
            Snew.p, int(nw), slab, d_slots.p, P->d_wsa.p, int(nwa), P->d_jsp.p, P->d_tsp.p, P->d_eps_i.p, A_b.p, int(ni));
        EPSP_LAUNCHED(ctx);
        spectral_colsum_kernel<<<dim3(unsigned(ni), unsigned(nA)), 256, 0, s>>>(A_b.p, int(nwa), int(ni), P->d_Wa.p,
                                                                              colsum_b.p);
        EPSP_LAUNCHED(ctx);
        min_kernel<<<unsigned(nA), 256, 0, s>>>(colsum_b.p, int(ni), d_slots.p, d_minA);
        EPSP_LAUNCHED(ctx);
        if (!fix_mu) {
          spectral_D_kernel<<<dim3(div_up(size_t(nwa), 32), unsigned(nA)), 256, 0, s>>>(A_b.p, int(nwa), int(ni),
                                                                                       P->d_w_i.p, P->d_Wa.p, D_b.p);
          EPSP_LAUNCHED(ctx);
        }
      }
      prof_end(ctx, psp);
      if (!fix_mu) {
        long pm = prof_begin(ctx, "mu");
        mu_prep_kernel<<<dim3(div_up(size_t(nwa), kMuPrepThreads), unsigned(nA)), kMuPrepThreads, 0, s>>>(
            D_b.p, P->d_wsa.p, int(nwa), d_slots.p, d_tp.p, br0, br1, P->w_E.p, P->w_R1.p);
        EPSP_LAUNCHED(ctx);
        mu_solve_kernel<<<unsigned(kMuCluster * nA), kMuThreads, 0, s>>>(
            D_b.p, P->d_wsa.p, int(nwa), d_slots.p, d_tp.p, P->W, P->nstates_base, occ->spin_degeneracy, br0, br1,
            P->w_E.p, P->w_R1.p, d_mu, d_status, d_evals);
        EPSP_LAUNCHED(ctx);
        prof_end(ctx, pm);
      }
      if (P->path != EPSP_PATH_GEMM_BF16) {  // (the tensor-core epilogue took err and the copy)
        err_copy_kernel<false><<<dim3(eb, unsigned(nA)), 256, 0, s>>>(Snew.p, S.p, slab, d_slots.p, d_err);
        EPSP_LAUNCHED(ctx);
      }
    };
    // iteration 1 replays a graph a previous run captured with the same key; otherwise it runs
    // eagerly (first launches set kernel attributes) and iteration 2 captures
    const bool have_graph = P->graph && [&] {
      const auto k = graph_key(nA);
      return std::equal(k.begin(), k.end(), P->graph_key);
    }();
    if (use_graph && (iter > 1 || have_graph)) {
      const auto key = graph_key(nA);
      if (!P->graph || !std::equal(key.begin(), key.end(), P->graph_key)) {
        if (P->graph) cudaGraphExecDestroy(P->graph), P->graph = nullptr;
        const int64_t l0 = ctx->launches;
        cudaGraph_t g = nullptr;
        EPSP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        try {
          body();
        } catch (...) {
          cudaStreamEndCapture(s, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        EPSP_CUDA(cudaStreamEndCapture(s, &g));
        cudaError_t ie = cudaGraphInstantiate(&P->graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) P->graph = nullptr;
        EPSP_CUDA(ie);
        P->graph_launches = ctx->launches - l0;
        ctx->launches = l0;
        std::copy(key.begin(), key.end(), P->graph_key);
      }
      EPSP_CUDA(cudaGraphLaunch(P->graph, s));
      ctx->launches += P->graph_launches;
    } else {
      body();
    }
    EPSP_CUDA(cudaMemcpyAsync(h_pack, d_pack.p, npack * sizeof(double), cudaMemcpyDeviceToHost, s));
    EPSP_CUDA(cudaStreamSynchronize(s));
    if (P->path == EPSP_PATH_GEMM_BF16) {
      int tcerr = 0;
      std::memcpy(&tcerr, &h_pack[size_t(4 * nT)], sizeof(int));
      if (tcerr) {
        EPSP_CUDA(cudaMemsetAsync(tc_err_ptr(P), 0, sizeof(int), s));  // the plan's next run starts clean
        fail(EPSP_EDEVICE_TIMEOUT, "a tensor-core GEMM wait ran out (bounded device wait)");
      }
    }
    const auto* h_err = reinterpret_cast<const unsigned long long*>(h_pack);
    const double* h_mu = h_pack + nT;
    const double* h_minA = h_pack + 2 * nT;
    const auto* h_status = reinterpret_cast<const int*>(h_pack + 3 * nT);
    for (int64_t iT = 0; iT < nT; ++iT) {
      if (!active[size_t(iT)]) continue;
      hist->min_spectral_weight[iT + nT * (iter - 1)] = h_minA[size_t(iT)];
      if (!fix_mu) {
        if (h_status[size_t(iT)] != 0) {
          char buf[400];
          std::snprintf(buf, sizeof buf,
                        "no chemical potential in (%g, %g) gives %g electrons per cell at T = %g: the window holds too "
                        "few states on one side of the gap, or the spectral weight it loses outside omegas_spectral "
                        "moves the count past the target. Pass mu_start with fix_mu, or widen the window or omegas.",
                        br0, br1, occ->nlist[iT] + occ->nelec, occ->Tlist[iT]);
          fail(EPSP_ENOROOT_MU, buf);
        }
        mu[size_t(iT)] = h_mu[size_t(iT)];
      }
      double err;
      std::memcpy(&err, &h_err[size_t(iT)], 8);
      hist->err[iT + nT * (iter - 1)] = err;
      hist->mu[iT + nT * (iter - 1)] = mu[size_t(iT)];
      if (err < tol) {
        active[size_t(iT)] = 0;
        hist->iter_frozen[iT] = iter;
      }
      if (P->verbosity >= 2)
        std::fprintf(stderr, "scgd0 iteration %d, T = %.6g: err = %.3e, mu = %.15g, mu evaluations %d\n", int(iter),
                     occ->Tlist[iT], err, mu[size_t(iT)], fix_mu ? 0 : h_status[size_t(nT + iT)]);
    }
    if (warm && iter == 1 && iter < maxiter)
      for (int64_t iT = 0; iT < nT; ++iT)
        if (active[size_t(iT)])
          warmstart_correct(warm, ctx, S.p + slab * iT, nw, ni, P->d_eps_i.p, occ->Tlist[iT], mu[size_t(iT)],
                            warm_scale[iT], P->path == EPSP_PATH_GEMM_BF16 ? tc_err_ptr(P) : nullptr);
    hist->wall[iter - 1] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    niter = iter;
    if (std::none_of(active.begin(), active.end(), [](char a) { return a != 0; })) break;
  }
  hist->niter = niter;
  long pd = prof_begin(ctx, "scgd0_io");
  if (sigma_out) S.download(reinterpret_cast<double2*>(sigma_out), size_t(slab * nT), s);
  P->sigma_nT = nT;
  prof_end(ctx, pd);
  EPSP_CUDA(cudaStreamSynchronize(s));
  for (int64_t iT = 0; iT < nT; ++iT) {
    mu_out[iT] = mu[size_t(iT)];
    converged[iT] = active[size_t(iT)] ? 0 : 1;
  }
}

}  // namespace epsp

using namespace epsp;

template <class F>
static epsp_status guarded(Ctx* c, F&& f) {
  try {
    EPSP_CUDA(cudaSetDevice(c->device));
    f();
    c->last_error.clear();
    return EPSP_OK;
  } catch (const Error& e) {
    c->last_error = e.msg;
    return epsp_status(e.code);
  } catch (const std::bad_alloc&) {
    c->last_error = "host allocation failed";
    return EPSP_ENOMEM;
  } catch (const std::exception& e) {
    c->last_error = e.what();
    return EPSP_EINVAL;
  }
}

extern "C" {

epsp_status epsp_scgd0_setup(epsp_ctx* ctx, const epsp_model* model, const epsp_options* opts, epsp_scgd0_plan** plan) {
  if (!ctx || !plan) return EPSP_EINVAL;
  *plan = nullptr;
  return guarded(&ctx->c, [&] { *plan = reinterpret_cast<epsp_scgd0_plan*>(scgd0_setup(&ctx->c, model, opts)); });
}

void epsp_scgd0_plan_destroy(epsp_scgd0_plan* plan) {
  if (!plan) return;
  auto* P = reinterpret_cast<Scgd0Plan*>(plan);
  cudaSetDevice(P->ctx->device);
  delete P;
}

epsp_status epsp_scgd0_run(epsp_scgd0_plan* plan, const epsp_occ* occ, const double* eta_min, double eta_init,
                           int32_t maxiter, double tol, int32_t fix_mu, const double* mu_start, const double* sigma_init,
                           double* sigma_out, double* mu_out, uint8_t* converged, epsp_scgd0_history* hist) {
  if (!plan) return EPSP_EINVAL;
  auto* P = reinterpret_cast<Scgd0Plan*>(plan);
  return guarded(P->ctx, [&] {
    scgd0_run(P, occ, eta_min, eta_init, maxiter, tol, fix_mu, mu_start, sigma_init, sigma_out, mu_out, converged, hist);
  });
}

epsp_status epsp_scgd0_run_warm(epsp_scgd0_plan* plan, epsp_warmstart* net, const double* coupling_scale,
                                const epsp_occ* occ, const double* eta_min, double eta_init, int32_t maxiter, double tol,
                                int32_t fix_mu, const double* mu_start, double* sigma_out, double* mu_out,
                                uint8_t* converged, epsp_scgd0_history* hist, int32_t* iters_total, int32_t* fallback) {
  if (!plan || !net || !coupling_scale || !iters_total || !fallback) return EPSP_EINVAL;
  auto* P = reinterpret_cast<Scgd0Plan*>(plan);
  return guarded(P->ctx, [&] {
    scgd0_run(P, occ, eta_min, eta_init, maxiter, tol, fix_mu, mu_start, nullptr, sigma_out, mu_out, converged, hist,
              net, coupling_scale);
    *iters_total = hist->niter;
    *fallback = 0;
    bool all = true;
    for (int64_t iT = 0; iT < occ->nT; ++iT) all = all && converged[iT];
    if (!all) {  // the plain start decides
      const int32_t used = hist->niter;
      scgd0_run(P, occ, eta_min, eta_init, maxiter, tol, fix_mu, mu_start, nullptr, sigma_out, mu_out, converged, hist);
      *iters_total = used + hist->niter;
      *fallback = 1;
    }
  });
}

epsp_status epsp_scgd0_sigma_device(const epsp_scgd0_plan* plan, const double** sigma_dev, int64_t* nT) {
  if (!plan || !sigma_dev) return EPSP_EINVAL;
  auto* P = reinterpret_cast<const Scgd0Plan*>(plan);
  if (P->sigma_nT < 1) return EPSP_EINVAL;  // no run yet
  *sigma_dev = reinterpret_cast<const double*>(P->w_S.p);
  if (nT) *nT = P->sigma_nT;
  return EPSP_OK;
}

epsp_status epsp_scgd0_imsigma(epsp_scgd0_plan* plan, const double* sigma_in, double mu, double T, double* imsigma) {
  if (!plan || !sigma_in || !imsigma) return EPSP_EINVAL;
  auto* P = reinterpret_cast<Scgd0Plan*>(plan);
  return guarded(P->ctx, [&] {
    if (!(T >= 0)) fail(EPSP_EINVAL, "Temperature must be positive");
    cudaStream_t s = P->ctx->stream;
    const size_t n = size_t(P->nw * P->ni);
    P->d_Sin.upload(reinterpret_cast<const double2*>(sigma_in), n, s);
    P->d_ImS.upload(imsigma, n, s);
    scgd0_imsigma(P, P->d_Sin.p, mu, T, P->d_ImS.p);
    P->d_ImS.download(imsigma, n, s);
    EPSP_CUDA(cudaStreamSynchronize(s));
  });
}

}  // extern "C"
