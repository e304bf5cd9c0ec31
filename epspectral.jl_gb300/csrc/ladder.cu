// ladder.cu -- the ladder plan: setup (_setup_ladder + _ladder_workspace, src/ladder.jl:112-233),
// one application of the ladder kernel (apply_ladder_kernel!, src/ladder.jl:245-296) and the (T, Ω)
// solves (_loop_ladder, src/ladder.jl:303-379) on one GPU.
//
// Index legend and layouts as in the reference (src/ladder_kernel.jl:1-13), column-major:
//   J, LJ, J0   [nω, 4, 3, 2, ni] double2   (ω, c12, cart, c0, i)
//   Gm, Gp      [nω, 4, ni] double2
// DIRECT_FP64 follows the reference's shift grid:
//   B̃ [nshift·3·ni, 6 ni] per temperature (the star-summed coupling of every chunk, kept for all
//   the solves at that temperature: it depends on T only), X [16 nω, nshift·3·nip] per chunk and
//   sign, C± [16 nω, 6 ni] += X B̃, the four channels with the Kramers-Kronig image, then
//   LJ = -Gm K Gp.
// GEMM_FP64 / GEMM_BF16X3 / GEMM_TF32 (dispersionless modes) regroup the shift sums per mode: a mode of
// frequency ω_ν = (m_ν + r_ν) h contributes (1 - r_ν) S_{m_ν} + r_ν S_{m_ν+1}, the same two shift
// tables and weights the shift grid gives it, so
//   U±, V± [row, (a, i)] = Σ_{ν, b, i'} X±_ν[row, (ν, b, i')] (1 or n_ν) G̃[(ν, b, i'), (a, i)],
//   G̃[(ν, b, i'), (a, i)] = Σ_{f in star(i')} R_f[a, b] w_f g2[ν, i, f]   (T-independent, setup),
// and the channel combinations are folded into the A operand rows: 6 combinations q per
// (c0, re/im) instead of the 16 of (c12, type) x sign, and K = nm·3·ni instead of nshift·3·ni.
// The tensor-core paths keep vertices and Krylov vectors in FP32 and run the contraction on tcgen05
// with BF16 hi/lo operands (three products) or TF32 operands (one product); the autotuner picks the
// kernel (one CTA per tile, persistent, CTA pairs) per plan.
#include "common.cuh"
#include "g2stream.cuh"
#include "gemm_f64.cuh"
#include "tc_gemm.cuh"

#include <algorithm>
#include <chrono>
#include <type_traits>
#include <complex>
#include <cstring>
#include <limits>
#include <memory>

namespace epsp {

using cplx = std::complex<double>;

// ---------------------------------------------------------------------------------------------
// plan
// ---------------------------------------------------------------------------------------------

// The GMRES state on the device, FP64 (Krylov.gmres, restart = false): the rotated Hessenberg R
// (packed columns), the rotations (c, s), the right-hand side z, and the status the host reads.
struct GmresDev {
  double nJ0, beta, atol, rnorm;  // ‖J0‖, ‖r0‖, atol = rtol ‖J0‖, the current residual
  double hbis, inv_hbis;          // H[k + 1, k] and its inverse (0 for a breakdown)
  int solved, breakdown, solved_x0, inner;
};

struct LadderChunk {
  long i0 = 0, i1 = 0;     // outer states [i0, i1)
  long f0 = 0, f1 = 0;     // positions [f0, f1) in star order
  long k_off = 0;          // row offset of the chunk in B̃
};

// zgather_kernel's launch shape: U nodes per thread, nranges node ranges of U threads nodes each,
// NC columns per block, staged rows of wstride float4s (the widest window + 4 zeros); smem bytes.
struct ZgatherShape {
  int U = 2, NC = 4, threads = 0, nranges = 1, wstride = 0;
  size_t smem = 0;
};

struct LadderPlan {
  Ctx* ctx = nullptr;
  int path = EPSP_PATH_DIRECT_FP64;
  double w_ac = 0, h = 0;
  long nm = 0, ni = 0, nf = 0, nw = 0, nshift = 0;
  GridHost ws;
  std::vector<double> Ww_h, v_h, w_i_h, wnu;
  std::vector<int32_t> m_nu;
  std::vector<double> r_nu;
  DBuf<double> d_ws, d_Ww, d_KK, d_eps_i, d_v;
  // DIRECT_FP64
  std::vector<LadderChunk> chunks;
  DBuf<int32_t> d_by_star, d_star_ptr, d_klo;
  DBuf<double> d_wlo, d_whi, d_g2, d_wq, d_wf, d_R, d_B, d_Bt, d_X, d_Cp, d_Cm;
  long Ktot = 0;
  double Bt_T = std::numeric_limits<double>::quiet_NaN();  // temperature B̃ was built for
  // GEMM paths: rows (j, q, c0, ri) with j padded to nwp (a multiple of 32), K = (ν, b, i') with ν
  // padded to nmp (a multiple of 16)
  long nwp = 0, nmp = 0;
  long Kx = 0, Kp2 = 0;
  // tensor-core paths: the contraction Z = Jr Bz (M = 16 nwp rows (ri, c0, p, c12), N = nm 3ni
  // columns (ν, a, i), K = 3ni pairs (b, i') padded to Kzp), then D from Z by zgather_kernel
  long Mz = 0, Nz = 0, Kz = 0, Kzp = 0;
  DBuf<float> d_ztab;            // [nm, 2, nwp][4] the weights of p0, p0 + 1, p0 + 2 (tent weights folded in), p0
                                 // (integer bits): the three nodes a mode's two shift tables read
  DBuf<int32_t> d_zwin;          // [node ranges, nm][2] zgather_kernel's staging windows (float4 chunks)
  ZgatherShape zg;               // zgather_kernel's launch shape
  DBuf<float> d_nnu_f;
  DBuf<__nv_bfloat16> d_KKh, d_KKl, d_Yh, d_Yl;
  DBuf<float> d_part2;
  TcOperand opKK{}, opY{};
  int bn2 = 128, splits2 = 1;
  DBuf<double> d_Gt, d_Af, d_D;   // G̃ [Kx, 3ni]; A (FP64) [24nω, Kx]; D [24nω, 3ni]
  DBuf<int32_t> d_mnu;
  DBuf<double> d_rnu, d_nnu;
  DBuf<__nv_bfloat16> d_Jh, d_Jl, d_Bzh, d_Bzl;  // GEMM_BF16: Jr and Bz as BF16 hi/lo rows of Kzp
  DBuf<float> d_Jt, d_Bzt;                        // GEMM_TF32: the same as TF32-rounded FP32
  DBuf<float> d_Z, d_Dz;  // Z (split-K partials, zsplit_cap of them at most) [Mz, Nz]; D [24 nwp, 3ni]
  int zsplit_cap = 1;
  DBuf<int> d_err;
  TcOperand opA{}, opG{}, opA64{}, opG128{}, opG256{}, opA32{}, opG256_32{};
  int bn = 128, splits = 1, bk = kTcBK;  // the contraction's tile shape, picked by the autotuner at setup
  bool persist = false;                  // ... and whether it runs as the persistent kernel
  int gm = 1;                            // ... in launch order (1) or grouped tile order
  bool pair = false;                     // ... or as the CTA-pair kernel (cta_group::2)
  std::vector<TcTune> tune_all;
  float tune_ms_heuristic = 0.f;
  // exchange (both paths)
  DBuf<double> d_Y, d_KY;
  // per (T, Ω)
  DBuf<double2> d_Gm, d_Gp, d_Sm, d_Sp, d_ST;
  DBuf<int32_t> d_jm, d_jp;
  DBuf<double> d_tm, d_tp;
  std::vector<int32_t> h_jm, h_jp;  // host copies behind the last upload of the tables
  std::vector<double> h_tm, h_tp;
  double tab_Om = std::numeric_limits<double>::quiet_NaN();
  double cur_T = 0, cur_mu = 0, cur_Om = 0;
  // GEMM_BF16: the propagators as FP32 complex
  DBuf<float2> d_Gmf, d_Gpf;
  // work buffers of the solves, kept across runs (vertex vectors: FP64 complex on the FP64 paths,
  // FP32 complex on the tensor-core path)
  DBuf<double2> w_J0, w_J, w_LJ, w_W, w_part, w_H, w_Y;
  std::vector<DBuf<double2>> w_V;
  DBuf<float2> w_J0f, w_Jf, w_LJf, w_Wf;
  std::vector<DBuf<float2>> w_Vf;
  // the device Arnoldi step: the two Gram-Schmidt passes' projections, ‖w‖^2, the rotated
  // Hessenberg (packed), the rotations, z, 1 / H[k + 1, k], the status, the Krylov vectors' pointers
  DBuf<double2> g_h1, g_h2, g_hsq, g_R, g_sn, g_z, g_inv;
  DBuf<double> g_cs;
  DBuf<GmresDev> g_st;
  DBuf<void*> g_vp;
  std::shared_ptr<void> w_batch;  // the LadderBatch of the batched solves, kept across runs
};

// ---------------------------------------------------------------------------------------------
// element kernels
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ long jidx(long nw, long w, int c12, int cart, int c0, long i) {
  return w + nw * (c12 + 4 * (cart + 3 * (c0 + 2 * i)));
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

// Complex arithmetic in R (double for the FP64 path; float for the BF16 path, whose products carry
// ~1e-5 relative error already and where FP64 would make this kernel compute-bound).
template <class R>
struct Cx {
  R x, y;
};
template <class R>
__device__ __forceinline__ Cx<R> cxmul(Cx<R> a, Cx<R> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class R>
__device__ __forceinline__ Cx<R> cxadd(Cx<R> a, Cx<R> b) {
  return {a.x + b.x, a.y + b.y};
}

// Complex element types of the vertex vectors: double2 on the FP64 paths; float2 on the tensor-core
// path, whose vertices carry ~1e-6 relative error from the BF16 split products already (FP32
// storage halves their traffic and keeps their arithmetic off the FP64 units, 1/64 of FP32 here).
template <class V>
struct VecOf;
template <>
struct VecOf<double2> {
  using R = double;
  static __device__ __forceinline__ double2 make(double x, double y) { return make_double2(x, y); }
};
template <>
struct VecOf<float2> {
  using R = float;
  static __device__ __forceinline__ float2 make(float x, float y) { return make_float2(x, y); }
};
template <class R>
using Vec2 = std::conditional_t<std::is_same_v<R, float>, float2, double2>;


// Julia's inv(::ComplexF64) (Smith's algorithm).
__device__ __forceinline__ double2 cinv_d(double c, double d) {
  if (fabs(d) <= fabs(c)) {
    double r = d / c, t = 1.0 / (c + d * r);
    return make_double2(t, -r * t);
  }
  double r = c / d, t = 1.0 / (d + c * r);
  return make_double2(r * t, -t);
}

// One contour component set at x = ωs ∓ Ω/2 (contour_greens!, src/ladder_kernel.jl:27-57): G^R =
// 1/(x - ε - Σ(x)), G^A, G^K = (G^R - G^A)(1 - 2f), combined into the four Keldysh components.
// F32 (tensor-core path): the difference x - ε - Re Σ in FP64, the reciprocal and the occupation
// in FP32 (FP64 division and exp would make the kernel compute-bound on the FP64 units).
// The four Keldysh components at one point in FP32 (the tensor-core path's contour_g).
__device__ __forceinline__ void contour_f32(const double2* __restrict__ col, int j, double t, double x, double eps,
                                            double mu, double T, float2 (&g)[4]) {
  const double2 lo = col[j], hi = col[j + 1];
  const double sr = (1 - t) * lo.x + t * hi.x, si = (1 - t) * lo.y + t * hi.y;
  const float c = float(x - eps - sr), d = float(-si);
  float gr, gi;  // Smith's 1/(c + i d)
  if (fabsf(d) <= fabsf(c)) {
    const float r = d / c, tt = 1.f / (c + d * r);
    gr = tt;
    gi = -r * tt;
  } else {
    const float r = c / d, tt = 1.f / (d + c * r);
    gr = r * tt;
    gi = -tt;
  }
  const float Tf = float(T);
  const float f = Tf > 1.4901161193847656e-08f ? 1.f / (expf(float(x - mu) / Tf) + 1.f)
                                               : (x - mu > 0 ? 0.f : (x - mu < 0 ? 1.f : 0.5f));
  const float fac = 1.f - 2.f * f;
  // GR = (gr, gi), GA = (gr, -gi), GK = (GR - GA) fac = (0, 2 gi fac)
  const float kk = 2.f * gi * fac;
  g[0] = make_float2(gr, 0.5f * kk);                 // (GR + GA + GK) / 2
  g[1] = make_float2(0.f, 0.5f * (2.f * gi + kk));   // (GR - GA + GK) / 2
  g[2] = make_float2(0.f, 0.5f * (-2.f * gi + kk));  // (GA - GR + GK) / 2
  g[3] = make_float2(-gr, 0.5f * kk);                // (GK - GR - GA) / 2
}

template <bool F32>
__device__ __forceinline__ void contour_g(const double2* __restrict__ col, int j, double t, double x, double eps,
                                          double mu, double T, Vec2<std::conditional_t<F32, float, double>>* __restrict__ G,
                                          int w, int nw, int i) {
  if constexpr (F32) {
    float2 g[4];
    contour_f32(col, j, t, x, eps, mu, T, g);
    for (int c = 0; c < 4; ++c) G[w + long(nw) * (c + 4 * i)] = g[c];
  } else {
    const double2 lo = col[j], hi = col[j + 1];
    const double sr = (1 - t) * lo.x + t * hi.x, si = (1 - t) * lo.y + t * hi.y;
    double2 GR = cinv_d(x - eps - sr, -si);
    double2 GA = make_double2(GR.x, -GR.y);
    double fac = 1 - 2 * occ_fermion_d(x - mu, T);
    double2 GK = cscale(csub(GR, GA), fac);
    double2 g[4];
    g[0] = cscale(cadd(cadd(GR, GA), GK), 0.5);
    g[1] = cscale(cadd(csub(GR, GA), GK), 0.5);
    g[2] = cscale(cadd(csub(GA, GR), GK), 0.5);
    g[3] = cscale(csub(csub(GK, GR), GA), 0.5);
    for (int c = 0; c < 4; ++c) G[w + long(nw) * (c + 4 * i)] = g[c];
  }
}

// contour_greens! (src/ladder_kernel.jl:27-57) of the self-energy read at ωs ∓ Ω/2 by the
// interpolation tables (jm, tm), (jp, tp) (src/ladder.jl:321-334).
template <bool F32>
__global__ void propagators_kernel(const double2* __restrict__ ST, const double* __restrict__ ws, int nw,
                                   const int32_t* __restrict__ jm, const double* __restrict__ tm,
                                   const int32_t* __restrict__ jp, const double* __restrict__ tp,
                                   const double* __restrict__ eps_i, double mu, double T, double Om,
                                   Vec2<std::conditional_t<F32, float, double>>* __restrict__ Gm,
                                   Vec2<std::conditional_t<F32, float, double>>* __restrict__ Gp, int ni) {
  int w = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y;
  if (w >= nw) return;
  const double2* col = ST + long(nw) * i;
  contour_g<F32>(col, jm[w], tm[w], ws[w] - Om / 2, eps_i[i], mu, T, Gm, w, nw, i);
  contour_g<F32>(col, jp[w], tp[w], ws[w] + Om / 2, eps_i[i], mu, T, Gp, w, nw, i);
}

// attach_greens_to_bare_vertex! (src/ladder_kernel.jl:70-73, 97-99): J0^{c1c2,c0} = Gm^{c1c0} v Gp^{c0c2}
// (float2: the tensor-core path, products in FP32).
// Grid (nω / 256, 6 ni, 4 slots): blockIdx.y = cart + 3 (c0 + 2 i), c12 = blockIdx.z % 4 (the column
// c12 + 4 blockIdx.y of J0).
// Batched over slots: blockIdx.z = c12 + 4 z writes J0 + z 24 nω ni from Gm, Gp + z 4 nω ni.
template <class V>
__global__ void attach_bare_kernel(const V* __restrict__ Gm_all, const V* __restrict__ Gp_all,
                                   const double* __restrict__ v, int nw, int ni, V* __restrict__ J0_all) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const int c12 = blockIdx.z % 4, rest = blockIdx.y;
  const long z = blockIdx.z / 4;
  const V* Gm = Gm_all + z * 4l * nw * ni;
  const V* Gp = Gp_all + z * 4l * nw * ni;
  const long idx = z * 24l * nw * ni + (long(c12) + 4l * rest) * nw + w;
  const int cart = rest % 3, c0 = (rest / 3) % 2;
  const long i = rest / 6;
  int c1 = c12 % 2, c2 = c12 / 2;
  const V a = Gm[w + long(nw) * (c1 + 2 * c0 + 4 * i)];
  const V b = Gp[w + long(nw) * (c0 + 2 * c2 + 4 * i)];
  if constexpr (std::is_same_v<V, float2>) {
    const float vv = float(v[cart + 3 * i]);
    const Cx<float> av{a.x * vv, a.y * vv}, bb{b.x, b.y};
    const Cx<float> zz = cxmul(av, bb);
    J0_all[idx] = make_float2(zz.x, zz.y);
  } else {
    J0_all[idx] = cmul(cscale(a, v[cart + 3 * i]), b);
  }
}

// Y[b, i] = Σ_ω Wω[ω] (J[ω, 22, b, c0=1, i] + J[ω, 11, b, c0=2, i]), the inner sum of
// conductivity_from_vertex (src/ladder_kernel.jl:116-122); fixed-order block sum.
// Batched over blockIdx.y: slot z reads J + z 24 nω ni and writes Y + z 3 ni.
template <class V>
__global__ void __launch_bounds__(256) cond_sum_kernel(const V* __restrict__ J_all, const double* __restrict__ Ww, int nw,
                                                       int ni, double2* __restrict__ Y_all) {
  __shared__ double sr[256], si[256];
  const long z = blockIdx.y;
  const V* J = J_all + z * 24l * nw * ni;
  double2* Y = Y_all + z * 3l * ni;
  int b = blockIdx.x % 3;
  long i = blockIdx.x / 3;
  double ar = 0, ai = 0;
  for (int w = threadIdx.x; w < nw; w += 256) {
    const V x = J[jidx(nw, w, 3, b, 0, i)], y = J[jidx(nw, w, 0, b, 1, i)];
    ar += Ww[w] * double(x.x + y.x);
    ai += Ww[w] * double(x.y + y.y);
  }
  sr[threadIdx.x] = ar;
  si[threadIdx.x] = ai;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sr[threadIdx.x] += sr[threadIdx.x + s];
      si[threadIdx.x] += si[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) Y[b + 3 * i] = make_double2(sr[0], si[0]);
}

// The start of a tensor-core solve in one pass per outer state i (block i, threads over ω): the
// propagators Gm, Gp (propagators_kernel<true>), the bare vertex J0 = Gm v Gp
// (attach_bare_kernel<float2>), its σ sums Y[b, i] (cond_sum_kernel: the same per-thread order and
// block tree) and the block partial of ‖J0‖² (FP32 per thread and ω, FP64 across).
__global__ void __launch_bounds__(256) prep_vertex_f32_kernel(const double2* __restrict__ ST, const double* __restrict__ ws,
                                                              int nw, const int32_t* __restrict__ jm,
                                                              const double* __restrict__ tm, const int32_t* __restrict__ jp,
                                                              const double* __restrict__ tp, const double* __restrict__ eps_i,
                                                              double mu, double T, double Om, const double* __restrict__ v,
                                                              const double* __restrict__ Ww, int ni, float2* __restrict__ Gm,
                                                              float2* __restrict__ Gp, float2* __restrict__ J0,
                                                              double2* __restrict__ Y, double2* __restrict__ part) {
  __shared__ double sr[256], si[256];
  const int i = blockIdx.x;
  const double2* col = ST + long(nw) * i;
  const double e = eps_i[i];
  const float vc[3] = {float(v[3 * i]), float(v[3 * i + 1]), float(v[3 * i + 2])};
  double yr[3] = {0, 0, 0}, yi[3] = {0, 0, 0}, nrm = 0;
  for (int w = threadIdx.x; w < nw; w += 256) {
    float2 gm[4], gp[4];
    contour_f32(col, jm[w], tm[w], ws[w] - Om / 2, e, mu, T, gm);
    contour_f32(col, jp[w], tp[w], ws[w] + Om / 2, e, mu, T, gp);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      Gm[w + long(nw) * (c + 4 * i)] = gm[c];
      Gp[w + long(nw) * (c + 4 * i)] = gp[c];
    }
    float n2 = 0.f;
    float2 j3[3];  // J0[ω, c12 = 3, b, c0 = 0], which Y adds to J0[ω, c12 = 0, b, c0 = 1]
#pragma unroll
    for (int c0 = 0; c0 < 2; ++c0)
#pragma unroll
      for (int cart = 0; cart < 3; ++cart)
#pragma unroll
        for (int c12 = 0; c12 < 4; ++c12) {
          const int c1 = c12 % 2, c2 = c12 / 2;
          const float2 a = gm[c1 + 2 * c0], b = gp[c0 + 2 * c2];
          const Cx<float> av{a.x * vc[cart], a.y * vc[cart]}, bb{b.x, b.y};
          const Cx<float> z = cxmul(av, bb);
          J0[jidx(nw, w, c12, cart, c0, i)] = make_float2(z.x, z.y);
          n2 += z.x * z.x + z.y * z.y;
          if (c12 == 3 && c0 == 0) j3[cart] = make_float2(z.x, z.y);
          if (c12 == 0 && c0 == 1) {  // as cond_sum_kernel: the two added in FP32, then weighted in FP64
            yr[cart] += Ww[w] * double(j3[cart].x + z.x);
            yi[cart] += Ww[w] * double(j3[cart].y + z.y);
          }
        }
    nrm += double(n2);
  }
  auto block_sum = [&](double a, double b, double& ra, double& rb) {
    sr[threadIdx.x] = a;
    si[threadIdx.x] = b;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
      if (threadIdx.x < st) {
        sr[threadIdx.x] += sr[threadIdx.x + st];
        si[threadIdx.x] += si[threadIdx.x + st];
      }
      __syncthreads();
    }
    ra = sr[0];
    rb = si[0];
    __syncthreads();
  };
  for (int b = 0; b < 3; ++b) {
    double ra, rb;
    block_sum(yr[b], yi[b], ra, rb);
    if (threadIdx.x == 0) Y[b + 3 * i] = make_double2(ra, rb);
  }
  double ra, rb;
  block_sum(nrm, 0.0, ra, rb);
  if (threadIdx.x == 0) part[i] = make_double2(ra, 0.0);
}

// ---- DIRECT_FP64: the reference's shift grid ----

// ωq of every (ν, inner state in star order, outer state) (gather_pair_table!, src/ladder.jl:259).
__global__ void gather_wq_star_kernel(const double* __restrict__ wph, const int32_t* __restrict__ iq_kk,
                                      const int32_t* __restrict__ iks_i, const int32_t* __restrict__ iks_f,
                                      const int32_t* __restrict__ by_star, int nm, long nf, int ni, long nk_i,
                                      double* __restrict__ wq) {
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= long(nm) * nf * ni) return;
  int nu = int(idx % nm);
  long fc = (idx / nm) % nf;
  int i = int(idx / (long(nm) * nf));
  long q = iq_kk[iks_i[i] + nk_i * long(iks_f[by_star[fc]])];
  wq[idx] = wph[nu + long(nm) * q];
}

// bin_coupling_on_shift_grid! (src/ladder_kernel.jl:195-236) for the inner states [f0, f1) in star
// order: B[m, fc, i, type] with each mode added to its two shifts in ascending ν, then times w_f.
// One thread per (fc, i, type) column, which it owns.
__global__ void bin_coupling_kernel(const double* __restrict__ g2, const double* __restrict__ wq, const int32_t* __restrict__ by_star,
                                    const double* __restrict__ w_f, int nm, int ni, long nf, long f0, long nfc, int ns, double h,
                                    double w_ac, double T, double* __restrict__ B) {
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= nfc * ni * 2) return;
  long fc = idx % nfc;
  int i = int((idx / nfc) % ni), type = int(idx / (nfc * ni));
  double* col = B + long(ns) * idx;
  for (int m = 0; m < ns; ++m) col[m] = 0.0;
  long f = by_star[f0 + fc];
  for (int nu = 0; nu < nm; ++nu) {
    double w = wq[nu + long(nm) * ((f0 + fc) + nf * i)];
    if (w < w_ac) continue;
    double x = w / h;
    long lo = long(floor(x));
    double g = g2[nu + long(nm) * (i + long(ni) * f)];
    for (long m = lo; m <= lo + 1; ++m) {
      double c = g * fmax(0.0, 1 - fabs(x - double(m)));
      if (m >= 0 && m < ns) col[m] += type == 0 ? c : c * occ_boson_d(w, T);
    }
  }
  double wf = w_f[f];
  for (int m = 0; m < ns; ++m) col[m] *= wf;
}

// star_sum_coupling! (src/ladder_kernel.jl:240-264) into the rows [k_off, k_off + ns·3·nip) of B̃:
// B̃[(m, b, ip), (a, i, type)] = Σ_{fc in star(ip)} R[a, b, f] B[m, fc, i, type].
__global__ void star_sum_kernel(const double* __restrict__ B, const double* __restrict__ R, const int32_t* __restrict__ by_star,
                                const int32_t* __restrict__ star_ptr, long i0, long nip, long f0, long nfc, int ns, int ni,
                                long Ktot, long k_off, double* __restrict__ Bt) {
  long kc = long(ns) * 3 * nip;
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= kc * 6 * ni) return;
  long k = idx % kc, col = idx / kc;
  int m = int(k % ns), b = int((k / ns) % 3);
  long ip = k / (3 * ns);
  int a = int(col % 3), i = int((col / 3) % ni), type = int(col / (3 * ni));
  long p0 = star_ptr[i0 + ip] - f0, p1 = star_ptr[i0 + ip + 1] - f0;
  double acc = 0.0;
  for (long fc = p0; fc < p1; ++fc) {
    long f = by_star[f0 + fc];
    acc += R[a + 3 * (b + 3 * f)] * B[m + long(ns) * (fc + nfc * (i + long(ni) * type))];
  }
  Bt[(k_off + k) + Ktot * col] = acc;
}

// gather_shifted_vertex! (src/ladder_kernel.jl:268-288) for one sign:
// X[(j, c12, c0, ri), (m, b, ip)] = re/im of wlo J[klo] + whi J[klo + 1] of outer state i0 + ip.
__global__ void shifted_vertex_kernel(const double2* __restrict__ J, const int32_t* __restrict__ klo,
                                      const double* __restrict__ wlo, const double* __restrict__ whi, int nw, int ns,
                                      long i0, long nip, double* __restrict__ X) {
  const long nrow = 16l * nw;
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= nrow * ns * 3 * nip) return;
  long row = idx % nrow, k = idx / nrow;
  int j = int(row % nw);
  int c12 = int((row / nw) % 4), c0 = int((row / (4l * nw)) % 2), ri = int(row / (8l * nw));
  int m = int(k % ns), b = int((k / ns) % 3);
  long i = i0 + k / (3 * ns);
  int kl = klo[j + long(nw) * m];
  double wl = wlo[j + long(nw) * m], wh = whi[j + long(nw) * m];
  double2 z0 = J[jidx(nw, kl, c12, b, c0, i)], z1 = J[jidx(nw, kl + 1, c12, b, c0, i)];
  X[idx] = ri == 0 ? wl * z0.x + wh * z1.x : wl * z0.y + wh * z1.y;
}

// Y = (C+ - C-)/2 of type 1 (src/ladder_kernel.jl:319): [nω, (c12, c0, ri, a, i)].
__global__ void y_direct_kernel(const double* __restrict__ Cp, const double* __restrict__ Cm, long n, double* __restrict__ Y) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) Y[k] = (Cp[k] - Cm[k]) / 2;
}

// The four channels (src/ladder_kernel.jl:296-307) from C± [nω, 4, 2, 2, 3, ni, 2] and KY, then
// LJ = -(Gm K Gp) as 2x2 contour matrices (src/ladder.jl:294-295). One thread per (ω, a, c0, i).
__global__ void finish_direct_kernel(const double* __restrict__ Cp, const double* __restrict__ Cm, const double* __restrict__ KY,
                                     const double2* __restrict__ Gm, const double2* __restrict__ Gp, int nw, int ni,
                                     double2* __restrict__ LJ) {
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= long(nw) * 6 * ni) return;
  long w = idx % nw;
  long r = idx / nw;
  int a = int(r % 3), c0 = int((r / 3) % 2);
  long i = r / 6;
  auto cidx = [&](int c12, int ri, int type) {
    return w + nw * (c12 + 4 * (c0 + 2 * (ri + 2 * (a + 3 * (i + long(ni) * type)))));
  };
  double2 K[4];
  for (int c12 = 0; c12 < 4; ++c12) {
    double2 Up = make_double2(Cp[cidx(c12, 0, 0)], Cp[cidx(c12, 1, 0)]);
    double2 Um = make_double2(Cm[cidx(c12, 0, 0)], Cm[cidx(c12, 1, 0)]);
    double2 Vp = make_double2(Cp[cidx(c12, 0, 1)], Cp[cidx(c12, 1, 1)]);
    double2 Vm = make_double2(Cm[cidx(c12, 0, 1)], Cm[cidx(c12, 1, 1)]);
    if (c12 == 0 || c12 == 3) {
      double2 ky = make_double2(KY[cidx(c12, 0, 0)], KY[cidx(c12, 1, 0)]);
      double2 iky = c12 == 0 ? make_double2(ky.y, -ky.x) : make_double2(-ky.y, ky.x);
      K[c12] = csub(csub(iky, cscale(cadd(Up, Um), 0.5)), cadd(Vp, Vm));
    } else if (c12 == 1) {
      K[c12] = cadd(cadd(Vp, Um), Vm);
    } else {
      K[c12] = cadd(cadd(Up, Vp), Vm);
    }
  }
  for (int c1 = 0; c1 < 2; ++c1)
    for (int c2 = 0; c2 < 2; ++c2) {
      auto gm = [&](int c) { return Gm[w + long(nw) * (c + 4 * i)]; };
      auto gp = [&](int c) { return Gp[w + long(nw) * (c + 4 * i)]; };
      double2 z = cmul(cmul(gm(c1), K[0]), gp(0 + 2 * c2));
      z = cadd(z, cmul(cmul(gm(c1 + 2), K[1]), gp(0 + 2 * c2)));
      z = cadd(z, cmul(cmul(gm(c1), K[2]), gp(1 + 2 * c2)));
      z = cadd(z, cmul(cmul(gm(c1 + 2), K[3]), gp(1 + 2 * c2)));
      LJ[jidx(nw, w, c1 + 2 * c2, a, c0, i)] = make_double2(-z.x, -z.y);
    }
}

// ---- GEMM paths: per-mode regrouped shift sums ----

// G̃[(ν, b, i'), (a, i)] = Σ_{f in star(i')} R_f[a, b] w_f g2[ν, i, f] (star sums of the regrouped
// paths; modes below ω_acoustic are 0), for the stars [c0, c1) of one streamed chunk: g2c
// [nm, ni, p - p0] holds their members p in star order.
template <class T>
__global__ void coupling_rot_chunk_kernel(const T* __restrict__ g2c, const double* __restrict__ R,
                                          const double* __restrict__ w_f, const int32_t* __restrict__ by_star,
                                          const int32_t* __restrict__ star_ptr, long c0, long c1, long p0,
                                          const double* __restrict__ wnu, double w_ac, int nm, int nmp, int ni, long Kx,
                                          double* __restrict__ Gt) {
  // thread (ν, i) of stars ip = c0 + blockIdx.y, + gridDim.y, ...: each star's members in order (a
  // star's nine outputs are its own, so the stars run side by side; R of a member is the same for
  // the block)
  const long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= long(nm) * ni) return;
  const int nu = int(idx % nm), i = int(idx / nm);
  const bool skip = wnu[nu] < w_ac;
  for (long ip = c0 + blockIdx.y; ip < c1; ip += gridDim.y) {
    double acc[3][3] = {};
    if (!skip)
      for (int p = star_ptr[ip]; p < star_ptr[ip + 1]; ++p) {
        const long f = by_star[p];
        const double g = w_f[f] * load_g2(g2c, nu + long(nm) * (i + long(ni) * (p - p0)));
        for (int b = 0; b < 3; ++b)
          for (int a = 0; a < 3; ++a) acc[a][b] += R[a + 3 * (b + 3 * f)] * g;
      }
    for (int b = 0; b < 3; ++b)
      for (int a = 0; a < 3; ++a) Gt[(nu + long(nmp) * (b + 3l * ip)) + Kx * (a + 3l * i)] = acc[a][b];
  }
}

// One element of the A operand: row (j, q, c0, ri), column k = (ν, b, i'). The shifted vertex of
// sign s at shift m, node j: wlo J[klo] + whi J[klo + 1]; the mode value
// X±_ν = (1 - r_ν) S_{m_ν} + r_ν S_{m_ν + 1}; the combination q folds the channel algebra:
//   q = 0, 2 : (X+ - X-)/2 of c12 = 11, 22        (the Kramers-Kronig argument)
//   q = 1, 3 : -(1/2 + n_ν)(X+ + X-) of c12 = 11, 22
//   q = 4    : n_ν X+ + (1 + n_ν) X- of c12 = 21
//   q = 5    : (1 + n_ν) X+ + n_ν X- of c12 = 12
__device__ __forceinline__ double xgen_value(const double2* __restrict__ J, const int32_t* __restrict__ klo,
                                             const double* __restrict__ wlo, const double* __restrict__ whi, int nw,
                                             int ns, int j, int q, int c0, int ri, int m, double r, double n, int b,
                                             long ip) {
  const int c12 = (q < 2) ? 0 : (q < 4 ? 3 : (q == 4 ? 1 : 2));
  double xs[2];
  for (int s = 0; s < 2; ++s) {
    double acc = 0;
    for (int dm = 0; dm < 2; ++dm) {
      const int mm = m + dm;
      const double wgt = dm == 0 ? 1 - r : r;
      if (wgt == 0.0 || mm >= ns) continue;
      const long t = j + long(nw) * (mm + long(ns) * s);
      const int kl = klo[t];
      const double2 z0 = J[jidx(nw, kl, c12, b, c0, ip)], z1 = J[jidx(nw, kl + 1, c12, b, c0, ip)];
      const double zz = ri == 0 ? wlo[t] * z0.x + whi[t] * z1.x : wlo[t] * z0.y + whi[t] * z1.y;
      acc += wgt * zz;
    }
    xs[s] = acc;
  }
  switch (q) {
    case 0:
    case 2: return (xs[0] - xs[1]) / 2;
    case 1:
    case 3: return -(0.5 + n) * (xs[0] + xs[1]);
    case 4: return n * xs[0] + (1 + n) * xs[1];
    default: return (1 + n) * xs[0] + n * xs[1];
  }
}

// FP64 A operand, column-major [24 nwp, Kx] (rows j >= nω and modes ν >= nm are zero).
__global__ void xgen_f64_kernel(const double2* __restrict__ J, const int32_t* __restrict__ klo, const double* __restrict__ wlo,
                                const double* __restrict__ whi, const int32_t* __restrict__ mnu, const double* __restrict__ rnu,
                                const double* __restrict__ nnu, int nw, int nwp, int ns, int nm, int nmp, int ni,
                                double* __restrict__ A) {
  const long nrow = 24l * nwp;
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= nrow * nmp * 3 * ni) return;
  long row = idx % nrow, k = idx / nrow;
  int j = int(row % nwp);
  int rr = int(row / nwp);
  int q = rr % 6, c0 = (rr / 6) % 2, ri = rr / 12;
  int nu = int(k % nmp), b = int((k / nmp) % 3);
  long ip = k / (3l * nmp);
  A[idx] = (j < nw && nu < nm) ? xgen_value(J, klo, wlo, whi, nw, ns, j, q, c0, ri, mnu[nu], rnu[nu], nnu[nu], b, ip) : 0.0;
}

// ---- the tensor-core contraction, interpolation after the product ----
// The shift interpolation of the regrouped sums acts on the frequency axis only, with weights that
// depend on (j, ν, sign) and not on the pair (b, i'), so it commutes with the contraction over the
// pairs:
//   Z_ν[(c12, c0, ri, p), (a, i)] = Σ_{b, i'} Jr[(c12, c0, ri, p), (b, i')] G̃[(ν, b, i'), (a, i)]
//   D[(q, c0, ri, j), (a, i)] = Σ_ν Σ_s c_q(ν, s) Σ_t w_{ν,s,t}(j) Z_ν[(c12(q), c0, ri, p_{ν,s}(j) + t), (a, i)]
// with Jr the vertex's re/im parts as rows. One product for all modes (N = nm 3ni columns (ν, a, i),
// K = 3ni) replaces the per-mode A operand (K = 16 3ni, 24 rows per node instead of 16): 0.62 of
// the tensor-core work, and the operand written and read back is Z instead of A (1.8 GB against
// 2.9 GB at 1251 nodes and 495 outer states). The channel combinations c_q (q = 0..5 on the
// components c12 = 11, 11, 22, 22, 21, 12) and the three taps of each mode and sign are applied by
// zgather_kernel; D's layout is the one the Kramers-Kronig and channel kernels read.

// Jr rows z 16 nwp + (ri 2 + c0) 4 nwp + 4 p + c12 (a node's four components adjacent, so that Z
// holds them as one float4), K-major with row stride Kzp (columns k = b + 3i',
// zero for p >= nω and k >= 3ni), from the vertex of right-hand side rmap[z] (z without rmap), FP32
// complex [nω, 4, 3, 2, ni] jstride apart: TF32-rounded (kTf32) or split into BF16 hi/lo. A block
// transposes a tile of 32 nodes x 32 pairs of one (c12, c0) through shared memory, reading node
// runs and writing 128-byte row segments. Grid (Kzp / 32, nwp / 32, 8 slots).
template <bool kTf32>
__global__ void __launch_bounds__(256) jmat_kernel(const float2* __restrict__ J_all, long jstride, const int* __restrict__ rmap,
                                                   int nw, int nwp, int ni, long Kzp, float* __restrict__ Jt,
                                                   __nv_bfloat16* __restrict__ Jh, __nv_bfloat16* __restrict__ Jl) {
  __shared__ float2 tile[32][33];
  const int k0 = blockIdx.x * 32, p0 = blockIdx.y * 32;
  const int comp = blockIdx.z % 8, z = blockIdx.z / 8;
  const int c12 = comp % 4, c0 = comp / 4;
  const int rhs = rmap ? rmap[z] : z;
  const float2* J = J_all + jstride * rhs;
  const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
  const long Kz = 3l * ni;
#pragma unroll
  for (int r = 0; r < 4; ++r) {  // pair k0 + ty + 8 r, node p0 + tx
    const long k = k0 + ty + 8 * r;
    const int p = p0 + tx;
    float2 v = make_float2(0.f, 0.f);
    if (k < Kz && p < nw) v = J[jidx(nw, p, c12, int(k % 3), c0, k / 3)];
    tile[ty + 8 * r][tx] = v;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 8; ++r) {  // row (ri, node p0 + ty + 4 (r % 4)... ): 8 rows of 32 columns per pass
    const int pl = ty + 8 * (r % 4), ri = r / 4;
    const float2 v = tile[tx][pl];
    const float x = ri ? v.y : v.x;
    const long row = long(z) * 16 * nwp + long(ri * 2 + c0) * 4 * nwp + long(p0 + pl) * 4 + c12;
    const long off = row * Kzp + k0 + tx;
    if constexpr (kTf32) {
      Jt[off] = round_tf32(x);
    } else {
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      Jh[off] = h;
      Jl[off] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
  }
}

// The contraction's B operand: rows (ν, a, i) = ν 3ni + n, K-major with row stride Kzp, from G̃
// [Kx, 3ni] column-major (rows k = ν + nmp (b + 3i')): TF32-rounded (Bt) or BF16 hi/lo (Bh, Bl).
__global__ void bz_build_kernel(const double* __restrict__ Gt, long Kx, int nmp, int nm, long N, long Kzp,
                                float* __restrict__ Bt, __nv_bfloat16* __restrict__ Bh, __nv_bfloat16* __restrict__ Bl) {
  const long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= long(nm) * N * Kzp) return;
  const long row = idx / Kzp, k = idx % Kzp;
  const long nu = row / N, n = row % N;
  const float x = k < N ? float(Gt[nu + nmp * k + Kx * n]) : 0.f;  // k < 3ni = N
  if (Bt) {
    Bt[idx] = round_tf32(x);
  } else {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    Bh[idx] = h;
    Bl[idx] = __float2bfloat16_rn(x - __bfloat162float(h));
  }
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// zgather_kernel: the largest block (two blocks resident per SM, the accumulators in registers).
constexpr int kZgMaxThreads = 320;

// D from Z (the formula above), FP32, modes in ascending order, both signs and three taps each.
// Z: [Mz, nm N] column-major (ld ldZ) as zsplits split-K partials zstride apart (summed in
// ascending order as they are staged); rows of slot z at z 16 nwp, then (ri 2 + c0) 4 nwp + 4 p +
// c12: a node's four components are one float4. ztab [nm][2][nwp]: per node, mode and sign the
// three tap weights (tent split folded in) and, in .w as integer bits, the first tap node p0 (the
// taps are p0, p0 + 1, p0 + 2); nnu_all 16 Bose occupations per right-hand side (rmap[z], or z).
// D[z 24 nwp + (q + 6 (c0 + 2 ri)) nwp + j + ldD n], rows j < nω.
// Grid (N / NC, 4 (c0, ri) x node ranges, slots), blockDim a multiple of 32 up to kZgMaxThreads: a
// block owns NC columns n of one (c0, ri) and the U blockDim nodes of its range; per mode it stages
// the window zwin[range][ν] (nodes [lo, hi): every node the range's taps read, as float4s) into
// rows of wstride float4s by asynchronous copies, double-buffered over ν, and each thread
// accumulates U nodes x NC columns, one shared-memory load per tap for the four components.
template <int U, int NC>
__global__ void __launch_bounds__(kZgMaxThreads, 2)
    zgather_kernel(const float* __restrict__ Z, long ldZ, int zsplits, long zstride, const float4* __restrict__ ztab,
                   const int2* __restrict__ zwin, int wstride, const float* __restrict__ nnu_all,
                   const int* __restrict__ rmap, int nw, int nwp, int nm, long N, float* __restrict__ D, long ldD) {
  extern __shared__ __align__(16) float4 zs4[];  // [2][NC][wstride]
  const long n0 = long(blockIdx.x) * NC;
  const int c0 = blockIdx.y & 1, ri = (blockIdx.y >> 1) & 1, rg = int(blockIdx.y >> 2);
  const long z = blockIdx.z;
  const int rhs = rmap ? rmap[z] : int(z);
  const float* nnu = nnu_all + 16 * rhs;
  const float* zb = Z + z * 16 * nwp + long(ri * 2 + c0) * 4 * nwp;  // the nodes' float4s, contiguous
  const int nthr = blockDim.x;
  const int jb = rg * U * nthr;  // the range's first node
  auto stage = [&](int nu, int buf, int2 win) {
    const int nn = win.y - win.x;  // nodes staged
    for (int c = 0; c < NC; ++c) {
      const long n = n0 + c;
      if (n >= N) break;
      float4* dst = zs4 + long(buf * NC + c) * wstride;
      // zeros after the staged nodes: a tap past the grid's last padded node (weight zero) reads them
      if (threadIdx.x < 4) dst[nn + threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
      const float* src = zb + ldZ * (long(nu) * N + n) + 4l * win.x;
      if (zsplits == 1) {
        for (int e = threadIdx.x; e < nn; e += nthr) cp_async16(dst + e, src + 4l * e);
      } else {  // split-K partials: summed here in ascending order (synchronous loads)
        for (int e = threadIdx.x; e < 4 * nn; e += nthr) {
          float acc = 0.f;
          for (int sp = 0; sp < zsplits; ++sp) acc += src[e + zstride * sp];
          reinterpret_cast<float*>(dst)[e] = acc;
        }
      }
    }
    cp_async_commit();
  };
  float acc[NC][U][6];
#pragma unroll
  for (int c = 0; c < NC; ++c)
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int q = 0; q < 6; ++q) acc[c][u][q] = 0.f;
  const int2* win_rg = zwin + long(rg) * nm;
  int2 win = win_rg[0];
  stage(0, 0, win);
  for (int nu = 0; nu < nm; ++nu) {
    const float nb = nnu[nu];
    const float hp = 0.5f + nb;
    const int2 win_next = win_rg[nu + 1 < nm ? nu + 1 : nu];  // loaded before the wait
    cp_async_wait_all();
    __syncthreads();  // mode nu's columns are in buffer nu & 1; buffer (nu + 1) & 1 is free
    if (nu + 1 < nm) stage(nu + 1, (nu + 1) & 1, win_next);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = jb + threadIdx.x + nthr * u;
      if (j >= nw) continue;
      float4 t[2];
      int pk[2];
#pragma unroll
      for (int sg = 0; sg < 2; ++sg) {
        t[sg] = ztab[(long(nu) * 2 + sg) * nwp + j];
        pk[sg] = __float_as_int(t[sg].w) - win.x;
      }
      // per sign s: the factors of components c12 = 0 (11, .x), 1 (21, .y), 2 (12, .z), 3 (22, .w)
      // in the six rows q (sign + : 1/2, -(1/2 + n), n, 1 + n; sign - : -1/2, -(1/2 + n), 1 + n, n)
#pragma unroll
      for (int sg = 0; sg < 2; ++sg) {
        const float half = sg ? -0.5f : 0.5f, fy = sg ? 1.f + nb : nb, fz = sg ? nb : 1.f + nb;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const float4* zc = zs4 + long((nu & 1) * NC + c) * wstride + pk[sg];
          const float4 r0 = zc[0], r1 = zc[1], r2 = zc[2];
          const float xx = t[sg].x * r0.x + t[sg].y * r1.x + t[sg].z * r2.x;
          const float xy = t[sg].x * r0.y + t[sg].y * r1.y + t[sg].z * r2.y;
          const float xz = t[sg].x * r0.z + t[sg].y * r1.z + t[sg].z * r2.z;
          const float xw = t[sg].x * r0.w + t[sg].y * r1.w + t[sg].z * r2.w;
          acc[c][u][0] += half * xx;
          acc[c][u][1] += -hp * xx;
          acc[c][u][2] += half * xw;
          acc[c][u][3] += -hp * xw;
          acc[c][u][4] += fy * xy;
          acc[c][u][5] += fz * xz;
        }
      }
    }
    win = win_next;
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const long n = n0 + c;
    if (n >= N) break;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = jb + threadIdx.x + nthr * u;
      if (j >= nw) continue;
#pragma unroll
      for (int q = 0; q < 6; ++q) D[z * 24 * nwp + long(q + 6 * (c0 + 2 * ri)) * nwp + j + ldD * n] = acc[c][u][q];
    }
  }
}

// Group size (M tiles) of the contraction's grouped tile order: 8 tiles of 128 rows of Jr.
constexpr int kZGroupM = 8;

// Threads and ranges for nω nodes (the windows, and with them NC and the staging, follow).
static ZgatherShape zgather_ranges(long nw, int U) {
  ZgatherShape g;
  g.U = U;
  const long nthr = (nw + U - 1) / U;  // threads for all nodes in one block
  g.nranges = int((nthr + kZgMaxThreads - 1) / kZgMaxThreads);
  g.threads = int(((nthr + g.nranges - 1) / g.nranges + 31) / 32 * 32);
  return g;
}
// The staging windows of zgather_kernel: for each node range and mode, the nodes [lo, hi) that
// hold every tap p0 .. p0 + 2 of the range's nodes (both signs), from the first-tap table hk
// [nm][2][nwp]; taps past nwp read the zeros staged after the window. Sets g.wstride (the widest
// window + 4, float4s), g.NC (4 while two double-buffered blocks fit an SM, else 2, else 1) and
// g.smem.
static std::vector<int32_t> zgather_windows(ZgatherShape& g, const std::vector<int32_t>& hk, long nw, long nwp, long nm) {
  std::vector<int32_t> win(size_t(2 * g.nranges * nm));
  const long span = long(g.U) * g.threads;
  long maxn = 1;
  for (long r = 0; r < g.nranges; ++r)
    for (long nu = 0; nu < nm; ++nu) {
      long lo = nwp, hi = 0;
      for (long j = r * span; j < std::min(nw, (r + 1) * span); ++j)
        for (long sg = 0; sg < 2; ++sg) {
          const long p0 = hk[size_t((nu * 2 + sg) * nwp + j)];
          if (p0 < 0 || p0 + 2 >= nwp + 4) fail(EPSP_EINVAL, "a shift-table tap outside the staged rows");
          lo = std::min(lo, p0);
          hi = std::max(hi, p0 + 3);
        }
      if (hi <= lo) lo = hi = 0;  // an empty range stages nothing
      hi = std::min(hi, nwp);
      win[size_t(2 * (r * nm + nu))] = int32_t(lo);
      win[size_t(2 * (r * nm + nu) + 1)] = int32_t(std::max(lo, hi));
      maxn = std::max(maxn, hi - lo);
    }
  g.wstride = int(maxn + 4);
  const size_t per_col = size_t(2 * g.wstride) * sizeof(float4);  // two buffers
  g.NC = per_col * 4 <= (size_t(110) << 10) ? 4 : per_col * 2 <= (size_t(110) << 10) ? 2 : 1;
  g.smem = per_col * size_t(g.NC);
  if (g.smem > (size_t(227) << 10))
    fail(EPSP_EUNSUPPORTED, "the ladder's interpolation windows do not fit shared memory (grid too fine for its modes)");
  return win;
}
template <int U, int NC>
static void launch_zgather_t(const ZgatherShape& g, dim3 grid, cudaStream_t s, const float* Z, long ldZ, int zsplits,
                             long zstride, const float4* ztab, const int2* zwin, const float* nnu, const int* rmap, int nw,
                             int nwp, int nm, long N, float* D, long ldD) {
  static size_t smem_set = 0;  // the largest dynamic shared memory allowed so far
  if (g.smem > smem_set) {
    EPSP_CUDA(cudaFuncSetAttribute(zgather_kernel<U, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(g.smem)));
    smem_set = g.smem;
  }
  zgather_kernel<U, NC><<<grid, g.threads, g.smem, s>>>(Z, ldZ, zsplits, zstride, ztab, zwin, g.wstride, nnu, rmap, nw,
                                                        nwp, nm, N, D, ldD);
}
// Grid (N / NC, 4 x node ranges, slots).
static void launch_zgather(const ZgatherShape& g, long N, unsigned slots, cudaStream_t s, const float* Z, long ldZ,
                           int zsplits, long zstride, const float4* ztab, const int2* zwin, const float* nnu,
                           const int* rmap, int nw, int nwp, int nm, float* D, long ldD) {
  const dim3 grid(unsigned((N + g.NC - 1) / g.NC), 4u * unsigned(g.nranges), slots);
  if (g.NC == 4)
    launch_zgather_t<2, 4>(g, grid, s, Z, ldZ, zsplits, zstride, ztab, zwin, nnu, rmap, nw, nwp, nm, N, D, ldD);
  else if (g.NC == 2)
    launch_zgather_t<2, 2>(g, grid, s, Z, ldZ, zsplits, zstride, ztab, zwin, nnu, rmap, nw, nwp, nm, N, D, ldD);
  else
    launch_zgather_t<2, 1>(g, grid, s, Z, ldZ, zsplits, zstride, ztab, zwin, nnu, rmap, nw, nwp, nm, N, D, ldD);
}

// Y (rows q = 0, 2 of D) as the BF16 hi/lo B operand of the Kramers-Kronig GEMM: row (qq, c0, ri, n),
// K = ω' contiguous, stride Kp2.
// Batched over blockIdx.y: slot z reads rows z 24 nwp.. of D (column stride ldD) and writes rows
// z 8N.. of Y.
// D is read as the sum of its dsplits split-K partials D + p dstride (in ascending p, as the FP32
// sum the GEMM's split-K parts take elsewhere). Grid (Kp2 / 256, N, slots): thread (ω', n) writes
// the 8 rows (qq, c0, ri, n).
__global__ void y_split_kernel(const float* __restrict__ D, long ldD, int dsplits, long dstride, int nw, int nwp, long N,
                               long Kp2, __nv_bfloat16* __restrict__ Yh, __nv_bfloat16* __restrict__ Yl) {
  const long w = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= Kp2) return;
  const long n = blockIdx.y, z = blockIdx.z;
  float x[8];
#pragma unroll
  for (int r8 = 0; r8 < 8; ++r8) x[r8] = 0.f;
  if (w < nw)
    for (int p = 0; p < dsplits; ++p) {  // the 8 loads of a partial issued together
      const float* src = D + z * 24 * nwp + w + ldD * n + dstride * p;
#pragma unroll
      for (int r8 = 0; r8 < 8; ++r8) {
        const int qq = r8 % 2, c0 = (r8 / 2) % 2, ri = r8 / 4;
        x[r8] += src[long(nwp) * ((qq == 0 ? 0 : 2) + 6 * (c0 + 2 * ri))];
      }
    }
#pragma unroll
  for (int r8 = 0; r8 < 8; ++r8) {
    const __nv_bfloat16 h = __float2bfloat16_rn(x[r8]);
    const long o = z * 8 * N * Kp2 + (r8 + 8 * n) * Kp2 + w;
    Yh[o] = h;
    Yl[o] = __float2bfloat16_rn(x[r8] - __bfloat162float(h));
  }
}

// out[r * Kp + c] = split(S[r + ldr c]) for c < cols (a column-major matrix read by rows).
__global__ void split_rows_t2_kernel(const double* __restrict__ S, long ldr, long rows, long cols, long Kp,
                                     __nv_bfloat16* __restrict__ oh, __nv_bfloat16* __restrict__ ol) {
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= rows * Kp) return;
  long r = idx / Kp, c = idx % Kp;
  float x = c < cols ? float(S[r + ldr * c]) : 0.f;
  __nv_bfloat16 h = __float2bfloat16_rn(x);
  oh[idx] = h;
  ol[idx] = __float2bfloat16_rn(x - __bfloat162float(h));
}

// Y of the regrouped path: the rows q = 0 (c12 = 11) and q = 2 (c12 = 22) of D, as [nω, (qq, c0, ri, n)].
__global__ void y_gemm_kernel(const double* __restrict__ D, int nw, int nwp, long ncol, double* __restrict__ Y) {
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  long total = long(nw) * 8 * ncol;
  if (idx >= total) return;
  long w = idx % nw, r = idx / nw;
  int qq = int(r % 2), c0 = int((r / 2) % 2), ri = int((r / 4) % 2);
  long n = r / 8;
  int q = qq == 0 ? 0 : 2;
  Y[idx] = D[w + long(nwp) * (q + 6 * (c0 + 2 * ri)) + 24l * nwp * n];
}


// Grid (nω / 256, 6 ni, slots): blockIdx.y is the (a, c0, i) row set; slot z = blockIdx.z reads rows
// z 24 nwp.. of D (column stride ldD) and KY + z nω 24ni, and writes LJ + 24 nω ni r with the
// propagators Gm, Gp + 4 nω ni r of right-hand side r = rmap[z] (r = z without rmap).
// With X_all, it writes X - L(X) instead of L(X) (the GMRES operator applied to X, in one pass).
// R = float (tensor-core path): D and KY (as split-K partials, summed in ascending order) in FP32 and
// the propagators and vertices FP32 complex; R = double: all FP64.
template <class R>
__global__ void finish_gemm_kernel(const R* __restrict__ D_all, long ldD, int dsplits, long dstride, const R* __restrict__ KY_all,
                                   int kysplits, long kystride,
                                   const Vec2<R>* __restrict__ Gm_all, const Vec2<R>* __restrict__ Gp_all,
                                   const int* __restrict__ rmap, int nw, int nwp, int ni, Vec2<R>* __restrict__ LJ_all,
                                   const Vec2<R>* __restrict__ X_all = nullptr) {
  using V = Vec2<R>;
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const int r = blockIdx.y;  // (a, c0, i)
  const long z = blockIdx.z;
  const long rhs = rmap ? rmap[z] : z;
  const R* D = D_all + z * 24 * nwp;
  const R* KY = KY_all + z * long(nw) * 24 * ni;
  const V* Gm = Gm_all + rhs * 4l * nw * ni;
  const V* Gp = Gp_all + rhs * 4l * nw * ni;
  V* LJ = LJ_all + rhs * 24l * nw * ni;
  const int a = r % 3, c0 = (r / 3) % 2;
  const long i = r / 6;
  const long n = a + 3 * i;
  // the 8 values of D this thread reads (rows q = 1, 3, 4, 5 of re and im; q = 0, 2 enter through
  // KY), summed over the split-K partials with all loads of a partial issued together
  R dv[2][6];
#pragma unroll
  for (int ri = 0; ri < 2; ++ri)
#pragma unroll
    for (int q = 0; q < 6; ++q) dv[ri][q] = 0;
  for (int p = 0; p < dsplits; ++p) {
    const R* src = D + w + ldD * n + dstride * p;
#pragma unroll
    for (int ri = 0; ri < 2; ++ri)
#pragma unroll
      for (int q = 1; q < 6; ++q)
        if (q != 2) dv[ri][q] += src[long(nwp) * (q + 6 * (c0 + 2 * ri))];
  }
  auto d = [&](int q, int ri) { return dv[ri][q]; };
  // KY as kysplits split-K partials kystride apart, summed in ascending order, the 4 values of a
  // partial loaded together
  R kv[2][2] = {{0, 0}, {0, 0}};  // [qq][ri]
  for (int p = 0; p < kysplits; ++p) {
    const R* src = KY + w + kystride * p;
#pragma unroll
    for (int qq = 0; qq < 2; ++qq)
#pragma unroll
      for (int ri = 0; ri < 2; ++ri) kv[qq][ri] += src[nw * (qq + 2 * (c0 + 2 * (ri + 2 * n)))];
  }
  auto ky = [&](int qq, int ri) { return kv[qq][ri]; };
  Cx<R> K[4];
  {
    const Cx<R> y0{ky(0, 0), ky(0, 1)};
    K[0] = {y0.y + d(1, 0), -y0.x + d(1, 1)};  // -i KY + rest
    const Cx<R> y3{ky(1, 0), ky(1, 1)};
    K[3] = {-y3.y + d(3, 0), y3.x + d(3, 1)};  // +i KY + rest
    K[1] = {d(4, 0), d(4, 1)};
    K[2] = {d(5, 0), d(5, 1)};
  }
  Cx<R> gm[4], gp[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const V a = Gm[w + long(nw) * (c + 4 * i)], b = Gp[w + long(nw) * (c + 4 * i)];
    gm[c] = {a.x, a.y};
    gp[c] = {b.x, b.y};
  }
#pragma unroll
  for (int c1 = 0; c1 < 2; ++c1)
#pragma unroll
    for (int c2 = 0; c2 < 2; ++c2) {
      Cx<R> z = cxmul(cxmul(gm[c1], K[0]), gp[0 + 2 * c2]);
      z = cxadd(z, cxmul(cxmul(gm[c1 + 2], K[1]), gp[0 + 2 * c2]));
      z = cxadd(z, cxmul(cxmul(gm[c1], K[2]), gp[1 + 2 * c2]));
      z = cxadd(z, cxmul(cxmul(gm[c1 + 2], K[3]), gp[1 + 2 * c2]));
      const long o = jidx(nw, w, c1 + 2 * c2, a, c0, i);
      V v = VecOf<V>::make(-z.x, -z.y);
      if (X_all) {
        const V x = X_all[rhs * 24l * nw * ni + o];
        v = VecOf<V>::make(x.x - v.x, x.y - v.y);
      }
      LJ[o] = v;
    }
}

// ---- GMRES BLAS-1 (fixed-order reductions) ----
// V = double2: FP64 throughout. V = float2: FP32 elements and products, each thread's sums carried
// in FP32 over runs of 8 elements and added into FP64, the block and grid sums in FP64.
// Batched over blockIdx.y: slot z works on the vectors of right-hand side r = rmap[z] (r = z without
// rmap), stored n apart.

constexpr int kDotBlocks = 1024;
constexpr int kRun = 8;  // elements per FP32 run of the float2 reductions

template <class V>
__device__ __forceinline__ long slot_rhs(const int* rmap) {
  return rmap ? rmap[blockIdx.y] : long(blockIdx.y);
}

// part[z gridDim.x + block] = block partial of conj(u) v.
template <class V>
__global__ void __launch_bounds__(256) dot_partial_kernel(const V* __restrict__ U, const V* __restrict__ Vv, long n,
                                                          const int* __restrict__ rmap, double2* __restrict__ part) {
  __shared__ double sr[256], si[256];
  const long r = slot_rhs<V>(rmap);
  const V* u = U + n * r;
  const V* v = Vv + n * r;
  double ar = 0, ai = 0;
  if constexpr (std::is_same_v<V, double2>) {
    for (long k = long(blockIdx.x) * 256 + threadIdx.x; k < n; k += long(gridDim.x) * 256) {
      double2 a = u[k], b = v[k];
      ar += a.x * b.x + a.y * b.y;  // conj(a) b
      ai += a.x * b.y - a.y * b.x;
    }
  } else {
    // runs of kRun strided elements, their loads issued together
    const long stride = long(gridDim.x) * 256;
    for (long k0 = long(blockIdx.x) * 256 + threadIdx.x; k0 < n; k0 += stride * kRun) {
      float2 a[kRun], b[kRun];
#pragma unroll
      for (int q = 0; q < kRun; ++q) {
        const long k = k0 + stride * q;
        a[q] = k < n ? u[k] : make_float2(0.f, 0.f);
        b[q] = k < n ? v[k] : make_float2(0.f, 0.f);
      }
      float fr = 0.f, fi = 0.f;
#pragma unroll
      for (int q = 0; q < kRun; ++q) {
        fr += a[q].x * b[q].x + a[q].y * b[q].y;
        fi += a[q].x * b[q].y - a[q].y * b[q].x;
      }
      ar += fr;
      ai += fi;
    }
  }
  sr[threadIdx.x] = ar;
  si[threadIdx.x] = ai;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sr[threadIdx.x] += sr[threadIdx.x + s];
      si[threadIdx.x] += si[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[long(blockIdx.y) * gridDim.x + blockIdx.x] = make_double2(sr[0], si[0]);
}

// out[rmap[z]] (out[z] without rmap) = Σ_b part[z][b] in order; one block per slot.
__global__ void __launch_bounds__(256) dot_final_kernel(const double2* __restrict__ part, int np, const int* __restrict__ rmap,
                                                        double2* __restrict__ out) {
  __shared__ double sr[256], si[256];
  double ar = 0, ai = 0;
  for (int k = threadIdx.x; k < np; k += 256) {
    ar += part[long(blockIdx.x) * np + k].x;
    ai += part[long(blockIdx.x) * np + k].y;
  }
  sr[threadIdx.x] = ar;
  si[threadIdx.x] = ai;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sr[threadIdx.x] += sr[threadIdx.x + s];
      si[threadIdx.x] += si[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[rmap ? rmap[blockIdx.x] : int(blockIdx.x)] = make_double2(sr[0], si[0]);
}

// Q[r] -= h[r] V[r] with h from device memory (one coefficient per right-hand side).
template <class V>
__global__ void axpy_dev_kernel(V* __restrict__ Q, const V* __restrict__ X, const double2* __restrict__ h, long n,
                                const int* __restrict__ rmap) {
  using R = typename VecOf<V>::R;
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const long r = slot_rhs<V>(rmap);
  const double2 hd = h[r];
  const R hx = R(hd.x), hy = R(hd.y);
  const V x = X[n * r + k], q = Q[n * r + k];
  Q[n * r + k] = VecOf<V>::make(q.x - (hx * x.x - hy * x.y), q.y - (hx * x.y + hy * x.x));
}

// Y[r] = a X[r] + b Y[r]: complex a, b from the host (a_dev, b_dev null) or per right-hand side
// from device memory.
template <class V>
__global__ void axpby_kernel(double2 a, const double2* __restrict__ a_dev, const V* __restrict__ X, double2 b,
                             const double2* __restrict__ b_dev, V* __restrict__ Y, long n, const int* __restrict__ rmap) {
  using R = typename VecOf<V>::R;
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const long r = slot_rhs<V>(rmap);
  if (a_dev) a = a_dev[r];
  if (b_dev) b = b_dev[r];
  const R ax = R(a.x), ay = R(a.y), bx = R(b.x), by = R(b.y);
  const V xv = X[n * r + k], yv = Y[n * r + k];
  Y[n * r + k] = VecOf<V>::make(ax * xv.x - ay * xv.y + bx * yv.x - by * yv.y, ax * xv.y + ay * xv.x + bx * yv.y + by * yv.x);
}

// Y[r] = a X[r] (Y is not read); a from the host or per right-hand side from device memory.
template <class V>
__global__ void scale_kernel(double2 a, const double2* __restrict__ a_dev, const V* __restrict__ X, V* __restrict__ Y, long n,
                             const int* __restrict__ rmap) {
  using R = typename VecOf<V>::R;
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const long r = slot_rhs<V>(rmap);
  if (a_dev) a = a_dev[r];
  const R ax = R(a.x), ay = R(a.y);
  const V xv = X[n * r + k];
  Y[n * r + k] = VecOf<V>::make(ax * xv.x - ay * xv.y, ax * xv.y + ay * xv.x);
}

// q -= h v (h from device memory) and the block partials of |q|^2 of the result, in the order of
// dot_partial_kernel (the norm of what the projection leaves, in the same pass). Single vectors.
template <class V>
__global__ void __launch_bounds__(256) axpy_norm_kernel(V* __restrict__ q, const V* __restrict__ v,
                                                        const double2* __restrict__ h, long n, double2* __restrict__ part) {
  using R = typename VecOf<V>::R;
  __shared__ double sr[256];
  const double2 hd = *h;
  const R hx = R(hd.x), hy = R(hd.y);
  double ar = 0;
  if constexpr (std::is_same_v<V, double2>) {
    for (long k = long(blockIdx.x) * 256 + threadIdx.x; k < n; k += long(gridDim.x) * 256) {
      const V x = v[k];
      V a = q[k];
      a = VecOf<V>::make(a.x - (hx * x.x - hy * x.y), a.y - (hx * x.y + hy * x.x));
      q[k] = a;
      ar += a.x * a.x + a.y * a.y;
    }
  } else {
    // runs of kRun strided elements, their loads issued together
    const long stride = long(gridDim.x) * 256;
    for (long k0 = long(blockIdx.x) * 256 + threadIdx.x; k0 < n; k0 += stride * kRun) {
      V xs[kRun], as[kRun];
#pragma unroll
      for (int t = 0; t < kRun; ++t) {
        const long k = k0 + stride * t;
        if (k < n) {
          xs[t] = v[k];
          as[t] = q[k];
        }
      }
      float fr = 0.f;
#pragma unroll
      for (int t = 0; t < kRun; ++t) {
        const long k = k0 + stride * t;
        if (k < n) {
          const V a = VecOf<V>::make(as[t].x - (hx * xs[t].x - hy * xs[t].y), as[t].y - (hx * xs[t].y + hy * xs[t].x));
          q[k] = a;
          fr += a.x * a.x + a.y * a.y;
        }
      }
      ar += fr;
    }
  }
  sr[threadIdx.x] = ar;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) sr[threadIdx.x] += sr[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = make_double2(sr[0], 0.0);
}

// Complex FP64 scalar arithmetic of the device Givens step (the operations of std::complex<double>
// on finite values: products without the C99 special cases, |z| as hypot, division by a real).
struct cuda_cplx {
  double x, y;
  static __device__ __forceinline__ cuda_cplx of(double2 v) { return {v.x, v.y}; }
  __device__ __forceinline__ double2 d2() const { return make_double2(x, y); }
  __device__ __forceinline__ cuda_cplx conj() const { return {x, -y}; }
  __device__ __forceinline__ double abs() const { return hypot(x, y); }
  __device__ __forceinline__ cuda_cplx operator*(cuda_cplx b) const { return {x * b.x - y * b.y, x * b.y + y * b.x}; }
  __device__ __forceinline__ cuda_cplx operator*(double s) const { return {x * s, y * s}; }
  __device__ __forceinline__ cuda_cplx operator/(double s) const { return {x / s, y / s}; }
  __device__ __forceinline__ cuda_cplx operator+(cuda_cplx b) const { return {x + b.x, y + b.y}; }
  __device__ __forceinline__ cuda_cplx operator-(cuda_cplx b) const { return {x - b.x, y - b.y}; }
};

// ---- the Arnoldi step on the device: classical Gram-Schmidt with one reorthogonalisation (CGS2)
// over the Krylov vectors (pointers vp[i]), m <= kMG vectors per pass, and the Givens update of
// Krylov.gmres's Hessenberg least-squares problem in FP64 on one thread ----
constexpr int kMG = 8;

// part[t kDotBlocks + block] = block partial of conj(V_{i0 + t}) w, t < m, in the reduction order of
// dot_partial_kernel (one pass over w for m vectors).
template <class V>
__global__ void __launch_bounds__(256) mdot_partial_kernel(V* const* __restrict__ vp, int i0, int m, const V* __restrict__ w,
                                                           long n, double2* __restrict__ part) {
  __shared__ double sr[256], si[256];
  double ar[kMG], ai[kMG];
  const V* vt[kMG];  // the m vectors' pointers, read once
#pragma unroll
  for (int t = 0; t < kMG; ++t) {
    ar[t] = ai[t] = 0;
    vt[t] = t < m ? vp[i0 + t] : w;
  }
  const long stride = long(gridDim.x) * 256;
  if constexpr (std::is_same_v<V, double2>) {
    for (long k = long(blockIdx.x) * 256 + threadIdx.x; k < n; k += stride) {
      const double2 b = w[k];
#pragma unroll
      for (int t = 0; t < kMG; ++t)
        if (t < m) {
          const double2 a = vt[t][k];
          ar[t] += a.x * b.x + a.y * b.y;  // conj(a) b
          ai[t] += a.x * b.y - a.y * b.x;
        }
    }
  } else {
    for (long k0 = long(blockIdx.x) * 256 + threadIdx.x; k0 < n; k0 += stride * kRun) {
      float2 b[kRun];
#pragma unroll
      for (int q = 0; q < kRun; ++q) {
        const long k = k0 + stride * q;
        b[q] = k < n ? w[k] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int t = 0; t < kMG; ++t)
        if (t < m) {
          const float2* v = vt[t];
          float fr = 0.f, fi = 0.f;
#pragma unroll
          for (int q = 0; q < kRun; ++q) {
            const long k = k0 + stride * q;
            const float2 a = k < n ? v[k] : make_float2(0.f, 0.f);
            fr += a.x * b[q].x + a.y * b[q].y;
            fi += a.x * b[q].y - a.y * b[q].x;
          }
          ar[t] += fr;
          ai[t] += fi;
        }
    }
  }
#pragma unroll
  for (int t = 0; t < kMG; ++t) {
    if (t >= m) break;  // m is the same for the whole block
    sr[threadIdx.x] = ar[t];
    si[threadIdx.x] = ai[t];
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
      if (threadIdx.x < st) {
        sr[threadIdx.x] += sr[threadIdx.x + st];
        si[threadIdx.x] += si[threadIdx.x + st];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) part[long(t) * gridDim.x + blockIdx.x] = make_double2(sr[0], si[0]);
    __syncthreads();
  }
}

// w -= Σ_{t < m} h[i0 + t] V_{i0 + t} (ascending t, in the arithmetic of axpy_dev_kernel); with part,
// also the block partials of |w|^2 of the result.
template <class V>
__global__ void __launch_bounds__(256) maxpy_kernel(V* __restrict__ w, V* const* __restrict__ vp, int i0, int m,
                                                    const double2* __restrict__ h, long n, double2* __restrict__ part) {
  using R = typename VecOf<V>::R;
  __shared__ double sr[256];
  R hx[kMG], hy[kMG];
  const V* vt[kMG];  // the m vectors' pointers, read once
#pragma unroll
  for (int t = 0; t < kMG; ++t) {
    const double2 hd = t < m ? h[i0 + t] : make_double2(0, 0);
    hx[t] = R(hd.x);
    hy[t] = R(hd.y);
    vt[t] = t < m ? vp[i0 + t] : w;
  }
  double ar = 0;
  const long stride = long(gridDim.x) * 256;
  for (long k0 = long(blockIdx.x) * 256 + threadIdx.x; k0 < n; k0 += stride * kRun) {
    R fr = 0;
#pragma unroll
    for (int q = 0; q < kRun; ++q) {
      const long k = k0 + stride * q;
      if (k < n) {
        V a = w[k];
#pragma unroll
        for (int t = 0; t < kMG; ++t)
          if (t < m) {
            const V x = vt[t][k];
            a = VecOf<V>::make(a.x - (hx[t] * x.x - hy[t] * x.y), a.y - (hx[t] * x.y + hy[t] * x.x));
          }
        w[k] = a;
        if constexpr (std::is_same_v<V, double2>)
          ar += a.x * a.x + a.y * a.y;
        else
          fr += a.x * a.x + a.y * a.y;
      }
    }
    if constexpr (!std::is_same_v<V, double2>) ar += fr;
  }
  if (!part) return;
  sr[threadIdx.x] = ar;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) sr[threadIdx.x] += sr[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = make_double2(sr[0], 0.0);
}

// One Givens step for Arnoldi column `inner` (1-based): h1 + h2 (the two Gram-Schmidt passes'
// projections, inner entries; h2 NULL after one pass) and ‖w‖^2 (hsq) complete the column; the
// previous rotations are applied, a new one annihilates H[k + 1, k], and z and the residual follow
// (src/ladder.jl:340-353 through Krylov.gmres). At inner = 1 it also takes ‖J0‖^2 and ‖r0‖^2 and sets
// atol and z[0]; a solve already solved at x0 stops there. inv_out receives 1 / H[k + 1, k] (0 for a
// breakdown), the scale of the next Krylov vector.
__global__ void gmres_givens_kernel(const double2* __restrict__ h1, const double2* __restrict__ h2,
                                    const double2* __restrict__ hsq, const double2* __restrict__ nJ0sq,
                                    const double2* __restrict__ beta_sq, double rtol, double btol, int inner,
                                    double2* __restrict__ Rp, double* __restrict__ cs, double2* __restrict__ sn,
                                    double2* __restrict__ zv, GmresDev* __restrict__ st, double2* __restrict__ inv_out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  using C = cuda_cplx;
  if (inner == 1) {
    st->nJ0 = sqrt(nJ0sq->x);
    st->atol = rtol * st->nJ0;
    st->beta = sqrt(beta_sq->x);
    st->rnorm = st->beta;
    st->solved = 0;
    st->breakdown = 0;
    st->solved_x0 = st->beta <= st->atol || st->beta == 0;
    zv[0] = make_double2(st->beta, 0);
    if (st->solved_x0) {
      st->solved = 1;
      st->inner = 0;
      inv_out->x = inv_out->y = 0;
      return;
    }
  }
  const long nr = long(inner - 1) * inner / 2;  // packed start of column inner - 1
  for (int i = 0; i < inner; ++i)
    Rp[nr + i] = h2 ? make_double2(h1[i].x + h2[i].x, h1[i].y + h2[i].y) : h1[i];
  const double Hbis = sqrt(hsq->x);
  for (int i = 0; i < inner - 1; ++i) {
    const C r0 = C::of(Rp[nr + i]), r1 = C::of(Rp[nr + i + 1]), sv = C::of(sn[i]);
    const C Rt = r0 * cs[i] + sv * r1;  // c R[i] + s R[i + 1]
    Rp[nr + i + 1] = (sv.conj() * r0 - r1 * cs[i]).d2();
    Rp[nr + i] = Rt.d2();
  }
  const C a = C::of(Rp[nr + inner - 1]);
  const double abs_a = a.abs();
  double cc;
  C ss, rho;
  if (Hbis == 0) {
    cc = 1;
    ss = C{0, 0};
    rho = a;
  } else if (abs_a == 0) {
    cc = 0;
    ss = C{1, 0};
    rho = C{Hbis, 0};
  } else {
    const double rr = hypot(abs_a, Hbis);
    const C psi = a / abs_a;
    cc = abs_a / rr;
    ss = psi * (Hbis / rr);
    rho = psi * rr;
  }
  cs[inner - 1] = cc;
  sn[inner - 1] = ss.d2();
  Rp[nr + inner - 1] = rho.d2();
  const C zk = C::of(zv[inner - 1]);
  const C zeta = ss.conj() * zk;
  zv[inner - 1] = (zk * cc).d2();
  zv[inner] = zeta.d2();
  st->rnorm = zeta.abs();
  st->solved = st->rnorm <= st->atol || st->rnorm + 1.0 <= 1.0;
  st->breakdown = Hbis <= btol;
  st->hbis = Hbis;
  st->inv_hbis = Hbis > 0 ? 1.0 / Hbis : 0.0;
  st->inner = inner;
  inv_out->x = st->inv_hbis;
  inv_out->y = 0;
}

// O[r] = X[r] - Y[r] resp. X[r] + Y[r].
template <class V>
__global__ void sub_kernel(const V* __restrict__ X, const V* __restrict__ Y, V* __restrict__ O, long n,
                           const int* __restrict__ rmap) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const long r = slot_rhs<V>(rmap);
  const V x = X[n * r + k], y = Y[n * r + k];
  O[n * r + k] = VecOf<V>::make(x.x - y.x, x.y - y.y);
}

template <class V>
__global__ void add_kernel(const V* __restrict__ X, const V* __restrict__ Y, V* __restrict__ O, long n) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const V x = X[k], y = Y[k];
  O[k] = VecOf<V>::make(x.x + y.x, x.y + y.y);
}

// FP32 <-> FP64 complex copies at the boundary of the tensor-core path (host vertices are FP64).
__global__ void to_f2_kernel(const double2* __restrict__ x, long n, float2* __restrict__ y) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) y[k] = make_float2(float(x[k].x), float(x[k].y));
}
__global__ void to_d2_kernel(const float2* __restrict__ x, long n, double2* __restrict__ y) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) y[k] = make_double2(double(x[k].x), double(x[k].y));
}

// ---------------------------------------------------------------------------------------------
// setup
// ---------------------------------------------------------------------------------------------

static void check_ladder_model(const epsp_model* m) {
  if (!m) fail(EPSP_EINVAL, "model is NULL");
  if (m->nm < 1 || m->ni < 1 || m->nf < 1) fail(EPSP_EINVAL, "nm, ni and nf must be positive");
  if (!m->g2 || !m->omega_ph || !m->iq_kk || !m->iks_i || !m->iks_f || !m->eps_i || !m->w_i || !m->w_f ||
      !m->f_to_i || !m->R || !m->v)
    fail(EPSP_EINVAL, "a required model array is NULL (the ladder needs R and v)");
  for (int64_t f = 0; f < m->nf; ++f) {
    if (m->f_to_i[f] < 0 || m->f_to_i[f] >= m->ni) fail(EPSP_EINVAL, "f_to_i out of range");
    if (m->iks_f[f] < 0 || m->iks_f[f] >= m->nk_f) fail(EPSP_EINVAL, "iks_f out of range");
  }
  for (int64_t i = 0; i < m->ni; ++i)
    if (m->iks_i[i] < 0 || m->iks_i[i] >= m->nk_i) fail(EPSP_EINVAL, "iks_i out of range");
  for (int64_t k = 0; k < m->nk_i * m->nk_f; ++k)
    if (m->iq_kk[k] < 0 || m->iq_kk[k] >= m->nq) fail(EPSP_EINVAL, "iq_kk out of range");
}

// The tensor-core paths: the contraction on tcgen05 (BF16x3 or TF32), FP32 vertices.
static bool tc_path(int path) { return path == EPSP_PATH_GEMM_BF16 || path == EPSP_PATH_GEMM_TF32; }

static TcOperand one_part_tf32(const float* a, long rows, long cols, long ld, int box_rows, int bk = 32) {
  TcOperand op;
  op.ns = 1;
  op.bk = bk;
  op.tf32 = true;
  op.m[0] = make_tmap_f32(a, rows, cols, ld, box_rows, bk);
  op.m[1] = op.m[0];
  op.m[2] = op.m[0];
  op.base[0] = op.base[1] = op.base[2] = a;
  op.rows = rows;
  op.cols = cols;
  op.ld = ld;
  return op;
}

// The contraction's operands for the plan's tile shape: BF16x3 maps with K boxes of 64 (opA64,
// opG128, opG256) or 32 (opA32, opG256_32); TF32 maps have K boxes of 32 only.
static void pick_contraction_operands(LadderPlan* P) {
  const bool narrow = P->path == EPSP_PATH_GEMM_BF16 && P->bk == 32;
  P->opA = narrow ? P->opA32 : P->opA64;
  P->opG = narrow ? P->opG256_32 : (P->bn == 256 ? P->opG256 : P->opG128);
}

static TcOperand two_part(const void* hi, const void* lo, long rows, long cols, long ld, int box_rows, int bk = kTcBK) {
  TcOperand op;
  op.ns = 2;
  op.bk = bk;
  op.m[0] = make_tmap_bf16(hi, rows, cols, ld, box_rows, bk);
  op.m[1] = make_tmap_bf16(lo, rows, cols, ld, box_rows, bk);
  op.m[2] = op.m[0];
  op.base[0] = op.base[2] = hi;
  op.base[1] = lo;
  op.rows = rows;
  op.cols = cols;
  op.ld = ld;
  return op;
}

static std::vector<double> g2_as_double(const epsp_model* m) {
  const size_t n = size_t(m->nm * m->ni * m->nf);
  std::vector<double> out(n);
  if (m->g2_dtype == EPSP_F64) {
    std::memcpy(out.data(), m->g2, n * 8);
  } else if (m->g2_dtype == EPSP_F32) {
    const float* p = static_cast<const float*>(m->g2);
    for (size_t k = 0; k < n; ++k) out[k] = double(p[k]);
  } else {
    const uint16_t* p = static_cast<const uint16_t*>(m->g2);
    for (size_t k = 0; k < n; ++k) {
      uint32_t u = uint32_t(p[k]) << 16;
      float x;
      std::memcpy(&x, &u, 4);
      out[k] = double(x);
    }
  }
  return out;
}

LadderPlan* ladder_setup(Ctx* ctx, const epsp_model* m, const epsp_options* opts) {
  check_ladder_model(m);
  if (!opts) fail(EPSP_EINVAL, "options are NULL");
  if (opts->gpu_tile < 0) fail(EPSP_EINVAL, "gpu_tile must be nothing or a positive number of inner states");
  if (!(opts->omega_acoustic > 0))
    fail(EPSP_EINVAL, "omega_acoustic must be positive: the shift-grid coupling build has no row for a negative phonon frequency");
  auto* P = new LadderPlan;
  std::unique_ptr<LadderPlan> guard(P);
  cudaStream_t s = ctx->stream;
  P->ctx = ctx;
  P->path = opts->path;
  P->w_ac = opts->omega_acoustic;
  P->nm = m->nm;
  P->ni = m->ni;
  P->nf = m->nf;
  P->ws = make_grid(m->omegas, "omegas");
  P->nw = P->ws.n;
  P->h = P->ws.unit;
  PhaseLog plog(ctx, "ladder", opts->verbosity);
  const long nm = P->nm, ni = P->ni, nf = P->nf, nw = P->nw;
  // nshift = ceil(max ωph / dω_unit) + 2 (src/ladder.jl:151)
  double mx = -std::numeric_limits<double>::infinity();
  for (int64_t k = 0; k < m->nm * m->nq; ++k) mx = std::max(mx, m->omega_ph[k]);
  if (!std::isfinite(mx)) fail(EPSP_EINVAL, "omega_ph must be finite");
  P->nshift = long(std::ceil(mx / P->h)) + 2;
  if (P->nshift < 2) P->nshift = 2;
  const long ns = P->nshift;
  P->Ww_h = trapezoid_weights(P->ws.nodes);
  P->v_h.assign(m->v, m->v + 3 * ni);
  P->w_i_h.assign(m->w_i, m->w_i + ni);
  P->d_ws = to_device(ctx, P->ws.nodes);
  P->d_Ww = to_device(ctx, P->Ww_h);
  P->d_eps_i = to_device(ctx, m->eps_i, size_t(ni));
  P->d_v = to_device(ctx, m->v, size_t(3 * ni));
  // KK (src/frequency_grids.jl:30-44), through the same device builder as the scGD0 plan
  kk_matrix_to_device(ctx, P->ws.nodes, P->d_KK);
  plog.mark("grid, KK matrix");
  // stars: sortperm(f_to_i) (stable) and the cumulative star sizes (src/ladder.jl:144-149)
  std::vector<int32_t> by_star(static_cast<size_t>(nf));
  for (long f = 0; f < nf; ++f) by_star[size_t(f)] = int32_t(f);
  std::stable_sort(by_star.begin(), by_star.end(), [&](int32_t a, int32_t b) { return m->f_to_i[a] < m->f_to_i[b]; });
  std::vector<int32_t> sp(size_t(ni + 1), 0);
  for (long f = 0; f < nf; ++f) sp[size_t(m->f_to_i[f] + 1)]++;
  for (long i = 0; i < ni; ++i) sp[size_t(i + 1)] += sp[size_t(i)];
  P->d_by_star = to_device(ctx, by_star);
  P->d_star_ptr = to_device(ctx, sp);
  // shift tables (src/ladder_kernel.jl:158-176): [nω, nshift, 2]
  {
    std::vector<int32_t> klo(size_t(nw * ns * 2));
    std::vector<double> wlo(klo.size()), whi(klo.size());
    const auto& off = P->ws.offsets;
    for (int sg = 0; sg < 2; ++sg)
      for (long mm = 0; mm < ns; ++mm)
        for (long j = 0; j < nw; ++j) {
          int64_t p = off[size_t(j)] + (sg == 0 ? mm : -mm);
          long ssl = long(std::upper_bound(off.begin(), off.end(), p) - off.begin());
          long k = std::clamp<long>(ssl, 1, nw - 1) - 1;
          double t = double(p - off[size_t(k)]) / double(off[size_t(k + 1)] - off[size_t(k)]);
          bool inside = off[0] <= p && p <= off[size_t(nw - 1)];
          size_t idx = size_t(j + nw * (mm + ns * sg));
          klo[idx] = int32_t(k);
          wlo[idx] = inside ? 1 - t : 0.0;
          whi[idx] = inside ? t : 0.0;
        }
    P->d_klo = to_device(ctx, klo);
    P->d_wlo = to_device(ctx, wlo);
    P->d_whi = to_device(ctx, whi);
  }
  if (P->path == EPSP_PATH_DIRECT_FP64) {  // the shift-grid coupling reads g2 in every application
    auto g2d = g2_as_double(m);
    P->d_g2 = to_device(ctx, g2d);
  }
  P->d_wf = to_device(ctx, m->w_f, size_t(nf));
  P->d_R = to_device(ctx, m->R, size_t(9 * nf));
  if (P->path == EPSP_PATH_DIRECT_FP64) {
    // chunks by whole stars (src/ladder.jl:180-202)
    const int64_t CB = int64_t(1) << 30;
    int64_t bytes_per_f = 8 * std::max(ns * ni * 2, nm * ni);
    int64_t bytes_per_i = 8 * std::max(ns * 9 * ni * 2, nw * 16 * ns * 3);
    int64_t max_f = opts->gpu_tile <= 0 ? std::max<int64_t>(CB / bytes_per_f, 1) : opts->gpu_tile;
    int64_t max_i = std::max<int64_t>(CB / bytes_per_i, 1);
    long i1 = 0, koff = 0, maxnf = 0, maxnip = 0;
    while (i1 < ni) {
      long i2 = i1;
      while (i2 < ni - 1 && i2 - i1 + 2 <= max_i && sp[size_t(i2 + 2)] - sp[size_t(i1)] <= max_f) ++i2;
      LadderChunk c;
      c.i0 = i1;
      c.i1 = i2 + 1;
      c.f0 = sp[size_t(i1)];
      c.f1 = sp[size_t(i2 + 1)];
      c.k_off = koff;
      koff += ns * 3 * (c.i1 - c.i0);
      maxnf = std::max(maxnf, c.f1 - c.f0);
      maxnip = std::max(maxnip, c.i1 - c.i0);
      P->chunks.push_back(c);
      i1 = i2 + 1;
    }
    P->Ktot = koff;
    auto d_wph = to_device(ctx, m->omega_ph, size_t(nm * m->nq));
    auto d_iq = to_device(ctx, m->iq_kk, size_t(m->nk_i * m->nk_f));
    auto d_iksi = to_device(ctx, m->iks_i, size_t(ni));
    auto d_iksf = to_device(ctx, m->iks_f, size_t(nf));
    P->d_wq.alloc(ctx, size_t(nm * nf * ni));
    gather_wq_star_kernel<<<div_up(size_t(nm * nf * ni), 256), 256, 0, s>>>(d_wph.p, d_iq.p, d_iksi.p, d_iksf.p, P->d_by_star.p,
                                                                           int(nm), nf, int(ni), m->nk_i, P->d_wq.p);
    EPSP_LAUNCHED(ctx);
    P->d_B.alloc(ctx, size_t(ns * maxnf * ni * 2));
    P->d_Bt.alloc(ctx, size_t(P->Ktot * 6 * ni));
    P->d_X.alloc(ctx, size_t(16 * nw * ns * 3 * maxnip));
    P->d_Cp.alloc(ctx, size_t(16 * nw * 6 * ni));
    P->d_Cm.alloc(ctx, size_t(16 * nw * 6 * ni));
    EPSP_CUDA(cudaStreamSynchronize(s));
  } else if (P->path == EPSP_PATH_GEMM_FP64 || tc_path(P->path)) {
    P->wnu.assign(size_t(nm), 0.0);
    for (long nu = 0; nu < nm; ++nu) {
      double w0 = m->omega_ph[nu];
      for (int64_t q = 1; q < m->nq; ++q)
        if (!(m->omega_ph[nu + nm * q] == w0))
          fail(EPSP_EUNSUPPORTED, "the GEMM paths need dispersionless modes (every row of omega_ph constant); use EPSP_PATH_DIRECT_FP64");
      P->wnu[size_t(nu)] = w0;
    }
    P->m_nu.resize(size_t(nm));
    P->r_nu.resize(size_t(nm));
    for (long nu = 0; nu < nm; ++nu) {
      double x = P->wnu[size_t(nu)] / P->h;  // the tent split of src/ladder_kernel.jl:199-206
      long lo = long(std::floor(x));
      P->m_nu[size_t(nu)] = int32_t(std::max<long>(lo, 0));
      P->r_nu[size_t(nu)] = x - double(lo);
      if (P->wnu[size_t(nu)] < P->w_ac) {
        P->m_nu[size_t(nu)] = 0;
        P->r_nu[size_t(nu)] = 0;
      }
    }
    P->d_mnu = to_device(ctx, P->m_nu);
    P->d_rnu = to_device(ctx, P->r_nu);
    P->d_nnu.alloc(ctx, size_t(nm));
    P->d_nnu_f.alloc(ctx, 16);
    auto d_wnu = to_device(ctx, P->wnu);
    P->nwp = (nw + 31) / 32 * 32;
    P->nmp = (nm + 15) / 16 * 16;
    if (tc_path(P->path) && P->nmp != 16)
      fail(EPSP_EUNSUPPORTED, "the tensor-core ladder paths take at most 16 modes; use EPSP_PATH_GEMM_FP64");
    if (6 * ni > 65535)  // the channel-algebra kernels put (a, c0, i) on the grid's y dimension
      fail(EPSP_EUNSUPPORTED, "the GEMM ladder paths take at most 10922 outer states");
    P->Kx = P->nmp * 3 * ni;
    P->d_Gt.alloc(ctx, size_t(P->Kx * 3 * ni));
    P->d_Gt.zero(s);
    plog.mark("stars, shift tables");
    // G̃ needs g2 once: it streams through the device star by star (gpu_tile inner states per chunk,
    // or about 64 MiB of g2), copies overlapped with the sums; g2 stays in the caller's memory
    {
      const size_t member_bytes = size_t(nm * ni) * g2_elem_bytes(m->g2_dtype);
      const long chunk_f =
          opts->gpu_tile > 0 ? long(opts->gpu_tile) : std::max<long>(1, long((size_t(64) << 20) / member_bytes));
      const unsigned grid = div_up(size_t(nm * ni), 128);
      stream_g2_by_columns(ctx, m, by_star, sp, chunk_f, [&](const void* g2c, long c0, long c1, long p0) {
        if (m->g2_dtype == EPSP_F64)
          coupling_rot_chunk_kernel<double><<<dim3(grid, unsigned(std::min<long>(c1 - c0, 65535))), 128, 0, s>>>(static_cast<const double*>(g2c), P->d_R.p, P->d_wf.p,
                                                                P->d_by_star.p, P->d_star_ptr.p, c0, c1, p0, d_wnu.p,
                                                                P->w_ac, int(nm), int(P->nmp), int(ni), P->Kx, P->d_Gt.p);
        else if (m->g2_dtype == EPSP_F32)
          coupling_rot_chunk_kernel<float><<<dim3(grid, unsigned(std::min<long>(c1 - c0, 65535))), 128, 0, s>>>(static_cast<const float*>(g2c), P->d_R.p, P->d_wf.p,
                                                               P->d_by_star.p, P->d_star_ptr.p, c0, c1, p0, d_wnu.p,
                                                               P->w_ac, int(nm), int(P->nmp), int(ni), P->Kx, P->d_Gt.p);
        else
          coupling_rot_chunk_kernel<uint16_t><<<dim3(grid, unsigned(std::min<long>(c1 - c0, 65535))), 128, 0, s>>>(static_cast<const uint16_t*>(g2c), P->d_R.p, P->d_wf.p,
                                                                  P->d_by_star.p, P->d_star_ptr.p, c0, c1, p0, d_wnu.p,
                                                                  P->w_ac, int(nm), int(P->nmp), int(ni), P->Kx,
                                                                  P->d_Gt.p);
        EPSP_LAUNCHED(ctx);
      });
    }
    const long M = 24 * P->nwp, N = 3 * ni;
    if (!tc_path(P->path)) P->d_D.alloc(ctx, size_t(M * N));  // the tensor-core paths keep D as split-K parts
    if (P->path == EPSP_PATH_GEMM_FP64) {
      P->d_Af.alloc(ctx, size_t(M * P->Kx));
    } else {
      plog.mark("g2 streamed, G~ built");
      // mode tables: for node j, mode ν and sign s, the two shift tables (m_ν, m_ν + 1) with the
      // tent weights (1 - r_ν, r_ν) folded into their interpolation weights (FP32). The two tables'
      // lower nodes differ by at most one (the grid's spacing is a multiple of its unit, the shift
      // step), so their four taps lie on three consecutive nodes p0, p0 + 1, p0 + 2: three weights
      // and the node (as integer bits in the fourth slot) per entry.
      {
        const long nwp = P->nwp;
        std::vector<int32_t> hk(size_t(nwp * nm * 2));
        std::vector<float> hw(size_t(nwp * nm * 2 * 4), 0.f);
        std::vector<int32_t> klo(size_t(nw * ns * 2));
        std::vector<double> wlo(klo.size()), whi(klo.size());
        P->d_klo.download(klo.data(), klo.size(), s);
        P->d_wlo.download(wlo.data(), wlo.size(), s);
        P->d_whi.download(whi.data(), whi.size(), s);
        EPSP_CUDA(cudaStreamSynchronize(s));
        for (long j = 0; j < nwp; ++j)
          for (long nu = 0; nu < nm; ++nu)
            for (long sg = 0; sg < 2; ++sg) {
              const size_t e = size_t((nu * 2 + sg) * nwp + j);  // [ν][s][j]: consecutive nodes adjacent
              hk[e] = int32_t(j);  // zero weights; the taps j.. j + 2 stay inside the staged rows and pads
              if (j >= nw || P->wnu[size_t(nu)] < P->w_ac) continue;
              const long mm = P->m_nu[size_t(nu)];
              const double r = P->r_nu[size_t(nu)];
              const size_t t0 = size_t(j + nw * (mm + ns * sg));
              long ka = klo[t0], kb = ka;
              double tw[4] = {(1 - r) * wlo[t0], (1 - r) * whi[t0], 0.0, 0.0};
              if (mm + 1 < ns && r != 0.0) {
                const size_t t1 = size_t(j + nw * (mm + 1 + ns * sg));
                kb = klo[t1];
                tw[2] = r * wlo[t1];
                tw[3] = r * whi[t1];
              }
              if (std::labs(kb - ka) > 1)
                fail(EPSP_EUNSUPPORTED, "neighbouring shift tables more than one node apart (the grid spacing is below its unit)");
              const long p0 = std::min(ka, kb);
              double cw[3] = {0, 0, 0};
              cw[ka - p0] += tw[0];
              cw[ka + 1 - p0] += tw[1];
              cw[kb - p0] += tw[2];
              cw[kb + 1 - p0] += tw[3];
              hk[e] = int32_t(p0);
              for (int t = 0; t < 3; ++t) hw[4 * e + size_t(t)] = float(cw[t]);
            }
        for (size_t e = 0; e < hk.size(); ++e) std::memcpy(&hw[4 * e + 3], &hk[e], sizeof(int32_t));
        P->d_ztab = to_device(ctx, hw);
        P->zg = zgather_ranges(nw, 2);
        P->d_zwin = to_device(ctx, zgather_windows(P->zg, hk, nw, nwp, nm));
      }
      P->Kp2 = (nw + 63) / 64 * 64;
      const bool tf = P->path == EPSP_PATH_GEMM_TF32;
      // the contraction Z = Jr Bz: Jr [16 nwp][Kzp] (written per application), Bz [nm 3ni][Kzp] from G̃
      P->Mz = 16 * P->nwp;
      P->Nz = nm * N;
      P->Kz = N;
      P->Kzp = (P->Kz + 63) / 64 * 64;
      const size_t nB = size_t(P->Nz * P->Kzp);
      if (tf) {
        P->d_Jt.alloc(ctx, size_t(P->Mz * P->Kzp));
        P->d_Bzt.alloc(ctx, nB);
        bz_build_kernel<<<div_up(nB, 256), 256, 0, s>>>(P->d_Gt.p, P->Kx, int(P->nmp), int(nm), N, P->Kzp, P->d_Bzt.p,
                                                        nullptr, nullptr);
      } else {
        P->d_Jh.alloc(ctx, size_t(P->Mz * P->Kzp));
        P->d_Jl.alloc(ctx, size_t(P->Mz * P->Kzp));
        P->d_Bzh.alloc(ctx, nB);
        P->d_Bzl.alloc(ctx, nB);
        bz_build_kernel<<<div_up(nB, 256), 256, 0, s>>>(P->d_Gt.p, P->Kx, int(P->nmp), int(nm), N, P->Kzp, nullptr,
                                                        P->d_Bzh.p, P->d_Bzl.p);
      }
      EPSP_LAUNCHED(ctx);
      plog.mark("mode tables, operand buffers");
      // the contraction's tile shape: the autotuner times the candidates on these operands (Jr
      // zeroed), in launch order and in grouped order (Bz, nm 3ni rows, is too large to stay in L2
      // across the M tiles), and keeps the fastest. Z holds two split-K partials while that costs
      // at most 512 MB, else one.
      const size_t zbytes = size_t(P->Mz) * size_t(P->Nz) * sizeof(float);
      P->zsplit_cap = zbytes * 2 <= (size_t(512) << 20) ? 2 : 1;
      const int Mi = int(P->Mz), Ni = int(P->Nz), Ki = int(P->Kz);
      int bn_h = 128, sp_h = 1;
      tc_gemm_shape(ctx, Mi, Ni, Ki, P->zsplit_cap, 2, &bn_h, &sp_h);
      P->d_Z.alloc(ctx, size_t(P->zsplit_cap) * size_t(P->Mz * P->Nz));
      P->d_Dz.alloc(ctx, size_t(M * N));
      P->d_err.alloc(ctx, 1);
      P->d_err.zero(s);
      if (tf) {  // one TF32 map per operand, K boxes of 32 (128 bytes); opA32 / opG256_32 alias them
        P->d_Jt.zero(s);
        P->opA64 = P->opA32 = one_part_tf32(P->d_Jt.p, P->Mz, P->Kz, P->Kzp, kTcBM);
        P->opG128 = one_part_tf32(P->d_Bzt.p, P->Nz, P->Kz, P->Kzp, 128);
        P->opG256 = P->opG256_32 = one_part_tf32(P->d_Bzt.p, P->Nz, P->Kz, P->Kzp, 256);
      } else {
        P->d_Jh.zero(s);
        P->d_Jl.zero(s);
        P->opA64 = two_part(P->d_Jh.p, P->d_Jl.p, P->Mz, P->Kz, P->Kzp, kTcBM);
        P->opG128 = two_part(P->d_Bzh.p, P->d_Bzl.p, P->Nz, P->Kz, P->Kzp, 128);
        P->opG256 = two_part(P->d_Bzh.p, P->d_Bzl.p, P->Nz, P->Kz, P->Kzp, 256);
        P->opA32 = two_part(P->d_Jh.p, P->d_Jl.p, P->Mz, P->Kz, P->Kzp, kTcBM, 32);
        P->opG256_32 = two_part(P->d_Bzh.p, P->d_Bzl.p, P->Nz, P->Kz, P->Kzp, 256, 32);
      }
      const TcTune best = tc_gemm_autotune(ctx, P->opA64, P->opG128, P->opG256, Mi, Ni, Ki, P->d_Z.p, P->Mz,
                                           P->Mz * P->Nz, P->zsplit_cap, P->d_err.p, 3, &P->tune_all, &P->opA32,
                                           &P->opG256_32, kZGroupM);
      for (const auto& c : P->tune_all)
        if (c.bn == bn_h && c.splits == sp_h && c.bk == (tf ? 32 : kTcBK) && !c.persist && c.gm == 1)
          P->tune_ms_heuristic = c.ms;
      P->bn = best.bn;
      P->splits = best.splits;
      P->bk = best.bk;
      P->persist = best.persist;
      P->pair = best.pair;
      P->gm = best.gm;
      pick_contraction_operands(P);
      int terr = 0;
      P->d_err.download(&terr, 1, s);
      EPSP_CUDA(cudaStreamSynchronize(s));
      if (terr) {
        P->d_err.zero(s);
        fail(EPSP_EDEVICE_TIMEOUT, "a tensor-core GEMM wait ran out while tuning (bounded device wait)");
      }
      plog.mark("tile shape (autotuner or cache)");
      // the Kramers-Kronig image on the tensor cores: A = KK [nω][nω'], B = Y [8N][nω']
      P->d_KKh.alloc(ctx, size_t(nw * P->Kp2));
      P->d_KKl.alloc(ctx, size_t(nw * P->Kp2));
      split_rows_t2_kernel<<<div_up(size_t(nw * P->Kp2), 256), 256, 0, s>>>(P->d_KK.p, nw, nw, nw, P->Kp2, P->d_KKh.p,
                                                                            P->d_KKl.p);
      EPSP_LAUNCHED(ctx);
      P->d_Yh.alloc(ctx, size_t(8 * N * P->Kp2));
      P->d_Yl.alloc(ctx, size_t(8 * N * P->Kp2));
      tc_gemm_shape(ctx, int(nw), int(8 * N), int(nw), 16, 2, &P->bn2, &P->splits2);
      P->d_part2.alloc(ctx, size_t(P->splits2) * size_t(nw * 8 * N));
      P->opKK = two_part(P->d_KKh.p, P->d_KKl.p, nw, nw, P->Kp2, kTcBM);
      P->opY = two_part(P->d_Yh.p, P->d_Yl.p, 8 * N, nw, P->Kp2, P->bn2);
    }
    EPSP_CUDA(cudaStreamSynchronize(s));
  } else {
    fail(EPSP_EINVAL, "unknown path");
  }
  if (tc_path(P->path)) {
    P->d_Gmf.alloc(ctx, size_t(nw * 4 * ni));
    P->d_Gpf.alloc(ctx, size_t(nw * 4 * ni));
  } else {
    P->d_Y.alloc(ctx, size_t(nw * 48 * ni));
    P->d_KY.alloc(ctx, size_t(nw * 48 * ni));
    P->d_Gm.alloc(ctx, size_t(nw * 4 * ni));
    P->d_Gp.alloc(ctx, size_t(nw * 4 * ni));
  }
  P->d_ST.alloc(ctx, size_t(nw * ni));
  P->d_jm.alloc(ctx, size_t(nw));
  P->d_jp.alloc(ctx, size_t(nw));
  P->d_tm.alloc(ctx, size_t(nw));
  P->d_tp.alloc(ctx, size_t(nw));
  plog.mark("KK operands, per-(T, Ω) buffers");
  return guard.release();
}

// ---------------------------------------------------------------------------------------------
// operator
// ---------------------------------------------------------------------------------------------

// Propagators of (T, μ, Ω) from Σ_T on the device (d_ST); with launch = false only the
// interpolation tables of Ω (for a kernel that forms the propagators itself).
static void set_propagators(LadderPlan* P, double mu, double T, double Om, bool launch = true) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  const long nw = P->nw, ni = P->ni;
  if (!(P->tab_Om == Om)) {  // the interpolation tables depend on Ω only
    // the previous uploads from these host tables must be done before they are rebuilt
    EPSP_CUDA(cudaStreamSynchronize(s));
    std::vector<double> xm(static_cast<size_t>(nw)), xp(static_cast<size_t>(nw));
    for (long k = 0; k < nw; ++k) {
      xm[size_t(k)] = P->ws.nodes[size_t(k)] - Om / 2;
      xp[size_t(k)] = P->ws.nodes[size_t(k)] + Om / 2;
    }
    interp_table(P->ws.nodes, xm, P->h_jm, P->h_tm);
    interp_table(P->ws.nodes, xp, P->h_jp, P->h_tp);
    P->d_jm.upload(P->h_jm.data(), size_t(nw), s);
    P->d_jp.upload(P->h_jp.data(), size_t(nw), s);
    P->d_tm.upload(P->h_tm.data(), size_t(nw), s);
    P->d_tp.upload(P->h_tp.data(), size_t(nw), s);
    P->tab_Om = Om;
  }
  P->cur_T = T;
  P->cur_mu = mu;
  P->cur_Om = Om;
  if (!launch) return;
  const dim3 grid(div_up(size_t(nw), 128), unsigned(ni));
  if (tc_path(P->path))
    propagators_kernel<true><<<grid, 128, 0, s>>>(P->d_ST.p, P->d_ws.p, int(nw), P->d_jm.p, P->d_tm.p, P->d_jp.p, P->d_tp.p,
                                                   P->d_eps_i.p, mu, T, Om, P->d_Gmf.p, P->d_Gpf.p, int(ni));
  else
    propagators_kernel<false><<<grid, 128, 0, s>>>(P->d_ST.p, P->d_ws.p, int(nw), P->d_jm.p, P->d_tm.p, P->d_jp.p,
                                                    P->d_tp.p, P->d_eps_i.p, mu, T, Om, P->d_Gm.p, P->d_Gp.p, int(ni));
  EPSP_LAUNCHED(ctx);
}

// B̃ of temperature T for every chunk (the B build and star sum of src/ladder.jl:257-281).
static void build_Bt(LadderPlan* P, double T) {
  if (P->Bt_T == T) return;
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  const long ni = P->ni, ns = P->nshift;
  for (const auto& c : P->chunks) {
    const long nfc = c.f1 - c.f0, nip = c.i1 - c.i0;
    bin_coupling_kernel<<<div_up(size_t(nfc * ni * 2), 128), 128, 0, s>>>(P->d_g2.p, P->d_wq.p, P->d_by_star.p, P->d_wf.p,
                                                                         int(P->nm), int(ni), P->nf, c.f0, nfc, int(ns), P->h,
                                                                         P->w_ac, T, P->d_B.p);
    EPSP_LAUNCHED(ctx);
    const long total = ns * 3 * nip * 6 * ni;
    star_sum_kernel<<<div_up(size_t(total), 256), 256, 0, s>>>(P->d_B.p, P->d_R.p, P->d_by_star.p, P->d_star_ptr.p, c.i0, nip,
                                                               c.f0, nfc, int(ns), int(ni), P->Ktot, c.k_off, P->d_Bt.p);
    EPSP_LAUNCHED(ctx);
  }
  P->Bt_T = T;
}

// LJ = L(J) with the current propagators (apply_ladder_kernel!, src/ladder.jl:245-296).
// The Bose occupations of the modes at T, for the regrouped GEMM paths (uploaded when T changes).
static void set_mode_occupations(LadderPlan* P, double T) {
  if (P->Bt_T == T) return;
  cudaStream_t s = P->ctx->stream;
  std::vector<double> nnu(size_t(P->nm));
  std::vector<float> nf16(16, 0.f);
  for (long nu = 0; nu < P->nm; ++nu) {
    double w = P->wnu[size_t(nu)];
    nnu[size_t(nu)] = w < P->w_ac ? 0.0 : (T > 1.4901161193847656e-08 ? (w == 0 ? -0.5 : 1.0 / std::expm1(w / T)) : (w > 0 ? 0.0 : -1.0));
    if (nu < 16) nf16[size_t(nu)] = float(nnu[size_t(nu)]);
  }
  P->d_nnu.upload(nnu.data(), size_t(P->nm), s);
  P->d_nnu_f.upload(nf16.data(), 16, s);
  EPSP_CUDA(cudaStreamSynchronize(s));
  P->Bt_T = T;
}

// LJ = L(J) on the FP64 paths (DIRECT_FP64, GEMM_FP64). With X (GEMM_FP64 only), LJ receives
// X - L(J) instead.
static void apply_L(LadderPlan* P, const double2* J, double2* LJ, const double2* X = nullptr) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  const long nw = P->nw, ni = P->ni, ns = P->nshift;
  const double T = P->cur_T;
  if (tc_path(P->path)) fail(EPSP_EINVAL, "internal: FP64 vertices on the tensor-core path");
  if (P->path == EPSP_PATH_DIRECT_FP64) {
    build_Bt(P, T);
    const long nrow = 16 * nw, ncol = 6 * ni;
    P->d_Cp.zero(s);
    P->d_Cm.zero(s);
    for (const auto& c : P->chunks) {
      const long nip = c.i1 - c.i0, kc = ns * 3 * nip;
      for (int sg = 0; sg < 2; ++sg) {
        shifted_vertex_kernel<<<div_up(size_t(nrow * kc), 256), 256, 0, s>>>(J, P->d_klo.p + nw * ns * sg, P->d_wlo.p + nw * ns * sg,
                                                                            P->d_whi.p + nw * ns * sg, int(nw), int(ns), c.i0, nip,
                                                                            P->d_X.p);
        EPSP_LAUNCHED(ctx);
        long pg = prof_begin(ctx, "ladder_gemm");
        gemm_f64(ctx, false, int(nrow), int(ncol), int(kc), 1.0, P->d_X.p, nrow, P->d_Bt.p + c.k_off, P->Ktot, 1.0,
                 sg == 0 ? P->d_Cp.p : P->d_Cm.p, nrow);
        prof_end(ctx, pg);
      }
    }
    const long ny = nw * 48 * ni;
    y_direct_kernel<<<div_up(size_t(ny), 256), 256, 0, s>>>(P->d_Cp.p, P->d_Cm.p, ny, P->d_Y.p);
    EPSP_LAUNCHED(ctx);
    gemm_f64(ctx, false, int(nw), int(48 * ni), int(nw), 1.0, P->d_KK.p, nw, P->d_Y.p, nw, 0.0, P->d_KY.p, nw);
    finish_direct_kernel<<<div_up(size_t(nw * 6 * ni), 256), 256, 0, s>>>(P->d_Cp.p, P->d_Cm.p, P->d_KY.p, P->d_Gm.p, P->d_Gp.p,
                                                                          int(nw), int(ni), LJ);
    EPSP_LAUNCHED(ctx);
    return;
  }
  // regrouped GEMM path, FP64
  set_mode_occupations(P, T);
  const long nwp = P->nwp, M = 24 * nwp, N = 3 * ni;
  long px = prof_begin(ctx, "xgen");
  xgen_f64_kernel<<<div_up(size_t(M * P->Kx), 256), 256, 0, s>>>(J, P->d_klo.p, P->d_wlo.p, P->d_whi.p, P->d_mnu.p, P->d_rnu.p,
                                                                 P->d_nnu.p, int(nw), int(nwp), int(ns), int(P->nm),
                                                                 int(P->nmp), int(ni), P->d_Af.p);
  EPSP_LAUNCHED(ctx);
  prof_end(ctx, px);
  long pg = prof_begin(ctx, "ladder_gemm");
  gemm_f64(ctx, false, int(M), int(N), int(P->Kx), 1.0, P->d_Af.p, M, P->d_Gt.p, P->Kx, 0.0, P->d_D.p, M);
  prof_end(ctx, pg);
  const long ny = nw * 8 * N;
  y_gemm_kernel<<<div_up(size_t(ny), 256), 256, 0, s>>>(P->d_D.p, int(nw), int(nwp), N, P->d_Y.p);
  EPSP_LAUNCHED(ctx);
  gemm_f64(ctx, false, int(nw), int(8 * N), int(nw), 1.0, P->d_KK.p, nw, P->d_Y.p, nw, 0.0, P->d_KY.p, nw);
  finish_gemm_kernel<double><<<dim3(div_up(size_t(nw), 256), unsigned(6 * ni), 1), 256, 0, s>>>(
      P->d_D.p, M, 1, 0, P->d_KY.p, 1, 0, P->d_Gm.p, P->d_Gp.p, nullptr, int(nw), int(nwp), int(ni), LJ, X);
  EPSP_LAUNCHED(ctx);
}

// Jr of nA vertices (rows z 16 nwp..) into the plan's or a batch's operand buffers.
static void launch_jmat(LadderPlan* P, const float2* J, long jstride, const int* rmap, int nA, float* Jt,
                        __nv_bfloat16* Jh, __nv_bfloat16* Jl) {
  Ctx* ctx = P->ctx;
  const dim3 grid(unsigned(P->Kzp / 32), unsigned(P->nwp / 32), unsigned(8 * nA));
  if (P->path == EPSP_PATH_GEMM_TF32)
    jmat_kernel<true><<<grid, 256, 0, ctx->stream>>>(J, jstride, rmap, int(P->nw), int(P->nwp), int(P->ni), P->Kzp, Jt,
                                                     nullptr, nullptr);
  else
    jmat_kernel<false><<<grid, 256, 0, ctx->stream>>>(J, jstride, rmap, int(P->nw), int(P->nwp), int(P->ni), P->Kzp,
                                                      nullptr, Jh, Jl);
  EPSP_LAUNCHED(ctx);
}

// The tensor-core paths (GEMM_BF16, GEMM_TF32), FP32 vertices: LJ = L(J), or X - L(J) with X.
static void apply_L(LadderPlan* P, const float2* J, float2* LJ, const float2* X = nullptr) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  const long nw = P->nw, ni = P->ni;
  if (!tc_path(P->path)) fail(EPSP_EINVAL, "internal: FP32 vertices on an FP64 path");
  set_mode_occupations(P, P->cur_T);
  const long nwp = P->nwp, M = 24 * nwp, N = 3 * ni;
  long px = prof_begin(ctx, "jmat");
  launch_jmat(P, J, 0, nullptr, 1, P->d_Jt.p, P->d_Jh.p, P->d_Jl.p);
  prof_end(ctx, px);
  const int sp = tc_gemm_launch_with(ctx, P->opA, P->opG, P->bn, P->splits, int(P->Mz), int(P->Nz), int(P->Kz), P->d_Z.p,
                                     P->Mz, P->Mz * P->Nz, P->d_err.p, "tc_ladder", P->persist, P->pair, P->gm);
  long pz = prof_begin(ctx, "zgather");
  launch_zgather(P->zg, N, 1, s, P->d_Z.p, P->Mz, sp, P->Mz * P->Nz, reinterpret_cast<const float4*>(P->d_ztab.p),
                 reinterpret_cast<const int2*>(P->d_zwin.p), P->d_nnu_f.p, nullptr, int(nw), int(nwp), int(P->nm),
                 P->d_Dz.p, M);
  EPSP_LAUNCHED(ctx);
  prof_end(ctx, pz);
  long pl = prof_begin(ctx, "lsum");
  y_split_kernel<<<dim3(div_up(size_t(P->Kp2), 256), unsigned(N), 1), 256, 0, s>>>(P->d_Dz.p, M, 1, 0, int(nw), int(nwp),
                                                                                  N, P->Kp2, P->d_Yh.p, P->d_Yl.p);
  EPSP_LAUNCHED(ctx);
  prof_end(ctx, pl);
  int sp2 = tc_gemm_launch(ctx, P->opKK, P->opY, int(nw), int(8 * N), int(nw), P->d_part2.p, nw, nw * 8 * N, 16, P->d_err.p,
                           "tc_ladder_kk");
  pl = prof_begin(ctx, "lfinish");
  finish_gemm_kernel<float><<<dim3(div_up(size_t(nw), 256), unsigned(6 * ni), 1), 256, 0, s>>>(
      P->d_Dz.p, M, 1, 0, P->d_part2.p, sp2, nw * 8 * N, P->d_Gmf.p, P->d_Gpf.p, nullptr, int(nw), int(nwp), int(ni), LJ,
      X);
  EPSP_LAUNCHED(ctx);
  prof_end(ctx, pl);
}

static void check_tc_err(LadderPlan* P) {
  if (!tc_path(P->path)) return;
  int e = 0;
  P->d_err.download(&e, 1, P->ctx->stream);
  EPSP_CUDA(cudaStreamSynchronize(P->ctx->stream));
  if (e) {
    P->d_err.zero(P->ctx->stream);  // cleared, so that the plan's next call starts clean
    fail(EPSP_EDEVICE_TIMEOUT, "a tensor-core GEMM wait ran out (bounded device wait)");
  }
}

// ---------------------------------------------------------------------------------------------
// solves (src/ladder.jl:327-375)
// ---------------------------------------------------------------------------------------------

template <class V>
static void dot_dev(LadderPlan* P, const V* u, const V* v, long n, DBuf<double2>& part, double2* out_dev) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  dot_partial_kernel<V><<<dim3(kDotBlocks, 1), 256, 0, s>>>(u, v, n, nullptr, part.p);
  EPSP_LAUNCHED(ctx);
  dot_final_kernel<<<1, 256, 0, s>>>(part.p, kDotBlocks, nullptr, out_dev);
  EPSP_LAUNCHED(ctx);
}

// conductivity_from_vertex (src/ladder_kernel.jl:116-122), in two halves: the device sums Y[b, i] of
// a vertex into Ydev (cond_launch, asynchronous), and σ from Y on the host (sigma_from_Y).
template <class V>
static void cond_launch(LadderPlan* P, const V* J, double2* Ydev) {
  Ctx* ctx = P->ctx;
  cond_sum_kernel<V><<<dim3(unsigned(3 * P->ni), 1), 256, 0, ctx->stream>>>(J, P->d_Ww.p, int(P->nw), int(P->ni), Ydev);
  EPSP_LAUNCHED(ctx);
}

static void sigma_from_Y(LadderPlan* P, const cplx* Y, double Om, double T, double* sigma) {
  const long ni = P->ni;
  cplx F = Om == 0 ? cplx(0, 1) / (4 * T)
                   : -1.0 / (cplx(0, 2) * Om * (1 + 2 * (T > 1.4901161193847656e-08 ? 1.0 / std::expm1(Om / T) : 0.0)));
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      cplx S = 0;
      for (long i = 0; i < ni; ++i) S += (P->v_h[size_t(a + 3 * i)] * P->w_i_h[size_t(i)]) * Y[size_t(b + 3 * i)];
      sigma[a + 3 * b] = (F / (2 * 3.14159265358979323846 * cplx(0, 1)) * S).real();
    }
}

// Both halves with a synchronisation in between.
template <class V>
static void conductivity_dev(LadderPlan* P, const V* J, double Om, double T, DBuf<double2>& Ybuf, double* sigma) {
  cudaStream_t s = P->ctx->stream;
  cond_launch(P, J, Ybuf.p);
  std::vector<cplx> Y(size_t(3 * P->ni));
  EPSP_CUDA(cudaMemcpyAsync(Y.data(), Ybuf.p, Y.size() * sizeof(cplx), cudaMemcpyDeviceToHost, s));
  EPSP_CUDA(cudaStreamSynchronize(s));
  sigma_from_Y(P, Y.data(), Om, T, sigma);
}

// c[0] = 1/sqrt(Re x[0]) (the scale of the first Krylov vector, without a round trip to the host).
__global__ void rsqrt_coef_kernel(const double2* __restrict__ x, double2* __restrict__ c) {
  if (threadIdx.x == 0 && blockIdx.x == 0) c[0] = make_double2(1.0 / sqrt(x[0].x), 0.0);
}

// A device vertex copied into host FP64 memory (FP32 vertices widened on the way).
static void vertex_to_host(LadderPlan* P, const double2* J, long n, double* out) {
  EPSP_CUDA(cudaMemcpyAsync(out, J, size_t(n) * sizeof(double2), cudaMemcpyDeviceToHost, P->ctx->stream));
  EPSP_CUDA(cudaStreamSynchronize(P->ctx->stream));
}
static void vertex_to_host(LadderPlan* P, const float2* J, long n, double* out) {
  std::vector<float2> h(static_cast<size_t>(n));
  EPSP_CUDA(cudaMemcpyAsync(h.data(), J, size_t(n) * sizeof(float2), cudaMemcpyDeviceToHost, P->ctx->stream));
  EPSP_CUDA(cudaStreamSynchronize(P->ctx->stream));
  for (long k = 0; k < n; ++k) {
    out[2 * k] = double(h[size_t(k)].x);
    out[2 * k + 1] = double(h[size_t(k)].y);
  }
}

static double mat3_norm(const double* a) {
  double s = 0;
  for (int k = 0; k < 9; ++k) s += a[k] * a[k];
  return std::sqrt(s);
}

// The solves of ladder_run with vertex vectors of element type V (double2 on the FP64 paths, float2
// on the tensor-core path).
template <class V>
static void ladder_run_t(LadderPlan* P, const double* sigma, const double* mu, const double* Tlist, int64_t nT,
                         const double* Omegas, int64_t nO, int32_t solver, double rtol, int32_t maxiter, double* sb,
                         double* sl, uint8_t* conv, int32_t* niter, epsp_ladder_history* hist, double* J_out,
                         DBuf<V>& J0, DBuf<V>& J, DBuf<V>& LJ, DBuf<V>& W, std::vector<DBuf<V>>& Vb) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  if (solver != EPSP_SOLVER_GMRES && solver != EPSP_SOLVER_FIXED_POINT) fail(EPSP_EINVAL, "solver must be :gmres or :fixed_point");
  if (maxiter < 1) fail(EPSP_EINVAL, "maxiter must be at least 1, got " + std::to_string(maxiter));
  if (nO < 1) fail(EPSP_EINVAL, "Omegas must hold at least one probe frequency");
  if (nT < 1 || !sigma || !mu || !Tlist || !Omegas || !sb || !sl || !conv || !niter) fail(EPSP_EINVAL, "an input or output array is NULL");
  for (int64_t iT = 0; iT < nT; ++iT)
    if (!(Tlist[iT] >= 0)) fail(EPSP_EINVAL, "Temperature must be positive");
  const long nw = P->nw, ni = P->ni;
  const long n = nw * 24 * ni;
  const unsigned eb = div_up(size_t(n), 256);
  DBuf<double2>& part = P->w_part;
  DBuf<double2>& Hdev = P->w_H;
  DBuf<double2>& Ybuf = P->w_Y;
  for (auto* b : {&J0, &J, &LJ, &W}) ensure(*b, ctx, size_t(n));
  ensure(part, ctx, size_t(std::max<long>(kMG * kDotBlocks, ni)));  // block partials of up to kMG dot products
  ensure(Hdev, ctx, size_t(maxiter + 5));  // (unused), ‖J0‖², β², 1/β
  ensure(Ybuf, ctx, size_t(3 * ni * (maxiter + 2)));  // σ sums of J0, x0 and each Krylov vector
  std::vector<DBuf<V>>& Vk = Vb;
  const double btol = std::pow(std::numeric_limits<double>::epsilon(), 0.75);
  {
    const size_t m1 = size_t(maxiter + 1);
    for (auto* b : {&P->g_h1, &P->g_h2, &P->g_z}) ensure(*b, ctx, m1);
    for (auto* b : {&P->g_hsq, &P->g_inv}) ensure(*b, ctx, 1);
    ensure(P->g_R, ctx, m1 * m1 / 2 + m1);
    ensure(P->g_sn, ctx, m1);
    ensure(P->g_cs, ctx, m1);
    ensure(P->g_st, ctx, 1);
    if (ensure(P->g_vp, ctx, m1)) {  // a new pointer table: the kept Krylov vectors' pointers again
      std::vector<void*> ptrs(m1, nullptr);
      for (size_t k = 0; k < std::min(Vk.size(), m1); ++k) ptrs[k] = Vk[k].p;
      P->g_vp.upload(ptrs.data(), m1, s);
      EPSP_CUDA(cudaStreamSynchronize(s));
    }
  }
  for (int64_t iT = 0; iT < nT; ++iT) {
    const double T = Tlist[iT];
    long pu = prof_begin(ctx, "ladder_io");
    // Σ_T from host or device memory (unified addressing: e.g. the scGD0 plan's own Σ)
    EPSP_CUDA(cudaMemcpyAsync(P->d_ST.p, reinterpret_cast<const double2*>(sigma) + size_t(nw * ni * iT),
                              size_t(nw * ni) * sizeof(double2), cudaMemcpyDefault, s));
    prof_end(ctx, pu);
    for (int64_t iO = 0; iO < nO; ++iO) {
      const double Om = Omegas[iO];
      const int64_t idx = iO + nO * iT;
      long plp = prof_begin(ctx, "lprep");
      const size_t hN0 = size_t(maxiter + 2), hB2 = size_t(maxiter + 3), hC = size_t(maxiter + 4);
      if constexpr (std::is_same_v<V, float2>) {
        // propagators, J0, its σ sums (slot 0) and ‖J0‖² in one pass
        set_propagators(P, mu[iT], T, Om, false);
        prep_vertex_f32_kernel<<<unsigned(ni), 256, 0, s>>>(P->d_ST.p, P->d_ws.p, int(nw), P->d_jm.p, P->d_tm.p, P->d_jp.p,
                                                            P->d_tp.p, P->d_eps_i.p, mu[iT], T, Om, P->d_v.p, P->d_Ww.p,
                                                            int(ni), P->d_Gmf.p, P->d_Gpf.p, J0.p, Ybuf.p, part.p);
        EPSP_LAUNCHED(ctx);
        dot_final_kernel<<<1, 256, 0, s>>>(part.p, int(ni), nullptr, Hdev.p + hN0);
        EPSP_LAUNCHED(ctx);
      } else {
        set_propagators(P, mu[iT], T, Om);
        const dim3 ab(div_up(size_t(nw), 256), unsigned(6 * ni), 4);
        attach_bare_kernel<double2><<<ab, 256, 0, s>>>(P->d_Gm.p, P->d_Gp.p, P->d_v.p, int(nw), int(ni), J0.p);
        EPSP_LAUNCHED(ctx);
      }
      auto op = [&](const V* x, V* y) {  // y = x - L(x)
        if (P->path == EPSP_PATH_DIRECT_FP64) {
          apply_L(P, x, LJ.p);
          sub_kernel<V><<<eb, 256, 0, s>>>(x, LJ.p, y, n, nullptr);
          EPSP_LAUNCHED(ctx);
        } else {
          apply_L(P, x, y, x);  // the last pass of the operator forms x - L(x)
        }
      };
      if (solver == EPSP_SOLVER_GMRES) {
        // Krylov.gmres(A, b[, x0]; atol = rtol ‖J0‖, rtol = 0, itmax = maxiter), restart = false,
        // Givens (src/ladder.jl:340-353), the Arnoldi step on the device: classical Gram-Schmidt with
        // one reorthogonalisation (CGS2; one pass while the basis holds one vector, where it is the
        // MGS step) in multi-vector passes, and the Givens update, the residual and the stopping test
        // in FP64 by gmres_givens_kernel. The host reads a small status once per iteration: the
        // first operator application starts before ‖J0‖ and β are known (the first Krylov vector
        // is scaled on the device), and they come back with the first status. σ of the
        // solution is Σ y_i σ(v_i) (+ σ(x0)) from the per-vector sums, unless the vertex itself is
        // wanted (stored, or the next Ω's start), when x is formed and summed.
        const bool warm = iO > 0;
        const bool needJ = J_out != nullptr || iO + 1 < nO;
        const long ny = 3 * ni;
        if constexpr (!std::is_same_v<V, float2>) {
          cond_launch(P, J0.p, Ybuf.p);  // slot 0: σ_bubble
          dot_dev(P, J0.p, J0.p, n, part, Hdev.p + hN0);
        }
        const V* r0 = J0.p;  // a cold start's r0 is J0 itself
        if (warm) {          // r0 = b - A x0
          if (!needJ) cond_launch(P, J.p, Ybuf.p + ny);  // slot 1: σ(x0)
          op(J.p, W.p);
          axpby_kernel<V><<<eb, 256, 0, s>>>(make_double2(1, 0), nullptr, J0.p, make_double2(-1, 0), nullptr, W.p, n, nullptr);
          EPSP_LAUNCHED(ctx);
          dot_dev(P, W.p, W.p, n, part, Hdev.p + hB2);
          r0 = W.p;
        }
        rsqrt_coef_kernel<<<1, 32, 0, s>>>(Hdev.p + (warm ? hB2 : hN0), Hdev.p + hC);
        EPSP_LAUNCHED(ctx);
        // the Krylov vectors and their pointers on the device (allocated as the basis grows, kept)
        auto vec = [&](int k) -> V* {
          if (Vk.size() < size_t(k + 1)) Vk.resize(size_t(k + 1));
          if (Vk[size_t(k)].n != size_t(n)) {
            Vk[size_t(k)].alloc(ctx, size_t(n));
            void* pv = Vk[size_t(k)].p;
            EPSP_CUDA(cudaMemcpyAsync(P->g_vp.p + k, &pv, sizeof(void*), cudaMemcpyHostToDevice, s));
            EPSP_CUDA(cudaStreamSynchronize(s));  // the pointer's host copy is a local
          }
          return Vk[size_t(k)].p;
        };
        scale_kernel<V><<<eb, 256, 0, s>>>(make_double2(0, 0), Hdev.p + hC, r0, vec(0), n, nullptr);
        EPSP_LAUNCHED(ctx);
        prof_end(ctx, plp);
        plp = -1;
        std::vector<double> res;
        bool solved = false, breakdown = false, tired = false;
        int inner = 0;
        std::vector<cplx> Yb(static_cast<size_t>(ny)), Yx0(static_cast<size_t>(ny), cplx(0, 0));
        std::vector<std::vector<cplx>> Yv;
        const bool tc = tc_path(P->path);
        V* const* vp = reinterpret_cast<V* const*>(P->g_vp.p);
        GmresDev gs{};
        int werr = 0;
        while (!(solved || tired || breakdown)) {
          ++inner;
          // a cold start's first Krylov vector is J0 times 1/β: its σ sums are J0's (slot 0) times
          // the same factor, formed on the host once β is read, instead of another pass
          const bool v_from_j0 = inner == 1 && !warm;
          op(Vk[size_t(inner - 1)].p, W.p);  // w = A v_k
          if (!needJ && !v_from_j0) cond_launch(P, Vk[size_t(inner - 1)].p, Ybuf.p + (2 + (inner - 1)) * ny);
          long pbl = prof_begin(ctx, "lblas");
          // CGS2: h1 = V^H w, w -= V h1; h2 = V^H w, w -= V h2 with ‖w‖^2; m <= kMG vectors per pass.
          // With one Krylov vector the second pass is left out (one projection: the MGS step itself).
          const int npass = inner >= 2 ? 2 : 1;
          for (int pass = 0; pass < npass; ++pass) {
            double2* hp = pass == 0 ? P->g_h1.p : P->g_h2.p;
            for (int i0 = 0; i0 < inner; i0 += kMG) {
              const int m = std::min(kMG, inner - i0);
              mdot_partial_kernel<V><<<kDotBlocks, 256, 0, s>>>(vp, i0, m, W.p, n, part.p);
              EPSP_LAUNCHED(ctx);
              dot_final_kernel<<<unsigned(m), 256, 0, s>>>(part.p, kDotBlocks, nullptr, hp + i0);
              EPSP_LAUNCHED(ctx);
            }
            for (int i0 = 0; i0 < inner; i0 += kMG) {
              const int m = std::min(kMG, inner - i0);
              const bool last = pass == npass - 1 && i0 + m >= inner;
              maxpy_kernel<V><<<kDotBlocks, 256, 0, s>>>(W.p, vp, i0, m, hp, n, last ? part.p : nullptr);
              EPSP_LAUNCHED(ctx);
            }
          }
          dot_final_kernel<<<1, 256, 0, s>>>(part.p, kDotBlocks, nullptr, P->g_hsq.p);
          EPSP_LAUNCHED(ctx);
          gmres_givens_kernel<<<1, 32, 0, s>>>(P->g_h1.p, npass == 2 ? P->g_h2.p : nullptr, P->g_hsq.p, Hdev.p + hN0,
                                               Hdev.p + (warm ? hB2 : hN0), rtol, btol, inner, P->g_R.p, P->g_cs.p,
                                               P->g_sn.p, P->g_z.p, P->g_st.p, P->g_inv.p);
          EPSP_LAUNCHED(ctx);
          P->g_st.download(&gs, 1, s);
          if (tc) P->d_err.download(&werr, 1, s);
          if (inner == 1) {
            EPSP_CUDA(cudaMemcpyAsync(Yb.data(), Ybuf.p, size_t(ny) * sizeof(cplx), cudaMemcpyDeviceToHost, s));
            if (warm && !needJ)
              EPSP_CUDA(cudaMemcpyAsync(Yx0.data(), Ybuf.p + ny, size_t(ny) * sizeof(cplx), cudaMemcpyDeviceToHost, s));
          }
          if (!needJ) {
            Yv.emplace_back(static_cast<size_t>(ny));
            if (!v_from_j0)
              EPSP_CUDA(cudaMemcpyAsync(Yv.back().data(), Ybuf.p + (2 + (inner - 1)) * ny, size_t(ny) * sizeof(cplx),
                                        cudaMemcpyDeviceToHost, s));
          }
          prof_end(ctx, pbl);
          EPSP_CUDA(cudaStreamSynchronize(s));
          if (werr) {
            P->d_err.zero(s);
            fail(EPSP_EDEVICE_TIMEOUT, "a tensor-core GEMM wait ran out (bounded device wait)");
          }
          if (inner == 1) {
            res.push_back(gs.beta);
            if (gs.solved_x0) {  // solved at x0: the speculative first step is dropped
              solved = true;
              inner = 0;
              Yv.clear();
              break;
            }
          }
          if (v_from_j0 && !needJ) {  // the factor the device scaled J0 by (rsqrt_coef, in R precision)
            const double c1 = 1.0 / gs.nJ0;
            const double cr = tc ? double(float(c1)) : c1;
            for (long k = 0; k < ny; ++k) Yv[0][size_t(k)] = Yb[size_t(k)] * cr;
          }
          res.push_back(gs.rnorm);
          solved = gs.solved != 0;
          breakdown = gs.breakdown != 0;
          tired = inner >= maxiter;
          if (!(solved || tired || breakdown)) {  // the next Krylov vector w / H[k + 1, k]
            scale_kernel<V><<<eb, 256, 0, s>>>(make_double2(0, 0), P->g_inv.p, W.p, vec(inner), n, nullptr);
            EPSP_LAUNCHED(ctx);
          }
        }
        // y = R \ z (the least-squares solution of Krylov.gmres, FP64, on the host)
        std::vector<cplx> y(static_cast<size_t>(inner)), Rh(static_cast<size_t>(inner * (inner + 1) / 2));
        if (inner > 0) {
          EPSP_CUDA(cudaMemcpyAsync(Rh.data(), P->g_R.p, Rh.size() * sizeof(cplx), cudaMemcpyDeviceToHost, s));
          EPSP_CUDA(cudaMemcpyAsync(y.data(), P->g_z.p, y.size() * sizeof(cplx), cudaMemcpyDeviceToHost, s));
          EPSP_CUDA(cudaStreamSynchronize(s));
        }
        {
          const int nr = inner * (inner + 1) / 2;
          for (int i = inner - 1; i >= 0; --i) {
            int pos = nr + i - inner;
            for (int jj = inner - 1; jj >= i + 1; --jj) {
              y[size_t(i)] -= Rh[size_t(pos)] * y[size_t(jj)];
              pos -= jj;
            }
            if (std::abs(Rh[size_t(pos)]) <= btol)
              y[size_t(i)] = 0;
            else
              y[size_t(i)] /= Rh[size_t(pos)];
          }
        }
        sigma_from_Y(P, Yb.data(), Om, T, sb + 9 * idx);
        if (needJ) {
          // x = x0 + V y (x0 = J for a warm start, else 0)
          long psl = prof_begin(ctx, "lsol");
          if (inner == 0 && !warm) J.zero(s);
          for (int i = 0; i < inner; ++i) {
            const double2 yi = make_double2(y[size_t(i)].real(), y[size_t(i)].imag());
            if (i == 0 && !warm)
              scale_kernel<V><<<eb, 256, 0, s>>>(yi, nullptr, Vk[0].p, J.p, n, nullptr);
            else
              axpby_kernel<V><<<eb, 256, 0, s>>>(yi, nullptr, Vk[size_t(i)].p, make_double2(1, 0), nullptr, J.p, n, nullptr);
            EPSP_LAUNCHED(ctx);
          }
          prof_end(ctx, psl);
          conductivity_dev(P, J.p, Om, T, Ybuf, sl + 9 * idx);
          if (J_out) vertex_to_host(P, J.p, n, J_out + 2 * size_t(n) * size_t(idx));
        } else {
          std::vector<cplx> Yx = Yx0;  // σ is linear in the vertex
          for (int i = 0; i < inner; ++i)
            for (long k = 0; k < ny; ++k) Yx[size_t(k)] += y[size_t(i)] * Yv[size_t(i)][size_t(k)];
          sigma_from_Y(P, Yx.data(), Om, T, sl + 9 * idx);
        }
        conv[idx] = solved ? 1 : 0;
        niter[idx] = inner;
        if (hist && hist->norms && hist->nnorms) {
          int32_t nn = int32_t(std::min<size_t>(res.size(), size_t(maxiter + 1)));
          for (int32_t k = 0; k < nn; ++k) hist->norms[size_t(maxiter + 1) * size_t(idx) + size_t(k)] = res[size_t(k)];
          hist->nnorms[idx] = nn;
        }
        if (hist && hist->nsigma) hist->nsigma[idx] = 0;
      } else {
        // J ← J0 + L(J) from J0 until the relative change of σ is below rtol (src/ladder.jl:354-369)
        prof_end(ctx, plp);
        plp = -1;
        conductivity_dev(P, J0.p, Om, T, Ybuf, sb + 9 * idx);
        EPSP_CUDA(cudaMemcpyAsync(J.p, J0.p, size_t(n) * sizeof(V), cudaMemcpyDeviceToDevice, s));
        double sprev[9] = {}, scur[9];
        conv[idx] = 0;
        int32_t ns_ = 0;
        for (int32_t it = 1; it <= maxiter; ++it) {
          apply_L(P, J.p, LJ.p);
          add_kernel<V><<<eb, 256, 0, s>>>(J0.p, LJ.p, J.p, n);
          EPSP_LAUNCHED(ctx);
          check_tc_err(P);
          conductivity_dev(P, J.p, Om, T, Ybuf, scur);
          if (hist && hist->sigma_iter)
            for (int k = 0; k < 9; ++k) hist->sigma_iter[9 * (size_t(maxiter) * size_t(idx) + size_t(it - 1)) + size_t(k)] = scur[k];
          ns_ = it;
          niter[idx] = it;
          if (it > 1) {
            double d[9];
            for (int k = 0; k < 9; ++k) d[k] = scur[k] - sprev[k];
            if (mat3_norm(d) < rtol * mat3_norm(scur)) {
              conv[idx] = 1;
              break;
            }
          }
          std::copy(scur, scur + 9, sprev);
        }
        if (hist && hist->nsigma) hist->nsigma[idx] = ns_;
        if (hist && hist->nnorms) hist->nnorms[idx] = 0;
        conductivity_dev(P, J.p, Om, T, Ybuf, sl + 9 * idx);
        if (J_out) vertex_to_host(P, J.p, n, J_out + 2 * size_t(n) * size_t(idx));
      }
    }
  }
}

void ladder_run(LadderPlan* P, const double* sigma, const double* mu, const double* Tlist, int64_t nT, const double* Omegas,
                int64_t nO, int32_t solver, double rtol, int32_t maxiter, double* sb, double* sl, uint8_t* conv, int32_t* niter,
                epsp_ladder_history* hist, double* J_out) {
  if (tc_path(P->path))
    ladder_run_t<float2>(P, sigma, mu, Tlist, nT, Omegas, nO, solver, rtol, maxiter, sb, sl, conv, niter, hist, J_out,
                         P->w_J0f, P->w_Jf, P->w_LJf, P->w_Wf, P->w_Vf);
  else
    ladder_run_t<double2>(P, sigma, mu, Tlist, nT, Omegas, nO, solver, rtol, maxiter, sb, sl, conv, niter, hist, J_out,
                          P->w_J0, P->w_J, P->w_LJ, P->w_W, P->w_V);
}

// ---------------------------------------------------------------------------------------------
// (T, Ω) pairs as simultaneous right-hand sides (GEMM_BF16)
// ---------------------------------------------------------------------------------------------

struct PairParams {
  double mu, T, Om;
  int iT, pad;
};

// contour_greens! of every pair of the batch: slot z uses Σ of temperature pp[z].iT, its own
// interpolation tables [z][nω] and writes Gm, Gp + 4 nω ni z.
__global__ void propagators_batch_kernel(const double2* __restrict__ S_all, const double* __restrict__ ws, int nw,
                                         const int32_t* __restrict__ jm_all, const double* __restrict__ tm_all,
                                         const int32_t* __restrict__ jp_all, const double* __restrict__ tp_all,
                                         const double* __restrict__ eps_i, const PairParams* __restrict__ pp,
                                         float2* __restrict__ Gm_all, float2* __restrict__ Gp_all, int ni) {
  int w = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y;
  const long z = blockIdx.z;
  if (w >= nw) return;
  const PairParams q = pp[z];
  const double2* col = S_all + long(nw) * ni * q.iT + long(nw) * i;
  contour_g<true>(col, jm_all[z * nw + w], tm_all[z * nw + w], ws[w] - q.Om / 2, eps_i[i], q.mu, q.T,
                  Gm_all + z * 4l * nw * ni, w, nw, i);
  contour_g<true>(col, jp_all[z * nw + w], tp_all[z * nw + w], ws[w] + q.Om / 2, eps_i[i], q.mu, q.T,
                  Gp_all + z * 4l * nw * ni, w, nw, i);
}

// The batched BLAS-1 are the kernels above with blockIdx.y over the slots and rmap.
constexpr int kDotBlocksB = 256;

// Buffers of a batch of right-hand sides (capacity cap), tensor maps over them.
struct LadderBatch {
  long cap = 0;
  int bk = 0;  // K block of the Jr maps
  DBuf<__nv_bfloat16> Jh, Jl, Yh, Yl;
  DBuf<float> Jt;  // GEMM_TF32: Jr as TF32-rounded FP32
  DBuf<float> Z, D, part2, nnu;
  DBuf<float2> Gm, Gp, J0, J, LJ, W;
  DBuf<double2> dpart, H, coef_a, coef_b;
  std::vector<DBuf<float2>> V;
  DBuf<int32_t> jm, jp;
  DBuf<double> tm, tp;
  DBuf<PairParams> pp;
  DBuf<int> rmap;
  DBuf<double2> Y;
  TcOperand opA{}, opY{};
};

static void batch_reserve(LadderPlan* P, LadderBatch& B, long R, int maxiter) {
  Ctx* ctx = P->ctx;
  const long nw = P->nw, ni = P->ni, nwp = P->nwp, M = 24 * nwp, N = 3 * ni, n = nw * 24 * ni;
  B.cap = R;
  const bool tf = P->path == EPSP_PATH_GEMM_TF32;
  if (tf) {
    B.Jt.alloc(ctx, size_t(R * P->Mz * P->Kzp));
  } else {
    B.Jh.alloc(ctx, size_t(R * P->Mz * P->Kzp));
    B.Jl.alloc(ctx, size_t(R * P->Mz * P->Kzp));
  }
  B.Yh.alloc(ctx, size_t(R * 8 * N * P->Kp2));
  B.Yl.alloc(ctx, size_t(R * 8 * N * P->Kp2));
  size_t p2 = 0;
  for (long a = 1; a <= R; ++a) {
    int bn, sp2;
    tc_gemm_shape(ctx, int(nw), int(a * 8 * N), int(nw), 16, 2, &bn, &sp2);
    p2 = std::max(p2, size_t(sp2) * size_t(a * nw * 8 * N));
  }
  B.Z.alloc(ctx, size_t(R * P->Mz) * size_t(P->Nz));  // one split: the stacked product has tiles for every SM
  B.D.alloc(ctx, size_t(R * M * N));
  B.part2.alloc(ctx, p2);
  B.nnu.alloc(ctx, size_t(16 * R));
  B.Gm.alloc(ctx, size_t(R * 4 * nw * ni));
  B.Gp.alloc(ctx, size_t(R * 4 * nw * ni));
  for (auto* b : {&B.J0, &B.J, &B.LJ, &B.W}) b->alloc(ctx, size_t(R * n));
  B.dpart.alloc(ctx, size_t(R * kDotBlocksB));
  B.H.alloc(ctx, size_t(R * (maxiter + 2)));
  B.coef_a.alloc(ctx, size_t(R));
  B.coef_b.alloc(ctx, size_t(R));
  B.jm.alloc(ctx, size_t(R * nw));
  B.jp.alloc(ctx, size_t(R * nw));
  B.tm.alloc(ctx, size_t(R * nw));
  B.tp.alloc(ctx, size_t(R * nw));
  B.pp.alloc(ctx, size_t(R));
  B.rmap.alloc(ctx, size_t(R));
  B.Y.alloc(ctx, size_t(R * 3 * ni));
  B.opA = tf ? one_part_tf32(B.Jt.p, R * P->Mz, P->Kz, P->Kzp, kTcBM, P->bk)
             : two_part(B.Jh.p, B.Jl.p, R * P->Mz, P->Kz, P->Kzp, kTcBM, P->bk);
  B.bk = P->bk;
  B.opY = two_part(B.Yh.p, B.Yl.p, R * 8 * N, nw, P->Kp2, P->bn2);
}

// LJ[r] = L(X[r]) for the nA right-hand sides listed in the device array rmap (host copy rmap_h).
static void apply_L_batch(LadderPlan* P, LadderBatch& B, const float2* X, int nA, float2* LJ) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  const long nw = P->nw, ni = P->ni, nwp = P->nwp, M = 24 * nwp, N = 3 * ni, n = nw * 24 * ni;
  const long Mt = M * nA, Mzt = P->Mz * nA;
  long px = prof_begin(ctx, "jmat");
  launch_jmat(P, X, n, B.rmap.p, nA, B.Jt.p, B.Jh.p, B.Jl.p);
  prof_end(ctx, px);
  tc_gemm_launch_with(ctx, B.opA, P->opG, P->bn, 1, int(Mzt), int(P->Nz), int(P->Kz), B.Z.p, Mzt, Mzt * P->Nz,
                      P->d_err.p, "tc_ladder", P->persist, P->pair, P->gm);
  launch_zgather(P->zg, N, unsigned(nA), s, B.Z.p, Mzt, 1, long(0), reinterpret_cast<const float4*>(P->d_ztab.p),
                 reinterpret_cast<const int2*>(P->d_zwin.p), B.nnu.p, B.rmap.p, int(nw), int(nwp), int(P->nm), B.D.p, Mt);
  EPSP_LAUNCHED(ctx);
  y_split_kernel<<<dim3(div_up(size_t(P->Kp2), 256), unsigned(N), unsigned(nA)), 256, 0, s>>>(
      B.D.p, Mt, 1, 0, int(nw), int(nwp), N, P->Kp2, B.Yh.p, B.Yl.p);
  EPSP_LAUNCHED(ctx);
  const long N2 = 8 * N * nA;
  int sp2 = tc_gemm_launch(ctx, P->opKK, B.opY, int(nw), int(N2), int(nw), B.part2.p, nw, nw * N2, 16, P->d_err.p,
                           "tc_ladder_kk");
  finish_gemm_kernel<float><<<dim3(div_up(size_t(nw), 256), unsigned(6 * ni), unsigned(nA)), 256, 0, s>>>(
      B.D.p, Mt, 1, 0, B.part2.p, sp2, nw * N2, B.Gm.p, B.Gp.p, B.rmap.p, int(nw), int(nwp), int(ni), LJ);
  EPSP_LAUNCHED(ctx);
}

// σ of every pair of the batch from the vertices J[z] (conductivity_from_vertex).
static void conductivity_batch(LadderPlan* P, LadderBatch& B, const float2* J, int nP, const std::vector<PairParams>& pp,
                               double* sigma_base, const std::vector<long>& idx) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  const long nw = P->nw, ni = P->ni;
  cond_sum_kernel<float2><<<dim3(unsigned(3 * ni), unsigned(nP)), 256, 0, s>>>(J, P->d_Ww.p, int(nw), int(ni), B.Y.p);
  EPSP_LAUNCHED(ctx);
  std::vector<double2> Y(static_cast<size_t>(3 * ni * nP));
  B.Y.download(Y.data(), Y.size(), s);
  EPSP_CUDA(cudaStreamSynchronize(s));
  for (int z = 0; z < nP; ++z) {
    const double T = pp[size_t(z)].T, Om = pp[size_t(z)].Om;
    cplx F = Om == 0 ? cplx(0, 1) / (4 * T)
                     : -1.0 / (cplx(0, 2) * Om * (1 + 2 * (T > 1.4901161193847656e-08 ? 1.0 / std::expm1(Om / T) : 0.0)));
    double* sig = sigma_base + 9 * idx[size_t(z)];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        cplx S = 0;
        for (long i = 0; i < ni; ++i) {
          const double2 y = Y[size_t(3 * ni * z + b + 3 * i)];
          S += (P->v_h[size_t(a + 3 * i)] * P->w_i_h[size_t(i)]) * cplx(y.x, y.y);
        }
        sig[a + 3 * b] = (F / (2 * 3.14159265358979323846 * cplx(0, 1)) * S).real();
      }
  }
}

// Host state of one right-hand side's GMRES (the recurrences of the sequential solver).
struct GmresState {
  double atol = 0, rNorm = 0;
  std::vector<double> res;
  std::vector<cplx> R, sv, z;
  std::vector<double> cv;
  int inner = 0, nr = 0;
  bool solved = false, tired = false, breakdown = false, active = false;
};

void ladder_run_batched(LadderPlan* P, const double* sigma, const double* mu, const double* Tlist, int64_t nT,
                        const double* Omegas, int64_t nO, double rtol, int32_t maxiter, int32_t max_rhs, double* sb,
                        double* sl, uint8_t* conv, int32_t* niter, epsp_ladder_history* hist, double* J_out) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  if (!tc_path(P->path))
    fail(EPSP_EUNSUPPORTED, "batched right-hand sides need a tensor-core ladder plan (GEMM_BF16 or GEMM_TF32)");
  if (maxiter < 1) fail(EPSP_EINVAL, "maxiter must be at least 1, got " + std::to_string(maxiter));
  if (max_rhs < 1) fail(EPSP_EINVAL, "max_rhs must be at least 1");
  if (nO < 1) fail(EPSP_EINVAL, "Omegas must hold at least one probe frequency");
  if (nT < 1 || !sigma || !mu || !Tlist || !Omegas || !sb || !sl || !conv || !niter) fail(EPSP_EINVAL, "an input or output array is NULL");
  for (int64_t iT = 0; iT < nT; ++iT)
    if (!(Tlist[iT] >= 0)) fail(EPSP_EINVAL, "Temperature must be positive");
  const long nw = P->nw, ni = P->ni, slab = nw * ni, n = nw * 24 * ni;
  const long nPairs = nT * nO;
  const long R = std::min<long>(max_rhs, nPairs);
  auto* Bp = static_cast<LadderBatch*>(P->w_batch.get());
  if (!Bp || Bp->cap < R || Bp->H.n < size_t(R * (maxiter + 2)) || Bp->bk != P->bk) {
    P->w_batch.reset();  // free the old buffers before the new ones are allocated
    auto nb = std::make_shared<LadderBatch>();
    batch_reserve(P, *nb, R, maxiter);
    P->w_batch = nb;
    Bp = nb.get();
  }
  LadderBatch& B = *Bp;
  DBuf<double2> S_all;
  S_all.alloc(ctx, size_t(slab * nT));
  EPSP_CUDA(cudaMemcpyAsync(S_all.p, sigma, size_t(slab * nT) * sizeof(double2), cudaMemcpyDefault, s));
  const double btol = std::pow(std::numeric_limits<double>::epsilon(), 0.75);
  const unsigned eb = div_up(size_t(n), 256);
  auto dot_batch = [&](const float2* U, const float2* V, int nA, double2* out) {
    dot_partial_kernel<float2><<<dim3(kDotBlocksB, unsigned(nA)), 256, 0, s>>>(U, V, n, B.rmap.p, B.dpart.p);
    EPSP_LAUNCHED(ctx);
    dot_final_kernel<<<unsigned(nA), 256, 0, s>>>(B.dpart.p, kDotBlocksB, B.rmap.p, out);
    EPSP_LAUNCHED(ctx);
  };
  auto set_rmap = [&](const std::vector<int>& rm) { B.rmap.upload(rm.data(), rm.size(), s); };
  for (long p0 = 0; p0 < nPairs; p0 += R) {
    const int nP = int(std::min<long>(R, nPairs - p0));
    std::vector<PairParams> pp(static_cast<size_t>(nP));
    std::vector<long> idx(static_cast<size_t>(nP));
    std::vector<int32_t> jm(static_cast<size_t>(nP * nw)), jp(static_cast<size_t>(nP * nw));
    std::vector<double> tm(static_cast<size_t>(nP * nw)), tp(static_cast<size_t>(nP * nw));
    std::vector<float> nnu(static_cast<size_t>(16 * nP), 0.f);
    for (int z = 0; z < nP; ++z) {
      const long pidx = p0 + z;  // = iO + nO iT
      const int iT = int(pidx / nO), iO = int(pidx % nO);
      const double T = Tlist[iT], Om = Omegas[iO];
      pp[size_t(z)] = PairParams{mu[iT], T, Om, iT, 0};
      idx[size_t(z)] = pidx;
      std::vector<double> xm(static_cast<size_t>(nw)), xp(static_cast<size_t>(nw)), t1, t2;
      std::vector<int32_t> j1, j2;
      for (long k = 0; k < nw; ++k) {
        xm[size_t(k)] = P->ws.nodes[size_t(k)] - Om / 2;
        xp[size_t(k)] = P->ws.nodes[size_t(k)] + Om / 2;
      }
      interp_table(P->ws.nodes, xm, j1, t1);
      interp_table(P->ws.nodes, xp, j2, t2);
      std::copy(j1.begin(), j1.end(), jm.begin() + z * nw);
      std::copy(j2.begin(), j2.end(), jp.begin() + z * nw);
      std::copy(t1.begin(), t1.end(), tm.begin() + z * nw);
      std::copy(t2.begin(), t2.end(), tp.begin() + z * nw);
      for (long nu = 0; nu < P->nm && nu < 16; ++nu) {
        const double w = P->wnu[size_t(nu)];
        nnu[size_t(16 * z + nu)] = float(w < P->w_ac ? 0.0
                                                     : (T > 1.4901161193847656e-08 ? (w == 0 ? -0.5 : 1.0 / std::expm1(w / T))
                                                                                   : (w > 0 ? 0.0 : -1.0)));
      }
    }
    B.jm.upload(jm.data(), jm.size(), s);
    B.jp.upload(jp.data(), jp.size(), s);
    B.tm.upload(tm.data(), tm.size(), s);
    B.tp.upload(tp.data(), tp.size(), s);
    B.nnu.upload(nnu.data(), nnu.size(), s);
    B.pp.upload(pp.data(), pp.size(), s);
    propagators_batch_kernel<<<dim3(div_up(size_t(nw), 128), unsigned(ni), unsigned(nP)), 128, 0, s>>>(
        S_all.p, P->d_ws.p, int(nw), B.jm.p, B.tm.p, B.jp.p, B.tp.p, P->d_eps_i.p, B.pp.p, B.Gm.p, B.Gp.p, int(ni));
    EPSP_LAUNCHED(ctx);
    attach_bare_kernel<float2><<<dim3(div_up(size_t(nw), 256), unsigned(6 * ni), unsigned(4 * nP)), 256, 0, s>>>(
        B.Gm.p, B.Gp.p, P->d_v.p, int(nw), int(ni), B.J0.p);
    EPSP_LAUNCHED(ctx);
    conductivity_batch(P, B, B.J0.p, nP, pp, sb, idx);
    // GMRES per right-hand side from x0 = 0: r0 = J0, ‖J0‖ gives atol and β
    std::vector<int> all(static_cast<size_t>(nP));
    for (int z = 0; z < nP; ++z) all[size_t(z)] = z;
    set_rmap(all);
    dot_batch(B.J0.p, B.J0.p, nP, B.H.p);
    std::vector<double2> h(static_cast<size_t>(nP));
    B.H.download(h.data(), size_t(nP), s);
    EPSP_CUDA(cudaStreamSynchronize(s));
    std::vector<GmresState> g(static_cast<size_t>(nP));
    std::vector<int> act;
    std::vector<double2> ca(static_cast<size_t>(nP)), cb(static_cast<size_t>(nP));
    for (int z = 0; z < nP; ++z) {
      GmresState& q = g[size_t(z)];
      const double beta = std::sqrt(h[size_t(z)].x);
      q.atol = rtol * beta;
      q.rNorm = beta;
      q.res.push_back(beta);
      q.solved = beta <= q.atol || beta == 0;
      if (!q.solved) {
        q.active = true;
        q.z.push_back(beta);
        act.push_back(z);
        ca[size_t(z)] = make_double2(1.0 / beta, 0);
      } else {
        ca[size_t(z)] = make_double2(0, 0);
      }
      cb[size_t(z)] = make_double2(0, 0);
    }
    if (B.V.empty()) B.V.emplace_back();
    if (B.V[0].n != size_t(R * n)) B.V[0].alloc(ctx, size_t(R * n));
    // V0 = J0 / β (every slot; solved ones get 0)
    B.coef_a.upload(ca.data(), ca.size(), s);
    scale_kernel<float2><<<dim3(eb, unsigned(nP)), 256, 0, s>>>(make_double2(0, 0), B.coef_a.p, B.J0.p, B.V[0].p, n, B.rmap.p);
    EPSP_LAUNCHED(ctx);
    int k = 0;
    while (!act.empty()) {
      ++k;
      const int nA = int(act.size());
      set_rmap(act);
      apply_L_batch(P, B, B.V[size_t(k - 1)].p, nA, B.LJ.p);  // LJ[r] = L(v_k)
      sub_kernel<float2><<<dim3(eb, unsigned(nA)), 256, 0, s>>>(B.V[size_t(k - 1)].p, B.LJ.p, B.W.p, n, B.rmap.p);
      EPSP_LAUNCHED(ctx);
      for (int i = 0; i < k; ++i) {
        dot_batch(B.V[size_t(i)].p, B.W.p, nA, B.H.p + long(i) * R);
        axpy_dev_kernel<float2><<<dim3(eb, unsigned(nA)), 256, 0, s>>>(B.W.p, B.V[size_t(i)].p, B.H.p + long(i) * R, n,
                                                                       B.rmap.p);
        EPSP_LAUNCHED(ctx);
      }
      dot_batch(B.W.p, B.W.p, nA, B.H.p + long(k) * R);
      std::vector<double2> hall(static_cast<size_t>((k + 1) * R));
      B.H.download(hall.data(), hall.size(), s);
      EPSP_CUDA(cudaStreamSynchronize(s));
      check_tc_err(P);
      std::vector<int> next;
      for (int z : act) {
        GmresState& q = g[size_t(z)];
        q.inner = k;
        for (int i = 0; i < k; ++i) q.R.push_back(cplx(hall[size_t(i * R + z)].x, hall[size_t(i * R + z)].y));
        const double Hbis = std::sqrt(hall[size_t(k * R + z)].x);
        for (int i = 0; i < k - 1; ++i) {
          cplx Rt = q.cv[size_t(i)] * q.R[size_t(q.nr + i)] + q.sv[size_t(i)] * q.R[size_t(q.nr + i + 1)];
          q.R[size_t(q.nr + i + 1)] = std::conj(q.sv[size_t(i)]) * q.R[size_t(q.nr + i)] - q.cv[size_t(i)] * q.R[size_t(q.nr + i + 1)];
          q.R[size_t(q.nr + i)] = Rt;
        }
        cplx a = q.R[size_t(q.nr + k - 1)];
        double abs_a = std::abs(a), cc;
        cplx ss, rho;
        if (Hbis == 0) {
          cc = 1;
          ss = 0;
          rho = a;
        } else if (abs_a == 0) {
          cc = 0;
          ss = 1;
          rho = Hbis;
        } else {
          double rr = std::hypot(abs_a, Hbis);
          cplx psi = a / abs_a;
          cc = abs_a / rr;
          ss = psi * (Hbis / rr);
          rho = psi * rr;
        }
        q.cv.push_back(cc);
        q.sv.push_back(ss);
        q.R[size_t(q.nr + k - 1)] = rho;
        cplx zeta = std::conj(ss) * q.z[size_t(k - 1)];
        q.z[size_t(k - 1)] = cc * q.z[size_t(k - 1)];
        q.rNorm = std::abs(zeta);
        q.res.push_back(q.rNorm);
        q.nr += k;
        q.solved = q.rNorm <= q.atol || q.rNorm + 1.0 <= 1.0;
        q.breakdown = Hbis <= btol;
        q.tired = k >= maxiter;
        if (!(q.solved || q.tired || q.breakdown)) {
          q.z.push_back(zeta);
          next.push_back(z);
          ca[size_t(z)] = make_double2(1.0 / Hbis, 0);
        } else {
          q.active = false;
        }
      }
      act = next;
      if (!act.empty()) {
        if (B.V.size() < size_t(k + 1)) B.V.emplace_back();
        if (B.V[size_t(k)].n != size_t(R * n)) B.V[size_t(k)].alloc(ctx, size_t(R * n));
        set_rmap(act);
        B.coef_a.upload(ca.data(), ca.size(), s);
        scale_kernel<float2><<<dim3(eb, unsigned(act.size())), 256, 0, s>>>(make_double2(0, 0), B.coef_a.p, B.W.p,
                                                                             B.V[size_t(k)].p, n, B.rmap.p);
        EPSP_LAUNCHED(ctx);
      }
    }
    // x = Σ_i y_i v_i per right-hand side (x0 = 0)
    B.J.zero(s);
    const int kmax = k;
    std::vector<std::vector<cplx>> ys(static_cast<size_t>(nP));
    for (int z = 0; z < nP; ++z) {
      GmresState& q = g[size_t(z)];
      std::vector<cplx> y = q.z;
      const int inner = q.inner;
      for (int i = inner - 1; i >= 0; --i) {
        int pos = q.nr + i - inner;
        for (int jj = inner - 1; jj >= i + 1; --jj) {
          y[size_t(i)] -= q.R[size_t(pos)] * y[size_t(jj)];
          pos -= jj;
        }
        if (std::abs(q.R[size_t(pos)]) <= btol)
          y[size_t(i)] = 0;
        else
          y[size_t(i)] /= q.R[size_t(pos)];
      }
      ys[size_t(z)] = y;
    }
    for (int i = 0; i < kmax; ++i) {
      std::vector<int> use;
      for (int z = 0; z < nP; ++z) {
        if (g[size_t(z)].inner > i) {
          use.push_back(z);
          ca[size_t(z)] = make_double2(ys[size_t(z)][size_t(i)].real(), ys[size_t(z)][size_t(i)].imag());
          cb[size_t(z)] = make_double2(1, 0);
        }
      }
      if (use.empty()) continue;
      set_rmap(use);
      B.coef_a.upload(ca.data(), ca.size(), s);
      B.coef_b.upload(cb.data(), cb.size(), s);
      axpby_kernel<float2><<<dim3(eb, unsigned(use.size())), 256, 0, s>>>(make_double2(0, 0), B.coef_a.p, B.V[size_t(i)].p,
                                                                           make_double2(0, 0), B.coef_b.p, B.J.p, n, B.rmap.p);
      EPSP_LAUNCHED(ctx);
    }
    conductivity_batch(P, B, B.J.p, nP, pp, sl, idx);
    for (int z = 0; z < nP; ++z) {
      const long pidx = idx[size_t(z)];
      const GmresState& q = g[size_t(z)];
      conv[pidx] = q.solved ? 1 : 0;
      niter[pidx] = q.inner;
      if (hist && hist->norms && hist->nnorms) {
        int32_t nn = int32_t(std::min<size_t>(q.res.size(), size_t(maxiter + 1)));
        for (int32_t kk = 0; kk < nn; ++kk) hist->norms[size_t(maxiter + 1) * size_t(pidx) + size_t(kk)] = q.res[size_t(kk)];
        hist->nnorms[pidx] = nn;
      }
      if (hist && hist->nsigma) hist->nsigma[pidx] = 0;
      if (J_out) vertex_to_host(P, B.J.p + size_t(n) * size_t(z), n, J_out + 2 * size_t(n) * size_t(pidx));
    }
    EPSP_CUDA(cudaStreamSynchronize(s));
  }
}

}  // namespace epsp

using namespace epsp;

template <class F>
static epsp_status lguard(Ctx* c, F&& f) {
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

epsp_status epsp_ladder_setup(epsp_ctx* ctx, const epsp_model* model, const epsp_options* opts, epsp_ladder_plan** plan) {
  if (!ctx || !plan) return EPSP_EINVAL;
  *plan = nullptr;
  return lguard(&ctx->c, [&] { *plan = reinterpret_cast<epsp_ladder_plan*>(ladder_setup(&ctx->c, model, opts)); });
}

void epsp_ladder_plan_destroy(epsp_ladder_plan* plan) {
  if (!plan) return;
  auto* P = reinterpret_cast<LadderPlan*>(plan);
  cudaSetDevice(P->ctx->device);
  delete P;
}

epsp_status epsp_ladder_run(epsp_ladder_plan* plan, const double* sigma, const double* mu, const double* Tlist, int64_t nT,
                            const double* Omegas, int64_t nOmega, int32_t solver, double rtol, int32_t maxiter,
                            double* sigma_bubble, double* sigma_ladder, uint8_t* converged, int32_t* niter,
                            epsp_ladder_history* hist, double* J_out) {
  if (!plan) return EPSP_EINVAL;
  auto* P = reinterpret_cast<LadderPlan*>(plan);
  return lguard(P->ctx, [&] {
    ladder_run(P, sigma, mu, Tlist, nT, Omegas, nOmega, solver, rtol, maxiter, sigma_bubble, sigma_ladder, converged, niter,
               hist, J_out);
  });
}

epsp_status epsp_ladder_run_batched(epsp_ladder_plan* plan, const double* sigma, const double* mu, const double* Tlist,
                                    int64_t nT, const double* Omegas, int64_t nOmega, double rtol, int32_t maxiter,
                                    int32_t max_rhs, double* sigma_bubble, double* sigma_ladder, uint8_t* converged,
                                    int32_t* niter, epsp_ladder_history* hist, double* J_out) {
  if (!plan) return EPSP_EINVAL;
  auto* P = reinterpret_cast<LadderPlan*>(plan);
  return lguard(P->ctx, [&] {
    ladder_run_batched(P, sigma, mu, Tlist, nT, Omegas, nOmega, rtol, maxiter, max_rhs, sigma_bubble, sigma_ladder,
                       converged, niter, hist, J_out);
  });
}

epsp_status epsp_ladder_set_gemm_config(epsp_ladder_plan* plan, int32_t bn, int32_t splits, int32_t bk) {
  if (!plan) return EPSP_EINVAL;
  auto* P = reinterpret_cast<LadderPlan*>(plan);
  return lguard(P->ctx, [&] {
    if (!tc_path(P->path)) fail(EPSP_EUNSUPPORTED, "tile shapes apply to tensor-core plans (GEMM_BF16, GEMM_TF32)");
    const bool tf = P->path == EPSP_PATH_GEMM_TF32;
    const bool ok = tf ? (bk == 32 && (bn == 128 || bn == 256))
                       : ((bk == 64 && (bn == 128 || bn == 256)) || (bk == 32 && bn == 256));
    if (!ok)
      fail(EPSP_EINVAL, tf ? "TF32 tile shape must be bn 128 or 256 with bk 32"
                           : "tile shape must be bn 128 or 256 with bk 64, or bn 256 with bk 32");
    const int max_sp = P->zsplit_cap;
    if (splits < 1 || splits > max_sp) fail(EPSP_EINVAL, "splits must be in [1, " + std::to_string(max_sp) + "]");
    P->bn = bn;
    P->splits = splits;
    P->bk = bk;
    pick_contraction_operands(P);
    if (!tf && !(bn == 256 && bk == 32)) P->persist = false;
    P->pair = false;
  });
}

epsp_status epsp_ladder_gemm_persistent(const epsp_ladder_plan* plan, int32_t* on) {
  if (!plan || !on) return EPSP_EINVAL;
  *on = reinterpret_cast<const LadderPlan*>(plan)->persist ? 1 : 0;
  return EPSP_OK;
}

epsp_status epsp_ladder_set_gemm_persistent(epsp_ladder_plan* plan, int32_t on) {
  if (!plan) return EPSP_EINVAL;
  auto* P = reinterpret_cast<LadderPlan*>(plan);
  return lguard(P->ctx, [&] {
    if (!tc_path(P->path)) fail(EPSP_EUNSUPPORTED, "tile shapes apply to tensor-core plans (GEMM_BF16, GEMM_TF32)");
    if (on && P->path == EPSP_PATH_GEMM_BF16 && !(P->bn == 256 && P->bk == 32))
      fail(EPSP_EINVAL, "the persistent BF16x3 kernel takes bn 256 with bk 32");
    P->persist = on != 0;  // with pair: the persistent CTA-pair kernel
  });
}

epsp_status epsp_ladder_gemm_pair(const epsp_ladder_plan* plan, int32_t* on) {
  if (!plan || !on) return EPSP_EINVAL;
  *on = reinterpret_cast<const LadderPlan*>(plan)->pair ? 1 : 0;
  return EPSP_OK;
}

epsp_status epsp_ladder_set_gemm_pair(epsp_ladder_plan* plan, int32_t on) {
  if (!plan) return EPSP_EINVAL;
  auto* P = reinterpret_cast<LadderPlan*>(plan);
  return lguard(P->ctx, [&] {
    if (!tc_path(P->path)) fail(EPSP_EUNSUPPORTED, "tile shapes apply to tensor-core plans (GEMM_BF16, GEMM_TF32)");
    if (on && (P->bn != 256 || P->bk != 32))
      fail(EPSP_EINVAL, "the CTA-pair kernels take bn 256 with bk 32");
    P->pair = on != 0;  // with persistent: the persistent CTA-pair kernel
  });
}

epsp_status epsp_ladder_gemm_config(const epsp_ladder_plan* plan, int32_t* bn, int32_t* splits, int32_t* bk,
                                    double* ms_chosen, double* ms_heuristic) {
  if (!plan || !bn || !splits) return EPSP_EINVAL;
  auto* P = reinterpret_cast<const LadderPlan*>(plan);
  *bn = P->bn;
  *splits = P->splits;
  if (bk) *bk = P->bk;
  double best = 0;
  for (const auto& c : P->tune_all)
    if (c.bn == P->bn && c.splits == P->splits && c.bk == P->bk && c.persist == P->persist && c.pair == P->pair &&
        c.gm == P->gm)
      best = c.ms;
  if (ms_chosen) *ms_chosen = best;
  if (ms_heuristic) *ms_heuristic = P->tune_ms_heuristic;
  return EPSP_OK;
}

epsp_status epsp_ladder_apply(epsp_ladder_plan* plan, const double* sigma_T, double mu, double T, double Omega, const double* J,
                              double* LJ) {
  if (!plan || !sigma_T || !J || !LJ) return EPSP_EINVAL;
  auto* P = reinterpret_cast<LadderPlan*>(plan);
  return lguard(P->ctx, [&] {
    if (!(T >= 0)) fail(EPSP_EINVAL, "Temperature must be positive");
    cudaStream_t s = P->ctx->stream;
    const long n = P->nw * 24 * P->ni;
    P->d_ST.upload(reinterpret_cast<const double2*>(sigma_T), size_t(P->nw * P->ni), s);
    set_propagators(P, mu, T, Omega);
    DBuf<double2> dJ, dLJ;
    dJ.alloc(P->ctx, size_t(n));
    dLJ.alloc(P->ctx, size_t(n));
    dJ.upload(reinterpret_cast<const double2*>(J), size_t(n), s);
    if (tc_path(P->path)) {  // FP32 vertices on the device
      DBuf<float2> fJ, fLJ;
      fJ.alloc(P->ctx, size_t(n));
      fLJ.alloc(P->ctx, size_t(n));
      to_f2_kernel<<<div_up(size_t(n), 256), 256, 0, s>>>(dJ.p, n, fJ.p);
      EPSP_LAUNCHED(P->ctx);
      apply_L(P, fJ.p, fLJ.p);
      to_d2_kernel<<<div_up(size_t(n), 256), 256, 0, s>>>(fLJ.p, n, dLJ.p);
      EPSP_LAUNCHED(P->ctx);
      dLJ.download(reinterpret_cast<double2*>(LJ), size_t(n), s);
      EPSP_CUDA(cudaStreamSynchronize(s));
    } else {
      apply_L(P, dJ.p, dLJ.p);
      dLJ.download(reinterpret_cast<double2*>(LJ), size_t(n), s);
      EPSP_CUDA(cudaStreamSynchronize(s));
    }
    check_tc_err(P);
  });
}

}  // extern "C"
