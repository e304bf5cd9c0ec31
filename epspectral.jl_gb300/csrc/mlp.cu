// mlp.cu -- the learned warm start: a small multilayer perceptron, its training and its inference,
// on the GPU with hand-written kernels.
//
// Network: L fully connected layers d_0 -> d_1 -> ... -> d_L, SiLU between layers, linear output.
// Weights W_l [d_{l+1}][d_l] (row-major) are kept in FP32 (the optimiser's master copy) and used in
// BF16 by the forward and backward products (BF16 weights, FP32 accumulation); biases FP32. The
// loss is the mean squared error over the batch and the outputs; the optimiser is Adam. The products
// are register-tiled SIMT GEMMs over arbitrary strides (the network is ~1e6 parameters: a training
// epoch over the warm-start set is tens of milliseconds), every reduction in fixed order, so a
// training run is bitwise reproducible.
#include "common.cuh"
#include "tc_gemm.cuh"
#include "warmstart.cuh"

#include <cuda_bf16.h>

#include <cmath>
#include <memory>

namespace epsp {

// C[m, n] = Σ_k A(m, k) B(k, n), with A(m, k) = A[m sam + k sak], B(k, n) = B[k sbk + n sbn],
// C[m scm + n scn]; 64x64 tiles, 256 threads with 4x4 outputs each, k in order. With gridDim.z > 1
// slice z sums k in [z kc, (z + 1) kc) and writes C + z M N (row-major partials, summed in order by
// partial_sum_kernel).
template <class TA, class TB>
__global__ void __launch_bounds__(256) mlp_gemm_kernel(int M, int N, int K, int kc, const TA* __restrict__ A, long sam,
                                                       long sak, const TB* __restrict__ B, long sbk, long sbn,
                                                       float* __restrict__ C, long scm, long scn) {
  __shared__ float As[16][64 + 1];
  __shared__ float Bs[16][64 + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  const int kb = blockIdx.z * kc, ke = min(K, kb + kc);
  if (gridDim.z > 1) C += long(blockIdx.z) * M * N;
  float acc[4][4] = {};
  for (int k0 = kb; k0 < ke; k0 += 16) {
    // consecutive threads walk the operand's unit-stride index (k when that stride is 1)
    for (int r = threadIdx.x; r < 1024; r += 256) {
      int kk = r / 64, mm = r % 64;
      if (sak == 1) kk = r % 16, mm = r / 16;
      const int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < ke) ? float(A[long(gm) * sam + long(gk) * sak]) : 0.f;
      kk = r / 64, mm = r % 64;
      if (sbk == 1) kk = r % 16, mm = r / 16;
      const int gn = n0 + mm, gk2 = k0 + kk;
      Bs[kk][mm] = (gn < N && gk2 < ke) ? float(B[long(gk2) * sbk + long(gn) * sbn]) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][tx + 16 * u];
        b[u] = Bs[kk][ty + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int gm = m0 + tx + 16 * u, gn = n0 + ty + 16 * v;
      if (gm < M && gn < N) {
        if (gridDim.z > 1)
          C[long(gm) * N + gn] = acc[u][v];
        else
          C[long(gm) * scm + long(gn) * scn] = acc[u][v];
      }
    }
}

// C[m scm + n scn] = Σ_z P[z][m][n], z ascending.
__global__ void partial_sum_kernel(const float* __restrict__ P, int M, int N, int nz, float* __restrict__ C, long scm,
                                   long scn) {
  const long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= long(M) * N) return;
  float acc = 0.f;
  for (int z = 0; z < nz; ++z) acc += P[long(z) * M * N + k];
  C[(k / N) * scm + (k % N) * scn] = acc;
}

// Slices of K for a product of few output tiles, so that the grid covers the GPU twice.
static int gemm_splits(const Ctx* ctx, int M, int N, int K) {
  const int tiles = int(div_up(size_t(M), 64) * div_up(size_t(N), 64));
  const int want = std::max(1, 2 * ctx->sm_count / tiles);
  return std::max(1, std::min(want, K / 128));
}

template <class TA, class TB>
static void mlp_gemm(Ctx* ctx, float* work, int M, int N, int K, const TA* A, long sam, long sak, const TB* B, long sbk,
                     long sbn, float* C, long scm, long scn) {
  const int sp = gemm_splits(ctx, M, N, K);
  const int kc = int(div_up(div_up(size_t(K), size_t(sp)), 16) * 16);
  const int nz = int(div_up(size_t(K), size_t(kc)));
  dim3 grid(div_up(size_t(M), 64), div_up(size_t(N), 64), unsigned(nz));
  mlp_gemm_kernel<TA, TB><<<grid, 256, 0, ctx->stream>>>(M, N, K, kc, A, sam, sak, B, sbk, sbn, nz > 1 ? work : C, scm,
                                                         scn);
  EPSP_LAUNCHED(ctx);
  if (nz > 1) {
    partial_sum_kernel<<<div_up(size_t(M) * N, 256), 256, 0, ctx->stream>>>(work, M, N, nz, C, scm, scn);
    EPSP_LAUNCHED(ctx);
  }
}

__device__ __forceinline__ float sigmoidf_(float x) { return 1.f / (1.f + expf(-x)); }

// Z += b (row-major [n][d]); X = SiLU(Z) if act, else X = Z.
__global__ void bias_act_kernel(float* __restrict__ Z, const float* __restrict__ b, long n, int d, bool act,
                                float* __restrict__ X) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n * d) return;
  float z = Z[k] + b[k % d];
  Z[k] = z;
  X[k] = act ? z * sigmoidf_(z) : z;
}

// dZ = dX * SiLU'(Z).
__global__ void act_back_kernel(const float* __restrict__ dX, const float* __restrict__ Z, long n, float* __restrict__ dZ) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float z = Z[k], s = sigmoidf_(z);
  dZ[k] = dX[k] * (s * (1.f + z * (1.f - s)));
}

// db[j] = Σ_m dZ[m][j] in ascending m.
__global__ void bias_grad_kernel(const float* __restrict__ dZ, long n, int d, float* __restrict__ db) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d) return;
  float s = 0.f;
  for (long m = 0; m < n; ++m) s += dZ[m * d + j];
  db[j] = s;
}

// dY = 2 (P - Y) / (n d) and per-row sums of squared errors; one block per row, fixed order.
__global__ void __launch_bounds__(256) mse_kernel(const float* __restrict__ P, const float* __restrict__ Y, int d,
                                                  float inv_nd2, float* __restrict__ dY, float* __restrict__ row_loss) {
  __shared__ float sh[256];
  const long m = blockIdx.x;
  float s = 0.f;
  for (int j = threadIdx.x; j < d; j += 256) {
    const float e = P[m * d + j] - Y[m * d + j];
    s += e * e;
    dY[m * d + j] = inv_nd2 * e;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) row_loss[m] = sh[0];
}

// out[slot] = Σ_k x[k] (one block, fixed order, FP64 accumulation).
__global__ void sum_kernel(const float* __restrict__ x, long n, double* __restrict__ out, int slot) {
  __shared__ double sh[256];
  double s = 0;
  for (long k = threadIdx.x; k < n; k += 256) s += x[k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[slot] = sh[0];
}

__global__ void step_kernel(int* t) { *t += 1; }

// Adam step t (read from the device, so a captured epoch replays with the right bias corrections)
// on one parameter block; writes the BF16 copy of the weights the products use.
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1, float* __restrict__ m2,
                            long n, float lr, float b1, float b2, float eps, const int* __restrict__ t,
                            __nv_bfloat16* __restrict__ wbf) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float c1 = 1.f - powf(b1, float(*t)), c2 = 1.f - powf(b2, float(*t));
  const float gk = g[k];
  const float a = b1 * m1[k] + (1.f - b1) * gk;
  const float v = b2 * m2[k] + (1.f - b2) * gk * gk;
  m1[k] = a;
  m2[k] = v;
  const float wn = w[k] - lr * (a / c1) / (sqrtf(v / c2) + eps);
  w[k] = wn;
  if (wbf) wbf[k] = __float2bfloat16_rn(wn);
}

__global__ void to_bf16_kernel(const float* __restrict__ w, long n, __nv_bfloat16* __restrict__ o) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) o[k] = __float2bfloat16_rn(w[k]);
}

// Gathers the rows idx[0..n) of X [N][d] into out [n][d].
__global__ void gather_rows_kernel(const float* __restrict__ X, const int64_t* __restrict__ idx, long n, int d,
                                   float* __restrict__ out) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n * d) return;
  out[k] = X[idx[k / d] * d + k % d];
}

struct Mlp {
  Ctx* ctx = nullptr;
  int L = 0;
  std::vector<int> dims;
  std::vector<DBuf<float>> W, b, gW, gb, mW, vW, mb, vb;
  std::vector<DBuf<__nv_bfloat16>> Wbf;
  std::vector<DBuf<float>> Z, X;  // per layer, sized for the largest batch
  DBuf<float> dA, dB, loss_rows, Yb, work;
  DBuf<double> loss_sum;
  DBuf<int> d_step;  // Adam's step counter
  long cap = 0;      // rows the activation buffers hold
  DBuf<float> dataX, dataY;
  long ndata = 0;
  DBuf<float> x_mean, x_std, y_mean;  // feature standardisation for the in-iteration hook
  float y_scale = 1.f;
  bool scaled = false;
  long wgen = 0;  // bumped whenever the weights change (set_params, train)
  // Tensor-core inference: weights as the B operand [d_{l+1}][d_l padded to 8] (hi = the BF16
  // weights, lo = 0), activations as the A operand (BF16 hi/lo of the FP32 values) [cap][d_l
  // padded], split-K partials; rebuilt when wgen or the row capacity changes.
  struct Infer {
    long wgen = -1, cap = 0;
    std::vector<int> dpad, bn;
    std::vector<DBuf<__nv_bfloat16>> Wh, Wl, Ah, Al;
    std::vector<TcOperand> opA, opB;
    DBuf<float> part;
  } inf;
};

// X[i][j] = (feature j of state i - x_mean[j]) / x_std[j]: Re Σ(ω_j), Im Σ(ω_j), T, μ, scale, ε_i - μ.
__global__ void features_kernel(const double2* __restrict__ S, int nw, int ni, const double* __restrict__ eps_i, double T,
                                double mu, double scale, const float* __restrict__ xm, const float* __restrict__ xs,
                                float* __restrict__ X) {
  const int d0 = 2 * nw + 4;
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j >= d0) return;
  double v;
  if (j < nw)
    v = S[long(i) * nw + j].x;
  else if (j < 2 * nw)
    v = S[long(i) * nw + j - nw].y;
  else if (j == 2 * nw)
    v = T;
  else if (j == 2 * nw + 1)
    v = mu;
  else if (j == 2 * nw + 2)
    v = scale;
  else
    v = eps_i[i] - mu;
  X[long(i) * d0 + j] = (float(v) - xm[j]) / xs[j];
}

// Σ(ω_j, i) += (Y[i][j] y_scale + y_mean[j]) + i (Y[i][nω + j] y_scale + y_mean[nω + j]).
__global__ void correct_kernel(double2* __restrict__ S, int nw, const float* __restrict__ Y, float ys,
                               const float* __restrict__ ym) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j >= nw) return;
  const float* y = Y + long(i) * 2 * nw;
  double2 v = S[long(i) * nw + j];
  v.x += double(y[j] * ys + ym[j]);
  v.y += double(y[nw + j] * ys + ym[nw + j]);
  S[long(i) * nw + j] = v;
}

static void ensure_cap(Mlp* P, long n) {
  if (n <= P->cap) return;
  Ctx* ctx = P->ctx;
  int dmax = 0;
  for (int d : P->dims) dmax = std::max(dmax, d);
  P->Z.resize(size_t(P->L));
  P->X.resize(size_t(P->L + 1));
  for (int l = 0; l <= P->L; ++l) P->X[size_t(l)].alloc(ctx, size_t(n) * size_t(P->dims[size_t(l)]));
  for (int l = 0; l < P->L; ++l) P->Z[size_t(l)].alloc(ctx, size_t(n) * size_t(P->dims[size_t(l + 1)]));
  P->dA.alloc(ctx, size_t(n) * size_t(dmax));
  P->dB.alloc(ctx, size_t(n) * size_t(dmax));
  P->loss_rows.alloc(ctx, size_t(n));
  P->Yb.alloc(ctx, size_t(n) * size_t(P->dims.back()));
  // split-K partials: a product is split only when its tiles cover the GPU less than twice, and
  // slices x M x N <= (2 SMs / tiles) x tiles x 64 x 64
  const size_t wmax = size_t(2) * size_t(ctx->sm_count) * 64 * 64;
  P->work.alloc(ctx, wmax);
  P->cap = n;
}

// ---- tensor-core inference (the scGD0 hook on the tensor-core path) ----

// out[r][c] = in[r][c] for c < cols, 0 for cols <= c < ldo (BF16 rows padded to 16 bytes).
__global__ void pad_rows_bf16_kernel(const __nv_bfloat16* __restrict__ in, long rows, int cols, int ldo,
                                     __nv_bfloat16* __restrict__ out) {
  const long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= rows * ldo) return;
  const long r = k / ldo;
  const int c = int(k % ldo);
  out[k] = c < cols ? in[r * cols + c] : __float2bfloat16_rn(0.f);
}

// A operand of the first product: X [n][d] FP32 rows split into BF16 hi/lo rows of ldo.
__global__ void split_rows_mlp_kernel(const float* __restrict__ X, int n, int d, int ldo, __nv_bfloat16* __restrict__ oh,
                                      __nv_bfloat16* __restrict__ ol) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j >= d || i >= n) return;
  const float x = X[long(i) * d + j];
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  oh[long(i) * ldo + j] = h;
  ol[long(i) * ldo + j] = __float2bfloat16_rn(x - __bfloat162float(h));
}

// z = Σ_s part[s][m + n j] + b[j] (the product's column-major FP32 splits, in order); SiLU when act;
// into the next product's A operand (BF16 hi/lo rows of ldo) or, for the last layer, X [n][dout].
__global__ void bias_act_split_kernel(const float* __restrict__ part, int splits, long stride, int n, int dout,
                                      const float* __restrict__ b, bool act, __nv_bfloat16* __restrict__ oh,
                                      __nv_bfloat16* __restrict__ ol, int ldo, float* __restrict__ X) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (m >= n) return;
  float z = 0.f;
  for (int p = 0; p < splits; ++p) z += part[stride * p + m + long(n) * j];
  z += b[j];
  const float x = act ? z * sigmoidf_(z) : z;
  if (oh) {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    oh[long(m) * ldo + j] = h;
    ol[long(m) * ldo + j] = __float2bfloat16_rn(x - __bfloat162float(h));
  } else {
    X[long(m) * dout + j] = x;
  }
}

static void infer_reserve(Mlp* P, long n) {
  Mlp::Infer& I = P->inf;
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  const bool grow = n > I.cap;
  if (I.wgen == P->wgen && !grow) return;
  const int L = P->L;
  if (I.dpad.empty()) {
    I.dpad.resize(size_t(L));
    I.bn.resize(size_t(L));
    I.Wh.resize(size_t(L));
    I.Wl.resize(size_t(L));
    I.Ah.resize(size_t(L));
    I.Al.resize(size_t(L));
    I.opA.resize(size_t(L));
    I.opB.resize(size_t(L));
    for (int l = 0; l < L; ++l) {
      const int din = P->dims[size_t(l)], dout = P->dims[size_t(l + 1)];
      I.dpad[size_t(l)] = (din + 7) / 8 * 8;
      int bn, sp;
      tc_gemm_shape(ctx, 1, dout, din, 16, 2, &bn, &sp);  // the tile width depends on N only
      I.bn[size_t(l)] = bn;
      I.Wh[size_t(l)].alloc(ctx, size_t(dout) * size_t(I.dpad[size_t(l)]));
      I.Wl[size_t(l)].alloc(ctx, size_t(dout) * size_t(I.dpad[size_t(l)]));
      I.Wl[size_t(l)].zero(s);  // the weights are exact in BF16: no low part
      I.opB[size_t(l)].ns = 2;
      I.opB[size_t(l)].m[0] = make_tmap_bf16(I.Wh[size_t(l)].p, dout, din, I.dpad[size_t(l)], bn);
      I.opB[size_t(l)].m[1] = make_tmap_bf16(I.Wl[size_t(l)].p, dout, din, I.dpad[size_t(l)], bn);
    }
  }
  if (I.wgen != P->wgen) {
    for (int l = 0; l < L; ++l) {
      const int din = P->dims[size_t(l)], dout = P->dims[size_t(l + 1)], dp = I.dpad[size_t(l)];
      pad_rows_bf16_kernel<<<div_up(size_t(dout) * size_t(dp), 256), 256, 0, s>>>(P->Wbf[size_t(l)].p, dout, din, dp,
                                                                                 I.Wh[size_t(l)].p);
      EPSP_LAUNCHED(ctx);
    }
    I.wgen = P->wgen;
  }
  if (grow) {
    size_t part = 0;
    for (int l = 0; l < L; ++l) {
      const int din = P->dims[size_t(l)], dout = P->dims[size_t(l + 1)], dp = I.dpad[size_t(l)];
      I.Ah[size_t(l)].alloc(ctx, size_t(n) * size_t(dp));
      I.Al[size_t(l)].alloc(ctx, size_t(n) * size_t(dp));
      I.Ah[size_t(l)].zero(s);  // the padding columns stay zero
      I.Al[size_t(l)].zero(s);
      I.opA[size_t(l)].ns = 2;
      I.opA[size_t(l)].m[0] = make_tmap_bf16(I.Ah[size_t(l)].p, n, din, dp, kTcBM);
      I.opA[size_t(l)].m[1] = make_tmap_bf16(I.Al[size_t(l)].p, n, din, dp, kTcBM);
      int bn, sp;
      tc_gemm_shape(ctx, int(n), dout, dp, 16, 2, &bn, &sp);
      part = std::max(part, size_t(sp) * size_t(n) * size_t(dout));
    }
    I.part.alloc(ctx, part);
    I.cap = n;
  }
}

// Forward over the rows in P->X[0] (n rows) on the tensor cores: each product A x W^T with A the
// FP32 activations as BF16 hi + lo (three products, the weights' lo part is zero: FP32-accurate
// activations times the BF16 weights, as the SIMT forward), FP32 accumulation; output in P->X[L].
// Bounded waits report to d_err.
static void forward_tc(Mlp* P, long n, int* d_err) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  infer_reserve(P, n);
  Mlp::Infer& I = P->inf;
  const int d0 = P->dims[0];
  split_rows_mlp_kernel<<<dim3(div_up(size_t(d0), 256), unsigned(n)), 256, 0, s>>>(P->X[0].p, int(n), d0, I.dpad[0],
                                                                                 I.Ah[0].p, I.Al[0].p);
  EPSP_LAUNCHED(ctx);
  for (int l = 0; l < P->L; ++l) {
    const int dout = P->dims[size_t(l + 1)], dp = I.dpad[size_t(l)];
    const int sp = tc_gemm_launch(ctx, I.opA[size_t(l)], I.opB[size_t(l)], int(n), dout, dp, I.part.p, n, n * long(dout),
                                  16, d_err, "mlp");
    const bool last = l + 1 == P->L;
    bias_act_split_kernel<<<dim3(div_up(size_t(n), 128), unsigned(dout)), 128, 0, s>>>(
        I.part.p, sp, n * long(dout), int(n), dout, P->b[size_t(l)].p, !last, last ? nullptr : I.Ah[size_t(l + 1)].p,
        last ? nullptr : I.Al[size_t(l + 1)].p, last ? 0 : I.dpad[size_t(l + 1)], P->X[size_t(P->L)].p);
    EPSP_LAUNCHED(ctx);
  }
}

// Forward over the rows in P->X[0] (n rows); output in P->X[L].
static void forward(Mlp* P, long n) {
  Ctx* ctx = P->ctx;
  for (int l = 0; l < P->L; ++l) {
    const int din = P->dims[size_t(l)], dout = P->dims[size_t(l + 1)];
    mlp_gemm<float, __nv_bfloat16>(ctx, P->work.p, int(n), dout, din, P->X[size_t(l)].p, din, 1, P->Wbf[size_t(l)].p, 1,
                                   din, P->Z[size_t(l)].p, dout, 1);
    bias_act_kernel<<<div_up(size_t(n * dout), 256), 256, 0, ctx->stream>>>(P->Z[size_t(l)].p, P->b[size_t(l)].p, n, dout,
                                                                          l + 1 < P->L, P->X[size_t(l + 1)].p);
    EPSP_LAUNCHED(ctx);
  }
}

// Gradients of the mean squared error of the batch in P->X[0], P->Yb (n rows, normalised by
// n_total rows) into gW, gb; the batch's sum of squared errors goes to P->loss_sum[slot].
static void backward(Mlp* P, long n, long n_total, int slot) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  const int dl = P->dims.back();
  mse_kernel<<<unsigned(n), 256, 0, s>>>(P->X[size_t(P->L)].p, P->Yb.p, dl, 2.f / (float(n_total) * float(dl)), P->dA.p,
                                         P->loss_rows.p);
  EPSP_LAUNCHED(ctx);
  sum_kernel<<<1, 256, 0, s>>>(P->loss_rows.p, n, P->loss_sum.p, slot);
  EPSP_LAUNCHED(ctx);
  float* dZ = P->dA.p;  // gradient w.r.t. the last pre-activation (linear output)
  float* other = P->dB.p;
  for (int l = P->L - 1; l >= 0; --l) {
    const int din = P->dims[size_t(l)], dout = P->dims[size_t(l + 1)];
    // gW[o][i] = Σ_m dZ[m][o] X[m][i]
    mlp_gemm<float, float>(ctx, P->work.p, dout, din, int(n), dZ, 1, dout, P->X[size_t(l)].p, din, 1, P->gW[size_t(l)].p,
                           din, 1);
    bias_grad_kernel<<<div_up(size_t(dout), 128), 128, 0, s>>>(dZ, n, dout, P->gb[size_t(l)].p);
    EPSP_LAUNCHED(ctx);
    if (l > 0) {
      // dX[m][i] = Σ_o dZ[m][o] W[o][i], then through SiLU of layer l-1
      mlp_gemm<float, __nv_bfloat16>(ctx, P->work.p, int(n), din, dout, dZ, dout, 1, P->Wbf[size_t(l)].p, din, 1, other,
                                     din, 1);
      act_back_kernel<<<div_up(size_t(n * din), 256), 256, 0, s>>>(other, P->Z[size_t(l - 1)].p, n * din, other);
      EPSP_LAUNCHED(ctx);
      std::swap(dZ, other);
    }
  }
}

static void adam(Mlp* P, float lr) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  step_kernel<<<1, 1, 0, s>>>(P->d_step.p);
  EPSP_LAUNCHED(ctx);
  for (int l = 0; l < P->L; ++l) {
    const long nw = long(P->dims[size_t(l)]) * P->dims[size_t(l + 1)], nb = P->dims[size_t(l + 1)];
    adam_kernel<<<div_up(size_t(nw), 256), 256, 0, s>>>(P->W[size_t(l)].p, P->gW[size_t(l)].p, P->mW[size_t(l)].p,
                                                        P->vW[size_t(l)].p, nw, lr, b1, b2, eps, P->d_step.p,
                                                        P->Wbf[size_t(l)].p);
    EPSP_LAUNCHED(ctx);
    adam_kernel<<<div_up(size_t(nb), 256), 256, 0, s>>>(P->b[size_t(l)].p, P->gb[size_t(l)].p, P->mb[size_t(l)].p,
                                                        P->vb[size_t(l)].p, nb, lr, b1, b2, eps, P->d_step.p, nullptr);
    EPSP_LAUNCHED(ctx);
  }
}

static long nparams(const Mlp* P) {
  long t = 0;
  for (int l = 0; l < P->L; ++l) t += long(P->dims[size_t(l)]) * P->dims[size_t(l + 1)] + P->dims[size_t(l + 1)];
  return t;
}

}  // namespace epsp

using namespace epsp;

struct epsp_warmstart {
  Mlp m;
};

namespace epsp {

void warmstart_correct(epsp_warmstart* w, Ctx* ctx, double2* S_T, long nw, long ni, const double* d_eps_i, double T,
                       double mu, double scale, int* tc_err) {
  Mlp& P = w->m;
  if (P.ctx != ctx) fail(EPSP_EINVAL, "the warm-start network belongs to another context");
  if (P.dims[0] != 2 * nw + 4 || P.dims.back() != 2 * nw)
    fail(EPSP_EINVAL, "the warm-start network's widths do not match 2 nω + 4 inputs and 2 nω outputs (nω = " +
                          std::to_string(nw) + ")");
  if (!P.scaled) fail(EPSP_EINVAL, "the warm-start network has no feature scaling (epsp_warmstart_set_scaling)");
  cudaStream_t s = ctx->stream;
  ensure_cap(&P, ni);
  features_kernel<<<dim3(div_up(size_t(2 * nw + 4), 256), unsigned(ni)), 256, 0, s>>>(
      S_T, int(nw), int(ni), d_eps_i, T, mu, scale, P.x_mean.p, P.x_std.p, P.X[0].p);
  EPSP_LAUNCHED(ctx);
  if (tc_err)
    forward_tc(&P, ni, tc_err);
  else
    forward(&P, ni);
  correct_kernel<<<dim3(div_up(size_t(nw), 256), unsigned(ni)), 256, 0, s>>>(S_T, int(nw), P.X[size_t(P.L)].p, P.y_scale,
                                                                            P.y_mean.p);
  EPSP_LAUNCHED(ctx);
}

}  // namespace epsp

template <class F>
static epsp_status wguard(Ctx* c, F&& f) {
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
  }
}

extern "C" {

epsp_status epsp_warmstart_create(epsp_ctx* ctx, int32_t nlayers, const int32_t* dims, epsp_warmstart** out) {
  if (!ctx || !out || !dims || nlayers < 1 || nlayers > 16) return EPSP_EINVAL;
  *out = nullptr;
  return wguard(&ctx->c, [&] {
    for (int l = 0; l <= nlayers; ++l)
      if (dims[l] < 1 || dims[l] > (1 << 20)) fail(EPSP_EINVAL, "layer widths must be in [1, 2^20]");
    auto* w = new epsp_warmstart;
    std::unique_ptr<epsp_warmstart> guard(w);
    Mlp& P = w->m;
    P.ctx = &ctx->c;
    P.L = nlayers;
    P.dims.assign(dims, dims + nlayers + 1);
    P.W.resize(size_t(nlayers));
    P.b.resize(size_t(nlayers));
    P.gW.resize(size_t(nlayers));
    P.gb.resize(size_t(nlayers));
    P.mW.resize(size_t(nlayers));
    P.vW.resize(size_t(nlayers));
    P.mb.resize(size_t(nlayers));
    P.vb.resize(size_t(nlayers));
    P.Wbf.resize(size_t(nlayers));
    for (int l = 0; l < nlayers; ++l) {
      const size_t nw = size_t(dims[l]) * size_t(dims[l + 1]), nb = size_t(dims[l + 1]);
      for (auto* v : {&P.W[size_t(l)], &P.gW[size_t(l)], &P.mW[size_t(l)], &P.vW[size_t(l)]}) v->alloc(P.ctx, nw);
      for (auto* v : {&P.b[size_t(l)], &P.gb[size_t(l)], &P.mb[size_t(l)], &P.vb[size_t(l)]}) v->alloc(P.ctx, nb);
      P.Wbf[size_t(l)].alloc(P.ctx, nw);
      for (auto* v : {&P.W[size_t(l)], &P.mW[size_t(l)], &P.vW[size_t(l)], &P.b[size_t(l)], &P.mb[size_t(l)], &P.vb[size_t(l)]})
        v->zero(P.ctx->stream);
    }
    P.loss_sum.alloc(P.ctx, 1);
    P.d_step.alloc(P.ctx, 1);
    P.d_step.zero(P.ctx->stream);
    EPSP_CUDA(cudaStreamSynchronize(P.ctx->stream));
    *out = guard.release();
  });
}

void epsp_warmstart_destroy(epsp_warmstart* w) {
  if (!w) return;
  cudaSetDevice(w->m.ctx->device);
  delete w;
}

int64_t epsp_warmstart_nparams(const epsp_warmstart* w) { return w ? nparams(&w->m) : 0; }

/* Parameters as one flat FP32 vector: for each layer, W [d_{l+1}][d_l] then b [d_{l+1}]. Setting
 * them resets the optimiser state. */
epsp_status epsp_warmstart_set_params(epsp_warmstart* w, const float* params) {
  if (!w || !params) return EPSP_EINVAL;
  Mlp& P = w->m;
  return wguard(P.ctx, [&] {
    cudaStream_t s = P.ctx->stream;
    long off = 0;
    for (int l = 0; l < P.L; ++l) {
      const long nw = long(P.dims[size_t(l)]) * P.dims[size_t(l + 1)], nb = P.dims[size_t(l + 1)];
      P.W[size_t(l)].upload(params + off, size_t(nw), s);
      off += nw;
      P.b[size_t(l)].upload(params + off, size_t(nb), s);
      off += nb;
      to_bf16_kernel<<<div_up(size_t(nw), 256), 256, 0, s>>>(P.W[size_t(l)].p, nw, P.Wbf[size_t(l)].p);
      EPSP_LAUNCHED(P.ctx);
      P.mW[size_t(l)].zero(s);
      P.vW[size_t(l)].zero(s);
      P.mb[size_t(l)].zero(s);
      P.vb[size_t(l)].zero(s);
    }
    P.d_step.zero(s);
    ++P.wgen;
    EPSP_CUDA(cudaStreamSynchronize(s));
  });
}

epsp_status epsp_warmstart_get_params(epsp_warmstart* w, float* params) {
  if (!w || !params) return EPSP_EINVAL;
  Mlp& P = w->m;
  return wguard(P.ctx, [&] {
    cudaStream_t s = P.ctx->stream;
    long off = 0;
    for (int l = 0; l < P.L; ++l) {
      const long nw = long(P.dims[size_t(l)]) * P.dims[size_t(l + 1)], nb = P.dims[size_t(l + 1)];
      P.W[size_t(l)].download(params + off, size_t(nw), s);
      off += nw;
      P.b[size_t(l)].download(params + off, size_t(nb), s);
      off += nb;
    }
    EPSP_CUDA(cudaStreamSynchronize(s));
  });
}

/* Standardisation used when the network corrects Σ inside the scGD0 iteration: inputs
 * (x - x_mean) / x_std, outputs y * y_scale + y_mean. */
epsp_status epsp_warmstart_set_scaling(epsp_warmstart* w, const float* x_mean, const float* x_std, const float* y_mean,
                                       float y_scale) {
  if (!w || !x_mean || !x_std || !y_mean || !(y_scale > 0.f) || !std::isfinite(y_scale)) return EPSP_EINVAL;
  Mlp& P = w->m;
  return wguard(P.ctx, [&] {
    const int d0 = P.dims[0], dl = P.dims.back();
    for (int j = 0; j < d0; ++j)
      if (!(x_std[j] > 0.f) || !std::isfinite(x_std[j]) || !std::isfinite(x_mean[j]))
        fail(EPSP_EINVAL, "x_std must be positive and x_mean finite");
    for (int j = 0; j < dl; ++j)
      if (!std::isfinite(y_mean[j])) fail(EPSP_EINVAL, "y_mean must be finite");
    cudaStream_t s = P.ctx->stream;
    P.x_mean.alloc(P.ctx, size_t(d0));
    P.x_std.alloc(P.ctx, size_t(d0));
    P.y_mean.alloc(P.ctx, size_t(dl));
    P.x_mean.upload(x_mean, size_t(d0), s);
    P.x_std.upload(x_std, size_t(d0), s);
    P.y_mean.upload(y_mean, size_t(dl), s);
    P.y_scale = y_scale;
    P.scaled = true;
    EPSP_CUDA(cudaStreamSynchronize(s));
  });
}

/* Inference: Y [n][d_L] from X [n][d_0] (host arrays, row-major). */
epsp_status epsp_warmstart_predict(epsp_warmstart* w, const float* X, int64_t n, float* Y) {
  if (!w || !X || !Y || n < 1) return EPSP_EINVAL;
  Mlp& P = w->m;
  return wguard(P.ctx, [&] {
    cudaStream_t s = P.ctx->stream;
    const long chunk = 8192;
    ensure_cap(&P, std::min<long>(n, chunk));
    for (long r0 = 0; r0 < n; r0 += chunk) {
      const long nb = std::min(chunk, n - r0);
      P.X[0].upload(X + r0 * P.dims[0], size_t(nb * P.dims[0]), s);
      forward(&P, nb);
      P.X[size_t(P.L)].download(Y + r0 * P.dims.back(), size_t(nb * P.dims.back()), s);
    }
    EPSP_CUDA(cudaStreamSynchronize(s));
  });
}

/* Loss (mean squared error) and its gradient with respect to every parameter (flat, as
 * epsp_warmstart_set_params) for the batch (X [n][d_0], Y [n][d_L]); no parameter update. */
epsp_status epsp_warmstart_grad(epsp_warmstart* w, const float* X, const float* Y, int64_t n, double* loss, float* grad) {
  if (!w || !X || !Y || n < 1 || !grad) return EPSP_EINVAL;
  Mlp& P = w->m;
  return wguard(P.ctx, [&] {
    cudaStream_t s = P.ctx->stream;
    ensure_cap(&P, n);
    P.X[0].upload(X, size_t(n * P.dims[0]), s);
    P.Yb.upload(Y, size_t(n * P.dims.back()), s);
    forward(&P, n);
    backward(&P, n, n, 0);
    long off = 0;
    for (int l = 0; l < P.L; ++l) {
      const long nw = long(P.dims[size_t(l)]) * P.dims[size_t(l + 1)], nb = P.dims[size_t(l + 1)];
      P.gW[size_t(l)].download(grad + off, size_t(nw), s);
      off += nw;
      P.gb[size_t(l)].download(grad + off, size_t(nb), s);
      off += nb;
    }
    double ls = 0;
    P.loss_sum.download(&ls, 1, s);
    EPSP_CUDA(cudaStreamSynchronize(s));
    if (loss) *loss = ls / (double(n) * P.dims.back());
  });
}

/* Training: the set (X [n][d_0], Y [n][d_L]) is uploaded once; `epochs` passes of Adam (learning
 * rate lr) over minibatches of `batch` rows in the order perm (n indices per epoch, epochs x n in
 * total, or NULL for the identity); each minibatch's loss is its own mean. loss_history [epochs]
 * receives each epoch's mean loss over the set. */
epsp_status epsp_warmstart_train(epsp_warmstart* w, const float* X, const float* Y, int64_t n, int32_t epochs,
                                 int32_t batch, float lr, const int64_t* perm, double* loss_history) {
  if (!w || !X || !Y || n < 1 || epochs < 1 || batch < 1 || !(lr > 0.f)) return EPSP_EINVAL;
  Mlp& P = w->m;
  return wguard(P.ctx, [&] {
    cudaStream_t s = P.ctx->stream;
    const int d0 = P.dims[0], dl = P.dims.back();
    if (perm)
      for (long k = 0; k < long(epochs) * n; ++k)
        if (perm[k] < 0 || perm[k] >= n) fail(EPSP_EINVAL, "perm holds an index outside [0, n)");
    const long nbat = (n + batch - 1) / batch;
    P.dataX.alloc(P.ctx, size_t(n) * size_t(d0));
    P.dataY.alloc(P.ctx, size_t(n) * size_t(dl));
    P.dataX.upload(X, size_t(n) * size_t(d0), s);
    P.dataY.upload(Y, size_t(n) * size_t(dl), s);
    DBuf<int64_t> d_perm;
    d_perm.alloc(P.ctx, size_t(n));
    P.loss_sum.alloc(P.ctx, size_t(nbat));
    ensure_cap(&P, std::min<long>(n, batch));
    std::vector<int64_t> ident;
    if (!perm) {
      ident.resize(size_t(n));
      for (long k = 0; k < n; ++k) ident[size_t(k)] = k;
    }
    std::vector<double> bl(static_cast<size_t>(nbat));
    // One epoch's launches (every minibatch: gather, forward, backward, Adam) are captured once in a
    // CUDA graph and replayed per epoch; only the row order (uploaded before each replay) changes.
    auto epoch_launches = [&] {
      for (long bi = 0; bi < nbat; ++bi) {
        const long r0 = bi * batch, nb = std::min<long>(batch, n - r0);
        gather_rows_kernel<<<div_up(size_t(nb * d0), 256), 256, 0, s>>>(P.dataX.p, d_perm.p + r0, nb, d0, P.X[0].p);
        EPSP_LAUNCHED(P.ctx);
        gather_rows_kernel<<<div_up(size_t(nb * dl), 256), 256, 0, s>>>(P.dataY.p, d_perm.p + r0, nb, dl, P.Yb.p);
        EPSP_LAUNCHED(P.ctx);
        forward(&P, nb);
        backward(&P, nb, nb, int(bi));
        adam(&P, lr);
      }
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    struct GraphGuard {
      cudaGraph_t* g;
      cudaGraphExec_t* e;
      ~GraphGuard() {
        if (*e) cudaGraphExecDestroy(*e);
        if (*g) cudaGraphDestroy(*g);
      }
    } gguard{&graph, &exec};
    const int64_t l0 = P.ctx->launches;
    EPSP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      epoch_launches();
    } catch (...) {
      cudaStreamEndCapture(s, &graph);
      throw;
    }
    EPSP_CUDA(cudaStreamEndCapture(s, &graph));
    EPSP_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    const int64_t per_epoch = P.ctx->launches - l0;
    P.ctx->launches = l0;
    for (int e = 0; e < epochs; ++e) {
      d_perm.upload(perm ? perm + long(e) * n : ident.data(), size_t(n), s);
      EPSP_CUDA(cudaGraphLaunch(exec, s));
      P.ctx->launches += per_epoch;
      P.loss_sum.download(bl.data(), size_t(nbat), s);
      EPSP_CUDA(cudaStreamSynchronize(s));
      double tot = 0;
      for (double v : bl) tot += v;
      if (loss_history) loss_history[e] = tot / (double(n) * dl);
    }
    P.dataX.release();
    P.dataY.release();
    P.loss_sum.alloc(P.ctx, 1);
    ++P.wgen;
  });
}

}  // extern "C"
