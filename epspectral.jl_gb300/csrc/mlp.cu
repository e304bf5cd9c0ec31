// mlp.cu -- the learned warm start: a small multilayer perceptron, its training and its inference,
// on the GPU with hand-written kernels.
//
// Network: L fully connected layers d_0 -> d_1 -> ... -> d_L, SiLU between layers, linear output.
// Weights W_l [d_{l+1}][d_l] (row-major) are kept in FP32 (the optimiser's master copy) and used in
// BF16 by the products (BF16 weights, FP32 accumulation); biases FP32. The loss is the mean squared
// error over the batch and the outputs; the optimiser is Adam. Every product of the training, of
// the gradient and of the prediction runs on the tensor cores (tc_gemm_launch: tcgen05, TMA, TMEM)
// with the FP32 activations and gradients split into three BF16 parts (six products, ~2^-24
// relative, as FP32; the BF16 weights' second and third parts are zero), every reduction in fixed
// order, so a training run is bitwise reproducible. The scGD0 hook's inference (forward_tc) splits
// the activations into two parts.
#include "common.cuh"
#include "tc_gemm.cuh"
#include "warmstart.cuh"

#include <cuda_bf16.h>

#include <cmath>
#include <memory>

namespace epsp {

// C[m scm + n scn] = Σ_z P[z][m][n], z ascending.
__global__ void partial_sum_kernel(const float* __restrict__ P, int M, int N, int nz, float* __restrict__ C, long scm,
                                   long scn) {
  const long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= long(M) * N) return;
  float acc = 0.f;
  for (int z = 0; z < nz; ++z) acc += P[long(z) * M * N + k];
  C[(k / N) * scm + (k % N) * scn] = acc;
}

__device__ __forceinline__ float sigmoidf_(float x) { return 1.f / (1.f + expf(-x)); }

// One pass over a [rows][cols] matrix in 32 x 32 tiles. The value v(m, j) is, by MODE:
//   kEmitCopy    src[m ld_src + j];
//   kEmitBiasAct z = Σ_s part[s pstride + j + cols m] + bias[j] (a product's split-K slabs, summed in
//                order), written to Zout[m cols + j] when given, then v = SiLU(z) if act, else z;
//   kEmitActBack Σ_s part[s pstride + j + cols m] times SiLU'(Zin[m cols + j]).
// v goes to out32[m cols + j] (FP32) and, as three BF16 parts, to rp[p rpart + m ldr + j] (rows)
// and tp[p tpart + j ldt + m] (transposed, through shared memory; columns m in [rows, ldt) get
// zeros, so that the padded K of a product over the rows adds nothing). Grid (cols / 32, M / 32)
// with M = ldt when tp is given, else rows; 32 x 8 threads.
enum { kEmitCopy = 0, kEmitBiasAct = 1, kEmitActBack = 2 };
template <int MODE>
__global__ void __launch_bounds__(256)
    emit_kernel(int rows, int cols, const float* __restrict__ src, long ld_src, const float* __restrict__ part, int splits,
                long pstride, const float* __restrict__ bias, bool act, const float* __restrict__ Zin,
                float* __restrict__ Zout, float* __restrict__ out32, __nv_bfloat16* __restrict__ rp, long ldr, long rpart,
                __nv_bfloat16* __restrict__ tp, long ldt, long tpart) {
  __shared__ float tile[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int j0 = blockIdx.x * 32, m0 = blockIdx.y * 32;
  const int j = j0 + tx;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int ml = ty + 8 * r, m = m0 + ml;
    float v = 0.f;
    if (m < rows && j < cols) {
      if constexpr (MODE == kEmitCopy) {
        v = src[long(m) * ld_src + j];
      } else {
        float acc = 0.f;
        for (int sp = 0; sp < splits; ++sp) acc += part[long(sp) * pstride + j + long(cols) * m];
        if constexpr (MODE == kEmitBiasAct) {
          const float z = acc + bias[j];
          if (Zout) Zout[long(m) * cols + j] = z;
          v = act ? z * sigmoidf_(z) : z;
        } else {
          const float z = Zin[long(m) * cols + j], sg = sigmoidf_(z);
          v = acc * (sg * (1.f + z * (1.f - sg)));
        }
      }
      if (out32) out32[long(m) * cols + j] = v;
      if (rp) {
        __nv_bfloat16 q[3];
        split_bf16_n(v, 3, q);
#pragma unroll
        for (int p = 0; p < 3; ++p) rp[p * rpart + long(m) * ldr + j] = q[p];
      }
    }
    tile[ml][tx] = v;
  }
  if (!tp) return;
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int jl = ty + 8 * r, jj = j0 + jl, m = m0 + tx;
    if (jj >= cols || m >= ldt) continue;
    __nv_bfloat16 q[3];
    split_bf16_n(tile[tx][jl], 3, q);  // zero for m >= rows
#pragma unroll
    for (int p = 0; p < 3; ++p) tp[p * tpart + long(jj) * ldt + m] = q[p];
  }
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

// BF16 copies of the weight element k = o d_in + i of W [d_out][d_in]: wbf[k], the tensor-core
// products' rows wp[o ldp + i] and the transposed rows wt[i ldt + o].
__device__ __forceinline__ void store_wbf(long k, float w, int din, __nv_bfloat16* __restrict__ wbf,
                                          __nv_bfloat16* __restrict__ wp, long ldp, __nv_bfloat16* __restrict__ wt,
                                          long ldt) {
  const __nv_bfloat16 h = __float2bfloat16_rn(w);
  wbf[k] = h;
  const long o = k / din, i = k % din;
  wp[o * ldp + i] = h;
  wt[i * ldt + o] = h;
}

// Adam step t (read from the device, so a captured epoch replays with the right bias corrections)
// on one parameter block; for a weight block (wbf given) writes the BF16 copies the products use.
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1, float* __restrict__ m2,
                            long n, float lr, float b1, float b2, float eps, const int* __restrict__ t,
                            __nv_bfloat16* __restrict__ wbf, int din, __nv_bfloat16* __restrict__ wp, long ldp,
                            __nv_bfloat16* __restrict__ wt, long ldt) {
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
  if (wbf) store_wbf(k, wn, din, wbf, wp, ldp, wt, ldt);
}

__global__ void to_bf16_kernel(const float* __restrict__ w, long n, int din, __nv_bfloat16* __restrict__ wbf,
                               __nv_bfloat16* __restrict__ wp, long ldp, __nv_bfloat16* __restrict__ wt, long ldt) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) store_wbf(k, w[k], din, wbf, wp, ldp, wt, ldt);
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
  DBuf<float> dA, dB, loss_rows, Yb;
  DBuf<int> d_err;                // the tensor-core products' bounded-wait flag
  DBuf<double> loss_sum;
  DBuf<int> d_step;  // Adam's step counter
  long cap = 0;      // rows the activation buffers hold
  DBuf<float> dataX, dataY;
  long ndata = 0;
  DBuf<float> x_mean, x_std, y_mean;  // feature standardisation for the in-iteration hook
  float y_scale = 1.f;
  bool scaled = false;
  long wgen = 0;  // bumped whenever the weights change (set_params, train)
  double train_ms = 0;  // device milliseconds of the last training's epochs
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
  // Tensor-core training and prediction (three BF16 parts per operand, FP32 accumulation). Layer l
  // (d_l -> d_{l+1}), batches of up to cap rows, rows padded to ldT = cap rounded up to 8:
  //   forward   Z_l^T = W_l X_l^T     A = W_l  [d_{l+1}][dp_l]  B = Xs_l  [cap][dp_l]      K = d_l
  //   gradient  gW_l^T = X_l^T dZ_l   A = XT_l [d_l][ldT]       B = dZT_l [d_{l+1}][ldT]   K = rows
  //   backward  dX_l^T = W_l^T dZ_l^T A = WT_l [d_l][dp_{l+1}]  B = dZs_l [cap][dp_{l+1}]  K = d_{l+1}
  // (dp_l = d_l padded to 8: 16-byte rows); the activation and gradient buffers hold their three
  // parts one after the other.
  struct Train {
    long cap = 0, ldT = 0;
    std::vector<int> dp;
    std::vector<DBuf<__nv_bfloat16>> Wp, WT, Xs, XT, dZs, dZT;
    DBuf<__nv_bfloat16> zero;  // the weights' second and third parts
    std::vector<TcOperand> opW, opWT, opXs, opXT, opdZs, opdZT;
    DBuf<float> part;
  } tr;
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

// A three-part operand over `parts` (three consecutive [rows][ld] BF16 blocks, or one block and
// the shared zero block twice when zero is given), boxes of box_rows rows.
static TcOperand three_part(const __nv_bfloat16* parts, const __nv_bfloat16* zero, long rows, long cols, long ld,
                            int box_rows) {
  TcOperand op;
  op.ns = 3;
  for (int p = 0; p < 3; ++p) {
    const __nv_bfloat16* base = p == 0 ? parts : zero ? zero : parts + long(p) * rows * ld;
    op.m[p] = make_tmap_bf16(base, rows, cols, ld, box_rows);
    op.base[p] = base;
  }
  op.rows = rows;
  op.cols = cols;
  op.ld = ld;
  return op;
}

// The BF16 weight rows of the products and their operands (fixed sizes; built once per network).
static void train_weights_init(Mlp* P) {
  Mlp::Train& T = P->tr;
  const int L = P->L;
  T.dp.resize(size_t(L + 1));
  for (int l = 0; l <= L; ++l) T.dp[size_t(l)] = (P->dims[size_t(l)] + 7) / 8 * 8;
  T.Wp.resize(size_t(L));
  T.WT.resize(size_t(L));
  size_t zmax = 0;
  for (int l = 0; l < L; ++l) {
    const long din = P->dims[size_t(l)], dout = P->dims[size_t(l + 1)];
    T.Wp[size_t(l)].alloc(P->ctx, size_t(dout * T.dp[size_t(l)]));
    T.WT[size_t(l)].alloc(P->ctx, size_t(din * T.dp[size_t(l + 1)]));
    T.Wp[size_t(l)].zero(P->ctx->stream);  // the padding columns stay zero
    T.WT[size_t(l)].zero(P->ctx->stream);
    zmax = std::max(zmax, std::max(size_t(dout * T.dp[size_t(l)]), size_t(din * T.dp[size_t(l + 1)])));
  }
  T.zero.alloc(P->ctx, zmax);
  T.zero.zero(P->ctx->stream);
  T.opW.resize(size_t(L));
  T.opWT.resize(size_t(L));
  for (int l = 0; l < L; ++l) {
    const long din = P->dims[size_t(l)], dout = P->dims[size_t(l + 1)];
    T.opW[size_t(l)] = three_part(T.Wp[size_t(l)].p, T.zero.p, dout, din, T.dp[size_t(l)], kTcBM);
    T.opWT[size_t(l)] = three_part(T.WT[size_t(l)].p, T.zero.p, din, dout, T.dp[size_t(l + 1)], kTcBM);
  }
}

static void ensure_cap(Mlp* P, long n) {
  if (n <= P->cap) return;
  Ctx* ctx = P->ctx;
  const int L = P->L;
  int dmax = 0;
  for (int d : P->dims) dmax = std::max(dmax, d);
  P->Z.resize(size_t(L));
  P->X.resize(size_t(L + 1));
  for (int l = 0; l <= L; ++l) P->X[size_t(l)].alloc(ctx, size_t(n) * size_t(P->dims[size_t(l)]));
  for (int l = 0; l < L; ++l) P->Z[size_t(l)].alloc(ctx, size_t(n) * size_t(P->dims[size_t(l + 1)]));
  P->dA.alloc(ctx, size_t(n) * size_t(dmax));
  P->dB.alloc(ctx, size_t(n) * size_t(dmax));
  P->loss_rows.alloc(ctx, size_t(n));
  P->Yb.alloc(ctx, size_t(n) * size_t(P->dims.back()));
  // the tensor-core operands of the activations and gradients, and the products' split-K slabs:
  // a product of t tiles takes at most ceil(SMs / t) splits, so splits x M x N stays below
  // (SMs + t) tiles of 128 x 128
  Mlp::Train& T = P->tr;
  T.cap = n;
  T.ldT = (n + 7) / 8 * 8;
  for (auto* v : {&T.Xs, &T.XT, &T.dZs, &T.dZT}) v->resize(size_t(L));
  for (auto* v : {&T.opXs, &T.opXT, &T.opdZs, &T.opdZT}) v->resize(size_t(L));
  const long sm = ctx->sm_count;
  auto tiles = [](long M, long N) { return ((M + 127) / 128) * ((N + 127) / 128); };
  long part = 0;
  for (int l = 0; l < L; ++l) {
    const long din = P->dims[size_t(l)], dout = P->dims[size_t(l + 1)];
    const long dpi = T.dp[size_t(l)], dpo = T.dp[size_t(l + 1)];
    T.Xs[size_t(l)].alloc(ctx, size_t(3 * n * dpi));
    T.XT[size_t(l)].alloc(ctx, size_t(3 * din * T.ldT));
    T.dZs[size_t(l)].alloc(ctx, size_t(3 * n * dpo));
    T.dZT[size_t(l)].alloc(ctx, size_t(3 * dout * T.ldT));
    T.opXs[size_t(l)] = three_part(T.Xs[size_t(l)].p, nullptr, n, din, dpi, 128);
    T.opXT[size_t(l)] = three_part(T.XT[size_t(l)].p, nullptr, din, T.ldT, T.ldT, kTcBM);
    T.opdZs[size_t(l)] = three_part(T.dZs[size_t(l)].p, nullptr, n, dout, dpo, 128);
    T.opdZT[size_t(l)] = three_part(T.dZT[size_t(l)].p, nullptr, dout, T.ldT, T.ldT, 128);
    for (const long t : {tiles(dout, n), tiles(din, dout), tiles(din, n)}) part = std::max(part, (sm + t) * 128 * 128);
  }
  T.part.alloc(ctx, size_t(part));
  P->cap = n;
}

// One three-part product into the split-K slabs T.part (out[s][m + ld_out n]); returns the splits.
static int mlp_product(Mlp* P, const TcOperand& A, const TcOperand& B, int M, int N, int K, long ld_out) {
  int bn = 0, sp = 0;
  tc_gemm_shape(P->ctx, M, N, K, 16, 3, &bn, &sp);
  if (bn != 128) fail(EPSP_EINVAL, "three-part products run with tiles of 128 columns");
  if (size_t(sp) * size_t(M) * size_t(N) > P->tr.part.n) fail(EPSP_EINVAL, "split-K slabs exceed their buffer");
  return tc_gemm_launch(P->ctx, A, B, M, N, K, P->tr.part.p, ld_out, long(M) * N, 16, P->d_err.p, "mlp");
}

static dim3 emit_grid(long cols, long rows) { return dim3(unsigned((cols + 31) / 32), unsigned((rows + 31) / 32)); }

// Forward over the n rows in P->X[0] on the tensor cores; output in P->X[L]. With `train` the
// transposed activations (the gradient products' operands) and the pre-activations Z are kept.
static void forward_train(Mlp* P, long n, bool train) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  Mlp::Train& T = P->tr;
  const dim3 blk(32, 8);
  const int d0 = P->dims[0];
  emit_kernel<kEmitCopy><<<emit_grid(d0, train ? T.ldT : n), blk, 0, s>>>(
      int(n), d0, P->X[0].p, d0, nullptr, 0, 0, nullptr, false, nullptr, nullptr, nullptr, T.Xs[0].p, T.dp[0],
      long(T.cap) * T.dp[0], train ? T.XT[0].p : nullptr, T.ldT, long(d0) * T.ldT);
  EPSP_LAUNCHED(ctx);
  for (int l = 0; l < P->L; ++l) {
    const int din = P->dims[size_t(l)], dout = P->dims[size_t(l + 1)];
    const bool last = l + 1 == P->L;
    const int sp = mlp_product(P, T.opW[size_t(l)], T.opXs[size_t(l)], dout, int(n), din, dout);
    const bool tpose = train && !last;
    emit_kernel<kEmitBiasAct><<<emit_grid(dout, tpose ? T.ldT : n), blk, 0, s>>>(
        int(n), dout, nullptr, 0, T.part.p, sp, long(dout) * n, P->b[size_t(l)].p, !last, nullptr,
        (train && !last) ? P->Z[size_t(l)].p : nullptr, last ? P->X[size_t(P->L)].p : nullptr,
        last ? nullptr : T.Xs[size_t(l + 1)].p, last ? 0 : T.dp[size_t(l + 1)], last ? 0 : long(T.cap) * T.dp[size_t(l + 1)],
        tpose ? T.XT[size_t(l + 1)].p : nullptr, T.ldT, long(dout) * T.ldT);
    EPSP_LAUNCHED(ctx);
  }
}

// Gradients of the mean squared error of the batch in P->X[0], P->Yb (n rows, normalised by
// n_total rows) into gW, gb; the batch's sum of squared errors goes to P->loss_sum[slot]. Needs the
// forward with `train`.
static void backward(Mlp* P, long n, long n_total, int slot) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  Mlp::Train& T = P->tr;
  const dim3 blk(32, 8);
  const int L = P->L, dl = P->dims.back();
  mse_kernel<<<unsigned(n), 256, 0, s>>>(P->X[size_t(L)].p, P->Yb.p, dl, 2.f / (float(n_total) * float(dl)), P->dA.p,
                                         P->loss_rows.p);
  EPSP_LAUNCHED(ctx);
  sum_kernel<<<1, 256, 0, s>>>(P->loss_rows.p, n, P->loss_sum.p, slot);
  EPSP_LAUNCHED(ctx);
  // dZ of the last layer (linear output) as the products' operands
  emit_kernel<kEmitCopy><<<emit_grid(dl, T.ldT), blk, 0, s>>>(
      int(n), dl, P->dA.p, dl, nullptr, 0, 0, nullptr, false, nullptr, nullptr, nullptr, T.dZs[size_t(L - 1)].p,
      T.dp[size_t(L)], long(T.cap) * T.dp[size_t(L)], T.dZT[size_t(L - 1)].p, T.ldT, long(dl) * T.ldT);
  EPSP_LAUNCHED(ctx);
  float* dZ = P->dA.p;  // FP32 dZ of layer l, [n][d_{l+1}]
  float* other = P->dB.p;
  for (int l = L - 1; l >= 0; --l) {
    const int din = P->dims[size_t(l)], dout = P->dims[size_t(l + 1)];
    // gW[o][i] = Σ_m dZ[m][o] X[m][i]: the product's slab element (i, o) at i + din o
    const int sg = mlp_product(P, T.opXT[size_t(l)], T.opdZT[size_t(l)], din, dout, int(n), din);
    partial_sum_kernel<<<div_up(size_t(dout) * size_t(din), 256), 256, 0, s>>>(T.part.p, dout, din, sg,
                                                                               P->gW[size_t(l)].p, din, 1);
    EPSP_LAUNCHED(ctx);
    bias_grad_kernel<<<div_up(size_t(dout), 128), 128, 0, s>>>(dZ, n, dout, P->gb[size_t(l)].p);
    EPSP_LAUNCHED(ctx);
    if (l > 0) {
      // dX[m][i] = Σ_o dZ[m][o] W[o][i] (slab element (i, m) at i + din m), through SiLU of layer l - 1
      const int sx = mlp_product(P, T.opWT[size_t(l)], T.opdZs[size_t(l)], din, int(n), dout, din);
      emit_kernel<kEmitActBack><<<emit_grid(din, T.ldT), blk, 0, s>>>(
          int(n), din, nullptr, 0, T.part.p, sx, long(din) * n, nullptr, false, P->Z[size_t(l - 1)].p, nullptr, other,
          T.dZs[size_t(l - 1)].p, T.dp[size_t(l)], long(T.cap) * T.dp[size_t(l)], T.dZT[size_t(l - 1)].p, T.ldT,
          long(din) * T.ldT);
      EPSP_LAUNCHED(ctx);
      std::swap(dZ, other);
    }
  }
}

// Reports (and clears) a bounded wait that ran out in the network's tensor-core products.
static void check_mlp_err(Mlp* P) {
  int e = 0;
  P->d_err.download(&e, 1, P->ctx->stream);
  EPSP_CUDA(cudaStreamSynchronize(P->ctx->stream));
  if (e) {
    P->d_err.zero(P->ctx->stream);
    fail(EPSP_EDEVICE_TIMEOUT, "a tensor-core GEMM wait ran out in the warm-start network (bounded device wait)");
  }
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

static void adam(Mlp* P, float lr) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  step_kernel<<<1, 1, 0, s>>>(P->d_step.p);
  EPSP_LAUNCHED(ctx);
  for (int l = 0; l < P->L; ++l) {
    const long nw = long(P->dims[size_t(l)]) * P->dims[size_t(l + 1)], nb = P->dims[size_t(l + 1)];
    adam_kernel<<<div_up(size_t(nw), 256), 256, 0, s>>>(
        P->W[size_t(l)].p, P->gW[size_t(l)].p, P->mW[size_t(l)].p, P->vW[size_t(l)].p, nw, lr, b1, b2, eps, P->d_step.p,
        P->Wbf[size_t(l)].p, P->dims[size_t(l)], P->tr.Wp[size_t(l)].p, P->tr.dp[size_t(l)], P->tr.WT[size_t(l)].p,
        P->tr.dp[size_t(l + 1)]);
    EPSP_LAUNCHED(ctx);
    adam_kernel<<<div_up(size_t(nb), 256), 256, 0, s>>>(P->b[size_t(l)].p, P->gb[size_t(l)].p, P->mb[size_t(l)].p,
                                                        P->vb[size_t(l)].p, nb, lr, b1, b2, eps, P->d_step.p, nullptr, 1,
                                                        nullptr, 0, nullptr, 0);
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
  if (tc_err) {
    forward_tc(&P, ni, tc_err);
  } else {
    forward_train(&P, ni, false);
    check_mlp_err(&P);
  }
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
    P.d_err.alloc(P.ctx, 1);
    P.d_err.zero(P.ctx->stream);
    train_weights_init(&P);
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

/* Device milliseconds of the epochs of the last epsp_warmstart_train (CUDA events around each
 * epoch's graph replay; the uploads and the capture are not included). */
double epsp_warmstart_train_ms(const epsp_warmstart* w) { return w ? w->m.train_ms : 0.0; }

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
      to_bf16_kernel<<<div_up(size_t(nw), 256), 256, 0, s>>>(P.W[size_t(l)].p, nw, P.dims[size_t(l)], P.Wbf[size_t(l)].p,
                                                             P.tr.Wp[size_t(l)].p, P.tr.dp[size_t(l)],
                                                             P.tr.WT[size_t(l)].p, P.tr.dp[size_t(l + 1)]);
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
      forward_train(&P, nb, false);
      P.X[size_t(P.L)].download(Y + r0 * P.dims.back(), size_t(nb * P.dims.back()), s);
    }
    check_mlp_err(&P);
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
    forward_train(&P, n, true);
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
    check_mlp_err(&P);
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
        forward_train(&P, nb, true);
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
    // one gradient pass on the first minibatch outside the capture (no parameter update), so that
    // every kernel's launch attributes are set before the capture
    {
      const long nb = std::min<long>(batch, n);
      d_perm.upload(perm ? perm : ident.data(), size_t(n), s);
      gather_rows_kernel<<<div_up(size_t(nb * d0), 256), 256, 0, s>>>(P.dataX.p, d_perm.p, nb, d0, P.X[0].p);
      EPSP_LAUNCHED(P.ctx);
      gather_rows_kernel<<<div_up(size_t(nb * dl), 256), 256, 0, s>>>(P.dataY.p, d_perm.p, nb, dl, P.Yb.p);
      EPSP_LAUNCHED(P.ctx);
      forward_train(&P, nb, true);
      backward(&P, nb, nb, 0);
      check_mlp_err(&P);
    }
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
    cudaEvent_t ev[2] = {nullptr, nullptr};
    struct EventGuard {
      cudaEvent_t* e;
      ~EventGuard() {
        for (int k = 0; k < 2; ++k)
          if (e[k]) cudaEventDestroy(e[k]);
      }
    } eguard{ev};
    for (auto& e : ev) EPSP_CUDA(cudaEventCreate(&e));
    P.train_ms = 0;
    for (int e = 0; e < epochs; ++e) {
      d_perm.upload(perm ? perm + long(e) * n : ident.data(), size_t(n), s);
      EPSP_CUDA(cudaEventRecord(ev[0], s));
      EPSP_CUDA(cudaGraphLaunch(exec, s));
      EPSP_CUDA(cudaEventRecord(ev[1], s));
      P.ctx->launches += per_epoch;
      P.loss_sum.download(bl.data(), size_t(nbat), s);
      check_mlp_err(&P);
      float ms = 0;
      EPSP_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
      P.train_ms += double(ms);
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
