// gemm_f64.cuh -- FP64 SIMT GEMM for the FP64 paths (the Kramers-Kronig map, the recast
// Fan-Migdal contraction and the ladder's shift sums in FP64).
//
// C[M, N] = alpha * op(A)[M, K] * B[K, N] + beta * C, column-major with leading dimensions; op(A)
// is A or A^T. 64x64 tiles, 256 threads with 4x4 outputs each, K staged 16 at a time in shared
// memory; each output sums its K terms in ascending order, so the result is bitwise reproducible.
// GB300's FP64 rate is ~1.25 TFLOP/s for the whole chip, so this is the plain baseline, not a fast
// path.
#pragma once

#include "common.cuh"

namespace epsp {

template <bool TRANS_A>
__global__ void __launch_bounds__(256) gemm_f64_kernel(int M, int N, int K, double alpha, const double* __restrict__ A,
                                                       long lda, const double* __restrict__ B, long ldb, double beta,
                                                       double* __restrict__ C, long ldc) {
  __shared__ double As[16][64 + 1];
  __shared__ double Bs[16][64 + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  double acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 16) {
    // A tile: 64 rows x 16 k; B tile: 16 k x 64 cols. 1024 elements each, 4 per thread.
    for (int r = threadIdx.x; r < 1024; r += 256) {
      int kk = r / 64, mm = r % 64;
      int gm = m0 + mm, gk = k0 + kk;
      double a = 0;
      if (gm < M && gk < K) a = TRANS_A ? A[gk + lda * long(gm)] : A[gm + lda * long(gk)];
      As[kk][mm] = a;
      int nn = r / 16, kb = r % 16;
      int gn = n0 + nn, gk2 = k0 + kb;
      Bs[kb][nn] = (gn < N && gk2 < K) ? B[gk2 + ldb * long(gn)] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][tx + 16 * u];
        b[u] = Bs[kk][ty + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      int gm = m0 + tx + 16 * u, gn = n0 + ty + 16 * v;
      if (gm < M && gn < N) {
        double* c = C + gm + ldc * long(gn);
        *c = beta == 0 ? alpha * acc[u][v] : alpha * acc[u][v] + beta * *c;
      }
    }
}

inline void gemm_f64(Ctx* ctx, bool transA, int M, int N, int K, double alpha, const double* A, long lda,
                     const double* B, long ldb, double beta, double* C, long ldc) {
  if (M <= 0 || N <= 0) return;
  dim3 grid(div_up(size_t(M), 64), div_up(size_t(N), 64));
  if (transA)
    gemm_f64_kernel<true><<<grid, 256, 0, ctx->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  else
    gemm_f64_kernel<false><<<grid, 256, 0, ctx->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  EPSP_LAUNCHED(ctx);
}

}  // namespace epsp
