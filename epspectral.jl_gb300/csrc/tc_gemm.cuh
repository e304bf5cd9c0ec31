// tc_gemm.cuh -- BF16x3 split-precision GEMM on the sm_103a tensor cores (tcgen05 + TMA + TMEM).
//
//   D[m, n] (FP32) = Σ_k A[m, k] B[n, k]   with   A ≈ A_hi + A_lo,  B ≈ B_hi + B_lo  (BF16 each)
//   evaluated as A_hi·B_hi + A_hi·B_lo + A_lo·B_hi, all three products accumulated in one TMEM
//   accumulator (FP32). A [M][K] and B [N][K] are row-major with K contiguous ("K-major"), row
//   stride `ldk` elements (a multiple of 8, so rows start on 16-byte boundaries).
//
// One CTA of 128 threads computes a 128 x BN tile of D over a range of 64-wide K blocks (split-K
// over blockIdx.z; each split writes its own FP32 slab, summed afterwards in fixed order):
//   warp 0, lane 0 : TMA producer, a ring of STAGES stages [A_hi | A_lo | B_hi | B_lo] with
//                    128-byte swizzle, completion through mbarriers (expect_tx);
//   warp 1, lane 0 : issues tcgen05.mma (M = 128, N = BN, K = 16 per instruction, three per K step)
//                    and tcgen05.commit to release a stage and, at the end, to signal the epilogue;
//   warps 0-3      : epilogue, tcgen05.ld of TMEM lanes 32w..32w+31 into registers, masked stores.
// Every mbarrier wait is bounded; on timeout the kernel records the error in *err and winds down
// (waits, again bounded, for its own copies and MMAs, frees TMEM and returns).
#pragma once

#include "common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <vector>

namespace epsp {

constexpr int kTcBM = 128, kTcBK = 64;
constexpr unsigned kWaitLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred P1;\nmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\nselp.b32 %0, 1, 0, P1;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of parity `parity` to complete; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (unsigned it = 0; it < kWaitLimit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it > 64) __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile with 128-byte swizzle: rows of 128 B
// (64 BF16), 8-row groups 1024 B apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return uint64_t((addr >> 4) & 0x3FFF) | (uint64_t(1024 >> 4) << 32) | (uint64_t(1) << 46) | (uint64_t(2) << 61);
}
// The same with 64-byte swizzle: rows of 64 B (32 BF16), 8-row groups 512 B apart.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t addr) {
  return uint64_t((addr >> 4) & 0x3FFF) | (uint64_t(512 >> 4) << 32) | (uint64_t(1) << 46) | (uint64_t(4) << 61);
}
// The descriptor for K blocks of BK elements (64: 128-byte rows, 32: 64-byte rows).
template <int BK>
__device__ __forceinline__ uint64_t sw_desc(uint32_t addr) {
  if constexpr (BK == 64)
    return sw128_desc(addr);
  else
    return sw64_desc(addr);
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(128 >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 lanes x 32 columns of 32-bit values from TMEM: thread `lane` gets row (lane base + lane),
// columns col..col+31.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,"
      "%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// NS = 2: operands split x = x0 + x1 (hi, lo), products 00, 01, 10 (BF16x3, ~2^-16 relative);
// NS = 3: x = x0 + x1 + x2 (hi, mid, lo), products 00, 01, 10, 02, 11, 20 (six, ~2^-23 relative).
template <int BN, int STAGES, int NS, int BK = kTcBK>
struct TcSmem {
  static constexpr int kA = kTcBM * BK * 2;   // bytes of one A tile
  static constexpr int kB = BN * BK * 2;      // bytes of one B tile
  static constexpr int kStage = NS * kA + NS * kB;
  static constexpr int kBars = 2 * STAGES + 1;
  static constexpr int kBytes = STAGES * kStage + 8 * kBars + 16 + 1024;  // + alignment slack
};

struct TcMaps {
  CUtensorMap a[3], b[3];
};

template <int BN, int STAGES, int NS, int BK = kTcBK>
__global__ void __launch_bounds__(128, 1)
    tc_gemm_split_kernel(const __grid_constant__ TcMaps maps, int M, int N, int kblocks, int kb_per_split,
                         float* __restrict__ out, long ld_out, long split_stride, int* __restrict__ err) {
  using L = TcSmem<BN, STAGES, NS, BK>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * L::kStage);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + L::kBars);
  __shared__ int s_abort;
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES), done_bar = smem_u32(bars + 2 * STAGES);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  // N tiles vary fastest over the launch order, so the CTAs resident together share A tiles
  // (the large operand) through L2 and A streams from DRAM about once
  const int n0 = blockIdx.x * BN, m0 = blockIdx.y * kTcBM;
  const int kb0 = blockIdx.z * kb_per_split;
  const int nkb = max(0, min(kblocks, kb0 + kb_per_split) - kb0);

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < 2 * STAGES + 1; ++s) mbar_init(smem_u32(bars + s), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)), "r"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer
    int issued = 0;
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % STAGES;
      const uint32_t ph = (kb / STAGES) & 1;
      if (kb >= STAGES && !mbar_wait(empty0 + 8 * s, ph ^ 1)) {
        atomicExch(&s_abort, 1);
        break;
      }
      if (*(volatile int*)&s_abort) break;
      uint8_t* st = smem + s * L::kStage;
      const uint32_t fb = full0 + 8 * s;
      mbar_expect_tx(fb, L::kStage);
      const int kc = (kb0 + kb) * BK;
#pragma unroll
      for (int p = 0; p < NS; ++p) {
        tma_load_2d(smem_u32(st + p * L::kA), &maps.a[p], kc, m0, fb);
        tma_load_2d(smem_u32(st + NS * L::kA + p * L::kB), &maps.b[p], kc, n0, fb);
      }
      issued = kb + 1;
    }
    if (*(volatile int*)&s_abort) {
      // wind down: wait (bounded) for the copies this thread issued into stages not yet consumed
      for (int kb = max(0, issued - STAGES); kb < issued; ++kb) mbar_wait(full0 + 8 * (kb % STAGES), (kb / STAGES) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = idesc_bf16_f32(BN);
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % STAGES;
      const uint32_t ph = (kb / STAGES) & 1;
      if (!mbar_wait(full0 + 8 * s, ph)) {
        atomicExch(&s_abort, 1);
        break;
      }
      if (*(volatile int*)&s_abort) break;
      tc_fence_after();
      const uint32_t a0 = smem_u32(smem + s * L::kStage);
      const uint32_t b0 = a0 + NS * L::kA;
#pragma unroll
      for (int ks = 0; ks < BK / 16; ++ks) {
        const uint32_t off = ks * 32;  // 16 BF16 along K inside the swizzled row
        // the split products of increasing order: 00; 01, 10; (NS = 3) 02, 11, 20
        umma_bf16(tmem, sw_desc<BK>(a0 + off), sw_desc<BK>(b0 + off), idesc, (kb | ks) != 0);
        umma_bf16(tmem, sw_desc<BK>(a0 + off), sw_desc<BK>(b0 + L::kB + off), idesc, 1);
        umma_bf16(tmem, sw_desc<BK>(a0 + L::kA + off), sw_desc<BK>(b0 + off), idesc, 1);
        if constexpr (NS == 3) {
          umma_bf16(tmem, sw_desc<BK>(a0 + off), sw_desc<BK>(b0 + 2 * L::kB + off), idesc, 1);
          umma_bf16(tmem, sw_desc<BK>(a0 + L::kA + off), sw_desc<BK>(b0 + L::kB + off), idesc, 1);
          umma_bf16(tmem, sw_desc<BK>(a0 + 2 * L::kA + off), sw_desc<BK>(b0 + off), idesc, 1);
        }
      }
      umma_commit(empty0 + 8 * s);
    }
    umma_commit(done_bar);  // completes when every MMA issued above has
  }
  __syncwarp();
  // epilogue
  bool ok = true;
  if (!mbar_wait(done_bar, 0)) {
    ok = false;
    atomicExch(&s_abort, 1);
  }
  tc_fence_after();
  __syncthreads();
  const bool aborted = *(volatile int*)&s_abort != 0;
  if (aborted && threadIdx.x == 0) atomicExch(err, 1);
  if (!aborted && ok) {
    const int row = m0 + warp * 32 + lane;
    float* o = out + long(blockIdx.z) * split_stride;
#pragma unroll 1
    for (int c = 0; c < BN; c += 32) {
      float v[32];
      tmem_ld32(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c), v);
      if (nkb == 0) {
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = 0.f;
      }
      if (row < M) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int n = n0 + c + j;
          if (n < N) o[row + ld_out * long(n)] = v[j];
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
}

// ---- persistent variant ----
// One CTA per SM runs the (N tile, M tile, split) items i = blockIdx.x, blockIdx.x + gridDim.x, ...
// (N tiles fastest, the launch order of the one-tile kernel), 192 threads:
//   warp 0, lane 0 : TMA producer; the operand ring runs on across items;
//   warp 1, lane 0 : MMA issuer; item t accumulates in TMEM columns (t % 2) BN.. (two accumulators);
//   warps 2-5      : epilogue of item t (TMEM lane quarter = warp % 4) while the MMAs of item t + 1
//                    run into the other accumulator; they release an accumulator by one arrive each.
// Per tile the MMAs run in the one-tile kernel's order, so the results are bitwise the same.
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

template <int BN, int STAGES, int NS, int BK>
struct TcPSmem {
  static constexpr int kA = kTcBM * BK * 2;
  static constexpr int kB = BN * BK * 2;
  static constexpr int kStage = NS * kA + NS * kB;
  static constexpr int kBars = 2 * STAGES + 5;  // full, empty, accumulator full x2, empty x2, done
  static constexpr int kBytes = STAGES * kStage + 8 * kBars + 16 + 1024;
};

template <int BN, int STAGES, int NS, int BK>
__global__ void __launch_bounds__(192, 1)
    tc_gemm_persist_kernel(const __grid_constant__ TcMaps maps, int M, int N, int kblocks, int kb_per_split, int nN,
                           int nM, int nitems, float* __restrict__ out, long ld_out, long split_stride,
                           int* __restrict__ err) {
  using L = TcPSmem<BN, STAGES, NS, BK>;
  static_assert(2 * BN <= 512, "two accumulators must fit TMEM");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * L::kStage);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + L::kBars);
  __shared__ int s_abort;
  const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * STAGES, accf0 = full0 + 16 * STAGES,
                 acce0 = accf0 + 16, done_bar = accf0 + 32;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  auto coords = [&](int item, int& n0, int& m0, int& z, int& kb0, int& nkb) {
    n0 = (item % nN) * BN;
    m0 = ((item / nN) % nM) * kTcBM;
    z = item / (nN * nM);
    kb0 = z * kb_per_split;
    nkb = max(0, min(kblocks, kb0 + kb_per_split) - kb0);
  };
  auto aborted = [&] { return *(volatile int*)&s_abort != 0; };

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < 2 * STAGES; ++s) mbar_init(smem_u32(bars + s), 1);
    mbar_init(accf0, 1);
    mbar_init(accf0 + 8, 1);
    mbar_init(acce0, 4);
    mbar_init(acce0 + 8, 4);
    mbar_init(done_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer
    int g = 0;
    bool stop = false;
    for (int item = blockIdx.x; item < nitems && !stop; item += gridDim.x) {
      int n0, m0, z, kb0, nkb;
      coords(item, n0, m0, z, kb0, nkb);
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = g % STAGES;
        const uint32_t ph = (g / STAGES) & 1;
        if (g >= STAGES && !mbar_wait(empty0 + 8 * s, ph ^ 1)) {
          atomicExch(&s_abort, 1);
          stop = true;
          break;
        }
        if (aborted()) {
          stop = true;
          break;
        }
        uint8_t* st = smem + s * L::kStage;
        const uint32_t fb = full0 + 8 * s;
        mbar_expect_tx(fb, L::kStage);
        const int kc = (kb0 + kb) * BK;
#pragma unroll
        for (int p = 0; p < NS; ++p) {
          tma_load_2d(smem_u32(st + p * L::kA), &maps.a[p], kc, m0, fb);
          tma_load_2d(smem_u32(st + NS * L::kA + p * L::kB), &maps.b[p], kc, n0, fb);
        }
        ++g;
      }
    }
    if (aborted()) {
      // wind down: wait (bounded) for the copies this thread issued into stages not yet consumed
      for (int k = max(0, g - STAGES); k < g; ++k) mbar_wait(full0 + 8 * (k % STAGES), (k / STAGES) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = idesc_bf16_f32(BN);
    int g = 0, t = 0;
    bool stop = false;
    for (int item = blockIdx.x; item < nitems && !stop; item += gridDim.x, ++t) {
      int n0, m0, z, kb0, nkb;
      coords(item, n0, m0, z, kb0, nkb);
      const int b = t & 1;
      const uint32_t acc = tmem + uint32_t(b * BN);
      if (t >= 2 && !mbar_wait(acce0 + 8 * b, ((t >> 1) & 1) ^ 1)) {  // the epilogue drained it
        atomicExch(&s_abort, 1);
        break;
      }
      tc_fence_after();
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = g % STAGES;
        const uint32_t ph = (g / STAGES) & 1;
        if (!mbar_wait(full0 + 8 * s, ph)) {
          atomicExch(&s_abort, 1);
          stop = true;
          break;
        }
        if (aborted()) {
          stop = true;
          break;
        }
        tc_fence_after();
        const uint32_t a0 = smem_u32(smem + s * L::kStage);
        const uint32_t b0 = a0 + NS * L::kA;
#pragma unroll
        for (int ks = 0; ks < BK / 16; ++ks) {
          const uint32_t off = ks * 32;
          umma_bf16(acc, sw_desc<BK>(a0 + off), sw_desc<BK>(b0 + off), idesc, (kb | ks) != 0);
          if constexpr (NS >= 2) {
            umma_bf16(acc, sw_desc<BK>(a0 + off), sw_desc<BK>(b0 + L::kB + off), idesc, 1);
            umma_bf16(acc, sw_desc<BK>(a0 + L::kA + off), sw_desc<BK>(b0 + off), idesc, 1);
          }
          if constexpr (NS == 3) {
            umma_bf16(acc, sw_desc<BK>(a0 + off), sw_desc<BK>(b0 + 2 * L::kB + off), idesc, 1);
            umma_bf16(acc, sw_desc<BK>(a0 + L::kA + off), sw_desc<BK>(b0 + L::kB + off), idesc, 1);
            umma_bf16(acc, sw_desc<BK>(a0 + 2 * L::kA + off), sw_desc<BK>(b0 + off), idesc, 1);
          }
        }
        umma_commit(empty0 + 8 * s);
        ++g;
      }
      umma_commit(accf0 + 8 * b);  // completes when the item's MMAs have
    }
    umma_commit(done_bar);  // completes when every MMA issued above has
  } else if (warp >= 2) {
    // epilogue
    const int q = warp % 4;
    int t = 0;
    for (int item = blockIdx.x; item < nitems; item += gridDim.x, ++t) {
      if (aborted()) break;
      int n0, m0, z, kb0, nkb;
      coords(item, n0, m0, z, kb0, nkb);
      const int b = t & 1;
      if (!mbar_wait(accf0 + 8 * b, (t >> 1) & 1)) {
        atomicExch(&s_abort, 1);
        break;
      }
      tc_fence_after();
      if (aborted()) break;
      const int row = m0 + q * 32 + lane;
      float* o = out + long(z) * split_stride;
#pragma unroll 1
      for (int c = 0; c < BN; c += 32) {
        float v[32];
        tmem_ld32(tmem + (uint32_t(q * 32) << 16) + uint32_t(b * BN + c), v);
        if (nkb == 0) {
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = 0.f;
        }
        if (row < M) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int n = n0 + c + j;
            if (n < N) o[row + ld_out * long(n)] = v[j];
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acce0 + 8 * b);
    }
  }
  __syncwarp();
  // every MMA issued has completed before TMEM is freed (bounded)
  if (!mbar_wait(done_bar, 0)) atomicExch(&s_abort, 1);
  tc_fence_after();
  __syncthreads();
  if (aborted() && threadIdx.x == 0) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN));
}

// ---- host side ----

// A 2-D BF16 tensor map over a row-major [rows][ld] array (K contiguous, rows of `cols` valid
// elements), box = 64 x box_rows, 128-byte swizzle; out-of-range elements read as zero.
// A 2-D tensor map of a row-major BF16 matrix [rows][cols] (row stride ld elements) whose box is
// bk columns (64: 128-byte swizzle; 32: 64-byte swizzle) by box_rows rows.
CUtensorMap make_tmap_bf16(const void* base, long rows, long cols, long ld, int box_rows, int bk = kTcBK);

// The BF16 parts of one operand: ns = 2 (hi, lo) or 3 (hi, mid, lo) tensor maps.
struct TcOperand {
  CUtensorMap m[3];
  int ns = 2;
  int bk = kTcBK;  // K columns of the maps' box
};

// Launches the split-precision product of A [M][K] and B [N][K] (K-major, both split into A.ns
// parts) into the FP32 slabs out[split][m + ld_out n]; returns the number of splits used. With
// kb_cap > 0 no FP32 accumulator sums more than kb_cap K-blocks of 64 (splits are added to bound
// the accumulation error of long same-sign sums), within max_splits.
int tc_gemm_launch(Ctx* ctx, const TcOperand& A, const TcOperand& B, int M, int N, int K, float* out, long ld_out,
                   long split_stride, int max_splits, int* d_err, const char* prof_name = "tc_gemm", int kb_cap = 0);

// The BN and split count tc_gemm_launch picks for (M, N, K), ns parts, at most max_splits splits.
void tc_gemm_shape(Ctx* ctx, int M, int N, int K, int max_splits, int ns, int* bn, int* splits, int kb_cap = 0);

// Launch with an explicit tile width bn (128: three pipeline stages; 256: two; two-part operands
// only) and split count (0: the heuristic's count for that bn); B's tensor maps must have boxes of
// bn rows. Returns the splits used.
int tc_gemm_launch_with(Ctx* ctx, const TcOperand& A, const TcOperand& B, int bn, int splits, int M, int N, int K,
                        float* out, long ld_out, long split_stride, int* d_err, const char* prof_name = "tc_gemm",
                        bool persist = false);
// The variant with K blocks of 32 (64-byte swizzle) and four pipeline stages, bn = 256; A and B
// maps built with bk = 32.

// The split count tc_gemm_launch_with uses for splits = 0.
int tc_splits_for(Ctx* ctx, int M, int N, int K, int bn);

// One measured candidate of the autotuner.
struct TcTune {
  int bn = 0, splits = 0, bk = kTcBK;
  float ms = 0.f;
  bool persist = false;  // the persistent kernel (one CTA per SM, two accumulators)
};

// The autotuner: times every candidate tile shape (bn 128 with three stages, bn 256 with two; the
// heuristic split count and twice it, within max_splits) of one two-part product on its own
// operands -- CUDA events on ctx's stream, one untimed and `reps` timed launches each -- and returns
// the fastest; every candidate's time goes to *all when given. B128 / B256: B's maps with boxes of
// 128 / 256 rows.
TcTune tc_gemm_autotune(Ctx* ctx, const TcOperand& A, const TcOperand& B128, const TcOperand& B256, int M, int N, int K,
                        float* out, long ld_out, long split_stride, int max_splits, int* d_err, int reps,
                        std::vector<TcTune>* all = nullptr, const TcOperand* A32 = nullptr,
                        const TcOperand* B256_32 = nullptr);

// x = Σ_p x_p with x_p BF16, p < ns (round to nearest at every step).
__device__ __forceinline__ void split_bf16_n(float x, int ns, __nv_bfloat16* out) {
  float r = x;
  for (int p = 0; p < ns; ++p) {
    __nv_bfloat16 h = __float2bfloat16_rn(r);
    out[p] = h;
    r -= __bfloat162float(h);
  }
}

}  // namespace epsp
