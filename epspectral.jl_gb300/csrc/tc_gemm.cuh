// tc_gemm.cuh -- split-precision and TF32 GEMMs on the sm_103a tensor cores (tcgen05 + TMA + TMEM).
//
//   D[m, n] (FP32) = Σ_k A[m, k] B[n, k]   with   A ≈ A_hi + A_lo,  B ≈ B_hi + B_lo  (BF16 each)
//   evaluated as A_hi·B_hi + A_hi·B_lo + A_lo·B_hi, all three products accumulated in one TMEM
//   accumulator (FP32). A [M][K] and B [N][K] are row-major with K contiguous ("K-major"), row
//   stride `ldk` elements (a multiple of 8, so rows start on 16-byte boundaries).
//   The TF32 variant (TF32 = true, one part per operand) runs one kind::tf32 product of FP32
//   operands already rounded to TF32 (10-bit mantissa): half the BF16 rate per product, so two
//   thirds of the BF16x3 tensor time for the same operand bytes, at ~2^-11 relative per element.
//
// One CTA of 128 threads computes a 128 x BN tile of D over a range of 64-wide K blocks (split-K
// over blockIdx.z; each split writes its own FP32 slab, summed afterwards in fixed order):
//   warp 0, lane 0 : TMA producer, a ring of STAGES stages [A_hi | A_lo | B_hi | B_lo] with
//                    128-byte swizzle, completion through mbarriers (expect_tx);
//   warp 1, lane 0 : issues tcgen05.mma (M = 128, N = BN, K = 16 per instruction, three per K step)
//                    and tcgen05.commit to release a stage and, at the end, to signal the epilogue;
//   warps 0-3      : epilogue, tcgen05.ld of TMEM lanes 32w..32w+31 into registers, masked stores.
// Every mbarrier wait is bounded; on timeout the kernel records the error in *err and winds down
// (waits, again bounded, for its own copies and MMAs, frees TMEM and returns). The one-CTA kernel
// takes its pipeline waits' limit as an argument, and a K block its producer skips (a test hook:
// the wait for that block's copies then runs out; the wind-down waits keep the full limit, and the
// epilogue's wait for the MMAs ends when the MMA thread, which always commits, gives up).
// Two more kernels below share that pipeline: the persistent one (a CTA per SM over all tiles,
// two TMEM accumulators) and the CTA-pair one (tcgen05 cta_group::2: a 256-row tile over two CTAs,
// each holding half of B). Every TMA load reads this GPU's own memory into the issuing CTA's
// shared memory (no multicast).
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
// Bounded wait for the phase of parity `parity` to complete; false after `limit` tries.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned limit = kWaitLimit) {
  for (unsigned it = 0; it < limit; ++it) {
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
__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// Every thread of every CTA of the cluster (a hardware barrier; all of them reach it).
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// The (N tile, M tile) of tile index L (0 <= L < nN nM) in launch order. gm <= 1: N tiles fastest
// (CTAs resident together share one A tile and sweep B). gm > 1: grouped order, the M tiles of a
// group of gm run fastest and the group sweeps every N tile before the next group starts, so a
// group's A tiles stay in L2 while B streams once per group -- for products whose B operand is too
// large to stay in L2 across the M tiles.
__device__ __forceinline__ void tile_of(int L, int nN, int nM, int gm, int& nt, int& mt) {
  if (gm <= 1) {
    nt = L % nN;
    mt = L / nN;
    return;
  }
  const int per = gm * nN, g = L / per, r = L % per;
  const int rows = min(gm, nM - g * gm);
  mt = g * gm + r % rows;
  nt = r / rows;
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
// The descriptor for K rows of RB bytes (128: 64 BF16 or 32 TF32; 64: 32 BF16).
template <int RB>
__device__ __forceinline__ uint64_t sw_desc(uint32_t addr) {
  static_assert(RB == 128 || RB == 64, "K rows of 128 or 64 bytes");
  if constexpr (RB == 128)
    return sw128_desc(addr);
  else
    return sw64_desc(addr);
}

// Instruction descriptor of kind::f16 (A and B BF16) or kind::tf32 (A and B TF32): D FP32, both
// K-major, M = 128, N = n.
template <bool TF32 = false>
__host__ __device__ constexpr uint32_t idesc_f32acc(int n) {
  return (1u << 4) | ((TF32 ? 2u : 1u) << 7) | ((TF32 ? 2u : 1u) << 10) | (uint32_t(n >> 3) << 17) |
         (uint32_t(128 >> 4) << 24);
}

// One MMA: K = 16 BF16 (kind::f16) or K = 8 TF32 (kind::tf32), 32 bytes of each operand row.
template <bool TF32 = false>
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  if constexpr (TF32)
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
  else
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

// x rounded to TF32 (nearest, ties away from zero), as an FP32 value with the low 13 bits zero.
__device__ __forceinline__ float round_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
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
// NS = 3: x = x0 + x1 + x2 (hi, mid, lo), products 00, 01, 10, 02, 11, 20 (six, ~2^-23 relative);
// NS = 1 with TF32: one TF32 product. BK counts elements (2 bytes, or 4 with TF32) per K row.
template <int BN, int STAGES, int NS, int BK = kTcBK, bool TF32 = false>
struct TcSmem {
  static constexpr int kES = TF32 ? 4 : 2;     // bytes per element
  static constexpr int kRB = BK * kES;         // bytes of one K row
  static constexpr int kA = kTcBM * kRB;       // bytes of one A tile
  static constexpr int kB = BN * kRB;          // bytes of one B tile
  static constexpr int kStage = NS * kA + NS * kB;
  static constexpr int kBars = 2 * STAGES + 1;
  static constexpr int kBytes = STAGES * kStage + 8 * kBars + 16 + 1024;  // + alignment slack
};

struct TcMaps {
  CUtensorMap a[3], b[3];
};

template <int BN, int STAGES, int NS, int BK = kTcBK, bool TF32 = false>
__global__ void __launch_bounds__(128, 1)
    tc_gemm_split_kernel(const __grid_constant__ TcMaps maps, int M, int N, int kblocks, int kb_per_split,
                         float* __restrict__ out, long ld_out, long split_stride, int* __restrict__ err, int gm = 1,
                         int skip_kb = -1, unsigned wait_limit = kWaitLimit) {
  using L = TcSmem<BN, STAGES, NS, BK, TF32>;
  static_assert(!TF32 || NS == 1, "TF32 operands have one part");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * L::kStage);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + L::kBars);
  __shared__ int s_abort;
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES), done_bar = smem_u32(bars + 2 * STAGES);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  // N tiles vary fastest over the launch order (gm <= 1), so the CTAs resident together share A
  // tiles (the large operand) through L2 and A streams from DRAM about once; gm > 1 groups M tiles
  int nt, mt;
  tile_of(int(blockIdx.y) * int(gridDim.x) + int(blockIdx.x), int(gridDim.x), int(gridDim.y), gm, nt, mt);
  const int n0 = nt * BN, m0 = mt * kTcBM;
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
      if (kb == skip_kb) continue;  // test hook: this K block's copies are never issued
      const int s = kb % STAGES;
      const uint32_t ph = (kb / STAGES) & 1;
      if (kb >= STAGES && !mbar_wait(empty0 + 8 * s, ph ^ 1, wait_limit)) {
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
      // (a skipped K block's stage is never reused: the wait for its release runs out first)
      for (int kb = max(0, issued - STAGES); kb < issued; ++kb)
        if (kb != skip_kb) mbar_wait(full0 + 8 * (kb % STAGES), (kb / STAGES) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = idesc_f32acc<TF32>(BN);
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % STAGES;
      const uint32_t ph = (kb / STAGES) & 1;
      if (!mbar_wait(full0 + 8 * s, ph, wait_limit)) {
        atomicExch(&s_abort, 1);
        break;
      }
      if (*(volatile int*)&s_abort) break;
      tc_fence_after();
      const uint32_t a0 = smem_u32(smem + s * L::kStage);
      const uint32_t b0 = a0 + NS * L::kA;
#pragma unroll
      for (int ks = 0; ks < L::kRB / 32; ++ks) {
        const uint32_t off = ks * 32;  // 16 BF16 (8 TF32) along K inside the swizzled row
        // the split products of increasing order: 00; 01, 10; (NS = 3) 02, 11, 20
        umma<TF32>(tmem, sw_desc<L::kRB>(a0 + off), sw_desc<L::kRB>(b0 + off), idesc, (kb | ks) != 0);
        if constexpr (NS >= 2) {
          umma<TF32>(tmem, sw_desc<L::kRB>(a0 + off), sw_desc<L::kRB>(b0 + L::kB + off), idesc, 1);
          umma<TF32>(tmem, sw_desc<L::kRB>(a0 + L::kA + off), sw_desc<L::kRB>(b0 + off), idesc, 1);
        }
        if constexpr (NS == 3) {
          umma<TF32>(tmem, sw_desc<L::kRB>(a0 + off), sw_desc<L::kRB>(b0 + 2 * L::kB + off), idesc, 1);
          umma<TF32>(tmem, sw_desc<L::kRB>(a0 + L::kA + off), sw_desc<L::kRB>(b0 + L::kB + off), idesc, 1);
          umma<TF32>(tmem, sw_desc<L::kRB>(a0 + 2 * L::kA + off), sw_desc<L::kRB>(b0 + off), idesc, 1);
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

template <int BN, int STAGES, int NS, int BK, bool TF32 = false>
struct TcPSmem {
  static constexpr int kES = TF32 ? 4 : 2;
  static constexpr int kRB = BK * kES;
  static constexpr int kA = kTcBM * kRB;
  static constexpr int kB = BN * kRB;
  static constexpr int kStage = NS * kA + NS * kB;
  static constexpr int kBars = 2 * STAGES + 5;  // full, empty, accumulator full x2, empty x2, done
  static constexpr int kBytes = STAGES * kStage + 8 * kBars + 16 + 1024;
};

template <int BN, int STAGES, int NS, int BK, bool TF32 = false>
__global__ void __launch_bounds__(192, 1)
    tc_gemm_persist_kernel(const __grid_constant__ TcMaps maps, int M, int N, int kblocks, int kb_per_split, int nN,
                           int nM, int nitems, float* __restrict__ out, long ld_out, long split_stride,
                           int* __restrict__ err, int gm = 1) {
  using L = TcPSmem<BN, STAGES, NS, BK, TF32>;
  static_assert(!TF32 || NS == 1, "TF32 operands have one part");
  static_assert(2 * BN <= 512, "two accumulators must fit TMEM");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * L::kStage);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + L::kBars);
  __shared__ int s_abort;
  const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * STAGES, accf0 = full0 + 16 * STAGES,
                 acce0 = accf0 + 16, done_bar = accf0 + 32;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int first = int(blockIdx.x), stride = int(gridDim.x);  // this CTA's items
  auto coords = [&](int item, int& n0, int& m0, int& z, int& kb0, int& nkb) {
    int nt, mt;
    tile_of(item % (nN * nM), nN, nM, gm, nt, mt);
    n0 = nt * BN;
    m0 = mt * kTcBM;
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
    for (int item = first; item < nitems && !stop; item += stride) {
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
    constexpr uint32_t idesc = idesc_f32acc<TF32>(BN);
    int g = 0, t = 0;
    bool stop = false;
    for (int item = first; item < nitems && !stop; item += stride, ++t) {
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
        for (int ks = 0; ks < L::kRB / 32; ++ks) {
          const uint32_t off = ks * 32;
          umma<TF32>(acc, sw_desc<L::kRB>(a0 + off), sw_desc<L::kRB>(b0 + off), idesc, (kb | ks) != 0);
          if constexpr (NS >= 2) {
            umma<TF32>(acc, sw_desc<L::kRB>(a0 + off), sw_desc<L::kRB>(b0 + L::kB + off), idesc, 1);
            umma<TF32>(acc, sw_desc<L::kRB>(a0 + L::kA + off), sw_desc<L::kRB>(b0 + off), idesc, 1);
          }
          if constexpr (NS == 3) {
            umma<TF32>(acc, sw_desc<L::kRB>(a0 + off), sw_desc<L::kRB>(b0 + 2 * L::kB + off), idesc, 1);
            umma<TF32>(acc, sw_desc<L::kRB>(a0 + L::kA + off), sw_desc<L::kRB>(b0 + L::kB + off), idesc, 1);
            umma<TF32>(acc, sw_desc<L::kRB>(a0 + 2 * L::kA + off), sw_desc<L::kRB>(b0 + off), idesc, 1);
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
    for (int item = first; item < nitems; item += stride, ++t) {
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

// ---- CTA-pair variant (tcgen05 cta_group::2) ----
// A cluster of two CTAs computes a 256 x BN tile: rank r holds A rows m0 + 128 r.. and B rows
// n0 + (BN / 2) r.. in its own shared memory (32 KB per TF32 stage instead of 48, so six stages fit
// where four did), and one thread of rank 0 (the leader) issues every MMA with M = 256, which reads
// both CTAs' operands and accumulates each CTA's 128 rows in that CTA's TMEM. Both CTAs' copies
// complete on the leader's full barrier (expect_tx of both stages, set by the leader); the leader's
// commits arrive on the empty barriers of both CTAs (each CTA's producer refills only its own
// stages) and on both done barriers. TMEM is allocated and freed by a warp of each CTA together.
// Per tile the K order is the one-tile kernel's, so the results are bitwise the same.
template <int BN, int STAGES, int NS, int BK, bool TF32>
struct TcPairSmem {
  static constexpr int kES = TF32 ? 4 : 2;
  static constexpr int kRB = BK * kES;
  static constexpr int kA = kTcBM * kRB;       // this CTA's 128 A rows
  static constexpr int kBh = (BN / 2) * kRB;   // this CTA's half of the B tile
  static constexpr int kStage = NS * kA + NS * kBh;
  static constexpr int kBars = 2 * STAGES + 1;  // full, empty, done
  static constexpr int kBytes = STAGES * kStage + 8 * kBars + 16 + 1024;
};

__device__ __forceinline__ uint32_t mapa_shared(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
// A tiled load into this CTA's shared memory completing on an mbarrier of either CTA of the pair.
__device__ __forceinline__ void tma_load_2d_pair(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}
template <bool TF32>
__device__ __forceinline__ void umma_pair(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  if constexpr (TF32)
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
  else
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit_pair(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(bar),
      "h"(uint16_t(3))
      : "memory");
}
// Instruction descriptor with M = 256 (the pair's tile).
template <bool TF32>
__host__ __device__ constexpr uint32_t idesc_pair(int n) {
  return (1u << 4) | ((TF32 ? 2u : 1u) << 7) | ((TF32 ? 2u : 1u) << 10) | (uint32_t(n >> 3) << 17) |
         (uint32_t(256 >> 4) << 24);
}

template <int BN, int STAGES, int NS, int BK, bool TF32>
__global__ void __launch_bounds__(128, 1)
    tc_gemm_pair_kernel(const __grid_constant__ TcMaps maps, int M, int N, int kblocks, int kb_per_split,
                        float* __restrict__ out, long ld_out, long split_stride, int* __restrict__ err, int gm = 1) {
  using L = TcPairSmem<BN, STAGES, NS, BK, TF32>;
  static_assert(!TF32 || NS == 1, "TF32 operands have one part");
  static_assert((BN / 2) % 8 == 0 && BN <= 256, "B halves of whole 8-row swizzle groups");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * L::kStage);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + L::kBars);
  __shared__ int s_abort;
  const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * STAGES, done_bar = full0 + 16 * STAGES;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const uint32_t rank = cluster_ctarank();  // 0: the leader, which issues the MMAs
  // clusters are consecutive blockIdx.x pairs; the pair's tile in the one-tile kernel's order (both
  // CTAs of a pair compute the same tile index)
  int nt, mt;
  tile_of(int(blockIdx.y) * int(gridDim.x >> 1) + int(blockIdx.x >> 1), int(gridDim.x >> 1), int(gridDim.y), gm, nt,
          mt);
  const int n0 = nt * BN, m0 = mt * 2 * kTcBM + int(rank) * kTcBM;
  const int kb0 = blockIdx.z * kb_per_split;
  const int nkb = max(0, min(kblocks, kb0 + kb_per_split) - kb0);

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < L::kBars; ++s) mbar_init(smem_u32(bars + s), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)), "r"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  cluster_sync_all();  // both CTAs' barriers initialised and TMEM allocated

  if (warp == 0 && lane == 0) {
    // producer: this CTA's A rows and B half, completing on the leader's full barrier
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
      const uint32_t fb = mapa_shared(full0 + 8 * s, 0);
      if (rank == 0) mbar_expect_tx(full0 + 8 * s, 2 * L::kStage);
      const int kc = (kb0 + kb) * BK;
#pragma unroll
      for (int p = 0; p < NS; ++p) {
        tma_load_2d_pair(smem_u32(st + p * L::kA), &maps.a[p], kc, m0, fb);
        tma_load_2d_pair(smem_u32(st + NS * L::kA + p * L::kBh), &maps.b[p], kc, n0 + int(rank) * (BN / 2), fb);
      }
      issued = kb + 1;
    }
    // the leader's last releases of this CTA's stages have landed (bounded)
    for (int kb = max(0, issued - STAGES); kb < issued; ++kb)
      if (!mbar_wait(empty0 + 8 * (kb % STAGES), (kb / STAGES) & 1)) {
        atomicExch(&s_abort, 1);
        break;
      }
  } else if (warp == 1 && lane == 0 && rank == 0) {
    // MMA issuer (leader only): M = 256 over both CTAs' operands
    constexpr uint32_t idesc = idesc_pair<TF32>(BN);
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
      for (int ks = 0; ks < L::kRB / 32; ++ks) {
        const uint32_t off = ks * 32;
        umma_pair<TF32>(tmem, sw_desc<L::kRB>(a0 + off), sw_desc<L::kRB>(b0 + off), idesc, (kb | ks) != 0);
        if constexpr (NS >= 2) {
          umma_pair<TF32>(tmem, sw_desc<L::kRB>(a0 + off), sw_desc<L::kRB>(b0 + L::kBh + off), idesc, 1);
          umma_pair<TF32>(tmem, sw_desc<L::kRB>(a0 + L::kA + off), sw_desc<L::kRB>(b0 + off), idesc, 1);
        }
      }
      umma_commit_pair(empty0 + 8 * s);  // the stage is free in both CTAs
    }
    umma_commit_pair(done_bar);  // both CTAs: every MMA issued above has completed
  }
  __syncwarp();
  // epilogue: this CTA's 128 rows from its own TMEM
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
  cluster_sync_all();  // neither CTA frees TMEM or leaves while its peer still runs
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
}

// ---- persistent CTA-pair variant ----
// The CTA-pair kernel run persistently: cluster p of two CTAs takes the items (pair of M tiles,
// N tile, split) i = p, p + npairs, ... in the one-tile kernel's order, with two TMEM accumulators
// of BN columns per CTA (allocated by both CTAs together), so that both CTAs' epilogues drain item
// t while the leader's products run item t + 1. Barriers: full (the leader's: both CTAs' copies
// of a stage, as in the one-tile pair kernel), empty and accumulator-full (each CTA's, from the
// leader's commits to both), accumulator-empty (the leader's: eight arrivals, the four epilogue
// warps of each CTA, the peer's through their cluster addresses), done. 192 threads: warp 0 the
// producer, warp 1 the leader's MMA issuer, warps 2-5 the epilogue (TMEM lanes 32 (warp % 4)..).
template <int BN, int STAGES, int NS, int BK, bool TF32>
struct TcPairPSmem {
  static constexpr int kES = TF32 ? 4 : 2;
  static constexpr int kRB = BK * kES;
  static constexpr int kA = kTcBM * kRB;        // this CTA's 128 A rows
  static constexpr int kBh = (BN / 2) * kRB;    // this CTA's half of the B tile
  static constexpr int kStage = NS * kA + NS * kBh;
  static constexpr int kBars = 2 * STAGES + 5;  // full, empty, accumulator full x2, empty x2, done
  static constexpr int kBytes = STAGES * kStage + 8 * kBars + 16 + 1024;
};

// Arrival on an mbarrier of another CTA of the cluster (addr from mapa).
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(addr) : "memory");
}

template <int BN, int STAGES, int NS, int BK, bool TF32>
__global__ void __launch_bounds__(192, 1)
    tc_gemm_pair_persist_kernel(const __grid_constant__ TcMaps maps, int M, int N, int kblocks, int kb_per_split,
                                int nN, int nM2, int nitems, float* __restrict__ out, long ld_out, long split_stride,
                                int* __restrict__ err, int gm = 1) {
  using L = TcPairPSmem<BN, STAGES, NS, BK, TF32>;
  static_assert(!TF32 || NS == 1, "TF32 operands have one part");
  static_assert((BN / 2) % 8 == 0 && 2 * BN <= 512, "B halves of whole 8-row swizzle groups; two accumulators");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * L::kStage);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + L::kBars);
  __shared__ int s_abort;
  const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * STAGES, accf0 = full0 + 16 * STAGES,
                 acce0 = accf0 + 16, done_bar = accf0 + 32;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const uint32_t rank = cluster_ctarank();  // 0: the leader, which issues the MMAs
  const int pair = int(blockIdx.x >> 1), npairs = int(gridDim.x >> 1);
  auto coords = [&](int item, int& n0, int& m0, int& z, int& kb0, int& nkb) {
    int nt, mt;
    tile_of(item % (nN * nM2), nN, nM2, gm, nt, mt);
    n0 = nt * BN;
    m0 = mt * 2 * kTcBM + int(rank) * kTcBM;
    z = item / (nN * nM2);
    kb0 = z * kb_per_split;
    nkb = max(0, min(kblocks, kb0 + kb_per_split) - kb0);
  };
  auto aborted = [&] { return *(volatile int*)&s_abort != 0; };

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < 2 * STAGES; ++s) mbar_init(smem_u32(bars + s), 1);
    mbar_init(accf0, 1);
    mbar_init(accf0 + 8, 1);
    mbar_init(acce0, 8);
    mbar_init(acce0 + 8, 8);
    mbar_init(done_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  cluster_sync_all();  // both CTAs' barriers initialised and TMEM allocated

  if (warp == 0 && lane == 0) {
    // producer: this CTA's A rows and B half of every item, completing on the leader's full barrier
    int g = 0;
    bool stop = false;
    for (int item = pair; item < nitems && !stop; item += npairs) {
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
        const uint32_t fb = mapa_shared(full0 + 8 * s, 0);
        if (rank == 0) mbar_expect_tx(full0 + 8 * s, 2 * L::kStage);
        const int kc = (kb0 + kb) * BK;
#pragma unroll
        for (int p = 0; p < NS; ++p) {
          tma_load_2d_pair(smem_u32(st + p * L::kA), &maps.a[p], kc, m0, fb);
          tma_load_2d_pair(smem_u32(st + NS * L::kA + p * L::kBh), &maps.b[p], kc, n0 + int(rank) * (BN / 2), fb);
        }
        ++g;
      }
    }
    // the leader's last releases of this CTA's stages have landed (bounded)
    for (int k = max(0, g - STAGES); k < g; ++k)
      if (!mbar_wait(empty0 + 8 * (k % STAGES), (k / STAGES) & 1)) {
        atomicExch(&s_abort, 1);
        break;
      }
  } else if (warp == 1 && lane == 0 && rank == 0) {
    // MMA issuer (leader only): M = 256 over both CTAs' operands, accumulators alternating per item
    constexpr uint32_t idesc = idesc_pair<TF32>(BN);
    int g = 0, t = 0;
    bool stop = false;
    for (int item = pair; item < nitems && !stop; item += npairs, ++t) {
      int n0, m0, z, kb0, nkb;
      coords(item, n0, m0, z, kb0, nkb);
      const int b = t & 1;
      const uint32_t acc = tmem + uint32_t(b * BN);
      if (t >= 2 && !mbar_wait(acce0 + 8 * b, ((t >> 1) & 1) ^ 1)) {  // both CTAs' epilogues drained it
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
        for (int ks = 0; ks < L::kRB / 32; ++ks) {
          const uint32_t off = ks * 32;
          umma_pair<TF32>(acc, sw_desc<L::kRB>(a0 + off), sw_desc<L::kRB>(b0 + off), idesc, (kb | ks) != 0);
          if constexpr (NS >= 2) {
            umma_pair<TF32>(acc, sw_desc<L::kRB>(a0 + off), sw_desc<L::kRB>(b0 + L::kBh + off), idesc, 1);
            umma_pair<TF32>(acc, sw_desc<L::kRB>(a0 + L::kA + off), sw_desc<L::kRB>(b0 + off), idesc, 1);
          }
        }
        umma_commit_pair(empty0 + 8 * s);  // the stage is free in both CTAs
        ++g;
      }
      umma_commit_pair(accf0 + 8 * b);  // both CTAs: the item's products are done
    }
    umma_commit_pair(done_bar);  // both CTAs: every MMA issued above has completed
  } else if (warp >= 2) {
    // epilogue: this CTA's 128 rows of each item from its own TMEM
    const int q = warp % 4;
    int t = 0;
    for (int item = pair; item < nitems; item += npairs, ++t) {
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
      if (lane == 0) {
        if (rank == 0)
          mbar_arrive(acce0 + 8 * b);
        else
          mbar_arrive_cluster(mapa_shared(acce0 + 8 * b, 0));
      }
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
  cluster_sync_all();  // neither CTA frees TMEM or leaves while its peer still runs
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN));
}

// ---- host side ----

// A 2-D BF16 tensor map over a row-major [rows][ld] array (K contiguous, rows of `cols` valid
// elements), box = 64 x box_rows, 128-byte swizzle; out-of-range elements read as zero.
// A 2-D tensor map of a row-major BF16 matrix [rows][cols] (row stride ld elements) whose box is
// bk columns (64: 128-byte swizzle; 32: 64-byte swizzle) by box_rows rows.
CUtensorMap make_tmap_bf16(const void* base, long rows, long cols, long ld, int box_rows, int bk = kTcBK);
// The same over an FP32 matrix (TF32 operands): box bk = 32 columns (128 bytes, 128-byte swizzle)
// or 16 (64 bytes, 64-byte swizzle).
CUtensorMap make_tmap_f32(const void* base, long rows, long cols, long ld, int box_rows, int bk = 32);

// The parts of one operand: ns = 2 (hi, lo) or 3 (hi, mid, lo) BF16 tensor maps, or one FP32 map
// of TF32-rounded values (tf32, ns = 1, bk = 32).
struct TcOperand {
  CUtensorMap m[3];
  int ns = 2;
  int bk = kTcBK;  // K columns of the maps' box
  bool tf32 = false;
  // the matrices behind the maps (for maps with other boxes: the B halves of a CTA-pair launch)
  const void* base[3] = {nullptr, nullptr, nullptr};
  long rows = 0, cols = 0, ld = 0;
};

// Launches the split-precision product of A [M][K] and B [N][K] (K-major, both split into A.ns
// parts) into the FP32 slabs out[split][m + ld_out n]; returns the number of splits used. With
// kb_cap > 0 no FP32 accumulator sums more than kb_cap K-blocks of 64 (splits are added to bound
// the accumulation error of long same-sign sums), within max_splits.
int tc_gemm_launch(Ctx* ctx, const TcOperand& A, const TcOperand& B, int M, int N, int K, float* out, long ld_out,
                   long split_stride, int max_splits, int* d_err, const char* prof_name = "tc_gemm", int kb_cap = 0);

// The BN and split count tc_gemm_launch picks for (M, N, K), ns parts, at most max_splits splits.
void tc_gemm_shape(Ctx* ctx, int M, int N, int K, int max_splits, int ns, int* bn, int* splits, int kb_cap = 0);

// Launch with an explicit tile width bn (128: three pipeline stages; 256: two; two-part BF16 or TF32
// operands) and split count (0: the heuristic's count for that bn); B's tensor maps must have boxes
// of bn rows. TF32 operands: bn 128 (six stages) or 256 (four), either kernel. Returns the splits
// used. pair: the CTA-pair kernel (bn 256; BF16 with K blocks of 32, or TF32), six stages.
int tc_gemm_launch_with(Ctx* ctx, const TcOperand& A, const TcOperand& B, int bn, int splits, int M, int N, int K,
                        float* out, long ld_out, long split_stride, int* d_err, const char* prof_name = "tc_gemm",
                        bool persist = false, bool pair = false, int gm = 1);
// The variant with K blocks of 32 (64-byte swizzle) and four pipeline stages, bn = 256; A and B
// maps built with bk = 32.

// The split count tc_gemm_launch_with uses for splits = 0.
int tc_splits_for(Ctx* ctx, int M, int N, int K, int bn);

// One measured candidate of the autotuner.
struct TcTune {
  int bn = 0, splits = 0, bk = kTcBK;
  float ms = 0.f;
  bool persist = false;  // the persistent kernel (one CTA per SM, two accumulators)
  bool pair = false;     // the CTA-pair kernel (tcgen05 cta_group::2, 256-row tiles)
  int gm = 1;            // tile order: N tiles fastest (1) or groups of gm M tiles
};

// The autotuner: times every candidate tile shape of one two-part BF16 or one-part TF32 product on
// its own operands -- BF16: bn 128 with three stages, bn 256 with two (K blocks of 64), and with
// A32 / B256_32 (K blocks of 32) bn 256 one-tile, persistent and CTA pairs; TF32: bn 128 and 256
// one-tile and persistent, and (bn 256) CTA pairs; each
// with the heuristic split count and twice it, capped at max_splits -- with CUDA events on ctx's
// stream (a first launch, then unless it took 20 ms or more the best of `reps` launches timed one
// by one), and returns the fastest; every candidate's time goes to *all when given. B128 / B256: B's maps
// with boxes of 128 / 256 rows. gm > 1 adds the one-tile, persistent and pair candidates in grouped
// tile order (groups of gm and of 4 gm M tiles). Results are cached per device and shape for the
// process.
TcTune tc_gemm_autotune(Ctx* ctx, const TcOperand& A, const TcOperand& B128, const TcOperand& B256, int M, int N, int K,
                        float* out, long ld_out, long split_stride, int max_splits, int* d_err, int reps,
                        std::vector<TcTune>* all = nullptr, const TcOperand* A32 = nullptr,
                        const TcOperand* B256_32 = nullptr, int gm = 1);

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
