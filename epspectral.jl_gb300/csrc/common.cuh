// common.cuh -- shared host and device pieces of libepspectral_gb300: errors, device buffers, the
// context, and the scalar element functions of the reference (occupations, grid interpolation)
// as device code.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <cmath>

#include "../../include/epspectral_gb300.h"

namespace epsp {

// ---- errors ----

struct Error {
  int code;
  std::string msg;
};

[[noreturn]] inline void fail(int code, const std::string& msg) { throw Error{code, msg}; }

inline void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
  if (e != cudaSuccess) {
    char buf[512];
    std::snprintf(buf, sizeof buf, "%s failed at %s:%d: %s", what, file, line, cudaGetErrorString(e));
    fail(e == cudaErrorMemoryAllocation ? EPSP_ENOMEM : EPSP_ECUDA, buf);
  }
}
#define EPSP_CUDA(call) ::epsp::cuda_check((call), #call, __FILE__, __LINE__)

// ---- context ----

// Pinned host memory (page-locked: copies to and from it are direct DMA, without staging).
struct HostPinned {
  void* p = nullptr;
  size_t bytes = 0;
  void ensure(size_t n) {
    if (n <= bytes) return;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    if (cudaHostAlloc(&p, n, cudaHostAllocDefault) != cudaSuccess) {
      p = nullptr;
      (void)cudaGetLastError();
      fail(EPSP_ENOMEM, "page-locked host allocation of " + std::to_string(n) + " bytes failed");
    }
    bytes = n;
  }
  HostPinned() = default;
  HostPinned(const HostPinned&) = delete;
  HostPinned& operator=(const HostPinned&) = delete;
  ~HostPinned() {
    if (p) cudaFreeHost(p);
  }
};

// The device copy of a streamed g2 that a context keeps on request (epsp_ctx_keep_g2): the host
// array it came from (null while incomplete), its size, element type and member order.
struct G2Kept {
  bool on = false;
  const void* host = nullptr;
  size_t bytes = 0;
  int dtype = -1;
  std::vector<int32_t> order;
  void* dev = nullptr;
  size_t dev_bytes = 0;
  void release() {
    if (dev) cudaFree(dev);
    dev = nullptr;
    dev_bytes = 0;
    host = nullptr;
    order.clear();
  }
  G2Kept() = default;
  G2Kept(const G2Kept&) = delete;
  G2Kept& operator=(const G2Kept&) = delete;
  ~G2Kept() { release(); }
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  int64_t launches = 0;
  int sm_count = 0;
  // Device-side timing of one named kernel family (enabled by epsp_profile_kernel).
  std::string prof_name;
  std::vector<cudaEvent_t> prof_events;  // pairs (start, stop)
  size_t prof_used = 0;
  // Host-side test hook: the next allocation of at least `fail_alloc_bytes` fails (0 = off).
  size_t fail_alloc_bytes = 0;
  // Test hook of the one-CTA tensor-core GEMM: the producer skips K block `stall_kb` of every tile
  // (-1 = off) and the pipeline waits give up after `stall_wait_limit` tries (0 = the default).
  int stall_kb = -1;
  unsigned stall_wait_limit = 0;
  // Test hook of the g2 stream: gather on the host and copy even where the GPU reads g2 in place.
  bool g2_host_gather = false;
  cudaEvent_t timer[2] = {nullptr, nullptr};
  // host time spent in device allocations (for the set-up phase log)
  double alloc_ms = 0;
  long alloc_calls = 0;
  // the g2 stream's double-buffered staging, kept for the next plan of this context
  HostPinned g2_stage[2];
  // the streamed g2 itself, when the caller asks the context to keep it
  G2Kept g2_kept;
};

// Set-up phase log (verbosity >= 2): host milliseconds of each phase since the previous mark (the
// stream synchronised, so device work is included) and of the device allocations in it, to stderr.
struct PhaseLog {
  Ctx* ctx;
  const char* who;
  bool on;
  std::chrono::steady_clock::time_point t;
  double a0;
  long c0;
  PhaseLog(Ctx* c, const char* w, int verbosity)
      : ctx(c), who(w), on(verbosity >= 2), t(std::chrono::steady_clock::now()), a0(c->alloc_ms), c0(c->alloc_calls) {}
  void mark(const char* phase) {
    if (!on) return;
    cudaStreamSynchronize(ctx->stream);
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "%s set-up: %-28s %8.2f ms (allocations %.2f ms in %ld)\n", who, phase,
                 std::chrono::duration<double, std::milli>(now - t).count(), ctx->alloc_ms - a0, ctx->alloc_calls - c0);
    t = now;
    a0 = ctx->alloc_ms;
    c0 = ctx->alloc_calls;
  }
};

// Records the start event of a profiled launch; returns the pair index or -1.
inline long prof_begin(Ctx* c, const char* name) {
  if (c->prof_name.empty() || c->prof_name != name) return -1;
  if (c->prof_used + 2 > c->prof_events.size()) {
    for (int k = 0; k < 64; ++k) {
      cudaEvent_t e;
      EPSP_CUDA(cudaEventCreate(&e));
      c->prof_events.push_back(e);
    }
  }
  long idx = long(c->prof_used);
  EPSP_CUDA(cudaEventRecord(c->prof_events[idx], c->stream));
  c->prof_used += 2;
  return idx;
}
inline void prof_end(Ctx* c, long idx) {
  if (idx >= 0) EPSP_CUDA(cudaEventRecord(c->prof_events[size_t(idx) + 1], c->stream));
}

#define EPSP_LAUNCHED(ctx) do { (ctx)->launches++; EPSP_CUDA(cudaGetLastError()); } while (0)

// ---- device buffers ----

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  Ctx* ctx = nullptr;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept { *this = std::move(o); }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p; n = o.n; ctx = o.ctx;
      o.p = nullptr; o.n = 0;
    }
    return *this;
  }
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(Ctx* c, size_t count) {
    release();
    ctx = c;
    n = count;
    if (count == 0) return;
    size_t bytes = count * sizeof(T);
    if (c && c->fail_alloc_bytes && bytes >= c->fail_alloc_bytes) {
      c->fail_alloc_bytes = 0;
      fail(EPSP_ENOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed (test hook)");
    }
    const auto t0 = std::chrono::steady_clock::now();
    cudaError_t e = cudaMalloc(&p, bytes);
    if (c) {
      c->alloc_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      ++c->alloc_calls;
    }
    if (e != cudaSuccess) {
      p = nullptr;
      (void)cudaGetLastError();
      fail(EPSP_ENOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
    }
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    EPSP_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void download(T* h, size_t count, cudaStream_t s) const {
    EPSP_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
  void zero(cudaStream_t s) {
    if (n) EPSP_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
};

// Work buffers kept by a plan across calls: (re)allocated only when they must grow.
template <class T>
bool ensure(DBuf<T>& b, Ctx* c, size_t count) {
  if (b.p && b.n >= count) return false;
  b.alloc(c, count);
  return true;
}

template <class T>
DBuf<T> to_device(Ctx* c, const T* h, size_t count) {
  DBuf<T> b;
  b.alloc(c, count);
  if (count) b.upload(h, count, c->stream);
  return b;
}
template <class T>
DBuf<T> to_device(Ctx* c, const std::vector<T>& h) {
  return to_device(c, h.data(), h.size());
}

// The Kramers-Kronig matrix of a grid (src/frequency_grids.jl:30-44), built on the device into K
// [n, n] (column-major) from the nodes padded by one spacing at either end; returns when K is made.
void kk_matrix_to_device(Ctx* ctx, const std::vector<double>& nodes, DBuf<double>& K);

inline unsigned div_up(size_t a, size_t b) { return unsigned((a + b - 1) / b); }

// ---- grids (host) ----

struct GridHost {
  std::vector<double> nodes;  // origin + offsets[j] * unit (src/frequency_grids.jl:140-141)
  std::vector<int64_t> offsets;
  double origin = 0, unit = 0, dw_min = 0;
  int64_t n = 0;
};

GridHost make_grid(const epsp_grid& g, const char* name);

// FrequencyGrid's constructor checks (src/frequency_grids.jl:124-132) on g, without allocating:
// returns the smallest gap between consecutive offsets (dω_min = unit x that gap).
int64_t check_grid(const epsp_grid& g, const char* name);

// cell_search_table (src/frequency_grids.jl:184-196)
struct CellTableHost {
  std::vector<int32_t> jtab;
  double x0 = 0, inv_h = 0;
};
CellTableHost make_cell_table(const GridHost& g);

// The two steps of cell_search_table on the strictly increasing nodes x[0..n), shared by the plans
// and the allocation-free entry point (which fills a fixed array): the bucket width 1 / inv_h,
// inv_h = 1 / ((1 - 1e-6) dω_min); the table's entry count, the last node's bucket + 1, with the
// bucket index clamped to 2^40 before it is converted to an integer; and the table itself,
// jtab[k] = the first node whose bucket is >= k, for k < entries (EPSP_EINVAL when two nodes fall
// in one bucket).
inline double cell_inv_h(double dw_min) { return 1.0 / ((1.0 - 1e-6) * dw_min); }
int64_t cell_table_entries(const double* x, int64_t n, double inv_h);
void fill_cell_table(const double* x, int64_t n, double inv_h, int32_t* jtab, int64_t entries);

// linear_interpolation_table (src/frequency_grids.jl:65-84), 0-based cells.
void interp_table(const std::vector<double>& ws, const std::vector<double>& xs, std::vector<int32_t>& j,
                  std::vector<double>& t);

std::vector<double> trapezoid_weights(const std::vector<double>& ws);

// ---- device element functions ----

struct CellTableDev {
  const int32_t* jtab;
  const double* ws;
  double x0, inv_h;
  int n;
};

// occ_fermion, src/utils.jl:14-22 (negative T is rejected on the host before any launch).
__device__ __forceinline__ double occ_fermion_d(double e, double T) {
  if (T > 1.4901161193847656e-08) return 1.0 / (exp(e / T) + 1.0);
  return e > 0 ? 0.0 : (e < 0 ? 1.0 : 0.5);
}

// occ_boson, src/utils.jl:24-38.
__device__ __forceinline__ double occ_boson_d(double e, double T) {
  if (T > 1.4901161193847656e-08) return e == 0 ? -0.5 : 1.0 / expm1(e / T);
  return e > 0 ? 0.0 : (e == 0 ? -0.5 : -1.0);
}

// _interp_linear_grid (src/frequency_grids.jl:207-219) of a complex column (interleaved) at x.
__device__ __forceinline__ double2 interp_grid_d(const double2* __restrict__ col, const CellTableDev& ct, double x) {
  if (!(x > ct.ws[0])) return col[0];
  if (x >= ct.ws[ct.n - 1]) return col[ct.n - 1];
  int c = __ldg(ct.jtab + (long long)((x - ct.x0) * ct.inv_h));
  int j = c - 1 + (__ldg(ct.ws + c) <= x ? 1 : 0);
  double wl = __ldg(ct.ws + j), wh = __ldg(ct.ws + j + 1);
  double t = (x - wl) / (wh - wl);
  double2 lo = col[j], hi = col[j + 1];
  return make_double2((1 - t) * lo.x + t * hi.x, (1 - t) * lo.y + t * hi.y);
}

}  // namespace epsp

// The opaque handle types of the ABI.
struct epsp_ctx {
  epsp::Ctx c;
};
