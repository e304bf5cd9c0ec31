// g2stream.cu -- host side of the star-order g2 stream (g2stream.cuh).
#include "g2stream.cuh"

#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>

namespace epsp {

size_t g2_elem_bytes(int dtype) { return dtype == EPSP_F64 ? 8 : (dtype == EPSP_F32 ? 4 : 2); }

namespace {
// Host threads for the star-order gather, started once per stream: the caller hands each chunk's
// member range to them (a generation count under a mutex), takes the first share itself and waits
// for the rest; the destructor stops and joins them.
struct GatherCrew {
  std::vector<std::thread> th;
  std::mutex mu;
  std::condition_variable go, done;
  long gen = 0;
  int pending = 0;
  bool stop = false;
  std::function<void(int)> work;  // work(t): thread t's share of the current chunk
  explicit GatherCrew(int n) {
    for (int t = 1; t < n; ++t)
      th.emplace_back([this, t] {
        long seen = 0;
        for (;;) {
          std::function<void(int)> w;
          {
            std::unique_lock<std::mutex> lk(mu);
            go.wait(lk, [&] { return stop || gen != seen; });
            if (stop) return;
            seen = gen;
            w = work;
          }
          w(t);
          std::lock_guard<std::mutex> lk(mu);
          if (--pending == 0) done.notify_one();
        }
      });
  }
  void run(const std::function<void(int)>& f) {
    {
      std::lock_guard<std::mutex> lk(mu);
      work = f;
      pending = int(th.size());
      ++gen;
    }
    go.notify_all();
    f(0);
    std::unique_lock<std::mutex> lk(mu);
    done.wait(lk, [&] { return pending == 0; });
  }
  ~GatherCrew() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stop = true;
    }
    go.notify_all();
    for (auto& x : th) x.join();
  }
};

// The star-order gather on the device, for a g2 this GPU reads in place: block x takes members
// p0 + x, p0 + x + gridDim.x, ... and copies g2[:, :, order[p]] (units V of the member's bytes)
// to slab p - p0 of dst, eight loads in flight per thread before their stores.
template <class V>
__global__ void __launch_bounds__(256) gather_members_kernel(const V* __restrict__ src, long units,
                                                             const int32_t* __restrict__ order, long p0, long n,
                                                             V* __restrict__ dst) {
  constexpr int kIn = 8;
  for (long p = blockIdx.x; p < n; p += gridDim.x) {
    const V* sp = src + long(order[p0 + p]) * units;
    V* dp = dst + p * units;
    for (long e = threadIdx.x; e < units; e += 256 * kIn) {
      V v[kIn];
#pragma unroll
      for (int u = 0; u < kIn; ++u)
        if (e + u * 256 < units) v[u] = sp[e + u * 256];
#pragma unroll
      for (int u = 0; u < kIn; ++u)
        if (e + u * 256 < units) dp[e + u * 256] = v[u];
    }
  }
}

// members [p0, p0 + n) of src into dst in `unit`-byte words (unit divides the member size and
// both base addresses)
void launch_gather_members(Ctx* ctx, const void* src, size_t slab, int unit, const int32_t* d_order, long p0,
                           long n, void* dst, cudaStream_t st) {
  if (n <= 0) return;
  const unsigned grid = unsigned(std::min<long>(n, long(std::max(ctx->sm_count, 1)) * 8));
  const long units = long(slab / size_t(unit));
  switch (unit) {
    case 16:
      gather_members_kernel<uint4><<<grid, 256, 0, st>>>(static_cast<const uint4*>(src), units, d_order, p0, n,
                                                        static_cast<uint4*>(dst));
      break;
    case 8:
      gather_members_kernel<uint2><<<grid, 256, 0, st>>>(static_cast<const uint2*>(src), units, d_order, p0, n,
                                                        static_cast<uint2*>(dst));
      break;
    case 4:
      gather_members_kernel<uint32_t><<<grid, 256, 0, st>>>(static_cast<const uint32_t*>(src), units, d_order, p0,
                                                           n, static_cast<uint32_t*>(dst));
      break;
    case 2:
      gather_members_kernel<uint16_t><<<grid, 256, 0, st>>>(static_cast<const uint16_t*>(src), units, d_order, p0,
                                                           n, static_cast<uint16_t*>(dst));
      break;
    default:
      gather_members_kernel<uint8_t><<<grid, 256, 0, st>>>(static_cast<const uint8_t*>(src), units, d_order, p0, n,
                                                          static_cast<uint8_t*>(dst));
  }
  EPSP_LAUNCHED(ctx);
}

// The largest g2 in host memory that is gathered on the device. On a GB300 node, the scGD0
// set-up's gather and coupling sums of a registered 365 MB g2 took 2.4 ms this way against 5.2 ms
// through the host gather, but those of a registered 8.6 GB g2 took 0.87-1.05 s against 0.15 s
// (also with each chunk's members read in ascending address order): the in-place reads slow down
// once the array is large, so a larger g2 goes through the host gather.
constexpr size_t kDeviceGatherMaxBytes = size_t(1) << 30;

// The address at which kernels read the caller's g2 of `bytes` bytes, or nullptr when it goes
// through the host gather. Device or managed memory is read in place; page-locked host memory
// registered with CUDA (epsp_host_register, cudaHostRegister, cudaHostAlloc) through its device
// alias, up to kDeviceGatherMaxBytes, when its first and last bytes lie in one contiguous device
// mapping of the same kind (a g2 registered only in part goes through the host gather). Pageable
// memory is not read in place even where the GPU could (cudaDevAttrPageableMemoryAccess on
// NVLink-C2C nodes): on a GB300 node, set-ups of a 365 MB g2 that the host had worked on meanwhile
// slowed several times over that way, as when the driver moves the pages the GPU reads.
const void* device_view(Ctx* ctx, const void* h, size_t bytes) {
  if (ctx->g2_host_gather || bytes == 0) return nullptr;
  cudaPointerAttributes a{}, z{};
  const void* last = static_cast<const uint8_t*>(h) + (bytes - 1);
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess || cudaPointerGetAttributes(&z, last) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (a.type != z.type || !a.devicePointer ||
      static_cast<const uint8_t*>(z.devicePointer) != static_cast<const uint8_t*>(a.devicePointer) + (bytes - 1))
    return nullptr;
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return a.devicePointer;
  if (a.type == cudaMemoryTypeHost && bytes <= kDeviceGatherMaxBytes) return a.devicePointer;
  return nullptr;
}

struct Events {
  cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaStream_t copy = nullptr;
  ~Events() {
    for (auto x : e)
      if (x) cudaEventDestroy(x);
    if (copy) cudaStreamDestroy(copy);
  }
};
}  // namespace

void stream_g2_by_columns(Ctx* ctx, const epsp_model* m, const std::vector<int32_t>& order,
                          const std::vector<int32_t>& cptr, long chunk_f,
                          const std::function<void(const void*, long, long, long)>& fn) {
  const long nc = long(cptr.size()) - 1;
  if (nc < 1) return;
  const size_t slab = size_t(m->nm) * size_t(m->ni) * g2_elem_bytes(m->g2_dtype);  // bytes of one member
  chunk_f = std::max<long>(chunk_f, 1);
  // chunk boundaries over whole columns
  std::vector<long> cb{0};
  long maxm = 0;
  for (long c = 0; c < nc;) {
    long c1 = c + 1;
    while (c1 < nc && cptr[size_t(c1 + 1)] - cptr[size_t(c)] <= chunk_f) ++c1;
    maxm = std::max<long>(maxm, cptr[size_t(c1)] - cptr[size_t(c)]);
    cb.push_back(c1);
    c = c1;
  }
  const long nchunk = long(cb.size()) - 1;
  const size_t bytes = size_t(std::max<long>(maxm, 1)) * slab;
  cudaStream_t s = ctx->stream;
  // the copy the context keeps (epsp_ctx_keep_g2): the same array, size, type and member order are
  // read there, chunk by chunk, without a host gather or a copy
  G2Kept& K = ctx->g2_kept;
  const size_t total = order.size() * slab;
  if (K.on && K.host == m->g2 && K.bytes == total && K.dtype == m->g2_dtype && K.order == order) {
    for (long k = 0; k < nchunk; ++k) {
      const long c0 = cb[size_t(k)], c1 = cb[size_t(k + 1)], p0 = cptr[size_t(c0)];
      fn(static_cast<uint8_t*>(K.dev) + size_t(p0) * slab, c0, c1, p0);
    }
    EPSP_CUDA(cudaStreamSynchronize(s));
    return;
  }
  // otherwise the chunks are streamed, into the kept copy's slots when the context keeps g2 (each
  // chunk its own slot: no double buffer on the device), else through two device buffers
  bool keep = K.on;
  if (keep) {
    K.host = nullptr;
    if (K.dev_bytes < total) {
      K.release();
      if (cudaMalloc(&K.dev, total) != cudaSuccess) {  // no room for a copy: stream as usual
        (void)cudaGetLastError();
        K.dev = nullptr;
        keep = false;
      } else {
        K.dev_bytes = total;
      }
    }
  }
  DBuf<uint8_t> dev[2];
  Events ev;
  EPSP_CUDA(cudaStreamCreateWithFlags(&ev.copy, cudaStreamNonBlocking));
  for (auto& e : ev.e) EPSP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  const int nb = nchunk > 1 ? 2 : 1;
  for (int b = 0; b < nb; ++b)
    if (!keep) dev[b].alloc(ctx, bytes);
  cudaEvent_t* copied = ev.e;
  cudaEvent_t* consumed = ev.e + 2;
  auto complete = [&] {
    EPSP_CUDA(cudaStreamSynchronize(s));
    EPSP_CUDA(cudaStreamSynchronize(ev.copy));
    if (keep) {  // complete: a later set-up of the same array and order reads it
      K.host = m->g2;
      K.bytes = total;
      K.dtype = m->g2_dtype;
      K.order = order;
    }
  };
  // When the GPU reads the caller's g2 in place, one kernel per chunk gathers it in star order on
  // the copy stream (no host staging and no separate copy); the chunks' consumers overlap the next
  // gathers as in the copy path below.
  if (const void* src = device_view(ctx, m->g2, size_t(m->nf) * slab)) {
    int unit = 16;  // the widest word that divides the member size and the address
    while (unit > 1 && (slab % size_t(unit) != 0 || reinterpret_cast<uintptr_t>(src) % uintptr_t(unit) != 0))
      unit /= 2;
    DBuf<int32_t> d_order = to_device(ctx, order);
    EPSP_CUDA(cudaEventRecord(copied[0], s));  // the order table is on the device
    EPSP_CUDA(cudaStreamWaitEvent(ev.copy, copied[0], 0));
    for (long k = 0; k < nchunk; ++k) {
      const int b = int(k % nb);
      const long c0 = cb[size_t(k)], c1 = cb[size_t(k + 1)];
      const long p0 = cptr[size_t(c0)], p1 = cptr[size_t(c1)];
      // the device buffer's previous chunk must be consumed before it is overwritten
      if (k >= nb && !keep) EPSP_CUDA(cudaStreamWaitEvent(ev.copy, consumed[b], 0));
      uint8_t* d = keep ? static_cast<uint8_t*>(K.dev) + size_t(p0) * slab : dev[b].p;
      launch_gather_members(ctx, src, slab, unit, d_order.p, p0, p1 - p0, d, ev.copy);
      EPSP_CUDA(cudaEventRecord(copied[b], ev.copy));
      EPSP_CUDA(cudaStreamWaitEvent(s, copied[b], 0));
      fn(d, c0, c1, p0);
      EPSP_CUDA(cudaEventRecord(consumed[b], s));
    }
    complete();
    return;
  }
  HostPinned* host = ctx->g2_stage;  // kept by the context for the next plan
  for (int b = 0; b < nb; ++b) host[b].ensure(bytes);
  // the star-order gather of a chunk into the staging buffer, over up to 16 host threads started
  // once for the stream (chunks of less than 8 MB are gathered by the caller alone)
  const int nthreads = int(std::clamp<unsigned>(std::thread::hardware_concurrency(), 1u, 16u));
  const bool crew_on = nthreads > 1 && size_t(std::max<long>(maxm, 1)) * slab >= (size_t(8) << 20);
  std::unique_ptr<GatherCrew> crew(crew_on ? new GatherCrew(nthreads) : nullptr);
  auto gather = [&](uint8_t* dst, long p0, long p1) {
    const auto* src = static_cast<const uint8_t*>(m->g2);
    auto part = [&](long a, long b) {
      for (long p = a; p < b; ++p) std::memcpy(dst + size_t(p - p0) * slab, src + size_t(order[size_t(p)]) * slab, slab);
    };
    const long n = p1 - p0;
    if (!crew || size_t(n) * slab < (size_t(8) << 20)) {
      part(p0, p1);
      return;
    }
    const long per = (n + nthreads - 1) / nthreads;
    crew->run([&](int t) {
      const long a = p0 + t * per, b = std::min(p1, a + per);
      if (a < b) part(a, b);
    });
  };
  for (long k = 0; k < nchunk; ++k) {
    const int b = int(k % nb);
    const long c0 = cb[size_t(k)], c1 = cb[size_t(k + 1)];
    const long p0 = cptr[size_t(c0)], p1 = cptr[size_t(c1)];
    // the staging buffer's previous copy must be done before it is refilled
    if (k >= nb) EPSP_CUDA(cudaEventSynchronize(copied[b]));
    gather(static_cast<uint8_t*>(host[b].p), p0, p1);
    // the device buffer's previous chunk must be consumed before it is overwritten
    if (k >= nb && !keep) EPSP_CUDA(cudaStreamWaitEvent(ev.copy, consumed[b], 0));
    uint8_t* d = keep ? static_cast<uint8_t*>(K.dev) + size_t(p0) * slab : dev[b].p;
    EPSP_CUDA(cudaMemcpyAsync(d, host[b].p, size_t(p1 - p0) * slab, cudaMemcpyHostToDevice, ev.copy));
    EPSP_CUDA(cudaEventRecord(copied[b], ev.copy));
    EPSP_CUDA(cudaStreamWaitEvent(s, copied[b], 0));
    fn(d, c0, c1, p0);
    EPSP_CUDA(cudaEventRecord(consumed[b], s));
  }
  complete();
}

}  // namespace epsp
