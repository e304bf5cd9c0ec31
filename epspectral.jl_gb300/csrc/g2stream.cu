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
  HostPinned* host = ctx->g2_stage;  // kept by the context for the next plan
  DBuf<uint8_t> dev[2];
  Events ev;
  EPSP_CUDA(cudaStreamCreateWithFlags(&ev.copy, cudaStreamNonBlocking));
  for (auto& e : ev.e) EPSP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  const int nb = nchunk > 1 ? 2 : 1;
  for (int b = 0; b < nb; ++b) {
    host[b].ensure(bytes);
    if (!keep) dev[b].alloc(ctx, bytes);
  }
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
  cudaEvent_t* copied = ev.e;
  cudaEvent_t* consumed = ev.e + 2;
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
  EPSP_CUDA(cudaStreamSynchronize(s));
  EPSP_CUDA(cudaStreamSynchronize(ev.copy));
  if (keep) {  // complete: a later set-up of the same array and order reads it
    K.host = m->g2;
    K.bytes = total;
    K.dtype = m->g2_dtype;
    K.order = order;
  }
}

}  // namespace epsp
