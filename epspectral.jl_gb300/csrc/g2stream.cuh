// g2stream.cuh -- the caller's host g2 [nm, ni, nf] streamed through the device in star order.
#pragma once
#include "common.cuh"

#include <functional>
#include <vector>

namespace epsp {

// g2's element as FP64 (FP64, FP32 or BF16 bit patterns in uint16_t storage).
template <class T>
__device__ __forceinline__ double load_g2(const T* p, long k);
template <>
__device__ __forceinline__ double load_g2<double>(const double* p, long k) { return p[k]; }
template <>
__device__ __forceinline__ double load_g2<float>(const float* p, long k) { return double(p[k]); }
template <>
__device__ __forceinline__ double load_g2<uint16_t>(const uint16_t* p, long k) {
  return double(__uint_as_float(uint32_t(p[k]) << 16));
}

size_t g2_elem_bytes(int dtype);

// Streams g2 through the device by column sets: column c holds the inner states order[p] for p in
// [cptr[c], cptr[c + 1]). Chunks are whole columns with at most chunk_f members (one column may
// exceed it alone). A chunk is laid out as [nm, ni, p - p0] (member-major slabs of
// g2[:, :, order[p]]) in one of two device buffers, filled on a second stream while the previous
// chunk is consumed on ctx->stream. A g2 the GPU reads in place (device memory, or registered
// page-locked host memory of at most 1 GiB) is gathered into the chunk by a kernel; otherwise
// each chunk is gathered on the host (over up to 16 threads) into page-locked staging (two buffers
// kept by the context for its next plan) and copied.
// fn(d_chunk, c0, c1, p0) enqueues the consumer of columns [c0, c1) on ctx->stream. Returns when
// every chunk has been consumed. The caller's g2 is read only.
void stream_g2_by_columns(Ctx* ctx, const epsp_model* m, const std::vector<int32_t>& order,
                          const std::vector<int32_t>& cptr, long chunk_f,
                          const std::function<void(const void*, long, long, long)>& fn);

}  // namespace epsp
