// context.cu -- the context entry points of the ABI and the host-side grid tables shared by the
// scGD0 and ladder plans.
#include "common.cuh"

#include <algorithm>
#include <limits>

namespace epsp {

int64_t check_grid(const epsp_grid& g, const char* name) {
  if (!(std::isfinite(g.origin) && std::isfinite(g.unit) && g.unit > 0))
    fail(EPSP_EINVAL, std::string(name) + ": origin must be finite and unit finite and positive");
  if (g.n < 2 || g.offsets == nullptr) fail(EPSP_EINVAL, std::string(name) + ": a FrequencyGrid needs at least two nodes");
  int64_t mg = std::numeric_limits<int64_t>::max();
  for (int64_t j = 0; j + 1 < g.n; ++j) {
    int64_t d = g.offsets[j + 1] - g.offsets[j];
    if (d <= 0) fail(EPSP_EINVAL, std::string(name) + ": offsets must be strictly increasing");
    mg = std::min(mg, d);
  }
  return mg;
}

GridHost make_grid(const epsp_grid& g, const char* name) {
  const int64_t mg = check_grid(g, name);
  GridHost h;
  h.origin = g.origin;
  h.unit = g.unit;
  h.n = g.n;
  h.offsets.assign(g.offsets, g.offsets + g.n);
  h.dw_min = g.unit * double(mg);
  h.nodes.resize(size_t(g.n));
  for (int64_t j = 0; j < g.n; ++j) h.nodes[size_t(j)] = g.origin + double(g.offsets[j]) * g.unit;
  return h;
}

int64_t cell_table_entries(const double* x, int64_t n, double inv_h) {
  return int64_t(std::min((x[n - 1] - x[0]) * inv_h, std::ldexp(1.0, 40))) + 1;
}

void fill_cell_table(const double* x, int64_t n, double inv_h, int32_t* jtab, int64_t entries) {
  // the caller checked entries against its table's capacity, so every bucket below is < 2^40
  auto bucket = [&](int64_t j) { return int64_t((x[j] - x[0]) * inv_h); };
  for (int64_t j = 0; j + 1 < n; ++j)
    if (bucket(j + 1) == bucket(j)) fail(EPSP_EINVAL, "two grid nodes fall in one bucket");
  int64_t c = 0;
  for (int64_t k = 0; k < entries; ++k) {
    while (c < n && bucket(c) < k) ++c;
    jtab[k] = int32_t(c);
  }
}

CellTableHost make_cell_table(const GridHost& g) {
  CellTableHost ct;
  ct.x0 = g.nodes[0];
  ct.inv_h = cell_inv_h(g.dw_min);
  const int64_t n = int64_t(g.nodes.size());
  const int64_t entries = cell_table_entries(g.nodes.data(), n, ct.inv_h);
  if (entries > (int64_t(1) << 24))
    fail(EPSP_EINVAL, "cell search table of more than 2^24 entries: use a grid without a near-coincident pair of nodes");
  ct.jtab.resize(size_t(entries));
  fill_cell_table(g.nodes.data(), n, ct.inv_h, ct.jtab.data(), entries);
  return ct;
}

void interp_table(const std::vector<double>& ws, const std::vector<double>& xs, std::vector<int32_t>& j,
                  std::vector<double>& t) {
  const size_t n = ws.size();
  j.resize(xs.size());
  t.resize(xs.size());
  for (size_t r = 0; r < xs.size(); ++r) {
    double x = xs[r];
    if (x <= ws[0]) {
      j[r] = 0;
      t[r] = 0;
    } else if (x >= ws[n - 1]) {
      j[r] = int32_t(n - 2);
      t[r] = 1;
    } else {
      size_t jr = size_t(std::upper_bound(ws.begin(), ws.end(), x) - ws.begin()) - 1;
      j[r] = int32_t(jr);
      t[r] = (x - ws[jr]) / (ws[jr + 1] - ws[jr]);
    }
  }
}

std::vector<double> trapezoid_weights(const std::vector<double>& ws) {  // src/frequency_grids.jl:53-54
  const size_t n = ws.size();
  std::vector<double> W(n);
  for (size_t j = 0; j < n; ++j) W[j] = (ws[std::min(j + 1, n - 1)] - ws[j == 0 ? 0 : j - 1]) / 2;
  return W;
}

}  // namespace epsp

using namespace epsp;

extern "C" {

epsp_status epsp_create(epsp_ctx** out, int32_t device) {
  if (!out) return EPSP_EINVAL;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return EPSP_ECUDA;
  if (device < 0 || device >= n) return EPSP_EINVAL;
  auto* c = new (std::nothrow) epsp_ctx;
  if (!c) return EPSP_ENOMEM;
  c->c.device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->c.stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return EPSP_ECUDA;
  }
  cudaDeviceGetAttribute(&c->c.sm_count, cudaDevAttrMultiProcessorCount, device);
  *out = c;
  return EPSP_OK;
}

void epsp_destroy(epsp_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->c.device);
  for (auto e : c->c.prof_events) cudaEventDestroy(e);
  for (auto e : c->c.timer)
    if (e) cudaEventDestroy(e);
  if (c->c.stream) cudaStreamDestroy(c->c.stream);
  delete c;
}

const char* epsp_last_error(const epsp_ctx* c) { return c ? c->c.last_error.c_str() : "null context"; }

int64_t epsp_kernel_launches(const epsp_ctx* c) { return c ? c->c.launches : 0; }

/* Kernel timing for the roofline report (not in the reference): every launch of the kernel family
 * `name` is bracketed by CUDA events on the context's stream until the next call. name = NULL or ""
 * switches it off. epsp_profile_read returns the summed milliseconds and the number of launches. */
epsp_status epsp_profile_kernel(epsp_ctx* c, const char* name) {
  if (!c) return EPSP_EINVAL;
  c->c.prof_name = name ? name : "";
  c->c.prof_used = 0;
  return EPSP_OK;
}

epsp_status epsp_profile_read(epsp_ctx* c, double* total_ms, int64_t* count) {
  if (!c) return EPSP_EINVAL;
  if (cudaStreamSynchronize(c->c.stream) != cudaSuccess) return EPSP_ECUDA;
  double tot = 0;
  size_t n = c->c.prof_used / 2;
  for (size_t k = 0; k < n; ++k) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, c->c.prof_events[2 * k], c->c.prof_events[2 * k + 1]) != cudaSuccess) return EPSP_ECUDA;
    tot += ms;
  }
  if (total_ms) *total_ms = tot;
  if (count) *count = int64_t(n);
  c->c.prof_used = 0;
  return EPSP_OK;
}

/* Device-side stopwatch on the context's stream (for benchmarks): epsp_timer_begin records a start
 * event, epsp_timer_end a stop event, waits for it and returns the elapsed milliseconds. */
epsp_status epsp_timer_begin(epsp_ctx* c) {
  if (!c) return EPSP_EINVAL;
  if (!c->c.timer[0]) {
    if (cudaEventCreate(&c->c.timer[0]) != cudaSuccess || cudaEventCreate(&c->c.timer[1]) != cudaSuccess) return EPSP_ECUDA;
  }
  return cudaEventRecord(c->c.timer[0], c->c.stream) == cudaSuccess ? EPSP_OK : EPSP_ECUDA;
}

epsp_status epsp_timer_end(epsp_ctx* c, double* ms) {
  if (!c || !c->c.timer[0]) return EPSP_EINVAL;
  if (cudaEventRecord(c->c.timer[1], c->c.stream) != cudaSuccess || cudaEventSynchronize(c->c.timer[1]) != cudaSuccess)
    return EPSP_ECUDA;
  float f = 0;
  if (cudaEventElapsedTime(&f, c->c.timer[0], c->c.timer[1]) != cudaSuccess) return EPSP_ECUDA;
  if (ms) *ms = double(f);
  return EPSP_OK;
}

/* Test hook (not in the reference): the next device allocation of at least `bytes` bytes made
 * through this context fails with EPSP_ENOMEM, as a device without room would. 0 switches it off. */
epsp_status epsp_test_fail_alloc(epsp_ctx* c, uint64_t bytes) {
  if (!c) return EPSP_EINVAL;
  c->c.fail_alloc_bytes = size_t(bytes);
  return EPSP_OK;
}

/* Not in the reference: with on, the context keeps on the device the last g2 a plan set-up streamed
 * (in that set-up's member order), and a later set-up whose model points at the same g2 array
 * (address, size, element type) in the same order reads that copy instead of streaming g2 again
 * (an scGD0 plan and a ladder plan of one model). The caller must not change the array in between.
 * on = 0 switches it off and frees the copy. */
epsp_status epsp_ctx_keep_g2(epsp_ctx* c, int32_t on) {
  if (!c) return EPSP_EINVAL;
  if (!on) c->c.g2_kept.release();
  c->c.g2_kept.on = on != 0;
  return EPSP_OK;
}

/* Test hook (not in the reference): the one-CTA tensor-core GEMM kernel's producer skips K block
 * `skip_kblock` of every tile (-1 switches it off), and that kernel's pipeline waits give up after
 * `wait_limit` tries (0 restores the default), so a call returns EPSP_EDEVICE_TIMEOUT from a wait
 * that runs out on the device rather than from a fault. */
epsp_status epsp_test_gemm_stall(epsp_ctx* c, int32_t skip_kblock, uint32_t wait_limit) {
  if (!c) return EPSP_EINVAL;
  if (skip_kblock < -1 || (wait_limit != 0 && wait_limit < 64)) {
    c->c.last_error = "epsp_test_gemm_stall: skip_kblock must be -1 or a K block, wait_limit 0 or at least 64";
    return EPSP_EINVAL;
  }
  c->c.stall_kb = skip_kblock;
  c->c.stall_wait_limit = wait_limit;
  return EPSP_OK;
}

/* Page-locks host memory [ptr, ptr + bytes) and maps it for the device (cudaHostRegister, portable
 * and mapped), so that plan set-ups read a g2 there in place; epsp_host_unregister undoes it. */
epsp_status epsp_host_register(epsp_ctx* c, void* ptr, uint64_t bytes) {
  if (!c) return EPSP_EINVAL;
  if (!ptr || bytes == 0) {
    c->c.last_error = "epsp_host_register: ptr must be non-NULL and bytes positive";
    return EPSP_EINVAL;
  }
  cudaSetDevice(c->c.device);
  const cudaError_t e = cudaHostRegister(ptr, size_t(bytes), cudaHostRegisterPortable | cudaHostRegisterMapped);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    c->c.last_error = std::string("cudaHostRegister: ") + cudaGetErrorString(e);
    return e == cudaErrorHostMemoryAlreadyRegistered ? EPSP_EINVAL : EPSP_ECUDA;
  }
  return EPSP_OK;
}

epsp_status epsp_host_unregister(epsp_ctx* c, void* ptr) {
  if (!c || !ptr) return EPSP_EINVAL;
  cudaSetDevice(c->c.device);
  const cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    c->c.last_error = std::string("cudaHostUnregister: ") + cudaGetErrorString(e);
    return e == cudaErrorHostMemoryNotRegistered ? EPSP_EINVAL : EPSP_ECUDA;
  }
  return EPSP_OK;
}

/* Test hook: on = 1 makes the g2 stream gather on the host and copy even for a g2 the GPU reads in
 * place (registered page-locked memory); on = 0 (the default) gathers such a g2 on the device. */
epsp_status epsp_test_g2_host_gather(epsp_ctx* c, int32_t on) {
  if (!c) return EPSP_EINVAL;
  c->c.g2_host_gather = on != 0;
  return EPSP_OK;
}

}  // extern "C"
