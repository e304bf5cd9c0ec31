// noalloc.cu -- the Fan-Migdal sum for callers that cannot allocate device memory.
//
// Some callers own every byte of device memory themselves: a Julia host whose CUDA.jl pool (or the
// ElectronPhonon backend's allocator) holds the memory budget, code that runs where a cudaMalloc
// would be refused or would stall other work on the device, or a host that hands the library only
// pointers into buffers it already has. epsp_scgd0_imsigma_noalloc serves them: the caller passes
// every input and the output as device pointers, and the only device memory the kernel needs beyond
// those -- the grid nodes and the O(1) cell-search table of _interp_linear_grid -- lives in the
// file-scope array g_noalloc_scratch below, of a fixed size held by every device that loads the
// library until the process exits.
//
// The computation is the reference's element sum (src/scgd0_kernel.jl:27-86), term by term in FP64,
// as the DIRECT_FP64 plan path: ImΣ[ω, i] += Σ_{νf} term in ascending νf, with ωq gathered per pair
// (src/scgd0.jl:270) and g2 read in its [ν, i, f] layout.
#include "common.cuh"

#include <mutex>

namespace epsp {

// Capacity of the scratch array: the grid nodes (doubles) followed by the cell-search table (int32).
constexpr int64_t kNoallocMaxNodes = 1 << 16;
constexpr int64_t kNoallocMaxTable = 1 << 20;
constexpr size_t kNoallocBytes = size_t(kNoallocMaxNodes) * 8 + size_t(kNoallocMaxTable) * 4;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// Host-side staging of the same two tables (no heap allocation per call).
static double g_nodes_host[kNoallocMaxNodes];
static int32_t g_table_host[kNoallocMaxTable];
static std::mutex g_noalloc_mutex;
static void* g_scratch_dev[64] = {};  // device address of g_noalloc_scratch, per device ordinal

__global__ void fm_direct_noalloc_kernel(const double* __restrict__ ws, int nw, CellTableDev ct,
                                         const double2* __restrict__ Sin, const double* __restrict__ g2,
                                         const double* __restrict__ wph, const int32_t* __restrict__ iq_kk,
                                         const int32_t* __restrict__ iks_i, const int32_t* __restrict__ iks_f,
                                         long nk_i, const double* __restrict__ eps_f, const double* __restrict__ w_f,
                                         const int32_t* __restrict__ f_to_i, int nm, int ni, long nf, double mu,
                                         double T, double w_ac, double* __restrict__ imsigma) {
  constexpr int kTile = 128;
  __shared__ double s_g2[kTile], s_wq[kTile], s_nq[kTile], s_eps[kTile], s_wf[kTile];
  __shared__ int s_col[kTile];
  const int i = blockIdx.y;
  const int iw = blockIdx.x * kTile + threadIdx.x;
  const double w = iw < nw ? ws[iw] : 0.0;
  const long nvf = long(nm) * nf;
  double acc = 0.0;
  for (long t0 = 0; t0 < nvf; t0 += kTile) {
    const long vf = t0 + threadIdx.x;
    if (vf < nvf) {
      const int nu = int(vf % nm);
      const long f = vf / nm;
      const long q = iq_kk[iks_i[i] + nk_i * long(iks_f[f])];
      const double wq = wph[nu + long(nm) * q];
      s_g2[threadIdx.x] = g2[nu + long(nm) * (i + long(ni) * f)];
      s_wq[threadIdx.x] = wq;
      s_nq[threadIdx.x] = wq < w_ac ? 0.0 : occ_boson_d(wq, T);
      s_eps[threadIdx.x] = eps_f[f];
      s_wf[threadIdx.x] = w_f[f];
      s_col[threadIdx.x] = f_to_i[f];
    }
    __syncthreads();
    const int nt = int(min(long(kTile), nvf - t0));
    if (iw < nw) {
      for (int k = 0; k < nt; ++k) {
        const double wq = s_wq[k];
        if (wq < w_ac) continue;
        const double2* col = Sin + long(nw) * s_col[k];
        const double xa = w + wq, xe = w - wq;
        const double2 sa = interp_grid_d(col, ct, xa);
        const double2 se = interp_grid_d(col, ct, xe);
        const double zar = xa - s_eps[k] - sa.x, zai = -sa.y;
        const double zer = xe - s_eps[k] - se.x, zei = -se.y;
        const double ga = -zai / (zar * zar + zai * zai);
        const double ge = -zei / (zer * zer + zei * zei);
        const double nq = s_nq[k];
        acc += s_wf[k] * s_g2[k] * (ga * (nq + occ_fermion_d(xa - mu, T)) + ge * (nq + 1 - occ_fermion_d(xe - mu, T)));
      }
    }
    __syncthreads();
  }
  if (iw < nw) imsigma[iw + long(nw) * i] += acc;
}

}  // namespace epsp

using namespace epsp;

extern "C" epsp_status epsp_scgd0_imsigma_noalloc(epsp_ctx* ctx, int64_t nm, int64_t ni, int64_t nf,
                                                  const double* g2, int64_t nq, const double* omega_ph,
                                                  int64_t nk_i, int64_t nk_f, const int32_t* iq_kk,
                                                  const int32_t* iks_i, const int32_t* iks_f, const double* eps_f,
                                                  const double* w_f, const int32_t* f_to_i, const epsp_grid* omegas,
                                                  double omega_acoustic, const double* sigma_in, double mu, double T,
                                                  double* imsigma) {
  if (!ctx) return EPSP_EINVAL;
  Ctx* c = &ctx->c;
  try {
    if (nm < 1 || ni < 1 || nf < 1 || nq < 1 || nk_i < 1 || nk_f < 1)
      fail(EPSP_EINVAL, "nm, ni, nf, nq, nk_i and nk_f must be positive");
    if (!g2 || !omega_ph || !iq_kk || !iks_i || !iks_f || !eps_f || !w_f || !f_to_i || !omegas || !sigma_in ||
        !imsigma)
      fail(EPSP_EINVAL, "an array pointer is NULL");
    if (!(T >= 0)) fail(EPSP_EINVAL, "Temperature must be positive");
    if (ni > 65535) fail(EPSP_EINVAL, "at most 65535 outer states");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    EPSP_CUDA(cudaSetDevice(c->device));
    // Set-up, once per device, with that device current: the device address of the scratch array.
    if (c->device < 0 || c->device >= 64) fail(EPSP_EINVAL, "device ordinal beyond 63");
    if (!g_scratch_dev[c->device]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) fail(EPSP_ECUDA, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      g_scratch_dev[c->device] = p;
    }
    // Grid checks and tables, as FrequencyGrid and cell_search_table (src/frequency_grids.jl:124-196),
    // by the helpers the plans use, into the fixed host staging arrays.
    const epsp_grid& g = *omegas;
    const int64_t mg = check_grid(g, "omegas");
    if (g.n > kNoallocMaxNodes)
      fail(EPSP_EINVAL, "omegas has " + std::to_string(g.n) + " nodes; epsp_scgd0_imsigma_noalloc takes at most " +
                            std::to_string(kNoallocMaxNodes));
    for (int64_t j = 0; j < g.n; ++j) g_nodes_host[j] = g.origin + double(g.offsets[j]) * g.unit;
    const double x0 = g_nodes_host[0];
    const double inv_h = cell_inv_h(g.unit * double(mg));
    const int64_t entries = cell_table_entries(g_nodes_host, g.n, inv_h);
    if (entries > kNoallocMaxTable)
      fail(EPSP_EINVAL, "the cell-search table of omegas needs " + std::to_string(entries) +
                            " entries; epsp_scgd0_imsigma_noalloc holds at most " + std::to_string(kNoallocMaxTable));
    fill_cell_table(g_nodes_host, g.n, inv_h, g_table_host, entries);
    unsigned char* base = static_cast<unsigned char*>(g_scratch_dev[c->device]);
    double* d_nodes = reinterpret_cast<double*>(base);
    int32_t* d_table = reinterpret_cast<int32_t*>(base + size_t(kNoallocMaxNodes) * 8);
    EPSP_CUDA(cudaMemcpyAsync(d_nodes, g_nodes_host, size_t(g.n) * 8, cudaMemcpyHostToDevice, c->stream));
    EPSP_CUDA(cudaMemcpyAsync(d_table, g_table_host, size_t(entries) * 4, cudaMemcpyHostToDevice, c->stream));
    CellTableDev ct{d_table, d_nodes, x0, inv_h, int(g.n)};
    dim3 grid(div_up(size_t(g.n), 128), unsigned(ni));
    fm_direct_noalloc_kernel<<<grid, 128, 0, c->stream>>>(d_nodes, int(g.n), ct, reinterpret_cast<const double2*>(sigma_in),
                                                          g2, omega_ph, iq_kk, iks_i, iks_f, nk_i, eps_f, w_f, f_to_i,
                                                          int(nm), int(ni), nf, mu, T, omega_acoustic, imsigma);
    EPSP_LAUNCHED(c);
    // The staging arrays and the scratch are reused by the next call: finish before returning.
    EPSP_CUDA(cudaStreamSynchronize(c->stream));
    c->last_error.clear();
    return EPSP_OK;
  } catch (const Error& e) {
    c->last_error = e.msg;
    return epsp_status(e.code);
  }
}
