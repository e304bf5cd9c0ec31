// scgd0_tc.cu -- the GEMM_BF16 path of the scGD0 iteration: the kernel tensor written directly as
// BF16 split operands, the Fan-Migdal contraction and the Kramers-Kronig map on the tcgen05 tensor
// cores (tc_gemm.cuh), split-K partials summed in fixed order.
//
//   ImΣ[ω, i] = Σ_k K_t[ω, k] G[k, i]      A = K_t  [nω][Kp]  (K-major),  B = G^T [ni][Kp]
//   ReΣ[ω, i] = Σ_ω' KK[ω, ω'] ImΣ[ω', i]   A = KK   [nω][Kp2],           B = ImΣ^T [ni][Kp2]
//
// Both contractions use the three-way split (x = hi + mid + lo, six products, ~2^-23 relative): the
// iteration's own convergence test compares successive Σ to tol (1e-6 eV for the benchmark), and a
// two-way split's ~2^-16 rounding of the map (~2e-6 eV here) would stall it above that.
#include "scgd0.cuh"
#include "fp_pair.cuh"
#include "tc_gemm.cuh"

#include <algorithm>

namespace epsp {

constexpr int kNs = 3;
// K-blocks of 64 summed by one FP32 accumulator at most: the Fan-Migdal sums are long and of one
// sign, and their FP32 rounding must stay well below the iteration's tol (1e-6 eV)
constexpr int kKbCap = 16;
// The Kramers-Kronig product's bound: its terms cancel (principal value), so the FP32 rounding of
// a long accumulation is large against the result (at 4101 nodes and 800 K, 16 K blocks per
// accumulator left |ΔReΣ| ~1e-5 eV against FP64, 4 K blocks ~3x less).
constexpr int kKbCapKK = 4;
// Split limit of a product of depth K: enough splits that no FP32 accumulator sums more than cap
// K blocks (the Fan-Migdal product of a 32^3 model has ~680), and at least 16.
static int max_splits_for(long K, int cap = kKbCap) {
  const long kb = (K + kTcBK - 1) / kTcBK;
  return int(std::max<long>(16, (kb + cap - 1) / cap));
}

struct Scgd0Plan::Tc {
  long Kp = 0, Kp2 = 0;
  int splits1 = 1, splits2 = 1, bn1 = 128, bn2 = 128;
  DBuf<__nv_bfloat16> Kt[kNs], G[kNs], KK[kNs], Im[kNs];
  DBuf<float> part;
  DBuf<int> err;
  TcOperand opK, opG, opKK, opIm;
  // FP32 forms of the K-tensor inputs: cell points as float pairs (hi, lo), cell weights, the cell
  // energies as pairs, the occupation tables, and per iteration Σin as {Re hi, Re lo, Im, 0}
  DBuf<float2> xf, ef;
  DBuf<float> tf, Ff;
  DBuf<float4> Sf;
  // 1 for modes below the acoustic cutoff (left out of the sum)
  DBuf<uint8_t> skip;
  // batched iteration: capacity in temperatures, ImΣ of every slot
  long capT = 1;
  DBuf<double> ImS_b;
};

__global__ void split_df_kernel(const double* __restrict__ x, long n, float2* __restrict__ out) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) out[k] = split_df(x[k]);
}

// gw[vf + nvf i] = w_f[f] g2t[vf + nvf i] rounded to FP32 (vf = ν + nm f).
__global__ void gw_f32_kernel(const double* __restrict__ g2t, const double* __restrict__ w_f, int nm, long nvf, long ni,
                              float* __restrict__ gw) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= nvf * ni) return;
  gw[k] = float(w_f[(k % nvf) / nm] * g2t[k]);
}

__global__ void to_f32_kernel(const double* __restrict__ x, long n, float* __restrict__ out) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) out[k] = float(x[k]);
}

__global__ void sigma_f32_kernel(const double2* __restrict__ S, long n, float4* __restrict__ out) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double2 z = S[k];
  const float2 r = split_df(z.x);
  out[k] = make_float4(r.x, r.y, float(z.y), 0.f);
}

// Kernel tensor of the recast Fan-Migdal sum (see kbuild_f64_kernel in scgd0.cu), written as BF16
// split rows K_t[ω][k], k = c nm + ν, through a shared-memory transpose. The cells of ω ± ω_ν come
// from the setup table; Re z = (x - ε) - Re Σ(x), which cancels near the quasiparticle pole, is
// formed exactly from float pairs (re_z), and Im Σ(x), the reciprocal and the occupation products
// are FP32: the kernel runs on the FP32 units only.
// Grid (nω / 16, Kp / (kKbCols nm), slots), 256 threads: thread (node ω0 + t % 16, modes t / 16,
// t / 16 + 16, ..) loads the cells and occupations of its (ω, ν) once and runs over the block's
// kKbCols columns c (their Σ column and energy from shared memory), so per element only the two
// interpolations of Σ and the arithmetic remain. Dynamic shared memory: the tile [kKbCols nm][17]
// floats. kKbCols nm must be a multiple of 8, so that the write-out's 16-byte chunks never
// straddle two blocks (nor Kp, a multiple of 64).
constexpr int kKbCols = 8;
constexpr int kKbW = 16;
__global__ void __launch_bounds__(256, 6) kbuild_bf16_kernel(int nw, long slab, const float4* __restrict__ Sf_all,
                                                          const int32_t* __restrict__ cell_j,
                                                          const float* __restrict__ cell_t,
                                                          const float2* __restrict__ cell_x,
                                                          const uint8_t* __restrict__ skip, int nm,
                                                          const float2* __restrict__ eps_c,
                                                          const int32_t* __restrict__ col_c, int nc,
                                                          const float* __restrict__ F_all,
                                                          __nv_bfloat16* __restrict__ K0, __nv_bfloat16* __restrict__ K1,
                                                          __nv_bfloat16* __restrict__ K2, long Kp) {
  extern __shared__ float kb_tile[];  // [kKbCols nm][kKbW + 1]
  __shared__ int s_col[kKbCols];
  __shared__ float2 s_eps[kKbCols];
  const int w0 = blockIdx.x * kKbW;
  const int cbeg = blockIdx.y * kKbCols;
  const int tw = threadIdx.x % kKbW, tm = threadIdx.x / kKbW;
  const int iw = w0 + tw;
  const int nwm = nw * nm;
  const float4* Sf = Sf_all + slab * blockIdx.z;
  const float* F = F_all + 2l * nwm * blockIdx.z;
  if (threadIdx.x < kKbCols) {
    const int c = cbeg + threadIdx.x;
    s_col[threadIdx.x] = c < nc ? nw * col_c[c] : -1;
    s_eps[threadIdx.x] = c < nc ? eps_c[c] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int nu = tm; nu < nm; nu += 256 / kKbW) {
    const bool on = iw < nw && !skip[nu];
    int ja = 0, je = 0;
    float ta = 0.f, te = 0.f, Fa = 0.f, Fe = 0.f;
    float2 xa = make_float2(0.f, 0.f), xe = xa;
    if (on) {
      const int ia = iw + nw * nu, ie = ia + nwm;
      ja = cell_j[ia];
      je = cell_j[ie];
      ta = cell_t[ia];
      te = cell_t[ie];
      xa = cell_x[ia];
      xe = cell_x[ie];
      Fa = F[ia];
      Fe = F[ie];
    }
#pragma unroll 4
    for (int cl = 0; cl < kKbCols; ++cl) {
      const int co = s_col[cl];
      float v = 0.f;
      if (on && co >= 0) {
        const float4* col = Sf + co;
        const float2 e = s_eps[cl];
        const float4 la = col[ja], ha = col[ja + 1], le = col[je], he = col[je + 1];
        const float zar = re_z(xa, e, la, ha, ta);
        const float zer = re_z(xe, e, le, he, te);
        const float sia = (1.f - ta) * la.z + ta * ha.z;  // Im Σ(x)
        const float sie = (1.f - te) * le.z + te * he.z;
        // Im 1/z with Im z = -Im Σ; the K tensor carries FP32 precision, so an approximate
        // division (2 ulp; denominators here lie far inside its range) is enough
        const float ga = __fdividef(sia, zar * zar + sia * sia);
        const float ge = __fdividef(sie, zer * zer + sie * sie);
        v = ga * Fa + ge * Fe;
      }
      kb_tile[(cl * nm + nu) * (kKbW + 1) + tw] = v;
    }
  }
  __syncthreads();
  // write-out: the block's columns [cbeg nm, (cbeg + kKbCols) nm) of rows ω0.., 8 BF16 per store; a
  // half-warp writes one row's chunks (contiguous)
  const long kbeg = long(cbeg) * nm;
  const int nchunk = kKbCols * nm / 8;
  const long krow0 = long(nw) * blockIdx.z;
  for (int wr = threadIdx.x / 16; wr < kKbW; wr += 16) {
    for (int ch = threadIdx.x % 16; ch < nchunk; ch += 16) {
      const int ow = w0 + wr;
      const long k = kbeg + 8 * ch;
      if (ow >= nw || k >= Kp) continue;
      __align__(16) __nv_bfloat16 p0[8], p1[8], p2[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        __nv_bfloat16 q[3];
        split_bf16_n(kb_tile[(8 * ch + j) * (kKbW + 1) + wr], 3, q);
        p0[j] = q[0];
        p1[j] = q[1];
        p2[j] = q[2];
      }
      const long off = (krow0 + ow) * Kp + k;
      *reinterpret_cast<uint4*>(K0 + off) = *reinterpret_cast<const uint4*>(p0);
      *reinterpret_cast<uint4*>(K1 + off) = *reinterpret_cast<const uint4*>(p1);
      *reinterpret_cast<uint4*>(K2 + off) = *reinterpret_cast<const uint4*>(p2);
    }
  }
}

static size_t kbuild_smem_bytes(long nm) { return size_t(kKbCols * nm * (kKbW + 1)) * sizeof(float); }

// ---- dispersive phonons: the Fan-Migdal sum term by term in FP32 ----
// The reference's element sum (src/scgd0_kernel.jl:27-39, 59-86) with ωq gathered per pair
// (ωq[ν, f, i] = ωph[ν, iq_kk[iks_i[i], iks_f[f]]], src/scgd0.jl:270): for each (ω, i) and every
// (ν, f) with ωq >= ω_acoustic, w_f g2 {Im[1/(x_a - ε_f - Σ_in(x_a))] (n + f(x_a - μ)) +
// Im[1/(x_e - ε_f - Σ_in(x_e))] (n + 1 - f(x_e - μ))}, x_a,e = ω ± ωq. FP32 arithmetic with float
// pairs where the value cancels: x = ω ± ωq, ε_f and Re Σ are float pairs and Re z = (x - ε) - Re Σ(x)
// is formed exactly on them (re_z), as in kbuild_bf16_kernel; the cell of x (the O(1) bucket table of
// _interp_linear_grid, flat outside the grid: a bucket, then one node entry that carries the inverse
// widths of both its cells, so the weight needs no division) is found on the pair; the weight, Im Σ,
// the reciprocal and the occupations are FP32, the Fermi factors from exp((ω - μ)/T) exp(±ωq/T)
// (one exponential per thread and one per staged mode instead of two per term; evaluated directly
// where a factor leaves FP32's range), and each thread sums its terms in FP32 runs of one tile
// (256 pairs (ν, f)) added into FP64. The (ν, f) tile of the block's outer state -- w_f g2, ωq,
// n(ωq), exp(±ωq/T), ε_f, the Σ column -- is staged in shared memory by the block; the node table
// and the bucket table too, when they fit.
// Grid (nω / 256, ni, slots), 256 threads, thread = node ω. Slot a reads Σ_in from Sf_all + a nω ni
// and T, μ from tp[slots[a]]. Output: with ImS_b, ImΣ of the slot (ImS_b + a nω ni) and its BF16
// split as the Kramers-Kronig product's B operand (rows a ni + i, columns ω, stride Kp2), as
// finalize_fm_batch_kernel writes them; else ImΣ added into add_out [nω, ni] (slot 0).
constexpr int kFdTile = 256;

__device__ __forceinline__ float2 pair_add(float2 a, float2 b) {  // a + b as a float pair
  float e;
  const float s = two_sum(a.x, b.x, e);
  e += a.y + b.y;
  const float h = s + e;
  return make_float2(h, e - (h - s));
}
__device__ __forceinline__ bool pair_le(float2 a, float2 b) {  // a <= b for float pairs (normalised)
  return a.x < b.x || (a.x == b.x && a.y <= b.y);
}
__device__ __forceinline__ float occ_fermion_f(float e, float T) {  // occ_fermion, src/utils.jl:14-22
  if (T > 1.4901161193847656e-08f) return 1.f / (__expf(e / T) + 1.f);
  return e > 0.f ? 0.f : (e < 0.f ? 1.f : 0.5f);
}
__device__ __forceinline__ float occ_boson_f(float e, float T) {  // occ_boson, src/utils.jl:24-38
  if (T > 1.4901161193847656e-08f) return e == 0.f ? -0.5f : 1.f / expm1f(e / T);
  return e > 0.f ? 0.f : (e == 0.f ? -0.5f : -1.f);
}

template <bool kSmemTab>
__global__ void __launch_bounds__(kFdTile) fm_disp_f32_kernel(
    int nw, long slab, const float4* __restrict__ Sf_all, const float4* __restrict__ wtab_g,
    const int32_t* __restrict__ jtab_g, float x0, float inv_h, long ntab, const float* __restrict__ gw,
    const double* __restrict__ wph, const int32_t* __restrict__ iq_kk, const int32_t* __restrict__ iks_i,
    const int32_t* __restrict__ iks_f, long nk_i, const double* __restrict__ eps_f, const int32_t* __restrict__ f_to_i,
    int nm, long nvf, int ni, double w_ac, const int* __restrict__ slots, const TParams* __restrict__ tp,
    double* __restrict__ ImS_b, __nv_bfloat16* __restrict__ Im0, __nv_bfloat16* __restrict__ Im1,
    __nv_bfloat16* __restrict__ Im2, long Kp2, double* __restrict__ add_out) {
  extern __shared__ __align__(16) unsigned char fd_tab[];  // kSmemTab: node table [nw] float4, then the buckets
  // the staged (ν, f) pairs: {w_f g2, n(ωq), exp(ωq/T), exp(-ωq/T)}, {ε - ωq, ε + ωq} as float pairs,
  // {ωq as a float pair, the Σ column's offset, 0}
  __shared__ float4 s_a[kFdTile], s_e[kFdTile], s_q[kFdTile];
  const float4* wtab = wtab_g;
  const int32_t* jtab = jtab_g;
  if constexpr (kSmemTab) {
    float4* sw = reinterpret_cast<float4*>(fd_tab);
    int32_t* sj = reinterpret_cast<int32_t*>(fd_tab + sizeof(float4) * size_t(nw));
    for (int k = threadIdx.x; k < nw; k += kFdTile) sw[k] = wtab_g[k];
    for (long k = threadIdx.x; k < ntab; k += kFdTile) sj[k] = jtab_g[k];
    wtab = sw;
    jtab = sj;
  }
  const int i = blockIdx.y, a = blockIdx.z;
  const int iw = blockIdx.x * kFdTile + threadIdx.x;
  const bool on = iw < nw;
  const TParams q = tp[slots[a]];
  const float T = float(q.T);
  const bool warm = T > 1.4901161193847656e-08f;
  const float invT = warm ? 1.f / T : 0.f;
  const float2 mu = split_df(q.mu);
  const float4* Sf = Sf_all + slab * a;
  const float4 wn = wtab_g[on ? iw : 0];
  const float2 w = make_float2(wn.x, wn.y);
  // exp((ω - μ)/T) of the thread's node: f(ω ± ωq - μ) = 1 / (E exp(±ωq/T) + 1); a node whose E
  // leaves FP32's range takes the exponential of each term directly
  const float wm = (w.x - mu.x) + (w.y - mu.y);
  const float E = warm ? __expf(wm * invT) : 0.f;
  const bool Eok = warm && E > 0.f && E < INFINITY;
  const int ntab_i = int(ntab), jmax = nw - 2;
  const int ki = iks_i[i];
  // one side of a term, x = ω + sg ωq (sg = ±1), with em = ε - sg ωq: Im 1/(x - ε - Σ(x)) times its
  // occupation bracket
  auto side = [&](const float4* col, float sgwq_hi, float sgwq_lo, float2 em, float nq, float eq, bool absorb) -> float {
    const float xh = w.x + sgwq_hi;
    const float v = fminf(fmaxf((xh - x0) * inv_h, -1.f), float(ntab_i)) - 0.5f;
    // the bucket floor((x - x0) / h) in 32-bit integer arithmetic (1.5 2^23 added: the integer part
    // lands in the mantissa; |v| < 2^22); an off-by-one bucket at a bucket edge still picks the
    // cell whose value is continuous there
    int b = __float_as_int(v + 12582912.f) - 0x4B400000;
    b = min(max(b, 0), ntab_i - 1);
    const int c = jtab[b];
    const float4 wc = wtab[c];  // node c: (hi, lo, 1 / (w[c+1] - w[c]), 1 / (w[c] - w[c-1]))
    const float dx = ((w.x - wc.x) + sgwq_hi) + ((w.y - wc.y) + sgwq_lo);
    const bool below = dx < 0.f;
    int j = below ? c - 1 : c;
    float t = below ? fmaf(dx, wc.w, 1.f) : dx * wc.z;
    if (j < 0 || j > jmax) {  // outside the grid the value is flat (the first or the last node)
      t = j < 0 ? 0.f : 1.f;
      j = j < 0 ? 0 : jmax;
    }
    const float4 lo = col[j], hi = col[j + 1];
    // Re z = (x - ε) - Re Σ(x) = (ω - em) - Re Σ(x), exact on the float pairs
    const float zr = re_z(w, em, lo, hi, t);
    const float si = fmaf(t, hi.z - lo.z, lo.z);  // Im Σ(x)
    const float g = __fdividef(si, fmaf(zr, zr, si * si));
    float y = E * eq;
    if (!Eok || y != y) {  // a factor out of range (stored as NaN), or T -> 0
      const float xm = (xh - mu.x) + ((w.y + sgwq_lo) - mu.y);
      y = warm ? __expf(xm * invT) : (xm > 0.f ? INFINITY : (xm < 0.f ? 0.f : 1.f));
    }
    const float f = __fdividef(1.f, y + 1.f);
    return g * (absorb ? nq + f : nq + 1.f - f);
  };
  double acc = 0.0;
  for (long t0 = 0; t0 < nvf; t0 += kFdTile) {
    const long vf = t0 + threadIdx.x;
    __syncthreads();  // the previous tile's readers are done (and, first, the tables are staged)
    // below ω_acoustic (and past the end) no term: zero coupling, the first column as a stand-in and
    // ε - ωq = -1e30, so that Re z^2 overflows and Im 1/z is exactly 0 whatever the column holds
    float4 sa = make_float4(0.f, 0.f, 0.f, 0.f), se = make_float4(-1e30f, 0.f, -1e30f, 0.f), sq = sa;
    if (vf < nvf) {
      const int nu = int(vf % nm);
      const long f = vf / nm;
      const double wq = wph[nu + long(nm) * iq_kk[ki + nk_i * long(iks_f[f])]];
      if (!(wq < w_ac)) {
        const double e = eps_f[f];
        const float wqf = float(wq);
        const float2 ea = split_df(e - wq), ee = split_df(e + wq), wqp = split_df(wq);
        float eq = warm ? __expf(wqf * invT) : 0.f, ieq = warm ? __expf(-wqf * invT) : 0.f;
        if (!(eq < INFINITY) || !(ieq > 0.f)) eq = ieq = __int_as_float(0x7fc00000);  // out of range: NaN
        sa = make_float4(gw[vf + nvf * i], occ_boson_f(wqf, T), eq, ieq);
        se = make_float4(ea.x, ea.y, ee.x, ee.y);
        sq = make_float4(wqp.x, wqp.y, __int_as_float(nw * f_to_i[f]), 0.f);
      }
    }
    s_a[threadIdx.x] = sa;
    s_e[threadIdx.x] = se;
    s_q[threadIdx.x] = sq;
    __syncthreads();
    float run0 = 0.f, run1 = 0.f;
    if (on) {
      const int nt = int(min(long(kFdTile), nvf - t0));
#pragma unroll 2
      for (int k = 0; k < nt; ++k) {
        const float4 A = s_a[k], Ee = s_e[k], Q = s_q[k];
        const float4* col = Sf + __float_as_int(Q.z);
        const float va = side(col, Q.x, Q.y, make_float2(Ee.x, Ee.y), A.y, A.z, true);
        const float ve = side(col, -Q.x, -Q.y, make_float2(Ee.z, Ee.w), A.y, A.w, false);
        const float v = A.x * (va + ve);
        if (k & 1)
          run1 += v;
        else
          run0 += v;
      }
    }
    acc += double(run0) + double(run1);
  }
  if (!on) return;
  const long k = iw + long(nw) * i;
  if (ImS_b) {
    ImS_b[slab * a + k] = acc;
    __nv_bfloat16 p[3];
    split_bf16_n(float(acc), 3, p);
    const long o = (long(a) * ni + i) * Kp2 + iw;
    Im0[o] = p[0];
    Im1[o] = p[1];
    Im2[o] = p[2];
  } else {
    add_out[k] += acc;
  }
}

// The node table of fm_disp_f32_kernel: node j as (hi, lo, 1 / (w[j+1] - w[j]), 1 / (w[j] - w[j-1]))
// (0 past the ends).
__global__ void fd_node_table_kernel(const double* __restrict__ ws, int nw, float4* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nw) return;
  const float2 p = split_df(ws[j]);
  const float up = j + 1 < nw ? float(1.0 / (ws[j + 1] - ws[j])) : 0.f;
  const float dn = j > 0 ? float(1.0 / (ws[j] - ws[j - 1])) : 0.f;
  out[j] = make_float4(p.x, p.y, up, dn);
}


// out_p[r * ld + c] = part p of S(r, c) for c < cols, 0 for cols <= c < ld, with S(r, c) =
// S[c + ldc r] (transposed = false: rows of the output are columns of the column-major S) or
// S[r + ldc c] (transposed = true).
__global__ void split3_rows_kernel(const double* __restrict__ S, long ldc, long rows, long cols, long ld, bool transposed,
                                   __nv_bfloat16* __restrict__ o0, __nv_bfloat16* __restrict__ o1,
                                   __nv_bfloat16* __restrict__ o2) {
  long idx = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= rows * ld) return;
  long r = idx / ld, c = idx % ld;
  float x = 0.f;
  if (c < cols) x = float(transposed ? S[r + ldc * c] : S[c + ldc * r]);
  __nv_bfloat16 q[3];
  split_bf16_n(x, 3, q);
  o0[idx] = q[0];
  o1[idx] = q[1];
  o2[idx] = q[2];
}

// ImΣ (FP64) += Σ_s part[s] in ascending s.
__global__ void finalize_add_kernel(const float* __restrict__ part, long n, int splits, long stride, double* __restrict__ out) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float s = 0.f;
  for (int p = 0; p < splits; ++p) s += part[k + stride * p];
  out[k] += double(s);
}

// Σ_new = Σ_s part[s] + i ImΣ.
__global__ void finalize_assemble_kernel(const float* __restrict__ part, long n, int splits, long stride,
                                         const double* __restrict__ im, double2* __restrict__ out) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float s = 0.f;
  for (int p = 0; p < splits; ++p) s += part[k + stride * p];
  out[k] = make_double2(double(s), im[k]);
}

// The occupation tables of the active temperatures as FP32 (computed in FP64 as occ_table_kernel):
// F[a][0 .. nω nm) absorption, F[a][nω nm .. 2 nω nm) emission.
__global__ void occ_table_f32_kernel(const double* __restrict__ ws, int nw, const double* __restrict__ wnu, int nm,
                                     const int* __restrict__ slots, const TParams* __restrict__ tp, double w_ac,
                                     float* __restrict__ F_all) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const long nwm = long(nw) * nm;
  if (k >= nwm) return;
  const int a = blockIdx.y;
  const TParams q = tp[slots[a]];
  float* F = F_all + 2 * nwm * a;
  const int iw = k % nw, nu = k / nw;
  const double wq = wnu[nu], w = ws[iw];
  if (wq < w_ac) {
    F[k] = 0.f;
    F[k + nwm] = 0.f;
    return;
  }
  const double nq = occ_boson_d(wq, q.T);
  F[k] = float(nq + occ_fermion_d(w + wq - q.mu, q.T));
  F[k + nwm] = float(nq + 1 - occ_fermion_d(w - wq - q.mu, q.T));
}

__global__ void sigma_f32_batch_kernel(const double2* __restrict__ S, long n, int nA, float4* __restrict__ out) {
  long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n * nA) return;
  const double2 z = S[k];
  const float2 r = split_df(z.x);
  out[k] = make_float4(r.x, r.y, float(z.y), 0.f);
}

// ImΣ of slot a: ImS[a][ω + nω i] = Σ_s part[s][(a nω + ω) + M i], M = nA nω (the stacked rows).
// With Im0 (the batched iteration), it also writes ImΣ split into the KK product's B operand (whose
// padding columns nω.. Kp2 stay zero from the reservation).
__global__ void finalize_fm_batch_kernel(const float* __restrict__ part, int nw, long slab, int nA, int splits,
                                         long stride, double* __restrict__ ImS, __nv_bfloat16* __restrict__ Im0 = nullptr,
                                         __nv_bfloat16* __restrict__ Im1 = nullptr, __nv_bfloat16* __restrict__ Im2 = nullptr,
                                         long Kp2 = 0) {
  const long k = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= slab) return;
  const int a = blockIdx.y;
  const long w = k % nw, i = k / nw;
  const long src = (long(a) * nw + w) + long(nA) * nw * i;
  float acc = 0.f;
  for (int p = 0; p < splits; ++p) acc += part[src + stride * p];
  ImS[slab * a + k] = double(acc);
  if (Im0) {  // and the B operand of the Kramers-Kronig product: row a ni + i, column ω, three parts
    __nv_bfloat16 q[3];
    split_bf16_n(acc, 3, q);
    const long o = (long(a) * (slab / nw) + i) * Kp2 + w;
    Im0[o] = q[0];
    Im1[o] = q[1];
    Im2[o] = q[2];
  }
}

// The Kramers-Kronig product's epilogue and the rest of the iteration's tail, in one pass over its
// split-K partials (src/scgd0.jl:287-301, 326-328): per state group of slot a -- a degenerate
// multiplet, or a single state -- Σ_new(ω_j) = Σ_s part[s] + i ImΣ of every member (the partials in
// ascending order), averaged over the members of a multiplet (their sum in member order divided by
// the count); then per member: err = max |Σ_new - Σ| over the slot's temperature (FP64 differences,
// FP32 magnitude, the maximum taken on the bit patterns as err_copy_kernel does), Σ ← Σ_new, and the
// spectral functions' per-node terms P[i][j] = (ε_i - ω_j + ReΣ_j, ReΣ_{j+1} - ReΣ_j, ImΣ_j, ImΣ_{j+1})
// of spectral_prep_f32_kernel (ImΣ_{j+1}, ReΣ_{j+1} = those of j at the last node). Bitwise the
// results of the separate kernels. Groups: CSR (gptr, gidx), members in order. Grid (nω / 255,
// groups, slots), 256 threads: thread t takes node j = 255 blockIdx.x + t; the last thread's node
// is the next block's first, formed again to give node 254 its neighbour.
__global__ void __launch_bounds__(256) kk_epilogue_kernel(const float* __restrict__ part, int splits, long stride,
                                                          const double* __restrict__ ImS_b, int nw, long slab,
                                                          const int* __restrict__ slots, const int32_t* __restrict__ gptr,
                                                          const int32_t* __restrict__ gidx, const double* __restrict__ ws,
                                                          const double* __restrict__ eps_i, double2* __restrict__ S_all,
                                                          float4* __restrict__ Pall,
                                                          unsigned long long* __restrict__ errbits_all,
                                                          double* __restrict__ minA_all) {
  __shared__ double2 sh[256];
  __shared__ unsigned long long she[256];
  const int a = blockIdx.z, t = slots[a];
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0)  // the minimum of spectral_fin starts at +inf
    minA_all[t] = INFINITY;
  const int j = blockIdx.x * 255 + threadIdx.x;
  const bool in = j < nw;
  const int p0 = gptr[blockIdx.y], p1 = gptr[blockIdx.y + 1];
  double sr = 0, si = 0;
  if (in) {
    for (int p = p0; p < p1; ++p) {
      const long src = slab * a + j + long(nw) * gidx[p];
      float acc = 0.f;
      for (int q = 0; q < splits; ++q) acc += part[src + stride * q];
      if (p1 - p0 == 1) {
        sr = double(acc);
        si = ImS_b[src];
      } else {
        sr += double(acc);
        si += ImS_b[src];
      }
    }
    if (p1 - p0 > 1) {
      const double len = double(p1 - p0);
      sr /= len;
      si /= len;
    }
  }
  sh[threadIdx.x] = make_double2(sr, si);
  __syncthreads();
  unsigned long long e = 0;
  if (in && threadIdx.x < 255) {
    const double2 lo = sh[threadIdx.x];
    const double2 hi = j + 1 < nw ? sh[threadIdx.x + 1] : lo;
    double2* S = S_all + slab * t;
    for (int p = p0; p < p1; ++p) {
      const int i = gidx[p];
      const long k = j + long(nw) * i;
      const double2 b = S[k];
      const double d = double(hypotf(float(lo.x - b.x), float(lo.y - b.y)));
      e = max(e, (unsigned long long)__double_as_longlong(d));
      S[k] = lo;
      Pall[slab * a + k] = make_float4(float(eps_i[i] - ws[j] + lo.x), float(hi.x - lo.x), float(lo.y), float(hi.y));
    }
  }
  she[threadIdx.x] = e;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) she[threadIdx.x] = max(she[threadIdx.x], she[threadIdx.x + st]);
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(errbits_all + t, she[0]);
}

static long pad64(long x) { return (x + 63) / 64 * 64; }

// K block of the three-part products' operand maps (64: two 96 KB pipeline stages; 32: four of
// 48 KB, measured no faster on these short products).
constexpr int kScgd0Bk = 64;

static TcOperand operand(DBuf<__nv_bfloat16>* parts, long rows, long cols, long ld, int box_rows) {
  TcOperand op;
  op.ns = kNs;
  op.bk = kScgd0Bk;
  for (int p = 0; p < kNs; ++p) op.m[p] = make_tmap_bf16(parts[p].p, rows, cols, ld, box_rows, kScgd0Bk);
  return op;
}

void tc_setup(Scgd0Plan* P) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  auto* T = new Scgd0Plan::Tc;
  P->tc = std::unique_ptr<Scgd0Plan::Tc, void (*)(Scgd0Plan::Tc*)>(T, [](Scgd0Plan::Tc* t) { delete t; });
  const long nw = P->nw, ni = P->ni, nk = P->nm * P->nc;
  T->Kp = pad64(nk);
  T->Kp2 = pad64(nw);
  if (nw > (1l << 30) || ni > (1l << 30) || nk > (1l << 30)) fail(EPSP_EINVAL, "sizes beyond the 32-bit tile grid");
  if (P->disp) {  // the Kramers-Kronig map's operands only: the Fan-Migdal sum is fm_disp_f32_kernel
    for (int p = 0; p < kNs; ++p) {
      T->KK[p].alloc(ctx, size_t(nw * T->Kp2));
      T->Im[p].alloc(ctx, size_t(ni * T->Kp2));
    }
    T->err.alloc(ctx, 1);
    T->err.zero(s);
    split3_rows_kernel<<<div_up(size_t(nw * T->Kp2), 256), 256, 0, s>>>(P->d_KK.p, nw, nw, nw, T->Kp2, true, T->KK[0].p,
                                                                        T->KK[1].p, T->KK[2].p);
    EPSP_LAUNCHED(ctx);
    tc_gemm_shape(ctx, int(nw), int(ni), int(nw), max_splits_for(nw, kKbCapKK), kNs, &T->bn2, &T->splits2, kKbCapKK);
    T->part.alloc(ctx, size_t(T->splits2) * size_t(nw * ni));
    T->Sf.alloc(ctx, size_t(nw * ni));
    T->opKK = operand(T->KK, nw, nw, T->Kp2, kTcBM);
    T->opIm = operand(T->Im, ni, nw, T->Kp2, T->bn2);
    return;
  }
  if (kbuild_smem_bytes(P->nm) > size_t(227 * 1024))
    fail(EPSP_EUNSUPPORTED, "the BF16 scGD0 path takes at most 427 modes; use EPSP_PATH_GEMM_FP64");
  if (kbuild_smem_bytes(P->nm) > size_t(48 * 1024))
    EPSP_CUDA(cudaFuncSetAttribute(kbuild_bf16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   int(kbuild_smem_bytes(P->nm))));
  for (int p = 0; p < kNs; ++p) {
    T->Kt[p].alloc(ctx, size_t(nw * T->Kp));
    T->G[p].alloc(ctx, size_t(ni * T->Kp));
    T->KK[p].alloc(ctx, size_t(nw * T->Kp2));
    T->Im[p].alloc(ctx, size_t(ni * T->Kp2));
  }
  T->err.alloc(ctx, 1);
  T->err.zero(s);
  {
    std::vector<double> wnu(static_cast<size_t>(P->nm));
    P->d_wnu.download(wnu.data(), wnu.size(), s);
    EPSP_CUDA(cudaStreamSynchronize(s));
    std::vector<uint8_t> skip(wnu.size());
    for (size_t nu = 0; nu < wnu.size(); ++nu) skip[nu] = wnu[nu] < P->w_ac ? 1 : 0;
    T->skip = to_device(ctx, skip);
  }
  // B of the contraction: G [nk, ni] column-major is G^T row-major [ni][nk].
  split3_rows_kernel<<<div_up(size_t(ni * T->Kp), 256), 256, 0, s>>>(P->d_G.p, nk, ni, nk, T->Kp, false, T->G[0].p,
                                                                     T->G[1].p, T->G[2].p);
  EPSP_LAUNCHED(ctx);
  // A of the Kramers-Kronig map: A[ω][ω'] = KK[ω + nω ω'].
  split3_rows_kernel<<<div_up(size_t(nw * T->Kp2), 256), 256, 0, s>>>(P->d_KK.p, nw, nw, nw, T->Kp2, true, T->KK[0].p,
                                                                      T->KK[1].p, T->KK[2].p);
  EPSP_LAUNCHED(ctx);
  tc_gemm_shape(ctx, int(nw), int(ni), int(nk), max_splits_for(nk), kNs, &T->bn1, &T->splits1, kKbCap);
  tc_gemm_shape(ctx, int(nw), int(ni), int(nw), max_splits_for(nw, kKbCapKK), kNs, &T->bn2, &T->splits2, kKbCapKK);
  T->part.alloc(ctx, size_t(std::max(T->splits1, T->splits2)) * size_t(nw * ni));
  const long nwm = nw * P->nm;
  T->xf.alloc(ctx, size_t(2 * nwm));
  T->tf.alloc(ctx, size_t(2 * nwm));
  T->Ff.alloc(ctx, size_t(2 * nwm));
  T->ef.alloc(ctx, size_t(P->nc));
  T->Sf.alloc(ctx, size_t(nw * ni));
  split_df_kernel<<<div_up(size_t(2 * nwm), 256), 256, 0, s>>>(P->d_cell_x.p, 2 * nwm, T->xf.p);
  EPSP_LAUNCHED(ctx);
  to_f32_kernel<<<div_up(size_t(2 * nwm), 256), 256, 0, s>>>(P->d_cell_t.p, 2 * nwm, T->tf.p);
  EPSP_LAUNCHED(ctx);
  split_df_kernel<<<div_up(size_t(P->nc), 256), 256, 0, s>>>(P->d_epsc.p, P->nc, T->ef.p);
  EPSP_LAUNCHED(ctx);
  T->opK = operand(T->Kt, nw, nk, T->Kp, kTcBM);
  T->opG = operand(T->G, ni, nk, T->Kp, T->bn1);
  T->opKK = operand(T->KK, nw, nw, T->Kp2, kTcBM);
  T->opIm = operand(T->Im, ni, nw, T->Kp2, T->bn2);
}

static void check_err(Scgd0Plan* P) {
  int e = 0;
  P->tc->err.download(&e, 1, P->ctx->stream);
  EPSP_CUDA(cudaStreamSynchronize(P->ctx->stream));
  if (e) {
    P->tc->err.zero(P->ctx->stream);  // cleared, so that the plan's next call starts clean
    fail(EPSP_EDEVICE_TIMEOUT, "a tensor-core GEMM wait ran out (bounded device wait)");
  }
}

// fm_disp_f32_kernel over nA slots (Σ_in in T->Sf): into ImS_b and the Kramers-Kronig operand, or
// added into add_out (one slot).
static void launch_fm_disp(Scgd0Plan* P, int nA, const int* d_slots, const TParams* d_tp, double* ImS_b,
                           double* add_out) {
  Ctx* ctx = P->ctx;
  auto* T = P->tc.get();
  const long nw = P->nw, ni = P->ni;
  // the grid nodes and the bucket table in shared memory when they fit 96 KB
  const size_t tab = sizeof(float4) * size_t(nw) + sizeof(int32_t) * size_t(P->ntab);
  const bool smem = tab <= (size_t(96) << 10);
  const dim3 grid(div_up(size_t(nw), kFdTile), unsigned(ni), unsigned(nA));
  static size_t smem_set = 0;
  if (smem && tab > smem_set) {
    EPSP_CUDA(cudaFuncSetAttribute(fm_disp_f32_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tab)));
    smem_set = tab;
  }
  auto args = [&](auto kern, size_t bytes) {
    kern<<<grid, kFdTile, bytes, ctx->stream>>>(
        int(nw), nw * ni, T->Sf.p, P->d_wtab.p, P->d_jtab.p, P->x0f, P->inv_hf, P->ntab, P->d_gwf.p, P->d_wph.p,
        P->d_iq.p, P->d_iksi.p, P->d_iksf.p, P->nk_i, P->d_epsf.p, P->d_fti.p, int(P->nm), P->nm * P->nf, int(ni),
        P->w_ac, d_slots, d_tp, ImS_b, T->Im[0].p, T->Im[1].p, T->Im[2].p, T->Kp2, add_out);
  };
  if (smem)
    args(fm_disp_f32_kernel<true>, tab);
  else
    args(fm_disp_f32_kernel<false>, size_t(0));
  EPSP_LAUNCHED(ctx);
}

// One Fan-Migdal sum at (μ, T) for a model with dispersive modes, added into d_ImS.
void tc_imsigma_disp(Scgd0Plan* P, const double2* d_Sin, double mu, double T, double* d_ImS) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  auto* T_ = P->tc.get();
  const long nw = P->nw, ni = P->ni;
  sigma_f32_kernel<<<div_up(size_t(nw * ni), 256), 256, 0, s>>>(d_Sin, nw * ni, T_->Sf.p);
  EPSP_LAUNCHED(ctx);
  TParams q{};
  q.T = T;
  q.mu = mu;
  DBuf<TParams> d_q = to_device(ctx, &q, 1);
  DBuf<int> d_slot0;
  d_slot0.alloc(ctx, 1);
  d_slot0.zero(s);
  long pk = prof_begin(ctx, "fm_disp");
  launch_fm_disp(P, 1, d_slot0.p, d_q.p, nullptr, d_ImS);
  prof_end(ctx, pk);
  EPSP_CUDA(cudaStreamSynchronize(s));  // the parameter buffers are locals
}

// The tables of fm_disp_f32_kernel (see Scgd0Plan): w_f g2 permuted to [ν f, i] and rounded to
// FP32, ωph, iq_kk, iks_i, iks_f, f_to_i, ε_f and the grid nodes as float pairs, the bucket table's
// origin and scale. ωq itself is gathered per term, never stored.
void tc_setup_dispersive(Scgd0Plan* P, const epsp_model* m) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  P->disp = true;
  const long nm = m->nm, ni = m->ni, nf = m->nf, nvf = nm * nf;
  {
    DBuf<double> g2t;
    upload_g2_permuted(ctx, m, g2t);
    auto d_wf = to_device(ctx, m->w_f, size_t(nf));
    auto d_fti = to_device(ctx, m->f_to_i, size_t(nf));
    P->d_gwf.alloc(ctx, size_t(nvf * ni));
    gw_f32_kernel<<<div_up(size_t(nvf * ni), 256), 256, 0, s>>>(g2t.p, d_wf.p, int(nm), nvf, ni, P->d_gwf.p);
    EPSP_LAUNCHED(ctx);
    EPSP_CUDA(cudaStreamSynchronize(s));
  }
  P->d_wph = to_device(ctx, m->omega_ph, size_t(nm * m->nq));
  P->d_iq = to_device(ctx, m->iq_kk, size_t(m->nk_i * m->nk_f));
  P->d_iksi = to_device(ctx, m->iks_i, size_t(ni));
  P->d_iksf = to_device(ctx, m->iks_f, size_t(nf));
  P->d_fti = to_device(ctx, m->f_to_i, size_t(nf));
  P->nk_i = m->nk_i;
  P->d_epsf = to_device(ctx, m->eps_f, size_t(nf));
  P->d_wtab.alloc(ctx, size_t(P->nw));
  fd_node_table_kernel<<<div_up(size_t(P->nw), 256), 256, 0, s>>>(P->d_ws.p, int(P->nw), P->d_wtab.p);
  EPSP_LAUNCHED(ctx);
  P->x0f = float(P->ct.x0);
  P->inv_hf = float(P->ct.inv_h);
  P->ntab = long(P->d_jtab.n);
  if (P->ntab >= (long(1) << 21))
    fail(EPSP_EUNSUPPORTED, "the grid's cell-search table is too long for the FP32 dispersive path (2^21 buckets at "
                            "most); use EPSP_PATH_DIRECT_FP64");
  EPSP_CUDA(cudaStreamSynchronize(s));
}

void tc_imsigma(Scgd0Plan* P, const double2* d_Sin, double* d_ImS) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  auto* T = P->tc.get();
  const long nw = P->nw, ni = P->ni, nk = P->nm * P->nc;
  long pk = prof_begin(ctx, "kbuild");
  const long nwm = nw * P->nm;
  sigma_f32_kernel<<<div_up(size_t(nw * ni), 256), 256, 0, s>>>(d_Sin, nw * ni, T->Sf.p);
  EPSP_LAUNCHED(ctx);

  to_f32_kernel<<<div_up(size_t(nwm), 256), 256, 0, s>>>(P->d_Fa.p, nwm, T->Ff.p);
  EPSP_LAUNCHED(ctx);
  to_f32_kernel<<<div_up(size_t(nwm), 256), 256, 0, s>>>(P->d_Fe.p, nwm, T->Ff.p + nwm);
  EPSP_LAUNCHED(ctx);
  kbuild_bf16_kernel<<<dim3(div_up(size_t(nw), kKbW), unsigned(div_up(size_t(T->Kp), size_t(kKbCols * P->nm))), 1), 256,
                       kbuild_smem_bytes(P->nm), s>>>(int(nw), nw * ni, T->Sf.p, P->d_cell_j.p, T->tf.p, T->xf.p,
                                                      T->skip.p, int(P->nm), T->ef.p, P->d_colc.p, int(P->nc), T->Ff.p,
                                                      T->Kt[0].p, T->Kt[1].p, T->Kt[2].p, T->Kp);
  EPSP_LAUNCHED(ctx);
  prof_end(ctx, pk);
  const long slab = nw * ni;
  int sp = tc_gemm_launch(ctx, T->opK, T->opG, int(nw), int(ni), int(nk), T->part.p, nw, slab, max_splits_for(nk),
                          T->err.p, "tc_fm", kKbCap);
  finalize_add_kernel<<<div_up(size_t(slab), 256), 256, 0, s>>>(T->part.p, slab, sp, slab, d_ImS);
  EPSP_LAUNCHED(ctx);
  check_err(P);
}

void tc_kk_assemble(Scgd0Plan* P, double2* d_Snew) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  auto* T = P->tc.get();
  const long nw = P->nw, ni = P->ni, slab = nw * ni;
  split3_rows_kernel<<<div_up(size_t(ni * T->Kp2), 256), 256, 0, s>>>(P->d_ImS.p, nw, ni, nw, T->Kp2, false, T->Im[0].p,
                                                                      T->Im[1].p, T->Im[2].p);
  EPSP_LAUNCHED(ctx);
  int sp = tc_gemm_launch(ctx, T->opKK, T->opIm, int(nw), int(ni), int(nw), T->part.p, nw, slab,
                          max_splits_for(nw, kKbCapKK), T->err.p, "tc_kk", kKbCapKK);
  finalize_assemble_kernel<<<div_up(size_t(slab), 256), 256, 0, s>>>(T->part.p, slab, sp, slab, P->d_ImS.p, d_Snew);
  EPSP_LAUNCHED(ctx);
}

void tc_reserve(Scgd0Plan* P, long nT) {
  auto* T = P->tc.get();
  if (nT <= T->capT && T->ImS_b.p) return;
  Ctx* ctx = P->ctx;
  const long nw = P->nw, ni = P->ni, nk = P->nm * P->nc, nwm = nw * P->nm, slab = nw * ni;
  nT = std::max(nT, T->capT);
  if (nT * nw > (1l << 30) || nT * ni > (1l << 30)) fail(EPSP_EINVAL, "too many temperatures for the 32-bit tile grid");
  for (int p = 0; p < kNs; ++p) {
    if (!P->disp) T->Kt[p].alloc(ctx, size_t(nT * nw * T->Kp));
    T->Im[p].alloc(ctx, size_t(nT * ni * T->Kp2));
    T->Im[p].zero(ctx->stream);  // the padding columns nω.. Kp2 of the KK operand stay zero
  }
  T->Sf.alloc(ctx, size_t(nT * slab));
  if (!P->disp) T->Ff.alloc(ctx, size_t(nT * 2 * nwm));
  T->ImS_b.alloc(ctx, size_t(nT * slab));
  size_t part = 0;
  for (long a = 1; a <= nT; ++a) {
    int bn, sp1 = 1, sp2;
    if (!P->disp) tc_gemm_shape(ctx, int(a * nw), int(ni), int(nk), max_splits_for(nk), kNs, &bn, &sp1, kKbCap);
    tc_gemm_shape(ctx, int(nw), int(a * ni), int(nw), max_splits_for(nw, kKbCapKK), kNs, &bn, &sp2, kKbCapKK);
    part = std::max(part, size_t(std::max(sp1, sp2)) * size_t(a * slab));
  }
  T->part.alloc(ctx, part);
  if (!P->disp) T->opK = operand(T->Kt, nT * nw, nk, T->Kp, kTcBM);
  T->opIm = operand(T->Im, nT * ni, nw, T->Kp2, T->bn2);
  T->capT = nT;
}

void tc_check(Scgd0Plan* P) { check_err(P); }

int* tc_err_ptr(Scgd0Plan* P) { return P->tc->err.p; }

long tc_capacity(Scgd0Plan* P) { return P->tc->ImS_b.p ? P->tc->capT : 0; }

float4* tc_sigma_f32(Scgd0Plan* P) { return P->tc->Sf.p; }

static void tc_kk_tail(Scgd0Plan* P, int nA, const int* d_slots, double2* d_S_all, float4* d_P,
                       unsigned long long* d_errbits, double* d_minA);

void tc_iterate(Scgd0Plan* P, int nA, const int* d_slots, const int* slots_h, const TParams* d_tp,
                const double2* d_Sin_b, double2* d_S_all, float4* d_P, unsigned long long* d_errbits, double* d_minA) {
  (void)slots_h;
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  auto* T = P->tc.get();
  if (nA > T->capT) fail(EPSP_EINVAL, "more active temperatures than reserved");
  const long nw = P->nw, ni = P->ni, nk = P->nm * P->nc, nwm = nw * P->nm, slab = nw * ni;
  const unsigned eb = div_up(size_t(slab), 256);
  long pp = prof_begin(ctx, "kprep");
  if (d_Sin_b) {
    sigma_f32_batch_kernel<<<div_up(size_t(slab * nA), 256), 256, 0, s>>>(d_Sin_b, slab, nA, T->Sf.p);
    EPSP_LAUNCHED(ctx);
  }
  if (P->disp) {  // dispersive modes: ImΣ of every slot term by term, then the same Kramers-Kronig tail
    prof_end(ctx, pp);
    long pk = prof_begin(ctx, "fm_disp");
    launch_fm_disp(P, nA, d_slots, d_tp, T->ImS_b.p, nullptr);
    prof_end(ctx, pk);
    tc_kk_tail(P, nA, d_slots, d_S_all, d_P, d_errbits, d_minA);
    return;
  }
  // small blocks: the FP64 exponentials of the table spread over every SM
  occ_table_f32_kernel<<<dim3(div_up(size_t(nwm), 64), unsigned(nA)), 64, 0, s>>>(
      P->d_ws.p, int(nw), P->d_wnu.p, int(P->nm), d_slots, d_tp, P->w_ac, T->Ff.p);
  EPSP_LAUNCHED(ctx);
  prof_end(ctx, pp);
  long pk = prof_begin(ctx, "kbuild");
  kbuild_bf16_kernel<<<dim3(div_up(size_t(nw), kKbW), unsigned(div_up(size_t(T->Kp), size_t(kKbCols * P->nm))),
                            unsigned(nA)),
                       256, kbuild_smem_bytes(P->nm), s>>>(int(nw), slab, T->Sf.p, P->d_cell_j.p, T->tf.p, T->xf.p,
                                                           T->skip.p, int(P->nm), T->ef.p, P->d_colc.p, int(P->nc), T->Ff.p,
                                                           T->Kt[0].p, T->Kt[1].p, T->Kt[2].p, T->Kp);
  EPSP_LAUNCHED(ctx);
  prof_end(ctx, pk);
  // ImΣ of every slot: the stacked K_t rows times G
  const long M = long(nA) * nw;
  int sp = tc_gemm_launch(ctx, T->opK, T->opG, int(M), int(ni), int(nk), T->part.p, M, M * ni, max_splits_for(nk),
                          T->err.p, "tc_fm", kKbCap);
  // ImΣ of every slot, and its BF16 split as the B operand of ReΣ = KK ImΣ (columns: the slots'
  // states in order)
  long pf = prof_begin(ctx, "finalize");
  finalize_fm_batch_kernel<<<dim3(eb, unsigned(nA)), 256, 0, s>>>(T->part.p, int(nw), slab, nA, sp, M * ni, T->ImS_b.p,
                                                                   T->Im[0].p, T->Im[1].p, T->Im[2].p, T->Kp2);
  EPSP_LAUNCHED(ctx);
  prof_end(ctx, pf);
  tc_kk_tail(P, nA, d_slots, d_S_all, d_P, d_errbits, d_minA);
}

// ReΣ = KK ImΣ for every slot (the split ImΣ rows already in T->Im) and the fused epilogue.
static void tc_kk_tail(Scgd0Plan* P, int nA, const int* d_slots, double2* d_S_all, float4* d_P,
                       unsigned long long* d_errbits, double* d_minA) {
  Ctx* ctx = P->ctx;
  cudaStream_t s = ctx->stream;
  auto* T = P->tc.get();
  const long nw = P->nw, ni = P->ni, slab = nw * ni;
  const long N2 = long(nA) * ni;
  int sp2 = tc_gemm_launch(ctx, T->opKK, T->opIm, int(nw), int(N2), int(nw), T->part.p, nw, nw * N2,
                           max_splits_for(nw, kKbCapKK), T->err.p, "tc_kk", kKbCapKK);
  long pf = prof_begin(ctx, "kk_epilogue");
  kk_epilogue_kernel<<<dim3(div_up(size_t(nw), 255), unsigned(P->ngroups), unsigned(nA)), 256, 0, s>>>(
      T->part.p, sp2, nw * N2, T->ImS_b.p, int(nw), slab, d_slots, P->d_gptr.p, P->d_gidx.p, P->d_ws.p, P->d_eps_i.p,
      d_S_all, d_P, d_errbits, d_minA);
  EPSP_LAUNCHED(ctx);
  prof_end(ctx, pf);
}

}  // namespace epsp
