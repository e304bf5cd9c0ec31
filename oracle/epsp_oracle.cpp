// epsp_oracle.cpp -- CPU FP64 restatement of EPSpectral.jl's scGD0 and ladder hot path.
//
// TEST INFRASTRUCTURE: the parity oracle and the CPU baseline (see epsp_oracle.h). Compiled with
// -ffp-contract=off so that a*b+c is rounded twice, as the reference's Julia code evaluates it.
// OpenMP splits the same axes the reference threads over (outer states i, GEMM columns), and each
// thread writes disjoint outputs, so results do not depend on the thread count
// (src/scgd0_kernel.jl:55-57).

#include "epsp_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using cplx = std::complex<double>;
constexpr double kPi = 3.14159265358979323846;
constexpr int64_t kChunkBytes = int64_t(1) << 30;  // CHUNK_BYTES, src/utils.jl:11

struct OracleError : std::runtime_error {
  int code;
  OracleError(int c, const std::string& s) : std::runtime_error(s), code(c) {}
};

int g_threads = 0;

void set_msg(char* msg, int32_t len, const char* s) {
  if (msg && len > 0) {
    std::snprintf(msg, size_t(len), "%s", s);
  }
}

// ---- scalars: src/utils.jl:14-38 ----

const double kSqrtEps = std::sqrt(std::numeric_limits<double>::epsilon());

double occ_fermion(double e, double T) {
  if (T > kSqrtEps) return 1.0 / (std::exp(e / T) + 1.0);
  if (T >= 0) {
    double s = (e > 0) ? 1.0 : (e < 0 ? -1.0 : 0.0);
    return (1.0 - s) / 2.0;
  }
  throw OracleError(EPSP_EINVAL, "Temperature must be positive");
}

double occ_boson(double e, double T) {
  if (T > kSqrtEps) return e == 0 ? -0.5 : 1.0 / std::expm1(e / T);
  if (T >= 0) {
    if (e > 0) return 0.0;
    if (e == 0) return -0.5;
    return -1.0;
  }
  throw OracleError(EPSP_EINVAL, "Temperature must be positive");
}

// Julia's inv(::ComplexF64) for finite arguments in the normal range: Smith's algorithm
// (Base.inv(w::ComplexF64)), as used by `inv.(…)` in src/scgd0.jl:305 and src/ladder_kernel.jl:28.
cplx julia_inv(cplx w) {
  double c = w.real(), d = w.imag();
  if (std::fabs(d) <= std::fabs(c)) {
    double r = d / c;
    double t = 1.0 / (c + d * r);
    return cplx(t, -r * t);
  }
  std::swap(c, d);
  double r = d / c;
  double t = 1.0 / (c + d * r);
  return cplx(r * t, -t);
}

double bits_to_double(uint64_t u) {
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}
uint64_t double_to_bits(double x) {
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
}

// The midpoint of Roots.jl's Bisection over floating-point values (Roots._middle): 0 when the
// two (nonzero) ends have opposite signs, otherwise the mean of the bit patterns of |x| and |y|
// with the common sign.
double float_middle(double x, double y) {
  if (!std::isfinite(x) || !std::isfinite(y)) return x + y;
  if (x != 0 && y != 0 && (std::signbit(x) != std::signbit(y))) return 0.0;
  bool negate = (x < 0) || (y < 0);
  uint64_t ux = double_to_bits(std::fabs(x)), uy = double_to_bits(std::fabs(y));
  double m = bits_to_double((ux + uy) >> 1);
  return negate ? -m : m;
}

// Bracketed root by bisection to adjacent floats (Roots.find_zero(f, (a, b)), Bisection()).
template <class F>
double bisect_root(F&& f, double a, double b, double fa, double fb) {
  if (fa == 0) return a;
  if (fb == 0) return b;
  for (int it = 0; it < 2100; ++it) {
    double m = float_middle(a, b);
    if (m == a || m == b) break;
    double fm = f(m);
    if (fm == 0) return m;
    if (std::signbit(fm) == std::signbit(fa)) {
      a = m;
      fa = fm;
    } else {
      b = m;
      fb = fm;
    }
  }
  return std::fabs(fa) <= std::fabs(fb) ? a : b;
}

// ---- frequency grids: src/frequency_grids.jl ----

std::vector<double> grid_nodes(const epsp_grid& g) {  // :140-141
  std::vector<double> w(size_t(g.n));
  for (int64_t j = 0; j < g.n; ++j) w[j] = g.origin + double(g.offsets[j]) * g.unit;
  return w;
}

void check_grid(const epsp_grid& g, const char* name) {  // :124-132
  if (!(std::isfinite(g.origin) && std::isfinite(g.unit) && g.unit > 0))
    throw OracleError(EPSP_EINVAL, std::string(name) + ": origin must be finite and unit finite and positive");
  if (g.n < 2) throw OracleError(EPSP_EINVAL, std::string(name) + ": a FrequencyGrid needs at least two nodes");
  for (int64_t j = 0; j + 1 < g.n; ++j)
    if (g.offsets[j + 1] <= g.offsets[j])
      throw OracleError(EPSP_EINVAL, std::string(name) + ": offsets must be strictly increasing");
}

double grid_dw_min(const epsp_grid& g) {
  int64_t mg = std::numeric_limits<int64_t>::max();
  for (int64_t j = 0; j + 1 < g.n; ++j) mg = std::min(mg, g.offsets[j + 1] - g.offsets[j]);
  return g.unit * double(mg);
}

std::vector<double> trapezoid_weights(const double* ws, int64_t n) {  // :53-54
  std::vector<double> W(static_cast<size_t>(n));
  for (int64_t j = 0; j < n; ++j) W[j] = (ws[std::min(j + 1, n - 1)] - ws[std::max<int64_t>(j - 1, 0)]) / 2;
  return W;
}

double xlogx(double x) { return x == 0 ? 0.0 : x * std::log(std::fabs(x)); }  // :5

double lskk(double x, double x1, double x2, double x3) {  // :13-19
  return xlogx(x1 - x) / (x2 - x1) - xlogx(x2 - x) * (x3 - x1) / (x2 - x1) / (x3 - x2) +
         xlogx(x3 - x) / (x3 - x2);
}

void kk_matrix(const double* ws, int64_t N, double* K) {  // :30-44
  std::vector<double> xs(size_t(N + 2));
  xs[0] = ws[0] - (ws[1] - ws[0]);
  for (int64_t j = 0; j < N; ++j) xs[j + 1] = ws[j];
  xs[N + 1] = ws[N - 1] + (ws[N - 1] - ws[N - 2]);
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < N; ++j)
    for (int64_t i = 0; i < N; ++i) K[i + N * j] = lskk(xs[i + 1], xs[j], xs[j + 1], xs[j + 2]) / kPi;
}

// linear_interpolation_table, :65-84 (0-based j).
void interp_table(const double* ws, int64_t n, const double* xs, int64_t nx, int32_t* j, double* t) {
  for (int64_t r = 0; r < nx; ++r) {
    double x = xs[r];
    if (x <= ws[0]) {
      j[r] = 0;
      t[r] = 0;
    } else if (x >= ws[n - 1]) {
      j[r] = int32_t(n - 2);
      t[r] = 1;
    } else {
      int64_t jr = int64_t(std::upper_bound(ws, ws + n, x) - ws) - 1;  // searchsortedlast
      j[r] = int32_t(jr);
      t[r] = (x - ws[jr]) / (ws[jr + 1] - ws[jr]);
    }
  }
}

// cell_search_table, :184-196.
struct CellTable {
  std::vector<int32_t> jtab;
  double x0 = 0, inv_h = 0;
};

CellTable cell_search_table(const epsp_grid& g, const std::vector<double>& ws) {
  CellTable ct;
  ct.x0 = ws[0];
  ct.inv_h = 1.0 / ((1.0 - 1e-6) * grid_dw_min(g));
  double span_b = std::min((ws.back() - ct.x0) * ct.inv_h, std::ldexp(1.0, 40));
  int64_t nbuckets = int64_t(span_b) + 1;
  if (nbuckets > (int64_t(1) << 24))
    throw OracleError(EPSP_EINVAL, "cell search table of more than 2^24 entries: use a grid without a near-coincident pair of nodes");
  std::vector<int64_t> buckets(ws.size());
  for (size_t j = 0; j < ws.size(); ++j) buckets[j] = int64_t((ws[j] - ct.x0) * ct.inv_h);
  for (size_t j = 0; j + 1 < ws.size(); ++j)
    if (buckets[j + 1] == buckets[j]) throw OracleError(EPSP_EINVAL, "two grid nodes fall in one bucket");
  ct.jtab.resize(size_t(buckets.back() + 1));
  size_t c = 0;
  for (int64_t b = 0; b <= buckets.back(); ++b) {
    while (c < buckets.size() && buckets[c] < b) ++c;
    ct.jtab[size_t(b)] = int32_t(c);
  }
  return ct;
}

// _interp_linear_grid, :207-219, on a complex column ys (interleaved), returns the value at x.
inline cplx interp_grid(const double* ys_col, const double* ws, int64_t n, const CellTable& ct, double x) {
  auto y = [&](int64_t k) { return cplx(ys_col[2 * k], ys_col[2 * k + 1]); };
  if (!(x > ws[0])) return y(0);
  if (x >= ws[n - 1]) return y(n - 1);
  int64_t c = ct.jtab[size_t(int64_t((x - ct.x0) * ct.inv_h))];
  int64_t j1 = c + (ws[c] <= x ? 1 : 0);  // 1-based index of the lower node
  int64_t j = j1 - 1;
  double t = (x - ws[j]) / (ws[j + 1] - ws[j]);
  cplx lo = y(j), hi = y(j + 1);
  return cplx((1 - t) * lo.real() + t * hi.real(), (1 - t) * lo.imag() + t * hi.imag());
}

// ---- model access ----

struct Model {
  const epsp_model* m;
  int64_t nm, ni, nf, nw, nwa;
  std::vector<double> ws, wsa;  // nodes of ωs and ωs_spectral
  double g2(int64_t nu, int64_t i, int64_t f) const {
    size_t k = size_t(nu + nm * (i + ni * f));
    switch (m->g2_dtype) {
      case EPSP_F64: return static_cast<const double*>(m->g2)[k];
      case EPSP_F32: return double(static_cast<const float*>(m->g2)[k]);
      default: {
        uint16_t h = static_cast<const uint16_t*>(m->g2)[k];
        uint32_t u = uint32_t(h) << 16;
        float x;
        std::memcpy(&x, &u, 4);
        return double(x);
      }
    }
  }
  // ωq[ν, f, i] = ωph[ν, iq_kk[iks_i[i], iks_f[f]]]: gather_pair_table! as called at
  // src/scgd0.jl:270 and src/ladder.jl:259 (pinned by test/test_scgd0_pb.jl:81).
  double omega_q(int64_t nu, int64_t f, int64_t i) const {
    int64_t ki = m->iks_i[i], kf = m->iks_f[f];
    int64_t q = m->iq_kk[ki + m->nk_i * kf];
    return m->omega_ph[nu + nm * q];
  }
};

Model make_model(const epsp_model* m) {
  Model M;
  M.m = m;
  M.nm = m->nm;
  M.ni = m->ni;
  M.nf = m->nf;
  if (M.nm < 1 || M.ni < 1 || M.nf < 1) throw OracleError(EPSP_EINVAL, "nm, ni and nf must be positive");
  check_grid(m->omegas, "omegas");
  check_grid(m->omegas_spectral, "omegas_spectral");
  M.ws = grid_nodes(m->omegas);
  M.wsa = grid_nodes(m->omegas_spectral);
  M.nw = m->omegas.n;
  M.nwa = m->omegas_spectral.n;
  return M;
}

// ---- Fan-Migdal sum: src/scgd0_kernel.jl ----

// _fan_migdal_imsigma_term, :27-39.
inline double fm_term(double w, double g2, double wq, double eps_f, const double* sin_col,
                      const Model& M, const CellTable& ct, double mu, double T, double w_f,
                      double w_ac) {
  if (wq < w_ac) return 0.0;
  double n_q = occ_boson(wq, T);
  cplx s_abs = interp_grid(sin_col, M.ws.data(), M.nw, ct, w + wq);
  cplx s_emi = interp_grid(sin_col, M.ws.data(), M.nw, ct, w - wq);
  double za_re = w + wq - eps_f - s_abs.real(), za_im = -s_abs.imag();
  double ze_re = w - wq - eps_f - s_emi.real(), ze_im = -s_emi.imag();
  double img_abs = -za_im / (za_re * za_re + za_im * za_im);
  double img_emi = -ze_im / (ze_re * ze_re + ze_im * ze_im);
  return w_f * g2 *
         (img_abs * (n_q + occ_fermion(w + wq - mu, T)) + img_emi * (n_q + 1 - occ_fermion(w - wq - mu, T)));
}

int64_t scgd0_nf_chunk(const Model& M, int64_t gpu_tile) {  // src/scgd0.jl:201-202
  if (gpu_tile <= 0) return std::clamp<int64_t>(kChunkBytes / (8 * M.nm * M.ni), 1, M.nf);
  return std::min(gpu_tile, M.nf);
}

// add_fan_migdal_imsigma! over all chunks of inner states (src/scgd0.jl:264-287): per chunk, the
// sum over νf = (ν, f) in order for each (ω, i), added to imsigma [nω, ni].
void fan_migdal(const Model& M, const CellTable& ct, int64_t nf_chunk, const double* sin,
                double mu, double T, double w_ac, double* imsigma, int64_t ia = 0, int64_t ib = -1) {
  if (ib < 0) ib = M.ni;
  for (int64_t f0 = 0; f0 < M.nf; f0 += nf_chunk) {
    int64_t f1 = std::min(M.nf, f0 + nf_chunk);
    // every (i, ω) element is summed on its own in ascending νf, so the split over threads does not
    // change the result
#pragma omp parallel for collapse(2) schedule(dynamic, 8)
    for (int64_t i = ia; i < ib; ++i) {
      for (int64_t iw = 0; iw < M.nw; ++iw) {
        double w = M.ws[iw];
        double acc = 0.0;
        for (int64_t f = f0; f < f1; ++f) {
          const double* col = sin + 2 * M.nw * M.m->f_to_i[f];
          double eps_f = M.m->eps_f[f], w_f = M.m->w_f[f];
          for (int64_t nu = 0; nu < M.nm; ++nu)
            acc += fm_term(w, M.g2(nu, i, f), M.omega_q(nu, f, i), eps_f, col, M, ct, mu, T, w_f, w_ac);
        }
        imsigma[iw + M.nw * i] += acc;
      }
    }
  }
}

// compute_ncarrier_spectral, src/scgd0.jl:361-366, with ElectronPhonon's compute_ncarrier
// (Σ D f(ωa - μ)) and compute_ncarrier_hole (Σ D (1 - f) written as f(μ - ωa)), pinned by
// test/test_scgd0_mu.jl:7-51.
double ncarrier_spectral(double mu, double T, const double* wa, const double* D, int64_t n, double W,
                         bool count_holes, double nstates_base, double spin_deg) {
  double s = 0.0;
  if (count_holes) {
    for (int64_t a = 0; a < n; ++a) s += D[a] * occ_fermion(mu - wa[a], T);
    return (W - s + nstates_base) * spin_deg;
  }
  for (int64_t a = 0; a < n; ++a) s += D[a] * occ_fermion(wa[a] - mu, T);
  return (s + nstates_base) * spin_deg;
}

// ---- scGD0 loop: src/scgd0.jl:189-346 ----

void scgd0_run(const epsp_model* mp, const epsp_options* opts, const epsp_occ* occ, const double* eta_min,
               double eta_init, int32_t maxiter, double tol, int32_t fix_mu, const double* mu_start,
               const double* sigma_init, double* sigma_out, double* mu_out, uint8_t* converged,
               epsp_scgd0_history* hist) {
  Model M = make_model(mp);
  const int64_t nT = occ->nT, nw = M.nw, ni = M.ni, nwa = M.nwa;
  if (maxiter < 1) throw OracleError(EPSP_EINVAL, "maxiter must be at least 1");
  if (nT < 1) throw OracleError(EPSP_EINVAL, "at least one temperature");
  const double w_ac = opts->omega_acoustic;
  CellTable ct = cell_search_table(mp->omegas, M.ws);
  std::vector<int32_t> jsp(static_cast<size_t>(nwa));
  std::vector<double> tsp(static_cast<size_t>(nwa));
  interp_table(M.ws.data(), nw, M.wsa.data(), nwa, jsp.data(), tsp.data());  // src/scgd0.jl:163
  std::vector<double> Wa = trapezoid_weights(M.wsa.data(), nwa);
  std::vector<double> KK(size_t(nw * nw));
  kk_matrix(M.ws.data(), nw, KK.data());
  const double br0 = M.wsa.front() - 0.1, br1 = M.wsa.back() + 0.1;  // src/scgd0.jl:197
  const int64_t nf_chunk = scgd0_nf_chunk(M, opts->gpu_tile);

  const size_t slab = size_t(2 * nw * ni);
  std::vector<double> S(slab * nT), Snew(slab * nT), Sin(slab), ImS(size_t(nw * ni)), ReS(size_t(nw * ni));
  if (sigma_init) {
    std::copy(sigma_init, sigma_init + slab * nT, S.begin());
  } else {
    for (size_t k = 0; k < slab * nT; k += 2) {
      S[k] = 0.0;
      S[k + 1] = -eta_init;
    }
  }
  Snew = S;
  std::vector<double> mu(mu_start, mu_start + nT);
  std::vector<char> active(size_t(nT), 1);
  const double nan = std::numeric_limits<double>::quiet_NaN();
  for (int64_t k = 0; k < nT * maxiter; ++k) hist->err[k] = hist->mu[k] = hist->min_spectral_weight[k] = nan;
  for (int32_t k = 0; k < maxiter; ++k) hist->wall[k] = 0;
  for (int64_t k = 0; k < nT; ++k) hist->iter_frozen[k] = 0;
  int32_t niter = 0;
  std::vector<double> A(size_t(nwa * ni)), D(static_cast<size_t>(nwa)), Ssp(size_t(2 * nwa * ni));

  for (int32_t iter = 1; iter <= maxiter; ++iter) {
    auto t0 = std::chrono::steady_clock::now();
    for (int64_t iT = 0; iT < nT; ++iT) {
      if (!active[iT]) continue;
      double* ST = S.data() + slab * iT;
      double* SnT = Snew.data() + slab * iT;
      // 1. clamp, src/scgd0.jl:256-260.
      for (size_t k = 0; k < slab; k += 2) {
        Sin[k] = ST[k];
        Sin[k + 1] = std::min(ST[k + 1], -eta_min[iT]);
      }
      // 2-3. Fan-Migdal, src/scgd0.jl:261-287.
      std::fill(ImS.begin(), ImS.end(), 0.0);
      fan_migdal(M, ct, nf_chunk, Sin.data(), mu[iT], occ->Tlist[iT], w_ac, ImS.data());
      // 4. Re Σ = KK · Im Σ, src/scgd0.jl:288-292.
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < ni; ++i) {
        for (int64_t r = 0; r < nw; ++r) ReS[r + nw * i] = 0.0;
        for (int64_t k = 0; k < nw; ++k) {
          double z = ImS[k + nw * i];
          const double* Kc = KK.data() + nw * k;
          for (int64_t r = 0; r < nw; ++r) ReS[r + nw * i] += Kc[r] * z;
        }
        for (int64_t r = 0; r < nw; ++r) {
          SnT[2 * (r + nw * i)] = ReS[r + nw * i];
          SnT[2 * (r + nw * i) + 1] = ImS[r + nw * i];
        }
      }
    }
    // 5. multiplet average, src/scgd0.jl:293-301.
    for (int64_t iT = 0; iT < nT; ++iT) {
      if (!active[iT]) continue;
      double* SnT = Snew.data() + slab * iT;
      for (int64_t g = 0; g < mp->nmult; ++g) {
        int32_t p0 = mp->mult_ptr[g], p1 = mp->mult_ptr[g + 1];
        double len = double(p1 - p0);
        for (int64_t r = 0; r < nw; ++r) {
          double sr = 0, si = 0;
          for (int32_t p = p0; p < p1; ++p) {
            int64_t i = mp->mult_idx[p];
            sr += SnT[2 * (r + nw * i)];
            si += SnT[2 * (r + nw * i) + 1];
          }
          for (int32_t p = p0; p < p1; ++p) {
            int64_t i = mp->mult_idx[p];
            SnT[2 * (r + nw * i)] = sr / len;
            SnT[2 * (r + nw * i) + 1] = si / len;
          }
        }
      }
    }
    for (int64_t iT = 0; iT < nT; ++iT) {
      if (!active[iT]) continue;
      double* ST = S.data() + slab * iT;
      double* SnT = Snew.data() + slab * iT;
      const double T = occ->Tlist[iT];
      // 6. spectral DOS, src/scgd0.jl:303-308.
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < ni; ++i) {
        for (int64_t a = 0; a < nwa; ++a) {
          int64_t j = jsp[a];
          double t = tsp[a];
          const double* lo = SnT + 2 * (j + nw * i);
          double sr = (1 - t) * lo[0] + t * lo[2];
          double si = (1 - t) * lo[1] + t * lo[3];
          cplx z = cplx(M.wsa[a] - mp->eps_i[i] - sr, -si);
          A[a + nwa * i] = -julia_inv(z).imag() / kPi;
        }
      }
      for (int64_t a = 0; a < nwa; ++a) {
        double s = 0;
        for (int64_t i = 0; i < ni; ++i) s += A[a + nwa * i] * mp->w_i[i];
        D[a] = s * Wa[a];
      }
      double minA = std::numeric_limits<double>::infinity();
      for (int64_t i = 0; i < ni; ++i) {
        double s = 0;
        for (int64_t a = 0; a < nwa; ++a) s += A[a + nwa * i] * Wa[a];
        minA = std::min(minA, s);
      }
      hist->min_spectral_weight[iT + nT * (iter - 1)] = minA;
      // 7. chemical potential, src/scgd0.jl:309-324.
      if (!fix_mu) {
        bool holes = occ->type == EPSP_SEMICONDUCTOR && occ->nlist[iT] < 0;
        double n_target = occ->nlist[iT] + occ->nelec;
        auto excess = [&](double m_) {
          return ncarrier_spectral(m_, T, M.wsa.data(), D.data(), nwa, mp->W, holes, mp->nstates_base,
                                   occ->spin_degeneracy) -
                 n_target;
        };
        double f0 = excess(br0), f1 = excess(br1);
        if (f0 * f1 > 0) {
          char buf[256];
          std::snprintf(buf, sizeof buf,
                        "no chemical potential in (%g, %g) gives %g electrons per cell at T = %g", br0, br1,
                        n_target, T);
          throw OracleError(EPSP_ENOROOT_MU, buf);
        }
        mu[iT] = bisect_root(excess, br0, br1, f0, f1);
      }
      // 8-9. convergence, src/scgd0.jl:325-333.
      double err = 0;
      for (size_t k = 0; k < slab; k += 2) err = std::max(err, std::hypot(SnT[k] - ST[k], SnT[k + 1] - ST[k + 1]));
      hist->err[iT + nT * (iter - 1)] = err;
      hist->mu[iT + nT * (iter - 1)] = mu[iT];
      std::copy(SnT, SnT + slab, ST);
      if (err < tol) {
        active[iT] = 0;
        hist->iter_frozen[iT] = iter;
      }
    }
    hist->wall[iter - 1] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    niter = iter;
    if (std::none_of(active.begin(), active.end(), [](char a) { return a != 0; })) break;
  }
  hist->niter = niter;
  std::copy(S.begin(), S.end(), sigma_out);
  for (int64_t iT = 0; iT < nT; ++iT) {
    mu_out[iT] = mu[iT];
    converged[iT] = active[iT] ? 0 : 1;
  }
}

// ---- ladder: src/ladder_kernel.jl and src/ladder.jl ----

// _contour_green, src/ladder_kernel.jl:27-40 (c12 0-based: 11, 21, 12, 22).
cplx contour_green(double w, double eps, cplx S, double mu, double T, int c12) {
  cplx GR = julia_inv(cplx(w - eps - S.real(), -S.imag()));
  cplx GA = std::conj(GR);
  cplx GK = (GR - GA) * (1 - 2 * occ_fermion(w - mu, T));
  switch (c12) {
    case 0: return (GR + GA + GK) / 2.0;
    case 1: return (GR - GA + GK) / 2.0;
    case 2: return (-GR + GA + GK) / 2.0;
    default: return (-GR - GA + GK) / 2.0;
  }
}

struct Ladder {
  Model M;
  int64_t nshift = 0;
  double h = 0;
  std::vector<int32_t> by_star, star_ptr;  // src/ladder.jl:144-149 (0-based)
  std::vector<int32_t> klo;                // [nω, nshift, 2]
  std::vector<double> wlo, whi, Ww, KK;
  struct Chunk {
    int64_t i0, i1;               // outer states [i0, i1)
    std::vector<int32_t> fidx;    // inner states of the chunk
    std::vector<int32_t> sptr;    // local star pointers [nip + 1]
  };
  std::vector<Chunk> chunks;
};

int64_t nshift_of(const epsp_model* m) {  // src/ladder.jl:151
  double mx = -std::numeric_limits<double>::infinity();
  for (int64_t k = 0; k < m->nm * m->nq; ++k) mx = std::max(mx, m->omega_ph[k]);
  return int64_t(std::ceil(mx / m->omegas.unit)) + 2;
}

// vertex_shift_tables, src/ladder_kernel.jl:158-176.
void shift_tables(const epsp_grid& g, int64_t nshift, int32_t* klo, double* wlo, double* whi) {
  const int64_t nw = g.n;
  const int64_t* off = g.offsets;
  for (int s = 0; s < 2; ++s) {
    int64_t sign = s == 0 ? 1 : -1;
    for (int64_t m = 0; m < nshift; ++m) {
      for (int64_t j = 0; j < nw; ++j) {
        int64_t p = off[j] + sign * m;
        int64_t ssl = int64_t(std::upper_bound(off, off + nw, p) - off);  // searchsortedlast (1-based)
        int64_t k = std::clamp<int64_t>(ssl, 1, nw - 1) - 1;
        double t = double(p - off[k]) / double(off[k + 1] - off[k]);
        bool inside = off[0] <= p && p <= off[nw - 1];
        size_t idx = size_t(j + nw * (m + nshift * s));
        klo[idx] = int32_t(k);
        wlo[idx] = inside ? 1 - t : 0.0;
        whi[idx] = inside ? t : 0.0;
      }
    }
  }
}

Ladder make_ladder(const epsp_model* mp, int64_t gpu_tile) {
  Ladder L;
  L.M = make_model(mp);
  const Model& M = L.M;
  if (!mp->R || !mp->v) throw OracleError(EPSP_EINVAL, "the ladder needs R and v");
  L.h = mp->omegas.unit;
  L.nshift = nshift_of(mp);
  // stars: sortperm(f_to_i) (stable) and the cumulative star sizes, src/ladder.jl:144-149.
  L.by_star.resize(size_t(M.nf));
  for (int64_t f = 0; f < M.nf; ++f) L.by_star[f] = int32_t(f);
  std::stable_sort(L.by_star.begin(), L.by_star.end(),
                   [&](int32_t a, int32_t b) { return mp->f_to_i[a] < mp->f_to_i[b]; });
  L.star_ptr.assign(size_t(M.ni + 1), 0);
  for (int64_t f = 0; f < M.nf; ++f) L.star_ptr[mp->f_to_i[f] + 1] += 1;
  for (int64_t i = 0; i < M.ni; ++i) L.star_ptr[i + 1] += L.star_ptr[i];
  const int64_t nw = M.nw;
  L.klo.resize(size_t(nw * L.nshift * 2));
  L.wlo.resize(L.klo.size());
  L.whi.resize(L.klo.size());
  shift_tables(mp->omegas, L.nshift, L.klo.data(), L.wlo.data(), L.whi.data());
  L.Ww = trapezoid_weights(M.ws.data(), nw);
  L.KK.resize(size_t(nw * nw));
  kk_matrix(M.ws.data(), nw, L.KK.data());
  // chunks by whole stars, src/ladder.jl:180-202.
  int64_t bytes_per_f = 8 * std::max(L.nshift * M.ni * 2, M.nm * M.ni);
  int64_t bytes_per_i = 8 * std::max(L.nshift * 9 * M.ni * 2, nw * 16 * L.nshift * 3);
  int64_t max_f = gpu_tile <= 0 ? std::max<int64_t>(kChunkBytes / bytes_per_f, 1) : gpu_tile;
  int64_t max_i = std::max<int64_t>(kChunkBytes / bytes_per_i, 1);
  const auto& sp = L.star_ptr;
  int64_t i1 = 0;
  while (i1 < M.ni) {
    int64_t i2 = i1;
    while (i2 < M.ni - 1 && i2 - i1 + 2 <= max_i && sp[i2 + 2] - sp[i1] <= max_f) ++i2;
    Ladder::Chunk c;
    c.i0 = i1;
    c.i1 = i2 + 1;
    c.fidx.assign(L.by_star.begin() + sp[i1], L.by_star.begin() + sp[i2 + 1]);
    for (int64_t i = i1; i <= i2 + 1; ++i) c.sptr.push_back(sp[i] - sp[i1]);
    L.chunks.push_back(std::move(c));
    i1 = i2 + 1;
  }
  return L;
}

// J[ω, c12, cart, c0, i] complex, interleaved.
inline size_t jidx(int64_t nw, int64_t w, int64_t c12, int64_t cart, int64_t c0, int64_t i) {
  return size_t(w + nw * (c12 + 4 * (cart + 3 * (c0 + 2 * i))));
}

// contour_greens! of the shifted self-energies, src/ladder.jl:321-334 and
// src/ladder_kernel.jl:51-57. Gm, Gp: [nω, 4, ni].
void propagators(const Ladder& L, const double* sigma_T, double mu, double T, double Omega,
                 std::vector<cplx>& Gm, std::vector<cplx>& Gp) {
  const Model& M = L.M;
  const int64_t nw = M.nw, ni = M.ni;
  std::vector<double> xm(static_cast<size_t>(nw)), xp(static_cast<size_t>(nw)), tm(static_cast<size_t>(nw)), tp(static_cast<size_t>(nw));
  std::vector<int32_t> jm(static_cast<size_t>(nw)), jp(static_cast<size_t>(nw));
  for (int64_t k = 0; k < nw; ++k) {
    xm[k] = M.ws[k] - Omega / 2;
    xp[k] = M.ws[k] + Omega / 2;
  }
  interp_table(M.ws.data(), nw, xm.data(), nw, jm.data(), tm.data());
  interp_table(M.ws.data(), nw, xp.data(), nw, jp.data(), tp.data());
  Gm.assign(size_t(nw * 4 * ni), cplx());
  Gp.assign(size_t(nw * 4 * ni), cplx());
  for (int64_t i = 0; i < ni; ++i) {
    const double* col = sigma_T + 2 * nw * i;
    for (int64_t w = 0; w < nw; ++w) {
      auto lerp = [&](int32_t j, double t) {
        return cplx((1 - t) * col[2 * j] + t * col[2 * j + 2], (1 - t) * col[2 * j + 1] + t * col[2 * j + 3]);
      };
      cplx sm = lerp(jm[w], tm[w]), spp = lerp(jp[w], tp[w]);
      for (int c = 0; c < 4; ++c) {
        Gm[size_t(w + nw * (c + 4 * i))] = contour_green(xm[w], M.m->eps_i[i], sm, mu, T, c);
        Gp[size_t(w + nw * (c + 4 * i))] = contour_green(xp[w], M.m->eps_i[i], spp, mu, T, c);
      }
    }
  }
}

// attach_greens_to_bare_vertex!, src/ladder_kernel.jl:70-73, 97-99: J0 = Gm V Gp with
// V^{c1 c2, c0} = δ_{c1 c2} δ_{c1 c0} v_i. Gm, Gp [nω, 4, ni]; v [3, ni].
void attach_bare_core(int64_t nw, int64_t ni, const cplx* Gm, const cplx* Gp, const double* v, double* J0) {
  for (int64_t i = 0; i < ni; ++i)
    for (int c0 = 0; c0 < 2; ++c0)
      for (int cart = 0; cart < 3; ++cart)
        for (int c12 = 0; c12 < 4; ++c12) {
          int c1 = c12 % 2, c2 = c12 / 2;
          for (int64_t w = 0; w < nw; ++w) {
            cplx z = Gm[size_t(w + nw * (c1 + 2 * c0 + 4 * i))] * v[cart + 3 * i] *
                     Gp[size_t(w + nw * (c0 + 2 * c2 + 4 * i))];
            size_t k = jidx(nw, w, c12, cart, c0, i);
            J0[2 * k] = z.real();
            J0[2 * k + 1] = z.imag();
          }
        }
}

void attach_bare(const Ladder& L, const std::vector<cplx>& Gm, const std::vector<cplx>& Gp, double* J0) {
  attach_bare_core(L.M.nw, L.M.ni, Gm.data(), Gp.data(), L.M.m->v, J0);
}

// attach_greens_to_vertex!, src/ladder_kernel.jl:61-67, 87-89: J = Gm X Gp per (ω, cart, c0, i),
// for the outer states [ia, ia + ni) of Gm, Gp [nω, 4, *]; X and J hold those ni states only.
void attach_core(int64_t nw, int64_t ni, const cplx* Gm, const cplx* Gp, const cplx* X, double* J, double scale,
                 int64_t ia) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < ni; ++i)
    for (int c0 = 0; c0 < 2; ++c0)
      for (int cart = 0; cart < 3; ++cart)
        for (int c12 = 0; c12 < 4; ++c12) {
          int c1 = c12 % 2, c2 = c12 / 2;
          for (int64_t w = 0; w < nw; ++w) {
            auto gm = [&](int c) { return Gm[size_t(w + nw * (c + 4 * (ia + i)))]; };
            auto gp = [&](int c) { return Gp[size_t(w + nw * (c + 4 * (ia + i)))]; };
            auto x = [&](int c) { return X[jidx(nw, w, c, cart, c0, i)]; };
            cplx z = gm(c1) * x(0) * gp(0 + 2 * c2) + gm(c1 + 2) * x(1) * gp(0 + 2 * c2) +
                     gm(c1) * x(2) * gp(1 + 2 * c2) + gm(c1 + 2) * x(3) * gp(1 + 2 * c2);
            size_t k = jidx(nw, w, c12, cart, c0, i);
            J[2 * k] = scale * z.real();
            J[2 * k + 1] = scale * z.imag();
          }
        }
}

// all outer states by default, or [ia, ia + n)
void attach(const Ladder& L, const std::vector<cplx>& Gm, const std::vector<cplx>& Gp,
            const std::vector<cplx>& X, double* J, double scale, int64_t ia = 0, int64_t n = -1) {
  attach_core(L.M.nw, n < 0 ? L.M.ni : n, Gm.data(), Gp.data(), X.data(), J, scale, ia);
}

// conductivity_from_vertex, src/ladder_kernel.jl:116-122.
void conductivity(const double* J, const double* v, const double* w_i, const double* Ww, int64_t nw,
                  int64_t ni, double Omega, double T, double* sigma) {
  cplx F = Omega == 0 ? cplx(0, 1) / (4 * T)
                      : -1.0 / (cplx(0, 2) * Omega * (1 + 2 * occ_boson(Omega, T)));
  std::vector<cplx> Y(size_t(3 * ni));
  for (int64_t i = 0; i < ni; ++i)
    for (int b = 0; b < 3; ++b) {
      cplx s = 0;
      for (int64_t w = 0; w < nw; ++w) {
        size_t k22 = jidx(nw, w, 3, b, 0, i), k11 = jidx(nw, w, 0, b, 1, i);
        s += Ww[w] * (cplx(J[2 * k22], J[2 * k22 + 1]) + cplx(J[2 * k11], J[2 * k11 + 1]));
      }
      Y[size_t(b + 3 * i)] = s;
    }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      cplx S = 0;
      for (int64_t i = 0; i < ni; ++i) S += (v[a + 3 * i] * w_i[i]) * Y[size_t(b + 3 * i)];
      sigma[a + 3 * b] = (F / (2 * kPi * cplx(0, 1)) * S).real();
    }
}

// B (bin_coupling_on_shift_grid!, src/ladder_kernel.jl:195-236) and B̃ (star_sum_coupling!,
// :240-264) of one chunk for the output columns col = (a, ii, type) of the outer states
// [ia, ia + nsel): Bt [nk, 6 nsel], nk = nshift·3·nip, rows (m, b, ip).
void chunk_coupling(const Ladder& L, const Ladder::Chunk& ch, double T, double w_ac, int64_t ia, int64_t nsel,
                    double* Bt) {
  const Model& M = L.M;
  const epsp_model* mp = M.m;
  const int64_t nm = M.nm, ns = L.nshift;
  const int64_t nfc = int64_t(ch.fidx.size()), nip = ch.i1 - ch.i0, ncol = 6 * nsel;
  std::vector<double> B(size_t(ns * nfc * nsel * 2), 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t fc = 0; fc < nfc; ++fc) {
    int64_t f = ch.fidx[size_t(fc)];
    for (int type = 0; type < 2; ++type)
      for (int64_t ii = 0; ii < nsel; ++ii) {
        int64_t i = ia + ii;
        double* col = B.data() + ns * (fc + nfc * (ii + nsel * type));
        for (int64_t nu = 0; nu < nm; ++nu) {
          double w = M.omega_q(nu, f, i);
          if (w < w_ac) continue;
          double x = w / L.h;
          int64_t lo = int64_t(std::floor(x));
          double g = M.g2(nu, i, f);
          for (int64_t m = lo; m <= lo + 1; ++m) {
            double c = g * std::max(0.0, 1 - std::fabs(x - double(m)));
            col[m] += type == 0 ? c : c * occ_boson(w, T);
          }
        }
        double wf = mp->w_f[f];
        for (int64_t m = 0; m < ns; ++m) col[m] *= wf;
      }
  }
  const int64_t nk = ns * 3 * nip;
#pragma omp parallel for schedule(static)
  for (int64_t col = 0; col < ncol; ++col) {  // col = (a, ii, type)
    int64_t a = col % 3, ii = (col / 3) % nsel, type = col / (3 * nsel);
    for (int64_t ip = 0; ip < nip; ++ip)
      for (int b = 0; b < 3; ++b)
        for (int64_t m = 0; m < ns; ++m) {
          double acc = 0.0;
          for (int32_t fc = ch.sptr[size_t(ip)]; fc < ch.sptr[size_t(ip + 1)]; ++fc)
            acc += mp->R[a + 3 * (b + 3 * int64_t(ch.fidx[size_t(fc)]))] *
                   B[size_t(m + ns * (fc + nfc * (ii + nsel * type)))];
          Bt[size_t(m + ns * (b + 3 * ip) + nk * col)] = acc;
        }
  }
}

// X of one chunk and sign s (gather_shifted_vertex!, src/ladder_kernel.jl:268-288): X [16 nω, nk],
// rows (j, c12, c0, ri), columns (m, b, ip).
void chunk_shifted_vertex(const Ladder& L, const Ladder::Chunk& ch, int s, const double* J, double* X) {
  const int64_t nw = L.M.nw, ns = L.nshift, nrow = nw * 16;
  const int64_t nk = ns * 3 * (ch.i1 - ch.i0);
  const int32_t* klo = L.klo.data() + nw * ns * s;
  const double* wlo = L.wlo.data() + nw * ns * s;
  const double* whi = L.whi.data() + nw * ns * s;
#pragma omp parallel for schedule(static)
  for (int64_t kk = 0; kk < nk; ++kk) {  // kk = (m, b, ip)
    int64_t m = kk % ns, b = (kk / ns) % 3, ip = kk / (3 * ns);
    int64_t i = ch.i0 + ip;
    for (int c0 = 0; c0 < 2; ++c0)
      for (int c12 = 0; c12 < 4; ++c12)
        for (int64_t j = 0; j < nw; ++j) {
          int64_t k = klo[j + nw * m];
          size_t a0 = jidx(nw, k, c12, b, c0, i), a1 = jidx(nw, k + 1, c12, b, c0, i);
          double wl = wlo[j + nw * m], wh = whi[j + nw * m];
          double zr = wl * J[2 * a0] + wh * J[2 * a1];
          double zi = wl * J[2 * a0 + 1] + wh * J[2 * a1 + 1];
          X[size_t(j + nw * (c12 + 4 * (c0 + 2 * 0)) + nrow * kk)] = zr;  // row (j, c12, c0, ri)
          X[size_t(j + nw * (c12 + 4 * (c0 + 2 * 1)) + nrow * kk)] = zi;
        }
  }
}

// apply_ladder_kernel!, src/ladder.jl:245-296, for the output states [ia, ib) (all of them by
// default): LJ [nω, 4, 3, 2, ib - ia]. An output state's columns of C± and of the exchange part
// depend on that state's columns of B̃ only, and each is summed in the same order whatever the
// range, so a range's LJ is bitwise the full LJ's slice.
void ladder_apply(const Ladder& L, const std::vector<cplx>& Gm, const std::vector<cplx>& Gp, double T,
                  double w_ac, const double* J, double* LJ, int64_t ia = 0, int64_t ib = -1) {
  const Model& M = L.M;
  if (ib < 0) ib = M.ni;
  const int64_t nw = M.nw, ni = ib - ia, ns = L.nshift;
  const int64_t nrow = nw * 16, ncol = 6 * ni;
  std::vector<double> Cp(size_t(nrow * ncol), 0.0), Cm(size_t(nrow * ncol), 0.0);
  for (const auto& ch : L.chunks) {
    const int64_t nk = ns * 3 * (ch.i1 - ch.i0);
    std::vector<double> Bt(size_t(nk * ncol));
    chunk_coupling(L, ch, T, w_ac, ia, ni, Bt.data());
    // C_s += X_s · B̃ (src/ladder.jl:283-290)
    std::vector<double> X(size_t(nrow * nk));
    for (int s = 0; s < 2; ++s) {
      chunk_shifted_vertex(L, ch, s, J, X.data());
      double* C = s == 0 ? Cp.data() : Cm.data();
#pragma omp parallel for schedule(static)
      for (int64_t col = 0; col < ncol; ++col) {
        double* Cc = C + nrow * col;
        const double* Bc = Bt.data() + nk * col;
        for (int64_t k = 0; k < nk; ++k) {
          double b = Bc[k];
          if (b == 0.0) continue;
          const double* Xk = X.data() + nrow * k;
          for (int64_t r = 0; r < nrow; ++r) Cc[r] += Xk[r] * b;
        }
      }
    }
  }
  // apply_phonon_exchange_kernel!, src/ladder_kernel.jl:296-322. C[ω, c12, c0, ri, a, i, type].
  auto cidx = [&](int64_t w, int64_t c12, int64_t c0, int64_t ri, int64_t a, int64_t i, int64_t type) {
    return size_t(w + nw * (c12 + 4 * (c0 + 2 * (ri + 2 * (a + 3 * (i + ni * type))))));
  };
  const int64_t ny = 48 * ni;  // columns of Y: (c12, c0, ri, a, i)
  std::vector<double> Y(size_t(nw * ny)), KY(size_t(nw * ny), 0.0);
  for (int64_t k = 0; k < nw * ny; ++k) Y[size_t(k)] = (Cp[size_t(k)] - Cm[size_t(k)]) / 2;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < ny; ++c)
    for (int64_t k = 0; k < nw; ++k) {
      double y = Y[size_t(k + nw * c)];
      const double* Kc = L.KK.data() + nw * k;
      for (int64_t r = 0; r < nw; ++r) KY[size_t(r + nw * c)] += Kc[r] * y;
    }
  std::vector<cplx> KJ(size_t(nw * 24 * ni));
  for (int64_t i = 0; i < ni; ++i)
    for (int c0 = 0; c0 < 2; ++c0)
      for (int a = 0; a < 3; ++a)
        for (int c12 = 0; c12 < 4; ++c12)
          for (int64_t w = 0; w < nw; ++w) {
            auto sumc = [&](const std::vector<double>& C, int type) {
              return cplx(C[cidx(w, c12, c0, 0, a, i, type)], C[cidx(w, c12, c0, 1, a, i, type)]);
            };
            cplx Up = sumc(Cp, 0), Um = sumc(Cm, 0), Vp = sumc(Cp, 1), Vm = sumc(Cm, 1);
            cplx r;
            if (c12 == 0 || c12 == 3) {
              cplx ky(KY[cidx(w, c12, c0, 0, a, i, 0)], KY[cidx(w, c12, c0, 1, a, i, 0)]);
              r = (c12 == 0 ? cplx(0, -1) : cplx(0, 1)) * ky - (Up + Um) / 2.0 - (Vp + Vm);
            } else if (c12 == 1) {
              r = Vp + Um + Vm;
            } else {
              r = Up + Vp + Vm;
            }
            KJ[jidx(nw, w, c12, a, c0, i)] = r;
          }
  attach(L, Gm, Gp, KJ, LJ, -1.0, ia, ni);  // src/ladder.jl:294-295
}

double vnorm(const std::vector<cplx>& x) {
  double s = 0;
  for (const auto& z : x) s += std::norm(z);
  return std::sqrt(s);
}

// Krylov.gmres (Krylov.jl 0.10, restart = false, MGS, Givens), as called at src/ladder.jl:340-353.
struct GmresStats {
  bool solved = false;
  int niter = 0;
  std::vector<double> residuals;
};

template <class Op>
GmresStats gmres(Op&& A, const std::vector<cplx>& b, std::vector<cplx>& x, bool warm, double atol,
                 int itmax) {
  const size_t n = b.size();
  GmresStats st;
  std::vector<cplx> r0(n), w(n), dx;
  if (warm) {
    dx = x;
    A(dx, w);
    for (size_t k = 0; k < n; ++k) r0[k] = b[k] - w[k];
  } else {
    r0 = b;
  }
  std::fill(x.begin(), x.end(), cplx());
  double beta = vnorm(r0);
  double rNorm = beta;
  st.residuals.push_back(beta);
  const double eps = atol;  // rtol = 0
  if (beta == 0) {
    st.solved = true;
    if (warm) x = dx;
    return st;
  }
  const double btol = std::pow(std::numeric_limits<double>::epsilon(), 0.75);
  bool solved = rNorm <= eps, breakdown = false;
  std::vector<std::vector<cplx>> V;
  std::vector<cplx> R, s, z;
  std::vector<double> c;
  int inner = 0;
  if (!solved && itmax > 0) {
    V.emplace_back(n);
    for (size_t k = 0; k < n; ++k) V[0][k] = r0[k] / rNorm;
    z.push_back(beta);
    int nr = 0;
    bool tired = false;
    std::vector<cplx> q(n);
    while (!(solved || tired || breakdown)) {
      ++inner;
      A(V[size_t(inner - 1)], q);
      for (int i = 0; i < inner; ++i) {
        cplx h = 0;
        const auto& vi = V[size_t(i)];
        for (size_t k = 0; k < n; ++k) h += std::conj(vi[k]) * q[k];
        for (size_t k = 0; k < n; ++k) q[k] -= h * vi[k];
        R.push_back(h);
      }
      double Hbis = vnorm(q);
      for (int i = 0; i < inner - 1; ++i) {
        cplx Rtmp = c[size_t(i)] * R[size_t(nr + i)] + s[size_t(i)] * R[size_t(nr + i + 1)];
        R[size_t(nr + i + 1)] = std::conj(s[size_t(i)]) * R[size_t(nr + i)] - c[size_t(i)] * R[size_t(nr + i + 1)];
        R[size_t(nr + i)] = Rtmp;
      }
      // sym_givens(a::Complex, b::Real)
      cplx a = R[size_t(nr + inner - 1)];
      double abs_a = std::abs(a), cc;
      cplx ss, rho;
      if (Hbis == 0) {
        cc = 1;
        ss = 0;
        rho = a;
      } else if (abs_a == 0) {
        cc = 0;
        ss = 1;
        rho = Hbis;
      } else {
        double rr = std::hypot(abs_a, Hbis);
        cplx psi = a / abs_a;
        cc = abs_a / rr;
        ss = psi * (Hbis / rr);
        rho = psi * rr;
      }
      c.push_back(cc);
      s.push_back(ss);
      R[size_t(nr + inner - 1)] = rho;
      cplx zeta = std::conj(ss) * z[size_t(inner - 1)];
      z[size_t(inner - 1)] = cc * z[size_t(inner - 1)];
      rNorm = std::abs(zeta);
      st.residuals.push_back(rNorm);
      nr += inner;
      bool mach = rNorm + 1.0 <= 1.0;
      solved = rNorm <= eps || mach;
      breakdown = Hbis <= btol;
      tired = inner >= itmax;
      if (!(solved || tired || breakdown)) {
        V.emplace_back(n);
        for (size_t k = 0; k < n; ++k) V.back()[k] = q[k] / Hbis;
        z.push_back(zeta);
      }
    }
    // back substitution R y = z and x = V y
    std::vector<cplx> y = z;
    for (int i = inner - 1; i >= 0; --i) {
      int pos = nr + i - inner;  // 0-based position of r_{i,k}
      for (int j = inner - 1; j >= i + 1; --j) {
        y[size_t(i)] -= R[size_t(pos)] * y[size_t(j)];
        pos = pos - (j + 1) + 1;
      }
      if (std::abs(R[size_t(pos)]) <= btol)
        y[size_t(i)] = 0;
      else
        y[size_t(i)] /= R[size_t(pos)];
    }
    for (int i = 0; i < inner; ++i)
      for (size_t k = 0; k < n; ++k) x[k] += y[size_t(i)] * V[size_t(i)][k];
  }
  if (warm)
    for (size_t k = 0; k < n; ++k) x[k] += dx[k];
  st.solved = solved;
  st.niter = inner;
  return st;
}

double mat3_norm(const double* a) {
  double s = 0;
  for (int k = 0; k < 9; ++k) s += a[k] * a[k];
  return std::sqrt(s);
}

void ladder_run(const epsp_model* mp, const epsp_options* opts, const double* sigma, const double* mu,
                const double* Tlist, int64_t nT, const double* Omegas, int64_t nO, int32_t solver,
                double rtol, int32_t maxiter, double* sb, double* sl, uint8_t* conv, int32_t* niter,
                epsp_ladder_history* hist, double* J_out) {
  if (solver != EPSP_SOLVER_GMRES && solver != EPSP_SOLVER_FIXED_POINT)
    throw OracleError(EPSP_EINVAL, "solver must be gmres or fixed_point");
  if (maxiter < 1) throw OracleError(EPSP_EINVAL, "maxiter must be at least 1");
  if (nO < 1) throw OracleError(EPSP_EINVAL, "Omegas must hold at least one probe frequency");
  if (!(opts->omega_acoustic > 0)) throw OracleError(EPSP_EINVAL, "omega_acoustic must be positive");
  Ladder L = make_ladder(mp, opts->gpu_tile);
  const int64_t nw = L.M.nw, ni = L.M.ni;
  const size_t nJ = size_t(nw * 24 * ni);
  std::vector<cplx> J0(nJ), J(nJ), LJ(nJ);
  std::vector<double> buf(2 * nJ), buf2(2 * nJ);
  auto to_c = [&](const std::vector<double>& d, std::vector<cplx>& c) {
    for (size_t k = 0; k < nJ; ++k) c[k] = cplx(d[2 * k], d[2 * k + 1]);
  };
  auto to_d = [&](const std::vector<cplx>& c, std::vector<double>& d) {
    for (size_t k = 0; k < nJ; ++k) {
      d[2 * k] = c[k].real();
      d[2 * k + 1] = c[k].imag();
    }
  };
  std::vector<cplx> Gm, Gp;
  for (int64_t iT = 0; iT < nT; ++iT) {
    const double T = Tlist[iT];
    const double* ST = sigma + 2 * nw * ni * iT;
    for (int64_t iO = 0; iO < nO; ++iO) {
      const double Om = Omegas[iO];
      const int64_t idx = iO + nO * iT;
      propagators(L, ST, mu[iT], T, Om, Gm, Gp);
      attach_bare(L, Gm, Gp, buf.data());
      to_c(buf, J0);
      conductivity(buf.data(), mp->v, mp->w_i, L.Ww.data(), nw, ni, Om, T, sb + 9 * idx);
      auto op = [&](const std::vector<cplx>& xin, std::vector<cplx>& yout) {  // y = (I - L) x
        to_d(xin, buf2);
        ladder_apply(L, Gm, Gp, T, opts->omega_acoustic, buf2.data(), buf.data());
        for (size_t k = 0; k < nJ; ++k) yout[k] = xin[k] - cplx(buf[2 * k], buf[2 * k + 1]);
      };
      if (solver == EPSP_SOLVER_GMRES) {
        GmresStats st = gmres(op, J0, J, iO > 0, rtol * vnorm(J0), maxiter);
        conv[idx] = st.solved ? 1 : 0;
        niter[idx] = st.niter;
        if (hist && hist->norms) {
          int32_t nn = int32_t(std::min<size_t>(st.residuals.size(), size_t(maxiter + 1)));
          for (int32_t k = 0; k < nn; ++k) hist->norms[size_t(maxiter + 1) * size_t(idx) + size_t(k)] = st.residuals[size_t(k)];
          hist->nnorms[idx] = nn;
        }
        if (hist && hist->nsigma) hist->nsigma[idx] = 0;
      } else {
        J = J0;
        std::vector<double> sprev(9), scur(9);
        conv[idx] = 0;
        int32_t ns = 0;
        for (int32_t it = 1; it <= maxiter; ++it) {
          to_d(J, buf2);
          ladder_apply(L, Gm, Gp, T, opts->omega_acoustic, buf2.data(), buf.data());
          for (size_t k = 0; k < nJ; ++k) J[k] = J0[k] + cplx(buf[2 * k], buf[2 * k + 1]);
          to_d(J, buf2);
          conductivity(buf2.data(), mp->v, mp->w_i, L.Ww.data(), nw, ni, Om, T, scur.data());
          if (hist && hist->sigma_iter)
            for (int k = 0; k < 9; ++k) hist->sigma_iter[9 * (size_t(maxiter) * size_t(idx) + size_t(it - 1)) + size_t(k)] = scur[size_t(k)];
          ns = it;
          niter[idx] = it;
          if (it > 1) {
            double d[9];
            for (int k = 0; k < 9; ++k) d[k] = scur[size_t(k)] - sprev[size_t(k)];
            if (mat3_norm(d) < rtol * mat3_norm(scur.data())) {
              conv[idx] = 1;
              break;
            }
          }
          sprev = scur;
        }
        if (hist && hist->nsigma) hist->nsigma[idx] = ns;
        if (hist && hist->nnorms) hist->nnorms[idx] = 0;
      }
      to_d(J, buf2);
      conductivity(buf2.data(), mp->v, mp->w_i, L.Ww.data(), nw, ni, Om, T, sl + 9 * idx);
      if (J_out) std::copy(buf2.begin(), buf2.end(), J_out + 2 * nJ * size_t(idx));
    }
  }
}

template <class F>
int guarded(char* msg, int32_t len, F&& f) {
  try {
    f();
    set_msg(msg, len, "");
    return EPSP_OK;
  } catch (const OracleError& e) {
    set_msg(msg, len, e.what());
    return e.code;
  } catch (const std::exception& e) {
    set_msg(msg, len, e.what());
    return EPSP_EINVAL;
  }
}

void apply_threads() {
#ifdef _OPENMP
  if (g_threads > 0) omp_set_num_threads(g_threads);
#endif
}

}  // namespace

extern "C" {

double epsp_oracle_occ_fermion(double e, double T) { return occ_fermion(e, T); }
double epsp_oracle_occ_boson(double e, double T) { return occ_boson(e, T); }

void epsp_oracle_grid_nodes(const epsp_grid* g, double* nodes) {
  auto w = grid_nodes(*g);
  std::copy(w.begin(), w.end(), nodes);
}

void epsp_oracle_trapezoid_weights(const double* ws, int64_t n, double* W) {
  auto w = trapezoid_weights(ws, n);
  std::copy(w.begin(), w.end(), W);
}

void epsp_oracle_kk_matrix(const double* ws, int64_t n, double* K) {
  apply_threads();
  kk_matrix(ws, n, K);
}

void epsp_oracle_interp_table(const double* ws, int64_t n, const double* xs, int64_t nx, int32_t* j, double* t) {
  interp_table(ws, n, xs, nx, j, t);
}

int epsp_oracle_interp_grid(const epsp_grid* g, const double* ys, int64_t col, const double* xs, int64_t nx,
                            double* out, char* msg, int32_t msglen) {
  return guarded(msg, msglen, [&] {
    check_grid(*g, "grid");
    auto ws = grid_nodes(*g);
    CellTable ct = cell_search_table(*g, ws);
    for (int64_t r = 0; r < nx; ++r) {
      cplx z = interp_grid(ys + 2 * g->n * col, ws.data(), g->n, ct, xs[r]);
      out[2 * r] = z.real();
      out[2 * r + 1] = z.imag();
    }
  });
}

double epsp_oracle_ncarrier_spectral(double mu, double T, const double* wa, const double* D, int64_t n, double W,
                                     int32_t count_holes, double nstates_base, double spin_degeneracy) {
  return ncarrier_spectral(mu, T, wa, D, n, W, count_holes != 0, nstates_base, spin_degeneracy);
}

int epsp_oracle_imsigma(const epsp_model* m, const epsp_options* opts, const double* sigma_in, double mu,
                        double T, double* imsigma, char* msg, int32_t msglen) {
  apply_threads();
  return guarded(msg, msglen, [&] {
    Model M = make_model(m);
    CellTable ct = cell_search_table(m->omegas, M.ws);
    fan_migdal(M, ct, scgd0_nf_chunk(M, opts->gpu_tile), sigma_in, mu, T, opts->omega_acoustic, imsigma);
  });
}

int epsp_oracle_scgd0_run(const epsp_model* m, const epsp_options* opts, const epsp_occ* occ, const double* eta_min,
                          double eta_init, int32_t maxiter, double tol, int32_t fix_mu, const double* mu_start,
                          const double* sigma_init, double* sigma_out, double* mu_out, uint8_t* converged,
                          epsp_scgd0_history* hist, char* msg, int32_t msglen) {
  apply_threads();
  return guarded(msg, msglen, [&] {
    scgd0_run(m, opts, occ, eta_min, eta_init, maxiter, tol, fix_mu, mu_start, sigma_init, sigma_out, mu_out,
              converged, hist);
  });
}

void epsp_oracle_contour_green(double w, double eps, double s_re, double s_im, double mu, double T, int32_t c12,
                               double* out) {
  cplx z = contour_green(w, eps, cplx(s_re, s_im), mu, T, c12);
  out[0] = z.real();
  out[1] = z.imag();
}

void epsp_oracle_shift_tables(const epsp_grid* g, int64_t nshift, int32_t* klo, double* wlo, double* whi) {
  shift_tables(*g, nshift, klo, wlo, whi);
}

int64_t epsp_oracle_nshift(const epsp_model* m) { return nshift_of(m); }

void epsp_oracle_bin_coupling(const epsp_model* mp, double w_ac, double T, double* B) {
  Model M = make_model(mp);
  std::vector<int32_t> by_star(size_t(M.nf));
  for (int64_t f = 0; f < M.nf; ++f) by_star[f] = int32_t(f);
  std::stable_sort(by_star.begin(), by_star.end(), [&](int32_t a, int32_t b) { return mp->f_to_i[a] < mp->f_to_i[b]; });
  const int64_t ns = nshift_of(mp), nf = M.nf, ni = M.ni;
  const double h = mp->omegas.unit;
  std::fill(B, B + ns * nf * ni * 2, 0.0);
  for (int64_t fc = 0; fc < nf; ++fc) {
    int64_t f = by_star[size_t(fc)];
    for (int type = 0; type < 2; ++type)
      for (int64_t i = 0; i < ni; ++i) {
        double* col = B + ns * (fc + nf * (i + ni * type));
        for (int64_t nu = 0; nu < M.nm; ++nu) {
          double w = M.omega_q(nu, f, i);
          if (w < w_ac) continue;
          double x = w / h;
          int64_t lo = int64_t(std::floor(x));
          double g = M.g2(nu, i, f);
          for (int64_t m = lo; m <= lo + 1; ++m) {
            double c = g * std::max(0.0, 1 - std::fabs(x - double(m)));
            col[m] += type == 0 ? c : c * occ_boson(w, T);
          }
        }
        for (int64_t m = 0; m < ns; ++m) col[m] *= mp->w_f[f];
      }
  }
}

void epsp_oracle_conductivity(const double* J, const double* v, const double* w_i, const double* Ww, int64_t nw,
                              int64_t ni, double Omega, double T, double* sigma) {
  conductivity(J, v, w_i, Ww, nw, ni, Omega, T, sigma);
}

// Gm, Gp [nω, 4, ni], X and J [nω, 4, 3, 2, ni]: complex, interleaved.
void epsp_oracle_attach_greens(int64_t nw, int64_t ni, const double* Gm, const double* Gp, const double* X,
                               double* J) {
  attach_core(nw, ni, reinterpret_cast<const cplx*>(Gm), reinterpret_cast<const cplx*>(Gp),
              reinterpret_cast<const cplx*>(X), J, 1.0, 0);
}

void epsp_oracle_attach_bare(int64_t nw, int64_t ni, const double* Gm, const double* Gp, const double* v,
                             double* J0) {
  attach_bare_core(nw, ni, reinterpret_cast<const cplx*>(Gm), reinterpret_cast<const cplx*>(Gp), v, J0);
}

int epsp_oracle_ladder_apply(const epsp_model* m, const epsp_options* opts, const double* sigma_T, double mu,
                             double T, double Omega, const double* J, double* LJ, char* msg, int32_t msglen) {
  apply_threads();
  return guarded(msg, msglen, [&] {
    Ladder L = make_ladder(m, opts->gpu_tile);
    std::vector<cplx> Gm, Gp;
    propagators(L, sigma_T, mu, T, Omega, Gm, Gp);
    ladder_apply(L, Gm, Gp, T, opts->omega_acoustic, J, LJ);
  });
}

int epsp_oracle_ladder_run(const epsp_model* m, const epsp_options* opts, const double* sigma, const double* mu,
                           const double* Tlist, int64_t nT, const double* Omegas, int64_t nOmega, int32_t solver,
                           double rtol, int32_t maxiter, double* sigma_bubble, double* sigma_ladder,
                           uint8_t* converged, int32_t* niter, epsp_ladder_history* hist, double* J_out, char* msg,
                           int32_t msglen) {
  apply_threads();
  return guarded(msg, msglen, [&] {
    ladder_run(m, opts, sigma, mu, Tlist, nT, Omegas, nOmega, solver, rtol, maxiter, sigma_bubble, sigma_ladder,
               converged, niter, hist, J_out);
  });
}

int epsp_oracle_imsigma_sample(const epsp_model* m, const epsp_options* opts, const double* sigma_in, double mu,
                               double T, int64_t i0, int64_t i1, double* imsigma, char* msg, int32_t msglen) {
  apply_threads();
  return guarded(msg, msglen, [&] {
    Model M = make_model(m);
    if (i0 < 0 || i1 > M.ni || i0 >= i1) throw OracleError(EPSP_EINVAL, "bad outer-state range");
    CellTable ct = cell_search_table(m->omegas, M.ws);
    fan_migdal(M, ct, scgd0_nf_chunk(M, opts->gpu_tile), sigma_in, mu, T, opts->omega_acoustic, imsigma, i0, i1);
  });
}

int epsp_oracle_ladder_apply_sample(const epsp_model* m, const epsp_options* opts, const double* sigma_T, double mu,
                                    double T, double Omega, const double* J, int64_t i0, int64_t i1, double* LJ,
                                    char* msg, int32_t msglen) {
  apply_threads();
  return guarded(msg, msglen, [&] {
    Ladder L = make_ladder(m, opts->gpu_tile);
    if (i0 < 0 || i1 > L.M.ni || i0 >= i1) throw OracleError(EPSP_EINVAL, "bad outer-state range");
    std::vector<cplx> Gm, Gp;
    propagators(L, sigma_T, mu, T, Omega, Gm, Gp);
    ladder_apply(L, Gm, Gp, T, opts->omega_acoustic, J, LJ, i0, i1);
  });
}

int epsp_oracle_ladder_chunks(const epsp_model* m, const epsp_options* opts, int64_t* n_chunks, int64_t* i_lo,
                              int64_t* i_hi, int64_t cap, int64_t* nshift, char* msg, int32_t msglen) {
  return guarded(msg, msglen, [&] {
    Ladder L = make_ladder(m, opts->gpu_tile);
    *n_chunks = int64_t(L.chunks.size());
    if (nshift) *nshift = L.nshift;
    for (int64_t c = 0; c < std::min<int64_t>(cap, *n_chunks); ++c) {
      i_lo[c] = L.chunks[size_t(c)].i0;
      i_hi[c] = L.chunks[size_t(c)].i1;
    }
  });
}

int epsp_oracle_ladder_chunk_operands(const epsp_model* m, const epsp_options* opts, double T, const double* J,
                                      int64_t chunk, double* Xp, double* Xm, double* Bt, char* msg, int32_t msglen) {
  apply_threads();
  return guarded(msg, msglen, [&] {
    Ladder L = make_ladder(m, opts->gpu_tile);
    if (chunk < 0 || chunk >= int64_t(L.chunks.size())) throw OracleError(EPSP_EINVAL, "bad chunk index");
    const auto& ch = L.chunks[size_t(chunk)];
    chunk_coupling(L, ch, T, opts->omega_acoustic, 0, L.M.ni, Bt);
    chunk_shifted_vertex(L, ch, 0, J, Xp);
    chunk_shifted_vertex(L, ch, 1, J, Xm);
  });
}

void epsp_oracle_set_threads(int32_t n) { g_threads = n; }

int32_t epsp_oracle_get_threads(void) {
#ifdef _OPENMP
  if (g_threads > 0) return g_threads;
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
