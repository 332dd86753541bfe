// Effective-Hamiltonian matvec and the device-resident Lanczos eigensolver.
//
// The matvec replaces update_tensor_eigs_f_handle_optimized (MPSClass.py:755-776):
//   H_eff psi = WL.psi(chi_l d, chi_r) + psi(chi_l, d chi_r).WR^T + sum_k SL_k psi SR_k^T
// where WL/WR are the enlarged-block operators (all left-/right-acting buckets of
// classify_and_update_env, MPSClass.py:684-733, summed into one matrix each) and
// SL/SR the straddling '1_0_1' pairs.
//
// The eigensolver replaces scipy's eigsh(..., which='LM') on I - tau*H_eff
// (MPSClass.py:800-807). Krylov vectors live in the caller's workspace; every
// inner product, the Gram-Schmidt projections (classical GS, applied twice) and
// the tridiagonal eigenproblem are FP64. The host only reads the alpha/beta
// coefficients every `check_every` steps to test convergence.
#include <math.h>
#include <string.h>

#include <vector>

#include "common.cuh"

int tn_dot_ws(int64_t n, const double* x, const double* y, double* out, void* ws, size_t ws_bytes, cudaStream_t s);
int tn_matvec_tf32x3(const tn_site_desc* d, const double* psi, double* y, double alpha, double beta,
                     void* ws, size_t ws_bytes, cudaStream_t s);
size_t tn_matvec_tf32x3_ws_bytes(const tn_site_desc* d);
int tn_tf32x3_prepare_static(const tn_site_desc* d, void* ws, size_t ws_bytes, cudaStream_t s);
int tn_matvec_tf32x3_fp64_region(const tn_site_desc* d, void* ws, size_t ws_bytes, void** out, size_t* out_bytes);

namespace {

constexpr int NT = 256;
constexpr int kMaxKrylov = 128;

size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// ---------------------------------------------------------------------------
// FP64 matvec through the CUDA-core GEMM

int matvec_fp64(const tn_site_desc* ds, const double* psi, double* y, double alpha, double beta, void* ws,
                size_t ws_bytes, cudaStream_t s) {
  const int64_t cl = ds->chil, d = ds->d, cr = ds->chir;
  const int64_t n = cl * d * cr;
  char* p = (char*)ws;
  size_t zbytes = align_up((size_t)ds->nstr * n * sizeof(double));
  double* Z = ds->nstr > 0 ? (double*)p : nullptr;
  void* gws = p + zbytes;
  size_t gws_bytes = ws_bytes > zbytes ? ws_bytes - zbytes : 0;
  if (ds->nstr > 0 && ws_bytes < zbytes) return tn_fail(TN_ERR_WORKSPACE, "matvec: workspace too small");
  bool first = true;
  if (ds->wl) {
    TnGemmF64 g{};
    g.M = cl * d; g.N = cr; g.K = cl * d;
    g.A = ds->wl; g.sAm = cl * d; g.sAk = 1;
    g.B = psi; g.sBk = cr; g.sBn = 1;
    g.C = y; g.sCm = cr; g.sCn = 1; g.Cin = psi;
    g.batch = 1; g.nred = 1;
    g.alpha = alpha; g.beta = beta;
    int st = tn_gemm_f64_ws(g, gws, gws_bytes, s);
    if (st) return st;
    first = false;
  }
  if (ds->wr) {
    TnGemmF64 g{};
    g.M = cl; g.N = d * cr; g.K = d * cr;
    g.A = psi; g.sAm = d * cr; g.sAk = 1;
    g.B = ds->wr; g.sBk = 1; g.sBn = d * cr;
    g.C = y; g.sCm = d * cr; g.sCn = 1; g.Cin = first ? psi : y;
    g.batch = 1; g.nred = 1;
    g.alpha = alpha; g.beta = first ? beta : 1.0;
    int st = tn_gemm_f64_ws(g, gws, gws_bytes, s);
    if (st) return st;
    first = false;
  }
  if (ds->nstr > 0) {
    TnGemmF64 g{};
    g.M = cl; g.N = d * cr; g.K = cl;
    g.A = ds->sl; g.sAm = cl; g.sAk = 1; g.sAb = cl * cl;
    g.B = psi; g.sBk = d * cr; g.sBn = 1; g.sBb = 0;
    g.C = Z; g.sCm = d * cr; g.sCn = 1; g.sCb = n;
    g.batch = ds->nstr; g.nred = 1;
    g.alpha = 1.0; g.beta = 0.0;
    int st = tn_gemm_f64_ws(g, gws, gws_bytes, s);
    if (st) return st;
    TnGemmF64 h{};
    h.M = cl * d; h.N = cr; h.K = cr;
    h.A = Z; h.sAm = cr; h.sAk = 1; h.sAr = n;
    h.B = ds->sr; h.sBk = 1; h.sBn = cr; h.sBr = cr * cr;
    h.C = y; h.sCm = cr; h.sCn = 1; h.Cin = first ? psi : y;
    h.batch = 1; h.nred = ds->nstr;
    h.alpha = alpha; h.beta = first ? beta : 1.0;
    st = tn_gemm_f64_ws(h, gws, gws_bytes, s);
    if (st) return st;
    first = false;
  }
  if (first) {
    // H_eff == 0: y = beta * psi
    TnGemmF64 g{};
    g.M = 1; g.N = n; g.K = 0;
    g.A = psi; g.sAm = 0; g.sAk = 0;
    g.B = psi; g.sBk = 0; g.sBn = 0;
    g.C = y; g.sCm = 0; g.sCn = 1; g.Cin = psi;
    g.batch = 1; g.nred = 0;
    g.alpha = 0.0; g.beta = beta;
    if (beta == 0.0) g.beta = 0.0;
    return tn_gemm_f64_ws(g, nullptr, 0, s);
  }
  return TN_OK;
}

size_t matvec_fp64_ws_bytes(const tn_site_desc* ds) {
  const int64_t cl = ds->chil, d = ds->d, cr = ds->chir;
  const int64_t n = cl * d * cr;
  size_t b = align_up((size_t)ds->nstr * n * sizeof(double));
  const int64_t mx = std::max<int64_t>(cl * d * cr, 1);
  b += align_up((size_t)16 * mx * sizeof(double));  // split-K partials of the largest output
  return b;
}

// ---------------------------------------------------------------------------
// Lanczos vector kernels. V is (ldv) x n row-major: vector i at V + i*n.

// The vector kernels are bound by L2/HBM latency times the bytes in flight: every thread keeps
// four grid-strided elements (UNR) of each operand in flight before it uses any of them.
constexpr int UNR = 4;

// part[i*nb + blockIdx.x] = sum over this block's chunk of V[i]·w ; last block per column reduces.
__global__ void multidot_kernel(int64_t n, int ncols, const double* __restrict__ V, const double* __restrict__ w,
                                double* part, unsigned int* tickets, double* out) {
  const int i = blockIdx.y;
  const double* v = V + (int64_t)i * n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double a4[UNR] = {0.0, 0.0, 0.0, 0.0};
  for (; k + (UNR - 1) * stride < n; k += UNR * stride) {
    double x[UNR], y[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      x[u] = v[k + u * stride];
      y[u] = w[k + u * stride];
    }
#pragma unroll
    for (int u = 0; u < UNR; ++u) a4[u] = fma(x[u], y[u], a4[u]);
  }
  for (; k < n; k += stride) a4[0] = fma(v[k], w[k], a4[0]);
  double acc = (a4[0] + a4[1]) + (a4[2] + a4[3]);
  __shared__ double red[NT / 32];
  __shared__ bool last;
  acc = tn_warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < NT / 32; ++q) t += red[q];
    part[(int64_t)i * gridDim.x + blockIdx.x] = t;
    __threadfence();
    last = (atomicAdd(tickets + i, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {  // uniform over the block
    const double t = tn_block_sum_partials(part + (int64_t)i * gridDim.x, gridDim.x);
    if (threadIdx.x == 0) {
      out[i] = t;
      tickets[i] = 0u;
    }
  }
}

// w -= sum_i h[i] V[i]; optionally nrm2 = ||w||^2 (deterministic last-block reduction).
__global__ void multiaxpy_kernel(int64_t n, int ncols, const double* __restrict__ V, const double* __restrict__ h,
                                 double* __restrict__ w, double* part, unsigned int* ticket, double* nrm2) {
  __shared__ double hs[kMaxKrylov + 1];
  for (int i = threadIdx.x; i < ncols; i += blockDim.x) hs[i] = h[i];
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double a4[UNR] = {0.0, 0.0, 0.0, 0.0};
  for (; k + (UNR - 1) * stride < n; k += UNR * stride) {
    double x[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) x[u] = w[k + u * stride];
    for (int i = 0; i < ncols; ++i) {
      const double* vi = V + (int64_t)i * n;
      double y[UNR];
#pragma unroll
      for (int u = 0; u < UNR; ++u) y[u] = vi[k + u * stride];
#pragma unroll
      for (int u = 0; u < UNR; ++u) x[u] = fma(-hs[i], y[u], x[u]);
    }
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      w[k + u * stride] = x[u];
      a4[u] = fma(x[u], x[u], a4[u]);
    }
  }
  for (; k < n; k += stride) {
    double x = w[k];
    for (int i = 0; i < ncols; ++i) x = fma(-hs[i], V[(int64_t)i * n + k], x);
    w[k] = x;
    a4[0] = fma(x, x, a4[0]);
  }
  double acc = (a4[0] + a4[1]) + (a4[2] + a4[3]);
  if (!nrm2) return;
  __shared__ double red[NT / 32];
  __shared__ bool last;
  acc = tn_warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < NT / 32; ++q) t += red[q];
    part[blockIdx.x] = t;
    __threadfence();
    last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {  // uniform over the block
    const double t = tn_block_sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      *nrm2 = t;
      *ticket = 0u;
    }
  }
}

// v = w / sqrt(nrm2) (0 on breakdown); block 0 records alpha[j] = h1[j] + h2[j], beta[j] = sqrt(nrm2).
__global__ void lanczos_finish_kernel(int64_t n, int j, const double* __restrict__ w, double* __restrict__ v,
                                      const double* h1, const double* h2, const double* nrm2, double* alpha,
                                      double* beta) {
  const double nn = *nrm2;
  const double b = nn > 0.0 ? sqrt(nn) : 0.0;
  const double inv = b > 1e-300 ? 1.0 / b : 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; k + (UNR - 1) * stride < n; k += UNR * stride) {
    double x[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) x[u] = w[k + u * stride];
#pragma unroll
    for (int u = 0; u < UNR; ++u) v[k + u * stride] = x[u] * inv;
  }
  for (; k < n; k += stride) v[k] = w[k] * inv;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    alpha[j] = h1[j] + h2[j];
    beta[j] = b;
  }
}

// x = sum_i s[i] V[i]
__global__ void combine_kernel(int64_t n, int ncols, const double* __restrict__ V, const double* __restrict__ s,
                               double* __restrict__ x) {
  __shared__ double ss[kMaxKrylov + 1];
  for (int i = threadIdx.x; i < ncols; i += blockDim.x) ss[i] = s[i];
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; k + (UNR - 1) * stride < n; k += UNR * stride) {
    double acc[UNR] = {0.0, 0.0, 0.0, 0.0};
    for (int i = 0; i < ncols; ++i) {
      const double* vi = V + (int64_t)i * n;
      double y[UNR];
#pragma unroll
      for (int u = 0; u < UNR; ++u) y[u] = vi[k + u * stride];
#pragma unroll
      for (int u = 0; u < UNR; ++u) acc[u] = fma(ss[i], y[u], acc[u]);
    }
#pragma unroll
    for (int u = 0; u < UNR; ++u) x[k + u * stride] = acc[u];
  }
  for (; k < n; k += stride) {
    double acc = 0.0;
    for (int i = 0; i < ncols; ++i) acc = fma(ss[i], V[(int64_t)i * n + k], acc);
    x[k] = acc;
  }
}

// dst = src * alpha / sqrt(nrm2)
__global__ void scaled_copy_kernel(int64_t n, const double* src, double* dst,
                                   const double* nrm2) {
  const double nn = *nrm2;
  const double inv = nn > 0.0 ? 1.0 / sqrt(nn) : 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; k + (UNR - 1) * stride < n; k += UNR * stride) {
    double x[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) x[u] = src[k + u * stride];
#pragma unroll
    for (int u = 0; u < UNR; ++u) dst[k + u * stride] = x[u] * inv;
  }
  for (; k < n; k += stride) dst[k] = src[k] * inv;
}

// r = w - e*x (e = x.w), nrm2 = ||r||^2 computed in the dot kernel afterwards
__global__ void residual_kernel(int64_t n, const double* __restrict__ x, const double* __restrict__ e,
                                double* __restrict__ w) {
  const double ev = *e;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    w[k] = fma(-ev, x[k], w[k]);
}

// ---------------------------------------------------------------------------
// Host-side symmetric tridiagonal: lowest eigenpair by Sturm bisection + inverse iteration.

int sturm_count(const double* a, const double* b, int m, double x) {
  // number of eigenvalues < x, via the pivots of the LDL^T factorisation of T - x I
  int cnt = 0;
  double q = a[0] - x;
  if (q < 0) ++cnt;
  for (int i = 1; i < m; ++i) {
    const double qq = fabs(q) < 1e-300 ? (q < 0 ? -1e-300 : 1e-300) : q;
    q = (a[i] - x) - b[i - 1] * b[i - 1] / qq;
    if (q < 0) ++cnt;
  }
  return cnt;
}

// Solve (T - lam I) z = r with Gaussian elimination and partial pivoting (tridiagonal -> 3 diagonals).
void tridiag_solve(const double* a, const double* b, int m, double lam, std::vector<double>& z) {
  std::vector<double> d0(m), d1(m, 0.0), d2(m, 0.0), rhs(z);
  std::vector<double> sub(m, 0.0);
  for (int i = 0; i < m; ++i) {
    d0[i] = a[i] - lam;
    if (i + 1 < m) d1[i] = b[i];
    if (i > 0) sub[i] = b[i - 1];
  }
  // Row i holds (sub[i], d0[i], d1[i], d2[i]) in columns i-1, i, i+1, i+2.
  for (int i = 0; i < m - 1; ++i) {
    if (fabs(sub[i + 1]) > fabs(d0[i])) {
      std::swap(d0[i], sub[i + 1]);
      std::swap(d1[i], d0[i + 1]);
      std::swap(d2[i], d1[i + 1]);
      std::swap(rhs[i], rhs[i + 1]);
    }
    double piv = d0[i];
    if (fabs(piv) < 1e-300) piv = 1e-300;
    const double f = sub[i + 1] / piv;
    d0[i + 1] -= f * d1[i];
    d1[i + 1] -= f * d2[i];
    rhs[i + 1] -= f * rhs[i];
    sub[i + 1] = 0.0;
  }
  for (int i = m - 1; i >= 0; --i) {
    double v = rhs[i];
    if (i + 1 < m) v -= d1[i] * z[i + 1];
    if (i + 2 < m) v -= d2[i] * z[i + 2];
    double piv = d0[i];
    if (fabs(piv) < 1e-300) piv = 1e-300;
    z[i] = v / piv;
  }
}

void lowest_eigenpair(const double* a, const double* b, int m, double* lam_out, std::vector<double>& s) {
  double lo = a[0], hi = a[0];
  for (int i = 0; i < m; ++i) {
    const double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i + 1 < m ? fabs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  const double scale = std::max(fabs(lo), fabs(hi)) + 1e-300;
  for (int it = 0; it < 200 && (hi - lo) > 4e-16 * scale; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_count(a, b, m, mid) >= 1) hi = mid; else lo = mid;
  }
  const double lam = 0.5 * (lo + hi);
  s.assign(m, 1.0);
  for (int i = 0; i < m; ++i) s[i] = 1.0 + 1e-3 * i;  // generic start
  for (int it = 0; it < 3; ++it) {
    std::vector<double> z(s);
    tridiag_solve(a, b, m, lam, z);
    double nrm = 0.0;
    for (double v : z) nrm += v * v;
    nrm = sqrt(nrm);
    if (!(nrm > 0) || !isfinite(nrm)) break;
    for (int i = 0; i < m; ++i) s[i] = z[i] / nrm;
  }
  *lam_out = lam;
}

struct LanczosWs {
  double *V, *w, *h1, *h2, *alpha, *beta, *nrm2, *s, *part, *e;
  unsigned int* tickets;
  void* mv_ws;
  size_t mv_bytes;
  int nblocks;
};

int lanczos_blocks(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(n, NT), 2LL * tn_sm_count()));
}

size_t lanczos_layout(const tn_site_desc* ds, const tn_lanczos_opts* o, char* base, LanczosWs* L) {
  const int64_t n = ds->chil * ds->d * ds->chir;
  const int m = std::max(2, std::min<int>(o->max_krylov, kMaxKrylov));
  const int nb = lanczos_blocks(n);
  size_t off = 0;
  auto take = [&](size_t bytes) { char* p = base ? base + off : nullptr; off += align_up(bytes); return p; };
  L->V = (double*)take((size_t)(m + 1) * n * sizeof(double));
  L->w = (double*)take((size_t)n * sizeof(double));
  L->h1 = (double*)take((kMaxKrylov + 1) * sizeof(double));
  L->h2 = (double*)take((kMaxKrylov + 1) * sizeof(double));
  L->alpha = (double*)take((kMaxKrylov + 1) * sizeof(double));
  L->beta = (double*)take((kMaxKrylov + 1) * sizeof(double));
  L->nrm2 = (double*)take(4 * sizeof(double));
  L->e = (double*)take(4 * sizeof(double));
  L->s = (double*)take((kMaxKrylov + 1) * sizeof(double));
  L->tickets = (unsigned int*)take((kMaxKrylov + 2) * sizeof(unsigned int));
  L->part = (double*)take((size_t)(kMaxKrylov + 1) * nb * sizeof(double));
  L->nblocks = nb;
  const size_t mvb = (o->precision == TN_PREC_TF32X3) ? tn_matvec_tf32x3_ws_bytes(ds) : matvec_fp64_ws_bytes(ds);
  L->mv_ws = take(mvb);
  L->mv_bytes = mvb;
  return off + 256;
}

}  // namespace

// ---------------------------------------------------------------------------

size_t tn_matvec_fp64_ws_bytes(const tn_site_desc* ds) { return matvec_fp64_ws_bytes(ds); }

// y += alpha * sum_k SL_k psi SR_k^T in FP64 (the straddling part of the matvec).
int tn_matvec_fp64_straddle(const tn_site_desc* ds, const double* psi, double* y, double alpha, void* ws,
                            size_t ws_bytes, cudaStream_t s) {
  if (ds->nstr <= 0) return TN_OK;
  const int64_t n = ds->chil * ds->d * ds->chir;
  const size_t zb = align_up((size_t)ds->nstr * n * sizeof(double));
  if (ws_bytes < zb) return tn_fail(TN_ERR_WORKSPACE, "straddle: workspace too small");
  const int64_t cl = ds->chil, d = ds->d, cr = ds->chir;
  double* Z = (double*)ws;
  TnGemmF64 g{};
  g.M = cl; g.N = d * cr; g.K = cl;
  g.A = ds->sl; g.sAm = cl; g.sAk = 1; g.sAb = cl * cl;
  g.B = psi; g.sBk = d * cr; g.sBn = 1; g.sBb = 0;
  g.C = Z; g.sCm = d * cr; g.sCn = 1; g.sCb = n;
  g.batch = ds->nstr; g.nred = 1; g.alpha = 1.0; g.beta = 0.0;
  int st = tn_gemm_f64_ws(g, (char*)ws + zb, ws_bytes - zb, s);
  if (st) return st;
  TnGemmF64 h{};
  h.M = cl * d; h.N = cr; h.K = cr;
  h.A = Z; h.sAm = cr; h.sAk = 1; h.sAr = n;
  h.B = ds->sr; h.sBk = 1; h.sBn = cr; h.sBr = cr * cr;
  h.C = y; h.sCm = cr; h.sCn = 1; h.Cin = y;
  h.batch = 1; h.nred = ds->nstr; h.alpha = alpha; h.beta = 1.0;
  return tn_gemm_f64_ws(h, (char*)ws + zb, ws_bytes - zb, s);
}

// Useful flops of one block-form matvec: WL.psi + psi.WR^T + straddling pairs.
static double matvec_flops(const tn_site_desc* ds) {
  const double cl = (double)ds->chil, d = (double)ds->d, cr = (double)ds->chir;
  double f = 0.0;
  if (ds->wl) f += 2.0 * (cl * d) * (cl * d) * cr;
  if (ds->wr) f += 2.0 * cl * (d * cr) * (d * cr);
  f += (double)ds->nstr * (2.0 * cl * cl * d * cr + 2.0 * cl * d * cr * cr);
  return f;
}

extern "C" size_t tn_matvec_workspace_bytes(const tn_site_desc* desc, int precision) {
  if (!desc) return 0;
  return precision == TN_PREC_TF32X3 ? tn_matvec_tf32x3_ws_bytes(desc) : matvec_fp64_ws_bytes(desc);
}

static int check_desc(const tn_site_desc* ds) {
  if (!ds || ds->chil <= 0 || ds->d <= 0 || ds->chir <= 0 || ds->nstr < 0)
    return tn_fail(TN_ERR_ARG, "site descriptor: bad dimensions");
  if (ds->nstr > 0 && (!ds->sl || !ds->sr)) return tn_fail(TN_ERR_ARG, "site descriptor: straddling pointers missing");
  return TN_OK;
}

extern "C" int tn_matvec(const tn_site_desc* desc, const double* psi, double* y, double alpha, double beta,
                         int precision, void* ws, size_t ws_bytes, void* stream) {
  int st = check_desc(desc);
  if (st) return st;
  if (!psi || !y) return tn_fail(TN_ERR_ARG, "matvec: null vector");
  if (psi == y) return tn_fail(TN_ERR_ARG, "matvec: psi and y must not alias");
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == TN_PREC_TF32X3) {
    if (ws_bytes < tn_matvec_tf32x3_ws_bytes(desc)) return tn_fail(TN_ERR_WORKSPACE, "matvec: workspace too small");
    st = tn_tf32x3_prepare_static(desc, ws, ws_bytes, s);
    if (st) return st;
    return tn_matvec_tf32x3(desc, psi, y, alpha, beta, ws, ws_bytes, s);
  }
  if (precision != TN_PREC_FP64) return tn_fail(TN_ERR_ARG, "matvec: unknown precision");
  return matvec_fp64(desc, psi, y, alpha, beta, ws, ws_bytes, s);
}

extern "C" size_t tn_lanczos_workspace_bytes(const tn_site_desc* desc, const tn_lanczos_opts* opts) {
  if (!desc || !opts) return 0;
  LanczosWs L;
  return lanczos_layout(desc, opts, nullptr, &L);
}

static int lanczos_impl(const tn_site_desc* desc, double* psi, const tn_lanczos_opts* o, void* ws,
                        size_t ws_bytes, tn_lanczos_result* res, void* stream) {
  int st = check_desc(desc);
  if (st) return st;
  if (!psi || !o || !res) return tn_fail(TN_ERR_ARG, "lanczos: null argument");
  if (o->precision != TN_PREC_FP64 && o->precision != TN_PREC_TF32X3) return tn_fail(TN_ERR_ARG, "lanczos: precision");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t n = desc->chil * desc->d * desc->chir;
  LanczosWs L;
  const size_t need = lanczos_layout(desc, o, nullptr, &L);
  if (!ws || ws_bytes < need) return tn_fail(TN_ERR_WORKSPACE, "lanczos: workspace too small");
  char* base = (char*)(((uintptr_t)ws + 255) & ~(uintptr_t)255);
  lanczos_layout(desc, o, base, &L);
  const int m = (int)std::min<int64_t>(std::max(2, std::min<int>(o->max_krylov, kMaxKrylov)), n);
  const int check = std::max(1, o->check_every);
  const int nb = L.nblocks;
  const bool mixed = (o->precision == TN_PREC_TF32X3);

  TN_CUDA(cudaMemsetAsync(L.tickets, 0, (kMaxKrylov + 2) * sizeof(unsigned int), s));
  // FP64 matvecs of a split-TF32 solve (refinement) work in the FP64 region of the split-TF32
  // workspace, which leaves the staged hi/lo operator copies intact
  void* f64_ws = L.mv_ws;
  size_t f64_bytes = L.mv_bytes;
  if (mixed) {
    st = tn_tf32x3_prepare_static(desc, L.mv_ws, L.mv_bytes, s);
    if (st) return st;
    st = tn_matvec_tf32x3_fp64_region(desc, L.mv_ws, L.mv_bytes, &f64_ws, &f64_bytes);
    if (st) return st;
  }
  auto matvec = [&](const double* x, double* y) -> int {
    cudaEvent_t ev = tn_profile_begin(s);
    const int r = mixed ? tn_matvec_tf32x3(desc, x, y, 1.0, 0.0, L.mv_ws, L.mv_bytes, s)
                        : matvec_fp64(desc, x, y, 1.0, 0.0, L.mv_ws, L.mv_bytes, s);
    tn_profile_end(ev, s, TN_PROF_MATVEC, matvec_flops(desc));
    return r;
  };
  // single dot product through the multi-dot kernel (its own ticket slot)
  auto dot2 = [&](const double* x, const double* y, double* out) -> int {
    multidot_kernel<<<dim3(nb, 1), NT, 0, s>>>(n, 1, x, y, L.part, L.tickets + kMaxKrylov + 1, out);
    TN_CHECK_LAUNCH();
    return TN_OK;
  };

  // V[0] = psi / ||psi||
  st = dot2(psi, psi, L.nrm2);
  if (st) return st;
  scaled_copy_kernel<<<nb, NT, 0, s>>>(n, psi, L.V, L.nrm2);
  TN_CHECK_LAUNCH();

  std::vector<double> ha(kMaxKrylov + 1), hb(kMaxKrylov + 1), sv;
  // the device error word (range flags of the split-TF32 staging, bounded waits) travels with
  // alpha/beta at every convergence check, so a mixed-precision solve needs no sync of its own
  int* dev_err = nullptr;
  if (mixed && (st = tn_error_word(s, &dev_err))) return st;
  int herr = 0;
  int matvecs = 0, restarts = 0;
  bool converged = false;
  double theta = 0.0, resid = INFINITY;
  // refine == 2 on the split-TF32 path: once the mixed-precision iteration has reached its floor,
  // every further restart cycle begins with an FP64 matvec of the current vector x. That step's
  // alpha = x.Hx and beta = ||Hx - alpha x|| are FP64-exact (the true Rayleigh quotient and
  // residual), the cycle's later matvecs act on vectors orthogonal to x with weights of order
  // beta/gap, so their split-TF32 error enters the next vector only at second order: each cycle
  // divides the true residual by ~(split-TF32 error x ||H|| / gap) until it meets the FP64 tolerance.
  const bool vec_refine = mixed && o->refine == 2;
  const int max_cycles = o->refine_cycles > 0 ? o->refine_cycles : 4;
  bool exact_phase = false;  // restart cycles open with an FP64 matvec
  int cycles = 0;
  double beta0 = INFINITY, theta0 = 0.0;
  for (;;) {
    int jj = 0;
    bool stop = false;
    for (int j = 0; j < m; ++j) {
      double* vj = L.V + (int64_t)j * n;
      const bool exact = exact_phase && j == 0;
      if (exact) {
        cudaEvent_t ev = tn_profile_begin(s);
        st = matvec_fp64(desc, vj, L.w, 1.0, 0.0, f64_ws, f64_bytes, s);
        tn_profile_end(ev, s, TN_PROF_MATVEC, matvec_flops(desc));
      } else {
        st = matvec(vj, L.w);
      }
      if (st) return st;
      ++matvecs;
      const int nc = j + 1;
      multidot_kernel<<<dim3(nb, nc), NT, 0, s>>>(n, nc, L.V, L.w, L.part, L.tickets, L.h1);
      TN_CHECK_LAUNCH();
      multiaxpy_kernel<<<nb, NT, 0, s>>>(n, nc, L.V, L.h1, L.w, nullptr, nullptr, nullptr);
      TN_CHECK_LAUNCH();
      multidot_kernel<<<dim3(nb, nc), NT, 0, s>>>(n, nc, L.V, L.w, L.part, L.tickets, L.h2);
      TN_CHECK_LAUNCH();
      multiaxpy_kernel<<<nb, NT, 0, s>>>(n, nc, L.V, L.h2, L.w, L.part, L.tickets + kMaxKrylov + 1, L.nrm2);
      TN_CHECK_LAUNCH();
      lanczos_finish_kernel<<<nb, NT, 0, s>>>(n, j, L.w, L.V + (int64_t)(j + 1) * n, L.h1, L.h2, L.nrm2, L.alpha,
                                             L.beta);
      TN_CHECK_LAUNCH();
      const bool last = (j + 1 == m);
      if ((j + 1) % check == 0 || last || exact) {
        TN_CUDA(cudaMemcpyAsync(ha.data(), L.alpha, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
        TN_CUDA(cudaMemcpyAsync(hb.data(), L.beta, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (mixed) TN_CUDA(cudaMemcpyAsync(&herr, dev_err, sizeof(int), cudaMemcpyDeviceToHost, s));
        TN_CUDA(cudaStreamSynchronize(s));
        if (herr) return tn_error_status(herr, s);
        for (int i = 0; i < nc; ++i)
          if (!isfinite(ha[i]) || !isfinite(hb[i])) return tn_fail(TN_ERR_NUMERIC, "lanczos: non-finite coefficient");
        // breakdown: truncate at the first negligible beta
        int mm = nc;
        double tnorm = 0.0;
        for (int i = 0; i < nc; ++i) tnorm = std::max(tnorm, fabs(ha[i]) + fabs(hb[i]));
        bool brk = false;
        for (int i = 0; i < nc - 1; ++i)
          if (hb[i] <= 1e-14 * std::max(tnorm, 1e-300)) { mm = i + 1; brk = true; break; }
        lowest_eigenpair(ha.data(), hb.data(), mm, &theta, sv);
        resid = brk ? 0.0 : fabs(hb[mm - 1] * sv[mm - 1]);
        if (hb[mm - 1] <= 1e-14 * std::max(tnorm, 1e-300)) { resid = 0.0; brk = true; }
        double tol;
        if (o->tau > 0) tol = o->eigs_tol / o->tau * fabs(1.0 - o->tau * theta);
        else tol = o->eigs_tol * std::max(1.0, fabs(theta));
        if (o->tol_cap > 0) tol = std::min(tol, o->tol_cap * std::max(1.0, fabs(theta)));
        if (exact_phase) {
          if (exact) {
            // FP64-exact Rayleigh quotient and residual of the current vector
            theta0 = ha[0];
            beta0 = hb[0];
            if (beta0 <= tol || brk) { converged = true; jj = 1; sv.assign(1, 1.0); stop = true; break; }
            continue;
          }
          // a cycle ends once its mixed-precision estimate has dropped well below the exact
          // residual it started from; the next cycle's FP64 step measures the true one
          if (resid <= std::max(tol, 1e-4 * beta0) || brk || nc >= n || last) { jj = mm; break; }
          continue;
        }
        if (mixed) tol = std::max(tol, std::max(o->mixed_floor, 0.0) * std::max(1.0, fabs(theta)));
        if (resid <= tol || brk || nc >= n) {
          jj = mm;
          if (vec_refine && !brk && nc < n) { exact_phase = true; break; }
          converged = true;
          stop = true;
          break;
        }
        if (last) { jj = mm; break; }
      }
    }
    // Ritz vector x = V s / ||s|| -> psi: the basis is orthonormal to ~1e-15 (Gram-Schmidt twice),
    // so ||V s|| = ||s|| to that accuracy and no separate normalisation pass is needed
    {
      double ss = 0.0;
      for (int i = 0; i < jj; ++i) ss += sv[i] * sv[i];
      const double inv = ss > 0.0 ? 1.0 / sqrt(ss) : 0.0;
      for (int i = 0; i < jj; ++i) sv[i] *= inv;
    }
    TN_CUDA(cudaMemcpyAsync(L.s, sv.data(), jj * sizeof(double), cudaMemcpyHostToDevice, s));
    combine_kernel<<<nb, NT, 0, s>>>(n, jj, L.V, L.s, psi);
    TN_CHECK_LAUNCH();
    if (stop) break;
    if (exact_phase) {
      if (cycles >= max_cycles) {
        // the FP64 residual measured at the start of the last cycle stands for the vector
        theta = theta0;
        resid = beta0;
        break;
      }
      ++cycles;
    } else {
      if (restarts >= o->max_restarts) break;
    }
    ++restarts;
    TN_CUDA(cudaMemcpyAsync(L.V, psi, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  if (vec_refine && exact_phase && converged) {
    theta = theta0;
    resid = beta0;
  }
  res->energy = theta;
  res->residual = resid;
  res->energy_fp64 = theta;
  if (o->refine == 1) {
    // FP64 residual and Rayleigh quotient of the final vector.
    st = matvec_fp64(desc, psi, L.w, 1.0, 0.0, f64_ws, f64_bytes, s);
    if (st) return st;
    ++matvecs;
    st = dot2(psi, L.w, L.e);
    if (st) return st;
    residual_kernel<<<nb, NT, 0, s>>>(n, psi, L.e, L.w);
    TN_CHECK_LAUNCH();
    st = dot2(L.w, L.w, L.nrm2);
    if (st) return st;
    double hv[2];
    TN_CUDA(cudaMemcpyAsync(&hv[0], L.e, sizeof(double), cudaMemcpyDeviceToHost, s));
    TN_CUDA(cudaMemcpyAsync(&hv[1], L.nrm2, sizeof(double), cudaMemcpyDeviceToHost, s));
    TN_CUDA(cudaStreamSynchronize(s));
    res->energy_fp64 = hv[0];
    res->residual = sqrt(std::max(hv[1], 0.0));
  }
  res->matvecs = matvecs;
  res->restarts = restarts;
  res->converged = converged ? 1 : 0;
  return converged ? TN_OK : TN_ERR_NOCONV;
}

extern "C" int tn_lanczos(const tn_site_desc* desc, double* psi, const tn_lanczos_opts* o, void* ws,
                          size_t ws_bytes, tn_lanczos_result* res, void* stream) {
  cudaEvent_t ev = tn_profile_begin((cudaStream_t)stream);
  const int st = lanczos_impl(desc, psi, o, ws, ws_bytes, res, stream);
  tn_profile_end(ev, (cudaStream_t)stream, TN_PROF_LANCZOS, 0.0);
  return st;
}
