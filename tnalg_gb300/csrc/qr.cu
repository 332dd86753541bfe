// FP64 Householder QR for the DMRG gauge move (K4).
//
// Replaces np.linalg.qr in left2right_decompose_tensor / right2left_decompose_tensor
// (TensorBasicModule.py:314-384). Blocked right-looking Householder with the
// compact WY form H_1..H_b = I - V T V^T (forward, column-wise):
//   * panel of NB columns factored by one CTA (reflectors, tau, T);
//   * trailing matrix updated by three FP64 GEMMs (V^T C, T^T W, C - V W);
//   * Q formed backwards from [I; 0] with the same block reflectors.
// The reflector convention (beta = -sign(alpha) ||x||, v(0) = 1) is LAPACK's
// dlarfg, so Q and R agree with numpy's up to rounding.
#include "common.cuh"

namespace {

constexpr int NB = 16;
constexpr int NTP = 512;

size_t al(size_t x) { return (x + 255) / 256 * 256; }

struct QrWs {
  double *Aw, *Vf, *Qw, *T, *W, *W2, *gws;
  size_t gws_bytes;
};

size_t qr_layout(int64_t m, int64_t n, char* base, QrWs* q) {
  const int64_t k = std::min(m, n);
  const int64_t np = tn_cdiv(k, NB);
  size_t off = 0;
  auto take = [&](size_t b) { char* p = base ? base + off : nullptr; off += al(b); return p; };
  q->Aw = (double*)take((size_t)m * n * 8);
  q->Vf = (double*)take((size_t)m * k * 8);
  q->Qw = (double*)take((size_t)m * k * 8);
  q->T = (double*)take((size_t)np * NB * NB * 8);
  q->W = (double*)take((size_t)NB * n * 8);
  q->W2 = (double*)take((size_t)NB * n * 8);
  q->gws_bytes = (size_t)16 * NB * std::max(n, k) * 8;
  q->gws = (double*)take(q->gws_bytes);
  return off + 256;
}

__global__ void qr_copy_in(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn, double* Aw) {
  const int64_t total = m * n;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = idx / m, i = idx % m;
    Aw[idx] = a[i * sAm + j * sAn];
  }
}

__global__ void qr_init_q(int64_t m, int64_t k, double* Qw, double* Vf) {
  const int64_t total = m * k;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = idx / m, i = idx % m;
    Qw[idx] = (i == j) ? 1.0 : 0.0;
    Vf[idx] = 0.0;
  }
}

// Factor columns j0..j0+jb-1 (rows j0..m-1) of the column-major Aw in place.
__global__ void __launch_bounds__(NTP) qr_panel(int64_t m, int64_t j0, int jb, double* Aw, double* Vf, double* T) {
  __shared__ double red[NTP / 32][NB];
  __shared__ double vals[NB];
  __shared__ double sc[3];  // tau, beta, scale
  __shared__ double Ts[NB][NB];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int i = tid; i < NB * NB; i += NTP) Ts[i / NB][i % NB] = 0.0;
  __syncthreads();
  for (int c = 0; c < jb; ++c) {
    const int64_t j = j0 + c;
    double* x = Aw + j * m;
    // (1) sigma = ||x(j+1:m)||^2
    double p = 0.0;
    for (int64_t i = j + 1 + tid; i < m; i += NTP) p = fma(x[i], x[i], p);
    p = tn_warp_sum(p);
    if (lane == 0) red[wid][0] = p;
    __syncthreads();
    if (tid == 0) {
      double sigma = 0.0;
      for (int w = 0; w < NTP / 32; ++w) sigma += red[w][0];
      const double alpha = x[j];
      double tau = 0.0, beta = alpha, scale = 0.0;
      if (sigma > 0.0) {
        const double nrm = sqrt(alpha * alpha + sigma);
        beta = alpha >= 0.0 ? -nrm : nrm;
        tau = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
      }
      sc[0] = tau; sc[1] = beta; sc[2] = scale;
    }
    __syncthreads();
    const double tau = sc[0], scale = sc[2];
    // (2) reflector v: v(j) = 1, v(i>j) = x(i)*scale; R(j,j) = beta
    double* v = Vf + j * m;
    for (int64_t i = j + tid; i < m; i += NTP) {
      if (i == j) { v[i] = 1.0; x[i] = sc[1]; }
      else { const double vi = x[i] * scale; v[i] = vi; x[i] = 0.0; }
    }
    __syncthreads();
    // (3)+(4): dots of v with the remaining panel columns and with earlier reflectors
    const int nr = jb - c - 1;  // remaining columns
    double acc[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) acc[q] = 0.0;
    for (int64_t i = j + tid; i < m; i += NTP) {
      const double vi = v[i];
#pragma unroll
      for (int q = 0; q < NB; ++q) {
        if (q < nr) acc[q] = fma(vi, Aw[(j + 1 + q) * m + i], acc[q]);
        else if (q - nr < c) acc[q] = fma(vi, Vf[(j0 + (q - nr)) * m + i], acc[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const double s = tn_warp_sum(acc[q]);
      if (lane == 0) red[wid][q] = s;
    }
    __syncthreads();
    if (tid < nr + c) {
      double s = 0.0;
      for (int w = 0; w < NTP / 32; ++w) s += red[w][tid];
      vals[tid] = s;
    }
    __syncthreads();
    for (int64_t i = j + tid; i < m; i += NTP) {
      const double vi = v[i];
      for (int q = 0; q < nr; ++q) Aw[(j + 1 + q) * m + i] -= tau * vals[q] * vi;
    }
    if (tid == 0) {
      // T(0:c, c) = -tau * T(0:c, 0:c) * (V(:,0:c)^T v);  T(c,c) = tau
      double z[NB];
      for (int q = 0; q < c; ++q) z[q] = -tau * vals[nr + q];
      for (int r = 0; r < c; ++r) {
        double t = 0.0;
        for (int q = r; q < c; ++q) t = fma(Ts[r][q], z[q], t);
        Ts[r][c] = t;
      }
      Ts[c][c] = tau;
    }
    __syncthreads();
  }
  for (int i = tid; i < NB * NB; i += NTP) T[i] = Ts[i / NB][i % NB];
}

__global__ void qr_extract(int64_t m, int64_t n, int64_t k, const double* Aw, const double* Qw, double* q,
                           int64_t sQm, int64_t sQn, double* r, int64_t sRm, int64_t sRn) {
  const int64_t tq = m * k, tr = k * n;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < tq + tr;
       idx += (int64_t)gridDim.x * blockDim.x) {
    if (idx < tq) {
      const int64_t j = idx / m, i = idx % m;
      if (q) q[i * sQm + j * sQn] = Qw[idx];
    } else {
      const int64_t e = idx - tq;
      const int64_t c = e / k, rr = e % k;
      if (r) r[rr * sRm + c * sRn] = (c >= rr) ? Aw[c * m + rr] : 0.0;
    }
  }
}

int blocks_for(int64_t total) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(total, 256), 8LL * tn_sm_count()));
}

}  // namespace

extern "C" size_t tn_qr_workspace_bytes(int64_t m, int64_t n) {
  if (m <= 0 || n <= 0) return 0;
  QrWs q;
  return qr_layout(m, n, nullptr, &q);
}

extern "C" int tn_qr(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn, double* q, int64_t sQm,
                     int64_t sQn, double* r, int64_t sRm, int64_t sRn, void* ws, size_t ws_bytes, void* stream) {
  if (m <= 0 || n <= 0 || !a) return tn_fail(TN_ERR_ARG, "qr: bad shape");
  QrWs w;
  const size_t need = qr_layout(m, n, nullptr, &w);
  if (!ws || ws_bytes < need) return tn_fail(TN_ERR_WORKSPACE, "qr: workspace too small");
  char* base = (char*)(((uintptr_t)ws + 255) & ~(uintptr_t)255);
  qr_layout(m, n, base, &w);
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t k = std::min(m, n);
  cudaEvent_t ev_all = tn_profile_begin(s);
  qr_copy_in<<<blocks_for(m * n), 256, 0, s>>>(m, n, a, sAm, sAn, w.Aw);
  TN_CHECK_LAUNCH();
  qr_init_q<<<blocks_for(m * k), 256, 0, s>>>(m, k, w.Qw, w.Vf);
  TN_CHECK_LAUNCH();
  const int64_t np = tn_cdiv(k, NB);
  for (int64_t p = 0; p < np; ++p) {
    const int64_t j0 = p * NB;
    const int jb = (int)std::min<int64_t>(NB, k - j0);
    double* Tp = w.T + p * NB * NB;
    cudaEvent_t ev_p = tn_profile_begin(s);
    qr_panel<<<1, NTP, 0, s>>>(m, j0, jb, w.Aw, w.Vf, Tp);
    TN_CHECK_LAUNCH();
    tn_profile_end(ev_p, s, TN_PROF_QR_PANEL, 0.0);
    const int64_t nc = n - j0 - jb;
    if (nc <= 0) continue;
    const int64_t mr = m - j0;
    TnGemmF64 g{};
    // W = V^T C
    g.M = jb; g.N = nc; g.K = mr;
    g.A = w.Vf + j0 + j0 * m; g.sAm = m; g.sAk = 1;
    g.B = w.Aw + j0 + (j0 + jb) * m; g.sBk = 1; g.sBn = m;
    g.C = w.W; g.sCm = nc; g.sCn = 1;
    g.batch = 1; g.nred = 1; g.alpha = 1.0; g.beta = 0.0;
    int st = tn_gemm_f64_ws(g, w.gws, w.gws_bytes, s);
    if (st) return st;
    // W2 = T^T W
    TnGemmF64 h{};
    h.M = jb; h.N = nc; h.K = jb;
    h.A = Tp; h.sAm = 1; h.sAk = NB;
    h.B = w.W; h.sBk = nc; h.sBn = 1;
    h.C = w.W2; h.sCm = nc; h.sCn = 1;
    h.batch = 1; h.nred = 1; h.alpha = 1.0; h.beta = 0.0;
    st = tn_gemm_f64_ws(h, nullptr, 0, s);
    if (st) return st;
    // C -= V W2
    TnGemmF64 u{};
    u.M = mr; u.N = nc; u.K = jb;
    u.A = w.Vf + j0 + j0 * m; u.sAm = 1; u.sAk = m;
    u.B = w.W2; u.sBk = nc; u.sBn = 1;
    u.C = w.Aw + j0 + (j0 + jb) * m; u.sCm = 1; u.sCn = m;
    u.batch = 1; u.nred = 1; u.alpha = -1.0; u.beta = 1.0;
    st = tn_gemm_f64_ws(u, nullptr, 0, s);
    if (st) return st;
  }
  cudaEvent_t ev_q = tn_profile_begin(s);
  if (q) {
    for (int64_t p = np - 1; p >= 0; --p) {
      const int64_t j0 = p * NB;
      const int jb = (int)std::min<int64_t>(NB, k - j0);
      const int64_t nc = k - j0;
      const int64_t mr = m - j0;
      double* Tp = w.T + p * NB * NB;
      TnGemmF64 g{};
      g.M = jb; g.N = nc; g.K = mr;
      g.A = w.Vf + j0 + j0 * m; g.sAm = m; g.sAk = 1;
      g.B = w.Qw + j0 + j0 * m; g.sBk = 1; g.sBn = m;
      g.C = w.W; g.sCm = nc; g.sCn = 1;
      g.batch = 1; g.nred = 1; g.alpha = 1.0; g.beta = 0.0;
      int st = tn_gemm_f64_ws(g, w.gws, w.gws_bytes, s);
      if (st) return st;
      TnGemmF64 h{};
      h.M = jb; h.N = nc; h.K = jb;
      h.A = Tp; h.sAm = NB; h.sAk = 1;
      h.B = w.W; h.sBk = nc; h.sBn = 1;
      h.C = w.W2; h.sCm = nc; h.sCn = 1;
      h.batch = 1; h.nred = 1; h.alpha = 1.0; h.beta = 0.0;
      st = tn_gemm_f64_ws(h, nullptr, 0, s);
      if (st) return st;
      TnGemmF64 u{};
      u.M = mr; u.N = nc; u.K = jb;
      u.A = w.Vf + j0 + j0 * m; u.sAm = 1; u.sAk = m;
      u.B = w.W2; u.sBk = nc; u.sBn = 1;
      u.C = w.Qw + j0 + j0 * m; u.sCm = 1; u.sCn = m;
      u.batch = 1; u.nred = 1; u.alpha = -1.0; u.beta = 1.0;
      st = tn_gemm_f64_ws(u, nullptr, 0, s);
      if (st) return st;
    }
  }
  tn_profile_end(ev_q, s, TN_PROF_QR_FORM_Q, 0.0);
  qr_extract<<<blocks_for(m * k + k * n), 256, 0, s>>>(m, n, k, w.Aw, w.Qw, q, sQm, sQn, r, sRm, sRn);
  TN_CHECK_LAUNCH();
  tn_profile_end(ev_all, s, TN_PROF_QR, 4.0 * m * n * n - 4.0 / 3.0 * n * n * (double)n);
  return TN_OK;
}
