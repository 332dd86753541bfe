// FP64 Householder QR for the DMRG gauge move.
//
// Replaces np.linalg.qr in left2right_decompose_tensor / right2left_decompose_tensor
// (TensorBasicModule.py:314-384). Blocked right-looking Householder with the
// compact WY form H_1..H_b = I - V T V^T (forward, column-wise):
//   * panel of NB columns factored by a cluster of 8 CTAs: the panel rows are split
//     across the CTAs (held in shared memory) and every column's norm and dot products
//     are reduced through distributed shared memory between two cluster barriers;
//   * trailing matrix updated by FP64 GEMMs (V^T C, T^T W, C - V W);
//   * Q formed backwards from [I; 0] with the same block reflectors.
// The whole launch sequence of one (m, n, strides, workspace) shape is captured once in
// a CUDA graph and replayed; the input/output pointers travel through a small argument
// block in the workspace, so replays need no graph updates.
// The reflector convention (beta = -sign(alpha) ||x||, v(0) = 1) is LAPACK's dlarfg, so
// Q and R agree with numpy's up to rounding.
#include <cooperative_groups.h>

#include <string.h>

#include <mutex>
#include <vector>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int NB = 16;
constexpr int NTP = 512;  // single-CTA panel
constexpr int CL = 8;     // CTAs per panel cluster
constexpr int PW = 32;    // one warp per cluster CTA
constexpr int PRW = 8;    // panel rows per lane -> <= CL * PW * PRW rows
constexpr int NSLOT = NB + 2;

size_t al(size_t x) { return (x + 255) / 256 * 256; }

struct QrArgs {
  const double* a;
  double* q;
  double* r;
};

struct QrWs {
  QrArgs* args;
  double *Aw, *Vf, *Qw, *T, *W, *W2, *gws;
  size_t gws_bytes;
};

size_t qr_layout(int64_t m, int64_t n, char* base, QrWs* q) {
  const int64_t k = std::min(m, n);
  const int64_t np = tn_cdiv(k, NB);
  size_t off = 0;
  auto take = [&](size_t b) { char* p = base ? base + off : nullptr; off += al(b); return p; };
  q->args = (QrArgs*)take(sizeof(QrArgs));
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

__global__ void qr_set_args(QrArgs* args, const double* a, double* q, double* r) {
  args->a = a;
  args->q = q;
  args->r = r;
}

__global__ void qr_copy_in(int64_t m, int64_t n, const QrArgs* args, int64_t sAm, int64_t sAn, double* Aw) {
  const double* a = args->a;
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

// Householder scalars of x = (alpha, tail) with ||tail||^2 = sigma (LAPACK dlarfg convention).
__device__ __forceinline__ void householder(double alpha, double sigma, double* tau, double* beta, double* scale) {
  *tau = 0.0;
  *beta = alpha;
  *scale = 0.0;
  if (sigma > 0.0) {
    const double nrm = sqrt(alpha * alpha + sigma);
    *beta = alpha >= 0.0 ? -nrm : nrm;
    *tau = (*beta - alpha) / *beta;
    *scale = 1.0 / (alpha - *beta);
  }
}

// Factor columns j0..j0+jb-1 (rows j0..m-1) of the column-major Aw in place; one CTA.
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
    double p = 0.0;
    for (int64_t i = j + 1 + tid; i < m; i += NTP) p = fma(x[i], x[i], p);
    p = tn_warp_sum(p);
    if (lane == 0) red[wid][0] = p;
    __syncthreads();
    if (tid == 0) {
      double sigma = 0.0;
      for (int w = 0; w < NTP / 32; ++w) sigma += red[w][0];
      householder(x[j], sigma, &sc[0], &sc[1], &sc[2]);
    }
    __syncthreads();
    const double tau = sc[0], scale = sc[2];
    double* v = Vf + j * m;
    for (int64_t i = j + tid; i < m; i += NTP) {
      if (i == j) { v[i] = 1.0; x[i] = sc[1]; }
      else { const double vi = x[i] * scale; v[i] = vi; x[i] = 0.0; }
    }
    __syncthreads();
    const int nr = jb - c - 1;
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

// The same panel factorisation spread over a cluster of CL CTAs of ONE warp each. CTA `rank`
// owns panel rows [r0, r0 + nr) in shared memory (PRW rows per lane). GB300 issues FP64 at ~2
// lanes/clock/SM, so every FP64 warp instruction costs ~16 cycles whatever it computes: the
// kernel keeps the FP64 instruction count per column low (one warp, a transposing 16-value warp
// reduction, unpredicated dot slots, a lane-parallel T column). Per column, each CTA pushes its
// partial sums into every rank's `gath` slot (remote shared-memory stores) and a cluster barrier
// publishes them; slots are double-buffered across columns.
__device__ __forceinline__ void warp_reduce16(double (&a)[16], int lane) {
  // afterwards lanes 2i and 2i+1 hold the warp-wide sum of slot i
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const bool up = lane & 16;
    const double send = up ? a[i] : a[i + 8], keep = up ? a[i + 8] : a[i];
    a[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const bool up = lane & 8;
    const double send = up ? a[i] : a[i + 4], keep = up ? a[i + 4] : a[i];
    a[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const bool up = lane & 4;
    const double send = up ? a[i] : a[i + 2], keep = up ? a[i + 2] : a[i];
    a[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  {
    const bool up = lane & 2;
    const double send = up ? a[0] : a[1], keep = up ? a[1] : a[0];
    a[0] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
  }
  a[0] += __shfl_xor_sync(0xffffffffu, a[0], 1);
}

__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(PW)
    qr_panel_cluster(int64_t m, int64_t j0, int jb, double* Aw, double* Vf, double* T) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  extern __shared__ double dyn[];
  double(*P)[NB + 1] = reinterpret_cast<double(*)[NB + 1]>(dyn);
  double(*Vs)[NB + 1] = reinterpret_cast<double(*)[NB + 1]>(dyn + PW * PRW * (NB + 1));
  __shared__ double gath[2][CL][NSLOT];
  __shared__ double Ts[NB][NB];
  const int lane = threadIdx.x;
  const int64_t chunk = tn_cdiv(m - j0, CL);
  const int64_t r0 = j0 + rank * chunk;
  const int64_t r1 = (m < r0 + chunk) ? m : r0 + chunk;
  const int nr = r1 > r0 ? (int)(r1 - r0) : 0;
  for (int e = lane; e < PW * PRW * (NB + 1); e += PW) (&Vs[0][0])[e] = 0.0;
  for (int e = lane; e < nr * jb; e += PW) {
    const int rr = e % nr, c = e / nr;
    P[rr][c] = Aw[(j0 + c) * m + r0 + rr];
  }
  for (int e = lane; e < NB * NB; e += PW) Ts[e / NB][e % NB] = 0.0;
  __syncwarp();
  int buf = 0;
  for (int c = 0; c < jb; ++c) {
    const int64_t j = j0 + c;
    // (a) partial ||x(j+1:)||^2 and the diagonal entry alpha
    double ps = 0.0, pa = 0.0;
#pragma unroll
    for (int q = 0; q < PRW; ++q) {
      const int rr = lane + q * PW;
      if (rr < nr) {
        const int64_t i = r0 + rr;
        const double x = P[rr][c];
        if (i > j) ps = fma(x, x, ps);
        else if (i == j) pa = x;
      }
    }
    ps = tn_warp_sum(ps);
    pa = tn_warp_sum(pa);
    if (lane < 2 * CL) cluster.map_shared_rank(&gath[buf][rank][0], lane >> 1)[lane & 1] = (lane & 1) ? pa : ps;
    cluster.sync();
    double sigma = 0.0, alpha = 0.0;
#pragma unroll
    for (int r = 0; r < CL; ++r) { sigma += gath[buf][r][0]; alpha += gath[buf][r][1]; }
    double tau, beta, scale;
    householder(alpha, sigma, &tau, &beta, &scale);
    double vq[PRW];
#pragma unroll
    for (int q = 0; q < PRW; ++q) {
      const int rr = lane + q * PW;
      vq[q] = 0.0;
      if (rr < nr) {
        const int64_t i = r0 + rr;
        if (i == j) { vq[q] = 1.0; P[rr][c] = beta; }
        else if (i > j) { vq[q] = P[rr][c] * scale; P[rr][c] = 0.0; }
        Vs[rr][c] = vq[q];
      }
    }
    __syncwarp();
    // (b) dot products: slot t < nrem with panel column c+1+t, slot t >= nrem with reflector t-nrem
    const int nrem = jb - c - 1;
    const int nd = nrem + c;
    double acc[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) acc[t] = 0.0;
#pragma unroll
    for (int q = 0; q < PRW; ++q) {
      const int rr = lane + q * PW;
      if (rr < nr && vq[q] != 0.0) {
#pragma unroll
        for (int t = 0; t < 16; ++t) {
          const double* src = (t < nrem) ? &P[rr][c + 1 + t] : &Vs[rr][t - nrem];
          acc[t] = fma(vq[q], *src, acc[t]);
        }
      }
    }
    warp_reduce16(acc, lane);
    const int slot_i = (lane >> 1) & 15;
    if (slot_i < nd) {
      const int half = lane & 1;
#pragma unroll
      for (int dd = 0; dd < CL / 2; ++dd)
        cluster.map_shared_rank(&gath[buf][rank][0], half * (CL / 2) + dd)[2 + slot_i] = acc[0];
    }
    cluster.sync();
    double wt = 0.0;
    if (slot_i < nd) {
#pragma unroll
      for (int r = 0; r < CL; ++r) wt += gath[buf][r][2 + slot_i];
    }
    // rank-1 update of the remaining panel columns: P(:, c+1+t) -= tau * w_t * v
    for (int t = 0; t < nrem; ++t) {
      const double coef = tau * __shfl_sync(0xffffffffu, wt, 2 * t);
#pragma unroll
      for (int q = 0; q < PRW; ++q) {
        const int rr = lane + q * PW;
        if (rr < nr && vq[q] != 0.0) P[rr][c + 1 + t] = fma(-coef, vq[q], P[rr][c + 1 + t]);
      }
    }
    // T(0:c, c) = -tau * T(0:c, 0:c) * (V(:, 0:c)^T v); lane r owns row r
    double tr = 0.0;
    for (int qq = 0; qq < c; ++qq) {
      const double z = -tau * __shfl_sync(0xffffffffu, wt, 2 * (nrem + qq));
      if (lane < c && qq >= lane) tr = fma(Ts[lane][qq], z, tr);
    }
    if (lane < c) Ts[lane][c] = tr;
    if (lane == 0) Ts[c][c] = tau;
    __syncwarp();
    buf ^= 1;
  }
  for (int e = lane; e < nr * jb; e += PW) {
    const int rr = e % nr, c = e / nr;
    Aw[(j0 + c) * m + r0 + rr] = P[rr][c];
    Vf[(j0 + c) * m + r0 + rr] = Vs[rr][c];
  }
  if (rank == 0)
    for (int e = lane; e < NB * NB; e += PW) T[e] = Ts[e / NB][e % NB];
  cluster.sync();  // no CTA leaves while another may still write into its slots
}

__global__ void qr_extract(int64_t m, int64_t n, int64_t k, const double* Aw, const double* Qw, const QrArgs* args,
                           int64_t sQm, int64_t sQn, int64_t sRm, int64_t sRn) {
  double* q = args->q;
  double* r = args->r;
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

constexpr size_t kClusterSmem = (size_t)2 * PW * PRW * (NB + 1) * sizeof(double);

int launch_panel(int64_t m, int64_t j0, int jb, const QrWs& w, double* Tp, cudaStream_t s) {
  if (m - j0 <= (int64_t)CL * PW * PRW) {
    int st = tn_set_smem_attr_once(TN_ATTR_QR_PANEL_CLUSTER, (const void*)qr_panel_cluster, (int)kClusterSmem);
    if (st) return st;
    qr_panel_cluster<<<CL, PW, kClusterSmem, s>>>(m, j0, jb, w.Aw, w.Vf, Tp);
  } else {
    qr_panel<<<1, NTP, 0, s>>>(m, j0, jb, w.Aw, w.Vf, Tp);
  }
  TN_CHECK_LAUNCH();
  return TN_OK;
}

// Every launch of one QR except qr_set_args (pointer-free, graph-capturable).
int qr_body(int64_t m, int64_t n, int64_t sAm, int64_t sAn, int64_t sQm, int64_t sQn, int64_t sRm, int64_t sRn,
            bool want_q, const QrWs& w, cudaStream_t s) {
  const int64_t k = std::min(m, n);
  qr_copy_in<<<blocks_for(m * n), 256, 0, s>>>(m, n, w.args, sAm, sAn, w.Aw);
  TN_CHECK_LAUNCH();
  qr_init_q<<<blocks_for(m * k), 256, 0, s>>>(m, k, w.Qw, w.Vf);
  TN_CHECK_LAUNCH();
  const int64_t np = tn_cdiv(k, NB);
  int st;
  for (int64_t p = 0; p < np; ++p) {
    const int64_t j0 = p * NB;
    const int jb = (int)std::min<int64_t>(NB, k - j0);
    double* Tp = w.T + p * NB * NB;
    if ((st = launch_panel(m, j0, jb, w, Tp, s))) return st;
    const int64_t nc = n - j0 - jb;
    if (nc <= 0) continue;
    const int64_t mr = m - j0;
    TnGemmF64 g{};  // W = V^T C
    g.M = jb; g.N = nc; g.K = mr;
    g.A = w.Vf + j0 + j0 * m; g.sAm = m; g.sAk = 1;
    g.B = w.Aw + j0 + (j0 + jb) * m; g.sBk = 1; g.sBn = m;
    g.C = w.W; g.sCm = nc; g.sCn = 1;
    g.batch = 1; g.nred = 1; g.alpha = 1.0; g.beta = 0.0;
    if ((st = tn_gemm_f64_ws(g, w.gws, w.gws_bytes, s))) return st;
    TnGemmF64 h{};  // W2 = T^T W
    h.M = jb; h.N = nc; h.K = jb;
    h.A = Tp; h.sAm = 1; h.sAk = NB;
    h.B = w.W; h.sBk = nc; h.sBn = 1;
    h.C = w.W2; h.sCm = nc; h.sCn = 1;
    h.batch = 1; h.nred = 1; h.alpha = 1.0; h.beta = 0.0;
    if ((st = tn_gemm_f64_ws(h, nullptr, 0, s))) return st;
    TnGemmF64 u{};  // C -= V W2
    u.M = mr; u.N = nc; u.K = jb;
    u.A = w.Vf + j0 + j0 * m; u.sAm = 1; u.sAk = m;
    u.B = w.W2; u.sBk = nc; u.sBn = 1;
    u.C = w.Aw + j0 + (j0 + jb) * m; u.sCm = 1; u.sCn = m;
    u.batch = 1; u.nred = 1; u.alpha = -1.0; u.beta = 1.0;
    if ((st = tn_gemm_f64_ws(u, nullptr, 0, s))) return st;
  }
  if (want_q) {
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
      if ((st = tn_gemm_f64_ws(g, w.gws, w.gws_bytes, s))) return st;
      TnGemmF64 h{};
      h.M = jb; h.N = nc; h.K = jb;
      h.A = Tp; h.sAm = NB; h.sAk = 1;
      h.B = w.W; h.sBk = nc; h.sBn = 1;
      h.C = w.W2; h.sCm = nc; h.sCn = 1;
      h.batch = 1; h.nred = 1; h.alpha = 1.0; h.beta = 0.0;
      if ((st = tn_gemm_f64_ws(h, nullptr, 0, s))) return st;
      TnGemmF64 u{};
      u.M = mr; u.N = nc; u.K = jb;
      u.A = w.Vf + j0 + j0 * m; u.sAm = 1; u.sAk = m;
      u.B = w.W2; u.sBk = nc; u.sBn = 1;
      u.C = w.Qw + j0 + j0 * m; u.sCm = 1; u.sCn = m;
      u.batch = 1; u.nred = 1; u.alpha = -1.0; u.beta = 1.0;
      if ((st = tn_gemm_f64_ws(u, nullptr, 0, s))) return st;
    }
  }
  qr_extract<<<blocks_for(m * k + k * n), 256, 0, s>>>(m, n, k, w.Aw, w.Qw, w.args, sQm, sQn, sRm, sRn);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

// Graph cache: one executable graph per (shape, strides, workspace, outputs requested).
struct QrGraph {
  int64_t key[11];
  cudaGraphExec_t exec;
  unsigned long long kernels;  // kernel launches recorded into the graph
};
// g_graphs, its eviction and the capture stream are shared by all host threads: g_graph_mu guards
// the lookup, a capture, the insertion and the launch of a cached graph (an eviction by another
// thread could otherwise destroy an executable graph between its lookup and its launch).
// Least recently used at the front. The keys include the workspace address, so every MPS (every
// job of a multi-job run) has its own graphs, a dozen or so shapes each (interior and edge moves
// in both directions): the cache holds enough for many interleaved jobs, so that round-robin
// over them replays graphs instead of capturing one at every move.
constexpr size_t kQrGraphCap = 512;
std::vector<QrGraph> g_graphs;
std::mutex g_graph_mu;
std::atomic<bool> g_use_graphs{true};

}  // namespace

extern "C" size_t tn_qr_workspace_bytes(int64_t m, int64_t n) {
  if (m <= 0 || n <= 0) return 0;
  QrWs q;
  return qr_layout(m, n, nullptr, &q);
}

extern "C" int tn_qr_use_graphs(int on) {
  g_use_graphs = on != 0;
  return TN_OK;
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
  cudaEvent_t ev_all = tn_profile_begin(s);
  qr_set_args<<<1, 1, 0, s>>>(w.args, a, q, r);
  TN_CHECK_LAUNCH();
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  TN_CUDA(cudaStreamIsCapturing(s, &cap));
  int st;
  if (!g_use_graphs || cap != cudaStreamCaptureStatusNone) {
    st = qr_body(m, n, sAm, sAn, sQm, sQn, sRm, sRn, q != nullptr, w, s);
  } else {
    std::lock_guard<std::mutex> lock(g_graph_mu);
    int dev = 0;
    if ((st = tn_current_device(&dev))) return st;
    const int64_t key[11] = {m, n, sAm, sAn, sQm, sQn, sRm, sRn, (int64_t)(uintptr_t)base, q != nullptr, dev};
    cudaGraphExec_t exec = nullptr;
    unsigned long long kernels = 0;
    for (size_t i = 0; i < g_graphs.size(); ++i)
      if (memcmp(g_graphs[i].key, key, sizeof(key)) == 0) {
        exec = g_graphs[i].exec;
        kernels = g_graphs[i].kernels;
        std::rotate(g_graphs.begin() + i, g_graphs.begin() + i + 1, g_graphs.end());  // now most recent
        break;
      }
    if (!exec) {
      // capture on a private stream (the caller's may be the legacy default stream, which
      // cannot capture); nothing runs during capture, the graph is launched on `s` below.
      // one capture stream per device (a stream belongs to the device it was created on)
      static cudaStream_t capture_streams[TN_MAX_DEVICES] = {nullptr};
      cudaStream_t& cs = capture_streams[dev];
      if (!cs) TN_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t graph;
      TN_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      const unsigned long long launches0 = g_tn_thread_launches;
      st = qr_body(m, n, sAm, sAn, sQm, sQn, sRm, sRn, q != nullptr, w, cs);
      cudaError_t e = cudaStreamEndCapture(cs, &graph);
      kernels = g_tn_thread_launches - launches0;
      g_tn_thread_launches = launches0;  // recorded, not run: counted at every replay below
      g_tn_launches.fetch_sub(kernels);
      if (st) return st;
      if (e != cudaSuccess) return tn_record_error(e);
      e = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return tn_record_error(e);
      if (g_graphs.size() >= kQrGraphCap) {
        cudaGraphExecDestroy(g_graphs.front().exec);
        g_graphs.erase(g_graphs.begin());
      }
      QrGraph gg;
      memcpy(gg.key, key, sizeof(key));
      gg.exec = exec;
      gg.kernels = kernels;
      g_graphs.push_back(gg);
    }
    TN_CUDA(cudaGraphLaunch(exec, s));
    g_tn_launches.fetch_add(kernels);
    g_tn_thread_launches += kernels;
    st = TN_OK;
  }
  // algorithmic work of the factorisation, 2mn^2 - 2n^3/3 (forming Q is not counted)
  tn_profile_end(ev_all, s, TN_PROF_QR, 2.0 * m * n * (double)n - 2.0 / 3.0 * n * n * (double)n);
  return st;
}
