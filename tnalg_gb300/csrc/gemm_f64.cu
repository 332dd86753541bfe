// FP64 batched / batch-reduced GEMM on the CUDA cores.
//
// C[b] = alpha * sum_r A[b,r] B[b,r] + beta * C[b]  with fully general strides.
// This is the plain-FP64 contraction engine behind the effective-Hamiltonian
// matvec, the environment updates and the QR trailing updates (it replaces the
// np.dot calls of TensorBasicModule.py:387-619 and MPSClass.py:755-776).
//
// GB300 has ~2 FP64 FMA/clk/SM, so the kernel is bound by the FP64 pipe, not by
// memory: what matters is spreading the work over all 152 SMs. Tiles are small
// (32x32) and the K loop is split across CTAs (deterministic two-stage
// reduction through the caller's workspace) when the tile grid is too small to
// fill the GPU.
#include "common.cuh"

namespace {

constexpr int BM = 32, BN = 32, BK = 16, NT = 128;

__global__ void __launch_bounds__(NT) gemm_f64_kernel(TnGemmF64 g, int ksplit, double* part) {
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;  // 16 x 8 threads, 4 rows x 2 cols each
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  const int64_t zb = blockIdx.z / ksplit;
  const int ks = blockIdx.z % ksplit;
  const int64_t kchunk = tn_cdiv(tn_cdiv(g.K, BK), ksplit) * BK;
  const int64_t kbeg = ks * kchunk;
  const int64_t kend = kbeg + kchunk < g.K ? kbeg + kchunk : g.K;
  const bool a_kc = (g.sAk == 1);
  const bool b_nc = (g.sBn == 1);
  double acc[4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i) acc[i][0] = acc[i][1] = 0.0;

  for (int64_t r = 0; r < g.nred; ++r) {
    const double* A = g.A + zb * g.sAb + r * g.sAr;
    const double* B = g.B + zb * g.sBb + r * g.sBr;
    for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
      for (int e = tid; e < BM * BK; e += NT) {
        int mm, kk;
        if (a_kc) { mm = e / BK; kk = e % BK; } else { kk = e / BM; mm = e % BM; }
        const int64_t gm = m0 + mm, gk = k0 + kk;
        As[kk][mm] = (gm < g.M && gk < kend) ? A[gm * g.sAm + gk * g.sAk] : 0.0;
      }
#pragma unroll
      for (int e = tid; e < BN * BK; e += NT) {
        int nn, kk;
        if (b_nc) { kk = e / BN; nn = e % BN; } else { nn = e / BK; kk = e % BK; }
        const int64_t gn = n0 + nn, gk = k0 + kk;
        Bs[kk][nn] = (gn < g.N && gk < kend) ? B[gk * g.sBk + gn * g.sBn] : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        double a[4], b[2];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
        b[0] = Bs[kk][tx * 2];
        b[1] = Bs[kk][tx * 2 + 1];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          acc[i][0] = fma(a[i], b[0], acc[i][0]);
          acc[i][1] = fma(a[i], b[1], acc[i][1]);
        }
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int64_t gm = m0 + ty * 4 + i, gn = n0 + tx * 2 + j;
      if (gm < g.M && gn < g.N) {
        if (ksplit == 1) {
          const int64_t off = zb * g.sCb + gm * g.sCm + gn * g.sCn;
          const double v = g.alpha * acc[i][j];
          g.C[off] = (g.beta == 0.0) ? v : fma(g.beta, (g.Cin ? g.Cin : g.C)[off], v);
        } else {
          part[((int64_t)ks * g.batch + zb) * g.M * g.N + gm * g.N + gn] = acc[i][j];
        }
      }
    }
  }
}

__global__ void splitk_reduce_kernel(TnGemmF64 g, int ksplit, const double* part) {
  const int64_t total = g.batch * g.M * g.N;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t zb = idx / (g.M * g.N);
    const int64_t rem = idx % (g.M * g.N);
    const int64_t gm = rem / g.N, gn = rem % g.N;
    double s = 0.0;
    for (int ks = 0; ks < ksplit; ++ks) s += part[(int64_t)ks * total + idx];
    const int64_t off = zb * g.sCb + gm * g.sCm + gn * g.sCn;
    const double v = g.alpha * s;
    g.C[off] = (g.beta == 0.0) ? v : fma(g.beta, (g.Cin ? g.Cin : g.C)[off], v);
  }
}

}  // namespace

static int gemm_f64_run(const TnGemmF64& g, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return TN_OK;
  if (g.K <= 0 || g.nred <= 0) {
    // C = beta*C: run the reduce kernel with zero partials is wasteful; use ksplit=1 GEMM with K=0.
    TnGemmF64 z = g;
    z.K = 0;
    z.nred = 1;
    dim3 grid((unsigned)tn_cdiv(g.N, BN), (unsigned)tn_cdiv(g.M, BM), (unsigned)g.batch);
    gemm_f64_kernel<<<grid, NT, 0, s>>>(z, 1, nullptr);
    TN_CHECK_LAUNCH();
    return TN_OK;
  }
  const int64_t tiles = tn_cdiv(g.M, BM) * tn_cdiv(g.N, BN) * g.batch;
  const int64_t target = 4LL * tn_sm_count();
  int ksplit = 1;
  const int64_t kt = tn_cdiv(g.K, BK);
  while (tiles * ksplit < target && ksplit * 2 <= kt / 4 && ksplit < 16) ksplit *= 2;
  const size_t need = (size_t)ksplit * g.batch * g.M * g.N * sizeof(double);
  if (ksplit > 1 && (ws == nullptr || ws_bytes < need)) ksplit = 1;
  if (tiles * ksplit > 65535LL * 65535LL) return tn_fail(TN_ERR_ARG, "gemm grid too large");
  dim3 grid((unsigned)tn_cdiv(g.N, BN), (unsigned)tn_cdiv(g.M, BM), (unsigned)(g.batch * ksplit));
  if (grid.z > 65535u) return tn_fail(TN_ERR_ARG, "gemm batch*ksplit exceeds 65535");
  gemm_f64_kernel<<<grid, NT, 0, s>>>(g, ksplit, (double*)ws);
  TN_CHECK_LAUNCH();
  if (ksplit > 1) {
    const int64_t total = g.batch * g.M * g.N;
    const int blocks = (int)std::min<int64_t>(tn_cdiv(total, 256), 8LL * tn_sm_count());
    splitk_reduce_kernel<<<blocks, 256, 0, s>>>(g, ksplit, (const double*)ws);
    TN_CHECK_LAUNCH();
  }
  return TN_OK;
}

int tn_gemm_f64_launch(const TnGemmF64& g, cudaStream_t s) { return gemm_f64_run(g, nullptr, 0, s); }

size_t tn_gemm_f64_ws_bytes(int64_t M, int64_t N, int64_t batch) {
  return (size_t)16 * batch * M * N * sizeof(double);
}

int tn_gemm_f64_ws(const TnGemmF64& g, void* ws, size_t ws_bytes, cudaStream_t s) {
  return gemm_f64_run(g, ws, ws_bytes, s);
}
