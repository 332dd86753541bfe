// FP32 Householder QR of one m x n matrix (n <= m <= 1024, n <= 512) by ONE 16-CTA thread-block
// cluster, the matrix resident in registers for the whole factorisation and Q formation.
//
// Role: step 1 of the mixed-precision gauge move (tn_qr_mixed): the FP32 factors it returns are
// re-orthogonalised in FP64 afterwards, so only backward stability in FP32 is needed here.
//
// Why a cluster: a Householder QR is a chain of n dependent column steps. On GB300 FP64 runs at
// ~2 lanes/clock/SM with a 64-cycle dependent latency, so the steps are done in FP32, and every
// step is one reduction over all rows: with the rows spread over 16 SMs the per-step cost is a
// distributed-shared-memory reduction (two cluster barriers) instead of a kernel launch and a
// round trip through global memory.
//
// Layout: CTA `rank` of the cluster owns rows [64 rank, 64 rank + 64); thread c of every CTA
// owns column c, so a thread keeps its column's 64 local rows in registers (a[64]). Column c's
// reductions are owned by CTA (c % 16), slot c / 16.
//
// Column step j of the factorisation (LAPACK dgeqr2/dlarfg conventions, beta = -sign(x1)||x||,
// v(j) = 1, tau = (beta - x1) / beta, v(g > j) = x(g) / (x1 - beta)):
//   1. thread c >= j: s_c = sum over local rows g >= j of x(g) a(g, c) (x = column j); thread j
//      instead forms the local sum of squares strictly below the pivot; the CTA holding row j
//      also publishes the pivot row a(j, c). Partials are pushed into the owner CTA's slots.
//   2. barrier; each owner forms w_c = v^T a_c = a(j,c) + (s_c - x1 a(j,c)) / (x1 - beta),
//      f_c = tau w_c, writes R(j, c) = a(j, c) - f_c and pushes f_c to every CTA.
//   3. barrier; every thread c > j updates a(g, c) -= v(g) f_c for its rows; thread j stores v.
// Q is then formed in place backwards (LAPACK dorg2r): step j applies H_j to columns c > j
// (one reduction of v^T q_c per column, same pattern) and sets column j to H_j e_j.
#include "common.cuh"

namespace {

constexpr int CL = 16;          // CTAs per cluster (non-portable size)
constexpr int RPC = 64;         // rows per CTA
constexpr int NT = 512;         // threads per CTA = maximum number of columns
constexpr int SLOTS = NT / CL;  // reduction slots owned per CTA

struct __align__(16) QcShared {
  float xb[2][RPC];      // pivot column of the current / next step (local rows, zero above)
  float vs[2][RPC];      // Householder vector, local rows (v(j) = 1, zero above j)
  float red[CL][SLOTS];  // partial dots pushed by every CTA for the columns this CTA owns
  float piv[SLOTS];      // pivot-row entries a(j, c) of the owned columns
  float sj[CL];          // partial sums of squares below the pivot, one per CTA
  float x1;              // the pivot a(j, j)
  float fb[NT];          // update coefficients f_c of every column (all-gathered)
  float tau[NT];         // tau_j of every reflector
};

// Store v into the copy of `local` (this CTA's shared variable) held by cluster CTA `rank`.
__device__ __forceinline__ void st_remote(const float* local, int rank, float v) {
  uint32_t ra;
  const uint32_t la = (uint32_t)__cvta_generic_to_shared(local);
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(la), "r"(rank));
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(ra), "f"(v) : "memory");
}

// Cluster-wide barrier; release/acquire order the remote stores issued before it.
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ int cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return (int)r;
}

// Rows in chunks of 16 with a compiler fence between chunks: at most 16 broadcast values from
// shared memory are live next to the 64-register column (no spills at 128 registers/thread).
constexpr int CH = 16;

// sum_i a[i] * x[i] over the 64 local rows, x in shared memory (16-byte aligned)
__device__ __forceinline__ float dot_rows(const float (&a)[RPC], const float* x) {
  float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f;
#pragma unroll
  for (int ch = 0; ch < RPC; ch += CH) {
#pragma unroll
    for (int i = ch; i < ch + CH; i += 4) {
      const float4 v = *reinterpret_cast<const float4*>(x + i);
      p0 = fmaf(a[i], v.x, p0);
      p1 = fmaf(a[i + 1], v.y, p1);
      p2 = fmaf(a[i + 2], v.z, p2);
      p3 = fmaf(a[i + 3], v.w, p3);
    }
    asm volatile("" ::: "memory");
  }
  return (p0 + p1) + (p2 + p3);
}

// a[i] -= v[i] * f over the 64 local rows, v in shared memory
__device__ __forceinline__ void axpy_rows(float (&a)[RPC], const float* v, float f) {
#pragma unroll
  for (int ch = 0; ch < RPC; ch += CH) {
#pragma unroll
    for (int i = ch; i < ch + CH; i += 4) {
      const float4 w = *reinterpret_cast<const float4*>(v + i);
      a[i] = fmaf(-w.x, f, a[i]);
      a[i + 1] = fmaf(-w.y, f, a[i + 1]);
      a[i + 2] = fmaf(-w.z, f, a[i + 2]);
      a[i + 3] = fmaf(-w.w, f, a[i + 3]);
    }
    asm volatile("" ::: "memory");
  }
}

__global__ void __launch_bounds__(NT, 1)
    qr32_cluster_kernel(int m, int n, const double* __restrict__ A, int64_t sAm, int64_t sAn, double* __restrict__ Q,
                        double* __restrict__ R, int64_t sRm, int64_t sRn) {
  __shared__ QcShared sh;
  const int rank = cluster_rank();
  const int c = threadIdx.x;
  const int row0 = rank * RPC;

  float a[RPC];
#pragma unroll
  for (int ch = 0; ch < RPC; ch += CH) {
#pragma unroll
    for (int i = ch; i < ch + CH; ++i) {
      const int g = row0 + i;
      a[i] = (c < n && g < m) ? (float)A[(int64_t)g * sAm + (int64_t)c * sAn] : 0.f;
    }
    asm volatile("" ::: "memory");
  }
  if (R && c < n) {  // strictly lower part of R (n x n): zeros, rows spread over the cluster
    int i0 = c + 1;
    i0 += ((rank - i0) % CL + CL) % CL;
    for (int i = i0; i < n; i += CL) R[(int64_t)i * sRm + (int64_t)c * sRn] = 0.0;
  }
  if (c == 0) {
#pragma unroll
    for (int i = 0; i < RPC; ++i) sh.xb[0][i] = a[i];
  }
  cluster_sync();  // every CTA is running (its shared memory exists) before the first remote store

  // ---- factorisation ----
  for (int j = 0; j < n; ++j) {
    const float* X = sh.xb[j & 1];
    const int lj = j - row0;  // local index of row j (outside [0, RPC) if another CTA holds it)
    const bool own_pivot = lj >= 0 && lj < RPC;
    if (c >= j && c < n) {
      float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f;
      if (c == j) {
#pragma unroll
        for (int i = 0; i < RPC; i += 4) {
          p0 = fmaf(a[i], (i > lj) ? a[i] : 0.f, p0);
          p1 = fmaf(a[i + 1], (i + 1 > lj) ? a[i + 1] : 0.f, p1);
          p2 = fmaf(a[i + 2], (i + 2 > lj) ? a[i + 2] : 0.f, p2);
          p3 = fmaf(a[i + 3], (i + 3 > lj) ? a[i + 3] : 0.f, p3);
        }
      }
      const float p = (c == j) ? (p0 + p1) + (p2 + p3) : dot_rows(a, X);
      float pv = 0.f;
      if (own_pivot) {
#pragma unroll
        for (int i = 0; i < RPC; ++i) pv = (i == lj) ? a[i] : pv;
      }
      if (c == j) {
        for (int q = 0; q < CL; ++q) {
          st_remote(&sh.sj[rank], q, p);
          if (own_pivot) st_remote(&sh.x1, q, pv);
        }
      } else {
        const int q = c % CL, t = c / CL;
        st_remote(&sh.red[rank][t], q, p);
        if (own_pivot) st_remote(&sh.piv[t], q, pv);
      }
    }
    cluster_sync();

    float sig = 0.f;
#pragma unroll
    for (int q = 0; q < CL; ++q) sig += sh.sj[q];
    const float x1 = sh.x1;
    float beta = x1, tau = 0.f, scale = 0.f;
    if (sig > 0.f) {
      const float nrm = sqrtf(fmaf(x1, x1, sig));
      beta = (x1 >= 0.f) ? -nrm : nrm;
      tau = (beta - x1) / beta;
      scale = 1.f / (x1 - beta);
    }
    if (c < SLOTS) {
      const int col = c * CL + rank;
      if (col > j && col < n) {
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < CL; ++q) s += sh.red[q][c];
        const float a1 = sh.piv[c];
        const float f = tau * fmaf(s - x1 * a1, scale, a1);
        if (R) R[(int64_t)j * sRm + (int64_t)col * sRn] = (double)(a1 - f);
        for (int q = 0; q < CL; ++q) st_remote(&sh.fb[col], q, f);
      }
    }
    if (R && c == j && own_pivot) R[(int64_t)j * sRm + (int64_t)j * sRn] = (double)beta;
    if (c == 0) sh.tau[j] = tau;
    if (c < RPC) sh.vs[0][c] = (c > lj) ? X[c] * scale : (c == lj ? 1.f : 0.f);
    cluster_sync();

    if (c > j && c < n) {
      axpy_rows(a, sh.vs[0], sh.fb[c]);
      if (c == j + 1) {
        float* Xn = sh.xb[(j + 1) & 1];
#pragma unroll
        for (int i = 0; i < RPC; ++i) Xn[i] = (i > lj) ? a[i] : 0.f;
      }
    } else if (c == j) {
#pragma unroll
      for (int i = 0; i < RPC; ++i) a[i] = (i > lj) ? a[i] * scale : a[i];
    }
    __syncthreads();  // the next pivot column is in shared memory
  }

  // ---- Q formation, backwards, in place ----
  for (int j = n - 1; j >= 0; --j) {
    const int lj = j - row0;
    const float tj = sh.tau[j];
    float* V = sh.vs[j & 1];
    if (c == j) {
#pragma unroll
      for (int i = 0; i < RPC; ++i) V[i] = (i > lj) ? a[i] : (i == lj ? 1.f : 0.f);
    }
    __syncthreads();
    if (c > j && c < n) st_remote(&sh.red[rank][c / CL], c % CL, dot_rows(a, V));
    cluster_sync();
    if (c < SLOTS) {
      const int col = c * CL + rank;
      if (col > j && col < n) {
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < CL; ++q) s += sh.red[q][c];
        const float f = tj * s;
        for (int q = 0; q < CL; ++q) st_remote(&sh.fb[col], q, f);
      }
    }
    cluster_sync();
    if (c > j && c < n) {
      axpy_rows(a, V, sh.fb[c]);
    } else if (c == j) {
#pragma unroll
      for (int i = 0; i < RPC; ++i) a[i] = (i > lj) ? -tj * a[i] : (i == lj ? 1.f - tj : 0.f);
    }
  }

  if (c < n) {
#pragma unroll
    for (int i = 0; i < RPC; ++i) {
      const int g = row0 + i;
      if (g < m) Q[g + (int64_t)c * m] = (double)a[i];
    }
  }
}

int g_cluster_state = -1;  // -1 unknown, 0 unavailable, 1 available

}  // namespace

// True when the 16-CTA cluster kernel can run this shape on the current device.
bool tn_qr32_cluster_supported(int64_t m, int64_t n) {
  if (n < 1 || n > NT || m < n || m > (int64_t)CL * RPC) return false;
  if (g_cluster_state < 0) {
    g_cluster_state = 0;
    if (cudaFuncSetAttribute(qr32_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
        cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(CL);
      cfg.blockDim = dim3(NT);
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = CL;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int clusters = 0;
      if (cudaOccupancyMaxActiveClusters(&clusters, qr32_cluster_kernel, &cfg) == cudaSuccess && clusters > 0)
        g_cluster_state = 1;
    }
    cudaGetLastError();  // an unsupported attribute leaves no sticky error behind
  }
  return g_cluster_state == 1;
}

// Q (column-major m x n, FP64 values of the FP32 factor) and, if R is given, R (n x n, strided).
int tn_qr32_cluster(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn, double* q, double* r,
                    int64_t sRm, int64_t sRn, cudaStream_t s) {
  if (!tn_qr32_cluster_supported(m, n)) return tn_fail(TN_ERR_ARG, "qr32 cluster: unsupported shape or device");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL);
  cfg.blockDim = dim3(NT);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  TN_CUDA(cudaLaunchKernelEx(&cfg, qr32_cluster_kernel, (int)m, (int)n, a, sAm, sAn, q, r, sRm, sRn));
  TN_CHECK_LAUNCH();
  return TN_OK;
}
