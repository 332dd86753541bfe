// Grouped building blocks and the batched gauge-move QR of the batched DMRG path.
//
// tn_grouped_ops: every item of a table in one launch, each item one of
//   * a block operator of an enlarged block (the classify_and_update_env buckets summed,
//     MPSClass.py:684-733), as tn_assemble_block;
//   * slot combinations out[g] = sum c E[slot] (straddling pairs, gathered carried operators), as
//     tn_combine_slots;
//   * site operators on the physical bond (TensorBasicModule.py:414-421), as tn_apply_site_ops.
// The environment stack of an item has general slot and row strides.
//
// tn_batched_qr_mixed: the gauge move of many jobs' site tensors at once (left2right_decompose_tensor
// / right2left_decompose_tensor, TensorBasicModule.py:314-384), in the mixed precision of tn_qr_mixed:
//   1. one CTA per matrix (m x n, n <= m, m n <= 32768): the input scaled by a power of two and
//      rounded to FP32 in shared memory, Householder QR column by column (LAPACK geqr2 order), R
//      written out (FP32-accurate, scaled back), Q formed in place (org2r order) and written as FP64
//      over the input and as FP32 into scratch;
//   2. E = Q^T Q - I in FP64 from the FP32 copy (every product of two FP32 values is exact in FP64);
//   3. Q <- Q - Q E / 2 with the grouped split-TF32 GEMM (the product is ~1e-6 in size, so its
//      ~1e-6 relative error is ~1e-12): Q orthonormal to ~1e-12, spanning col(A) to FP32 accuracy.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "grouped.cuh"

namespace {

constexpr int NT = 256;
constexpr int CHUNK = 1024;  // work units per block of tn_grouped_ops

__device__ __forceinline__ int find_item(const int* prefix, int n, int t) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ double op_elem(const double* ops, int op, int64_t d, int64_t r, int64_t c) {
  return op < 0 ? (r == c ? 1.0 : 0.0) : ops[(int64_t)op * d * d + r * d + c];
}

// Work units of an item: a block operator is computed one (environment row, column) pair at a time
// (its d x d block of outputs, d <= 4); the other kinds one output element at a time.
__host__ __device__ __forceinline__ int64_t op_units(const tn_batch_op& it) {
  return (it.kind == TN_BOP_BLOCK_LEFT || it.kind == TN_BOP_BLOCK_RIGHT) ? (int64_t)it.chi * it.chi : it.total;
}

constexpr int MAX_D = 4;

__global__ void __launch_bounds__(NT) grouped_ops_kernel(const tn_batch_op* items, int nitems, const int* prefix) {
  const int t = blockIdx.x;
  const int i = find_item(prefix, nitems, t);
  const tn_batch_op it = items[i];
  if (it.active && *it.active == 0) return;
  const int64_t u0 = (int64_t)(t - prefix[i]) * CHUNK;
  const int64_t u1 = min(op_units(it), u0 + CHUNK);
  const int chi = it.chi, d = it.d;
  const tn_block_term* terms = (const tn_block_term*)it.terms;
  if (it.kind == TN_BOP_BLOCK_LEFT || it.kind == TN_BOP_BLOCK_RIGHT) {
    // unit (r, c) of the environment: W[(r s'), (c s)] (left) or W[(s' r), (s c)] (right) for all s', s
    const int n = chi * d;
    for (int64_t u = u0 + threadIdx.x; u < u1; u += blockDim.x) {
      const int r = (int)(u / chi), c = (int)(u - (int64_t)r * chi);
      double acc[MAX_D * MAX_D];
#pragma unroll
      for (int q = 0; q < MAX_D * MAX_D; ++q) acc[q] = 0.0;
      for (int q = 0; q < it.nterms; ++q) {
        const tn_block_term tt = terms[q];
        const double e = tt.slot < 0 ? (r == c ? 1.0 : 0.0) : it.src[(int64_t)tt.slot * it.s_slot + (int64_t)r * it.s_row + c];
        if (e == 0.0) continue;
        const double ce = tt.coeff * e;
        // fully unrolled over the MAX_D x MAX_D block so that acc stays in registers
        if (tt.op < 0) {
#pragma unroll
          for (int x = 0; x < MAX_D; ++x)
            if (x < d) acc[x * MAX_D + x] += ce;
        } else {
          const double* o = it.ops + (int64_t)tt.op * d * d;
#pragma unroll
          for (int x = 0; x < MAX_D; ++x)
#pragma unroll
            for (int y = 0; y < MAX_D; ++y)
              if (x < d && y < d) acc[x * MAX_D + y] = fma(ce, o[x * d + y], acc[x * MAX_D + y]);
        }
      }
#pragma unroll
      for (int x = 0; x < MAX_D; ++x)
#pragma unroll
        for (int y = 0; y < MAX_D; ++y)
          if (x < d && y < d) {
            const int64_t row = (it.kind == TN_BOP_BLOCK_LEFT) ? (int64_t)r * d + x : (int64_t)x * chi + r;
            const int64_t col = (it.kind == TN_BOP_BLOCK_LEFT) ? (int64_t)c * d + y : (int64_t)y * chi + c;
            it.out[row * n + col] = acc[x * MAX_D + y];
          }
    }
  } else if (it.kind == TN_BOP_COMBINE) {
    const int64_t m = (int64_t)chi * chi;
    for (int64_t idx = u0 + threadIdx.x; idx < u1; idx += blockDim.x) {
      const int g = (int)(idx / m);
      const int e = (int)(idx - g * m);
      const int r = e / chi, c = e - r * chi;
      double acc = 0.0;
      for (int q = 0; q < it.nterms; ++q) {
        const tn_block_term tt = terms[q];
        if (tt.op != g) continue;
        const double v = tt.slot < 0 ? (r == c ? 1.0 : 0.0) : it.src[(int64_t)tt.slot * it.s_slot + (int64_t)r * it.s_row + c];
        acc = fma(tt.coeff, v, acc);
      }
      it.out[(int64_t)g * it.out_stride + e] = acc;
    }
  } else {  // TN_BOP_SITE_OPS: out[k][a, s', b] = sum_s ops[opidx[k]][s', s] src[a, s, b]
    const int chir = it.chir;
    const int64_t per = (int64_t)chi * d * chir;
    for (int64_t idx = u0 + threadIdx.x; idx < u1; idx += blockDim.x) {
      const int k = (int)(idx / per);
      const int64_t e = idx - k * per;
      const int64_t a = e / ((int64_t)d * chir);
      const int rem = (int)(e - a * d * chir);
      const int sp = rem / chir, b = rem - sp * chir;
      const int op = ((const int32_t*)it.terms)[k];
      double acc = 0.0;
      for (int s2 = 0; s2 < d; ++s2) {
        const double o = op < 0 ? (sp == s2 ? 1.0 : 0.0) : it.ops[(int64_t)op * d * d + sp * d + s2];
        acc = fma(o, it.src[(a * d + s2) * chir + b], acc);
      }
      it.out[(int64_t)k * it.out_stride + e] = acc;
    }
  }
}

// ---------------------------------------------------------------------------
// batched mixed-precision QR

constexpr int QR_NT = 256;
constexpr int QR_MAX_ELEMS = 32768;  // m * n floats in shared memory (128 KB)

struct QrbItem {
  int32_t m, n;
  double* a;
  int64_t sAm, sAn;
  double* r;
  int64_t sRm, sRn;
  float* qs;     // FP32 copy of Q, column-major (m x n)
  double* e;     // n x n Gram correction
  const int32_t* active;
};

__device__ __forceinline__ float block_sumf(float v, float* red) {
  v = tn_warp_sumf(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = 0.f;
  for (int w = 0; w < QR_NT / 32; ++w) t += red[w];
  __syncthreads();
  return t;
}

// Columns c > j of A (column-major, ld m) <- H_j A: w = A[j, c] + v . A[j+1:, c] (v_j = 1, v below
// the diagonal in column j), A[:, c] -= tau w v. Warp `warp` takes columns j + 1 + warp + 8 i, four
// at a time so that four independent load / FMA / shuffle chains overlap; each column's arithmetic
// (per-lane partial sums in row order, then the warp sum) is that of one column at a time.
__device__ __forceinline__ void apply_reflector_cols(float* A, int m, int n, int j, float tj, int warp, int lane) {
  constexpr int NWARP = QR_NT / 32, G = 4;
  for (int c0 = j + 1 + warp; c0 < n; c0 += G * NWARP) {
    float ajc[G], w[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int c = c0 + g * NWARP;
      ajc[g] = (c < n) ? A[j + c * m] : 0.f;  // read by every lane before lane 0 rewrites it
      w[g] = 0.f;
    }
    for (int r = j + 1 + lane; r < m; r += 32) {
      const float v = A[r + j * m];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const int c = c0 + g * NWARP;
        if (c < n) w[g] = fmaf(v, A[r + c * m], w[g]);
      }
    }
    float tw[G];
#pragma unroll
    for (int g = 0; g < G; ++g) tw[g] = tj * (tn_warp_sumf(w[g]) + ajc[g]);
    __syncwarp();
    if (lane == 0) {
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const int c = c0 + g * NWARP;
        if (c < n) A[j + c * m] = ajc[g] - tw[g];
      }
    }
    for (int r = j + 1 + lane; r < m; r += 32) {
      const float v = A[r + j * m];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const int c = c0 + g * NWARP;
        if (c < n) A[r + c * m] = fmaf(-tw[g], v, A[r + c * m]);
      }
    }
  }
}

// one CTA per matrix; dynamic shared memory: A as column-major m x n floats (ld = m) + tau (n)
__global__ void __launch_bounds__(QR_NT) qrb_householder_kernel(const QrbItem* items) {
  extern __shared__ float sm[];
  __shared__ float red[QR_NT / 32];
  __shared__ float sv[2];
  __shared__ int sexp;
  const QrbItem it = items[blockIdx.x];
  if (it.active && *it.active == 0) return;
  const int m = it.m, n = it.n;
  float* A = sm;             // A[r + c * m]
  float* tau = sm + m * n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // scale: max |a| to [1, 2) by an exact power of two
  double mx = 0.0;
  for (int idx = threadIdx.x; idx < m * n; idx += QR_NT) {
    const int r = idx % m, c = idx / m;
    mx = fmax(mx, fabs(it.a[(int64_t)r * it.sAm + (int64_t)c * it.sAn]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  __shared__ double wmax[QR_NT / 32];
  if (lane == 0) wmax[warp] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < QR_NT / 32; ++w) t = fmax(t, wmax[w]);
    sexp = (t > 0.0 && isfinite(t)) ? ilogb(t) : 0;
  }
  __syncthreads();
  const int ex = sexp;
  for (int idx = threadIdx.x; idx < m * n; idx += QR_NT) {
    const int r = idx % m, c = idx / m;
    A[idx] = (float)ldexp(it.a[(int64_t)r * it.sAm + (int64_t)c * it.sAn], -ex);
  }
  __syncthreads();
  // Householder QR: column j -> reflector v (v_j = 1 implicit, v below the diagonal stored in A),
  // tau_j, beta_j on the diagonal
  for (int j = 0; j < n; ++j) {
    float ss = 0.f;
    for (int r = j + 1 + threadIdx.x; r < m; r += QR_NT) ss = fmaf(A[r + j * m], A[r + j * m], ss);
    ss = block_sumf(ss, red);
    if (threadIdx.x == 0) {
      const float alpha = A[j + j * m];
      float t = 0.f, scale = 0.f, beta = alpha;
      if (ss > kHhTiny) {  // smaller sub-columns are taken as zero (see kHhTiny)
        beta = -copysignf(sqrtf(fmaf(alpha, alpha, ss)), alpha);
        t = (beta - alpha) / beta;
        scale = 1.f / (alpha - beta);
      }
      tau[j] = t;
      sv[0] = scale;
      A[j + j * m] = beta;
    }
    __syncthreads();
    const float scale = sv[0];
    for (int r = j + 1 + threadIdx.x; r < m; r += QR_NT) A[r + j * m] *= scale;
    __syncthreads();
    const float tj = tau[j];
    if (tj != 0.f) apply_reflector_cols(A, m, n, j, tj, warp, lane);
    __syncthreads();
  }
  // R (upper n x n), scaled back
  for (int idx = threadIdx.x; idx < n * n; idx += QR_NT) {
    const int r = idx / n, c = idx % n;
    it.r[(int64_t)r * it.sRm + (int64_t)c * it.sRn] = (r <= c) ? ldexp((double)A[r + c * m], ex) : 0.0;
  }
  __syncthreads();
  // Q in place, backwards (org2r): column j of Q from reflector j applied to e_j, after the
  // columns j+1.. have received reflector j
  for (int j = n - 1; j >= 0; --j) {
    const float tj = tau[j];
    // w = v . Q[j:, c] with v_j = 1 (Q[j, c] is still 0 here: column c > j has no entries above its
    // own diagonal yet)
    if (j < n - 1) apply_reflector_cols(A, m, n, j, tj, warp, lane);
    __syncthreads();
    for (int r = threadIdx.x; r < m; r += QR_NT) {
      if (r < j) A[r + j * m] = 0.f;
      else if (r == j) A[r + j * m] = 1.f - tj;
      else A[r + j * m] = -tj * A[r + j * m];
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < m * n; idx += QR_NT) {
    const int r = idx % m, c = idx / m;
    const float q = A[idx];
    it.qs[idx] = q;
    it.a[(int64_t)r * it.sAm + (int64_t)c * it.sAn] = (double)q;
  }
}

// a * b added to the double-float (hi, lo): TwoProduct by FMA and TwoSum (Ogita, Rump and Oishi's
// Dot2); the _rn intrinsics are never contracted into FMAs, which would break both transformations
__device__ __forceinline__ void qrb_dot2_step(float a, float b, float& hi, float& lo) {
  const float h = __fmul_rn(a, b);
  const float r = fmaf(a, b, -h);
  const float t = __fadd_rn(hi, h);
  const float z = __fsub_rn(t, hi);
  const float q = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, z)), __fsub_rn(h, z));
  hi = t;
  lo = __fadd_rn(lo, __fadd_rn(q, r));
}

// E = Q^T Q - I (n x n) from the FP32 copy. Every product of two FP32 values is exact as a pair of
// floats; the 32 products of a shared-memory stage are summed in double-float on the FP32 pipe and
// each stage's sum is added in FP64 (one FP64 add per 32 products: GB300's FP64 pipe issues ~64
// times fewer lanes per clock than its FP32 pipe).
// One block per (item, 32 x 32 tile of E); tiles below the diagonal are skipped and mirrored.
__global__ void qrb_gram_kernel(const QrbItem* items, const int* prefix, int nitems) {
  __shared__ float Qi[32][33], Qj[32][33];
  const int t = blockIdx.x;
  const int k = find_item(prefix, nitems, t);
  const QrbItem it = items[k];
  if (it.active && *it.active == 0) return;
  const int nt = (it.n + 31) / 32;
  const int local = t - prefix[k];
  const int ti = local / nt, tj = local % nt;
  if (tj < ti) return;
  const int m = it.m, n = it.n;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads, 4 entries each
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int r0 = 0; r0 < m; r0 += 32) {
    for (int q = threadIdx.x; q < 32 * 32; q += 256) {
      const int rr = q & 31, cc = q >> 5;
      const int r = r0 + rr;
      Qi[cc][rr] = (r < m && ti * 32 + cc < n) ? it.qs[r + (int64_t)(ti * 32 + cc) * m] : 0.f;
      Qj[cc][rr] = (r < m && tj * 32 + cc < n) ? it.qs[r + (int64_t)(tj * 32 + cc) * m] : 0.f;
    }
    __syncthreads();
    float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
    for (int rr = 0; rr < 32; ++rr) {
      const float b = Qj[tx][rr];
#pragma unroll
      for (int u = 0; u < 4; ++u) qrb_dot2_step(Qi[ty + 8 * u][rr], b, hi[u], lo[u]);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] += (double)hi[u] + (double)lo[u];
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = ti * 32 + ty + 8 * u, j = tj * 32 + tx;
    if (i < n && j < n) {
      const double v = acc[u] - (i == j ? 1.0 : 0.0);
      it.e[(int64_t)i * n + j] = v;
      it.e[(int64_t)j * n + i] = v;
    }
  }
}

size_t al(size_t x, size_t a = 1024) { return (x + a - 1) / a * a; }

}  // namespace

// ---------------------------------------------------------------------------

extern "C" int tn_grouped_ops(const tn_batch_op* items, int count, void* ws, size_t ws_bytes, void* stream) {
  if (count <= 0) return TN_OK;
  if (!items) return tn_fail(TN_ERR_ARG, "grouped ops: null table");
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<int> prefix(1, 0);
  for (int i = 0; i < count; ++i) {
    const tn_batch_op& it = items[i];
    if (it.kind < TN_BOP_BLOCK_LEFT || it.kind > TN_BOP_SITE_OPS || it.total < 0 || (it.total > 0 && !it.out))
      return tn_fail(TN_ERR_ARG, "grouped ops: bad item");
    if ((it.kind == TN_BOP_BLOCK_LEFT || it.kind == TN_BOP_BLOCK_RIGHT) && (it.d > MAX_D || it.d < 1))
      return tn_fail(TN_ERR_ARG, "grouped ops: block operators need 1 <= d <= 4");
    prefix.push_back(prefix.back() + (int)tn_cdiv(op_units(it), CHUNK));
  }
  const size_t tb = al(sizeof(tn_batch_op) * (size_t)count), pb = al(sizeof(int) * prefix.size());
  if (!ws || ws_bytes < tb + pb + 1024) return tn_fail(TN_ERR_WORKSPACE, "grouped ops: workspace too small");
  char* base = (char*)al((uintptr_t)ws);
  TN_CUDA(cudaMemcpyAsync(base, items, sizeof(tn_batch_op) * (size_t)count, cudaMemcpyHostToDevice, s));
  TN_CUDA(cudaMemcpyAsync(base + tb, prefix.data(), sizeof(int) * prefix.size(), cudaMemcpyHostToDevice, s));
  if (prefix.back() > 0) {
    grouped_ops_kernel<<<prefix.back(), NT, 0, s>>>((const tn_batch_op*)base, count, (const int*)(base + tb));
    TN_CHECK_LAUNCH();
  }
  return TN_OK;
}

extern "C" size_t tn_grouped_ops_workspace_bytes(int count) {
  return al(sizeof(tn_batch_op) * (size_t)std::max(count, 1)) + al(sizeof(int) * (size_t)(count + 1)) + 2048;
}

namespace {
struct QrbPlan {
  std::vector<QrbItem> items;
  std::vector<int> gram_prefix;
  std::vector<tn_grouped_gemm_problem> fix;
  size_t bytes = 0, tab = 0, scratch = 0;
  int max_smem = 0;
};

int qrb_plan(const tn_qr_item* in, int count, char* base, QrbPlan* P) {
  size_t off = 0;
  P->tab = off;
  off += al(sizeof(QrbItem) * (size_t)count) + al(sizeof(int) * (size_t)(count + 1));
  P->gram_prefix.assign(1, 0);
  // largest factorisations first (m n^2 work each, one CTA per matrix): the long ones start in the
  // first wave and the short ones fill the SMs behind them
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return (int64_t)in[x].m * in[x].n * in[x].n > (int64_t)in[y].m * in[y].n * in[y].n;
  });
  for (int oi = 0; oi < count; ++oi) {
    const tn_qr_item& q = in[order[oi]];
    if (q.n < 1 || q.m < q.n || (int64_t)q.m * q.n > QR_MAX_ELEMS || !q.a || !q.r)
      return tn_fail(TN_ERR_ARG, "batched qr: need 1 <= n <= m and m n <= 32768");
    QrbItem it{};
    it.m = q.m; it.n = q.n;
    it.a = q.a; it.sAm = q.sAm; it.sAn = q.sAn;
    it.r = q.r; it.sRm = q.sRm; it.sRn = q.sRn;
    it.active = q.active;
    it.qs = base ? (float*)(base + off) : nullptr;
    off += al(sizeof(float) * (size_t)q.m * q.n);
    it.e = base ? (double*)(base + off) : nullptr;
    off += al(sizeof(double) * (size_t)q.n * q.n);
    P->items.push_back(it);
    const int nt = (q.n + 31) / 32;
    P->gram_prefix.push_back(P->gram_prefix.back() + nt * nt);
    P->max_smem = std::max(P->max_smem, (int)(sizeof(float) * ((size_t)q.m * q.n + q.n)));
    // Q <- Q - 1/2 Q E: the operands are staged before the product runs, so C may alias A
    tn_grouped_gemm_problem f{};
    f.M = q.m; f.N = q.n; f.K = q.n; f.nred = 1; f.batch = 1;
    f.A = q.a; f.sAm = q.sAm; f.sAk = q.sAn;
    f.B = it.e; f.sBk = q.n; f.sBn = 1;
    f.C = q.a; f.sCm = q.sAm; f.sCn = q.sAn;
    f.alpha = -0.5; f.beta = 1.0; f.accumulate = 0; f.active = q.active;
    P->fix.push_back(f);
  }
  P->scratch = off;
  P->bytes = off + 2048;
  return TN_OK;
}
}  // namespace

size_t tn_grouped_gemm_workspace_bytes(int precision, const tn_grouped_gemm_problem* problems, int count);
int tn_grouped_gemm(int precision, const tn_grouped_gemm_problem* problems, int count, void* ws, size_t ws_bytes,
                    void* stream);

// Sizes only depend on the shapes: plans that are only measured are laid out at this placeholder
// address (the correction GEMM's table needs non-null operand pointers to be planned).
char* const kMeasureBase = (char*)(uintptr_t)(1 << 20);

extern "C" size_t tn_batched_qr_mixed_workspace_bytes(const tn_qr_item* items, int count) {
  if (!items || count <= 0) return 4096;
  QrbPlan P;
  if (qrb_plan(items, count, kMeasureBase, &P)) return 0;
  // the correction GEMM's staging goes behind the plan's own scratch
  return P.bytes + tn_grouped_gemm_workspace_bytes(TN_PREC_TF32X3, P.fix.data(), count) + 2048;
}

extern "C" int tn_batched_qr_mixed(const tn_qr_item* items, int count, void* ws, size_t ws_bytes, void* stream) {
  if (count <= 0) return TN_OK;
  if (!items) return tn_fail(TN_ERR_ARG, "batched qr: null table");
  if (!tn_tf32x3_supported()) return tn_fail(TN_ERR_ARG, "batched qr: needs an sm_103 device (split-TF32 correction)");
  cudaStream_t s = (cudaStream_t)stream;
  QrbPlan M0;
  int st = qrb_plan(items, count, kMeasureBase, &M0);
  if (st) return st;
  const size_t gg = tn_grouped_gemm_workspace_bytes(TN_PREC_TF32X3, M0.fix.data(), count);
  if (!ws || ws_bytes < M0.bytes + gg + 2048) return tn_fail(TN_ERR_WORKSPACE, "batched qr: workspace too small");
  char* base = (char*)al((uintptr_t)ws);
  QrbPlan P;
  if ((st = qrb_plan(items, count, base, &P))) return st;
  QrbItem* d_items = (QrbItem*)(base + P.tab);
  int* d_gp = (int*)(base + P.tab + al(sizeof(QrbItem) * (size_t)count));
  TN_CUDA(cudaMemcpyAsync(d_items, P.items.data(), sizeof(QrbItem) * (size_t)count, cudaMemcpyHostToDevice, s));
  TN_CUDA(cudaMemcpyAsync(d_gp, P.gram_prefix.data(), sizeof(int) * P.gram_prefix.size(), cudaMemcpyHostToDevice, s));
  if ((st = tn_set_smem_attr_once(TN_ATTR_BATCH_QR, (const void*)qrb_householder_kernel,
                                  (int)(sizeof(float) * (QR_MAX_ELEMS + 512)))))
    return st;
  qrb_householder_kernel<<<count, QR_NT, P.max_smem, s>>>(d_items);
  TN_CHECK_LAUNCH();
  qrb_gram_kernel<<<P.gram_prefix.back(), 256, 0, s>>>(d_items, d_gp, count);
  TN_CHECK_LAUNCH();
  char* gws = base + al(P.bytes);
  return tn_grouped_gemm(TN_PREC_TF32X3, P.fix.data(), count, gws, ws_bytes - (size_t)(gws - (char*)ws), stream);
}
