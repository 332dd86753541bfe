// Mixed-precision gauge move: FP32 Householder QR + FP64 re-orthogonalisation (split-TF32 path).
//
// On GB300 a dependent FP64 operation costs ~64 cycles and the FP64 pipe issues ~2 lanes/clock
// per SM, which makes the column-sequential Householder panel the bottleneck of an FP64 QR.
// In a sweep the R factor of a gauge move only seeds the next local solve (the site it is
// absorbed into is re-optimised right away), so only Q has to be accurate:
//   1. Householder QR of the FP64 input scaled by a power of two (exact; any finite FP64 input fits
//      FP32) and rounded to FP32: Q32 with ||Q32^T Q32 - I|| ~ 1e-6 whatever the conditioning of
//      the input, R32 accurate to FP32 and scaled back. For n <= m <= 1024,
//      n <= 512 the whole factorisation runs in one 16-CTA cluster kernel (qr_cluster.cu);
//      otherwise one-CTA FP32 panels with FP32 GEMM trailing updates, Q formed backwards;
//   2. E = Q^T Q - I to double-float accuracy on the FP32 pipe (Q32's entries are FP32 values, so
//      every product is exact as a pair of floats), then Q <- Q - Q E / 2 on the tensor cores
//      (split TF32; the product is ~1e-6 in size, so its 1e-6 relative error is ~1e-12): the
//      returned Q is orthonormal to ~1e-12 and spans col(A) to FP32 accuracy.
// Used by tn_qr_mixed; the plain FP64 path keeps tn_qr.
#include "common.cuh"

int tn_gemm_tf32x3(const TnGemmF64& g, void* ws, size_t ws_bytes, cudaStream_t s);
size_t tn_gemm_tf32x3_ws_bytes(int64_t M, int64_t N, int64_t K, int64_t batch, int64_t nred);
bool tn_qr32_cluster_supported(int64_t m, int64_t n);
size_t tn_qr32_cluster_scratch_floats(int64_t m, int64_t n);
int tn_qr32_cluster(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn, double* q, double* r,
                    int64_t sRm, int64_t sRn, float* scratch, cudaStream_t s);

namespace {

constexpr int NB = 16;
constexpr int NTP = 512;

struct G32 {
  int64_t M, N, K;
  const float* A; int64_t sAm, sAk;
  const float* B; int64_t sBk, sBn;
  float* C; int64_t sCm, sCn;
  float alpha, beta;
};

// FP32 SIMT GEMM, 64x64 tiles, 256 threads with 4x4 micro-tiles, general strides.
constexpr int TM = 64, TN = 64, TK = 16, T32 = 256;

__global__ void __launch_bounds__(T32) gemm32_kernel(G32 g) {
  __shared__ float As[TK][TM + 4];
  __shared__ float Bs[TK][TN + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t m0 = (int64_t)blockIdx.y * TM, n0 = (int64_t)blockIdx.x * TN;
  const bool a_kc = (g.sAk == 1), b_nc = (g.sBn == 1);
  float acc[4][4] = {};
  for (int64_t k0 = 0; k0 < g.K; k0 += TK) {
    for (int e = tid; e < TM * TK; e += T32) {
      int mm, kk;
      if (a_kc) { mm = e / TK; kk = e % TK; } else { kk = e / TM; mm = e % TM; }
      const int64_t gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < g.M && gk < g.K) ? g.A[gm * g.sAm + gk * g.sAk] : 0.f;
    }
    for (int e = tid; e < TN * TK; e += T32) {
      int nn, kk;
      if (b_nc) { kk = e / TN; nn = e % TN; } else { nn = e / TK; kk = e % TK; }
      const int64_t gn = n0 + nn, gk = k0 + kk;
      Bs[kk][nn] = (gn < g.N && gk < g.K) ? g.B[gk * g.sBk + gn * g.sBn] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) { a[i] = As[kk][ty * 4 + i]; b[i] = Bs[kk][tx * 4 + i]; }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
      if (gm < g.M && gn < g.N) {
        float* c = g.C + gm * g.sCm + gn * g.sCn;
        const float v = g.alpha * acc[i][j];
        *c = (g.beta == 0.f) ? v : fmaf(g.beta, *c, v);
      }
    }
}

int gemm32(const G32& g, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0) return TN_OK;
  dim3 grid((unsigned)tn_cdiv(g.N, TN), (unsigned)tn_cdiv(g.M, TM));
  gemm32_kernel<<<grid, T32, 0, s>>>(g);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

// max |a| as the bits of a non-negative double (ordered like the values), into *amax (zeroed)
__global__ void amax_kernel(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn,
                            unsigned long long* amax) {
  double mx = 0.0;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < m * n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = idx / m, i = idx % m;
    mx = fmax(mx, fabs(a[i * sAm + j * sAn]));
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(amax, (unsigned long long)__double_as_longlong(mx));
}

// exponent of the power of two that brings max |a| to [1, 2) (0 for a zero or non-finite max)
__device__ __forceinline__ int scale_exponent(const unsigned long long* amax) {
  const double mx = __longlong_as_double((long long)*amax);
  return (mx > 0.0 && isfinite(mx)) ? ilogb(mx) : 0;
}

// FP64 -> FP32 copy scaled by an exact power of two, so any finite FP64 input fits FP32
__global__ void copy_in32(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn, float* Aw,
                          const unsigned long long* amax) {
  const double down = ldexp(1.0, -scale_exponent(amax));
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < m * n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = idx / m, i = idx % m;
    Aw[idx] = (float)(a[i * sAm + j * sAn] * down);
  }
}

__global__ void init_q32(int64_t m, int64_t k, float* Qw, float* Vf) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < m * k;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = idx / m, i = idx % m;
    Qw[idx] = (i == j) ? 1.f : 0.f;
    Vf[idx] = 0.f;
  }
}

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// FP32 Householder panel, one CTA (LAPACK sign convention), forward compact-WY T.
__global__ void __launch_bounds__(NTP) panel32(int64_t m, int64_t j0, int jb, float* Aw, float* Vf, float* T) {
  __shared__ float red[NTP / 32][NB];
  __shared__ float vals[NB];
  __shared__ float sc[3];
  __shared__ float Ts[NB][NB];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int i = tid; i < NB * NB; i += NTP) Ts[i / NB][i % NB] = 0.f;
  __syncthreads();
  for (int c = 0; c < jb; ++c) {
    const int64_t j = j0 + c;
    float* x = Aw + j * m;
    float p = 0.f;
    for (int64_t i = j + 1 + tid; i < m; i += NTP) p = fmaf(x[i], x[i], p);
    p = warp_sumf(p);
    if (lane == 0) red[wid][0] = p;
    __syncthreads();
    if (tid == 0) {
      float sigma = 0.f;
      for (int w = 0; w < NTP / 32; ++w) sigma += red[w][0];
      const float alpha = x[j];
      float tau = 0.f, beta = alpha, scale = 0.f;
      if (sigma > kHhTiny) {  // smaller sub-columns are taken as zero (see kHhTiny)
        const float nrm = sqrtf(alpha * alpha + sigma);
        beta = alpha >= 0.f ? -nrm : nrm;
        tau = (beta - alpha) / beta;
        scale = 1.f / (alpha - beta);
      }
      sc[0] = tau; sc[1] = beta; sc[2] = scale;
    }
    __syncthreads();
    const float tau = sc[0], scale = sc[2];
    float* v = Vf + j * m;
    for (int64_t i = j + tid; i < m; i += NTP) {
      if (i == j) { v[i] = 1.f; x[i] = sc[1]; }
      else { const float vi = x[i] * scale; v[i] = vi; x[i] = 0.f; }
    }
    __syncthreads();
    const int nr = jb - c - 1;
    float acc[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) acc[q] = 0.f;
    for (int64_t i = j + tid; i < m; i += NTP) {
      const float vi = v[i];
#pragma unroll
      for (int q = 0; q < NB; ++q) {
        if (q < nr) acc[q] = fmaf(vi, Aw[(j + 1 + q) * m + i], acc[q]);
        else if (q - nr < c) acc[q] = fmaf(vi, Vf[(j0 + (q - nr)) * m + i], acc[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const float s = warp_sumf(acc[q]);
      if (lane == 0) red[wid][q] = s;
    }
    __syncthreads();
    if (tid < nr + c) {
      float s = 0.f;
      for (int w = 0; w < NTP / 32; ++w) s += red[w][tid];
      vals[tid] = s;
    }
    __syncthreads();
    for (int64_t i = j + tid; i < m; i += NTP) {
      const float vi = v[i];
      for (int q = 0; q < nr; ++q) Aw[(j + 1 + q) * m + i] -= tau * vals[q] * vi;
    }
    if (tid < c) {  // T(0:c, c) = -tau T(0:c, 0:c) (V(:,0:c)^T v), one thread per row
      float t = 0.f;
      for (int q = tid; q < c; ++q) t = fmaf(Ts[tid][q], -tau * vals[nr + q], t);
      Ts[tid][c] = t;
    }
    if (tid == 0) Ts[c][c] = tau;
    __syncthreads();
  }
  for (int i = tid; i < NB * NB; i += NTP) T[i] = Ts[i / NB][i % NB];
}

__global__ void extract_mixed(int64_t m, int64_t n, int64_t k, const float* Aw, const float* Qw, double* Q64,
                              double* r, int64_t sRm, int64_t sRn, const unsigned long long* amax) {
  const double up = ldexp(1.0, scale_exponent(amax));
  const int64_t tq = m * k, tr = k * n;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < tq + tr;
       idx += (int64_t)gridDim.x * blockDim.x) {
    if (idx < tq) {
      Q64[idx] = (double)Qw[idx];  // column-major m x k
    } else {
      const int64_t e = idx - tq;
      const int64_t c = e / k, rr = e % k;
      if (r) r[rr * sRm + c * sRn] = (c >= rr) ? (double)Aw[c * m + rr] * up : 0.0;
    }
  }
}

// E = Q^T Q - I for a Q whose entries are FP32 values (column-major m x k, held in FP64), exact
// to double-float accuracy on the FP32 pipe: each product a*b is split error-free into
// h + fma(a, b, -h) (TwoProduct), the h are summed error-free (Knuth's TwoSum) into a running
// FP32 head and all low-order parts into an FP32 tail (the compensated dot product "Dot2" of
// Ogita, Rump and Oishi, SIAM J. Sci. Comput. 26 (2005)); every CTA sums at most GRAM_ROWS rows
// of one 64 x 64 tile on or above the diagonal, so the tail's own rounding stays ~1e-16 for
// columns of unit norm. Ten FP32 operations per product against one FP64 FMA: the FP64 pipe
// issues 64 times fewer lanes per clock on this part.
constexpr int GT = 64;          // output tile edge
constexpr int GK = 32;          // rows per shared-memory stage
constexpr int GRAM_ROWS = 128;  // rows summed per CTA (the split of the row range)
constexpr int GNT = 256;

// (the _rn intrinsics are never contracted into FMAs, which would break both transformations)
__device__ __forceinline__ void dot2_step(float a, float b, float& hi, float& lo) {
  const float h = __fmul_rn(a, b);
  const float r = fmaf(a, b, -h);
  const float t = __fadd_rn(hi, h);
  const float z = __fsub_rn(t, hi);
  const float q = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, z)), __fsub_rn(h, z));
  hi = t;
  lo = __fadd_rn(lo, __fadd_rn(q, r));
}

__device__ __forceinline__ int gram_tile_id(int ib, int jb, int nt) { return ib * nt - ib * (ib - 1) / 2 + (jb - ib); }

// part[(tile * nsplit + split) * GT * GT + li * GT + lj] = sum over the split's rows of
// Q(r, 64 ib + li) Q(r, 64 jb + lj) for every tile jb >= ib (grid: tiles x splits). Thread (ti, tj)
// owns rows ti + 16 a and columns tj + 16 b of the tile (a, b < 4), so both shared-memory reads of a
// stage step are conflict-free.
__global__ void __launch_bounds__(GNT) gram_dot2_kernel(int64_t m, int64_t k, const double* __restrict__ Q,
                                                        int nsplit, double* __restrict__ part) {
  __shared__ float As[GK][GT + 1], Bs[GK][GT + 1];
  const int nt = (int)tn_cdiv(k, GT);
  int tile = blockIdx.x, ib = 0;
  while (tile >= nt - ib) {
    tile -= nt - ib;
    ++ib;
  }
  const int jb = ib + tile;
  const int64_t r_begin = (int64_t)blockIdx.y * GRAM_ROWS, r_end = min(m, r_begin + GRAM_ROWS);
  const int t = threadIdx.x, ti = t >> 4, tj = t & 15;
  float hi[4][4], lo[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) hi[a][b] = lo[a][b] = 0.f;
  for (int64_t r0 = r_begin; r0 < r_end; r0 += GK) {
    for (int e = t; e < GK * GT; e += GNT) {
      const int c = e / GK, rr = e % GK;  // a warp reads 32 consecutive rows of one column
      const int64_t r = r0 + rr, ca = (int64_t)ib * GT + c, cb = (int64_t)jb * GT + c;
      As[rr][c] = (r < r_end && ca < k) ? (float)Q[r + ca * m] : 0.f;
      Bs[rr][c] = (r < r_end && cb < k) ? (float)Q[r + cb * m] : 0.f;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < GK; ++kk) {
      float av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) av[a] = As[kk][ti + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) bv[b] = Bs[kk][tj + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) dot2_step(av[a], bv[b], hi[a][b], lo[a][b]);
    }
    __syncthreads();
  }
  double* out = part + ((size_t)gram_tile_id(ib, jb, nt) * nsplit + blockIdx.y) * GT * GT;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) out[(ti + 16 * a) * GT + tj + 16 * b] = (double)hi[a][b] + (double)lo[a][b];
}

// E (k x k, row-major) = sum of the splits' partial Gram tiles (mirrored below the diagonal) - I
__global__ void gram_finish_kernel(int64_t k, int nsplit, const double* __restrict__ part, double* __restrict__ E) {
  const int nt = (int)tn_cdiv(k, GT);
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < k * k;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = idx / k, j = idx % k;
    if (i / GT > j / GT) {
      const int64_t x = i;
      i = j;
      j = x;
    }
    const int ib = (int)(i / GT), jb = (int)(j / GT);
    const double* p = part + (size_t)gram_tile_id(ib, jb, nt) * nsplit * GT * GT + (i % GT) * GT + (j % GT);
    double s = 0.0;
    for (int sp = 0; sp < nsplit; ++sp) s += p[(size_t)sp * GT * GT];
    E[idx] = s - ((idx / k == idx % k) ? 1.0 : 0.0);
  }
}

// out(i, j) (strided) = Q(i, j) - Qc(i, j): Q, Qc column-major m x k
__global__ void write_q(int64_t m, int64_t k, const double* Q64, const double* QE, double* q, int64_t sQm,
                        int64_t sQn) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < m * k;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = idx / m, i = idx % m;
    q[i * sQm + j * sQn] = Q64[idx] - 0.5 * QE[idx];
  }
}

int blocks_for(int64_t total) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(total, 256), 8LL * tn_sm_count()));
}

size_t al(size_t x) { return (x + 1023) / 1024 * 1024; }

struct MixWs {
  float *Aw, *Vf, *Qw, *T, *W, *W2, *Vc;
  double *Q64, *E, *QE;
  unsigned long long* amax;
  char* tf_ws;
  size_t tf_bytes;
  double* gram;  // partial Gram tiles of the re-orthogonalisation
};

size_t mix_layout(int64_t m, int64_t n, char* base, MixWs* w) {
  const int64_t k = std::min(m, n), np = tn_cdiv(k, NB);
  size_t off = 0;
  auto take = [&](size_t b) { char* p = base ? base + off : nullptr; off += al(b); return p; };
  w->Aw = (float*)take((size_t)m * n * 4);
  w->Vf = (float*)take((size_t)m * k * 4);
  w->Qw = (float*)take((size_t)m * k * 4);
  w->T = (float*)take((size_t)np * NB * NB * 4);
  w->W = (float*)take((size_t)NB * std::max(n, k) * 4);
  w->W2 = (float*)take((size_t)NB * std::max(n, k) * 4);
  w->Vc = (float*)take(tn_qr32_cluster_scratch_floats(m, k) * 4);
  w->Q64 = (double*)take((size_t)m * k * 8);
  w->amax = (unsigned long long*)take(sizeof(unsigned long long));
  w->E = (double*)take((size_t)k * k * 8);
  w->QE = (double*)take((size_t)m * k * 8);
  w->tf_bytes = tn_gemm_tf32x3_ws_bytes(m, k, k, 1, 1);
  w->tf_ws = take(w->tf_bytes);
  {
    const int64_t nt = tn_cdiv(k, GT), nsplit = tn_cdiv(m, GRAM_ROWS);
    w->gram = (double*)take((size_t)(nt * (nt + 1) / 2) * nsplit * GT * GT * 8);
  }
  return off + 1024;
}

int qr32_blocked(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn, double* r, int64_t sRm,
                 int64_t sRn, const MixWs& w, cudaStream_t s);
int refine_q(int64_t m, int64_t k, double* q, int64_t sQm, int64_t sQn, const MixWs& w, cudaStream_t s);

}  // namespace

extern "C" size_t tn_qr_mixed_workspace_bytes(int64_t m, int64_t n) {
  if (m <= 0 || n <= 0) return 0;
  MixWs w;
  return mix_layout(m, n, nullptr, &w);
}

extern "C" int tn_qr_mixed(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn, double* q, int64_t sQm,
                           int64_t sQn, double* r, int64_t sRm, int64_t sRn, void* ws, size_t ws_bytes,
                           void* stream) {
  if (m <= 0 || n <= 0 || !a || !q) return tn_fail(TN_ERR_ARG, "qr_mixed: bad arguments");
  MixWs w;
  if (!ws || ws_bytes < mix_layout(m, n, nullptr, &w)) return tn_fail(TN_ERR_WORKSPACE, "qr_mixed: workspace");
  char* base = (char*)(((uintptr_t)ws + 1023) & ~(uintptr_t)1023);
  mix_layout(m, n, base, &w);
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t ev = tn_profile_begin(s);
  const int64_t k = std::min(m, n), np = tn_cdiv(k, NB);
  int st;
  if (m >= n && tn_qr32_cluster_supported(m, n)) {
    // whole FP32 factorisation and Q formation in one cluster-resident kernel
    if ((st = tn_qr32_cluster(m, n, a, sAm, sAn, w.Q64, r, sRm, sRn, w.Vc, s))) return st;
  } else {
    if ((st = qr32_blocked(m, n, a, sAm, sAn, r, sRm, sRn, w, s))) return st;
  }
  if ((st = refine_q(m, k, q, sQm, sQn, w, s))) return st;
  // algorithmic work of the factorisation, 2mn^2 - 2n^3/3 (for m >= n; forming Q is not counted)
  tn_profile_end(ev, s, TN_PROF_QR, 2.0 * m * k * (double)k - 2.0 / 3.0 * k * k * (double)k);
  return TN_OK;
}

namespace {

// FP32 blocked Householder QR on global memory (one-CTA panels + FP32 GEMM updates): Q64, R.
int qr32_blocked(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn, double* r, int64_t sRm,
                 int64_t sRn, const MixWs& w, cudaStream_t s) {
  const int64_t k = std::min(m, n), np = tn_cdiv(k, NB);
  TN_CUDA(cudaMemsetAsync(w.amax, 0, sizeof(unsigned long long), s));
  amax_kernel<<<blocks_for(m * n), 256, 0, s>>>(m, n, a, sAm, sAn, w.amax);
  TN_CHECK_LAUNCH();
  copy_in32<<<blocks_for(m * n), 256, 0, s>>>(m, n, a, sAm, sAn, w.Aw, w.amax);
  TN_CHECK_LAUNCH();
  init_q32<<<blocks_for(m * k), 256, 0, s>>>(m, k, w.Qw, w.Vf);
  TN_CHECK_LAUNCH();
  int st;
  for (int64_t p = 0; p < np; ++p) {
    const int64_t j0 = p * NB;
    const int jb = (int)std::min<int64_t>(NB, k - j0);
    float* Tp = w.T + p * NB * NB;
    panel32<<<1, NTP, 0, s>>>(m, j0, jb, w.Aw, w.Vf, Tp);
    TN_CHECK_LAUNCH();
    const int64_t nc = n - j0 - jb, mr = m - j0;
    if (nc <= 0) continue;
    // W = V^T C ; W2 = T^T W ; C -= V W2
    if ((st = gemm32({jb, nc, mr, w.Vf + j0 + j0 * m, m, 1, w.Aw + j0 + (j0 + jb) * m, 1, m, w.W, nc, 1, 1.f, 0.f}, s)))
      return st;
    if ((st = gemm32({jb, nc, jb, Tp, 1, NB, w.W, nc, 1, w.W2, nc, 1, 1.f, 0.f}, s))) return st;
    if ((st = gemm32({mr, nc, jb, w.Vf + j0 + j0 * m, 1, m, w.W2, nc, 1, w.Aw + j0 + (j0 + jb) * m, 1, m, -1.f, 1.f},
                     s)))
      return st;
  }
  for (int64_t p = np - 1; p >= 0; --p) {
    const int64_t j0 = p * NB;
    const int jb = (int)std::min<int64_t>(NB, k - j0);
    const int64_t nc = k - j0, mr = m - j0;
    float* Tp = w.T + p * NB * NB;
    if ((st = gemm32({jb, nc, mr, w.Vf + j0 + j0 * m, m, 1, w.Qw + j0 + j0 * m, 1, m, w.W, nc, 1, 1.f, 0.f}, s)))
      return st;
    if ((st = gemm32({jb, nc, jb, Tp, NB, 1, w.W, nc, 1, w.W2, nc, 1, 1.f, 0.f}, s))) return st;
    if ((st = gemm32({mr, nc, jb, w.Vf + j0 + j0 * m, 1, m, w.W2, nc, 1, w.Qw + j0 + j0 * m, 1, m, -1.f, 1.f}, s)))
      return st;
  }
  extract_mixed<<<blocks_for(m * k + k * n), 256, 0, s>>>(m, n, k, w.Aw, w.Qw, w.Q64, r, sRm, sRn, w.amax);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

// FP64 re-orthogonalisation of Q64 (column-major m x k, FP32-accurate) into q (strided).
int refine_q(int64_t m, int64_t k, double* q, int64_t sQm, int64_t sQn, const MixWs& w, cudaStream_t s) {
  int st;
  // E = Q^T Q - I, double-float exact on the FP32 pipe (Q64 holds FP32 values)
  {
    const int nt = (int)tn_cdiv(k, GT), nsplit = (int)tn_cdiv(m, GRAM_ROWS);
    gram_dot2_kernel<<<dim3((unsigned)(nt * (nt + 1) / 2), (unsigned)nsplit), GNT, 0, s>>>(m, k, w.Q64, nsplit,
                                                                                          w.gram);
    TN_CHECK_LAUNCH();
    gram_finish_kernel<<<blocks_for(k * k), 256, 0, s>>>(k, nsplit, w.gram, w.E);
    TN_CHECK_LAUNCH();
  }
  // QE = Q E on the tensor cores (split TF32), then q = Q - QE / 2
  TnGemmF64 h{};
  h.M = m; h.N = k; h.K = k;
  h.A = w.Q64; h.sAm = 1; h.sAk = m;
  h.B = w.E; h.sBk = k; h.sBn = 1;
  h.C = w.QE; h.sCm = 1; h.sCn = m;
  h.batch = 1; h.nred = 1; h.alpha = 1.0; h.beta = 0.0;
  if ((st = tn_gemm_tf32x3(h, w.tf_ws, w.tf_bytes, s))) return st;
  write_q<<<blocks_for(m * k), 256, 0, s>>>(m, k, w.Q64, w.QE, q, sQm, sQn);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

}  // namespace
