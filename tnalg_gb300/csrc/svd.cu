// One-sided (Hestenes) Jacobi singular values in FP64 (K5).
//
// Replaces the np.linalg.svd of decompose(..., way='svd') used by
// calculate_entanglement_spectrum (MPSClass.py:812-832,
// TensorBasicModule.py:338-342,374-377): the Schmidt values of a bond are the
// singular values of the R factor of the centre tensor.
//
// Rows of X are rotated pairwise until mutually orthogonal; the row norms are
// the singular values. Pairs follow a round-robin tournament, so each round is
// k/2 independent pairs (one CTA each); a sweep is k-1 rounds. The host reads a
// single "rotated" flag per sweep and stops when a sweep rotates nothing.
#include <math.h>

#include "common.cuh"

namespace {

constexpr int NT = 256;

__global__ void svd_copy_in(int64_t k, int64_t kp, int64_t n, const double* x, int64_t sr, int64_t sc, double* X) {
  const int64_t total = kp * n;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx / n, c = idx % n;
    X[idx] = r < k ? x[r * sr + c * sc] : 0.0;
  }
}

// Round-robin pairing: player 0 fixed, others rotate. Round r pairs slot i with slot kp-1-i.
__device__ __forceinline__ int64_t rr_player(int64_t slot, int64_t r, int64_t kp) {
  if (slot == 0) return 0;
  return 1 + (slot - 1 + r) % (kp - 1);
}

__global__ void jacobi_round(int64_t kp, int64_t n, int64_t r, double* X, double tol, int* rotated) {
  const int64_t i = blockIdx.x;  // pair index 0..kp/2-1
  const int64_t p = rr_player(i, r, kp), q = rr_player(kp - 1 - i, r, kp);
  double* xp = X + p * n;
  double* xq = X + q * n;
  double a = 0.0, b = 0.0, g = 0.0;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) {
    const double u = xp[t], v = xq[t];
    a = fma(u, u, a);
    b = fma(v, v, b);
    g = fma(u, v, g);
  }
  __shared__ double red[3][NT / 32];
  __shared__ double cs[2];
  a = tn_warp_sum(a);
  b = tn_warp_sum(b);
  g = tn_warp_sum(g);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { red[0][wid] = a; red[1][wid] = b; red[2][wid] = g; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double A = 0, B = 0, G = 0;
    for (int w = 0; w < NT / 32; ++w) { A += red[0][w]; B += red[1][w]; G += red[2][w]; }
    double c = 1.0, s = 0.0;
    if (fabs(G) > tol * sqrt(A * B) && G != 0.0) {
      const double zeta = (B - A) / (2.0 * G);
      const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
      c = 1.0 / sqrt(1.0 + t * t);
      s = c * t;
      *rotated = 1;
    }
    cs[0] = c; cs[1] = s;
  }
  __syncthreads();
  const double c = cs[0], s = cs[1];
  if (s == 0.0) return;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) {
    const double u = xp[t], v = xq[t];
    xp[t] = c * u - s * v;
    xq[t] = s * u + c * v;
  }
}

__global__ void row_norms(int64_t k, int64_t n, const double* X, double* out) {
  const int64_t r = blockIdx.x;
  if (r >= k) return;
  double a = 0.0;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) a = fma(X[r * n + t], X[r * n + t], a);
  __shared__ double red[NT / 32];
  a = tn_warp_sum(a);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double A = 0;
    for (int w = 0; w < NT / 32; ++w) A += red[w];
    out[r] = sqrt(A);
  }
}

}  // namespace

extern "C" size_t tn_singular_values_workspace_bytes(int64_t k, int64_t n) {
  const int64_t kp = k + (k & 1);
  return (size_t)kp * n * sizeof(double) + 512;
}

extern "C" int tn_singular_values(int64_t k, int64_t n, const double* x, int64_t sXr, int64_t sXc, double* s_out,
                                  double tol, int max_sweeps, void* ws, size_t ws_bytes, void* stream) {
  if (k <= 0 || n <= 0 || !x || !s_out) return tn_fail(TN_ERR_ARG, "singular_values: bad args");
  const int64_t kp = k + (k & 1);
  if (!ws || ws_bytes < tn_singular_values_workspace_bytes(k, n))
    return tn_fail(TN_ERR_WORKSPACE, "singular_values: workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  int* flag = (int*)ws;
  double* X = (double*)((char*)ws + 256);
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(kp * n, NT), 8LL * tn_sm_count()));
  svd_copy_in<<<blocks, NT, 0, s>>>(k, kp, n, x, sXr, sXc, X);
  TN_CHECK_LAUNCH();
  if (kp >= 2) {
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
      TN_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
      for (int64_t r = 0; r < kp - 1; ++r) {
        jacobi_round<<<(unsigned)(kp / 2), NT, 0, s>>>(kp, n, r, X, tol, flag);
        TN_CHECK_LAUNCH();
      }
      int h = 0;
      TN_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
      TN_CUDA(cudaStreamSynchronize(s));
      if (!h) break;
    }
  }
  row_norms<<<(unsigned)k, NT, 0, s>>>(k, n, X, s_out);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant. Some hosts cannot allocate device memory themselves: a Go or JVM
// service that may only use buffers registered by its own allocator, or a process whose device
// memory is held entirely by another framework's caching allocator. They can still compute an
// entanglement spectrum with tn_singular_values_noalloc, whose scratch (the rotated copy of X and
// the "rotated" flag) lives in this static device array instead of a caller workspace.
//
// Limit: (k rounded up to even) * n <= TN_SV_NOALLOC_MAX_ELEMS doubles (512 KiB; e.g. 256 x 256).
// Every GPU that loads the library holds the array until the process exits. All calls share it:
// calls that overlap on the GPU (different streams, or different host threads on one device) race
// and must be serialised by the caller. The flag is cleared at the start of every sweep; the copy
// of X is rewritten by every call, so no state leaks from one call into the next.
#define TN_SV_NOALLOC_MAX_ELEMS 65536
#define TN_SV_NOALLOC_FLAG_SLOTS 32
static __device__ __align__(256) double g_sv_noalloc_scratch[TN_SV_NOALLOC_FLAG_SLOTS + TN_SV_NOALLOC_MAX_ELEMS];

namespace {
constexpr int kMaxDevices = 64;
void* g_sv_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of the static scratch on the current device, resolved once per device.
int sv_noalloc_scratch(void** out) {
  int dev = 0;
  TN_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return tn_fail(TN_ERR_ARG, "singular_values_noalloc: device ordinal >= 64");
  if (!g_sv_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_sv_noalloc_scratch);
    if (e != cudaSuccess) return tn_record_error(e);
    g_sv_noalloc_ptr[dev] = p;
  }
  *out = g_sv_noalloc_ptr[dev];
  return TN_OK;
}
}  // namespace

extern "C" int tn_singular_values_noalloc(int64_t k, int64_t n, const double* x, int64_t sXr, int64_t sXc,
                                          double* s_out, double tol, int max_sweeps, void* stream) {
  if (k <= 0 || n <= 0 || !x || !s_out) return tn_fail(TN_ERR_ARG, "singular_values_noalloc: bad args");
  const int64_t kp = k + (k & 1);
  if (kp > TN_SV_NOALLOC_MAX_ELEMS / n || kp * n > TN_SV_NOALLOC_MAX_ELEMS)
    return tn_fail(TN_ERR_ARG,
                   "singular_values_noalloc: (k rounded up to even) * n exceeds the 65536-element static scratch");
  void* base = nullptr;
  int st = sv_noalloc_scratch(&base);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  int* flag = (int*)base;
  double* X = (double*)base + TN_SV_NOALLOC_FLAG_SLOTS;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(kp * n, NT), 8LL * tn_sm_count()));
  svd_copy_in<<<blocks, NT, 0, s>>>(k, kp, n, x, sXr, sXc, X);
  TN_CHECK_LAUNCH();
  if (kp >= 2) {
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
      TN_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
      for (int64_t r = 0; r < kp - 1; ++r) {
        jacobi_round<<<(unsigned)(kp / 2), NT, 0, s>>>(kp, n, r, X, tol, flag);
        TN_CHECK_LAUNCH();
      }
      int h = 0;
      TN_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
      TN_CUDA(cudaStreamSynchronize(s));
      if (!h) break;
    }
  }
  row_norms<<<(unsigned)k, NT, 0, s>>>(k, n, X, s_out);
  TN_CHECK_LAUNCH();
  return TN_OK;
}
