// One-sided (Hestenes) Jacobi singular values in FP64 (entanglement spectrum).
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
// A pair is left alone when its off-diagonal is below tol relative to the rows, or when one
// of its rows is numerically null (squared norm below (4 eps)^2 max(k, n) ||X||_F^2): rounding
// noise keeps such rows from ever becoming orthogonal, and their norms are noise-level singular
// values either way (LAPACK's are accurate to ~eps ||X|| too). A row that is small but above the
// null level (squared norm below (64 eps)^2 k n ||X||_F^2, e.g. a direction left over from the
// cancellation of two large rows) still rotates, but its rotations do not count as "rotated": its
// dot products carry the rounding of the large rows it came from (relative error up to
// eps ||X|| / ||row||), so they may never fall below tol, and would otherwise keep every sweep
// going until max_sweeps. Its singular value is then accurate to ~eps ||X||, LAPACK's accuracy.
// A sweep that still rotated after max_sweeps makes the call return TN_ERR_NOCONV (the values are
// written all the same).
#include <math.h>

#include <vector>

#include <mutex>

#include "common.cuh"

namespace {

constexpr int NT = 256;

// Squared norm below which a row counts as numerically null, relative to ||X||_F^2.
inline double null_row_rel2(int64_t k, int64_t n) {
  const double e = 4.0 * 2.220446049250313e-16;
  return e * e * (double)std::max<int64_t>(k, n);
}

// X = x (rows padded to kp with zeros); *fro2 += ||x||_F^2 (*fro2 zeroed by the caller).
__global__ void svd_copy_in(int64_t k, int64_t kp, int64_t n, const double* x, int64_t sr, int64_t sc, double* X,
                            double* fro2) {
  const int64_t total = kp * n;
  double acc = 0.0;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx / n, c = idx % n;
    const double v = r < k ? x[r * sr + c * sc] : 0.0;
    X[idx] = v;
    acc = fma(v, v, acc);
  }
  acc = tn_warp_sum(acc);
  if ((threadIdx.x & 31) == 0 && acc != 0.0) atomicAdd(fro2, acc);
}

// Round-robin pairing: player 0 fixed, others rotate. Round r pairs slot i with slot kp-1-i.
__device__ __forceinline__ int64_t rr_player(int64_t slot, int64_t r, int64_t kp) {
  if (slot == 0) return 0;
  return 1 + (slot - 1 + r) % (kp - 1);
}

// Pair i of round r, by the whole block: J, the accumulated rotations (kp x kp, row-major), is
// rotated with X's rows when not null.
__device__ __forceinline__ void jacobi_pair(int64_t kp, int64_t n, int64_t i, int64_t r, double* X, double tol,
                                            const double* fro2, double null_rel2, int* rotated, double* J) {
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
    const double f2 = *fro2;
    if (G != 0.0 && fabs(G) > tol * sqrt(A * B) && fmin(A, B) > null_rel2 * f2) {
      const double zeta = (B - A) / (2.0 * G);
      const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
      c = 1.0 / sqrt(1.0 + t * t);
      s = c * t;
      // rows below the "small" level rotate without holding up convergence (see the top)
      if (s != 0.0 && fmin(A, B) > null_rel2 * 256.0 * (double)min(kp, n) * f2) *rotated = 1;
    }
    cs[0] = c; cs[1] = s;
  }
  __syncthreads();
  const double c = cs[0], s = cs[1];
  // every thread has read cs: the next pair of this block may overwrite it
  __syncthreads();
  if (s == 0.0) return;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) {
    const double u = xp[t], v = xq[t];
    xp[t] = c * u - s * v;
    xq[t] = s * u + c * v;
  }
  if (J) {
    double* jp = J + p * kp;
    double* jq = J + q * kp;
    for (int64_t t = threadIdx.x; t < kp; t += blockDim.x) {
      const double u = jp[t], v = jq[t];
      jp[t] = c * u - s * v;
      jq[t] = s * u + c * v;
    }
  }
}

__global__ void jacobi_round(int64_t kp, int64_t n, int64_t r, double* X, double tol, const double* fro2,
                             double null_rel2, int* rotated, double* J = nullptr) {
  jacobi_pair(kp, n, blockIdx.x, r, X, tol, fro2, null_rel2, rotated, J);
}

constexpr long long kBarrierCycles = 4000000000LL;  // ~2 s at 2 GHz

// Grid-wide barrier of a cooperative launch (every block is resident): an arrival count and a
// generation word in global memory (bar[0], bar[1]). The last block to arrive resets the count and
// advances the generation; the others wait for it, for at most kBarrierCycles. Returns false in
// every thread of a block whose wait gave up.
__device__ bool grid_barrier(unsigned int* bar, unsigned int nblocks) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = bar + 1;
    const unsigned int g = *gen;
    __threadfence();
    int good = 1;
    if (atomicAdd(bar, 1u) == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const long long t0 = clock64();
      while (*gen == g) {
        if (clock64() - t0 > kBarrierCycles) {
          good = 0;
          break;
        }
      }
    }
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Self-test of the bounded barrier: every block waits at a barrier that expects one block more
// than the grid holds, so no block can pass; each gives up after kBarrierCycles and records
// TN_DEVERR_SVD_WAIT. No copies are in flight and no other resource is held, so the blocks just end.
__global__ void barrier_timeout_selftest_kernel(unsigned int* bar, int* err) {
  if (!grid_barrier(bar, gridDim.x + 1u) && threadIdx.x == 0) atomicExch(err, TN_DEVERR_SVD_WAIT);
}

// Every sweep of the one-sided Jacobi in ONE launch: block i takes pair i of every round, and a
// grid barrier separates the rounds (the round-robin schedule of jacobi_round, the same pair
// arithmetic, so the result equals the one-launch-per-round loop bit for bit). The "rotated" flag
// of sweep w is flags[w % 3]; block 0 clears flags[(w + 1) % 3] as sweep w starts, which no block
// reads or writes during sweeps w - 1 and w. After each sweep every block reads its flag behind
// the sweep's last barrier and stops when it is clear. out[0] = sweeps run, out[1] = 1 if the last
// sweep still rotated. bar: 2 words, zero at launch. A barrier that gives up records
// TN_DEVERR_SVD_WAIT in *err and ends the block.
__global__ void __launch_bounds__(NT) jacobi_sweeps_kernel(int64_t kp, int64_t n, double* X, double tol,
                                                           const double* fro2, double null_rel2, int* flags, double* J,
                                                           int max_sweeps, unsigned int* bar, int* out, int* err) {
  const unsigned int nb = gridDim.x;
  int sweeps = 0, still = 0;
  for (int w = 0; w < max_sweeps; ++w) {
    if (blockIdx.x == 0 && threadIdx.x == 0) flags[(w + 1) % 3] = 0;
    for (int64_t r = 0; r < kp - 1; ++r) {
      jacobi_pair(kp, n, blockIdx.x, r, X, tol, fro2, null_rel2, flags + (w % 3), J);
      if (!grid_barrier(bar, nb)) {
        if (threadIdx.x == 0) atomicExch(err, TN_DEVERR_SVD_WAIT);
        return;
      }
    }
    ++sweeps;
    still = *(volatile int*)(flags + (w % 3));
    if (!still) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    out[0] = sweeps;
    out[1] = still;
  }
}

__global__ void eye_kernel(int64_t kp, double* J) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < kp * kp;
       idx += (int64_t)gridDim.x * blockDim.x)
    J[idx] = (idx / kp == idx % kp) ? 1.0 : 0.0;
}

// s[i] = ||X_i||, Vt[i] = X_i / s[i] (0 for a zero row), U[:, i] = J[i, :k]
__global__ void svd_finish_kernel(int64_t k, int64_t kp, int64_t n, const double* X, const double* J, double* s_out,
                                  double* U, int64_t ldu, double* Vt, int64_t ldvt) {
  const int64_t i = blockIdx.x;
  if (i >= k) return;
  double a = 0.0;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) a = fma(X[i * n + t], X[i * n + t], a);
  __shared__ double red[NT / 32];
  __shared__ double sv;
  a = tn_warp_sum(a);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < NT / 32; ++w) t += red[w];
    sv = sqrt(t);
    s_out[i] = sv;
  }
  __syncthreads();
  const double inv = sv > 0.0 ? 1.0 / sv : 0.0;
  if (Vt)
    for (int64_t t = threadIdx.x; t < n; t += blockDim.x) Vt[i * ldvt + t] = X[i * n + t] * inv;
  if (U)
    for (int64_t r = threadIdx.x; r < k; r += blockDim.x) U[r * ldu + i] = J[i * kp + r];
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

// The whole one-matrix solve on scratch X (kp x n), flag (int) and fro2 (double).
int jacobi_run(int64_t k, int64_t kp, int64_t n, const double* x, int64_t sXr, int64_t sXc, double* s_out,
               double tol, int max_sweeps, double* X, int* flag, double* fro2, cudaStream_t s) {
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(kp * n, NT), 8LL * tn_sm_count()));
  TN_CUDA(cudaMemsetAsync(fro2, 0, sizeof(double), s));
  svd_copy_in<<<blocks, NT, 0, s>>>(k, kp, n, x, sXr, sXc, X, fro2);
  TN_CHECK_LAUNCH();
  const double nr2 = null_row_rel2(k, n);
  int h = 0;
  if (kp >= 2) {
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
      TN_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
      for (int64_t r = 0; r < kp - 1; ++r) {
        jacobi_round<<<(unsigned)(kp / 2), NT, 0, s>>>(kp, n, r, X, tol, fro2, nr2, flag);
        TN_CHECK_LAUNCH();
      }
      TN_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
      TN_CUDA(cudaStreamSynchronize(s));
      if (!h) break;
    }
  }
  row_norms<<<(unsigned)k, NT, 0, s>>>(k, n, X, s_out);
  TN_CHECK_LAUNCH();
  if (h) return tn_fail(TN_ERR_NOCONV, "singular values: Jacobi still rotating after max_sweeps");
  return TN_OK;
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
  double* fro2 = (double*)((char*)ws + 8);
  double* X = (double*)((char*)ws + 256);
  return jacobi_run(k, kp, n, x, sXr, sXc, s_out, tol, max_sweeps, X, flag, fro2, s);
}

// ---------------------------------------------------------------------------
// Batched variant: the singular values of many independent matrices (e.g. the R factors of every
// bond of a chain) with one launch per Jacobi round for the whole batch, so the ~k launches per
// sweep are paid once instead of once per matrix. Each matrix runs its own round-robin schedule
// (round r uses r mod (kp - 1)); a matrix with fewer rows simply repeats rounds, which only
// rotates pairs that are still non-orthogonal. FP64 throughout: with FP32 rows the rounded
// rotations drift the row norms by ~1e-4 over the thousands of rotations a 512-row matrix takes.

namespace {

template <typename T>
struct SvItem {
  int64_t k, kp, n;
  const double* x;
  int64_t sXr, sXc;
  double* s_out;
  T* X;
  double* fro2;      // ||x||_F^2, accumulated by the copy-in
  double null_rel2;  // null-row threshold relative to fro2
};

template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__global__ void svb_copy_in(const SvItem<T>* items) {
  const SvItem<T> it = items[blockIdx.y];
  const int64_t total = it.kp * it.n;
  double acc = 0.0;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx / it.n, c = idx % it.n;
    const double v = r < it.k ? it.x[r * it.sXr + c * it.sXc] : 0.0;
    it.X[idx] = (T)v;
    acc = fma(v, v, acc);
  }
  acc = tn_warp_sum(acc);
  if ((threadIdx.x & 31) == 0 && acc != 0.0) atomicAdd(it.fro2, acc);
}

template <typename T>
__global__ void svb_round(const SvItem<T>* items, int64_t r, T tol, int* rotated) {
  const SvItem<T> it = items[blockIdx.y];
  const int64_t i = blockIdx.x;
  if (it.kp < 2 || i >= it.kp / 2) return;
  const int64_t rr = r % (it.kp - 1);
  const int64_t p = rr_player(i, rr, it.kp), q = rr_player(it.kp - 1 - i, rr, it.kp);
  T* xp = it.X + p * it.n;
  T* xq = it.X + q * it.n;
  T a = 0, b = 0, g = 0;
  for (int64_t t = threadIdx.x; t < it.n; t += blockDim.x) {
    const T u = xp[t], v = xq[t];
    a += u * u;
    b += v * v;
    g += u * v;
  }
  __shared__ T red[3][NT / 32];
  __shared__ T cs[2];
  a = warp_sum_t(a);
  b = warp_sum_t(b);
  g = warp_sum_t(g);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][wid] = a;
    red[1][wid] = b;
    red[2][wid] = g;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    T A = 0, B = 0, G = 0;
    for (int w = 0; w < NT / 32; ++w) {
      A += red[0][w];
      B += red[1][w];
      G += red[2][w];
    }
    T c = 1, sn = 0;
    const double f2 = *it.fro2;
    if (G != (T)0 && fabs(G) > tol * sqrt(A * B) && (double)fmin(A, B) > it.null_rel2 * f2) {
      const T zeta = (B - A) / (2 * G);
      const T tt = (zeta >= 0 ? (T)1 : (T)-1) / (fabs(zeta) + sqrt((T)1 + zeta * zeta));
      c = (T)1 / sqrt((T)1 + tt * tt);
      sn = c * tt;
      // rows below the "small" level rotate without holding up convergence (see the top)
      if (sn != (T)0 && (double)fmin(A, B) > it.null_rel2 * 256.0 * (double)min(it.kp, it.n) * f2) *rotated = 1;
    }
    cs[0] = c;
    cs[1] = sn;
  }
  __syncthreads();
  const T c = cs[0], sn = cs[1];
  if (sn == (T)0) return;
  for (int64_t t = threadIdx.x; t < it.n; t += blockDim.x) {
    const T u = xp[t], v = xq[t];
    xp[t] = c * u - sn * v;
    xq[t] = sn * u + c * v;
  }
}

template <typename T>
__global__ void svb_row_norms(const SvItem<T>* items) {
  const SvItem<T> it = items[blockIdx.y];
  const int64_t r = blockIdx.x;
  if (r >= it.k) return;
  double a = 0.0;
  for (int64_t t = threadIdx.x; t < it.n; t += blockDim.x) {
    const double v = (double)it.X[r * it.n + t];
    a = fma(v, v, a);
  }
  __shared__ double red[NT / 32];
  a = tn_warp_sum(a);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double A = 0;
    for (int w = 0; w < NT / 32; ++w) A += red[w];
    it.s_out[r] = sqrt(A);
  }
}

size_t svb_align(size_t x) { return (x + 255) / 256 * 256; }

template <typename T>
size_t svb_layout(int count, const tn_sv_item* items, char* base, std::vector<SvItem<T>>* out) {
  size_t off = 256 + svb_align(sizeof(SvItem<T>) * (size_t)count);
  double* fro2 = base ? (double*)(base + off) : nullptr;   // one accumulator per matrix
  off += svb_align(sizeof(double) * (size_t)count);
  for (int b = 0; b < count; ++b) {
    const int64_t k = items[b].k, n = items[b].n, kp = k + (k & 1);
    if (out) {
      SvItem<T> it;
      it.k = k;
      it.kp = kp;
      it.n = n;
      it.x = items[b].x;
      it.sXr = items[b].sXr;
      it.sXc = items[b].sXc;
      it.s_out = items[b].s_out;
      it.X = (T*)(base + off);
      it.fro2 = fro2 + b;
      it.null_rel2 = null_row_rel2(k, n);
      out->push_back(it);
    }
    off += svb_align(sizeof(T) * (size_t)kp * n);
  }
  return off;
}

template <typename T>
int svb_run(int count, const tn_sv_item* items, T tol, int max_sweeps, void* ws, cudaStream_t s) {
  char* base = (char*)ws;
  std::vector<SvItem<T>> host;
  svb_layout<T>(count, items, base, &host);
  int* flag = (int*)base;
  SvItem<T>* dev_items = (SvItem<T>*)(base + 256);
  TN_CUDA(cudaMemcpyAsync(dev_items, host.data(), sizeof(SvItem<T>) * host.size(), cudaMemcpyHostToDevice, s));
  int64_t kpmax = 0, kmax = 0, nmax = 0;
  for (const auto& it : host) {
    kpmax = std::max(kpmax, it.kp);
    kmax = std::max(kmax, it.k);
    nmax = std::max(nmax, it.n);
  }
  const dim3 cgrid((unsigned)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(kpmax * nmax, NT), 64)), (unsigned)count);
  TN_CUDA(cudaMemsetAsync(host[0].fro2, 0, sizeof(double) * (size_t)count, s));
  svb_copy_in<T><<<cgrid, NT, 0, s>>>(dev_items);
  TN_CHECK_LAUNCH();
  int h = 0;
  if (kpmax >= 2) {
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
      TN_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
      for (int64_t r = 0; r < kpmax - 1; ++r) {
        svb_round<T><<<dim3((unsigned)(kpmax / 2), (unsigned)count), NT, 0, s>>>(dev_items, r, tol, flag);
        TN_CHECK_LAUNCH();
      }
      TN_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
      TN_CUDA(cudaStreamSynchronize(s));
      if (!h) break;
    }
  }
  svb_row_norms<T><<<dim3((unsigned)std::max<int64_t>(kmax, 1), (unsigned)count), NT, 0, s>>>(dev_items);
  TN_CHECK_LAUNCH();
  // the item table is read by the launches above: keep the host copy alive until they ran
  TN_CUDA(cudaStreamSynchronize(s));
  if (h) return tn_fail(TN_ERR_NOCONV, "singular values: Jacobi still rotating after max_sweeps");
  return TN_OK;
}

}  // namespace

extern "C" size_t tn_singular_values_batched_workspace_bytes(int count, const tn_sv_item* items) {
  if (count <= 0 || !items) return 256;
  return svb_layout<double>(count, items, nullptr, nullptr);
}

extern "C" int tn_singular_values_batched(int count, const tn_sv_item* items, double tol, int max_sweeps, void* ws,
                                          size_t ws_bytes, void* stream) {
  if (count <= 0) return TN_OK;
  if (!items || count > 65535) return tn_fail(TN_ERR_ARG, "singular_values_batched: bad item table");
  for (int b = 0; b < count; ++b)
    if (items[b].k <= 0 || items[b].n <= 0 || !items[b].x || !items[b].s_out)
      return tn_fail(TN_ERR_ARG, "singular_values_batched: bad item");
  if (!ws || ws_bytes < tn_singular_values_batched_workspace_bytes(count, items) ||
      ((uintptr_t)ws & 255) != 0)
    return tn_fail(TN_ERR_WORKSPACE, "singular_values_batched: workspace too small or not 256-byte aligned");
  return svb_run<double>(count, items, tol, max_sweeps, ws, (cudaStream_t)stream);
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
// and must be serialised by the caller. The flag is cleared at the start of every sweep, the norm
// accumulator at the start of every call, and the copy of X is rewritten by every call, so no
// state leaks from one call into the next.
#define TN_SV_NOALLOC_MAX_ELEMS 65536
#define TN_SV_NOALLOC_FLAG_SLOTS 32
static __device__ __align__(256) double g_sv_noalloc_scratch[TN_SV_NOALLOC_FLAG_SLOTS + TN_SV_NOALLOC_MAX_ELEMS];

namespace {
void* g_sv_noalloc_ptr[TN_MAX_DEVICES] = {nullptr};
std::mutex g_sv_noalloc_mu;

// Device address of the static scratch on the current device, resolved once per device (under a
// mutex: host threads of a multi-job host may make their first calls at the same time).
int sv_noalloc_scratch(void** out) {
  int dev = 0;
  int st = tn_current_device(&dev);
  if (st) return st;
  std::lock_guard<std::mutex> lk(g_sv_noalloc_mu);
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
  int* flag = (int*)base;                   // flag slots: the "rotated" flag, then ||X||_F^2
  double* fro2 = (double*)base + 1;
  double* X = (double*)base + TN_SV_NOALLOC_FLAG_SLOTS;
  return jacobi_run(k, kp, n, x, sXr, sXc, s_out, tol, max_sweeps, X, flag, fro2, s);
}

// ---------------------------------------------------------------------------
// Thin SVD with singular vectors (the same Jacobi, rotations accumulated).

extern "C" int tn_selftest_wait_timeout(void* ws, size_t ws_bytes, void* stream) {
  if (!ws || ws_bytes < 256 || ((uintptr_t)ws & 255)) return tn_fail(TN_ERR_WORKSPACE, "selftest: workspace");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int* bar = (unsigned int*)ws;
  int* err = nullptr;
  int st = tn_error_word(s, &err);
  if (st) return st;
  TN_CUDA(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned int), s));
  barrier_timeout_selftest_kernel<<<2, NT, 0, s>>>(bar, err);
  TN_CHECK_LAUNCH();
  return tn_error_check(s);
}

extern "C" size_t tn_svd_jacobi_workspace_bytes(int64_t k, int64_t n) {
  const int64_t kp = k + (k & 1);
  return 256 + (size_t)kp * n * sizeof(double) + 256 + (size_t)kp * kp * sizeof(double) + 512;
}

namespace {

// Can jacobi_sweeps_kernel run kp/2 blocks co-resident on the current device? (once per device)
bool jacobi_coop_fits(int64_t kp) {
  static std::mutex mu;
  static int per_sm[TN_MAX_DEVICES] = {0};   // resident blocks per SM, -1: no cooperative launch
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= TN_MAX_DEVICES) return false;
  int b;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!per_sm[dev]) {
      int coop = 0, nb = 0;
      if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, jacobi_sweeps_kernel, NT, 0) != cudaSuccess || nb <= 0)
        nb = -1;
      cudaGetLastError();
      per_sm[dev] = nb;
    }
    b = per_sm[dev];
  }
  return b > 0 && kp / 2 <= (int64_t)b * tn_sm_count();
}

}  // namespace

extern "C" int tn_svd_jacobi(int64_t k, int64_t n, const double* x, int64_t sXr, int64_t sXc, double* s_out,
                             double* U, int64_t ldu, double* Vt, int64_t ldvt, double tol, int max_sweeps, void* ws,
                             size_t ws_bytes, void* stream) {
  if (k <= 0 || n <= 0 || !x || !s_out) return tn_fail(TN_ERR_ARG, "svd: bad args");
  if ((U && ldu < k) || (Vt && ldvt < n)) return tn_fail(TN_ERR_ARG, "svd: leading dimension too small");
  if (!ws || ws_bytes < tn_svd_jacobi_workspace_bytes(k, n) || ((uintptr_t)ws & 255))
    return tn_fail(TN_ERR_WORKSPACE, "svd: workspace too small or not 256-byte aligned");
  const int64_t kp = k + (k & 1);
  cudaStream_t s = (cudaStream_t)stream;
  int* flag = (int*)ws;
  double* fro2 = (double*)((char*)ws + 8);
  double* X = (double*)((char*)ws + 256);
  double* J = (double*)((char*)X + ((size_t)kp * n * sizeof(double) + 255) / 256 * 256);
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(kp * n, NT), 8LL * tn_sm_count()));
  TN_CUDA(cudaMemsetAsync(fro2, 0, sizeof(double), s));
  svd_copy_in<<<blocks, NT, 0, s>>>(k, kp, n, x, sXr, sXc, X, fro2);
  TN_CHECK_LAUNCH();
  eye_kernel<<<(int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(kp * kp, NT), 8LL * tn_sm_count())), NT, 0, s>>>(kp, J);
  TN_CHECK_LAUNCH();
  const double nr2 = null_row_rel2(k, n);
  int h = 0;
  if (kp >= 2 && max_sweeps > 0 && jacobi_coop_fits(kp)) {
    // all sweeps in one cooperative launch; flags, barrier and result words in the header bytes
    // of the workspace (flag at 0, fro2 at 8): flags[3] at 16, bar[2] at 32, out[2] at 40
    int* flags = (int*)((char*)ws + 16);
    unsigned int* bar = (unsigned int*)((char*)ws + 32);
    int* out = (int*)((char*)ws + 40);
    int* err = nullptr;
    int st = tn_error_word(s, &err);
    if (st) return st;
    TN_CUDA(cudaMemsetAsync(flags, 0, 32, s));
    int64_t a_kp = kp, a_n = n;
    double a_tol = tol, a_nr2 = nr2;
    int a_max = max_sweeps;
    void* args[] = {&a_kp, &a_n, &X, &a_tol, &fro2, &a_nr2, &flags, &J, &a_max, &bar, &out, &err};
    TN_CUDA(cudaLaunchCooperativeKernel((const void*)jacobi_sweeps_kernel, dim3((unsigned)(kp / 2)), dim3(NT), args,
                                        0, s));
    TN_CHECK_LAUNCH();
    svd_finish_kernel<<<(unsigned)k, NT, 0, s>>>(k, kp, n, X, J, s_out, U, ldu, Vt, ldvt);
    TN_CHECK_LAUNCH();
    int hv[2] = {0, 0}, herr = 0;
    TN_CUDA(cudaMemcpyAsync(hv, out, sizeof(hv), cudaMemcpyDeviceToHost, s));
    TN_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    TN_CUDA(cudaStreamSynchronize(s));
    if (herr) return tn_error_status(herr, s);
    if (hv[1]) return tn_fail(TN_ERR_NOCONV, "svd: Jacobi still rotating after max_sweeps");
    return TN_OK;
  }
  if (kp >= 2) {
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
      TN_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
      for (int64_t r = 0; r < kp - 1; ++r) {
        jacobi_round<<<(unsigned)(kp / 2), NT, 0, s>>>(kp, n, r, X, tol, fro2, nr2, flag, J);
        TN_CHECK_LAUNCH();
      }
      TN_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
      TN_CUDA(cudaStreamSynchronize(s));
      if (!h) break;
    }
  }
  svd_finish_kernel<<<(unsigned)k, NT, 0, s>>>(k, kp, n, X, J, s_out, U, ldu, Vt, ldvt);
  TN_CHECK_LAUNCH();
  if (h) return tn_fail(TN_ERR_NOCONV, "svd: Jacobi still rotating after max_sweeps");
  return TN_OK;
}
