// Batched local solves: the Lanczos eigensolver of many independent DMRG jobs advanced together.
//
// Every job of the batch has its own effective Hamiltonian (block form WL (x) 1 + 1 (x) WR +
// sum SL (x) 1 (x) SR, the classify_and_update_env buckets of MPSClass.py:684-733 summed) and its
// own start vector, and replaces scipy's eigsh of update_tensor_eigs (MPSClass.py:778-809) by a
// Lanczos iteration with full reorthogonalisation (classical Gram-Schmidt twice), as tn_lanczos
// does for one job. Here one launch serves all jobs:
//   * matvec: one grouped GEMM launch (grouped_gemm.cu) over every job's WL.x and x.WR^T (split
//     TF32 on the tensor cores, or FP64), with the static operands staged once per solve;
//   * Gram-Schmidt, norms and the next Krylov vector: grouped vector kernels over a flattened list
//     of (job, 1024-element chunk) blocks, with deterministic last-block reductions per job;
//   * convergence: the lowest eigenpair of every job's tridiagonal matrix on the device (one warp
//     per job: 32-point multisection with division-free Sturm counts for the eigenvalue, inverse
//     iteration for the vector), the residual test of tn_lanczos, and the Ritz vector formed on
//     the device. The host reads one counter (jobs still running) per convergence check.
// All active jobs take their Lanczos steps together, so their Krylov bases have the same size;
// a job that converges drops out of every later launch (its blocks return at once).
#include <math.h>
#include <stddef.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "grouped.cuh"

namespace {

constexpr int NT = 256;
constexpr int CH = 1024;         // elements per vector block
constexpr int kMaxM = 64;        // Krylov vectors per restart (batched)

struct BjJob {
  int64_t n;
  double *V, *w, *x;
  double *alpha, *beta, *h1, *h2, *s, *part, *nrm2;
  unsigned int* tickets;  // kMaxM + 2
  const double* psi_in;
  double* psi_out;
  int32_t chunk0, nchunks;
  int32_t active, converged, combine, restarts, brk, steps;
  double theta, resid, tol;
};

__device__ __forceinline__ int find_job(const int* prefix, int n, int t) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

// block-wide sum returned in thread 0
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[NT / 32];
  v = tn_warp_sum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int q = 0; q < NT / 32; ++q) t += red[q];
  __syncthreads();
  return t;
}

// partial -> part[slot * nchunks + c]; the last block of the job for this slot sums the partials
// in chunk order into out (deterministic)
__device__ void reduce_partial(BjJob& J, int c, int slot, double v, double* out) {
  __shared__ bool last;
  const double t = block_sum(v);
  if (threadIdx.x == 0) {
    J.part[(int64_t)slot * J.nchunks + c] = t;
    __threadfence();
    last = (atomicAdd(J.tickets + slot, 1u) == (unsigned)J.nchunks - 1);
  }
  __syncthreads();
  if (last) {
    const double tot = tn_block_sum_partials(J.part + (int64_t)slot * J.nchunks, J.nchunks);
    if (threadIdx.x == 0) {
      *out = tot;
      J.tickets[slot] = 0u;
    }
  }
}

// w = psi_in (block copy) and ||w||^2
__global__ void bl_init_kernel(BjJob* jobs, int njobs, const int* prefix) {
  const int t = blockIdx.x;
  const int j = find_job(prefix, njobs, t);
  BjJob J = jobs[j];
  const int c = t - prefix[j];
  const int64_t e0 = (int64_t)c * CH;
  double acc = 0.0;
  for (int64_t e = e0 + threadIdx.x; e < min(J.n, e0 + CH); e += NT) {
    const double v = J.psi_in[e];
    J.w[e] = v;
    acc = fma(v, v, acc);
  }
  reduce_partial(J, c, kMaxM + 1, acc, J.nrm2);
}

constexpr int EPT = CH / NT;  // vector elements per thread

// Sum over the 32 lanes of G = 8 values at once: on return lane L holds the sum over the warp of
// v[L & 7] (3 halving exchanges, then 2 on the single value left: 9 shuffles instead of 40).
__device__ __forceinline__ double warp_transpose_sum8(double (&v)[8], int lane) {
#pragma unroll
  for (int half = 4; half >= 1; half >>= 1) {
    const bool upper = (lane & half) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const double send = upper ? v[i] : v[i + half];
      const double keep = upper ? v[i + half] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, half);
    }
  }
  double t = v[0];
  t += __shfl_xor_sync(0xffffffffu, t, 8);
  t += __shfl_xor_sync(0xffffffffu, t, 16);
  return t;
}

// h[i] = V[i] . x for i < k over the block's chunk (x: this thread's EPT elements, at e0 + tid +
// q NT), reduced over the block, then, by the last block of the job, over the chunks in chunk order
// (deterministic). One block computes all k dots of its chunk: the w chunk is read once and the
// basis chunks stream through eight at a time (8 EPT independent loads per thread in flight), the
// eight partial dots of a group reduced over the warp together.
__device__ void chunk_dots(BjJob& J, int c, int k, const double (&x)[EPT], int64_t e0, double* out) {
  __shared__ double red[NT / 32][kMaxM + 8];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t nrem = J.n - e0;
  for (int i0 = 0; i0 < k; i0 += 8) {
    double acc[8];
#pragma unroll
    for (int g = 0; g < 8; ++g) {
      acc[g] = 0.0;
      if (i0 + g < k) {
        const double* v = J.V + (int64_t)(i0 + g) * J.n + e0;
#pragma unroll
        for (int q = 0; q < EPT; ++q) {
          const int idx = threadIdx.x + q * NT;
          if (idx < nrem) acc[g] = fma(v[idx], x[q], acc[g]);
        }
      }
    }
    const double t = warp_transpose_sum8(acc, lane);
    if (lane < 8) red[wid][i0 + lane] = t;
  }
  __syncthreads();
  if (threadIdx.x < k) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) t += red[w][threadIdx.x];
    J.part[(int64_t)threadIdx.x * J.nchunks + c] = t;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(J.tickets + kMaxM, 1u) == (unsigned)J.nchunks - 1);
  __syncthreads();
  if (last) {
    __threadfence();
    // warp w sums dots w, w + 8, ...: its lanes stride over the chunks, then a warp sum
    for (int i = wid; i < k; i += NT / 32) {
      const volatile double* pp = J.part + (int64_t)i * J.nchunks;
      double t = 0.0;
      for (int q = lane; q < J.nchunks; q += 32) t += pp[q];
      t = tn_warp_sum(t);
      if (lane == 0) out[i] = t;
    }
    if (threadIdx.x == 0) J.tickets[kMaxM] = 0u;
  }
}

__device__ __forceinline__ void load_chunk(const BjJob& J, int64_t e0, double (&x)[EPT]) {
  const int64_t nrem = J.n - e0;
#pragma unroll
  for (int q = 0; q < EPT; ++q) {
    const int idx = threadIdx.x + q * NT;
    x[q] = idx < nrem ? J.w[e0 + idx] : 0.0;
  }
}

// x -= sum_{i<k} h[i] V[i] on this thread's elements (EPT independent chains)
__device__ __forceinline__ void chunk_axpy(const BjJob& J, int64_t e0, int k, const double* hs, double (&x)[EPT]) {
  const int64_t nrem = J.n - e0;
#pragma unroll 8
  for (int i = 0; i < k; ++i) {
    const double* v = J.V + (int64_t)i * J.n + e0;
    const double h = hs[i];
#pragma unroll
    for (int q = 0; q < EPT; ++q) {
      const int idx = threadIdx.x + q * NT;
      if (idx < nrem) x[q] = fma(-h, v[idx], x[q]);
    }
  }
}

__device__ __forceinline__ void store_chunk(const BjJob& J, int64_t e0, const double (&x)[EPT]) {
  const int64_t nrem = J.n - e0;
#pragma unroll
  for (int q = 0; q < EPT; ++q) {
    const int idx = threadIdx.x + q * NT;
    if (idx < nrem) J.w[e0 + idx] = x[q];
  }
}

// pass 1 of the Gram-Schmidt: h1 = V[0..k) . w
__global__ void __launch_bounds__(NT) bl_dots_kernel(BjJob* jobs, int njobs, const int* prefix, int k) {
  const int t = blockIdx.x;
  const int j = find_job(prefix, njobs, t);
  BjJob J = jobs[j];
  if (!J.active) return;
  const int c = t - prefix[j];
  const int64_t e0 = (int64_t)c * CH;
  double x[EPT];
  load_chunk(J, e0, x);
  chunk_dots(J, c, k, x, e0, J.h1);
}

// w -= sum h1[i] V[i] (pass 1), then h2 = V[0..k) . w (pass 2's projections) in the same block
__global__ void __launch_bounds__(NT) bl_axpy_dots_kernel(BjJob* jobs, int njobs, const int* prefix, int k) {
  const int t = blockIdx.x;
  const int j = find_job(prefix, njobs, t);
  BjJob J = jobs[j];
  if (!J.active) return;
  const int c = t - prefix[j];
  __shared__ double hs[kMaxM + 1];
  for (int i = threadIdx.x; i < k; i += NT) hs[i] = J.h1[i];
  __syncthreads();
  const int64_t e0 = (int64_t)c * CH;
  double x[EPT];
  load_chunk(J, e0, x);
  chunk_axpy(J, e0, k, hs, x);
  store_chunk(J, e0, x);
  chunk_dots(J, c, k, x, e0, J.h2);
}

// w -= sum h2[i] V[i] (pass 2) and ||w||^2 into nrm2
__global__ void __launch_bounds__(NT) bl_axpy_norm_kernel(BjJob* jobs, int njobs, const int* prefix, int k) {
  const int t = blockIdx.x;
  const int j = find_job(prefix, njobs, t);
  BjJob J = jobs[j];
  if (!J.active) return;
  const int c = t - prefix[j];
  __shared__ double hs[kMaxM + 1];
  for (int i = threadIdx.x; i < k; i += NT) hs[i] = J.h2[i];
  __syncthreads();
  const int64_t e0 = (int64_t)c * CH;
  double x[EPT];
  load_chunk(J, e0, x);
  chunk_axpy(J, e0, k, hs, x);
  store_chunk(J, e0, x);
  double acc = 0.0;
#pragma unroll
  for (int q = 0; q < EPT; ++q) acc = fma(x[q], x[q], acc);
  reduce_partial(J, c, kMaxM + 1, acc, J.nrm2);
}

// V[k] = w / ||w||, x = V[k], w = 0; alpha[k-1] = h1 + h2, beta[k-1] = ||w|| (k >= 1; k == 0 is
// the start vector)
__global__ void bl_finish_kernel(BjJob* jobs, int njobs, const int* prefix, int k) {
  const int t = blockIdx.x;
  const int j = find_job(prefix, njobs, t);
  BjJob J = jobs[j];
  if (!J.active) return;
  const int c = t - prefix[j];
  const double nn = *J.nrm2;
  const double b = nn > 0.0 ? sqrt(nn) : 0.0;
  const double inv = b > 1e-300 ? 1.0 / b : 0.0;
  const int64_t e0 = (int64_t)c * CH;
  double* vk = J.V + (int64_t)k * J.n;
  for (int64_t e = e0 + threadIdx.x; e < min(J.n, e0 + CH); e += NT) {
    const double v = J.w[e] * inv;
    vk[e] = v;
    J.x[e] = v;
    J.w[e] = 0.0;
  }
  if (c == 0 && threadIdx.x == 0 && k >= 1) {
    jobs[j].alpha[k - 1] = J.h1[k - 1] + J.h2[k - 1];
    jobs[j].beta[k - 1] = b;
    jobs[j].steps += 1;
  }
}

// ---------------------------------------------------------------------------
// lowest eigenpair of each job's k x k tridiagonal matrix, one warp per job

// number of eigenvalues of T (diagonal a, off-diagonal b, size m) below x: sign changes of the
// leading principal minors det(T_i - x I), by their three-term recurrence (no division); both
// carried minors are rescaled by the same power of two when they leave [2^-400, 2^400]
__device__ int sturm_count(const double* a, const double* b, int m, double x) {
  double p0 = 1.0, p1 = a[0] - x;
  int cnt = (p1 < 0.0) ? 1 : 0;
  bool neg = p1 < 0.0;
  for (int i = 1; i < m; ++i) {
    const double p2 = (a[i] - x) * p1 - b[i - 1] * b[i - 1] * p0;
    p0 = p1;
    p1 = p2;
    const bool n2 = (p1 < 0.0) || (p1 == 0.0 && !neg);
    if (n2 != neg) ++cnt;
    neg = n2;
    const double ap = fabs(p1);
    if (ap > 0x1p400 || (ap < 0x1p-400 && ap > 0.0)) {
      const int e = ilogb(ap);
      p1 = ldexp(p1, -e);
      p0 = ldexp(p0, -e);
    }
  }
  return cnt;
}

// LU factorisation of the tridiagonal T - lam I with partial pivoting (one thread): U has the
// diagonal d0 (stored as reciprocals rp) and two superdiagonals d1, d2; row i's multiplier is f[i]
// and sw[i] says whether rows i and i+1 were swapped. Factored once per eigenvector, solved twice.
// lam is an eigenvalue to working accuracy, so a pivot may vanish: it is replaced by 1e-18 of the
// matrix scale tn (inverse iteration then magnifies the eigenvector by ~1e18 / tn, and the
// normalisation stays in range; a pivot of 1e-300 would overflow the norm).
__device__ void tri_factor(const double* a, const double* b, int m, double lam, double tn, double* rp, double* d1,
                           double* d2, double* f, unsigned char* sw) {
  const double tiny = 1e-18 * fmax(tn, 1e-280);
  double p0 = a[0] - lam, p1 = (m > 1) ? b[0] : 0.0, p2 = 0.0;   // working row i
  for (int i = 0; i < m; ++i) {
    if (i + 1 < m) {
      // next row (below the diagonal b[i], then a[i+1] - lam, then b[i+1])
      double n0 = b[i], n1 = a[i + 1] - lam, n2 = (i + 2 < m) ? b[i + 1] : 0.0;
      const bool swp = fabs(n0) > fabs(p0);
      if (swp) {
        double t;
        t = p0; p0 = n0; n0 = t;
        t = p1; p1 = n1; n1 = t;
        t = p2; p2 = n2; n2 = t;
      }
      double piv = p0;
      if (fabs(piv) < tiny) piv = (piv < 0.0) ? -tiny : tiny;
      const double r = 1.0 / piv;
      const double fi = n0 * r;
      rp[i] = r;
      d1[i] = p1;
      d2[i] = p2;
      f[i] = fi;
      sw[i] = swp ? 1 : 0;
      p0 = n1 - fi * p1;
      p1 = n2 - fi * p2;
      p2 = 0.0;
    } else {
      double piv = p0;
      if (fabs(piv) < tiny) piv = (piv < 0.0) ? -tiny : tiny;
      rp[i] = 1.0 / piv;
      d1[i] = 0.0;
      d2[i] = 0.0;
    }
  }
}

// z <- (T - lam I)^{-1} z with the factorisation of tri_factor (multiplications only)
__device__ void tri_apply(int m, const double* rp, const double* d1, const double* d2, const double* f,
                          const unsigned char* sw, double* z) {
  for (int i = 0; i + 1 < m; ++i) {
    if (sw[i]) {
      const double t = z[i];
      z[i] = z[i + 1];
      z[i + 1] = t;
    }
    z[i + 1] = fma(-f[i], z[i], z[i + 1]);
  }
  for (int i = m - 1; i >= 0; --i) {
    double v = z[i];
    if (i + 1 < m) v = fma(-d1[i], z[i + 1], v);
    if (i + 2 < m) v = fma(-d2[i], z[i + 2], v);
    z[i] = v * rp[i];
  }
}

struct TriOpts {
  double eigs_tol, tau, tol_cap, mixed_floor;
  int32_t mixed, m, restart_at_m, pad;
  int64_t nmin;  // unused
};

// one warp per job; k = Lanczos steps taken (size of T)
__global__ void bl_tridiag_kernel(BjJob* jobs, int njobs, int k, TriOpts o) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int wl = threadIdx.x >> 5;
  __shared__ double sa[4][kMaxM], sb[4][kMaxM], sz[4][kMaxM];
  __shared__ double w0[4][kMaxM], w1[4][kMaxM], w2[4][kMaxM], wf[4][kMaxM];
  __shared__ unsigned char wsw[4][kMaxM];
  __shared__ double lohi[4][2];
  if (warp >= njobs) return;
  BjJob& J = jobs[warp];
  if (!J.active) return;
  double* a = sa[wl];
  double* b = sb[wl];
  for (int i = lane; i < k; i += 32) {
    a[i] = J.alpha[i];
    b[i] = J.beta[i];
  }
  __syncwarp();
  // norm scale and the first negligible off-diagonal (breakdown: T splits there)
  double tn = 0.0;
  for (int i = lane; i < k; i += 32) tn = fmax(tn, fabs(a[i]) + fabs(b[i]));
#pragma unroll
  for (int o2 = 16; o2 > 0; o2 >>= 1) tn = fmax(tn, __shfl_xor_sync(0xffffffffu, tn, o2));
  int mm = k;
  for (int base = 0; base < k - 1; base += 32) {
    const int i = base + lane;
    const bool small = (i < k - 1) && (b[i] <= 1e-14 * fmax(tn, 1e-300));
    const unsigned bal = __ballot_sync(0xffffffffu, small);
    if (bal) { mm = base + __ffs(bal); break; }  // first i with small b: size i + 1
  }
  const bool brk = mm < k || (b[mm - 1] <= 1e-14 * fmax(tn, 1e-300));
  // Gershgorin bracket of the spectrum of the leading mm x mm block; its smallest diagonal entry is
  // a Rayleigh quotient, hence an upper bound of the lowest eigenvalue
  double lo = INFINITY, hi = INFINITY;
  for (int i = lane; i < mm; i += 32) {
    const double r = (i > 0 ? fabs(b[i - 1]) : 0.0) + (i + 1 < mm ? fabs(b[i]) : 0.0);
    lo = fmin(lo, a[i] - r);
    hi = fmin(hi, a[i]);
  }
#pragma unroll
  for (int o2 = 16; o2 > 0; o2 >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o2));
    hi = fmin(hi, __shfl_xor_sync(0xffffffffu, hi, o2));
  }
  // 32-point multisection: lane q tests x_q = lo + (q + 1) (hi - lo) / 33
  const double scale = fmax(fabs(lo), fabs(hi)) + 1e-300;
  for (int it = 0; it < 16 && (hi - lo) > 4e-16 * scale; ++it) {
    const double x = lo + (double)(lane + 1) * ((hi - lo) / 33.0);
    const bool ge = sturm_count(a, b, mm, x) >= 1;
    const unsigned bal = __ballot_sync(0xffffffffu, ge);
    const int q = bal ? __ffs(bal) - 1 : 32;  // first lane whose point lies above the eigenvalue
    const double nlo = (q == 0) ? lo : lo + (double)q * ((hi - lo) / 33.0);
    const double nhi = (q == 32) ? hi : lo + (double)(q + 1) * ((hi - lo) / 33.0);
    lo = nlo;
    hi = nhi;
  }
  const double lam = 0.5 * (lo + hi);
  if (lane == 0) {
    // eigenvector of the leading mm x mm block by inverse iteration (one factorisation, two
    // solves from a generic start); its last component gives the residual |beta_mm s_mm|
    double* z = sz[wl];
    tri_factor(a, b, mm, lam, tn, w0[wl], w1[wl], w2[wl], wf[wl], wsw[wl]);
    for (int i = 0; i < mm; ++i) z[i] = 1.0 + 1e-3 * i;
    for (int rep = 0; rep < 2; ++rep) {
      tri_apply(mm, w0[wl], w1[wl], w2[wl], wf[wl], wsw[wl], z);
      double nrm = 0.0;
      for (int i = 0; i < mm; ++i) nrm = fma(z[i], z[i], nrm);
      nrm = sqrt(nrm);
      if (!(nrm > 0.0) || !isfinite(nrm)) break;
      const double inv = 1.0 / nrm;
      for (int i = 0; i < mm; ++i) z[i] *= inv;
    }
    const double resid = brk ? 0.0 : fabs(b[mm - 1] * z[mm - 1]);
    double tol;
    if (o.tau > 0.0) tol = o.eigs_tol / o.tau * fabs(1.0 - o.tau * lam);
    else tol = o.eigs_tol * fmax(1.0, fabs(lam));
    if (o.tol_cap > 0.0) tol = fmin(tol, o.tol_cap * fmax(1.0, fabs(lam)));
    if (o.mixed) tol = fmax(tol, fmax(o.mixed_floor, 0.0) * fmax(1.0, fabs(lam)));
    const bool conv = resid <= tol || brk || (int64_t)k >= J.n;
    J.theta = lam;
    J.resid = resid;
    J.tol = tol;
    J.brk = brk ? 1 : 0;
    J.combine = conv ? 1 : ((k >= o.m) ? 2 : 0);
    if (J.combine)
      for (int i = 0; i < k; ++i) J.s[i] = (i < mm) ? z[i] : 0.0;
  }
}

// x = sum_i s[i] V[i] for jobs whose combine flag is set: into psi_out (converged) or V[0] and the
// current vector (restart)
__global__ void bl_combine_kernel(BjJob* jobs, int njobs, const int* prefix, int k) {
  const int t = blockIdx.x;
  const int j = find_job(prefix, njobs, t);
  BjJob J = jobs[j];
  if (!J.active || !J.combine) return;
  const int c = t - prefix[j];
  __shared__ double ss[kMaxM];
  for (int i = threadIdx.x; i < k; i += NT) ss[i] = J.s[i];
  __syncthreads();
  const int64_t e0 = (int64_t)c * CH;
  for (int64_t e = e0 + threadIdx.x; e < min(J.n, e0 + CH); e += NT) {
    double acc = 0.0;
    for (int i = 0; i < k; ++i) acc = fma(ss[i], J.V[(int64_t)i * J.n + e], acc);
    if (J.combine == 1) {
      J.psi_out[e] = acc;
    } else {
      J.V[e] = acc;
      J.x[e] = acc;
      J.w[e] = 0.0;
    }
  }
}

// job states after a combine; counts the jobs still running
__global__ void bl_post_kernel(BjJob* jobs, int njobs, int* running) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= njobs) return;
  BjJob& J = jobs[j];
  if (!J.active) return;
  if (J.combine == 1) {
    J.active = 0;
    J.converged = 1;
  } else {
    if (J.combine == 2) J.restarts += 1;
    atomicAdd(running, 1);
  }
  J.combine = 0;
}

// jobs that never converged: their last Ritz vector into psi_out
__global__ void bl_flush_kernel(BjJob* jobs, int njobs, const int* prefix) {
  const int t = blockIdx.x;
  const int j = find_job(prefix, njobs, t);
  BjJob J = jobs[j];
  if (!J.active) return;
  const int c = t - prefix[j];
  const int64_t e0 = (int64_t)c * CH;
  for (int64_t e = e0 + threadIdx.x; e < min(J.n, e0 + CH); e += NT) J.psi_out[e] = J.V[e];
}

size_t al(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

struct Layout {
  std::vector<BjJob> jobs;
  std::vector<int> chunk_prefix;
  // matvec tables; phase 2 (straddling pairs: y += sum_g Z_g SR_g^T after Z = [SL_g] x) runs after
  // phase 1 (WL x, x WR^T, Z)
  std::vector<GgStage> st_static, st_iter, st_iter2;
  std::vector<int> pf_static, pf_iter, pf_iter2;
  std::vector<GgProblem> probs, probs2;
  std::vector<int> pf_probs, pf_probs2;
  std::vector<GgF64Problem> f64, f64b;
  std::vector<int> pf_f64, pf_f64b;
  int bn = 128;  // split-TF32 tile width (gg_tile_n of the calling thread)
  BjJob* d_jobs = nullptr;
  unsigned int* tickets = nullptr;
  size_t tickets_bytes = 0;
  size_t tab_off = 0, bytes = 0;
};

// Builds every table and places every per-job buffer; base == nullptr only measures. Layout of
// the workspace: [256: running-jobs counter][job table][tickets][per-job buffers][other tables].
int layout(const tn_batch_solve* in, int count, const tn_lanczos_opts* o, char* base, Layout* L) {
  const bool mixed = o->precision == TN_PREC_TF32X3;
  const int m = std::max(2, std::min<int>(o->max_krylov, kMaxM));
  const int bn = gg_tile_n();
  L->bn = bn;
  size_t off = 256;
  auto take = [&](size_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off += al(bytes, 1024);
    return p;
  };
  L->d_jobs = (BjJob*)take(sizeof(BjJob) * (size_t)count);
  L->tickets_bytes = sizeof(unsigned int) * (size_t)(kMaxM + 2) * count;
  L->tickets = (unsigned int*)take(L->tickets_bytes);
  L->chunk_prefix.assign(1, 0);
  L->pf_static.assign(1, 0);
  L->pf_iter.assign(1, 0);
  L->pf_iter2.assign(1, 0);
  L->pf_probs.assign(1, 0);
  L->pf_probs2.assign(1, 0);
  L->pf_f64.assign(1, 0);
  L->pf_f64b.assign(1, 0);
  for (int i = 0; i < count; ++i) {
    const tn_site_desc& d = in[i].site;
    if (d.chil <= 0 || d.d <= 0 || d.chir <= 0 || d.nstr < 0) return tn_fail(TN_ERR_ARG, "batched lanczos: bad site shape");
    if (d.nstr > 0 && (!d.sl || !d.sr)) return tn_fail(TN_ERR_ARG, "batched lanczos: straddling pointers missing");
    if (!in[i].psi_in || !in[i].psi_out) return tn_fail(TN_ERR_ARG, "batched lanczos: null vector");
    const int64_t cl = d.chil, dd = d.d, cr = d.chir, n = cl * dd * cr;
    if (n > (1LL << 30)) return tn_fail(TN_ERR_ARG, "batched lanczos: site too large");
    const int32_t* active = base ? (const int32_t*)((char*)(L->d_jobs + i) + offsetof(BjJob, active)) : nullptr;
    BjJob J{};
    J.n = n;
    J.nchunks = (int32_t)tn_cdiv(n, CH);
    J.chunk0 = L->chunk_prefix.back();
    L->chunk_prefix.push_back(J.chunk0 + J.nchunks);
    J.V = (double*)take(sizeof(double) * (size_t)(m + 1) * n);
    J.w = (double*)take(sizeof(double) * n);
    J.x = (double*)take(sizeof(double) * n);
    J.alpha = (double*)take(sizeof(double) * (kMaxM + 2));
    J.beta = (double*)take(sizeof(double) * (kMaxM + 2));
    J.h1 = (double*)take(sizeof(double) * (kMaxM + 2));
    J.h2 = (double*)take(sizeof(double) * (kMaxM + 2));
    J.s = (double*)take(sizeof(double) * (kMaxM + 2));
    J.nrm2 = (double*)take(sizeof(double) * 4);
    J.part = (double*)take(sizeof(double) * (size_t)(kMaxM + 2) * J.nchunks);
    J.tickets = base ? L->tickets + (size_t)(kMaxM + 2) * i : nullptr;
    J.psi_in = in[i].psi_in;
    J.psi_out = in[i].psi_out;
    J.active = 1;
    L->jobs.push_back(J);
    const int64_t ng = d.nstr;
    double* Z = ng > 0 ? (double*)take(sizeof(double) * (size_t)ng * n) : nullptr;
    // matvec problems: WL . x  and  x . WR^T, both added into w; straddling pairs in two phases
    if (mixed) {
      auto stage = [&](std::vector<GgStage>& v, std::vector<int>& pf, const double* src, int64_t rows, int64_t K,
                       int64_t s_row, int64_t s_k, int64_t nred = 1, int64_t s_red = 0) -> const float* {
        GgStage g{};
        g.src = src; g.s_row = s_row; g.s_k = s_k; g.s_red = s_red; g.active = active;
        gg_stage_shape(&g, rows, K, nred);
        g.dst = (float*)take(sizeof(float) * gg_staged_floats(rows, K, nred));
        v.push_back(g);
        pf.push_back(pf.back() + gg_stage_tiles(g));
        return g.dst;
      };
      if (ng > 0) {
        // phase 1: Z (ng chil x d chir) = [SL_1; ...; SL_ng] (ng chil x chil) . x (chil x d chir)
        GgProblem p{};
        p.nbatch = 1; p.n_mt = (int32_t)tn_cdiv(ng * cl, 128);
        p.M = (int32_t)(ng * cl); p.N = (int32_t)(dd * cr); p.nred = 1;
        p.n_kb = (int32_t)tn_cdiv(cl, 32); p.n_nt = (int32_t)tn_cdiv(dd * cr, bn);
        p.a = stage(L->st_static, L->pf_static, d.sl, ng * cl, cl, cl, 1);
        p.a_nrt = (int32_t)tn_cdiv(ng * cl, 128);
        p.b = stage(L->st_iter, L->pf_iter, J.x, dd * cr, cl, 1, dd * cr);  // B^T rows (s b), k = a
        p.b_nrt = (int32_t)tn_cdiv(dd * cr, 128);
        p.C = Z; p.sCm = dd * cr; p.sCn = 1; p.alpha = 1.0; p.beta = 0.0; p.accumulate = 0; p.active = active;
        L->probs.push_back(p);
        L->pf_probs.push_back(L->pf_probs.back() + gg_tf32_tiles(p, bn));
        // phase 2: w += sum_g Z_g (chil d x chir) . SR_g^T
        GgProblem q{};
        q.nbatch = 1; q.n_mt = (int32_t)tn_cdiv(cl * dd, 128);
        q.M = (int32_t)(cl * dd); q.N = (int32_t)cr; q.nred = (int32_t)ng;
        q.n_kb = (int32_t)tn_cdiv(cr, 32); q.n_nt = (int32_t)tn_cdiv(cr, bn);
        q.a = stage(L->st_iter2, L->pf_iter2, Z, cl * dd, cr, cr, 1, ng, n);
        q.a_nrt = (int32_t)tn_cdiv(cl * dd, 128);
        q.b = stage(L->st_static, L->pf_static, d.sr, cr, cr, cr, 1, ng, cr * cr);  // B^T rows b = SR_g rows
        q.b_nrt = (int32_t)tn_cdiv(cr, 128);
        q.C = J.w; q.sCm = cr; q.sCn = 1; q.alpha = 1.0; q.accumulate = 1; q.active = active;
        L->probs2.push_back(q);
        L->pf_probs2.push_back(L->pf_probs2.back() + gg_tf32_tiles(q, bn));
      }
      if (d.wl) {
        GgProblem p{};
        p.nbatch = 1; p.n_mt = (int32_t)tn_cdiv(cl * dd, 128);
        p.M = (int32_t)(cl * dd); p.N = (int32_t)cr; p.nred = 1;
        p.n_kb = (int32_t)tn_cdiv(cl * dd, 32); p.n_nt = (int32_t)tn_cdiv(cr, bn);
        p.a = stage(L->st_static, L->pf_static, d.wl, cl * dd, cl * dd, cl * dd, 1);
        p.a_nrt = (int32_t)tn_cdiv(cl * dd, 128);
        p.b = stage(L->st_iter, L->pf_iter, J.x, cr, cl * dd, 1, cr);  // B^T rows b, k = (a s)
        p.b_nrt = (int32_t)tn_cdiv(cr, 128);
        p.C = J.w; p.sCm = cr; p.sCn = 1; p.alpha = 1.0; p.accumulate = 1; p.active = active;
        L->probs.push_back(p);
        L->pf_probs.push_back(L->pf_probs.back() + gg_tf32_tiles(p, bn));
      }
      if (d.wr) {
        GgProblem p{};
        p.nbatch = 1; p.n_mt = (int32_t)tn_cdiv(cl, 128);
        p.M = (int32_t)cl; p.N = (int32_t)(dd * cr); p.nred = 1;
        p.n_kb = (int32_t)tn_cdiv(dd * cr, 32); p.n_nt = (int32_t)tn_cdiv(dd * cr, bn);
        p.a = stage(L->st_iter, L->pf_iter, J.x, cl, dd * cr, dd * cr, 1);
        p.a_nrt = (int32_t)tn_cdiv(cl, 128);
        p.b = stage(L->st_static, L->pf_static, d.wr, dd * cr, dd * cr, dd * cr, 1);  // B^T = WR rows
        p.b_nrt = (int32_t)tn_cdiv(dd * cr, 128);
        p.C = J.w; p.sCm = dd * cr; p.sCn = 1; p.alpha = 1.0; p.accumulate = 1; p.active = active;
        L->probs.push_back(p);
        L->pf_probs.push_back(L->pf_probs.back() + gg_tf32_tiles(p, bn));
      }
    } else {
      if (ng > 0) {
        GgF64Problem f{};
        f.nbatch = 1;
        f.M = (int32_t)(ng * cl); f.N = (int32_t)(dd * cr); f.K = (int32_t)cl; f.nred = 1;
        f.A = d.sl; f.sAm = cl; f.sAk = 1;
        f.B = J.x; f.sBk = dd * cr; f.sBn = 1;
        f.C = Z; f.sCm = dd * cr; f.sCn = 1; f.alpha = 1.0; f.beta = 0.0; f.accumulate = 0; f.active = active;
        L->f64.push_back(f);
        L->pf_f64.push_back(L->pf_f64.back() + gg_f64_tiles(f));
        GgF64Problem g{};
        g.nbatch = 1;
        g.M = (int32_t)(cl * dd); g.N = (int32_t)cr; g.K = (int32_t)cr; g.nred = (int32_t)ng;
        g.A = Z; g.sAm = cr; g.sAk = 1; g.sAr = n;
        g.B = d.sr; g.sBk = 1; g.sBn = cr; g.sBr = cr * cr;
        g.C = J.w; g.sCm = cr; g.sCn = 1; g.alpha = 1.0; g.accumulate = 1; g.active = active;
        L->f64b.push_back(g);
        L->pf_f64b.push_back(L->pf_f64b.back() + gg_f64_tiles(g));
      }
      if (d.wl) {
        GgF64Problem f{};
        f.nbatch = 1;
        f.M = (int32_t)(cl * dd); f.N = (int32_t)cr; f.K = (int32_t)(cl * dd); f.nred = 1;
        f.A = d.wl; f.sAm = cl * dd; f.sAk = 1;
        f.B = J.x; f.sBk = cr; f.sBn = 1;
        f.C = J.w; f.sCm = cr; f.sCn = 1; f.alpha = 1.0; f.accumulate = 1; f.active = active;
        L->f64.push_back(f);
        L->pf_f64.push_back(L->pf_f64.back() + gg_f64_tiles(f));
      }
      if (d.wr) {
        GgF64Problem f{};
        f.nbatch = 1;
        f.M = (int32_t)cl; f.N = (int32_t)(dd * cr); f.K = (int32_t)(dd * cr); f.nred = 1;
        f.A = J.x; f.sAm = dd * cr; f.sAk = 1;
        f.B = d.wr; f.sBk = 1; f.sBn = dd * cr;
        f.C = J.w; f.sCm = dd * cr; f.sCn = 1; f.alpha = 1.0; f.accumulate = 1; f.active = active;
        L->f64.push_back(f);
        L->pf_f64.push_back(L->pf_f64.back() + gg_f64_tiles(f));
      }
    }
  }
  // the remaining device tables
  L->tab_off = off;
  auto tab = [&](size_t bytes) { take(bytes + 64); };
  tab(sizeof(int) * L->chunk_prefix.size());
  tab(sizeof(GgStage) * L->st_static.size());
  tab(sizeof(int) * L->pf_static.size());
  tab(sizeof(GgStage) * L->st_iter.size());
  tab(sizeof(int) * L->pf_iter.size());
  tab(sizeof(GgStage) * L->st_iter2.size());
  tab(sizeof(int) * L->pf_iter2.size());
  tab(sizeof(GgProblem) * L->probs.size());
  tab(sizeof(int) * L->pf_probs.size());
  tab(sizeof(GgProblem) * L->probs2.size());
  tab(sizeof(int) * L->pf_probs2.size());
  tab(sizeof(GgF64Problem) * L->f64.size());
  tab(sizeof(int) * L->pf_f64.size());
  tab(sizeof(GgF64Problem) * L->f64b.size());
  tab(sizeof(int) * L->pf_f64b.size());
  L->bytes = off + 1024;
  return TN_OK;
}

}  // namespace

extern "C" size_t tn_batched_lanczos_workspace_bytes(const tn_batch_solve* jobs, int count,
                                                     const tn_lanczos_opts* opts) {
  if (!jobs || count <= 0 || !opts) return 4096;
  Layout L;
  if (layout(jobs, count, opts, nullptr, &L)) return 0;
  return L.bytes;
}

extern "C" int tn_batched_lanczos(const tn_batch_solve* in, int count, const tn_lanczos_opts* o, void* ws,
                                  size_t ws_bytes, tn_lanczos_result* results, void* stream) {
  if (count <= 0) return TN_OK;
  if (!in || !o || !results) return tn_fail(TN_ERR_ARG, "batched lanczos: null argument");
  if (o->precision != TN_PREC_FP64 && o->precision != TN_PREC_TF32X3)
    return tn_fail(TN_ERR_ARG, "batched lanczos: precision");
  if (o->precision == TN_PREC_TF32X3 && !tn_tf32x3_supported())
    return tn_fail(TN_ERR_ARG, "tf32x3 needs an sm_103 device");
  if (o->refine == 2) return tn_fail(TN_ERR_ARG, "batched lanczos: refine == 2 is not supported");
  if (o->max_krylov > kMaxM) return tn_fail(TN_ERR_ARG, "batched lanczos: max_krylov > 64");
  cudaStream_t s = (cudaStream_t)stream;
  Layout Lm;
  int st = layout(in, count, o, nullptr, &Lm);
  if (st) return st;
  if (!ws || ws_bytes < Lm.bytes) return tn_fail(TN_ERR_WORKSPACE, "batched lanczos: workspace too small");
  char* base = (char*)al((uintptr_t)ws, 1024);
  Layout L;
  if ((st = layout(in, count, o, base, &L))) return st;
  char* p = base + L.tab_off;
  auto put = [&](const void* src, size_t bytes) -> char* {
    char* at = p;
    if (bytes) {
      if (cudaMemcpyAsync(at, src, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) return nullptr;
    }
    p += al(bytes + 64, 1024);
    return at;
  };
  BjJob* d_jobs = L.d_jobs;
  TN_CUDA(cudaMemcpyAsync(d_jobs, L.jobs.data(), sizeof(BjJob) * L.jobs.size(), cudaMemcpyHostToDevice, s));
  TN_CUDA(cudaMemsetAsync(L.tickets, 0, L.tickets_bytes, s));
  int* d_cpf = (int*)put(L.chunk_prefix.data(), sizeof(int) * L.chunk_prefix.size());
  GgStage* d_sst = (GgStage*)put(L.st_static.data(), sizeof(GgStage) * L.st_static.size());
  int* d_pst = (int*)put(L.pf_static.data(), sizeof(int) * L.pf_static.size());
  GgStage* d_sit = (GgStage*)put(L.st_iter.data(), sizeof(GgStage) * L.st_iter.size());
  int* d_pit = (int*)put(L.pf_iter.data(), sizeof(int) * L.pf_iter.size());
  GgStage* d_sit2 = (GgStage*)put(L.st_iter2.data(), sizeof(GgStage) * L.st_iter2.size());
  int* d_pit2 = (int*)put(L.pf_iter2.data(), sizeof(int) * L.pf_iter2.size());
  GgProblem* d_pr = (GgProblem*)put(L.probs.data(), sizeof(GgProblem) * L.probs.size());
  int* d_ppr = (int*)put(L.pf_probs.data(), sizeof(int) * L.pf_probs.size());
  GgProblem* d_pr2 = (GgProblem*)put(L.probs2.data(), sizeof(GgProblem) * L.probs2.size());
  int* d_ppr2 = (int*)put(L.pf_probs2.data(), sizeof(int) * L.pf_probs2.size());
  GgF64Problem* d_f = (GgF64Problem*)put(L.f64.data(), sizeof(GgF64Problem) * L.f64.size());
  int* d_pf = (int*)put(L.pf_f64.data(), sizeof(int) * L.pf_f64.size());
  GgF64Problem* d_f2 = (GgF64Problem*)put(L.f64b.data(), sizeof(GgF64Problem) * L.f64b.size());
  int* d_pf2 = (int*)put(L.pf_f64b.data(), sizeof(int) * L.pf_f64b.size());
  if (!d_cpf || !d_sst || !d_pst || !d_sit || !d_pit || !d_sit2 || !d_pit2 || !d_pr || !d_ppr || !d_pr2 ||
      !d_ppr2 || !d_f || !d_pf || !d_f2 || !d_pf2)
    return tn_record_error(cudaGetLastError());
  // the counter of running jobs lives in the first bytes of the workspace
  int* running = (int*)base;
  const int njobs = count;
  const int chunks = L.chunk_prefix.back();
  const bool mixed = o->precision == TN_PREC_TF32X3;
  const int m = std::max(2, std::min<int>(o->max_krylov, kMaxM));
  const int check = std::max(1, o->check_every);
  TriOpts to{o->eigs_tol, o->tau, o->tol_cap, o->mixed_floor, mixed ? 1 : 0, m, 1, 0, 0};

  if (mixed) {
    st = gg_launch_stage(d_sst, (int)L.st_static.size(), d_pst, L.pf_static.back(), s);
    if (st) return st;
  }
  bl_init_kernel<<<chunks, NT, 0, s>>>(d_jobs, njobs, d_cpf);
  TN_CHECK_LAUNCH();
  bl_finish_kernel<<<chunks, NT, 0, s>>>(d_jobs, njobs, d_cpf, 0);
  TN_CHECK_LAUNCH();
  int k = 0;  // Lanczos steps in the current cycle (size of T)
  const int max_steps = m * std::max(1, o->max_restarts + 1);
  int total = 0, left = njobs;
  for (; total < max_steps && left > 0; ++total) {
    // w = H x
    if (mixed) {
      if ((st = gg_launch_stage(d_sit, (int)L.st_iter.size(), d_pit, L.pf_iter.back(), s))) return st;
      if ((st = gg_launch_tf32(d_pr, (int)L.probs.size(), d_ppr, L.pf_probs.back(), L.bn, 0, s))) return st;
      if (!L.probs2.empty()) {
        if ((st = gg_launch_stage(d_sit2, (int)L.st_iter2.size(), d_pit2, L.pf_iter2.back(), s))) return st;
        if ((st = gg_launch_tf32(d_pr2, (int)L.probs2.size(), d_ppr2, L.pf_probs2.back(), L.bn, 0, s))) return st;
      }
    } else {
      if ((st = gg_launch_f64(d_f, (int)L.f64.size(), d_pf, L.pf_f64.back(), s))) return st;
      if (!L.f64b.empty() && (st = gg_launch_f64(d_f2, (int)L.f64b.size(), d_pf2, L.pf_f64b.back(), s))) return st;
    }
    const int nc = k + 1;
    // classical Gram-Schmidt twice against V[0..nc): dots, update + second dots, update + norm
    bl_dots_kernel<<<chunks, NT, 0, s>>>(d_jobs, njobs, d_cpf, nc);
    TN_CHECK_LAUNCH();
    bl_axpy_dots_kernel<<<chunks, NT, 0, s>>>(d_jobs, njobs, d_cpf, nc);
    TN_CHECK_LAUNCH();
    bl_axpy_norm_kernel<<<chunks, NT, 0, s>>>(d_jobs, njobs, d_cpf, nc);
    TN_CHECK_LAUNCH();
    bl_finish_kernel<<<chunks, NT, 0, s>>>(d_jobs, njobs, d_cpf, nc);
    TN_CHECK_LAUNCH();
    k = nc;
    if (k % check == 0 || k >= m) {
      bl_tridiag_kernel<<<(unsigned)tn_cdiv(njobs, 4), 128, 0, s>>>(d_jobs, njobs, k, to);
      TN_CHECK_LAUNCH();
      bl_combine_kernel<<<chunks, NT, 0, s>>>(d_jobs, njobs, d_cpf, k);
      TN_CHECK_LAUNCH();
      TN_CUDA(cudaMemsetAsync(running, 0, sizeof(int), s));
      bl_post_kernel<<<(unsigned)tn_cdiv(njobs, 128), 128, 0, s>>>(d_jobs, njobs, running);
      TN_CHECK_LAUNCH();
      int h = 0;
      TN_CUDA(cudaMemcpyAsync(&h, running, sizeof(int), cudaMemcpyDeviceToHost, s));
      int herr = 0;
      int* err;
      if ((st = tn_error_word(s, &err))) return st;
      TN_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
      TN_CUDA(cudaStreamSynchronize(s));
      if (herr) return tn_error_status(herr, s);
      left = h;
      if (k >= m) k = 0;  // restarted jobs continue from their Ritz vector in V[0]
    }
  }
  if (left > 0) {
    bl_flush_kernel<<<chunks, NT, 0, s>>>(d_jobs, njobs, d_cpf);
    TN_CHECK_LAUNCH();
  }
  std::vector<BjJob> out(njobs);
  TN_CUDA(cudaMemcpyAsync(out.data(), d_jobs, sizeof(BjJob) * njobs, cudaMemcpyDeviceToHost, s));
  TN_CUDA(cudaStreamSynchronize(s));
  int unconverged = 0;
  for (int i = 0; i < njobs; ++i) {
    results[i].energy = out[i].theta;
    results[i].residual = out[i].resid;
    results[i].energy_fp64 = out[i].theta;
    results[i].matvecs = out[i].steps;
    results[i].restarts = out[i].restarts;
    results[i].converged = out[i].converged;
    if (!out[i].converged) ++unconverged;
  }
  return unconverged ? TN_ERR_NOCONV : TN_OK;
}
