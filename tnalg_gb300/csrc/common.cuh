// Shared helpers for the tnalg_gb300 CUDA kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>

#include "tnalg_gb300.h"

// Every kernel launch site of the library is followed by TN_CHECK_LAUNCH(), which also counts
// the launch (tn_launch_count in the C ABI): in a process-wide atomic counter, and in a per-thread
// one that lets a graph capture count its own launches while other host threads launch theirs.
extern std::atomic<unsigned long long> g_tn_launches;
extern thread_local unsigned long long g_tn_thread_launches;

// Codes written into a device error word: 1-3 name the split-TF32 GEMM pipeline wait that gave
// up, TN_DEVERR_RANGE a finite operand beyond FP32's range (split TF32 cannot represent it), and
// TN_DEVERR_QR_WAIT a cluster-QR panel wait that timed out.
constexpr int TN_DEVERR_RANGE = 16;
constexpr int TN_DEVERR_QR_WAIT = 32;
// TN_DEVERR_SVD_WAIT: a grid barrier of the single-launch Jacobi SVD that timed out.
constexpr int TN_DEVERR_SVD_WAIT = 64;

// FP32 Householder QR (inputs scaled by a power of two to max |a| ~ 1): a sub-column whose squared
// norm is at most kHhTiny gets no reflector and is taken as zero. Below ~1e-19 the squares are
// subnormal or flushed, the computed |x|^2 can be off by an O(1) factor, and a reflector built from
// it is not orthogonal; with the threshold at 1e-24 the squares that matter are normal numbers, and
// the entries dropped are below 1e-12 of the largest, under the FP32 accuracy of R.
constexpr float kHhTiny = 1e-24f;

// Per-device host state (device_state.cu). Device ordinals 0..TN_MAX_DEVICES-1.
constexpr int TN_MAX_DEVICES = 64;
int tn_current_device(int* dev);
// The error word of stream s on the current device (device memory, zeroed at creation).
int tn_error_word(cudaStream_t s, int** out);
// Status for a value h read from stream s's error word; clears the word (on s) when h != 0.
int tn_error_status(int h, cudaStream_t s);
// Synchronise s, read and clear its error word.
int tn_error_check(cudaStream_t s);
// cudaFuncAttributeMaxDynamicSharedMemorySize = bytes for func, once per device (key: one bit per
// kernel configuration, TN_ATTR_*).
int tn_set_smem_attr_once(int key, const void* func, int bytes);
enum {
  TN_ATTR_TF32_BN64 = 0,
  TN_ATTR_TF32_BN128 = 1,
  TN_ATTR_QR_PANEL_CLUSTER = 2,
  TN_ATTR_GROUPED_GEMM = 3,
  TN_ATTR_BATCH_QR = 4,
};
#define TN_CHECK_LAUNCH()                                   \
  do {                                                      \
    g_tn_launches.fetch_add(1, std::memory_order_relaxed);  \
    ++g_tn_thread_launches;                                 \
    cudaError_t e_ = cudaGetLastError();                    \
    if (e_ != cudaSuccess) return tn_record_error(e_);      \
  } while (0)

#define TN_CUDA(call)                                       \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return tn_record_error(e_);      \
  } while (0)

// Records the CUDA error text for tn_last_error() and maps it to a status code.
int tn_record_error(cudaError_t e);
int tn_fail(int status, const char* msg);

__host__ __device__ static inline int64_t tn_cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

__device__ __forceinline__ double tn_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of part[0..count) by the whole block (every thread calls it; the result is returned in
// thread 0). Deterministic for a given block size; the partials are read after a fence, for the
// "last block of a grid reduces everyone's partials" pattern. Replaces a one-thread loop, whose
// dependent FP64 adds (64-cycle latency on GB300) took ~10 us for a few hundred partials.
__device__ __forceinline__ double tn_block_sum_partials(const double* part, unsigned count) {
  __shared__ double tn_red_partials[32];
  __threadfence();
  double t = 0.0;
  for (unsigned b = threadIdx.x; b < count; b += blockDim.x) t += ((const volatile double*)part)[b];
  t = tn_warp_sum(t);
  if ((threadIdx.x & 31) == 0) tn_red_partials[threadIdx.x >> 5] = t;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (unsigned w = 0; w < (blockDim.x + 31) / 32; ++w) s += tn_red_partials[w];
  return s;
}

__device__ __forceinline__ float tn_warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Internal launchers shared between translation units.
struct TnGemmF64 {
  int64_t M, N, K;
  const double* A; int64_t sAm, sAk;
  const double* B; int64_t sBk, sBn;
  double* C; int64_t sCm, sCn;
  const double* Cin;  // nullptr: beta scales C itself
  int64_t batch; int64_t sAb, sBb, sCb;
  int64_t nred; int64_t sAr, sBr;
  double alpha, beta;
};
int tn_gemm_f64_launch(const TnGemmF64& g, cudaStream_t s);
int tn_gemm_f64_ws(const TnGemmF64& g, void* ws, size_t ws_bytes, cudaStream_t s);
size_t tn_gemm_f64_ws_bytes(int64_t M, int64_t N, int64_t batch);
int tn_sm_count();

// Optional CUDA-event profiling of kernel classes (tn_profile_* in the C ABI).
enum {
  TN_PROF_MATVEC = 0,    // effective-Hamiltonian matvec inside tn_lanczos
  TN_PROF_QR = 1,        // whole tn_qr call
  TN_PROF_QR_PANEL = 2,  // QR panel factorisations
  TN_PROF_QR_FORM_Q = 3, // explicit Q formation
  TN_PROF_LANCZOS = 4,   // whole tn_lanczos call
  TN_PROF_NCLASS = 8
};
// begin returns nullptr when profiling is off; end(nullptr, ...) is a no-op. Pairs may nest.
cudaEvent_t tn_profile_begin(cudaStream_t s);
void tn_profile_end(cudaEvent_t start, cudaStream_t s, int cls, double flops);
