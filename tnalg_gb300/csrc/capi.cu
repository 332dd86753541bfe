// C-ABI plumbing: error reporting, device info and the public GEMM entry point.
#include <stdio.h>
#include <string.h>

#include "common.cuh"

int tn_gemm_tf32x3(const TnGemmF64& g, void* ws, size_t ws_bytes, cudaStream_t s);
size_t tn_gemm_tf32x3_ws_bytes(int64_t M, int64_t N, int64_t K, int64_t batch, int64_t nred);

namespace {
thread_local char g_err[512] = "";
}

int tn_record_error(cudaError_t e) {
  snprintf(g_err, sizeof(g_err), "CUDA error %d: %s", (int)e, cudaGetErrorString(e));
  return TN_ERR_CUDA;
}

int tn_fail(int status, const char* msg) {
  snprintf(g_err, sizeof(g_err), "%s", msg);
  return status;
}

std::atomic<unsigned long long> g_tn_launches{0};
thread_local unsigned long long g_tn_thread_launches = 0;
bool tn_tf32x3_supported();

extern "C" const char* tn_last_error(void) { return g_err; }

extern "C" int tn_version(void) { return 100; }

extern "C" unsigned long long tn_launch_count(void) { return g_tn_launches.load(); }

extern "C" int tn_precision_available(int precision) {
  if (precision == TN_PREC_FP64) return 1;
  if (precision == TN_PREC_TF32X3) return tn_tf32x3_supported() ? 1 : 0;
  return 0;
}

extern "C" int tn_device_info(int* sm_count, int* cc_major, int* cc_minor) {
  int dev = 0;
  TN_CUDA(cudaGetDevice(&dev));
  if (sm_count) TN_CUDA(cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev));
  if (cc_major) TN_CUDA(cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev));
  if (cc_minor) TN_CUDA(cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
  return TN_OK;
}

extern "C" size_t tn_gemm_workspace_bytes(int precision, int64_t M, int64_t N, int64_t K, int64_t batch,
                                          int64_t nred) {
  if (precision == TN_PREC_TF32X3) return tn_gemm_tf32x3_ws_bytes(M, N, K, batch, nred);
  return tn_gemm_f64_ws_bytes(M, N, batch);
}

extern "C" int tn_check_device_status(void* stream) {
  // the error word of this stream on the current device: kernels of other streams (other jobs)
  // record their failures in their own words
  return tn_error_check((cudaStream_t)stream);
}

extern "C" int tn_gemm(int precision, int64_t M, int64_t N, int64_t K, const double* A, int64_t sAm, int64_t sAk,
                       const double* B, int64_t sBk, int64_t sBn, double* C, int64_t sCm, int64_t sCn,
                       const double* Cin, int64_t batch, int64_t sAb, int64_t sBb, int64_t sCb, int64_t nred,
                       int64_t sAr, int64_t sBr, double alpha, double beta, void* ws, size_t ws_bytes,
                       void* stream) {
  if (M < 0 || N < 0 || K < 0 || batch < 0 || nred < 0) return tn_fail(TN_ERR_ARG, "gemm: negative size");
  if (!C) return tn_fail(TN_ERR_ARG, "gemm: C is null");
  TnGemmF64 g{};
  g.M = M; g.N = N; g.K = K;
  g.A = A; g.sAm = sAm; g.sAk = sAk;
  g.B = B; g.sBk = sBk; g.sBn = sBn;
  g.C = C; g.sCm = sCm; g.sCn = sCn; g.Cin = Cin;
  g.batch = batch; g.sAb = sAb; g.sBb = sBb; g.sCb = sCb;
  g.nred = nred; g.sAr = sAr; g.sBr = sBr;
  g.alpha = alpha; g.beta = beta;
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == TN_PREC_TF32X3) return tn_gemm_tf32x3(g, ws, ws_bytes, s);
  if (precision != TN_PREC_FP64) return tn_fail(TN_ERR_ARG, "gemm: unknown precision");
  return tn_gemm_f64_ws(g, ws, ws_bytes, s);
}

// ---------------------------------------------------------------------------
// Event profiler: begin/end pairs recorded on the launching stream; elapsed times are
// accumulated when read (or when the event pool runs dry). Single host thread.
#include <vector>

namespace {
struct ProfRec {
  cudaEvent_t a, b;
  int cls;
  double flops;
};
bool g_prof_on = false;
std::vector<cudaEvent_t> g_pool;
std::vector<ProfRec> g_pending;
double g_ms[TN_PROF_NCLASS] = {0}, g_flops[TN_PROF_NCLASS] = {0};
int64_t g_cnt[TN_PROF_NCLASS] = {0};

cudaEvent_t pool_get() {
  if (g_pool.empty()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
  }
  cudaEvent_t e = g_pool.back();
  g_pool.pop_back();
  return e;
}

void flush_pending() {
  for (auto& r : g_pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      g_ms[r.cls] += ms;
      g_cnt[r.cls] += 1;
      g_flops[r.cls] += r.flops;
    }
    g_pool.push_back(r.a);
    g_pool.push_back(r.b);
  }
  g_pending.clear();
}
}  // namespace

cudaEvent_t tn_profile_begin(cudaStream_t s) {
  if (!g_prof_on) return nullptr;
  if (g_pending.size() > 4096) flush_pending();
  cudaEvent_t a = pool_get();
  if (a) cudaEventRecord(a, s);
  return a;
}

void tn_profile_end(cudaEvent_t a, cudaStream_t s, int cls, double flops) {
  if (!a) return;
  cudaEvent_t b = pool_get();
  if (!b) {
    g_pool.push_back(a);
    return;
  }
  cudaEventRecord(b, s);
  g_pending.push_back({a, b, cls, flops});
}

extern "C" int tn_profile_enable(int on) {
  g_prof_on = on != 0;
  return TN_OK;
}

extern "C" int tn_profile_reset(void) {
  flush_pending();
  for (int i = 0; i < TN_PROF_NCLASS; ++i) { g_ms[i] = 0; g_flops[i] = 0; g_cnt[i] = 0; }
  return TN_OK;
}

extern "C" int tn_profile_read(int cls, double* ms, int64_t* count, double* flops) {
  if (cls < 0 || cls >= TN_PROF_NCLASS) return tn_fail(TN_ERR_ARG, "profile: bad class");
  flush_pending();
  if (ms) *ms = g_ms[cls];
  if (count) *count = g_cnt[cls];
  if (flops) *flops = g_flops[cls];
  return TN_OK;
}
