// C-ABI plumbing: error reporting, device info and the public GEMM entry point.
#include <stdio.h>
#include <string.h>

#include "common.cuh"

int tn_gemm_tf32x3(const TnGemmF64& g, void* ws, size_t ws_bytes, cudaStream_t s);
size_t tn_gemm_tf32x3_ws_bytes(int64_t M, int64_t N, int64_t K, int64_t batch);

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

extern "C" const char* tn_last_error(void) { return g_err; }

extern "C" int tn_version(void) { return 100; }

extern "C" int tn_device_info(int* sm_count, int* cc_major, int* cc_minor) {
  int dev = 0;
  TN_CUDA(cudaGetDevice(&dev));
  if (sm_count) TN_CUDA(cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev));
  if (cc_major) TN_CUDA(cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev));
  if (cc_minor) TN_CUDA(cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
  return TN_OK;
}

extern "C" size_t tn_gemm_workspace_bytes(int precision, int64_t M, int64_t N, int64_t K, int64_t batch) {
  if (precision == TN_PREC_TF32X3) return tn_gemm_tf32x3_ws_bytes(M, N, K, batch);
  return tn_gemm_f64_ws_bytes(M, N, batch);
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
