// Split-TF32 tensor-core GEMM (tcgen05) — placeholder until the kernel lands.
#include "common.cuh"

int tn_gemm_tf32x3(const TnGemmF64& g, void* ws, size_t ws_bytes, cudaStream_t s) {
  (void)g; (void)ws; (void)ws_bytes; (void)s;
  return tn_fail(TN_ERR_ARG, "tf32x3 precision not available in this build");
}
size_t tn_gemm_tf32x3_ws_bytes(int64_t M, int64_t N, int64_t K, int64_t batch) {
  (void)M; (void)N; (void)K; (void)batch;
  return 0;
}
int tn_matvec_tf32x3(const tn_site_desc* d, const double* psi, double* y, double alpha, double beta, void* ws,
                     size_t ws_bytes, cudaStream_t s) {
  (void)d; (void)psi; (void)y; (void)alpha; (void)beta; (void)ws; (void)ws_bytes; (void)s;
  return tn_fail(TN_ERR_ARG, "tf32x3 precision not available in this build");
}
size_t tn_matvec_tf32x3_ws_bytes(const tn_site_desc* d) { (void)d; return 0; }
int tn_tf32x3_prepare_static(const tn_site_desc* d, void* ws, size_t ws_bytes, cudaStream_t s) {
  (void)d; (void)ws; (void)ws_bytes; (void)s;
  return tn_fail(TN_ERR_ARG, "tf32x3 precision not available in this build");
}
