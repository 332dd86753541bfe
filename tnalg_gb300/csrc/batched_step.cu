// tn_batched_step: one local update of every job of a batch in one call.
//
// A local update of one-site DMRG (the body of the sweep loop of dmrg_finite_size,
// DMRG_anyH.py:43-64, i.e. correct_orthogonal_center + update_tensor_eigs of MPSClass.py:188-198,
// 778-809) is, for every job of the batch, a fixed sequence of grouped launches whose records the
// host builds once per (site, direction) of each job:
//   ops1   block operator of the environment being extended (MPSClass.py:684-733)
//   qr     the gauge move of the site left behind, Q in place (TensorBasicModule.py:314-384)
//   gemm1  R absorbed into the next site; the products of the environment update
//   ops2   site operators of the environment update (TensorBasicModule.py:414-421)
//   gemm2  the new environment slots (transfer_left / transfer_right, TensorBasicModule.py:530-619)
//   ops3   the effective Hamiltonian of the next site: WL, WR and straddling pairs
//   solve  the batched Lanczos of every job (tn_batched_lanczos)
// The phases run in this order on one stream; each reuses the same scratch (stream order makes
// that safe). Gauge moves larger than tn_batched_qr_mixed's shared-memory limit run one by one
// through tn_qr_mixed with Q staged in scratch and copied back.
#include <algorithm>
#include <vector>

#include "common.cuh"

namespace {

constexpr int64_t kQrSmemElems = 32768;  // tn_batched_qr_mixed's m n limit

bool dense_layout(const tn_qr_item& q) {
  return (q.sAm == q.n && q.sAn == 1) || (q.sAm == 1 && q.sAn == q.m);
}

size_t al(size_t x) { return (x + 1023) / 1024 * 1024; }

// the items that go through tn_batched_qr_mixed and those that need tn_qr_mixed
void split_qr(const tn_batch_step_desc* d, std::vector<tn_qr_item>* small, std::vector<tn_qr_item>* big) {
  for (int i = 0; i < d->n_qr; ++i) {
    const tn_qr_item& q = d->qr[i];
    if ((int64_t)q.m * q.n > kQrSmemElems) big->push_back(q);
    else small->push_back(q);
  }
}

}  // namespace

extern "C" size_t tn_batched_step_workspace_bytes(const tn_batch_step_desc* d, const tn_lanczos_opts* opts) {
  if (!d || !opts) return 0;
  size_t need = 4096;
  need = std::max(need, tn_grouped_ops_workspace_bytes(std::max({d->n_ops1, d->n_ops2, d->n_ops3, 1})));
  std::vector<tn_qr_item> small, big;
  split_qr(d, &small, &big);
  if (!small.empty()) need = std::max(need, tn_batched_qr_mixed_workspace_bytes(small.data(), (int)small.size()));
  for (const tn_qr_item& q : big)
    need = std::max(need, al(sizeof(double) * (size_t)q.m * q.n) + tn_qr_mixed_workspace_bytes(q.m, q.n));
  if (d->n_gemm1 > 0) need = std::max(need, tn_grouped_gemm_workspace_bytes(d->precision, d->gemm1, d->n_gemm1));
  if (d->n_gemm2 > 0) need = std::max(need, tn_grouped_gemm_workspace_bytes(d->precision, d->gemm2, d->n_gemm2));
  if (d->n_solves > 0) need = std::max(need, tn_batched_lanczos_workspace_bytes(d->solves, d->n_solves, opts));
  return need + 1024;
}

extern "C" int tn_batched_step(const tn_batch_step_desc* d, const tn_lanczos_opts* opts, void* ws, size_t ws_bytes,
                               tn_lanczos_result* results, void* stream) {
  if (!d || !opts) return tn_fail(TN_ERR_ARG, "batched step: null argument");
  if (d->n_solves > 0 && !results) return tn_fail(TN_ERR_ARG, "batched step: null results");
  if (d->n_ops1 < 0 || d->n_qr < 0 || d->n_gemm1 < 0 || d->n_ops2 < 0 || d->n_gemm2 < 0 || d->n_ops3 < 0 ||
      d->n_solves < 0)
    return tn_fail(TN_ERR_ARG, "batched step: negative count");
  const size_t need = tn_batched_step_workspace_bytes(d, opts);
  if (!ws || ws_bytes < need) return tn_fail(TN_ERR_WORKSPACE, "batched step: workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  int st;
  if (d->n_ops1 > 0 && (st = tn_grouped_ops(d->ops1, d->n_ops1, ws, ws_bytes, stream))) return st;
  std::vector<tn_qr_item> small, big;
  split_qr(d, &small, &big);
  if (!small.empty() && (st = tn_batched_qr_mixed(small.data(), (int)small.size(), ws, ws_bytes, stream))) return st;
  for (const tn_qr_item& q : big) {
    if (!dense_layout(q)) return tn_fail(TN_ERR_ARG, "batched step: a large gauge move needs a dense layout");
    if (q.active) return tn_fail(TN_ERR_ARG, "batched step: a large gauge move cannot be masked");
    double* qs = (double*)ws;
    const size_t qbytes = al(sizeof(double) * (size_t)q.m * q.n);
    if ((st = tn_qr_mixed(q.m, q.n, q.a, q.sAm, q.sAn, qs, q.sAm, q.sAn, q.r, q.sRm, q.sRn, (char*)ws + qbytes,
                          ws_bytes - qbytes, stream)))
      return st;
    TN_CUDA(cudaMemcpyAsync(q.a, qs, sizeof(double) * (size_t)q.m * q.n, cudaMemcpyDeviceToDevice, s));
  }
  if (d->n_gemm1 > 0 && (st = tn_grouped_gemm(d->precision, d->gemm1, d->n_gemm1, ws, ws_bytes, stream))) return st;
  if (d->n_ops2 > 0 && (st = tn_grouped_ops(d->ops2, d->n_ops2, ws, ws_bytes, stream))) return st;
  if (d->n_gemm2 > 0 && (st = tn_grouped_gemm(d->precision, d->gemm2, d->n_gemm2, ws, ws_bytes, stream))) return st;
  if (d->n_ops3 > 0 && (st = tn_grouped_ops(d->ops3, d->n_ops3, ws, ws_bytes, stream))) return st;
  if (d->n_solves > 0) return tn_batched_lanczos(d->solves, d->n_solves, opts, ws, ws_bytes, results, stream);
  return TN_OK;
}
