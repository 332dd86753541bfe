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
// that safe). Gauge moves larger than tn_batched_qr_mixed's shared-memory limit go through
// tn_qr_mixed (one 16-CTA cluster each) with Q staged in scratch and copied back; they are spread
// over up to kLanes side streams forked from and joined back into the caller's stream, each lane
// with its own slice of the scratch, so the clusters of different jobs run side by side (a step of
// a batch with chi = 256 or 512 jobs otherwise runs their factorisations one after another on ~16
// of the 152 SMs). A bounded wait that gives up inside a lane is recorded in the lane stream's
// error word and moved into the caller's stream's word after the join.
#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace {

constexpr int64_t kQrSmemElems = 32768;  // tn_batched_qr_mixed's m n limit
constexpr int kLanes = 8;                 // side streams for the large gauge moves of one step

// Side streams and fork/join events of one device, created on first use there. The enqueue of a
// step's lanes (fork, launches, join) holds the mutex, so concurrent callers on one device never
// interleave their records of the shared events.
struct Lanes {
  bool ready = false;
  cudaStream_t s[kLanes];
  cudaEvent_t fork;
  cudaEvent_t join[kLanes];
};
Lanes g_lanes[TN_MAX_DEVICES];
std::mutex g_lanes_mu;

int lanes_of_device(Lanes** out) {
  int dev = 0;
  int st = tn_current_device(&dev);
  if (st) return st;
  Lanes& L = g_lanes[dev];
  if (!L.ready) {
    TN_CUDA(cudaEventCreateWithFlags(&L.fork, cudaEventDisableTiming));
    for (int i = 0; i < kLanes; ++i) {
      TN_CUDA(cudaStreamCreateWithFlags(&L.s[i], cudaStreamNonBlocking));
      TN_CUDA(cudaEventCreateWithFlags(&L.join[i], cudaEventDisableTiming));
    }
    L.ready = true;
  }
  *out = &L;
  return TN_OK;
}

// *dst |= what a lane recorded in *src (the first error code wins), and *src cleared
__global__ void move_error_kernel(int* dst, int* src) {
  const int e = *src;
  if (e) {
    atomicCAS(dst, 0, e);
    *src = 0;
  }
}

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

// scratch of one lane: the staged Q and tn_qr_mixed's workspace of the largest move
size_t big_lane_bytes(const std::vector<tn_qr_item>& big) {
  size_t b = 0;
  for (const tn_qr_item& q : big)
    b = std::max(b, al(sizeof(double) * (size_t)q.m * q.n) + al(tn_qr_mixed_workspace_bytes(q.m, q.n)));
  return b;
}

// The large gauge moves: move i on lane i mod nl, every lane forked from and joined into s.
int run_big_qr(const std::vector<tn_qr_item>& big, void* ws, size_t ws_bytes, cudaStream_t s) {
  for (const tn_qr_item& q : big) {
    if (!dense_layout(q)) return tn_fail(TN_ERR_ARG, "batched step: a large gauge move needs a dense layout");
    if (q.active) return tn_fail(TN_ERR_ARG, "batched step: a large gauge move cannot be masked");
  }
  const int nl = (int)std::min<size_t>(big.size(), kLanes);
  const size_t slice = big_lane_bytes(big);
  if ((size_t)nl * slice > ws_bytes) return tn_fail(TN_ERR_WORKSPACE, "batched step: workspace too small");
  // a single move needs no fork
  if (nl == 1) {
    for (const tn_qr_item& q : big) {
      double* qs = (double*)ws;
      const size_t qbytes = al(sizeof(double) * (size_t)q.m * q.n);
      int st = tn_qr_mixed(q.m, q.n, q.a, q.sAm, q.sAn, qs, q.sAm, q.sAn, q.r, q.sRm, q.sRn, (char*)ws + qbytes,
                           slice - qbytes, s);
      if (st) return st;
      TN_CUDA(cudaMemcpyAsync(q.a, qs, sizeof(double) * (size_t)q.m * q.n, cudaMemcpyDeviceToDevice, s));
    }
    return TN_OK;
  }
  Lanes* L = nullptr;
  std::lock_guard<std::mutex> lk(g_lanes_mu);
  int st = lanes_of_device(&L);
  if (st) return st;
  int* main_err = nullptr;
  if ((st = tn_error_word(s, &main_err))) return st;
  TN_CUDA(cudaEventRecord(L->fork, s));
  for (int i = 0; i < nl; ++i) TN_CUDA(cudaStreamWaitEvent(L->s[i], L->fork, 0));
  for (size_t j = 0; j < big.size(); ++j) {
    const tn_qr_item& q = big[j];
    const int lane = (int)(j % nl);
    cudaStream_t ls = L->s[lane];
    char* base = (char*)ws + (size_t)lane * slice;
    double* qs = (double*)base;
    const size_t qbytes = al(sizeof(double) * (size_t)q.m * q.n);
    if ((st = tn_qr_mixed(q.m, q.n, q.a, q.sAm, q.sAn, qs, q.sAm, q.sAn, q.r, q.sRm, q.sRn, base + qbytes,
                          slice - qbytes, ls)))
      return st;
    TN_CUDA(cudaMemcpyAsync(q.a, qs, sizeof(double) * (size_t)q.m * q.n, cudaMemcpyDeviceToDevice, ls));
  }
  for (int i = 0; i < nl; ++i) {
    TN_CUDA(cudaEventRecord(L->join[i], L->s[i]));
    TN_CUDA(cudaStreamWaitEvent(s, L->join[i], 0));
    int* lane_err = nullptr;
    if ((st = tn_error_word(L->s[i], &lane_err))) return st;
    move_error_kernel<<<1, 1, 0, s>>>(main_err, lane_err);
    TN_CHECK_LAUNCH();
  }
  return TN_OK;
}

}  // namespace

extern "C" size_t tn_batched_step_workspace_bytes(const tn_batch_step_desc* d, const tn_lanczos_opts* opts) {
  if (!d || !opts) return 0;
  size_t need = 4096;
  need = std::max(need, tn_grouped_ops_workspace_bytes(std::max({d->n_ops1, d->n_ops2, d->n_ops3, 1})));
  std::vector<tn_qr_item> small, big;
  split_qr(d, &small, &big);
  if (!small.empty()) need = std::max(need, tn_batched_qr_mixed_workspace_bytes(small.data(), (int)small.size()));
  if (!big.empty()) need = std::max(need, big_lane_bytes(big) * std::min<size_t>(big.size(), kLanes));
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
  if (!big.empty() && (st = run_big_qr(big, ws, ws_bytes, s))) return st;
  if (d->n_gemm1 > 0 && (st = tn_grouped_gemm(d->precision, d->gemm1, d->n_gemm1, ws, ws_bytes, stream))) return st;
  if (d->n_ops2 > 0 && (st = tn_grouped_ops(d->ops2, d->n_ops2, ws, ws_bytes, stream))) return st;
  if (d->n_gemm2 > 0 && (st = tn_grouped_gemm(d->precision, d->gemm2, d->n_gemm2, ws, ws_bytes, stream))) return st;
  if (d->n_ops3 > 0 && (st = tn_grouped_ops(d->ops3, d->n_ops3, ws, ws_bytes, stream))) return st;
  if (d->n_solves > 0) return tn_batched_lanczos(d->solves, d->n_solves, opts, ws, ws_bytes, results, stream);
  return TN_OK;
}
