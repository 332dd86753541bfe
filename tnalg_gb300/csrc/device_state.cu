// Per-device host state of the library: SM counts, one-time kernel attributes, and the device
// error words that bounded waits and range checks write.
//
// A process may drive several GPUs (one MPS per device, or a multi-job host with jobs on different
// devices), so nothing here is set up once per process: every value is looked up for the device
// that is current when the call is made. Error words are kept per (device, stream): a job's
// kernels record a failure in the word of the stream they run on, and only that stream's
// tn_check_device_status (or the Lanczos convergence check on that stream) reads and clears it, so
// concurrent jobs on their own streams never see or clear each other's errors.
#include <mutex>
#include <unordered_map>

#include "common.cuh"

namespace {

constexpr int kWordsPerDevice = 4096;

struct DeviceRecord {
  std::atomic<int> sm_count{0};
  std::atomic<uint64_t> attrs_set{0};   // bit k: attribute key k applied on this device
  int* words = nullptr;                 // kWordsPerDevice device ints, zeroed at creation
  int next_word = 0;
  std::unordered_map<cudaStream_t, int> word_of;
};

DeviceRecord g_dev[TN_MAX_DEVICES];
std::mutex g_words_mu;
std::mutex g_attr_mu;

}  // namespace

int tn_current_device(int* dev) {
  int d = 0;
  TN_CUDA(cudaGetDevice(&d));
  if (d < 0 || d >= TN_MAX_DEVICES) return tn_fail(TN_ERR_ARG, "device ordinal outside 0..63");
  *dev = d;
  return TN_OK;
}

int tn_sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= TN_MAX_DEVICES) return 152;
  int c = g_dev[dev].sm_count.load(std::memory_order_relaxed);
  if (c == 0) {
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    if (c <= 0) c = 152;
    g_dev[dev].sm_count.store(c, std::memory_order_relaxed);  // every thread computes the same value
  }
  return c;
}

int tn_set_smem_attr_once(int key, const void* func, int bytes) {
  int dev = 0;
  int st = tn_current_device(&dev);
  if (st) return st;
  if (key < 0 || key >= 64) return tn_fail(TN_ERR_ARG, "attribute key outside 0..63");
  const uint64_t bit = 1ull << key;
  if (g_dev[dev].attrs_set.load(std::memory_order_acquire) & bit) return TN_OK;
  std::lock_guard<std::mutex> lk(g_attr_mu);
  if (g_dev[dev].attrs_set.load(std::memory_order_acquire) & bit) return TN_OK;
  TN_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  g_dev[dev].attrs_set.fetch_or(bit, std::memory_order_release);
  return TN_OK;
}

int tn_error_word(cudaStream_t s, int** out) {
  int dev = 0;
  int st = tn_current_device(&dev);
  if (st) return st;
  std::lock_guard<std::mutex> lk(g_words_mu);
  DeviceRecord& r = g_dev[dev];
  if (!r.words) {
    int* p = nullptr;
    TN_CUDA(cudaMalloc(&p, kWordsPerDevice * sizeof(int)));
    cudaError_t e = cudaMemset(p, 0, kWordsPerDevice * sizeof(int));
    if (e != cudaSuccess) {
      cudaFree(p);
      return tn_record_error(e);
    }
    r.words = p;
  }
  auto it = r.word_of.find(s);
  int k;
  if (it != r.word_of.end()) {
    k = it->second;
  } else {
    // after kWordsPerDevice distinct streams the table starts over; a stream then shares a word
    // with a stream created long before it (handles of destroyed streams are never told apart)
    if ((int)r.word_of.size() >= kWordsPerDevice) r.word_of.clear();
    k = r.next_word;
    r.next_word = (r.next_word + 1) % kWordsPerDevice;
    r.word_of.emplace(s, k);
  }
  *out = r.words + k;
  return TN_OK;
}

int tn_error_status(int h, cudaStream_t s) {
  if (!h) return TN_OK;
  int* err;
  int st = tn_error_word(s, &err);
  if (st) return st;
  TN_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  if (h == TN_DEVERR_RANGE)
    return tn_fail(TN_ERR_NUMERIC, "tf32x3 gemm: an operand lies outside the FP32 range (|x| >= 3.4e38)");
  if (h == TN_DEVERR_QR_WAIT) return tn_fail(TN_ERR_TIMEOUT, "qr32 cluster: a bounded panel wait gave up");
  if (h == TN_DEVERR_SVD_WAIT) return tn_fail(TN_ERR_TIMEOUT, "svd: a bounded grid barrier gave up");
  return tn_fail(TN_ERR_TIMEOUT, "tf32x3 gemm: a bounded pipeline wait gave up");
}

int tn_error_check(cudaStream_t s) {
  int* err;
  int st = tn_error_word(s, &err);
  if (st) return st;
  int h = 0;
  TN_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  TN_CUDA(cudaStreamSynchronize(s));
  return tn_error_status(h, s);
}
