// Split-TF32 ("3xTF32") GEMM on the 5th-generation tensor cores (tcgen05), FP64 in/out.
//
// C[z] = alpha * sum_r A[z,r] B[z,r] + beta * Cin[z] for the mixed-precision effective-Hamiltonian
// matvec and environment contractions (the np.dot calls of MPSClass.py:755-776 and
// TensorBasicModule.py:530-619). Every FP64 operand x is split into x_hi = tf32(x) and
// x_lo = tf32(x - x_hi); the tensor cores accumulate hi*hi + hi*lo + lo*hi in FP32 in TMEM,
// which keeps ~FP32 accuracy while running on the TF32 pipe.
//
// Kernel structure (one 128 x BN output tile per CTA, 4 warps):
//   * warp 0 / lane 0: TMA producer, 3-stage ring of {A_hi, A_lo, B_hi, B_lo} K-blocks of 32
//     elements (128 B rows, 128B swizzle), completion tracked by mbarriers;
//   * warp 1 / lane 0: issues tcgen05.mma (M=128, N=BN, K=8) x 3 products x 4 k-steps per
//     K-block into one TMEM accumulator, and tcgen05.commit frees the stage;
//   * all warps: epilogue, tcgen05.ld of the accumulator rows (warp w owns TMEM lanes
//     32w..32w+31), alpha/beta applied in FP64 and stored (or atomically added for split K).
// Every wait is bounded by a clock budget; on timeout the kernel records an error code,
// skips its remaining work and frees its TMEM.
#include <cuda.h>
#include <string.h>

#include <mutex>

#include "common.cuh"
#include "tcgen05.cuh"

size_t tn_matvec_fp64_ws_bytes(const tn_site_desc* ds);
int tn_matvec_fp64_straddle(const tn_site_desc* ds, const double* psi, double* y, double alpha, void* ws,
                            size_t ws_bytes, cudaStream_t s);

namespace {

constexpr int BM = 128;
constexpr int BK = 32;  // fp32 elements per K-block = 128 bytes
constexpr int STAGES = 3;
constexpr int NTHREADS = 128;
using namespace tc;

// K-blocks rotate over NACC accumulators in TMEM (summed in FP64 by the epilogue): each FP32
// tensor-core accumulation chain is NACC times shorter.
constexpr int NACC = 4;

template <int BN>
struct Cfg {
  static constexpr int A_BYTES = BM * BK * 4;
  static constexpr int B_BYTES = BN * BK * 4;
  static constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 + 256;
  static constexpr uint32_t TMEM_COLS = NACC * BN;  // 256 or 512: powers of two
};

template <int BN>
__global__ void __launch_bounds__(NTHREADS, 1)
    tf32x3_gemm_kernel(const __grid_constant__ CUtensorMap mAhi, const __grid_constant__ CUtensorMap mAlo,
                       const __grid_constant__ CUtensorMap mBhi, const __grid_constant__ CUtensorMap mBlo, int M,
                       int N, int K, int R, int ksplit, double* C, int64_t sCm, int64_t sCn, int64_t sCb,
                       const double* Cin, double alpha, double beta, int atomic_out, int* err) {
  using cfg = Cfg<BN>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * cfg::STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accb = empty + STAGES;
  uint32_t* tmem_slot = (uint32_t*)(accb + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_tile = blockIdx.x, m_tile = blockIdx.y;
  const int z = blockIdx.z / ksplit, ks = blockIdx.z % ksplit;
  const int kb_per = (K + BK - 1) / BK;
  const int total_kb = R * kb_per;
  const int chunk = (total_kb + ksplit - 1) / ksplit;
  const int kb0 = ks * chunk;
  const int kb1 = min(total_kb, kb0 + chunk);
  const int nkb = max(0, kb1 - kb0);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accb, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tmem_slot, cfg::TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  auto stage = [&](int s, int part) -> uint8_t* {
    return smem + s * cfg::STAGE_BYTES + (part < 2 ? part * cfg::A_BYTES : 2 * cfg::A_BYTES + (part - 2) * cfg::B_BYTES);
  };

  if (warp == 0 && lane == 0) {
    for (int i = 0; i < nkb; ++i) {
      const int s = i % STAGES, round = i / STAGES;
      if (round > 0 && !mbar_wait(&empty[s], (round - 1) & 1, err, 1)) break;
      mbar_expect_tx(&full[s], cfg::STAGE_BYTES);
      const int kb = kb0 + i;
      const int r = kb / kb_per;
      const int kx = (kb % kb_per) * BK;
      const int zr = z * R + r;
      tma_load_3d(stage(s, 0), &mAhi, &full[s], kx, m_tile * BM, zr);
      tma_load_3d(stage(s, 1), &mAlo, &full[s], kx, m_tile * BM, zr);
      tma_load_3d(stage(s, 2), &mBhi, &full[s], kx, n_tile * BN, zr);
      tma_load_3d(stage(s, 3), &mBlo, &full[s], kx, n_tile * BN, zr);
    }
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = make_idesc(BM, BN);
    bool ok = true;
    for (int i = 0; i < nkb && ok; ++i) {
      const int s = i % STAGES, round = i / STAGES;
      if (!mbar_wait(&full[s], round & 1, err, 2)) { ok = false; break; }
      tc_fence_after();
      const uint64_t dAhi = smem_desc(stage(s, 0)), dAlo = smem_desc(stage(s, 1));
      const uint64_t dBhi = smem_desc(stage(s, 2)), dBlo = smem_desc(stage(s, 3));
      const uint32_t dacc = tmem + (uint32_t)((i % NACC) * BN);
#pragma unroll
      for (int k = 0; k < BK / 8; ++k) {
        const uint64_t o = (uint64_t)(k * 32) >> 4;  // 8 tf32 = 32 bytes along the swizzled row
        mma_tf32(dacc, dAhi + o, dBhi + o, idesc, (i >= NACC || k > 0) ? 1u : 0u);
        mma_tf32(dacc, dAhi + o, dBlo + o, idesc, 1u);
        mma_tf32(dacc, dAlo + o, dBhi + o, idesc, 1u);
      }
      mma_commit(&empty[s]);
    }
    if (nkb > 0) mma_commit(accb);
  }
  __syncwarp();

  bool have = nkb > 0;
  if (have) {
    have = mbar_wait(accb, 0, err, 3);
    tc_fence_after();
  }
  have = __all_sync(0xffffffffu, have);  // tcgen05.ld below is warp-collective
  const int row = m_tile * BM + warp * 32 + lane;
  const int64_t base = (int64_t)z * sCb;
  if (have) {
    // The NACC partial accumulators are summed error-free in FP32 (TwoSum: a head and a tail per
    // element) and widened with integer operations; only the final head + tail, alpha and beta
    // use the FP64 pipe, which issues 64 times fewer lanes per clock than FP32 on this part.
    const int nacc = min(nkb, NACC);
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float hi[16], lo[16];
      {
        uint32_t r[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          hi[j] = __uint_as_float(r[j]);
          lo[j] = 0.f;
        }
      }
#pragma unroll 1
      for (int a = 1; a < nacc; ++a) {
        uint32_t r[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(a * BN + c0), r);
#pragma unroll
        for (int j = 0; j < 16; ++j) two_sum_acc(hi[j], lo[j], __uint_as_float(r[j]));
      }
      if (row < M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = n_tile * BN + c0 + j;
          if (col < N) {
            const int64_t off = base + (int64_t)row * sCm + (int64_t)col * sCn;
            const double sum = f32_to_f64(hi[j]) + f32_to_f64(lo[j]);
            const double v = (alpha == 1.0) ? sum : alpha * sum;
            if (atomic_out) atomicAdd(C + off, v);
            else C[off] = (beta == 0.0) ? v : fma(beta, (Cin ? Cin : C)[off], v);
          }
        }
      }
    }
  } else if (!atomic_out && row < M && nkb == 0) {
    for (int col = n_tile * BN; col < min(N, n_tile * BN + BN); ++col) {
      const int64_t off = base + (int64_t)row * sCm + (int64_t)col * sCn;
      C[off] = (beta == 0.0) ? 0.0 : beta * (Cin ? Cin : C)[off];
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, cfg::TMEM_COLS);
}

// ---------------------------------------------------------------------------
// FP64 -> (tf32 hi, tf32 lo) staging, K-major rows of pitch Kp (multiple of 4).

struct PrepArgs {
  const double* src;
  int64_t Z, R, rows, K;
  int64_t sZ, sR, sRow, sK;
  float *hi, *lo;
  int64_t Kp;
  int* err;  // set by prep(): the kernels' device error word
};

constexpr int kErrRange = TN_DEVERR_RANGE;

__device__ __forceinline__ void stage_value(const PrepArgs& a, double x, int64_t o) {
  float h, l;
  split_tf32(x, h, l);
  if (!isfinite(h) && finite_f64(x)) atomicExch(a.err, kErrRange);
  a.hi[o] = h;
  a.lo[o] = l;
}

// Both prep kernels also write zeros into the pitch padding k in [K, Kp): the staging buffers are
// reused scratch, and the padding must never feed the product whatever the tensor map's bounds.
// prep_direct: block (64, 4) = 64 consecutive k of 4 staged rows; every thread stages 4 elements
// 64 apart with its row index split once (staged row g = zr * rows + row, zr = z * R + r).
constexpr int PD_K = 64, PD_ROWS = 4, PD_PER = 4;
__global__ void __launch_bounds__(PD_K * PD_ROWS) prep_direct_kernel(PrepArgs a) {
  const int64_t g = (int64_t)blockIdx.x * PD_ROWS + threadIdx.y;
  if (g >= a.Z * a.R * a.rows) return;
  const int64_t zr = g / a.rows, row = g - zr * a.rows;
  const int64_t z = zr / a.R, r = zr - z * a.R;
  const double* src = a.src + z * a.sZ + r * a.sR + row * a.sRow;
  const int64_t k0 = (int64_t)blockIdx.y * (PD_K * PD_PER) + threadIdx.x;
  double x[PD_PER];
#pragma unroll
  for (int i = 0; i < PD_PER; ++i) {
    const int64_t k = k0 + i * PD_K;
    x[i] = (k < a.K) ? src[k * a.sK] : 0.0;
  }
#pragma unroll
  for (int i = 0; i < PD_PER; ++i) {
    const int64_t k = k0 + i * PD_K;
    if (k < a.Kp) stage_value(a, x[i], g * a.Kp + k);
  }
}

// sRow == 1: read 32x32 tiles along rows, write along K.
__global__ void prep_transpose_kernel(PrepArgs a) {
  __shared__ double tile[32][33];
  const int64_t zr = blockIdx.z;
  const int64_t z = zr / a.R, r = zr % a.R;
  const int64_t k0 = (int64_t)blockIdx.y * 32, r0 = (int64_t)blockIdx.x * 32;
  const double* src = a.src + z * a.sZ + r * a.sR;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int64_t k = k0 + i, row = r0 + threadIdx.x;
    tile[i][threadIdx.x] = (k < a.K && row < a.rows) ? src[row + k * a.sK] : 0.0;
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int64_t row = r0 + i, k = k0 + threadIdx.x;
    // the grid's K extent, cdiv(K, 32) * 32, covers Kp; the tile holds zeros for k >= K
    if (row < a.rows && k < a.Kp) stage_value(a, tile[threadIdx.x][i], (zr * a.rows + row) * a.Kp + k);
  }
}

__global__ void scale_out_kernel(int64_t Z, int64_t M, int64_t N, double* C, int64_t sCm, int64_t sCn, int64_t sCb,
                                 const double* Cin, double beta) {
  const int64_t total = Z * M * N;
  const double* src = Cin ? Cin : C;
  if (Z == 1 && M == 1 && sCn == 1) {  // one contiguous vector: no index arithmetic
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N; idx += (int64_t)gridDim.x * blockDim.x)
      C[idx] = (beta == 0.0) ? 0.0 : beta * src[idx];
    return;
  }
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t z = idx / (M * N), e = idx % (M * N);
    const int64_t off = z * sCb + (e / N) * sCm + (e % N) * sCn;
    C[off] = (beta == 0.0) ? 0.0 : beta * src[off];
  }
}

int blocks_for(int64_t total) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(total, 256), 16LL * tn_sm_count()));
}

int prep(const PrepArgs& args, cudaStream_t s) {
  if (args.Z * args.R * args.rows * args.K == 0) return TN_OK;
  PrepArgs a = args;
  int st = tn_error_word(s, &a.err);
  if (st) return st;
  if (a.sRow == 1 && a.sK != 1) {
    dim3 grid((unsigned)tn_cdiv(a.rows, 32), (unsigned)tn_cdiv(a.K, 32), (unsigned)(a.Z * a.R));
    if (grid.z > 65535u || grid.y > 65535u) return tn_fail(TN_ERR_ARG, "tf32 prep: grid too large");
    prep_transpose_kernel<<<grid, dim3(32, 8), 0, s>>>(a);
  } else {
    const int64_t nrows = a.Z * a.R * a.rows;
    const int64_t kchunks = tn_cdiv(a.Kp, PD_K * PD_PER);
    if (kchunks > 65535 || tn_cdiv(nrows, PD_ROWS) > 0x7fffffffLL) return tn_fail(TN_ERR_ARG, "tf32 prep: grid too large");
    prep_direct_kernel<<<dim3((unsigned)tn_cdiv(nrows, PD_ROWS), (unsigned)kchunks), dim3(PD_K, PD_ROWS), 0, s>>>(a);
  }
  TN_CHECK_LAUNCH();
  return TN_OK;
}

// ---------------------------------------------------------------------------
// Tensor maps through the driver entry point (no link-time dependency on libcuda).

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  // resolved once; the initialisation of a function-local static is thread-safe
  static const EncodeTiledFn fn = []() -> EncodeTiledFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (EncodeTiledFn)p;
    return nullptr;
  }();
  return fn;
}

int make_map(CUtensorMap* m, const float* base, int64_t K, int64_t rows, int64_t nmat, int64_t Kp, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return tn_fail(TN_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  if (((uintptr_t)base & 15) || (Kp * 4) % 16) return tn_fail(TN_ERR_ARG, "tf32 operand misaligned");
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)nmat};
  cuuint64_t strides[2] = {(cuuint64_t)(Kp * 4), (cuuint64_t)(rows * Kp * 4)};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return tn_fail(TN_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return TN_OK;
}

int64_t padk(int64_t K) { return (K + 3) / 4 * 4; }
size_t al(size_t x) { return (x + 1023) / 1024 * 1024; }

struct Staged {
  float *hi, *lo;
  int64_t rows, K, Kp, nmat;
};

size_t staged_bytes(int64_t rows, int64_t K, int64_t nmat) { return 2 * al((size_t)nmat * rows * padk(K) * 4); }

Staged carve(char*& p, int64_t rows, int64_t K, int64_t nmat) {
  Staged st;
  st.rows = rows; st.K = K; st.Kp = padk(K); st.nmat = nmat;
  const size_t b = al((size_t)nmat * rows * st.Kp * 4);
  st.hi = (float*)p; p += b;
  st.lo = (float*)p; p += b;
  return st;
}

template <int BN>
int launch_kernel(const Staged& A, const Staged& B, int64_t M, int64_t N, int64_t K, int64_t Z, int64_t R,
                  double* C, int64_t sCm, int64_t sCn, int64_t sCb, const double* Cin, double alpha, double beta,
                  bool atomic_out, int ksplit, cudaStream_t s) {
  using cfg = Cfg<BN>;
  CUtensorMap ma[2], mb[2];
  int st;
  if ((st = make_map(&ma[0], A.hi, K, M, Z * R, A.Kp, BM))) return st;
  if ((st = make_map(&ma[1], A.lo, K, M, Z * R, A.Kp, BM))) return st;
  if ((st = make_map(&mb[0], B.hi, K, N, Z * R, B.Kp, BN))) return st;
  if ((st = make_map(&mb[1], B.lo, K, N, Z * R, B.Kp, BN))) return st;
  if ((st = tn_set_smem_attr_once(BN == 128 ? TN_ATTR_TF32_BN128 : TN_ATTR_TF32_BN64,
                                   (const void*)tf32x3_gemm_kernel<BN>, cfg::SMEM)))
    return st;
  int* err;
  if ((st = tn_error_word(s, &err))) return st;
  dim3 grid((unsigned)tn_cdiv(N, BN), (unsigned)tn_cdiv(M, BM), (unsigned)(Z * ksplit));
  if (grid.y > 65535u || grid.z > 65535u) return tn_fail(TN_ERR_ARG, "tf32 gemm grid too large");
  tf32x3_gemm_kernel<BN><<<grid, NTHREADS, cfg::SMEM, s>>>(ma[0], ma[1], mb[0], mb[1], (int)M, (int)N, (int)K,
                                                           (int)R, ksplit, C, sCm, sCn, sCb, Cin, alpha, beta,
                                                           atomic_out ? 1 : 0, err);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

// Tile width and K split for a problem: fill the SMs with at least ~one CTA each.
void plan(int64_t M, int64_t N, int64_t K, int64_t Z, int64_t R, int* bn, int* ksplit) {
  const int64_t sms = tn_sm_count();
  *bn = (tn_cdiv(M, BM) * tn_cdiv(N, 128) * Z >= sms) ? 128 : 64;
  const int64_t tiles = tn_cdiv(M, BM) * tn_cdiv(N, *bn) * Z;
  const int64_t kbs = R * tn_cdiv(K, BK);
  int ks = 1;
  while (tiles * ks * 2 <= sms && kbs / (ks * 2) >= 8 && ks < 8) ks *= 2;
  *ksplit = ks;
}

int gemm_staged(const Staged& A, const Staged& B, int64_t M, int64_t N, int64_t K, int64_t Z, int64_t R, double* C,
                int64_t sCm, int64_t sCn, int64_t sCb, const double* Cin, double alpha, double beta, bool accumulate,
                cudaStream_t s) {
  // accumulate: C already holds beta*Cin (caller initialised it); add alpha*A.B atomically.
  int bn, ks;
  plan(M, N, K, Z, R, &bn, &ks);
  bool atomic_out = accumulate || ks > 1;
  if (ks > 1 && !accumulate) {
    scale_out_kernel<<<blocks_for(Z * M * N), 256, 0, s>>>(Z, M, N, C, sCm, sCn, sCb, Cin, beta);
    TN_CHECK_LAUNCH();
  }
  if (bn == 128)
    return launch_kernel<128>(A, B, M, N, K, Z, R, C, sCm, sCn, sCb, Cin, alpha, beta, atomic_out, ks, s);
  return launch_kernel<64>(A, B, M, N, K, Z, R, C, sCm, sCn, sCb, Cin, alpha, beta, atomic_out, ks, s);
}

}  // namespace

bool tn_tf32x3_supported() {
  int dev = 0, maj = 0, min = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  cudaDeviceGetAttribute(&maj, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&min, cudaDevAttrComputeCapabilityMinor, dev);
  return maj == 10 && min == 3 && encode_fn() != nullptr;
}

size_t tn_gemm_tf32x3_ws_bytes(int64_t M, int64_t N, int64_t K, int64_t batch, int64_t nred) {
  const int64_t zr = batch * std::max<int64_t>(nred, 1);
  return staged_bytes(M, K, zr) + staged_bytes(N, K, zr) + 4096;
}

int tn_gemm_tf32x3(const TnGemmF64& g, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (!tn_tf32x3_supported()) return tn_fail(TN_ERR_ARG, "tf32x3 needs an sm_103 device");
  if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return TN_OK;
  if (g.M > (1LL << 30) || g.N > (1LL << 30) || g.K > (1LL << 30)) return tn_fail(TN_ERR_ARG, "tf32 gemm too large");
  const int64_t Z = g.batch, R = std::max<int64_t>(g.nred, 1);
  if (g.K <= 0 || g.nred <= 0) {
    scale_out_kernel<<<blocks_for(Z * g.M * g.N), 256, 0, s>>>(Z, g.M, g.N, g.C, g.sCm, g.sCn, g.sCb, g.Cin, g.beta);
    TN_CHECK_LAUNCH();
    return TN_OK;
  }
  const size_t need = staged_bytes(g.M, g.K, Z * R) + staged_bytes(g.N, g.K, Z * R) + 2048;
  if (!ws || ws_bytes < need) return tn_fail(TN_ERR_WORKSPACE, "tf32 gemm: workspace too small");
  char* p = (char*)(((uintptr_t)ws + 1023) & ~(uintptr_t)1023);
  Staged A = carve(p, g.M, g.K, Z * R);
  Staged B = carve(p, g.N, g.K, Z * R);
  PrepArgs pa{g.A, Z, R, g.M, g.K, g.sAb, g.sAr, g.sAm, g.sAk, A.hi, A.lo, A.Kp};
  int st = prep(pa, s);
  if (st) return st;
  PrepArgs pb{g.B, Z, R, g.N, g.K, g.sBb, g.sBr, g.sBn, g.sBk, B.hi, B.lo, B.Kp};
  if ((st = prep(pb, s))) return st;
  return gemm_staged(A, B, g.M, g.N, g.K, Z, R, g.C, g.sCm, g.sCn, g.sCb, g.Cin, g.alpha, g.beta, false, s);
}

// ---------------------------------------------------------------------------
// Mixed-precision matvec: WL and WR staged once per local solve, psi staged per call.

namespace {
struct MvLayout {
  Staged wl, wr, psi, psit;
  Staged sl, sr, psiz, zs;  // straddling pairs: stacked SL, SR blocks, psi for SL psi, Z for Z SR^T
  char* fp64_ws;            // Z = [SL_1; ...] psi (FP64, nstr x chil d chir) first
  size_t fp64_bytes;
};

size_t mv_layout(const tn_site_desc* d, char* base, MvLayout* L) {
  const int64_t cl = d->chil, dd = d->d, cr = d->chir;
  char* p = base ? (char*)(((uintptr_t)base + 1023) & ~(uintptr_t)1023) : nullptr;
  size_t off = 1024;
  auto take = [&](int64_t rows, int64_t K, Staged* st, int64_t nmat = 1) {
    const size_t b = staged_bytes(rows, K, nmat);
    if (p) {
      char* q = p;
      *st = carve(q, rows, K, nmat);
      p += b;
    }
    off += b;
  };
  take(cl * dd, cl * dd, &L->wl);
  take(dd * cr, dd * cr, &L->wr);
  take(cl, dd * cr, &L->psi);
  take(cr, cl * dd, &L->psit);
  if (d->nstr > 0) {
    const int64_t ng = d->nstr;
    take(ng * cl, cl, &L->sl);     // A of Z = [SL_1; ...; SL_ng] psi: the SL blocks stacked by rows
    take(dd * cr, cl, &L->psiz);   // B of the same product: psi read with (s b) as the row, a as k
    take(cl * dd, cr, &L->zs, ng);  // A of y += sum_g Z_g SR_g^T
    take(cr, cr, &L->sr, ng);       // B of the same product: SR_g as stored
  }
  const size_t fb = tn_matvec_fp64_ws_bytes(d) + (size_t)8 * d->nstr * cl * dd * cr + 4096;
  if (p) {
    L->fp64_ws = p;
    L->fp64_bytes = fb;
  }
  off += fb;
  return off;
}
}  // namespace

size_t tn_matvec_fp64_ws_bytes(const tn_site_desc* ds);
int tn_matvec_fp64_straddle(const tn_site_desc* ds, const double* psi, double* y, double alpha, void* ws,
                            size_t ws_bytes, cudaStream_t s);

size_t tn_matvec_tf32x3_ws_bytes(const tn_site_desc* d) {
  MvLayout L;
  return mv_layout(d, nullptr, &L);
}

// The FP64 scratch region inside a split-TF32 matvec workspace: an FP64 matvec run between
// split-TF32 ones (the FP64 steps of a refined Lanczos solve) must use this region, not the start
// of the workspace, where the staged hi/lo copies of WL, WR, SL and SR live.
int tn_matvec_tf32x3_fp64_region(const tn_site_desc* d, void* ws, size_t ws_bytes, void** out, size_t* out_bytes) {
  MvLayout L;
  if (!ws || ws_bytes < mv_layout(d, nullptr, &L)) return tn_fail(TN_ERR_WORKSPACE, "tf32 matvec: workspace");
  mv_layout(d, (char*)ws, &L);
  *out = L.fp64_ws;
  *out_bytes = L.fp64_bytes;
  return TN_OK;
}

int tn_tf32x3_prepare_static(const tn_site_desc* d, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (!tn_tf32x3_supported()) return tn_fail(TN_ERR_ARG, "tf32x3 needs an sm_103 device");
  MvLayout L;
  if (!ws || ws_bytes < mv_layout(d, nullptr, &L)) return tn_fail(TN_ERR_WORKSPACE, "tf32 matvec: workspace");
  mv_layout(d, (char*)ws, &L);
  const int64_t cl = d->chil, dd = d->d, cr = d->chir;
  int st;
  if (d->wl) {
    PrepArgs a{d->wl, 1, 1, cl * dd, cl * dd, 0, 0, cl * dd, 1, L.wl.hi, L.wl.lo, L.wl.Kp};
    if ((st = prep(a, s))) return st;
  }
  if (d->wr) {
    PrepArgs a{d->wr, 1, 1, dd * cr, dd * cr, 0, 0, dd * cr, 1, L.wr.hi, L.wr.lo, L.wr.Kp};
    if ((st = prep(a, s))) return st;
  }
  if (d->nstr > 0) {
    const int64_t ng = d->nstr;
    PrepArgs a{d->sl, 1, 1, ng * cl, cl, 0, 0, cl, 1, L.sl.hi, L.sl.lo, L.sl.Kp};
    if ((st = prep(a, s))) return st;
    PrepArgs b{d->sr, 1, ng, cr, cr, 0, cr * cr, cr, 1, L.sr.hi, L.sr.lo, L.sr.Kp};
    if ((st = prep(b, s))) return st;
  }
  return TN_OK;
}

int tn_matvec_tf32x3(const tn_site_desc* d, const double* psi, double* y, double alpha, double beta, void* ws,
                     size_t ws_bytes, cudaStream_t s) {
  MvLayout L;
  if (!ws || ws_bytes < mv_layout(d, nullptr, &L)) return tn_fail(TN_ERR_WORKSPACE, "tf32 matvec: workspace");
  mv_layout(d, (char*)ws, &L);
  const int64_t cl = d->chil, dd = d->d, cr = d->chir;
  const int64_t n = cl * dd * cr;
  int st;
  // y = beta * psi, then every product is added atomically
  if (beta == 0.0) {
    TN_CUDA(cudaMemsetAsync(y, 0, (size_t)n * sizeof(double), s));
  } else {
    scale_out_kernel<<<blocks_for(n), 256, 0, s>>>(1, 1, n, y, 0, 1, 0, psi, beta);
    TN_CHECK_LAUNCH();
  }
  if (d->wl) {
    // psi^T staged: B-op[n = b][k = (a s)] = psi[(a s) * cr + b]
    PrepArgs pt{psi, 1, 1, cr, cl * dd, 0, 0, 1, cr, L.psit.hi, L.psit.lo, L.psit.Kp};
    if ((st = prep(pt, s))) return st;
    if ((st = gemm_staged(L.wl, L.psit, cl * dd, cr, cl * dd, 1, 1, y, cr, 1, 0, nullptr, alpha, 1.0, true, s)))
      return st;
  }
  if (d->wr) {
    PrepArgs pp{psi, 1, 1, cl, dd * cr, 0, 0, dd * cr, 1, L.psi.hi, L.psi.lo, L.psi.Kp};
    if ((st = prep(pp, s))) return st;
    if ((st = gemm_staged(L.psi, L.wr, cl, dd * cr, dd * cr, 1, 1, y, dd * cr, 1, 0, nullptr, alpha, 1.0, true, s)))
      return st;
  }
  if (d->nstr > 0) {
    // straddling pairs (absent in nearest-neighbour chains), the products of the FP64 path
    // (tn_matvec_fp64_straddle) in split TF32: Z = [SL_1; ...; SL_ng] psi as one GEMM, whose
    // (ng chil) x (d chir) output is Z_g stacked, then y += alpha sum_g Z_g SR_g^T, one GEMM
    // reduced over g
    const int64_t ng = d->nstr;
    double* Z = (double*)L.fp64_ws;
    PrepArgs pz{psi, 1, 1, dd * cr, cl, 0, 0, 1, dd * cr, L.psiz.hi, L.psiz.lo, L.psiz.Kp};
    if ((st = prep(pz, s))) return st;
    if ((st = gemm_staged(L.sl, L.psiz, ng * cl, dd * cr, cl, 1, 1, Z, dd * cr, 1, 0, nullptr, 1.0, 0.0, false, s)))
      return st;
    PrepArgs pa{Z, 1, ng, cl * dd, cr, 0, n, cr, 1, L.zs.hi, L.zs.lo, L.zs.Kp};
    if ((st = prep(pa, s))) return st;
    if ((st = gemm_staged(L.zs, L.sr, cl * dd, cr, cr, 1, ng, y, cr, 1, 0, nullptr, alpha, 1.0, true, s)))
      return st;
  }
  return TN_OK;
}
