// Grouped GEMMs: many independent contractions of uneven shapes in one launch.
//
// The batched DMRG path advances many independent jobs (chains of different lengths and bond
// dimensions) one local update at a time; every local update is a handful of dense contractions
// per job (the block matvec WL.psi + psi.WR^T of MPSClass.py:755-776, the environment transfers
// of TensorBasicModule.py:530-619, the R-absorb of :387-424). A group lists them all; one launch
// runs every output tile of every problem.
//
// Split-TF32 (tcgen05) path:
//   1. gg_stage_kernel: every operand (A as rows m, B as rows n; both K-contiguous) is converted
//      from FP64 to (tf32 hi, tf32 lo) pairs in 128-row x 32-element tiles whose 128-byte rows are
//      already in the 128B-swizzled order the tensor-core descriptors read, so a tile moves to
//      shared memory with one untiled bulk copy (cp.async.bulk), with no tensor map per problem;
//      rows and K past the operand's extent are written as zeros.
//   2. gg_tf32x3_kernel: a persistent kernel, one CTA per SM; each CTA walks the flattened tile
//      list (problem found by binary search in the tile prefix), with a 3-stage bulk-copy ring,
//      one thread issuing tcgen05.mma.kind::tf32 (hi.hi + hi.lo + lo.hi) into NACC rotating TMEM
//      accumulators, and all four warps in the epilogue (TwoSum of the partial accumulators,
//      FP64 out, plain store or atomic add).
// FP64 path: gg_f64_kernel, 64 x 64 CUDA-core tiles over the same flattened tile list.
//
// Every mbarrier wait is bounded; on a timeout the CTA records an error in the stream's error
// word, waits (bounded) for the bulk copies it issued, frees its TMEM and returns.
#include <string.h>

#include <vector>

#include "common.cuh"
#include "grouped.cuh"
#include "tcgen05.cuh"

using namespace tc;

namespace {

constexpr int BM = 128;
constexpr int BK = 32;
constexpr int STAGES = 3;
constexpr int NTHREADS = 128;
constexpr int NACC = 4;
constexpr int TILE_FLOATS = BM * BK;          // one 128 x 32 tf32 tile (16 KB)
constexpr int PAIR_FLOATS = 2 * TILE_FLOATS;  // hi tile, then lo tile

template <int BN>
struct GgCfg {
  static constexpr int A_BYTES = BM * BK * 4;
  static constexpr int B_BYTES = BN * BK * 4;
  static constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 + 256;
  static constexpr uint32_t TMEM_COLS = NACC * BN;
};

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// swizzled position of element (row, k) inside a 128-row x 32 tile: 128-byte rows, 16-byte chunk
// index XOR (row mod 8) -- the layout of a TMA SWIZZLE_128B box, which the descriptors expect
__device__ __forceinline__ int swz(int row, int k) { return row * BK + ((((k >> 2) ^ (row & 7)) << 2) | (k & 3)); }

__device__ __forceinline__ int find_item(const int* prefix, int n, int t) {
  int lo = 0, hi = n;  // prefix[lo] <= t < prefix[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// staging: one CTA per 128 x 32 tile of one operand

__global__ void __launch_bounds__(256) gg_stage_kernel(const GgStage* items, int nitems, const int* prefix, int* err) {
  __shared__ double tile[BM][BK + 1];
  const int t = blockIdx.x;
  const int i = find_item(prefix, nitems, t);
  const GgStage it = items[i];
  if (it.active && *it.active == 0) return;
  const int local = t - prefix[i];
  const int per_red = it.n_rt * it.n_kb;
  const int r = local / per_red;
  const int rt = (local % per_red) / it.n_kb, kb = local % it.n_kb;
  const double* src = it.src + (int64_t)r * it.s_red;
  const int row0 = rt * BM, k0 = kb * BK;
  if (it.s_k == 1 || it.s_row != 1) {
    for (int e = threadIdx.x; e < BM * BK; e += blockDim.x) {
      const int row = e >> 5, k = e & 31;
      const int gr = row0 + row, gk = k0 + k;
      tile[row][k] = (gr < it.rows && gk < it.K) ? src[(int64_t)gr * it.s_row + (int64_t)gk * it.s_k] : 0.0;
    }
  } else {  // rows contiguous: walk rows with the lanes
    for (int e = threadIdx.x; e < BM * BK; e += blockDim.x) {
      const int row = e & (BM - 1), k = e >> 7;
      const int gr = row0 + row, gk = k0 + k;
      tile[row][k] = (gr < it.rows && gk < it.K) ? src[(int64_t)gr + (int64_t)gk * it.s_k] : 0.0;
    }
  }
  __syncthreads();
  float* hi = it.dst + (size_t)local * PAIR_FLOATS;
  float* lo = hi + TILE_FLOATS;
  for (int e = threadIdx.x; e < BM * BK; e += blockDim.x) {
    const int row = e >> 5, k = e & 31;
    const double x = tile[row][k];
    float h, l;
    split_tf32(x, h, l);
    if (!isfinite(h) && isfinite(x)) atomicExch(err, TN_DEVERR_RANGE);
    const int o = swz(row, k);
    hi[o] = h;
    lo[o] = l;
  }
}

// ---------------------------------------------------------------------------
// split-TF32 grouped GEMM

template <int BN>
__global__ void __launch_bounds__(NTHREADS, 1)
    gg_tf32x3_kernel(const GgProblem* probs, int nprobs, const int* prefix, int total_tiles, int* err) {
  using cfg = GgCfg<BN>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * cfg::STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accb = empty + STAGES;
  uint32_t* tmem_slot = (uint32_t*)(accb + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
  volatile int* consumed = abort_flag + 1;  // k-blocks the MMA thread has taken (for the abort drain)

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accb, 1);
    *abort_flag = 0;
    *consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tmem_slot, cfg::TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  auto stage = [&](int s) -> uint8_t* { return smem + s * cfg::STAGE_BYTES; };

  uint32_t issued = 0;    // k-blocks issued by the producer (ring position), thread 0 only
  uint32_t taken = 0;     // k-blocks consumed by the MMA thread, thread 32 only
  uint32_t acc_uses = 0;  // tiles that committed the accumulator barrier (its parity)
  for (int t = blockIdx.x; t < total_tiles; t += gridDim.x) {
    if (*abort_flag) break;
    const int p = find_item(prefix, nprobs, t);
    const GgProblem P = probs[p];
    const int local = t - prefix[p];
    const int per_z = P.n_mt * P.n_nt;
    const int z = local / per_z;
    const int mt = (local % per_z) / P.n_nt, nt = local % P.n_nt;
    const bool skip = P.active && *P.active == 0;
    const int nkb = skip ? 0 : P.n_kb * P.nred;
    double* const Cz = P.C + (int64_t)z * P.sCb;

    if (warp == 0 && lane == 0) {
      const int b_rt = (nt * BN) / BM, b_half = (nt * BN) % BM;  // B rows of this tile in its 128-row tile
      for (int i = 0; i < nkb; ++i, ++issued) {
        const int s = issued % STAGES;
        const uint32_t round = issued / STAGES;
        if (round > 0 && !mbar_wait(&empty[s], (round - 1) & 1, err, 1)) { *abort_flag = 1; break; }
        const int r = z * P.nred + i / P.n_kb, kb = i % P.n_kb;
        const float* a = P.a + ((size_t)(r * P.a_nrt + mt) * P.n_kb + kb) * PAIR_FLOATS;
        const float* b = P.b + ((size_t)(r * P.b_nrt + b_rt) * P.n_kb + kb) * PAIR_FLOATS;
        mbar_expect_tx(&full[s], cfg::STAGE_BYTES);
        bulk_load(stage(s), a, 2 * cfg::A_BYTES, &full[s]);
        if (BN == BM) {
          bulk_load(stage(s) + 2 * cfg::A_BYTES, b, 2 * cfg::B_BYTES, &full[s]);
        } else {
          bulk_load(stage(s) + 2 * cfg::A_BYTES, b + b_half * BK, cfg::B_BYTES, &full[s]);
          bulk_load(stage(s) + 2 * cfg::A_BYTES + cfg::B_BYTES, b + TILE_FLOATS + b_half * BK, cfg::B_BYTES,
                    &full[s]);
        }
      }
    } else if (warp == 1 && lane == 0) {
      constexpr uint32_t idesc = make_idesc(BM, BN);
      for (int i = 0; i < nkb; ++i, ++taken) {
        const int s = taken % STAGES;
        const uint32_t round = taken / STAGES;
        if (!mbar_wait(&full[s], round & 1, err, 2)) { *abort_flag = 1; break; }
        *consumed = (int)taken + 1;
        tc_fence_after();
        const uint64_t dAhi = smem_desc(stage(s)), dAlo = smem_desc(stage(s) + cfg::A_BYTES);
        const uint64_t dBhi = smem_desc(stage(s) + 2 * cfg::A_BYTES);
        const uint64_t dBlo = smem_desc(stage(s) + 2 * cfg::A_BYTES + cfg::B_BYTES);
        const uint32_t dacc = tmem + (uint32_t)((i % NACC) * BN);
#pragma unroll
        for (int k = 0; k < BK / 8; ++k) {
          const uint64_t o = (uint64_t)(k * 32) >> 4;
          mma_tf32(dacc, dAhi + o, dBhi + o, idesc, (i >= NACC || k > 0) ? 1u : 0u);
          mma_tf32(dacc, dAhi + o, dBlo + o, idesc, 1u);
          mma_tf32(dacc, dAlo + o, dBhi + o, idesc, 1u);
        }
        mma_commit(&empty[s]);
      }
      if (nkb > 0) mma_commit(accb);
    }
    __syncwarp();
    __syncthreads();  // abort_flag is final for this tile
    if (nkb > 0) {
      bool have = !*abort_flag;
      if (have) {
        have = mbar_wait(accb, acc_uses & 1, err, 3);
        tc_fence_after();
      }
      ++acc_uses;
      have = __all_sync(0xffffffffu, have);
      const int row = mt * BM + warp * 32 + lane;
      if (have) {
        const int nacc = min(nkb, NACC);
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
          float hi[16], lo[16];
          {
            uint32_t rr[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, rr);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              hi[j] = __uint_as_float(rr[j]);
              lo[j] = 0.f;
            }
          }
#pragma unroll 1
          for (int a = 1; a < nacc; ++a) {
            uint32_t rr[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(a * BN + c0), rr);
#pragma unroll
            for (int j = 0; j < 16; ++j) two_sum_acc(hi[j], lo[j], __uint_as_float(rr[j]));
          }
          if (row < P.M) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int col = nt * BN + c0 + j;
              if (col < P.N) {
                double* c = Cz + (int64_t)row * P.sCm + (int64_t)col * P.sCn;
                const double v = P.alpha * (f32_to_f64(hi[j]) + f32_to_f64(lo[j]));
                if (P.accumulate) atomicAdd(c, v);
                else *c = (P.beta == 0.0) ? v : fma(P.beta, *c, v);
              }
            }
          }
        }
      }
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
    } else if (!skip && !P.accumulate && P.n_kb * P.nred == 0) {
      // K == 0: C = beta C
      const int row = mt * BM + warp * 32 + lane;
      if (row < P.M)
        for (int col = nt * BN; col < min(P.N, nt * BN + BN); ++col) {
          double* c = Cz + (int64_t)row * P.sCm + (int64_t)col * P.sCn;
          *c = (P.beta == 0.0) ? 0.0 : P.beta * *c;
        }
    }
  }
  __syncthreads();
  if (*abort_flag && threadIdx.x == 0) {
    // drain: every bulk copy this CTA issued must land before its shared memory is released
    for (uint32_t q = (uint32_t)*consumed; q < issued; ++q)
      if (!mbar_wait(&full[q % STAGES], (q / STAGES) & 1, err, 4)) break;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, cfg::TMEM_COLS);
}

// ---------------------------------------------------------------------------
// FP64 grouped GEMM on the CUDA cores: 64 x 64 output tiles, 256 threads with 4 x 4 micro-tiles.

constexpr int FT = 64, FK = 16, FNT = 256;

__global__ void __launch_bounds__(FNT) gg_f64_kernel(const GgF64Problem* probs, int nprobs, const int* prefix) {
  __shared__ double As[FK][FT + 1];
  __shared__ double Bs[FK][FT + 1];
  const int t = blockIdx.x;
  const int p = find_item(prefix, nprobs, t);
  const GgF64Problem P = probs[p];
  if (P.active && *P.active == 0) return;
  const int local0 = t - prefix[p];
  const int n_nt = (P.N + FT - 1) / FT, n_mt = (P.M + FT - 1) / FT;
  const int z = local0 / (n_mt * n_nt), local = local0 % (n_mt * n_nt);
  const int64_t m0 = (int64_t)(local / n_nt) * FT, n0 = (int64_t)(local % n_nt) * FT;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const bool a_kc = (P.sAk == 1), b_nc = (P.sBn == 1);
  double acc[4][4] = {};
  for (int r = 0; r < P.nred; ++r) {
    const double* A = P.A + (int64_t)z * P.sAb + (int64_t)r * P.sAr;
    const double* B = P.B + (int64_t)z * P.sBb + (int64_t)r * P.sBr;
    for (int64_t k0 = 0; k0 < P.K; k0 += FK) {
      for (int e = tid; e < FT * FK; e += FNT) {
        int mm, kk;
        if (a_kc) { mm = e / FK; kk = e % FK; } else { kk = e / FT; mm = e % FT; }
        const int64_t gm = m0 + mm, gk = k0 + kk;
        As[kk][mm] = (gm < P.M && gk < P.K) ? A[gm * P.sAm + gk * P.sAk] : 0.0;
      }
      for (int e = tid; e < FT * FK; e += FNT) {
        int nn, kk;
        if (b_nc) { kk = e / FT; nn = e % FT; } else { nn = e / FK; kk = e % FK; }
        const int64_t gn = n0 + nn, gk = k0 + kk;
        Bs[kk][nn] = (gn < P.N && gk < P.K) ? B[gk * P.sBk + gn * P.sBn] : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < FK; ++kk) {
        double a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) { a[i] = As[kk][ty * 4 + i]; b[i] = Bs[kk][tx * 4 + i]; }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
      if (gm < P.M && gn < P.N) {
        double* c = P.C + (int64_t)z * P.sCb + gm * P.sCm + gn * P.sCn;
        const double v = P.alpha * acc[i][j];
        if (P.accumulate) atomicAdd(c, v);
        else *c = (P.beta == 0.0) ? v : fma(P.beta, *c, v);
      }
    }
}

size_t al(size_t x, size_t a = 1024) { return (x + a - 1) / a * a; }

}  // namespace

// ---------------------------------------------------------------------------
// internal launchers (grouped.cuh)

size_t gg_staged_floats(int64_t rows, int64_t K, int64_t nred) {
  return (size_t)nred * tn_cdiv(rows, BM) * tn_cdiv(K, BK) * PAIR_FLOATS;
}

void gg_stage_shape(GgStage* it, int64_t rows, int64_t K, int64_t nred) {
  it->rows = (int32_t)rows;
  it->K = (int32_t)K;
  it->nred = (int32_t)nred;
  it->n_rt = (int32_t)tn_cdiv(rows, BM);
  it->n_kb = (int32_t)tn_cdiv(K, BK);
}

int gg_stage_tiles(const GgStage& it) { return it.nred * it.n_rt * it.n_kb; }

int gg_tf32_tiles(const GgProblem& p, int bn) {
  return (int)(std::max(p.nbatch, 1) * tn_cdiv(p.M, BM) * tn_cdiv(p.N, bn));
}

int gg_launch_stage(const GgStage* dev_items, int nitems, const int* dev_prefix, int total_tiles, cudaStream_t s) {
  if (total_tiles <= 0) return TN_OK;
  int* err;
  int st = tn_error_word(s, &err);
  if (st) return st;
  gg_stage_kernel<<<(unsigned)total_tiles, 256, 0, s>>>(dev_items, nitems, dev_prefix, err);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

int gg_launch_tf32(const GgProblem* dev_probs, int nprobs, const int* dev_prefix, int total_tiles, int bn, int ctas,
                   cudaStream_t s) {
  if (total_tiles <= 0) return TN_OK;
  int* err;
  int st = tn_error_word(s, &err);
  if (st) return st;
  const int grid = std::max(1, std::min(total_tiles, ctas > 0 ? ctas : tn_sm_count()));
  if (bn == 128) {
    if ((st = tn_set_smem_attr_once(TN_ATTR_GROUPED_GEMM, (const void*)gg_tf32x3_kernel<128>, GgCfg<128>::SMEM)))
      return st;
    gg_tf32x3_kernel<128><<<grid, NTHREADS, GgCfg<128>::SMEM, s>>>(dev_probs, nprobs, dev_prefix, total_tiles, err);
  } else if (bn == 64) {
    if ((st = tn_set_smem_attr_once(TN_ATTR_GROUPED_GEMM + 8, (const void*)gg_tf32x3_kernel<64>, GgCfg<64>::SMEM)))
      return st;
    gg_tf32x3_kernel<64><<<grid, NTHREADS, GgCfg<64>::SMEM, s>>>(dev_probs, nprobs, dev_prefix, total_tiles, err);
  } else {
    return tn_fail(TN_ERR_ARG, "grouped gemm: tile width must be 64 or 128");
  }
  TN_CHECK_LAUNCH();
  return TN_OK;
}

int gg_f64_tiles(const GgF64Problem& p) { return (int)(std::max(p.nbatch, 1) * tn_cdiv(p.M, FT) * tn_cdiv(p.N, FT)); }

int gg_launch_f64(const GgF64Problem* dev_probs, int nprobs, const int* dev_prefix, int total_tiles, cudaStream_t s) {
  if (total_tiles <= 0) return TN_OK;
  gg_f64_kernel<<<(unsigned)total_tiles, FNT, 0, s>>>(dev_probs, nprobs, dev_prefix);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

// ---------------------------------------------------------------------------
// public entry point: stage every operand, then one grouped launch

namespace {

struct GroupPlan {
  std::vector<GgStage> stages;
  std::vector<int> stage_prefix;
  std::vector<GgProblem> probs;
  std::vector<int> prob_prefix;
  std::vector<GgF64Problem> f64;
  std::vector<int> f64_prefix;
  size_t staged_floats = 0;
};

bool problem_ok(const tn_grouped_gemm_problem& q) {
  return q.M >= 0 && q.N >= 0 && q.K >= 0 && q.nred >= 1 && q.batch >= 0 && (q.batch <= 1 || q.nred == 1) &&
         (q.C || q.M * q.N == 0) && (q.K == 0 || (q.A && q.B));
}

int plan_group(int precision, const tn_grouped_gemm_problem* pr, int count, int bn, GroupPlan* g) {
  if (precision == TN_PREC_FP64) {
    g->f64_prefix.push_back(0);
    for (int i = 0; i < count; ++i) {
      const auto& q = pr[i];
      if (!problem_ok(q)) return tn_fail(TN_ERR_ARG, "grouped gemm: bad problem");
      GgF64Problem f{};
      f.M = q.M; f.N = q.N; f.K = q.K; f.nred = q.nred;
      f.A = q.A; f.sAm = q.sAm; f.sAk = q.sAk; f.sAr = q.sAr;
      f.B = q.B; f.sBk = q.sBk; f.sBn = q.sBn; f.sBr = q.sBr;
      f.C = q.C; f.sCm = q.sCm; f.sCn = q.sCn;
      f.alpha = q.alpha; f.beta = q.beta; f.accumulate = q.accumulate; f.active = q.active;
      f.nbatch = std::max(q.batch, 1); f.sAb = q.sAb; f.sBb = q.sBb; f.sCb = q.sCb;
      g->f64.push_back(f);
      g->f64_prefix.push_back(g->f64_prefix.back() + (q.M * q.N ? gg_f64_tiles(f) : 0));
    }
    return TN_OK;
  }
  g->stage_prefix.push_back(0);
  g->prob_prefix.push_back(0);
  size_t off = 0;
  for (int i = 0; i < count; ++i) {
    const auto& q = pr[i];
    if (!problem_ok(q)) return tn_fail(TN_ERR_ARG, "grouped gemm: bad problem");
    GgProblem p{};
    const int32_t nb = std::max(q.batch, 1);
    p.M = q.M; p.N = q.N;
    p.nred = q.nred;
    p.nbatch = nb;
    p.n_kb = (int32_t)tn_cdiv(q.K, BK);
    p.n_nt = (int32_t)tn_cdiv(q.N, bn);
    p.n_mt = (int32_t)tn_cdiv(q.M, BM);
    p.C = q.C; p.sCm = q.sCm; p.sCn = q.sCn; p.sCb = q.sCb;
    p.alpha = q.alpha; p.beta = q.beta; p.accumulate = q.accumulate; p.active = q.active;
    if (q.K > 0 && q.M > 0 && q.N > 0) {
      // a batch is staged like a reduction over z (the two never combine: nred == 1 when batch > 1)
      const int64_t nr = nb > 1 ? nb : q.nred;
      GgStage a{}, b{};
      a.src = q.A; a.s_row = q.sAm; a.s_k = q.sAk; a.s_red = nb > 1 ? q.sAb : q.sAr; a.active = q.active;
      gg_stage_shape(&a, q.M, q.K, nr);
      a.dst = (float*)(uintptr_t)off;  // offset now, pointer once the workspace is known
      off += gg_staged_floats(q.M, q.K, nr);
      b.src = q.B; b.s_row = q.sBn; b.s_k = q.sBk; b.s_red = nb > 1 ? q.sBb : q.sBr; b.active = q.active;
      gg_stage_shape(&b, q.N, q.K, nr);
      b.dst = (float*)(uintptr_t)off;
      off += gg_staged_floats(q.N, q.K, nr);
      p.a = a.dst; p.a_nrt = a.n_rt;
      p.b = b.dst; p.b_nrt = b.n_rt;
      g->stages.push_back(a);
      g->stage_prefix.push_back(g->stage_prefix.back() + gg_stage_tiles(a));
      g->stages.push_back(b);
      g->stage_prefix.push_back(g->stage_prefix.back() + gg_stage_tiles(b));
    } else {
      p.n_kb = 0;
    }
    g->probs.push_back(p);
    g->prob_prefix.push_back(g->prob_prefix.back() + (q.M * q.N ? gg_tf32_tiles(p, bn) : 0));
  }
  g->staged_floats = off;
  return TN_OK;
}

size_t tables_bytes(const GroupPlan& g) {
  return al(g.stages.size() * sizeof(GgStage) + 64) + al(g.stage_prefix.size() * sizeof(int) + 64) +
         al(g.probs.size() * sizeof(GgProblem) + 64) + al(g.prob_prefix.size() * sizeof(int) + 64) +
         al(g.f64.size() * sizeof(GgF64Problem) + 64) + al(g.f64_prefix.size() * sizeof(int) + 64);
}

int pick_bn(int precision) { return precision == TN_PREC_TF32X3 ? gg_tile_n() : 64; }

// the split-TF32 tile width chosen for the calls of this host thread (0: the default, 128)
thread_local int t_tile_n = 0;

}  // namespace

int gg_tile_n() { return t_tile_n ? t_tile_n : 128; }

extern "C" int tn_set_grouped_tile(int tile_n) {
  if (tile_n != 0 && tile_n != 64 && tile_n != 128) return tn_fail(TN_ERR_ARG, "grouped tile width must be 0, 64 or 128");
  t_tile_n = tile_n;
  return TN_OK;
}

extern "C" int tn_get_grouped_tile(void) { return gg_tile_n(); }

extern "C" size_t tn_grouped_gemm_workspace_bytes(int precision, const tn_grouped_gemm_problem* problems, int count) {
  if (!problems || count <= 0) return 1024;
  GroupPlan g;
  if (plan_group(precision, problems, count, pick_bn(precision), &g)) return 0;
  return 2048 + tables_bytes(g) + al(g.staged_floats * sizeof(float));
}

extern "C" int tn_grouped_gemm(int precision, const tn_grouped_gemm_problem* problems, int count, void* ws,
                               size_t ws_bytes, void* stream) {
  if (count <= 0) return TN_OK;
  if (!problems) return tn_fail(TN_ERR_ARG, "grouped gemm: null problem table");
  if (precision != TN_PREC_FP64 && precision != TN_PREC_TF32X3) return tn_fail(TN_ERR_ARG, "grouped gemm: precision");
  if (precision == TN_PREC_TF32X3 && !tn_tf32x3_supported()) return tn_fail(TN_ERR_ARG, "tf32x3 needs an sm_103 device");
  cudaStream_t s = (cudaStream_t)stream;
  GroupPlan g;
  const int bn = pick_bn(precision);
  int st = plan_group(precision, problems, count, bn, &g);
  if (st) return st;
  const size_t need = 2048 + tables_bytes(g) + al(g.staged_floats * sizeof(float));
  if (!ws || ws_bytes < need) return tn_fail(TN_ERR_WORKSPACE, "grouped gemm: workspace too small");
  char* base = (char*)al((size_t)(uintptr_t)ws);
  char* p = base;
  auto put = [&](const void* src, size_t bytes) -> char* {
    char* at = p;
    if (bytes) {
      cudaError_t e = cudaMemcpyAsync(at, src, bytes, cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) return nullptr;
    }
    p += al(bytes + 64);
    return at;
  };
  if (precision == TN_PREC_FP64) {
    char* dp = put(g.f64.data(), g.f64.size() * sizeof(GgF64Problem));
    char* dx = put(g.f64_prefix.data(), g.f64_prefix.size() * sizeof(int));
    if (!dp || !dx) return tn_record_error(cudaGetLastError());
    st = gg_launch_f64((const GgF64Problem*)dp, (int)g.f64.size(), (const int*)dx, g.f64_prefix.back(), s);
    if (st) return st;
    // the tables were copied from pageable host memory: the copies finished before the calls returned
    return TN_OK;
  }
  // place the tables first, then the staging area; fix up the staged pointers
  char* tab = p;
  p += tables_bytes(g);
  float* staged = (float*)al((size_t)(uintptr_t)p);
  for (auto& it : g.stages) it.dst = staged + (size_t)(uintptr_t)it.dst;
  for (auto& pr : g.probs) {
    if (pr.n_kb) {
      pr.a = staged + (size_t)(uintptr_t)pr.a;
      pr.b = staged + (size_t)(uintptr_t)pr.b;
    }
  }
  p = tab;
  char* d_st = put(g.stages.data(), g.stages.size() * sizeof(GgStage));
  char* d_sx = put(g.stage_prefix.data(), g.stage_prefix.size() * sizeof(int));
  char* d_pr = put(g.probs.data(), g.probs.size() * sizeof(GgProblem));
  char* d_px = put(g.prob_prefix.data(), g.prob_prefix.size() * sizeof(int));
  if (!d_st || !d_sx || !d_pr || !d_px) return tn_record_error(cudaGetLastError());
  st = gg_launch_stage((const GgStage*)d_st, (int)g.stages.size(), (const int*)d_sx, g.stage_prefix.back(), s);
  if (st) return st;
  return gg_launch_tf32((const GgProblem*)d_pr, (int)g.probs.size(), (const int*)d_px, g.prob_prefix.back(), bn, 0,
                        s);
}
