// FP32 Householder QR of one m x n matrix (n <= m <= 1024, n <= 512) by ONE 16-CTA thread-block
// cluster (blocked, column-distributed), then Q formed by a wide grid.
//
// Role: step 1 of the mixed-precision gauge move (tn_qr_mixed): the FP32 factors it returns are
// re-orthogonalised in FP64 afterwards, so only backward stability in FP32 is needed here.
//
// Why this shape: a Householder QR is a chain of n dependent column steps, each a reduction over
// the rows. On GB300 FP64 issues ~2 lanes/clock/SM with a 64-cycle dependent latency, so the
// steps run in FP32; and a reduction across SMs (cluster barrier + distributed shared memory,
// ~1 us) per column would dominate, so every column step stays inside one CTA:
//   * The columns form panels of 16 (block b = columns [16b, 16b + 16)); CTA q owns blocks q and
//     q + 16 for ALL rows, in shared memory (column-major, odd leading dimension 1025, so
//     row-parallel and column-parallel accesses are both free of bank conflicts). Panel b is
//     factorised by its owner alone (LAPACK dgeqr2 conventions per column, then the compact-WY
//     factor T of dlarft, forward/columnwise), by 8 of its warps on a named barrier, with no
//     synchronisation outside the CTA.
//   * The owner publishes V_b (row-major m x 16 in global memory, unit diagonal, zeros above) and
//     T_b, then arrives on mbarrier ready[b] of every CTA of the cluster (release at cluster
//     scope).
//   * A CTA with blocks to the right of b waits on its own ready[b] (bounded), stages V_b in its
//     shared memory once and applies H_b^T = I - V_b T_b^T V_b^T to those blocks. The chain of the
//     factorisation is, per panel: stage V_b, form W2 = T_b^T V_b^T C of block b + 1 and fold
//     C -= V_b W2 into the register prologue of its factorisation, factorise, publish; every
//     other update runs beside it. The block two panels ahead is updated after the
//     factorisation, so it never delays the chain.
//   * Q = H_0 H_1 ... E is formed by a second kernel over 128 CTAs (4 columns each) from the
//     published V_b, T_b: the chain H_q, ..., H_0 of the last column block would otherwise run on
//     one SM after the last panel while the rest of the cluster sits idle.
// Every wait is bounded by a clock budget; on timeout the CTA records an error code, skips its
// remaining work and still joins the final cluster barrier.
#include <mutex>

#include "common.cuh"


namespace {

constexpr int CL = 16;           // CTAs per cluster (non-portable size)
constexpr int BW = 16;           // columns per panel
constexpr int NBMAX = 2 * CL;    // panels (two per CTA)
constexpr int NT = 512;          // threads per CTA
constexpr int NW = NT / 32;      // warps per CTA
constexpr int MMAX = 1024;       // maximum rows
constexpr int LDC = MMAX + 1;    // leading dimension of a shared column block
constexpr int LDW = BW + 1;
constexpr int LDW2 = BW + 4;     // W2 row pitch (16-byte aligned rows)
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

struct Smem {
  float C[2][BW * LDC];       // own column blocks q and q + 16, column-major
  float Vs[MMAX * BW];        // V of the panel being applied, row-major, 16-byte chunks swizzled
  float Wred[NW * BW * LDW];  // per-warp partial products
  float W2[BW * LDW2];        // W2 = T^T W, 16-byte aligned rows
  float T[BW * LDW];          // T of the panel being factorised
  float G[BW * LDW];          // G(l, i) = v_l^T v_i of the panel being factorised (l < i)
  float Tapp[BW * LDW];       // T of the panel being applied
  float red[NW * LDW];        // per-warp partials of the panel reductions
  float f[BW];                // update coefficients of the current panel column
  float prow[BW];             // the pivot row of the panel (16-byte aligned)
  float tau[BW];              // tau of every reflector of the panel
  float rb[2];                // beta and scale of the current reflector
  unsigned long long ready[NBMAX];  // mbarrier per panel
  double amax[CL];            // largest |a| of every CTA's blocks
  double wmax[NW];            // per-warp maxima of this CTA's blocks
  int failed;
};

constexpr size_t kSmemBytes = sizeof(Smem) + 16;
static_assert(kSmemBytes <= 227 * 1024, "shared memory budget of one CTA");
static_assert(offsetof(Smem, Vs) % 16 == 0 && offsetof(Smem, W2) % 16 == 0 && offsetof(Smem, f) % 16 == 0 &&
                  offsetof(Smem, prow) % 16 == 0,
              "float4 members");

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ int cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return (int)r;
}

__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Arrive (release, cluster scope) on the copy of mbarrier `bar` held by cluster CTA `rank`.
__device__ __forceinline__ void remote_arrive(unsigned long long* bar, int rank) {
  uint32_t ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(smem_u32(bar)), "r"(rank));
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(ra) : "memory");
}

// Bounded wait for phase 0 of a local mbarrier (acquire, cluster scope).
__device__ __forceinline__ bool wait_ready(unsigned long long* bar) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], 0;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar))
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > kWaitCycles) return false;
  }
}

// Float index of 16-byte chunk ch (0..3) of row r in Vs: the chunk index is XOR-ed with bits 1-2
// of the row, so 8 consecutive rows at one chunk, and 4 consecutive rows at two chunks, fall on
// distinct banks.
__device__ __forceinline__ int vs_idx(int r, int ch) { return r * BW + ((ch ^ ((r >> 1) & 3)) << 2); }

// Sum over the 32 lanes of 16 values at once: on return lane L holds sum over lanes of v[L & 15].
__device__ __forceinline__ float warp_transpose_sum(float (&v)[BW], int lane) {
#pragma unroll
  for (int half = BW / 2; half >= 1; half >>= 1) {
    const bool upper = (lane & half) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      // keep the half of the vector this lane is responsible for, send the other half
      const float send = upper ? v[i] : v[i + half];
      const float keep = upper ? v[i + half] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, half);
    }
  }
  return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 16);
}

// Vs(rows >= r0) <- V_p (published, row-major m x 16) and Tapp <- T_p. Every thread issues all its
// loads before its first store.
__device__ void stage_v(Smem& sh, int m, int r0, const float* __restrict__ Vp, const float* __restrict__ Tp) {
  const int t = threadIdx.x;
  const float tv = (t < BW * BW) ? Tp[t] : 0.f;
  const int total = (m - r0) * 4;  // 16-byte chunks
  const float4* src = reinterpret_cast<const float4*>(Vp + (size_t)r0 * BW);
  float4* dst = reinterpret_cast<float4*>(sh.Vs);
  constexpr int PER = MMAX * 4 / NT;  // 8 chunks per thread at most
  float4 x[PER];
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = t + NT * i;
    x[i] = (e < total) ? src[e] : make_float4(0.f, 0.f, 0.f, 0.f);
  }
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = t + NT * i;
    if (e < total) dst[vs_idx(r0 + (e >> 2), e & 3) >> 2] = x[i];
  }
  if (t < BW * BW) sh.Tapp[(t / BW) * LDW + t % BW] = tv;
}

// Block `slot` (rows >= r0) <- H_p^T C = (I - V T^T V^T) C with V = V_p staged in Vs and T = T_p
// staged in Tapp.
//   W = V^T C  (16 x 16): thread = (8 reflectors kb, 4 columns cb) x row group g (64 groups);
//   C -= V W2  (rows x 16): thread = 8 rows (128 apart) x 4 columns cb.
// W2 = T^T V^T C (rows >= r0): the first half of apply_block; ends with a barrier.
__device__ void apply_w(Smem& sh, int slot, int m, int r0) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const float* Cs = sh.C[slot];
  {
    const int tile = t & 7, kb = tile >> 2, cb = tile & 3, g = t >> 3;
    float acc[8][4];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = 0.f;
    for (int r = r0 + g; r < m; r += NT / 8) {
      const float4 v0 = *reinterpret_cast<const float4*>(sh.Vs + vs_idx(r, 2 * kb));
      const float4 v1 = *reinterpret_cast<const float4*>(sh.Vs + vs_idx(r, 2 * kb + 1));
      const float v[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
      float cv[4];
#pragma unroll
      for (int b = 0; b < 4; ++b) cv[b] = Cs[(4 * cb + b) * LDC + r];
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fmaf(v[a], cv[b], acc[a][b]);
    }
    // the warp's 4 row groups differ in lane bits 3 and 4
#pragma unroll
    for (int o = 8; o <= 16; o <<= 1)
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] += __shfl_xor_sync(0xffffffffu, acc[a][b], o);
    if (lane < 8) {
      float* Wp = sh.Wred + warp * BW * LDW;
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) Wp[(8 * kb + a) * LDW + 4 * cb + b] = acc[a][b];
    }
  }
  __syncthreads();
  // reduce the warps' partials into Wred[0] (each thread reads and writes only its own element)
  for (int o = t; o < BW * BW; o += NT) {
    const int k = o / BW, c = o % BW;
    float s = 0.f;
#pragma unroll
    for (int w = 0; w < NW; ++w) s += sh.Wred[w * BW * LDW + k * LDW + c];
    sh.Wred[k * LDW + c] = s;
  }
  __syncthreads();
  // W2 = T^T W (T upper triangular)
  for (int o = t; o < BW * BW; o += NT) {
    const int k = o / BW, c = o % BW;
    float s = 0.f;
    for (int l = 0; l <= k; ++l) s = fmaf(sh.Tapp[l * LDW + k], sh.Wred[l * LDW + c], s);
    sh.W2[k * LDW2 + c] = s;
  }
  __syncthreads();
}

// C(rows >= r0) -= V W2: the second half of apply_block.
__device__ void apply_c(Smem& sh, int slot, int m, int r0) {
  const int t = threadIdx.x;
  float* Cs = sh.C[slot];
  // C -= V W2: a warp covers 32 consecutive rows of one column group (Vs reads conflict-free by the
  // swizzle, W2 reads broadcast, C accesses on 32 distinct banks by the odd pitch)
  {
    const int rs = t & 127, cb = t >> 7;
    float out[8][4];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) out[a][b] = 0.f;
#pragma unroll
    for (int k4 = 0; k4 < BW / 4; ++k4) {
      float v[8][4];
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        const int r = r0 + rs + 128 * a;
        const float4 x = (r < m) ? *reinterpret_cast<const float4*>(sh.Vs + vs_idx(r, k4))
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
        v[a][0] = x.x;
        v[a][1] = x.y;
        v[a][2] = x.z;
        v[a][3] = x.w;
      }
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const float4 w4 = *reinterpret_cast<const float4*>(sh.W2 + (4 * k4 + kk) * LDW2 + 4 * cb);
        const float w[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) out[a][b] = fmaf(v[a][kk], w[b], out[a][b]);
      }
    }
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const int r = r0 + rs + 128 * a;
      if (r < m) {
#pragma unroll
        for (int b = 0; b < 4; ++b) Cs[(4 * cb + b) * LDC + r] -= out[a][b];
      }
    }
  }
  __syncthreads();
}

__device__ void apply_block(Smem& sh, int slot, int m, int r0) {
  apply_w(sh, slot, m, r0);
  apply_c(sh, slot, m, r0);
}

// Householder QR of panel `slot` (columns 0..jb-1 of the block, rows >= j0 = 16 b), then its
// compact-WY factor T (dlarft, forward, columnwise) in sh.T.
// One reduction per column: with x the pivot column below the pivot row j and v = e_j + scale x
// (dlarfg), v^T a_c = a_c(j) + scale * (x^T a_c), so the sums sig = x^T x and h_c = x^T a_c over
// the rows > j, taken together in one transposed warp reduction before the reflector is known,
// give the reflector, every update coefficient f_c = tau v^T a_c (unfinished slots) and the Gram
// entries v_l^T v_i of T (finished slots). A column step is then: partial sums (8 warps) -> barrier
// -> warp 0 finishes the sums, the reflector and f -> barrier -> update. Every warp taking part
// repeats a transposed reduction, so 8 warps (4 rows per thread, named barrier 1) do it and the
// other 8 only wait.
// The panel is held in registers: thread t < 256 owns rows t + 256 k (k < 4) of the 16 columns,
// a[4][16], used as a ring. At step i the slots 0..15-i hold the unfinished columns i..15 (slot 0 =
// the pivot column) and the slots 16-i..15 hold the finished reflectors v_0..v_{i-1} (masked: 0
// above the diagonal, 1 on it). Every step works on slot 0 and then rotates the ring by one, so all
// steps run the same code with static register indices (unrolled by two, which halves the moves of
// the rotation).
constexpr int FW = 8;           // warps of the panel factorisation
constexpr int FT = FW * 32;     // its threads
constexpr int RPT = MMAX / FT;  // rows per thread

__device__ __forceinline__ void bar_factor() { asm volatile("bar.sync 1, %0;" ::"n"(FT) : "memory"); }

// fr0 >= 0: the block has not yet received the update C -= V W2 of the previous panel (rows >= fr0,
// V staged in Vs, W2 from apply_w); it is applied here, in registers, on the way in (the panel is
// retired into shared memory column by column, all rows).
__device__ void factor_panel(Smem& sh, int slot, int m, int j0, int jb, int fr0) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  float* Cs = sh.C[slot];
  if (t < FT) {
    float a[RPT][BW];
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
      const int r = t + rr * FT;
#pragma unroll
      for (int c = 0; c < BW; ++c) a[rr][c] = (r < m) ? Cs[c * LDC + r] : 0.f;
    }
    if (fr0 >= 0) {
#pragma unroll 1
      for (int k4 = 0; k4 < BW / 4; ++k4) {
        float v[RPT][4];
#pragma unroll
        for (int rr = 0; rr < RPT; ++rr) {
          const int r = t + rr * FT;
          const float4 x = (r >= fr0 && r < m) ? *reinterpret_cast<const float4*>(sh.Vs + vs_idx(r, k4))
                                               : make_float4(0.f, 0.f, 0.f, 0.f);
          v[rr][0] = x.x;
          v[rr][1] = x.y;
          v[rr][2] = x.z;
          v[rr][3] = x.w;
        }
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          float w[BW];
#pragma unroll
          for (int c4 = 0; c4 < BW / 4; ++c4) {
            const float4 w4 = *reinterpret_cast<const float4*>(sh.W2 + (4 * k4 + kk) * LDW2 + 4 * c4);
            w[4 * c4] = w4.x;
            w[4 * c4 + 1] = w4.y;
            w[4 * c4 + 2] = w4.z;
            w[4 * c4 + 3] = w4.w;
          }
#pragma unroll
          for (int rr = 0; rr < RPT; ++rr)
#pragma unroll
            for (int c = 0; c < BW; ++c) a[rr][c] = fmaf(-v[rr][kk], w[c], a[rr][c]);
        }
      }
    }
#pragma unroll 2
    for (int i = 0; i < jb; ++i) {
      const int j = j0 + i;
      // partial sums over this thread's rows below the pivot: slot 0 -> sig, slot c -> h_c; the
      // owner of the pivot row publishes it
      float x[RPT];
#pragma unroll
      for (int rr = 0; rr < RPT; ++rr) x[rr] = (t + rr * FT > j) ? a[rr][0] : 0.f;  // rows >= m hold 0
      float p[BW];
#pragma unroll
      for (int c = 0; c < BW; ++c) {
        float y = x[0] * a[0][c];
#pragma unroll
        for (int rr = 1; rr < RPT; ++rr) y = fmaf(x[rr], a[rr][c], y);
        p[c] = y;
      }
#pragma unroll
      for (int rr = 0; rr < RPT; ++rr)
        if (t + rr * FT == j) {
#pragma unroll
          for (int c4 = 0; c4 < BW / 4; ++c4)
            reinterpret_cast<float4*>(sh.prow)[c4] =
                make_float4(a[rr][4 * c4], a[rr][4 * c4 + 1], a[rr][4 * c4 + 2], a[rr][4 * c4 + 3]);
        }
      const float ws = warp_transpose_sum(p, lane);
      if (lane < BW) sh.red[warp * LDW + lane] = ws;
      bar_factor();
      // warp 0, lane c: the total of slot c, then the reflector (every lane) and slot c's coefficient
      if (warp == 0 && lane < BW) {
        float t0 = 0.f, t1 = 0.f;
#pragma unroll
        for (int w = 0; w < FW; w += 2) {
          t0 += sh.red[w * LDW + lane];
          t1 += sh.red[(w + 1) * LDW + lane];
        }
        const float tot = t0 + t1;
        const float sig = __shfl_sync(0x0000ffffu, tot, 0);
        const float x1 = sh.prow[0];
        float beta = x1, tau = 0.f, scale = 0.f;
        // a sub-column below kHhTiny in squared norm is taken as zero (no reflector): its squares
        // would be subnormal or flushed, sig would misstate |x|^2 and the reflector built from it
        // would not be orthogonal (input scaled to max |a| ~ 1, so the dropped entries are < 1e-12
        // of the largest, below the FP32 accuracy of R)
        if (sig > kHhTiny) {
          // hardware reciprocal square root and reciprocal (a few ulp, which the FP64
          // re-orthogonalisation absorbs) on the critical path of every column
          const float s2 = fmaf(x1, x1, sig);
          const float nrm = s2 * rsqrtf(s2);
          beta = (x1 >= 0.f) ? -nrm : nrm;
          tau = (beta - x1) * __fdividef(1.f, beta);
          scale = __fdividef(1.f, x1 - beta);
        }
        const float pc = fmaf(scale, tot, sh.prow[lane]);  // v_i^T (slot lane)
        const bool unfinished = lane >= 1 && lane <= BW - 1 - i && i + lane < jb;
        sh.f[lane] = unfinished ? tau * pc : 0.f;
        if (lane >= BW - i) sh.G[(lane - BW + i) * LDW + i] = pc;  // slot 16 - i + l holds v_l
        if (lane == 0) {
          sh.tau[i] = tau;
          sh.rb[0] = beta;
          sh.rb[1] = scale;
        }
      }
      bar_factor();
      // v_i (masked) of this thread's rows into the pivot slot, R(j, j) on the pivot row; update of
      // the unfinished slots (f is zero on the others)
      const float beta = sh.rb[0], scale = sh.rb[1];
      float fc[BW];
#pragma unroll
      for (int c4 = 0; c4 < BW / 4; ++c4) {
        const float4 f4 = reinterpret_cast<const float4*>(sh.f)[c4];
        fc[4 * c4] = f4.x;
        fc[4 * c4 + 1] = f4.y;
        fc[4 * c4 + 2] = f4.z;
        fc[4 * c4 + 3] = f4.w;
      }
#pragma unroll
      for (int rr = 0; rr < RPT; ++rr) {
        const int r = t + rr * FT;
        float v = 0.f;
        if (r > j) {
          v = x[rr] * scale;
          a[rr][0] = v;
        } else if (r == j) {
          v = 1.f;
          a[rr][0] = beta;
        }
#pragma unroll
        for (int c = 1; c < BW; ++c) a[rr][c] = fmaf(-v, fc[c], a[rr][c]);
        // retire the pivot column: R part and v to shared memory, masked v into the ring
        if (r < m) Cs[i * LDC + r] = a[rr][0];
#pragma unroll
        for (int c = 0; c < BW - 1; ++c) a[rr][c] = a[rr][c + 1];
        a[rr][BW - 1] = v;
      }
      // no barrier here: the next step writes prow/red before its first barrier and f/rb after it,
      // and every reader of this step's values has passed this step's second barrier
    }
    bar_factor();
    // T(k, i) = -tau_i sum_{l=k}^{i-1} T(k, l) G(l, i), T(i, i) = tau_i: lane k of warp 0 runs row k
    // with the row in registers
    if (warp == 0 && lane < BW) {
      const int k = lane;
      float tr[BW];
#pragma unroll
      for (int i = 0; i < BW; ++i) {
        float a0 = 0.f, a1 = 0.f;
#pragma unroll
        for (int l = 0; l < i; ++l) {
          const float g = sh.G[l * LDW + i];
          if (l & 1) a1 = fmaf((l >= k) ? tr[l] : 0.f, g, a1);
          else a0 = fmaf((l >= k) ? tr[l] : 0.f, g, a0);
        }
        const float ti = sh.tau[i];
        tr[i] = (i >= jb || k >= jb || k > i) ? 0.f : ((k == i) ? ti : -ti * (a0 + a1));
      }
#pragma unroll
      for (int i = 0; i < BW; ++i) sh.T[k * LDW + i] = tr[i];
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(NT, 1)
    qr32_cluster_kernel(int m, int n, const double* __restrict__ A, int64_t sAm, int64_t sAn, double* __restrict__ R,
                        int64_t sRm, int64_t sRn, float* __restrict__ Vg, float* __restrict__ Tg, int* err) {
  extern __shared__ unsigned char smem_raw[];
  Smem& sh = *reinterpret_cast<Smem*>(((uintptr_t)smem_raw + 15) & ~(uintptr_t)15);
  const int q = cluster_rank();
  const int t = threadIdx.x;
  const int nblk = (n + BW - 1) / BW;
  const int blk[2] = {q, q + CL};  // own blocks, slot 0 and slot 1
  int jbs[2];
#pragma unroll
  for (int sl = 0; sl < 2; ++sl) jbs[sl] = max(0, min(BW, n - blk[sl] * BW));
  if (t == 0) {
    for (int p = 0; p < NBMAX; ++p)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&sh.ready[p])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sh.failed = 0;
  }
  // element e of block slot sl (columns beyond n are zero), coalesced along the unit stride
  auto elem = [&](int sl, int e, int& r, int& c) -> double {
    if (sAn == 1) {
      r = e / BW;
      c = e % BW;
    } else {
      c = e / m;
      r = e % m;
    }
    return (c < jbs[sl]) ? A[(int64_t)r * sAm + (int64_t)(blk[sl] * BW + c) * sAn] : 0.0;
  };
  cluster_sync();  // every CTA of the cluster is running before any remote store into it
  // largest |a| of the blocks, published to every CTA: the whole matrix is scaled by one power of
  // two (exact) so that any finite FP64 input fits FP32; R is scaled back on output
  {
    double mx = 0.0;
    for (int sl = 0; sl < 2; ++sl)
      for (int e = t; e < m * BW; e += NT) {
        int r, c;
        mx = fmax(mx, fabs(elem(sl, e, r, c)));
      }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((t & 31) == 0) sh.wmax[t >> 5] = mx;
    __syncthreads();
    if (t < CL) {
      double cm = 0.0;
      for (int w = 0; w < NW; ++w) cm = fmax(cm, sh.wmax[w]);
      uint32_t ra;
      asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(smem_u32(&sh.amax[q])), "r"(t));
      asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(ra), "d"(cm) : "memory");
    }
  }
  cluster_sync();  // maxima published; mbarriers of every CTA initialised before any remote arrive
  double gmax = 0.0;
  for (int p = 0; p < CL; ++p) gmax = fmax(gmax, sh.amax[p]);
  const int ex = (gmax > 0.0 && isfinite(gmax)) ? ilogb(gmax) : 0;
  const double down = ldexp(1.0, -ex), up = ldexp(1.0, ex);
  for (int sl = 0; sl < 2; ++sl)
    for (int e = t; e < m * BW; e += NT) {
      int r, c;
      const double v = elem(sl, e, r, c);
      sh.C[sl][c * LDC + r] = (float)(v * down);
    }
  __syncthreads();

  // V_p into Vs (waiting for panel p first unless this CTA owns it); false after a failed wait
  auto acquire = [&](int p) -> bool {
    if (p % CL != q && !wait_ready(&sh.ready[p])) {
      if (t == 0) atomicExch(err, TN_DEVERR_QR_WAIT);
      sh.failed = 1;
    }
    __syncthreads();
    if (sh.failed) return false;
    stage_v(sh, m, p * BW, Vg + (size_t)p * m * BW, Tg + p * BW * BW);
    __syncthreads();
    return true;
  };
  auto apply = [&](int sl, int p) { apply_block(sh, sl, m, p * BW); };
  // factorise block slot sl (fr0 >= 0: with the pending update of the previous panel folded in),
  // publish V and T, release the waiters, write the R block
  auto factor_publish = [&](int sl, int fr0) {
    const int b = blk[sl], jb = jbs[sl], col0 = b * BW;
    factor_panel(sh, sl, m, col0, jb, fr0);
    float* Vb = Vg + (size_t)b * m * BW;
    for (int e = t; e < m * BW; e += NT) {
      const int r = e / BW, c = e % BW;
      const int d = col0 + c;
      Vb[e] = (c < jb && r >= d) ? ((r == d) ? 1.f : sh.C[sl][c * LDC + r]) : 0.f;
    }
    for (int e = t; e < BW * BW; e += NT) {
      const int k = e / BW, l = e % BW;
      Tg[b * BW * BW + e] = (k < jb && l < jb) ? sh.T[k * LDW + l] : 0.f;
    }
    __threadfence();
    __syncthreads();
    if (t < CL) remote_arrive(&sh.ready[b], t);
    // R block (not needed by the other CTAs): rows <= diagonal from the block, zeros below
    if (R) {
      for (int e = t; e < n * BW; e += NT) {
        const int r = e / BW, c = e % BW;
        if (c < jb) {
          const int d = col0 + c;
          R[(int64_t)r * sRm + (int64_t)d * sRn] = (r <= d) ? (double)sh.C[sl][c * LDC + r] * up : 0.0;
        }
      }
    }
  };

  if (jbs[0] > 0) {
    const bool two = jbs[1] > 0;
    // panels left of block q, in order; the last one is folded into the factorisation of block q
    // (the link of the chain), and reaches block q + 16 only after it (it stays in Vs meanwhile)
    for (int p = 0; p < blk[0]; ++p) {
      if (!acquire(p)) break;
      if (p == blk[0] - 1) {
        apply_w(sh, 0, m, p * BW);
      } else {
        apply(0, p);
        if (two) apply(1, p);
      }
    }
    if (!sh.failed) {
      factor_publish(0, blk[0] > 0 ? (blk[0] - 1) * BW : -1);
      if (two) {
        if (blk[0] > 0) apply(1, blk[0] - 1);
        for (int p = blk[0]; p < blk[1]; ++p) {
          if (!acquire(p)) break;
          if (p == blk[1] - 1) apply_w(sh, 1, m, p * BW);
          else apply(1, p);
        }
        if (!sh.failed) factor_publish(1, (blk[1] - 1) * BW);
      }
    }
  }
  (void)nblk;
  cluster_sync();  // no CTA exits while another may still arrive on its barriers
}

// Q = H_0 H_1 ... H_{np-1} [I_n; 0] from the published V_p, T_p, formed by a wide grid after the
// factorisation: one CTA per (column block q, chunk of QF_CW columns). H_p with p > q leaves the
// identity columns of block q unchanged (they are zero on rows >= 16p), so the CTA applies
// H_q, ..., H_0 to its columns, each on rows >= 16p only.
constexpr int QF_CW = 4;    // columns of Q per CTA (128 CTAs at n = 512: short per-CTA chains)
constexpr int QF_NT = 256;  // threads per CTA (the chain of the last blocks is issue-bound)
constexpr int QF_NW = QF_NT / 32;
constexpr int QF_ROWS = MMAX / QF_NT;  // rows per thread in the update
constexpr int QF_W = BW * QF_CW;       // elements of W (threads t < QF_W own one)
static_assert(QF_W <= QF_NT && QF_CW % 4 == 0 && BW % QF_CW == 0, "one W element per thread, float4 rows");

__global__ void __launch_bounds__(QF_NT) qr32_form_q_kernel(int m, int n, const float* __restrict__ Vg,
                                                            const float* __restrict__ Tg, double* __restrict__ Q) {
  __shared__ __align__(16) float X[MMAX * QF_CW];  // the CTA's Q columns, row-major m x QF_CW
  __shared__ __align__(16) float Wp[QF_NW][QF_W];
  __shared__ __align__(16) float W[QF_W];
  __shared__ __align__(16) float W2[QF_W];
  __shared__ float T[BW * LDW];
  constexpr int chunks = BW / QF_CW;
  const int q = blockIdx.x / chunks, c0 = q * BW + (blockIdx.x % chunks) * QF_CW;
  if (c0 >= n) return;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  for (int e = t; e < m * QF_CW; e += QF_NT) {
    const int r = e / QF_CW, c = e % QF_CW;
    X[e] = (r == c0 + c && c0 + c < n) ? 1.f : 0.f;
  }
  for (int p = q; p >= 0; --p) {
    const float* __restrict__ Vp = Vg + (size_t)p * m * BW;
    const float* __restrict__ Tp = Tg + p * BW * BW;
    const int r0 = p * BW;
    for (int o = t; o < BW * BW; o += QF_NT) T[(o / BW) * LDW + o % BW] = Tp[o];
    __syncthreads();  // X (initial values or the previous update) and T are in place
    // W = V_p^T X over rows >= r0: thread = (4 reflectors kq, row group g of 64), 4 x 8 partials
    {
      const int kq = lane & 3, g = warp * 8 + (lane >> 2);
      float acc[4][QF_CW];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < QF_CW; ++b) acc[a][b] = 0.f;
      for (int r = r0 + g; r < m; r += QF_NW * 8) {
        const float4 v4 = reinterpret_cast<const float4*>(Vp + (size_t)r * BW)[kq];
        const float4* xr = reinterpret_cast<const float4*>(X + r * QF_CW);
        const float v[4] = {v4.x, v4.y, v4.z, v4.w};
        float x[QF_CW];
#pragma unroll
        for (int h = 0; h < QF_CW / 4; ++h) {
          const float4 x4 = xr[h];
          x[4 * h] = x4.x;
          x[4 * h + 1] = x4.y;
          x[4 * h + 2] = x4.z;
          x[4 * h + 3] = x4.w;
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < QF_CW; ++b) acc[a][b] = fmaf(v[a], x[b], acc[a][b]);
      }
      // the warp's 8 row groups differ in lane bits 2..4
#pragma unroll
      for (int o = 4; o <= 16; o <<= 1)
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < QF_CW; ++b) acc[a][b] += __shfl_xor_sync(0xffffffffu, acc[a][b], o);
      if (lane < 4) {
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < QF_CW; ++b) Wp[warp][(4 * kq + a) * QF_CW + b] = acc[a][b];
      }
    }
    __syncthreads();
    if (t < QF_W) {
      float s = 0.f;
#pragma unroll
      for (int w = 0; w < QF_NW; ++w) s += Wp[w][t];
      W[t] = s;
    }
    __syncthreads();
    // W2 = T_p W (T upper triangular)
    if (t < QF_W) {
      const int k = t / QF_CW, c = t % QF_CW;
      float s = 0.f;
      for (int l = k; l < BW; ++l) s = fmaf(T[k * LDW + l], W[l * QF_CW + c], s);
      W2[t] = s;
    }
    __syncthreads();
    // X -= V_p W2 over rows >= r0: thread t owns rows r0 + t + 256 i of the 8 columns, so every W2
    // value read from shared memory feeds QF_ROWS rows
    {
      float out[QF_ROWS][QF_CW];
#pragma unroll
      for (int i = 0; i < QF_ROWS; ++i)
#pragma unroll
        for (int b = 0; b < QF_CW; ++b) out[i][b] = 0.f;
#pragma unroll 1
      for (int k4 = 0; k4 < BW / 4; ++k4) {
        float v[QF_ROWS][4];
#pragma unroll
        for (int i = 0; i < QF_ROWS; ++i) {
          const int r = r0 + t + QF_NT * i;
          const float4 x = (r < m) ? reinterpret_cast<const float4*>(Vp + (size_t)r * BW)[k4]
                                   : make_float4(0.f, 0.f, 0.f, 0.f);
          v[i][0] = x.x;
          v[i][1] = x.y;
          v[i][2] = x.z;
          v[i][3] = x.w;
        }
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const float4* wr = reinterpret_cast<const float4*>(W2 + (4 * k4 + kk) * QF_CW);
          float w[QF_CW];
#pragma unroll
          for (int h = 0; h < QF_CW / 4; ++h) {
            const float4 w4 = wr[h];
            w[4 * h] = w4.x;
            w[4 * h + 1] = w4.y;
            w[4 * h + 2] = w4.z;
            w[4 * h + 3] = w4.w;
          }
#pragma unroll
          for (int i = 0; i < QF_ROWS; ++i)
#pragma unroll
            for (int b = 0; b < QF_CW; ++b) out[i][b] = fmaf(v[i][kk], w[b], out[i][b]);
        }
      }
#pragma unroll
      for (int i = 0; i < QF_ROWS; ++i) {
        const int r = r0 + t + QF_NT * i;
        if (r < m) {
          float4* xr = reinterpret_cast<float4*>(X + r * QF_CW);
#pragma unroll
          for (int h = 0; h < QF_CW / 4; ++h) {
            const float4 x4 = xr[h];
            xr[h] = make_float4(x4.x - out[i][4 * h], x4.y - out[i][4 * h + 1], x4.z - out[i][4 * h + 2],
                                x4.w - out[i][4 * h + 3]);
          }
        }
      }
    }
  }
  __syncthreads();
  for (int e = t; e < m * QF_CW; e += QF_NT) {
    const int c = e / m, r = e % m;
    if (c0 + c < n) Q[(int64_t)r + (int64_t)(c0 + c) * m] = (double)X[r * QF_CW + c];
  }
}


cudaLaunchConfig_t launch_config(cudaLaunchAttribute* at, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = kSmemBytes;
  cfg.stream = s;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cfg;
}

}  // namespace

// True when the 16-CTA cluster kernel can run this shape on the current device.
bool tn_qr32_cluster_supported(int64_t m, int64_t n) {
  if (n < 1 || n > (int64_t)NBMAX * BW || m < n || m > MMAX) return false;
  // probed once per device (under a mutex, so concurrent first callers all see the probe's answer)
  static std::mutex mu;
  static signed char probed[TN_MAX_DEVICES] = {0};  // 0 unknown, 1 yes, -1 no
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= TN_MAX_DEVICES) return false;
  std::lock_guard<std::mutex> lk(mu);
  if (probed[dev]) return probed[dev] > 0;
  const bool available = [] {
    bool ok = false;
    if (cudaFuncSetAttribute(qr32_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess &&
        cudaFuncSetAttribute(qr32_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes) ==
            cudaSuccess) {
      cudaLaunchAttribute at[1];
      cudaLaunchConfig_t cfg = launch_config(at, 0);
      int clusters = 0;
      if (cudaOccupancyMaxActiveClusters(&clusters, qr32_cluster_kernel, &cfg) == cudaSuccess && clusters > 0)
        ok = true;
    }
    cudaGetLastError();  // an unsupported attribute leaves no sticky error behind
    return ok;
  }();
  probed[dev] = available ? 1 : -1;
  return available;
}

// Scratch floats for V and T of all panels of an m x n factorisation.
size_t tn_qr32_cluster_scratch_floats(int64_t m, int64_t n) {
  const int64_t np = tn_cdiv(n, BW);
  return (size_t)np * (m * BW + BW * BW);
}

// Q (column-major m x n, FP64 values of the FP32 factor) and, if r is given, R (n x n, strided).
// scratch: tn_qr32_cluster_scratch_floats(m, n) floats, 16-byte aligned.
int tn_qr32_cluster(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn, double* q, double* r,
                    int64_t sRm, int64_t sRn, float* scratch, cudaStream_t s) {
  if (!tn_qr32_cluster_supported(m, n)) return tn_fail(TN_ERR_ARG, "qr32 cluster: unsupported shape or device");
  if (((uintptr_t)scratch & 15) != 0) return tn_fail(TN_ERR_ARG, "qr32 cluster: scratch misaligned");
  int* err;
  int st = tn_error_word(s, &err);
  if (st) return st;
  const int64_t np = tn_cdiv(n, BW);
  float* Vg = scratch;
  float* Tg = scratch + (size_t)np * m * BW;
  cudaLaunchAttribute at[1];
  cudaLaunchConfig_t cfg = launch_config(at, s);
  TN_CUDA(cudaLaunchKernelEx(&cfg, qr32_cluster_kernel, (int)m, (int)n, a, sAm, sAn, r, sRm, sRn, Vg, Tg, err));
  TN_CHECK_LAUNCH();
  qr32_form_q_kernel<<<(unsigned)(np * (BW / QF_CW)), QF_NT, 0, s>>>((int)m, (int)n, Vg, Tg, q);
  TN_CHECK_LAUNCH();
  return TN_OK;
}
