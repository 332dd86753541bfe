// Internal tables of the grouped GEMMs (grouped_gemm.cu) shared with the batched DMRG kernels.
#pragma once
#include <stdint.h>

#include "common.cuh"

// One FP64 operand view converted to split-TF32 tile pairs: element (row, k) of reduction term r
// at src[r * s_red + row * s_row + k * s_k]; written as nred x n_rt x n_kb tile pairs of
// 128 rows x 32 (hi tile, then lo tile, 128B-swizzled rows) at dst.
struct GgStage {
  const double* src;
  int64_t s_row, s_k, s_red;
  int32_t rows, K, nred, n_rt, n_kb, pad;
  float* dst;
  const int32_t* active;  // skipped when *active == 0
};

// One split-TF32 problem over staged operands: C (M x N) = alpha sum_r A_r B_r (+ beta C, or
// added atomically when accumulate).
struct GgProblem {
  int32_t M, N, n_kb, nred, n_nt, a_nrt, b_nrt, accumulate;
  int32_t nbatch, n_mt;  // batch entries z (each its own staged A_z, B_z and output C + z sCb)
  const float* a;
  const float* b;
  double* C;
  int64_t sCm, sCn, sCb;
  double alpha, beta;
  const int32_t* active;
};

// One FP64 problem read in place.
struct GgF64Problem {
  int32_t M, N, K, nred;
  const double* A;
  int64_t sAm, sAk, sAr;
  const double* B;
  int64_t sBk, sBn, sBr;
  double* C;
  int64_t sCm, sCn;
  double alpha, beta;
  int32_t accumulate, nbatch;
  int64_t sAb, sBb, sCb;
  const int32_t* active;
};

size_t gg_staged_floats(int64_t rows, int64_t K, int64_t nred);
void gg_stage_shape(GgStage* it, int64_t rows, int64_t K, int64_t nred);
int gg_stage_tiles(const GgStage& it);
int gg_tf32_tiles(const GgProblem& p, int bn);
int gg_f64_tiles(const GgF64Problem& p);
int gg_launch_stage(const GgStage* dev_items, int nitems, const int* dev_prefix, int total_tiles, cudaStream_t s);
// ctas <= 0: one CTA per SM
int gg_launch_tf32(const GgProblem* dev_probs, int nprobs, const int* dev_prefix, int total_tiles, int bn, int ctas,
                   cudaStream_t s);
int gg_launch_f64(const GgF64Problem* dev_probs, int nprobs, const int* dev_prefix, int total_tiles, cudaStream_t s);
bool tn_tf32x3_supported();
// output tile width (64 or 128 columns) of the split-TF32 grouped GEMMs issued by the calling host
// thread: tn_set_grouped_tile, 128 unless set
int gg_tile_n();
