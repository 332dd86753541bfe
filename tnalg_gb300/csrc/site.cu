// Effective-operator building blocks and small vector kernels.
//
// These replace the bookkeeping of MPSClass.py:684-733 (bucket accumulation),
// the physical-bond absorption of TensorBasicModule.py:414-421 and the traces of
// MPSClass.py:857-909. All are HBM-bound elementwise/reduction kernels.
#include "common.cuh"

namespace {

constexpr int NT = 256;

__device__ __forceinline__ double op_elem(const double* ops, int op, int64_t d, int64_t r, int64_t c) {
  return op < 0 ? (r == c ? 1.0 : 0.0) : ops[(int64_t)op * d * d + r * d + c];
}
__device__ __forceinline__ double env_elem(const double* env, int slot, int64_t chi, int64_t r, int64_t c) {
  return slot < 0 ? (r == c ? 1.0 : 0.0) : env[(int64_t)slot * chi * chi + r * chi + c];
}

// side 0: W[(a',s'),(a,s)] = sum_t c E[a',a] O[s',s];  side 1: W[(s',b'),(s,b)] = sum_t c O[s',s] E[b',b]
__global__ void assemble_block_kernel(int side, int64_t chi, int64_t d, const double* __restrict__ env,
                                      const double* __restrict__ ops, const tn_block_term* __restrict__ terms,
                                      int64_t nterms, double* __restrict__ w) {
  const int64_t n = chi * d;
  const int64_t total = n * n;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = idx / n, col = idx % n;
    int64_t er, ec, orr, oc;
    if (side == 0) {
      er = row / d; orr = row % d; ec = col / d; oc = col % d;
    } else {
      orr = row / chi; er = row % chi; oc = col / chi; ec = col % chi;
    }
    double acc = 0.0;
    for (int64_t t = 0; t < nterms; ++t) {
      const tn_block_term tt = terms[t];
      const double o = op_elem(ops, tt.op, d, orr, oc);
      if (o == 0.0) continue;
      const double e = env_elem(env, tt.slot, chi, er, ec);
      acc = fma(tt.coeff * o, e, acc);
    }
    w[idx] = acc;
  }
}

// out[g][r][c] = sum_{t: group(t)==g} coeff_t * env[slot_t][r][c]
__global__ void combine_slots_kernel(int64_t chi, const double* __restrict__ env,
                                     const tn_block_term* __restrict__ terms, int64_t nterms, int64_t ngroups,
                                     double* __restrict__ out) {
  const int64_t m = chi * chi;
  const int64_t total = ngroups * m;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = idx / m, e = idx % m;
    double acc = 0.0;
    for (int64_t t = 0; t < nterms; ++t) {
      const tn_block_term tt = terms[t];
      if (tt.op != g) continue;
      const double v = tt.slot < 0 ? ((e / chi) == (e % chi) ? 1.0 : 0.0) : env[(int64_t)tt.slot * m + e];
      acc = fma(tt.coeff, v, acc);
    }
    out[idx] = acc;
  }
}

__global__ void apply_site_ops_kernel(int64_t chil, int64_t d, int64_t chir, const double* __restrict__ in,
                                      const double* __restrict__ ops, const int32_t* __restrict__ opidx,
                                      int64_t nout, double* __restrict__ out, int64_t out_stride) {
  const int64_t per = chil * d * chir;
  const int64_t total = nout * per;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = idx / per, e = idx % per;
    const int64_t a = e / (d * chir), sp = (e / chir) % d, b = e % chir;
    const int op = opidx[k];
    double acc = 0.0;
    for (int64_t s = 0; s < d; ++s) acc = fma(op_elem(ops, op, d, sp, s), in[(a * d + s) * chir + b], acc);
    out[k * out_stride + e] = acc;
  }
}

// out[s',s] += alpha * sum_{x,z} M[x,s',z] T[x,s,z]; d <= 4. One atomicAdd per block per entry.
__global__ void pair_contract_kernel(int64_t chil, int64_t d, int64_t chir, const double* __restrict__ m,
                                     const double* __restrict__ t, double alpha, double* out) {
  double acc[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) acc[i] = 0.0;
  const int64_t total = chil * chir;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = idx / chir, z = idx % chir;
    double mv[4], tv[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      mv[s] = s < d ? m[(x * d + s) * chir + z] : 0.0;
      tv[s] = s < d ? t[(x * d + s) * chir + z] : 0.0;
    }
#pragma unroll
    for (int sp = 0; sp < 4; ++sp)
#pragma unroll
      for (int s = 0; s < 4; ++s) acc[sp * 4 + s] = fma(mv[sp], tv[s], acc[sp * 4 + s]);
  }
  __shared__ double red[16][NT / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const double v = tn_warp_sum(acc[i]);
    if (lane == 0) red[i][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < 16) {
    const int i = threadIdx.x;
    const int sp = i / 4, s = i % 4;
    if (sp < d && s < d) {
      double v = 0.0;
      for (int w = 0; w < NT / 32; ++w) v += red[i][w];
      atomicAdd(out + sp * d + s, alpha * v);
    }
  }
}

// Deterministic dot: per-block partials, last block sums them in order.
__global__ void dot_kernel(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                           double* part, unsigned int* ticket, double* out) {
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc = fma(x[i], y[i], acc);
  __shared__ double red[NT / 32];
  __shared__ bool last;
  acc = tn_warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < NT / 32; ++w) v += red[w];
    part[blockIdx.x] = v;
    __threadfence();
    last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {  // uniform over the block
    const double v = tn_block_sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      *out = v;
      *ticket = 0u;
    }
  }
}

__global__ void scale_kernel(int64_t n, double* x, double alpha, const double* nrm2) {
  const double s = nrm2 ? alpha / sqrt(*nrm2) : alpha;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= s;
}

__global__ void set_identity_kernel(int64_t n, double* a, int64_t lda) {
  const int64_t total = n * n;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx / n, c = idx % n;
    a[r * lda + c] = (r == c) ? 1.0 : 0.0;
  }
}

int grid_for(int64_t total) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(total, NT), 16LL * tn_sm_count()));
}

}  // namespace

extern "C" int tn_assemble_block(int side, int64_t chi, int64_t d, const double* env, const double* ops,
                                 const tn_block_term* terms, int64_t nterms, double* w, void* stream) {
  if (chi <= 0 || d <= 0 || !w || (side != 0 && side != 1) || nterms < 0) return tn_fail(TN_ERR_ARG, "assemble_block: bad args");
  const int64_t total = chi * d * chi * d;
  assemble_block_kernel<<<grid_for(total), NT, 0, (cudaStream_t)stream>>>(side, chi, d, env, ops, terms, nterms, w);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

extern "C" int tn_combine_slots(int64_t chi, const double* env, const tn_block_term* terms, int64_t nterms,
                                int64_t ngroups, double* out, void* stream) {
  if (chi <= 0 || ngroups < 0 || nterms < 0) return tn_fail(TN_ERR_ARG, "combine_slots: bad args");
  if (ngroups == 0) return TN_OK;
  const int64_t total = ngroups * chi * chi;
  combine_slots_kernel<<<grid_for(total), NT, 0, (cudaStream_t)stream>>>(chi, env, terms, nterms, ngroups, out);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

extern "C" int tn_apply_site_ops(int64_t chil, int64_t d, int64_t chir, const double* in, const double* ops,
                                 const int32_t* opidx, int64_t nout, double* out, int64_t out_stride, void* stream) {
  if (chil <= 0 || d <= 0 || chir <= 0 || nout < 0 || out_stride < chil * d * chir)
    return tn_fail(TN_ERR_ARG, "apply_site_ops: bad args");
  if (nout == 0) return TN_OK;
  const int64_t total = nout * chil * d * chir;
  apply_site_ops_kernel<<<grid_for(total), NT, 0, (cudaStream_t)stream>>>(chil, d, chir, in, ops, opidx, nout, out,
                                                                          out_stride);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

extern "C" int tn_pair_contract(int64_t chil, int64_t d, int64_t chir, const double* m, const double* t,
                                double alpha, double* out, void* stream) {
  if (d < 1 || d > 4 || chil <= 0 || chir <= 0) return tn_fail(TN_ERR_ARG, "pair_contract: need 1 <= d <= 4");
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(chil * chir, NT), 2LL * tn_sm_count()));
  pair_contract_kernel<<<blocks, NT, 0, (cudaStream_t)stream>>>(chil, d, chir, m, t, alpha, out);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

// ws layout for tn_dot: [ticket (8 B)] [partials: blocks doubles]
int tn_dot_ws(int64_t n, const double* x, const double* y, double* out, void* ws, size_t ws_bytes, cudaStream_t s) {
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tn_cdiv(n, NT), 2LL * tn_sm_count()));
  if (!ws || ws_bytes < 16 + (size_t)blocks * sizeof(double)) return tn_fail(TN_ERR_WORKSPACE, "dot: workspace too small");
  unsigned int* ticket = (unsigned int*)ws;
  double* part = (double*)((char*)ws + 16);
  dot_kernel<<<blocks, NT, 0, s>>>(n, x, y, part, ticket, out);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

extern "C" int tn_dot(int64_t n, const double* x, const double* y, double* out, void* ws, size_t ws_bytes,
                      void* stream) {
  if (n <= 0) return tn_fail(TN_ERR_ARG, "dot: n <= 0");
  return tn_dot_ws(n, x, y, out, ws, ws_bytes, (cudaStream_t)stream);
}

extern "C" int tn_scale(int64_t n, double* x, double alpha, const double* nrm2, void* stream) {
  if (n <= 0) return TN_OK;
  scale_kernel<<<grid_for(n), NT, 0, (cudaStream_t)stream>>>(n, x, alpha, nrm2);
  TN_CHECK_LAUNCH();
  return TN_OK;
}

extern "C" int tn_set_identity(int64_t n, double* a, int64_t lda, void* stream) {
  if (n <= 0 || lda < n) return tn_fail(TN_ERR_ARG, "set_identity: bad args");
  set_identity_kernel<<<grid_for(n * n), NT, 0, (cudaStream_t)stream>>>(n, a, lda);
  TN_CHECK_LAUNCH();
  return TN_OK;
}
