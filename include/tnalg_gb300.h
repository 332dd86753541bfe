/*
 * tnalg_gb300 — C ABI of the GB300-native finite-size DMRG sweep.
 *
 * The reference (T-Nalg) is pure Python/numpy and has no FFI layer; its hot path
 * is MpsOpenBoundaryClass (MPSClass.py:26-1098) driven by dmrg_finite_size
 * (DMRG_anyH.py:18-101). Each entry point below replaces a numpy/scipy step of
 * that path, cited as file:line. The Python host (tnalg_gb300/MPSClass.py) binds
 * these functions with ctypes (tnalg_gb300/_lib.py).
 *
 * Conventions
 *  - All pointers except descriptor/option structs are DEVICE pointers owned by the
 *    caller (plain cudaMalloc or torch storage). Descriptor and option structs and
 *    result structs live in HOST memory.
 *  - Every function returns an int status (TN_OK == 0); nothing throws across the
 *    ABI. tn_last_error() returns a thread-local message for the last failure.
 *  - `stream` is a cudaStream_t passed as void*; every kernel of a call is queued
 *    on it. Calls are not re-entrant on one stream with one workspace.
 *  - Host threads: several threads may call the library at once, each with its own
 *    stream and workspaces (a multi-job host runs one job per thread). The library's
 *    shared host state (launch counter, FP64-QR graph cache, lazily resolved entry
 *    points) is synchronised. Process-wide and not for concurrent use: the profiler
 *    (tn_profile_*) and tn_qr_use_graphs.
 *  - Devices: every call works on the CURRENT device (cudaSetDevice); `stream` and all
 *    pointers must belong to it. Per-device state (SM count, kernel attributes, QR
 *    capture streams and graphs) is set up for each device on first use there.
 *  - Device errors (bounded waits that gave up, operands outside FP32 range) are
 *    recorded in an error word of the stream the failing kernel ran on, and reported
 *    by the next tn_check_device_status / tn_lanczos convergence check on that stream:
 *    jobs on their own streams never see or clear each other's errors.
 *  - Tensors are row-major FP64. An MPS site tensor is (chi_l, d, chi_r); an
 *    environment is (chi, chi) indexed [bra, ket] (TensorBasicModule.py:530-619).
 *  - Strides are in elements.
 */
#ifndef TNALG_GB300_H
#define TNALG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  TN_OK = 0,
  TN_ERR_ARG = 1,        /* invalid argument / unsupported shape */
  TN_ERR_CUDA = 2,       /* a CUDA runtime call failed */
  TN_ERR_WORKSPACE = 3,  /* workspace missing or too small */
  TN_ERR_NOCONV = 4,     /* eigensolver hit its iteration limit (result still usable) */
  TN_ERR_NUMERIC = 5,    /* NaN/Inf detected */
  TN_ERR_TIMEOUT = 6     /* a bounded device-side wait gave up */
};

enum { TN_PREC_FP64 = 0, TN_PREC_TF32X3 = 1 };

/* ---- library --------------------------------------------------------------- */
const char* tn_last_error(void);
int tn_version(void);
/* SM count and compute capability of the current device. */
int tn_device_info(int* sm_count, int* cc_major, int* cc_minor);
/* 1 if `precision` can run on the current device with this build. */
int tn_precision_available(int precision);
/* Kernels launched by this library so far (all entry points, all threads). */
unsigned long long tn_launch_count(void);

/* ---- contraction primitive -------------------------------------------------- */
/*
 * C[b] = alpha * sum_r A[b,r] . B[b,r] + beta * Cin[b]
 * A[b,r](m,k) = A[b*sAb + r*sAr + m*sAm + k*sAk], same pattern for B(k,n), C(m,n).
 * Cin may equal C or be NULL (then beta multiplies C itself).
 * Replaces the np.dot calls inside absorb_matrix2tensor / bound_vec_operator_*
 * (TensorBasicModule.py:387-424, 530-619).
 * precision: TN_PREC_FP64 (CUDA-core FP64) or TN_PREC_TF32X3 (tcgen05 tensor cores,
 * split-TF32 products with FP32 accumulation, FP64 in/out).
 * ws may be NULL; with ws the FP64 path splits K across CTAs for small outputs.
 */
int tn_gemm(int precision, int64_t M, int64_t N, int64_t K,
            const double* A, int64_t sAm, int64_t sAk,
            const double* B, int64_t sBk, int64_t sBn,
            double* C, int64_t sCm, int64_t sCn, const double* Cin,
            int64_t batch, int64_t sAb, int64_t sBb, int64_t sCb,
            int64_t nred, int64_t sAr, int64_t sBr,
            double alpha, double beta, void* ws, size_t ws_bytes, void* stream);
size_t tn_gemm_workspace_bytes(int precision, int64_t M, int64_t N, int64_t K, int64_t batch, int64_t nred);
/* Synchronise `stream` and report any error a bounded device-side wait recorded
 * (TN_ERR_TIMEOUT); the CUDA context stays usable. */
int tn_check_device_status(void* stream);

/* ---- effective-operator building blocks ------------------------------------ */
/* One term of a block operator: coeff * E[slot] (x) ops[op]; slot < 0 -> identity,
 * op < 0 -> identity. */
typedef struct {
  int32_t slot;
  int32_t op;
  double coeff;
} tn_block_term;

/*
 * Dense block operator of an enlarged block (classify_and_update_env buckets,
 * MPSClass.py:684-733, summed into one matrix):
 *   side == 0 (left):  W[(a',s'),(a,s)] = sum_t c_t E_t[a',a] O_t[s',s]   (chi*d)^2
 *   side == 1 (right): W[(s',b'),(s,b)] = sum_t c_t O_t[s',s] E_t[b',b]   (d*chi)^2
 * env: nslots x chi x chi (slot stride chi*chi); ops: nops x d x d; terms: DEVICE array.
 */
int tn_assemble_block(int side, int64_t chi, int64_t d, const double* env, const double* ops,
                      const tn_block_term* terms, int64_t nterms, double* w, void* stream);

/* out[g] = sum over terms t with group g of coeff_t * env[slot_t]; groups listed as a
 * DEVICE array of (group, slot, coeff) triples encoded as tn_block_term{slot, op=group}. */
int tn_combine_slots(int64_t chi, const double* env, const tn_block_term* terms, int64_t nterms,
                     int64_t ngroups, double* out, void* stream);

/* out[k][a,s',b] = sum_s ops[opidx[k]][s',s] in[a,s,b]   (absorb_matrix2tensor on the
 * physical bond, TensorBasicModule.py:414-421). opidx: DEVICE int32 array (-1 = identity). */
int tn_apply_site_ops(int64_t chil, int64_t d, int64_t chir, const double* in, const double* ops,
                      const int32_t* opidx, int64_t nout, double* out, int64_t out_stride, void* stream);

/* out[s',s] += alpha * sum_{x,z} M[x,s',z] T[x,s,z]   (d <= 4): the local reduced density
 * matrix used by observation_s1 / observation_s1_s2 (MPSClass.py:857-909). out: d*d DEVICE. */
int tn_pair_contract(int64_t chil, int64_t d, int64_t chir, const double* m, const double* t,
                     double alpha, double* out, void* stream);

/* ---- effective Hamiltonian matvec ----------------------------------------------- */
typedef struct {
  int64_t chil, d, chir;
  const double* wl;   /* (chil*d)^2 left block incl. on-site terms, or NULL */
  const double* wr;   /* (d*chir)^2 right block, or NULL */
  int64_t nstr;       /* straddling pairs: sum_k SL[k] (x) 1 (x) SR[k] */
  const double* sl;   /* nstr x chil x chil (coefficients folded in) */
  const double* sr;   /* nstr x chir x chir */
} tn_site_desc;

/*
 * y = beta * psi + alpha * H_eff psi  with H_eff = WL (x) 1 + 1 (x) WR + sum_k SL_k (x) 1 (x) SR_k.
 * Replaces update_tensor_eigs_f_handle_optimized (MPSClass.py:755-776), which is the
 * case alpha = -tau, beta = 1.
 */
int tn_matvec(const tn_site_desc* desc, const double* psi, double* y, double alpha, double beta,
              int precision, void* ws, size_t ws_bytes, void* stream);
size_t tn_matvec_workspace_bytes(const tn_site_desc* desc, int precision);

/* ---- local eigensolver ---------------------------------------------------------- */
typedef struct {
  double eigs_tol;      /* tolerance as passed to the reference's eigsh */
  double tau;           /* the reference's shift; tol on ||Hx - t x|| = eigs_tol/tau*|1-tau*t| */
  double tol_cap;       /* if > 0: residual tol = min(above, tol_cap * max(1, |t|)) */
  double mixed_floor;   /* TF32X3: residual floor relative to |t| (precision limit) */
  int32_t max_krylov;   /* Lanczos vectors per restart */
  int32_t max_restarts;
  int32_t check_every;  /* steps between host convergence checks */
  int32_t precision;    /* matvec precision */
  int32_t refine;       /* 1: FP64 residual + Rayleigh quotient of the final vector;
                           2 (TF32X3): refine the vector itself: after the split-TF32 iteration
                           reaches mixed_floor, restart cycles that open with an FP64 matvec run
                           until the FP64 residual meets the FP64 tolerance (energy = FP64 x.Hx) */
  int32_t refine_cycles; /* refine == 2: at most this many FP64-opened cycles (0 = 4) */
} tn_lanczos_opts;

typedef struct {
  double energy;        /* Ritz value of H_eff */
  double residual;      /* ||H x - energy x|| (estimate, or FP64 value when refined) */
  double energy_fp64;   /* FP64 Rayleigh quotient x.Hx (refine == 1 or 2) */
  int32_t matvecs;
  int32_t restarts;
  int32_t converged;
  int32_t reserved;
} tn_lanczos_result;

/*
 * Lowest eigenpair of H_eff by Lanczos with full (classical Gram-Schmidt, twice)
 * reorthogonalisation; Krylov basis, dot products and the tridiagonal problem in
 * FP64. psi_inout: start vector in, unit eigenvector out.
 * Replaces eigsh(LinearOperator(I - tau*H_eff), k=1, which='LM', v0=psi, tol)
 * (MPSClass.py:800-807; same eigenvector, eigenvalue reported for H_eff).
 */
int tn_lanczos(const tn_site_desc* desc, double* psi_inout, const tn_lanczos_opts* opts,
               void* ws, size_t ws_bytes, tn_lanczos_result* result, void* stream);
size_t tn_lanczos_workspace_bytes(const tn_site_desc* desc, const tn_lanczos_opts* opts);

/* ---- gauge move ------------------------------------------------------------------ */
/*
 * Thin Householder QR in FP64 of the m x n matrix A (general strides):
 * A = Q R, Q: m x k with orthonormal columns, R: k x n upper trapezoidal, k = min(m, n).
 * Replaces np.linalg.qr in left2right_decompose_tensor / right2left_decompose_tensor
 * (TensorBasicModule.py:314-384). Columns of Q are those of LAPACK up to sign.
 */
int tn_qr(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn,
          double* q, int64_t sQm, int64_t sQn, double* r, int64_t sRm, int64_t sRn,
          void* ws, size_t ws_bytes, void* stream);
size_t tn_qr_workspace_bytes(int64_t m, int64_t n);
/*
 * Gauge move of the mixed-precision sweep: same outputs as tn_qr, but Q comes from an FP32
 * Householder QR re-orthogonalised in FP64 (||Q^T Q - I|| ~ 1e-12, col(Q) = col(A) to FP32
 * accuracy) and R is accurate to FP32 only. Meant for moves whose R is absorbed into a site
 * that is re-optimised next (the seed of the next local solve). q is required.
 */
int tn_qr_mixed(int64_t m, int64_t n, const double* a, int64_t sAm, int64_t sAn,
                double* q, int64_t sQm, int64_t sQn, double* r, int64_t sRm, int64_t sRn,
                void* ws, size_t ws_bytes, void* stream);
size_t tn_qr_mixed_workspace_bytes(int64_t m, int64_t n);
/* tn_qr replays one captured CUDA graph per (shape, strides, workspace) (default on); 0 turns
 * replay off (plain launches). A stream that is already capturing always gets plain launches. */
int tn_qr_use_graphs(int on);

/* ---- entanglement spectrum ---------------------------------------------------------- */
/*
 * Singular values of the k x n matrix X (general strides) by parallel one-sided
 * Jacobi in FP64; s_out (DEVICE, k values, unsorted). Replaces np.linalg.svd in the
 * SVD moves of calculate_entanglement_spectrum (MPSClass.py:812-832,
 * TensorBasicModule.py:338-342,374-377). tol: relative off-diagonal threshold.
 */
int tn_singular_values(int64_t k, int64_t n, const double* x, int64_t sXr, int64_t sXc, double* s_out,
                       double tol, int max_sweeps, void* ws, size_t ws_bytes, void* stream);
size_t tn_singular_values_workspace_bytes(int64_t k, int64_t n);

/*
 * Thin SVD X = U diag(s) Vt of the k x n matrix X (general strides) by the same one-sided Jacobi,
 * with the rotations accumulated: s (k values, unsorted, DEVICE), U (k x k, column i belongs to s[i],
 * row-major with leading dimension ldu; may be NULL), Vt (k x n, row i = the rotated row i / s[i],
 * zero for s[i] == 0; leading dimension ldvt; may be NULL). The decomposition behind truncation:
 * keeping the largest chi values of s with their columns of U and rows of Vt gives the best rank-chi
 * approximation (the truncated svd of decompose(..., way='svd'), TensorBasicModule.py:338-342).
 * ws: 256-byte aligned DEVICE scratch of tn_svd_jacobi_workspace_bytes(k, n).
 */
int tn_svd_jacobi(int64_t k, int64_t n, const double* x, int64_t sXr, int64_t sXc, double* s_out, double* U,
                  int64_t ldu, double* Vt, int64_t ldvt, double tol, int max_sweeps, void* ws, size_t ws_bytes,
                  void* stream);
size_t tn_svd_jacobi_workspace_bytes(int64_t k, int64_t n);

/*
 * Self-test of the library's bounded device waits: a 2-block kernel waits at a grid barrier that
 * can never complete (it expects a third block); every block gives up after its wait limit (~2 s)
 * and records the timeout in the error word of `stream`, which this call reads and clears. Returns
 * TN_ERR_TIMEOUT when the bounded wait worked; the context stays usable. ws: 256-byte aligned DEVICE
 * scratch of at least 256 bytes. Synchronises stream. Diagnostic only; no counterpart in the
 * reference.
 */
int tn_selftest_wait_timeout(void* ws, size_t ws_bytes, void* stream);

/*
 * tn_singular_values without a workspace argument and without any device allocation. It has no
 * counterpart in the reference: it exists for hosts that cannot allocate device memory
 * themselves (a service that may only use buffers registered by its own allocator, or a process
 * whose device memory is owned by another framework's allocator) but still want an
 * entanglement spectrum. Its scratch is a static device array of 65536 + 32 doubles (512 KiB)
 * that every GPU loading the library keeps until the process exits; (k rounded up to even) * n
 * must be <= 65536, larger sizes return TN_ERR_ARG. The first call on each device resolves the
 * array's device address (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture. All calls share the array: calls that overlap on the GPU race, so
 * the caller serialises them. Same arguments and results as tn_singular_values otherwise.
 */
int tn_singular_values_noalloc(int64_t k, int64_t n, const double* x, int64_t sXr, int64_t sXc,
                               double* s_out, double tol, int max_sweeps, void* stream);

/*
 * Singular values of `count` independent matrices at once (the same FP64 Jacobi algorithm, one
 * launch per round for the whole batch): the R factors of every bond collected by one sweep of
 * gauge moves, which is how calculate_entanglement_spectrum (MPSClass.py:812-832) fills lm for
 * all bonds. items is a HOST array; x and s_out in every item are DEVICE pointers. ws: 256-byte
 * aligned DEVICE scratch of tn_singular_values_batched_workspace_bytes(count, items) bytes.
 * Synchronises stream. No counterpart in the reference (which takes one SVD per move).
 */
typedef struct tn_sv_item {
  int64_t k, n;        /* rows, columns */
  const double* x;     /* DEVICE, element (r, c) at x[r * sXr + c * sXc] */
  int64_t sXr, sXc;
  double* s_out;       /* DEVICE, k singular values (unsorted) */
} tn_sv_item;
int tn_singular_values_batched(int count, const tn_sv_item* items, double tol, int max_sweeps, void* ws,
                               size_t ws_bytes, void* stream);
size_t tn_singular_values_batched_workspace_bytes(int count, const tn_sv_item* items);

/* ---- grouped contractions (many independent jobs per launch) --------------------------- */
/*
 * One contraction of a group (or `batch` contractions A_z . B_z -> C_z at strides sAb, sBb, sCb):
 * C = alpha * sum_r A_r . B_r + beta * C (accumulate == 0; the problem
 * must then be the only writer of its C in the call), or C += alpha * sum_r A_r . B_r added
 * atomically (accumulate == 1; several problems may add into one C).
 * A_r(m, k) = A[r*sAr + m*sAm + k*sAk], B_r(k, n) = B[r*sBr + k*sBk + n*sBn], C(m, n) = C[m*sCm + n*sCn].
 * active: DEVICE int32 flag or NULL; the problem is skipped when *active == 0 at launch time.
 * These are the per-job np.dot calls of a local update (MPSClass.py:755-776, transfer
 * contractions TensorBasicModule.py:530-619, R-absorb :387-424) of many independent jobs.
 */
typedef struct {
  int32_t M, N, K, nred;
  const double* A; int64_t sAm, sAk, sAr;
  const double* B; int64_t sBk, sBn, sBr;
  double* C; int64_t sCm, sCn;
  double alpha, beta;
  int32_t accumulate, batch;       /* batch: z = 0..batch-1 (0 counts as 1); nred must be 1 when batch > 1 */
  int64_t sAb, sBb, sCb;           /* batch strides of A, B and C */
  const int32_t* active;
} tn_grouped_gemm_problem;

/*
 * Every problem of a HOST table in one grouped launch. TN_PREC_TF32X3: operands staged as split-TF32
 * tiles (one launch), then one persistent tcgen05 launch over all output tiles; TN_PREC_FP64:
 * CUDA-core FP64 tiles. ws: DEVICE scratch of tn_grouped_gemm_workspace_bytes bytes (tables and
 * staged operands). No counterpart in the reference, which runs these products one at a time.
 */
int tn_grouped_gemm(int precision, const tn_grouped_gemm_problem* problems, int count, void* ws, size_t ws_bytes,
                    void* stream);
size_t tn_grouped_gemm_workspace_bytes(int precision, const tn_grouped_gemm_problem* problems, int count);

/*
 * Output tile width (64 or 128 columns; 0 restores the default, 128) of the split-TF32 grouped GEMMs
 * that the CALLING HOST THREAD issues from now on (tn_grouped_gemm, tn_batched_lanczos,
 * tn_batched_step, tn_batched_qr_mixed). The setting is thread-local, so engines on different
 * threads tune independently; the results do not depend on it (the same products are summed in
 * the same order). Picked by tnalg_gb300/tuner.py from a measured table. No counterpart in the
 * reference.
 */
int tn_set_grouped_tile(int tile_n);
int tn_get_grouped_tile(void);

/* ---- grouped building blocks and the batched gauge move --------------------------------- */
enum { TN_BOP_BLOCK_LEFT = 0, TN_BOP_BLOCK_RIGHT = 1, TN_BOP_COMBINE = 2, TN_BOP_SITE_OPS = 3 };

/*
 * One item of tn_grouped_ops:
 *  TN_BOP_BLOCK_LEFT / _RIGHT: a block operator as tn_assemble_block (side 0 / 1) into out,
 *      (chi*d)^2 values; terms: DEVICE tn_block_term[nterms];
 *  TN_BOP_COMBINE: out[g] = sum_t c_t E[slot_t] as tn_combine_slots (group in the op field), groups
 *      out_stride apart, total = ngroups * chi^2;
 *  TN_BOP_SITE_OPS: out[k] = ops[opidx[k]] on the physical bond of the (chi, d, chir) tensor src, as
 *      tn_apply_site_ops; terms: DEVICE int32 opidx[nterms], outputs out_stride apart.
 * Environment element (slot, r, c) at src[slot*s_slot + r*s_row + c]. total: output elements.
 * active: DEVICE flag or NULL (skipped when *active == 0).
 */
typedef struct {
  int32_t kind;
  int32_t chi, d, chir;
  int32_t nterms, reserved;
  const double* src;
  int64_t s_slot, s_row;
  const double* ops;
  const void* terms;
  double* out;
  int64_t out_stride;
  int64_t total;
  const int32_t* active;
} tn_batch_op;

/* Every item of a HOST table in one launch (the per-job block assembly, slot gathers and site
 * operators of MPSClass.py:684-733 and TensorBasicModule.py:414-421 for many jobs). ws: DEVICE
 * scratch of tn_grouped_ops_workspace_bytes(count). No counterpart in the reference. */
int tn_grouped_ops(const tn_batch_op* items, int count, void* ws, size_t ws_bytes, void* stream);
size_t tn_grouped_ops_workspace_bytes(int count);

/* One gauge move of tn_batched_qr_mixed: A (m x n, 1 <= n <= m, m*n <= 32768, general strides) is
 * replaced by Q (orthonormal columns), R (n x n upper) written to r. */
typedef struct {
  int32_t m, n;
  double* a; int64_t sAm, sAn;
  double* r; int64_t sRm, sRn;
  const int32_t* active;
} tn_qr_item;

/*
 * The QR gauge moves (left2right / right2left_decompose_tensor, TensorBasicModule.py:314-384) of
 * many jobs at once, in tn_qr_mixed's precision: FP32 Householder per matrix (one CTA each, the
 * matrix in shared memory), Q re-orthogonalised in FP64 (||Q^T Q - I|| ~ 1e-12, col(Q) = col(A) to
 * FP32 accuracy), R accurate to FP32 (it seeds the next local solve). Q overwrites A in place.
 * Needs an sm_103 device. items: HOST table; ws: DEVICE scratch.
 */
int tn_batched_qr_mixed(const tn_qr_item* items, int count, void* ws, size_t ws_bytes, void* stream);
size_t tn_batched_qr_mixed_workspace_bytes(const tn_qr_item* items, int count);

/* ---- batched local solves -------------------------------------------------------------- */
/* One job of a batched solve: its effective Hamiltonian and its start / result vectors. */
typedef struct {
  tn_site_desc site;       /* WL, WR and straddling pairs SL, SR */
  const double* psi_in;    /* DEVICE start vector, chil*d*chir values */
  double* psi_out;         /* DEVICE unit eigenvector (may equal psi_in) */
} tn_batch_solve;

/*
 * The lowest eigenpair of every job's effective Hamiltonian, all jobs advanced together: the
 * eigsh of update_tensor_eigs (MPSClass.py:778-809) for many independent DMRG jobs. Lanczos with
 * classical Gram-Schmidt applied twice, as tn_lanczos; one grouped matvec launch (split TF32 or
 * FP64 by opts->precision) and grouped vector kernels per step for all jobs, the tridiagonal
 * eigenpairs and the convergence test on the device (one warp per job); the host reads one
 * counter per check (opts->check_every steps). max_krylov <= 64; refine must be 0 or 1 (1 is
 * accepted and ignored: energy_fp64 = energy). jobs and results are HOST arrays; ws is DEVICE
 * scratch of tn_batched_lanczos_workspace_bytes bytes. Returns TN_ERR_NOCONV if any job hit the
 * restart limit (its last Ritz vector is written). results[i].matvecs counts the batch's steps.
 */
int tn_batched_lanczos(const tn_batch_solve* jobs, int count, const tn_lanczos_opts* opts, void* ws,
                       size_t ws_bytes, tn_lanczos_result* results, void* stream);
size_t tn_batched_lanczos_workspace_bytes(const tn_batch_solve* jobs, int count, const tn_lanczos_opts* opts);

/* ---- one local update of many jobs ------------------------------------------------------ */
/*
 * The launch records of one local update (one step of the sweep loop of dmrg_finite_size,
 * DMRG_anyH.py:43-64: the gauge move and environment update of correct_orthogonal_center,
 * MPSClass.py:188-198, 202-325, then update_tensor_eigs, MPSClass.py:778-809) for every job of a
 * batch, concatenated over the jobs. They run in this order on one stream:
 *   ops1  block operator of the environment being extended (tn_grouped_ops)
 *   qr    the gauge move of the site left behind, Q in place (tn_batched_qr_mixed; a matrix with
 *         m n > 32768 goes through tn_qr_mixed and must have a dense layout and no active flag)
 *   gemm1 R absorbed into the next site and the products of the environment update
 *   ops2  site operators of the environment update
 *   gemm2 the new environment slots
 *   ops3  the effective Hamiltonian of the next site (WL, WR, straddling pairs)
 *   solves the local solve of every job (tn_batched_lanczos with opts)
 * gemm1 and gemm2 run in `precision` (TN_PREC_TF32X3 or TN_PREC_FP64). Every table is a HOST
 * array; a count of 0 skips its phase. No counterpart in the reference, which runs one job's
 * update at a time.
 */
typedef struct {
  const tn_batch_op* ops1;
  const tn_qr_item* qr;
  const tn_grouped_gemm_problem* gemm1;
  const tn_batch_op* ops2;
  const tn_grouped_gemm_problem* gemm2;
  const tn_batch_op* ops3;
  const tn_batch_solve* solves;
  int32_t n_ops1, n_qr, n_gemm1, n_ops2, n_gemm2, n_ops3, n_solves;
  int32_t precision;
} tn_batch_step_desc;

/* One local update of every job: the phases above, then results[i] of solves[i]. ws: DEVICE
 * scratch of tn_batched_step_workspace_bytes bytes (shared by the phases). Returns TN_ERR_NOCONV as
 * tn_batched_lanczos does. */
int tn_batched_step(const tn_batch_step_desc* desc, const tn_lanczos_opts* opts, void* ws, size_t ws_bytes,
                    tn_lanczos_result* results, void* stream);
size_t tn_batched_step_workspace_bytes(const tn_batch_step_desc* desc, const tn_lanczos_opts* opts);

/* ---- profiling ----------------------------------------------------------------------- */
/* CUDA-event timing of kernel classes on their launching stream (0 = effective-Hamiltonian
 * matvecs inside tn_lanczos). Off by default; reading synchronises the recorded events. */
int tn_profile_enable(int on);
int tn_profile_reset(void);
int tn_profile_read(int cls, double* ms, int64_t* count, double* flops);

/* ---- small vector helpers ------------------------------------------------------- */
/* out[0] = sum x[i]*y[i] (FP64, deterministic two-stage reduction). */
int tn_dot(int64_t n, const double* x, const double* y, double* out, void* ws, size_t ws_bytes,
           void* stream);
/* x[i] *= alpha / sqrt(nrm2[0]) when nrm2 != NULL, else x[i] *= alpha. */
int tn_scale(int64_t n, double* x, double alpha, const double* nrm2, void* stream);
/* eye: n x n identity into a (row stride lda). */
int tn_set_identity(int64_t n, double* a, int64_t lda, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TNALG_GB300_H */
