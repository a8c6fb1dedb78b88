/*
 * stile_gb300 -- C ABI of the GB300 (sm_103a) hybrid sparse-tile SpMM / SDDMM
 * path.  Plain pointers and sizes only; every entry point returns 0 on
 * success or a negative status (STILE_E_*), never aborts, and records a
 * message readable through stile_last_error().
 *
 * Reference interfaces replaced (STile, paths relative to the project root):
 *   stile_spmm_plan_upload / stile_sddmm_plan_upload
 *       -- prepare_inputs_BSPMM / prepare_inputs_BSDDMM upload the packed
 *          format arrays with tvm.nd.array(..., device=dev)
 *          (MY_sparse/my_fuse_formats.py:3321-3332, :3544-3678)
 *   stile_spmm_run / stile_spmm_run_bf16
 *       -- the fused SpMM PackedFunc f(*args_nd) launched by
 *          measure_latency_BSPMM (MY_sparse/my_fuse_formats.py:4152-4173),
 *          fp32 or bf16 dense operand
 *   stile_sddmm_run
 *       -- the fused SDDMM PackedFunc launched by measure_latency_BSDDMM
 *          (MY_sparse/my_fuse_formats.py:4292-4330) plus the host-side
 *          output reorder order_output_BSDDMM (:4247-4288), done on device
 *   stile_spmm_dvals
 *       -- no counterpart: value gradient of the SpMM (SDDMM on A's pattern
 *          walking the forward tile layout), used by the autograd backward
 *   stile_csr_spmm_run
 *       -- the plain CSR SpMM comparator (the reference times cuSPARSE CSR
 *          through torch.sparse_csr_tensor @ B, gen_formats_v2.py:3079-3106)
 *   stile_spmm_plan_free / stile_sddmm_plan_free / stile_last_error /
 *   stile_spmm_plan_error_flag / stile_spmm_plan_set_wait_policy
 *       -- ownership and error reporting (the reference relies on TVM
 *          NDArray lifetimes and asserts)
 *
 * Streams are passed as void* (a cudaStream_t; NULL = legacy default
 * stream).  All device pointers are caller-owned except the plan arrays,
 * which the plan handle owns.
 */
#ifndef STILE_GB300_H_
#define STILE_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define STILE_OK 0
#define STILE_E_INVALID (-1)   /* bad argument or malformed plan */
#define STILE_E_CUDA (-2)      /* a CUDA runtime call failed */
#define STILE_E_DEVICE (-3)    /* a kernel reported a device-side error */
#define STILE_E_UNSUPPORTED (-4)

/* element types of dense operands / tensor-tile values */
#define STILE_F32 0
#define STILE_BF16 1
#define STILE_F16 2
/* tensor-tile precision modes */
#define STILE_TC_BF16 1        /* A, B rounded to bf16, fp32 accumulate */
#define STILE_TC_F16 2         /* A, B rounded to fp16, fp32 accumulate */
#define STILE_TC_SPLIT_BF16 4  /* hi+lo bf16 split of A and B, 4 products */
#define STILE_TC_FP8 3         /* A e4m3 (per-tensor scale), B e4m3 (per tile-row
                                  scale), fp32 accumulate; fp32 B operands */


/*
 * SpMM plan, device-ready host arrays (built by the emitter).
 *
 * Tensor-core items: one per (format, compressed 16-row block).  Each item
 * owns k-steps [tc_item_kbeg[i], tc_item_kbeg[i+1]) of 16 columns.
 * tc_vals holds, per k-step, the 16x16 block values as the shared-memory
 * image of one tcgen05.mma B operand (K-major, no swizzle):
 *   element (row n, col k) at byte (n/8)*256 + (k/8)*128 + (n%8)*16 + (k%8)*2
 * for 16-bit modes (bf16 / fp16); STILE_TC_SPLIT_BF16 stores the hi image
 * followed by the lo image (1024 B per k-step).  STILE_TC_FP8 stores, per
 * k-step, the e4m3 bytes of value / tc_row_scale[item * 16 + n] as a K = 32
 * operand whose upper 16 k are zero: byte (n/8)*256 + (k/16)*128 +
 * (n%8)*16 + k%16 (512 B per k-step).
 *
 * ELL items: one per row-bucket tile; rows [ell_item_row0[i],
 * ell_item_row0[i+1]), every row with ell_item_K[i] slots starting at
 * ell_item_slot0[i] + r*K (the reference's indices_k layout).
 *
 * out rows equal to -1 are never written.  zero_rows lists the output rows
 * that no owned (non-atomic) tile stores; stile_spmm_run zeroes them before
 * the fused kernel so atomic tiles can accumulate.
 */
typedef struct StileSpmmPlanHost {
  int32_t M, K;
  int32_t tc_mode;
  int32_t tc_n_items, tc_n_ksteps;
  const int32_t* tc_item_kbeg;   /* [tc_n_items + 1] */
  const int32_t* tc_item_flags;  /* [tc_n_items] bit0: atomic */
  const int32_t* tc_out_rows;    /* [tc_n_items * 16] */
  const int32_t* tc_cols;        /* [tc_n_ksteps * 16] */
  const void* tc_vals;           /* [tc_n_ksteps * tc_kstep_bytes] */
  int32_t tc_kstep_bytes;        /* 512 (bf16/fp16), 1024 (split) */
  const int32_t* tc_nnz_id;      /* [tc_n_ksteps * 256] row-major (n,k); -1: empty */
  int32_t ell_n_items, ell_n_rows, ell_n_slots;
  const int32_t* ell_item_row0;  /* [ell_n_items + 1] */
  const int32_t* ell_item_K;     /* [ell_n_items] */
  const int32_t* ell_item_slot0; /* [ell_n_items] */
  const int32_t* ell_item_flags; /* [ell_n_items] bit0: atomic */
  const int32_t* ell_out_row;    /* [ell_n_rows] */
  const int32_t* ell_row_len;    /* [ell_n_rows] live slots */
  const float* ell_vals;         /* [ell_n_slots] */
  const int32_t* ell_kidx;       /* [ell_n_slots] original column */
  const int32_t* ell_nnz_id;     /* [ell_n_slots] -1: padding */
  int32_t n_zero_rows;
  const int32_t* zero_rows;      /* [n_zero_rows] */
  int64_t nnz;                   /* nonzeros of the pattern (dvals length) */
  const float* tc_row_scale;     /* [tc_n_items * 16] STILE_TC_FP8: scale of every
                                    tensor-tile row (its largest |value| / 448); else NULL */
} StileSpmmPlanHost;

/*
 * SDDMM plan.  1D items: flattened nonzeros (mid_idx, j_idx, remap of the
 * reference, my_fuse_formats.py:3568-3600).  Block items: TC_sddmm tiles
 * (i_indices, j_indices, indptr, indicesDense, indices, :3607-3661);
 * block width = bn (16), block height = bm (16).
 */
typedef struct StileSddmmPlanHost {
  int32_t M, K;
  int64_t nnz;
  int32_t n_1d;
  const int32_t* mid_idx;        /* [n_1d] */
  const int32_t* j_idx;          /* [n_1d] */
  const int32_t* remap;          /* [n_1d] output nonzero id */
  int32_t n_blk, bm, bn, n_blk_nnz;
  const int32_t* blk_i;          /* [n_blk * bm] */
  const int32_t* blk_j;          /* [n_blk * bn] */
  const int32_t* blk_indptr;     /* [n_blk + 1] */
  const int32_t* blk_dense_pos;  /* [n_blk_nnz] m*bn + n */
  const int32_t* blk_out;        /* [n_blk_nnz] output nonzero id */
} StileSddmmPlanHost;

typedef struct StileSpmmPlan StileSpmmPlan;
typedef struct StileSddmmPlan StileSddmmPlan;

/* Copy a host plan to the current device; the handle owns the copies. */
int stile_spmm_plan_upload(const StileSpmmPlanHost* host, StileSpmmPlan** out);
int stile_sddmm_plan_upload(const StileSddmmPlanHost* host, StileSddmmPlan** out);
int stile_spmm_plan_free(StileSpmmPlan* plan);
int stile_sddmm_plan_free(StileSddmmPlan* plan);

/*
 * C[M, N] = A @ B[K, N] (fp32 in / fp32 out; row strides ldb, ldc in
 * elements, multiples of 4).  C is fully written (rows without nonzeros
 * become 0).  Stream-ordered; returns after enqueueing.
 */
int stile_spmm_run(const StileSpmmPlan* plan, const float* B, int64_t ldb,
                   float* C, int64_t ldc, int32_t N, void* stream);

/*
 * The same product with B in bf16 (raw bfloat16 bits; fp32 accumulation and
 * fp32 C): row tiles convert the gathered rows to fp32, tensor tiles feed
 * them to the MMA unconverted.  ldb is in elements and must be a multiple
 * of 8 (16-byte rows chunks), B 16-byte aligned; the plan's tensor tiles
 * must be bf16 (STILE_TC_BF16), else STILE_E_UNSUPPORTED.  Counterpart: the
 * reference's fused SpMM built for dtype "float16" / bf16 activations
 * (SPMM/SPMMbench_our_method.py:187-222, the MydtypeIn knob).
 */
int stile_spmm_run_bf16(const StileSpmmPlan* plan, const uint16_t* B,
                        int64_t ldb, float* C, int64_t ldc, int32_t N,
                        void* stream);

/*
 * Batched (multi-head) SpMM: H value sets on the plan's pattern, one launch
 * of each kernel for all of them.  stile_spmm_values_pack packs
 * vals[H][nnz] (CSR order, fp32) into `packed`, caller-owned device memory
 * of stile_spmm_values_bytes(plan, H) bytes, 256-byte aligned; then
 *   C + h * c_head_stride  =  A_h @ (B + h * b_head_stride)   for h < H
 * (strides in elements, multiples of 4; heads may not overlap).  fp32 B.
 * Counterpart: batched_spmm, the reference's multi-head SpMM whose value
 * buffer carries a batch dimension (MY_sparse/my_fuse_formats.py:1296-1428).
 */
int64_t stile_spmm_values_bytes(const StileSpmmPlan* plan, int32_t heads);
int stile_spmm_values_pack(const StileSpmmPlan* plan, const float* vals,
                           int32_t heads, void* packed, void* stream);
int stile_spmm_run_batched(const StileSpmmPlan* plan, const void* packed,
                           int32_t heads, const float* B, int64_t ldb,
                           int64_t b_head_stride, float* C, int64_t ldc,
                           int64_t c_head_stride, int32_t N, void* stream);

/* dvals[nnz] = <dY[row(t)], B[col(t)]> for every nonzero t of A (CSR order),
 * walking the forward plan's tiles. */
int stile_spmm_dvals(const StileSpmmPlan* plan, const float* dY, int64_t lddy,
                     const float* B, int64_t ldb, float* dvals, int32_t N,
                     void* stream);

/* dvals with B in bf16 (the operand of stile_spmm_run_bf16; dY fp32).  No
 * counterpart in the reference, like stile_spmm_dvals. */
int stile_spmm_dvals_bf16(const StileSpmmPlan* plan, const float* dY,
                          int64_t lddy, const uint16_t* B, int64_t ldb,
                          float* dvals, int32_t N, void* stream);

/* out[nnz] = <X[row(t)], Y[col(t)]> (fp32), CSR order of the mask.  A plan
 * of an empty mask returns 0 without reading any pointer. */
int stile_sddmm_run(const StileSddmmPlan* plan, const float* X, int64_t ldx,
                    const float* Y, int64_t ldy, float* out, int32_t F,
                    void* stream);

/* The same with X and Y in bf16 (raw bfloat16 bits, row strides multiples
 * of 8, 16-byte aligned; products and sums in fp32).  Counterpart: the
 * fused SDDMM built for 16-bit inputs (measure_latency_BSDDMM with
 * dtype "float16", MY_sparse/my_fuse_formats.py:4292-4330). */
int stile_sddmm_run_bf16(const StileSddmmPlan* plan, const uint16_t* X,
                         int64_t ldx, const uint16_t* Y, int64_t ldy,
                         float* out, int32_t F, void* stream);

/* Plain CSR SpMM (fp32) with nonzero-balanced ranges per warp group
 * (stile_csr_group_nnz() nonzeros each), vectorised B loads; nnz = indptr[M]
 * (passed so no device read is needed).  group_rows[g] (optional, may be
 * NULL) is the row holding nonzero g * stile_csr_group_nnz(); without it
 * every group binary-searches indptr. */
int stile_csr_spmm_run(int32_t M, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                       const float* vals, const int32_t* group_rows, const float* B, int64_t ldb,
                       float* C, int64_t ldc, int32_t N, void* stream);

/* Nonzeros per warp group of the CSR kernel (for building group_rows). */
int32_t stile_csr_group_nnz(void);

/*
 * Row softmax over a CSR pattern, for `batch` value sets (heads) of nnz
 * entries each, stored one after another:
 *   out[h][t] = exp(scale * x[h][t] - max_r) / sum over row r's entries,
 * the entries outside the pattern taken as -inf (x and out may alias).
 * Counterpart: the sparse-transformer softmax the reference's attention
 * benchmarks use (my_3rdparty/Magicube/Magicube1/end2end_eval/
 * sparse_transformer_magicube/src/cuda/softmax_kernel.cu, checked against
 * torch.softmax(dense * scaler) in verify/bsoftmax.py).
 */
int stile_csr_row_softmax(int32_t M, const int32_t* indptr, int64_t nnz,
                          const float* x, float* out, float scale,
                          int32_t batch, void* stream);

/*
 * Fused sparse attention, every head in one launch (no counterpart kernel in
 * the reference, which runs the three steps as separate operators):
 *   out[h][r] = sum_t p_t V[h][c_t],  p = softmax over row r's stored
 *   entries c_t of scale * <Q[h][r], K[h][c_t]> (the others count as -inf)
 * for the CSR pattern (indptr[n_rows + 1], indices: column ids < the rows of
 * K and V, not checked).  One pass per row with an online softmax: neither
 * the scores nor the probabilities are stored.  fp32; 1 <= F, Fv <= 128;
 * row strides multiples of 4 elements, 16-byte aligned rows; head h's
 * operands start h * stride elements further.  A row without entries gives
 * zeros.  It replaces the chain SDDMM -> stile_csr_row_softmax -> batched
 * SpMM of the LogSparse / Strided attention operators
 * (MY_sparse/gen_formats_v2.py:2926-3003).
 */
int stile_sparse_attention(int32_t n_rows, const int32_t* indptr, const int32_t* indices, const float* Q,
                           const float* K, const float* V, int64_t ldq, int64_t ldk, int64_t ldv,
                           int64_t q_head_stride, int64_t k_head_stride, int64_t v_head_stride, float* out,
                           int64_t ldo, int64_t out_head_stride, int32_t F, int32_t Fv, float scale, int32_t heads,
                           void* stream);

/* Learned tile cost model (replaces get_MLP_pred / PyTorchMLP,
 * my_cost_model.py:1010-1093, and its trainer MLP_train_cost_model.py:81-204):
 * a STILE_MLP_FEATURES -> 64 -> 32 -> 1 ReLU network over standardised tile
 * features, STILE_MLP_PARAMS floats laid out W1[F][64], b1[64], W2[64][32],
 * b2[32], W3[32], b3.  All pointers are device pointers.
 * stile_mlp_forward: y[n] = net(x[n][F]), every candidate in one launch.
 * stile_mlp_gradient: loss = sum (y - t)^2 / n and grad[STILE_MLP_PARAMS];
 *   work holds n * 192 floats, dy n floats (scratch of the caller).
 * stile_mlp_adam: one Adam step (bias-corrected, step >= 1). */
#define STILE_MLP_FEATURES 12
#define STILE_MLP_PARAMS 2945
int stile_mlp_forward(const float* params, const float* x, int64_t n, float* y, void* stream);
int stile_mlp_gradient(const float* params, const float* x, const float* t, int64_t n,
                       float* work, float* dy, float* grad, float* loss, void* stream);
int stile_mlp_adam(float* params, const float* grad, float* m, float* v, int64_t count,
                   float lr, float beta1, float beta2, float eps, int32_t step, void* stream);

/* Plain CSR SpMM that allocates nothing.  No counterpart in the reference.
 * For callers that must not allocate device memory: their memory belongs to
 * another allocator (a host framework's caching pool, an arena handed out up
 * front), and a cudaMalloc / cudaFree of their own may also synchronise the
 * device and stall other streams.  Same result as stile_csr_spmm_run with a
 * group_rows map, but the map is built on the device into a scratch array
 * compiled into the library: STILE_CSR_NOALLOC_MAX_GROUPS entries (1 MiB),
 * held by every GPU that loads the library until the process exits, so
 * nnz <= STILE_CSR_NOALLOC_MAX_GROUPS * stile_csr_group_nnz() (16,777,216);
 * larger inputs are rejected with STILE_E_INVALID.  Every call looks up
 * the array's address on the current device (cudaGetSymbolAddress, which
 * allocates nothing); the first call on a device loads the library's module
 * there, so make that first call before any stream capture.  All calls on a device
 * share the array: every entry a call reads it writes first, but calls that
 * overlap on the GPU (unordered streams) race on it. */
#define STILE_CSR_NOALLOC_MAX_GROUPS (1 << 18)
int stile_csr_spmm_run_noalloc(int32_t M, int64_t nnz, const int32_t* indptr,
                               const int32_t* indices, const float* vals,
                               const float* B, int64_t ldb, float* C, int64_t ldc,
                               int32_t N, void* stream);

/*
 * Fused backward of C = A @ B (no counterpart in the reference, like
 * stile_spmm_dvals).  planT is the plan of A^T (its own pattern and tiles);
 * stile_spmm_plan_set_transpose_ids tells it, once, the forward's numbering:
 * perm[t] (device, nnz entries) is the nonzero of A that nonzero t of A^T
 * (CSR order of A^T) is.  Then
 *   dB[K, N]  = A^T @ dC[M, N]             (fp32, fully written)
 *   dvals[s]  = <dC[row(s)], B[col(s)]>    for every nonzero s of A
 * in one pass over A^T's row tiles: each dC row gathered for dB also gives
 * the value gradients of its entries (B's row is held per row run); the
 * tensor-tile nonzeros take a second pass (see stile_spmm_plan_set_dvals_mode).
 * N > 128 runs the product and the gradient pass one after the other.  dvals
 * is fully written when A^T's tiles hold every nonzero. */
int stile_spmm_plan_set_transpose_ids(StileSpmmPlan* planT, const int32_t* perm, int64_t nnz, void* stream);
int stile_spmm_backward(const StileSpmmPlan* planT, const float* dC, int64_t lddc,
                        const float* B, int64_t ldb, float* dB, int64_t lddb,
                        float* dvals, int32_t N, void* stream);

/* How stile_spmm_dvals and stile_spmm_backward compute the value gradients
 * of the tensor-tile nonzeros (no counterpart in the reference, whose
 * dvals is a separate SDDMM): mode 1 on the tensor cores (a unit of up to 8
 * k-steps of one tile row block is one M = 128, N = 16 MMA chain over the
 * gathered fp32 rows split into hi + lo bf16, hi.hi + hi.lo + lo.hi, fp32
 * accumulation: the item's 16 rows are gathered once per unit and each
 * k-step's 16 columns once, against one row per nonzero), mode 2 by the
 * row runs of the entry list (fp32 on CUDA cores), mode 0 (the default at
 * upload) the row runs, which measured faster on the 232,965-node GCN
 * graph; the operator API times both once per width.  Row-tile
 * nonzeros always take the row runs or
 * the fused ELL pass.  A bf16 B (stile_spmm_dvals_bf16) always takes the
 * row runs.  The mode is read when a call is enqueued; setting it is not
 * thread-safe against calls on the same plan from other host threads. */
int stile_spmm_plan_set_dvals_mode(StileSpmmPlan* plan, int32_t mode);

/* Refresh the tile values of a plan from vals[nnz] (device, CSR order of the
 * pattern the plan was built for); the pattern and index arrays are kept.
 * Used when A's values change between calls (training the values). */
int stile_spmm_plan_set_values(StileSpmmPlan* plan, const float* vals, void* stream);

/* Device-side error flag of a plan's kernels (bounded waits that gave up):
 * synchronises the stream, returns the flag (0 = none) and clears it. */
int stile_spmm_plan_error_flag(StileSpmmPlan* plan, void* stream, int32_t* flag);
int stile_sddmm_plan_error_flag(StileSddmmPlan* plan, void* stream, int32_t* flag);

/* Wait policy of the plan's tensor-core kernel (failure detection; no
 * counterpart in the reference).  Every pipeline wait of the kernel (on an
 * operand slot or an accumulator) gives up after `polls` polls (polls <= 0:
 * the default, 2^22), sets the plan's error flag and ends its role; the
 * kernel's wait for its own MMAs before freeing tensor memory keeps the
 * default.  stall_test != 0 (needs polls > 0) makes the MMA issuer first
 * wait on a barrier that nothing arrives on, so that wait, and then the
 * other roles' waits, run out: the run returns with the error flag set and
 * its output undefined, and later runs with stall_test = 0 are unaffected.
 * Not thread-safe against runs of the same plan in flight on other host
 * threads. */
int stile_spmm_plan_set_wait_policy(StileSpmmPlan* plan, int32_t polls, int32_t stall_test);

/* Tensor-core layout self-check (no counterpart in the reference): runs one
 * tcgen05.mma (M=128, N=16; kind = 0: kind::f16, K=16; kind = 1:
 * kind::tf32, K=8; kind = 2: kind::f8f6f4, K=32; fp32 accumulate) on two 16 KB shared-memory images copied
 * verbatim from a_img / b_img, with descriptor fields desc6 = {a_lbo, a_sbo,
 * a_layout, b_lbo, b_sbo, b_layout} (bytes, multiples of 16, <= 2048) and
 * instruction descriptor idesc; writes the 128x16 fp32 accumulator row-major
 * to out.  *err is set if the MMA did not complete within the bounded wait. */
int stile_debug_umma_probe(const void* a_img, const void* b_img, const uint32_t* desc6,
                           uint32_t idesc, int32_t kind, float* out, int32_t* err, void* stream);

/* Copy the last error message of the calling thread into buf. */
int stile_last_error(char* buf, size_t n);

/* Number of kernels launched by this library since load (for accounting). */
int64_t stile_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* STILE_GB300_H_ */
