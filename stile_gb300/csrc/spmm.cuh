// Kernel argument block and launchers of the SpMM kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/stile_gb300.h"

namespace stile {

struct SpmmArgs {
  // dense operands
  const float* B;  // fp32, or bf16 bits when b_bf16 (ldb in elements either way)
  long ldb;
  int b_bf16;
  int ell_fc_span;  // features per ELL block row (blockIdx.y); set by the launcher
  int ell_lazy_wait;  // the ELL kernel's predecessor is the zero-rows kernel: only its adds wait
  // heads of a batched run (blockIdx.z; 0 and unused otherwise): per head, B
  // and C start head * stride elements further, the value images head *
  // tc_vals_head_stride bytes further and the ELL records head * ell_n_pos
  // records further
  long b_head_stride, c_head_stride, tc_vals_head_stride;
  int heads;  // grid.z of the ELL and tensor-core launches (0 or 1: one head)
  int tc_slice_per;      // 128-feature slices per tensor-core CTA (blockIdx.y); set by the launcher
  int tc_max_cta_steps;  // most k-steps the chunk schedule gives one CTA
  float* C;
  long ldc;
  int N;
  int K;          // rows of B
  int n_fchunks;  // ceil(N / 128): tensor-core feature chunks
  int tc_mode;
  // tensor-core work chunks (items split into runs of <= kChunkSteps k-steps)
  int tc_n_chunks;
  const int* tc_chunk_kbeg;   // [tc_n_chunks] first k-step
  const int* tc_chunk_nk;     // [tc_n_chunks] k-steps
  // persistent schedule: CTA b owns chunks [tc_cta_chunk[b], tc_cta_chunk[b + 1]),
  // whose k-steps are contiguous
  int tc_grid;
  const int* tc_cta_chunk;    // [tc_grid + 1]
  const int* tc_chunk_item;   // [tc_n_chunks]
  const int* tc_chunk_flags;  // [tc_n_chunks] bit0: atomic
  // tensor-core items
  int tc_n_items, tc_n_ksteps;
  const int* tc_item_kbeg;
  const int* tc_item_flags;
  const int* tc_out_rows;
  const int* tc_cols;
  const void* tc_vals;
  const int* tc_nnz_id;
  // STILE_TC_FP8: scale of every (item, row) and the device word that holds
  // the bits of max |B| of the run (written by an amax pass before the
  // kernels; B's e4m3 scale is that / 448)
  const float* tc_row_scale;
  unsigned* tc_xamax;
  // ELL tiles, compacted at upload into a stream of live entries in row
  // order, cut into groups of at most kSegNnz entries at row boundaries
  // (rows longer than that are split into atomic pieces of their own)
  int ell_n_groups;
  long ell_n_pos;
  const int* ell_group_ptr;  // [ell_n_groups + 1]
  // [ell_n_pos] {column of B, value bits, 2 * row code + run end, 0}; row
  // code r stores into C row r, -(r + 1) adds; run end is 1 when the entry
  // ends its row's run in the group
  const int4* ell_entry;
  const int* ell_nnz_id;     // [ell_n_pos] nonzero id (or NULL)
  // value-gradient entry list enumerated from the tiles: tensor-core entries
  // (item, row, k-step, column order) then ELL slots (row, slot order)
  long dv_n;
  const int* dv_row;
  const int* dv_col;
  const int* dv_id;
  // the same list cut into runs of one row (at most kRunGroup entries):
  // run g is entries [dv_gptr[g], dv_gptr[g + 1]) of row dv_grow[g]
  int dv_n_groups;
  const int* dv_gptr;
  const int* dv_grow;
  // device error flag (bounded waits that gave up)
  int* err_flag;
  // polls of every pipeline wait of the tensor-core kernel before it gives
  // up (0: the default); the final wait for the kernel's own MMAs always
  // uses the default, so TMEM is freed only after they completed
  uint32_t poll_limit;
  // failure-detection test: the MMA thread first waits on a barrier that
  // nothing arrives on, so that wait and then every other role's wait runs
  // out and the kernel returns with the error flag set
  int stall_test;
  // fused backward (this plan is the transposed operator's): the ELL pass
  // that computes dB = A^T dC also writes dvals[id] = <dC[col], dvx[row]>
  // for its entries, id in the fourth word of each record (dvx: the
  // forward's dense operand), and the run list's tensor-core prefix
  // (dv_n_groups_tc groups) gives the rest with ids dvp_id; ids in the
  // forward operator's nonzero numbering (set by set_transpose_ids)
  const float* dvx;
  long dvx_ld;
  float* dv_out;
  int ell_ids_set;
  const int* dvp_id;
  int dv_n_groups_tc;
  // value gradients of the tensor-tile nonzeros on the tensor cores: units
  // of up to 8 k-steps of one chunk (tcdv_unit_ks: first k-step in schedule
  // order; tcdv_unit_meta: item * 8 + k-steps - 1); tcdv_id: the k-steps'
  // nonzero ids ([tc_n_ksteps * 256], (row, column) order) in the numbering
  // of the gradient (the plan's own, or the forward operator's after
  // set_transpose_ids); tcdv_use: use them (else the row runs)
  int tcdv_n_units;
  const int* tcdv_unit_ks;
  const int* tcdv_unit_meta;
  const int* tcdv_id;
  int tcdv_use;
};

cudaError_t launch_csr_spmm(int M, const int* indptr, const int* indices, const float* vals,
                            const float* B, long ldb, float* C, long ldc, int N, long nnz,
                            const int* group_rows, cudaStream_t st);
constexpr int kCsrGroupNnz = 64;  // nonzeros per warp group of the CSR kernel
constexpr int kSegNnz = 64;       // entries per group of the ELL stream kernel
cudaError_t launch_zero_rows(const int* rows, int n, float* C, long ldc, int N, cudaStream_t st, int heads = 1,
                             long c_head_stride = 0);
cudaError_t launch_tc(const SpmmArgs& p, cudaStream_t st);
// C-ABI bookkeeping shared by the entry points of every translation unit:
// record `msg` as the calling thread's last error and return `code`; count
// kernel launches
int report_error(int code, const char* msg);
void note_launches(int n);
// CTAs of the persistent tensor-core kernel resident on the current device
// (0 on error)
int tc_persistent_ctas(int mode);
// streaming multiprocessors of the current device (cached; 1 on error)
int device_sm_count();
cudaError_t launch_ell(const SpmmArgs& p, cudaStream_t st);
// the ELL pass of the fused backward (fp32, N <= 128, one head)
cudaError_t launch_ell_bwd(const SpmmArgs& p, cudaStream_t st);
// out[i] = in[i] >= 0 ? perm[in[i]] : -1
cudaError_t launch_permute_ids(const int* in, long n, const int* perm, int* out, cudaStream_t st);
// ent[i].w = ids[i] >= 0 ? perm[ids[i]] : -1
cudaError_t launch_record_ids(int4* ent, const int* ids, long n, const int* perm, cudaStream_t st);
cudaError_t launch_dvals(const SpmmArgs& p, const float* dY, long lddy, float* dvals, cudaStream_t st);
// out[id] = <X[item row], Y[k-step column]> for the tensor-tile nonzeros
// (fp32 X and Y, F features), on the tensor cores with hi + lo bf16
// operands; ids from p.tcdv_id
cudaError_t launch_tc_dvals(const SpmmArgs& p, const float* X, long ldx, const float* Y, long ldy, float* out, int F,
                            cudaStream_t st);
constexpr int kTcDvUnit = 8;  // k-steps per unit of the tensor-tile value-gradient kernel
constexpr int kChunkSteps = 32;
cudaError_t launch_pack_values(const SpmmArgs& p, const float* vals, long nnz, int heads, void* ell_out,
                               void* tc_out, long n_ell, long tc_head_bytes, cudaStream_t st);
cudaError_t launch_repack(const SpmmArgs& p, const float* vals, long n_ell_slots, cudaStream_t st);
// *amax_bits = bits of max |B[r][f]| over K rows x N features (atomicMax on
// the non-negative floats' bits; *amax_bits starts at 0); an ordinary launch
cudaError_t launch_amax(const float* B, long ldb, int K, int N, unsigned* amax_bits, cudaStream_t st);

struct SddmmArgs {
  const float* X;  // fp32, or bf16 bits when xy_bf16 (X and Y alike)
  long ldx;
  const float* Y;
  long ldy;
  int xy_bf16;
  float* out;
  int F;
  int n_1d;
  const int* mid_idx;
  const int* j_idx;
  const int* remap;
  // the 1D entries as runs of one row (at most kRunGroup entries each)
  int n_runs;
  const int* run_ptr;
  const int* run_row;
  int n_blk, bm, bn;
  const int* blk_i;
  const int* blk_j;
  const int* blk_indptr;
  const int* blk_dense_pos;
  const int* blk_out;
  // device error flag (the block kernel's bounded MMA wait gave up)
  int* err_flag;
};

cudaError_t launch_sddmm(const SddmmArgs& p, cudaStream_t st);
cudaError_t launch_csr_row_softmax(int M, const int* indptr, long nnz, const float* x, float* out, float scale,
                                   int batch, cudaStream_t st);
cudaError_t launch_sddmm_list(long n, const int* rows, const int* cols, const int* outs, const void* X, bool x_bf16,
                              long ldx, const void* Y, bool y_bf16, long ldy, float* out, int F, cudaStream_t st);
// row-run SDDMM: group g is entries [gptr[g], gptr[g+1]) of row grow[g]
constexpr int kRunGroup = 64;  // entries per run group at most
cudaError_t launch_sddmm_runs(int n_groups, const int* gptr, const int* grow, const int* cols, const int* outs,
                              const void* X, bool x_bf16, long ldx, const void* Y, bool y_bf16, long ldy, float* out,
                              int F, cudaStream_t st);

cudaError_t launch_sparse_attention(int n_rows, const int* indptr, const int* indices, const float* Q,
                                    const float* K, const float* V, long ldq, long ldk, long ldv, long q_head,
                                    long k_head, long v_head, float* out, long ldo, long o_head, int F, int Fv,
                                    float scale, int heads, cudaStream_t st);

cudaError_t launch_umma_probe(const void* a_img, const void* b_img, const uint32_t* desc6,
                              uint32_t idesc, uint32_t kind, float* out, int* err, cudaStream_t st);

}  // namespace stile
