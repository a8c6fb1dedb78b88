// SpMM kernels for sm_103a.
//
//  * csr_spmm_kernel     plain CSR-row SpMM (the comparator)
//  * zero_rows_kernel    zeroes output rows that no owned tile stores
//  * spmm_tc_kernel      dense 16-row block tiles on the tensor cores
//                        (tcgen05.mma, accumulator in TMEM), cp.async ring
//  * spmm_ell_kernel     ELL row-bucket tiles on CUDA cores
//                        The two launches together are the reference's
//                        horizontally fused kernel (my_fuse_formats.py:2437):
//                        the same tiles, split by template into two grids so
//                        that each gets its own block shape and shared memory.
//  * spmm_dvals_kernel   value gradient <dY[row], B[col]> for every nonzero,
//                        walking the same tiles.
#include "common.cuh"
#include "spmm.cuh"

namespace stile {

// ===========================================================================
// plain CSR SpMM (the comparator)
// ===========================================================================
// Nonzero-balanced CSR: every LPR-lane group owns kCsrNnz consecutive
// nonzeros, finds its first row by binary search in indptr and walks the
// rows it touches (4 B rows in flight per lane).  A row lying wholly inside
// the range is stored; a row that straddles a range boundary is accumulated
// with atomics into a row that csr_prezero_kernel zeroed first.
constexpr int kCsrNnz = 64;

__device__ __forceinline__ int row_of_nnz(const int* __restrict__ indptr, int M, long t) {
  // largest r with indptr[r] <= t
  int lo = 0, hi = M;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (indptr[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

__global__ void csr_prezero_kernel(int M, const int* __restrict__ indptr, float* __restrict__ C, long ldc,
                                   int N) {
  // one thread per row: rows without nonzeros and rows that straddle a
  // range boundary (accumulated with atomics) start at zero
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= M) return;
  const long rb = indptr[r], re = indptr[r + 1];
  const bool empty = rb == re;
  const bool split = !empty && (rb / kCsrNnz) != ((re - 1) / kCsrNnz);
  if (!empty && !split) return;
  float* row = C + (long)r * ldc;
  for (int f = 0; f < N; f += 4) st_row4(row, f, N, make_float4(0.f, 0.f, 0.f, 0.f));
}

template <int LPR>
__global__ void __launch_bounds__(256) csr_spmm_kernel(int M, const int* __restrict__ indptr,
                                                       const int* __restrict__ indices,
                                                       const float* __restrict__ vals,
                                                       const float* __restrict__ B, long ldb,
                                                       float* __restrict__ C, long ldc, int N,
                                                       int n_groups) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / LPR, sl = lane % LPR;
  const int g = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (kWarp / LPR) + sub;
  if (g >= n_groups) return;
  const long nnz = indptr[M];
  const long t0 = (long)g * kCsrNnz;
  const long t1 = min(t0 + kCsrNnz, nnz);
  int r = row_of_nnz(indptr, M, t0);
  long t = t0;
  while (r < M && t < t1) {
    const long rb = indptr[r], re = indptr[r + 1];
    const long a = max(rb, t0), b = min(re, t1);
    if (a >= b) {  // empty row (already zero)
      t = re;
      ++r;
      continue;
    }
    const bool whole = (rb >= t0) && (re <= t1);
    for (int fc = 0; fc < N; fc += 4 * LPR) {
      const int f = fc + 4 * sl;
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      long k = a;
      for (; k + 4 <= b; k += 4) {
        const int c0 = __ldg(indices + k), c1 = __ldg(indices + k + 1), c2 = __ldg(indices + k + 2),
                  c3 = __ldg(indices + k + 3);
        const float v0 = __ldg(vals + k), v1 = __ldg(vals + k + 1), v2 = __ldg(vals + k + 2),
                    v3 = __ldg(vals + k + 3);
        const float4 b0 = ld_row4(B + (long)c0 * ldb, f, N);
        const float4 b1 = ld_row4(B + (long)c1 * ldb, f, N);
        const float4 b2 = ld_row4(B + (long)c2 * ldb, f, N);
        const float4 b3 = ld_row4(B + (long)c3 * ldb, f, N);
        fma4(acc, v0, b0);
        fma4(acc, v1, b1);
        fma4(acc, v2, b2);
        fma4(acc, v3, b3);
      }
      for (; k < b; ++k) fma4(acc, __ldg(vals + k), ld_row4(B + (long)__ldg(indices + k) * ldb, f, N));
      if (whole) st_row4(C + (long)r * ldc, f, N, acc); else red_row4(C + (long)r * ldc, f, N, acc);
    }
    t = re;
    ++r;
  }
}

// ===========================================================================
// zero rows
// ===========================================================================
__global__ void zero_rows_kernel(const int* __restrict__ rows, int n_rows, float* __restrict__ C,
                                 long ldc, int N) {
  // one warp per row, float4 stores
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp_global >= n_rows) return;
  float* row = C + (long)rows[warp_global] * ldc;
  for (int f = 4 * lane; f < N; f += 128) st_row4(row, f, N, make_float4(0.f, 0.f, 0.f, 0.f));
}

// ===========================================================================
// hybrid SpMM: tensor-core kernel + ELL kernel (launched back to back)
// ===========================================================================
// Tensor-core chunks.  A chunk is a run of at most kChunkSteps k-steps of
// one item (items longer than that are split; the split parts accumulate
// with atomics into pre-zeroed rows).  Per k-step the CTA gathers the 16
// referenced B rows (fp32, 128 features) with cp.async into a 4-stage ring
// together with the step's 16x16 value image, converts its own copies to the
// bf16 / fp16 A-operand image and one thread issues the tcgen05.mma.
//
// Shared-memory operand layouts (checked by the layout probe):
//   A: [128 features (M) x 16 k (K)], MN-major, 128-byte swizzle: two
//      64-feature atoms (LBO 2048 B), two 8-row k groups (SBO 1024 B)
//   B: the 16x16 block values (N = 16 rows x K = 16), K-major, no swizzle:
//      core matrices 8 rows x 16 B, LBO 128 B (k), SBO 256 B (rows); the
//      plan stores this image and it is used in place.
constexpr uint32_t kAStage = 4096;   // bytes of one A image (16-bit)
constexpr uint32_t kBStage = 512;    // bytes of one B image (16-bit)
constexpr uint32_t kALbo = 2048, kASbo = 1024;
constexpr uint32_t kBLbo = 128, kBSbo = 256;
constexpr int kTcThreads = 128;
constexpr int kStages = 4;           // cp.async ring depth
constexpr uint32_t kRawRows = 8192;  // 16 rows x 128 fp32 per stage

__device__ __forceinline__ uint32_t a_img_off(int m, int k) {
  // m: feature (0..127), k: column within the k-step (0..15)
  const int atom = m >> 6, grp = k >> 3, r = k & 7, chunk = (m & 63) >> 3;
  return (uint32_t)(atom * kALbo + grp * kASbo + r * 128 + ((chunk ^ r) << 4) + (m & 7) * 2);
}

template <bool kSplit>
struct TcLayout {
  static constexpr uint32_t kVals = kSplit ? 2 * kBStage : kBStage;
  static constexpr uint32_t kStage = kRawRows + kVals;
  static constexpr uint32_t kAImg = kSplit ? 2 * kAStage : kAStage;
  static constexpr uint32_t kRing = kStages * kStage;                 // multiple of 1024
  static constexpr uint32_t kBytes = 1024 + kRing + 2 * kAImg + 64;  // + alignment slack
};

template <int MODE>
__global__ void __launch_bounds__(kTcThreads) spmm_tc_kernel(SpmmArgs p) {
  constexpr bool kSplit = (MODE == STILE_TC_SPLIT_BF16);
  using L = TcLayout<kSplit>;
  extern __shared__ uint8_t smem_raw[];
  const int chunk = blockIdx.x / p.n_fchunks;
  const int f0 = (blockIdx.x % p.n_fchunks) * 128;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const uint32_t ring = base;
  const uint32_t aimg = base + L::kRing;
  const uint32_t bar = aimg + 2 * L::kAImg;
  const uint32_t tmem_slot = bar + 8;

  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(tmem_slot, 32);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  uint32_t tmem;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(tmem) : "r"(tmem_slot) : "memory");

  const int kb = p.tc_chunk_kbeg[chunk];
  const int n = p.tc_chunk_kbeg[chunk + 1] - kb;
  const int item = p.tc_chunk_item[chunk];
  const int N = p.N;
  const uint8_t* vals = reinterpret_cast<const uint8_t*>(p.tc_vals);
  const uint32_t idesc = (MODE == STILE_TC_F16) ? make_idesc(0, 0, 1, 0, 128, 16)
                                                : make_idesc(1, 1, 1, 0, 128, 16);

  // this thread's 4 copies per stage: rows warp + 4j, features 4*lane..+3
  auto issue = [&](int ks, int stg) {
    const uint32_t sb = ring + stg * L::kStage;
    const int f = f0 + 4 * lane;
    const uint32_t bytes = (f + 4 <= N) ? 16u : (f < N ? (uint32_t)(N - f) * 4u : 0u);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int kk = warp + 4 * j;
      const float* row = p.B + (long)p.tc_cols[(long)ks * 16 + kk] * p.ldb;
      cp_async16(sb + kk * 512 + lane * 16, bytes ? (const void*)(row + f) : (const void*)row, bytes);
    }
    if (tid < (int)(L::kVals / 16))
      cp_async16(sb + kRawRows + tid * 16, vals + (long)ks * L::kVals + tid * 16, 16u);
  };

  // k-steps per accumulation chain before the accumulator is drained into
  // fp32 registers (bounds the tensor core's accumulation chain)
  constexpr int kGroup = kSplit ? 4 : 16;
  float acc[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) acc[i] = 0.f;
  const uint32_t my_lanes = tmem + ((uint32_t)(32 * warp) << 16);
  bool ok = true;

#pragma unroll 1
  for (int j = 0; j < kStages - 1; ++j) {
    if (j < n) issue(kb + j, j);
    cp_async_commit();
  }
#pragma unroll 1
  for (int step = 0; step < n; ++step) {
    // the MMA of the previous step has read the stage the next copy overwrites
    bool w_ok = true;
    if (step >= 1) w_ok = mbar_wait_bounded(bar, (uint32_t)(step - 1) & 1u);
    if (w_ok && step + kStages - 1 < n) issue(kb + step + kStages - 1, (step + kStages - 1) % kStages);
    cp_async_commit();
    cp_async_wait<kStages - 1>();
    const uint32_t sb = ring + (step % kStages) * L::kStage;
    const uint32_t ai = aimg + (step & 1) * L::kAImg;
    if (w_ok) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int kk = warp + 4 * j;
        const uint4 raw = ld_shared_v4(sb + kk * 512 + lane * 16);
        const float4 v = make_float4(__uint_as_float(raw.x), __uint_as_float(raw.y),
                                     __uint_as_float(raw.z), __uint_as_float(raw.w));
        const uint32_t o = a_img_off(4 * lane, kk);
        if (MODE == STILE_TC_F16) {
          st_shared_v2(ai + o, pack_f16x2(v.x, v.y), pack_f16x2(v.z, v.w));
        } else {
          const uint32_t h0 = pack_bf16x2(v.x, v.y), h1 = pack_bf16x2(v.z, v.w);
          st_shared_v2(ai + o, h0, h1);
          if (kSplit) {
            const __nv_bfloat162 b0 = *reinterpret_cast<const __nv_bfloat162*>(&h0);
            const __nv_bfloat162 b1 = *reinterpret_cast<const __nv_bfloat162*>(&h1);
            const float2 r0 = __bfloat1622float2(b0), r1 = __bfloat1622float2(b1);
            st_shared_v2(ai + kAStage + o, pack_bf16x2(v.x - r0.x, v.y - r0.y),
                         pack_bf16x2(v.z - r1.x, v.w - r1.y));
          }
        }
      }
    }
    fence_proxy_async_smem();
    ok = __syncthreads_and(w_ok && ok) != 0;
    if (!ok) break;
    const bool group_start = (step % kGroup) == 0;
    const bool group_end = ((step % kGroup) == kGroup - 1) || (step == n - 1);
    if (tid == 0) {
      tc_fence_after();
      const uint64_t ad = smem_desc(ai, kALbo, kASbo, kSwizzle128B);
      const uint64_t bd = smem_desc(sb + kRawRows, kBLbo, kBSbo, kSwizzleNone);
      umma_f16(tmem, ad, bd, idesc, group_start ? 0u : 1u);
      if (kSplit) {
        const uint64_t ad_lo = smem_desc(ai + kAStage, kALbo, kASbo, kSwizzle128B);
        const uint64_t bd_lo = smem_desc(sb + kRawRows + kBStage, kBLbo, kBSbo, kSwizzleNone);
        umma_f16(tmem, ad, bd_lo, idesc, 1u);
        umma_f16(tmem, ad_lo, bd, idesc, 1u);
        umma_f16(tmem, ad_lo, bd_lo, idesc, 1u);
      }
      umma_commit(bar);
    }
    if (group_end) {
      const bool done = __syncthreads_and(mbar_wait_bounded(bar, (uint32_t)step & 1u)) != 0;
      if (!done) {
        ok = false;
        break;
      }
      tc_fence_after();
      uint32_t r[16];
      tmem_ld16(my_lanes, r);
      tmem_wait_ld();
#pragma unroll
      for (int i = 0; i < 16; ++i) acc[i] += __uint_as_float(r[i]);
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
    }
  }
  cp_async_wait<0>();
  if (!ok && tid == 0) atomicOr(p.err_flag, 1);

  // epilogue: warp w owns features f0+32w+lane, 16 tile rows in registers
  const int f = f0 + 32 * warp + lane;
  const bool atomic = (p.tc_chunk_flags[chunk] & 1) != 0;
  if (f < N && n > 0 && ok) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int row = p.tc_out_rows[(long)item * 16 + i];
      if (row < 0) continue;
      float* dst = p.C + (long)row * p.ldc + f;
      if (atomic) atomicAdd(dst, acc[i]); else *dst = acc[i];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 32);
}

// tf32 tensor-core kernel (B in fp32).  No conversion pass: each gathered B
// row is copied by cp.async straight into the A operand of kind::tf32
// (features = M = 128, MN-major, 128-byte swizzle, 32-feature atoms,
// LBO 1024 B; the two 8-row k groups of a k-step are 4096 B apart and feed
// one MMA each, so the descriptor's k-group stride is never used).  The block values sit in the plan as the fp32 B-operand
// image (K-major, no swizzle, LBO 128 B, SBO 256 B; k halves 512 B apart).
// Warps 0-3 produce (4 x 16 B copies per thread per k-step, completion
// signalled on a full barrier by cp.async.mbarrier.arrive) and run the
// epilogue; warp 4 waits on the full barrier, issues the two MMAs and
// commits to the stage's empty barrier.
constexpr int kTfStages = 4;
constexpr uint32_t kTfA = 8192;                 // 16 k x 128 features x 4 B
constexpr uint32_t kTfB = 1024;                 // 16 rows x 16 k x 4 B
constexpr uint32_t kTfStage = kTfA + kTfB;      // 9216 = 9 x 1024
constexpr uint32_t kTfBytes = 1024 + kTfStages * kTfStage + 128;
constexpr int kTfThreads = 160;

__global__ void __launch_bounds__(kTfThreads) spmm_tc_tf32_kernel(SpmmArgs p) {
  extern __shared__ uint8_t smem_raw[];
  const int chunk = blockIdx.x / p.n_fchunks;
  const int f0 = (blockIdx.x % p.n_fchunks) * 128;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const uint32_t bars = base + kTfStages * kTfStage;  // full[S], empty[S], done
  const uint32_t tmem_slot = bars + 8 * (2 * kTfStages + 1);
  auto full = [&](int s) { return bars + 8 * s; };
  auto empty = [&](int s) { return bars + 8 * (kTfStages + s); };
  const uint32_t done = bars + 8 * (2 * kTfStages);

  if (tid == 0) {
    for (int s = 0; s < kTfStages; ++s) {
      mbar_init(full(s), 128);
      mbar_init(empty(s), 1);
    }
    mbar_init(done, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(tmem_slot, 32);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  uint32_t tmem;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(tmem) : "r"(tmem_slot) : "memory");

  const int kb = p.tc_chunk_kbeg[chunk];
  const int n = p.tc_chunk_kbeg[chunk + 1] - kb;
  const int item = p.tc_chunk_item[chunk];
  const int N = p.N;
  bool ok = true;

  if (warp < 4) {
    // ---------------- producers ----------------
    const int f = f0 + 4 * lane;
    const uint32_t bytes = (f + 4 <= N) ? 16u : (f < N ? (uint32_t)(N - f) * 4u : 0u);
    const int atom = lane >> 3, cic = lane & 7;
    const uint8_t* vals = reinterpret_cast<const uint8_t*>(p.tc_vals);
#pragma unroll 1
    for (int step = 0; step < n; ++step) {
      const int s = step % kTfStages;
      if (step >= kTfStages) {
        if (!mbar_wait_bounded(empty(s), (uint32_t)((step / kTfStages) - 1) & 1u)) {
          ok = false;
          break;
        }
      }
      const uint32_t sa = base + s * kTfStage;
      const long ks = kb + step;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int kk = warp + 4 * j;
        const int g = kk >> 3, r = kk & 7;
        const float* row = p.B + (long)p.tc_cols[ks * 16 + kk] * p.ldb;
        const uint32_t dst = sa + g * 4096 + atom * 1024 + r * 128 + ((cic ^ r) << 4);
        cp_async16(dst, bytes ? (const void*)(row + f) : (const void*)row, bytes);
      }
      if (tid < 64) cp_async16(sa + kTfA + tid * 16, vals + ks * kTfB + tid * 16, 16u);
      cp_async_mbar_arrive_noinc(full(s));
    }
  } else if (lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t idesc = make_idesc(2, 2, 1, 0, 128, 16);
#pragma unroll 1
    for (int step = 0; step < n; ++step) {
      const int s = step % kTfStages;
      if (!mbar_wait_bounded(full(s), (uint32_t)(step / kTfStages) & 1u)) {
        ok = false;
        break;
      }
      fence_proxy_async_smem();
      tc_fence_after();
      const uint32_t sa = base + s * kTfStage;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const uint64_t ad = smem_desc(sa + h * 4096, 1024, 2048, kSwizzle128B);
        const uint64_t bd = smem_desc(sa + kTfA + h * 512, 128, 256, kSwizzleNone);
        umma_tf32(tmem, ad, bd, idesc, (step > 0 || h > 0) ? 1u : 0u);
      }
      umma_commit(empty(s));
    }
    umma_commit(done);
  }
  cp_async_wait<0>();

  // ---------------- epilogue (warps 0-3) ----------------
  if (warp < 4) {
    const bool fin = mbar_wait_bounded(done, 0u);
    tc_fence_after();
    uint32_t r[16];
    tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16), r);
    tmem_wait_ld();
    const int f = f0 + 32 * warp + lane;
    const bool atomic = (p.tc_chunk_flags[chunk] & 1) != 0;
    if (fin && ok && n > 0 && f < N) {
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int row = p.tc_out_rows[(long)item * 16 + i];
        if (row < 0) continue;
        float* dst = p.C + (long)row * p.ldc + f;
        const float v = __uint_as_float(r[i]);
        if (atomic) atomicAdd(dst, v); else *dst = v;
      }
    }
    if (!fin || !ok) atomicOr(p.err_flag, 1);
  } else if (!ok) {
    atomicOr(p.err_flag, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 32);
}

// ELL tiles: one CTA (8 warps) per tile.  An LPR-lane group owns 4 rows at a
// time and loads two slots of each per iteration (8 B-row loads of 16 B in
// flight per lane), so short rows still keep the memory system busy.
constexpr int kEllThreads = 256;
constexpr int kEllRows = 4;

template <int LPR>
__global__ void __launch_bounds__(kEllThreads, 2) spmm_ell_kernel(SpmmArgs p) {
  constexpr int RPW = kWarp / LPR;
  constexpr int kGroups = (kEllThreads / kWarp) * RPW;
  const int item = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int sub = lane / LPR, sl = lane % LPR;
  const int row0 = p.ell_item_row0[item];
  const int nrows = p.ell_item_row0[item + 1] - row0;
  const int K = p.ell_item_K[item];
  const long slot0 = p.ell_item_slot0[item];
  const bool atomic = (p.ell_item_flags[item] & 1) != 0;
  const int N = p.N;
  const int g = warp * RPW + sub;
  for (int rb = g * kEllRows; rb < nrows; rb += kGroups * kEllRows) {
    int orow[kEllRows], len[kEllRows];
    int maxlen = 0;
#pragma unroll
    for (int q = 0; q < kEllRows; ++q) {
      const int r = rb + q;
      orow[q] = -1;
      len[q] = 0;
      if (r < nrows) {
        orow[q] = p.ell_out_row[row0 + r];
        len[q] = orow[q] >= 0 ? p.ell_row_len[row0 + r] : 0;
      }
      maxlen = max(maxlen, len[q]);
    }
    if (maxlen == 0) continue;
    for (int fc = 0; fc < N; fc += 4 * LPR) {
      const int f = fc + 4 * sl;
      float4 acc[kEllRows];
#pragma unroll
      for (int q = 0; q < kEllRows; ++q) acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int k = 0; k < maxlen; k += 2) {
        // two slots of each of the 4 rows: 8 B-row loads in flight per lane
        float4 b[2 * kEllRows];
        float v[2 * kEllRows];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
#pragma unroll
          for (int q = 0; q < kEllRows; ++q) {
            const int i = u * kEllRows + q;
            v[i] = 0.f;
            b[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k + u < len[q]) {
              const long s = slot0 + (long)(rb + q) * K + k + u;
              v[i] = __ldg(p.ell_vals + s);
              b[i] = ld_row4(p.B + (long)__ldg(p.ell_kidx + s) * p.ldb, f, N);
            }
          }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
#pragma unroll
          for (int q = 0; q < kEllRows; ++q) fma4(acc[q], v[u * kEllRows + q], b[u * kEllRows + q]);
        }
      }
#pragma unroll
      for (int q = 0; q < kEllRows; ++q) {
        if (orow[q] < 0) continue;
        float* crow = p.C + (long)orow[q] * p.ldc;
        if (atomic) red_row4(crow, f, N, acc[q]); else st_row4(crow, f, N, acc[q]);
      }
    }
  }
}

// ===========================================================================
// value gradient: dvals[t] = <dY[row(t)], B[col(t)]> over the plan's entry
// list (launch_dvals -> launch_sddmm_list)
// ===========================================================================

// ===========================================================================
// value re-pack: refresh the plan's tile values from a CSR-ordered value
// array (used when the matrix values change but the pattern does not)
// ===========================================================================
__global__ void repack_values_kernel(SpmmArgs p, const float* __restrict__ vals, float* ell_vals,
                                     uint16_t* tc_img, long n_ell_slots) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long n_tc = (long)p.tc_n_ksteps * 256;
  if (i < n_tc) {
    const long ks = i >> 8;
    const int e = (int)(i & 255), n = e >> 4, k = e & 15;
    const int id = p.tc_nnz_id[i];
    const float v = id >= 0 ? vals[id] : 0.f;
    const int img = (n >> 3) * 128 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7);
    if (p.tc_mode == STILE_TC_TF32) {
      const int fi = (k >> 3) * 128 + (n >> 3) * 64 + ((k & 7) >> 2) * 32 + (n & 7) * 4 + (k & 3);
      uint32_t t;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v));
      reinterpret_cast<uint32_t*>(tc_img)[ks * 256 + fi] = t;
    } else if (p.tc_mode == STILE_TC_F16) {
      __half h = __float2half_rn(v);
      tc_img[ks * 256 + img] = *reinterpret_cast<uint16_t*>(&h);
    } else {
      __nv_bfloat16 h = __float2bfloat16_rn(v);
      if (p.tc_mode == STILE_TC_SPLIT_BF16) {
        __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
        tc_img[ks * 512 + img] = *reinterpret_cast<uint16_t*>(&h);
        tc_img[ks * 512 + 256 + img] = *reinterpret_cast<uint16_t*>(&l);
      } else {
        tc_img[ks * 256 + img] = *reinterpret_cast<uint16_t*>(&h);
      }
    }
  } else if (i - n_tc < n_ell_slots) {
    const long s = i - n_tc;
    const int id = p.ell_nnz_id[s];
    ell_vals[s] = id >= 0 ? vals[id] : 0.f;
  }
}

cudaError_t launch_repack(const SpmmArgs& p, const float* vals, long n_ell_slots, cudaStream_t st) {
  const long total = (long)p.tc_n_ksteps * 256 + n_ell_slots;
  if (total == 0) return cudaSuccess;
  const long grid = (total + 255) / 256;
  repack_values_kernel<<<(unsigned)grid, 256, 0, st>>>(
      p, vals, const_cast<float*>(p.ell_vals),
      reinterpret_cast<uint16_t*>(const_cast<void*>(p.tc_vals)), n_ell_slots);
  return cudaGetLastError();
}

// ===========================================================================
// host-side launchers
// ===========================================================================
static int lpr_for(int N) {
  const int lanes = (N + 3) / 4;
  if (lanes >= 32) return 32;
  int l = 1;
  while (l < lanes) l <<= 1;
  return l < 4 ? 4 : l;
}

template <template <int> class F, typename... Args>
static cudaError_t dispatch_lpr(int lpr, Args... args) {
  switch (lpr) {
    case 4: return F<4>::run(args...);
    case 8: return F<8>::run(args...);
    case 16: return F<16>::run(args...);
    default: return F<32>::run(args...);
  }
}

template <int LPR>
struct CsrLaunch {
  static cudaError_t run(int M, const int* indptr, const int* indices, const float* vals, const float* B,
                         long ldb, float* C, long ldc, int N, long nnz, cudaStream_t st) {
    const int n_groups = (int)((nnz + kCsrNnz - 1) / kCsrNnz);
    csr_prezero_kernel<<<(M + 255) / 256, 256, 0, st>>>(M, indptr, C, ldc, N);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    constexpr int GPB = 256 / LPR;
    const int grid = (n_groups + GPB - 1) / GPB;
    if (grid == 0) return cudaSuccess;
    csr_spmm_kernel<LPR><<<grid, 256, 0, st>>>(M, indptr, indices, vals, B, ldb, C, ldc, N, n_groups);
    return cudaGetLastError();
  }
};

cudaError_t launch_csr_spmm(int M, const int* indptr, const int* indices, const float* vals,
                            const float* B, long ldb, float* C, long ldc, int N, long nnz, cudaStream_t st) {
  return dispatch_lpr<CsrLaunch>(lpr_for(N), M, indptr, indices, vals, B, ldb, C, ldc, N, nnz, st);
}

cudaError_t launch_zero_rows(const int* rows, int n, float* C, long ldc, int N, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int grid = (n + 7) / 8;
  zero_rows_kernel<<<grid, 256, 0, st>>>(rows, n, C, ldc, N);
  return cudaGetLastError();
}

size_t tc_smem_bytes(int mode) {
  return mode == STILE_TC_SPLIT_BF16 ? TcLayout<true>::kBytes : TcLayout<false>::kBytes;
}

template <int MODE>
static cudaError_t launch_tc_t(const SpmmArgs& p, cudaStream_t st) {
  const size_t smem = tc_smem_bytes(MODE);
  auto k = spmm_tc_kernel<MODE>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int grid = p.tc_n_chunks * p.n_fchunks;
  if (grid == 0) return cudaSuccess;
  k<<<grid, kTcThreads, smem, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_tc(const SpmmArgs& p, cudaStream_t st) {
  if (p.tc_mode == STILE_TC_TF32) {
    cudaError_t e = cudaFuncSetAttribute(spmm_tc_tf32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kTfBytes);
    if (e != cudaSuccess) return e;
    const int grid = p.tc_n_chunks * p.n_fchunks;
    if (grid == 0) return cudaSuccess;
    spmm_tc_tf32_kernel<<<grid, kTfThreads, kTfBytes, st>>>(p);
    return cudaGetLastError();
  }
  switch (p.tc_mode) {
    case STILE_TC_F16: return launch_tc_t<STILE_TC_F16>(p, st);
    case STILE_TC_SPLIT_BF16: return launch_tc_t<STILE_TC_SPLIT_BF16>(p, st);
    default: return launch_tc_t<STILE_TC_BF16>(p, st);
  }
}

template <int LPR>
struct EllLaunch {
  static cudaError_t run(const SpmmArgs& p, cudaStream_t st) {
    if (p.ell_n_items == 0) return cudaSuccess;
    spmm_ell_kernel<LPR><<<p.ell_n_items, kEllThreads, 0, st>>>(p);
    return cudaGetLastError();
  }
};

cudaError_t launch_ell(const SpmmArgs& p, cudaStream_t st) {
  return dispatch_lpr<EllLaunch>(lpr_for(p.N), p, st);
}

cudaError_t launch_dvals(const SpmmArgs& p, const float* dY, long lddy, float* dvals, cudaStream_t st) {
  return launch_sddmm_list(p.dv_n, p.dv_row, p.dv_col, p.dv_id, dY, lddy, p.B, p.ldb, dvals, p.N, st);
}

}  // namespace stile
