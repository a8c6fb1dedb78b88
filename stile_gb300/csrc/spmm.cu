// SpMM kernels for sm_103a.
//
//  * csr_spmm_kernel     plain CSR-row SpMM (the comparator)
//  * zero_rows_kernel    zeroes output rows that no owned tile stores
//  * spmm_tc_ws_kernel   dense 16-row block tiles on the tensor cores
//                        (tcgen05.mma, accumulator in TMEM): warp-specialised
//                        cp.async producers + MMA issuer (bf16 / fp16, and
//                        split-bf16 hi+lo products with periodic accumulator
//                        drains for fp32-level accuracy)
//  * spmm_ell_seg_kernel ELL row-bucket tiles on CUDA cores, as a stream of
//                        live entries cut into groups at row boundaries
//                        The two launches together are the reference's
//                        horizontally fused kernel (my_fuse_formats.py:2437):
//                        the same tiles, split by template into two grids so
//                        that each gets its own block shape and shared memory.
//  * dvals               value gradient <dY[row], B[col]> for every nonzero,
//                        over an entry list built from the same tiles (the
//                        SDDMM entry-list kernel of sddmm.cu)
//  * pack_values_kernel  per-head value sets of a batched run
#include "common.cuh"
#include <algorithm>
#include <map>
#include <mutex>

#include "spmm.cuh"

namespace stile {

// ===========================================================================
// plain CSR SpMM (the comparator)
// ===========================================================================
// Nonzero-balanced CSR: every LPR-lane group owns kCsrNnz consecutive
// nonzeros, takes its first row from group_rows (or, when that is NULL,
// from a binary search in indptr) and walks the
// rows it touches (4 B rows in flight per lane).  A row lying wholly inside
// the range is stored; a row that straddles a range boundary is accumulated
// with atomics into a row that csr_prezero_kernel zeroed first.
constexpr int kCsrNnz = kCsrGroupNnz;

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
                                                       int n_groups, const int* __restrict__ group_rows) {
  const int lane = threadIdx.x & 31;
  const int sub = lane / LPR, sl = lane % LPR;
  const int g = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (kWarp / LPR) + sub;
  if (g >= n_groups) return;
  const long nnz = indptr[M];
  const long t0 = (long)g * kCsrNnz;
  const long t1 = min(t0 + kCsrNnz, nnz);
  int r = group_rows ? __ldg(group_rows + g) : row_of_nnz(indptr, M, t0);
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
                                 long ldc, int N, long c_head_stride) {
  // one warp per row, float4 stores.  Launched dependent on the previous
  // kernel, whose reads of C must be done first; the ELL kernel may launch
  // meanwhile (it waits for this grid before adding into these rows)
  griddep_wait();
  griddep_launch_dependents();
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp_global >= n_rows) return;
  float* row = C + blockIdx.y * c_head_stride + (long)rows[warp_global] * ldc;
  for (int f = 4 * lane; f < N; f += 128) st_row4(row, f, N, make_float4(0.f, 0.f, 0.f, 0.f));
}

// ===========================================================================
// hybrid SpMM: tensor-core kernel + ELL kernel (launched back to back)
// ===========================================================================
// Tensor-core chunks.  A chunk is a run of at most kChunkSteps k-steps of
// one item (items longer than that are split; the parts add into rows that
// another writer initialises).  Per k-step the kernel gathers the 16
// referenced B rows (fp32, 128 features) and the step's 16x16 value image,
// converts the rows to the bf16 / fp16 A-operand image and one thread
// issues the tcgen05.mma.
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
constexpr uint32_t kRawRows = 8192;  // 16 rows x 128 fp32 per stage
// fp8 operands (K = 32 bytes, K-major, no swizzle): core matrices of 8 rows
// x 16 bytes, the two k halves 128 B apart (LBO), 8-row groups 256 B apart
// (SBO); the A image is 4 KB, a k-step's value image 512 B
constexpr uint32_t kF8Lbo = 128, kF8Sbo = 256;
constexpr float kE4m3Max = 448.f;

__device__ __forceinline__ uint32_t a_img_off(int m, int k) {
  // m: feature (0..127), k: column within the k-step (0..15)
  const int atom = m >> 6, grp = k >> 3, r = k & 7, chunk = (m & 63) >> 3;
  return (uint32_t)(atom * kALbo + grp * kASbo + r * 128 + ((chunk ^ r) << 4) + (m & 7) * 2);
}

// Persistent bf16 / fp16 tensor-core kernel.
//
// The upload assigns chunks to the kernel's CTAs (longest first, each to the
// least loaded CTA) and stores every CTA's k-steps contiguously, so a CTA's
// work is the step range [s_beg, s_beg + S), walked once per 128-feature
// slice; its units are (slice, chunk) pairs in that order.
// Roles (kProdWarps producer warps, then one warp whose lane 0 issues the
// MMAs, then four epilogue warps):
//  * Producers: warp w fills the steps g = w, w + kProdWarps, ... and owns
//    raw stage w and operand slot g % kWsSlots.  Per step each lane copies
//    features 4l..4l+3 of the step's 16 B rows and 16 bytes of its 512-byte
//    value image with cp.async into the stage (the rows' column ids, one per
//    lane 0-15, were loaded one step earlier and are broadcast by shuffle),
//    then, once the copies landed and the MMA that last read the slot has
//    committed its empty barrier, converts its own copies to the bf16 / fp16
//    A image in the slot, and lane 0 arrives on the slot's full barrier.
//    The next step's copies go out right after, so every producer warp keeps
//    one step in flight while the others convert: the steps of one CTA
//    overlap kProdWarps ways, and no producer waits on another.
//  * MMA: per unit t waits until the epilogue released accumulator t % 4
//    (TMEM columns 16 * (t % 4)), then per step waits for a full slot,
//    issues tcgen05.mma and commits to the slot's empty barrier; a unit's
//    last step also commits to the accumulator's full barrier.
//  * Epilogue: per unit waits for its accumulator, reads it (warp w reads
//    TMEM lanes 32 * (w % 4)..+31), releases it and writes C.
// Every wait is bounded; a wait that gives up sets the error flag and ends
// that role, and the others then end at their next (bounded) wait.
constexpr int kProdWarps = 4;                            // producer warps, one step in flight each
constexpr int kAccBufs = 4;                              // accumulators of 16 TMEM columns
constexpr int kWsThreads = (kProdWarps + 1 + 4) * 32;   // producers, MMA warp, 4 epilogue warps

// Per-mode layout.  Split-bf16 (fp32-level accuracy) keeps hi and lo images
// of both operands: A = hi(B rows) | lo(B rows), values = hi | lo, and
// issues three MMAs per step (hi*hi + hi*lo + lo*hi); its accumulator is
// drained into the epilogue's fp32 registers every kGroup steps, which
// bounds the tensor core's accumulation chain.
//
// A bf16 B (kIn16) needs no conversion: the producers copy its rows with
// cp.async straight into the swizzled A image of the slot (each 16-byte
// chunk of a row is 8 features, one chunk of the layout), so there is no raw
// stage and every producer warp keeps two steps in flight in its two slots.
// Slot s holds the A image(s) at a_off(s) (1024-aligned) and the value
// image(s) at v_off(s): A images first, then all value images.
template <int MODE, bool kIn16 = false>
struct WsCfg {
  static constexpr bool kSplit = MODE == STILE_TC_SPLIT_BF16;
  static constexpr int kSlots = kIn16 ? 3 * kProdWarps : kProdWarps;  // warp w fills slots w, w + 4, ..
  static constexpr uint32_t kVals = kSplit ? 2 * kBStage : kBStage;   // value image(s) per step
  static constexpr uint32_t kAImg = kSplit ? 2 * kAStage : kAStage;   // A image(s) per step
  static constexpr uint32_t kSlotBytes = kSlots * (kAImg + kVals);
  static constexpr uint32_t kRaw = kIn16 ? 0 : kRawRows + kVals;      // 16 fp32 rows + value image(s)
  // full / empty barrier per slot, full / empty per accumulator, drain, TMEM address
  static constexpr uint32_t kBarBytes = (16 * kSlots + 16 * kAccBufs + 16 + 63) / 64 * 64;
  static constexpr uint32_t kBytes = 1024 + kSlotBytes + kProdWarps * kRaw + kBarBytes;
  static __device__ __forceinline__ uint32_t a_off(int s) { return (uint32_t)s * kAImg; }
  static __device__ __forceinline__ uint32_t v_off(int s) { return kSlots * kAImg + (uint32_t)s * kVals; }
  static constexpr int kCtas = kSplit ? 3 : 4;                        // resident CTAs per SM
  static constexpr int kGroup = kSplit ? 4 : (1 << 30);               // k-steps per accumulator drain
  static_assert(!(kIn16 && MODE != STILE_TC_BF16), "a bf16 B feeds bf16 MMAs");
};

// kFull: every 128-feature slice is complete (N % 128 == 0)
template <int MODE, bool kFull, bool kIn16>
__global__ void __launch_bounds__(kWsThreads, WsCfg<MODE, kIn16>::kCtas) spmm_tc_ws_kernel(SpmmArgs p) {
  using W = WsCfg<MODE, kIn16>;
  constexpr int kWsSlots = W::kSlots;
  griddep_launch_dependents();  // the next kernel waits for this grid before using its results
  extern __shared__ uint8_t smem_raw[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t slots = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const uint32_t ring = slots + W::kSlotBytes;
  const uint32_t bars = ring + kProdWarps * W::kRaw;
  // full[kWsSlots], empty[kWsSlots], acc_full[kAccBufs], acc_empty[kAccBufs], drain
  const uint32_t full0 = bars, empty0 = bars + 8 * kWsSlots;
  const uint32_t accf0 = bars + 16 * kWsSlots, acce0 = accf0 + 8 * kAccBufs;
  const uint32_t drain = acce0 + 8 * kAccBufs;
  const uint32_t tmem_slot = drain + 8;

  if (tid == 0) {
    for (int s = 0; s < kWsSlots; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < kAccBufs; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, 4);
    }
    mbar_init(drain, 1);
    fence_mbar_init();
  }
  if constexpr (MODE == STILE_TC_FP8) {
    // the A images' upper k halves stay zero (each k-step fills the lower
    // half of a K = 32 operand); made visible to the tensor core's proxy
    for (int i = tid; i < (int)(kWsSlots * W::kAImg / 16); i += kWsThreads)
      st_shared_v4(slots + W::a_off(0) + 16 * i, make_uint4(0u, 0u, 0u, 0u));
    fence_proxy_async_smem();
  }
  if (warp == 0) {
    __syncwarp();
    tmem_alloc(tmem_slot, 16 * kAccBufs);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  uint32_t tmem;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(tmem) : "r"(tmem_slot) : "memory");

  // this CTA's chunks and their contiguous k-steps
  const int cb = __ldg(p.tc_cta_chunk + blockIdx.x);
  const int nc = __ldg(p.tc_cta_chunk + blockIdx.x + 1) - cb;
  const int s_beg = nc > 0 ? __ldg(p.tc_chunk_kbeg + cb) : 0;
  const int S = nc > 0 ? __ldg(p.tc_chunk_kbeg + cb + nc - 1) + __ldg(p.tc_chunk_nk + cb + nc - 1) - s_beg : 0;
  // feature slices of this CTA: blockIdx.y takes [sl0, sl0 + nf) (a wide B
  // spreads its slices over more CTAs than the chunk schedule has)
  const int sl0 = blockIdx.y * p.tc_slice_per;
  const int nf = min(p.tc_slice_per, p.n_fchunks - sl0);
  const long T = (long)S * nf;  // this CTA's k-steps over its slices
  const int n_units = nc * nf;
  const int N = p.N;
  const uint32_t polls = p.poll_limit ? p.poll_limit : kDefaultPolls;  // pipeline waits
  bool ok = true;

  if (warp < kProdWarps) {
    // ---------------- producers ----------------
    const uint8_t* vals = reinterpret_cast<const uint8_t*>(p.tc_vals) + blockIdx.z * p.tc_vals_head_stride;
    const uint32_t stage = ring + (uint32_t)warp * W::kRaw;
    // step g is k-step s_beg + loc of feature slice f0 / 128 (g = f0 / 128 * S + loc)
    long g = warp;
    int loc = 0, f0 = 0;
    if (g < T) {
      loc = warp % S;
      f0 = (sl0 + warp / S) * 128;
    }
    auto step_cols = [&](long gg, int l) {
      return (gg < T && lane < 16) ? __ldg(p.tc_cols + (long)(s_beg + l) * 16 + lane) : 0;
    };
    // (loc, f0) of this warp's step after the one at (l, ff)
    auto next_of = [&](int l, int ff, int& ln, int& fn) {
      ln = l + kProdWarps;
      fn = ff;
      while (ln >= S) {
        ln -= S;
        fn += 128;
      }
    };
    if constexpr (kIn16) {
      const uint16_t* B16 = reinterpret_cast<const uint16_t*>(p.B) + blockIdx.z * p.b_head_stride;
      const int ch = lane & 15, rh = lane >> 4;  // this lane's 16-byte chunk (8 features) and row parity
      // the step at (l, ff) into `slot`: rows 2j + rh, features ff + 8 ch ..
      auto issue16 = [&](int cols, int l, int ff, int slot) {
        const uint32_t sa = slots + W::a_off(slot);
        const int f = ff + 8 * ch;
        const uint32_t bytes = kFull ? 16u : ((f + 8 <= N) ? 16u : (f < N ? (uint32_t)(N - f) * 2u : 0u));
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int r = 2 * j + rh;
          const int col = __shfl_sync(0xffffffffu, cols, r);
          const uint16_t* row = B16 + (long)col * p.ldb;
          cp_async16(sa + a_img_off(8 * ch, r), bytes ? (const void*)(row + f) : (const void*)row, bytes);
        }
        cp_async16(slots + W::v_off(slot) + lane * 16, vals + (long)(s_beg + l) * kBStage + lane * 16, 16u);
        cp_async_commit();
      };
      // kD steps of this warp in flight; once the oldest (g) has landed and
      // the MMA that read its slot last time is done, step g + kD kProdWarps
      // refills that slot
      constexpr int kD = kWsSlots / kProdWarps;
      static_assert(kD >= 1 && kD <= 3, "one to three steps in flight per warp");
      long gi = g;  // the next step to issue, at (li, fi)
      int li = loc, fi = f0;
      for (int d = 0; d < kD && gi < T; ++d) {
        issue16(step_cols(gi, li), li, fi, (int)(gi % kWsSlots));
        gi += kProdWarps;
        next_of(li, fi, li, fi);
      }
#pragma unroll 1
      for (; g < T; g += kProdWarps) {
        const int cols_i = step_cols(gi, li);
        const long pend = (gi - g) / kProdWarps;  // this warp's steps in flight, g the oldest
        if (pend >= 3) cp_async_wait<2>();
        else if (pend == 2) cp_async_wait<1>();
        else cp_async_wait<0>();
        fence_proxy_async_smem();
        __syncwarp();
        const int slot = (int)(g % kWsSlots);
        if (lane == 0) mbar_arrive(full0 + 8 * slot);
        if (gi < T) {
          const uint32_t par = (uint32_t)(g / kWsSlots) & 1u;
          bool got = true;
          if (lane == 0) got = mbar_wait_bounded(empty0 + 8 * slot, par, polls);
          if (!__shfl_sync(0xffffffffu, got, 0)) {
            ok = false;
            break;
          }
          if (lane != 0) mbar_wait_bounded(empty0 + 8 * slot, par, polls);  // completed: returns at once
          issue16(cols_i, li, fi, slot);
          gi += kProdWarps;
          next_of(li, fi, li, fi);
        }
      }
      cp_async_wait<0>();
    } else {
    // fp8: B's e4m3 scale comes from the run's amax pass, which finished
    // before this kernel started (an ordinary launch never lets a dependent
    // start early)
    float xinv = 1.f;
    if constexpr (MODE == STILE_TC_FP8) {
      const float amax = __uint_as_float(*p.tc_xamax);
      xinv = amax > 0.f ? kE4m3Max / amax : 0.f;
    }
    auto issue = [&](int cols, int l, int ff) {
      const int f = ff + 4 * lane;
      const uint32_t bytes = kFull ? 16u : ((f + 4 <= N) ? 16u : (f < N ? (uint32_t)(N - f) * 4u : 0u));
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        const int col = __shfl_sync(0xffffffffu, cols, r);
        const float* row = p.B + blockIdx.z * p.b_head_stride + (long)col * p.ldb;
        cp_async16(stage + r * 512 + lane * 16, bytes ? (const void*)(row + f) : (const void*)row, bytes);
      }
#pragma unroll
      for (int c = lane; c < (int)(W::kVals / 16); c += 32)
        cp_async16(stage + kRawRows + c * 16, vals + (long)(s_beg + l) * W::kVals + c * 16, 16u);
      cp_async_commit();
    };
    if (g < T) issue(step_cols(g, loc), loc, f0);
#pragma unroll 1
    for (; g < T; g += kProdWarps) {
      // this warp's next step and its column ids (used after the convert)
      const long gn = g + kProdWarps;
      int locn, f0n;
      next_of(loc, f0, locn, f0n);
      const int coln = step_cols(gn, locn);
      cp_async_wait<0>();
      const int slot = (int)(g % kWsSlots);
      if (g >= kWsSlots) {
        const uint32_t par = (uint32_t)((g - kWsSlots) / kWsSlots) & 1u;
        bool got = true;
        if (lane == 0) got = mbar_wait_bounded(empty0 + 8 * slot, par, polls);
        if (!__shfl_sync(0xffffffffu, got, 0)) {
          ok = false;
          break;
        }
        if (lane != 0) mbar_wait_bounded(empty0 + 8 * slot, par, polls);  // completed: returns at once
      }
      const uint32_t sa = slots + W::a_off(slot);
      if constexpr (MODE == STILE_TC_FP8) {
        // this lane's 4 features x the step's 16 rows -> four K-major
        // 16-byte rows of the A image (feature m: the e4m3 bytes of x / s_x
        // for k = 0..15), core matrices of 8 features x 16 bytes
        uint32_t wd[4][4];
#pragma unroll
        for (int r = 0; r < 16; r += 2) {
          const uint4 ra = ld_shared_v4(stage + r * 512 + lane * 16);
          const uint4 rb = ld_shared_v4(stage + (r + 1) * 512 + lane * 16);
          const uint32_t ua[4] = {ra.x, ra.y, ra.z, ra.w}, ub[4] = {rb.x, rb.y, rb.z, rb.w};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const uint32_t h = pack_e4m3x2(__uint_as_float(ua[j]) * xinv, __uint_as_float(ub[j]) * xinv);
            if ((r & 2) == 0) wd[j][r >> 2] = h; else wd[j][r >> 2] |= h << 16;
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int m = 4 * lane + j;
          st_shared_v4(sa + (uint32_t)((m >> 3) * kF8Sbo + (m & 7) * 16),
                       make_uint4(wd[j][0], wd[j][1], wd[j][2], wd[j][3]));
        }
      }
#pragma unroll
      for (int r = 0; r < (MODE == STILE_TC_FP8 ? 0 : 16); ++r) {
        const uint4 raw = ld_shared_v4(stage + r * 512 + lane * 16);
        const float4 v = make_float4(__uint_as_float(raw.x), __uint_as_float(raw.y), __uint_as_float(raw.z),
                                     __uint_as_float(raw.w));
        const uint32_t o = a_img_off(4 * lane, r);
        if (MODE == STILE_TC_F16) {
          st_shared_v2(sa + o, pack_f16x2(v.x, v.y), pack_f16x2(v.z, v.w));
        } else {
          const uint32_t h01 = pack_bf16x2(v.x, v.y), h23 = pack_bf16x2(v.z, v.w);
          st_shared_v2(sa + o, h01, h23);
          if (W::kSplit) {
            // lo = v - float(hi): exact in fp32, then rounded to bf16
            const float4 hf = make_float4(__uint_as_float(h01 << 16), __uint_as_float(h01 & 0xffff0000u),
                                          __uint_as_float(h23 << 16), __uint_as_float(h23 & 0xffff0000u));
            st_shared_v2(sa + kAStage + o, pack_bf16x2(v.x - hf.x, v.y - hf.y), pack_bf16x2(v.z - hf.z, v.w - hf.w));
          }
        }
      }
#pragma unroll
      for (int c = lane; c < (int)(W::kVals / 16); c += 32)
        st_shared_v4(slots + W::v_off(slot) + c * 16, ld_shared_v4(stage + kRawRows + c * 16));
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(full0 + 8 * slot);
      if (gn < T) issue(coln, locn, f0n);
      loc = locn;
      f0 = f0n;
    }
    cp_async_wait<0>();
    }
  } else if (warp == kProdWarps) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      // fp8: e4m3 x e4m3, both operands K-major
      const uint32_t idesc = (MODE == STILE_TC_F16)   ? make_idesc(0, 0, 1, 0, 128, 16)
                             : (MODE == STILE_TC_FP8) ? make_idesc(0, 0, 0, 0, 128, 16)
                                                      : make_idesc(1, 1, 1, 0, 128, 16);
      long g = 0;
      int u = 0;  // accumulation groups issued so far (accumulator u % kAccBufs)
      // failure-detection test: nothing arrives on `drain` before the
      // commit below, so this wait runs out
      if (p.stall_test && !mbar_wait_bounded(drain, 0u, polls)) ok = false;
#pragma unroll 1
      for (int t = 0; t < n_units && ok; ++t) {
        const int n = __ldg(p.tc_chunk_nk + cb + t % nc);
#pragma unroll 1
        for (int s0 = 0; s0 < n && ok; s0 += W::kGroup, ++u) {
          const int b = u % kAccBufs;
          if (u >= kAccBufs && !mbar_wait_bounded(acce0 + 8 * b, (uint32_t)((u - kAccBufs) / kAccBufs) & 1u, polls)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem + (uint32_t)(16 * b);
          const int s1 = min(n, s0 + W::kGroup);
#pragma unroll 1
          for (int s = s0; s < s1; ++s, ++g) {
            const int slot = (int)(g % kWsSlots);
            if (!mbar_wait_bounded(full0 + 8 * slot, (uint32_t)(g / kWsSlots) & 1u, polls)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sa = slots + W::a_off(slot), sv = slots + W::v_off(slot);
            const uint64_t a_hi = smem_desc(sa, kALbo, kASbo, kSwizzle128B);
            const uint64_t v_hi = smem_desc(sv, kBLbo, kBSbo, kSwizzleNone);
            if constexpr (MODE == STILE_TC_FP8)
              umma_f8(d, smem_desc(sa, kF8Lbo, kF8Sbo, kSwizzleNone), smem_desc(sv, kF8Lbo, kF8Sbo, kSwizzleNone),
                      idesc, s > s0 ? 1u : 0u);
            else
              umma_f16(d, a_hi, v_hi, idesc, s > s0 ? 1u : 0u);
            if (W::kSplit) {
              umma_f16(d, a_hi, smem_desc(sv + kBStage, kBLbo, kBSbo, kSwizzleNone), idesc, 1u);
              umma_f16(d, smem_desc(sa + kAStage, kALbo, kASbo, kSwizzle128B), v_hi, idesc, 1u);
            }
            umma_commit(empty0 + 8 * slot);
          }
          if (ok) umma_commit(accf0 + 8 * b);
        }
      }
      // every MMA this thread issued has completed before TMEM is freed
      umma_commit(drain);
      if (!mbar_wait_bounded(drain, 0u)) ok = false;
    }
    __syncwarp();
  } else {
    // ---------------- epilogue ----------------
    // launched dependent on the ELL kernel: the producers and the MMA start
    // while it drains, the C writes (adds to rows it stores) wait for it
    griddep_wait();
    const int quarter = warp & 3;
    int u = 0;  // accumulation groups consumed so far
#pragma unroll 1
    for (int t = 0; t < n_units && ok; ++t) {
      const int n = __ldg(p.tc_chunk_nk + cb + t % nc);
      float acc[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) acc[i] = 0.f;
#pragma unroll 1
      for (int s0 = 0; s0 < n; s0 += W::kGroup, ++u) {
        const int b = u % kAccBufs;
        const uint32_t par = (uint32_t)(u / kAccBufs) & 1u;
        bool got = true;
        if (lane == 0) got = mbar_wait_bounded(accf0 + 8 * b, par, polls);
        if (!__shfl_sync(0xffffffffu, got, 0)) {
          ok = false;
          break;
        }
        if (lane != 0) mbar_wait_bounded(accf0 + 8 * b, par, polls);  // completed: returns at once
        tc_fence_after();
        uint32_t r[16];
        tmem_ld16(tmem + (uint32_t)(16 * b) + ((uint32_t)(32 * quarter) << 16), r);
        tmem_wait_ld();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(acce0 + 8 * b);
#pragma unroll
        for (int i = 0; i < 16; ++i) acc[i] += __uint_as_float(r[i]);
      }
      if (!ok) break;
      const int c = cb + t % nc;
      const int f = (sl0 + t / nc) * 128 + 32 * quarter + lane;
      if (kFull || f < N) {
        const int item = __ldg(p.tc_chunk_item + c);
        const bool atomic = (__ldg(p.tc_chunk_flags + c) & 1) != 0;
        const int* orows = p.tc_out_rows + (long)item * 16;
        if constexpr (MODE == STILE_TC_FP8) {
          // undo the scales: B's (per tensor) and the tile row's
          const float sx = __uint_as_float(*p.tc_xamax) / kE4m3Max;
#pragma unroll
          for (int i = 0; i < 16; ++i) acc[i] *= sx * __ldg(p.tc_row_scale + (long)item * 16 + i);
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int row = __ldg(orows + i);
          if (row < 0) continue;
          float* dst = p.C + blockIdx.z * p.c_head_stride + (long)row * p.ldc + f;
          if (atomic) atomicAdd(dst, acc[i]); else __stcs(dst, acc[i]);  // C is not read again: evict first
        }
      }
    }
  }
  if (!ok) atomicOr(p.err_flag, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, 16 * kAccBufs);
}

// ELL tiles as a stream of live entries in row order, packed as 16-byte
// records {column, value, 2 * row code + run end, 0}.  An LPR-lane
// sub-group owns one group of <= kSegNnz entries; each lane covers 4 * VEC
// features of a row, float4 w at features 4 (w LPR + lane), so that every
// load instruction of the sub-group reads 16 LPR contiguous bytes (whole
// 128-byte lines: the L1 tag stage, not DRAM, limits these gathers, and an
// interleaved 8-features-per-lane split touched twice the lines per
// instruction).  The sub-group holds the group's records LPR at a time
// (one per lane, the next LPR loaded while these are consumed), broadcasts
// them by shuffle, keeps 4 float4 B-row gathers in flight per lane and
// flushes the running sum after every entry that ends its row's run (store
// for a row the ELL kernel initialises, atomic add otherwise).  With
// VEC = 2 two sub-groups share every warp-wide shuffle and branch, so the
// instructions per gathered byte halve; no gather waits on a metadata load,
// and few registers leave room for many warps per SM.
// kFull: N % (4 * VEC * LPR) == 0, every lane's features are in range
// (otherwise a float4 that starts past N reads as zero).
// kOff32: every B row offset col * ldb fits in 32 bits.
// kSpanY: blockIdx.y takes features [y span, (y + 1) span) (a wide B over
// few groups; span = p.ell_fc_span, a multiple of the pass width).
// kHeads: a batched run (blockIdx.z = head offsets B, C and the records).
template <int LPR, int VEC, bool kFull, bool kOff32, bool kSpanY = false, bool kHeads = false>
__global__ void __launch_bounds__(256, 5) spmm_ell_seg_kernel(SpmmArgs p) {
  constexpr int kBatch = 4 / VEC;  // entries per batch: 4 float4 in flight per lane
  // Launched dependent on the previous kernel.  When that is the zero-rows
  // kernel (p.ell_lazy_wait), only the atomic adds (into rows it zeroes)
  // wait for it, and every thread waits before it exits, so that this
  // grid's completion implies that kernel's; otherwise (B may come from the
  // previous kernel) everything waits.  The tensor-core kernel may launch
  // once this grid is running.
  if (!p.ell_lazy_wait) griddep_wait();
  griddep_launch_dependents();
  const int lane = threadIdx.x & 31, sub = lane / LPR, sl = lane % LPR;
  const unsigned mask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << (sub * LPR));
  const int g = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (kWarp / LPR) + sub;
  if (g >= p.ell_n_groups) {  // the whole sub-group leaves together
    if (p.ell_lazy_wait) griddep_wait();
    return;
  }
  const int p0 = __ldg(p.ell_group_ptr + g);
  const int n = __ldg(p.ell_group_ptr + g + 1) - p0;
  const long head = kHeads ? blockIdx.z : 0;
  const int4* __restrict__ ent = p.ell_entry + head * p.ell_n_pos + p0;
  const int N = p.N;
  const int ldb32 = (int)p.ldb;
  // records are read once: streaming loads leave L2 to the B rows
  auto rec = [&](int i) { return i < n ? __ldcs(ent + i) : make_int4(0, 0, 0, 0); };
  for (int fc = kSpanY ? blockIdx.y * p.ell_fc_span : 0;
       fc < (kSpanY ? min(N, (int)(blockIdx.y + 1) * p.ell_fc_span) : N); fc += 4 * VEC * LPR) {
    // float4 w of this lane holds features f + 4 LPR w: each load
    // instruction of the group reads 16 LPR contiguous bytes of a row
    const int f = fc + 4 * sl;
    const float* Bf = p.B + head * p.b_head_stride + f;
    float4 acc[VEC];
#pragma unroll
    for (int w = 0; w < VEC; ++w) acc[w] = make_float4(0.f, 0.f, 0.f, 0.f);
    int4 mcur = rec(sl);
#pragma unroll 1
    for (int c0 = 0; c0 < n; c0 += LPR) {
      const int4 mnext = rec(c0 + LPR + sl);
#pragma unroll 1
      for (int b0 = c0; b0 < min(n, c0 + LPR); b0 += kBatch) {
        float4 bv[kBatch][VEC];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
          const int c = __shfl_sync(mask, mcur.x, b0 - c0 + u, LPR);
          // records past n hold column 0: a valid row, multiplied by 0
          if (kFull) {
            const float* row = kOff32 ? Bf + (unsigned)(c * ldb32) : Bf + (long)c * p.ldb;
#pragma unroll
            for (int w = 0; w < VEC; ++w) bv[u][w] = ldg4(row + 4 * LPR * w);
          } else {
            // float4 past N read as zero; padding features inside the last
            // live float4 only reach features that are never stored
            const float* row = p.B + head * p.b_head_stride + (long)c * p.ldb;
#pragma unroll
            for (int w = 0; w < VEC; ++w) bv[u][w] = ld4_pad(row, f + 4 * LPR * w, N);
          }
        }
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
          const float v = __int_as_float(__shfl_sync(mask, mcur.y, b0 - c0 + u, LPR));
          const int ce = __shfl_sync(mask, mcur.z, b0 - c0 + u, LPR);
#pragma unroll
          for (int w = 0; w < VEC; ++w) fma4(acc[w], v, bv[u][w]);  // records past n: value 0, no run end
          if (ce & 1) {
            const int code = ce >> 1;
            float* row = p.C + head * p.c_head_stride + (long)(code >= 0 ? code : -code - 1) * p.ldc;
#pragma unroll
            for (int w = 0; w < VEC; ++w) {
              const int fw = f + 4 * LPR * w;
              if (code < 0 && p.ell_lazy_wait) griddep_wait();
              if (kFull) {
                if (code >= 0) __stcs(reinterpret_cast<float4*>(row + fw), acc[w]);  // evict first
                else atomicAdd(reinterpret_cast<float4*>(row + fw), acc[w]);
              } else {
                if (code >= 0) st_row4(row, fw, N, acc[w]); else red_row4(row, fw, N, acc[w]);
              }
              acc[w] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
          }
        }
      }
      mcur = mnext;
    }
  }
  if (p.ell_lazy_wait) griddep_wait();
}

// The fused backward's ELL pass, run over the transposed operator's tiles
// with B = dC: the stream kernel above for VEC = 2 in one feature pass
// (N <= 8 LPR), and for every entry (row r, column c) of A^T also
//   dv_out[id] = <dC[c], dvx[r]>,
// the value gradient of the forward's nonzero (c, r); id, in the forward's
// numbering, rides in the entry record's fourth word.  The dC row gathered
// for the product is the one the gradient needs; dvx[r] (the forward's
// dense operand) is loaded where a row run starts, for both entries of a
// batch before either is used, so those loads overlap the dC gathers.  The
// two entries reduce their dot products together with the transposing
// butterfly (lanes whose high bit spells the entry hold its sum).
// kFull: N == 8 LPR.
template <int LPR, bool kFull>
__global__ void __launch_bounds__(256, 4) spmm_ell_bwd_kernel(SpmmArgs p) {
  static_assert(LPR >= 2, "two entries per batch");
  if (!p.ell_lazy_wait) griddep_wait();
  griddep_launch_dependents();
  const int lane = threadIdx.x & 31, sub = lane / LPR, sl = lane % LPR;
  const unsigned mask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << (sub * LPR));
  const int g = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (kWarp / LPR) + sub;
  if (g >= p.ell_n_groups) {  // the whole sub-group leaves together
    if (p.ell_lazy_wait) griddep_wait();
    return;
  }
  const int p0 = __ldg(p.ell_group_ptr + g);
  const int n = __ldg(p.ell_group_ptr + g + 1) - p0;
  const int4* __restrict__ ent = p.ell_entry + p0;
  const int N = p.N;
  // this lane's features: f .. f + 3 and f + 4 LPR .. f + 4 LPR + 3 (each
  // load instruction of the group reads 16 LPR contiguous bytes of a row)
  const int f = 4 * sl, f2 = f + 4 * LPR;
  auto rec = [&](int i) { return i < n ? __ldcs(ent + i) : make_int4(0, 0, 0, -1); };
  auto row_of = [](int ce) { const int code = ce >> 1; return code >= 0 ? code : -code - 1; };
  auto ld8 = [&](const float* row, float4& a, float4& b) {
    a = kFull ? ldg4(row + f) : ld4_live(row, f, N);
    b = kFull ? ldg4(row + f2) : ld4_live(row, f2, N);
  };
  float4 acc0 = make_float4(0.f, 0.f, 0.f, 0.f), acc1 = acc0;
  float4 xa0 = acc0, xa1 = acc0;  // dvx row of the last entry handled
  int xrow = -1;
  int4 mcur = rec(sl);
#pragma unroll 1
  for (int c0 = 0; c0 < n; c0 += LPR) {
#pragma unroll 1
    for (int b0 = c0; b0 < min(n, c0 + LPR); b0 += 2) {
      const int j = b0 - c0;
      const int col0 = __shfl_sync(mask, mcur.x, j, LPR), col1 = __shfl_sync(mask, mcur.x, j + 1, LPR);
      const int ce0 = __shfl_sync(mask, mcur.z, j, LPR), ce1 = __shfl_sync(mask, mcur.z, j + 1, LPR);
      const float v0 = __int_as_float(__shfl_sync(mask, mcur.y, j, LPR));
      const float v1 = __int_as_float(__shfl_sync(mask, mcur.y, j + 1, LPR));
      const int id0 = __shfl_sync(mask, mcur.w, j, LPR), id1 = __shfl_sync(mask, mcur.w, j + 1, LPR);
      const int r0 = row_of(ce0), r1 = row_of(ce1);
      // records past n: row 0, column 0, value 0, no run end, id -1
      float4 b00, b01, b10, b11;
      ld8(p.B + (long)col0 * p.ldb, b00, b01);
      ld8(p.B + (long)col1 * p.ldb, b10, b11);
      float4 x00 = xa0, x01 = xa1;
      if (r0 != xrow) ld8(p.dvx + (long)r0 * p.dvx_ld, x00, x01);
      float4 x10 = x00, x11 = x01;
      if (r1 != r0) ld8(p.dvx + (long)r1 * p.dvx_ld, x10, x11);
      xa0 = x10;
      xa1 = x11;
      xrow = r1;
      const float s0 = dot4(x00, b00) + dot4(x01, b01);
      const float s1 = dot4(x10, b10) + dot4(x11, b11);
      fma4(acc0, v0, b00);
      fma4(acc1, v0, b01);
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int ce = u ? ce1 : ce0;
        if (u) {
          fma4(acc0, v1, b10);
          fma4(acc1, v1, b11);
        }
        if (ce & 1) {
          const int code = ce >> 1;
          float* crow = p.C + (long)(u ? r1 : r0) * p.ldc;
          if (code < 0 && p.ell_lazy_wait) griddep_wait();
          if (kFull) {
            if (code >= 0) {
              __stcs(reinterpret_cast<float4*>(crow + f), acc0);
              __stcs(reinterpret_cast<float4*>(crow + f2), acc1);
            } else {
              atomicAdd(reinterpret_cast<float4*>(crow + f), acc0);
              atomicAdd(reinterpret_cast<float4*>(crow + f2), acc1);
            }
          } else if (code >= 0) {
            st_row4(crow, f, N, acc0);
            st_row4(crow, f2, N, acc1);
          } else {
            red_row4(crow, f, N, acc0);
            red_row4(crow, f2, N, acc1);
          }
          acc0 = make_float4(0.f, 0.f, 0.f, 0.f);
          acc1 = acc0;
        }
      }
      // transposing butterfly over the pair: the upper half keeps entry 1
      const bool up = (sl & (LPR / 2)) != 0;
      float t = (up ? s1 : s0) + __shfl_xor_sync(mask, up ? s0 : s1, LPR / 2);
#pragma unroll
      for (int o = LPR / 4; o > 0; o >>= 1) t += __shfl_xor_sync(mask, t, o);
      const int id = up ? id1 : id0;
      if ((sl & (LPR / 2 - 1)) == 0 && id >= 0) __stcs(p.dv_out + id, t);
    }
    if (c0 + LPR < n) mcur = rec(c0 + LPR + sl);
  }
  if (p.ell_lazy_wait) griddep_wait();
}

// fourth word of every ELL record := the forward operator's id of its
// nonzero (perm of the record's own id), -1 for padding
__global__ void record_ids_kernel(int4* __restrict__ ent, const int* __restrict__ ids, long n,
                                  const int* __restrict__ perm) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int v = ids[i];
  ent[i].w = v >= 0 ? perm[v] : -1;
}

cudaError_t launch_record_ids(int4* ent, const int* ids, long n, const int* perm, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  record_ids_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(ent, ids, n, perm);
  return cudaGetLastError();
}

__global__ void permute_ids_kernel(const int* __restrict__ in, long n, const int* __restrict__ perm,
                                   int* __restrict__ out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int v = in[i];
  out[i] = v >= 0 ? perm[v] : -1;
}

cudaError_t launch_permute_ids(const int* in, long n, const int* perm, int* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  permute_ids_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, n, perm, out);
  return cudaGetLastError();
}

// The same entry stream over a bf16 B: each lane covers 8 features with one
// 16-byte load (half the gathered bytes of fp32 rows), converts them to
// fp32 and accumulates in fp32; 4 entries' rows in flight per lane.
template <int LPR, bool kFull, bool kOff32, bool kSpanY = false>
__global__ void __launch_bounds__(256, 4) spmm_ell_seg_bf16_kernel(SpmmArgs p) {
  constexpr int kBatch = 4;
  static_assert(LPR % kBatch == 0, "batches stay inside one record block");
  // Launched dependent on the previous kernel.  When that is the zero-rows
  // kernel (p.ell_lazy_wait), only the atomic adds (into rows it zeroes)
  // wait for it, and every thread waits before it exits, so that this
  // grid's completion implies that kernel's; otherwise (B may come from the
  // previous kernel) everything waits.  The tensor-core kernel may launch
  // once this grid is running.
  if (!p.ell_lazy_wait) griddep_wait();
  griddep_launch_dependents();
  const int lane = threadIdx.x & 31, sub = lane / LPR, sl = lane % LPR;
  const unsigned mask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << (sub * LPR));
  const int g = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (kWarp / LPR) + sub;
  if (g >= p.ell_n_groups) {  // the whole sub-group leaves together
    if (p.ell_lazy_wait) griddep_wait();
    return;
  }
  const int p0 = __ldg(p.ell_group_ptr + g);
  const int n = __ldg(p.ell_group_ptr + g + 1) - p0;
  const int4* __restrict__ ent = p.ell_entry + blockIdx.z * p.ell_n_pos + p0;
  const uint16_t* __restrict__ B16 = reinterpret_cast<const uint16_t*>(p.B) + blockIdx.z * p.b_head_stride;
  float* __restrict__ Ch = p.C + blockIdx.z * p.c_head_stride;
  const int N = p.N;
  const int ldb32 = (int)p.ldb;
  // records are read once: streaming loads leave L2 to the B rows
  auto rec = [&](int i) { return i < n ? __ldcs(ent + i) : make_int4(0, 0, 0, 0); };
  for (int fc = kSpanY ? blockIdx.y * p.ell_fc_span : 0;
       fc < (kSpanY ? min(N, (int)(blockIdx.y + 1) * p.ell_fc_span) : N); fc += 8 * LPR) {
    const int f = fc + 8 * sl;
    float4 acc0 = make_float4(0.f, 0.f, 0.f, 0.f), acc1 = acc0;
    int4 mcur = rec(sl);
#pragma unroll 1
    for (int c0 = 0; c0 < n; c0 += LPR) {
      const int4 mnext = rec(c0 + LPR + sl);
#pragma unroll 1
      for (int b0 = c0; b0 < min(n, c0 + LPR); b0 += kBatch) {
        uint4 bv[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
          const int c = __shfl_sync(mask, mcur.x, b0 - c0 + u, LPR);
          // records past n hold column 0: a valid row, multiplied by 0
          const uint16_t* row = kOff32 ? B16 + (unsigned)(c * ldb32) : B16 + (long)c * p.ldb;
          bv[u] = kFull ? ldg_u4(row + f) : ld_row8_bf16(row, f, N);
        }
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
          const float v = __int_as_float(__shfl_sync(mask, mcur.y, b0 - c0 + u, LPR));
          const int ce = __shfl_sync(mask, mcur.z, b0 - c0 + u, LPR);
          float4 lo, hi;
          bf16x8_to_f32(bv[u], lo, hi);
          fma4(acc0, v, lo);
          fma4(acc1, v, hi);
          if (ce & 1) {
            const int code = ce >> 1;
            float* row = Ch + (long)(code >= 0 ? code : -code - 1) * p.ldc;
            if (code < 0 && p.ell_lazy_wait) griddep_wait();
            if (kFull) {
              if (code >= 0) {
                __stcs(reinterpret_cast<float4*>(row + f), acc0);
                __stcs(reinterpret_cast<float4*>(row + f + 4), acc1);
              } else {
                atomicAdd(reinterpret_cast<float4*>(row + f), acc0);
                atomicAdd(reinterpret_cast<float4*>(row + f + 4), acc1);
              }
            } else if (code >= 0) {
              st_row4(row, f, N, acc0);
              st_row4(row, f + 4, N, acc1);
            } else {
              red_row4(row, f, N, acc0);
              red_row4(row, f + 4, N, acc1);
            }
            acc0 = make_float4(0.f, 0.f, 0.f, 0.f);
            acc1 = acc0;
          }
        }
      }
      mcur = mnext;
    }
  }
  if (p.ell_lazy_wait) griddep_wait();
}

// ===========================================================================
// value gradient: dvals[t] = <dY[row(t)], B[col(t)]> over the plan's entry
// list (launch_dvals -> launch_sddmm_list)
// ===========================================================================

// ===========================================================================
// value re-pack: refresh the plan's tile values from a CSR-ordered value
// array (used when the matrix values change but the pattern does not)
// ===========================================================================
__global__ void repack_values_kernel(SpmmArgs p, const float* __restrict__ vals, int4* ell_entry,
                                     uint16_t* tc_img, long n_ell_slots) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long n_tc = (long)p.tc_n_ksteps * 256;
  if (i < n_tc) {
    const long ks = i >> 8;
    const int e = (int)(i & 255), n = e >> 4, k = e & 15;
    const int id = p.tc_nnz_id[i];
    const float v = id >= 0 ? vals[id] : 0.f;
    const int img = (n >> 3) * 128 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7);
    if (p.tc_mode == STILE_TC_F16) {
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
    ell_entry[s].y = __float_as_int(id >= 0 ? vals[id] : 0.f);
  }
}

// Value sets of a batched run: for head blockIdx.y, the tensor-tile images
// (in the plan's k-step order and mode) and the ELL records (the plan's
// column and row code, the head's value) built from vals + head * nnz.
__global__ void pack_values_kernel(SpmmArgs p, const float* __restrict__ vals, long nnz, int4* __restrict__ ell_out,
                                   uint16_t* __restrict__ tc_out, long n_ell, long tc_head_elems) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long h = blockIdx.y;
  const float* hv = vals + h * nnz;
  const long n_tc = (long)p.tc_n_ksteps * 256;
  if (i < n_tc) {
    const long ks = i >> 8;
    const int e = (int)(i & 255), n = e >> 4, k = e & 15;
    const int id = p.tc_nnz_id[i];
    const float v = id >= 0 ? hv[id] : 0.f;
    const int img = (n >> 3) * 128 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7);
    uint16_t* out = tc_out + h * tc_head_elems;
    if (p.tc_mode == STILE_TC_F16) {
      __half x = __float2half_rn(v);
      out[ks * 256 + img] = *reinterpret_cast<uint16_t*>(&x);
    } else {
      __nv_bfloat16 x = __float2bfloat16_rn(v);
      if (p.tc_mode == STILE_TC_SPLIT_BF16) {
        __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(x));
        out[ks * 512 + img] = *reinterpret_cast<uint16_t*>(&x);
        out[ks * 512 + 256 + img] = *reinterpret_cast<uint16_t*>(&l);
      } else {
        out[ks * 256 + img] = *reinterpret_cast<uint16_t*>(&x);
      }
    }
  } else if (i - n_tc < n_ell) {
    const long s = i - n_tc;
    const int id = p.ell_nnz_id[s];
    int4 r = p.ell_entry[s];
    r.y = __float_as_int(id >= 0 ? hv[id] : 0.f);
    ell_out[h * n_ell + s] = r;
  }
}

// bits of max |B| over K rows x N features into *out (atomicMax on the bits
// of non-negative floats, which order like the floats)
__global__ void amax_kernel(const float* __restrict__ B, long ldb, int K, int N, unsigned* __restrict__ out) {
  float m = 0.f;
  const long total = (long)K * N;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(B[(i / N) * ldb + i % N]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(out, __float_as_uint(m));
}

cudaError_t launch_amax(const float* B, long ldb, int K, int N, unsigned* amax_bits, cudaStream_t st) {
  const long total = (long)K * N;
  if (total == 0) return cudaSuccess;
  const long cap = (long)device_sm_count() * 8;
  const long grid = std::min((total + 255) / 256, cap);
  amax_kernel<<<(unsigned)grid, 256, 0, st>>>(B, ldb, K, N, amax_bits);
  return cudaGetLastError();
}

cudaError_t launch_pack_values(const SpmmArgs& p, const float* vals, long nnz, int heads, void* ell_out,
                               void* tc_out, long n_ell, long tc_head_bytes, cudaStream_t st) {
  const long total = (long)p.tc_n_ksteps * 256 + n_ell;
  if (total == 0 || heads == 0) return cudaSuccess;
  pack_values_kernel<<<dim3((unsigned)((total + 255) / 256), heads), 256, 0, st>>>(
      p, vals, nnz, static_cast<int4*>(ell_out), static_cast<uint16_t*>(tc_out), n_ell, tc_head_bytes / 2);
  return cudaGetLastError();
}

cudaError_t launch_repack(const SpmmArgs& p, const float* vals, long n_ell_slots, cudaStream_t st) {
  const long total = (long)p.tc_n_ksteps * 256 + n_ell_slots;
  if (total == 0) return cudaSuccess;
  const long grid = (total + 255) / 256;
  repack_values_kernel<<<(unsigned)grid, 256, 0, st>>>(
      p, vals, const_cast<int4*>(p.ell_entry),
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
                         long ldb, float* C, long ldc, int N, long nnz, const int* group_rows, cudaStream_t st) {
    const int n_groups = (int)((nnz + kCsrNnz - 1) / kCsrNnz);
    csr_prezero_kernel<<<(M + 255) / 256, 256, 0, st>>>(M, indptr, C, ldc, N);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    constexpr int GPB = 256 / LPR;
    const int grid = (n_groups + GPB - 1) / GPB;
    if (grid == 0) return cudaSuccess;
    csr_spmm_kernel<LPR><<<grid, 256, 0, st>>>(M, indptr, indices, vals, B, ldb, C, ldc, N, n_groups, group_rows);
    return cudaGetLastError();
  }
};

cudaError_t launch_csr_spmm(int M, const int* indptr, const int* indices, const float* vals,
                            const float* B, long ldb, float* C, long ldc, int N, long nnz,
                            const int* group_rows, cudaStream_t st) {
  return dispatch_lpr<CsrLaunch>(lpr_for(N), M, indptr, indices, vals, B, ldb, C, ldc, N, nnz, group_rows, st);
}

cudaError_t launch_zero_rows(const int* rows, int n, float* C, long ldc, int N, cudaStream_t st, int heads,
                             long c_head_stride) {
  if (n == 0 || heads == 0) return cudaSuccess;
  const int grid = (n + 7) / 8;
  return launch_dependent(zero_rows_kernel, dim3(grid, heads), dim3(256), 0, st, rows, n, C, ldc, N, c_head_stride);
}

// CTAs of `kernel` resident per SM at `threads` threads and `smem` bytes of
// dynamic shared memory, from the device's limits (shared memory with the
// per-block reservation, registers, threads, blocks); at least 1.
template <typename K>
static cudaError_t resident_ctas(K kernel, int threads, size_t smem, int* sms, int* per_sm) {
  int dev = 0, smem_sm = 0, reserved = 0, regs_sm = 0, thr_sm = 0, blk_sm = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess)
    return e;
  if ((e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess)
    return e;
  if ((e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev)) != cudaSuccess)
    return e;
  if ((e = cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&blk_sm, cudaDevAttrMaxBlocksPerMultiprocessor, dev)) != cudaSuccess) return e;
  cudaFuncAttributes fa;
  if ((e = cudaFuncGetAttributes(&fa, kernel)) != cudaSuccess) return e;
  const int warps = (threads + 31) / 32;
  const int regs_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
  const long by_smem = (long)smem_sm / (long)(smem + fa.sharedSizeBytes + reserved);
  const long by_regs = regs_warp > 0 ? (long)(regs_sm / regs_warp) / warps : blk_sm;
  const long by_thr = thr_sm / (warps * 32);
  long n = std::min(std::min(by_smem, by_regs), std::min(by_thr, (long)blk_sm));
  *per_sm = (int)std::max(1L, n);
  return cudaSuccess;
}

template <int MODE, bool kFull, bool kIn16 = false>
static cudaError_t launch_ws_t(const SpmmArgs& p, cudaStream_t st) {
  auto k = spmm_tc_ws_kernel<MODE, kFull, kIn16>;
  constexpr uint32_t kWsBytes = WsCfg<MODE, kIn16>::kBytes;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWsBytes);
  if (e != cudaSuccess) return e;
  // shared memory for the resident CTAs; the rest of the unified L1 /
  // shared storage stays L1
  e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  if (p.tc_n_chunks == 0 || p.tc_grid == 0) return cudaSuccess;
  return launch_dependent(k, dim3(p.tc_grid, (p.n_fchunks + p.tc_slice_per - 1) / p.tc_slice_per, std::max(1, p.heads)),
                          dim3(kWsThreads),
                          kWsBytes, st, p);
}

// resident CTAs of the tensor-core kernel on the current device, computed
// once per (device, split mode)
int tc_persistent_ctas(int mode) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  const std::pair<int, int> key{dev, mode == STILE_TC_SPLIT_BF16 ? 1 : 0};
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  int sms = 0, per_sm = 0;
  const cudaError_t e =
      mode == STILE_TC_SPLIT_BF16
          ? resident_ctas(spmm_tc_ws_kernel<STILE_TC_SPLIT_BF16, true, false>, kWsThreads,
                          WsCfg<STILE_TC_SPLIT_BF16>::kBytes, &sms, &per_sm)
          : resident_ctas(spmm_tc_ws_kernel<STILE_TC_BF16, true, false>, kWsThreads, WsCfg<STILE_TC_BF16>::kBytes,
                          &sms, &per_sm);
  if (e != cudaSuccess) return 0;
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = sms * per_sm;
  return sms * per_sm;
}

// Feature slices per CTA of the tensor-core grid.  The chunk schedule
// balances k-steps over tc_grid CTAs; with nf slices a CTA's work is its
// k-steps times nf.  When that makes the longest CTA much longer than the
// average over all resident CTAs (a wide B over few chunks), the slices are
// split over grid.y so that no CTA holds more than about the average.
static int tc_slices_per_cta(const SpmmArgs& p) {
  const int nf = p.n_fchunks;
  if (nf <= 1 || p.tc_max_cta_steps <= 0) return nf;
  const int resident = tc_persistent_ctas(p.tc_mode);
  if (resident <= 0) return nf;
  const long avg = ((long)p.tc_n_ksteps * nf + resident - 1) / resident;  // step-slices per CTA
  const long per = avg / p.tc_max_cta_steps;
  return (int)std::max(1L, std::min<long>(per, nf));
}

cudaError_t launch_tc(const SpmmArgs& args, cudaStream_t st) {
  SpmmArgs p = args;
  p.tc_slice_per = tc_slices_per_cta(p);
  if (p.b_bf16) {
    if (p.tc_mode != STILE_TC_BF16) return cudaErrorNotSupported;
    return p.N % 128 == 0 ? launch_ws_t<STILE_TC_BF16, true, true>(p, st)
                          : launch_ws_t<STILE_TC_BF16, false, true>(p, st);
  }
  switch (p.tc_mode) {
    case STILE_TC_F16:
      return p.N % 128 == 0 ? launch_ws_t<STILE_TC_F16, true>(p, st) : launch_ws_t<STILE_TC_F16, false>(p, st);
    case STILE_TC_FP8:
      return p.N % 128 == 0 ? launch_ws_t<STILE_TC_FP8, true>(p, st) : launch_ws_t<STILE_TC_FP8, false>(p, st);
    case STILE_TC_SPLIT_BF16:
      return p.N % 128 == 0 ? launch_ws_t<STILE_TC_SPLIT_BF16, true>(p, st)
                            : launch_ws_t<STILE_TC_SPLIT_BF16, false>(p, st);
    default:
      return p.N % 128 == 0 ? launch_ws_t<STILE_TC_BF16, true>(p, st) : launch_ws_t<STILE_TC_BF16, false>(p, st);
  }
}

// Streaming multiprocessors of the current device (cached per device; 1 if
// the query fails, which only shrinks grids).
int device_sm_count() {
  static std::mutex mu;
  static std::map<int, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
  cache[dev] = sms;
  return sms;
}

// Blocks of the ELL kernels: x over groups; when that leaves the GPU short
// of blocks (a wide B over few groups), y splits the feature passes, up to
// about ten blocks per SM in all.
// (sets p.ell_fc_span to the features of one block row)
static dim3 ell_grid(SpmmArgs& p, int groups_per_block, int pass) {
  const long gx = (p.ell_n_groups + groups_per_block - 1) / groups_per_block;
  const int n_pass = (p.N + pass - 1) / pass;
  const long want = (long)device_sm_count() * 10;
  long gy = gx >= want ? 1 : (want + gx - 1) / gx;
  gy = std::max(1L, std::min<long>(gy, n_pass));
  const int per = (int)((n_pass + gy - 1) / gy);
  gy = (n_pass + per - 1) / per;
  p.ell_fc_span = per * pass;
  return dim3((unsigned)gx, (unsigned)gy, (unsigned)std::max(1, p.heads));
}

template <int LPR>
struct EllLaunch {
  static cudaError_t run(SpmmArgs p, cudaStream_t st) {
    if (p.ell_n_groups == 0) return cudaSuccess;
    const dim3 grid = ell_grid(p, 256 / LPR, 4 * LPR);
    if (grid.z > 1)
      return launch_dependent(spmm_ell_seg_kernel<LPR, 1, false, false, true, true>, grid, dim3(256), 0, st, p);
    if (grid.y > 1)
      return launch_dependent(spmm_ell_seg_kernel<LPR, 1, false, false, true>, grid, dim3(256), 0, st, p);
    return launch_dependent(spmm_ell_seg_kernel<LPR, 1, false, false>, grid, dim3(256), 0, st, p);
  }
};

// Narrow fp32 B (N < 128): LPR-lane sub-groups of 8 features per lane (two
// float4), LPR the power of two covering N, so a 41-wide row takes 6 of 8
// lanes instead of 11 of 16 single-float4 lanes.
template <int LPR>
struct EllNarrowLaunch {
  static cudaError_t run(SpmmArgs p, cudaStream_t st) {
    const dim3 grid = ell_grid(p, 256 / LPR, 8 * LPR);
    const bool full = p.N % (8 * LPR) == 0;
    if (grid.z > 1)
      return full ? launch_dependent(spmm_ell_seg_kernel<LPR, 2, true, false, true, true>, grid, dim3(256), 0, st, p)
                  : launch_dependent(spmm_ell_seg_kernel<LPR, 2, false, false, true, true>, grid, dim3(256), 0, st, p);
    if (grid.y > 1)
      return full ? launch_dependent(spmm_ell_seg_kernel<LPR, 2, true, false, true>, grid, dim3(256), 0, st, p)
                  : launch_dependent(spmm_ell_seg_kernel<LPR, 2, false, false, true>, grid, dim3(256), 0, st, p);
    // (4 entries per batch at 4 blocks per SM measured slower at N = 41,
    // 159 against 154 us on the GCN graph)
    return full ? launch_dependent(spmm_ell_seg_kernel<LPR, 2, true, false>, grid, dim3(256), 0, st, p)
                : launch_dependent(spmm_ell_seg_kernel<LPR, 2, false, false>, grid, dim3(256), 0, st, p);
  }
};

template <int LPR>
struct EllBf16Launch {
  static cudaError_t run(SpmmArgs p, cudaStream_t st) {
    const dim3 grid = ell_grid(p, 256 / LPR, 8 * LPR);
    if (grid.y > 1)
      return launch_dependent(spmm_ell_seg_bf16_kernel<LPR, false, false, true>, grid, dim3(256), 0, st, p);
    return launch_dependent(spmm_ell_seg_bf16_kernel<LPR, false, false>, grid, dim3(256), 0, st, p);
  }
};

static int lpr_for_bf16(int N) {
  const int lanes = (N + 7) / 8;
  if (lanes >= 32) return 32;
  int l = 4;
  while (l < lanes) l <<= 1;
  return l;
}

cudaError_t launch_ell(const SpmmArgs& args, cudaStream_t st) {
  if (args.ell_n_groups == 0) return cudaSuccess;
  SpmmArgs p = args;
  const bool off32 = (long)p.K * p.ldb < (1L << 31);
  if (p.b_bf16) {
    if (p.N % 128 == 0) {
      // 16-lane sub-groups of 8 features per lane (two groups per warp)
      const dim3 grid = ell_grid(p, 16, 128);
      if (grid.y > 1)
      return launch_dependent(spmm_ell_seg_bf16_kernel<16, true, false, true>, grid, dim3(256), 0, st, p);
      else if (off32) return launch_dependent(spmm_ell_seg_bf16_kernel<16, true, true>, grid, dim3(256), 0, st, p);
      return launch_dependent(spmm_ell_seg_bf16_kernel<16, true, false>, grid, dim3(256), 0, st, p);
    }
    return dispatch_lpr<EllBf16Launch>(lpr_for_bf16(p.N), p, st);
  }
  if (p.N % 128 == 0) {
    // 16-lane sub-groups of 8 features per lane (two groups per warp)
    const dim3 grid = ell_grid(p, 16, 128);
    if (grid.z > 1)
      return launch_dependent(spmm_ell_seg_kernel<16, 2, true, false, true, true>, grid, dim3(256), 0, st, p);
    if (grid.y > 1)
      return launch_dependent(spmm_ell_seg_kernel<16, 2, true, false, true>, grid, dim3(256), 0, st, p);
    else if (off32) return launch_dependent(spmm_ell_seg_kernel<16, 2, true, true>, grid, dim3(256), 0, st, p);
    return launch_dependent(spmm_ell_seg_kernel<16, 2, true, false>, grid, dim3(256), 0, st, p);
  }
  if (p.N < 128) {
    int lpr = 4;
    while (lpr < (p.N + 7) / 8) lpr <<= 1;
    return dispatch_lpr<EllNarrowLaunch>(lpr, p, st);
  }
  return dispatch_lpr<EllLaunch>(lpr_for(p.N), p, st);
}

// dvals[t] = <dY[row(t)], B[col(t)]> over the plan's entry list, as runs of
// one row (the row-run SDDMM kernel holds the dY row and gathers B rows)
template <int LPR>
static cudaError_t launch_ell_bwd_t(SpmmArgs p, cudaStream_t st) {
  const long gx = (p.ell_n_groups + (256 / LPR) - 1) / (256 / LPR);
  const dim3 grid((unsigned)gx, 1, 1);
  return p.N == 8 * LPR ? launch_dependent(spmm_ell_bwd_kernel<LPR, true>, grid, dim3(256), 0, st, p)
                        : launch_dependent(spmm_ell_bwd_kernel<LPR, false>, grid, dim3(256), 0, st, p);
}

cudaError_t launch_ell_bwd(const SpmmArgs& p, cudaStream_t st) {
  if (p.ell_n_groups == 0) return cudaSuccess;
  if (p.N > 128 || p.b_bf16 || p.heads > 1) return cudaErrorNotSupported;
  int lpr = 4;
  while (8 * lpr < p.N) lpr <<= 1;
  switch (lpr) {
    case 4: return launch_ell_bwd_t<4>(p, st);
    case 8: return launch_ell_bwd_t<8>(p, st);
    default: return launch_ell_bwd_t<16>(p, st);
  }
}

// Value gradients of the tensor-tile nonzeros on the tensor cores.
//
// A unit is up to 8 k-steps of one chunk (one item): its 128 k-step columns
// (16 per k-step) are the M = 128 rows of the MMA's A operand, the item's 16
// rows its N = 16 B operand, the features its K, so
//   D[16 j + k][r] = <Y[col(j, k)], X[row r]>
// is the gradient of the nonzero (r, k) of k-step j.  The item's 16 X rows
// are gathered once per unit, the columns once per k-step (the row-run
// kernel gathers one row per nonzero: ~41 per k-step on the GCN graph).
// Per 64-feature chunk each of the 16 half-warps (256 threads) issues the
// loads of its 8 columns and 1 item row at once (a float4 a lane, 256
// contiguous bytes a row), then splits every row into hi = bf16(x) and
// lo = bf16(x - hi), and stores both into K-major images with the 128-byte
// swizzle (128-byte rows of 64 features, the 16-byte chunk q of row m at
// q ^ (m % 8), 8-row atoms 1 KB apart), so each half-warp writes one
// 128-byte row: no bank conflicts.  One thread issues hi.hi + hi.lo + lo.hi
// per 16-feature slice (the K advance is 32 bytes inside the atom row) into
// a 16-column TMEM accumulator; the epilogue reads lane m = 16 j + k and
// writes the live entries through the k-step's id table.  The wait for the
// MMAs is bounded; a wait that runs out sets the error flag and ends the
// kernel's work.
constexpr uint32_t kDvYImg = 16384;  // 128 rows x 64 bf16
constexpr uint32_t kDvXImg = 2048;   // 16 rows x 64 bf16
constexpr uint32_t kDvBytes = 1024 + 2 * kDvYImg + 2 * kDvXImg + 64 + 64;

__device__ __forceinline__ uint32_t sw128_off(int row, int q) {
  return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((q ^ (row & 7)) << 4));
}

constexpr int kDvThreads = 256;

__global__ void __launch_bounds__(kDvThreads, 3) spmm_tc_dvals_kernel(SpmmArgs p, const float* __restrict__ X, long ldx,
                                                              const float* __restrict__ Y, long ldy,
                                                              float* __restrict__ out, int F) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const uint32_t yhi = base, ylo = base + kDvYImg, xhi = base + 2 * kDvYImg, xlo = xhi + kDvXImg;
  const uint32_t orow_s = xlo + kDvXImg, bar = orow_s + 64, tmem_slot = bar + 8;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, hw = lane >> 4, sl = lane & 15;
  griddep_wait();  // X and Y may come from the previous kernel
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
  // kind::f16, bf16 x bf16, M = 128, N = 16, both operands K-major
  constexpr uint32_t idesc = make_idesc(1, 1, 0, 0, 128, 16);
  uint32_t phase = 0;
  bool ok = true;
  // one float4 of a gathered row -> hi and lo bf16 halves of its 16-byte chunk
  auto put = [&](uint32_t hi_img, uint32_t lo_img, int row, float4 v) {
    const uint32_t o = sw128_off(row, sl >> 1) + (sl & 1) * 8;
    const uint32_t h01 = pack_bf16x2(v.x, v.y), h23 = pack_bf16x2(v.z, v.w);
    st_shared_v2(hi_img + o, h01, h23);
    st_shared_v2(lo_img + o, pack_bf16x2(v.x - __uint_as_float(h01 << 16), v.y - __uint_as_float(h01 & 0xffff0000u)),
                 pack_bf16x2(v.z - __uint_as_float(h23 << 16), v.w - __uint_as_float(h23 & 0xffff0000u)));
  };
#pragma unroll 1
  for (int u = blockIdx.x; u < p.tcdv_n_units && ok; u += gridDim.x) {
    const int ks0 = __ldg(p.tcdv_unit_ks + u);
    const int meta = __ldg(p.tcdv_unit_meta + u);
    const int item = meta >> 3, nks = (meta & 7) + 1;
    // this half-warp (hg = 0..15) gathers columns m = 16 i + hg (i < 8) and
    // item row hg
    const int hg = 2 * warp + hw;
    int ycol[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int m = 16 * i + hg, j = m >> 4;
      ycol[i] = j < nks ? __ldg(p.tc_cols + (long)(ks0 + j) * 16 + (m & 15)) : -1;
    }
    const int xrow = __ldg(p.tc_out_rows + (long)item * 16 + hg);
    if (sl == 0) asm volatile("st.shared.b32 [%0], %1;" ::"r"(orow_s + 4 * hg), "r"(xrow) : "memory");
#pragma unroll 1
    for (int fc = 0; fc < F; fc += 64) {
      const int f = fc + 4 * sl;
      // every load of the chunk in flight at once, then the conversions
      float4 v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i)
        v[i] = ycol[i] >= 0 ? ld4_live(Y + (long)ycol[i] * ldy, f, F) : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 xv = xrow >= 0 ? ld4_live(X + (long)xrow * ldx, f, F) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int i = 0; i < 8; ++i) put(yhi, ylo, 16 * i + hg, v[i]);
      put(xhi, xlo, hg, xv);
      fence_proxy_async_smem();
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      if (tid == 0) {
        const int ns = min(4, (F - fc + 15) / 16);
        for (int s = 0; s < ns; ++s) {
          const uint64_t ah = smem_desc(yhi + 32 * s, 16, 1024, kSwizzle128B);
          const uint64_t bh = smem_desc(xhi + 32 * s, 16, 1024, kSwizzle128B);
          umma_f16(tmem, ah, bh, idesc, (fc > 0 || s > 0) ? 1u : 0u);
          umma_f16(tmem, ah, smem_desc(xlo + 32 * s, 16, 1024, kSwizzle128B), idesc, 1u);
          umma_f16(tmem, smem_desc(ylo + 32 * s, 16, 1024, kSwizzle128B), bh, idesc, 1u);
        }
        umma_commit(bar);
      }
      // the MMAs read the images: nobody rewrites them, or reads TMEM, first
      const bool done = __syncthreads_and(tid == 0 ? mbar_wait_bounded(bar, phase) : true) != 0;
      phase ^= 1u;
      if (!done) {
        ok = false;
        break;
      }
      if (tid != 0) mbar_wait_bounded(bar, phase ^ 1u);  // completed: returns at once
      tc_fence_after();
    }
    if (!ok) break;
    // epilogue (warps 0-3): warp w holds TMEM lanes m = 32 w .. 32 w + 31
    // (k-steps 2 w and 2 w + 1), columns r = 0..15
    const int m = 32 * warp + lane, j = m >> 4, k = m & 15;
    uint32_t v[16];
    if (warp < 4) {
      tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16), v);
      tmem_wait_ld();
    }
    if (warp < 4 && j < nks) {
      const int* ids = p.tcdv_id + (long)(ks0 + j) * 256 + k;
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        int orow;
        asm volatile("ld.shared.b32 %0, [%1];" : "=r"(orow) : "r"(orow_s + 4 * r) : "memory");
        const int id = __ldcs(ids + 16 * r);
        if (id >= 0 && orow >= 0) __stcs(out + id, __uint_as_float(v[r]));
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  if (!ok && tid == 0 && p.err_flag) atomicOr(p.err_flag, 1);
  // every MMA this CTA issued has completed before TMEM is freed
  if (!ok && tid == 0) mbar_wait_bounded(bar, phase ^ 1u);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, 32);
}

cudaError_t launch_tc_dvals(const SpmmArgs& p, const float* X, long ldx, const float* Y, long ldy, float* out, int F,
                            cudaStream_t st) {
  if (p.tcdv_n_units == 0) return cudaSuccess;
  if (!p.tcdv_id) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(spmm_tc_dvals_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kDvBytes);
  if (e != cudaSuccess) return e;
  // 37 KB of shared memory, 256 threads at 80 registers and 32 TMEM columns
  // per CTA: 3 CTAs per SM
  const int grid = std::min(p.tcdv_n_units, device_sm_count() * 3);
  return launch_dependent(spmm_tc_dvals_kernel, dim3((unsigned)grid), dim3(kDvThreads), kDvBytes, st, p, X, ldx, Y,
                          ldy, out, F);
}

cudaError_t launch_dvals(const SpmmArgs& p, const float* dY, long lddy, float* dvals, cudaStream_t st) {
  return launch_sddmm_runs(p.dv_n_groups, p.dv_gptr, p.dv_grow, p.dv_col, p.dv_id, dY, false, lddy, p.B,
                           p.b_bf16 != 0, p.ldb, dvals, p.N, st);
}

}  // namespace stile
