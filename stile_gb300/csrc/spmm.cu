// SpMM kernels for sm_103a.
//
//  * csr_spmm_kernel     plain CSR-row SpMM (the comparator)
//  * zero_rows_kernel    zeroes output rows that no owned tile stores
//  * spmm_fused_kernel   one launch for every tile of a plan: the first
//                        tc_ctas CTAs run dense 16-row block tiles on the
//                        tensor cores (tcgen05.mma, accumulator in TMEM), the
//                        rest run ELL row-bucket tiles on CUDA cores.  This is
//                        the reference's horizontally fused kernel
//                        (my_fuse_formats.py:2437, blockIdx-range dispatch).
//  * spmm_dvals_kernel   value gradient <dY[row], B[col]> for every nonzero,
//                        walking the same tiles.
#include "common.cuh"
#include "spmm.cuh"

namespace stile {

// ===========================================================================
// plain CSR-row kernel
// ===========================================================================
// LPR lanes per row (each lane owns 4 consecutive features per chunk); a warp
// handles 32/LPR rows at once.  Column indices / values of a row are loaded
// cooperatively 32 at a time and broadcast with shuffles.
template <int LPR>
__global__ void __launch_bounds__(256) csr_spmm_kernel(int M, const int* __restrict__ indptr,
                                                       const int* __restrict__ indices,
                                                       const float* __restrict__ vals,
                                                       const float* __restrict__ B, long ldb,
                                                       float* __restrict__ C, long ldc, int N) {
  constexpr int RPW = kWarp / LPR;
  const int lane = threadIdx.x & 31;
  const int sub = lane / LPR;
  const int sl = lane % LPR;
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int row = warp_global * RPW + sub;
  const bool valid = row < M;
  const int beg = valid ? indptr[row] : 0;
  const int end = valid ? indptr[row + 1] : 0;
  const unsigned gmask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << (sub * LPR));
  for (int fc = 0; fc < N; fc += 4 * LPR) {
    const int f = fc + 4 * sl;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int base = beg; base < end; base += LPR) {
      const int my = base + sl;
      const int mcol = (my < end) ? indices[my] : 0;
      const float mval = (my < end) ? vals[my] : 0.f;
      const int cnt = min(LPR, end - base);
      int j = 0;
      for (; j + 4 <= cnt; j += 4) {
        const int c0 = __shfl_sync(gmask, mcol, sub * LPR + j);
        const int c1 = __shfl_sync(gmask, mcol, sub * LPR + j + 1);
        const int c2 = __shfl_sync(gmask, mcol, sub * LPR + j + 2);
        const int c3 = __shfl_sync(gmask, mcol, sub * LPR + j + 3);
        const float v0 = __shfl_sync(gmask, mval, sub * LPR + j);
        const float v1 = __shfl_sync(gmask, mval, sub * LPR + j + 1);
        const float v2 = __shfl_sync(gmask, mval, sub * LPR + j + 2);
        const float v3 = __shfl_sync(gmask, mval, sub * LPR + j + 3);
        const float4 b0 = ld_row4(B + (long)c0 * ldb, f, N);
        const float4 b1 = ld_row4(B + (long)c1 * ldb, f, N);
        const float4 b2 = ld_row4(B + (long)c2 * ldb, f, N);
        const float4 b3 = ld_row4(B + (long)c3 * ldb, f, N);
        fma4(acc, v0, b0);
        fma4(acc, v1, b1);
        fma4(acc, v2, b2);
        fma4(acc, v3, b3);
      }
      for (; j < cnt; ++j) {
        const int c = __shfl_sync(gmask, mcol, sub * LPR + j);
        const float v = __shfl_sync(gmask, mval, sub * LPR + j);
        fma4(acc, v, ld_row4(B + (long)c * ldb, f, N));
      }
    }
    if (valid) st_row4(C + (long)row * ldc, f, N, acc);
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
// fused hybrid kernel
// ===========================================================================
// Tensor-core item layout in shared memory (per pipeline stage):
//   A operand: gathered B rows, transposed -> [128 features (M) x 16 k (K)],
//              MN-major, 128-byte swizzle: two 64-feature atoms (LBO 2048 B),
//              two 8-row k groups (SBO 1024 B).
//   B operand: the 16x16 block values (N = 16 tile rows x K = 16), K-major,
//              no swizzle: core matrices 8 rows x 16 B, LBO 128 B (k
//              direction), SBO 256 B (row direction); copied verbatim from
//              the plan (the host writes this image).
constexpr uint32_t kAStage = 4096;   // bytes of one A image
constexpr uint32_t kBStage = 512;    // bytes of one B image (16-bit)
constexpr uint32_t kALbo = 2048, kASbo = 1024;
constexpr uint32_t kBLbo = 128, kBSbo = 256;
constexpr int kTcThreads = 128;

__device__ __forceinline__ uint32_t a_img_off(int m, int k) {
  // m: feature (0..127), k: column within the k-step (0..15)
  const int atom = m >> 6, grp = k >> 3, r = k & 7, chunk = (m & 63) >> 3;
  return (uint32_t)(atom * kALbo + grp * kASbo + r * 128 + ((chunk ^ r) << 4) + (m & 7) * 2);
}

struct TcSmem {
  uint32_t a[2][2];   // [stage][hi/lo] A image addresses
  uint32_t b[2];      // [stage] B image(s) address
  uint32_t bar[3];    // stage 0, stage 1, final
  uint32_t tmem_slot;
};

template <int MODE>
__device__ void tc_item(const SpmmArgs& p, int cta, uint8_t* smem_raw) {
  constexpr bool kSplit = (MODE == STILE_TC_SPLIT_BF16);
  constexpr uint32_t kBBytes = kSplit ? 2 * kBStage : kBStage;
  const int item = cta / p.n_fchunks;
  const int f0 = (cta % p.n_fchunks) * 128;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // carve shared memory (1024-byte aligned for the 128B swizzle atoms)
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  TcSmem s;
  uint32_t off = base;
  for (int st = 0; st < 2; ++st) {
    s.a[st][0] = off; off += kAStage;
    s.a[st][1] = off; if (kSplit) off += kAStage;
  }
  for (int st = 0; st < 2; ++st) { s.b[st] = off; off += kBBytes; }
  s.bar[0] = off; s.bar[1] = off + 8; s.bar[2] = off + 16;
  s.tmem_slot = off + 24;

  if (tid == 0) {
    mbar_init(s.bar[0], 1);
    mbar_init(s.bar[1], 1);
    mbar_init(s.bar[2], 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(s.tmem_slot, 32);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  uint32_t tmem;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(tmem) : "r"(s.tmem_slot) : "memory");

  const int kb = p.tc_item_kbeg[item];
  const int ke = p.tc_item_kbeg[item + 1];
  const int N = p.N;
  const uint32_t idesc = (MODE == STILE_TC_F16) ? make_idesc(0, 0, 1, 0, 128, 16)
                                                : make_idesc(1, 1, 1, 0, 128, 16);
  uint32_t parity[2] = {0u, 0u};
  uint32_t drain_parity = 0u;
  bool ok = true;
  const uint8_t* vals = reinterpret_cast<const uint8_t*>(p.tc_vals);
  // The accumulator is drained into fp32 registers every kGroup k-steps and
  // the MMA chain restarts, which bounds how many partial sums the tensor
  // core accumulates in a row (long rows otherwise drift in split mode).
  constexpr int kGroup = kSplit ? 4 : 16;
  float acc[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) acc[i] = 0.f;
  const uint32_t my_lanes = tmem + ((uint32_t)(32 * warp) << 16);

  for (int ks = kb; ks < ke; ++ks) {
    const int step = ks - kb;
    const int st = step & 1;
    bool free_ok = true;
    if (step >= 2) {
      // the MMA that read this stage two steps ago must be finished
      free_ok = mbar_wait_bounded(s.bar[st], parity[st]);
      parity[st] ^= 1u;
    }
    if (free_ok) {
      // gather 16 rows of B (this k-step's columns) for features [f0, f0+128)
      // warp w handles columns 4w..4w+3, lane l handles features 4l..4l+3
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int kk = warp * 4 + r;
        const int col = p.tc_cols[(long)ks * 16 + kk];
        const int f = f0 + 4 * lane;
        const float4 v = ld_row4(p.B + (long)col * p.ldb, f, N);
        const uint32_t o = a_img_off(4 * lane, kk);
        if (MODE == STILE_TC_F16) {
          st_shared_v2(s.a[st][0] + o, pack_f16x2(v.x, v.y), pack_f16x2(v.z, v.w));
        } else {
          const uint32_t h0 = pack_bf16x2(v.x, v.y), h1 = pack_bf16x2(v.z, v.w);
          st_shared_v2(s.a[st][0] + o, h0, h1);
          if (kSplit) {
            const __nv_bfloat162 b0 = *reinterpret_cast<const __nv_bfloat162*>(&h0);
            const __nv_bfloat162 b1 = *reinterpret_cast<const __nv_bfloat162*>(&h1);
            const float2 r0 = __bfloat1622float2(b0), r1 = __bfloat1622float2(b1);
            st_shared_v2(s.a[st][1] + o, pack_bf16x2(v.x - r0.x, v.y - r0.y),
                         pack_bf16x2(v.z - r1.x, v.w - r1.y));
          }
        }
      }
      // block values: verbatim copy of the operand image(s)
      const uint4* src = reinterpret_cast<const uint4*>(vals + (long)ks * kBBytes);
      for (int i = tid; i < (int)(kBBytes / 16); i += kTcThreads) st_shared_v4(s.b[st] + 16 * i, src[i]);
    }
    fence_proxy_async_smem();
    // uniform decision: every thread saw its stage free
    ok = __syncthreads_and(free_ok && ok) != 0;
    if (!ok) break;
    const bool group_start = (step % kGroup) == 0;
    const bool group_end = ((step % kGroup) == kGroup - 1) || (ks == ke - 1);
    if (tid == 0) {
      tc_fence_after();
      const uint64_t ad = smem_desc(s.a[st][0], kALbo, kASbo, kSwizzle128B);
      const uint64_t bd = smem_desc(s.b[st], kBLbo, kBSbo, kSwizzleNone);
      umma_f16(tmem, ad, bd, idesc, group_start ? 0u : 1u);
      if (kSplit) {
        const uint64_t bd_lo = smem_desc(s.b[st] + kBStage, kBLbo, kBSbo, kSwizzleNone);
        const uint64_t ad_lo = smem_desc(s.a[st][1], kALbo, kASbo, kSwizzle128B);
        umma_f16(tmem, ad, bd_lo, idesc, 1u);
        umma_f16(tmem, ad_lo, bd, idesc, 1u);
        umma_f16(tmem, ad_lo, bd_lo, idesc, 1u);
      }
      umma_commit(s.bar[st]);
      if (group_end) umma_commit(s.bar[2]);
    }
    if (group_end) {
      // drain: wait for the group's MMAs, add the partial sums in fp32
      const bool done = __syncthreads_and(mbar_wait_bounded(s.bar[2], drain_parity)) != 0;
      drain_parity ^= 1u;
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
      // every warp has read the accumulator before the next group resets it
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
    }
  }
  if (!ok && tid == 0) atomicOr(p.err_flag, 1);

  // epilogue: warp w owns features f0+32w+lane, 16 tile rows in registers
  const bool have = (ke > kb) && ok;
  const int f = f0 + 32 * warp + lane;
  const bool atomic = (p.tc_item_flags[item] & 1) != 0;
  if (f < N && have) {
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

// ELL tile: 4 warps; LPR lanes per row own 4 features each, rows of the tile
// are distributed round-robin over the 32/LPR row slots of every warp.
template <int LPR>
__device__ void ell_item(const SpmmArgs& p, int item) {
  constexpr int RPW = kWarp / LPR;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int sub = lane / LPR, sl = lane % LPR;
  const int row0 = p.ell_item_row0[item];
  const int nrows = p.ell_item_row0[item + 1] - row0;
  const int K = p.ell_item_K[item];
  const long slot0 = p.ell_item_slot0[item];
  const bool atomic = (p.ell_item_flags[item] & 1) != 0;
  const int N = p.N;
  for (int r = warp * RPW + sub; r < nrows; r += (kTcThreads / kWarp) * RPW) {
    const int gr = row0 + r;
    const int orow = p.ell_out_row[gr];
    if (orow < 0) continue;
    const int len = p.ell_row_len[gr];
    const float* vr = p.ell_vals + slot0 + (long)r * K;
    const int* kr = p.ell_kidx + slot0 + (long)r * K;
    float* crow = p.C + (long)orow * p.ldc;
    for (int fc = 0; fc < N; fc += 4 * LPR) {
      const int f = fc + 4 * sl;
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      int k = 0;
      for (; k + 4 <= len; k += 4) {
        const int c0 = __ldg(kr + k), c1 = __ldg(kr + k + 1), c2 = __ldg(kr + k + 2),
                  c3 = __ldg(kr + k + 3);
        const float v0 = __ldg(vr + k), v1 = __ldg(vr + k + 1), v2 = __ldg(vr + k + 2),
                    v3 = __ldg(vr + k + 3);
        const float4 b0 = ld_row4(p.B + (long)c0 * p.ldb, f, N);
        const float4 b1 = ld_row4(p.B + (long)c1 * p.ldb, f, N);
        const float4 b2 = ld_row4(p.B + (long)c2 * p.ldb, f, N);
        const float4 b3 = ld_row4(p.B + (long)c3 * p.ldb, f, N);
        fma4(acc, v0, b0);
        fma4(acc, v1, b1);
        fma4(acc, v2, b2);
        fma4(acc, v3, b3);
      }
      for (; k < len; ++k) fma4(acc, __ldg(vr + k), ld_row4(p.B + (long)__ldg(kr + k) * p.ldb, f, N));
      if (atomic) red_row4(crow, f, N, acc); else st_row4(crow, f, N, acc);
    }
  }
}

template <int MODE, int LPR>
__global__ void __launch_bounds__(kTcThreads) spmm_fused_kernel(SpmmArgs p) {
  extern __shared__ uint8_t smem_raw[];
  const int cta = blockIdx.x;
  if (cta < p.tc_ctas) {
    tc_item<MODE>(p, cta, smem_raw);
  } else {
    ell_item<LPR>(p, cta - p.tc_ctas);
  }
}

// ===========================================================================
// value gradient: dvals[t] = <dY[row(t)], B[col(t)]>
// ===========================================================================
// One CTA (4 warps) per ELL item or per TC k-step.  An LPR-lane group computes
// one dot product, reducing over the features with shuffles.
template <int LPR>
__device__ __forceinline__ float group_dot(const float* a, const float* b, int N, int sl,
                                           unsigned gmask) {
  float s = 0.f;
  for (int f = 4 * sl; f < N; f += 4 * LPR) s += dot4(ld_row4(a, f, N), ld_row4(b, f, N));
#pragma unroll
  for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(gmask, s, o);
  return s;
}

template <int LPR>
__global__ void __launch_bounds__(128) spmm_dvals_kernel(SpmmArgs p, const float* __restrict__ dY,
                                                         long lddy, float* __restrict__ dvals) {
  constexpr int RPW = kWarp / LPR;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int sub = lane / LPR, sl = lane % LPR;
  const unsigned gmask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << (sub * LPR));
  const int N = p.N;
  const int cta = blockIdx.x;
  const int groups = 4 * RPW;
  const int g = warp * RPW + sub;
  if (cta < p.tc_n_ksteps) {
    // TC k-step: 16 rows x 16 columns, entries with a nonzero id
    const int ks = cta;
    // which item owns this k-step: binary search in tc_item_kbeg
    int lo = 0, hi = p.tc_n_items;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (p.tc_item_kbeg[mid] <= ks) lo = mid; else hi = mid;
    }
    const int item = lo;
    for (int e = g; e < 256; e += groups) {
      const int id = p.tc_nnz_id[(long)ks * 256 + e];  // uniform within the group
      if (id < 0) continue;
      const int n = e >> 4, k = e & 15;
      const int row = p.tc_out_rows[(long)item * 16 + n];
      const int col = p.tc_cols[(long)ks * 16 + k];
      const float d = group_dot<LPR>(dY + (long)row * lddy, p.B + (long)col * p.ldb, N, sl, gmask);
      if (sl == 0) dvals[id] = d;
    }
  } else {
    const int item = cta - p.tc_n_ksteps;
    const int row0 = p.ell_item_row0[item];
    const int nrows = p.ell_item_row0[item + 1] - row0;
    const int K = p.ell_item_K[item];
    const long slot0 = p.ell_item_slot0[item];
    const int total = nrows * K;
    for (int e = g; e < total; e += groups) {
      const int r = e / K, k = e - r * K;
      const int gr = row0 + r;
      const int orow = p.ell_out_row[gr];
      if (orow < 0 || k >= p.ell_row_len[gr]) continue;
      const long s = slot0 + (long)r * K + k;
      const int id = p.ell_nnz_id[s];
      if (id < 0) continue;
      const float d =
          group_dot<LPR>(dY + (long)orow * lddy, p.B + (long)p.ell_kidx[s] * p.ldb, N, sl, gmask);
      if (sl == 0) dvals[id] = d;
    }
  }
}

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
  static cudaError_t run(int M, const int* indptr, const int* indices, const float* vals,
                         const float* B, long ldb, float* C, long ldc, int N, cudaStream_t st) {
    constexpr int RPW = kWarp / LPR;
    const int rows_per_cta = 8 * RPW;
    const int grid = (M + rows_per_cta - 1) / rows_per_cta;
    if (grid == 0) return cudaSuccess;
    csr_spmm_kernel<LPR><<<grid, 256, 0, st>>>(M, indptr, indices, vals, B, ldb, C, ldc, N);
    return cudaGetLastError();
  }
};

cudaError_t launch_csr_spmm(int M, const int* indptr, const int* indices, const float* vals,
                            const float* B, long ldb, float* C, long ldc, int N, cudaStream_t st) {
  return dispatch_lpr<CsrLaunch>(lpr_for(N), M, indptr, indices, vals, B, ldb, C, ldc, N, st);
}

cudaError_t launch_zero_rows(const int* rows, int n, float* C, long ldc, int N, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int grid = (n + 7) / 8;
  zero_rows_kernel<<<grid, 256, 0, st>>>(rows, n, C, ldc, N);
  return cudaGetLastError();
}

size_t fused_smem_bytes(int mode) {
  const bool split = mode == STILE_TC_SPLIT_BF16;
  const size_t a = 2 * (split ? 2 : 1) * kAStage;
  const size_t b = 2 * (split ? 2 : 1) * kBStage;
  return 1024 + a + b + 64;
}

template <int MODE, int LPR>
static cudaError_t launch_fused_t(const SpmmArgs& p, cudaStream_t st) {
  const size_t smem = fused_smem_bytes(MODE);
  auto k = spmm_fused_kernel<MODE, LPR>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int grid = p.tc_ctas + p.ell_n_items;
  if (grid == 0) return cudaSuccess;
  k<<<grid, kTcThreads, smem, st>>>(p);
  return cudaGetLastError();
}

template <int LPR>
struct FusedLaunch {
  static cudaError_t run(int mode, const SpmmArgs& p, cudaStream_t st) {
    switch (mode) {
      case STILE_TC_F16: return launch_fused_t<STILE_TC_F16, LPR>(p, st);
      case STILE_TC_SPLIT_BF16: return launch_fused_t<STILE_TC_SPLIT_BF16, LPR>(p, st);
      default: return launch_fused_t<STILE_TC_BF16, LPR>(p, st);
    }
  }
};

cudaError_t launch_fused(const SpmmArgs& p, cudaStream_t st) {
  return dispatch_lpr<FusedLaunch>(lpr_for(p.N), p.tc_mode, p, st);
}

template <int LPR>
struct DvalsLaunch {
  static cudaError_t run(const SpmmArgs& p, const float* dY, long lddy, float* dvals,
                         cudaStream_t st) {
    const int grid = p.tc_n_ksteps + p.ell_n_items;
    if (grid == 0) return cudaSuccess;
    spmm_dvals_kernel<LPR><<<grid, 128, 0, st>>>(p, dY, lddy, dvals);
    return cudaGetLastError();
  }
};

cudaError_t launch_dvals(const SpmmArgs& p, const float* dY, long lddy, float* dvals,
                         cudaStream_t st) {
  return dispatch_lpr<DvalsLaunch>(lpr_for(p.N), p, dY, lddy, dvals, st);
}

}  // namespace stile
