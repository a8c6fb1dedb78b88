// SDDMM kernels for sm_103a: out[t] = <X[row(t)], Y[col(t)]> on a mask.
//
//  * 1D tiles (the reference's "1D_sddmm", my_fuse_formats.py:2263-2317):
//    the entry-list kernel below over (mid_idx, j_idx, remap); results go
//    straight to their CSR position -- the reference writes a tile-ordered
//    buffer and reorders on the host (order_output_BSDDMM, :4247-4288).
//  * block tiles (the reference's "TC_sddmm", :2324-2415, whose kernel runs
//    each 16x16 block as a wmma product, my_wmmas1.py:422-466): tcgen05.mma
//    over units of 8 blocks, below; only the live entries of a block
//    (indicesDense) are written.
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "spmm.cuh"

namespace stile {

// Entry-list SDDMM: out[outs[t]] = <X[rows[t]], Y[cols[t]]>.  An LPR-lane
// group takes V consecutive entries per iteration: lanes 0..V-1 load the
// entries' (row, column, output) and broadcast them by shuffle where used;
// the Y rows are gathered 4 at a time (128-bit per lane) and an X row is
// gathered only where the row changes from the previous entry (lists
// grouped by row, as both callers' are, read each X row about once per
// run).  The V dot products are reduced together with a transposing
// butterfly: each halving step sends half of the partial sums across and
// keeps the other half, so after log2(V) steps every lane holds one entry's
// partial sum (8 dots cost 9 shuffles instead of 40).
constexpr int kSddmmV = 8;           // entries per group iteration
constexpr int kSddmmBlocks = 4;      // resident 256-thread blocks per SM (register budget)

// kVec: F % 4 == 0, so a lane's float4 of features is all in range or all
// out.  VEC float4 per lane: with VEC = 2 (16-lane groups for F >= 128) two
// groups share every warp-wide shuffle, halving the instructions per byte.
//
// kXb / kYb: X / Y hold bf16 (8 features per 16-byte load, converted to
// fp32; VEC = 2 so that a lane covers the 8 features of one load).
template <int VEC, bool kVec, bool kB16>
__device__ __forceinline__ void load_feats(const void* row, int f, int F, float4 (&o)[VEC]) {
  if constexpr (kB16) {
    static_assert(VEC == 2, "a bf16 load covers 8 features");
    bf16x8_to_f32(ld_row8_bf16(static_cast<const uint16_t*>(row), f, F), o[0], o[1]);
  } else {
    const float* r = static_cast<const float*>(row);
#pragma unroll
    for (int w = 0; w < VEC; ++w) {
      const int fw = f + 4 * w;
      if (kVec) o[w] = fw < F ? ldg4(r + fw) : make_float4(0.f, 0.f, 0.f, 0.f);
      else o[w] = ld_row4(r, fw, F);
    }
  }
}

template <int LPR, int V, bool kVec, int VEC = 1, bool kXb = false, bool kYb = false>
__global__ void __launch_bounds__(256, kSddmmBlocks) sddmm_list_kernel(long n, const int* __restrict__ rows,
                                                                     const int* __restrict__ cols,
                                                                     const int* __restrict__ outs,
                                                                     const void* __restrict__ Xv, long ldx,
                                                                     const void* __restrict__ Yv, long ldy,
                                                                     float* __restrict__ out, int F) {
  static_assert(V % 4 == 0, "entries are gathered 4 at a time");
  static_assert(VEC == 1 || kVec || kXb || kYb, "wide fp32 lanes need F % 4 == 0");
  // launched dependent on the previous kernel: wait for its results (X or Y
  // may be one of them), then let the next dependent kernel launch
  griddep_wait();
  griddep_launch_dependents();
  using TX = typename std::conditional<kXb, uint16_t, float>::type;
  using TY = typename std::conditional<kYb, uint16_t, float>::type;
  const TX* __restrict__ X = static_cast<const TX*>(Xv);
  const TY* __restrict__ Y = static_cast<const TY*>(Yv);
  constexpr int kPh = 4 / VEC;  // entries per gather phase: 8 float4 loads in flight per lane
  constexpr int GPB = 256 / LPR;
  const int lane = threadIdx.x & 31;
  const int sub = lane / LPR, sl = lane % LPR;
  const unsigned gmask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << (sub * LPR));
  const long g = (long)blockIdx.x * GPB + threadIdx.x / LPR;
  const long stride = (long)gridDim.x * GPB;
  for (long base = g * V; base < n; base += stride * V) {
    const int cnt = (int)min((long)V, n - base);
    // groups of >= V lanes: lanes 0..V-1 load one entry each; smaller
    // groups load every entry
    int rl = 0, cl = 0, ol = 0;
    if (LPR >= V) {
      const bool mine = sl < V && sl < cnt;
      rl = mine ? __ldg(rows + base + sl) : 0;
      cl = mine ? __ldg(cols + base + sl) : 0;
      ol = mine ? __ldg(outs + base + sl) : 0;
    }
    auto row_of = [&](int v) {
      return LPR >= V ? __shfl_sync(gmask, rl, v, LPR) : (v < cnt ? __ldg(rows + base + v) : 0);
    };
    auto col_of = [&](int v) {
      return LPR >= V ? __shfl_sync(gmask, cl, v, LPR) : (v < cnt ? __ldg(cols + base + v) : 0);
    };
    float a[V];
#pragma unroll
    for (int v = 0; v < V; ++v) a[v] = 0.f;
    for (int fc = 0; fc < F; fc += 4 * VEC * LPR) {
      const int f = fc + 4 * VEC * sl;
      // phases of kPh entries; xlast carries the previous phase's last X row
      float4 xlast[VEC];
#pragma unroll
      for (int w = 0; w < VEC; ++w) xlast[w] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int h = 0; h < V; h += kPh) {
        float4 xv[kPh][VEC], yv[kPh][VEC];
#pragma unroll
        for (int v = 0; v < kPh; ++v)
          load_feats<VEC, kVec, kYb>(Y + (long)col_of(h + v) * ldy, f, F, yv[v]);
        // X rows: a gather only where the row changes (entry 0 always loads)
#pragma unroll
        for (int v = 0; v < kPh; ++v) {
          const int i = h + v;
          const int ri = row_of(i);
          const bool same = i > 0 && ri == row_of(i > 0 ? i - 1 : 0);
          if (!same) {
            load_feats<VEC, kVec, kXb>(X + (long)ri * ldx, f, F, xv[v]);
          } else {
#pragma unroll
            for (int w = 0; w < VEC; ++w) xv[v][w] = v > 0 ? xv[v > 0 ? v - 1 : 0][w] : xlast[w];
          }
        }
#pragma unroll
        for (int v = 0; v < kPh; ++v) {
#pragma unroll
          for (int w = 0; w < VEC; ++w) a[h + v] += dot4(xv[v][w], yv[v][w]);
        }
#pragma unroll
        for (int w = 0; w < VEC; ++w) xlast[w] = xv[kPh - 1][w];
      }
    }
    if (LPR >= V) {
      // transposing butterfly: entry e ends in the lanes whose bits at the
      // halving strides spell e
      int e = 0;
#pragma unroll
      for (int m = V, hw = LPR / 2; m > 1; m >>= 1, hw >>= 1) {
        const bool up = (sl & hw) != 0;
#pragma unroll
        for (int i = 0; i < m / 2; ++i) {
          const float send = up ? a[i] : a[i + m / 2];
          const float keep = up ? a[i + m / 2] : a[i];
          a[i] = keep + __shfl_xor_sync(gmask, send, hw);
        }
        if (up) e += m / 2;
      }
#pragma unroll
      for (int o = LPR / (2 * V); o > 0; o >>= 1) a[0] += __shfl_xor_sync(gmask, a[0], o);
      const int oe = __shfl_sync(gmask, ol, e, LPR);
      if ((sl & (LPR / V - 1)) == 0 && e < cnt) out[oe] = a[0];
    } else {
#pragma unroll
      for (int v = 0; v < V; ++v) {
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1) a[v] += __shfl_xor_sync(gmask, a[v], o);
      }
      if (sl == 0) {
#pragma unroll
        for (int v = 0; v < V; ++v)
          if (v < cnt) out[__ldg(outs + base + v)] = a[v];
      }
    }
  }
}

static int lpr_for_f(int F) {
  const int lanes = (F + 3) / 4;
  if (lanes >= 32) return 32;
  int l = 1;
  while (l < lanes) l <<= 1;
  return l < 4 ? 4 : l;
}

static int lpr_for_f8(int F) {
  const int lanes = (F + 7) / 8;
  if (lanes >= 32) return 32;
  int l = 4;
  while (l < lanes) l <<= 1;
  return l;
}

template <bool kXb, bool kYb>
static cudaError_t launch_list_b16(long n, const int* rows, const int* cols, const int* outs, const void* X,
                                   long ldx, const void* Y, long ldy, float* out, int F, cudaStream_t st) {
  // 8 features per lane (one bf16 load, two float4 of an fp32 operand)
  const int lpr = F % 128 == 0 ? 16 : lpr_for_f8(F);
  const long groups = (n + kSddmmV - 1) / kSddmmV;
  long grid = (groups + (256 / lpr) - 1) / (256 / lpr);
  const long cap = (long)device_sm_count() * 32;  // persistent-style cap: 32 blocks per SM
  if (grid > cap) grid = cap;
#define STILE_SDDMM_B16(L)                                                                                      \
  launch_dependent(sddmm_list_kernel<L, kSddmmV, false, 2, kXb, kYb>, dim3((unsigned)grid), dim3(256), 0, st, n, \
                   rows, cols, outs, X, ldx, Y, ldy, out, F)
  cudaError_t e;
  switch (lpr) {
    case 4: e = STILE_SDDMM_B16(4); break;
    case 8: e = STILE_SDDMM_B16(8); break;
    case 16: e = STILE_SDDMM_B16(16); break;
    default: e = STILE_SDDMM_B16(32); break;
  }
#undef STILE_SDDMM_B16
  return e;
}

cudaError_t launch_sddmm_list(long n, const int* rows, const int* cols, const int* outs, const void* X, bool x_bf16,
                              long ldx, const void* Y, bool y_bf16, long ldy, float* out, int F, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (x_bf16 && y_bf16) return launch_list_b16<true, true>(n, rows, cols, outs, X, ldx, Y, ldy, out, F, st);
  if (y_bf16) return launch_list_b16<false, true>(n, rows, cols, outs, X, ldx, Y, ldy, out, F, st);
  if (x_bf16) return cudaErrorNotSupported;  // no caller has a bf16 X with an fp32 Y
  const int lpr = lpr_for_f(F);
  const int gpb = 256 / lpr;
  long groups = (n + kSddmmV - 1) / kSddmmV;
  long grid = (groups + gpb - 1) / gpb;
  const long cap = (long)device_sm_count() * 32;  // persistent-style cap: 32 blocks per SM
  if (grid > cap) grid = cap;
  if (F % 128 == 0) {
    // 16-lane groups of 8 features per lane (two groups per warp)
    long groups2 = (n + kSddmmV - 1) / kSddmmV;
    long grid2 = (groups2 + 15) / 16;
    if (grid2 > cap) grid2 = cap;
    return launch_dependent(sddmm_list_kernel<16, kSddmmV, true, 2>, dim3((unsigned)grid2), dim3(256), 0, st, n, rows,
                            cols, outs, X, ldx, Y, ldy, out, F);
  }
  const bool vec = F % 4 == 0;
  cudaError_t e;
#define STILE_SDDMM_CASE(L)                                                                                   \
  e = vec ? launch_dependent(sddmm_list_kernel<L, kSddmmV, true>, dim3((unsigned)grid), dim3(256), 0, st, n, rows,  \
                             cols, outs, X, ldx, Y, ldy, out, F)                                               \
          : launch_dependent(sddmm_list_kernel<L, kSddmmV, false>, dim3((unsigned)grid), dim3(256), 0, st, n, rows, \
                             cols, outs, X, ldx, Y, ldy, out, F);
  switch (lpr) {
    case 4: STILE_SDDMM_CASE(4) break;
    case 8: STILE_SDDMM_CASE(8) break;
    case 16: STILE_SDDMM_CASE(16) break;
    default: STILE_SDDMM_CASE(32) break;
  }
#undef STILE_SDDMM_CASE
  return e;
}

// Row-run SDDMM: the entries come in groups that share one row (runs of a
// row-grouped list, cut at kRunGroup entries):
//   out[outs[t]] = <X[grow[g]], Y[cols[t]]>  for t in [gptr[g], gptr[g+1]).
// An LPR-lane group takes one run: it holds the run's X row in registers
// (one pass: F <= 4 VEC LPR; longer rows reload their slice per batch, an
// L1 hit) and streams the run's Y rows U at a time, each lane covering
// 4 VEC features with VEC float4 (or one 16-byte bf16 load) per row.  The U
// partial dot products are reduced with the transposing butterfly of the
// entry-list kernel, so the lanes whose high bits spell an entry index hold
// that entry's sum.  Few registers (no X gather per entry, no entry
// records in flight) leave room for more warps per SM than the entry-list
// kernel, and gathers grow with resident warps.
constexpr int kRunU = 2;       // Y rows in flight per group
constexpr int kRunBlocks = 6;  // resident 256-thread blocks per SM (register budget)

// kOne: F <= 4 VEC LPR (one pass; the X row stays in registers).
// kFull: F == 4 VEC LPR exactly (no masking at all).
template <int LPR, int VEC, int U, int MINB, bool kYb, bool kOne, bool kFull, bool kXb = false>
__global__ void __launch_bounds__(256, MINB) sddmm_run_kernel(int n_groups, const int* __restrict__ gptr,
                                                                const int* __restrict__ grow,
                                                                const int* __restrict__ cols,
                                                                const int* __restrict__ outs,
                                                                const void* __restrict__ Xv, long ldx,
                                                                const void* __restrict__ Yv, long ldy,
                                                                float* __restrict__ out, int F) {
  static_assert(U <= LPR && (U & (U - 1)) == 0, "U must be a power of two no larger than the group");
  static_assert((!kYb && !kXb) || VEC == 2, "a bf16 load covers 8 features");
  static_assert(!kFull || kOne, "a full pass is one pass");
  // launched dependent on the previous kernel: wait for its results (X may
  // be one of them), then let the next dependent kernel launch
  griddep_wait();
  griddep_launch_dependents();
  using TY = typename std::conditional<kYb, uint16_t, float>::type;
  const TY* __restrict__ Y = static_cast<const TY*>(Yv);
  const int lane = threadIdx.x & 31, sub = lane / LPR, sl = lane % LPR;
  const unsigned gmask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << (sub * LPR));
  const long g = ((long)blockIdx.x * blockDim.x + threadIdx.x) / LPR;
  if (g >= n_groups) return;  // the whole group leaves together
  const int p0 = __ldg(gptr + g), p1 = __ldg(gptr + g + 1);
  using TX = typename std::conditional<kXb, uint16_t, float>::type;
  const TX* __restrict__ xr = static_cast<const TX*>(Xv) + (long)__ldg(grow + g) * ldx;
  // A bf16 Y row gives a lane 8 consecutive features (one 16-byte load);
  // fp32 rows give it float4 w at features 4 (w LPR + lane), so that each
  // load instruction of the group reads 16 LPR contiguous bytes.  X follows
  // Y's split.
  constexpr int FP = 4 * VEC * LPR;  // features per pass
  constexpr int kStep = kYb ? 4 : 4 * LPR;  // features between a lane's float4
  const int f0 = kYb ? 4 * VEC * sl : 4 * sl;
  // X's features of this lane as VEC float4 (masked past F)
  auto load_x = [&](int f, float4 (&x)[VEC]) {
    if constexpr (kXb) {
      bf16x8_to_f32(kFull ? ldg_u4(xr + f) : ld_row8_bf16(xr, f, F), x[0], x[1]);
    } else {
#pragma unroll
      for (int w = 0; w < VEC; ++w) x[w] = kFull ? ldg4(xr + f + kStep * w) : ld4_live(xr, f + kStep * w, F);
    }
  };
  auto load_y = [&](int c, int f, float4 (&y)[VEC]) {
    const TY* row = Y + (long)c * ldy;
    if constexpr (kYb) {
      bf16x8_to_f32(kFull ? ldg_u4(row + f) : ld_row8_bf16(row, f, F), y[0], y[1]);
    } else {
#pragma unroll
      for (int w = 0; w < VEC; ++w) y[w] = kFull ? ldg4(row + f + kStep * w) : ld4_live(row, f + kStep * w, F);
    }
  };
  float4 x1[VEC];
  if constexpr (kOne) load_x(f0, x1);
#pragma unroll 1
  for (int b0 = p0; b0 < p1; b0 += U) {
    int c[U];
#pragma unroll
    for (int u = 0; u < U; ++u) c[u] = __ldg(cols + min(b0 + u, p1 - 1));  // past the run: a valid row, unused
    float s[U];
#pragma unroll
    for (int u = 0; u < U; ++u) s[u] = 0.f;
    if constexpr (kOne) {
      float4 y[U][VEC];
#pragma unroll
      for (int u = 0; u < U; ++u) load_y(c[u], f0, y[u]);
#pragma unroll
      for (int u = 0; u < U; ++u) {
#pragma unroll
        for (int w = 0; w < VEC; ++w) s[u] += dot4(x1[w], y[u][w]);
      }
    } else {
#pragma unroll 1
      for (int fc = 0; fc < F; fc += FP) {
        const int f = fc + f0;
        float4 xv[VEC];
        load_x(f, xv);
        float4 y[U][VEC];
#pragma unroll
        for (int u = 0; u < U; ++u) load_y(c[u], f, y[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
          for (int w = 0; w < VEC; ++w) s[u] += dot4(xv[w], y[u][w]);
        }
      }
    }
    int e = 0;
#pragma unroll
    for (int m = U, hw = LPR / 2; m > 1; m >>= 1, hw >>= 1) {
      const bool up = (sl & hw) != 0;
#pragma unroll
      for (int i = 0; i < m / 2; ++i) {
        const float send = up ? s[i] : s[i + m / 2];
        const float keep = up ? s[i + m / 2] : s[i];
        s[i] = keep + __shfl_xor_sync(gmask, send, hw);
      }
      if (up) e += m / 2;
    }
#pragma unroll
    for (int o = LPR / (2 * U); o > 0; o >>= 1) s[0] += __shfl_xor_sync(gmask, s[0], o);
    if ((sl & (LPR / U - 1)) == 0 && b0 + e < p1) __stcs(out + __ldg(outs + b0 + e), s[0]);  // evict first
  }
}

template <int L, bool kYb, bool kXb = false>
static cudaError_t launch_runs_t(int grid, bool one, bool full, cudaStream_t st, int n_groups, const int* gptr,
                                 const int* grow, const int* cols, const int* outs, const void* X, long ldx,
                                 const void* Y, long ldy, float* out, int F) {
  // narrow rows (8 lanes or fewer: 64 features or fewer) keep 4 Y rows in
  // flight per group at 5 blocks per SM: a narrow row is few bytes, and the
  // gathers are bound by the bytes in flight
  constexpr int U = L <= 8 ? 4 : kRunU, MINB = L <= 8 ? 5 : kRunBlocks;
  if (full)
    return launch_dependent(sddmm_run_kernel<L, 2, U, MINB, kYb, true, true, kXb>, dim3((unsigned)grid), dim3(256), 0,
                            st, n_groups, gptr, grow, cols, outs, X, ldx, Y, ldy, out, F);
  if (one)
    return launch_dependent(sddmm_run_kernel<L, 2, U, MINB, kYb, true, false, kXb>, dim3((unsigned)grid), dim3(256),
                            0, st, n_groups, gptr, grow, cols, outs, X, ldx, Y, ldy, out, F);
  return launch_dependent(sddmm_run_kernel<L, 2, U, MINB, kYb, false, false, kXb>, dim3((unsigned)grid), dim3(256), 0,
                          st, n_groups, gptr, grow, cols, outs, X, ldx, Y, ldy, out, F);
}

cudaError_t launch_sddmm_runs(int n_groups, const int* gptr, const int* grow, const int* cols, const int* outs,
                              const void* X, bool x_bf16, long ldx, const void* Y, bool y_bf16, long ldy, float* out,
                              int F, cudaStream_t st) {
  if (n_groups <= 0) return cudaSuccess;
  if (x_bf16 && !y_bf16) return cudaErrorNotSupported;  // no caller has a bf16 X with an fp32 Y
  // lanes per run: 8 features per lane (two float4, or one bf16 load);
  // 128 features per pass at most (longer rows take several passes)
  int lpr = 16;
  if (F < 128) {
    const int lanes = (F + 7) / 8;
    lpr = 4;
    while (lpr < lanes) lpr <<= 1;
  }
  const bool one = F <= 8 * lpr, full = F == 8 * lpr;
  const int grid = (int)(((long)n_groups * lpr + 255) / 256);
#define STILE_RUNS_ARGS grid, one, full, st, n_groups, gptr, grow, cols, outs, X, ldx, Y, ldy, out, F
  switch (lpr) {
    case 4:
      return x_bf16 ? launch_runs_t<4, true, true>(STILE_RUNS_ARGS)
                    : (y_bf16 ? launch_runs_t<4, true>(STILE_RUNS_ARGS) : launch_runs_t<4, false>(STILE_RUNS_ARGS));
    case 8:
      return x_bf16 ? launch_runs_t<8, true, true>(STILE_RUNS_ARGS)
                    : (y_bf16 ? launch_runs_t<8, true>(STILE_RUNS_ARGS) : launch_runs_t<8, false>(STILE_RUNS_ARGS));
    default:
      return x_bf16 ? launch_runs_t<16, true, true>(STILE_RUNS_ARGS)
                    : (y_bf16 ? launch_runs_t<16, true>(STILE_RUNS_ARGS) : launch_runs_t<16, false>(STILE_RUNS_ARGS));
  }
#undef STILE_RUNS_ARGS
}

// Block tiles on the tensor cores.  A unit is up to 8 consecutive 16x16
// blocks: its 128 Y rows (16 per block) form the MMA's A operand (M = 128)
// and its 128 X rows its B operand (N = 128), both K-major with the
// features along K exactly as the rows are stored, so
//   D[16 j + n][16 j + m] = <X[blk_i[j][m]], Y[blk_j[j][n]]>
// on the 8 diagonal 16x16 sub-blocks (the off-diagonal ones are products
// nobody asked for; the tensor pipe has time to spare).  Per 64-feature
// chunk every thread gathers one Y row and one X row, converts them to bf16
// (fp32 inputs: hi = bf16(x) and lo = bf16(x - hi), three MMAs per K-slice,
// hi.hi + hi.lo + lo.hi), stores them in the no-swizzle K-major layout
// (core matrices of 8 rows x 16 B, k halves 128 B apart, 8-row groups 256 B
// apart, one 4 KB slice per 16 features), and one thread issues the MMAs
// into a 128-column TMEM accumulator.  The epilogue reads each warp's 32 Y
// rows from TMEM, stages the diagonal blocks in shared memory and writes
// only the blocks' live entries (indicesDense).  The wait for the MMAs is
// bounded; a wait that runs out sets the error flag and skips the unit's
// output.
constexpr int kBlkUnit = 8;                      // blocks per unit
constexpr int kBlkFc = 64;                       // features per chunk: 4 K-slices of 16
constexpr uint32_t kBlkSlice = 4096;             // one K = 16 slice of 128 bf16 rows
constexpr uint32_t kBlkImg = 4 * kBlkSlice;      // 64 features of 128 rows
constexpr int kBlkDPad = 17;                     // staged D rows (floats), padded against bank conflicts

template <bool kB16>
struct BlkCfg {
  static constexpr int kImgs = kB16 ? 2 : 4;     // Y hi, X hi (+ Y lo, X lo)
  static constexpr uint32_t kDBytes = kBlkUnit * 16 * kBlkDPad * 4;
  static constexpr uint32_t kBytes = 1024 + kImgs * kBlkImg + kDBytes + 64;
};

// 16 bytes of 8 bf16 features at element (row, k = 8 q) of a 128-row
// K-major image (slice q / 2, k half q % 2)
__device__ __forceinline__ uint32_t blk_off(int row, int q) {
  return (uint32_t)((q >> 1) * kBlkSlice + (row >> 3) * 256 + (q & 1) * 128 + (row & 7) * 16);
}

template <bool kB16>
__global__ void __launch_bounds__(128) sddmm_block_tc_kernel(SddmmArgs p, int n_units) {
  using Cfg = BlkCfg<kB16>;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const uint32_t yhi = base, xhi = base + kBlkImg, ylo = base + 2 * kBlkImg, xlo = base + 3 * kBlkImg;
  const uint32_t dst = base + Cfg::kImgs * kBlkImg;
  float* dstage = reinterpret_cast<float*>(smem_raw + (dst - smem_u32(smem_raw)));
  const uint32_t bar = dst + Cfg::kDBytes, tmem_slot = bar + 8;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(tmem_slot, 128);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  uint32_t tmem;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(tmem) : "r"(tmem_slot) : "memory");
  // kind::f16, bf16 x bf16, M = 128, N = 128, both operands K-major
  constexpr uint32_t idesc = make_idesc(1, 1, 0, 0, 128, 128);
  const int F = p.F;
  uint32_t phase = 0;
  bool ok = true;
#pragma unroll 1
  for (int u = blockIdx.x; u < n_units && ok; u += gridDim.x) {
    const int b0 = u * kBlkUnit;
    const int nb = min(kBlkUnit, p.n_blk - b0);
    const int j = tid >> 4, r = tid & 15;
    const int yrow = j < nb ? __ldg(p.blk_j + (long)(b0 + j) * 16 + r) : -1;
    const int xrow = j < nb ? __ldg(p.blk_i + (long)(b0 + j) * 16 + r) : -1;
#pragma unroll 1
    for (int fc = 0; fc < F; fc += kBlkFc) {
      // gather and convert: this thread's Y row and X row, 64 features
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const int row = side ? xrow : yrow;
        const uint32_t hi = side ? xhi : yhi, lo = side ? xlo : ylo;
#pragma unroll 2
        for (int q = 0; q < kBlkFc / 8; ++q) {
          const int f = fc + 8 * q;
          float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
          if (row >= 0) {
            if constexpr (kB16) {
              const uint16_t* src = reinterpret_cast<const uint16_t*>(side ? (const void*)p.X : (const void*)p.Y);
              bf16x8_to_f32(ld_row8_bf16(src + (long)row * (side ? p.ldx : p.ldy), f, F), a, b);
            } else {
              const float* src = (side ? p.X : p.Y) + (long)row * (side ? p.ldx : p.ldy);
              a = ld4_live(src, f, F);
              b = ld4_live(src, f + 4, F);
            }
          }
          const uint32_t h01 = pack_bf16x2(a.x, a.y), h23 = pack_bf16x2(a.z, a.w);
          const uint32_t h45 = pack_bf16x2(b.x, b.y), h67 = pack_bf16x2(b.z, b.w);
          st_shared_v4(hi + blk_off(tid, q), make_uint4(h01, h23, h45, h67));
          if constexpr (!kB16) {
            auto lo2 = [](uint32_t h, float x0, float x1) {
              return pack_bf16x2(x0 - __uint_as_float(h << 16), x1 - __uint_as_float(h & 0xffff0000u));
            };
            st_shared_v4(lo + blk_off(tid, q),
                         make_uint4(lo2(h01, a.x, a.y), lo2(h23, a.z, a.w), lo2(h45, b.x, b.y), lo2(h67, b.z, b.w)));
          }
        }
      }
      fence_proxy_async_smem();
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      if (tid == 0) {
        const int ns = min(4, (F - fc + 15) / 16);
        for (int s = 0; s < ns; ++s) {
          const uint64_t ah = smem_desc(yhi + s * kBlkSlice, 128, 256, kSwizzleNone);
          const uint64_t bh = smem_desc(xhi + s * kBlkSlice, 128, 256, kSwizzleNone);
          umma_f16(tmem, ah, bh, idesc, (fc > 0 || s > 0) ? 1u : 0u);
          if constexpr (!kB16) {
            umma_f16(tmem, ah, smem_desc(xlo + s * kBlkSlice, 128, 256, kSwizzleNone), idesc, 1u);
            umma_f16(tmem, smem_desc(ylo + s * kBlkSlice, 128, 256, kSwizzleNone), bh, idesc, 1u);
          }
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
    // epilogue: warp w holds TMEM lanes (Y rows) 32 w .. 32 w + 31, i.e.
    // blocks 2 w and 2 w + 1, whose X rows are TMEM columns 16 j .. 16 j + 15
    uint32_t v0[16], v1[16];
    tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(32 * warp), v0);
    tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(32 * warp + 16), v1);
    tmem_wait_ld();
    {
      const int jj = tid >> 4, n = tid & 15;
#pragma unroll
      for (int m = 0; m < 16; ++m)
        dstage[(jj * 16 + n) * kBlkDPad + m] = __uint_as_float(lane < 16 ? v0[m] : v1[m]);
    }
    tc_fence_before();
    __syncthreads();
    for (int jj = 0; jj < nb; ++jj) {
      const int e0 = __ldg(p.blk_indptr + b0 + jj), e1 = __ldg(p.blk_indptr + b0 + jj + 1);
      for (int e = e0 + tid; e < e1; e += 128) {
        const int pos = __ldg(p.blk_dense_pos + e);
        const int m = pos / p.bn, n = pos % p.bn;
        __stcs(p.out + __ldg(p.blk_out + e), dstage[(jj * 16 + n) * kBlkDPad + m]);
      }
    }
    __syncthreads();
  }
  if (!ok && tid == 0 && p.err_flag) atomicOr(p.err_flag, 1);
  // every MMA this CTA issued has completed before TMEM is freed
  if (!ok && tid == 0) mbar_wait_bounded(bar, phase ^ 1u);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, 128);
}

cudaError_t launch_sddmm(const SddmmArgs& p, cudaStream_t st) {
  // block tiles first, then 1D tiles: where both cover a nonzero the 1D
  // result is the one kept, as in the reference's host reorder
  // (order_output_BSDDMM writes the TC results first, then the 1D ones)
  if (p.n_blk > 0) {
    if (p.bm != 16 || p.bn != 16) return cudaErrorNotSupported;
    const int n_units = (p.n_blk + kBlkUnit - 1) / kBlkUnit;
    // at least 57 KB of shared memory per CTA: at most 4 CTAs share an SM,
    // whose 512 TMEM columns then hold their 128-column accumulators
    const size_t smem = std::max<size_t>(p.xy_bf16 ? BlkCfg<true>::kBytes : BlkCfg<false>::kBytes, 57 * 1024);
    auto k = p.xy_bf16 ? sddmm_block_tc_kernel<true> : sddmm_block_tc_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int grid = std::min(n_units, device_sm_count() * (p.xy_bf16 ? 4 : 2));
    k<<<grid, 128, smem, st>>>(p, n_units);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  // 1D tiles: the flattened entries come in runs of one row (cut at upload)
  return launch_sddmm_runs(p.n_runs, p.run_ptr, p.run_row, p.j_idx, p.remap, p.X, p.xy_bf16, p.ldx, p.Y, p.xy_bf16,
                           p.ldy, p.out, p.F, st);
}

// Row softmax over a CSR pattern (the sparse-attention step between the
// SDDMM of the scores and the SpMM with the values, as in the reference's
// sparse-transformer softmax, my_3rdparty/Magicube/Magicube1/end2end_eval/
// sparse_transformer_magicube/verify/bsoftmax.py: softmax over each row's
// stored entries of scale * x, the others being -inf).  One warp per row,
// blockIdx.y = head (x and out hold `batch` value sets of nnz entries).
__global__ void __launch_bounds__(256) csr_row_softmax_kernel(int M, const int* __restrict__ indptr, long nnz,
                                                               const float* __restrict__ x, float* __restrict__ out,
                                                               float scale) {
  const int row = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= M) return;
  const long off = (long)blockIdx.y * nnz;
  const int b = __ldg(indptr + row), e = __ldg(indptr + row + 1);
  float m = -INFINITY;
  for (int t = b + lane; t < e; t += 32) m = fmaxf(m, scale * __ldg(x + off + t));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  float sum = 0.f;
  for (int t = b + lane; t < e; t += 32) sum += expf(scale * __ldg(x + off + t) - m);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  const float inv = 1.f / sum;
  for (int t = b + lane; t < e; t += 32) out[off + t] = expf(scale * __ldg(x + off + t) - m) * inv;
}

cudaError_t launch_csr_row_softmax(int M, const int* indptr, long nnz, const float* x, float* out, float scale,
                                   int batch, cudaStream_t st) {
  if (M == 0 || batch == 0) return cudaSuccess;
  const dim3 grid((unsigned)((M + 7) / 8), (unsigned)batch);
  csr_row_softmax_kernel<<<grid, 256, 0, st>>>(M, indptr, nnz, x, out, scale);
  return cudaGetLastError();
}

}  // namespace stile
