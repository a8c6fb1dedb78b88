// SDDMM kernels for sm_103a: out[t] = <X[row(t)], Y[col(t)]> on a mask.
//
//  * 1D tiles (the reference's "1D_sddmm", my_fuse_formats.py:2263-2317):
//    the entry-list kernel below over (mid_idx, j_idx, remap); results go
//    straight to their CSR position -- the reference writes a tile-ordered
//    buffer and reorders on the host (order_output_BSDDMM, :4247-4288).
//  * block tiles (the reference's "TC_sddmm", :2324-2415): one CTA per
//    bm x bn block; the X / Y rows of the block are staged in shared memory
//    one 128-feature chunk at a time and only the live entries of the block
//    (indicesDense) are computed.
#include "common.cuh"
#include "spmm.cuh"

namespace stile {

// Entry-list SDDMM: out[outs[t]] = <X[rows[t]], Y[cols[t]]>.  An LPR-lane
// group takes 8 consecutive entries per iteration (row loads 8 at a time,
// 128-bit each) and reduces the 8 dot products together with a
// transposing butterfly: after the three halving steps every lane holds one
// entry's partial sum, so 8 dots cost 9 shuffles instead of 40.  Entries
// sorted by row reuse the X row from L1.
template <int LPR>
__global__ void __launch_bounds__(256, 2) sddmm_list_kernel(long n, const int* __restrict__ rows,
                                                            const int* __restrict__ cols,
                                                            const int* __restrict__ outs,
                                                            const float* __restrict__ X, long ldx,
                                                            const float* __restrict__ Y, long ldy,
                                                            float* __restrict__ out, int F) {
  constexpr int V = 8;
  constexpr int GPB = 256 / LPR;
  const int lane = threadIdx.x & 31;
  const int sub = lane / LPR, sl = lane % LPR;
  const unsigned gmask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << (sub * LPR));
  const long g = (long)blockIdx.x * GPB + threadIdx.x / LPR;
  const long stride = (long)gridDim.x * GPB;
  for (long base = g * V; base < n; base += stride * V) {
    const int cnt = (int)min((long)V, n - base);
    int r[V], c[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      r[v] = v < cnt ? __ldg(rows + base + v) : 0;
      c[v] = v < cnt ? __ldg(cols + base + v) : 0;
    }
    float a[V];
#pragma unroll
    for (int v = 0; v < V; ++v) a[v] = 0.f;
    for (int fc = 0; fc < F; fc += 4 * LPR) {
      const int f = fc + 4 * sl;
      // two phases of 4 entries: 8 row loads in flight, 8 float4 live
#pragma unroll
      for (int h = 0; h < V; h += 4) {
        float4 xv[4], yv[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          xv[v] = ld_row4(X + (long)r[h + v] * ldx, f, F);
          yv[v] = ld_row4(Y + (long)c[h + v] * ldy, f, F);
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) a[h + v] += dot4(xv[v], yv[v]);
      }
    }
    if (LPR >= 8) {
      constexpr int h1 = LPR / 2, h2 = LPR / 4, h3 = LPR / 8;
      {
        const bool up = (sl & h1) != 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float send = up ? a[i] : a[i + 4];
          const float keep = up ? a[i + 4] : a[i];
          a[i] = keep + __shfl_xor_sync(gmask, send, h1);
        }
      }
      {
        const bool up = (sl & h2) != 0;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const float send = up ? a[i] : a[i + 2];
          const float keep = up ? a[i + 2] : a[i];
          a[i] = keep + __shfl_xor_sync(gmask, send, h2);
        }
      }
      {
        const bool up = (sl & h3) != 0;
        const float send = up ? a[0] : a[1];
        const float keep = up ? a[1] : a[0];
        a[0] = keep + __shfl_xor_sync(gmask, send, h3);
      }
#pragma unroll
      for (int o = h3 / 2; o > 0; o >>= 1) a[0] += __shfl_xor_sync(gmask, a[0], o);
      const int e = ((sl & h1) ? 4 : 0) + ((sl & h2) ? 2 : 0) + ((sl & h3) ? 1 : 0);
      if ((sl & (h3 - 1)) == 0 && e < cnt) out[__ldg(outs + base + e)] = a[0];
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

cudaError_t launch_sddmm_list(long n, const int* rows, const int* cols, const int* outs, const float* X,
                              long ldx, const float* Y, long ldy, float* out, int F, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int lpr = lpr_for_f(F);
  const int gpb = 256 / lpr;
  long groups = (n + 7) / 8;
  long grid = (groups + gpb - 1) / gpb;
  if (grid > 152L * 32) grid = 152L * 32;
  switch (lpr) {
    case 4: sddmm_list_kernel<4><<<(unsigned)grid, 256, 0, st>>>(n, rows, cols, outs, X, ldx, Y, ldy, out, F); break;
    case 8: sddmm_list_kernel<8><<<(unsigned)grid, 256, 0, st>>>(n, rows, cols, outs, X, ldx, Y, ldy, out, F); break;
    case 16: sddmm_list_kernel<16><<<(unsigned)grid, 256, 0, st>>>(n, rows, cols, outs, X, ldx, Y, ldy, out, F); break;
    default: sddmm_list_kernel<32><<<(unsigned)grid, 256, 0, st>>>(n, rows, cols, outs, X, ldx, Y, ldy, out, F); break;
  }
  return cudaGetLastError();
}

constexpr int kChunk = 128;
constexpr int kPadRow = kChunk + 4;

__global__ void __launch_bounds__(128) sddmm_block_kernel(SddmmArgs p) {
  __shared__ __align__(16) float xs[16 * kPadRow];
  __shared__ __align__(16) float ys[16 * kPadRow];
  const int b = blockIdx.x;
  const int tid = threadIdx.x;
  const int e0 = p.blk_indptr[b], e1 = p.blk_indptr[b + 1];
  const int n_e = e1 - e0;  // <= bm * bn <= 256
  float acc[2] = {0.f, 0.f};
  int pos[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int e = tid + q * 128;
    pos[q] = (e < n_e) ? p.blk_dense_pos[e0 + e] : 0;
  }
  for (int fc = 0; fc < p.F; fc += kChunk) {
    __syncthreads();
    // stage: bm rows of X and bn rows of Y, 32 float4 per row
    for (int i = tid; i < 16 * (kChunk / 4); i += 128) {
      const int r = i / (kChunk / 4), c = (i % (kChunk / 4)) * 4;
      float4 vx = make_float4(0.f, 0.f, 0.f, 0.f), vy = vx;
      if (r < p.bm) vx = ld_row4(p.X + (long)p.blk_i[(long)b * p.bm + r] * p.ldx, fc + c, p.F);
      if (r < p.bn) vy = ld_row4(p.Y + (long)p.blk_j[(long)b * p.bn + r] * p.ldy, fc + c, p.F);
      *reinterpret_cast<float4*>(&xs[r * kPadRow + c]) = vx;
      *reinterpret_cast<float4*>(&ys[r * kPadRow + c]) = vy;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int e = tid + q * 128;
      if (e < n_e) {
        const int m = pos[q] / p.bn, n = pos[q] % p.bn;
        const float* xr = &xs[m * kPadRow];
        const float* yr = &ys[n * kPadRow];
        float s = 0.f;
#pragma unroll 8
        for (int c = 0; c < kChunk; c += 4) {
          const float4 a = *reinterpret_cast<const float4*>(xr + c);
          const float4 bb = *reinterpret_cast<const float4*>(yr + c);
          s += dot4(a, bb);
        }
        acc[q] += s;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int e = tid + q * 128;
    if (e < n_e) p.out[p.blk_out[e0 + e]] = acc[q];
  }
}

cudaError_t launch_sddmm(const SddmmArgs& p, cudaStream_t st) {
  // block tiles first, then 1D tiles: where both cover a nonzero the 1D
  // result is the one kept, as in the reference's host reorder
  // (order_output_BSDDMM writes the TC results first, then the 1D ones)
  if (p.n_blk > 0) {
    sddmm_block_kernel<<<p.n_blk, 128, 0, st>>>(p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return launch_sddmm_list(p.n_1d, p.mid_idx, p.j_idx, p.remap, p.X, p.ldx, p.Y, p.ldy, p.out, p.F, st);
}

}  // namespace stile
