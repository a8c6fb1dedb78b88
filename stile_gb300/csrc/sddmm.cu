// SDDMM kernels for sm_103a: out[t] = <X[row(t)], Y[col(t)]> on a mask.
//
//  * 1D tiles (the reference's "1D_sddmm", my_fuse_formats.py:2263-2317):
//    an LPR-lane group per nonzero, 128-bit feature loads, shuffle
//    reduction, result written straight to its CSR position (remap) -- the
//    reference writes a tile-ordered buffer and reorders on the host
//    (order_output_BSDDMM, :4247-4288).
//  * block tiles (the reference's "TC_sddmm", :2324-2415): one CTA per
//    bm x bn block; the X / Y rows of the block are staged in shared memory
//    one 128-feature chunk at a time and only the live entries of the block
//    (indicesDense) are computed.
#include "common.cuh"
#include "spmm.cuh"

namespace stile {

template <int LPR>
__global__ void __launch_bounds__(256) sddmm_1d_kernel(SddmmArgs p) {
  constexpr int GPB = 256 / LPR;  // groups per block
  const int lane = threadIdx.x & 31;
  const int sub = lane / LPR, sl = lane % LPR;
  const unsigned gmask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << (sub * LPR));
  const int g = blockIdx.x * GPB + threadIdx.x / LPR;
  const int stride = gridDim.x * GPB;
  for (int t = g; t < p.n_1d; t += stride) {
    const float* x = p.X + (long)p.mid_idx[t] * p.ldx;
    const float* y = p.Y + (long)p.j_idx[t] * p.ldy;
    float s = 0.f;
    for (int f = 4 * sl; f < p.F; f += 4 * LPR) s += dot4(ld_row4(x, f, p.F), ld_row4(y, f, p.F));
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(gmask, s, o);
    if (sl == 0) p.out[p.remap[t]] = s;
  }
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

static int lpr_for_f(int F) {
  const int lanes = (F + 3) / 4;
  if (lanes >= 32) return 32;
  int l = 1;
  while (l < lanes) l <<= 1;
  return l < 4 ? 4 : l;
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
  if (p.n_1d > 0) {
    const int lpr = lpr_for_f(p.F);
    const int gpb = 256 / lpr;
    int grid = (p.n_1d + gpb - 1) / gpb;
    if (grid > 152 * 64) grid = 152 * 64;
    switch (lpr) {
      case 4: sddmm_1d_kernel<4><<<grid, 256, 0, st>>>(p); break;
      case 8: sddmm_1d_kernel<8><<<grid, 256, 0, st>>>(p); break;
      case 16: sddmm_1d_kernel<16><<<grid, 256, 0, st>>>(p); break;
      default: sddmm_1d_kernel<32><<<grid, 256, 0, st>>>(p); break;
    }
    return cudaGetLastError();
  }
  return cudaSuccess;
}

}  // namespace stile
