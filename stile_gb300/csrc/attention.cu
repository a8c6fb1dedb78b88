// Fused sparse attention for sm_103a:
//   out[h][r] = sum_t softmax_t(scale * <Q[h][r], K[h][c_t]>) * V[h][c_t]
// over the stored entries c_t of row r of a CSR pattern (entries outside the
// pattern count as -inf), every head in one launch (blockIdx.y = head).
//
// This is the sparse-attention step the reference's LogSparse / Strided
// operators come from (MY_sparse/gen_formats_v2.py:2926-3003): the SDDMM of
// the scores on the pattern, the row softmax of the sparse transformer
// (my_3rdparty/Magicube/Magicube1/end2end_eval/sparse_transformer_magicube/
// src/cuda/softmax_kernel.cu) and the SpMM with the probabilities as values,
// here in one pass per row: an LPR-lane group holds its query row (8
// features a lane, as two float4 4 LPR features apart), gathers the K and V rows of two entries at a time,
// reduces the two scores with a transposing butterfly, broadcasts them, and
// keeps an online softmax -- running maximum m, running sum l and an output
// accumulator rescaled by exp(m_old - m_new) whenever the maximum grows --
// so neither the scores nor the probabilities are written anywhere.
#include "common.cuh"
#include "spmm.cuh"

namespace stile {

template <int LPR>
__global__ void __launch_bounds__(256, 4) sparse_attention_kernel(int n_rows, const int* __restrict__ indptr,
                                                                   const int* __restrict__ indices,
                                                                   const float* __restrict__ Q,
                                                                   const float* __restrict__ K,
                                                                   const float* __restrict__ V, long ldq, long ldk,
                                                                   long ldv, long q_head, long k_head, long v_head,
                                                                   float* __restrict__ out, long ldo, long o_head,
                                                                   int F, int Fv, float scale) {
  static_assert(LPR >= 2, "two entries per batch");
  const int lane = threadIdx.x & 31, sub = lane / LPR, sl = lane % LPR;
  const unsigned mask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << (sub * LPR));
  const long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) / LPR;
  if (r >= n_rows) return;  // the whole group leaves together
  const long h = blockIdx.y;
  const float* Qh = Q + h * q_head;
  const float* Kh = K + h * k_head;
  const float* Vh = V + h * v_head;
  // this lane's features: f .. f + 3 and f2 .. f2 + 3 (each load
  // instruction of the group reads 16 LPR contiguous bytes of a row)
  const int f = 4 * sl, f2 = f + 4 * LPR;
  const float* qr = Qh + r * ldq;
  const float4 q0 = ld4_live(qr, f, F), q1 = ld4_live(qr, f2, F);
  const int rb = __ldg(indptr + r), re = __ldg(indptr + r + 1);
  float m = -INFINITY, l = 0.f;
  float4 acc0 = make_float4(0.f, 0.f, 0.f, 0.f), acc1 = acc0;
#pragma unroll 1
  for (int b0 = rb; b0 < re; b0 += 2) {
    const bool v1 = b0 + 1 < re;
    const int c0 = __ldg(indices + b0), c1 = v1 ? __ldg(indices + b0 + 1) : c0;
    const float* k0 = Kh + (long)c0 * ldk;
    const float* k1 = Kh + (long)c1 * ldk;
    const float* w0 = Vh + (long)c0 * ldv;
    const float* w1 = Vh + (long)c1 * ldv;
    const float4 ka0 = ld4_live(k0, f, F), kb0 = ld4_live(k0, f2, F);
    const float4 ka1 = ld4_live(k1, f, F), kb1 = ld4_live(k1, f2, F);
    const float4 va0 = ld4_live(w0, f, Fv), vb0 = ld4_live(w0, f2, Fv);
    const float4 va1 = ld4_live(w1, f, Fv), vb1 = ld4_live(w1, f2, Fv);
    const float s0 = dot4(q0, ka0) + dot4(q1, kb0);
    const float s1 = dot4(q0, ka1) + dot4(q1, kb1);
    // transposing butterfly: the upper half of the group keeps entry 1
    const bool up = (sl & (LPR / 2)) != 0;
    float t = (up ? s1 : s0) + __shfl_xor_sync(mask, up ? s0 : s1, LPR / 2);
#pragma unroll
    for (int o = LPR / 4; o > 0; o >>= 1) t += __shfl_xor_sync(mask, t, o);
    const float e0 = scale * __shfl_sync(mask, t, 0, LPR);
    const float e1 = v1 ? scale * __shfl_sync(mask, t, LPR / 2, LPR) : -INFINITY;
    const float mn = fmaxf(m, fmaxf(e0, e1));
    const float alpha = expf(m - mn);  // 0 for the first batch (m = -inf)
    const float p0 = expf(e0 - mn), p1 = expf(e1 - mn);
    l = l * alpha + p0 + p1;
    acc0 = make_float4(acc0.x * alpha + p0 * va0.x + p1 * va1.x, acc0.y * alpha + p0 * va0.y + p1 * va1.y,
                       acc0.z * alpha + p0 * va0.z + p1 * va1.z, acc0.w * alpha + p0 * va0.w + p1 * va1.w);
    acc1 = make_float4(acc1.x * alpha + p0 * vb0.x + p1 * vb1.x, acc1.y * alpha + p0 * vb0.y + p1 * vb1.y,
                       acc1.z * alpha + p0 * vb0.z + p1 * vb1.z, acc1.w * alpha + p0 * vb0.w + p1 * vb1.w);
    m = mn;
  }
  // a row without entries attends to nothing: zeros
  const float inv = l > 0.f ? 1.f / l : 0.f;
  float* orow = out + h * o_head + r * ldo;
  st_row4(orow, f, Fv, make_float4(acc0.x * inv, acc0.y * inv, acc0.z * inv, acc0.w * inv));
  st_row4(orow, f2, Fv, make_float4(acc1.x * inv, acc1.y * inv, acc1.z * inv, acc1.w * inv));
}

cudaError_t launch_sparse_attention(int n_rows, const int* indptr, const int* indices, const float* Q,
                                    const float* K, const float* V, long ldq, long ldk, long ldv, long q_head,
                                    long k_head, long v_head, float* out, long ldo, long o_head, int F, int Fv,
                                    float scale, int heads, cudaStream_t st) {
  if (n_rows == 0 || heads == 0) return cudaSuccess;
  const int width = F > Fv ? F : Fv;  // features per lane: 8; lanes: the power of two covering the wider row
  int lpr = 2;
  while (8 * lpr < width) lpr <<= 1;
  const dim3 grid((unsigned)(((long)n_rows * lpr + 255) / 256), (unsigned)heads);
#define STILE_ATT(L)                                                                                              \
  sparse_attention_kernel<L><<<grid, 256, 0, st>>>(n_rows, indptr, indices, Q, K, V, ldq, ldk, ldv, q_head, k_head, \
                                                   v_head, out, ldo, o_head, F, Fv, scale)
  switch (lpr) {
    case 2: STILE_ATT(2); break;
    case 4: STILE_ATT(4); break;
    case 8: STILE_ATT(8); break;
    default: STILE_ATT(16); break;
  }
#undef STILE_ATT
  return cudaGetLastError();
}

}  // namespace stile
