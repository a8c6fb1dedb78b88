// Layout self-check for the tensor-core path: one CTA copies two operand
// images verbatim into shared memory, issues one tcgen05.mma (M=128, N=16;
// kind::f16 with K=16, kind::tf32 with K=8 or kind::f8f6f4 with K=32; fp32
// accumulate) with caller-chosen descriptor fields and writes the 128x16
// accumulator to global memory.  Every descriptor the caller can pass stays
// inside the CTA's shared memory: each operand gets a 48 KB zero-filled
// region, the image occupies its first 16 KB (a 128-row K-major operand
// with the 128-byte swizzle spans 16 KB), and the host limits strides to
// 2048 B so that 16 groups along one direction times the largest stride
// plus a 16 KB span stay below 48 KB.  A wrong layout yields wrong numbers,
// never an out-of-bounds access.
#include "common.cuh"
#include "spmm.cuh"

namespace stile {

constexpr int kProbeImage = 16384;   // bytes of one operand image
constexpr int kProbeRegion = 49152;  // shared-memory region per operand

__global__ void __launch_bounds__(128) umma_probe_kernel(const uint4* __restrict__ a_img,
                                                         const uint4* __restrict__ b_img,
                                                         uint32_t a_lbo, uint32_t a_sbo,
                                                         uint32_t a_layout, uint32_t b_lbo,
                                                         uint32_t b_sbo, uint32_t b_layout,
                                                         uint32_t idesc, uint32_t kind,
                                                         float* __restrict__ out, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const uint32_t sa = base, sb = base + kProbeRegion;
  const uint32_t bar = base + 2 * kProbeRegion, slot = bar + 8;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint4 z = make_uint4(0u, 0u, 0u, 0u);
  for (int i = tid; i < kProbeRegion / 16; i += 128) {
    const bool img = i < kProbeImage / 16;
    st_shared_v4(sa + 16 * i, img ? a_img[i] : z);
    st_shared_v4(sb + 16 * i, img ? b_img[i] : z);
  }
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(slot, 32);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  uint32_t tmem;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(tmem) : "r"(slot) : "memory");
  if (tid == 0) {
    const uint64_t ad = smem_desc(sa, a_lbo, a_sbo, a_layout), bd = smem_desc(sb, b_lbo, b_sbo, b_layout);
    if (kind == 1) umma_tf32(tmem, ad, bd, idesc, 0u);
    else if (kind == 2) umma_f8(tmem, ad, bd, idesc, 0u);
    else umma_f16(tmem, ad, bd, idesc, 0u);
    umma_commit(bar);
  }
  const bool done = __syncthreads_and(mbar_wait_bounded(bar, 0)) != 0;
  if (!done && tid == 0) atomicOr(err, 1);
  tc_fence_after();
  uint32_t r[16];
  tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16), r);
  tmem_wait_ld();
  const int m = 32 * warp + lane;
#pragma unroll
  for (int n = 0; n < 16; ++n) out[m * 16 + n] = done ? __uint_as_float(r[n]) : 0.f;
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 32);
}

cudaError_t launch_umma_probe(const void* a_img, const void* b_img, const uint32_t* desc6,
                              uint32_t idesc, uint32_t kind, float* out, int* err, cudaStream_t st) {
  const size_t smem = 1024 + 2 * kProbeRegion + 64;
  cudaError_t e = cudaFuncSetAttribute(umma_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  umma_probe_kernel<<<1, 128, smem, st>>>(static_cast<const uint4*>(a_img),
                                          static_cast<const uint4*>(b_img), desc6[0], desc6[1], desc6[2],
                                          desc6[3], desc6[4], desc6[5], idesc, kind, out, err);
  return cudaGetLastError();
}

}  // namespace stile
