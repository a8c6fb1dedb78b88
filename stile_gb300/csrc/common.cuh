// Shared device helpers for the sm_103a kernels: vector loads, tcgen05 /
// mbarrier inline PTX, shared-memory descriptors and bounded waits.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace stile {

constexpr int kWarp = 32;

// ---------------------------------------------------------------------------
// global memory
// ---------------------------------------------------------------------------
__device__ __forceinline__ float4 ldg4(const float* p) {
  return __ldg(reinterpret_cast<const float4*>(p));
}

// float4 load of features [f, f+4) of a row, masked by N (the row stride is a
// multiple of 4 elements, so the full vector is in bounds whenever f < N).
__device__ __forceinline__ float4 ld_row4(const float* row, int f, int N) {
  if (f + 3 < N) return ldg4(row + f);
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (f < N) {
    float4 t = ldg4(row + f);
    v.x = t.x;
    if (f + 1 < N) v.y = t.y;
    if (f + 2 < N) v.z = t.z;
  }
  return v;
}

// A float4 of features [f, f + 4) of a row whose stride is a multiple of 4
// elements: loaded when f < N (the vector then lies inside the row's
// storage), components at or past N set to zero by selects (padding may
// hold anything, NaN included).
__device__ __forceinline__ float4 ld4_live(const float* row, int f, int N) {
  const int live = N - f;
  float4 v = live > 0 ? ldg4(row + f) : make_float4(0.f, 0.f, 0.f, 0.f);
  v.y = live > 1 ? v.y : 0.f;
  v.z = live > 2 ? v.z : 0.f;
  v.w = live > 3 ? v.w : 0.f;
  return v;
}

// The float4 at feature f when f < N, else zeros: the features of that
// float4 past N are the row's padding (any bits).  Only for sums kept per
// feature (SpMM rows), whose padding features are never stored; a dot
// product over features needs ld4_live.
__device__ __forceinline__ float4 ld4_pad(const float* row, int f, int N) {
  return f < N ? ldg4(row + f) : make_float4(0.f, 0.f, 0.f, 0.f);
}

// Output rows are written once and not read again by the writing kernel:
// streaming (evict-first) stores leave L2 to the gathered operand rows.
__device__ __forceinline__ void st_row4(float* row, int f, int N, float4 v) {
  if (f + 3 < N) {
    __stcs(reinterpret_cast<float4*>(row + f), v);
  } else if (f < N) {
    row[f] = v.x;
    if (f + 1 < N) row[f + 1] = v.y;
    if (f + 2 < N) row[f + 2] = v.z;
  }
}

__device__ __forceinline__ void red_row4(float* row, int f, int N, float4 v) {
  if (f + 3 < N) {
    atomicAdd(reinterpret_cast<float4*>(row + f), v);
  } else if (f < N) {
    atomicAdd(row + f, v.x);
    if (f + 1 < N) atomicAdd(row + f + 1, v.y);
    if (f + 2 < N) atomicAdd(row + f + 2, v.z);
  }
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start while the previous kernel on the stream drains.
// griddep_wait() returns once that kernel has completed and its writes are
// visible (at once when the launch was an ordinary one);
// griddep_launch_dependents() lets the next such kernel start.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// The kernels of one C-API call chain as programmatic dependents, but the
// first kernel a call launches is an ordinary launch: it starts only after
// everything before it on the stream (the previous call's kernels) has
// completed.  Blocks of the next operator launched early onto the SMs of
// the previous operator's persistent tensor-core grid slowed that grid's
// tail: the two-layer GCN step (four operator calls) took 2.26 ms with the
// chain running across calls and 1.96 ms with it cut at every call.
// Every entry point that launches kernels calls begin_call() first.
inline thread_local bool t_call_start = false;
inline void begin_call() { t_call_start = true; }

// Launch with programmatic stream serialization (see griddep_wait): the
// kernel may start while the previous kernel on the stream drains; the
// first launch after begin_call() is an ordinary launch.
template <typename... KArgs, typename... Args>
static inline cudaError_t launch_dependent(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                    Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = t_call_start ? 0 : 1;
  t_call_start = false;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

// bf16 rows: 16-byte vectors of 8 features
__device__ __forceinline__ uint4 ldg_u4(const void* p) {
  return __ldg(reinterpret_cast<const uint4*>(p));
}

// features [f, f+8) of a bf16 row, masked by N (the row stride is a multiple
// of 8 elements, so the 16-byte vector is in bounds whenever f < N)
__device__ __forceinline__ uint4 ld_row8_bf16(const uint16_t* row, int f, int N) {
  if (f + 7 < N) return ldg_u4(row + f);
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (f < N) {
    const uint4 t = ldg_u4(row + f);
    const int live = N - f;  // 1..7 features
    const uint32_t w[4] = {t.x, t.y, t.z, t.w};
    uint32_t o[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const uint32_t keep = (2 * i + 1 < live) ? 0xffffffffu : (2 * i < live ? 0x0000ffffu : 0u);
      o[i] = w[i] & keep;
    }
    v = make_uint4(o[0], o[1], o[2], o[3]);
  }
  return v;
}

// 8 bf16 values (feature order: low half of word 0 first) as two float4
__device__ __forceinline__ void bf16x8_to_f32(uint4 u, float4& lo, float4& hi) {
  lo = make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u), __uint_as_float(u.y << 16),
                   __uint_as_float(u.y & 0xffff0000u));
  hi = make_float4(__uint_as_float(u.z << 16), __uint_as_float(u.z & 0xffff0000u), __uint_as_float(u.w << 16),
                   __uint_as_float(u.w & 0xffff0000u));
}

__device__ __forceinline__ void fma4(float4& acc, float a, float4 b) {
  acc.x = fmaf(a, b.x, acc.x);
  acc.y = fmaf(a, b.y, acc.y);
  acc.z = fmaf(a, b.z, acc.z);
  acc.w = fmaf(a, b.w, acc.w);
}

__device__ __forceinline__ float dot4(float4 a, float4 b) {
  return fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, a.w * b.w)));
}

// ---------------------------------------------------------------------------
// shared memory / async proxy
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void st_shared_v2(uint32_t addr, uint32_t a, uint32_t b) {
  asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(addr), "r"(a), "r"(b) : "memory");
}

__device__ __forceinline__ void st_shared_u32(uint32_t addr, uint32_t a) {
  asm volatile("st.shared.b32 [%0], %1;" ::"r"(addr), "r"(a) : "memory");
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint4 v) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y),
               "r"(v.z), "r"(v.w)
               : "memory");
}

// make generic-proxy shared-memory writes visible to the async proxy
// (tcgen05.mma reads its operands through the async proxy)
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 16-byte asynchronous global -> shared copy; src_bytes < 16 zero-fills the
// rest (0 copies nothing, the address is not read)
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// arrive on an mbarrier once all of this thread's prior cp.async copies have
// landed (the barrier's expected count includes this arrival)
__device__ __forceinline__ void cp_async_mbar_arrive_noinc(uint32_t bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ uint4 ld_shared_v4(uint32_t addr) {
  uint4 v;
  asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "r"(addr)
               : "memory");
  return v;
}

// ---------------------------------------------------------------------------
// mbarrier
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.release.cta.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(bar)
      : "memory");
}

// Arrive on the barrier and raise its expected transaction bytes.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 st, [%0], %1;\n\t}\n" ::"r"(bar),
      "r"(bytes)
      : "memory");
}

// Bounded wait: gives up after `polls` polls (default 2^22; each try_wait
// suspends for a bounded, implementation-defined time) and reports failure
// to the caller.  After a few failed polls the thread sleeps between polls,
// so that waiting warps leave the issue slots to the warps doing the work.
constexpr uint32_t kDefaultPolls = 1u << 22;
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint32_t polls = kDefaultPolls) {
  for (uint32_t i = 0; i < polls; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i >= 4) __nanosleep(32);
  }
  return false;
}

// ---------------------------------------------------------------------------
// tcgen05 (5th-generation tensor core, accumulator in tensor memory)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem], kind::f16 (bf16 / fp16 inputs, fp32 accumulate)
__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// D[tmem] (+)= A[smem] * B[smem], kind::tf32 (fp32 storage, tf32 multiply,
// fp32 accumulate); K = 8 per instruction
__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// D[tmem] (+)= A[smem] * B[smem], kind::f8f6f4 (e4m3 inputs here, fp32
// accumulate); K = 32 per instruction
__device__ __forceinline__ void umma_f8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                        uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// arrive on an mbarrier once all previously issued tcgen05 ops of this thread finish
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

// 32 TMEM lanes x 16 columns of 32 bits -> 16 registers per thread
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor (tcgen05): start address, leading / stride
// byte offsets (16-byte units), version 1, layout type in bits 61-63.
enum SmemLayout : uint32_t { kSwizzleNone = 0, kSwizzle128B = 2, kSwizzle64B = 4, kSwizzle32B = 6 };

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo,
                                              uint32_t layout) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)(layout & 0x7u) << 61;
  return d;
}

// Instruction descriptor for kind::f16 / kind::tf32 / kind::f8f6f4 with fp32
// accumulate.  a_fmt/b_fmt: kind::f16 -> 0 = f16, 1 = bf16; kind::tf32 -> 2;
// kind::f8f6f4 -> 0 = e4m3.
// a_mn_major / b_mn_major: 1 = MN-major operand, 0 = K-major.
__host__ __device__ constexpr uint32_t make_idesc(uint32_t a_fmt, uint32_t b_fmt,
                                                  uint32_t a_mn_major, uint32_t b_mn_major,
                                                  uint32_t M, uint32_t N) {
  return (1u << 4)                 // D = f32
         | (a_fmt << 7) | (b_fmt << 10) | (a_mn_major << 15) | (b_mn_major << 16) |
         ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
// two floats -> two e4m3 bytes (round to nearest even, saturated to +-448),
// lo in the low byte
__device__ __forceinline__ uint32_t pack_e4m3x2(float lo, float hi) {
  unsigned short d;
  asm("cvt.rn.satfinite.e4m3x2.f32 %0, %1, %2;" : "=h"(d) : "f"(hi), "f"(lo));
  return (uint32_t)d;
}

__device__ __forceinline__ uint32_t pack_f16x2(float lo, float hi) {
  __half2 v = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

}  // namespace stile
