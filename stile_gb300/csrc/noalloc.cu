// Plain CSR SpMM for callers that must not allocate device memory.
//
// stile_csr_spmm_run reads a group -> first-row map (group_rows) that the
// caller builds and stores in a device buffer of its own.  Some callers
// cannot make that buffer: their device memory belongs to another
// allocator (a host framework's caching pool or an arena handed out up
// front), and a cudaMalloc / cudaFree of their own may also synchronise the
// device and stall every other stream.  stile_csr_spmm_run_noalloc builds
// the same map on the device, into the scratch array below, and then runs
// the same CSR kernel; it allocates nothing.
//
// The scratch array is part of the library image: every GPU that loads the
// library holds kCsrNoallocMaxGroups * 4 bytes (1 MiB) of it until the
// process exits.  All calls on a device share it, and it keeps whatever the
// last call wrote; every entry a call reads is written earlier in that same
// call (nothing has to start at zero), but calls whose kernels overlap on
// the GPU (different streams, no ordering between them) overwrite each
// other's map and race.
#include <cuda_runtime.h>

#include <string>

#include "../../include/stile_gb300.h"
#include "common.cuh"
#include "spmm.cuh"

namespace stile {

constexpr int kCsrNoallocMaxGroups = STILE_CSR_NOALLOC_MAX_GROUPS;
static_assert(kCsrNoallocMaxGroups == (1 << 18), "1 MiB of group -> row entries");

// group g -> the row holding nonzero g * kCsrGroupNnz
static __device__ __align__(256) int g_csr_group_rows[kCsrNoallocMaxGroups];

__global__ void csr_group_rows_kernel(int M, const int* __restrict__ indptr, int n_groups,
                                      int* __restrict__ group_rows) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_groups) return;
  const long t = (long)g * kCsrGroupNnz;
  // largest r with indptr[r] <= t: the row whose range holds nonzero t
  int lo = 0, hi = M;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(indptr + mid) <= t) lo = mid; else hi = mid;
  }
  group_rows[g] = lo;
}

// Device address of the scratch array on the current device, looked up on
// every call (cudaGetSymbolAddress allocates nothing and is cheap).  Not
// caching it keeps the address right after a cudaDeviceReset, which reloads
// the library's module at another address.  The first lookup on a device
// loads the module there, which is why the first call should come before
// any stream capture.
static cudaError_t scratch_for_current_device(int** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_csr_group_rows);
  if (e != cudaSuccess) return e;
  *out = static_cast<int*>(p);
  return cudaSuccess;
}

}  // namespace stile

extern "C" int stile_csr_spmm_run_noalloc(int32_t M, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                                          const float* vals, const float* B, int64_t ldb, float* C, int64_t ldc,
                                          int32_t N, void* stream) {
  if (M < 0 || N <= 0) return stile::report_error(STILE_E_INVALID, "bad shape");
  if (nnz < 0) return stile::report_error(STILE_E_INVALID, "negative nnz");
  const long max_nnz = (long)stile::kCsrNoallocMaxGroups * stile::kCsrGroupNnz;
  if (nnz > max_nnz) {
    const std::string msg = "nnz " + std::to_string((long long)nnz) +
                            " exceeds the no-allocation CSR limit of " + std::to_string(max_nnz) +
                            " nonzeros; use stile_csr_spmm_run with a caller-allocated group_rows map";
    return stile::report_error(STILE_E_INVALID, msg.c_str());
  }
  if (M == 0) return STILE_OK;
  if (!indptr || !indices || !vals || !B || !C) return stile::report_error(STILE_E_INVALID, "null array");
  if (ldb < N || ldb % 4 != 0 || ldc < N || ldc % 4 != 0)
    return stile::report_error(STILE_E_INVALID, "row strides must be >= N and multiples of 4");
  if ((reinterpret_cast<uintptr_t>(B) & 15) != 0 || (reinterpret_cast<uintptr_t>(C) & 15) != 0)
    return stile::report_error(STILE_E_INVALID, "B and C must be 16-byte aligned");
  stile::begin_call();
  int* group_rows = nullptr;
  cudaError_t e = stile::scratch_for_current_device(&group_rows);
  if (e != cudaSuccess) return stile::report_error(STILE_E_CUDA, cudaGetErrorString(e));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int n_groups = (int)((nnz + stile::kCsrGroupNnz - 1) / stile::kCsrGroupNnz);
  if (n_groups > 0) {
    stile::csr_group_rows_kernel<<<(n_groups + 255) / 256, 256, 0, st>>>(M, indptr, n_groups, group_rows);
    e = cudaGetLastError();
    if (e != cudaSuccess) return stile::report_error(STILE_E_CUDA, cudaGetErrorString(e));
  }
  e = stile::launch_csr_spmm(M, indptr, indices, vals, B, ldb, C, ldc, N, nnz, group_rows, st);
  if (e != cudaSuccess) return stile::report_error(STILE_E_CUDA, cudaGetErrorString(e));
  stile::note_launches(n_groups > 0 ? 2 : 1);
  return STILE_OK;
}
