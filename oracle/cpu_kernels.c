/*
 * CPU oracle kernels (TEST INFRASTRUCTURE: used by tests/, smoke() and the
 * CPU-baseline leg of bench.py only).
 *
 * The reference's CPU comparison for this path is scipy / torch CSR SpMM and
 * a gather-dot SDDMM on the host cores (the reference's accuracy check
 * multiplies A.dot(B) with scipy, MY_sparse/my_fuse_formats.py:4197-4214;
 * its SDDMM golden is DGL u_dot_v, :4331-4341).  These are the same
 * operations in plain C with pthreads, fp32 data and fp32 accumulation,
 * rows / nonzeros split evenly over the threads.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int64_t r0, r1;
  const int32_t* indptr;
  const int32_t* indices;
  const float* vals;
  const float* B;
  int64_t ldb;
  float* C;
  int64_t ldc;
  int32_t N;
} spmm_job;

static void* spmm_worker(void* arg) {
  spmm_job* j = (spmm_job*)arg;
  for (int64_t r = j->r0; r < j->r1; ++r) {
    float* c = j->C + r * j->ldc;
    memset(c, 0, sizeof(float) * (size_t)j->N);
    for (int32_t p = j->indptr[r]; p < j->indptr[r + 1]; ++p) {
      const float v = j->vals[p];
      const float* b = j->B + (int64_t)j->indices[p] * j->ldb;
      for (int32_t f = 0; f < j->N; ++f) c[f] += v * b[f];
    }
  }
  return NULL;
}

int oracle_csr_spmm(int32_t M, const int32_t* indptr, const int32_t* indices, const float* vals,
                    const float* B, int64_t ldb, float* C, int64_t ldc, int32_t N, int32_t threads) {
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t tid[256];
  spmm_job jobs[256];
  /* balance by nonzeros */
  const int64_t nnz = indptr[M];
  int64_t r = 0;
  for (int t = 0; t < threads; ++t) {
    const int64_t target = nnz * (t + 1) / threads;
    int64_t r1 = r;
    while (r1 < M && indptr[r1] < target) ++r1;
    if (t == threads - 1) r1 = M;
    spmm_job j = {r, r1, indptr, indices, vals, B, ldb, C, ldc, N};
    jobs[t] = j;
    r = r1;
  }
  for (int t = 0; t < threads; ++t) pthread_create(&tid[t], NULL, spmm_worker, &jobs[t]);
  for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
  return 0;
}

typedef struct {
  int64_t t0, t1;
  const int32_t* rows;
  const int32_t* cols;
  const float* X;
  int64_t ldx;
  const float* Y;
  int64_t ldy;
  float* out;
  int32_t F;
} sddmm_job;

static void* sddmm_worker(void* arg) {
  sddmm_job* j = (sddmm_job*)arg;
  for (int64_t t = j->t0; t < j->t1; ++t) {
    const float* x = j->X + (int64_t)j->rows[t] * j->ldx;
    const float* y = j->Y + (int64_t)j->cols[t] * j->ldy;
    float s = 0.f;
    for (int32_t f = 0; f < j->F; ++f) s += x[f] * y[f];
    j->out[t] = s;
  }
  return NULL;
}

int oracle_sddmm(int64_t nnz, const int32_t* rows, const int32_t* cols, const float* X, int64_t ldx,
                 const float* Y, int64_t ldy, float* out, int32_t F, int32_t threads) {
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t tid[256];
  sddmm_job jobs[256];
  for (int t = 0; t < threads; ++t) {
    sddmm_job j = {nnz * t / threads, nnz * (t + 1) / threads, rows, cols, X, ldx, Y, ldy, out, F};
    jobs[t] = j;
  }
  for (int t = 0; t < threads; ++t) pthread_create(&tid[t], NULL, sddmm_worker, &jobs[t]);
  for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
  return 0;
}
