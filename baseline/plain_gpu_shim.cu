// Library calls of the reference's plain GPU path, for the comparator arm of
// bench.py (never part of the product library).
//
// The reference drives cuFFT and cuBLAS through two small C wrappers:
//  * albatros_analysis/src/utils/pycufft.cu:68-199 and :201-324 — batched 1-D
//    R2C / C2R transforms along the last axis, out of place, from plans made
//    once per (batch, n, type) with automatic work-area allocation off and
//    one caller-owned work area shared by every plan (PlanCache,
//    albatros_analysis/src/utils/pycufft.py:27-81); no scaling (the Python
//    side divides by n after a C2R);
//  * albatros_analysis/src/correlations/cgemm_batch.cu:8-53 — C = A * B^H per
//    batch with cublasCgemmStridedBatched, column-major, lda = M, ldb = N,
//    ldc = M, strides M*K, N*K, M*N, with a cuBLAS handle created and
//    destroyed on every call.
// This file makes the same library calls through its own entry points; it is
// written here, not taken from the reference.  Every entry returns 0 on
// success and a nonzero library status otherwise (nothing prints or exits).
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <cstddef>
#include <cstdint>

struct pg_plan {
  cufftHandle h;
  int type;  // 0 = R2C, 1 = C2R
};

extern "C" {

// Plan `batch` transforms of length n; *work_bytes receives the work-area
// size the plan needs (set with pg_fft_set_work before the first exec).
int pg_fft_plan(int type, int batch, int n, void** plan_out, size_t* work_bytes) {
  if (!plan_out || !work_bytes || batch < 1 || n < 2 || (type != 0 && type != 1)) return -1;
  pg_plan* p = new pg_plan{0, type};
  cufftResult r = cufftCreate(&p->h);
  if (r == CUFFT_SUCCESS) r = cufftSetAutoAllocation(p->h, 0);
  if (r == CUFFT_SUCCESS) r = cufftMakePlan1d(p->h, n, type == 0 ? CUFFT_R2C : CUFFT_C2R, batch, work_bytes);
  if (r != CUFFT_SUCCESS) {
    cufftDestroy(p->h);
    delete p;
    return (int)r;
  }
  *plan_out = p;
  return 0;
}

int pg_fft_set_work(void* plan, void* work) {
  if (!plan) return -1;
  return (int)cufftSetWorkArea(static_cast<pg_plan*>(plan)->h, work);
}

int pg_fft_exec(void* plan, const void* in, void* out, void* stream) {
  if (!plan || !in || !out) return -1;
  pg_plan* p = static_cast<pg_plan*>(plan);
  cufftResult r = cufftSetStream(p->h, static_cast<cudaStream_t>(stream));
  if (r != CUFFT_SUCCESS) return (int)r;
  if (p->type == 0)
    r = cufftExecR2C(p->h, (cufftReal*)in, (cufftComplex*)out);
  else
    r = cufftExecC2R(p->h, (cufftComplex*)in, (cufftReal*)out);
  return (int)r;
}

int pg_fft_destroy(void* plan) {
  if (!plan) return 0;
  pg_plan* p = static_cast<pg_plan*>(plan);
  int r = (int)cufftDestroy(p->h);
  delete p;
  return r;
}

// C[:, :, b] = A[:, :, b] * B[:, :, b]^H for b < batch (complex64,
// column-major; A is M x K, B is N x K, C is M x N per batch).
int pg_cgemm_strided_batched(const void* A, const void* B, void* C, int M, int N, int K, int batch, void* stream) {
  if (!A || !B || !C || M < 1 || N < 1 || K < 1 || batch < 1) return -1;
  cublasHandle_t h;
  cublasStatus_t st = cublasCreate(&h);
  if (st != CUBLAS_STATUS_SUCCESS) return (int)st;
  st = cublasSetStream(h, static_cast<cudaStream_t>(stream));
  const cuComplex one = make_cuComplex(1.f, 0.f), zero = make_cuComplex(0.f, 0.f);
  if (st == CUBLAS_STATUS_SUCCESS)
    st = cublasCgemmStridedBatched(h, CUBLAS_OP_N, CUBLAS_OP_C, M, N, K, &one, (const cuComplex*)A, M,
                                   (long long)M * K, (const cuComplex*)B, N, (long long)N * K, &zero, (cuComplex*)C,
                                   M, (long long)M * N, batch);
  cublasStatus_t d = cublasDestroy(h);
  return st != CUBLAS_STATUS_SUCCESS ? (int)st : (int)d;
}

}  // extern "C"
