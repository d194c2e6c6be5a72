// cblas_sgemm stand-in for building the reference's include/dsgl.hpp with -DUSE_MKL
// (MKL is not installed here).  Row-major only, which is all dsgl.hpp uses
// (dsgl.hpp:1241, 1290, 1309).  Each output element is a sequential-k sum of fused
// multiply-adds: the arithmetic contract the oracle and the CUDA kernels follow.
#pragma once
#include <cmath>

enum CBLAS_LAYOUT { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112 };

inline void mkl_set_num_threads(int) {}

inline void cblas_sgemm(CBLAS_LAYOUT, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int M, int N, int K,
                        float alpha, const float* A, int lda, const float* B, int ldb, float beta,
                        float* C, int ldc) {
  for (int i = 0; i < M; i++)
    for (int j = 0; j < N; j++) {
      float acc = 0.f;
      for (int k = 0; k < K; k++) {
        float a = ta == CblasNoTrans ? A[i * lda + k] : A[k * lda + i];
        float b = tb == CblasNoTrans ? B[k * ldb + j] : B[j * ldb + k];
        acc = fmaf(a, b, acc);
      }
      C[i * ldc + j] = beta == 0.f ? alpha * acc : alpha * acc + beta * C[i * ldc + j];
    }
}
