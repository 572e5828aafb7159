// mixed.cuh — shared declarations of the mixed-precision solver's pieces.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace bola {

// Tensor map for a K-major operand buffer of `rows` rows x 64 K values
// (bf16 or fp32 elements), boxes of 128 rows x 128 bytes, 128-byte swizzle.
int make_kmajor_map(CUtensorMap *map, const void *ptr, int64_t rows, bool bf16);

// W(m x n, column-major, ld ldw) -= A * B^T on tcgen05 (kind 0 bf16, 1 tf32,
// 2 3xTF32 with the lo maps); *err is set non-zero if a bounded wait expired.
int tc_update(cudaStream_t s, int kind, int64_t m, int64_t n, const CUtensorMap &A, const CUtensorMap &B,
              const CUtensorMap &Alo, const CUtensorMap &Blo, float *W, int64_t ldw, int32_t *err);

// Buffers and tensor maps of the low-precision LU (slu.cu), reusable across
// factorisations of size <= capacity.
struct MixedLU {
  int64_t n = 0, cap_n = 0;
  int kind = -1;  // 0 bf16, 1 tf32, 2 3xTF32 update operands
  void *aop = nullptr, *bop = nullptr;
  float *aop_lo = nullptr, *bop_lo = nullptr;
  int32_t *err = nullptr;
  int32_t *plan = nullptr;  // the current panel's composed interchanges: count, rows[128], src[128]
  CUtensorMap mapA, mapB, mapAlo, mapBlo;
  int reserve(int64_t n, int kind, cudaStream_t s);
  void release(cudaStream_t s);
  // LU with partial pivoting of the FP32 matrix W (n x n, ld ldw) in place.
  int factor(cudaStream_t s, float *W, int64_t ldw, int32_t *ipiv, int32_t *info);
};

}  // namespace bola
