// Tensor-core (tcgen05 / TMEM / TMA) GEMM engine for sm_103a.
//
// C[m][n] = alpha * sum_k A[m][k] * B[n][k]   ("TN": both operands K-major)
// with BF16 operands and FP32 accumulation in tensor memory.  In 3xBF16 mode
// each operand is the unevaluated sum hi + lo of two BF16 arrays and the
// kernel accumulates hi*hi + hi*lo + lo*hi, which carries about 16
// significant bits per operand (split-precision product).
#pragma once
#include <cuda_bf16.h>

#include "ctm_common.cuh"

namespace ctm {

using bf16 = __nv_bfloat16;

enum class TcMode { kBf16x1 = 1, kBf16x3 = 3 };

// K-major BF16 operand: rows x k, leading dimension ld (elements, multiple of 8).
struct TcOperand {
  const bf16* hi = nullptr;
  const bf16* lo = nullptr;  // required in 3xBF16 mode
  int64_t rows = 0, k = 0, ld = 0;
};

// Destinations of the reduced result (any subset).
struct TcOut {
  double alpha = 1.0;
  double* f64 = nullptr;       // C (M x N) row-major with ld_f64, or C^T when f64_trans
  int64_t ld_f64 = 0;
  bool f64_trans = false;
  float* f32 = nullptr;        // C (M x N) row-major with ld_f32
  int64_t ld_f32 = 0;
  bf16* hi_t = nullptr;        // C^T (N x M) split into BF16 hi (+ lo), ld_t
  bf16* lo_t = nullptr;
  int64_t ld_t = 0;
};

// Leading dimension used for BF16 operand arrays of width k.
inline int64_t tc_ld(int64_t k) { return (k + 63) / 64 * 64; }

void tc_gemm(Ctx& c, const TcOperand& A, const TcOperand& B, TcMode mode, const TcOut& out);

// src (rows x cols FP64, leading dimension ld_src) -> hi/lo BF16 split; with
// transpose the destination is (cols x rows).  lo may be null.
void split_bf16(Ctx& c, const double* src, int64_t rows, int64_t cols, int64_t ld_src,
                bool transpose, bf16* hi, bf16* lo, int64_t ld_dst);

}  // namespace ctm
