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

// Output layout: offset(m, n) = sum_j i_j(m) * ms[j] + sum_j i_j(n) * ns[j]
// where m and n are decoded mixed-radix over (me[0..nm), last fastest);
// up to six modes each.
constexpr int kTcModes = 6;
struct TcLayout {
  int nm = 1, nn = 1;
  int64_t me[kTcModes] = {1, 1, 1, 1, 1, 1}, ms[kTcModes] = {0, 0, 0, 0, 0, 0};
  int64_t ne[kTcModes] = {1, 1, 1, 1, 1, 1}, ns[kTcModes] = {0, 0, 0, 0, 0, 0};
  static TcLayout rows(int64_t M, int64_t N, int64_t ld) {  // C[m][n] at m*ld + n
    TcLayout l;
    l.me[0] = M; l.ms[0] = ld; l.ne[0] = N; l.ns[0] = 1;
    return l;
  }
  static TcLayout cols(int64_t M, int64_t N, int64_t ld) {  // C[m][n] at n*ld + m
    TcLayout l;
    l.me[0] = M; l.ms[0] = 1; l.ne[0] = N; l.ns[0] = ld;
    return l;
  }
};

enum class TcKind { kF64 = 0, kF32 = 1, kBf16Hi = 2, kBf16Lo = 3 };

struct TcDest {
  TcKind kind = TcKind::kF64;
  void* p = nullptr;
  TcLayout lay;
};

// Destinations of the reduced result: alpha * C written to every entry of d.
struct TcOut {
  double alpha = 1.0;
  const double* inv_scale = nullptr;   // device scalars: results are divided by *inv_scale
  const double* inv_scale2 = nullptr;  // and by *inv_scale2 when non-null
  int extra_tag = -1;                  // profiling class timed besides "tensor-core GEMM"
  const char* name = nullptr;          // kernel-class name in the per-kernel profile
  double algo_flops = -1.0;            // algorithmic FLOPs of the product (default 2 M N K)
  int nd = 0;
  TcDest d[4];
  TcOut& add(TcKind k, void* p, const TcLayout& l) {
    d[nd].kind = k;
    d[nd].p = p;
    d[nd].lay = l;
    ++nd;
    return *this;
  }
};

// Leading dimension used for BF16 operand arrays of width k.
inline int64_t tc_ld(int64_t k) { return (k + 63) / 64 * 64; }

void tc_gemm(Ctx& c, const TcOperand& A, const TcOperand& B, TcMode mode, const TcOut& out);

// As tc_gemm without a K split, and also writes max |output| to *absmax
// (device scalar, FP32-accumulated values).
void tc_gemm_absmax(Ctx& c, const TcOperand& A, const TcOperand& B, TcMode mode,
                    const TcOut& out, double* absmax);

// dst (cols x rows, leading dimension ld_dst) = src^T for BF16 hi and lo
// arrays (src rows x cols, leading dimension ld_src); lo pointers may be null.
void transpose_bf16(Ctx& c, const bf16* src_hi, const bf16* src_lo, int64_t rows, int64_t cols,
                    int64_t ld_src, bf16* dst_hi, bf16* dst_lo, int64_t ld_dst);

// out (rows x cols FP64, contiguous) = hi + lo (BF16, leading dimension ld).
void join_bf16(Ctx& c, const bf16* hi, const bf16* lo, int64_t rows, int64_t cols, int64_t ld,
               double* out);

// Gather-and-split of a strided FP64 tensor into a K-major BF16 operand:
// dst[r][k] (ld) = src[off(r, k)], off decoded mixed-radix from row modes
// (re, rs) and column modes (ke, ks), last mode fastest.
struct Gather {
  int nr = 1, nk = 1;
  int64_t re[4] = {1, 1, 1, 1}, rs[4] = {0, 0, 0, 0};
  int64_t ke[4] = {1, 1, 1, 1}, ks[4] = {0, 0, 0, 0};
};
void gather_split_bf16(Ctx& c, const double* src, const Gather& g, bf16* hi, bf16* lo,
                       int64_t ld);
void gather_split_bf16(Ctx& c, const float* src, const Gather& g, bf16* hi, bf16* lo,
                       int64_t ld);

// src (rows x cols FP64, leading dimension ld_src) -> hi/lo BF16 split; with
// transpose the destination is (cols x rows).  lo may be null.
void split_bf16(Ctx& c, const double* src, int64_t rows, int64_t cols, int64_t ld_src,
                bool transpose, bf16* hi, bf16* lo, int64_t ld_dst);
void split_bf16(Ctx& c, const float* src, int64_t rows, int64_t cols, int64_t ld_src,
                bool transpose, bf16* hi, bf16* lo, int64_t ld_dst);

}  // namespace ctm
