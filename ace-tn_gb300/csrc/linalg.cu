// FP64 dense linear algebra for the projector construction:
//  * orthonormalize(): QR of a tall-skinny matrix.  Shifted Cholesky-QR3
//    (Fukaya, Kannan, Nakatsukasa, Yamamoto, Yanagisawa, SIAM J. Sci. Comput.
//    42 (2020) A477) built on the GETT engine, with an orthogonality check
//    and a one-CTA Householder QR that runs instead when the check fails
//    (numerically rank-deficient input) or the problem is small.
//  * svd_thin(): one-sided (Hestenes) Jacobi SVD with the round-robin pair
//    ordering, run as a cooperative multi-CTA kernel with a bounded grid
//    barrier (Demmel & Veselic, SIAM J. Matrix Anal. Appl. 13 (1992) 1204).
//  * truncation of the singular spectrum and column scaling of the
//    projectors (acetn/renormalization/projectors.py:163-167).
#include "engine.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <type_traits>
#include <cmath>

namespace ctm {

namespace {

__device__ int g_status_flags;
__device__ unsigned long long g_qr_fallbacks;

// Asynchronous global -> shared copies (cp.async): 16 bytes, or one element
// of 4 or 8 bytes; cp_async_wait_all() waits for this thread's copies.
__device__ __forceinline__ void cp_async_f32x4(float* s, const float* g) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(s));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_f32(float* s, const float* g) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(s));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_elem(float* s, const float* g) { cp_async_f32(s, g); }
__device__ __forceinline__ void cp_async_elem(double* s, const double* g) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(s));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Paired FP32 FMA of Blackwell (fma.rn.f32x2): d = a * b + c in each lane,
// rounded as fmaf, one instruction for two.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;"
      : "=l"(d)
      : "l"(*reinterpret_cast<unsigned long long*>(&a)),
        "l"(*reinterpret_cast<unsigned long long*>(&b)),
        "l"(*reinterpret_cast<unsigned long long*>(&c)));
  return *reinterpret_cast<float2*>(&d);
}

constexpr int LT = 256;  // threads of one-CTA linear-algebra kernels

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum (all threads get the result).  sh must hold LT/32 values.
template <class T>
__device__ T block_sum(T v, T* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  T t = T(0);
  for (int i = 0; i < int(blockDim.x >> 5); ++i) t += sh[i];
  return t;
}

// ------------------------------------------------------------- Householder QR
// One CTA.  Y (n x q, row-major) is overwritten by the explicit Q; R (q x q)
// receives the triangular factor when non-null.  V (n x q) and beta (q) are
// scratch.  Runs only when (flags == nullptr) or (*flags & 1) != 0, and then
// first copies restore (n x q, when non-null) into Y.
template <class T>
__global__ void __launch_bounds__(LT) householder_qr_kernel(T* Y, int64_t n, int64_t q,
                                                            T* R, T* V, T* beta,
                                                            const int* flags, int clear_bit,
                                                            const T* restore = nullptr) {
  if (flags != nullptr && ((*flags) & clear_bit) == 0) return;
  if (flags != nullptr && threadIdx.x == 0) atomicAdd(&g_qr_fallbacks, 1ull);
  if (restore != nullptr) {
    for (int64_t i = threadIdx.x; i < n * q; i += LT) Y[i] = restore[i];
    __syncthreads();
  }
  __shared__ T sh[LT / 32];
  __shared__ T s_beta, s_alpha;
  for (int64_t j = 0; j < q; ++j) {
    // norm of the column below the diagonal
    T part = T(0);
    for (int64_t i = j + threadIdx.x; i < n; i += LT) {
      const T x = Y[i * q + j];
      part = fma(x, x, part);
    }
    const T nrm2 = block_sum(part, sh);
    if (threadIdx.x == 0) {
      const T x0 = Y[j * q + j];
      const T nrm = sqrt(nrm2);
      if (nrm == T(0)) {
        s_alpha = T(0);
        s_beta = T(0);
      } else {
        const T alpha = x0 >= T(0) ? -nrm : nrm;
        const T v0 = x0 - alpha;
        // v = x - alpha e1, stored with v0 in place; beta = 2 / (v^T v)
        const T vtv = nrm2 - x0 * x0 + v0 * v0;
        s_alpha = alpha;
        s_beta = vtv > T(0) ? T(2) / vtv : T(0);
        Y[j * q + j] = v0;
      }
    }
    __syncthreads();
    const T bj = s_beta;
    for (int64_t i = j + threadIdx.x; i < n; i += LT) V[i * q + j] = Y[i * q + j];
    __syncthreads();
    // trailing update Y[j:, j+1:] -= beta v (v^T Y)
    for (int64_t c = j + 1; c < q; ++c) {
      T d = T(0);
      for (int64_t i = j + threadIdx.x; i < n; i += LT) d = fma(V[i * q + j], Y[i * q + c], d);
      const T w = block_sum(d, sh) * bj;
      for (int64_t i = j + threadIdx.x; i < n; i += LT) Y[i * q + c] -= w * V[i * q + j];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      beta[j] = bj;
      Y[j * q + j] = s_alpha;  // R diagonal
    }
    __syncthreads();
  }
  if (R != nullptr) {
    for (int64_t idx = threadIdx.x; idx < q * q; idx += LT) {
      const int64_t r = idx / q, c = idx % q;
      R[idx] = (c >= r) ? Y[r * q + c] : T(0);
    }
  }
  __syncthreads();
  // explicit Q = H_0 ... H_{q-1} [I; 0], applied right to left
  for (int64_t idx = threadIdx.x; idx < n * q; idx += LT) {
    const int64_t r = idx / q, c = idx % q;
    Y[idx] = (r == c) ? T(1) : T(0);
  }
  __syncthreads();
  for (int64_t j = q - 1; j >= 0; --j) {
    const T bj = beta[j];
    if (bj == T(0)) continue;
    for (int64_t c = j; c < q; ++c) {
      T d = T(0);
      for (int64_t i = j + threadIdx.x; i < n; i += LT) d = fma(V[i * q + j], Y[i * q + c], d);
      const T w = block_sum(d, sh) * bj;
      for (int64_t i = j + threadIdx.x; i < n; i += LT) Y[i * q + c] -= w * V[i * q + j];
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------- Cholesky
// One CTA of kCholThreads threads factorises G + shift I = L L^T (q x q).
// Right-looking elimination on the upper triangle with the pivot division
// deferred: step j subtracts (W[j][i] / W[j][j]) * row j from every row
// i > j, so row j ends as d_j * (row j of L_unit^T) with d_j = W[j][j], and
// L^T[j][c] = W[j][c] / sqrt(d_j).  When Linv is requested the same row
// operations run on an identity block E, which ends as L_unit^-1, and
// L^-1 = diag(d)^-1/2 E.
//
// The pivots go in blocks of kCholNb: (a) one thread eliminates inside the
// kCholNb x kCholNb diagonal block and publishes pivots and multipliers;
// (b) one thread per column applies them to the block's pivot rows (of W,
// and of E on other threads) and stores the scaled multipliers
// S[t][i] = W[J+t][i] / d_t of the rows below; (c) every thread takes 4 x 4
// tiles of the trailing rows (W: upper-triangular tiles only) and subtracts
// sum_t S[t][i] row_(J+t) with 128-bit shared-memory accesses.  (A
// look-ahead, warp 0 eliminating the next diagonal block during (c), saved
// under 1% at q = 160: (a) outlasts the rest of (c) in most blocks.)
// W and E are q4 x ld (q4 = q rounded up to kCholNb, ld = q4 + 4) with zero
// padding, so the pivot rows of the last block and every 4 x 4 tile are in
// bounds.
//
// A pivot that is not positive (numerically semidefinite G) contributes a
// zero column to L and a zero row to L^-1, and sets bit 1 of *flags.
// shift_mode 0: none; 1: 11 (n q + q (q + 1)) u tr(G) (Fukaya et al.);
// 2: 1000 u tr(G) (FP32 stages of the mixed path).
// Outputs (each may be null): Lout = L (lower, row-major), Linv = L^-1
// (lower), Lt = L^T (upper), LinvT = L^-T (upper).  Wg / Eg are cholesky_scratch(q) elements of
// global scratch used for W / E when they are not in shared memory.
constexpr int kCholThreads = 1024;
constexpr int kCholNb = 8;
constexpr size_t kSmemOptin = 227 * 1024;

__host__ __device__ inline int chol_q4(int q) { return (q + kCholNb - 1) / kCholNb * kCholNb; }
__host__ __device__ inline int chol_ld(int q) { return chol_q4(q) + 4; }
inline size_t cholesky_scratch(int64_t q) { return size_t(chol_q4(int(q))) * chol_ld(int(q)); }

template <class T>
struct Vec4;
template <>
struct Vec4<float> {
  using type = float4;
};
template <>
struct Vec4<double> {
  using type = double4_32a;
};

// kPlace: 0 = W and E in global scratch, 1 = W in shared memory, 2 = both
// in shared memory (a compile-time choice, so shared accesses stay LDS/STS).
// FP64 tiles need twice the registers: 512 threads for T = double.
template <class T>
constexpr int chol_threads() { return sizeof(T) == 8 ? 512 : kCholThreads; }

// (a) for the diagonal block at rows / columns [J, J + jb) of W, by one
// thread with the block in registers (fully unrolled: every index is a
// compile-time constant): pivots d_t, 1 / d_t and multipliers W[t][v] / d_t.
template <class T>
__device__ __forceinline__ void chol_diag_block(const T* W, int ld, int J, int jb, T* s_d,
                                                T* s_rd, T (*s_mul)[kCholNb], int* s_fail) {
  T blk[kCholNb][kCholNb];
#pragma unroll
  for (int t = 0; t < kCholNb; ++t)
#pragma unroll
    for (int v = 0; v < kCholNb; ++v)
      blk[t][v] = (v >= t && t < jb && v < jb) ? W[(J + t) * ld + J + v] : T(0);
  bool fail = false;
#pragma unroll
  for (int t = 0; t < kCholNb; ++t) {
    const T dt = blk[t][t];
    const bool ok = t < jb && dt > T(0);
    fail = fail || (t < jb && !ok);
    s_d[t] = ok ? dt : T(0);
    // FP32: the hardware reciprocal (about 1 ulp) instead of the IEEE
    // division sequence on this serial chain; FP64 keeps the division
    T rinv = T(0);
    if (ok) {
      if constexpr (sizeof(T) == 4) rinv = __fdividef(1.f, dt);
      else rinv = T(1) / dt;
    }
    s_rd[t] = rinv;
    T m[kCholNb];
#pragma unroll
    for (int v = 0; v < kCholNb; ++v) {
      m[v] = v > t ? blk[t][v] * rinv : T(0);
      s_mul[t][v] = m[v];
    }
#pragma unroll
    for (int r = t + 1; r < kCholNb; ++r)
#pragma unroll
      for (int v = r; v < kCholNb; ++v) blk[r][v] -= m[r] * blk[t][v];
  }
  if (fail) *s_fail = 1;
}

template <class T, int kPlace>
__global__ void __launch_bounds__(chol_threads<T>()) cholesky_kernel(
    const T* G, int q, int64_t n, int shift_mode, T* Wg, T* Eg, T* Lout, T* Linv, T* Lt,
    T* LinvT, int* flags) {
  using V4 = typename Vec4<T>::type;
  extern __shared__ __align__(32) unsigned char chol_smem[];
  __shared__ T sh[32];
  __shared__ T s_d[kCholNb];
  __shared__ T s_rd[kCholNb];
  __shared__ T s_mul[kCholNb][kCholNb];
  __shared__ int s_fail;
  const int q4 = chol_q4(q), ld = chol_ld(q);
  T* dg = reinterpret_cast<T*>(chol_smem);              // q4: sqrt(d_j)
  T* rdg = dg + q4;                                      // q4: 1 / sqrt(d_j)
  T* S = rdg + q4;                                       // kCholNb x ld
  T* W = kPlace >= 1 ? S + kCholNb * ld : Wg;            // q4 x ld
  T* E = kPlace == 2 ? W + size_t(q4) * ld : Eg;         // q4 x ld
  const bool want_inv = Linv != nullptr || LinvT != nullptr;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5, nth = blockDim.x;
  // trace -> shift (every thread ends with the same value)
  T tr = T(0);
  for (int i = tid; i < q; i += nth) tr += G[size_t(i) * q + i];
  tr = warp_sum(tr);
  if (lane == 0) sh[warp] = tr;
  if (tid == 0) s_fail = 0;
  __syncthreads();
  tr = T(0);
  for (int w = 0; w < nwarps; ++w) tr += sh[w];
  const double u = sizeof(T) == 8 ? 1.1102230246251565e-16 : 5.9604644775390625e-08;
  double factor = 0.0;
  if (shift_mode == 1) factor = 11.0 * (double(n) * q + double(q) * (q + 1));
  if (shift_mode == 2) factor = 1000.0;
  const T shift = T(factor * u * double(tr));
  // W = upper triangle of G (asynchronous copies when W is in shared
  // memory, so that the loads overlap), zero elsewhere; E = I
  // (rows over warps, columns over lanes: no index division)
  for (int r = warp; r < q4; r += nwarps)
    for (int c = lane; c < ld; c += 32) {
      const int idx = r * ld + c;
      const bool from_g = r < q && c < q && c >= r;
      if (kPlace >= 1 && from_g)
        cp_async_elem(W + idx, G + size_t(r) * q + c);
      else
        W[idx] = from_g ? G[size_t(r) * q + c] : T(0);
      if (want_inv) E[idx] = (r == c) ? T(1) : T(0);
    }
  if (kPlace >= 1) cp_async_wait_all();
  __syncthreads();
  for (int j = tid; j < q; j += nth) W[j * ld + j] += shift;
  __syncthreads();
  for (int J = 0; J < q; J += kCholNb) {
    if (tid == 0) chol_diag_block(W, ld, J, min(kCholNb, q - J), s_d, s_rd, s_mul, &s_fail);
    __syncthreads();
    // (b) pivot rows at every column k >= J (threads from 0 up), and the
    //     pivot rows of E at the columns c < J + kCholNb (threads from the
    //     top down); s_mul is read from shared memory: a broadcast, and it
    //     keeps registers free
    const int nE = want_inv ? min(J + kCholNb, q4) : 0;
    for (int k = J + tid; k < q4; k += nth) {
      T x[kCholNb];
#pragma unroll
      for (int t = 0; t < kCholNb; ++t) x[t] = (J + t <= k) ? W[(J + t) * ld + k] : T(0);
#pragma unroll
      for (int t = 0; t < kCholNb; ++t)
#pragma unroll
        for (int r = t + 1; r < kCholNb; ++r) x[r] -= s_mul[t][r] * x[t];
#pragma unroll
      for (int t = 0; t < kCholNb; ++t) {
        if (J + t <= k) W[(J + t) * ld + k] = x[t];
        S[t * ld + k] = k >= J + kCholNb ? x[t] * s_rd[t] : T(0);
      }
    }
    for (int c = nth - 1 - tid; c < nE; c += nth) {
      T x[kCholNb];
#pragma unroll
      for (int t = 0; t < kCholNb; ++t) x[t] = E[(J + t) * ld + c];
#pragma unroll
      for (int t = 0; t < kCholNb; ++t)
#pragma unroll
        for (int r = t + 1; r < kCholNb; ++r) x[r] -= s_mul[t][r] * x[t];
#pragma unroll
      for (int t = 0; t < kCholNb; ++t) E[(J + t) * ld + c] = x[t];
    }
    __syncthreads();
    // (c) trailing rows i >= i0 in 4 x 4 tiles:
    //     W[i][k] -= sum_t S[t][i] W[J+t][k] (k >= i), E[i][c] likewise (c < i0).
    //     Tiles t < tw are the upper-triangular W tiles in row-major order
    //     (tile row bi starts at bi nbr - bi (bi - 1) / 2), then the E tiles.
    const int i0 = J + kCholNb;
    const int nbr = i0 < q4 ? (q4 - i0) / 4 : 0;  // tile rows (and columns) of W; even
    const int nbc = want_inv ? min(i0, q4) / 4 : 0;
    const int tw = nbr * (nbr + 1) / 2, te = nbr * nbc;
    auto tile = [&](int t) {
      int row0, col0;
      T* Dst;
      const T* Piv;
      if (t < tw) {
        const int m = 2 * nbr + 1;
        int bi = int((float(m) - sqrtf(float(m * m - 8 * t))) * 0.5f);
        bi = max(0, min(bi, nbr - 1));
        while (bi + 1 < nbr && (bi + 1) * nbr - (bi + 1) * bi / 2 <= t) ++bi;
        while (bi * nbr - bi * (bi - 1) / 2 > t) --bi;
        const int bk = bi + (t - (bi * nbr - bi * (bi - 1) / 2));
        row0 = i0 + 4 * bi;
        col0 = i0 + 4 * bk;
        Dst = W;
        Piv = W + J * ld;
      } else {
        const int e = t - tw;
        const int bi = e / nbc;
        row0 = i0 + 4 * bi;
        col0 = 4 * (e - bi * nbc);
        Dst = E;
        Piv = E + J * ld;
      }
      T acc[4][4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = T(0);
#pragma unroll
      for (int t2 = 0; t2 < kCholNb; ++t2) {
        const V4 a = *reinterpret_cast<const V4*>(S + t2 * ld + row0);
        const V4 pv = *reinterpret_cast<const V4*>(Piv + t2 * ld + col0);
        const T av[4] = {a.x, a.y, a.z, a.w}, pw[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) acc[r][c] = fma(av[r], pw[c], acc[r][c]);
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        V4* d4 = reinterpret_cast<V4*>(Dst + (row0 + r) * ld + col0);
        V4 w = *d4;
        w.x -= acc[r][0];
        w.y -= acc[r][1];
        w.z -= acc[r][2];
        w.w -= acc[r][3];
        *d4 = w;
      }
    };
    for (int t = tid; t < tw + te; t += nth) tile(t);
    __syncthreads();
  }
  if (tid == 0 && s_fail) atomicOr(flags, 1);
  for (int j = tid; j < q; j += nth) {
    const T dj = W[j * ld + j];
    const T sq = dj > T(0) ? sqrt(dj) : T(0);
    dg[j] = sq;
    rdg[j] = dj > T(0) ? T(1) / sq : T(0);
  }
  __syncthreads();
  for (int r = warp; r < q; r += nwarps)
    for (int c = lane; c < q; c += 32) {
      const int idx = r * q + c;
      if (Lout != nullptr)
        Lout[idx] = c < r ? W[c * ld + r] * rdg[c] : (c == r ? dg[c] : T(0));
      if (Lt != nullptr)
        Lt[idx] = c > r ? W[r * ld + c] * rdg[r] : (c == r ? dg[r] : T(0));
      if (Linv != nullptr) Linv[idx] = c <= r ? E[r * ld + c] * rdg[r] : T(0);
      if (LinvT != nullptr) LinvT[idx] = r <= c ? E[c * ld + r] * rdg[c] : T(0);
    }
}

// Launches cholesky_kernel with W and E in shared memory whenever both fit,
// else W alone.  Wg / Eg: cholesky_scratch(q) elements each, used for what
// is not in shared memory.
template <class T>
void cholesky(cudaStream_t st, const T* G, int64_t q, int64_t n, int shift_mode, T* Wg, T* Eg,
              T* Lout, T* Linv, T* Lt, int* flags, T* LinvT = nullptr) {
  const size_t mat = cholesky_scratch(q) * sizeof(T);
  const size_t head = (2 * size_t(chol_q4(int(q))) + size_t(kCholNb) * chol_ld(int(q))) * sizeof(T);
  // both scratch matrices in shared memory whenever they fit, also without
  // the inverse (that variant of the kernel compiles without spills)
  const int place = (head + 2 * mat <= kSmemOptin) ? 2 : (head + mat <= kSmemOptin ? 1 : 0);
  const size_t smem = head + (place >= 1 ? mat : 0) + (place == 2 ? mat : 0);
  auto launch = [&](auto kern) {
    CTM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    KernelTimer kt(st, sizeof(T) == 8 ? "cholesky_kernel<double>" : "cholesky_kernel<float>",
                   kUnitFlop, double(q) * q * q / 3.0);
    kern<<<1, chol_threads<T>(), smem, st>>>(G, int(q), n, shift_mode, Wg, Eg, Lout, Linv, Lt,
                                             LinvT, flags);
  };
  if (place == 2) launch(cholesky_kernel<T, 2>);
  else if (place == 1) launch(cholesky_kernel<T, 1>);
  else launch(cholesky_kernel<T, 0>);
  CTM_LAUNCH_CHECK();
}

// One-sided (Hestenes) Jacobi in FP32 on one CTA: the q rows of Mc (the
// columns of M = L^T, length q) are made mutually orthogonal by plane
// rotations, which are accumulated as rows of Jc.  Singular values are the
// final row norms; with M = L^T, L = J Sigma W^T, so the left singular
// vectors of L are the columns of J, orthogonal to working precision (the
// rotations are), which keeps V = B^T U / s accurate for small s as well.
// 8 threads per pair, each owning float4 chunks of the two rows: rows are
// padded with zeros to ld = jacobi_ld(q) (a multiple of 32 floats), so a
// warp's four groups read four 128-byte row segments per access phase.
// Mc and Jc live in shared memory (kSmem) or in the global scratch Wg
// (2 q ld floats).
__host__ __device__ inline int jacobi_ld(int q) { return (q + 31) / 32 * 32; }

// kCh > 0: rows of kCh float4 chunks per thread (ld = 32 kCh), held in
// registers between the dot products and the rotation; kCh = 0: any ld,
// rows re-read from memory.
// (q <= 32 kCh gives at most 16 kCh pairs: 128 kCh threads.)
template <bool kSmem, int kCh>
__global__ void __launch_bounds__(kCh > 0 ? 128 * kCh : 1024) jacobi_onesided_f32_kernel(const float* Mc_g, int q, int pp,
                                                                   float* Jc_g, float* norms,
                                                                   int max_sweeps, float tol,
                                                                   int* flags, float* Wg) {
  extern __shared__ __align__(16) float osm[];
  const int ld = jacobi_ld(q);
  float* Mc = kSmem ? osm : Wg;  // resolved at compile time: shared loads stay LDS
  float* Jc = Mc + size_t(q) * ld;
  __shared__ int s_rot;
  for (int idx = threadIdx.x; idx < q * ld; idx += blockDim.x) {
    const int r = idx / ld, c = idx - r * ld;
    Mc[idx] = c < q ? Mc_g[r * q + c] : 0.f;
    Jc[idx] = (r == c) ? 1.f : 0.f;
  }
  const int npairs = pp / 2;
  const int g = threadIdx.x >> 3, sub = threadIdx.x & 7;  // groups of 8 threads
  const int ngroups = blockDim.x >> 3;
  const int nchunk = kCh > 0 ? kCh : ld / 32;               // float4 chunks per thread
  __syncthreads();
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) s_rot = 0;
    __syncthreads();
    for (int r = 0; r < pp - 1; ++r) {
      // every warp runs the same number of trips (groups of 8 threads whose
      // pair index is out of range compute zeros), so the full-mask shuffles
      // below always see all 32 lanes
      for (int kb = 0; kb < npairs; kb += ngroups) {
        const int k = kb + g;
        int i = 0, j = q;
        if (k < npairs) {
          const int i0 = k == 0 ? 0 : ((k - 1 + r) % (pp - 1)) + 1;
          const int k2 = pp - 1 - k;
          const int j0 = k2 == 0 ? 0 : ((k2 - 1 + r) % (pp - 1)) + 1;
          i = min(i0, j0);
          j = max(i0, j0);
        }
        const bool active = j < q;
        float4* a = reinterpret_cast<float4*>(Mc + size_t(i) * ld) + sub;
        float4* b = reinterpret_cast<float4*>(Mc + size_t(active ? j : i) * ld) + sub;
        constexpr int kR = kCh > 0 ? kCh : 1;
        float4 xa[kR], xb[kR];
        float al = 0.f, be = 0.f, ga = 0.f;
        if (active) {
          if (kCh > 0) {
#pragma unroll
            for (int m = 0; m < kR; ++m) {
              xa[m] = a[8 * m];
              xb[m] = b[8 * m];
            }
            // two partial sums per quantity: half the dependent-FMA chain
            float al2 = 0.f, be2 = 0.f, ga2 = 0.f;
#pragma unroll
            for (int m = 0; m < kR; ++m) {
              const float4 x = xa[m], y = xb[m];
              al = fmaf(x.x, x.x, fmaf(x.y, x.y, al));
              al2 = fmaf(x.z, x.z, fmaf(x.w, x.w, al2));
              be = fmaf(y.x, y.x, fmaf(y.y, y.y, be));
              be2 = fmaf(y.z, y.z, fmaf(y.w, y.w, be2));
              ga = fmaf(x.x, y.x, fmaf(x.y, y.y, ga));
              ga2 = fmaf(x.z, y.z, fmaf(x.w, y.w, ga2));
            }
            al += al2;
            be += be2;
            ga += ga2;
          } else {
            for (int m = 0; m < nchunk; ++m) {
              const float4 x = a[8 * m], y = b[8 * m];
              al = fmaf(x.x, x.x, fmaf(x.y, x.y, fmaf(x.z, x.z, fmaf(x.w, x.w, al))));
              be = fmaf(y.x, y.x, fmaf(y.y, y.y, fmaf(y.z, y.z, fmaf(y.w, y.w, be))));
              ga = fmaf(x.x, y.x, fmaf(x.y, y.y, fmaf(x.z, y.z, fmaf(x.w, y.w, ga))));
            }
          }
        }
        for (int o = 4; o > 0; o >>= 1) {
          al += __shfl_xor_sync(0xffffffffu, al, o);
          be += __shfl_xor_sync(0xffffffffu, be, o);
          ga += __shfl_xor_sync(0xffffffffu, ga, o);
        }
        if (!active || al == 0.f || be == 0.f || !(fabsf(ga) > tol * sqrtf(al) * sqrtf(be)))
          continue;
        const float zeta = (be - al) / (2.f * ga);
        const float t = copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
        // Rutishauser's form of the rotation (x' = x - s (y + tau x),
        // y' = y + s (x - tau y), tau = s / (1 + c)): the second-order term
        // s tau ~ t^2 / 2 is applied explicitly; with c rounded to 1 for
        // t^2 < 2^-24, c x - s y would lengthen the pair by a factor 1 + t^2
        // per rotation, a bias that builds up over the sweeps
        const float cs = 1.f / sqrtf(1.f + t * t), sn = cs * t, tau = sn / (1.f + cs);
        float4* ja = reinterpret_cast<float4*>(Jc + size_t(i) * ld) + sub;
        float4* jb = reinterpret_cast<float4*>(Jc + size_t(j) * ld) + sub;
        auto rot = [&](float4* pa, float4* pb, const float4 x, const float4 y) {
          *pa = make_float4(fmaf(-sn, fmaf(tau, x.x, y.x), x.x), fmaf(-sn, fmaf(tau, x.y, y.y), x.y),
                            fmaf(-sn, fmaf(tau, x.z, y.z), x.z), fmaf(-sn, fmaf(tau, x.w, y.w), x.w));
          *pb = make_float4(fmaf(sn, fmaf(-tau, y.x, x.x), y.x), fmaf(sn, fmaf(-tau, y.y, x.y), y.y),
                            fmaf(sn, fmaf(-tau, y.z, x.z), y.z), fmaf(sn, fmaf(-tau, y.w, x.w), y.w));
        };
        if (kCh > 0) {
          float4 u[kR], v[kR];
#pragma unroll
          for (int m = 0; m < kR; ++m) {
            u[m] = ja[8 * m];
            v[m] = jb[8 * m];
          }
#pragma unroll
          for (int m = 0; m < kR; ++m) {
            rot(a + 8 * m, b + 8 * m, xa[m], xb[m]);
            rot(ja + 8 * m, jb + 8 * m, u[m], v[m]);
          }
        } else {
          for (int m = 0; m < nchunk; ++m) {
            rot(a + 8 * m, b + 8 * m, a[8 * m], b[8 * m]);
            rot(ja + 8 * m, jb + 8 * m, ja[8 * m], jb[8 * m]);
          }
        }
        if (sub == 0) s_rot = 1;
      }
      __syncthreads();
    }
    if (s_rot == 0) break;
    __syncthreads();
  }
  if (threadIdx.x == 0 && sweep == max_sweeps) atomicOr(flags, 2);
  for (int j = threadIdx.x; j < q; j += blockDim.x) {
    float nn = 0.f;
    for (int t = 0; t < q; ++t) nn = fmaf(Mc[j * ld + t], Mc[j * ld + t], nn);
    norms[j] = sqrtf(nn);
  }
  for (int idx = threadIdx.x; idx < q * q; idx += blockDim.x) {
    const int r = idx / q, c = idx - r * q;
    Jc_g[idx] = Jc[r * ld + c];
  }
}

// One plane rotation of the one-sided Jacobi on a pair of rows (ra, rb) of
// kCh float4 chunks per thread, kTP threads per pair (thread sub owns chunks
// sub + kTP m); the accumulated-rotation rows follow at ra + ld, rb + ld.
// Every lane of the pair's group must call it (group-mask shuffles).
// Returns whether the pair was rotated.
template <int kCh, int kTP>
__device__ __forceinline__ bool jacobi_rotate_pair(float* ra, float* rb, int ld, int sub,
                                                   float tol) {
  float4* a = reinterpret_cast<float4*>(ra) + sub;
  float4* b = reinterpret_cast<float4*>(rb) + sub;
  float4* ja = reinterpret_cast<float4*>(ra + ld) + sub;
  float4* jb = reinterpret_cast<float4*>(rb + ld) + sub;
  // the rotation rows are loaded with the data rows, ahead of the decision
  float4 xa[kCh], xb[kCh], u[kCh], v[kCh];
#pragma unroll
  for (int m = 0; m < kCh; ++m) {
    xa[m] = a[kTP * m];
    xb[m] = b[kTP * m];
  }
#pragma unroll
  for (int m = 0; m < kCh; ++m) {
    u[m] = ja[kTP * m];
    v[m] = jb[kTP * m];
  }
  // dot products in paired FMAs: four partial sums per quantity
  float2 al2a = make_float2(0.f, 0.f), al2b = al2a, be2a = al2a, be2b = al2a, ga2a = al2a,
         ga2b = al2a;
#pragma unroll
  for (int m = 0; m < kCh; ++m) {
    const float2 x0 = make_float2(xa[m].x, xa[m].y), x1 = make_float2(xa[m].z, xa[m].w);
    const float2 y0 = make_float2(xb[m].x, xb[m].y), y1 = make_float2(xb[m].z, xb[m].w);
    al2a = fma2(x0, x0, al2a);
    al2b = fma2(x1, x1, al2b);
    be2a = fma2(y0, y0, be2a);
    be2b = fma2(y1, y1, be2b);
    ga2a = fma2(x0, y0, ga2a);
    ga2b = fma2(x1, y1, ga2b);
  }
  float al = (al2a.x + al2a.y) + (al2b.x + al2b.y);
  float be = (be2a.x + be2a.y) + (be2b.x + be2b.y);
  float ga = (ga2a.x + ga2a.y) + (ga2b.x + ga2b.y);
  // the shuffles stay inside the pair's group of kTP lanes (its mask): the
  // groups of a warp beyond the last pair may skip the call
  const unsigned gmask =
      kTP >= 32 ? 0xffffffffu : (((1u << kTP) - 1u) << ((threadIdx.x & 31) & ~(kTP - 1)));
  for (int o = kTP / 2; o > 0; o >>= 1) {
    al += __shfl_xor_sync(gmask, al, o);
    be += __shfl_xor_sync(gmask, be, o);
    ga += __shfl_xor_sync(gmask, ga, o);
  }
  // |ga| > tol sqrt(al be) without square roots
  if (al == 0.f || be == 0.f || !(ga * ga > (tol * tol * al) * be)) return false;
  // Rotation parameters from approximate reciprocals and square roots: in
  // Rutishauser's form an error e in c changes the orthogonality of the
  // rotation by only ~s^2 e, so 2-ulp parameters cost nothing, while the
  // correctly rounded divisions and roots sat on the critical path of every
  // round.  |zeta| is capped at 1e18 so that zeta^2 stays finite (t is then
  // ~1/(2 zeta), a negligible rotation either way); zeta = 0 gives t = 1.
  const float zeta = __fdividef(be - al, 2.f * ga);
  const float az = fminf(fabsf(zeta), 1e18f);
  const float t = copysignf(__fdividef(1.f, az + sqrtf(fmaf(az, az, 1.f))), zeta);
  const float cs = rsqrtf(fmaf(t, t, 1.f)), sn = cs * t, tau = __fdividef(sn, 1.f + cs);
  const float2 s2 = make_float2(sn, sn), ms2 = make_float2(-sn, -sn);
  const float2 t2 = make_float2(tau, tau), mt2 = make_float2(-tau, -tau);
  auto rot = [&](float4* pa, float4* pb, const float4 x, const float4 y) {
    const float2 x0 = make_float2(x.x, x.y), x1 = make_float2(x.z, x.w);
    const float2 y0 = make_float2(y.x, y.y), y1 = make_float2(y.z, y.w);
    const float2 p0 = fma2(ms2, fma2(t2, x0, y0), x0), p1 = fma2(ms2, fma2(t2, x1, y1), x1);
    const float2 q0 = fma2(s2, fma2(mt2, y0, x0), y0), q1 = fma2(s2, fma2(mt2, y1, x1), y1);
    *pa = make_float4(p0.x, p0.y, p1.x, p1.y);
    *pb = make_float4(q0.x, q0.y, q1.x, q1.y);
  };
#pragma unroll
  for (int m = 0; m < kCh; ++m) {
    rot(a + kTP * m, b + kTP * m, xa[m], xb[m]);
    rot(ja + kTP * m, jb + kTP * m, u[m], v[m]);
  }
  return true;
}

// Block one-sided Jacobi on a cluster of P CTAs (same rotations and
// convergence test as jacobi_onesided_f32_kernel, another cyclic order).
// kTP threads per pair (b groups; the CTA's threads are rounded up to whole
// warps, the extra groups idle).  The rows (padded with zero rows to 2 P b,
// b even) form 2 P blocks of b rows; CTA k holds the blocks at tournament positions k ("top")
// and 2P-1-k ("bottom") in shared memory, each row stored as ld floats of Mc
// followed by ld floats of the accumulated rotations J.  A sweep is 2P-1
// block rounds of the circle method (position 0 fixed, the others advance by
// one per round): in a round every CTA rotates all b^2 top-bottom pairs, b
// disjoint pairs at a time (bottom row (i + s) mod b against top row i), and
// in the first round of a sweep also the pairs inside each of its two blocks
// (b - 1 rounds of the circle method on b rows).  Every pair of rows is thus
// visited once per sweep.  After a round each CTA writes the blocks that move
// into the receiving CTAs' second buffers (distributed shared memory) and the
// cluster synchronises; after 2P-1 rounds the blocks are back home.  The
// sweep loop ends when no CTA rotated in a sweep: every CTA reads all CTAs'
// per-sweep flags after the same cluster barrier, so all take the same
// decision and arrive at the same barriers.
template <int kCh, int kTP>
__global__ void __launch_bounds__(256) jacobi_cluster_f32_kernel(const float* Mc_g, int q, int b,
                                                                 float* Jc_g, float* norms,
                                                                 int max_sweeps, float tol,
                                                                 int* flags) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int P = int(cluster.num_blocks());
  const int k = int(cluster.block_rank());
  extern __shared__ __align__(16) float jcl_smem[];
  __shared__ int s_rot[64];
  constexpr int ld = 4 * kTP * kCh;
  constexpr int RS = 2 * ld;  // row stride: Mc, then J
  const int blk = b * RS;     // floats per block
  float* cur = jcl_smem;      // top block, then bottom block
  float* nxt = jcl_smem + 2 * blk;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int g = tid / kTP, sub = tid % kTP;
  for (int half = 0; half < 2; ++half) {
    const int beta = half == 0 ? k : 2 * P - 1 - k;
    float* base = cur + half * blk;
    for (int r = tid >> 5; r < b; r += nth >> 5)
      for (int c = tid & 31; c < RS; c += 32) {
        const int gr = beta * b + r;
        float v = 0.f;
        if (gr < q) v = c < ld ? (c < q ? Mc_g[size_t(gr) * q + c] : 0.f) : (c - ld == gr ? 1.f : 0.f);
        base[r * RS + c] = v;
      }
  }
  for (int i = tid; i < 64; i += nth) s_rot[i] = 0;
  cluster.sync();
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    bool rotated = false;
    for (int t = 0; t < 2 * P - 1; ++t) {
      const int nin = t == 0 ? b - 1 : 0;  // rounds inside the blocks
      for (int lr = 0; lr < nin + b; ++lr) {
        int ia, ib;
        if (lr < nin) {
          const int half = g < b / 2 ? 0 : 1;
          const int kk = half == 0 ? g : g - b / 2;
          const int i0 = kk == 0 ? 0 : ((kk - 1 + lr) % (b - 1)) + 1;
          const int k2 = b - 1 - kk;
          const int j0 = k2 == 0 ? 0 : ((k2 - 1 + lr) % (b - 1)) + 1;
          ia = half * blk + i0 * RS;
          ib = half * blk + j0 * RS;
        } else {
          const int sft = lr - nin;
          ia = g * RS;
          ib = blk + ((g + sft) % b) * RS;
        }
        if (g < b) rotated |= jacobi_rotate_pair<kCh, kTP>(cur + ia, cur + ib, ld, sub, tol);
        __syncthreads();
      }
      // move the blocks: position p -> p + 1 (2P-1 -> 1, 0 stays)
      float* dst_top;
      float* dst_bot;
      if (k == 0) {
        dst_top = nxt;
        dst_bot = cluster.map_shared_rank(nxt, 1);
      } else if (k < P - 1) {
        dst_top = cluster.map_shared_rank(nxt, k + 1);
        dst_bot = cluster.map_shared_rank(nxt + blk, k - 1);
      } else {
        dst_top = nxt + blk;
        dst_bot = cluster.map_shared_rank(nxt + blk, k - 1);
      }
      const float4* st4 = reinterpret_cast<const float4*>(cur);
      const float4* sb4 = reinterpret_cast<const float4*>(cur + blk);
      for (int i = tid; i < blk / 4; i += nth) {
        reinterpret_cast<float4*>(dst_top)[i] = st4[i];
        reinterpret_cast<float4*>(dst_bot)[i] = sb4[i];
      }
      cluster.sync();
      float* tmp = cur;
      cur = nxt;
      nxt = tmp;
    }
    if (rotated) s_rot[sweep] = 1;
    cluster.sync();
    int any = 0;
    for (int r = 0; r < P; ++r) any |= *cluster.map_shared_rank(&s_rot[sweep], r);
    if (any == 0) break;
  }
  if (tid == 0 && k == 0 && sweep == max_sweeps) atomicOr(flags, 2);
  // the blocks are home: top = block k, bottom = block 2P-1-k
  for (int rr = tid; rr < 2 * b; rr += nth) {
    const int half = rr < b ? 0 : 1, r = rr - half * b;
    const int gr = (half == 0 ? k : 2 * P - 1 - k) * b + r;
    if (gr >= q) continue;
    const float* row = cur + half * blk + r * RS;
    float nn = 0.f;
    for (int c = 0; c < q; ++c) nn = fmaf(row[c], row[c], nn);
    norms[gr] = sqrtf(nn);
  }
  for (int half = 0; half < 2; ++half) {
    const int beta = half == 0 ? k : 2 * P - 1 - k;
    for (int r = tid >> 5; r < b; r += nth >> 5) {
      const int gr = beta * b + r;
      if (gr >= q) continue;
      const float* jrow = cur + half * blk + r * RS + ld;
      for (int c = tid & 31; c < q; c += 32) Jc_g[size_t(gr) * q + c] = jrow[c];
    }
  }
  // no CTA may leave while others can still read its shared memory
  cluster.sync();
}

// Ub[:, r] = J[:, order[r]] (J columns stored as rows of Jc), S[r] = norm,
// inv_s[r] = 1 / S[r] (0 for a zero norm); order by descending norm.
// One CTA (q <= 1024): the rank of every row norm (descending, ties by
// index) from a shared-memory copy of the norms, then Ub[t][rank[j]] =
// Jc[j][t].  With kStaged (q <= kSortStagedMax) Jc goes through shared
// memory first and Ub is written row by row, contiguously (scattered
// 8-byte stores of one CTA bound the direct form).
constexpr int kSortThreads = 1024;
constexpr int kSortStagedMax = 224;
template <bool kStaged>
__global__ void __launch_bounds__(kSortThreads) sort_singular_kernel(const float* Jc,
                                                                     const float* norms, int q,
                                                                     double* Ub, double* S,
                                                                     double* inv_s) {
  extern __shared__ float jc_s[];  // kStaged: q rows of q + 1 floats
  __shared__ float s_norm[kSortThreads];
  __shared__ int s_rank[kSortThreads];
  for (int j = threadIdx.x; j < q; j += blockDim.x) s_norm[j] = norms[j];
  if (kStaged)
    for (int idx = threadIdx.x; idx < q * q; idx += blockDim.x) {
      const int j = idx / q, t = idx - j * q;
      jc_s[j * (q + 1) + t] = Jc[idx];
    }
  __syncthreads();
  for (int j = threadIdx.x; j < q; j += blockDim.x) {
    int rank = 0;
    const float nj = s_norm[j];
    for (int i = 0; i < q; ++i)
      if (s_norm[i] > nj || (s_norm[i] == nj && i < j)) ++rank;
    if (kStaged) s_rank[rank] = j;  // the inverse permutation
    else s_rank[j] = rank;
    S[rank] = double(nj);
    inv_s[rank] = nj > 0.f ? 1.0 / double(nj) : 0.0;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < q * q; idx += blockDim.x) {
    const int a = idx / q, b = idx - a * q;
    if (kStaged) Ub[idx] = double(jc_s[s_rank[b] * (q + 1) + a]);  // Ub[a][b], row-major
    else Ub[size_t(b) * q + s_rank[a]] = double(Jc[idx]);          // a = j, b = t
  }
}

void sort_singular(cudaStream_t st, const float* Jc, const float* norms, int64_t q, double* Ub,
                   double* S, double* inv_s) {
  if (q <= kSortStagedMax) {
    const size_t smem = size_t(q) * (q + 1) * sizeof(float);
    CTM_CUDA(cudaFuncSetAttribute(sort_singular_kernel<true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    sort_singular_kernel<true><<<1, kSortThreads, smem, st>>>(Jc, norms, int(q), Ub, S, inv_s);
  } else {
    sort_singular_kernel<false><<<1, kSortThreads, 0, st>>>(Jc, norms, int(q), Ub, S, inv_s);
  }
  CTM_LAUNCH_CHECK();
}


// Sets flag bit 1 when max |G - I| exceeds tol (NaN counts as failure).
template <class T>
__global__ void __launch_bounds__(1024) orthogonality_check_kernel(const T* G, int q, T tol,
                                                                   int* flags) {
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  bool local = false;
  for (int idx = threadIdx.x; idx < q * q; idx += blockDim.x) {
    const int r = idx / q, c = idx - r * q;
    const T e = fabs(G[idx] - (r == c ? T(1) : T(0)));
    local = local || !(e <= tol);
  }
  if (local) bad = 1;
  __syncthreads();
  if (threadIdx.x == 0 && bad) atomicOr(flags, 1);
}

// ------------------------------------------------------------- Jacobi SVD
struct JacobiArgs {
  double* W;      // p x L, row j = column j being orthogonalised
  double* J;      // p x p, row j = column j of the accumulated rotation
  int64_t p, L;
  int64_t pp;     // p rounded up to even
  double tol;
  int max_sweeps;
  unsigned* bar;  // [0] arrival count, [1] generation, [2] abort, [3..4] sweep flags
  int* flags;
  int64_t spin_limit;
};

// Bounded grid barrier.  Returns false when this CTA gave up waiting (the
// abort word is then set and the status flag records the timeout).
__device__ bool grid_sync(const JacobiArgs& a) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0) {
    volatile unsigned* gen = a.bar + 1;
    volatile unsigned* abort_w = a.bar + 2;
    ok = 1;
    const unsigned g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(a.bar, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(a.bar, 0u);
      __threadfence();
      atomicAdd(const_cast<unsigned*>(gen), 1u);
    } else {
      int64_t it = 0;
      while (*gen == g) {
        if (*abort_w != 0u || ++it > a.spin_limit) {
          atomicExch(const_cast<unsigned*>(abort_w), 1u);
          atomicOr(a.flags, 2);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

__device__ __forceinline__ int64_t rr_pos(int64_t i, int64_t r, int64_t pp) {
  return i == 0 ? 0 : ((i - 1 + r) % (pp - 1)) + 1;
}

__global__ void __launch_bounds__(64) jacobi_sweeps_kernel(const JacobiArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t warps_per_cta = blockDim.x >> 5;
  const int64_t gw = blockIdx.x * warps_per_cta + (threadIdx.x >> 5);
  const int64_t total_w = gridDim.x * warps_per_cta;
  const int64_t npairs = a.pp / 2;
  for (int sweep = 0; sweep < a.max_sweeps; ++sweep) {
    unsigned* rotated = a.bar + 3 + (sweep & 1);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(a.bar + 3 + ((sweep + 1) & 1), 0u);
    for (int64_t r = 0; r < a.pp - 1; ++r) {
      for (int64_t k = gw; k < npairs; k += total_w) {
        int64_t i = rr_pos(k, r, a.pp), j = rr_pos(a.pp - 1 - k, r, a.pp);
        if (i > j) { const int64_t t = i; i = j; j = t; }
        if (j >= a.p) continue;  // dummy partner
        double* wi = a.W + i * a.L;
        double* wj = a.W + j * a.L;
        double al = 0.0, be = 0.0, ga = 0.0;
        for (int64_t t = lane; t < a.L; t += 32) {
          const double x = wi[t], y = wj[t];
          al = fma(x, x, al);
          be = fma(y, y, be);
          ga = fma(x, y, ga);
        }
        al = warp_sum(al);
        be = warp_sum(be);
        ga = warp_sum(ga);
        if (al == 0.0 || be == 0.0 || !(fabs(ga) > a.tol * sqrt(al) * sqrt(be))) continue;
        const double zeta = (be - al) / (2.0 * ga);
        const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(fma(zeta, zeta, 1.0)));
        const double cs = 1.0 / sqrt(fma(t, t, 1.0));
        const double sn = cs * t;
        for (int64_t u = lane; u < a.L; u += 32) {
          const double x = wi[u], y = wj[u];
          wi[u] = cs * x - sn * y;
          wj[u] = sn * x + cs * y;
        }
        double* ji = a.J + i * a.p;
        double* jj = a.J + j * a.p;
        for (int64_t u = lane; u < a.p; u += 32) {
          const double x = ji[u], y = jj[u];
          ji[u] = cs * x - sn * y;
          jj[u] = sn * x + cs * y;
        }
        if (lane == 0) atomicExch(rotated, 1u);
      }
      if (!grid_sync(a)) return;
    }
    const unsigned any = *(volatile unsigned*)rotated;
    if (!grid_sync(a)) return;
    if (any == 0u) return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.flags, 2);
}

// Sorts the Jacobi result by descending column norm and writes U, S, V.
// trans == 0: W rows are columns of X (m >= n): U = W_j / s_j, V = J.
// trans == 1: W rows are rows of X (m < n):  U = J, V = W_j / s_j.
__global__ void jacobi_finish_kernel(const double* W, const double* J, int64_t p, int64_t L,
                                     int trans, double* U, double* S, double* V) {
  const int64_t j = blockIdx.x;
  if (j >= p) return;
  __shared__ double sh[LT / 32];
  __shared__ double s_norm;
  __shared__ int64_t s_rank;
  double part = 0.0;
  for (int64_t t = threadIdx.x; t < L; t += blockDim.x) part = fma(W[j * L + t], W[j * L + t], part);
  const double nj2 = block_sum(part, sh);
  // rank: strictly larger norms (ties broken by index); norms recomputed per
  // column so every block sees identical values
  int64_t cnt = 0;
  for (int64_t i = threadIdx.x; i < p; i += blockDim.x) {
    if (i == j) continue;
    double ni2 = 0.0;
    for (int64_t t = 0; t < L; ++t) ni2 = fma(W[i * L + t], W[i * L + t], ni2);
    if (ni2 > nj2 || (ni2 == nj2 && i < j)) ++cnt;
  }
  const double c = block_sum(double(cnt), sh);
  if (threadIdx.x == 0) {
    s_norm = sqrt(nj2);
    s_rank = static_cast<int64_t>(c + 0.5);
  }
  __syncthreads();
  const double sj = s_norm;
  const int64_t rk = s_rank;
  const double inv = sj > 0.0 ? 1.0 / sj : 0.0;
  if (threadIdx.x == 0) S[rk] = sj;
  if (trans == 0) {
    for (int64_t t = threadIdx.x; t < L; t += blockDim.x) U[t * p + rk] = W[j * L + t] * inv;
    for (int64_t t = threadIdx.x; t < p; t += blockDim.x) V[t * p + rk] = J[j * p + t];
  } else {
    for (int64_t t = threadIdx.x; t < p; t += blockDim.x) U[t * p + rk] = J[j * p + t];
    for (int64_t t = threadIdx.x; t < L; t += blockDim.x) V[t * p + rk] = W[j * L + t] * inv;
  }
}

__global__ void identity_kernel(double* X, int64_t p) {
  for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < p * p;
       idx += int64_t(gridDim.x) * blockDim.x)
    X[idx] = (idx / p == idx % p) ? 1.0 : 0.0;
}

// ------------------------------------------------------------- truncation
__global__ void truncation_kernel(const double* s, int64_t r, int64_t chi, double cutoff,
                                  double* f, int64_t cap, int64_t* chi_new) {
  __shared__ double sh[LT / 32];
  const double s0 = s[0];
  double cnt = 0.0;
  for (int64_t i = threadIdx.x; i < r; i += LT) cnt += (s[i] / s0 > cutoff) ? 1.0 : 0.0;
  cnt = block_sum(cnt, sh);
  const int64_t count = static_cast<int64_t>(cnt + 0.5);
  const int64_t cn = count < chi ? count : chi;
  for (int64_t i = threadIdx.x; i < cap; i += LT)
    f[i] = (i < cn) ? 1.0 / sqrt(s[i] / s0) : 0.0;
  if (threadIdx.x == 0) *chi_new = cn;
}

__global__ void scale_compact_kernel(const double* in, int64_t rows, int64_t cap, const double* f,
                                     const int64_t* chi_new, double* out) {
  const int64_t cn = *chi_new;
  const int64_t total = rows * cn;
  if (total < (int64_t(1) << 31)) {  // 32-bit decoding (a 64-bit division is a long sequence)
    const uint32_t ucn = uint32_t(cn);
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < uint32_t(total);
         idx += gridDim.x * blockDim.x) {
      const uint32_t r = idx / ucn, c = idx - r * ucn;
      const double v = in[int64_t(r) * cap + c];
      out[idx] = f != nullptr ? v * f[c] : v;
    }
    return;
  }
  for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = idx / cn, c = idx % cn;
    out[idx] = f != nullptr ? in[r * cap + c] * f[c] : in[r * cap + c];
  }
}

}  // namespace

int sm_count_linalg() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return 152;
  }
  return n;
}

unsigned long long* qr_fallback_counter() {
  unsigned long long* p = nullptr;
  CTM_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_qr_fallbacks));
  return p;
}

int* status_flags(Ctx& c) {
  (void)c;
  int* p = nullptr;
  CTM_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_status_flags));
  return p;
}

// ------------------------------------------------------------- tall-skinny
// FP32 stages of the Cholesky-QR (q <= 192): one kernel per stage applies the
// previous stage's L^-T to a slab of rows and accumulates the slab's Gram
// matrix; a second kernel sums the per-slab Grams in slab order.
namespace {

// cnt contiguous floats g -> s, issued asynchronously by the whole CTA
// (16-byte copies when kVec: both addresses 16-byte aligned, cnt % 4 == 0)
template <bool kVec>
__device__ __forceinline__ void slab_copy(float* s, const float* g, int64_t cnt) {
  if (kVec) {
    for (int64_t i = int64_t(threadIdx.x) * 4; i < cnt; i += int64_t(blockDim.x) * 4)
      cp_async_f32x4(s + i, g + i);
  } else {
    for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x) cp_async_f32(s + i, g + i);
  }
}

constexpr int kSlabThreads = 1024;

// Dynamic shared memory of a slab stage: rpb rows of q rounded up to 4
// floats, and q rows of L^T padded to 32-float multiples.
inline size_t slab_smem_bytes(int64_t q, int64_t rpb) {
  const int64_t ldq = (q + 3) / 4 * 4, ldl = (q + 31) / 32 * 32;
  return size_t(rpb * ldq + q * ldl) * sizeof(float);
}

// Tile t of the upper triangle (row-major, diagonal included) of an
// nt4 x nt4 grid of 4 x 4 tiles: its tile row ti and tile column tj >= ti.
__device__ __forceinline__ void slab_tri_tile(int t, int nt4, int& ti, int& tj) {
  const int m = 2 * nt4 + 1;
  int bi = int((float(m) - sqrtf(float(m * m - 8 * t))) * 0.5f);
  bi = max(0, min(bi, nt4 - 1));
  while (bi + 1 < nt4 && (bi + 1) * nt4 - (bi + 1) * bi / 2 <= t) ++bi;
  while (bi * nt4 - bi * (bi - 1) / 2 > t) --bi;
  ti = bi;
  tj = bi + (t - (bi * nt4 - bi * (bi - 1) / 2));
}

// One slab of rows [r0, r0 + nr) of Y (n x q, row-major), r0 = blockIdx.x * rpb.
// With Lt (q x q, the upper triangular L^T of a Cholesky factor L; entries
// below the diagonal do not matter): X = Y L^-T for the slab by forward substitution (x L^T = y
// row by row; written to X and kept in shared memory), then the slab's Gram
// matrix X^T X; without Lt: Y^T Y.  A zero diagonal of L (a pivot the
// factorisation dropped) gives a zero column of X.
// Shared memory: the slab (rpb rows of ldq = q rounded up to 4 floats, zero
// past column q) and Lt (q rows of 32 kT floats; once the reciprocal pivots
// are taken, row b holds L[a][b] / L[b][b] for a > b and zeros elsewhere, so
// the update loop reads every column unconditionally).
// Solve: warp w owns rows 4w..4w+3 (+128 per pass), lane the columns
// lane + 32 j, which hold residuals r_a; column b's residual is broadcast
// from its owner lane with a shuffle and every lane subtracts r_b times its
// entry of scaled row b (read conflict-free); at the end of each block of 32
// columns the lanes turn their residuals into x_a = r_a / L[a][a].  Full
// blocks are unrolled (the shuffle source and the loop bounds constant).
// Gram: the upper triangle of the slab's Gram matrix in 4 x 4 tiles, one
// tile per thread (two 16-byte reads per 16 FMAs and row), written packed:
// part[blockIdx.x][t][4][4] for tile t (slab_tri_tile order).
template <int kT, bool kVec>
__global__ void __launch_bounds__(kSlabThreads) slab_stage_kernel(
    const float* __restrict__ Y, int64_t n, int q, int rpb, const float* __restrict__ Lt,
    float* __restrict__ X, float* __restrict__ part) {
  extern __shared__ __align__(16) float slab_smem[];
  __shared__ float s_rdiag[32 * kT];
  constexpr int ldl = 32 * kT;
  const int ldq = (q + 3) & ~3;
  float* Ys = slab_smem;                      // rpb x ldq
  float* Us = slab_smem + size_t(rpb) * ldq;  // q x ldl
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t r0 = int64_t(blockIdx.x) * rpb;
  const int nr = int(n - r0 < rpb ? n - r0 : rpb);
  if (kVec) {  // q % 4 == 0 (ldq == q: the slab is contiguous), 16-byte aligned rows
    const int c4 = q / 4;
    for (int i = threadIdx.x; i < nr * c4; i += blockDim.x)
      cp_async_f32x4(Ys + 4 * i, Y + r0 * q + 4 * i);
    if (Lt != nullptr)
      for (int i = threadIdx.x; i < q * c4; i += blockDim.x) {
        const int r = i / c4, c = i - r * c4;
        cp_async_f32x4(Us + r * ldl + 4 * c, Lt + size_t(r) * q + 4 * c);
      }
  } else {
    for (int i = threadIdx.x; i < nr * q; i += blockDim.x) {
      const int r = i / q, c = i - r * q;
      cp_async_f32(Ys + r * ldq + c, Y + (r0 + r) * q + c);
    }
    if (Lt != nullptr)
      for (int i = threadIdx.x; i < q * q; i += blockDim.x) {
        const int r = i / q, c = i - r * q;
        cp_async_f32(Us + r * ldl + c, Lt + size_t(r) * q + c);
      }
  }
  // the slab's padding columns (not touched by the copies; those of Lt are
  // zeroed with the scaling below)
  if (ldq > q)
    for (int i = threadIdx.x; i < nr * (ldq - q); i += blockDim.x) {
      const int r = i / (ldq - q);
      Ys[r * ldq + q + (i - r * (ldq - q))] = 0.f;
    }
  cp_async_wait_all();
  __syncthreads();
  if (Lt != nullptr) {
    for (int b = threadIdx.x; b < q; b += blockDim.x) {
      const float d = Us[b * ldl + b];
      s_rdiag[b] = d > 0.f ? 1.f / d : 0.f;
    }
    __syncthreads();
    // row b of L^T scaled by 1 / L[b][b], zero at and below the diagonal:
    // the update of the residual r_a by column b is then r_a -= r_b Us[b][a]
    for (int i = threadIdx.x; i < q * ldl; i += blockDim.x) {
      const int b = i / ldl, a = i - b * ldl;
      Us[i] = (a > b && a < q) ? Us[i] * s_rdiag[b] : 0.f;
    }
    __syncthreads();
    for (int rg = warp * 4; rg < nr; rg += 4 * 32) {
      float y[4][kT];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < kT; ++j) {
          const int a = lane + 32 * j;
          y[i][j] = (rg + i < nr && a < q) ? Ys[(rg + i) * ldq + a] : 0.f;
        }
      // column b: its residual (final once the columns before it are done)
      // broadcast from its owner lane, subtracted from the columns after it
      auto step = [&](int jb, int bl) {
        float rb[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) rb[i] = __shfl_sync(0xffffffffu, y[i][jb], bl);
        const float* lrow = Us + (32 * jb + bl) * ldl + lane;
#pragma unroll
        for (int j = 0; j < kT; ++j) {
          if (j < jb) continue;
          const float l = lrow[32 * j];
#pragma unroll
          for (int i = 0; i < 4; ++i) y[i][j] = fmaf(-rb[i], l, y[i][j]);
        }
      };
#pragma unroll
      for (int jb = 0; jb < kT; ++jb) {
        const int nb = q - 32 * jb < 32 ? q - 32 * jb : 32;
        if (nb == 32) {
#pragma unroll
          for (int bl = 0; bl < 32; ++bl) step(jb, bl);
        } else {
          for (int bl = 0; bl < nb; ++bl) step(jb, bl);
        }
        // the block's columns are final: x = r / L[b][b]
        const int a = lane + 32 * jb;
        const float rd = a < q ? s_rdiag[a] : 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i) y[i][jb] *= rd;
      }
      // every warp reads only its own rows of Ys: overwrite them in place
      __syncwarp();
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int r = rg + i;
        if (r >= nr) continue;
#pragma unroll
        for (int j = 0; j < kT; ++j) {
          const int a = lane + 32 * j;
          if (a < q) {
            Ys[r * ldq + a] = y[i][j];
            X[(r0 + r) * q + a] = y[i][j];
          }
        }
      }
    }
    __syncthreads();
  }
  const int nt4 = ldq / 4;
  const int ntiles = nt4 * (nt4 + 1) / 2;
  float4* P = reinterpret_cast<float4*>(part) + size_t(blockIdx.x) * ntiles * 4;
  for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
    int ti, tj;
    slab_tri_tile(t, nt4, ti, tj);
    const float* ya = Ys + 4 * ti;
    const float* yb = Ys + 4 * tj;
    float g[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) g[i][j] = 0.f;
#pragma unroll 2
    for (int r = 0; r < nr; ++r) {
      const float4 a4 = *reinterpret_cast<const float4*>(ya + r * ldq);
      const float4 b4 = *reinterpret_cast<const float4*>(yb + r * ldq);
      const float av[4] = {a4.x, a4.y, a4.z, a4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) g[i][j] = fmaf(av[i], bv[j], g[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) P[size_t(t) * 4 + i] = make_float4(g[i][0], g[i][1], g[i][2], g[i][3]);
  }
}

// G = sum over slabs of the packed tile partials, in a fixed order, written
// to both triangles.  Each CTA: 16 tile rows (float4) x 16 slab ranges
// (about 5 slabs each at 81 slabs), combined through shared memory in range
// order; thread grp 0 writes the tile row and its mirror.  With tol > 0 it
// also checks the orthonormality of the slab stage's result: flag bit 1
// when an entry of G - I exceeds tol in magnitude (NaN counts as failure).
constexpr int kReduceEntries = 16, kReduceRanges = 16;

__global__ void __launch_bounds__(256) slab_reduce_kernel(const float* __restrict__ part,
                                                          int nblk, int q, int nt4,
                                                          float* __restrict__ G, float tol,
                                                          int* flags) {
  __shared__ float4 s[kReduceRanges][kReduceEntries];
  const int t = threadIdx.x % kReduceEntries, grp = threadIdx.x / kReduceEntries;
  const int ne = nt4 * (nt4 + 1) / 2 * 4;
  const int e = blockIdx.x * kReduceEntries + t;
  const int b0 = grp * nblk / kReduceRanges, b1 = (grp + 1) * nblk / kReduceRanges;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  if (e < ne) {
    const float4* pv = reinterpret_cast<const float4*>(part);
#pragma unroll 4
    for (int b = b0; b < b1; ++b) {
      const float4 v = pv[size_t(b) * ne + e];
      acc.x += v.x;
      acc.y += v.y;
      acc.z += v.z;
      acc.w += v.w;
    }
  }
  s[grp][t] = acc;
  __syncthreads();
  if (grp == 0 && e < ne) {
    float4 r = s[0][t];
#pragma unroll
    for (int k = 1; k < kReduceRanges; ++k) {
      r.x += s[k][t].x;
      r.y += s[k][t].y;
      r.z += s[k][t].z;
      r.w += s[k][t].w;
    }
    int ti, tj;
    slab_tri_tile(e / 4, nt4, ti, tj);
    const int row = 4 * ti + (e & 3), col0 = 4 * tj;
    if (row < q) {
      const float v[4] = {r.x, r.y, r.z, r.w};
      bool bad = false;
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        const int col = col0 + cc;
        if (col < q) {
          G[size_t(row) * q + col] = v[cc];
          if (ti != tj) G[size_t(col) * q + row] = v[cc];
          bad = bad || !(fabsf(v[cc] - (row == col ? 1.f : 0.f)) <= tol);
        }
      }
      if (tol > 0.f && bad) atomicOr(flags, 1);
    }
  }
}

template <int kT, bool kVec>
void slab_stage_launch(Ctx& c, const float* Y, int64_t n, int64_t q, int rpb, int nblk,
                       const float* Lt, float* X, float* part) {
  const size_t smem = slab_smem_bytes(q, rpb);
  CTM_CUDA(cudaFuncSetAttribute(slab_stage_kernel<kT, kVec>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  // forward substitution (n q^2 / 2 FMA) and the slab Gram matrices (n q^2 / 2 FMA)
  KernelTimer kt(c.stream, "slab_stage_kernel", kUnitFlop, 2.0 * double(n) * q * q);
  slab_stage_kernel<kT, kVec><<<nblk, kSlabThreads, smem, c.stream>>>(Y, n, int(q), rpb, Lt, X,
                                                                      part);
}

template <bool kVec>
void slab_stage_dispatch(Ctx& c, const float* Y, int64_t n, int64_t q, int rpb, int nblk,
                         const float* Lt, float* X, float* part) {
  switch ((q + 31) / 32) {
    case 1: slab_stage_launch<1, kVec>(c, Y, n, q, rpb, nblk, Lt, X, part); break;
    case 2: slab_stage_launch<2, kVec>(c, Y, n, q, rpb, nblk, Lt, X, part); break;
    case 3: slab_stage_launch<3, kVec>(c, Y, n, q, rpb, nblk, Lt, X, part); break;
    case 4: slab_stage_launch<4, kVec>(c, Y, n, q, rpb, nblk, Lt, X, part); break;
    case 5: slab_stage_launch<5, kVec>(c, Y, n, q, rpb, nblk, Lt, X, part); break;
    default: slab_stage_launch<6, kVec>(c, Y, n, q, rpb, nblk, Lt, X, part); break;
  }
}

// rows per slab: about two slabs per SM, as the slab stages of several rows
// of a move run concurrently (at n = 5184: 64 rows, 81 slabs, measured
// faster in the concurrent move than one slab of 35 rows per SM); at most 64
// rows and what shared memory holds
int slab_rows(int64_t n, int64_t q) {
  const int64_t sms = sm_count_linalg();
  int64_t rpb = (2 * n + sms - 1) / sms;
  rpb = std::max<int64_t>(4, std::min<int64_t>(64, rpb));
  while (rpb > 4 && slab_smem_bytes(q, rpb) > kSmemOptin) --rpb;
  return int(rpb);
}

}  // namespace

// G (q x q) = X^T X where X = Y L^-T (Lt = L^T, q x q upper triangular;
// X written) or X = Y when Lt is null; FP32, q <= 192, one pass over Y.
// check_tol > 0: sets bit 1 of *flags when max |G - I| > check_tol.
void slab_gram(Ctx& c, const float* Y, int64_t n, int64_t q, const float* Lt, float* X,
               float* G, float check_tol, int* flags) {
  CTM_REQUIRE(q >= 1 && q <= 192, CTM_ERR_INVALID, "slab_gram: needs 1 <= q <= 192");
  const int rpb = slab_rows(n, q);
  const int nblk = int((n + rpb - 1) / rpb);
  const int nt4 = int((q + 3) / 4);
  const int ne = nt4 * (nt4 + 1) / 2 * 4;  // float4 tile rows per slab
  Scope scope(c);
  float* part = c.alloc<float>(size_t(nblk) * ne * 4);
  if (c.sizing()) return;
  const bool vec = q % 4 == 0 && (reinterpret_cast<uintptr_t>(Y) & 15) == 0 &&
                   (Lt == nullptr || (reinterpret_cast<uintptr_t>(Lt) & 15) == 0);
  if (vec)
    slab_stage_dispatch<true>(c, Y, n, q, rpb, nblk, Lt, X, part);
  else
    slab_stage_dispatch<false>(c, Y, n, q, rpb, nblk, Lt, X, part);
  CTM_LAUNCH_CHECK();
  KernelTimer kt(c.stream, "slab_reduce_kernel", kUnitByte,
                 16.0 * double(nblk) * ne + 4.0 * double(q) * q);
  const unsigned grid = unsigned((ne + kReduceEntries - 1) / kReduceEntries);
  slab_reduce_kernel<<<grid, kReduceEntries * kReduceRanges, 0, c.stream>>>(
      part, nblk, int(q), nt4, G, check_tol, flags);
  CTM_LAUNCH_CHECK();
}

template <class T>
void orthonormalize_impl(Ctx& c, T* Y, int64_t n, int64_t q, T* R, int stages) {
  CTM_REQUIRE(n >= q && q >= 1, CTM_ERR_INVALID, "orthonormalize: needs n >= q >= 1");
  CTM_REQUIRE(stages == 2 || stages == 3, CTM_ERR_INVALID, "orthonormalize: 2 or 3 stages");
  Scope scope(c);
  T* V = c.alloc<T>(size_t(n) * q);
  T* beta = c.alloc<T>(q);
  // the one-CTA Householder QR for small problems (its cost grows as q^2
  // barriers); the FP32 slab kernels beat it from q = 32 on
  const bool small = (sizeof(T) == 4 && q >= 32) ? false : double(n) * q * q <= 4.0e6;
  if (small) {
    if (c.sizing()) return;
    KernelTimer kt(c.stream, "householder_qr_kernel", kUnitFlop, 4.0 * double(n) * q * q);
    householder_qr_kernel<T><<<1, LT, 0, c.stream>>>(Y, n, q, R, V, beta, nullptr, 1);
    CTM_LAUNCH_CHECK();
    return;
  }
  // shifted Cholesky-QR3 with a Householder re-run when the check fails
  T* X2 = c.alloc<T>(size_t(n) * q);
  T* G = c.alloc<T>(size_t(q) * q);
  T* Wk = c.alloc<T>(cholesky_scratch(q));
  T* Ek = c.alloc<T>(cholesky_scratch(q));
  T* Li = c.alloc<T>(size_t(q) * q);
  T* Lt = c.alloc<T>(size_t(q) * q);
  T* Rt = c.alloc<T>(size_t(q) * q);
  T* Rt2 = c.alloc<T>(size_t(q) * q);
  int* flags = c.alloc<int>(1);
  // keep the input for the fallback in V
  if (!c.sizing()) {
    CTM_CUDA(cudaMemcpyAsync(V, Y, sizeof(T) * n * q, cudaMemcpyDeviceToDevice, c.stream));
    CTM_CUDA(cudaMemsetAsync(flags, 0, sizeof(int), c.stream));
  }
  T* cur = Y;
  T* nxt = X2;
  // Shifted Cholesky-QR3 (or -QR2) in both precisions: one shifted stage (FP32 shift
  // 1000 u tr(G): the result has cond <= ~1e2 whenever cond(Y) < 1/u) and two
  // plain ones.  The mixed range finder orthonormalises after every half
  // step, so its bases have the condition number of Q1 Q4 restricted to the
  // subspace (<= ~1e5 at D=6 chi=144), well inside that range; the check
  // below catches anything else.
  const int shifted_stages = 1;
  // FP32 with q <= 192: one slab kernel per stage applies the previous
  // stage's L^-T (forward substitution with L^T) and forms the next Gram
  // matrix in the same pass over the rows; the factorisation forms no inverse
  const bool fast_f32 = sizeof(T) == 4 && q <= 192;
  const T tol = sizeof(T) == 8 ? T(stages == 3 ? 1e-11 : 1e-6) : T(stages == 3 ? 2e-4 : 5e-2);
  auto accumulate_r = [&](int stage) {
    if (R == nullptr) return;
    if (stage == 0) {
      if (!c.sizing())
        CTM_CUDA(cudaMemcpyAsync(Rt, Lt, sizeof(T) * q * q, cudaMemcpyDeviceToDevice, c.stream));
    } else {
      einsum(c, "ab,bc->ac", ViewT<T>(Lt, {q, q}), ViewT<T>(Rt, {q, q}), ViewT<T>(Rt2, {q, q}));
      std::swap(Rt, Rt2);
    }
  };
  if (fast_f32) {
    float* const Yf = reinterpret_cast<float*>(cur);
    slab_gram(c, Yf, n, q, nullptr, nullptr, reinterpret_cast<float*>(G), -1.f, nullptr);
    for (int stage = 0; stage < stages; ++stage) {
      const int mode = stage < shifted_stages ? 2 : 0;
      if (!c.sizing())
        cholesky<T>(c.stream, G, q, n, mode, Wk, Ek, nullptr, nullptr, Lt, flags);
      accumulate_r(stage);
      // nxt = cur L^-T and G = nxt^T nxt; after the last stage the
      // reduction also checks G against the identity
      slab_gram(c, reinterpret_cast<const float*>(cur), n, q, reinterpret_cast<const float*>(Lt),
                reinterpret_cast<float*>(nxt), reinterpret_cast<float*>(G),
                stage == stages - 1 ? float(tol) : -1.f, flags);
      std::swap(cur, nxt);
    }
  } else {
    for (int stage = 0; stage < stages; ++stage) {
      einsum(c, "ia,ib->ab", ViewT<T>(cur, {n, q}), ViewT<T>(cur, {n, q}), ViewT<T>(G, {q, q}));
      const int mode = stage < shifted_stages ? (sizeof(T) == 8 ? 1 : 2) : 0;
      if (!c.sizing())
        cholesky<T>(c.stream, G, q, n, mode, Wk, Ek, nullptr, Li, R != nullptr ? Lt : nullptr,
                    flags);
      // nxt = cur @ Linv^T
      einsum(c, "ia,ba->ib", ViewT<T>(cur, {n, q}), ViewT<T>(Li, {q, q}), ViewT<T>(nxt, {n, q}));
      accumulate_r(stage);
      std::swap(cur, nxt);
    }
    einsum(c, "ia,ib->ab", ViewT<T>(cur, {n, q}), ViewT<T>(cur, {n, q}), ViewT<T>(G, {q, q}));
  }
  // cur holds Q after the stages and G its Gram matrix; check it and fall
  // back when needed
  T* hv = c.alloc<T>(size_t(n) * q);
  if (c.sizing()) return;
  if (!fast_f32) {  // (the FP32 slab path checked G in its last reduction)
    KernelTimer kt(c.stream, "orthogonality_check_kernel", kUnitByte, double(sizeof(T)) * q * q);
    orthogonality_check_kernel<T><<<1, 1024, 0, c.stream>>>(G, int(q), tol, flags);
    CTM_LAUNCH_CHECK();
  }
  if (cur != Y)
    CTM_CUDA(cudaMemcpyAsync(Y, cur, sizeof(T) * n * q, cudaMemcpyDeviceToDevice, c.stream));
  if (R != nullptr)
    CTM_CUDA(cudaMemcpyAsync(R, Rt, sizeof(T) * q * q, cudaMemcpyDeviceToDevice, c.stream));
  // when flagged: Y = the saved input, then its Householder QR
  householder_qr_kernel<T><<<1, LT, 0, c.stream>>>(Y, n, q, R, hv, beta, flags, 1, V);
  CTM_LAUNCH_CHECK();
}

void orthonormalize(Ctx& c, double* Y, int64_t n, int64_t q, double* R, int stages) {
  orthonormalize_impl<double>(c, Y, n, q, R, stages);
}

void orthonormalize(Ctx& c, float* Y, int64_t n, int64_t q, float* R, int stages) {
  orthonormalize_impl<float>(c, Y, n, q, R, stages);
}

void svd_thin(Ctx& c, const double* X, int64_t m, int64_t n, double* U, double* S, double* V) {
  CTM_REQUIRE(m >= 1 && n >= 1, CTM_ERR_INVALID, "svd_thin: empty matrix");
  const int trans = m >= n ? 0 : 1;
  const int64_t p = std::min(m, n), L = std::max(m, n);
  Scope scope(c);
  double* W = c.alloc<double>(size_t(p) * L);
  double* J = c.alloc<double>(size_t(p) * p);
  unsigned* bar = c.alloc<unsigned>(8);
  if (c.sizing()) return;
  // W rows = columns of X (trans 0) or rows of X (trans 1)
  if (trans == 0)
    copy2d(c, View(X, {m, n}).permute({1, 0}), W, L);
  else
    CTM_CUDA(cudaMemcpyAsync(W, X, sizeof(double) * m * n, cudaMemcpyDeviceToDevice, c.stream));
  identity_kernel<<<grid_for(p * p, 256), 256, 0, c.stream>>>(J, p);
  CTM_LAUNCH_CHECK();
  CTM_CUDA(cudaMemsetAsync(bar, 0, 8 * sizeof(unsigned), c.stream));
  JacobiArgs a{};
  a.W = W;
  a.J = J;
  a.p = p;
  a.L = L;
  a.pp = p + (p & 1);
  a.tol = 2.220446049250313e-16 * std::sqrt(double(L));
  a.max_sweeps = 60;
  a.bar = bar;
  a.flags = status_flags(c);
  a.spin_limit = int64_t(20) * 1000 * 1000;  // ~1-2 s of 64 ns sleeps
  if (p > 1) {
    int dev = 0, sms = 0, per_sm = 0;
    CTM_CUDA(cudaGetDevice(&dev));
    CTM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int threads = 64;
    CTM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, jacobi_sweeps_kernel, threads, 0));
    const int64_t npairs = a.pp / 2;
    int64_t blocks = (npairs + 1) / 2;
    blocks = std::min<int64_t>(blocks, int64_t(sms) * std::max(per_sm, 1));
    blocks = std::min<int64_t>(blocks, sms);
    blocks = std::max<int64_t>(blocks, 1);
    void* args[] = {&a};
    KernelTimer kt(c.stream, "jacobi_sweeps_kernel", kUnitFlop, 0.0);
    CTM_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(jacobi_sweeps_kernel),
                                         dim3(unsigned(blocks)), dim3(threads), args, 0, c.stream));
    CTM_LAUNCH_CHECK();
  }
  {
    KernelTimer kt(c.stream, "jacobi_finish_kernel", kUnitFlop, 2.0 * double(p) * p * L);
    jacobi_finish_kernel<<<unsigned(p), LT, 0, c.stream>>>(W, J, p, L, trans, U, S, V);
    CTM_LAUNCH_CHECK();
  }
}

void truncation_factors(Ctx& c, const double* s, int64_t r, int64_t chi, double cutoff, double* f,
                        int64_t cap, int64_t* chi_new) {
  if (c.sizing()) return;
  truncation_kernel<<<1, LT, 0, c.stream>>>(s, r, chi, cutoff, f, cap, chi_new);
  CTM_LAUNCH_CHECK();
}

__global__ void scale_columns_kernel(double* x, int64_t rows, int64_t cols, int64_t ld,
                                     const double* f) {
  if (rows * cols < (int64_t(1) << 31)) {  // 32-bit decoding
    const uint32_t uc = uint32_t(cols), total = uint32_t(rows * cols);
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += gridDim.x * blockDim.x) {
      const uint32_t r = idx / uc, c = idx - r * uc;
      x[int64_t(r) * ld + c] *= f[c];
    }
    return;
  }
  for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < rows * cols;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = idx / cols, c = idx % cols;
    x[r * ld + c] *= f[c];
  }
}

void scale_columns(Ctx& c, double* x, int64_t rows, int64_t cols, int64_t ld, const double* f) {
  if (c.sizing() || rows * cols == 0) return;
  KernelTimer kt(c.stream, "scale_columns_kernel", kUnitByte, 16.0 * rows * cols);
  scale_columns_kernel<<<grid_for(rows * cols, 256), 256, 0, c.stream>>>(x, rows, cols, ld, f);
  CTM_LAUNCH_CHECK();
}

void scale_columns_compact(Ctx& c, const double* in, int64_t rows, int64_t cap, const double* f,
                           const int64_t* chi_new, double* out) {
  if (c.sizing() || rows * cap == 0) return;
  KernelTimer kt(c.stream, "scale_compact_kernel", kUnitByte, 16.0 * rows * cap);
  scale_compact_kernel<<<grid_for(rows * cap, 256), 256, 0, c.stream>>>(in, rows, cap, f, chi_new,
                                                                         out);
  CTM_LAUNCH_CHECK();
}

}  // namespace ctm

// ======================================================================
// Mixed-precision SVD of the Rayleigh-Ritz matrix.
namespace ctm {

namespace {

__global__ void transpose_f32_kernel(const float* src, int q, float* dst) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < q * q; idx += gridDim.x * blockDim.x) {
    const int r = idx / q, c = idx - r * q;
    dst[c * q + r] = src[idx];
  }
}

__global__ void scale_columns_f32_kernel(float* x, int64_t rows, int cols, const double* f) {
  if (rows * cols < (int64_t(1) << 31)) {  // 32-bit decoding
    const uint32_t total = uint32_t(rows * cols), uc = uint32_t(cols);
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += gridDim.x * blockDim.x)
      x[idx] = float(double(x[idx]) * f[idx - (idx / uc) * uc]);
    return;
  }
  for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < rows * cols;
       idx += int64_t(gridDim.x) * blockDim.x)
    x[idx] = float(double(x[idx]) * f[idx % cols]);
}

// Singular values and left singular vectors of L (q x q) given as the rows
// of Mc (FP32): one-sided Jacobi on the columns of L^T with the rotations
// accumulated, then sorted.  Ub (q x q FP64), S, inv_s (q).
void jacobi_left_singular(Ctx& c, const float* Mc, int64_t q, double* Ub, double* S,
                          double* inv_s) {
  Scope scope(c);
  float* Jc = c.alloc<float>(size_t(q) * q);
  float* norms = c.alloc<float>(q);
  // the Jacobi matrices stay in shared memory up to q = 160, in global
  // memory (L2) beyond
  const size_t wjac = size_t(2) * q * jacobi_ld(int(q)) * sizeof(float);
  const bool jac_smem = wjac <= (227 - 1) * 1024;
  float* Wg = jac_smem ? nullptr : c.alloc<float>(size_t(2) * q * jacobi_ld(int(q)));
  const int64_t pp = q + (q & 1);
  if (c.sizing()) return;
  // q >= 96: the block Jacobi on a cluster of kJacobiCluster CTAs with
  // kPairThreads threads per pair (rows padded to a multiple of 4
  // kJacobiCluster: b even), when its four blocks of b rows fit in shared
  // memory.  At q = 160: 16 blocks of 10 rows, no padding rows, 159 pair
  // rounds per sweep (blocks of 12 rows, a multiple of 4 so that 8 b threads
  // filled whole warps, padded q to 192 and took 191 rounds); 8 threads per
  // pair measured faster per round than 16 (one shuffle level less)
  constexpr int kJacobiCluster = 8, kPairThreads = 8;
  const int P = kJacobiCluster;
  const int qp = int((q + 4 * P - 1) / (4 * P) * (4 * P));
  const int b = qp / (2 * P);
  const int ldj = int((q + 4 * kPairThreads - 1) / (4 * kPairThreads) * (4 * kPairThreads));
  const unsigned jthreads_c = unsigned((kPairThreads * b + 31) / 32 * 32);
  const size_t smem = size_t(4) * b * 2 * ldj * sizeof(float);
  if (q >= 96 && ldj <= 256 && smem <= size_t(227) * 1024) {
    auto launch = [&](auto kern) {
      CTM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
      KernelTimer kt(c.stream, "jacobi_cluster_f32_kernel", kUnitFlop, 0.0);
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3(P);
      cfg.blockDim = dim3(jthreads_c);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = c.stream;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = unsigned(P);
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      CTM_CUDA(cudaLaunchKernelEx(&cfg, kern, static_cast<const float*>(Mc), int(q), b, Jc, norms,
                                  40, 4e-6f, status_flags(c)));
    };
    switch (ldj / (4 * kPairThreads)) {
      case 3: launch(jacobi_cluster_f32_kernel<3, kPairThreads>); break;
      case 4: launch(jacobi_cluster_f32_kernel<4, kPairThreads>); break;
      case 5: launch(jacobi_cluster_f32_kernel<5, kPairThreads>); break;
      case 6: launch(jacobi_cluster_f32_kernel<6, kPairThreads>); break;
      case 7: launch(jacobi_cluster_f32_kernel<7, kPairThreads>); break;
      default: launch(jacobi_cluster_f32_kernel<8, kPairThreads>); break;
    }
    CTM_LAUNCH_CHECK();
    sort_singular(c.stream, Jc, norms, q, Ub, S, inv_s);
    return;
  }
  // FP32 dot products of length q carry ~sqrt(q) u relative error: 4e-6
  // is the smallest coupling the sweeps can drive below.  One group of 8
  // threads per pair of a round (no idle warps at the round barriers).
  const unsigned jthreads = unsigned(std::min<int64_t>(1024, ((pp / 2) * 8 + 31) / 32 * 32));
  if (jac_smem) {
    auto launch = [&](auto kern) {
      CTM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(wjac)));
      KernelTimer kt(c.stream, "jacobi_onesided_f32_kernel", kUnitFlop, 0.0);
      kern<<<1, jthreads, wjac, c.stream>>>(Mc, int(q), int(pp), Jc, norms, 40, 4e-6f,
                                           status_flags(c), nullptr);
    };
    switch (jacobi_ld(int(q)) / 32) {
      case 1: launch(jacobi_onesided_f32_kernel<true, 1>); break;
      case 2: launch(jacobi_onesided_f32_kernel<true, 2>); break;
      case 3: launch(jacobi_onesided_f32_kernel<true, 3>); break;
      case 4: launch(jacobi_onesided_f32_kernel<true, 4>); break;
      case 5: launch(jacobi_onesided_f32_kernel<true, 5>); break;
      default: launch(jacobi_onesided_f32_kernel<true, 0>); break;
    }
  } else {
    KernelTimer kt(c.stream, "jacobi_onesided_f32_kernel", kUnitFlop, 0.0);
    jacobi_onesided_f32_kernel<false, 0><<<1, jthreads, 0, c.stream>>>(
        Mc, int(q), int(pp), Jc, norms, 40, 4e-6f, status_flags(c), Wg);
  }
  CTM_LAUNCH_CHECK();
  sort_singular(c.stream, Jc, norms, q, Ub, S, inv_s);
}

}  // namespace

void svd_via_qr(Ctx& c, const float* Bt, int64_t q, int64_t n, double* Ub, double* S, float* V) {
  CTM_REQUIRE(q >= 1 && q <= 1024 && q <= n, CTM_ERR_UNSUPPORTED,
              "mixed SVD: needs 1 <= q <= min(n, 1024) (chi + oversampling)");
  Scope scope(c);
  float* Y = c.alloc<float>(size_t(n) * q);
  float* R = c.alloc<float>(size_t(q) * q);
  float* Mc = c.alloc<float>(size_t(q) * q);
  double* inv_s = c.alloc<double>(q);
  // B^T = Qb R (shifted Cholesky-QR3 in FP32, R backward stable to ~u |B|),
  // so B = L Qb^T with L = R^T and the SVD of B is that of L.  (A QR of L
  // first, Drmac-Veselic preconditioning, does not reduce the sweep count
  // here: B comes out of the range finder already graded, 7 sweeps at D=6,
  // chi=144, with or without it.)
  if (!c.sizing())
    CTM_CUDA(cudaMemcpyAsync(Y, Bt, sizeof(float) * n * q, cudaMemcpyDeviceToDevice, c.stream));
  orthonormalize(c, Y, n, q, R);
  if (!c.sizing()) {
    // Mc rows = rows of L = columns of R
    transpose_f32_kernel<<<grid_for(q * q, 256), 256, 0, c.stream>>>(R, int(q), Mc);
    CTM_LAUNCH_CHECK();
  }
  jacobi_left_singular(c, Mc, q, Ub, S, inv_s);
  // V = B^T Ub diag(1/s), FP32
  float* uf = c.alloc<float>(size_t(q) * q);
  to_f32(c, Ub, uf, q * q);
  einsum(c, "ik,kj->ij", ViewF(Bt, {n, q}), ViewF(uf, {q, q}), ViewF(V, {n, q}));
  if (!c.sizing()) {
    scale_columns_f32_kernel<<<grid_for(n * q, 256), 256, 0, c.stream>>>(V, n, int(q), inv_s);
    CTM_LAUNCH_CHECK();
  }
}

}  // namespace ctm
