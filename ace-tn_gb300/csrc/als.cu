// The full update's ALS solver for the reduced tensors of one bond
// (ALSSolver, acetn/evolution/als_solver.py:6-270) on the GPU, FP64.
//
// The reference runs the loop as ~30 torch operations per iteration (or
// cuTENSOR plans and cuSOLVER potrf/potrs in its optional extension).  Here
// the contractions go through the strided GETT engine and each least-squares
// step is one kernel: the symmetrised, shifted system is factorised in one
// CTA with the matrix in shared memory (right-looking Cholesky, then the two
// triangular solves with one warp per right-hand side; Gaussian elimination
// with partial pivoting when a pivot is not positive, the reference's
// torch.linalg.solve fallback).  The pseudo-inverse method runs the FP64
// one-sided Jacobi SVD of the symmetrised system.  The host loop reads the
// cost once per iteration for the reference's convergence test.
#include <cmath>

#include "engine.cuh"

namespace ctm {
namespace {

constexpr int kAlsThreads = 256;
constexpr int kAlsMaxM = 160;  // nD bD: the system fits in shared memory
constexpr int kAlsMaxP = kAlsThreads / 32;

__device__ double block_max(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < int(blockDim.x >> 5); ++w) r = fmax(r, red[w]);
  return r;
}

// W (m x m, leading dimension ld) = (R + R^T) / 2 + shift * max|.| * I
__device__ void load_system(const double* R, int m, int ld, double eps, double* W, double* red) {
  double mx = 0.0;
  for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
    const int i = idx / m, j = idx - i * m;
    const double v = 0.5 * (R[size_t(i) * m + j] + R[size_t(j) * m + i]);
    W[i * ld + j] = v;
    mx = fmax(mx, fabs(v));
  }
  mx = block_max(mx, red);
  for (int i = threadIdx.x; i < m; i += blockDim.x) W[i * ld + i] += eps * mx;
  __syncthreads();
}

// One warp solves L y = b (lower = true: forward, L[i][k] at W[i*ld+k]) or
// L^T x = y (lower = false: backward, L^T[i][k] = W[k*ld+i]) for column p of
// the right-hand sides x (m x np, in place), lane-parallel dot products.
__device__ void tri_solve_warp(const double* W, int m, int ld, double* x, int np, int p,
                               bool lower) {
  const int lane = threadIdx.x & 31;
  for (int s = 0; s < m; ++s) {
    const int i = lower ? s : m - 1 - s;
    double acc = 0.0;
    if (lower) {
      for (int k = lane; k < i; k += 32) acc += W[i * ld + k] * x[k * np + p];
    } else {
      for (int k = i + 1 + lane; k < m; k += 32) acc += W[k * ld + i] * x[k * np + p];
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) x[i * np + p] = (x[i * np + p] - acc) / W[i * ld + i];
    __syncwarp();
  }
}

// solve_ar (als_solver.py:212-238), method "cholesky": X (m x np) solves
// (sym(R) + eps max|sym(R)| I) X = S.  *used_lu is set when the Cholesky
// met a non-positive pivot and the pivoted elimination ran instead.
__global__ void __launch_bounds__(kAlsThreads) als_cholesky_solve_kernel(
    const double* R, const double* S, int m, int np, double eps, double* X, int* used_lu) {
  extern __shared__ double als_smem[];
  __shared__ double red[32];
  __shared__ int s_piv;
  const int ld = m + 1;
  double* W = als_smem;           // m x ld
  double* x = W + size_t(m) * ld;  // m x np
  const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5;
  load_system(R, m, ld, eps, W, red);
  for (int idx = tid; idx < m * np; idx += nth) x[idx] = S[idx];
  __syncthreads();
  bool ok = true;
  for (int j = 0; j < m; ++j) {
    const double d = W[j * ld + j];  // the same value in every thread
    if (!(d > 0.0)) {
      ok = false;
      break;
    }
    const double ljj = sqrt(d);
    for (int i = j + 1 + tid; i < m; i += nth) W[i * ld + j] /= ljj;
    __syncthreads();
    if (tid == 0) W[j * ld + j] = ljj;
    const int t = m - j - 1;
    for (int idx = tid; idx < t * t; idx += nth) {
      const int i = j + 1 + idx / t, k = j + 1 + idx % t;
      if (k <= i) W[i * ld + k] -= W[i * ld + j] * W[k * ld + j];
    }
    __syncthreads();
  }
  if (ok) {
    if (warp < np) {
      tri_solve_warp(W, m, ld, x, np, warp, true);
      tri_solve_warp(W, m, ld, x, np, warp, false);
    }
    __syncthreads();
    for (int idx = tid; idx < m * np; idx += nth) X[idx] = x[idx];
    return;
  }
  // Gaussian elimination with partial pivoting on the shifted system
  __syncthreads();
  if (tid == 0) *used_lu = 1;
  load_system(R, m, ld, eps, W, red);
  for (int idx = tid; idx < m * np; idx += nth) x[idx] = S[idx];
  __syncthreads();
  for (int j = 0; j < m; ++j) {
    if (tid == 0) {
      int p = j;
      double best = fabs(W[j * ld + j]);
      for (int i = j + 1; i < m; ++i)
        if (fabs(W[i * ld + j]) > best) {
          best = fabs(W[i * ld + j]);
          p = i;
        }
      s_piv = p;
    }
    __syncthreads();
    const int p = s_piv;
    if (p != j) {
      for (int k = tid; k < m; k += nth) {
        const double a = W[j * ld + k];
        W[j * ld + k] = W[p * ld + k];
        W[p * ld + k] = a;
      }
      for (int q = tid; q < np; q += nth) {
        const double a = x[j * np + q];
        x[j * np + q] = x[p * np + q];
        x[p * np + q] = a;
      }
    }
    __syncthreads();
    const double piv = W[j * ld + j];
    const int t = m - j - 1;
    // multipliers first (column j below the pivot), then the trailing block
    for (int i = j + 1 + tid; i < m; i += nth) W[i * ld + j] = piv != 0.0 ? W[i * ld + j] / piv : 0.0;
    __syncthreads();
    for (int idx = tid; idx < t * (t + np); idx += nth) {
      const int i = j + 1 + idx / (t + np), c = idx % (t + np);
      const double f = W[i * ld + j];
      if (c < t) W[i * ld + j + 1 + c] -= f * W[j * ld + j + 1 + c];
      else x[i * np + (c - t)] -= f * x[j * np + (c - t)];
    }
    __syncthreads();
  }
  // back substitution with the upper factor (one warp per column)
  if (warp < np) {
    const int lane = tid & 31;
    for (int i = m - 1; i >= 0; --i) {
      double acc = 0.0;
      for (int k = i + 1 + lane; k < m; k += 32) acc += W[i * ld + k] * x[k * np + warp];
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) x[i * np + warp] = (x[i * np + warp] - acc) / W[i * ld + i];
      __syncwarp();
    }
  }
  __syncthreads();
  for (int idx = tid; idx < m * np; idx += nth) X[idx] = x[idx];
}

// W = (R + R^T) / 2 (m x m)
__global__ void als_symmetrize_kernel(const double* R, int m, double* W) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < m * m; idx += gridDim.x * blockDim.x) {
    const int i = idx / m, j = idx - i * m;
    W[idx] = 0.5 * (R[size_t(i) * m + j] + R[size_t(j) * m + i]);
  }
}

// f[i] = 1 / s[i] where s[i] > rcond s[0], else 0 (pinv's cutoff)
__global__ void als_pinv_factors_kernel(const double* s, int m, double rcond, double* f) {
  for (int i = threadIdx.x; i < m; i += blockDim.x) f[i] = s[i] > rcond * s[0] ? 1.0 / s[i] : 0.0;
}

// y[i][p] *= f[i]
__global__ void als_scale_rows_kernel(double* y, int m, int np, const double* f) {
  for (int idx = threadIdx.x; idx < m * np; idx += blockDim.x) y[idx] *= f[idx / np];
}

// M[(y,p)][(x,q)] = a12g[y][x][p][q]  (nD pD x nD pD)
__global__ void als_pair_matrix_kernel(const double* a12g, int nD, int pD, double* M) {
  const int n = nD * pD;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n * n; idx += gridDim.x * blockDim.x) {
    const int r = idx / n, c = idx - r * n;
    const int y = r / pD, p = r - y * pD, x = c / pD, q = c - x * pD;
    M[idx] = a12g[((size_t(y) * nD + x) * pD + p) * pD + q];
  }
}

// initialize_reduced_tensors (als_solver.py:120-147) from M = U diag(s) V^T:
// a1r[y][u][p] = U[(y,p)][u] sqrt(s_u / s_0), a2r[x][v][q] = V[(x,q)][v] sqrt(s_v / s_0)
__global__ void als_init_kernel(const double* U, const double* s, const double* V, int nD,
                                int bD, int pD, double* a1r, double* a2r) {
  const int n = nD * pD, tot = nD * bD * pD;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < tot; idx += gridDim.x * blockDim.x) {
    const int y = idx / (bD * pD), u = (idx / pD) % bD, p = idx % pD;
    const double sc = sqrt(s[u] / s[0]);
    a1r[idx] = U[size_t(y * pD + p) * n + u] * sc;
    a2r[idx] = V[size_t(y * pD + p) * n + u] * sc;
  }
}

// cost = sum Na a12n - 2 sum n12g a12n (one CTA, fixed order)
__global__ void als_cost_kernel(const double* na, const double* n12g, const double* a12n, int n,
                                double* cost) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += (na[i] - 2.0 * n12g[i]) * a12n[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) r += red[w];
    *cost = r;
  }
}

struct AlsDims {
  int64_t nD, bD, pD;
  int64_t m() const { return nD * bD; }
  int64_t pair() const { return nD * nD * pD * pD; }
};

View v4(const double* p, int64_t a, int64_t b, int64_t c, int64_t d) { return View(p, {a, b, c, d}); }
View v3(const double* p, int64_t a, int64_t b, int64_t c) { return View(p, {a, b, c}); }
View v5(const double* p, int64_t a, int64_t b, int64_t c, int64_t d, int64_t e) {
  return View(p, {a, b, c, d, e});
}

// calculate_cost (als_solver.py:253-262) into *cost, n12g = n12 . a12g given
void als_cost(Ctx& c, const AlsDims& g, const double* a1r, const double* a2r, const double* n12,
              const double* n12g, double* cost) {
  const int64_t nD = g.nD, bD = g.bD, pD = g.pD;
  Scope scope(c);
  double* a12n = c.alloc<double>(g.pair());
  double* na = c.alloc<double>(g.pair());
  einsum(c, "yup,xuq->yxpq", v3(a1r, nD, bD, pD), v3(a2r, nD, bD, pD), v4(a12n, nD, nD, pD, pD));
  einsum(c, "yxYX,yxpq->YXpq", v4(n12, nD, nD, nD, nD), v4(a12n, nD, nD, pD, pD),
         v4(na, nD, nD, pD, pD));
  if (c.sizing()) return;
  KernelTimer kt(c.stream, "als_cost_kernel", kUnitFlop, 4.0 * double(g.pair()));
  als_cost_kernel<<<1, 256, 0, c.stream>>>(na, n12g, a12n, int(g.pair()), cost);
  CTM_LAUNCH_CHECK();
}

// solve_ar (als_solver.py:212-243): X (m x pD) from R (m x m) and S (m x pD)
void als_solve_ar(Ctx& c, const AlsDims& g, const double* R, const double* S, int method,
                  double eps, double* X, int* used_lu) {
  const int m = int(g.m()), np = int(g.pD);
  if (method == 0) {
    if (c.sizing()) return;
    const size_t smem = (size_t(m) * (m + 1) + size_t(m) * np) * sizeof(double);
    CTM_CUDA(cudaFuncSetAttribute(als_cholesky_solve_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    KernelTimer kt(c.stream, "als_cholesky_solve_kernel", kUnitFlop, double(m) * m * m / 3.0);
    als_cholesky_solve_kernel<<<1, kAlsThreads, smem, c.stream>>>(R, S, m, np, eps, X, used_lu);
    CTM_LAUNCH_CHECK();
    return;
  }
  // pinv(R, hermitian=True, rcond=eps) @ S from the SVD of the symmetrised R:
  // for symmetric R the singular values are |eigenvalues| and
  // V diag(1/s) U^T = sum_i v_i v_i^T / lambda_i
  Scope scope(c);
  double* W = c.alloc<double>(size_t(m) * m);
  double* U = c.alloc<double>(size_t(m) * m);
  double* s = c.alloc<double>(m);
  double* V = c.alloc<double>(size_t(m) * m);
  double* f = c.alloc<double>(m);
  double* t = c.alloc<double>(size_t(m) * np);
  if (!c.sizing()) {
    als_symmetrize_kernel<<<grid_for(int64_t(m) * m, 256), 256, 0, c.stream>>>(R, m, W);
    CTM_LAUNCH_CHECK();
  }
  svd_thin(c, W, m, m, U, s, V);
  einsum(c, "ki,kp->ip", View(U, {m, m}), View(S, {m, np}), View(t, {m, np}));
  if (!c.sizing()) {
    als_pinv_factors_kernel<<<1, 256, 0, c.stream>>>(s, m, eps, f);
    CTM_LAUNCH_CHECK();
    als_scale_rows_kernel<<<1, 256, 0, c.stream>>>(t, m, np, f);
    CTM_LAUNCH_CHECK();
  }
  einsum(c, "ij,jp->ip", View(V, {m, m}), View(t, {m, np}), View(X, {m, np}));
}

double read_scalar(Ctx& c, const double* p) {
  double h = 0.0;
  CTM_CUDA(cudaMemcpyAsync(&h, p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  CTM_CUDA(cudaStreamSynchronize(c.stream));
  return h;
}

}  // namespace

void als_solve(Ctx& c, const double* n12, const double* a12g, int64_t nD, int64_t bD,
               int64_t pD, int niter, double tol, int method, double eps, double* a1r,
               double* a2r, int* iterations) {
  const AlsDims g{nD, bD, pD};
  CTM_REQUIRE(nD >= 1 && bD >= 1 && pD >= 1 && bD <= nD * pD, CTM_ERR_INVALID,
              "ALS: need 1 <= bD <= nD pD");
  CTM_REQUIRE(method == 0 || method == 1, CTM_ERR_INVALID,
              "ALS method must be 0 (cholesky) or 1 (pinv)");
  CTM_REQUIRE(niter >= 0, CTM_ERR_INVALID, "ALS: niter must be >= 0");
  CTM_REQUIRE(method == 1 || (g.m() <= kAlsMaxM && pD <= kAlsMaxP), CTM_ERR_UNSUPPORTED,
              "ALS cholesky: needs nD bD <= 160 and pD <= 8");
  const int64_t n = nD * pD, m = g.m();
  Scope scope(c);
  double* M = c.alloc<double>(size_t(n) * n);
  double* U = c.alloc<double>(size_t(n) * n);
  double* sv = c.alloc<double>(n);
  double* V = c.alloc<double>(size_t(n) * n);
  double* n12g = c.alloc<double>(g.pair());
  double* T = c.alloc<double>(size_t(nD) * nD * nD * bD * pD);
  double* R = c.alloc<double>(size_t(m) * m);
  double* S = c.alloc<double>(size_t(m) * pD);
  double* cost = c.alloc<double>(1);
  int* used_lu = c.alloc<int>(1);
  const View N = v4(n12, nD, nD, nD, nD);
  // initialize_tensors (als_solver.py:114-118)
  if (!c.sizing()) {
    als_pair_matrix_kernel<<<grid_for(n * n, 256), 256, 0, c.stream>>>(a12g, int(nD), int(pD), M);
    CTM_LAUNCH_CHECK();
    CTM_CUDA(cudaMemsetAsync(used_lu, 0, sizeof(int), c.stream));
  }
  svd_thin(c, M, n, n, U, sv, V);
  if (!c.sizing()) {
    als_init_kernel<<<grid_for(m * pD, 256), 256, 0, c.stream>>>(U, sv, V, int(nD), int(bD),
                                                                 int(pD), a1r, a2r);
    CTM_LAUNCH_CHECK();
  }
  einsum(c, "yxYX,yxpq->YXpq", N, v4(a12g, nD, nD, pD, pD), v4(n12g, nD, nD, pD, pD));
  auto half_step = [&](const double* fixed, double* solved, bool first) {
    const View fx = v3(fixed, nD, bD, pD);
    if (first) {
      // build_s1 / build_r1 (als_solver.py:245-251)
      einsum(c, "YXpQ,XUQ->YUp", v4(n12g, nD, nD, pD, pD), fx, v3(S, nD, bD, pD));
      einsum(c, "yxYX,xuq->yYXuq", N, fx, v5(T, nD, nD, nD, bD, pD));
      einsum(c, "yYXuQ,XUQ->YUyu", v5(T, nD, nD, nD, bD, pD), fx, v4(R, nD, bD, nD, bD));
    } else {
      // build_s2 / build_r2
      einsum(c, "YXPq,YVP->XVq", v4(n12g, nD, nD, pD, pD), fx, v3(S, nD, bD, pD));
      einsum(c, "yxYX,yvp->xYXvp", N, fx, v5(T, nD, nD, nD, bD, pD));
      einsum(c, "xYXvP,YVP->XVxv", v5(T, nD, nD, nD, bD, pD), fx, v4(R, nD, bD, nD, bD));
    }
    als_solve_ar(c, g, R, S, method, eps, solved, used_lu);
  };
  als_cost(c, g, a1r, a2r, n12, n12g, cost);
  if (c.sizing()) {
    half_step(a2r, a1r, true);
    half_step(a1r, a2r, false);
    return;
  }
  // solve_torch (als_solver.py:56-82)
  double d1 = std::fabs(read_scalar(c, cost));
  int it = 0;
  for (int i = 0; i < niter; ++i) {
    half_step(a2r, a1r, true);
    half_step(a1r, a2r, false);
    als_cost(c, g, a1r, a2r, n12, n12g, cost);
    const double d2 = read_scalar(c, cost);
    it = i + 1;
    const double err = std::fabs(d2 - d1) / std::fabs(d1);
    if (err < tol && i > 1) break;
    d1 = d2;
  }
  if (iterations != nullptr) *iterations = it;
}

void als_cost_only(Ctx& c, const double* a1r, const double* a2r, const double* a12g,
                   const double* n12, int64_t nD, int64_t bD, int64_t pD, double* cost) {
  const AlsDims g{nD, bD, pD};
  Scope scope(c);
  double* n12g = c.alloc<double>(g.pair());
  einsum(c, "yxYX,yxpq->YXpq", v4(n12, nD, nD, nD, nD), v4(a12g, nD, nD, pD, pD),
         v4(n12g, nD, nD, pD, pD));
  als_cost(c, g, a1r, a2r, n12, n12g, cost);
}

}  // namespace ctm

// ---------------------------------------------------------------- C ABI
using namespace ctm;

extern "C" {

int ctm_als_solve(const double* n12, const double* a12g, int64_t nD, int64_t bD, int64_t pD,
                  int32_t niter, double tol, int32_t method, double epsilon, double* a1r,
                  double* a2r, int32_t* iterations, void* ws, size_t* ws_bytes,
                  ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, reinterpret_cast<cudaStream_t>(stream), [&](Ctx& c) {
    if (!c.sizing())
      CTM_REQUIRE(n12 != nullptr && a12g != nullptr && a1r != nullptr && a2r != nullptr,
                  CTM_ERR_INVALID, "NULL tensor pointer");
    int it = 0;
    als_solve(c, n12, a12g, nD, bD, pD, niter, tol, method, epsilon, a1r, a2r, &it);
    if (iterations != nullptr && !c.sizing()) *iterations = it;
  });
}

int ctm_als_cost(const double* a1r, const double* a2r, const double* a12g, const double* n12,
                 int64_t nD, int64_t bD, int64_t pD, double* cost, void* ws, size_t* ws_bytes,
                 ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, reinterpret_cast<cudaStream_t>(stream), [&](Ctx& c) {
    CTM_REQUIRE(nD >= 1 && bD >= 1 && pD >= 1, CTM_ERR_INVALID, "ALS: bad dimensions");
    if (!c.sizing())
      CTM_REQUIRE(a1r != nullptr && a2r != nullptr && a12g != nullptr && n12 != nullptr &&
                      cost != nullptr,
                  CTM_ERR_INVALID, "NULL tensor pointer");
    als_cost_only(c, a1r, a2r, a12g, n12, nD, bD, pD, cost);
  });
}

}  // extern "C"
