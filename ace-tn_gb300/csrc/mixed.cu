// Mixed-precision projector construction (CTM_PREC_MIXED), half-system rSVD:
//  * range finder (the power-iteration products) in one BF16 tensor-core
//    pass with FP32 accumulation;
//  * Rayleigh-Ritz products B = Q^T Q1 Q4 and the projector products
//    P1 = Q1^T U, P2 = Q4 V in 3xBF16 split precision;
//  * orthonormalization, the SVD of B, the truncation and the s^(-1/2)
//    scaling in FP64.
// Algorithm of acetn/renormalization/projectors.py:138-174 with
// acetn/linalg/fused_matmul_svd_lowrank.py:4-52.
#include "engine.cuh"
#include "tc_gemm.cuh"

#include <algorithm>

namespace ctm {

namespace {

// BF16 operands of one quarter matrix Q (rows x cols): Q itself (K = cols)
// and its transpose (K = rows), hi and lo parts.
// The stored values are Q * max|Q| relative to the normalised quarter tensor
// of the reference: *scale (device) holds max|Q|, and every product that
// leaves the range finder divides by it.
struct QOps {
  bf16 *q_hi = nullptr, *q_lo = nullptr, *t_hi = nullptr, *t_lo = nullptr;
  double* scale = nullptr;
  int64_t rows = 0, cols = 0, ld = 0, ldt = 0;
  TcOperand q(bool lo) const { return TcOperand{q_hi, lo ? q_lo : nullptr, rows, cols, ld}; }
  TcOperand t(bool lo) const { return TcOperand{t_hi, lo ? t_lo : nullptr, cols, rows, ldt}; }
};

QOps alloc_ops(Ctx& c, int64_t rows, int64_t cols) {
  QOps o;
  o.rows = rows;
  o.cols = cols;
  o.ld = tc_ld(cols);
  o.ldt = tc_ld(rows);
  o.q_hi = c.alloc<bf16>(size_t(rows) * o.ld);
  o.q_lo = c.alloc<bf16>(size_t(rows) * o.ld);
  o.t_hi = c.alloc<bf16>(size_t(cols) * o.ldt);
  o.t_lo = c.alloc<bf16>(size_t(cols) * o.ldt);
  o.scale = c.alloc<double>(1);
  return o;
}

// Double-layer site matrix of A = S.A(k) (dims l, u, r, d, p):
//   DL[(r,R,d,D)][(l,L,u,U)] = sum_p A[l][u][r][d][p] A*[L][U][R][D][p]
// as a K-major BF16 hi/lo operand (K = (l,L,u,U)), leading dimension ld.
// Contracting a ket-bra pair of environment legs against it replaces the two
// one-layer contractions of make_quarter_tensor / renormalize_ej, whose
// K = D^2 and D^2 d are too short to keep the tensor cores busy.
// Each CTA copies A into shared memory in FP32 (legs l, u, r, d, p, p
// fastest) with the per-column offsets of the ket (l, u) and bra (L, U)
// legs, then forms kDlRows rows: one FP32 FMA chain over p per entry (its
// rounding, ~1e-7 of the terms, sits far below the hi/lo pair's 16 bits) and
// the hi/lo split in FP32 (x - hi is exact).  FP64 arithmetic and the
// per-entry index decoding made the earlier form several times slower.
constexpr int kDlRows = 8;

// x / d for x, d < 2^16 with m = ceil(2^32 / d) (d >= 2): q = (x m) >> 32 is
// exact, as x (m d - 2^32) < x d < 2^32.  The double-layer kernels decode
// every index through it instead of 32-bit division sequences.
struct Div16 {
  uint32_t d, m;
};
inline Div16 make_div16(int d) {
  return Div16{uint32_t(d), d >= 2 ? uint32_t(((uint64_t(1) << 32) + uint64_t(d) - 1) / d) : 0u};
}
__device__ __forceinline__ uint32_t div16(uint32_t x, Div16 v) {
  return v.d == 1 ? x : __umulhi(x, v.m);
}

inline size_t double_layer_smem(int64_t D, int64_t d) {
  const int64_t D4 = D * D * D * D;
  return size_t(D4 * d + 2 * D4) * 4;
}

__global__ void __launch_bounds__(256) double_layer_kernel(const double* A, int64_t s0,
                                                           int64_t s1, int64_t s2, int64_t s3,
                                                           int64_t s4, Div16 vD, Div16 vd,
                                                           bf16* hi, bf16* lo, int64_t ld) {
  extern __shared__ float dl_smem[];
  const int D = int(vD.d), d = int(vd.d);
  const int D2 = D * D, D4 = D2 * D2;
  const int c1 = D2 * d, c0 = D * c1, c2 = D * d, c3 = d;  // canonical strides of l, u, r, d
  float* As = dl_smem;                                       // D^4 d
  int* kofs = reinterpret_cast<int*>(As + D4 * d);           // ket offset of column k
  int* bofs = kofs + D4;                                     // bra offset of column k
  for (int i = threadIdx.x; i < D4 * d; i += blockDim.x) {
    uint32_t t = uint32_t(i), q = div16(t, vd);
    const int p = int(t - q * d);
    t = q;
    q = div16(t, vD);
    const int dd = int(t - q * D);
    t = q;
    q = div16(t, vD);
    const int r = int(t - q * D);
    t = q;
    q = div16(t, vD);
    const int u = int(t - q * D), l = int(q);
    As[i] = float(A[l * s0 + u * s1 + r * s2 + dd * s3 + p * s4]);
  }
  for (int k = threadIdx.x; k < D4; k += blockDim.x) {
    uint32_t t = uint32_t(k), q = div16(t, vD);
    const int U = int(t - q * D);
    t = q;
    q = div16(t, vD);
    const int u = int(t - q * D);
    t = q;
    q = div16(t, vD);
    const int L = int(t - q * D), l = int(q);
    kofs[k] = l * c0 + u * c1;
    bofs[k] = L * c0 + U * c1;
  }
  __syncthreads();
  const int n_end = min(D4, int(blockIdx.x + 1) * kDlRows);
  for (int n = int(blockIdx.x) * kDlRows; n < n_end; ++n) {
    uint32_t t = uint32_t(n), q = div16(t, vD);
    const int DD = int(t - q * D);
    t = q;
    q = div16(t, vD);
    const int dd = int(t - q * D);
    t = q;
    q = div16(t, vD);
    const int R = int(t - q * D), r = int(q);
    const int kn = r * c2 + dd * c3, bn = R * c2 + DD * c3;
    bf16* hrow = hi + int64_t(n) * ld;
    bf16* lrow = lo + int64_t(n) * ld;
    for (int k = threadIdx.x; k < D4; k += blockDim.x) {
      const float* ket = As + kofs[k] + kn;
      const float* bra = As + bofs[k] + bn;
      float v = 0.f;
      for (int p = 0; p < d; ++p) v = fmaf(ket[p], bra[p], v);
      const bf16 h = __float2bfloat16(v);
      hrow[k] = h;
      lrow[k] = __float2bfloat16(v - __bfloat162float(h));
    }
  }
}

struct DLOp {
  bf16 *hi = nullptr, *lo = nullptr;
  int64_t n = 0, ld = 0;
  TcOperand op() const { return TcOperand{hi, lo, n, n, ld}; }
};

DLOp double_layer(Ctx& c, const View& ak, int64_t D, int64_t d) {
  DLOp o;
  o.n = D * D * D * D;
  o.ld = tc_ld(o.n);
  o.hi = c.alloc<bf16>(size_t(o.n) * o.ld);
  o.lo = c.alloc<bf16>(size_t(o.n) * o.ld);
  if (!c.sizing()) {
    const size_t smem = double_layer_smem(D, d);
    CTM_REQUIRE(o.n * o.n < (int64_t(1) << 31) && smem <= size_t(200) * 1024 &&
                    o.n * d < (int64_t(1) << 16),
                CTM_ERR_UNSUPPORTED,
                "double layer: needs D^4 d < 2^16 and D^4 (d + 2) floats in shared memory "
                "(the one-layer form serves larger D)");
    KernelTimer kt(c.stream, "double_layer_kernel", kUnitByte, 4.0 * double(o.n) * o.n);
    CTM_CUDA(cudaFuncSetAttribute(double_layer_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    double_layer_kernel<<<unsigned((o.n + kDlRows - 1) / kDlRows), 256, smem, c.stream>>>(
        ak.p, ak.stride[0], ak.stride[1], ak.stride[2], ak.stride[3], ak.stride[4],
        make_div16(int(D)), make_div16(int(d)), o.hi, o.lo, o.ld);
    CTM_LAUNCH_CHECK();
  }
  return o;
}

// The two site-tensor steps of the enlarged corner and of the edge
// renormalization run either as one GEMM against the double-layer matrix
// (K = D^4: few, long products; D^8 entries) or as the reference's two
// one-layer steps (K = D^2 and D^2 d: the algorithmic FLOP count, larger
// intermediates).  0: double layer up to D = 6, one layer from D = 8;
// 1: always the double layer; 2: always one layer.
int g_contraction_form = 0;

bool one_layer_for(int64_t D) {
  return g_contraction_form == 2 || (g_contraction_form == 0 && D >= 8);
}

// Site-tensor operands of the one-layer steps (A = S.A(k), legs l u r d p):
//   bra[(R,D,P)][(L,U)] = A[L][U][R][D][P]   (K = D^2, leading dimension ldb)
//   ket[(r,d)][(p,l,u)] = A[l][u][r][d][p]   (K = D^2 d, leading dimension ldk)
__global__ void site_operands_kernel(const double* A, int64_t s0, int64_t s1, int64_t s2,
                                     int64_t s3, int64_t s4, int D, int d, bf16* bh, bf16* bl,
                                     int64_t ldb, bf16* kh, bf16* kl, int64_t ldk) {
  const int64_t D2 = int64_t(D) * D, nb = D2 * d * D2;
  for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < 2 * nb;
       idx += int64_t(gridDim.x) * blockDim.x) {
    double v;
    bf16 *h, *l;
    int64_t off;
    if (idx < nb) {
      const int64_t n = idx / D2, k = idx - n * D2;
      const int P = int(n % d), Dd = int((n / d) % D), R = int(n / (int64_t(d) * D));
      const int U = int(k % D), L = int(k / D);
      v = A[L * s0 + U * s1 + R * s2 + Dd * s3 + P * s4];
      h = bh;
      l = bl;
      off = n * ldb + k;
    } else {
      const int64_t i = idx - nb, n = i / (D2 * d), k = i - n * (D2 * d);
      const int dd = int(n % D), r = int(n / D);
      const int u = int(k % D), lg = int((k / D) % D), p = int(k / D2);
      v = A[lg * s0 + u * s1 + r * s2 + dd * s3 + p * s4];
      h = kh;
      l = kl;
      off = n * ldk + k;
    }
    const bf16 hv = __double2bfloat16(v);
    h[off] = hv;
    l[off] = __double2bfloat16(v - double(__bfloat162float(hv)));
  }
}

// The one-layer form of the two site-tensor steps (3xBF16):
//   T1[(i,j,R,D)][(p,l,u)] = sum_(L,U) X[(i,j,l,u)][(L,U)] A*[L,U,R,D,P]
//   out[(i,j,R,D)][(r,d)]  = sum_(p,l,u) T1 A[l,u,r,d,p]
// X has rows (i,j,l,u) (i, j the two boundary indices) and K = (L,U) padded
// to ldx; outB gives the layout of the result (rows (i,j,R,D), columns
// (r,d)); with want_absmax, *absmax receives max |result|.
void one_layer_steps(Ctx& c, const View& ak, int64_t D, int64_t d, int64_t ni, int64_t nj,
                     const bf16* xh, const bf16* xl, int64_t ldx, TcOut outB, bool want_absmax,
                     double* absmax, const char* step_a, const char* step_b) {
  const int64_t D2 = D * D, Kb = D2 * d, ldb = tc_ld(D2), ldt = tc_ld(Kb);
  const int64_t rows = ni * nj * D2;
  const TcMode x3 = TcMode::kBf16x3;
  Scope scope(c);
  bf16* bh = c.alloc<bf16>(size_t(Kb) * ldb);
  bf16* bl = c.alloc<bf16>(size_t(Kb) * ldb);
  bf16* kh = c.alloc<bf16>(size_t(D2) * ldt);
  bf16* kl = c.alloc<bf16>(size_t(D2) * ldt);
  if (!c.sizing()) {
    KernelTimer kt(c.stream, "site_operands_kernel", kUnitByte, 2.0 * 4.0 * double(Kb) * D2);
    site_operands_kernel<<<grid_for(2 * Kb * D2, 256), 256, 0, c.stream>>>(
        ak.p, ak.stride[0], ak.stride[1], ak.stride[2], ak.stride[3], ak.stride[4], int(D),
        int(d), bh, bl, ldb, kh, kl, ldt);
    CTM_LAUNCH_CHECK();
  }
  bf16* th = c.alloc<bf16>(size_t(rows) * ldt);
  bf16* tl = c.alloc<bf16>(size_t(rows) * ldt);
  {
    TcLayout l;  // rows (i,j,l,u) of X; columns (R,D,P) of bra
    l.nm = 4;
    l.me[0] = ni; l.ms[0] = nj * D2 * ldt;
    l.me[1] = nj; l.ms[1] = D2 * ldt;
    l.me[2] = D;  l.ms[2] = D;
    l.me[3] = D;  l.ms[3] = 1;
    l.nn = 3;
    l.ne[0] = D; l.ns[0] = D * ldt;
    l.ne[1] = D; l.ns[1] = ldt;
    l.ne[2] = d; l.ns[2] = D2;
    TcOut out;
    out.add(TcKind::kBf16Hi, th, l).add(TcKind::kBf16Lo, tl, l);
    out.name = step_a;
    tc_gemm(c, TcOperand{xh, xl, rows, D2, ldx}, TcOperand{bh, bl, Kb, D2, ldb}, x3, out);
  }
  outB.name = step_b;
  outB.algo_flops = 2.0 * double(rows) * D2 * Kb;
  if (want_absmax)
    tc_gemm_absmax(c, TcOperand{th, tl, rows, Kb, ldt}, TcOperand{kh, kl, D2, Kb, ldt}, x3, outB,
                   absmax);
  else
    tc_gemm(c, TcOperand{th, tl, rows, Kb, ldt}, TcOperand{kh, kl, D2, Kb, ldt}, x3, outB);
}

// X[(c,e)][(l,L,u,U)] = sum_a (C_k E_k)[a][(c,u,U)] E_{k+3}[e][a][l][L]: the
// boundary part of the enlarged corner of direction k (the first two einsums
// of make_quarter_tensor, acetn/renormalization/projectors.py:52-53), as a
// K-major BF16 hi/lo operand (K = (l,L,u,U) = D^4).  t1 = C E_k in FP32, then
// a K = chi tensor-core GEMM whose epilogue writes X.  For the one-layer
// steps (one_layer) the same values are laid out as X[(c,e,l,u)][(L,U)]
// with K = D^2 padded to 64.
struct XOp {
  bf16 *hi = nullptr, *lo = nullptr;
  int64_t rows = 0, k = 0, ld = 0, cc = 0, e = 0;
};

XOp x_operand(Ctx& c, const Site& S, int k, const char* name = "enlarged corner, edge step",
               bool one_layer = false) {
  int64_t sh[6], rows, cols;
  quarter_dims(S, k, rows, cols, sh);
  const View ck = S.C(k), ek1 = S.E(3 + k), ek2 = S.E(k);
  const int64_t a = ck.shape[0], cc = sh[0], E = sh[3], D = S.D, D2 = D * D;
  const TcMode x3 = TcMode::kBf16x3;
  XOp x;
  x.cc = cc;
  x.e = E;
  x.rows = one_layer ? cc * E * D2 : cc * E;
  x.k = one_layer ? D2 : D2 * D2;
  x.ld = tc_ld(x.k);
  x.hi = c.alloc<bf16>(size_t(x.rows) * x.ld);
  x.lo = c.alloc<bf16>(size_t(x.rows) * x.ld);
  bf16 *xh = x.hi, *xl = x.lo;
  const int64_t ldx = x.ld;
  Scope scope(c);
  // t1 = C E_k (a x (c,u,U)), FP32
  float* t1 = c.alloc<float>(size_t(a) * cc * D2);
  {
    Scope s2(c);
    float* cf = c.alloc<float>(size_t(ck.numel()));
    float* ef = c.alloc<float>(size_t(ek2.numel()));
    to_f32(c, ck.p, cf, ck.numel());
    to_f32(c, ek2.p, ef, ek2.numel());
    einsum(c, "ab,bcuU->acuU", ViewF(cf, {ck.shape[0], ck.shape[1]}),
           ViewF(ef, {ek2.shape[0], ek2.shape[1], D, D}), ViewF(t1, {a, cc, D, D}));
  }
  // GEMM 1 operands: E_{k+3} as ((e,l,L) x a) and t1^T as ((c,u,U) x a)
  const int64_t ld2 = tc_ld(a);
  bf16* eh = c.alloc<bf16>(size_t(E) * D2 * ld2);
  bf16* el = c.alloc<bf16>(size_t(E) * D2 * ld2);
  {
    Gather g;
    g.nr = 2;
    g.re[0] = E; g.rs[0] = ek1.stride[0];
    g.re[1] = D2; g.rs[1] = 1;
    g.nk = 1;
    g.ke[0] = a; g.ks[0] = ek1.stride[1];
    gather_split_bf16(c, ek1.p, g, eh, el, ld2);
  }
  bf16* th = c.alloc<bf16>(size_t(cc) * D2 * ld2);
  bf16* tl = c.alloc<bf16>(size_t(cc) * D2 * ld2);
  split_bf16(c, t1, a, cc * D2, cc * D2, true, th, tl, ld2);
  // X[(c,e)][(l,L,u,U)]: rows of GEMM 1 are (e,l,L), columns (c,u,U), so
  // that each epilogue thread's consecutive columns are consecutive (u,U)
  // in X: aligned groups of 4 (D^2 % 4 == 0) go out as one 8-byte store
  // (with rows (c,u,U) every element was a separate 2-byte store and this
  // K = chi GEMM ran at a few per cent of the tensor pipe)
  {
    TcLayout l;
    l.nm = 3;
    l.nn = 3;
    l.me[0] = E;  l.me[1] = D; l.me[2] = D;
    l.ne[0] = cc; l.ne[1] = D; l.ne[2] = D;
    if (one_layer) {  // X[((c E + e) D + l) D + u][L D + U]
      l.ms[0] = D2 * ldx; l.ms[1] = D * ldx; l.ms[2] = D;
      l.ns[0] = E * D2 * ldx; l.ns[1] = ldx; l.ns[2] = 1;
    } else {          // X[c E + e][((l D + L) D + u) D + U]
      l.ms[0] = ldx; l.ms[1] = D * D2; l.ms[2] = D2;
      l.ns[0] = E * ldx; l.ns[1] = D; l.ns[2] = 1;
    }
    TcOut out;
    out.add(TcKind::kBf16Hi, xh, l).add(TcKind::kBf16Lo, xl, l);
    out.name = name;
    tc_gemm(c, TcOperand{eh, el, E * D2, a, ld2}, TcOperand{th, tl, cc * D2, a, ld2}, x3, out);
  }
  return x;
}

// make_quarter_tensor (acetn/renormalization/projectors.py:35-60) on tensor
// cores, 3xBF16 throughout.  The four einsums become
//   t1 = C E_k (FP32, the small chi^3 D^2 step),
//   X[(c,e)][(l,L,u,U)] = sum_a t1[a][(c,u,U)] E_{k+3}[e][a][l][L]      (K = chi),
//   Q[(c,r,R)][(e,d,D)] = sum_(l,L,u,U) DL[(r,R,d,D)][(l,L,u,U)] X    (K = D^4),
// with the double-layer matrix DL of the site tensor (the two A / A* steps
// of the reference in one GEMM with a long K).  Each epilogue stores into the
// layout the next step reads, with the GEMM rows (one per epilogue lane) on
// the index that is contiguous in that layout; Q^T comes from a tiled
// transpose, and max|Q| from the last epilogue.
QOps quarter_mixed(Ctx& c, const Site& S, int k, bool fp64 = false) {
  int64_t sh[6], rows, cols;
  quarter_dims(S, k, rows, cols, sh);
  QOps o = alloc_ops(c, rows, cols);
  if (fp64) {
    // contracted in FP64 (already divided by max|Q|), then split
    Scope s0(c);
    double* Qd = c.alloc<double>(size_t(rows) * cols);
    int64_t qs[6];
    quarter_tensor(c, S, k, Qd, qs);
    split_bf16(c, Qd, rows, cols, cols, false, o.q_hi, o.q_lo, o.ld);
    fill(c, o.scale, 1, 1.0);
    transpose_bf16(c, o.q_hi, o.q_lo, rows, cols, o.ld, o.t_hi, o.t_lo, o.ldt);
    return o;
  }
  const View ak = S.A(k);
  const int64_t cc = sh[0], E = sh[3], D = S.D, d = S.d, D2 = D * D;
  const TcMode x3 = TcMode::kBf16x3;
  Scope scope(c);
  if (one_layer_for(D)) {
    const XOp x = x_operand(c, S, k, "enlarged corner, edge step", true);
    TcLayout lq;  // Q[(c,r,R)][(e,d,D)] from rows (c,e,R,D), columns (r,d)
    lq.nm = 4;
    lq.me[0] = cc; lq.ms[0] = D2 * o.ld;
    lq.me[1] = E;  lq.ms[1] = D2;
    lq.me[2] = D;  lq.ms[2] = o.ld;
    lq.me[3] = D;  lq.ms[3] = 1;
    lq.nn = 2;
    lq.ne[0] = D; lq.ns[0] = D * o.ld;
    lq.ne[1] = D; lq.ns[1] = D;
    TcOut out;
    out.add(TcKind::kBf16Hi, o.q_hi, lq).add(TcKind::kBf16Lo, o.q_lo, lq);
    one_layer_steps(c, ak, D, d, cc, E, x.hi, x.lo, x.ld, out, true, o.scale,
                    "enlarged corner, bra step", "enlarged corner, ket step");
    transpose_bf16(c, o.q_hi, o.q_lo, rows, cols, o.ld, o.t_hi, o.t_lo, o.ldt);
    return o;
  }
  const XOp x = x_operand(c, S, k);
  const bf16 *xh = x.hi, *xl = x.lo;
  const int64_t K2 = x.k, ldx = x.ld;
  // GEMM 2 against the double-layer matrix -> Q[(c,r,R)][(e,d,D)] and max|Q|;
  // rows (c,e) from X, columns (r,R,d,D) from DL: consecutive columns are
  // consecutive (d,D) in Q, stored 4 at a time, and N = D^4 = 1296 splits
  // into six 224-wide tiles
  const DLOp dl = double_layer(c, ak, D, d);
  {
    TcLayout lq;
    lq.nm = 2;
    lq.me[0] = cc; lq.ms[0] = D2 * o.ld;
    lq.me[1] = E;  lq.ms[1] = D2;
    lq.nn = 4;
    lq.ne[0] = D; lq.ns[0] = D * o.ld;
    lq.ne[1] = D; lq.ns[1] = o.ld;
    lq.ne[2] = D; lq.ns[2] = D;
    lq.ne[3] = D; lq.ns[3] = 1;
    TcOut out;
    out.add(TcKind::kBf16Hi, o.q_hi, lq).add(TcKind::kBf16Lo, o.q_lo, lq);
    out.extra_tag = kTagTcDoubleLayer;
    out.name = "enlarged corner, double-layer step";
    // the reference's two one-layer site-tensor steps (projectors.py:54-55)
    out.algo_flops = 4.0 * double(cc) * E * D2 * D2 * D2 * d;
    tc_gemm_absmax(c, TcOperand{xh, xl, cc * E, K2, ldx}, dl.op(), x3, out, o.scale);
  }
  transpose_bf16(c, o.q_hi, o.q_lo, rows, cols, o.ld, o.t_hi, o.t_lo, o.ldt);
  return o;
}

// Y^T as a BF16 operand (q x n) from Y (n x q, ld)
TcOperand yt_operand(Ctx& c, const double* Y, int64_t n, int64_t q, int64_t ldy, bool lo) {
  const int64_t ld = tc_ld(n);
  bf16* hi = c.alloc<bf16>(size_t(q) * ld);
  bf16* lw = lo ? c.alloc<bf16>(size_t(q) * ld) : nullptr;
  split_bf16(c, Y, n, q, ldy, true, hi, lw, ld);
  return TcOperand{hi, lw, q, n, ld};
}

TcOperand yt_operand_f32(Ctx& c, const float* Y, int64_t n, int64_t q, int64_t ldy, bool lo) {
  const int64_t ld = tc_ld(n);
  bf16* hi = c.alloc<bf16>(size_t(q) * ld);
  bf16* lw = lo ? c.alloc<bf16>(size_t(q) * ld) : nullptr;
  split_bf16(c, Y, n, q, ldy, true, hi, lw, ld);
  return TcOperand{hi, lw, q, n, ld};
}

// C = A @ B^T written as the next operand (C^T, BF16 hi [+ lo]).
TcOperand gemm_to_operand(Ctx& c, const TcOperand& A, const TcOperand& B, TcMode mode, bool lo,
                          const char* name = nullptr, const double* inv_scale = nullptr) {
  const int64_t M = A.rows, N = B.rows;
  const int64_t ld = tc_ld(M);
  bf16* hi = c.alloc<bf16>(size_t(N) * ld);
  bf16* lw = lo ? c.alloc<bf16>(size_t(N) * ld) : nullptr;
  TcOut out;
  out.add(TcKind::kBf16Hi, hi, TcLayout::cols(M, N, ld));
  if (lo) out.add(TcKind::kBf16Lo, lw, TcLayout::cols(M, N, ld));
  out.name = name;
  out.inv_scale = inv_scale;
  tc_gemm(c, A, B, mode, out);
  return TcOperand{hi, lw, N, M, ld};
}

void gemm_to_f64(Ctx& c, const TcOperand& A, const TcOperand& B, TcMode mode, double* C,
                 int64_t ldc, bool transposed, const double* inv_scale,
                 const char* name = nullptr) {
  TcOut out;
  out.add(TcKind::kF64, C,
          transposed ? TcLayout::cols(A.rows, B.rows, ldc) : TcLayout::rows(A.rows, B.rows, ldc));
  out.inv_scale = inv_scale;
  out.name = name;
  tc_gemm(c, A, B, mode, out);
}

}  // namespace

// renormalize_ej (acetn/renormalization/directional_mover.py:345-366) on
// tensor cores in 3xBF16.  The four einsums become three GEMMs, the two
// site-tensor steps merged into one against the double-layer matrix DL:
//   G1 X[(a,x)][(l,L,u,U)]   = sum_b P1[b][u][U][x] E[a][b][l][L]     (K = chi)
//   G2 T[(x,r,R)][(a,d,D)]   = sum_(l,L,u,U) DL[(r,R,d,D)][(l,L,u,U)] X
//   G3 E'[y][(x,r,R)]        = sum_(a,d,D) T P2[a][d][D][y]             (K = chi D^2)
// each epilogue storing the next GEMM's K-major operand; the last writes the
// FP64 result, normalised in FP64.
void renormalize_ej_mixed(Ctx& c, const Site& S, int k, const double* P2i, int64_t Y,
                          const double* P1j, int64_t X, double* Eout) {
  const View ei = S.E(3 + k), ak = S.A(k);
  const int64_t Aa = ei.shape[0], B = ei.shape[1], D = S.D, d = S.d, D2 = D * D;
  const TcMode x3 = TcMode::kBf16x3;
  Scope scope(c);
  // G1 operands: E as ((a,l,L) x b), P1 as ((x,u,U) x b)
  const int64_t ld1 = tc_ld(B);
  bf16* a1h = c.alloc<bf16>(size_t(Aa) * D2 * ld1);
  bf16* a1l = c.alloc<bf16>(size_t(Aa) * D2 * ld1);
  {
    Gather g;
    g.nr = 2;
    g.re[0] = Aa; g.rs[0] = ei.stride[0];
    g.re[1] = D2; g.rs[1] = 1;
    g.nk = 1;
    g.ke[0] = B; g.ks[0] = ei.stride[1];
    gather_split_bf16(c, ei.p, g, a1h, a1l, ld1);
  }
  bf16* b1h = c.alloc<bf16>(size_t(X) * D2 * ld1);
  bf16* b1l = c.alloc<bf16>(size_t(X) * D2 * ld1);
  {
    Gather g;  // P1j is (b,u,U) x X row-major
    g.nr = 2;
    g.re[0] = X;  g.rs[0] = 1;
    g.re[1] = D2; g.rs[1] = X;
    g.nk = 1;
    g.ke[0] = B; g.ks[0] = D2 * X;
    gather_split_bf16(c, P1j, g, b1h, b1l, ld1);
  }
  const int64_t K4 = Aa * D2;
  const int64_t ld4 = tc_ld(K4);
  bf16* t3h = c.alloc<bf16>(size_t(X) * D2 * ld4);
  bf16* t3l = c.alloc<bf16>(size_t(X) * D2 * ld4);
  if (one_layer_for(D)) {
    // G1 -> X[(a,x,l,u)][(L,U)] (K = D^2 padded), then the one-layer steps
    // -> T[(x,r,R)][(a,d,D)]
    const int64_t ldk = tc_ld(D2);
    bf16* xh = c.alloc<bf16>(size_t(Aa) * X * D2 * ldk);
    bf16* xl = c.alloc<bf16>(size_t(Aa) * X * D2 * ldk);
    {
      TcLayout l;
      l.nm = 3;
      l.me[0] = Aa; l.ms[0] = X * D2 * ldk;
      l.me[1] = D;  l.ms[1] = D * ldk;
      l.me[2] = D;  l.ms[2] = D;
      l.nn = 3;
      l.ne[0] = X; l.ns[0] = D2 * ldk;
      l.ne[1] = D; l.ns[1] = ldk;
      l.ne[2] = D; l.ns[2] = 1;
      TcOut out;
      out.add(TcKind::kBf16Hi, xh, l).add(TcKind::kBf16Lo, xl, l);
      out.name = "edge renormalization, projector step";
      tc_gemm(c, TcOperand{a1h, a1l, Aa * D2, B, ld1}, TcOperand{b1h, b1l, X * D2, B, ld1}, x3,
              out);
    }
    TcLayout l;  // T from rows (a,x,R,D), columns (r,d)
    l.nm = 4;
    l.me[0] = Aa; l.ms[0] = D2;
    l.me[1] = X;  l.ms[1] = D2 * ld4;
    l.me[2] = D;  l.ms[2] = ld4;
    l.me[3] = D;  l.ms[3] = 1;
    l.nn = 2;
    l.ne[0] = D; l.ns[0] = D * ld4;
    l.ne[1] = D; l.ns[1] = D;
    TcOut out;
    out.add(TcKind::kBf16Hi, t3h, l).add(TcKind::kBf16Lo, t3l, l);
    one_layer_steps(c, ak, D, d, Aa, X, xh, xl, ldk, out, false, nullptr,
                    "edge renormalization, bra step", "edge renormalization, ket step");
  } else {
  // G1 -> X[(x,a)][(l,L,u,U)]; rows (a,l,L) from E, columns (x,u,U) from
  // P1: consecutive columns are consecutive (u,U), stored 4 at a time (as in
  // quarter_mixed's GEMM 1).  X's rows run over a fastest, so that the
  // double-layer step below (its rows are X's rows) writes the rows of one
  // tile to adjacent runs of T (a before x there as well)
  const int64_t K2 = D2 * D2, ldx = tc_ld(K2);
  bf16* xh = c.alloc<bf16>(size_t(Aa) * X * ldx);
  bf16* xl = c.alloc<bf16>(size_t(Aa) * X * ldx);
  {
    TcLayout l;
    l.nm = 3;
    l.me[0] = Aa; l.ms[0] = ldx;
    l.me[1] = D;  l.ms[1] = D * D2;
    l.me[2] = D;  l.ms[2] = D2;
    l.nn = 2;
    l.ne[0] = X;  l.ns[0] = Aa * ldx;
    l.ne[1] = D2; l.ns[1] = 1;
    TcOut out;
    out.add(TcKind::kBf16Hi, xh, l).add(TcKind::kBf16Lo, xl, l);
    out.name = "edge renormalization, projector step";
    tc_gemm(c, TcOperand{a1h, a1l, Aa * D2, B, ld1}, TcOperand{b1h, b1l, X * D2, B, ld1}, x3, out);
  }
  // G2 -> T[(x,r,R)][(a,d,D)]
  const DLOp dl = double_layer(c, ak, D, d);
  {
    TcLayout l;  // rows (x,a) from X, columns (r,R,d,D) from DL (as in quarter_mixed)
    l.nm = 2;
    l.me[0] = X;  l.ms[0] = D2 * ld4;
    l.me[1] = Aa; l.ms[1] = D2;
    l.nn = 4;
    l.ne[0] = D; l.ns[0] = D * ld4;
    l.ne[1] = D; l.ns[1] = ld4;
    l.ne[2] = D; l.ns[2] = D;
    l.ne[3] = D; l.ns[3] = 1;
    TcOut out;
    out.add(TcKind::kBf16Hi, t3h, l).add(TcKind::kBf16Lo, t3l, l);
    out.extra_tag = kTagTcDoubleLayer;
    out.name = "edge renormalization, double-layer step";
    // the reference's two one-layer site-tensor steps (directional_mover.py:363-364)
    out.algo_flops = 4.0 * double(Aa) * X * D2 * D2 * D2 * d;
    tc_gemm(c, TcOperand{xh, xl, Aa * X, K2, ldx}, dl.op(), x3, out);
  }
  }
  // G3: B4[y][(a,d,D)] = P2[a][d][D][y]
  bf16* b4h = c.alloc<bf16>(size_t(Y) * ld4);
  bf16* b4l = c.alloc<bf16>(size_t(Y) * ld4);
  {
    Gather g;
    g.nr = 1;
    g.re[0] = Y; g.rs[0] = 1;
    g.nk = 1;
    g.ke[0] = K4; g.ks[0] = Y;
    gather_split_bf16(c, P2i, g, b4h, b4l, ld4);
  }
  {
    TcLayout l;  // E'[y][x][r][R]
    l.nm = 3;
    l.me[0] = X; l.ms[0] = D2;
    l.me[1] = D; l.ms[1] = D;
    l.me[2] = D; l.ms[2] = 1;
    l.nn = 1;
    l.ne[0] = Y; l.ns[0] = X * D2;
    TcOut out;
    out.add(TcKind::kF64, Eout, l);
    out.name = "edge renormalization, last projector step";
    tc_gemm(c, TcOperand{t3h, t3l, X * D2, K4, ld4}, TcOperand{b4h, b4l, Y, K4, ld4}, x3, out);
  }
  double* nrm = c.alloc<double>(1);
  sumsq(c, Eout, Y * X * D2, nrm);
  divide_by(c, Eout, Y * X * D2, nrm, 1);
}

namespace {

// Double-layer matrix of one half of a bond RDM with the physical legs and
// the two legs leaving the half open (the site tensor A = S.A(k), legs
// l=0, u=1, r=2, d=3, p=4; ket lowercase, bra uppercase):
//   DLo[(Bo,Bp,Ko,Kp,Kd,Bd)][(K1,B1,K2,B2)] = A[ket] A[bra]
// where legs g1, g2 are contracted with the half's boundary operand X and
// leg o (toward the other site) and d stay open.  No sum: every entry is
// one product.
__global__ void double_layer_open_kernel(const double* A, int64_t s0, int64_t s1, int64_t s2,
                                         int64_t s3, int64_t s4, int D, int d, int g1, int g2,
                                         int o, bf16* hi, bf16* lo, int64_t ld) {
  // 32-bit index decoding (D^8 d^2 < 2^31, checked on the host)
  const uint32_t uD = uint32_t(D), ud = uint32_t(d);
  const uint32_t D4 = uD * uD * uD * uD, N = D4 * ud * ud;
  const int64_t st[5] = {s0, s1, s2, s3, s4};
  for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < N * D4;
       idx += gridDim.x * blockDim.x) {
    const uint32_t row = idx / D4, k = idx - row * D4;
    const int B2 = int(k % uD), K2 = int((k / uD) % uD), B1 = int((k / (uD * uD)) % uD),
              K1 = int(k / (uD * uD * uD));
    uint32_t n = row;
    const int Bd = int(n % uD);
    n /= uD;
    const int Kd = int(n % uD);
    n /= uD;
    const int Kp = int(n % ud);
    n /= ud;
    const int Ko = int(n % uD);
    n /= uD;
    const int Bp = int(n % ud);
    const int Bo = int(n / ud);
    const int64_t ket = K1 * st[g1] + K2 * st[g2] + Ko * st[o] + Kd * st[3] + Kp * st[4];
    const int64_t bra = B1 * st[g1] + B2 * st[g2] + Bo * st[o] + Bd * st[3] + Bp * st[4];
    // one product: FP32 (~1e-7) is far inside the hi/lo pair's 16 bits
    const float v = float(A[ket]) * float(A[bra]);
    const bf16 h = __float2bfloat16(v);
    hi[int64_t(row) * ld + k] = h;
    lo[int64_t(row) * ld + k] = __float2bfloat16(v - __bfloat162float(h));
  }
}

// One half of build_bond_rdm_core (acetn/measurement/rdm.py:102-120) on
// tensor cores, r[f][(x,Bo,Bp,Ko,Kp)] in FP64:
//   X = the boundary operand of the quarter of direction kq
//       (rows (c,e), K = the contracted leg pairs g1, g2),
//   Y = X DLo^T                                       (K = D^4, 3xBF16),
//   r = Rb Y, contracted over (t, Kd, Bd)              (K = chi D^2, 3xBF16),
// where t is c (contract_first) or e, x the other one, and Rb the corner
// times edge that closes the half (Rb[t][f][d][D], FP32).
void bond_rdm_half(Ctx& c, const Site& S, int kq, const View& ak, int g1, int g2, int o,
                   const float* rb, int64_t F, bool contract_first, double* r) {
  const int64_t D = S.D, d = S.d, D2 = D * D, D4 = D2 * D2;
  const TcMode x3 = TcMode::kBf16x3;
  Scope scope(c);
  const XOp x = x_operand(c, S, kq, "bond RDM, edge step");
  const int64_t T = contract_first ? x.cc : x.e, Xn = contract_first ? x.e : x.cc;
  const int64_t N = D4 * d * d, ldo = tc_ld(D4);
  bf16* oh = c.alloc<bf16>(size_t(N) * ldo);
  bf16* ol = c.alloc<bf16>(size_t(N) * ldo);
  if (!c.sizing()) {
    CTM_REQUIRE(N * D4 < (int64_t(1) << 31), CTM_ERR_UNSUPPORTED,
                "open double layer: D^8 d^2 must be below 2^31");
    KernelTimer kt(c.stream, "double_layer_open_kernel", kUnitByte, 4.0 * double(N) * D4);
    double_layer_open_kernel<<<grid_for(N * D4, 256), 256, 0, c.stream>>>(
        ak.p, ak.stride[0], ak.stride[1], ak.stride[2], ak.stride[3], ak.stride[4], int(D),
        int(d), g1, g2, o, oh, ol, ldo);
    CTM_LAUNCH_CHECK();
  }
  // Y stored K-major for the closing GEMM: rows (x,Bo,Bp,Ko,Kp), K (t,Kd,Bd)
  const int64_t K3 = T * D2, ld3 = tc_ld(K3), rows3 = Xn * D2 * d * d;
  bf16* yh = c.alloc<bf16>(size_t(rows3) * ld3);
  bf16* yl = c.alloc<bf16>(size_t(rows3) * ld3);
  {
    TcLayout l;
    const int64_t xs = D * d * D * d * ld3;  // stride of x in Y's rows
    l.nm = 2;
    l.me[0] = x.cc; l.ms[0] = contract_first ? D2 : xs;
    l.me[1] = x.e;  l.ms[1] = contract_first ? xs : D2;
    l.nn = 6;
    l.ne[0] = D; l.ns[0] = d * D * d * ld3;  // Bo
    l.ne[1] = d; l.ns[1] = D * d * ld3;      // Bp
    l.ne[2] = D; l.ns[2] = d * ld3;          // Ko
    l.ne[3] = d; l.ns[3] = ld3;              // Kp
    l.ne[4] = D; l.ns[4] = D;                // Kd
    l.ne[5] = D; l.ns[5] = 1;                // Bd
    TcOut out;
    out.add(TcKind::kBf16Hi, yh, l).add(TcKind::kBf16Lo, yl, l);
    out.name = "bond RDM, double-layer step";
    // the reference's two one-layer site-tensor steps (rdm.py:106-107)
    out.algo_flops = 2.0 * double(x.cc) * x.e * D4 * D2 * d * (1 + d);
    tc_gemm(c, TcOperand{x.hi, x.lo, x.rows, D4, x.ld}, TcOperand{oh, ol, N, D4, ldo}, x3, out);
  }
  // Rb as the A operand: [f][(t,d,D)] from rb[t][f][d][D]
  bf16* bh = c.alloc<bf16>(size_t(F) * ld3);
  bf16* bl = c.alloc<bf16>(size_t(F) * ld3);
  {
    Gather g;
    g.nr = 1;
    g.re[0] = F; g.rs[0] = D2;
    g.nk = 2;
    g.ke[0] = T;  g.ks[0] = F * D2;
    g.ke[1] = D2; g.ks[1] = 1;
    gather_split_bf16(c, rb, g, bh, bl, ld3);
  }
  TcOut out;
  out.add(TcKind::kF64, r, TcLayout::rows(F, rows3, rows3));
  out.name = "bond RDM, closing step";
  tc_gemm(c, TcOperand{bh, bl, F, K3, ld3}, TcOperand{yh, yl, rows3, K3, ld3}, x3, out);
}

ViewF f32_view(Ctx& c, const View& v) {
  CTM_REQUIRE(v.contiguous(), CTM_ERR_INVALID, "f32_view: expects a contiguous view");
  float* p = c.alloc<float>(size_t(v.numel()));
  to_f32(c, v.p, p, v.numel());
  ViewF out;
  out.p = p;
  out.nd = v.nd;
  for (int i = 0; i < v.nd; ++i) out.shape[i] = v.shape[i], out.stride[i] = v.stride[i];
  return out;
}

}  // namespace

// RDM.build_bond_rdm (acetn/measurement/rdm.py:69-99) with the contraction
// of build_bond_rdm_core (rdm.py:102-120) on tensor cores.  Right half: the
// boundary operand of site s1's quarter of direction k+1 (C12 E12 E11; its K
// legs are u and r of A(k)), the open double layer of A(k) with leg l toward
// s2, closed by C13 E13 over (c, d, D).  Left half: site s2's quarter
// operand of direction k (C21 E21 E24; K legs l and u), leg r open, closed
// by C24 E23 over (e, d, D).  Both halves come out in FP64 and the last
// contraction over (f, c, bond legs) is an FP64 GETT.
void bond_rdm_mixed(Ctx& c, const Site& S1, const Site& S2, int k, double* out) {
  const int64_t D = S1.D, d = S1.d;
  Scope scope(c);
  const View c13 = S1.C(k + 2), e13 = S1.E(k + 2), c24 = S2.C(k + 3), e23 = S2.E(k + 2);
  // closing tensors (FP32): r1a[a][f][d][D] = C13 E13, r2a[e][f][d][D] = C24^T E23
  const int64_t fa = c13.shape[0], ff = e13.shape[1];
  float* r1a = c.alloc<float>(size_t(fa) * ff * D * D);
  const int64_t ea = c24.shape[1], ef = e23.shape[0];
  float* r2a = c.alloc<float>(size_t(ea) * ef * D * D);
  {
    Scope s2(c);
    einsum(c, "ab,bfdD->afdD", f32_view(c, c13), f32_view(c, e13), ViewF(r1a, {fa, ff, D, D}));
    einsum(c, "ae,fadD->efdD", f32_view(c, c24), f32_view(c, e23), ViewF(r2a, {ea, ef, D, D}));
  }
  int64_t sh1[6], sh2[6], rr, cq;
  quarter_dims(S1, k + 1, rr, cq, sh1);
  quarter_dims(S2, k, rr, cq, sh2);
  CTM_REQUIRE(sh1[0] == fa && sh2[3] == ea, CTM_ERR_INVALID,
              "bond RDM: closing corner and edge do not chain with the halves");
  const int64_t e1 = sh1[3], c2 = sh2[0];  // the legs that stay open in each half
  double* r1 = c.alloc<double>(size_t(ff) * e1 * D * d * D * d);
  double* r2 = c.alloc<double>(size_t(ef) * c2 * D * d * D * d);
  const View a1 = S1.A(k), a2 = S2.A(k);
  bond_rdm_half(c, S1, k + 1, a1, 1, 2, 0, r1a, ff, true, r1);
  bond_rdm_half(c, S2, k, a2, 0, 1, 2, r2a, ef, false, r2);
  einsum(c, "fcRPrp,fcRQrq->PQpq", View(r1, {ff, e1, D, d, D, d}), View(r2, {ef, c2, D, d, D, d}),
         View(out, {d, d, d, d}));
}

int set_contraction_form(int form) {
  CTM_REQUIRE(form >= 0 && form <= 2, CTM_ERR_INVALID, "contraction form must be 0, 1 or 2");
  const int old = g_contraction_form;
  g_contraction_form = form;
  return old;
}

void quarter_tensor_mixed_f64(Ctx& c, const Site& S, int k, double* Q) {
  Scope scope(c);
  const QOps o = quarter_mixed(c, S, k);
  join_bf16(c, o.q_hi, o.q_lo, o.rows, o.cols, o.ld, Q);
  divide_by(c, Q, o.rows * o.cols, o.scale, 0);
}

namespace {

// SVD of the Rayleigh-Ritz matrix B (q x n, given as B^T in FP32) and
// U = Q Ub with Q the final basis Y (m x q, FP32): Ud (m x q), s, Vd (n x q)
// in FP64; with Ud null, Ub itself (q x q FP64) goes to Ub_out instead.
// FP32: Cholesky-QR of B^T and one-sided Jacobi on its triangular factor;
// fp64_svd: B in FP64 and the FP64 one-sided Jacobi.
void rayleigh_ritz_svd(Ctx& c, const float* Bt, const float* Y, int64_t m, int64_t n, int64_t q,
                       bool fp64_svd, double* Ud, double* s, double* Vd,
                       double* Ub_out = nullptr) {
  Scope scope(c);
  double* Ub = Ud != nullptr ? c.alloc<double>(size_t(q) * q) : Ub_out;
  if (fp64_svd) {
    double* btd = c.alloc<double>(size_t(n) * q);
    double* Bd = c.alloc<double>(size_t(q) * n);
    to_f64(c, Bt, btd, n * q);
    copy2d(c, View(btd, {n, q}).permute({1, 0}), Bd, n);
    svd_thin(c, Bd, q, n, Ub, s, Vd);
    if (Ud == nullptr) return;
    double* Yd = c.alloc<double>(size_t(m) * q);
    to_f64(c, Y, Yd, m * q);
    einsum(c, "ik,kj->ij", View(Yd, {m, q}), View(Ub, {q, q}), View(Ud, {m, q}));
    return;
  }
  float* V = c.alloc<float>(size_t(n) * q);
  svd_via_qr(c, Bt, q, n, Ub, s, V);
  to_f64(c, V, Vd, n * q);
  if (Ud == nullptr) return;
  float* U = c.alloc<float>(size_t(m) * q);
  float* ubf = c.alloc<float>(size_t(q) * q);
  to_f32(c, Ub, ubf, q * q);
  einsum(c, "ik,kj->ij", ViewF(Y, {m, q}), ViewF(ubf, {q, q}), ViewF(U, {m, q}));
  to_f64(c, U, Ud, m * q);
}

// The projectors' final form: fixed width (cap columns, zero past the
// truncation count) or compact (chi_new columns).
void store_projectors(Ctx& c, const ctm_ctmrg_opts& o, const double* P1f, int64_t rows1,
                      const double* P2f, int64_t rows2, int64_t cap, const int64_t* chi_new,
                      double* P1, double* P2) {
  if (o.fixed_width) {
    if (!c.sizing()) {
      CTM_CUDA(cudaMemcpyAsync(P1, P1f, sizeof(double) * rows1 * cap, cudaMemcpyDeviceToDevice,
                               c.stream));
      CTM_CUDA(cudaMemcpyAsync(P2, P2f, sizeof(double) * rows2 * cap, cudaMemcpyDeviceToDevice,
                               c.stream));
    }
  } else {
    scale_columns_compact(c, P1f, rows1, cap, nullptr, chi_new, P1);
    scale_columns_compact(c, P2f, rows2, cap, nullptr, chi_new, P2);
  }
}

// ProjectorCalculator.calculate_full_system with the randomized SVD
// (acetn/renormalization/projectors.py:196-217; the chain of
// acetn/linalg/fused_3matmul_svd_lowrank.py:26-52) in the arithmetic of the
// mixed half-system form: F = Q2 Q1 Q4 Q3 is never formed; every product of
// the chain runs on tensor cores against the four quarter tensors (3xBF16
// range finder, Rayleigh-Ritz and projector products), each step
// divided by its quarter tensor's max |entry| (the reference's normalised
// quarters; the intermediates stay O(1)); FP32 orthonormalization after
// every half step (the reference's four-factor variant also
// orthonormalises Z); SVD as in the half-system form; FP64 truncation;
// proj1 = Q1^T (Q2^T U), proj2 = Q4 (Q3 V).
void projectors_mixed_full_system(Ctx& c, const Site* S[4], int k, const ctm_ctmrg_opts& o,
                                  const double* omega, double* P1, double* P2,
                                  int64_t* chi_new) {
  Scope scope(c);
  // chain order: F0 = Q2 (site 1, k+1), F1 = Q1 (site 0, k), F2 = Q4
  // (site 3, k+3), F3 = Q3 (site 2, k+2)
  const int site_of[4] = {1, 0, 3, 2};
  const int dir_of[4] = {k + 1, k, k + 3, k + 2};
  int64_t sh[6], rows[4], cols[4];
  for (int i = 0; i < 4; ++i) quarter_dims(*S[site_of[i]], dir_of[i], rows[i], cols[i], sh);
  CTM_REQUIRE(cols[0] == rows[1] && cols[1] == rows[2] && cols[2] == rows[3], CTM_ERR_INVALID,
              "full-system: quarter tensors do not chain");
  const int64_t m = rows[0], n = cols[3];
  const int64_t q = std::min({o.chi + o.rsvd_oversampling, m, n});
  const int64_t cap = std::min(o.chi, q);
  const TcMode x3 = TcMode::kBf16x3;
  // the range finder is always 3xBF16 here: the spectrum of the four-factor
  // product spans the square of the half system's range, and one BF16 pass
  // per chain step left 5e-4 - 1.3e-3 of the largest bond energy between
  // the mixed and the FP64 move at D=4, chi=32 / 64 (3xBF16: 3e-5 / 7e-5,
  // the FP64 algorithm's own draw-to-draw spread 1.5e-5 / 4.4e-5)
  const bool rf3 = true;
  const bool svd64 = (o.mixed_flags & CTM_MIXED_SVD64) != 0;
  const bool q64 = (o.mixed_flags & CTM_MIXED_Q64) != 0;
  CTM_REQUIRE((o.mixed_flags & CTM_MIXED_F32) == 0, CTM_ERR_UNSUPPORTED,
              "the FP32 reference form covers half-system projectors only");
  const TcMode xr = rf3 ? x3 : TcMode::kBf16x1;
  const int inner_stages = rf3 ? 3 : 2;
  float* Y = c.alloc<float>(size_t(m) * q);
  float* Bt = c.alloc<float>(size_t(n) * q);
  QOps F[4];
  {
    KernelTimer span(c.stream, kTagQuarter, 0.0);
    for (int i = 0; i < 4; ++i) F[i] = quarter_mixed(c, *S[site_of[i]], dir_of[i], q64);
  }
  // out (m x q, FP32) = F0 F1 F2 F3 x, from x^T (q x n)
  auto forward = [&](const TcOperand& xt, TcMode mode, bool lo, float* out, const char* name) {
    Scope s1(c);
    TcOperand t = xt;
    for (int i = 3; i >= 1; --i) t = gemm_to_operand(c, F[i].q(lo), t, mode, lo, name, F[i].scale);
    TcOut to;
    to.add(TcKind::kF32, out, TcLayout::rows(m, q, q));
    to.inv_scale = F[0].scale;
    to.name = name;
    tc_gemm(c, F[0].q(lo), t, mode, to);
  };
  // out (n x q, FP32) = F3^T F2^T F1^T F0^T y, from y^T (q x m)
  auto backward = [&](const TcOperand& yt, TcMode mode, bool lo, float* out, const char* name) {
    Scope s1(c);
    TcOperand t = yt;
    for (int i = 0; i <= 2; ++i) t = gemm_to_operand(c, F[i].t(lo), t, mode, lo, name, F[i].scale);
    TcOut to;
    to.add(TcKind::kF32, out, TcLayout::rows(n, q, q));
    to.inv_scale = F[3].scale;
    to.name = name;
    tc_gemm(c, F[3].t(lo), t, mode, to);
  };
  KernelTimer* rf_span = new KernelTimer(c.stream, kTagRangeFinder, 0.0);
  {
    Scope s2(c);
    forward(yt_operand(c, omega, n, q, q, rf3), xr, rf3, Y, "range finder");
  }
  for (int it = 0; it < o.rsvd_niter; ++it) {
    {
      KernelTimer span(c.stream, kTagOrtho, 0.0);
      orthonormalize(c, Y, m, q, nullptr, inner_stages);
    }
    Scope s2(c);
    float* Z = c.alloc<float>(size_t(n) * q);
    {
      Scope s3(c);
      backward(yt_operand_f32(c, Y, m, q, q, rf3), xr, rf3, Z, "range finder");
    }
    {
      KernelTimer span(c.stream, kTagOrtho, 0.0);
      orthonormalize(c, Z, n, q, nullptr, inner_stages);
    }
    forward(yt_operand_f32(c, Z, n, q, q, rf3), xr, rf3, Y, "range finder");
  }
  {
    KernelTimer span(c.stream, kTagOrtho, 0.0);
    orthonormalize(c, Y, m, q, nullptr);
  }
  delete rf_span;
  double* s = c.alloc<double>(q);
  double* Ud = c.alloc<double>(size_t(m) * q);
  double* Vd = c.alloc<double>(size_t(n) * q);
  {
    KernelTimer span(c.stream, kTagSvd, 0.0);
    {
      Scope s2(c);
      backward(yt_operand_f32(c, Y, m, q, q, true), x3, true, Bt, "Rayleigh-Ritz");
    }
    rayleigh_ritz_svd(c, Bt, Y, m, n, q, svd64, Ud, s, Vd);
  }
  KernelTimer proj_span(c.stream, kTagProject, 0.0);
  double* f = c.alloc<double>(cap);
  truncation_factors(c, s, q, o.chi, std::max({o.svd_cutoff, o.mixed_floor, 1e-8}), f, cap,
                     chi_new);
  const int64_t rows1 = cols[1], rows2 = rows[2];
  double* P1f = c.alloc<double>(size_t(rows1) * cap);
  double* P2f = c.alloc<double>(size_t(rows2) * cap);
  {
    Scope s2(c);
    scale_columns(c, Ud, m, cap, q, f);
    scale_columns(c, Vd, n, cap, q, f);
    // proj1 = Q1^T (Q2^T U f)
    const TcOperand ut = yt_operand(c, Ud, m, cap, q, true);                       // cap x m
    const TcOperand u2 = gemm_to_operand(c, F[0].t(true), ut, x3, true, "projector", F[0].scale);
    gemm_to_f64(c, F[1].t(true), u2, x3, P1f, cap, false, F[1].scale, "projector");
    // proj2 = Q4 (Q3 V f)
    const TcOperand vt = yt_operand(c, Vd, n, cap, q, true);                       // cap x n
    const TcOperand v3 = gemm_to_operand(c, F[3].q(true), vt, x3, true, "projector", F[3].scale);
    gemm_to_f64(c, F[2].q(true), v3, x3, P2f, cap, false, F[2].scale, "projector");
  }
  store_projectors(c, o, P1f, rows1, P2f, rows2, cap, chi_new, P1, P2);
}

}  // namespace

void calculate_projectors_mixed(Ctx& c, const Site* S[4], int k, const ctm_ctmrg_opts& o,
                                const double* omega, double* P1, double* P2, int64_t* chi_new) {
  CTM_REQUIRE(o.svd_type == CTM_SVD_RSVD, CTM_ERR_INVALID,
              "calculate_projectors_mixed: randomized SVD only (full-rank runs in "
              "calculate_projectors)");
  if (o.projectors == CTM_PROJ_FULL) {
    projectors_mixed_full_system(c, S, k, o, omega, P1, P2, chi_new);
    return;
  }
  CTM_REQUIRE(o.projectors == CTM_PROJ_HALF, CTM_ERR_INVALID, "Invalid ctmrg projector type");
  Scope scope(c);
  int64_t sh1[6], sh4[6], r1, c1, r4, c4;
  quarter_dims(*S[0], k, r1, c1, sh1);
  quarter_dims(*S[3], k + 3, r4, c4, sh4);
  CTM_REQUIRE(c1 == r4, CTM_ERR_INVALID, "half-system: quarter tensors do not chain");
  const int64_t m = r1, n = c4;
  const int64_t q = std::min({o.chi + o.rsvd_oversampling, m, n});
  const int64_t cap = std::min(o.chi, q);
  const TcMode x3 = TcMode::kBf16x3;
  const bool rf3 = (o.mixed_flags & CTM_MIXED_RF3) != 0;
  const bool svd64 = (o.mixed_flags & CTM_MIXED_SVD64) != 0;
  const bool q64 = (o.mixed_flags & CTM_MIXED_Q64) != 0;
  const bool f32 = (o.mixed_flags & CTM_MIXED_F32) != 0;
  // range-finder products: one BF16 pass, or 3xBF16 with FP32 bases
  // orthonormal to working precision
  const TcMode xr = rf3 ? x3 : TcMode::kBf16x1;
  const int inner_stages = rf3 ? 3 : 2;
  float* Y = c.alloc<float>(size_t(m) * q);
  float* Bt = c.alloc<float>(size_t(n) * q);
  float *Q1f = nullptr, *Q4f = nullptr;
  if (f32) {
    // every product on FP32 copies of FP64 quarter tensors (SIMT FP32 FMAs):
    // a precision reference for the tensor-core forms
    Q1f = c.alloc<float>(size_t(m) * c1);
    Q4f = c.alloc<float>(size_t(r4) * n);
    {
      Scope s0(c);
      double* Qd = c.alloc<double>(size_t(std::max(m * c1, r4 * n)));
      int64_t qs[6];
      quarter_tensor(c, *S[0], k, Qd, qs);
      to_f32(c, Qd, Q1f, m * c1);
      quarter_tensor(c, *S[3], k + 3, Qd, qs);
      to_f32(c, Qd, Q4f, r4 * n);
    }
    Scope s0(c);
    float* T = c.alloc<float>(size_t(std::max(c1, n)) * q);
    float* Z = c.alloc<float>(size_t(n) * q);
    float* omf = c.alloc<float>(size_t(n) * q);
    to_f32(c, omega, omf, n * q);
    einsum(c, "ik,kj->ij", ViewF(Q4f, {r4, n}), ViewF(omf, {n, q}), ViewF(T, {r4, q}));
    einsum(c, "ik,kj->ij", ViewF(Q1f, {m, c1}), ViewF(T, {c1, q}), ViewF(Y, {m, q}));
    for (int it = 0; it < o.rsvd_niter; ++it) {
      orthonormalize(c, Y, m, q, nullptr, 3);
      einsum(c, "ki,kj->ij", ViewF(Q1f, {m, c1}), ViewF(Y, {m, q}), ViewF(T, {c1, q}));
      einsum(c, "ki,kj->ij", ViewF(Q4f, {r4, n}), ViewF(T, {r4, q}), ViewF(Z, {n, q}));
      orthonormalize(c, Z, n, q, nullptr, 3);
      einsum(c, "ik,kj->ij", ViewF(Q4f, {r4, n}), ViewF(Z, {n, q}), ViewF(T, {r4, q}));
      einsum(c, "ik,kj->ij", ViewF(Q1f, {m, c1}), ViewF(T, {c1, q}), ViewF(Y, {m, q}));
    }
    orthonormalize(c, Y, m, q, nullptr, 3);
    einsum(c, "ki,kj->ij", ViewF(Q1f, {m, c1}), ViewF(Y, {m, q}), ViewF(T, {c1, q}));
    einsum(c, "ki,kj->ij", ViewF(Q4f, {r4, n}), ViewF(T, {r4, q}), ViewF(Bt, {n, q}));
  }
  // ---- quarter tensors as BF16 operands (tensor cores, 3xBF16)
  QOps A1, A4;
  if (!f32) {
    KernelTimer span(c.stream, kTagQuarter, 0.0);
    A1 = quarter_mixed(c, *S[0], k, q64);
    A4 = quarter_mixed(c, *S[3], k + 3, q64);
  }
  // ---- range finder in BF16 with FP32 orthonormalization (on the unscaled
  //      quarter tensors: every product is orthonormalised before use):
  //      Y = Q1 (Q4 Omega), niter x [QR; Z = Q4^T Q1^T Y; QR; Y = Q1 Q4 Z].
  //      The reference orthonormalises once per power iteration; the extra
  //      QR of the half step spans the same space in exact arithmetic and
  //      keeps the matrices that FP32 has to orthonormalise at the condition
  //      number of Q1 Q4 instead of its square.
  KernelTimer* rf_span = new KernelTimer(c.stream, kTagRangeFinder, 0.0);
  if (!f32) {
    Scope s2(c);
    const TcOperand om = yt_operand(c, omega, n, q, q, rf3);           // Omega^T (q x n)
    const TcOperand t = gemm_to_operand(c, A4.q(rf3), om, xr, rf3, "range finder");  // (Q4 Om)^T
    TcOut out;
    out.add(TcKind::kF32, Y, TcLayout::rows(m, q, q));
    out.name = "range finder";
    tc_gemm(c, A1.q(rf3), t, xr, out);
  }
  // The bases inside the power iteration are only multiplied again in BF16
  // (~4e-3 relative): two Cholesky-QR stages (orthonormal to ~1e-3) suffice
  // there; the final Q, which forms B in 3xBF16, gets three.
  for (int it = 0; it < (f32 ? 0 : o.rsvd_niter); ++it) {
    {
      KernelTimer span(c.stream, kTagOrtho, 0.0);
      orthonormalize(c, Y, m, q, nullptr, inner_stages);
    }
    Scope s2(c);
    float* Z = c.alloc<float>(size_t(n) * q);
    {
      Scope s3(c);
      const TcOperand yt = yt_operand_f32(c, Y, m, q, q, rf3);
      const TcOperand z1 = gemm_to_operand(c, A1.t(rf3), yt, xr, rf3, "range finder");  // (Q1^T Y)^T
      TcOut out;
      out.add(TcKind::kF32, Z, TcLayout::rows(n, q, q));
      out.name = "range finder";
      tc_gemm(c, A4.t(rf3), z1, xr, out);                                 // Z = Q4^T Q1^T Y
    }
    {
      KernelTimer span(c.stream, kTagOrtho, 0.0);
      orthonormalize(c, Z, n, q, nullptr, inner_stages);
    }
    const TcOperand zt = yt_operand_f32(c, Z, n, q, q, rf3);
    const TcOperand z3 = gemm_to_operand(c, A4.q(rf3), zt, xr, rf3, "range finder");  // (Q4 Z)^T
    TcOut out;
    out.add(TcKind::kF32, Y, TcLayout::rows(m, q, q));
    out.name = "range finder";
    tc_gemm(c, A1.q(rf3), z3, xr, out);
  }
  if (!f32) {
    KernelTimer span(c.stream, kTagOrtho, 0.0);
    orthonormalize(c, Y, m, q, nullptr);
  }
  delete rf_span;
  // ---- Rayleigh-Ritz: B = (Q^T Q1) Q4 in 3xBF16 (written as B^T in FP32),
  //      its SVD from an FP32 QR of B^T and one-sided Jacobi.  The product
  //      Q1^T Q is kept (c1 x q, K-major over q): the projector Q1^T U f with
  //      U = Q Ub is then (Q1^T Q) (Ub f), a K = q product instead of K = m.
  double* s = c.alloc<double>(q);
  double* Ud = f32 ? c.alloc<double>(size_t(m) * q) : nullptr;
  double* Ub = f32 ? nullptr : c.alloc<double>(size_t(q) * q);
  double* Vd = c.alloc<double>(size_t(n) * q);
  const int64_t ldwt = tc_ld(q);
  bf16* wt_hi = f32 ? nullptr : c.alloc<bf16>(size_t(c1) * ldwt);
  bf16* wt_lo = f32 ? nullptr : c.alloc<bf16>(size_t(c1) * ldwt);
  KernelTimer* svd_span = new KernelTimer(c.stream, kTagSvd, 0.0);
  if (!f32) {
    Scope s2(c);
    const TcOperand qt = yt_operand_f32(c, Y, m, q, q, true);           // Q^T (q x m)
    // Q1^T Q (c1 x q): as W = Q^T Q1 (q rows, K = c1) for B and as its
    // transpose (c1 rows, K = q) for the projector
    const int64_t ldw = tc_ld(c1);
    bf16* w_hi = c.alloc<bf16>(size_t(q) * ldw);
    bf16* w_lo = c.alloc<bf16>(size_t(q) * ldw);
    {
      TcOut ow;
      ow.add(TcKind::kBf16Hi, w_hi, TcLayout::cols(c1, q, ldw));
      ow.add(TcKind::kBf16Lo, w_lo, TcLayout::cols(c1, q, ldw));
      ow.add(TcKind::kBf16Hi, wt_hi, TcLayout::rows(c1, q, ldwt));
      ow.add(TcKind::kBf16Lo, wt_lo, TcLayout::rows(c1, q, ldwt));
      ow.name = "Rayleigh-Ritz";
      tc_gemm(c, A1.t(true), qt, x3, ow);
    }
    const TcOperand w{w_hi, w_lo, q, c1, ldw};
    TcOut out;
    out.add(TcKind::kF32, Bt, TcLayout::rows(A4.cols, q, q));            // B^T (n x q)
    out.inv_scale = A1.scale;  // normalised quarter tensors
    out.inv_scale2 = A4.scale;
    out.name = "Rayleigh-Ritz";
    tc_gemm(c, A4.t(true), w, x3, out);
  }
  rayleigh_ritz_svd(c, Bt, Y, m, n, q, svd64 || f32, Ud, s, Vd, Ub);
  delete svd_span;
  // ---- truncation (FP64 spectrum) and projector products (3xBF16)
  KernelTimer proj_span(c.stream, kTagProject, 0.0);
  double* f = c.alloc<double>(cap);
  // below ~1e-8 s_0 the spectrum is the noise of the 3xBF16 products: keeping
  // it would weight noise by s^-1/2 (and grows the environment without bound)
  truncation_factors(c, s, q, o.chi, std::max({o.svd_cutoff, o.mixed_floor, 1e-8}), f, cap,
                     chi_new);
  double* P1f = c.alloc<double>(size_t(c1) * cap);
  double* P2f = c.alloc<double>(size_t(r4) * cap);
  {
    Scope s2(c);
    if (f32) scale_columns(c, Ud, m, cap, q, f);
    else scale_columns(c, Ub, q, cap, q, f);
    scale_columns(c, Vd, n, cap, q, f);
    if (f32) {
      float* uf = c.alloc<float>(size_t(m) * q);
      float* vf = c.alloc<float>(size_t(n) * q);
      float* pf = c.alloc<float>(size_t(std::max(c1, r4)) * cap);
      to_f32(c, Ud, uf, m * q);
      to_f32(c, Vd, vf, n * q);
      ViewF uv(uf, {m, cap}), vv(vf, {n, cap});
      uv.stride[0] = q;
      vv.stride[0] = q;
      einsum(c, "ki,kz->iz", ViewF(Q1f, {m, c1}), uv, ViewF(pf, {c1, cap}));
      to_f64(c, pf, P1f, c1 * cap);
      einsum(c, "ik,kz->iz", ViewF(Q4f, {r4, n}), vv, ViewF(pf, {r4, cap}));
      to_f64(c, pf, P2f, r4 * cap);
    } else {
    const TcOperand ubt = yt_operand(c, Ub, q, cap, q, true);  // (Ub f)^T (cap x q)
    const TcOperand wt{wt_hi, wt_lo, c1, q, ldwt};               // Q1^T Q (c1 x q)
    gemm_to_f64(c, wt, ubt, x3, P1f, cap, false, A1.scale, "projector");  // Q1^T Q Ub f (c1 x cap)
    const TcOperand vt = yt_operand(c, Vd, n, cap, q, true);  // (V f)^T (cap x n)
    gemm_to_f64(c, A4.q(true), vt, x3, P2f, cap, false, A4.scale, "projector");  // Q4 V f (r4 x cap)
    }
  }
  store_projectors(c, o, P1f, c1, P2f, r4, cap, chi_new, P1, P2);
}

}  // namespace ctm
