// CTMRG operations of Ace-TN's renormalization and measurement path, built
// from the FP64 engine (gett.cu, linalg.cu) and the tensor-core engine
// (tc_gemm.cu), and the extern "C" entry points of include/ctm_gb300.h.
//
// Each function below follows one function of the reference; the einsum
// strings are the reference's own index expressions, evaluated by the
// strided GETT engine without permute copies.
#include "engine.cuh"
#include "tc_gemm.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <string>

namespace ctm {

namespace {

thread_local std::string g_last_error;

void check_site(const ctm_site_f64* s, int64_t D, int64_t d) {
  CTM_REQUIRE(s != nullptr && s->A != nullptr, CTM_ERR_INVALID, "site tensor A is NULL");
  CTM_REQUIRE(D >= 1 && d >= 1, CTM_ERR_INVALID, "bond and physical dimensions must be >= 1");
  for (int k = 0; k < 4; ++k) {
    CTM_REQUIRE(s->C[k] != nullptr && s->E[k] != nullptr, CTM_ERR_INVALID,
                "corner/edge tensor pointer is NULL");
    CTM_REQUIRE(s->c_rows[k] >= 1 && s->c_cols[k] >= 1 && s->e_rows[k] >= 1 && s->e_cols[k] >= 1,
                CTM_ERR_INVALID, "corner/edge tensor with an empty dimension");
  }
}

}  // namespace

// Quarter-tensor matrix dimensions of direction k: rows = (c, r, R), cols = (e, d, D).
void quarter_dims(const Site& S, int k, int64_t& rows, int64_t& cols, int64_t sh[6]) {
  const View ck = S.C(k), ek1 = S.E(3 + k), ek2 = S.E(k);
  CTM_REQUIRE(ck.shape[1] == ek2.shape[0], CTM_ERR_INVALID,
              "quarter tensor: C[k] columns do not match E[k] rows");
  CTM_REQUIRE(ck.shape[0] == ek1.shape[1], CTM_ERR_INVALID,
              "quarter tensor: C[k] rows do not match E[k+3] columns");
  sh[0] = ek2.shape[1];
  sh[1] = S.D;
  sh[2] = S.D;
  sh[3] = ek1.shape[0];
  sh[4] = S.D;
  sh[5] = S.D;
  rows = sh[0] * S.D * S.D;
  cols = sh[3] * S.D * S.D;
}


void set_last_error(const std::string& msg) { g_last_error = msg; }

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
const char* g_last_error_cstr() { return g_last_error.c_str(); }

// ------------------------------------------------------------------ quarter
// ProjectorCalculator.make_quarter_tensor (acetn/renormalization/projectors.py:35-60).
void quarter_tensor(Ctx& c, const Site& S, int k, double* Q, int64_t qshape[6]) {
  int64_t rows, cols;
  quarter_dims(S, k, rows, cols, qshape);
  const View ak = S.A(k), ck = S.C(k), ek1 = S.E(3 + k), ek2 = S.E(k);
  const int64_t a = ck.shape[0], cc = qshape[0], e = qshape[3], D = S.D, d = S.d;
  Scope scope(c);
  double* t1 = c.alloc<double>(size_t(a) * cc * D * D);
  double* t2 = c.alloc<double>(size_t(cc) * D * D * e * D * D);
  double* t3 = c.alloc<double>(size_t(cc) * D * e * D * D * D * d);
  double* mx = c.alloc<double>(1);
  einsum(c, "ab,bcuU->acuU", ck, ek2, View(t1, {a, cc, D, D}));
  einsum(c, "acuU,ealL->cuUelL", View(t1, {a, cc, D, D}), ek1, View(t2, {cc, D, D, e, D, D}));
  einsum(c, "cuUelL,LURDP->cuelRDP", View(t2, {cc, D, D, e, D, D}), ak,
         View(t3, {cc, D, e, D, D, D, d}));
  einsum(c, "lurdp,cuelRDp->crRedD", ak, View(t3, {cc, D, e, D, D, D, d}),
         View(Q, {cc, D, D, e, D, D}));
  absmax(c, Q, rows * cols, mx);
  divide_by(c, Q, rows * cols, mx, 0);
}

// ------------------------------------------------------------------ rSVD
// fused_matmul_svd_lowrank and friends (acetn/linalg/*.py) on a chain of
// factors F[0] @ F[1] @ ... (each rows x cols, row-major).
struct Factor {
  const double* p;
  int64_t rows, cols;
};

namespace {

View mat(const double* p, int64_t r, int64_t c) { return View(p, {r, c}); }

// C (M x N) = A (M x K) B (K x N), row-major FP64: the FP64 GETT, or (mixed)
// tcgen05 3xBF16 products of the split operands with FP32 accumulation.
void product(Ctx& c, const double* A, const double* B, double* C, int64_t M, int64_t N,
             int64_t K, int prec) {
  if (prec != CTM_PREC_MIXED) {
    einsum(c, "ik,kj->ij", mat(A, M, K), mat(B, K, N), mat(C, M, N));
    return;
  }
  const int64_t ld = tc_ld(K);
  Scope scope(c);
  bf16* ah = c.alloc<bf16>(size_t(M) * ld);
  bf16* al = c.alloc<bf16>(size_t(M) * ld);
  bf16* bh = c.alloc<bf16>(size_t(N) * ld);
  bf16* bl = c.alloc<bf16>(size_t(N) * ld);
  split_bf16(c, A, M, K, K, false, ah, al, ld);
  split_bf16(c, B, K, N, N, true, bh, bl, ld);
  TcOut out;
  out.add(TcKind::kF64, C, TcLayout::rows(M, N, N));
  out.name = "full-rank product";
  tc_gemm(c, TcOperand{ah, al, M, K, ld}, TcOperand{bh, bl, N, K, ld}, TcMode::kBf16x3, out);
}

// y (f.rows x q) = f @ x (f.cols x q)
void apply(Ctx& c, const Factor& f, const double* x, double* y, int64_t q, int prec) {
  (void)prec;
  einsum(c, "ik,kj->ij", mat(f.p, f.rows, f.cols), mat(x, f.cols, q), mat(y, f.rows, q));
}
// y (f.cols x q) = f^T @ x (f.rows x q)
void apply_t(Ctx& c, const Factor& f, const double* x, double* y, int64_t q, int prec) {
  (void)prec;
  einsum(c, "ki,kj->ij", mat(f.p, f.rows, f.cols), mat(x, f.rows, q), mat(y, f.cols, q));
}

}  // namespace

// Randomized SVD of prod(F).  U (m x q), S (q), V (n x q).
// Rayleigh-Ritz (B = Q^T prod(F)) in FP64 or 3xBF16, SVD in FP64.
void rsvd_chain(Ctx& c, const std::vector<Factor>& F, int64_t q, int niter, const double* omega,
                double* U, double* S, double* V, int prec) {
  const int nf = static_cast<int>(F.size());
  for (int i = 0; i + 1 < nf; ++i)
    CTM_REQUIRE(F[i].cols == F[i + 1].rows, CTM_ERR_INVALID, "rsvd: factor shapes do not chain");
  const int64_t m = F[0].rows, n = F[nf - 1].cols;
  CTM_REQUIRE(q >= 1 && q <= std::min(m, n), CTM_ERR_INVALID, "rsvd: q must satisfy 1 <= q <= min(m, n)");
  int64_t kmax = std::max(m, n);
  for (auto& f : F) kmax = std::max({kmax, f.rows, f.cols});
  Scope scope(c);
  double* Y = c.alloc<double>(size_t(m) * q);
  double* t0 = c.alloc<double>(size_t(kmax) * q);
  double* t1 = c.alloc<double>(size_t(kmax) * q);
  double* B = c.alloc<double>(size_t(q) * kmax);
  double* B2 = c.alloc<double>(size_t(q) * kmax);
  double* Ub = c.alloc<double>(size_t(q) * q);
  const int rr_prec = prec;  // Rayleigh-Ritz product precision
  // Y = F0 (F1 (... (F_{nf-1} omega)))
  auto forward = [&](const double* x, double* y) {
    const double* cur = x;
    double* bufs[2] = {t0, t1};
    int w = 0;
    for (int i = nf - 1; i >= 1; --i) {
      apply(c, F[i], cur, bufs[w], q, prec);
      cur = bufs[w];
      w ^= 1;
    }
    apply(c, F[0], cur, y, q, prec);
  };
  // y = F_{nf-1}^T (... (F0^T x))
  auto backward = [&](const double* x, double* y) {
    const double* cur = x;
    double* bufs[2] = {t0, t1};
    int w = 0;
    for (int i = 0; i < nf - 1; ++i) {
      apply_t(c, F[i], cur, bufs[w], q, prec);
      cur = bufs[w];
      w ^= 1;
    }
    apply_t(c, F[nf - 1], cur, y, q, prec);
  };
  double* Z = c.alloc<double>(size_t(n) * q);
  forward(omega, Y);
  for (int it = 0; it < niter; ++it) {
    orthonormalize(c, Y, m, q, nullptr);
    backward(Y, Z);
    // only the four-factor variant re-orthonormalises between the two halves
    // (acetn/linalg/fused_3matmul_svd_lowrank.py:43-48)
    if (nf == 4) orthonormalize(c, Z, n, q, nullptr);
    forward(Z, Y);
  }
  orthonormalize(c, Y, m, q, nullptr);
  // B = ((Q^T F0) F1) ... (q x n), left to right
  {
    int64_t cols = F[0].cols;
    (void)rr_prec;
    einsum(c, "kq,kj->qj", mat(Y, m, q), mat(F[0].p, F[0].rows, F[0].cols), mat(B, q, cols));
    double* cur = B;
    double* other = B2;
    for (int i = 1; i < nf; ++i) {
      einsum(c, "qk,kj->qj", mat(cur, q, F[i].rows), mat(F[i].p, F[i].rows, F[i].cols),
             mat(other, q, F[i].cols));
      std::swap(cur, other);
      cols = F[i].cols;
    }
    // thin SVD of B (q x n): Ub (q x q), S, V (n x q)
    svd_thin(c, cur, q, n, Ub, S, V);
  }
  // U = Q Ub
  einsum(c, "ik,kj->ij", mat(Y, m, q), mat(Ub, q, q), mat(U, m, q));
}

// ------------------------------------------------------------------ projectors
namespace {

void truncate_and_project(Ctx& c, double* U, double* V, int64_t m, int64_t n, int64_t ldu,
                          const double* s, int64_t r, const ctm_ctmrg_opts& o,
                          const Factor& left1, const Factor* left2, const Factor& right1,
                          const Factor* right2, double* P1, double* P2, int64_t* chi_new,
                          int prec) {
  // caps and scaling
  const int64_t cap = std::min<int64_t>(o.chi, r);
  Scope scope(c);
  double* f = c.alloc<double>(cap);
  truncation_factors(c, s, r, o.chi, o.svd_cutoff, f, cap, chi_new);
  scale_columns(c, U, m, cap, ldu, f);
  scale_columns(c, V, n, cap, ldu, f);
  // proj1 = left1^T (left2^T U) ; proj2 = right1 (right2 V)
  const int64_t p1rows = left1.cols, p2rows = right1.rows;
  double* P1f = c.alloc<double>(size_t(p1rows) * cap);
  double* P2f = c.alloc<double>(size_t(p2rows) * cap);
  View Uv(U, {m, cap});
  Uv.stride[0] = ldu;
  View Vv(V, {n, cap});
  Vv.stride[0] = ldu;
  if (left2 != nullptr) {
    double* tmp = c.alloc<double>(size_t(left2->cols) * cap);
    einsum(c, "ki,kz->iz", mat(left2->p, left2->rows, left2->cols), Uv, mat(tmp, left2->cols, cap));
    einsum(c, "ki,kz->iz", mat(left1.p, left1.rows, left1.cols), mat(tmp, left1.rows, cap),
           mat(P1f, p1rows, cap));
  } else {
    einsum(c, "ki,kz->iz", mat(left1.p, left1.rows, left1.cols), Uv, mat(P1f, p1rows, cap));
  }
  if (right2 != nullptr) {
    double* tmp = c.alloc<double>(size_t(right2->rows) * cap);
    einsum(c, "ik,kz->iz", mat(right2->p, right2->rows, right2->cols), Vv, mat(tmp, right2->rows, cap));
    einsum(c, "ik,kz->iz", mat(right1.p, right1.rows, right1.cols), mat(tmp, right1.cols, cap),
           mat(P2f, p2rows, cap));
  } else {
    einsum(c, "ik,kz->iz", mat(right1.p, right1.rows, right1.cols), Vv, mat(P2f, p2rows, cap));
  }
  if (o.fixed_width) {
    if (!c.sizing()) {
      CTM_CUDA(cudaMemcpyAsync(P1, P1f, sizeof(double) * p1rows * cap, cudaMemcpyDeviceToDevice,
                               c.stream));
      CTM_CUDA(cudaMemcpyAsync(P2, P2f, sizeof(double) * p2rows * cap, cudaMemcpyDeviceToDevice,
                               c.stream));
    }
  } else {
    scale_columns_compact(c, P1f, p1rows, cap, nullptr, chi_new, P1);
    scale_columns_compact(c, P2f, p2rows, cap, nullptr, chi_new, P2);
  }
}

}  // namespace

struct ProjDims {
  int64_t p1_rows, p2_rows, omega_rows, q, cap;
};

ProjDims projector_dims(const Site* S[4], int k, const ctm_ctmrg_opts& o) {
  ProjDims pd{};
  int64_t sh[6];
  int64_t r1, c1, r4, c4;
  quarter_dims(*S[0], k, r1, c1, sh);
  quarter_dims(*S[3], k + 3, r4, c4, sh);
  CTM_REQUIRE(o.projectors == CTM_PROJ_HALF || o.projectors == CTM_PROJ_FULL, CTM_ERR_INVALID,
              "Invalid ctmrg projector type");
  CTM_REQUIRE(o.svd_type == CTM_SVD_RSVD || o.svd_type == CTM_SVD_FULL, CTM_ERR_INVALID,
              "Invalid svd type");
  CTM_REQUIRE(o.chi >= 1, CTM_ERR_INVALID, "chi must be >= 1");
  pd.p1_rows = c1;
  pd.p2_rows = r4;
  int64_t m, n;
  if (o.projectors == CTM_PROJ_HALF) {
    CTM_REQUIRE(c1 == r4, CTM_ERR_INVALID, "half-system: quarter tensors do not chain");
    m = r1;
    n = c4;
  } else {
    int64_t r2, c2, r3, c3;
    quarter_dims(*S[1], k + 1, r2, c2, sh);
    quarter_dims(*S[2], k + 2, r3, c3, sh);
    CTM_REQUIRE(c2 == r1 && c1 == r4 && c4 == r3, CTM_ERR_INVALID,
                "full-system: quarter tensors do not chain");
    m = r2;
    n = c3;
  }
  pd.omega_rows = n;
  if (o.svd_type == CTM_SVD_RSVD) {
    CTM_REQUIRE(o.rsvd_niter >= 0 && o.rsvd_oversampling >= 0, CTM_ERR_INVALID,
                "rsvd_niter and rsvd_oversampling must be >= 0");
    pd.q = std::min({o.chi + o.rsvd_oversampling, m, n});
    pd.cap = std::min(o.chi, pd.q);
  } else {
    pd.q = 0;
    pd.cap = std::min({o.chi, m, n});
  }
  return pd;
}

// ProjectorCalculator.calculate_half_system / calculate_full_system
// (acetn/renormalization/projectors.py:114-217).
void calculate_projectors(Ctx& c, const Site* S[4], int k, const ctm_ctmrg_opts& o,
                          const double* omega, double* P1, double* P2, int64_t* chi_new) {
  const ProjDims pd = projector_dims(S, k, o);
  const int prec = o.precision;
  CTM_REQUIRE(prec == CTM_PREC_FP64 || prec == CTM_PREC_MIXED, CTM_ERR_INVALID, "bad precision");
  // here the mixed precision is the full-rank form: quarter tensors and the
  // products that feed the SVD in 3xBF16, the SVD and the projector products
  // in FP64, singular values below the mixed floor dropped (the spectrum of
  // the 3xBF16 products is noise there)
  CTM_REQUIRE(prec == CTM_PREC_FP64 || o.svd_type == CTM_SVD_FULL, CTM_ERR_INVALID,
              "mixed randomized-SVD projectors run in calculate_projectors_mixed");
  ctm_ctmrg_opts om = o;
  if (prec == CTM_PREC_MIXED) om.svd_cutoff = std::max({o.svd_cutoff, o.mixed_floor, 1e-8});
  auto quarter = [&](const Site& site, int kk, double* Q, int64_t* qs) {
    if (prec == CTM_PREC_MIXED) quarter_tensor_mixed_f64(c, site, kk, Q);
    else quarter_tensor(c, site, kk, Q, qs);
  };
  Scope scope(c);
  int64_t sh1[6], sh4[6], r1, c1, r4, c4;
  quarter_dims(*S[0], k, r1, c1, sh1);
  quarter_dims(*S[3], k + 3, r4, c4, sh4);
  double* Q1 = c.alloc<double>(size_t(r1) * c1);
  double* Q4 = c.alloc<double>(size_t(r4) * c4);
  quarter(*S[0], k, Q1, sh1);
  quarter(*S[3], k + 3, Q4, sh4);
  const Factor F1{Q1, r1, c1}, F4{Q4, r4, c4};
  if (o.projectors == CTM_PROJ_HALF) {
    if (o.svd_type == CTM_SVD_RSVD) {
      const int64_t q = pd.q;
      double* U = c.alloc<double>(size_t(r1) * q);
      double* s = c.alloc<double>(q);
      double* V = c.alloc<double>(size_t(c4) * q);
      rsvd_chain(c, {F1, F4}, q, o.rsvd_niter, omega, U, s, V, prec);
      truncate_and_project(c, U, V, r1, c4, q, s, q, o, F1, nullptr, F4, nullptr, P1, P2, chi_new,
                           prec);
    } else {
      // contract_half_system (projectors.py:62-82): R = Q1 Q4 / max|R|
      const int64_t r = std::min(r1, c4);
      double* R = c.alloc<double>(size_t(r1) * c4);
      double* mx = c.alloc<double>(1);
      double* U = c.alloc<double>(size_t(r1) * r);
      double* s = c.alloc<double>(r);
      double* V = c.alloc<double>(size_t(c4) * r);
      product(c, Q1, Q4, R, r1, c4, c1, prec);
      absmax(c, R, r1 * c4, mx);
      divide_by(c, R, r1 * c4, mx, 0);
      svd_thin(c, R, r1, c4, U, s, V);
      truncate_and_project(c, U, V, r1, c4, r, s, r, om, F1, nullptr, F4, nullptr, P1, P2,
                           chi_new, CTM_PREC_FP64);
    }
    return;
  }
  // full system
  int64_t sh2[6], sh3[6], r2, c2, r3, c3;
  quarter_dims(*S[1], k + 1, r2, c2, sh2);
  quarter_dims(*S[2], k + 2, r3, c3, sh3);
  double* Q2 = c.alloc<double>(size_t(r2) * c2);
  double* Q3 = c.alloc<double>(size_t(r3) * c3);
  quarter(*S[1], k + 1, Q2, sh2);
  quarter(*S[2], k + 2, Q3, sh3);
  const Factor F2{Q2, r2, c2}, F3{Q3, r3, c3};
  if (o.svd_type == CTM_SVD_RSVD) {
    const int64_t q = pd.q;
    double* U = c.alloc<double>(size_t(r2) * q);
    double* s = c.alloc<double>(q);
    double* V = c.alloc<double>(size_t(c3) * q);
    rsvd_chain(c, {F2, F1, F4, F3}, q, o.rsvd_niter, omega, U, s, V, CTM_PREC_FP64);
    truncate_and_project(c, U, V, r2, c3, q, s, q, o, F1, &F2, F4, &F3, P1, P2, chi_new,
                         CTM_PREC_FP64);
    return;
  }
  // contract_full_system (projectors.py:84-112)
  double* R1 = c.alloc<double>(size_t(r2) * c1);
  double* R2 = c.alloc<double>(size_t(r4) * c3);
  double* Fm = c.alloc<double>(size_t(r2) * c3);
  double* mx = c.alloc<double>(3);
  product(c, Q2, Q1, R1, r2, c1, c2, prec);
  product(c, Q4, Q3, R2, r4, c3, c4, prec);
  absmax(c, R1, r2 * c1, mx);
  divide_by(c, R1, r2 * c1, mx, 0);
  absmax(c, R2, r4 * c3, mx + 1);
  divide_by(c, R2, r4 * c3, mx + 1, 0);
  product(c, R1, R2, Fm, r2, c3, c1, prec);
  absmax(c, Fm, r2 * c3, mx + 2);
  divide_by(c, Fm, r2 * c3, mx + 2, 0);
  const int64_t r = std::min(r2, c3);
  double* U = c.alloc<double>(size_t(r2) * r);
  double* s = c.alloc<double>(r);
  double* V = c.alloc<double>(size_t(c3) * r);
  svd_thin(c, Fm, r2, c3, U, s, V);
  truncate_and_project(c, U, V, r2, c3, r, s, r, om, Factor{R1, r2, c1}, nullptr,
                       Factor{R2, r4, c3}, nullptr, P1, P2, chi_new, CTM_PREC_FP64);
}

// ------------------------------------------------------------------ renormalization
namespace {

// renormalize_cj1 / renormalize_cj2 of the mixed path: FP32 contractions,
// FP64 normalisation.
void renormalize_corners_f32(Ctx& c, const Site& S, int k, const double* P1i, int64_t x1i,
                             const double* P2j, int64_t x2j, double* Cout1, double* Cout2) {
  const int64_t D = S.D;
  Scope scope(c);
  double* nrm = c.alloc<double>(2);
  auto f32 = [&](const double* p, int64_t n) {
    float* y = c.alloc<float>(size_t(n));
    to_f32(c, p, y, n);
    return y;
  };
  {  // renormalize_cj1
    const View ci = S.C(3 + k), ei = S.E(2 + k);
    const int64_t a = ei.shape[0], b = ei.shape[1], cc = ci.shape[1];
    CTM_REQUIRE(ci.shape[0] == b, CTM_ERR_INVALID, "cj1: C and E do not chain");
    Scope s2(c);
    float* cf = f32(ci.p, ci.numel());
    float* ef = f32(ei.p, ei.numel());
    float* pf = f32(P1i, cc * D * D * x1i);
    float* t = c.alloc<float>(size_t(a) * D * D * cc);
    float* o = c.alloc<float>(size_t(a) * x1i);
    einsum(c, "ablL,bc->alLc", ViewF(ef, {a, b, D, D}), ViewF(cf, {b, cc}), ViewF(t, {a, D, D, cc}));
    einsum(c, "alLc,clLx->ax", ViewF(t, {a, D, D, cc}), ViewF(pf, {cc, D, D, x1i}),
           ViewF(o, {a, x1i}));
    to_f64(c, o, Cout1, a * x1i);
    sumsq(c, Cout1, a * x1i, nrm);
    divide_by(c, Cout1, a * x1i, nrm, 1);
  }
  {  // renormalize_cj2
    const View ci = S.C(k), ei = S.E(k);
    const int64_t a = ci.shape[0], b = ci.shape[1], cc = ei.shape[1];
    CTM_REQUIRE(ei.shape[0] == b, CTM_ERR_INVALID, "cj2: C and E do not chain");
    Scope s2(c);
    float* cf = f32(ci.p, ci.numel());
    float* ef = f32(ei.p, ei.numel());
    float* pf = f32(P2j, a * D * D * x2j);
    float* t = c.alloc<float>(size_t(a) * cc * D * D);
    float* o = c.alloc<float>(size_t(x2j) * cc);
    einsum(c, "ab,bcrR->acrR", ViewF(cf, {a, b}), ViewF(ef, {b, cc, D, D}), ViewF(t, {a, cc, D, D}));
    einsum(c, "arRx,acrR->xc", ViewF(pf, {a, D, D, x2j}), ViewF(t, {a, cc, D, D}),
           ViewF(o, {x2j, cc}));
    to_f64(c, o, Cout2, x2j * cc);
    sumsq(c, Cout2, x2j * cc, nrm + 1);
    divide_by(c, Cout2, x2j * cc, nrm + 1, 1);
  }
}

}  // namespace

// DirectionalMover.renormalize_boundary and its three kernels
// (acetn/renormalization/directional_mover.py:273-366).
void renormalize_boundary(Ctx& c, const Site& S, int k, const double* P1i, int64_t x1i,
                          const double* P2j, int64_t x2j, const double* P2i, int64_t x2i,
                          const double* P1j, int64_t x1j, double* Cout1, double* Cout2,
                          double* Eout, int precision) {
  const int64_t D = S.D, d = S.d;
  KernelTimer span(c.stream, kTagRenorm, 0.0);
  Scope scope(c);
  double* nrm = c.alloc<double>(3);
  if (precision == CTM_PREC_MIXED) {
    renormalize_corners_f32(c, S, k, P1i, x1i, P2j, x2j, Cout1, Cout2);
    renormalize_ej_mixed(c, S, k, P2i, x2i, P1j, x1j, Eout);
    return;
  }
  {  // renormalize_cj1
    const View ci = S.C(3 + k), ei = S.E(2 + k);
    const int64_t a = ei.shape[0], b = ei.shape[1], cc = ci.shape[1];
    CTM_REQUIRE(ci.shape[0] == b, CTM_ERR_INVALID, "cj1: C and E do not chain");
    Scope s2(c);
    double* t = c.alloc<double>(size_t(a) * D * D * cc);
    einsum(c, "ablL,bc->alLc", ei, ci, View(t, {a, D, D, cc}));
    einsum(c, "alLc,clLx->ax", View(t, {a, D, D, cc}), View(P1i, {cc, D, D, x1i}),
           View(Cout1, {a, x1i}));
    sumsq(c, Cout1, a * x1i, nrm);
    divide_by(c, Cout1, a * x1i, nrm, 1);
  }
  {  // renormalize_cj2
    const View ci = S.C(k), ei = S.E(k);
    const int64_t a = ci.shape[0], b = ci.shape[1], cc = ei.shape[1];
    CTM_REQUIRE(ei.shape[0] == b, CTM_ERR_INVALID, "cj2: C and E do not chain");
    Scope s2(c);
    double* t = c.alloc<double>(size_t(a) * cc * D * D);
    einsum(c, "ab,bcrR->acrR", ci, ei, View(t, {a, cc, D, D}));
    einsum(c, "arRx,acrR->xc", View(P2j, {a, D, D, x2j}), View(t, {a, cc, D, D}),
           View(Cout2, {x2j, cc}));
    sumsq(c, Cout2, x2j * cc, nrm + 1);
    divide_by(c, Cout2, x2j * cc, nrm + 1, 1);
  }
  {  // renormalize_ej
    const View ei = S.E(3 + k), ai = S.A(k);
    const int64_t a = ei.shape[0], b = ei.shape[1];
    Scope s2(c);
    double* t1 = c.alloc<double>(size_t(a) * D * D * D * D * x1j);
    double* t2 = c.alloc<double>(size_t(D) * D * d * a * D * D * x1j);
    double* t3 = c.alloc<double>(size_t(D) * D * D * D * a * x1j);
    einsum(c, "ablL,buUx->alLuUx", ei, View(P1j, {b, D, D, x1j}), View(t1, {a, D, D, D, D, x1j}));
    einsum(c, "LURDP,alLuUx->RDPalux", ai, View(t1, {a, D, D, D, D, x1j}),
           View(t2, {D, D, d, a, D, D, x1j}));
    einsum(c, "lurdp,RDpalux->rdRDax", ai, View(t2, {D, D, d, a, D, D, x1j}),
           View(t3, {D, D, D, D, a, x1j}));
    einsum(c, "rdRDax,adDy->yxrR", View(t3, {D, D, D, D, a, x1j}), View(P2i, {a, D, D, x2i}),
           View(Eout, {x2i, x1j, D, D}));
    sumsq(c, Eout, x2i * x1j * D * D, nrm + 2);
    divide_by(c, Eout, x2i * x1j * D * D, nrm + 2, 1);
  }
}

// ------------------------------------------------------------------ RDMs
namespace {

// The site RDM chain of RDM.build_site_rdm on views of element type T
// (FP64 or FP32 GETT).
template <class T>
void site_rdm_chain(Ctx& c, const ViewT<T>& c1, const ViewT<T>& c2, const ViewT<T>& c3,
                    const ViewT<T>& c4, const ViewT<T>& e1, const ViewT<T>& e2,
                    const ViewT<T>& e3, const ViewT<T>& e4, const ViewT<T>& a1, int64_t D,
                    int64_t d, T* out) {
  using V = ViewT<T>;
  Scope scope(c);
  // tmp1 = einsum("ab,bclL->aclL", c4, e4)
  const int64_t A4 = c4.shape[0], C4 = e4.shape[1];
  T* t1a = c.alloc<T>(size_t(A4) * C4 * D * D);
  einsum(c, "ab,bclL->aclL", c4, e4, V(t1a, {A4, C4, D, D}));
  // einsum("aclL,eadD->clLedD", tmp1, e3)
  const int64_t E3 = e3.shape[0];
  T* t1b = c.alloc<T>(size_t(C4) * D * D * E3 * D * D);
  einsum(c, "aclL,eadD->clLedD", V(t1a, {A4, C4, D, D}), e3, V(t1b, {C4, D, D, E3, D, D}));
  // einsum("clLedD,LURDP->cledURP", tmp1, conj(a1))
  T* t1c = c.alloc<T>(size_t(C4) * D * E3 * D * D * D * d);
  einsum(c, "clLedD,LURDP->cledURP", V(t1b, {C4, D, D, E3, D, D}), a1,
         V(t1c, {C4, D, E3, D, D, D, d}));
  // tmp2 = einsum("ab,bcuU->acuU", c1, e1)
  const int64_t A1 = c1.shape[0], C1 = e1.shape[1];
  T* t2 = c.alloc<T>(size_t(A1) * C1 * D * D);
  einsum(c, "ab,bcuU->acuU", c1, e1, V(t2, {A1, C1, D, D}));
  // tmp3 = einsum("ab,carR->bcrR", c3, e2)
  const int64_t B3 = c3.shape[1], CE2 = e2.shape[0];
  T* t3a = c.alloc<T>(size_t(B3) * CE2 * D * D);
  einsum(c, "ab,carR->bcrR", c3, e2, V(t3a, {B3, CE2, D, D}));
  // tmp3 = einsum("ec,bcrR->ebrR", c2, tmp3)
  const int64_t E2r = c2.shape[0];
  T* t3b = c.alloc<T>(size_t(E2r) * B3 * D * D);
  einsum(c, "ec,bcrR->ebrR", c2, V(t3a, {B3, CE2, D, D}), V(t3b, {E2r, B3, D, D}));
  // tmp3 = einsum("ebrR,aeuU->brRauU", tmp3, tmp2)
  T* t3c = c.alloc<T>(size_t(B3) * D * D * A1 * D * D);
  einsum(c, "ebrR,aeuU->brRauU", V(t3b, {E2r, B3, D, D}), V(t2, {A1, C1, D, D}),
         V(t3c, {B3, D, D, A1, D, D}));
  // tmp3 = einsum("erRcuU,cledURP->ruldP", tmp3, tmp1)
  T* t3d = c.alloc<T>(size_t(D) * D * D * D * d);
  einsum(c, "erRcuU,cledURP->ruldP", V(t3c, {B3, D, D, A1, D, D}),
         V(t1c, {C4, D, E3, D, D, D, d}), V(t3d, {D, D, D, D, d}));
  // rdm = einsum("ruldP,lurdp->Pp", tmp3, a1)
  einsum(c, "ruldP,lurdp->Pp", V(t3d, {D, D, D, D, d}), a1, V(out, {d, d}));
}

// FP32 copy of an FP64 view: the whole underlying tensor is converted and
// the view's shape and strides are kept (a bond_permute view stays a view).
ViewF f32_copy(Ctx& c, const View& v) {
  int64_t n = 1;
  for (int i = 0; i < v.nd; ++i) n += (v.shape[i] - 1) * v.stride[i];
  float* p = c.alloc<float>(size_t(n));
  to_f32(c, v.p, p, n);
  ViewF out;
  out.p = p;
  out.nd = v.nd;
  for (int i = 0; i < v.nd; ++i) out.shape[i] = v.shape[i], out.stride[i] = v.stride[i];
  return out;
}

}  // namespace

// RDM.build_site_rdm (acetn/measurement/rdm.py:35-67).  CTM_PREC_MIXED runs
// the same chain with FP32 FMAs and FP32 accumulation (FP64 result).
void site_rdm(Ctx& c, const Site& S, double* out, int precision) {
  const int64_t D = S.D, d = S.d;
  if (precision == CTM_PREC_FP64) {
    site_rdm_chain<double>(c, S.C(0), S.C(1), S.C(2), S.C(3), S.E(0), S.E(1), S.E(2), S.E(3),
                           S.A(0), D, d, out);
    return;
  }
  Scope scope(c);
  float* o = c.alloc<float>(size_t(d) * d);
  site_rdm_chain<float>(c, f32_copy(c, S.C(0)), f32_copy(c, S.C(1)), f32_copy(c, S.C(2)),
                        f32_copy(c, S.C(3)), f32_copy(c, S.E(0)), f32_copy(c, S.E(1)),
                        f32_copy(c, S.E(2)), f32_copy(c, S.E(3)), f32_copy(c, S.A(0)), D, d, o);
  to_f64(c, o, out, d * d);
}

// RDM.build_bond_rdm (acetn/measurement/rdm.py:69-99) with the unblocked core
// build_bond_rdm_core (rdm.py:102-120), the same sum as the blocked loop of
// build_bond_rdm_core_blocked (rdm.py:123-153).
void bond_rdm(Ctx& c, const Site& S1, const Site& S2, int k, double* out) {
  const int64_t D = S1.D, d = S1.d;
  const View c12 = S1.C(k + 1), e12 = S1.E(k + 1), e11 = S1.E(k), c13 = S1.C(k + 2),
             e13 = S1.E(k + 2), a1 = S1.A(k);
  const View c21 = S2.C(k), e21 = S2.E(k), e24 = S2.E(k + 3), c24 = S2.C(k + 3),
             e23 = S2.E(k + 2), a2 = S2.A(k);
  Scope scope(c);
  // right half
  const int64_t ra = c12.shape[0], rc = e12.shape[1], re = e11.shape[0];
  double* t = c.alloc<double>(size_t(ra) * rc * D * D);
  einsum(c, "ab,bcrR->acrR", c12, e12, View(t, {ra, rc, D, D}));
  double* tt = c.alloc<double>(size_t(rc) * D * D * re * D * D);
  einsum(c, "acrR,eauU->crReuU", View(t, {ra, rc, D, D}), e11, View(tt, {rc, D, D, re, D, D}));
  double* t3 = c.alloc<double>(size_t(rc) * D * re * D * D * D * d);
  einsum(c, "crReuU,LURDP->creuLDP", View(tt, {rc, D, D, re, D, D}), a1,
         View(t3, {rc, D, re, D, D, D, d}));
  double* t4 = c.alloc<double>(size_t(rc) * re * D * D * d * D * D * d);
  einsum(c, "creuLDP,lurdp->ceLDPldp", View(t3, {rc, D, re, D, D, D, d}), a1,
         View(t4, {rc, re, D, D, d, D, D, d}));
  const int64_t fa = c13.shape[0], ff = e13.shape[1];
  double* r1a = c.alloc<double>(size_t(fa) * ff * D * D);
  einsum(c, "ab,bfdD->afdD", c13, e13, View(r1a, {fa, ff, D, D}));
  double* r1 = c.alloc<double>(size_t(ff) * re * D * d * D * d);
  einsum(c, "afdD,acLDPldp->fcLPlp", View(r1a, {fa, ff, D, D}), View(t4, {rc, re, D, D, d, D, D, d}),
         View(r1, {ff, re, D, d, D, d}));
  // left half
  const int64_t la = c21.shape[0], lc = e21.shape[1], le = e24.shape[0];
  double* u = c.alloc<double>(size_t(la) * lc * D * D);
  einsum(c, "ab,bcuU->acuU", c21, e21, View(u, {la, lc, D, D}));
  double* uu = c.alloc<double>(size_t(lc) * D * D * le * D * D);
  einsum(c, "acuU,ealL->cuUelL", View(u, {la, lc, D, D}), e24, View(uu, {lc, D, D, le, D, D}));
  double* u3 = c.alloc<double>(size_t(lc) * D * le * D * D * D * d);
  einsum(c, "cuUelL,LURDQ->cuelRDQ", View(uu, {lc, D, D, le, D, D}), a2,
         View(u3, {lc, D, le, D, D, D, d}));
  double* u4 = c.alloc<double>(size_t(lc) * le * D * D * d * D * D * d);
  einsum(c, "cuelRDQ,lurdq->ceRDQrdq", View(u3, {lc, D, le, D, D, D, d}), a2,
         View(u4, {lc, le, D, D, d, D, D, d}));
  const int64_t ea = c24.shape[1], ef = e23.shape[0];
  double* r2a = c.alloc<double>(size_t(ea) * ef * D * D);
  einsum(c, "ae,fadD->efdD", c24, e23, View(r2a, {ea, ef, D, D}));
  double* r2 = c.alloc<double>(size_t(ef) * lc * D * d * D * d);
  einsum(c, "efdD,ceRDQrdq->fcRQrq", View(r2a, {ea, ef, D, D}),
         View(u4, {lc, le, D, D, d, D, D, d}), View(r2, {ef, lc, D, d, D, d}));
  einsum(c, "fcRPrp,fcRQrq->PQpq", View(r1, {ff, re, D, d, D, d}), View(r2, {ef, lc, D, d, D, d}),
         View(out, {d, d, d, d}));
}

// The full update's norm tensor: build_norm_tensor with
// build_norm_tensor_core (acetn/evolution/full_update.py:163-236), the
// environment of bond (s1, s2, k) -- the bond RDM's chain -- contracted with
// the reduced site tensors a1q (r, d, u, y) and a2q (d, l, u, x) of width nD
// into n12[y][x][Y][X].  Real tensors: the reference's conj() is the identity.
void norm_tensor(Ctx& c, const Site& S1, const Site& S2, int k, const double* a1q,
                 const double* a2q, int64_t nD, double* out) {
  const int64_t D = S1.D;
  const View c12 = S1.C(k + 1), e12 = S1.E(k + 1), e11 = S1.E(k), c13 = S1.C(k + 2),
             e13 = S1.E(k + 2);
  const View c21 = S2.C(k), e21 = S2.E(k), e24 = S2.E(k + 3), c24 = S2.C(k + 3),
             e23 = S2.E(k + 2);
  const View q1(a1q, {D, D, D, nD}), q2(a2q, {D, D, D, nD});
  Scope scope(c);
  // right half
  const int64_t ra = c12.shape[0], rc = e12.shape[1], re = e11.shape[0];
  double* t = c.alloc<double>(size_t(ra) * rc * D * D);
  einsum(c, "ab,bcrR->acrR", c12, e12, View(t, {ra, rc, D, D}));
  double* tt = c.alloc<double>(size_t(rc) * D * D * re * D * D);
  einsum(c, "acrR,eauU->crReuU", View(t, {ra, rc, D, D}), e11, View(tt, {rc, D, D, re, D, D}));
  double* t3 = c.alloc<double>(size_t(rc) * D * re * D * D * nD);
  einsum(c, "crReuU,RDUY->creuDY", View(tt, {rc, D, D, re, D, D}), q1,
         View(t3, {rc, D, re, D, D, nD}));
  double* t4 = c.alloc<double>(size_t(rc) * re * D * nD * D * nD);
  einsum(c, "creuDY,rduy->ceDYdy", View(t3, {rc, D, re, D, D, nD}), q1,
         View(t4, {rc, re, D, nD, D, nD}));
  const int64_t fa = c13.shape[0], ff = e13.shape[1];
  double* n1a = c.alloc<double>(size_t(fa) * ff * D * D);
  einsum(c, "ab,bfdD->afdD", c13, e13, View(n1a, {fa, ff, D, D}));
  double* n1 = c.alloc<double>(size_t(ff) * re * nD * nD);
  einsum(c, "afdD,aeDYdy->feYy", View(n1a, {fa, ff, D, D}), View(t4, {rc, re, D, nD, D, nD}),
         View(n1, {ff, re, nD, nD}));
  // left half
  const int64_t la = c21.shape[0], lc = e21.shape[1], le = e24.shape[0];
  double* u = c.alloc<double>(size_t(la) * lc * D * D);
  einsum(c, "ab,bcuU->acuU", c21, e21, View(u, {la, lc, D, D}));
  double* uu = c.alloc<double>(size_t(lc) * D * D * le * D * D);
  einsum(c, "acuU,ealL->cuUelL", View(u, {la, lc, D, D}), e24, View(uu, {lc, D, D, le, D, D}));
  double* u3 = c.alloc<double>(size_t(lc) * D * le * D * nD * D);
  einsum(c, "cuUelL,DLUX->cuelXD", View(uu, {lc, D, D, le, D, D}), q2,
         View(u3, {lc, D, le, D, nD, D}));
  double* u4 = c.alloc<double>(size_t(lc) * le * nD * D * nD * D);
  einsum(c, "cuelXD,dlux->ceXDxd", View(u3, {lc, D, le, D, nD, D}), q2,
         View(u4, {lc, le, nD, D, nD, D}));
  const int64_t bb = c24.shape[1], bf = e23.shape[0];
  double* n2a = c.alloc<double>(size_t(bb) * bf * D * D);
  einsum(c, "ab,fadD->bfdD", c24, e23, View(n2a, {bb, bf, D, D}));
  double* n2 = c.alloc<double>(size_t(bf) * lc * nD * nD);
  einsum(c, "bfdD,cbXDxd->fcXx", View(n2a, {bb, bf, D, D}), View(u4, {lc, le, nD, D, nD, D}),
         View(n2, {bf, lc, nD, nD}));
  einsum(c, "fcYy,fcXx->yxYX", View(n1, {ff, re, nD, nD}), View(n2, {bf, lc, nD, nD}),
         View(out, {nD, nD, nD, nD}));
}

}  // namespace ctm

// ====================================================================== C ABI
using namespace ctm;

namespace {
cudaStream_t as_stream(ctm_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }
}  // namespace

extern "C" {

const char* ctm_version(void) { return "ctm_gb300 0.1 (sm_103a)"; }

const char* ctm_last_error(void) { return ctm::g_last_error_cstr(); }

int ctm_set_mixed_contraction(int32_t form, int32_t* previous) {
  return guarded([&] {
    const int old = set_contraction_form(form);
    if (previous != nullptr) *previous = old;
  });
}

unsigned long long ctm_kernel_launches(void) { return g_launches.load(); }

int ctm_qr_fallbacks(unsigned long long* count, ctm_stream_t stream) {
  return guarded([&] {
    CTM_REQUIRE(count != nullptr, CTM_ERR_INVALID, "count is NULL");
    unsigned long long* d = qr_fallback_counter();
    CTM_CUDA(cudaMemcpyAsync(count, d, sizeof(*count), cudaMemcpyDeviceToHost, as_stream(stream)));
    CTM_CUDA(cudaStreamSynchronize(as_stream(stream)));
    CTM_CUDA(cudaMemsetAsync(d, 0, sizeof(*count), as_stream(stream)));
  });
}

int ctm_device_status(int* flags_out, ctm_stream_t stream) {
  return guarded([&] {
    CTM_REQUIRE(flags_out != nullptr, CTM_ERR_INVALID, "flags_out is NULL");
    Ctx c;
    int* dflags = status_flags(c);
    CTM_CUDA(cudaMemcpyAsync(flags_out, dflags, sizeof(int), cudaMemcpyDeviceToHost, as_stream(stream)));
    CTM_CUDA(cudaStreamSynchronize(as_stream(stream)));
    CTM_CUDA(cudaMemsetAsync(dflags, 0, sizeof(int), as_stream(stream)));
  });
}

int ctm_quarter_tensor(const ctm_site_f64* site, int64_t D, int64_t d, int32_t k, double* Q,
                       int64_t* qshape, int32_t precision, void* ws, size_t* ws_bytes,
                       ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    check_site(site, D, d);
    CTM_REQUIRE(precision == CTM_PREC_FP64 || precision == CTM_PREC_MIXED, CTM_ERR_INVALID,
                "bad precision");
    Site S{site, D, d};
    int64_t sh[6], rows, cols;
    if (!c.sizing()) CTM_REQUIRE(Q != nullptr, CTM_ERR_INVALID, "Q is NULL");
    if (precision == CTM_PREC_MIXED) {
      quarter_dims(S, k, rows, cols, sh);
      quarter_tensor_mixed_f64(c, S, k, Q);
    } else {
      quarter_tensor(c, S, k, Q, sh);
    }
    if (qshape != nullptr)
      for (int i = 0; i < 6; ++i) qshape[i] = sh[i];
  });
}

int ctm_projector_dims(const ctm_site_f64* const* sites, int64_t D, int32_t k,
                       const ctm_ctmrg_opts* opts, int64_t* p1_rows, int64_t* p2_rows,
                       int64_t* omega_rows, int64_t* q, int64_t* chi_cap) {
  return guarded([&] {
    CTM_REQUIRE(sites != nullptr && opts != nullptr, CTM_ERR_INVALID, "NULL argument");
    Site Ss[4];
    const Site* S[4];
    for (int i = 0; i < 4; ++i) {
      CTM_REQUIRE(sites[i] != nullptr, CTM_ERR_INVALID, "site pointer is NULL");
      Ss[i] = Site{sites[i], D, 1};
      S[i] = &Ss[i];
    }
    const ProjDims pd = projector_dims(S, k, *opts);
    if (p1_rows) *p1_rows = pd.p1_rows;
    if (p2_rows) *p2_rows = pd.p2_rows;
    if (omega_rows) *omega_rows = pd.omega_rows;
    if (q) *q = pd.q;
    if (chi_cap) *chi_cap = pd.cap;
  });
}

int ctm_calculate_projectors(const ctm_site_f64* const* sites, int64_t D, int64_t d, int32_t k,
                             const ctm_ctmrg_opts* opts, const double* omega, double* P1,
                             double* P2, int64_t* chi_new, void* ws, size_t* ws_bytes,
                             ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    CTM_REQUIRE(sites != nullptr && opts != nullptr, CTM_ERR_INVALID, "NULL argument");
    Site Ss[4];
    const Site* S[4];
    for (int i = 0; i < 4; ++i) {
      check_site(sites[i], D, d);
      Ss[i] = Site{sites[i], D, d};
      S[i] = &Ss[i];
    }
    if (!c.sizing()) {
      CTM_REQUIRE(P1 != nullptr && P2 != nullptr && chi_new != nullptr, CTM_ERR_INVALID,
                  "output pointer is NULL");
      CTM_REQUIRE(opts->svd_type != CTM_SVD_RSVD || omega != nullptr, CTM_ERR_INVALID,
                  "omega is NULL for the randomized SVD");
    }
    if (opts->precision == CTM_PREC_MIXED && opts->svd_type == CTM_SVD_RSVD)
      calculate_projectors_mixed(c, S, k, *opts, omega, P1, P2, chi_new);
    else
      calculate_projectors(c, S, k, *opts, omega, P1, P2, chi_new);
  });
}

int ctm_renormalize_boundary(const ctm_site_f64* s1, int64_t D, int64_t d, int32_t k,
                             const double* P1_i, int64_t chi_p1i, const double* P2_j,
                             int64_t chi_p2j, const double* P2_i, int64_t chi_p2i,
                             const double* P1_j, int64_t chi_p1j, double* Cout1, double* Cout2,
                             double* Eout, int32_t precision, void* ws, size_t* ws_bytes,
                             ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    check_site(s1, D, d);
    CTM_REQUIRE(precision == CTM_PREC_FP64 || precision == CTM_PREC_MIXED, CTM_ERR_INVALID,
                "bad precision");
    CTM_REQUIRE(chi_p1i >= 1 && chi_p2j >= 1 && chi_p2i >= 1 && chi_p1j >= 1, CTM_ERR_INVALID,
                "projector widths must be >= 1");
    if (!c.sizing())
      CTM_REQUIRE(P1_i && P2_j && P2_i && P1_j && Cout1 && Cout2 && Eout, CTM_ERR_INVALID,
                  "NULL tensor pointer");
    Site S{s1, D, d};
    renormalize_boundary(c, S, k, P1_i, chi_p1i, P2_j, chi_p2j, P2_i, chi_p2i, P1_j, chi_p1j,
                         Cout1, Cout2, Eout, precision);
  });
}

int ctm_move_batched(const ctm_site_f64* sites, int32_t nx, int32_t ny, int64_t D, int64_t d,
                     const int32_t* moves, int32_t nmoves, const ctm_ctmrg_opts* opts,
                     const double* const* omegas, double* const* out, int64_t* chi_new, void* ws,
                     size_t* ws_bytes, ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    CTM_REQUIRE(sites != nullptr && moves != nullptr && opts != nullptr, CTM_ERR_INVALID,
                "NULL argument");
    CTM_REQUIRE(nx >= 1 && ny >= 1 && int64_t(nx) * ny <= 1024, CTM_ERR_INVALID,
                "unit cell must have 1 <= nx * ny <= 1024 sites");
    CTM_REQUIRE(nmoves == 1 || nmoves == 2, CTM_ERR_INVALID, "one or two moves per call");
    for (int m = 0; m < nmoves; ++m)
      CTM_REQUIRE(moves[2 * m] >= 0 && moves[2 * m] <= 3, CTM_ERR_INVALID,
                  "move direction must be 0..3");
    if (nmoves == 2)
      CTM_REQUIRE(moves[0] % 2 == moves[2] % 2 && moves[0] != moves[2], CTM_ERR_INVALID,
                  "two moves must be a left/right or an up/down pair");
    std::vector<Site> S(size_t(nx) * ny);
    for (int i = 0; i < nx * ny; ++i) {
      check_site(&sites[i], D, d);
      S[size_t(i)] = Site{&sites[i], D, d};
    }
    auto at = [&](int x, int y) -> const Site* {
      x = ((x % nx) + nx) % nx;
      y = ((y % ny) + ny) % ny;
      return &S[size_t(x) * ny + y];
    };
    ctm_ctmrg_opts o = *opts;
    o.fixed_width = 1;
    struct Row {
      const Site* q[4];
      int k;
      double *P1, *P2;
      int64_t cap;
    };
    std::vector<Row> rows;
    std::vector<int> first(nmoves), count(nmoves);
    for (int m = 0; m < nmoves; ++m) {
      const int k = moves[2 * m], idx = moves[2 * m + 1];
      const int nr = (k % 2 == 0) ? ny : nx;
      first[m] = int(rows.size());
      count[m] = nr;
      for (int r = 0; r < nr; ++r) {
        Row w{};
        w.k = k;
        // the site quadruples of calculate_{left,up,right,down}_projectors
        // (acetn/renormalization/directional_mover.py:99-181)
        if (k == 0) {
          w.q[0] = at(idx, r); w.q[1] = at(idx + 1, r); w.q[2] = at(idx + 1, r - 1); w.q[3] = at(idx, r - 1);
        } else if (k == 1) {
          w.q[0] = at(r, idx); w.q[1] = at(r, idx - 1); w.q[2] = at(r - 1, idx - 1); w.q[3] = at(r - 1, idx);
        } else if (k == 2) {
          w.q[0] = at(idx, r); w.q[1] = at(idx - 1, r); w.q[2] = at(idx - 1, r + 1); w.q[3] = at(idx, r + 1);
        } else {
          w.q[0] = at(r, idx); w.q[1] = at(r, idx + 1); w.q[2] = at(r + 1, idx + 1); w.q[3] = at(r + 1, idx);
        }
        const ProjDims pd = projector_dims(w.q, k, o);
        w.cap = pd.cap;
        w.P1 = c.alloc<double>(size_t(pd.p1_rows) * pd.cap);
        w.P2 = c.alloc<double>(size_t(pd.p2_rows) * pd.cap);
        rows.push_back(w);
      }
    }
    if (!c.sizing()) {
      CTM_REQUIRE(out != nullptr && chi_new != nullptr, CTM_ERR_INVALID, "output pointer is NULL");
      for (size_t t = 0; t < rows.size(); ++t) {
        CTM_REQUIRE(out[3 * t] && out[3 * t + 1] && out[3 * t + 2], CTM_ERR_INVALID,
                    "output tensor pointer is NULL");
        CTM_REQUIRE(o.svd_type != CTM_SVD_RSVD || (omegas != nullptr && omegas[t] != nullptr),
                    CTM_ERR_INVALID, "omega is NULL for the randomized SVD");
      }
    }
    // phase A: the projector pairs of every row of every move
    for (size_t t = 0; t < rows.size(); ++t) {
      Row& w = rows[t];
      const double* om = (omegas != nullptr) ? omegas[t] : nullptr;
      if (o.precision == CTM_PREC_MIXED && o.svd_type == CTM_SVD_RSVD)
        calculate_projectors_mixed(c, w.q, w.k, o, om, w.P1, w.P2, chi_new ? chi_new + t : nullptr);
      else
        calculate_projectors(c, w.q, w.k, o, om, w.P1, w.P2, chi_new ? chi_new + t : nullptr);
    }
    // phase B: renormalize_boundary of every row (directional_mover.py:273-303)
    for (int m = 0; m < nmoves; ++m) {
      const int k = moves[2 * m], idx = moves[2 * m + 1], nr = count[m];
      for (int r = 0; r < nr; ++r) {
        const Site* s1;
        int i = r, j;
        if (k == 0) { s1 = at(idx, r); j = (r + 1) % nr; }
        else if (k == 1) { s1 = at(r, idx); j = (r + 1) % nr; }
        else if (k == 2) { s1 = at(idx, r); j = (r - 1 + nr) % nr; }
        else { s1 = at(r, idx); j = (r - 1 + nr) % nr; }
        const Row& ri = rows[size_t(first[m] + i)];
        const Row& rj = rows[size_t(first[m] + j)];
        const size_t t = size_t(first[m] + r);
        renormalize_boundary(c, *s1, k, ri.P1, ri.cap, rj.P2, rj.cap, ri.P2, ri.cap, rj.P1, rj.cap,
                             out ? out[3 * t] : nullptr, out ? out[3 * t + 1] : nullptr,
                             out ? out[3 * t + 2] : nullptr, o.precision);
      }
    }
  });
}

int ctm_site_rdm(const ctm_site_f64* site, int64_t D, int64_t d, int32_t precision, double* rdm,
                 void* ws, size_t* ws_bytes, ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    check_site(site, D, d);
    CTM_REQUIRE(precision == CTM_PREC_FP64 || precision == CTM_PREC_MIXED, CTM_ERR_INVALID,
                "bad precision");
    if (!c.sizing()) CTM_REQUIRE(rdm != nullptr, CTM_ERR_INVALID, "rdm is NULL");
    Site S{site, D, d};
    site_rdm(c, S, rdm, precision);
  });
}

int ctm_bond_rdm(const ctm_site_f64* s1, const ctm_site_f64* s2, int64_t D, int64_t d, int32_t k,
                 int32_t precision, double* rdm, void* ws, size_t* ws_bytes, ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    check_site(s1, D, d);
    check_site(s2, D, d);
    CTM_REQUIRE(precision == CTM_PREC_FP64 || precision == CTM_PREC_MIXED, CTM_ERR_INVALID,
                "bad precision");
    if (!c.sizing()) CTM_REQUIRE(rdm != nullptr, CTM_ERR_INVALID, "rdm is NULL");
    Site S1{s1, D, d}, S2{s2, D, d};
    if (precision == CTM_PREC_MIXED)
      bond_rdm_mixed(c, S1, S2, k, rdm);
    else
      bond_rdm(c, S1, S2, k, rdm);
  });
}

int ctm_norm_tensor(const ctm_site_f64* s1, const ctm_site_f64* s2, int64_t D, int64_t d,
                    int32_t k, const double* a1q, const double* a2q, int64_t nD, double* n12,
                    void* ws, size_t* ws_bytes, ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    check_site(s1, D, d);
    check_site(s2, D, d);
    CTM_REQUIRE(nD >= 1, CTM_ERR_INVALID, "nD must be >= 1");
    if (!c.sizing())
      CTM_REQUIRE(a1q != nullptr && a2q != nullptr && n12 != nullptr, CTM_ERR_INVALID,
                  "a1q, a2q and n12 must not be NULL");
    Site S1{s1, D, d}, S2{s2, D, d};
    norm_tensor(c, S1, S2, k, a1q, a2q, nD, n12);
  });
}

int ctm_svd_lowrank(const double* a, int64_t m, int64_t n, int64_t q, int32_t niter,
                    const double* omega, double* U, double* S, double* V, void* ws,
                    size_t* ws_bytes, ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    CTM_REQUIRE(m >= 1 && n >= 1 && niter >= 0, CTM_ERR_INVALID, "bad size");
    rsvd_chain(c, {Factor{a, m, n}}, q, niter, omega, U, S, V, CTM_PREC_FP64);
  });
}

int ctm_fused_matmul_svd_lowrank(const double* a, const double* b, int64_t m, int64_t k, int64_t n,
                                 int64_t q, int32_t niter, const double* omega, double* U,
                                 double* S, double* V, int32_t precision, void* ws,
                                 size_t* ws_bytes, ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    CTM_REQUIRE(m >= 1 && n >= 1 && k >= 1 && niter >= 0, CTM_ERR_INVALID, "bad size");
    CTM_REQUIRE(precision == CTM_PREC_FP64 || precision == CTM_PREC_MIXED, CTM_ERR_INVALID,
                "bad precision");
    rsvd_chain(c, {Factor{a, m, k}, Factor{b, k, n}}, q, niter, omega, U, S, V, precision);
  });
}

int ctm_fused_3matmul_svd_lowrank(const double* a, const double* b, const double* cc,
                                  const double* e, int64_t m, int64_t k1, int64_t k2, int64_t k3,
                                  int64_t n, int64_t q, int32_t niter, const double* omega,
                                  double* U, double* S, double* V, void* ws, size_t* ws_bytes,
                                  ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    CTM_REQUIRE(m >= 1 && n >= 1 && k1 >= 1 && k2 >= 1 && k3 >= 1 && niter >= 0, CTM_ERR_INVALID,
                "bad size");
    rsvd_chain(c, {Factor{a, m, k1}, Factor{b, k1, k2}, Factor{cc, k2, k3}, Factor{e, k3, n}}, q,
               niter, omega, U, S, V, CTM_PREC_FP64);
  });
}

int ctm_svd_f64(const double* a, int64_t m, int64_t n, double* U, double* S, double* V, void* ws,
                size_t* ws_bytes, ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    CTM_REQUIRE(m >= 1 && n >= 1 && m <= 4096 && n <= 4096, CTM_ERR_UNSUPPORTED,
                "ctm_svd_f64: 1 <= m, n <= 4096");
    svd_thin(c, a, m, n, U, S, V);
  });
}

int ctm_qr(void* Y, int64_t n, int64_t q, void* R, int32_t dtype, void* ws, size_t* ws_bytes,
           ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    CTM_REQUIRE(n >= q && q >= 1, CTM_ERR_INVALID, "ctm_qr: needs n >= q >= 1");
    if (dtype == CTM_DTYPE_F64) {
      orthonormalize(c, static_cast<double*>(Y), n, q, static_cast<double*>(R));
    } else {
      CTM_REQUIRE(dtype == CTM_DTYPE_F32, CTM_ERR_INVALID, "ctm_qr: bad dtype");
      orthonormalize(c, static_cast<float*>(Y), n, q, static_cast<float*>(R));
    }
  });
}

int ctm_svd_f32(const float* bt, int64_t n, int64_t q, double* U, double* S, float* V, void* ws,
                size_t* ws_bytes, ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    CTM_REQUIRE(q >= 1 && q <= 1024 && q <= n, CTM_ERR_UNSUPPORTED,
                "ctm_svd_f32: 1 <= q <= min(n, 1024)");
    svd_via_qr(c, bt, q, n, U, S, V);
  });
}

int ctm_matmul(const double* A, const double* B, double* C, int64_t M, int64_t N, int64_t K,
               int32_t precision, void* ws, size_t* ws_bytes, ctm_stream_t stream) {
  return with_workspace(ws, ws_bytes, as_stream(stream), [&](Ctx& c) {
    CTM_REQUIRE(M >= 1 && N >= 1 && K >= 1, CTM_ERR_INVALID, "bad size");
    if (precision == CTM_PREC_FP64) {
      einsum(c, "ik,kj->ij", View(A, {M, K}), View(B, {K, N}), View(C, {M, N}));
    } else {
      CTM_REQUIRE(precision == CTM_PREC_MIXED || precision == CTM_PREC_BF16, CTM_ERR_INVALID,
                  "bad precision");
      const bool x3 = precision == CTM_PREC_MIXED;
      const int64_t lda = tc_ld(K);
      Scope scope(c);
      bf16* ah = c.alloc<bf16>(size_t(M) * lda);
      bf16* al = x3 ? c.alloc<bf16>(size_t(M) * lda) : nullptr;
      bf16* bh = c.alloc<bf16>(size_t(N) * lda);
      bf16* bl = x3 ? c.alloc<bf16>(size_t(N) * lda) : nullptr;
      split_bf16(c, A, M, K, K, false, ah, al, lda);
      split_bf16(c, B, K, N, N, true, bh, bl, lda);
      TcOperand a{ah, al, M, K, lda}, b{bh, bl, N, K, lda};
      TcOut out;
      out.add(TcKind::kF64, C, TcLayout::rows(M, N, N));
      tc_gemm(c, a, b, x3 ? TcMode::kBf16x3 : TcMode::kBf16x1, out);
    }
  });
}

}  // extern "C"
