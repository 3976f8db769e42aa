// Internal operations of the CTMRG library (FP64 engine and helpers).
#pragma once
#include "ctm_common.cuh"

namespace ctm {

// C = alpha * einsum(spec, A, B) + beta * C for two-operand contractions whose
// labels split into batch / row / column / contracted groups (no traces, no
// outer-only labels).  All views are strided; nothing is copied.
void einsum(Ctx& c, const char* spec, const View& A, const View& B, const View& C,
            double alpha = 1.0, double beta = 0.0);
// The same contraction in FP32 (FP32 FMAs, FP32 accumulation).
void einsum(Ctx& c, const char* spec, const ViewF& A, const ViewF& B, const ViewF& C,
            double alpha = 1.0, double beta = 0.0);

// Deterministic reductions into a device scalar.
// Number of SMs of the current device.
int sm_count_linalg();

void absmax(Ctx& c, const double* x, int64_t n, double* out);
void sumsq(Ctx& c, const double* x, int64_t n, double* out);
// x[i] = x[i] / s  (mode 0: s = *scal, mode 1: s = sqrt(*scal)) for i < n.
void divide_by(Ctx& c, double* x, int64_t n, const double* scal, int mode);
// dst (rows x cols, row-major, ld_dst) = src view (2-D strided)
void copy2d(Ctx& c, const View& src, double* dst, int64_t ld_dst);
void fill(Ctx& c, double* x, int64_t n, double v);
// Element-wise precision conversions (n elements, contiguous).
void to_f32(Ctx& c, const double* x, float* y, int64_t n);
void to_f64(Ctx& c, const float* x, double* y, int64_t n);

// --- linear algebra (FP64) ---------------------------------------------------
// Orthonormal basis of the columns of Y (n x q, row-major): Y := Q.
// If R != nullptr it receives the q x q upper-triangular factor with Y_in = Q R.
// stages: Cholesky-QR stages (3: orthonormal to working precision; 2: to
// ~u cond^2 after the shifted stage, i.e. about 1e-3 in FP32, for bases that
// are only multiplied again in lower precision).
void orthonormalize(Ctx& c, double* Y, int64_t n, int64_t q, double* R, int stages = 3);
// The same in FP32 arithmetic (mixed path).
void orthonormalize(Ctx& c, float* Y, int64_t n, int64_t q, float* R, int stages = 3);
// Thin SVD of X (m x n, row-major, m >= n is not required):
// X = U diag(S) V^T, U (m x r), S (r) descending, V (n x r), r = min(m, n).
void svd_thin(Ctx& c, const double* X, int64_t m, int64_t n, double* U, double* S,
              double* V);
// Thin SVD of B (q x n, q <= min(n, 1024)) for the mixed path, from
// Bt = B^T (n x q, FP32): R of a shifted Cholesky-QR3 of Bt (B = R^T Qb^T),
// FP32 one-sided Jacobi on the columns of R with accumulated rotations
// (Ub = its left singular vectors, orthogonal to ~1e-6; singular values to
// ~1e-6 s_0, below the ~1e-5 s_0 of the 3xBF16 products that form B),
// V = B^T Ub diag(1/s) in FP32.
void svd_via_qr(Ctx& c, const float* Bt, int64_t q, int64_t n, double* Ub, double* S, float* V);
// Truncation of acetn/renormalization/projectors.py:163-167 on a descending
// spectrum s (len r): chi_new = min(chi, #{s/s0 > cutoff}); f[i] = 1/sqrt(s_i/s_0)
// for i < chi_new else 0 (i < cap).
void truncation_factors(Ctx& c, const double* s, int64_t r, int64_t chi, double cutoff,
                        double* f, int64_t cap, int64_t* chi_new);
// x[r, c] *= f[c] for a (rows x cols) block with leading dimension ld.
void scale_columns(Ctx& c, double* x, int64_t rows, int64_t cols, int64_t ld, const double* f);
// out (rows x chi_new) contiguous = in (rows x cap, ld cap) * f (per column;
// f == nullptr: no scaling), with chi_new read from device memory.
void scale_columns_compact(Ctx& c, const double* in, int64_t rows, int64_t cap,
                           const double* f, const int64_t* chi_new, double* out);

const char* g_last_error_cstr();

// One site's tensors in the reference layouts (acetn/ipeps/site_tensor.py:41-83).
struct Site {
  const ctm_site_f64* s;
  int64_t D, d;
  View A(int k) const { return bond_permute(s->A, D, d, k); }
  View C(int k) const {
    k = ((k % 4) + 4) % 4;
    return View(s->C[k], {s->c_rows[k], s->c_cols[k]});
  }
  View E(int k) const {
    k = ((k % 4) + 4) % 4;
    return View(s->E[k], {s->e_rows[k], s->e_cols[k], D, D});
  }
};

// Quarter-tensor matrix shape of direction k: rows (c, r, R), cols (e, d, D).
void quarter_dims(const Site& S, int k, int64_t& rows, int64_t& cols, int64_t sh[6]);
// make_quarter_tensor in FP64 (acetn/renormalization/projectors.py:35-60).
void quarter_tensor(Ctx& c, const Site& S, int k, double* Q, int64_t qshape[6]);
// make_quarter_tensor on tensor cores (3xBF16), returned as FP64 hi + lo.
void quarter_tensor_mixed_f64(Ctx& c, const Site& S, int k, double* Q);
// renormalize_ej on tensor cores (3xBF16), FP64 output normalised in FP64.
void renormalize_ej_mixed(Ctx& c, const Site& S, int k, const double* P2i, int64_t Y,
                          const double* P1j, int64_t X, double* Eout);
// Form of the site-tensor steps of the mixed path (0 automatic, 1 double
// layer, 2 one layer); returns the previous setting.
int set_contraction_form(int form);
// RDM.build_bond_rdm on tensor cores (3xBF16 contractions, FP64 halves and
// final contraction).
void bond_rdm_mixed(Ctx& c, const Site& S1, const Site& S2, int k, double* out);
// Half-system rSVD projectors with tensor-core arithmetic (CTM_PREC_MIXED).
void calculate_projectors_mixed(Ctx& c, const Site* S[4], int k, const ctm_ctmrg_opts& o,
                                const double* omega, double* P1, double* P2, int64_t* chi_new);

// Device-side failure flags (bit set by kernels: 1 = factorization failed,
// 2 = iteration limit reached); read and cleared by ctm_device_status().
int* status_flags(Ctx& c);
// Device counter of Cholesky-QR results rejected by the orthogonality check
// (the Householder fallback ran), read by ctm_qr_fallbacks().
unsigned long long* qr_fallback_counter();

}  // namespace ctm
