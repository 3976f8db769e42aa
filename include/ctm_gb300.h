/*
 * ctm_gb300.h - C ABI of the GB300 (sm_103a) CTMRG library.
 *
 * Every entry point takes device pointers to contiguous row-major tensors in
 * the layouts of Ace-TN's torch tensors, plain integer sizes, a caller-owned
 * device workspace and a cudaStream_t.  The library allocates no device
 * memory besides a file-scope status word; all launches go to the given
 * stream and only ctm_device_status() synchronizes (that stream).
 *
 * Workspace protocol: call with ws == NULL and *ws_bytes ignored; the entry
 * point stores the bytes it needs in *ws_bytes and returns CTM_OK without
 * launching anything.  Call again with a buffer of at least that size
 * (256-byte aligned).
 *
 * Tensor layouts (reference: acetn/ipeps/site_tensor.py:41-83):
 *   A    (D, D, D, D, d)          legs (left, up, right, down, phys)
 *   C[k] (c_rows[k], c_cols[k])   k = 0 left, 1 up, 2 right, 3 down
 *   E[k] (e_rows[k], e_cols[k], D, D)
 *
 * Status codes are returned by every function; ctm_last_error() gives the
 * message of the last failure on the calling thread.
 */
#ifndef CTM_GB300_H
#define CTM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* ctm_stream_t; /* == cudaStream_t */

enum {
  CTM_OK = 0,
  CTM_ERR_INVALID = 1,      /* bad shape, size, pointer or option         */
  CTM_ERR_UNSUPPORTED = 2,  /* valid request this library does not handle  */
  CTM_ERR_WORKSPACE = 3,    /* workspace smaller than the queried size     */
  CTM_ERR_CUDA = 4,         /* a CUDA runtime call failed                  */
  CTM_ERR_NUMERIC = 5,      /* non-finite input or failed factorization    */
  CTM_ERR_TIMEOUT = 6       /* a bounded device-side wait expired          */
};

/* Arithmetic of a projector computation. */
enum {
  CTM_PREC_FP64 = 0,   /* every product in FP64: the drop-in path                     */
  CTM_PREC_MIXED = 1,  /* tensor cores: BF16 range finder, 3xBF16 enlarged corners,
                          Rayleigh-Ritz and projector products, FP32 Cholesky-QR and
                          one-sided Jacobi SVD of the Rayleigh-Ritz matrix; FP64
                          spectrum, truncation and s^-1/2 scaling (ctm_ctmrg_opts
                          .mixed_flags selects higher precision per stage); half-
                          and full-system (four-factor chain) projectors.  With
                          CTM_SVD_FULL: 3xBF16 quarter tensors and products, FP64
                          SVD and projector products                              */
  CTM_PREC_BF16 = 2    /* ctm_matmul only: one BF16 tensor-core pass, FP32 accumulation */
};

/* Stage precision of CTM_PREC_MIXED (bits of ctm_ctmrg_opts.mixed_flags). */
enum {
  CTM_MIXED_RF3 = 1,    /* range-finder products in 3xBF16 (default: one BF16 pass) */
  CTM_MIXED_SVD64 = 2,  /* SVD of the Rayleigh-Ritz matrix in FP64                  */
  CTM_MIXED_Q64 = 8,    /* quarter tensors contracted in FP64, then split to BF16   */
  CTM_MIXED_F32 = 16    /* FP64 quarter tensors, every product in FP32 SIMT         */
};

/* Projector construction (acetn/ipeps/ipeps_config.py:16-24 CTMRGConfig). */
enum { CTM_PROJ_HALF = 0, CTM_PROJ_FULL = 1 };
enum { CTM_SVD_RSVD = 0, CTM_SVD_FULL = 1 };

typedef struct ctm_site_f64 {
  const double* A;
  const double* C[4];
  const double* E[4];
  int64_t c_rows[4], c_cols[4];
  int64_t e_rows[4], e_cols[4];
} ctm_site_f64;

typedef struct ctm_ctmrg_opts {
  int64_t chi;          /* dims["chi"]                                  */
  int32_t projectors;   /* CTM_PROJ_HALF | CTM_PROJ_FULL                */
  int32_t svd_type;     /* CTM_SVD_RSVD | CTM_SVD_FULL                  */
  double svd_cutoff;    /* relative singular-value cutoff (1e-12)       */
  int32_t rsvd_niter;   /* power iterations (2)                         */
  int32_t rsvd_oversampling; /* q = chi + oversampling (2)              */
  int32_t precision;    /* CTM_PREC_FP64 | CTM_PREC_MIXED               */
  int32_t fixed_width;  /* 1: write P1/P2 with exactly chi_cap columns, zero
                           beyond the truncation count (shape-stable output
                           for CUDA-graph capture); chi_new still receives
                           the count.  0: compact chi_new columns        */
  double mixed_floor;   /* CTM_PREC_MIXED only: singular values below
                           mixed_floor * s_0 are dropped as well (they are
                           below the resolution of the 3xBF16 products);
                           never less than 1e-8                            */
  int32_t mixed_flags;  /* CTM_PREC_MIXED only: precision of its stages
                           (CTM_MIXED_* bits, 0 = the defaults)          */
} ctm_ctmrg_opts;

/* Library version string and message of the last failure on this thread. */
const char* ctm_version(void);
const char* ctm_last_error(void);

/* Form of the two site-tensor steps of CTM_PREC_MIXED (enlarged corners and
 * edge renormalization), for the whole process: 0 = automatic (one GEMM
 * against the double-layer site matrix, K = D^4, up to D = 6; the two
 * one-layer GEMMs of the reference's einsum order, K = D^2 and D^2 d, from
 * D = 8, where the double layer's D^8 entries would multiply the FLOPs by
 * D^2 / (2 d)), 1 = always the double layer, 2 = always one layer.
 * *previous (if not NULL) receives the former setting.  No counterpart in
 * the reference (its einsums are always one-layer). */
int ctm_set_mixed_contraction(int32_t form, int32_t* previous);

/* Tile-plan autotuner of the tensor-core GEMMs.  enable = 1 turns tuning on,
 * 0 off, -1 leaves it, -2 also forgets every tuned shape.  While it is on,
 * the first call outside stream capture of each new product shape (M, N, K,
 * passes, epilogue) times the candidate plans (N tiles of 256 or 128
 * columns, K split to fill the SMs or not) with CUDA events, which
 * synchronises that call's stream, and keeps the fastest for later calls,
 * captured ones included.  Results do not depend on the plan up to FP32
 * summation order inside a K split.  *entries (if not NULL) receives the
 * number of tuned shapes.  No counterpart in the reference. */
int ctm_autotune(int32_t enable, int32_t* entries);

/* Tuned shape i (0 <= i < entries): mnk[3] = M, N, K; mode_choice[2] =
 * passes (1 = BF16, 3 = 3xBF16) and the chosen candidate (bit 0: 128-wide
 * N tiles, bit 1: no K split); the chosen and the default plan's times. */
int ctm_autotune_entry(int32_t i, int64_t* mnk, int32_t* mode_choice, double* best_ms,
                       double* default_ms);

/* Synchronizes `stream`, stores and clears the device-side failure flags of
 * the current device: bit 0 = a factorization failed and its fallback ran,
 * bit 1 = an iteration limit or a bounded wait expired.  No counterpart in
 * the reference (its torch calls raise synchronously). */
int ctm_device_status(int* flags, ctm_stream_t stream);

/* Number of CUDA kernels this library has launched in the process (for
 * launch accounting in benchmarks).  No counterpart in the reference. */
unsigned long long ctm_kernel_launches(void);

/* Synchronizes `stream`, stores and clears the device counter of Cholesky-QR
 * factorizations whose orthogonality check failed so that the one-CTA
 * Householder QR ran instead (a performance diagnostic).  No counterpart in
 * the reference. */
int ctm_qr_fallbacks(unsigned long long* count, ctm_stream_t stream);

/* Live kernel timing for benchmarks.  Between ctm_profile_begin() and
 * ctm_profile_end() the main kernels are bracketed by CUDA events on their
 * stream; ctm_profile_end() waits for them and ctm_profile_query(tag, ...)
 * returns total milliseconds, algorithmic work (FLOPs) and launch count of a
 * kernel class: 0 = FP64 contraction (GETT), 1 = tensor-core GEMM; or of a
 * span of stream work: 2 = quarter tensors, 3 = rSVD range finder,
 * 4 = orthonormalization, 5 = Rayleigh-Ritz SVD, 6 = projector products,
 * 7 = boundary renormalization; 9 = the double-layer tensor-core GEMMs of the
 * mixed enlarged corner and edge renormalization (a subset of 1).  No counterpart in the
 * reference (its benchmarking decorators time whole Python calls). */
void ctm_profile_begin(void);
int ctm_profile_end(void);
int ctm_profile_query(int tag, double* total_ms, double* total_work, long long* launches);
/* Per-kernel table of the same profile: the number of kernel classes timed,
 * and class i's name, work unit (0 = algorithmic FLOP, 1 = algorithmic
 * bytes read + written), total milliseconds, total work and launch count.
 * The name stays valid until the next ctm_profile_begin().  No counterpart
 * in the reference. */
int ctm_profile_kernel_count(int* count);
int ctm_profile_kernel(int i, const char** name, int* unit, double* total_ms, double* total_work,
                       long long* launches);

/* Enlarged corner (quarter tensor) of one site in direction k, reshaped to a
 * (rows x cols) matrix, rows = (c, r, R), cols = (e, d, D), divided by its
 * largest |entry|.  qshape receives the six leg sizes.  CTM_PREC_MIXED
 * computes it on tensor cores in 3xBF16 and returns the FP64 sum hi + lo of
 * its split form.
 * Reference: ProjectorCalculator.make_quarter_tensor,
 * acetn/renormalization/projectors.py:35-60. */
int ctm_quarter_tensor(const ctm_site_f64* site, int64_t D, int64_t d, int32_t k,
                       double* Q, int64_t* qshape, int32_t precision,
                       void* ws, size_t* ws_bytes, ctm_stream_t stream);

/* Projector pair of one row/column of a directional move.
 * sites[0..3] = (s1, s2, s3, s4) as built by calculate_{left,up,right,down}_projectors
 * (acetn/renormalization/directional_mover.py:99-181).
 * omega: (n x q) N(0,1) matrix for the rSVD (ignored for CTM_SVD_FULL); n is
 * the column count of the last factor, q = min(chi + oversampling, m, n).
 * P1 receives (e, D, D, chi_new) and P2 (c, D, D, chi_new), both written
 * contiguously in the first rows*chi_new entries of buffers that must hold
 * rows*min(chi, q) (rSVD) or rows*min(chi, n) (full-rank) doubles.
 * chi_new (device int64) receives min(chi, #{s/s0 > cutoff}).
 * Reference: ProjectorCalculator.calculate_half_system / calculate_full_system,
 * acetn/renormalization/projectors.py:114-217. */
int ctm_calculate_projectors(const ctm_site_f64* const* sites, int64_t D, int64_t d,
                             int32_t k, const ctm_ctmrg_opts* opts, const double* omega,
                             double* P1, double* P2, int64_t* chi_new,
                             void* ws, size_t* ws_bytes, ctm_stream_t stream);

/* Number of rows of P1/P2 and the sketch width q of ctm_calculate_projectors
 * (host-side shape query, no device access). */
int ctm_projector_dims(const ctm_site_f64* const* sites, int64_t D, int32_t k,
                       const ctm_ctmrg_opts* opts, int64_t* p1_rows, int64_t* p2_rows,
                       int64_t* omega_rows, int64_t* q, int64_t* chi_cap);

/* Boundary renormalization of one row of a move: writes
 *   Cout1 = renormalize_cj1(C[(3+k)%4], E[(2+k)%4], P1_i)   (rows_a x chi_i)
 *   Cout2 = renormalize_cj2(C[k], E[k], P2_j)               (chi_j x cols)
 *   Eout  = renormalize_ej(E[(3+k)%4], A perm k, P2_i, P1_j) (chi_i, chi_j, D, D)
 * each divided by its Frobenius norm.  P*_x point to (rows, D, D, chi_x) tensors.
 * Reference: DirectionalMover.renormalize_boundary / renormalize_cj1 /
 * renormalize_cj2 / renormalize_ej, acetn/renormalization/directional_mover.py:273-366. */
int ctm_renormalize_boundary(const ctm_site_f64* s1, int64_t D, int64_t d, int32_t k,
                             const double* P1_i, int64_t chi_p1i,
                             const double* P2_j, int64_t chi_p2j,
                             const double* P2_i, int64_t chi_p2i,
                             const double* P1_j, int64_t chi_p1j,
                             double* Cout1, double* Cout2, double* Eout,
                             int32_t precision, void* ws, size_t* ws_bytes,
                             ctm_stream_t stream);

/* One directional move, or a left/right or up/down pair of moves (which
 * read and write disjoint tensors), of a whole nx x ny unit cell in one call:
 * the projector pairs of every row (column) of the move(s), then the boundary
 * renormalization of every row, all on `stream`.
 * sites: nx * ny sites, site (x, y) at index x * ny + y.  moves: nmoves
 * (direction k, index) pairs (k = 0 left, 1 up, 2 right, 3 down; index = the
 * column of a left/right move, the row of an up/down move).  Rows of a move:
 * ny for left/right, nx for up/down; row t (over all moves, in order) takes
 * omegas[t] (n x q, as ctm_calculate_projectors; ignored for CTM_SVD_FULL)
 * and writes chi_new[t] (device int64) and the three new tensors of its
 * renormalised site: out[3t] = C[(3+k)%4] (a x cap), out[3t+1] = C[k]
 * (cap x c), out[3t+2] = E[(3+k)%4] (cap x cap x D x D), all with the fixed
 * width cap = min(chi, q) (rSVD) or min(chi, n) (full rank) and zero beyond
 * the truncation count, so that every size is known before the call.  The
 * site tensors are only read; the caller puts the new ones in place.
 * Reference: DirectionalMover.left/up/right/down_move and
 * calculate_*_projectors / renormalize_boundary,
 * acetn/renormalization/directional_mover.py:23-181, 273-366 (the pair:
 * left_right_move_dist / up_down_move_dist, :183-271). */
int ctm_move_batched(const ctm_site_f64* sites, int32_t nx, int32_t ny, int64_t D, int64_t d,
                     const int32_t* moves, int32_t nmoves, const ctm_ctmrg_opts* opts,
                     const double* const* omegas, double* const* out, int64_t* chi_new,
                     void* ws, size_t* ws_bytes, ctm_stream_t stream);

/* Site reduced density matrix (d x d), not trace-normalised.  precision:
 * CTM_PREC_FP64, or CTM_PREC_MIXED (the same contraction chain in FP32 FMAs
 * with FP32 accumulation; FP64 result).
 * Reference: RDM.build_site_rdm, acetn/measurement/rdm.py:35-67. */
int ctm_site_rdm(const ctm_site_f64* site, int64_t D, int64_t d, int32_t precision,
                 double* rdm, void* ws, size_t* ws_bytes, ctm_stream_t stream);

/* Bond reduced density matrix (d, d, d, d) of bond (s1, s2, k), not normalised.
 * precision: CTM_PREC_FP64, or CTM_PREC_MIXED (each half on tensor cores:
 * the boundary operand, a double layer of the site tensor with the physical
 * and the bond legs open, and the closing corner-edge product, 3xBF16 with
 * FP32 accumulation; FP64 halves and final contraction).
 * Reference: RDM.build_bond_rdm / build_bond_rdm_core(_blocked),
 * acetn/measurement/rdm.py:69-153. */
int ctm_bond_rdm(const ctm_site_f64* s1, const ctm_site_f64* s2, int64_t D, int64_t d,
                 int32_t k, int32_t precision, double* rdm, void* ws, size_t* ws_bytes,
                 ctm_stream_t stream);

/* Norm tensor of the full update for bond (s1, s2, k): the bond's environment
 * contracted with the reduced site tensors a1q (r, d, u, y) and a2q
 * (d, l, u, x), both (D, D, D, nD) contiguous, into n12 (nD, nD, nD, nD)
 * indexed [y][x][Y][X] (FP64).
 * Reference: build_norm_tensor / build_norm_tensor_core,
 * acetn/evolution/full_update.py:163-236. */
int ctm_norm_tensor(const ctm_site_f64* s1, const ctm_site_f64* s2, int64_t D, int64_t d,
                    int32_t k, const double* a1q, const double* a2q, int64_t nD, double* n12,
                    void* ws, size_t* ws_bytes, ctm_stream_t stream);

/* ALS solver of the full update for the reduced tensors a1r, a2r (nD, bD,
 * pD) of one bond, FP64 on the device: initial guess from the truncated SVD
 * of a12g[(y,p)][(x,q)], then up to niter alternating least-squares updates
 * of a1r and a2r; method 0 ("cholesky"): the symmetrised system shifted by
 * epsilon max|R| on the diagonal, Cholesky factor and two triangular solves
 * (Gaussian elimination with partial pivoting when a pivot is not positive;
 * needs nD bD <= 160 and pD <= 8); method 1 ("pinv"): the Hermitian
 * pseudo-inverse with relative cutoff epsilon.  Stops when the relative
 * change of the cost falls below tol after the second iteration.  n12 (nD^4,
 * [y][x][Y][X]) and a12g (nD^2 pD^2, [y][x][p][q]) contiguous device arrays;
 * *iterations (host, may be NULL) receives the iterations run.  Reads the
 * cost to the host once per iteration (synchronises `stream`).
 * Reference: ALSSolver.solve / solve_torch / initialize_reduced_tensors /
 * solve_ar, acetn/evolution/als_solver.py:35-82, 120-147, 212-243. */
int ctm_als_solve(const double* n12, const double* a12g, int64_t nD, int64_t bD, int64_t pD,
                  int32_t niter, double tol, int32_t method, double epsilon, double* a1r,
                  double* a2r, int32_t* iterations, void* ws, size_t* ws_bytes,
                  ctm_stream_t stream);

/* <a12n|N|a12n> - 2 <a12n|N|a12g> with a12n = a1r . a2r, into *cost (device).
 * Reference: ALSSolver.calculate_cost, acetn/evolution/als_solver.py:253-262. */
int ctm_als_cost(const double* a1r, const double* a2r, const double* a12g, const double* n12,
                 int64_t nD, int64_t bD, int64_t pD, double* cost, void* ws, size_t* ws_bytes,
                 ctm_stream_t stream);

/* Randomized SVD of a (m x n), of a @ b (a: m x k, b: k x n), or of
 * a @ b @ c @ e (shapes chained); omega (n x q) supplied by the caller.
 * Writes U (m x q), S (q), V (n x q) with a @ ... ~= U diag(S) V^T.
 * Reference: acetn/linalg/svd_lowrank.py:4-44,
 * acetn/linalg/fused_matmul_svd_lowrank.py:4-52,
 * acetn/linalg/fused_3matmul_svd_lowrank.py:4-56. */
int ctm_svd_lowrank(const double* a, int64_t m, int64_t n, int64_t q, int32_t niter,
                    const double* omega, double* U, double* S, double* V,
                    void* ws, size_t* ws_bytes, ctm_stream_t stream);
int ctm_fused_matmul_svd_lowrank(const double* a, const double* b, int64_t m, int64_t k,
                                 int64_t n, int64_t q, int32_t niter, const double* omega,
                                 double* U, double* S, double* V, int32_t precision,
                                 void* ws, size_t* ws_bytes, ctm_stream_t stream);
int ctm_fused_3matmul_svd_lowrank(const double* a, const double* b, const double* c,
                                  const double* e, int64_t m, int64_t k1, int64_t k2,
                                  int64_t k3, int64_t n, int64_t q, int32_t niter,
                                  const double* omega, double* U, double* S, double* V,
                                  void* ws, size_t* ws_bytes, ctm_stream_t stream);

/* Thin QR of a tall matrix in place: Y (n x q, row-major, n >= q >= 1) is
 * overwritten by Q with orthonormal columns and, when R is not NULL, R
 * (q x q, upper triangular) is written with Y = Q R.  dtype CTM_DTYPE_F64
 * (double buffers) or CTM_DTYPE_F32 (float buffers; the arithmetic of the
 * mixed range finder).  Signs of Q's columns may differ from LAPACK's.
 * Reference: the torch.linalg.qr calls of the range finders,
 * acetn/linalg/svd_lowrank.py:36,39, fused_matmul_svd_lowrank.py:38,43,
 * fused_3matmul_svd_lowrank.py:40,43,47. */
#define CTM_DTYPE_F64 0
#define CTM_DTYPE_F32 1
int ctm_qr(void* Y, int64_t n, int64_t q, void* R, int32_t dtype, void* ws, size_t* ws_bytes,
           ctm_stream_t stream);

/* Thin SVD of an (m x n) FP64 matrix, m, n <= 4096: U (m x r), S (r), V (n x r),
 * r = min(m, n), singular values descending.  Used by svd_type "full-rank"
 * (acetn/renormalization/projectors.py:219-236). */
int ctm_svd_f64(const double* a, int64_t m, int64_t n, double* U, double* S, double* V,
                void* ws, size_t* ws_bytes, ctm_stream_t stream);

/* Thin SVD of the mixed path's Rayleigh-Ritz step: B = bt^T (q x n, given as
 * bt, n x q FP32 row-major, 1 <= q <= min(n, 1024)) = U diag(S) V^T with U
 * (q x q, FP64), S (q, descending, FP64), V (n x q, FP32).  FP32 shifted
 * Cholesky-QR3 of bt, then FP32 one-sided Jacobi with accumulated rotations
 * (on an 8-CTA cluster from q = 96).  Replaces the torch.linalg.svd of the
 * projected matrix in acetn/linalg/fused_matmul_svd_lowrank.py:45-51 on the
 * mixed path; no direct counterpart, exposed to test and measure that stage. */
int ctm_svd_f32(const float* bt, int64_t n, int64_t q, double* U, double* S, float* V,
                void* ws, size_t* ws_bytes, ctm_stream_t stream);

/* Matrix product C = A @ B of FP64 row-major matrices, with the library's
 * arithmetic: CTM_PREC_FP64 (FP64 FMAs), CTM_PREC_MIXED (3xBF16 split
 * products on tcgen05 tensor cores, FP32 accumulation) or CTM_PREC_BF16 (one
 * BF16 tensor-core pass).
 * No counterpart in the reference (torch.matmul); exposed to test and
 * measure the GEMM engines behind every entry point above. */
int ctm_matmul(const double* A, const double* B, double* C, int64_t M, int64_t N,
               int64_t K, int32_t precision, void* ws, size_t* ws_bytes,
               ctm_stream_t stream);

/* C = A @ B (FP64 in and out, 3xBF16 tensor-core arithmetic as ctm_matmul
 * with CTM_PREC_MIXED) for callers that cannot allocate device memory: a
 * host that hands a plugin only its input and output buffers, or a host
 * whose own memory pool has reserved the device, so that a cudaMalloc from
 * the plugin fails or fragments that pool.  No workspace:
 * the scratch (BF16 operand copies, split-K partial sums) lives in a 32 MiB
 * file-scope device array that every GPU loading the library keeps until the
 * process exits; products needing more scratch (about M = N = K > 1000)
 * return CTM_ERR_WORKSPACE.  The first call on a device looks up that
 * device's address of the array (cudaGetSymbolAddress): make it before any
 * stream capture.  All calls share the array and it keeps the last call's
 * contents, so calls that overlap on the GPU (different streams, or threads
 * without ordering) race; serialise them.  Allocates nothing: no cudaMalloc,
 * cudaFree or allocating library call.  No counterpart in the reference. */
int ctm_matmul_mixed_noalloc(const double* A, const double* B, double* C, int64_t M,
                             int64_t N, int64_t K, ctm_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* CTM_GB300_H */
