// FP64 tensor-contraction engine: a strided GETT kernel (no permute copies)
// behind a two-operand einsum planner, plus deterministic reductions and
// elementwise helpers.
//
// Every einsum of the reference's CTMRG path (acetn/renormalization/*.py,
// acetn/measurement/rdm.py) is a two-operand contraction; the planner sorts
// its labels into batch / row (M) / column (N) / contracted (K) groups,
// merges modes that are adjacent in every operand, and launches one kernel
// whose tile loaders decode multi-mode indices into strided addresses.
#include "engine.cuh"

#include <algorithm>
#include <map>

namespace ctm {

namespace {

constexpr int kMaxModes = 4;

struct Mode {
  int64_t ext;
  int64_t s0;  // stride in the first operand of the pair
  int64_t s1;  // stride in the second operand of the pair
};

struct Group {
  int n;
  Mode m[kMaxModes];
};

template <class T>
struct GettArgs {
  const T* A;
  const T* B;
  T* C;
  Group M, N, K;  // M: (A, C) strides, N: (B, C), K: (A, B)
  int64_t Mt, Nt, Kt;
  int64_t bext, bsa, bsb, bsc;
  T alpha, beta;
  int splitk;
  int64_t kchunk;
  T* part;
  int kfa, kfb;  // tile loaders walk K fastest (K is the unit-stride mode of A / B)
  int swap_xy;   // grid x runs over column tiles (more than 65535 of them)
};

// Group index -> the two operands' offsets.  Decoded in 32-bit arithmetic
// (every group's extent is below 2^31, checked on the host): a 64-bit
// division by a run-time divisor is a long software sequence, and the tile
// loaders decode 16 K indices per step.
__device__ __forceinline__ void decode(const Group& g, int64_t idx, int64_t& o0, int64_t& o1) {
  o0 = 0;
  o1 = 0;
  uint32_t rem = uint32_t(idx);
#pragma unroll
  for (int j = kMaxModes - 1; j >= 0; --j) {
    if (j < g.n) {
      const uint32_t e = uint32_t(g.m[j].ext);
      const uint32_t q = rem / e;
      const int64_t r = int64_t(rem - q * e);
      rem = q;
      o0 += r * g.m[j].s0;
      o1 += r * g.m[j].s1;
    }
  }
}

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

// One 64x64 output tile per CTA, 4x4 outputs per thread, K staged through
// shared memory 16 at a time with a register prefetch of the next step (its
// global loads are in flight while the current step computes).  Each tile
// loader walks whichever of its two index groups has unit stride, so warps
// read contiguous memory for either operand orientation.
template <class T>
__global__ void __launch_bounds__(NT) gett_kernel(const GettArgs<T> p) {
  __shared__ int64_t sAm[BM], sCm[BM], sBn[BN], sCn[BN];
  __shared__ int64_t sAk[2][BK], sBk[2][BK];
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  constexpr int E = (BM * BK) / NT;

  const int tid = threadIdx.x;
  const int64_t m0 = static_cast<int64_t>(p.swap_xy ? blockIdx.y : blockIdx.x) * BM;
  const int64_t n0 = static_cast<int64_t>(p.swap_xy ? blockIdx.x : blockIdx.y) * BN;
  const int64_t z = blockIdx.z;
  const int64_t batch = z % p.bext;
  const int64_t split = z / p.bext;
  const T* A = p.A + batch * p.bsa;
  const T* B = p.B + batch * p.bsb;

  if (tid < BM) {
    const int64_t m = m0 + tid;
    if (m < p.Mt) decode(p.M, m, sAm[tid], sCm[tid]);
    else { sAm[tid] = -1; sCm[tid] = -1; }
  } else if (tid < BM + BN) {
    const int t = tid - BM;
    const int64_t n = n0 + t;
    if (n < p.Nt) decode(p.N, n, sBn[t], sCn[t]);
    else { sBn[t] = -1; sCn[t] = -1; }
  }
  const int64_t kb = split * p.kchunk;
  const int64_t ke = min(kb + p.kchunk, p.Kt);
  const int nsteps = ke > kb ? int((ke - kb + BK - 1) / BK) : 0;
  auto decode_k = [&](int step, int buf) {
    if (tid < BK) {
      const int64_t k = kb + int64_t(step) * BK + tid;
      if (step < nsteps && k < ke) decode(p.K, k, sAk[buf][tid], sBk[buf][tid]);
      else { sAk[buf][tid] = -1; sBk[buf][tid] = -1; }
    }
  };
  // element e of this thread: (row, k) of the A tile and (column, k) of the B tile
  auto a_idx = [&](int e, int& mm, int& kk) {
    const int lin = tid + e * NT;
    if (p.kfa) { mm = lin / BK; kk = lin % BK; } else { mm = lin % BM; kk = lin / BM; }
  };
  auto b_idx = [&](int e, int& nn, int& kk) {
    const int lin = tid + e * NT;
    if (p.kfb) { nn = lin / BK; kk = lin % BK; } else { nn = lin % BN; kk = lin / BN; }
  };
  T ra[E], rb[E];
  auto load = [&](int buf) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
      int mm, kk;
      a_idx(e, mm, kk);
      const int64_t am = sAm[mm], ak = sAk[buf][kk];
      ra[e] = (am >= 0 && ak >= 0) ? A[am + ak] : T(0);
      int nn, kb2;
      b_idx(e, nn, kb2);
      const int64_t bn = sBn[nn], bk = sBk[buf][kb2];
      rb[e] = (bn >= 0 && bk >= 0) ? B[bk + bn] : T(0);
    }
  };

  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);

  const int tx = tid & 15, ty = tid >> 4;
  decode_k(0, 0);
  __syncthreads();
  if (nsteps > 0) load(0);
  decode_k(1, 1);
  for (int st = 0; st < nsteps; ++st) {
    __syncthreads();  // the previous step's reads of As/Bs are done
#pragma unroll
    for (int e = 0; e < E; ++e) {
      int mm, kk;
      a_idx(e, mm, kk);
      As[kk][mm] = ra[e];
      int nn, kb2;
      b_idx(e, nn, kb2);
      Bs[kb2][nn] = rb[e];
    }
    __syncthreads();
    if (st + 1 < nsteps) load((st + 1) & 1);
    decode_k(st + 2, st & 1);  // buffer st & 1 was last read by load(st)
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
  }

#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int mi = ty + 16 * i;
    const int64_t m = m0 + mi;
    if (m >= p.Mt) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int nj = tx + 16 * j;
      const int64_t n = n0 + nj;
      if (n >= p.Nt) continue;
      if (p.splitk > 1) {
        p.part[((split * p.bext + batch) * p.Mt + m) * p.Nt + n] = acc[i][j];
      } else {
        T* c = p.C + batch * p.bsc + sCm[mi] + sCn[nj];
        const T v = p.alpha * acc[i][j];
        *c = (p.beta != T(0)) ? fma(p.beta, *c, v) : v;
      }
    }
  }
}

// Contractions with few outputs and a long K (the last steps of the RDMs:
// 4 x 4 outputs over chi^2 D^2 terms) would use one 64 x 64 tile of the GETT
// kernel for a handful of outputs.  Here every CTA takes one K chunk for all
// Mt x Nt <= 256 outputs (one per thread; Mt + Nt <= 128), staging KS K
// indices of both operands in shared memory per step (128 when the operands
// have at most 32 rows together, so that each thread has several loads in
// flight), and writes its partial sums for gett_small_reduce.
template <class T, int KS>
__global__ void __launch_bounds__(256) gett_small_kernel(const GettArgs<T> p) {
  __shared__ int64_t sAm[128], sBn[128], sAk[KS], sBk[KS];
  extern __shared__ __align__(16) unsigned char small_smem[];
  const int64_t Mt = p.Mt, Nt = p.Nt;
  T (*As)[KS + 1] = reinterpret_cast<T (*)[KS + 1]>(small_smem);
  T (*Bs)[KS + 1] = reinterpret_cast<T (*)[KS + 1]>(small_smem) + Mt;
  const int tid = threadIdx.x;
  for (int i = tid; i < Mt; i += blockDim.x) {
    int64_t a, c;
    decode(p.M, i, a, c);
    sAm[i] = a;
  }
  for (int i = tid; i < Nt; i += blockDim.x) {
    int64_t b, c;
    decode(p.N, i, b, c);
    sBn[i] = b;
  }
  const int64_t k0 = int64_t(blockIdx.x) * p.kchunk;
  const int64_t k1 = min(k0 + p.kchunk, p.Kt);
  const int m = tid / int(Nt), n = tid % int(Nt);
  const bool owner = tid < Mt * Nt;
  T acc = T(0);
  for (int64_t kb = k0; kb < k1; kb += KS) {
    __syncthreads();
    if (tid < KS) {
      int64_t a = 0, b = 0;
      if (kb + tid < k1) decode(p.K, kb + tid, a, b);
      sAk[tid] = a;
      sBk[tid] = b;
    }
    __syncthreads();
#pragma unroll 4
    for (int e = tid; e < Mt * KS; e += blockDim.x) {
      const int i = e / KS, kk = e % KS;
      As[i][kk] = (kb + kk < k1) ? p.A[sAm[i] + sAk[kk]] : T(0);
    }
#pragma unroll 4
    for (int e = tid; e < Nt * KS; e += blockDim.x) {
      const int j = e / KS, kk = e % KS;
      Bs[j][kk] = (kb + kk < k1) ? p.B[sBn[j] + sBk[kk]] : T(0);
    }
    __syncthreads();
    if (owner) {
#pragma unroll 8
      for (int kk = 0; kk < KS; ++kk) acc = fma(As[m][kk], Bs[n][kk], acc);
    }
  }
  if (owner) p.part[(int64_t(blockIdx.x) * Mt + m) * Nt + n] = acc;
}

// Sums the many partial sums of gett_small_kernel: one CTA per output, each
// thread a strided subset of the splits, then a fixed-order tree in shared
// memory (deterministic; a thread per output looping over ~1000 splits was
// latency-bound at ~100 us).
template <class T>
__global__ void __launch_bounds__(256) gett_small_reduce(const GettArgs<T> p) {
  __shared__ T red[256];
  const int64_t out = blockIdx.x;
  const int64_t outs = p.Mt * p.Nt;
  T s = T(0);
  for (int t = threadIdx.x; t < p.splitk; t += blockDim.x) s += p.part[t * outs + out];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    int64_t am, cm, bn, cn;
    decode(p.M, out / p.Nt, am, cm);
    decode(p.N, out % p.Nt, bn, cn);
    T* c = p.C + cm + cn;
    const T v = p.alpha * red[0];
    *c = (p.beta != T(0)) ? fma(p.beta, *c, v) : v;
  }
}

// Sums split-K partial tiles in a fixed order (deterministic) into C.
template <class T>
__global__ void gett_splitk_reduce(const GettArgs<T> p) {
  const int64_t total = p.bext * p.Mt * p.Nt;
  for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t n = idx % p.Nt;
    const int64_t m = (idx / p.Nt) % p.Mt;
    const int64_t b = idx / (p.Nt * p.Mt);
    // two interleaved partial sums in a fixed order: two loads in flight
    T s0 = T(0), s1 = T(0);
    const int64_t stride = p.bext * p.Mt * p.Nt;
    const T* pt = p.part + (b * p.Mt + m) * p.Nt + n;
    int t = 0;
    for (; t + 1 < p.splitk; t += 2) {
      s0 += pt[t * stride];
      s1 += pt[(t + 1) * stride];
    }
    if (t < p.splitk) s0 += pt[t * stride];
    const T s = s0 + s1;
    int64_t am, cm, bn, cn;
    decode(p.M, m, am, cm);
    decode(p.N, n, bn, cn);
    T* c = p.C + b * p.bsc + cm + cn;
    const T v = p.alpha * s;
    *c = (p.beta != T(0)) ? fma(p.beta, *c, v) : v;
  }
}

struct Label {
  char ch;
  int64_t ext;
  int64_t sa, sb, sc;  // 0 when absent
  bool ia, ib, ic;
};

// Merges modes (already ordered outer -> inner) that are contiguous in both
// operands; drops unit extents.
void merge(std::vector<Mode>& v) {
  std::vector<Mode> out;
  for (const Mode& md : v) {
    if (md.ext == 1) continue;
    if (!out.empty()) {
      Mode& o = out.back();
      if (o.s0 == md.ext * md.s0 && o.s1 == md.ext * md.s1) {
        o.ext *= md.ext;
        o.s0 = md.s0;
        o.s1 = md.s1;
        continue;
      }
    }
    out.push_back(md);
  }
  v.swap(out);
}

Group to_group(std::vector<Mode> v, const char* what) {
  merge(v);
  CTM_REQUIRE(v.size() <= size_t(kMaxModes), CTM_ERR_UNSUPPORTED,
              std::string("einsum: too many ") + what + " modes after merging");
  Group g{};
  g.n = static_cast<int>(v.size());
  for (size_t i = 0; i < v.size(); ++i) g.m[i] = v[i];
  return g;
}

int64_t group_size(const Group& g) {
  int64_t s = 1;
  for (int i = 0; i < g.n; ++i) s *= g.m[i].ext;
  return s;
}

}  // namespace

template <class T>
void einsum_impl(Ctx& c, const char* spec, const ViewT<T>& A, const ViewT<T>& B, const ViewT<T>& C,
                 double alpha, double beta) {
  std::string s(spec);
  const size_t comma = s.find(','), arrow = s.find("->");
  CTM_REQUIRE(comma != std::string::npos && arrow != std::string::npos, CTM_ERR_INVALID,
              "einsum: bad spec " + s);
  const std::string la = s.substr(0, comma), lb = s.substr(comma + 1, arrow - comma - 1),
                    lc = s.substr(arrow + 2);
  CTM_REQUIRE(int(la.size()) == A.nd && int(lb.size()) == B.nd && int(lc.size()) == C.nd,
              CTM_ERR_INVALID, "einsum: rank mismatch in " + s);
  std::map<char, Label> labels;
  auto add = [&](const std::string& l, const ViewT<T>& v, int which) {
    for (size_t i = 0; i < l.size(); ++i) {
      Label& L = labels[l[i]];
      if (L.ch == 0) {
        L.ch = l[i];
        L.ext = v.shape[i];
      }
      CTM_REQUIRE(L.ext == v.shape[i], CTM_ERR_INVALID,
                  std::string("einsum: extent mismatch for label ") + l[i] + " in " + s);
      if (which == 0) { L.ia = true; L.sa = v.stride[i]; }
      if (which == 1) { L.ib = true; L.sb = v.stride[i]; }
      if (which == 2) { L.ic = true; L.sc = v.stride[i]; }
    }
  };
  add(la, A, 0);
  add(lb, B, 1);
  add(lc, C, 2);

  std::vector<Label> bl, ml, nl, kl;
  for (auto& kv : labels) {
    const Label& L = kv.second;
    if (L.ia && L.ib && L.ic) bl.push_back(L);
    else if (L.ia && L.ic && !L.ib) ml.push_back(L);
    else if (L.ib && L.ic && !L.ia) nl.push_back(L);
    else if (L.ia && L.ib && !L.ic) kl.push_back(L);
    else
      CTM_REQUIRE(L.ext == 1, CTM_ERR_UNSUPPORTED,
                  std::string("einsum: unsupported label pattern for ") + L.ch + " in " + s);
  }
  auto by = [](int64_t Label::*key) {
    return [key](const Label& x, const Label& y) { return x.*key > y.*key; };
  };
  std::sort(ml.begin(), ml.end(), by(&Label::sc));
  std::sort(nl.begin(), nl.end(), by(&Label::sc));
  std::sort(kl.begin(), kl.end(), by(&Label::sa));
  std::sort(bl.begin(), bl.end(), by(&Label::sc));

  std::vector<Mode> mm, nn, kk, bb;
  for (auto& L : ml) mm.push_back({L.ext, L.sa, L.sc});
  for (auto& L : nl) nn.push_back({L.ext, L.sb, L.sc});
  for (auto& L : kl) kk.push_back({L.ext, L.sa, L.sb});
  GettArgs<T> p{};
  p.M = to_group(mm, "row");
  p.N = to_group(nn, "column");
  p.K = to_group(kk, "contracted");
  // batch: at most one mode after merging (all three strides must merge)
  int64_t bext = 1, bsa = 0, bsb = 0, bsc = 0;
  {
    std::vector<Label> bv;
    for (auto& L : bl)
      if (L.ext != 1) bv.push_back(L);
    for (size_t i = 0; i < bv.size(); ++i) {
      if (i == 0) {
        bext = bv[0].ext; bsa = bv[0].sa; bsb = bv[0].sb; bsc = bv[0].sc;
      } else {
        const Label& L = bv[i];
        CTM_REQUIRE(bsa == L.ext * L.sa && bsb == L.ext * L.sb && bsc == L.ext * L.sc,
                    CTM_ERR_UNSUPPORTED, "einsum: non-mergeable batch modes in " + s);
        bext *= L.ext; bsa = L.sa; bsb = L.sb; bsc = L.sc;
      }
    }
  }
  p.A = A.p;
  p.B = B.p;
  p.C = C.p;
  p.Mt = group_size(p.M);
  p.Nt = group_size(p.N);
  p.Kt = group_size(p.K);
  CTM_REQUIRE(p.Mt < (int64_t(1) << 31) && p.Nt < (int64_t(1) << 31) &&
                  p.Kt < (int64_t(1) << 31),
              CTM_ERR_UNSUPPORTED, "einsum: index groups must have fewer than 2^31 entries");
  p.bext = bext; p.bsa = bsa; p.bsb = bsb; p.bsc = bsc;
  p.alpha = T(alpha);
  p.beta = T(beta);
  if (p.Mt == 0 || p.Nt == 0) return;
  // loaders walk K fastest when K, not the row / column group, is unit-stride
  p.kfa = (p.K.n > 0 && p.K.m[p.K.n - 1].s0 == 1 &&
           !(p.M.n > 0 && p.M.m[p.M.n - 1].s0 == 1)) ? 1 : 0;
  p.kfb = (p.K.n > 0 && p.K.m[p.K.n - 1].s1 == 1 &&
           !(p.N.n > 0 && p.N.m[p.N.n - 1].s0 == 1)) ? 1 : 0;

  if (bext == 1 && p.Mt * p.Nt <= 256 && p.Mt + p.Nt <= 128 && p.Kt >= 8192) {
    // few outputs, long K: one K chunk per CTA for all outputs
    int splits = static_cast<int>(std::min<int64_t>(1024, (p.Kt + 511) / 512));
    const int ks = (p.Mt + p.Nt <= 32) ? 128 : 32;
    p.kchunk = ((p.Kt + splits - 1) / splits + ks - 1) / ks * ks;
    splits = static_cast<int>((p.Kt + p.kchunk - 1) / p.kchunk);
    p.splitk = splits;
    Scope scope(c);
    p.part = c.alloc<T>(size_t(splits) * p.Mt * p.Nt);
    if (c.sizing()) return;
    {
      const double flops = 2.0 * double(p.Mt) * p.Nt * p.Kt;
      KernelTimer timer(c.stream, sizeof(T) == 8 ? kTagGettF64 : kTagGettF32, flops);
      KernelTimer kt(c.stream, sizeof(T) == 8 ? "gett_small_kernel<double>"
                                             : "gett_small_kernel<float>", kUnitFlop, flops);
      const size_t smem = size_t(p.Mt + p.Nt) * (ks + 1) * sizeof(T);
      if (ks == 128) gett_small_kernel<T, 128><<<splits, 256, smem, c.stream>>>(p);
      else gett_small_kernel<T, 32><<<splits, 256, smem, c.stream>>>(p);
      CTM_LAUNCH_CHECK();
    }
    KernelTimer kt(c.stream, "gett_small_reduce", kUnitByte,
                   double(sizeof(T)) * (splits + 1.0) * p.Mt * p.Nt);
    gett_small_reduce<T><<<unsigned(p.Mt * p.Nt), 256, 0, c.stream>>>(p);
    CTM_LAUNCH_CHECK();
    return;
  }
  const int64_t tiles = ((p.Mt + BM - 1) / BM) * ((p.Nt + BN - 1) / BN) * bext;
  int splitk = 1;
  // split K until the grid holds about one CTA per SM: two per SM measured
  // slower in the concurrent move (the CTAs of other rows' kernels share the
  // SMs; the split-K partials double), far fewer lengthens the row
  const int64_t target = sm_count_linalg();
  if (tiles < target && p.Kt >= 2 * BK) {
    splitk = static_cast<int>(std::min<int64_t>((target + tiles - 1) / tiles, p.Kt / BK));
    splitk = std::max(splitk, 1);
  }
  p.kchunk = ((p.Kt + splitk - 1) / splitk + BK - 1) / BK * BK;
  if (p.Kt == 0) p.kchunk = BK;
  splitk = static_cast<int>(std::max<int64_t>(1, (p.Kt + p.kchunk - 1) / p.kchunk));
  p.splitk = splitk;
  Scope scope(c);
  if (splitk > 1) p.part = c.alloc<T>(size_t(splitk) * bext * p.Mt * p.Nt);
  if (c.sizing()) return;
  const int64_t mtiles = (p.Mt + BM - 1) / BM, ntiles = (p.Nt + BN - 1) / BN;
  p.swap_xy = ntiles > 65535 ? 1 : 0;
  dim3 grid(static_cast<unsigned>(p.swap_xy ? ntiles : mtiles),
            static_cast<unsigned>(p.swap_xy ? mtiles : ntiles), static_cast<unsigned>(bext * splitk));
  CTM_REQUIRE(grid.y <= 65535 && grid.z <= 65535 && grid.x <= 0x7fffffffLL, CTM_ERR_UNSUPPORTED,
              "einsum: grid too large");
  {
    const double flops = 2.0 * double(p.Mt) * p.Nt * p.Kt * bext;
    KernelTimer timer(c.stream, sizeof(T) == 8 ? kTagGettF64 : kTagGettF32, flops);
    KernelTimer kt(c.stream, sizeof(T) == 8 ? "gett_kernel<double>" : "gett_kernel<float>",
                   kUnitFlop, flops);
    gett_kernel<T><<<grid, NT, 0, c.stream>>>(p);
    CTM_LAUNCH_CHECK();
  }
  if (splitk > 1) {
    KernelTimer kt(c.stream, "gett_splitk_reduce", kUnitByte,
                   double(sizeof(T)) * (splitk + 1.0) * bext * p.Mt * p.Nt);
    gett_splitk_reduce<T><<<grid_for(bext * p.Mt * p.Nt, 256), 256, 0, c.stream>>>(p);
    CTM_LAUNCH_CHECK();
  }
}

void einsum(Ctx& c, const char* spec, const View& A, const View& B, const View& C, double alpha,
            double beta) {
  einsum_impl<double>(c, spec, A, B, C, alpha, beta);
}

void einsum(Ctx& c, const char* spec, const ViewF& A, const ViewF& B, const ViewF& C, double alpha,
            double beta) {
  einsum_impl<float>(c, spec, A, B, C, alpha, beta);
}

// ----------------------------------------------------------------- reductions
namespace {

constexpr int RT = 256;

__device__ __forceinline__ double combine(double a, double b, int op) {
  return op == 0 ? fmax(a, b) : a + b;
}

// Grid-stride partial reduction: op 0 = max |x|, op 1 = sum x^2.
__global__ void reduce_partial(const double* __restrict__ x, int64_t n, double* part, int op) {
  __shared__ double sh[RT];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * int64_t(RT) + threadIdx.x; i < n; i += int64_t(gridDim.x) * RT) {
    const double v = x[i];
    acc = op == 0 ? fmax(acc, fabs(v)) : fma(v, v, acc);
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = RT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = combine(sh[threadIdx.x], sh[threadIdx.x + s], op);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void reduce_final(const double* part, int nparts, double* out, int op) {
  __shared__ double sh[RT];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nparts; i += RT) acc = combine(acc, part[i], op);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = RT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = combine(sh[threadIdx.x], sh[threadIdx.x + s], op);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

void reduce(Ctx& c, const double* x, int64_t n, double* out, int op) {
  const int blocks = grid_for(n, RT, 152 * 4);
  Scope scope(c);
  double* part = c.alloc<double>(blocks);
  if (c.sizing()) return;
  {
    KernelTimer kt(c.stream, "reduce_partial", kUnitByte, 8.0 * n);
    reduce_partial<<<blocks, RT, 0, c.stream>>>(x, n, part, op);
    CTM_LAUNCH_CHECK();
  }
  reduce_final<<<1, RT, 0, c.stream>>>(part, blocks, out, op);
  CTM_LAUNCH_CHECK();
}

// x /= s (mode 0) or x /= sqrt(s) (mode 1), as a product with the
// reciprocal (within an ulp of the quotient; an FP64 division per entry is a
// long sequence on the FP64 units)
__global__ void divide_kernel(double* x, int64_t n, const double* scal, int mode) {
  const double r = 1.0 / (mode == 0 ? scal[0] : sqrt(scal[0]));
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    x[i] *= r;
}

__global__ void copy2d_kernel(const double* src, int64_t rows, int64_t cols, int64_t s0,
                              int64_t s1, double* dst, int64_t ld) {
  const int64_t total = rows * cols;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = i / cols, q = i % cols;
    dst[r * ld + q] = src[r * s0 + q * s1];
  }
}

__global__ void fill_kernel(double* x, int64_t n, double v) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    x[i] = v;
}

}  // namespace

void absmax(Ctx& c, const double* x, int64_t n, double* out) { reduce(c, x, n, out, 0); }
void sumsq(Ctx& c, const double* x, int64_t n, double* out) { reduce(c, x, n, out, 1); }

void divide_by(Ctx& c, double* x, int64_t n, const double* scal, int mode) {
  if (c.sizing() || n == 0) return;
  KernelTimer kt(c.stream, "divide_kernel", kUnitByte, 16.0 * n);
  divide_kernel<<<grid_for(n, 256), 256, 0, c.stream>>>(x, n, scal, mode);
  CTM_LAUNCH_CHECK();
}

void copy2d(Ctx& c, const View& src, double* dst, int64_t ld_dst) {
  CTM_REQUIRE(src.nd == 2, CTM_ERR_INVALID, "copy2d: expects a 2-D view");
  if (c.sizing() || src.numel() == 0) return;
  KernelTimer kt(c.stream, "copy2d_kernel", kUnitByte, 16.0 * src.numel());
  copy2d_kernel<<<grid_for(src.numel(), 256), 256, 0, c.stream>>>(
      src.p, src.shape[0], src.shape[1], src.stride[0], src.stride[1], dst, ld_dst);
  CTM_LAUNCH_CHECK();
}

namespace {
__global__ void cvt_f32_kernel(const double* x, float* y, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    y[i] = float(x[i]);
}
__global__ void cvt_f64_kernel(const float* x, double* y, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    y[i] = double(x[i]);
}
}  // namespace

void to_f32(Ctx& c, const double* x, float* y, int64_t n) {
  if (c.sizing() || n == 0) return;
  KernelTimer kt(c.stream, "cvt_f32_kernel", kUnitByte, 12.0 * n);
  cvt_f32_kernel<<<grid_for(n, 256), 256, 0, c.stream>>>(x, y, n);
  CTM_LAUNCH_CHECK();
}

void to_f64(Ctx& c, const float* x, double* y, int64_t n) {
  if (c.sizing() || n == 0) return;
  KernelTimer kt(c.stream, "cvt_f64_kernel", kUnitByte, 12.0 * n);
  cvt_f64_kernel<<<grid_for(n, 256), 256, 0, c.stream>>>(x, y, n);
  CTM_LAUNCH_CHECK();
}

void fill(Ctx& c, double* x, int64_t n, double v) {
  if (c.sizing() || n == 0) return;
  fill_kernel<<<grid_for(n, 256), 256, 0, c.stream>>>(x, n, v);
  CTM_LAUNCH_CHECK();
}

}  // namespace ctm
