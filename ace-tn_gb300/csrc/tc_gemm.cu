// tcgen05 GEMM for sm_103a: TMA loads (128-byte swizzle) into a multi-stage
// shared-memory ring, one thread issuing tcgen05.mma into a TMEM accumulator
// (M = 128 rows per CTA, N up to 256 columns).  Without a K split the
// epilogue reads TMEM with tcgen05.ld and stores every destination directly
// (each thread owns one output row; groups of four consecutive columns that
// are contiguous in a destination go out as one vector store).  With a K
// split over the grid's z dimension the epilogue writes FP32 partial tiles
// that a second kernel reduces in a fixed order.
//
// Every mbarrier wait is bounded: on expiry the kernel records bit 2 in the
// status word, stops issuing work, waits (bounded) for its own outstanding
// copies and MMAs, frees its tensor memory and returns.
#include <cuda.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <tuple>

#include "engine.cuh"
#include "tc_gemm.cuh"

namespace ctm {

namespace {

constexpr int kBM = 128;         // rows of A per CTA (MMA M)
// K per stage: 64 BF16 (128-byte rows, 128-byte swizzle); the kernel and the
// tensor maps also take 32 (64-byte rows, 64-byte swizzle).
constexpr int kThreads = 256;    // 8 warps: in the epilogue warp w reads TMEM lanes
                                 // 32 (w % 4) .. +31 for half (w / 4) of the columns
constexpr uint32_t kTmemCols = 256;
constexpr int64_t kSpinLimit = 4LL * 1000 * 1000;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      " .reg .pred P1;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
      " selp.b32 %0, 1, 0, P1;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      " .reg .pred P1;\n"
      " mbarrier.test_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
      " selp.b32 %0, 1, 0, P1;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait of the single producer / MMA thread on a pipeline barrier:
// a non-blocking test in a tight loop (no suspension, so the thread resumes
// as soon as the phase flips); gives up after about 0.1 s.
__device__ __forceinline__ bool mbar_wait_spin(uint64_t* bar, uint32_t parity) {
  for (int64_t i = 0; i < 8 * kSpinLimit; ++i)
    if (mbar_test_wait(bar, parity)) return true;
  return false;
}

// Bounded wait on an mbarrier phase; false when the limit expired.  Polls
// without sleeping for the first few thousand tries (a pipeline stage turns
// over in about a microsecond), then backs off.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (int64_t i = 0; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i > 4096) __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand with rows of bk BF16
// (bk = 64: 128-byte swizzle; bk = 32: 64-byte swizzle), 8-row core-matrix
// groups 8 * 2 * bk bytes apart.
__device__ __forceinline__ uint64_t smem_desc(const void* p, int bk) {
  const uint64_t addr = smem_u32(p);
  uint64_t d = (addr >> 4) & 0x3FFFull;              // start address
  d |= uint64_t(1) << 16;                            // leading byte offset (unused when swizzled)
  d |= uint64_t((16 * bk) >> 4) << 32;               // stride byte offset
  d |= uint64_t(1) << 46;                            // descriptor version (tcgen05)
  d |= uint64_t(bk == 64 ? 2 : 4) << 61;             // SWIZZLE_128B / SWIZZLE_64B
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B,
// both K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Row / column offsets of a separable layout.  The indices are decoded in
// 32-bit arithmetic (M and N are below 2^31, checked at launch; a 64-bit
// division by a run-time divisor is a long software sequence, and the
// epilogue decodes a tile's 256 columns and 128 rows for every destination);
// the offsets themselves stay 64-bit.
__device__ __forceinline__ int64_t lay_row(const TcLayout& l, int64_t m) {
  int64_t o = 0;
  uint32_t r = uint32_t(m);
  for (int j = l.nm - 1; j >= 0; --j) {
    const uint32_t e = uint32_t(l.me[j]);
    const uint32_t q = r / e;
    o += int64_t(r - q * e) * l.ms[j];
    r = q;
  }
  return o;
}

__device__ __forceinline__ int64_t lay_col(const TcLayout& l, int64_t n) {
  int64_t o = 0;
  uint32_t r = uint32_t(n);
  for (int j = l.nn - 1; j >= 0; --j) {
    const uint32_t e = uint32_t(l.ne[j]);
    const uint32_t q = r / e;
    o += int64_t(r - q * e) * l.ns[j];
    r = q;
  }
  return o;
}

// One value / four consecutive values (destination offset a multiple of 4)
// of an FP32 accumulator tile, scaled by sc, in the destination's format.
// FP32 arithmetic throughout (FP64 units are scarce on this part); an FP64
// destination receives the FP32 product widened.
__device__ __forceinline__ void store1(const TcDest& d, int64_t off, float v, float sc) {
  const float x = v * sc;
  switch (d.kind) {
    case TcKind::kF64: static_cast<double*>(d.p)[off] = double(x); break;
    case TcKind::kF32: static_cast<float*>(d.p)[off] = x; break;
    case TcKind::kBf16Hi: static_cast<bf16*>(d.p)[off] = __float2bfloat16(x); break;
    case TcKind::kBf16Lo:
      static_cast<bf16*>(d.p)[off] = __float2bfloat16(x - __bfloat162float(__float2bfloat16(x)));
      break;
  }
}

__device__ __forceinline__ void store4(const TcDest& d, int64_t off, const float* v, float sc) {
  const float x0 = v[0] * sc, x1 = v[1] * sc, x2 = v[2] * sc, x3 = v[3] * sc;
  switch (d.kind) {
    case TcKind::kF64: {
      double2* q = reinterpret_cast<double2*>(static_cast<double*>(d.p) + off);
      q[0] = make_double2(double(x0), double(x1));
      q[1] = make_double2(double(x2), double(x3));
      break;
    }
    case TcKind::kF32:
      *reinterpret_cast<float4*>(static_cast<float*>(d.p) + off) = make_float4(x0, x1, x2, x3);
      break;
    case TcKind::kBf16Hi:
    case TcKind::kBf16Lo: {
      float y[4] = {x0, x1, x2, x3};
      if (d.kind == TcKind::kBf16Lo) {
#pragma unroll
        for (int i = 0; i < 4; ++i) y[i] -= __bfloat162float(__float2bfloat16(y[i]));
      }
      const __nv_bfloat162 o0 = __halves2bfloat162(__float2bfloat16(y[0]), __float2bfloat16(y[1]));
      const __nv_bfloat162 o1 = __halves2bfloat162(__float2bfloat16(y[2]), __float2bfloat16(y[3]));
      *reinterpret_cast<uint2*>(static_cast<bf16*>(d.p) + off) =
          make_uint2(*reinterpret_cast<const uint32_t*>(&o0), *reinterpret_cast<const uint32_t*>(&o1));
      break;
    }
  }
}

struct GemmParams {
  int m_tiles, n_tiles, tiles;  // persistent kernel: the tile grid
  int ntile;         // MMA N (multiple of 16, <= 256)
  int bk;            // K per stage (64 or 32)
  int kb_total;      // 64-wide K blocks
  int kb_per_split;
  int stages;
  int mode;          // 1 or 3
  float* part;       // [split][m_pad][n_pad] (unfused epilogue)
  int m_pad, n_pad;
  int* status;
  // direct epilogue (single K split): the tile goes straight to the destinations
  int direct;
  int n_fast;        // grid x runs over N tiles (CTAs sharing an A tile run together)
  int nd;
  double alpha;
  const double* scale1;  // outputs divided by *scale1 and *scale2 when non-null
  const double* scale2;
  unsigned long long* absmax;  // max |output| accumulated as ordered bits when non-null
  int64_t M, N;
  int staged;        // persistent epilogue through shared memory (BF16 destinations, nd <= 2)
  TcDest d[4];
};

__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tAl,
                   const __grid_constant__ CUtensorMap tB, const __grid_constant__ CUtensorMap tBl,
                   const GemmParams p) {
  extern __shared__ uint8_t dyn_smem[];
  uint8_t* base = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(dyn_smem) + 1023) & ~uintptr_t(1023));
  const int bk = p.bk;
  const uint32_t a_bytes = kBM * bk * 2;
  const uint32_t b_bytes = uint32_t(p.ntile) * bk * 2;
  const uint32_t half_bytes = a_bytes + b_bytes;
  const uint32_t stage_bytes = half_bytes * (p.mode == 3 ? 2 : 1);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + size_t(p.stages) * stage_bytes);
  uint64_t* empty = full + p.stages;
  uint64_t* tfull = empty + p.stages;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(tfull + 1);
  __shared__ int s_fail;
  __shared__ int64_t s_co[4][256];

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int s = 0; s < p.stages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(tfull, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_holder)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_holder;

  const int kb0 = blockIdx.z * p.kb_per_split;
  const int kb1 = min(kb0 + p.kb_per_split, p.kb_total);
  const int nkb = kb1 - kb0;
  const int m0 = (p.n_fast ? blockIdx.y : blockIdx.x) * kBM;
  const int n0 = (p.n_fast ? blockIdx.x : blockIdx.y) * p.ntile;
  int issued_loads = 0;  // producer: stages handed to TMA

  // Lane 0 of warp 0 produces and lane 0 of warp 1 issues the MMAs; the other
  // lanes of those two warps wait at __syncwarp for their lane 0 (spinning on
  // the epilogue's barrier next to it, they held up the pipeline thread of
  // their own warp) and then join the epilogue.
  if (warp == 0) {
    if (lane == 0) {
      // ---------------- TMA producer
      for (int i = 0; i < nkb; ++i) {
        const int s = i % p.stages;
        const uint32_t ph = (i / p.stages) & 1;
        if (!mbar_wait_spin(&empty[s], ph ^ 1)) {
          atomicOr(&s_fail, 1);
          break;
        }
        uint8_t* st = base + size_t(s) * stage_bytes;
        mbar_expect_tx(&full[s], stage_bytes);
        const int x = (kb0 + i) * bk;
        tma_load_2d(st, &tA, x, m0, &full[s]);
        tma_load_2d(st + a_bytes, &tB, x, n0, &full[s]);
        if (p.mode == 3) {
          tma_load_2d(st + half_bytes, &tAl, x, m0, &full[s]);
          tma_load_2d(st + half_bytes + a_bytes, &tBl, x, n0, &full[s]);
        }
        issued_loads = i + 1;
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer
      const uint32_t idesc = idesc_bf16(kBM, p.ntile);
      for (int i = 0; i < nkb; ++i) {
        const int s = i % p.stages;
        const uint32_t ph = (i / p.stages) & 1;
        if (!mbar_wait_spin(&full[s], ph)) {
          atomicOr(&s_fail, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        uint8_t* st = base + size_t(s) * stage_bytes;
#pragma unroll
        for (int kk = 0; kk < bk / 16; ++kk) {
          const uint64_t ah = smem_desc(st + kk * 32, bk);
          const uint64_t bh = smem_desc(st + a_bytes + kk * 32, bk);
          mma_bf16(tmem, ah, bh, idesc, (i > 0 || kk > 0) ? 1u : 0u);
          if (p.mode == 3) {
            const uint64_t al = smem_desc(st + half_bytes + kk * 32, bk);
            const uint64_t bl = smem_desc(st + half_bytes + a_bytes + kk * 32, bk);
            mma_bf16(tmem, ah, bl, idesc, 1u);
            mma_bf16(tmem, al, bh, idesc, 1u);
          }
        }
        mma_commit(&empty[s]);
      }
      mma_commit(tfull);
    }
    __syncwarp();
  }

  // ---------------- epilogue: TMEM -> FP32 partial tile
  bool ok = mbar_wait(tfull, 0);
  if (!ok) atomicOr(&s_fail, 1);
  __syncwarp();
  // tcgen05.ld is warp-collective: decide per warp, never per lane
  ok = __all_sync(0xffffffffu, ok);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const int lane_base = (warp & 3) * 32;
  const int row = m0 + lane_base + lane;
  const uint32_t trow = uint32_t(lane_base) << 16;
  // column slice of this warp: [c_begin, c_end), 16-aligned
  constexpr int kSlices = kThreads / 128;
  const int slice_w = ((p.ntile + kSlices - 1) / kSlices + 15) / 16 * 16;
  const int c_begin = min(p.ntile, (warp >> 2) * slice_w);
  const int c_end = min(p.ntile, c_begin + slice_w);
  if (p.direct) {
    // column offsets of this tile in every destination (-1 beyond N)
    for (int k = 0; k < p.nd; ++k)
      for (int cc = threadIdx.x; cc < p.ntile; cc += kThreads) {
        const int64_t n = int64_t(n0) + cc;
        s_co[k][cc] = n < p.N ? lay_col(p.d[k].lay, n) : int64_t(-1);
      }
    __syncthreads();
    const bool mvalid = row < p.M;
    int64_t ro[4] = {0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k < p.nd && mvalid) ro[k] = lay_row(p.d[k].lay, row);
    double scd = p.alpha;
    if (p.scale1 != nullptr) scd /= p.scale1[0];
    if (p.scale2 != nullptr) scd /= p.scale2[0];
    const float sc = float(scd);
    float amax = 0.f;
    if (ok) {
      for (int c = c_begin; c < c_end; c += 16) {
        float v[16];
        __syncwarp();
        tmem_ld16(tmem + trow + uint32_t(c), v);
        if (mvalid) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (k >= p.nd) break;
            const TcDest& d = p.d[k];
#pragma unroll
            for (int g = 0; g < 4; ++g) {
              const int cb = c + 4 * g;
              const int64_t c0 = s_co[k][cb];
              const bool vec = c0 >= 0 && ((ro[k] + c0) & 3) == 0 && s_co[k][cb + 1] == c0 + 1 &&
                               s_co[k][cb + 2] == c0 + 2 && s_co[k][cb + 3] == c0 + 3;
              if (vec) {
                store4(d, ro[k] + c0, v + 4 * g, sc);
              } else {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                  const int64_t ci = s_co[k][cb + i];
                  if (ci >= 0) store1(d, ro[k] + ci, v[4 * g + i], sc);
                }
              }
            }
          }
          if (p.absmax != nullptr) {
#pragma unroll
            for (int i = 0; i < 16; ++i)
              if (s_co[0][c + i] >= 0) amax = fmaxf(amax, fabsf(v[i] * sc));
          }
        }
      }
    }
    if (p.absmax != nullptr) {
      for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
      // non-negative doubles order like their bit patterns
      if (lane == 0 && amax > 0.f)
        atomicMax(p.absmax, (unsigned long long)__double_as_longlong(double(amax)));
    }
  }
  float* out = p.part + (size_t(blockIdx.z) * p.m_pad + row) * p.n_pad + n0;
  if (ok && !p.direct) {
    for (int c = c_begin; c < c_end; c += 16) {
      float v[16];
      __syncwarp();
      tmem_ld16(tmem + trow + uint32_t(c), v);
      if (row < p.m_pad) {
#pragma unroll
        for (int j = 0; j < 16; j += 4)
          *reinterpret_cast<float4*>(out + c + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
      }
    }
  }
  // on failure: let in-flight copies land before the CTA's memory goes away
  if (threadIdx.x == 0 && s_fail) {
    for (int i = 0; i < issued_loads; ++i) {
      const int s = i % p.stages;
      (void)mbar_wait(&full[s], (i / p.stages) & 1);
    }
    atomicOr(p.status, 2);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void epi_bar_sync() {
  asm volatile("bar.sync 1, 256;" ::: "memory");  // the eight epilogue warps
}

// Persistent form for direct-epilogue products with more tiles than SMs: one
// CTA per SM walks tiles blockIdx.x, + gridDim.x, ...; the accumulator is
// double-buffered in tensor memory (2 x 256 columns), so while eight
// epilogue warps drain tile i the MMA thread already accumulates tile i + 1
// and the producer keeps the shared-memory ring full across tiles.
// Warp 0 lane 0: TMA producer; warp 1 lane 0: MMA issuer; warps 4-11:
// epilogue (warp w reads TMEM lanes 32 (w % 4).. for half (w - 4) / 4 of the
// columns).  Waits are bounded as in tc_gemm_kernel; the epilogue warps
// agree on failure through shared memory, so their named barriers are always
// reached by all eight.
constexpr int kPThreads = 384;
constexpr uint32_t kPTmemCols = 512;

__global__ void __launch_bounds__(kPThreads, 1)
    tc_gemm_persistent_kernel(const __grid_constant__ CUtensorMap tA,
                              const __grid_constant__ CUtensorMap tAl,
                              const __grid_constant__ CUtensorMap tB,
                              const __grid_constant__ CUtensorMap tBl, const GemmParams p) {
  extern __shared__ uint8_t dyn_smem[];
  uint8_t* base = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(dyn_smem) + 1023) & ~uintptr_t(1023));
  const int bk = p.bk;
  const uint32_t a_bytes = kBM * bk * 2;
  const uint32_t b_bytes = uint32_t(p.ntile) * bk * 2;
  const uint32_t half_bytes = a_bytes + b_bytes;
  const uint32_t stage_bytes = half_bytes * (p.mode == 3 ? 2 : 1);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + size_t(p.stages) * stage_bytes);
  uint64_t* empty = full + p.stages;
  uint64_t* tfull = empty + p.stages;  // [2]
  uint64_t* tempty = tfull + 2;        // [2]
  uint64_t* mdone = tempty + 2;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(mdone + 1);
  __shared__ int s_fail;
  __shared__ int s_epi_fail;
  __shared__ int64_t s_co[4][256];
  // staged epilogue: per epilogue warp and destination, 32 rows x 16 BF16
  // columns of the tile, and the rows' destination offsets
  __shared__ __align__(16) bf16 s_stage[8][2][32][16];
  __shared__ int64_t s_ro[8][2][32];
  // staged epilogue: per destination and group of 4 columns, the offset of
  // the first column when the 4 are contiguous and 4-aligned, else -1
  __shared__ int64_t s_v4[2][64];

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    s_fail = 0;
    s_epi_fail = 0;
    for (int st = 0; st < p.stages; ++st) {
      mbar_init(&full[st], 1);
      mbar_init(&empty[st], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 8);  // one arrival per epilogue warp
    }
    mbar_init(mdone, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_holder)),
                 "r"(kPTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_holder;
  const int ntl = (p.tiles - int(blockIdx.x) + int(gridDim.x) - 1) / int(gridDim.x);
  auto tile_origin = [&](int lt, int& m0, int& n0) {
    const int t = int(blockIdx.x) + lt * int(gridDim.x);
    int mt, nt;
    if (p.n_fast) {
      nt = t % p.n_tiles;
      mt = t / p.n_tiles;
    } else {
      mt = t % p.m_tiles;
      nt = t / p.m_tiles;
    }
    m0 = mt * kBM;
    n0 = nt * p.ntile;
  };
  int issued_loads = 0;

  if (threadIdx.x == 0) {
    // ---------------- TMA producer, across tiles
    int g = 0;
    bool fail = false;
    for (int lt = 0; lt < ntl && !fail; ++lt) {
      int m0, n0;
      tile_origin(lt, m0, n0);
      for (int kb = 0; kb < p.kb_total; ++kb, ++g) {
        const int st = g % p.stages;
        const uint32_t ph = (g / p.stages) & 1;
        if (!mbar_wait_spin(&empty[st], ph ^ 1)) {
          atomicOr(&s_fail, 1);
          fail = true;
          break;
        }
        uint8_t* sp = base + size_t(st) * stage_bytes;
        mbar_expect_tx(&full[st], stage_bytes);
        const int x = kb * bk;
        tma_load_2d(sp, &tA, x, m0, &full[st]);
        tma_load_2d(sp + a_bytes, &tB, x, n0, &full[st]);
        if (p.mode == 3) {
          tma_load_2d(sp + half_bytes, &tAl, x, m0, &full[st]);
          tma_load_2d(sp + half_bytes + a_bytes, &tBl, x, n0, &full[st]);
        }
        issued_loads = g + 1;
      }
    }
  } else if (threadIdx.x == 32) {
    // ---------------- MMA issuer, accumulating tile lt into buffer lt & 1
    const uint32_t idesc = idesc_bf16(kBM, p.ntile);
    int g = 0;
    bool fail = false;
    for (int lt = 0; lt < ntl && !fail; ++lt) {
      const int b = lt & 1;
      const uint32_t use = uint32_t(lt >> 1);
      if (!mbar_wait_spin(&tempty[b], (use & 1) ^ 1)) {
        atomicOr(&s_fail, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t acc = tmem + uint32_t(b) * 256u;
      for (int kb = 0; kb < p.kb_total; ++kb, ++g) {
        const int st = g % p.stages;
        const uint32_t ph = (g / p.stages) & 1;
        if (!mbar_wait_spin(&full[st], ph)) {
          atomicOr(&s_fail, 1);
          fail = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        uint8_t* sp = base + size_t(st) * stage_bytes;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          if (kk * 16 >= bk) break;
          const uint64_t ah = smem_desc(sp + kk * 32, bk);
          const uint64_t bh = smem_desc(sp + a_bytes + kk * 32, bk);
          mma_bf16(acc, ah, bh, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
          if (p.mode == 3) {
            const uint64_t al = smem_desc(sp + half_bytes + kk * 32, bk);
            const uint64_t bl = smem_desc(sp + half_bytes + a_bytes + kk * 32, bk);
            mma_bf16(acc, ah, bl, idesc, 1u);
            mma_bf16(acc, al, bh, idesc, 1u);
          }
        }
        mma_commit(&empty[st]);
      }
      if (!fail) mma_commit(&tfull[b]);
    }
    // every MMA issued by this thread has completed once mdone flips
    mma_commit(mdone);
    (void)mbar_wait(mdone, 0);
  } else if (warp >= 4) {
    // ---------------- epilogue warps
    const int etid = int(threadIdx.x) - 128;  // 0..255
    const int lane_base = (warp & 3) * 32;
    const uint32_t trow = uint32_t(lane_base) << 16;
    const int slice_w = ((p.ntile + 1) / 2 + 15) / 16 * 16;
    const int c_begin = min(p.ntile, ((warp - 4) >> 2) * slice_w);
    const int c_end = min(p.ntile, c_begin + slice_w);
    double scd = p.alpha;
    if (p.scale1 != nullptr) scd /= p.scale1[0];
    if (p.scale2 != nullptr) scd /= p.scale2[0];
    const float sc = float(scd);
    const bool hilo_pair = p.staged && p.nd == 2 && p.d[0].kind == TcKind::kBf16Hi &&
                           p.d[1].kind == TcKind::kBf16Lo;
    float amax = 0.f;
    for (int lt = 0; lt < ntl; ++lt) {
      const int b = lt & 1;
      const uint32_t use = uint32_t(lt >> 1);
      int m0, n0;
      tile_origin(lt, m0, n0);
      bool ok = mbar_wait(&tfull[b], use & 1);
      __syncwarp();
      ok = __all_sync(0xffffffffu, ok);
      if (!ok && lane == 0) s_epi_fail = 1;
      epi_bar_sync();  // all eight warps arrive: failure is decided together
      if (s_epi_fail) {
        if (etid == 0) atomicOr(&s_fail, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int k = 0; k < p.nd; ++k)
        for (int cc = etid; cc < p.ntile; cc += 256) {
          const int64_t n = int64_t(n0) + cc;
          s_co[k][cc] = n < p.N ? lay_col(p.d[k].lay, n) : int64_t(-1);
        }
      epi_bar_sync();
      if (p.staged) {
        for (int k = 0; k < min(p.nd, 2); ++k)
          for (int g4 = etid; g4 < p.ntile / 4; g4 += 256) {
            const int64_t c0 = s_co[k][4 * g4];
            const bool vec = c0 >= 0 && (c0 & 3) == 0 && s_co[k][4 * g4 + 1] == c0 + 1 &&
                             s_co[k][4 * g4 + 2] == c0 + 2 && s_co[k][4 * g4 + 3] == c0 + 3;
            s_v4[k][g4] = vec ? c0 : int64_t(-1);
          }
        epi_bar_sync();
      }
      const int row = m0 + lane_base + lane;
      const bool mvalid = row < p.M;
      int64_t ro[4] = {0, 0, 0, 0};
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k < p.nd && mvalid) ro[k] = lay_row(p.d[k].lay, row);
      const uint32_t tb = tmem + uint32_t(b) * 256u + trow;
      const int ew = warp - 4;
      if (p.staged) {
        if (p.nd > 0) s_ro[ew][0][lane] = ro[0];
        if (p.nd > 1) s_ro[ew][1][lane] = ro[1];
      }
      for (int c = c_begin; c < c_end; c += 16) {
        float v[16];
        __syncwarp();
        tmem_ld16(tb + uint32_t(c), v);
        if (p.staged) {
          // Staged: each lane converts its row's 16 values into shared
          // memory; then 4 lanes cover one row's 16 columns (8 bytes each),
          // so that one store instruction writes 8 rows x 32 bytes instead
          // of 32 scattered 8-byte pieces
          if (hilo_pair) {
            // the hi / lo pair from one rounding per value (the same bits as
            // rounding x for hi and x - hi for lo separately)
            uint32_t wh[8], wl[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              const float x0 = v[2 * i] * sc, x1 = v[2 * i + 1] * sc;
              const __nv_bfloat162 h2 = __floats2bfloat162_rn(x0, x1);
              const __nv_bfloat162 l2 = __floats2bfloat162_rn(x0 - __low2float(h2),
                                                              x1 - __high2float(h2));
              wh[i] = *reinterpret_cast<const uint32_t*>(&h2);
              wl[i] = *reinterpret_cast<const uint32_t*>(&l2);
            }
            uint4* dh = reinterpret_cast<uint4*>(&s_stage[ew][0][lane][0]);
            uint4* dl = reinterpret_cast<uint4*>(&s_stage[ew][1][lane][0]);
            dh[0] = make_uint4(wh[0], wh[1], wh[2], wh[3]);
            dh[1] = make_uint4(wh[4], wh[5], wh[6], wh[7]);
            dl[0] = make_uint4(wl[0], wl[1], wl[2], wl[3]);
            dl[1] = make_uint4(wl[4], wl[5], wl[6], wl[7]);
          } else {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              if (k >= p.nd) break;
              const bool lo = p.d[k].kind == TcKind::kBf16Lo;
              uint32_t w[8];
#pragma unroll
              for (int i = 0; i < 8; ++i) {
                float x0 = v[2 * i] * sc, x1 = v[2 * i + 1] * sc;
                if (lo) {
                  x0 -= __bfloat162float(__float2bfloat16(x0));
                  x1 -= __bfloat162float(__float2bfloat16(x1));
                }
                const __nv_bfloat162 h2 = __floats2bfloat162_rn(x0, x1);
                w[i] = *reinterpret_cast<const uint32_t*>(&h2);
              }
              uint4* dst4 = reinterpret_cast<uint4*>(&s_stage[ew][k][lane][0]);
              dst4[0] = make_uint4(w[0], w[1], w[2], w[3]);
              dst4[1] = make_uint4(w[4], w[5], w[6], w[7]);
            }
          }
          __syncwarp();
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            if (k >= p.nd) break;
            bf16* dp = static_cast<bf16*>(p.d[k].p);
#pragma unroll
            for (int it = 0; it < 4; ++it) {
              const int g = it * 32 + lane, r = g >> 2, c4 = (g & 3) * 4;
              if (m0 + lane_base + r >= p.M) continue;
              const int64_t rr = s_ro[ew][k][r];
              const int64_t v0 = s_v4[k][(c + c4) >> 2];
              if (v0 >= 0 && (rr & 3) == 0) {
                *reinterpret_cast<uint2*>(dp + rr + v0) =
                    *reinterpret_cast<const uint2*>(&s_stage[ew][k][r][c4]);
              } else {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                  const int64_t ci = s_co[k][c + c4 + i];
                  if (ci >= 0) dp[rr + ci] = s_stage[ew][k][r][c4 + i];
                }
              }
            }
          }
          __syncwarp();  // the staging buffer is rewritten by the next chunk
        } else if (mvalid) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (k >= p.nd) break;
            const TcDest& d = p.d[k];
#pragma unroll
            for (int gq = 0; gq < 4; ++gq) {
              const int cb = c + 4 * gq;
              const int64_t c0 = s_co[k][cb];
              const bool vec = c0 >= 0 && ((ro[k] + c0) & 3) == 0 && s_co[k][cb + 1] == c0 + 1 &&
                               s_co[k][cb + 2] == c0 + 2 && s_co[k][cb + 3] == c0 + 3;
              if (vec) {
                store4(d, ro[k] + c0, v + 4 * gq, sc);
              } else {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                  const int64_t ci = s_co[k][cb + i];
                  if (ci >= 0) store1(d, ro[k] + ci, v[4 * gq + i], sc);
                }
              }
            }
          }
        }
        if (mvalid) {
          if (p.absmax != nullptr) {
#pragma unroll
            for (int i = 0; i < 16; ++i)
              if (s_co[0][c + i] >= 0) amax = fmaxf(amax, fabsf(v[i] * sc));
          }
        }
      }
      // this warp's reads of buffer b are complete (tmem_ld16 waits): hand it back
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[b]);
    }
    if (p.absmax != nullptr) {
      for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
      if (lane == 0 && amax > 0.f)
        atomicMax(p.absmax, (unsigned long long)__double_as_longlong(double(amax)));
    }
  }
  // on failure: let in-flight copies land before the CTA's memory goes away
  if (threadIdx.x == 0 && s_fail) {
    for (int i = 0; i < issued_loads; ++i) (void)mbar_wait(&full[i % p.stages], (i / p.stages) & 1);
    atomicOr(p.status, 2);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kPTmemCols)
                 : "memory");
  }
}

// Sums the split-K partials in order and writes every destination.
struct ReduceParams {
  const float* part;
  int splits, m_pad, n_pad;
  int64_t M, N;
  double alpha;
  const double* inv_scale;
  const double* inv_scale2;
  int nd;
  TcDest d[4];
};

// 32 x 32 output tile per block (32 x 8 threads).  Every layout is separable
// (offset = row part + column part), so each block decodes its 32 row and 32
// column offsets once per destination.  Destinations whose innermost column
// stride is 1 are written with the column index fastest, the others with the
// row index fastest, so warps store contiguously in the common cases.
__global__ void tc_reduce_kernel(const ReduceParams r) {
  __shared__ float tile[32][33];
  __shared__ int64_t ro[32], co[32];
  const int64_t m0 = int64_t(blockIdx.x) * 32, n0 = int64_t(blockIdx.y) * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  double scd = r.alpha;
  if (r.inv_scale != nullptr) scd /= r.inv_scale[0];
  if (r.inv_scale2 != nullptr) scd /= r.inv_scale2[0];
  const float sc = float(scd);
  // the four rows of a thread are summed together, split by split, so that
  // four independent loads are in flight (one row at a time left the
  // kernel waiting on one memory latency per split and row)
  {
    const int64_t n = n0 + tx;
    float s[4] = {0.f, 0.f, 0.f, 0.f};
    bool in[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) in[j] = m0 + ty + 8 * j < r.M && n < r.N;
    for (int t = 0; t < r.splits; ++t) {
      const float* pt = r.part + (size_t(t) * r.m_pad + m0 + ty) * r.n_pad + n;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (in[j]) s[j] += pt[size_t(8 * j) * r.n_pad];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) tile[ty + 8 * j][tx] = s[j];
  }
  for (int k = 0; k < r.nd; ++k) {
    const TcDest& d = r.d[k];
    __syncthreads();
    if (threadIdx.x < 32) ro[threadIdx.x] = lay_row(d.lay, m0 + threadIdx.x);
    else if (threadIdx.x < 64) co[threadIdx.x - 32] = lay_col(d.lay, n0 + threadIdx.x - 32);
    __syncthreads();
    const bool n_fast = d.lay.ns[d.lay.nn - 1] == 1;
    for (int yy = ty; yy < 32; yy += 8) {
      const int mi = n_fast ? yy : tx, ni = n_fast ? tx : yy;
      if (m0 + mi >= r.M || n0 + ni >= r.N) continue;
      store1(d, ro[mi] + co[ni], tile[mi][ni], sc);
    }
  }
}

template <class S>
__global__ void split_bf16_kernel(const S* src, int64_t rows, int64_t cols, int64_t ld_src,
                                  int transpose, bf16* hi, bf16* lo, int64_t ld_dst) {
  // the split in the source's precision: for an FP32 source x - hi is exact
  // in FP32, so FP32 arithmetic gives the bits FP64 would (FP64 is slow here)
  __shared__ S tile[32][33];
  const int64_t r0 = int64_t(blockIdx.y) * 32, c0 = int64_t(blockIdx.x) * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  auto split = [&](S x, bf16& h, bf16& l) {
    if constexpr (sizeof(S) == 4) {
      h = __float2bfloat16(x);
      l = __float2bfloat16(x - __bfloat162float(h));
    } else {
      h = __double2bfloat16(x);
      l = __double2bfloat16(x - double(__bfloat162float(h)));
    }
  };
  if (!transpose) {
    for (int yy = ty; yy < 32; yy += 8) {
      const int64_t r = r0 + yy, c = c0 + tx;
      if (r < rows && c < cols) {
        bf16 h, l;
        split(src[r * ld_src + c], h, l);
        hi[r * ld_dst + c] = h;
        if (lo != nullptr) lo[r * ld_dst + c] = l;
      }
    }
    return;
  }
  for (int yy = ty; yy < 32; yy += 8) {
    const int64_t r = r0 + yy, c = c0 + tx;
    tile[yy][tx] = (r < rows && c < cols) ? src[r * ld_src + c] : S(0);
  }
  __syncthreads();
  for (int yy = ty; yy < 32; yy += 8) {
    const int64_t c = c0 + yy, r = r0 + tx;  // destination row c, column r
    if (r < rows && c < cols) {
      bf16 h, l;
      split(tile[tx][yy], h, l);
      hi[c * ld_dst + r] = h;
      if (lo != nullptr) lo[c * ld_dst + r] = l;
    }
  }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point, so the
// library does not link libcuda (it still loads on machines without a driver).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  if (fn == nullptr) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    CTM_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                              cudaEnableDefault, &q));
    CTM_REQUIRE(p != nullptr && q == cudaDriverEntryPointSuccess, CTM_ERR_CUDA,
                "cuTensorMapEncodeTiled is not available from the driver");
    fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

void make_map(CUtensorMap* map, const bf16* ptr, int64_t rows, int64_t k, int64_t ld,
              uint32_t box_rows, int bk) {
  CTM_REQUIRE(ptr != nullptr, CTM_ERR_INVALID, "tc_gemm: operand pointer is NULL");
  CTM_REQUIRE((reinterpret_cast<uintptr_t>(ptr) & 15) == 0, CTM_ERR_INVALID,
              "tc_gemm: operand must be 16-byte aligned");
  CTM_REQUIRE(ld % 8 == 0 && ld >= k, CTM_ERR_INVALID, "tc_gemm: leading dimension");
  const cuuint64_t dims[2] = {cuuint64_t(k), cuuint64_t(rows)};
  const cuuint64_t strides[1] = {cuuint64_t(ld) * 2};
  const cuuint32_t box[2] = {uint32_t(bk), box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult res = encode_tiled()(
      map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(ptr), dims, strides, box, estr,
      CU_TENSOR_MAP_INTERLEAVE_NONE,
      bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  CTM_REQUIRE(res == CUDA_SUCCESS, CTM_ERR_CUDA,
              "cuTensorMapEncodeTiled failed with code " + std::to_string(int(res)));
}

// Kernel-class names built at run time, kept for the life of the process.
const char* intern_name(const std::string& s) {
  static std::mutex mu;
  static std::set<std::string> names;
  std::lock_guard<std::mutex> lk(mu);
  return names.insert(s).first->c_str();
}

// SM count of the current device (152 on GB300), used by both the sizing
// pass and the launch so that they choose the same split-K; 152 when no
// device is visible (workspace queries on a machine without a GPU).
int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return 152;
  }
  return n;
}

}  // namespace

template <class S>
void split_bf16_impl(Ctx& c, const S* src, int64_t rows, int64_t cols, int64_t ld_src,
                     bool transpose, bf16* hi, bf16* lo, int64_t ld_dst) {
  if (c.sizing() || rows * cols == 0) return;
  dim3 grid(unsigned((cols + 31) / 32), unsigned((rows + 31) / 32));
  CTM_REQUIRE(grid.y <= 65535, CTM_ERR_UNSUPPORTED, "split_bf16: too many rows");
  KernelTimer kt(c.stream, "split_bf16_kernel", kUnitByte,
                 double(rows) * cols * (sizeof(S) + (lo != nullptr ? 4.0 : 2.0)));
  split_bf16_kernel<S><<<grid, 256, 0, c.stream>>>(src, rows, cols, ld_src, transpose ? 1 : 0, hi,
                                                   lo, ld_dst);
  CTM_LAUNCH_CHECK();
}

void split_bf16(Ctx& c, const double* src, int64_t rows, int64_t cols, int64_t ld_src,
                bool transpose, bf16* hi, bf16* lo, int64_t ld_dst) {
  split_bf16_impl<double>(c, src, rows, cols, ld_src, transpose, hi, lo, ld_dst);
}

void split_bf16(Ctx& c, const float* src, int64_t rows, int64_t cols, int64_t ld_src,
                bool transpose, bf16* hi, bf16* lo, int64_t ld_dst) {
  split_bf16_impl<float>(c, src, rows, cols, ld_src, transpose, hi, lo, ld_dst);
}

namespace {

template <class S>
__global__ void gather_split_kernel(const S* src, const Gather g, int64_t rows, int64_t K,
                                    bf16* hi, bf16* lo, int64_t ld) {
  // 32-bit index decoding (rows K < 2^31, checked on the host)
  const uint32_t total = uint32_t(rows * K), uk = uint32_t(K);
  for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += gridDim.x * blockDim.x) {
    uint32_t r = idx / uk, k = idx - (idx / uk) * uk;
    const int64_t r0 = r, k0 = k;
    int64_t off = 0;
    for (int j = g.nr - 1; j >= 0; --j) {
      const uint32_t e = uint32_t(g.re[j]), q = r / e;
      off += int64_t(r - q * e) * g.rs[j];
      r = q;
    }
    for (int j = g.nk - 1; j >= 0; --j) {
      const uint32_t e = uint32_t(g.ke[j]), q = k / e;
      off += int64_t(k - q * e) * g.ks[j];
      k = q;
    }
    bf16 h, l;
    if constexpr (sizeof(S) == 4) {  // exact in FP32 for an FP32 source (see split_bf16_kernel)
      const float x = src[off];
      h = __float2bfloat16(x);
      l = __float2bfloat16(x - __bfloat162float(h));
    } else {
      const double x = src[off];
      h = __double2bfloat16(x);
      l = __double2bfloat16(x - double(__bfloat162float(h)));
    }
    hi[r0 * ld + k0] = h;
    if (lo != nullptr) lo[r0 * ld + k0] = l;
  }
}

}  // namespace

__global__ void join_bf16_kernel(const bf16* hi, const bf16* lo, int64_t rows, int64_t cols,
                                 int64_t ld, double* out) {
  for (int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < rows * cols;
       idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = idx / cols, q = idx % cols;
    double v = double(__bfloat162float(hi[r * ld + q]));
    if (lo != nullptr) v += double(__bfloat162float(lo[r * ld + q]));
    out[idx] = v;
  }
}

namespace {

// dst = src^T for one 64 x 64 cell of BF16, of the hi and (when given) the
// lo array in the same CTA, so that each thread has four 16-byte loads in
// flight.  A cell goes through shared memory as 64 rows of 32 words (two
// BF16 each; rows padded to 33 words, so that the 16-byte loads' four
// words and the column reads below spread over the banks); a destination
// word is a 2 x 2 block transposed in registers: lane i of a warp reads the
// words of source rows 2i and 2i + 1 at one word column and writes word i of
// the two destination rows that column holds (a warp stores 128 contiguous
// bytes per destination row; the reads hit at most two words per bank).
__global__ void __launch_bounds__(256) transpose_bf16_kernel(
    const bf16* src_hi, const bf16* src_lo, int64_t rows, int64_t cols, int64_t ld_src,
    bf16* dst_hi, bf16* dst_lo, int64_t ld_dst) {
  __shared__ uint32_t tile[2][64][33];
  const int na = src_lo != nullptr ? 2 : 1;
  const int64_t r0 = int64_t(blockIdx.y) * 64, c0 = int64_t(blockIdx.x) * 64;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool vsrc = (ld_src & 7) == 0 && (reinterpret_cast<uintptr_t>(src_hi) & 15) == 0 &&
                    (na == 1 || (reinterpret_cast<uintptr_t>(src_lo) & 15) == 0);
  const bool vdst = (ld_dst & 1) == 0 && (reinterpret_cast<uintptr_t>(dst_hi) & 3) == 0 &&
                    (na == 1 || (reinterpret_cast<uintptr_t>(dst_lo) & 3) == 0);
  const bf16 z = __float2bfloat16(0.f);
  uint4 v[2][2];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const bf16* src = a == 0 ? src_hi : src_lo;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int i = tid + 256 * j, rr = i >> 3, ch = i & 7;
      const int64_t r = r0 + rr, cc = c0 + ch * 8;
      v[a][j] = make_uint4(0u, 0u, 0u, 0u);
      if (a < na && r < rows && cc < cols) {
        if (vsrc && cc + 8 <= cols) {
          v[a][j] = *reinterpret_cast<const uint4*>(src + r * ld_src + cc);
        } else {
          __align__(16) bf16 e[8];
          for (int t = 0; t < 8; ++t) e[t] = cc + t < cols ? src[r * ld_src + cc + t] : z;
          v[a][j] = *reinterpret_cast<const uint4*>(e);
        }
      }
    }
  }
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int i = tid + 256 * j, rr = i >> 3, ch = i & 7;
      tile[a][rr][ch * 4 + 0] = v[a][j].x;
      tile[a][rr][ch * 4 + 1] = v[a][j].y;
      tile[a][rr][ch * 4 + 2] = v[a][j].z;
      tile[a][rr][ch * 4 + 3] = v[a][j].w;
    }
  __syncthreads();
  const int64_t dc = r0 + 2 * lane;  // destination column of the word's first element
  for (int a = 0; a < na; ++a) {
    bf16* dst = a == 0 ? dst_hi : dst_lo;
    for (int wc = warp; wc < 32; wc += 8) {
      const uint32_t x0 = tile[a][2 * lane][wc], x1 = tile[a][2 * lane + 1][wc];
      // destination rows c0 + 2 wc (low halves) and c0 + 2 wc + 1 (high halves)
      const uint32_t w[2] = {__byte_perm(x0, x1, 0x5410), __byte_perm(x0, x1, 0x7632)};
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t dr = c0 + 2 * wc + h;
        if (dr >= cols || dc >= rows) continue;
        bf16* p = dst + dr * ld_dst + dc;
        if (vdst && dc + 2 <= ld_dst) {
          *reinterpret_cast<uint32_t*>(p) = w[h];
        } else {
          const uint32_t x = w[h];
          p[0] = *reinterpret_cast<const bf16*>(&x);
          if (dc + 1 < rows) p[1] = reinterpret_cast<const bf16*>(&x)[1];
        }
      }
    }
  }
}

}  // namespace

void transpose_bf16(Ctx& c, const bf16* src_hi, const bf16* src_lo, int64_t rows, int64_t cols,
                    int64_t ld_src, bf16* dst_hi, bf16* dst_lo, int64_t ld_dst) {
  if (c.sizing() || rows * cols == 0) return;
  CTM_REQUIRE((src_lo == nullptr) == (dst_lo == nullptr), CTM_ERR_INVALID,
              "transpose_bf16: lo arrays must be given on both sides or neither");
  const dim3 grid(unsigned((cols + 63) / 64), unsigned((rows + 63) / 64), 1u);
  CTM_REQUIRE(grid.y <= 65535, CTM_ERR_UNSUPPORTED, "transpose_bf16: too many rows");
  KernelTimer kt(c.stream, "transpose_bf16_kernel", kUnitByte,
                 4.0 * double(rows) * cols * (src_lo != nullptr ? 2.0 : 1.0));
  transpose_bf16_kernel<<<grid, 256, 0, c.stream>>>(src_hi, src_lo, rows, cols, ld_src, dst_hi,
                                                    dst_lo, ld_dst);
  CTM_LAUNCH_CHECK();
}

void join_bf16(Ctx& c, const bf16* hi, const bf16* lo, int64_t rows, int64_t cols, int64_t ld,
               double* out) {
  if (c.sizing() || rows * cols == 0) return;
  KernelTimer kt(c.stream, "join_bf16_kernel", kUnitByte,
                 double(rows) * cols * (8.0 + (lo != nullptr ? 4.0 : 2.0)));
  join_bf16_kernel<<<grid_for(rows * cols, 256), 256, 0, c.stream>>>(hi, lo, rows, cols, ld, out);
  CTM_LAUNCH_CHECK();
}

template <class S>
void gather_split_impl(Ctx& c, const S* src, const Gather& g, bf16* hi, bf16* lo, int64_t ld) {
  int64_t rows = 1, K = 1;
  for (int j = 0; j < g.nr; ++j) rows *= g.re[j];
  for (int j = 0; j < g.nk; ++j) K *= g.ke[j];
  if (c.sizing() || rows * K == 0) return;
  CTM_REQUIRE(rows * K < (int64_t(1) << 31), CTM_ERR_UNSUPPORTED,
              "gather_split: fewer than 2^31 elements");
  KernelTimer kt(c.stream, "gather_split_kernel", kUnitByte,
                 double(rows) * K * (sizeof(S) + (lo != nullptr ? 4.0 : 2.0)));
  gather_split_kernel<S><<<grid_for(rows * K, 256), 256, 0, c.stream>>>(src, g, rows, K, hi, lo,
                                                                       ld);
  CTM_LAUNCH_CHECK();
}

void gather_split_bf16(Ctx& c, const double* src, const Gather& g, bf16* hi, bf16* lo, int64_t ld) {
  gather_split_impl<double>(c, src, g, hi, lo, ld);
}

void gather_split_bf16(Ctx& c, const float* src, const Gather& g, bf16* hi, bf16* lo, int64_t ld) {
  gather_split_impl<float>(c, src, g, hi, lo, ld);
}

namespace {

// Tile plan of one product.  Candidate bits: 1 = N tiles of at most 128
// columns (default: 256), 2 = no K split (default: split K so that the grid
// fills the SMs in one wave).
struct TcPlan {
  int ntile = 0, bk = 64, kb_total = 0, splits = 1, kb_per_split = 0, stages = 2, p_stages = 2;
  int64_t n_tiles = 0, m_tiles = 0, base_ctas = 0;
  bool direct = true, n_fast = false, persistent = false;
  int m_pad = 0, n_pad = 0;
  uint32_t stage_bytes = 0;
  size_t smem = 0, p_smem = 0;
  size_t part_elems() const { return direct ? 0 : size_t(splits) * m_pad * n_pad; }
};

constexpr int kTcCandidates = 4;

TcPlan tc_plan(int64_t M, int64_t N, int64_t K, int imode, bool absmax, int cand) {
  TcPlan pl;
  // N tiling: MMA N must be a multiple of 16 up to 256 (256-wide 3xBF16
  // tiles with two stages measured faster than 128-wide ones with three:
  // 373 us against 551 us for the double-layer GEMM at D=6)
  const int64_t nmax = (cand & 1) ? 128 : 256;
  pl.n_tiles = (N + nmax - 1) / nmax;
  pl.ntile = static_cast<int>(((N + pl.n_tiles - 1) / pl.n_tiles + 15) / 16 * 16);
  pl.ntile = std::max(pl.ntile, 16);
  pl.m_tiles = (M + kBM - 1) / kBM;
  // 64-wide K steps: measured faster than 32-wide ones with a deeper ring
  // (64-byte swizzle) even where only two 3xBF16 stages fit (the double-layer
  // GEMM at D=6: 373 us against 469 us)
  pl.bk = 64;
  pl.kb_total = static_cast<int>((K + pl.bk - 1) / pl.bk);
  pl.base_ctas = pl.m_tiles * pl.n_tiles;
  const int sms = sm_count();
  // split K so that the grid fills the SMs in one wave: a partial second wave
  // costs as much time as a full one
  int splits = static_cast<int>(std::min<int64_t>(std::max<int64_t>(1, sms / pl.base_ctas),
                                                  std::max(1, pl.kb_total / 4)));
  splits = std::max(splits, 1);
  if (absmax || (cand & 2)) splits = 1;  // the maximum is taken over complete sums
  pl.kb_per_split = (pl.kb_total + splits - 1) / splits;
  pl.splits = (pl.kb_total + pl.kb_per_split - 1) / pl.kb_per_split;
  pl.direct = pl.splits == 1;
  pl.m_pad = static_cast<int>(pl.m_tiles * kBM);
  pl.n_pad = static_cast<int>(pl.n_tiles * pl.ntile);
  pl.stage_bytes = uint32_t(kBM * pl.bk * 2 + pl.ntile * pl.bk * 2) * (imode == 3 ? 2 : 1);
  // dynamic shared memory: the stage ring (the kernel's static arrays take ~8 KB)
  pl.stages = std::max(2, std::min(6, int((210 * 1024) / pl.stage_bytes)));
  pl.smem = size_t(pl.stages) * pl.stage_bytes + 256 + 1024;
  // grid x over N tiles when A is the larger operand: the CTAs that share an
  // A tile are then resident together and A streams from DRAM once
  pl.n_fast = pl.n_tiles > 1 && pl.m_tiles > pl.n_tiles && pl.m_tiles <= 65535;
  // more tiles than SMs with a direct epilogue: one persistent CTA per SM;
  // its static shared memory (offset tables and the staged epilogue, ~29 KB)
  // leaves 196 KB for the stage ring
  pl.persistent = pl.direct && pl.base_ctas > sms;
  pl.p_stages = std::max(2, std::min(6, int((196 * 1024) / pl.stage_bytes)));
  pl.p_smem = size_t(pl.p_stages) * pl.stage_bytes + 256 + 1024;
  return pl;
}

void tc_launch(Ctx& c, const TcOperand& A, const TcOperand& B, int imode, const TcOut& out,
               double* absmax, const TcPlan& pl, float* part) {
  const int64_t M = A.rows, N = B.rows, K = A.k;
  const int sms = sm_count();
  CTM_REQUIRE(pl.m_tiles <= 0x7fffffff && pl.n_tiles <= 65535 && pl.splits <= 65535,
              CTM_ERR_UNSUPPORTED, "tc_gemm: grid too large");
  CTM_REQUIRE(M < (int64_t(1) << 31) && N < (int64_t(1) << 31), CTM_ERR_UNSUPPORTED,
              "tc_gemm: M and N must be below 2^31");
  for (int i = 0; i < out.nd; ++i)
    for (int j = 0; j < kTcModes; ++j)
      CTM_REQUIRE(out.d[i].lay.me[j] >= 1 && out.d[i].lay.me[j] < (int64_t(1) << 32) &&
                      out.d[i].lay.ne[j] >= 1 && out.d[i].lay.ne[j] < (int64_t(1) << 32),
                  CTM_ERR_INVALID, "tc_gemm: layout extents must be in [1, 2^32)");
  CUtensorMap tA, tAl, tB, tBl;
  make_map(&tA, A.hi, A.rows, K, A.ld, kBM, pl.bk);
  make_map(&tB, B.hi, B.rows, K, B.ld, uint32_t(pl.ntile), pl.bk);
  if (imode == 3) {
    make_map(&tAl, A.lo, A.rows, K, A.ld, kBM, pl.bk);
    make_map(&tBl, B.lo, B.rows, K, B.ld, uint32_t(pl.ntile), pl.bk);
  } else {
    tAl = tA;
    tBl = tB;
  }
  bool bf16_dests = out.nd >= 1 && out.nd <= 2;
  for (int i = 0; i < out.nd; ++i)
    bf16_dests = bf16_dests && (out.d[i].kind == TcKind::kBf16Hi || out.d[i].kind == TcKind::kBf16Lo);
  GemmParams p{};
  p.m_tiles = int(pl.m_tiles);
  p.n_tiles = int(pl.n_tiles);
  p.tiles = int(pl.m_tiles * pl.n_tiles);
  p.ntile = pl.ntile;
  p.bk = pl.bk;
  p.kb_total = pl.kb_total;
  p.kb_per_split = pl.kb_per_split;
  p.stages = pl.persistent ? pl.p_stages : pl.stages;
  p.mode = imode;
  p.part = part;
  p.m_pad = pl.m_pad;
  p.n_pad = pl.n_pad;
  p.status = status_flags(c);
  p.direct = pl.direct ? 1 : 0;
  p.n_fast = pl.n_fast ? 1 : 0;
  p.nd = out.nd;
  p.alpha = out.alpha;
  p.scale1 = out.inv_scale;
  p.scale2 = out.inv_scale2;
  p.absmax = reinterpret_cast<unsigned long long*>(absmax);
  p.M = M;
  p.N = N;
  p.staged = (pl.persistent && bf16_dests) ? 1 : 0;
  for (int i = 0; i < out.nd; ++i) p.d[i] = out.d[i];
  if (absmax != nullptr) CTM_CUDA(cudaMemsetAsync(absmax, 0, sizeof(double), c.stream));
  CTM_CUDA(cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(pl.smem)));
  const dim3 grid(static_cast<unsigned>(pl.n_fast ? pl.n_tiles : pl.m_tiles),
                  static_cast<unsigned>(pl.n_fast ? pl.m_tiles : pl.n_tiles),
                  static_cast<unsigned>(pl.splits));
  {
    const double work = 2.0 * double(M) * N * K * imode;
    KernelTimer timer(c.stream, kTagTcGemm, work);
    KernelTimer timer2(c.stream, out.extra_tag >= 0 ? out.extra_tag : kTagTcGemm,
                       out.extra_tag >= 0 ? work : -1.0);
    const char* kname = pl.persistent ? "tc_gemm_persistent_kernel" : "tc_gemm_kernel";
    if (out.name != nullptr) kname = intern_name(std::string(kname) + " (" + out.name + ")");
    KernelTimer timer3(c.stream, kname, kUnitFlop,
                       out.algo_flops >= 0.0 ? out.algo_flops : 2.0 * double(M) * N * K);
    if (pl.persistent) {
      CTM_CUDA(cudaFuncSetAttribute(tc_gemm_persistent_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, int(pl.p_smem)));
      tc_gemm_persistent_kernel<<<unsigned(std::min<int64_t>(pl.base_ctas, sms)), kPThreads,
                                  pl.p_smem, c.stream>>>(tA, tAl, tB, tBl, p);
    } else {
      tc_gemm_kernel<<<grid, kThreads, pl.smem, c.stream>>>(tA, tAl, tB, tBl, p);
    }
    CTM_LAUNCH_CHECK();
  }
  if (pl.direct) return;
  ReduceParams r{};
  r.part = part;
  r.splits = pl.splits;
  r.m_pad = pl.m_pad;
  r.n_pad = pl.n_pad;
  r.M = M;
  r.N = N;
  r.alpha = out.alpha;
  r.inv_scale = out.inv_scale;
  r.inv_scale2 = out.inv_scale2;
  r.nd = out.nd;
  for (int i = 0; i < out.nd; ++i) r.d[i] = out.d[i];
  dim3 rg(unsigned((M + 31) / 32), unsigned((N + 31) / 32));
  CTM_REQUIRE(rg.y <= 65535, CTM_ERR_UNSUPPORTED, "tc_gemm: output too wide");
  KernelTimer kt(c.stream, "tc_reduce_kernel", kUnitByte, 4.0 * (pl.splits + 1.0) * double(M) * N);
  tc_reduce_kernel<<<rg, 256, 0, c.stream>>>(r);
  CTM_LAUNCH_CHECK();
}

// ---------------------------------------------------------------- autotuner
// Per product shape (M, N, K, passes, epilogue) the tile plan is one of the
// candidates above.  While tuning is on, the first eager call of a new shape
// runs every distinct candidate twice, timed with CUDA events on its stream
// (which synchronises that stream), keeps the fastest, and runs it again so
// that the output is the chosen plan's; later calls use the table.  Without
// an entry the default plan (candidate 0) runs.  Calls under stream capture
// never tune.
struct TuneKey {
  int64_t M, N, K;
  int mode, absmax, nd, kind0;
  std::string name;
  bool operator<(const TuneKey& o) const {
    return std::tie(M, N, K, mode, absmax, nd, kind0, name) <
           std::tie(o.M, o.N, o.K, o.mode, o.absmax, o.nd, o.kind0, o.name);
  }
};
struct TuneEntry {
  int choice = 0;
  double best_ms = 0.0, default_ms = 0.0;
};
std::mutex g_tune_mu;
bool g_tuning = false;
std::map<TuneKey, TuneEntry> g_tune;

void tc_gemm_impl(Ctx& c, const TcOperand& A, const TcOperand& B, TcMode mode, TcOut out,
                  double* absmax) {
  CTM_REQUIRE(A.k == B.k && A.k >= 1 && A.rows >= 1 && B.rows >= 1, CTM_ERR_INVALID,
              "tc_gemm: operand shapes");
  const int imode = static_cast<int>(mode);
  const int64_t M = A.rows, N = B.rows, K = A.k;
  TcPlan plans[kTcCandidates];
  size_t part_elems = 0;
  for (int i = 0; i < kTcCandidates; ++i) {
    plans[i] = tc_plan(M, N, K, imode, absmax != nullptr, i);
    part_elems = std::max(part_elems, plans[i].part_elems());
  }
  // the split-K buffer fits every candidate, so the workspace size does not
  // depend on what the tuner picks
  Scope scope(c);
  float* part = part_elems ? c.alloc<float>(part_elems) : nullptr;
  if (c.sizing()) return;
  CTM_REQUIRE(imode == 1 || (A.lo != nullptr && B.lo != nullptr), CTM_ERR_INVALID,
              "tc_gemm: 3xBF16 needs lo parts");
  const TuneKey key{M, N, K, imode, absmax != nullptr ? 1 : 0, out.nd,
                    out.nd ? int(out.d[0].kind) : -1, out.name ? out.name : ""};
  int choice = 0;
  bool tune = false;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) choice = it->second.choice;
    else tune = g_tuning;
  }
  if (tune) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CTM_CUDA(cudaStreamIsCapturing(c.stream, &cs));
    tune = cs == cudaStreamCaptureStatusNone;
  }
  if (!tune) {
    tc_launch(c, A, B, imode, out, absmax, plans[choice], part);
    return;
  }
  TuneEntry e;
  double best = 1e30;
  cudaEvent_t ev0, ev1;
  CTM_CUDA(cudaEventCreate(&ev0));
  CTM_CUDA(cudaEventCreate(&ev1));
  for (int i = 0; i < kTcCandidates; ++i) {
    bool dup = false;  // identical to an earlier candidate
    for (int j = 0; j < i; ++j)
      dup = dup || (plans[j].ntile == plans[i].ntile && plans[j].splits == plans[i].splits);
    if (dup) continue;
    float ms = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {  // the first run also loads the kernel's attributes
      CTM_CUDA(cudaEventRecord(ev0, c.stream));
      tc_launch(c, A, B, imode, out, absmax, plans[i], part);
      CTM_CUDA(cudaEventRecord(ev1, c.stream));
      CTM_CUDA(cudaEventSynchronize(ev1));
      float t = 0.f;
      CTM_CUDA(cudaEventElapsedTime(&t, ev0, ev1));
      ms = std::min(ms, t);
    }
    if (i == 0) e.default_ms = ms;
    if (ms < best) {
      best = ms;
      e.choice = i;
    }
  }
  CTM_CUDA(cudaEventDestroy(ev0));
  CTM_CUDA(cudaEventDestroy(ev1));
  e.best_ms = best;
  tc_launch(c, A, B, imode, out, absmax, plans[e.choice], part);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = e;
}

}  // namespace

void tc_gemm(Ctx& c, const TcOperand& A, const TcOperand& B, TcMode mode, const TcOut& out) {
  tc_gemm_impl(c, A, B, mode, out, nullptr);
}

void tc_gemm_absmax(Ctx& c, const TcOperand& A, const TcOperand& B, TcMode mode,
                    const TcOut& out, double* absmax) {
  CTM_REQUIRE(absmax != nullptr || c.sizing(), CTM_ERR_INVALID, "absmax scalar is NULL");
  tc_gemm_impl(c, A, B, mode, out, c.sizing() ? reinterpret_cast<double*>(16) : absmax);
}

}  // namespace ctm

// ---------------------------------------------------------------- C ABI of the autotuner
using namespace ctm;

extern "C" {

int ctm_autotune(int32_t enable, int32_t* entries) {
  return guarded([&] {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (enable >= 0) g_tuning = enable != 0;
    if (enable == -2) g_tune.clear();
    if (entries != nullptr) *entries = static_cast<int32_t>(g_tune.size());
  });
}

int ctm_autotune_entry(int32_t i, int64_t* mnk, int32_t* mode_choice, double* best_ms,
                       double* default_ms) {
  return guarded([&] {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    CTM_REQUIRE(i >= 0 && i < static_cast<int32_t>(g_tune.size()), CTM_ERR_INVALID,
                "bad autotune entry");
    auto it = g_tune.begin();
    std::advance(it, i);
    if (mnk != nullptr) {
      mnk[0] = it->first.M;
      mnk[1] = it->first.N;
      mnk[2] = it->first.K;
    }
    if (mode_choice != nullptr) {
      mode_choice[0] = it->first.mode;
      mode_choice[1] = it->second.choice;
    }
    if (best_ms != nullptr) *best_ms = it->second.best_ms;
    if (default_ms != nullptr) *default_ms = it->second.default_ms;
  });
}

// Test hook, not part of the plugin interface (no declaration in the
// public header): transpose_bf16 on caller-owned BF16 device arrays (src
// rows x cols with leading dimension ld_src; dst cols x rows with ld_dst; lo
// arrays optional), on the given stream.
int ctm_test_transpose_bf16(const void* src_hi, const void* src_lo, int64_t rows, int64_t cols,
                            int64_t ld_src, void* dst_hi, void* dst_lo, int64_t ld_dst,
                            void* stream) {
  return guarded([&] {
    CTM_REQUIRE(rows >= 1 && cols >= 1 && ld_src >= cols && ld_dst >= rows, CTM_ERR_INVALID,
                "transpose: bad sizes");
    Ctx c;
    c.stream = static_cast<cudaStream_t>(stream);
    c.base = reinterpret_cast<char*>(16);  // not sizing; nothing is allocated
    transpose_bf16(c, static_cast<const bf16*>(src_hi), static_cast<const bf16*>(src_lo), rows,
                   cols, ld_src, static_cast<bf16*>(dst_hi), static_cast<bf16*>(dst_lo), ld_dst);
  });
}

}  // extern "C"
