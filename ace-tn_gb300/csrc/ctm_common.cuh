// Shared host/device infrastructure of the CTMRG library: status handling,
// the workspace arena, tensor views and launch helpers.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <stdexcept>
#include <vector>
#include <initializer_list>

#include "../../include/ctm_gb300.h"

namespace ctm {

// ----------------------------------------------------------------- errors
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define CTM_REQUIRE(cond, code, msg)                                     \
  do {                                                                    \
    if (!(cond)) throw ::ctm::Error((code), std::string(msg));            \
  } while (0)

#define CTM_CUDA(call)                                                    \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess)                                                \
      throw ::ctm::Error(CTM_ERR_CUDA, std::string(#call) + ": " +        \
                                           cudaGetErrorString(e_));       \
  } while (0)

// Every kernel launch of the library is followed by CTM_LAUNCH_CHECK(), which
// also counts it (ctm_kernel_launches()).
void count_launch();
#define CTM_LAUNCH_CHECK()            \
  do {                                \
    ::ctm::count_launch();            \
    CTM_CUDA(cudaGetLastError());     \
  } while (0)

// Kernel classes of the live timer (ctm_profile_*).
// Tags 0-1 bracket single kernels (work = FLOPs); tags 2-7 bracket spans of
// a projector computation or a renormalization (work = 0).
enum ProfileTag {
  kTagGettF64 = 0,
  kTagTcGemm = 1,
  kTagQuarter = 2,
  kTagRangeFinder = 3,
  kTagOrtho = 4,
  kTagSvd = 5,
  kTagProject = 6,
  kTagRenorm = 7,
  kTagGettF32 = 8,
  kTagTcDoubleLayer = 9
};
constexpr int kProfileTags = 10;

// Unit of the work figure of a named kernel class.
enum WorkUnit { kUnitFlop = 0, kUnitByte = 1 };

// Brackets one launch (or a span of launches) with CUDA events while
// profiling is on; `work` is the algorithmic FLOP (or byte) count.  The tag
// form adds to one of the classes above; the named form adds to a per-kernel
// table keyed by `name` (a string literal), with its work unit.
class KernelTimer {
 public:
  KernelTimer(cudaStream_t s, int tag, double work);
  KernelTimer(cudaStream_t s, const char* name, int unit, double work);
  ~KernelTimer();

 private:
  void start(int tag, const char* name, int unit, double work);
  cudaStream_t stream_;
  bool active_ = false;
  size_t idx_ = 0;
};

// Runs f(), turning exceptions into status codes for the C ABI.
template <class F>
int guarded(F&& f) {
  try {
    f();
    return CTM_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return CTM_ERR_INVALID;
  }
}

// ----------------------------------------------------------------- workspace
// Bump allocator over the caller's buffer.  In sizing mode (base == nullptr)
// it only records the high-water mark and hands out null pointers; every
// launch helper skips work when the context is sizing.
struct Ctx {
  cudaStream_t stream = nullptr;
  char* base = nullptr;
  size_t capacity = 0;
  size_t offset = 0;
  size_t high = 0;
  bool sizing() const { return base == nullptr; }

  template <class T>
  T* alloc(size_t count) {
    size_t bytes = ((count * sizeof(T)) + 255) & ~size_t(255);
    size_t off = offset;
    offset += bytes;
    if (offset > high) high = offset;
    if (sizing()) return nullptr;
    CTM_REQUIRE(offset <= capacity, CTM_ERR_WORKSPACE,
                "workspace too small: need at least " + std::to_string(offset) + " bytes");
    return reinterpret_cast<T*>(base + off);
  }
  size_t mark() const { return offset; }
  void release(size_t m) { offset = m; }
};

// Scoped release of arena allocations.
struct Scope {
  Ctx& c;
  size_t m;
  explicit Scope(Ctx& ctx) : c(ctx), m(ctx.mark()) {}
  ~Scope() { c.release(m); }
};

// Runs body(ctx) once in sizing mode or once for real, following the
// workspace protocol of the C ABI.
template <class F>
int with_workspace(void* ws, size_t* ws_bytes, cudaStream_t stream, F&& body) {
  return guarded([&] {
    CTM_REQUIRE(ws_bytes != nullptr, CTM_ERR_INVALID, "ws_bytes must not be NULL");
    Ctx ctx;
    ctx.stream = stream;
    if (ws == nullptr) {
      body(ctx);
      *ws_bytes = ctx.high + 256;
      return;
    }
    CTM_REQUIRE((reinterpret_cast<uintptr_t>(ws) & 255) == 0, CTM_ERR_INVALID,
                "workspace must be 256-byte aligned");
    ctx.base = static_cast<char*>(ws);
    ctx.capacity = *ws_bytes;
    body(ctx);
  });
}

// ----------------------------------------------------------------- tensor views
constexpr int kMaxDims = 8;

template <class T>
struct ViewT {
  T* p = nullptr;
  int nd = 0;
  int64_t shape[kMaxDims] = {0};
  int64_t stride[kMaxDims] = {0};

  ViewT() = default;
  ViewT(const T* ptr, std::initializer_list<int64_t> dims) {
    p = const_cast<T*>(ptr);
    nd = static_cast<int>(dims.size());
    int i = 0;
    for (int64_t v : dims) shape[i++] = v;
    int64_t s = 1;
    for (int j = nd - 1; j >= 0; --j) {
      stride[j] = s;
      s *= shape[j];
    }
  }
  int64_t numel() const {
    int64_t n = 1;
    for (int i = 0; i < nd; ++i) n *= shape[i];
    return n;
  }
  // Axis permutation without a copy: out.dim[i] = in.dim[perm[i]].
  ViewT permute(std::initializer_list<int> perm) const {
    ViewT v = *this;
    int i = 0;
    for (int a : perm) {
      v.shape[i] = shape[a];
      v.stride[i] = stride[a];
      ++i;
    }
    return v;
  }
  bool contiguous() const {
    int64_t s = 1;
    for (int j = nd - 1; j >= 0; --j) {
      if (shape[j] != 1 && stride[j] != s) return false;
      s *= shape[j];
    }
    return true;
  }
};

using View = ViewT<double>;
using ViewF = ViewT<float>;

// The site tensor A permuted by bond_permute(k): legs (l,u,r,d,p) rotated by k
// (acetn/ipeps/site_tensor.py:138-150).
inline View bond_permute(const double* A, int64_t D, int64_t d, int k) {
  View a(A, {D, D, D, D, d});
  k = ((k % 4) + 4) % 4;
  return a.permute({(0 + k) % 4, (1 + k) % 4, (2 + k) % 4, (3 + k) % 4, 4});
}

inline int grid_for(int64_t n, int threads, int cap = 152 * 16) {
  int64_t b = (n + threads - 1) / threads;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return static_cast<int>(b);
}

}  // namespace ctm
