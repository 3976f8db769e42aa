// Matrix product for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a host framework that
// hands a plugin only its input and output buffers and no allocator, or one
// whose own memory pool has reserved the device, so that an allocation by
// the plugin fails or fragments that pool.  ctm_matmul_mixed_noalloc serves
// them: it is the 3xBF16
// tensor-core product of ctm_matmul (CTM_PREC_MIXED) with its scratch (the
// BF16 operand copies and the split-K partial sums) placed in a file-scope
// device array instead of a caller workspace.
#include <mutex>
#include <unordered_map>

#include "engine.cuh"
#include "tc_gemm.cuh"

namespace ctm {
namespace {

// Every GPU that loads the library holds this array until the process exits.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the scratch array on the current device.  The host-side
// symbol is only a stand-in: the address is taken once per device with
// cudaGetSymbolAddress while that device is current.
char* noalloc_scratch() {
  static std::mutex mu;
  static std::unordered_map<int, char*> by_device;
  int dev = 0;
  CTM_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto it = by_device.find(dev);
  if (it != by_device.end()) return it->second;
  void* p = nullptr;
  CTM_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  CTM_REQUIRE(p != nullptr, CTM_ERR_CUDA, "cudaGetSymbolAddress returned NULL for the scratch array");
  by_device[dev] = static_cast<char*>(p);
  return static_cast<char*>(p);
}

void matmul_mixed_body(Ctx& c, const double* A, const double* B, double* C, int64_t M,
                       int64_t N, int64_t K) {
  const int64_t lda = tc_ld(K);
  bf16* ah = c.alloc<bf16>(size_t(M) * lda);
  bf16* al = c.alloc<bf16>(size_t(M) * lda);
  bf16* bh = c.alloc<bf16>(size_t(N) * lda);
  bf16* bl = c.alloc<bf16>(size_t(N) * lda);
  split_bf16(c, A, M, K, K, false, ah, al, lda);
  split_bf16(c, B, K, N, N, true, bh, bl, lda);
  TcOut out;
  out.add(TcKind::kF64, C, TcLayout::rows(M, N, N));
  tc_gemm(c, TcOperand{ah, al, M, K, lda}, TcOperand{bh, bl, N, K, lda}, TcMode::kBf16x3, out);
}

}  // namespace
}  // namespace ctm

using namespace ctm;

extern "C" int ctm_matmul_mixed_noalloc(const double* A, const double* B, double* C, int64_t M,
                                        int64_t N, int64_t K, ctm_stream_t stream) {
  return guarded([&] {
    CTM_REQUIRE(M >= 1 && N >= 1 && K >= 1, CTM_ERR_INVALID, "bad size");
    CTM_REQUIRE(A != nullptr && B != nullptr && C != nullptr, CTM_ERR_INVALID, "NULL pointer");
    Ctx sizing;
    sizing.stream = reinterpret_cast<cudaStream_t>(stream);
    matmul_mixed_body(sizing, A, B, C, M, N, K);
    CTM_REQUIRE(sizing.high <= kNoAllocScratchBytes, CTM_ERR_WORKSPACE,
                "ctm_matmul_mixed_noalloc: this product needs " + std::to_string(sizing.high) +
                    " bytes of scratch; the static scratch holds " +
                    std::to_string(kNoAllocScratchBytes) + " bytes (use ctm_matmul with a workspace)");
    Ctx c;
    c.stream = reinterpret_cast<cudaStream_t>(stream);
    c.base = noalloc_scratch();
    c.capacity = kNoAllocScratchBytes;
    matmul_mixed_body(c, A, B, C, M, N, K);
  });
}
