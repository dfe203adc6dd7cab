// negf_zgemm_noalloc: the tensor-core sliced complex GEMM for callers that must not
// allocate device memory.
//
// Who needs it: code whose device memory belongs to another allocator (a framework's
// caching pool that must see every byte, or a serving process whose HBM budget is fixed
// at start-up), and latency-critical loops that cannot afford cudaMalloc/cudaFree, which
// synchronise the whole device.  negf_zgemm allocates its slice planes on every call; this
// variant keeps them in one static device array instead.
//
// The scratch is a file-scope __device__ array of NEGF_NOALLOC_SCRATCH_BYTES (about 26 MB).
// A GPU holds it from the first negf_zgemm_noalloc call on that device (or from library
// load, when CUDA loads modules eagerly) until the process exits.  It bounds the problem
// size: m, n, k <= NEGF_NOALLOC_MAX_DIM and slices <= NEGF_NOALLOC_MAX_SLICES.  All calls
// share it and it keeps the previous call's contents, so calls that overlap on the GPU
// (different streams or host threads without ordering) race on it; calls must be
// serialised by the caller.  The slicing kernels overwrite every scratch byte a call reads,
// and the device error flag is cleared at the start of each call.
//
// Host code may not use the array's name as a device address (on the host it names a
// shadow object): the first call on each device, with that device current, resolves the
// device address with cudaGetSymbolAddress and caches it.
//
// Every call ends by copying the device error flag to the host and synchronising
// `stream`, so it blocks until the product is complete and cannot be recorded into a CUDA
// graph.  The first beta = 0 call of each shape with K' = 2k <= 800 also runs the kernel
// variant choice of the tensor-core GEMM: it launches the product nine times on `stream`
// and waits for their events before it returns.
#include <mutex>

#include "engine.h"
#include "zgemm_tc.h"

namespace {

constexpr int kMaxDim = NEGF_NOALLOC_MAX_DIM;
constexpr int kMaxSlices = NEGF_NOALLOC_MAX_SLICES;
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
// layout: A slices (2m rows of 2k) | B slices (n rows of 2k) | row exponents | column
// exponents | error flag
constexpr size_t kABytes = align256(sizeof(__nv_bfloat16) * (size_t)kMaxSlices * 2 * kMaxDim * 2 * kMaxDim);
constexpr size_t kBBytes = align256(sizeof(__nv_bfloat16) * (size_t)kMaxSlices * kMaxDim * 2 * kMaxDim);
constexpr size_t kEBytes = align256(sizeof(int) * (size_t)kMaxDim);
constexpr size_t kScratchBytes = kABytes + kBBytes + 2 * kEBytes + 256;
static_assert(kScratchBytes <= NEGF_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the declared size");

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NEGF_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_scratch_dev[kMaxDevices] = {};

// device address of the scratch on the current device (resolved once per device)
int scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  NEGF_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return NEGF_EINVAL;
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    NEGF_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_scratch_dev[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_dev[dev];
  return NEGF_OK;
}

}  // namespace

extern "C" int negf_zgemm_noalloc(int32_t slices, int32_t m, int32_t n, int32_t k, const double* alpha,
                                  const double* A, int32_t lda, const double* B, int32_t ldb, const double* beta,
                                  double* C, int32_t ldc, void* stream) {
  using namespace negf;
  if (!alpha || !beta || !A || !B || !C) return NEGF_EINVAL;
  if (m <= 0 || n <= 0 || k <= 0 || lda < m || ldb < k || ldc < m) return NEGF_EINVAL;
  if (slices < 3 || slices > 8 || !tc_supported_slices(slices)) return NEGF_EINVAL;
  if (m > kMaxDim || n > kMaxDim || k > kMaxDim || slices > kMaxSlices) return NEGF_ESCRATCH;
  unsigned char* base = nullptr;
  NEGF_TRY(scratch_for_current_device(&base));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int* err = reinterpret_cast<int*>(base + kABytes + kBBytes + 2 * kEBytes);
  NEGF_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  SlicedOperand oa, ob;
  oa.data = reinterpret_cast<__nv_bfloat16*>(base);
  ob.data = reinterpret_cast<__nv_bfloat16*>(base + kABytes);
  oa.exps = reinterpret_cast<int*>(base + kABytes + kBBytes);
  ob.exps = reinterpret_cast<int*>(base + kABytes + kBBytes + kEBytes);
  oa.data_bytes = kABytes; ob.data_bytes = kBBytes;
  oa.exps_count = ob.exps_count = (size_t)kMaxDim;
  const double2 al = make_double2(alpha[0], alpha[1]), be = make_double2(beta[0], beta[1]);
  NEGF_TRY(slice_a(reinterpret_cast<const double2*>(A), lda, 0, m, k, 1, slices, oa, st));
  NEGF_TRY(slice_b(reinterpret_cast<const double2*>(B), ldb, 0, k, n, 1, slices, ob, st));
  NEGF_TRY(zgemm_tc(oa, ob, al, be, reinterpret_cast<double2*>(C), ldc, 0, err, st));
  int herr = 0;
  NEGF_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  NEGF_CUDA_TRY(cudaStreamSynchronize(st));
  return herr ? NEGF_ETIMEDOUT : NEGF_OK;
}
