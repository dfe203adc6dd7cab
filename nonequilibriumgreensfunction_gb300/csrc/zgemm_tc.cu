// Complex GEMM on the tcgen05 tensor cores with exact integer-sliced BF16 operands.
//
// C = alpha * A * B + beta * C for batches of complex FP64 matrices (column-major).
//
// Number format.  Every row i of A is scaled by 2^-e_i (e_i from frexp of the row's
// largest |re|,|im|) and every column j of B by 2^-f_j, so all scaled entries lie in
// (-1, 1).  An entry a is then cut into S integer slices of 7 bits,
//     a = 2^-6 (s_0 + 2^-7 (s_1 + 2^-7 (s_2 + ...))),   s_p in [-64, 64],
// each of which is exact in BF16.  The complex product is one real product of K' = 2K with
// the complex rows of A expanded into pairs of real rows,
//     row 2i:   [Ar(i,:)  -Ai(i,:)] . [Br(:,j); Bi(:,j)] = Cr(i,j)
//     row 2i+1: [Ai(i,:)   Ar(i,:)] . [Br(:,j); Bi(:,j)] = Ci(i,j),
// so the MMA's M side covers the 2M real rows (M = 400: 800 rows in 7 tiles of 128, against
// 4 tiles of 128 for 400 rows, 22% of them padding) and its N side the N complex columns.
// The slice products S_p T_q are integer matrices with |entries| <= K' * 2^12.  The MMAs
// of one anti-diagonal d = p + q (at most S pairs) accumulate into one FP32 TMEM
// accumulator; for d < 5 and K' <= 800 every partial sum stays below (d+1) 800 2^12 < 2^24,
// so those accumulators are EXACT (products of 7-bit integers and their sums are
// representable).  For 800 < K' <= 1600 (M up to 800) the K blocks are split in two halves
// of at most 800, each accumulated into its own set of TMEM accumulators and summed in
// int64 by the epilogue, so the same argument holds per half; K' > 1600 is refused.
// Higher diagonals carry weight <= 2^-35 and their rounding is far below FP64 epsilon of
// the leading term.  The epilogue recombines sum_d acc_d 2^(7(S-1-d)) in int64 (two words
// for S >= 7, each converted and then added), converts to FP64 and scales by
// 2^(e_i + f_j - 12 - 7(S-1)).  Accuracy
// is set by S: truncation <= 2^-7S of the row/column maximum (S = 4: 4e-9, S = 5: 3e-11,
// S = 7: 2e-15).
//
// Kernel structure (one 128 x NT output tile per CTA, 10 warps):
//   warp 0      TMA producer: for each K block of 32, S A-slices (128 x 32) and S B-slices
//               (NT x 32) into a ring of shared-memory stages (SWIZZLE_64B, K-major).
//   warp 1      TMEM allocation and the single-thread tcgen05.mma issue loop (one MMA per
//               A slice, spanning the B slices it pairs with); commits release the stage
//               and, at the end, signal the epilogue.
//   warps 2-9   epilogue, two warps per TMEM lane quarter taking the tile's column chunks
//               in turn: tcgen05.ld of the S accumulators, FP64 recombination; lanes
//               2i and 2i+1 hold the real and imaginary parts of C row i and exchange
//               them with one shuffle, the even lane storing the even columns and the
//               odd lane the odd ones.
// Every mbarrier wait is bounded; on expiry the kernel records an error code and returns
// after draining its own TMA copies and freeing its TMEM.
//
// Replaces, in the mixed form, the ZGEMM calls of Source/Recursive_Greens.F90 and the
// G Gamma products of Source/Calculate_Gnp.F90.
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <map>
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "negf_internal.cuh"
#include "zgemm_tc.h"

namespace negf {

namespace {

// Epilogue warps of both kernels: two per TMEM lane quarter (a warp reaches the 32 lanes of
// quarter warp % 4), which split the tile's columns chunk by chunk.  The epilogue's work per
// output (S accumulator loads, integer recombination, the exact conversion to FP64, the beta
// term) is long dependent integer code; with one warp per sub-partition nothing hides its
// latency, and at 3 slices, whose K loop is short, it outlasted the MMAs of the next tile.
constexpr int TC_EPI_WARPS = 8;
constexpr int TC_THREADS = 64 + 32 * TC_EPI_WARPS;   // producer, MMA issuer, epilogue
#ifndef TC_BK
#define TC_BK 32
#endif
constexpr int BK = TC_BK;           // K elements (bf16) per stage row: 64 bytes with SWIZZLE_64B
constexpr int ROW_BYTES = BK * 2;   // (32 bytes with SWIZZLE_32B when BK = 16)
static_assert(BK == 32 || BK == 16, "stage rows of 64 or 32 bytes");
// tcgen05 shared-memory descriptor swizzle field: 4 = 64-byte, 6 = 32-byte swizzling
constexpr uint64_t DESC_SWIZZLE = BK == 32 ? 4 : 6;
constexpr int TILE_M = 128;
constexpr uint32_t kWaitLimit = 1u << 22;   // ~1 s of polling

// ---------------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred P1;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, P1;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: true on success, false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// SWIZZLE_64B, K-major shared-memory matrix descriptor (tcgen05 "matrix descriptor"):
// start address >> 4 at [0,14), leading byte offset >> 4 at [16,30) (unused for swizzled
// K-major), stride byte offset >> 4 at [32,46) = 8 rows * 64 B, version 1 at [46,48),
// layout type at [61,64) = 4 (64-byte swizzle).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)(16 >> 4) << 16;
  d |= (uint64_t)((8 * ROW_BYTES) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= DESC_SWIZZLE << 61;
  return d;
}

// instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16 (bits 7-9,
// 10-12 = 1), both K-major, N >> 3 at [17,23), M >> 4 at [24,29)
__host__ __device__ constexpr uint32_t make_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accum));
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// An integer-valued FP32 accumulator as an int, with integer operations only.  Every TMEM
// accumulator holds a sum of products of 7-bit integers, |sum| <= S K' 2^12 < 2^31, and is
// integer-valued even where it rounded (an FP32 of magnitude >= 2^24 is an even integer),
// so value = mantissa * 2^(exponent - 150) is exact in an int.  The FP32 -> int64
// conversion instruction would run on the FP64 pipe, which on this part issues about two
// operations per clock per SM and otherwise bounds the epilogue.
__device__ __forceinline__ int acc_to_int(uint32_t bits) {
  const int e = (int)((bits >> 23) & 0xFFu) - 150;
  const int mant = (int)((bits & 0x7FFFFFu) | 0x800000u);
  const int mag = e >= 0 ? (mant << e) : (e > -24 ? (mant >> -e) : 0);
  return (bits >> 31) ? -mag : mag;
}

// u * 2^scale with the given sign bit as a double, rounded to nearest even, built from
// integer operations only (results below the normal range flush to zero)
__device__ __forceinline__ double scaled_uint_to_double(unsigned long long u, unsigned long long sign, int scale) {
  int top = 63 - __clzll((long long)u);
  unsigned long long mant;
  if (top <= 52) {
    mant = u << (52 - top);
  } else {
    const int sh = top - 52;
    const unsigned long long rem = u & ((1ULL << sh) - 1), halfu = 1ULL << (sh - 1);
    mant = u >> sh;
    if (rem > halfu || (rem == halfu && (mant & 1))) {
      ++mant;
      if (mant >> 53) { mant >>= 1; ++top; }
    }
  }
  const int ex = top + scale + 1023;
  if (ex <= 0) return __longlong_as_double((long long)sign);
  if (ex >= 2047) return __longlong_as_double((long long)(sign | (0x7FFULL << 52)));
  return __longlong_as_double((long long)(sign | ((unsigned long long)ex << 52) | (mant & ((1ULL << 52) - 1))));
}

// v * 2^scale as a double, rounded to nearest even, built from integer operations only
__device__ __forceinline__ double scaled_int_to_double(long long v, int scale) {
  if (v == 0) return 0.0;
  const unsigned long long sign = v < 0 ? (1ULL << 63) : 0ULL;
  return scaled_uint_to_double(v < 0 ? (unsigned long long)(-v) : (unsigned long long)v, sign, scale);
}

// sum_d acc_d 2^(7(S-1-d)) 2^sc from the words hi (d < DH, weight 2^(7(S-DH)) relative to lo)
// and lo (d >= DH).  For S >= 7 the two words are rounded separately and added in FP64: an
// exact 128-bit join with one rounding measured slower (568 against 596 TFLOP/s at 7 slices)
// than the one FP64 addition per output it saves.
template <int S, int DH>
__device__ __forceinline__ double recombine(long long hi, long long lo, int sc) {
  if constexpr (DH == S) {
    return scaled_int_to_double(hi, sc);
  } else {
    return scaled_int_to_double(hi, sc + 7 * (S - DH)) + scaled_int_to_double(lo, sc);
  }
}

// TMEM loads without the wait: issue several, then one tcgen05.wait::ld
__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------------
// slicing
// ---------------------------------------------------------------------------------
// Slices of x at scale exponent e (|x| < 2^e): the fixed-point integer
// F = round(x 2^(6 + 7(S-1) - e)), |F| <= 2^(6 + 7(S-1)) <= 2^55, built from the bits of x
// with integer operations only (GB300's FP64 pipe is 1/64 of its FP32 rate), then written
// as balanced base-128 digits: F = sum_p s_p 128^(S-1-p), lower digits in [-64, 63], the
// top digit in [-64, 64].  Every digit is exact in BF16; the truncation is <= 2^-7S of 2^e.
template <int S>
__device__ __forceinline__ void slice_value(double x, int e, __nv_bfloat16 (&out)[S]) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((bits >> 52) & 0x7FF);
  long long F = 0;
  if (ex != 0 && ex != 0x7FF) {                      // zero and subnormals slice to 0
    const unsigned long long m = (bits & ((1ULL << 52) - 1)) | (1ULL << 52);   // x = m 2^(ex - 1075)
    const int r = e - (ex - 1075) - (6 + 7 * (S - 1));                          // F = m 2^-r, r >= 46 - 7(S-1)
    if (r <= 0) F = (long long)(m << (-r));                                      // S = 8: exact, |F| < 2^55
    else if (r < 64) F = (long long)((m + (1ULL << (r - 1))) >> r);
    if (bits >> 63) F = -F;
  }
  // Balanced digits from the bottom, d_p = F_p - 128 floor((F_p + 64) / 128), in 32-bit
  // arithmetic: the low 28 bits give up to four digits and a carry into F >> 28 (|F| < 2^55,
  // so that part fits an int).  The digits are unique, so this equals the 64-bit recurrence.
  int hi = (int)(F >> 28);
  int lo = (int)(F & ((1LL << 28) - 1));
  constexpr int NL = S - 1 < 4 ? S - 1 : 4;   // digits taken from the low word
#pragma unroll
  for (int t = 0; t < NL; ++t) {
    const int nx = (lo + 64) >> 7;
    out[S - 1 - t] = __float2bfloat16_rn((float)(lo - nx * 128));
    lo = nx;
  }
  if constexpr (S - 1 < 4) {
    // S <= 4: what is left of the low word and the high word form the top digit
    out[0] = __float2bfloat16_rn((float)(lo + hi * (1 << (28 - 7 * NL))));
  } else {
    hi += lo;   // carry out of the low 28 bits
#pragma unroll
    for (int p = S - 1 - NL; p >= 1; --p) {
      const int nx = (hi + 64) >> 7;
      out[p] = __float2bfloat16_rn((float)(hi - nx * 128));
      hi = nx;
    }
    out[0] = __float2bfloat16_rn((float)hi);
  }
}

// Row and column maxima are taken on bit patterns: |x| as an unsigned integer orders like
// |x| itself, NaN maps to 0 as fmax would ignore it, and the exponent of the maximum is
// read from its bits -- all integer operations, none on GB300's slow FP64 pipe.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  const unsigned long long a = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFULL;
  return a > 0x7FF0000000000000ULL ? 0ULL : a;
}

// e with m = f 2^e, f in [0.5, 1) (frexp), for m = the double with bit pattern a >= 0;
// 0 for zero and infinity
__device__ __forceinline__ int scale_exponent(unsigned long long a) {
  const int E = (int)(a >> 52);
  if (a == 0 || E == 0x7FF) return 0;
  if (E == 0) {   // subnormal maximum: its row slices to zero whatever e is
    int e;
    frexp(__longlong_as_double((long long)a), &e);
    return e;
  }
  return E - 1022;
}

// row exponents of A (M x K complex, column-major): a CTA covers 32 rows, its 8 thread
// rows stride over the columns (coalesced 512-byte row segments), reduced in shared memory
__global__ void row_exp_kernel(const double2* A, int lda, long long sA, int m, int k, int* ea) {
  __shared__ unsigned long long part[8][32];
  const int b = blockIdx.y;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = blockIdx.x * 32 + tx;
  const double2* Ab = A + (long long)b * sA;
  unsigned long long mx = 0;
  if (i < m)
    for (int kk = ty; kk < k; kk += 8) {
      const double2 v = Ab[(long long)kk * lda + i];
      mx = max(mx, max(abs_bits(v.x), abs_bits(v.y)));
    }
  part[ty][tx] = mx;
  __syncthreads();
  if (ty == 0 && i < m) {
    for (int q = 1; q < 8; ++q) mx = max(mx, part[q][tx]);
    ea[(long long)b * m + i] = scale_exponent(mx);
  }
}

// A slices, K-major, two real rows per complex row i (kp = 2*half):
//     out[((b*S + p)*2m + 2i)*kp + k]   = [Ar(i, :), -Ai(i, :)]
//     out[((b*S + p)*2m + 2i+1)*kp + k] = [Ai(i, :),  Ar(i, :)],
// zero in the padding k in [K, half).  A tile of 32 rows x 64 k is staged through shared
// memory (coalesced column-major reads); each thread then slices one row x 8 consecutive
// k and writes 16-byte vectors.
template <int S>
__global__ void __launch_bounds__(256) slice_a_kernel(const double2* A, int lda, long long sA, int m, int k,
                                                      const int* ea, __nv_bfloat16* out, int half) {
  __shared__ double2 tile[64][33];
  const int kp = 2 * half;
  const int b = blockIdx.z;
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 64;
  const double2* Ab = A + (long long)b * sA;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int kk = k0 + ty + 8 * r, i = i0 + tx;
    tile[ty + 8 * r][tx] = (i < m && kk < k) ? Ab[(long long)kk * lda + i] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  const int row = threadIdx.x >> 3, kg = threadIdx.x & 7;
  const int i = i0 + row, kb = k0 + 8 * kg;
  if (i >= m || kb >= half) return;
  const int e = ea[(long long)b * m + i];
  __align__(16) __nv_bfloat16 sr[S][8], si[S][8], ni[S][8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const double2 v = tile[8 * kg + q][row];
    __nv_bfloat16 a[S], c[S];
    slice_value<S>(v.x, e, a);
    slice_value<S>(v.y, e, c);
#pragma unroll
    for (int p = 0; p < S; ++p) { sr[p][q] = a[p]; si[p][q] = c[p]; ni[p][q] = __hneg(c[p]); }
  }
#pragma unroll
  for (int p = 0; p < S; ++p) {
    __nv_bfloat16* re_row = out + ((long long)(b * S + p) * 2 * m + 2 * i) * kp;
    __nv_bfloat16* im_row = re_row + kp;
    *reinterpret_cast<uint4*>(re_row + kb) = *reinterpret_cast<const uint4*>(sr[p]);
    *reinterpret_cast<uint4*>(re_row + half + kb) = *reinterpret_cast<const uint4*>(ni[p]);
    *reinterpret_cast<uint4*>(im_row + kb) = *reinterpret_cast<const uint4*>(si[p]);
    *reinterpret_cast<uint4*>(im_row + half + kb) = *reinterpret_cast<const uint4*>(sr[p]);
  }
}

// B slices: one warp per column j of B (K x N complex, column-major).  Row j of the
// K-major operand is [Br(:,j); Bi(:,j)], zero in the padding: out[((b*S + p)*n + j)*kp + k].
// Chunks of 256 k are read coalesced into shared memory; each lane then slices 8
// consecutive k and writes 16-byte vectors.
template <int S>
__global__ void __launch_bounds__(256) slice_b_kernel(const double2* B, int ldb, long long sB, int k, int n, int* fb,
                                                      __nv_bfloat16* out, int half) {
  __shared__ double2 chunk[8][256];
  const int kp = 2 * half;
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * 8 + warp;
  if (j >= n) return;   // whole warps leave together; no block-wide barrier below
  const double2* col = B + (long long)b * sB + (long long)j * ldb;
  unsigned long long mx = 0;
  for (int kk = lane; kk < k; kk += 32) mx = max(mx, max(abs_bits(col[kk].x), abs_bits(col[kk].y)));
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  const int e = scale_exponent(mx);
  if (lane == 0) fb[(long long)b * n + j] = e;
  double2* ch = chunk[warp];
  for (int c0 = 0; c0 < half; c0 += 256) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int kk = c0 + lane + 32 * q;
      ch[lane + 32 * q] = kk < k ? col[kk] : make_double2(0.0, 0.0);
    }
    __syncwarp();
    const int kb = c0 + 8 * lane;
    if (kb < half) {
      __align__(16) __nv_bfloat16 rr[S][8], ri[S][8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const double2 v = ch[8 * lane + q];
        __nv_bfloat16 a[S], c[S];
        slice_value<S>(v.x, e, a);
        slice_value<S>(v.y, e, c);
#pragma unroll
        for (int p = 0; p < S; ++p) { rr[p][q] = a[p]; ri[p][q] = c[p]; }
      }
#pragma unroll
      for (int p = 0; p < S; ++p) {
        __nv_bfloat16* rowp = out + ((long long)(b * S + p) * n + j) * kp;
        *reinterpret_cast<uint4*>(rowp + kb) = *reinterpret_cast<const uint4*>(rr[p]);
        *reinterpret_cast<uint4*>(rowp + half + kb) = *reinterpret_cast<const uint4*>(ri[p]);
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------
// the MMA kernel
// ---------------------------------------------------------------------------------
// MINB = CTAs resident per SM: 1 (deep pipeline, up to 200 KB of stages) or 2 (two CTAs
// share an SM, so one's prologue/epilogue overlaps the other's MMAs; <= 110 KB of stages
// and <= 256 TMEM columns each).  KS = accumulator sets along K: 2 splits the K blocks in
// two halves of at most 800 K' each (exact accumulators for 800 < K' <= 1600).
template <int S, int NT, int MINB = 1, int KS = 1>
struct TcCfg {
  static constexpr int A_TILE = TILE_M * ROW_BYTES;            // bytes of one A slice tile
  static constexpr int B_TILE = NT * ROW_BYTES;                // bytes of one B slice tile
  static constexpr int STAGE = S * (A_TILE + B_TILE);
  static constexpr int BUDGET = MINB == 2 ? 110 * 1024 : 200 * 1024;
#ifndef TC_MAX_STAGES
#define TC_MAX_STAGES 4
#endif
  static constexpr int STAGES = BUDGET / STAGE > TC_MAX_STAGES ? TC_MAX_STAGES : BUDGET / STAGE;
  static constexpr int SMEM = STAGES * STAGE + 1024 + 256 + 4 * NT;   // + alignment, barriers, exponents
  static constexpr int TMEM_COLS_USED = KS * S * NT;
  static constexpr int TMEM_COLS = TMEM_COLS_USED <= 32 ? 32 : TMEM_COLS_USED <= 64 ? 64
                                 : TMEM_COLS_USED <= 128 ? 128 : TMEM_COLS_USED <= 256 ? 256 : 512;
  static_assert(STAGES >= 2, "at least two stages");
  static_assert(TMEM_COLS_USED <= 512 / MINB, "TMEM holds 512 columns per SM");
  static_assert(NT % 16 == 0 && NT >= 16 && NT <= 256, "UMMA N");
  static_assert(KS == 1 || KS == 2, "one or two accumulator sets along K");
};

// The MMAs of one stage.  Accumulator d (TMEM columns [d NT, (d+1) NT) from acc_base) sums
// the slice pairs (p, q) with p + q = d.  The stage's B slice tiles lie back to back (slice q
// at q * B_TILE, NT rows each, one K-major SWIZZLE_64B layout whose 512-byte atoms continue
// across the tiles), so for one A slice p the B slices q0 .. q0+qn-1 form one (qn NT)-row
// operand, and one MMA of N = qn NT adds the pairs (p, q0), ..., (p, q0+qn-1) into the
// accumulators p+q0 .. p+q0+qn-1, which are contiguous in TMEM.  Per K step of 16 that is S
// MMAs (a few more where S NT > 256, the largest N at M = 128) instead of S (S+1)/2, and each
// A slice is read from shared memory once instead of S - p times.  Every accumulator still
// receives its pairs in the same order (p ascending), and its partial sums are the same
// exact integers.  `overwrite`: the first K block of an accumulator set, whose first MMA per
// accumulator (p = 0, first K step) replaces what TMEM held.
template <int S, int NT, int A_TILE, int B_TILE>
__device__ __forceinline__ void issue_stage_mmas(uint32_t acc_base, uint64_t da0, uint64_t db0, bool overwrite) {
  constexpr int QMAX = 256 / NT;
  static_assert(QMAX >= 1, "one B slice per MMA at least");
#pragma unroll
  for (int p = 0; p < S; ++p) {
#pragma unroll
    for (int q0 = 0; q0 < S - p; q0 += QMAX) {
      const int qn = (S - p - q0) < QMAX ? (S - p - q0) : QMAX;
      const uint32_t idesc = make_idesc(TILE_M, qn * NT);
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        const uint64_t da = da0 + (uint64_t)((p * A_TILE + kk * 32) >> 4);
        const uint64_t db = db0 + (uint64_t)((q0 * B_TILE + kk * 32) >> 4);
        const uint32_t acc = (!overwrite || p > 0 || kk > 0) ? 1u : 0u;
        tc_mma(acc_base + (uint32_t)((p + q0) * NT), da, db, idesc, acc);
      }
    }
  }
}

struct TcArgs {
  int m, n, kp;            // rows of C, complex columns of C, K' = 2K
  int batch;
  long long rowsA;         // rows of one (item, slice) plane in the A map (= 2m)
  long long rowsB;         // rows of one (item, slice) plane in the B map (= n)
  int planesA, planesB;    // slice planes stored per item (>= S: the leading S are used)
  const int* ea;           // [batch][m]
  const int* fb;           // [batch][n]
  double2* C; int ldc; long long sC;
  double2 alpha, beta;
  int alpha_one;           // alpha == 1
  int beta_kind;           // 0: beta == 0, 1: beta == 1, 2: general
  int* err;
};

// Stores one chunk of CW tile columns.  Each lane holds, for its real output row, the exact
// integer sums of the real part (even row, part 0) or the imaginary part (odd row, part 1)
// of C(row / 2, col0 + c); it converts them to doubles, and lanes 2i and 2i+1 swap what
// the other one stores -- the even lane stores the even columns, the odd lane the odd
// ones -- with one shuffle per pair of columns.  Every lane of the warp must call it (the
// shuffles); `valid` masks the stores.
template <int S, int DH, int CW>
__device__ __forceinline__ void store_chunk(const long long (&hi)[CW], const long long (&lo)[CW], const int* cexp,
                                            int e_row, int part, int row, int col0, bool valid, const TcArgs& a,
                                            double2* Cb) {
  double v[CW];
#pragma unroll
  for (int c = 0; c < CW; ++c) v[c] = recombine<S, DH>(hi[c], lo[c], e_row + cexp[c] - 12 - 7 * (S - 1));
  double recv[CW / 2];   // the partner's half of the columns this lane stores
#pragma unroll
  for (int h = 0; h < CW / 2; ++h) recv[h] = __shfl_xor_sync(0xffffffffu, part ? v[2 * h] : v[2 * h + 1], 1);
  if (!valid) return;
  double2 cin[CW / 2];
  if (a.beta_kind != 0) {                // issue all loads of the chunk before any store
#pragma unroll
    for (int h = 0; h < CW / 2; ++h) {
      const int col = col0 + 2 * h + part;
      cin[h] = col < a.n ? Cb[(long long)col * a.ldc + row] : make_double2(0.0, 0.0);
    }
  }
#pragma unroll
  for (int h = 0; h < CW / 2; ++h) {
    const int col = col0 + 2 * h + part;
    if (col >= a.n) continue;
    const double mine = part ? v[2 * h + 1] : v[2 * h];
    double2 out = part ? make_double2(recv[h], mine) : make_double2(mine, recv[h]);
    if (!a.alpha_one) out = cmul(a.alpha, out);
    if (a.beta_kind == 1) out = cadd(out, cin[h]);
    else if (a.beta_kind == 2) out = cadd(out, cmul(a.beta, cin[h]));
    Cb[(long long)col * a.ldc + row] = out;
  }
}

template <int S, int NT, int MINB, int KS>
__global__ void __launch_bounds__(TC_THREADS, MINB)
    zgemm_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, TcArgs a) {
  using Cfg = TcCfg<S, NT, MINB, KS>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Cfg::STAGES * Cfg::STAGE);
  uint64_t* empty = full + Cfg::STAGES;
  uint64_t* done = empty + Cfg::STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);
  int* col_exp = abort_flag + 1;   // NT column exponents of this tile

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tm = blockIdx.x, tn = blockIdx.y, b = blockIdx.z;
  const int nk = (a.kp + BK - 1) / BK;
  // K blocks [0, ksplit) accumulate into set 0, [ksplit, nk) into set 1 (KS = 2 only)
  const int ksplit = KS == 1 ? nk : (nk + 1) / 2;
  const int nsets = (KS == 2 && ksplit < nk) ? 2 : 1;

  if (threadIdx.x == 0) {
    for (int s = 0; s < Cfg::STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"((uint32_t)Cfg::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
      // ---- TMA producer
      const int a_row0 = tm * TILE_M;
      const int b_row0 = tn * NT;
      int issued = 0;
      for (int kb = 0; kb < nk; ++kb) {
        const int st = kb % Cfg::STAGES;
        if (!mbar_wait(&empty[st], ((kb / Cfg::STAGES) & 1) ^ 1)) {
          atomicExch(abort_flag, 1);
          if (a.err) atomicCAS(a.err, 0, 1);
          break;
        }
        if (*((volatile int*)abort_flag)) break;
        uint8_t* sa = smem + st * Cfg::STAGE;
        uint8_t* sb = sa + S * Cfg::A_TILE;
        mbar_expect_tx(&full[st], (uint32_t)Cfg::STAGE);
#pragma unroll
        for (int p = 0; p < S; ++p) {
          tma_load_2d(sa + p * Cfg::A_TILE, &mapA, kb * BK,
                      (int)((long long)(b * a.planesA + p) * a.rowsA + a_row0), &full[st]);
          tma_load_2d(sb + p * Cfg::B_TILE, &mapB, kb * BK,
                      (int)((long long)(b * a.planesB + p) * a.rowsB + b_row0), &full[st]);
        }
        ++issued;
      }
      // drain: every issued stage must have landed before the CTA may exit
      for (int kb = (issued > Cfg::STAGES ? issued - Cfg::STAGES : 0); kb < issued; ++kb)
        mbar_wait(&full[kb % Cfg::STAGES], (kb / Cfg::STAGES) & 1);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issue
      for (int kb = 0; kb < nk; ++kb) {
        const int st = kb % Cfg::STAGES;
        if (!mbar_wait(&full[st], (kb / Cfg::STAGES) & 1)) {
          atomicExch(abort_flag, 1);
          if (a.err) atomicCAS(a.err, 0, 2);
          break;
        }
        tc_fence_after();
        const uint32_t sa = smem_u32(smem + st * Cfg::STAGE);
        const uint32_t sb = sa + S * Cfg::A_TILE;
        // descriptors of the stage's first tiles; the others differ only in the start
        // address field (bits 0-13, address >> 4), and shared addresses stay below 2^18,
        // so a tile's descriptor is the base plus its byte offset >> 4
        const uint64_t da0 = make_desc(sa), db0 = make_desc(sb);
        const bool second = KS == 2 && kb >= ksplit;
        const uint32_t acc_base = tmem + (second ? (uint32_t)(S * NT) : 0u);
        const bool first_kb = kb == (second ? ksplit : 0);   // the set's first K block overwrites it
        issue_stage_mmas<S, NT, Cfg::A_TILE, Cfg::B_TILE>(acc_base, da0, db0, first_kb);
        tc_commit(&empty[st]);
      }
      tc_commit(done);
    }
  } else {
    // ---- epilogue: warps 2..5 -> TMEM lane quarter (warp % 4); lane l of the tile is real
    // output row tm*128 + l.  While the MMAs run, stage the tile's column exponents in
    // shared memory.
    const int quarter = warp & 3;
    for (int c = threadIdx.x - 64; c < NT; c += 32 * TC_EPI_WARPS) {
      const int col = tn * NT + c;
      col_exp[c] = col < a.n ? a.fb[(long long)b * a.n + col] : 0;
    }
    asm volatile("bar.sync 1, %0;" ::"n"(32 * TC_EPI_WARPS) : "memory");   // the epilogue warps only
    const bool ok = mbar_wait(done, 0);
    if (!ok && a.err) atomicCAS(a.err, 0, 3);
    tc_fence_after();
    const int rr = tm * TILE_M + quarter * 32 + lane;
    const int row = rr >> 1, part = rr & 1;          // C row, real (0) or imaginary (1) part
    const bool aborted = !ok || *((volatile int*)abort_flag);
    const int e_row = (row < a.m) ? a.ea[(long long)b * a.m + row] : 0;
    double2* Cb = a.C + (long long)b * a.sC;
    constexpr int CW = (S >= 7 || MINB == 2 || KS == 2 || NT % 16 != 0) ? 8 : 16;   // fp32 columns per chunk
    constexpr int NGRP = TC_EPI_WARPS / 4;   // warps per lane quarter, taking chunks in turn
    const int grp = (warp - 2) >> 2;
#pragma unroll 1
    for (int c0 = grp * CW; c0 < NT; c0 += NGRP * CW) {
      // exact recombination of the diagonal accumulators (integer-valued FP32) in int64:
      // hi = sum_{d<DH} acc_d 2^(7(DH-1-d)), lo = sum_{d>=DH} acc_d 2^(7(S-1-d))
      constexpr int DH = S <= 6 ? S : 3;   // S <= 6 fits one int64; S >= 7 splits
      long long hi[CW], lo[CW];
#pragma unroll
      for (int i = 0; i < CW; ++i) { hi[i] = 0; lo[i] = 0; }
      if (ok) {
        // all S accumulator reads of this chunk (per K set) in flight together, one wait;
        // the sets' exact integer values add in int64
#pragma unroll 1
        for (int set = 0; set < nsets; ++set) {
          uint32_t raw[S][CW];
#pragma unroll
          for (int d = 0; d < S; ++d) {
            const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(set * S * NT + d * NT + c0);
#pragma unroll
            for (int h = 0; h < CW / 8; ++h) {
              uint32_t (&r8)[8] = *reinterpret_cast<uint32_t(*)[8]>(&raw[d][8 * h]);
              tmem_ld8_nowait(ta + 8 * h, r8);
            }
          }
          tmem_wait_ld();
#pragma unroll
          for (int d = 0; d < S; ++d) {
#pragma unroll
            for (int i = 0; i < CW; ++i) {
              const long long q = (long long)acc_to_int(raw[d][i]);
              if (d < DH) hi[i] += q * (1LL << (7 * (DH - 1 - d)));
              else lo[i] += q * (1LL << (7 * (S - 1 - d)));
            }
          }
        }
      }
      store_chunk<S, DH, CW>(hi, lo, col_exp + c0, e_row, part, row, tn * NT + c0, row < a.m && !aborted, a, Cb);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)Cfg::TMEM_COLS));
  }
}

// ---------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------
// ---------------------------------------------------------------------------------
// Persistent form: one CTA per SM walks the output tiles (tn fastest, so the CTAs running
// at the same time share their A tiles in L2).  A ring of STAGES shared-memory stages runs
// across tile boundaries, and TMEM holds two accumulator sets, so the epilogue of one tile
// overlaps the MMAs of the next and the producer keeps STAGES - 1 stages in flight.
//   warp 0     TMA producer over (tile, K block)
//   warp 1     TMEM allocation; MMA issue into accumulator set (tile count & 1)
//   warps 2-9  epilogue of each tile from its accumulator set, then release the set
// Barriers: full/empty per stage (as the per-tile kernel), tfull[2] (MMA commit -> epilogue)
// and tempty[2] (one arrival per epilogue thread -> MMA).  Every wait is bounded; a timeout sets the
// abort flag and the error code, every role leaves its loop, and the MMA warp waits for
// its issued MMAs to complete before TMEM is freed.
// ---------------------------------------------------------------------------------
template <int S, int NT>
struct TcPCfg {
  static constexpr int A_TILE = TILE_M * ROW_BYTES;
  static constexpr int B_TILE = NT * ROW_BYTES;
  static constexpr int STAGE = S * (A_TILE + B_TILE);
  static constexpr int BUDGET = 220 * 1024;
  static constexpr int STAGES = BUDGET / STAGE > 6 ? 6 : BUDGET / STAGE;
  static constexpr int ACC = S * NT;   // TMEM columns of one accumulator set
  static constexpr int SMEM = STAGES * STAGE + 1024 + 256 + 8 * NT;   // + alignment, barriers, 2 x NT exponents
  static_assert(STAGES >= 2, "at least two stages");
  static_assert(2 * ACC <= 512, "two accumulator sets in TMEM");
  static_assert(SMEM <= 227 * 1024, "shared memory of one CTA");
  static_assert(NT % 16 == 0 && NT >= 16 && NT <= 256, "UMMA N");
};

// named barrier 1 over the epilogue threads that also ORs a predicate: every thread gets
// the same answer, so the epilogue warps always take the same branch out of a loop
__device__ __forceinline__ bool epi_barrier_any(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, 1, %2, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "n"(32 * TC_EPI_WARPS)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <int S, int NT>
__global__ void __launch_bounds__(TC_THREADS, 1)
    zgemm_tc_persistent(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, TcArgs a,
                        int tiles_m, int tiles_n) {
  using Cfg = TcPCfg<S, NT>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Cfg::STAGES * Cfg::STAGE);
  uint64_t* empty = full + Cfg::STAGES;
  uint64_t* tfull = empty + Cfg::STAGES;
  uint64_t* tempty = tfull + 2;
  uint64_t* fin = tempty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(fin + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);
  int* col_exp = abort_flag + 1;   // [2][NT] column exponents of the tiles in flight

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = (a.kp + BK - 1) / BK;
  const long long tiles_item = (long long)tiles_m * tiles_n;
  const long long ntiles = tiles_item * a.batch;

  if (threadIdx.x == 0) {
    for (int s = 0; s < Cfg::STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    for (int s = 0; s < 2; ++s) { mbar_init(&tfull[s], 1); mbar_init(&tempty[s], 32 * TC_EPI_WARPS); }
    mbar_init(fin, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512u));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
      uint32_t kg = 0;   // stage-ring position, continuous across tiles
      for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int b = (int)(t / tiles_item);
        const int r = (int)(t % tiles_item);
        const int a_row0 = (r / tiles_n) * TILE_M, b_row0 = (r % tiles_n) * NT;
        bool stop = false;
        for (int kb = 0; kb < nk; ++kb, ++kg) {
          const int st = (int)(kg % Cfg::STAGES);
          if (!mbar_wait(&empty[st], ((kg / Cfg::STAGES) & 1) ^ 1)) {
            atomicExch(abort_flag, 1);
            if (a.err) atomicCAS(a.err, 0, 1);
            stop = true;
            break;
          }
          if (*((volatile int*)abort_flag)) { stop = true; break; }
          uint8_t* sa = smem + st * Cfg::STAGE;
          uint8_t* sb = sa + S * Cfg::A_TILE;
          mbar_expect_tx(&full[st], (uint32_t)Cfg::STAGE);
#pragma unroll
          for (int p = 0; p < S; ++p) {
            tma_load_2d(sa + p * Cfg::A_TILE, &mapA, kb * BK,
                        (int)((long long)(b * a.planesA + p) * a.rowsA + a_row0), &full[st]);
            tma_load_2d(sb + p * Cfg::B_TILE, &mapB, kb * BK,
                        (int)((long long)(b * a.planesB + p) * a.rowsB + b_row0), &full[st]);
          }
        }
        if (stop) break;
      }
      // drain: every issued stage must have landed before the CTA may exit
      for (uint32_t k = (kg > (uint32_t)Cfg::STAGES ? kg - Cfg::STAGES : 0); k < kg; ++k)
        mbar_wait(&full[k % Cfg::STAGES], (k / Cfg::STAGES) & 1);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      uint32_t kg = 0;
      int it = 0;
      bool stop = false;
      for (long long t = blockIdx.x; t < ntiles && !stop; t += gridDim.x, ++it) {
        const int buf = it & 1;
        if (!mbar_wait(&tempty[buf], ((it >> 1) & 1) ^ 1)) {
          atomicExch(abort_flag, 1);
          if (a.err) atomicCAS(a.err, 0, 4);
          break;
        }
        tc_fence_after();
        const uint32_t acc0 = tmem + (uint32_t)(buf * Cfg::ACC);
        for (int kb = 0; kb < nk; ++kb, ++kg) {
          const int st = (int)(kg % Cfg::STAGES);
          if (!mbar_wait(&full[st], (kg / Cfg::STAGES) & 1)) {
            atomicExch(abort_flag, 1);
            if (a.err) atomicCAS(a.err, 0, 2);
            stop = true;
            break;
          }
          tc_fence_after();
          const uint32_t sa = smem_u32(smem + st * Cfg::STAGE);
          const uint32_t sb = sa + S * Cfg::A_TILE;
          const uint64_t da0 = make_desc(sa), db0 = make_desc(sb);
          issue_stage_mmas<S, NT, Cfg::A_TILE, Cfg::B_TILE>(acc0, da0, db0, kb == 0);
          tc_commit(&empty[st]);
        }
        if (!stop) tc_commit(&tfull[buf]);
      }
      // every issued MMA has completed before TMEM may be freed
      tc_commit(fin);
      mbar_wait(fin, 0);
    }
  } else {
    const int quarter = warp & 3;
    int it = 0;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
      const int buf = it & 1;
      const int b = (int)(t / tiles_item);
      const int r = (int)(t % tiles_item);
      const int tm = r / tiles_n, tn = r % tiles_n;
      int* cexp = col_exp + buf * NT;
      for (int c = threadIdx.x - 64; c < NT; c += 32 * TC_EPI_WARPS) {
        const int col = tn * NT + c;
        cexp[c] = col < a.n ? a.fb[(long long)b * a.n + col] : 0;
      }
      // the exponents are visible to all epilogue warps, and all agree on stopping
      if (epi_barrier_any(*((volatile int*)abort_flag) != 0)) break;
      const bool ok = mbar_wait(&tfull[buf], (it >> 1) & 1);
      if (epi_barrier_any(!ok)) {
        atomicExch(abort_flag, 1);
        if (a.err) atomicCAS(a.err, 0, 3);
        break;
      }
      tc_fence_after();
      const int rr = tm * TILE_M + quarter * 32 + lane;
      const int row = rr >> 1, part = rr & 1;        // C row, real (0) or imaginary (1) part
      const int e_row = (row < a.m) ? a.ea[(long long)b * a.m + row] : 0;
      double2* Cb = a.C + (long long)b * a.sC;
      const uint32_t acc0 = tmem + (uint32_t)(buf * Cfg::ACC);
      constexpr int CW = 8;   // fp32 columns per chunk
      constexpr int NGRP = TC_EPI_WARPS / 4;   // warps per lane quarter
      const int grp = (warp - 2) >> 2;
#pragma unroll 1
      for (int c0 = grp * CW; c0 < NT; c0 += NGRP * CW) {
        constexpr int DH = S <= 6 ? S : 3;   // S <= 6 fits one int64; S >= 7 splits
        long long hi[CW], lo[CW];
#pragma unroll
        for (int i = 0; i < CW; ++i) { hi[i] = 0; lo[i] = 0; }
        uint32_t raw[S][CW];
#pragma unroll
        for (int d = 0; d < S; ++d) {
          const uint32_t ta = acc0 + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(d * NT + c0);
          tmem_ld8_nowait(ta, *reinterpret_cast<uint32_t(*)[8]>(&raw[d][0]));
        }
        tmem_wait_ld();
#pragma unroll
        for (int d = 0; d < S; ++d) {
#pragma unroll
          for (int i = 0; i < CW; ++i) {
            const long long q = (long long)acc_to_int(raw[d][i]);
            if (d < DH) hi[i] += q * (1LL << (7 * (DH - 1 - d)));
            else lo[i] += q * (1LL << (7 * (S - 1 - d)));
          }
        }
        store_chunk<S, DH, CW>(hi, lo, cexp + c0, e_row, part, row, tn * NT + c0, row < a.m, a, Cb);
      }
      tc_fence_before();
      mbar_arrive(&tempty[buf]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512u));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 2D bf16 map {inner = kp, outer = rows}, box {BK, box_rows}, 64-byte swizzle
int make_map(CUtensorMap* map, const void* base, int kp, long long rows, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return NEGF_ECUDA;
  if (((uintptr_t)base & 15) != 0 || ((long long)kp * 2) % 16 != 0) return NEGF_EINVAL;
  cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, BK == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? NEGF_OK : NEGF_ECUDA;
}

// Kernel variants, timed per shape by the autotuner below (results are bitwise the same
// in every variant): 0 and 1 are per-tile kernels <N tile, CTAs per SM> with different N
// tiles (the N tile sets how evenly the N columns divide, and with the slice count how
// much TMEM a CTA needs: S x N columns <= 512 / CTAs per SM), 2 is the persistent kernel.
constexpr int kVariants = 3;

template <int S, int NT, int MINB, int KS = 1>
int launch_mma(const SlicedOperand& A, const SlicedOperand& B, const TcArgs& args, cudaStream_t st) {
  using Cfg = TcCfg<S, NT, MINB, KS>;
  // one set of accumulators holds at most 800 K' exactly (two sets: 1600)
  if (args.kp > 800 * KS) return NEGF_EINVAL;
  CUtensorMap ma, mb;
  NEGF_TRY(make_map(&ma, A.data, args.kp, (long long)args.batch * args.planesA * args.rowsA, TILE_M));
  NEGF_TRY(make_map(&mb, B.data, args.kp, (long long)args.batch * args.planesB * args.rowsB, NT));
  NEGF_CUDA_TRY(
      cudaFuncSetAttribute(zgemm_tc_kernel<S, NT, MINB, KS>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM));
  dim3 grid((unsigned)((2LL * args.m + TILE_M - 1) / TILE_M), (unsigned)((args.n + NT - 1) / NT), args.batch);
  cudaEvent_t ev;
  const double cflops = 8.0 * args.m * (double)args.n * (args.kp / 2) * args.batch;
  add_tc_complex_flops(cflops);
  timed_begin(st, TK_TC, cflops * (S * (S + 1) / 2), &ev);
  zgemm_tc_kernel<S, NT, MINB, KS><<<grid, TC_THREADS, Cfg::SMEM, st>>>(ma, mb, args);
  NEGF_CUDA_TRY(cudaGetLastError());
  timed_end(st, TK_TC, ev);
  count_launch();
  return NEGF_OK;
}

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
  }
  return n;
}

template <int S, int NT>
int launch_persistent(const SlicedOperand& A, const SlicedOperand& B, const TcArgs& args, cudaStream_t st) {
  using Cfg = TcPCfg<S, NT>;
  CUtensorMap ma, mb;
  NEGF_TRY(make_map(&ma, A.data, args.kp, (long long)args.batch * args.planesA * args.rowsA, TILE_M));
  NEGF_TRY(make_map(&mb, B.data, args.kp, (long long)args.batch * args.planesB * args.rowsB, NT));
  NEGF_CUDA_TRY(cudaFuncSetAttribute(zgemm_tc_persistent<S, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM));
  const int tiles_m = (int)((2LL * args.m + TILE_M - 1) / TILE_M);
  const int tiles_n = (int)((args.n + NT - 1) / NT);
  const long long ntiles = (long long)tiles_m * tiles_n * args.batch;
  const int grid = (int)std::min<long long>(ntiles, sm_count());
  cudaEvent_t ev;
  const double cflops = 8.0 * args.m * (double)args.n * (args.kp / 2) * args.batch;
  add_tc_complex_flops(cflops);
  timed_begin(st, TK_TC, cflops * (S * (S + 1) / 2), &ev);
  zgemm_tc_persistent<S, NT><<<grid, TC_THREADS, Cfg::SMEM, st>>>(ma, mb, args, tiles_m, tiles_n);
  NEGF_CUDA_TRY(cudaGetLastError());
  timed_end(st, TK_TC, ev);
  count_launch();
  return NEGF_OK;
}

template <int S>
int slice_a_t(const double2* A, int lda, long long sA, int m, int k, int batch, SlicedOperand& out, cudaStream_t st) {
  cudaEvent_t ev;
  timed_begin(st, TK_SLICE, 0.0, &ev);
  dim3 g1((m + 31) / 32, batch);
  row_exp_kernel<<<g1, dim3(32, 8), 0, st>>>(A, lda, sA, m, k, out.exps);
  NEGF_CUDA_TRY(cudaGetLastError());
  dim3 g2((m + 31) / 32, (out.k + 63) / 64, batch);
  slice_a_kernel<S><<<g2, 256, 0, st>>>(A, lda, sA, m, k, out.exps, out.data, out.k);
  NEGF_CUDA_TRY(cudaGetLastError());
  timed_end(st, TK_SLICE, ev);
  count_launch(2);
  return NEGF_OK;
}

template <int S>
int slice_b_t(const double2* B, int ldb, long long sB, int k, int n, int batch, SlicedOperand& out, cudaStream_t st) {
  dim3 g((n + 7) / 8, batch);
  cudaEvent_t ev;
  timed_begin(st, TK_SLICE, 0.0, &ev);
  slice_b_kernel<S><<<g, 256, 0, st>>>(B, ldb, sB, k, n, out.exps, out.data, out.k);
  NEGF_CUDA_TRY(cudaGetLastError());
  timed_end(st, TK_SLICE, ev);
  count_launch();
  return NEGF_OK;
}

}  // namespace

bool tc_supported_slices(int s) { return s >= 3 && s <= 8; }

size_t sliced_bytes(int rows, int k, int slices, int batch) {
  return sizeof(__nv_bfloat16) * (size_t)batch * slices * rows * 2 * (size_t)k;
}
size_t sliced_bytes_a(int m, int k, int slices, int batch) { return sliced_bytes(2 * m, k, slices, batch); }
size_t sliced_bytes_b(int n, int k, int slices, int batch) { return sliced_bytes(n, k, slices, batch); }

int padded_k(int k) { return (k + 7) & ~7; }   // 16-byte slice vectors and TMA rows

int slice_a(const double2* A, int lda, long long sA, int m, int k, int batch, int slices, SlicedOperand& out,
            cudaStream_t st) {
  if (sliced_bytes_a(m, padded_k(k), slices, batch) > out.data_bytes || (size_t)m * batch > out.exps_count)
    return NEGF_EINVAL;
  out.rows = 2 * m; out.k = padded_k(k); out.slices = slices; out.batch = batch;
  switch (slices) {
    case 2: return slice_a_t<2>(A, lda, sA, m, k, batch, out, st);
    case 3: return slice_a_t<3>(A, lda, sA, m, k, batch, out, st);
    case 4: return slice_a_t<4>(A, lda, sA, m, k, batch, out, st);
    case 5: return slice_a_t<5>(A, lda, sA, m, k, batch, out, st);
    case 6: return slice_a_t<6>(A, lda, sA, m, k, batch, out, st);
    case 7: return slice_a_t<7>(A, lda, sA, m, k, batch, out, st);
    case 8: return slice_a_t<8>(A, lda, sA, m, k, batch, out, st);
  }
  return NEGF_EINVAL;
}

int slice_b(const double2* B, int ldb, long long sB, int k, int n, int batch, int slices, SlicedOperand& out,
            cudaStream_t st) {
  if (sliced_bytes_b(n, padded_k(k), slices, batch) > out.data_bytes || (size_t)n * batch > out.exps_count)
    return NEGF_EINVAL;
  out.rows = n; out.k = padded_k(k); out.slices = slices; out.batch = batch;
  switch (slices) {
    case 2: return slice_b_t<2>(B, ldb, sB, k, n, batch, out, st);
    case 3: return slice_b_t<3>(B, ldb, sB, k, n, batch, out, st);
    case 4: return slice_b_t<4>(B, ldb, sB, k, n, batch, out, st);
    case 5: return slice_b_t<5>(B, ldb, sB, k, n, batch, out, st);
    case 6: return slice_b_t<6>(B, ldb, sB, k, n, batch, out, st);
    case 7: return slice_b_t<7>(B, ldb, sB, k, n, batch, out, st);
    case 8: return slice_b_t<8>(B, ldb, sB, k, n, batch, out, st);
  }
  return NEGF_EINVAL;
}

int launch_variant(int v, int S, const SlicedOperand& A, const SlicedOperand& B, const TcArgs& args,
                   cudaStream_t st);

namespace {

// Autotuner of the kernel variant per shape (slices, m, n, K', batch rounded up to a power
// of two): the two per-tile kernels (N tiles of different widths; two CTAs per SM where
// TMEM and shared memory allow) and the persistent kernel.  All issue each output
// element's MMAs in the same K order into the same exact accumulators and run the same
// epilogue, so their results are bitwise identical and the choice never changes a number.
// The first call of a shape with beta = 0 runs every variant three times (each run
// overwrites C with the same values), times the last two runs with events on the caller's
// stream and keeps the fastest.  A first call with beta != 0 is tuned the same way when the
// caller lends a scratch output (the timings run with beta = 0 into it, so C keeps its
// input for the product itself); without one it uses variant 0 and leaves the shape
// untuned.  Beyond K' = 800 only the per-tile kernel with two accumulator sets along K
// exists.
struct TuneKey {
  int S, m, n, kp, batch;
  bool operator<(const TuneKey& o) const {
    if (S != o.S) return S < o.S;
    if (m != o.m) return m < o.m;
    if (n != o.n) return n < o.n;
    if (kp != o.kp) return kp < o.kp;
    return batch < o.batch;
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune;   // the chosen variant

float time_variant(int v, int S, const SlicedOperand& A, const SlicedOperand& B, const TcArgs& args, cudaStream_t st) {
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return -1.0f;
  if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return -1.0f; }
  cudaEventRecord(e0, st);
  const int rc = launch_variant(v, S, A, B, args, st);
  cudaEventRecord(e1, st);
  float ms = -1.0f;
  if (rc == NEGF_OK && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc == NEGF_OK ? ms : -1.0f;
}

}  // namespace

// returns the variant to launch, or -2 when tuning already ran the product (C is written)
int choose_variant(int S, const SlicedOperand& A, const SlicedOperand& B, const TcArgs& args, cudaStream_t st,
                   double2* tune_c) {
  int bb = 1;
  while (bb < args.batch) bb <<= 1;
  const TuneKey key{S, args.m, args.n, args.kp, bb};
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return it->second;
  }
  if (args.kp > 800 || (args.beta_kind != 0 && !tune_c)) return 0;
  TcArgs targs = args;
  if (args.beta_kind != 0) {   // time into the scratch with beta = 0
    targs.C = tune_c;
    targs.sC = (long long)args.ldc * args.n;
    targs.beta = make_double2(0.0, 0.0);
    targs.beta_kind = 0;
  }
  // two timings each, after a first run of each that pays one-time costs
  float best[kVariants];
  for (int v = 0; v < kVariants; ++v) best[v] = 1e30f;
  for (int rep = 0; rep < 3; ++rep)
    for (int v = 0; v < kVariants; ++v) {
      const float ms = time_variant(v, S, A, B, targs, st);
      if (ms < 0.0f) return -3;
      if (rep > 0 && ms < best[v]) best[v] = ms;
    }
  int choice = 0;
  for (int v = 1; v < kVariants; ++v)
    if (best[v] < best[choice]) choice = v;
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tune[key] = choice;
  return args.beta_kind != 0 ? choice : -2;   // with beta != 0 the product itself is still to run
}

int zgemm_tc(const SlicedOperand& A, const SlicedOperand& B, double2 alpha, double2 beta, double2* C, int ldc,
             long long sC, int* err, cudaStream_t st, int slices, double2* tune_c) {
  // the leading `slices` digit planes of each operand (its own count by default); the
  // leading planes of a finer slicing are a coarser slicing of the same values
  const int S = slices ? slices : A.slices;
  if (S > A.slices || S > B.slices || (!slices && A.slices != B.slices)) return NEGF_EINVAL;
  if (A.k != B.k || A.batch != B.batch) return NEGF_EINVAL;
  // every accumulator is exact for K' <= 800 per accumulator set, and the per-tile kernel
  // has at most two sets along K
  if (2 * A.k > 1600) return NEGF_EINVAL;
  TcArgs args{};
  if (A.rows % 2 != 0) return NEGF_EINVAL;
  args.m = A.rows / 2; args.n = B.rows; args.kp = 2 * A.k; args.batch = A.batch;
  args.rowsA = A.rows; args.rowsB = B.rows;
  args.planesA = A.slices; args.planesB = B.slices;
  args.ea = A.exps; args.fb = B.exps;
  args.C = C; args.ldc = ldc; args.sC = sC;
  args.alpha = alpha; args.beta = beta; args.err = err;
  args.alpha_one = (alpha.x == 1.0 && alpha.y == 0.0) ? 1 : 0;
  args.beta_kind = (beta.x == 0.0 && beta.y == 0.0) ? 0 : (beta.x == 1.0 && beta.y == 0.0) ? 1 : 2;
  // NEGF_TC_VARIANT = 0, 1 or 2 runs that kernel variant instead of the autotuner's choice
  // (to compare or profile variants; all give bitwise the same result)
  if (const char* ev = std::getenv("NEGF_TC_VARIANT")) {
    const int v = std::atoi(ev);
    if (ev[0] >= '0' && ev[0] <= '9' && v < kVariants) return launch_variant(v, S, A, B, args, st);
  }
  const int variant = choose_variant(S, A, B, args, st, tune_c);
  if (variant == -2) return NEGF_OK;        // the tuning runs computed C
  if (variant == -3) return NEGF_ECUDA;
  return launch_variant(variant, S, A, B, args, st);
}

int launch_variant(int v, int S, const SlicedOperand& A, const SlicedOperand& B, const TcArgs& args,
                   cudaStream_t st) {
  if (args.kp > 800) {
    // two accumulator sets along K, one CTA per SM: 2 S NT <= 512 TMEM columns
    switch (S) {
      case 3: return launch_mma<3, 80, 1, 2>(A, B, args, st);
      case 4: return launch_mma<4, 64, 1, 2>(A, B, args, st);
      case 5: return launch_mma<5, 48, 1, 2>(A, B, args, st);
      case 6: return launch_mma<6, 32, 1, 2>(A, B, args, st);
      case 7: return launch_mma<7, 32, 1, 2>(A, B, args, st);
      case 8: return launch_mma<8, 32, 1, 2>(A, B, args, st);
    }
    return NEGF_EINVAL;
  }
  if (v == 2) {
    switch (S) {
      case 2: return launch_persistent<2, 128>(A, B, args, st);
      case 3: return launch_persistent<3, 80>(A, B, args, st);
      case 4: return launch_persistent<4, 64>(A, B, args, st);
      case 5: return launch_persistent<5, 48>(A, B, args, st);
      case 6: return launch_persistent<6, 32>(A, B, args, st);
      case 7: return launch_persistent<7, 32>(A, B, args, st);
      case 8: return launch_persistent<8, 32>(A, B, args, st);
    }
    return NEGF_EINVAL;
  }
  switch (S) {
    case 2: return v ? launch_mma<2, 64, 2>(A, B, args, st) : launch_mma<2, 128, 2>(A, B, args, st);
    case 3: return v ? launch_mma<3, 48, 2>(A, B, args, st) : launch_mma<3, 80, 2>(A, B, args, st);
    case 4: return v ? launch_mma<4, 80, 1>(A, B, args, st) : launch_mma<4, 64, 2>(A, B, args, st);
    case 5: return v ? launch_mma<5, 80, 1>(A, B, args, st) : launch_mma<5, 48, 2>(A, B, args, st);
    case 6: return v ? launch_mma<6, 80, 1>(A, B, args, st) : launch_mma<6, 64, 1>(A, B, args, st);
    case 7: return v ? launch_mma<7, 48, 1>(A, B, args, st) : launch_mma<7, 64, 1>(A, B, args, st);
    case 8: return v ? launch_mma<8, 48, 1>(A, B, args, st) : launch_mma<8, 64, 1>(A, B, args, st);
  }
  return NEGF_EINVAL;
}

}  // namespace negf
