// Exact FP64 contractions on the bf16 tensor cores (shared by the
// reconstruction, recon_tc.cu, and the quadratures of the implicit solve,
// recon_solve.cu).
//
// An operand row or column is scaled by a power of two into an integer of 56
// significant bits and written as seven balanced base-256 digits (the top
// digit in [-256, 256], the others in [-128, 127]), each exact in bf16.
// Digit products of level l = i + k accumulate in FP32 through mma.sync
// m16n8k16; with at most 112 terms per chunk a level's partial sums stay
// below 2^24, so FP32 holds them exactly.  Levels l < 7 are kept (the rest
// lie below 2^-56 of the operands' scale), recombined exactly in 64-bit
// integers and rounded once to FP64.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include <cstring>
#include <vector>

#include "chn_common.cuh"

namespace chn {

static constexpr int kDig = 7;      // base-256 digits per operand
static constexpr int kChunkKT = 7;  // k-tiles per exact FP32 accumulation chunk (K <= 112)

inline uint16_t bf16_bits_of_int(int d) {
  const float f = (float)d;  // |d| <= 256: exact in bf16, low 16 bits zero
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (uint16_t)(u >> 16);
}

// seven balanced base-256 digits of x (|x| < 2^56), most significant first
inline void digits56(long long x, int* d) {
  for (int i = kDig - 1; i >= 1; --i) {
    const long long lo = ((x + 128) & 255) - 128;
    d[i] = (int)lo;
    x = (x - lo) >> 8;
  }
  d[0] = (int)x;
}

__device__ __forceinline__ void mma_bf16_16816(float* d, const uint4& a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b0), "r"(b1));
}

// the seven digits of v * 2^(56 - ex) from the bit pattern (integer ops only);
// ex bounds the column: |v| < 2^ex
__device__ __forceinline__ long long scaled56(double v, int ex) {
  const long long bits = __double_as_longlong(v);
  const int ef = (int)((bits >> 52) & 0x7FF);
  if (ef == 0) return 0;  // zero (denormals are below every scale in use)
  long long sig = (bits & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
  const int s = ef - 1019 - ex;  // <= 3
  if (s >= 0) sig <<= s;
  else if (s > -62) sig = (sig + (1LL << (-s - 1))) >> (-s);
  else sig = 0;
  return bits < 0 ? -sig : sig;
}

// (H 2^32 + L) 2^e with one FP64 conversion: the sum is folded into one
// int64 keeping at least 62 significant bits (|H| < 2^41, |L| < 2^50), the
// conversion rounds it, and the power of two goes into the exponent field
// with integer arithmetic.  Faithful (the folded-away low bits lie more
// than 8 bits below the result's last place); the FP64 pipe sees one
// conversion per value.
__device__ __forceinline__ double round_fast(long long H, long long L, int e) {
  const unsigned long long aH = (unsigned long long)(H < 0 ? -H : H);
  const int sh = max(0, 34 - __clzll((long long)aH));  // |T| < 2^63
  const long long T = (long long)((unsigned long long)H << (32 - sh)) + (L >> sh);
  if (T == 0) return 0.0;
  const double v = (double)T;
  const long long bits = __double_as_longlong(v);
  const int es = e + sh;
  const int ex = (int)((bits >> 52) & 0x7FF) + es;
  if (ex > 0 && ex < 2047) return __longlong_as_double(bits + ((long long)es << 52));
  return scalbn(v, es);
}

// round_fast for an output of a column whose largest biased exponent field
// is ce: a column that held an infinity or a NaN (ce = 0x7FF; its digits
// carry no meaning) gives NaN, as the FP64 sum would
__device__ __forceinline__ double round_col(long long H, long long L, int e, int ce) {
  return ce == 0x7FF ? __longlong_as_double(0x7FF8000000000000LL) : round_fast(H, L, e);
}

// x is neither infinite nor NaN (integer test on the exponent field)
__device__ __forceinline__ bool finite_bits(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7FF) != 0x7FF;
}

// Balanced digits without a carry chain: with B = sum_{i<6} 128 * 256^i,
// x + B = sum_{q>=1} (d_q + 128) 256^(6-q) + d_0 256^6, so every lower digit
// is an unsigned byte of x + B less 128 and the top digit (in [-256, 256])
// its arithmetic shift by 48.  The digits come out as FP32 values without an
// integer-to-float conversion: for 0 <= u < 2^23 the bit pattern
// 0x4B000000 | u is the float 2^23 + u, so a byte b placed under that
// exponent (one byte permute) less 2^23 + 128 is b - 128, exactly (one FP32
// add); the top digit goes the same way through u = d_0 + 256.  Every digit
// has at most 8 significant bits, so the float's upper half is its exact bf16.
__device__ __forceinline__ void balanced_digits_f32(long long x, float (&f)[kDig]) {
  const long long xb = x + 0x808080808080LL;
  const unsigned lo = (unsigned)xb, hi = (unsigned)(xb >> 32);
  constexpr float kOff = 8388736.0f;  // 2^23 + 128
  // __byte_perm selector 0x765k: byte 0 from byte k of the word, bytes 1-3 from 0x4B000000
  f[6] = __uint_as_float(__byte_perm(lo, 0x4B000000u, 0x7650)) - kOff;
  f[5] = __uint_as_float(__byte_perm(lo, 0x4B000000u, 0x7651)) - kOff;
  f[4] = __uint_as_float(__byte_perm(lo, 0x4B000000u, 0x7652)) - kOff;
  f[3] = __uint_as_float(__byte_perm(lo, 0x4B000000u, 0x7653)) - kOff;
  f[2] = __uint_as_float(__byte_perm(hi, 0x4B000000u, 0x7650)) - kOff;
  f[1] = __uint_as_float(__byte_perm(hi, 0x4B000000u, 0x7651)) - kOff;
  f[0] = __uint_as_float((unsigned)(((int)hi >> 16) + (0x4B000000 + 256))) - 8388864.0f;  // 2^23 + 256
}

// seven balanced digits of x (|x| < 2^56) as bf16 bit patterns, most significant first
__device__ __forceinline__ void digits_bf16(long long x, uint16_t* out, size_t stride) {
  float f[kDig];
  balanced_digits_f32(x, f);
#pragma unroll
  for (int q = 0; q < kDig; ++q) out[(size_t)q * stride] = (uint16_t)(__float_as_uint(f[q]) >> 16);
}

// the balanced digits of two values (re, im) packed per digit into one 32-bit
// word (re in the low half): out[q * stride] for q = 0..6
__device__ __forceinline__ void digits_pair_bf16(long long xr, long long xi, uint32_t* out, size_t stride) {
  float fr[kDig], fi[kDig];
  balanced_digits_f32(xr, fr);
  balanced_digits_f32(xi, fi);
#pragma unroll
  for (int q = 0; q < kDig; ++q)  // the upper halves of the two floats
    out[(size_t)q * stride] = __byte_perm(__float_as_uint(fr[q]), __float_as_uint(fi[q]), 0x7632);
}

// the exact level sums of one mma accumulator element added to (H, L): the
// sum is (H 2^32 + L) 2^(e_row + e_col - 64) for operands scaled to 56-bit
// integers.  Each level enters as a 32 x 32 -> 64-bit multiply-add onto the
// running 64-bit sum (exact integer arithmetic: the order does not matter).
__device__ __forceinline__ void fold_levels_add(const float (&acc)[kDig][4], int r, long long& H, long long& L) {
  int lv[kDig];
#pragma unroll
  for (int l = 0; l < kDig; ++l) lv[l] = __float2int_rn(acc[l][r]);
  H += (long long)lv[2];
  H += (long long)lv[1] * 256LL;
  H += (long long)lv[0] * 65536LL;
  L += (long long)lv[6];
  L += (long long)lv[5] * 256LL;
  L += (long long)lv[4] * 65536LL;
  L += (long long)lv[3] * 16777216LL;
}

// One exact digit GEMM tile of a fixed table A (fragment order
// [mt][KT][7][32][4]) against the smem digits of column n, over the k-tiles
// [k0, k1): FP32 level sums per chunk of at most 7 k-tiles (exact), folded
// into the 64-bit integers H, L per accumulator element (exact across
// chunks: |H| < 2^41, |L| < 2^50 per chunk); an empty range gives zeros
__device__ __forceinline__ void tc_tile_range(const uint4* __restrict__ A, int mt, int KT, int k0, int k1,
                                              const uint16_t* dig, size_t KS, size_t dstride, int n, int lane, int t,
                                              long long (&H)[4], long long (&L)[4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) { H[r] = 0; L[r] = 0; }
  for (int kc = k0; kc < k1; kc += kChunkKT) {
    float acc[kDig][4];
#pragma unroll
    for (int l = 0; l < kDig; ++l)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[l][r] = 0.f;
    const int kend = min(k1, kc + kChunkKT);
    for (int kt = kc; kt < kend; ++kt) {
      const uint32_t* brow = reinterpret_cast<const uint32_t*>(dig + (size_t)n * KS + kt * 16);
      uint32_t b0[kDig], b1[kDig];
#pragma unroll
      for (int k = 0; k < kDig; ++k) {
        b0[k] = brow[(size_t)k * dstride / 2 + t];
        b1[k] = brow[(size_t)k * dstride / 2 + t + 4];
      }
#pragma unroll
      for (int i = 0; i < kDig; ++i) {
        const uint4 af = __ldg(&A[(((size_t)mt * KT + kt) * kDig + i) * 32 + lane]);
#pragma unroll
        for (int k = 0; k < kDig - i; ++k) mma_bf16_16816(acc[i + k], af, b0[k], b1[k]);
      }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) fold_levels_add(acc, r, H[r], L[r]);
  }
}

__device__ __forceinline__ void tc_tile(const uint4* __restrict__ A, int mt, int KT, const uint16_t* dig, size_t KS,
                                        size_t dstride, int n, int lane, int t, long long (&H)[4],
                                        long long (&L)[4]) {
  tc_tile_range(A, mt, KT, 0, KT, dig, KS, dstride, n, lane, t, H, L);
}

// The same tile over the k-tiles [0, k1) of a table with KT k-tiles per row
// tile, with the table fragments of k-tile kt + 1 loaded while kt's products
// run (for tables that live in L2)
__device__ __forceinline__ void tc_tile_pf(const uint4* __restrict__ A, int mt, int KT, int k1, const uint16_t* dig,
                                           size_t KS, size_t dstride, int n, int lane, int t, long long (&H)[4],
                                           long long (&L)[4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) { H[r] = 0; L[r] = 0; }
  const uint4* Am = A + (size_t)mt * KT * kDig * 32 + lane;
  for (int kc = 0; kc < k1; kc += kChunkKT) {
    float acc[kDig][4];
#pragma unroll
    for (int l = 0; l < kDig; ++l)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[l][r] = 0.f;
    const int kend = min(k1, kc + kChunkKT);
    uint4 af[kDig];
#pragma unroll
    for (int i = 0; i < kDig; ++i) af[i] = __ldg(Am + ((size_t)kc * kDig + i) * 32);
    for (int kt = kc; kt < kend; ++kt) {
      const int kn = min(kt + 1, kend - 1);
      uint4 an[kDig];
#pragma unroll
      for (int i = 0; i < kDig; ++i) an[i] = __ldg(Am + ((size_t)kn * kDig + i) * 32);
      const uint32_t* brow = reinterpret_cast<const uint32_t*>(dig + (size_t)n * KS + kt * 16);
      uint32_t b0[kDig], b1[kDig];
#pragma unroll
      for (int k = 0; k < kDig; ++k) {
        b0[k] = brow[(size_t)k * dstride / 2 + t];
        b1[k] = brow[(size_t)k * dstride / 2 + t + 4];
      }
#pragma unroll
      for (int i = 0; i < kDig; ++i)
#pragma unroll
        for (int k = 0; k < kDig - i; ++k) mma_bf16_16816(acc[i + k], af[i], b0[k], b1[k]);
#pragma unroll
      for (int i = 0; i < kDig; ++i) af[i] = an[i];
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) fold_levels_add(acc, r, H[r], L[r]);
  }
}

// host: digit table of a row-major matrix M[rows][K] in mma A-fragment order
// [MT][KT][7][32 lanes][4] (appended to frag), row exponents appended to ex
bool append_digit_table(const double* M, int rows, int K, int MT, int KT, std::vector<uint32_t>& frag,
                        std::vector<int>& ex);

}  // namespace chn
