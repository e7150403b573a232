// The inverse 3/2-padded transforms (channel/pass1.c:42-114,
// channel/spec2phys.c:39-76) as exact digit GEMMs on the fifth-generation
// tensor cores: tcgen05.mma with the level sums accumulated in tensor memory.
//
// Same arithmetic as k_phys_inverse_tc (phys_tc.cu): the same DFT matrices,
// row exponents and 56-bit column scaling, seven balanced base-256 digits
// per operand, the even / odd (radix-2) split of each stage, level sums
// l = i + k of digit products exact in FP32, folded exactly into 64-bit
// integers and rounded once.  The integer sums do not depend on the order of
// the products, so the outputs equal the mma.sync kernel's bit for bit.
//
// Layout of one tcgen05.mma (cta_group::1, kind::f16, M = 128, K = 16):
//   A  the data digits: one row per data column of the stage (the z stage:
//      (field, x); the x stage: (field, m)), K-major, no swizzle, in 8 x 16-
//      byte core matrices ([row group][k half][8 rows][8 bf16]);
//   B  the table digits with the seven digit planes stacked along N: row
//      k Np + r holds digit k of table row r, so ONE instruction multiplies
//      data digit i by all table digits k = 0 .. 6 - i at once;
//   D  tensor memory: level l of table row r at column l Np + r, so the
//      instruction for data digit i writes at column offset i Np and every
//      product block k lands on its level i + k.
// Per k-tile: 7 instructions (9 where (7 - i) Np exceeds N = 256) instead of
// 28.  The first instruction of a stage overwrites (levels 0..6 all fresh),
// the rest accumulate.  Each lane of the accumulator is one data column, so
// every thread folds its own column's outputs (tcgen05.ld 32x32b).
//
// A persistent grid of one CTA per SM walks the (instance, plane) items.
// The tables are loaded once per CTA with a bulk copy (cp.async.bulk).  Per
// plane:
//   z stage, all fields at once: stage the kept spectral rows, column
//   exponents, digits of every k-tile; MMA the even-mode k-tiles, fold them
//   into (H, L) pairs kept in the Z buffer (H in the slot of output m, L in
//   that of m + pz/2: the two outputs the pair feeds); MMA the odd-mode
//   k-tiles into the same tensor memory and fold E + O -> Z[m],
//   E - O -> Z[m + pz/2] in place, gathering the x stage's column exponents.
//   x stage, in tiles of 128 columns: digits, even and odd k-tiles into two
//   accumulator sets, fold to P[xp], P[xp + px/2], stage the tile in shared
//   memory and write it out coalesced.
// Every wait on an mbarrier is bounded; on expiry the kernel records an error
// word, stops taking items, and frees its tensor memory.
#include <cstdio>
#include <vector>

#include "chn_common.cuh"
#include "kernels.h"
#include "phys_common.cuh"
#include "phys_tc.cuh"
#include "setup.h"
#include "tc_common.cuh"

namespace chn {

static constexpr int kT5Threads = 512;       // 16 warps: latency hiding at one CTA per SM
static constexpr int kT5Groups = kT5Threads / 128;  // warps sharing a tensor-memory lane quarter
static constexpr int kT5Cols = 512;        // tensor-memory columns per CTA (one CTA per SM)
static constexpr int kT5XO = 256;          // x stage: odd-class accumulators at this column
static constexpr long long kT5WaitCycles = 2000000000LL;  // ~1 s at 2 GHz

// set when a bounded wait expired (the host reads and clears it)
static __device__ int g_tc5_error;

// ---------------------------------------------------------------------------
// sizes
// ---------------------------------------------------------------------------

struct T5Dims {
  PhysTcDims d;
  int nf;           // fields
  int ncz, RGz;     // z stage: data columns (nf X) and their 8-row groups
  int ncx, ntile;   // x stage: data columns (nf pz) and tiles of 128
  int NpZ, NpX;     // table rows padded to 16 (z: 2 pz/2 rows, x: px/2)
  size_t tabZ, tabX, areg, zbuf;  // region bytes
  int stage_ld;     // doubles per staged output row (px + 1)
};

__host__ __device__ inline int round16(int n) { return (n + 15) / 16 * 16; }

__host__ __device__ inline T5Dims t5_dims(const Grid& g, int nf) {
  T5Dims t;
  t.d = phys_tc_dims(g);
  t.nf = nf;
  t.ncz = nf * g.X;
  t.RGz = (t.ncz + 7) / 8;
  t.ncx = nf * g.pz;
  t.ntile = (t.ncx + 127) / 128;
  t.NpZ = round16(2 * t.d.pzh);
  t.NpX = round16(t.d.pxh);
  t.tabZ = (size_t)t.d.KTz * (7 * t.NpZ / 8) * 256;
  t.tabX = (size_t)t.d.KTx * (7 * t.NpX / 8) * 256;
  t.stage_ld = g.px + 1;
  const size_t az = (size_t)kDig * t.d.KTz * t.RGz * 256;
  const size_t ax = (size_t)kDig * t.d.KTx * 16 * 256;
  const size_t st = (size_t)128 * t.stage_ld * sizeof(double);
  size_t a = az > ax ? az : ax;
  a = a > st ? a : st;
  t.areg = (a + 1023) / 1024 * 1024;
  // the Z buffer also holds the staged spectral rows (nf X (Nz - 1) < nf X pz)
  t.zbuf = ((size_t)nf * g.pz * g.X * sizeof(cpx) + 1023) / 1024 * 1024;
  return t;
}

// shared-memory plan: tables, A region, Z buffer, then the small arrays
__host__ __device__ inline size_t t5_small_off(const T5Dims& t) { return t.tabZ + t.tabX + t.areg + t.zbuf; }

__host__ __device__ inline size_t t5_smem_bytes(const T5Dims& t) {
  return t5_small_off(t) + 128 * sizeof(int) + (size_t)((t.ncx + 3) / 4 * 4) * sizeof(int) +
         kT5Threads * sizeof(double) + 64;
}

// ---------------------------------------------------------------------------
// host tables: digits of the rows of M[rows][K] (row exponents exactly as
// append_digit_table) as a stacked B operand, k-tile blocks of
// 7 Np / 8 row groups x 256 bytes
// ---------------------------------------------------------------------------

__host__ __device__ inline size_t umma_off(int row, int k, int rgroups) {
  return ((((size_t)(k / 16) * rgroups + row / 8) * 2 + (k % 16) / 8) * 128) + (row % 8) * 16 + (k % 8) * 2;
}

static void append_umma_table(const double* M, int rows, int K, int Np, std::vector<uint8_t>& out) {
  const int KT = K / 16, rg = 7 * Np / 8;
  out.assign((size_t)KT * rg * 256, 0);
  for (int y = 0; y < rows; ++y) {
    double mx = 0.0;
    for (int j = 0; j < K; ++j) mx = std::fmax(mx, std::fabs(M[(size_t)y * K + j]));
    if (mx == 0.0) continue;
    int e = 0;
    std::frexp(mx, &e);
    for (int j = 0; j < K; ++j) {
      int d[kDig];
      digits56(std::llround(std::ldexp(M[(size_t)y * K + j], 56 - e)), d);
      for (int i = 0; i < kDig; ++i) {
        const uint16_t b = bf16_bits_of_int(d[i]);
        const size_t o = umma_off(i * Np + y, j, rg);
        out[o] = (uint8_t)(b & 0xFF);
        out[o + 1] = (uint8_t)(b >> 8);
      }
    }
  }
}

bool build_phys_tc5_tables(const HostTables& h, std::vector<uint8_t>& zt, std::vector<uint8_t>& xt) {
  std::vector<double> Az, Ax;
  std::vector<int> zmap;
  int zrows = 0, Kz = 0, xrows = 0, Kx = 0;
  if (!phys_tc_matrices(h, Az, Ax, zmap, zrows, Kz, xrows, Kx)) return false;
  append_umma_table(Az.data(), zrows, Kz, round16(zrows), zt);
  append_umma_table(Ax.data(), xrows, Kx, round16(xrows), xt);
  return true;
}

// ---------------------------------------------------------------------------
// tcgen05 / mbarrier / bulk-copy primitives
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, no swizzle; lbo = byte distance
// of core matrices adjacent in K, sbo = of 8-row groups; version 1
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor, kind::f16: D f32, A and B bf16, both K-major
__device__ __forceinline__ uint32_t umma_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, int acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count));
}

// bounded wait for the phase with the given parity; false when it expired
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > kT5WaitCycles) return false;
  }
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

template <int N>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, float (&v)[N]) {
  uint32_t r[N];
  if constexpr (N == 8) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
  } else {
    static_assert(N == 4, "x4 or x8");
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
  }
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// exact (H, L) of seven FP32 level sums (levels at lv[0..6])
__device__ __forceinline__ void fold7(const float (&lv)[kDig], long long& H, long long& L) {
  int v[kDig];
#pragma unroll
  for (int l = 0; l < kDig; ++l) v[l] = __float2int_rn(lv[l]);
  H = (long long)v[2] + (long long)v[1] * 256LL + (long long)v[0] * 65536LL;
  L = (long long)v[6] + (long long)v[5] * 256LL + (long long)v[4] * 65536LL + (long long)v[3] * 16777216LL;
}

// One stage's MMAs over the k-tiles [k0, k1): data digits (A, blocks of
// `ablk` bytes per (digit, k-tile), digit-major with KT k-tiles) against the
// stacked table (B, k-tile blocks of 7 Np / 8 row groups) into the level
// accumulators at tensor-memory column d0.  Issued by one thread.
__device__ __forceinline__ void t5_mma_stage(uint32_t tm, uint32_t d0, uint32_t a0, size_t ablk, int KT, uint32_t b0,
                                             int Np, int k0, int k1) {
  const size_t bblk = (size_t)(7 * Np / 8) * 256;
  for (int kt = k0; kt < k1; ++kt) {
#pragma unroll
    for (int i = 0; i < kDig; ++i) {
      const uint64_t ad = umma_desc(a0 + (uint32_t)(((size_t)i * KT + kt) * ablk), 128, 256);
      const int acc = (kt == k0 && i == 0) ? 0 : 1;
      // table digits k = 0 .. 6 - i, at most 256 rows of N per instruction
      int k = 0;
      while (k < kDig - i) {
        int kn = kDig - i;
        while ((kn - k) * Np > 256) --kn;
        const uint64_t bd = umma_desc(b0 + (uint32_t)(kt * bblk + (size_t)k * (Np / 8) * 256), 128, 256);
        umma_bf16(tm + d0 + (uint32_t)((i + k) * Np), ad, bd, umma_idesc(128, (kn - k) * Np), acc);
        k = kn;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// kernel
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kT5Threads, 1) k_phys_inverse_tc5(const __grid_constant__ Grid g, PhysArgs a) {
  const T5Dims t = t5_dims(g, a.nfields);
  const PhysTcDims& d = t.d;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* tabZ = smem;
  unsigned char* tabX = tabZ + t.tabZ;
  unsigned char* areg = tabX + t.tabX;
  cpx* Zb = reinterpret_cast<cpx*>(areg + t.areg);
  unsigned char* sp = smem + t5_small_off(t);
  int* exz = reinterpret_cast<int*>(sp);
  sp += 128 * sizeof(int);
  int* exx = reinterpret_cast<int*>(sp);
  sp += (size_t)((t.ncx + 3) / 4 * 4) * sizeof(int);
  double* red = reinterpret_cast<double*>(sp);
  sp += kT5Threads * sizeof(double);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sp);  // [0] tables, [1] MMA completion
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sp + 16);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int q = warp & 3, grp = warp >> 2;  // tensor-memory lane quarter, row group of the folds
  const uint32_t bar_tab = smem_u32(&bars[0]), bar_mma = smem_u32(&bars[1]);
  if (tid == 0) {
    mbar_init(bar_tab, 1);
    mbar_init(bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tslot)),
                 "r"(kT5Cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tm = *tslot;
  if (tid == 0) {
    mbar_expect_tx(bar_tab, (uint32_t)(t.tabZ + t.tabX));
    bulk_load(tabZ, g.t5Z, (uint32_t)t.tabZ, bar_tab);
    bulk_load(tabX, g.t5X, (uint32_t)t.tabX, bar_tab);
  }
  bool ok = !__syncthreads_or(!mbar_wait(bar_tab, 0));
  const bool tab_ok = ok;
  uint32_t mph = 0;  // parity of the next MMA completion

  const int Kk = g.Nz - 1;
  const size_t plane = (size_t)g.pz * g.px;
  const uint32_t a0 = smem_u32(areg), bz0 = smem_u32(tabZ), bx0 = smem_u32(tabX);
  const size_t ablkz = (size_t)t.RGz * 256, ablkx = (size_t)16 * 256;
  const long long nitems = (long long)a.ninst * g.Q;

  for (long long item = blockIdx.x; ok && item < nitems; item += gridDim.x) {
    const int inst = (int)(item / g.Q), y = (int)(item - (long long)inst * g.Q);
    if (a.skip_blocked && blocked(a.status, a.sdiv, inst)) continue;
    const cpx* __restrict__ U = a.U.at(inst);
    double* __restrict__ P = a.P.at(inst);
    if (a.pslot.stride) P += (long long)a.pslot.slot() * a.pslot.stride;
    bool nonfinite = false;

    // ---- z stage inputs: the kept spectral rows of every field, staged in
    // the Z buffer [n][kk] (n = f X + x), and each column's exponent
    for (int i = tid; i < 128; i += kT5Threads) exz[i] = 0;
    for (int i = tid; i < t.ncx; i += kT5Threads) exx[i] = 0;
    __syncthreads();
    cpx* Fin = Zb;
    {
      const int per = kT5Threads / t.ncz;
      if (tid < per * t.ncz) {
        const int n = tid % t.ncz, f = n / g.X, x = n - f * g.X;
        int emax = 0;
        for (int kk = tid / t.ncz; kk < Kk; kk += per) {
          const int z = kk < g.Nz / 2 ? kk : kk + 1;
          const cpx v = field_value(g, U, f, z, y, x);
          Fin[(size_t)n * Kk + kk] = v;
          emax = max(emax, max((int)((__double_as_longlong(v.re) >> 52) & 0x7FF),
                               (int)((__double_as_longlong(v.im) >> 52) & 0x7FF)));
        }
        if (emax) atomicMax(&exz[n], emax);
      }
    }
    __syncthreads();
    // ---- digits of every z k-tile (even modes, then odd): A blocks [i][kt]
    {
      // a warp's 32 stores fill one 128-byte row set of a core matrix pair
      // (8 rows x 4 words): lane = (n & 7) + 8 (w & 3), conflict-free
      const int KW = d.KTz * 8;
      for (int idx = tid; idx < t.RGz * 8 * KW; idx += kT5Threads) {
        const int rest = idx >> 5, ng = rest % t.RGz, wg = rest / t.RGz;
        const int n = ng * 8 + (idx & 7), w = wg * 4 + ((idx >> 3) & 3);
        if (n >= t.ncz) continue;
        const int kk = g.tcZM[w];
        cpx v = {0.0, 0.0};
        if (kk >= 0) v = Fin[(size_t)n * Kk + kk];
        const int ex = exz[n] - 1022;
        const int kt = w >> 3;
        uint32_t* dst = reinterpret_cast<uint32_t*>(areg + (size_t)kt * ablkz +
                                                    ((size_t)((n >> 3) * 2 + ((w & 7) >> 2)) * 128) + (n & 7) * 16 +
                                                    (w & 3) * 4);
        digits_pair_bf16(scaled56(v.re, ex), scaled56(v.im, ex), dst, (size_t)d.KTz * ablkz / 4);
      }
    }
    fence_async_smem();
    __syncthreads();
    // ---- even-mode k-tiles
    if (tid == 0) {
      fence_after();
      t5_mma_stage(tm, 0, a0, ablkz, d.KTz, bz0, t.NpZ, 0, d.KTzE);
      umma_commit(bar_mma);
    }
    ok = !__syncthreads_or(!mbar_wait(bar_mma, mph));
    mph ^= 1;
    if (!ok) break;
    fence_after();
    const bool zwarp = 32 * q < t.ncz;
    const int nz = 32 * q + lane;
    const int rows_grp = t.NpZ / kT5Groups;  // a multiple of 4
    // fold the even sums into (H, L) pairs in the Z buffer slots of the two
    // outputs they feed
    if (zwarp) {
      for (int r0 = grp * rows_grp; r0 < (grp + 1) * rows_grp; r0 += 4) {
        float lv[kDig][4];
#pragma unroll
        for (int l = 0; l < kDig; ++l) tmem_ld<4>(tm + ((uint32_t)(32 * q) << 16) + (uint32_t)(l * t.NpZ + r0), lv[l]);
        tmem_wait_ld();
        if (nz < t.ncz) {
          const int f = nz / g.X, x = nz - f * g.X;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int r = r0 + j;
            if (r >= 2 * d.pzh) break;
            float c[kDig];
#pragma unroll
            for (int l = 0; l < kDig; ++l) c[l] = lv[l][j];
            long long H, L;
            fold7(c, H, L);
            const bool im = r >= d.pzh;
            const int m = im ? r - d.pzh : r;
            double* sp_ = reinterpret_cast<double*>(&Zb[((size_t)f * g.pz + m) * g.X + x]) + (im ? 1 : 0);
            double* sm_ = reinterpret_cast<double*>(&Zb[((size_t)f * g.pz + m + d.pzh) * g.X + x]) + (im ? 1 : 0);
            *sp_ = __longlong_as_double(H);
            *sm_ = __longlong_as_double(L);
          }
        }
      }
    }
    fence_before();
    __syncthreads();
    // ---- odd-mode k-tiles into the same tensor memory
    if (tid == 0) {
      fence_after();
      t5_mma_stage(tm, 0, a0, ablkz, d.KTz, bz0, t.NpZ, d.KTzE, d.KTz);
      umma_commit(bar_mma);
    }
    ok = !__syncthreads_or(!mbar_wait(bar_mma, mph));
    mph ^= 1;
    if (!ok) break;
    fence_after();
    if (zwarp) {
      for (int r0 = grp * rows_grp; r0 < (grp + 1) * rows_grp; r0 += 4) {
        float lv[kDig][4];
#pragma unroll
        for (int l = 0; l < kDig; ++l) tmem_ld<4>(tm + ((uint32_t)(32 * q) << 16) + (uint32_t)(l * t.NpZ + r0), lv[l]);
        tmem_wait_ld();
        if (nz < t.ncz) {
          const int f = nz / g.X, x = nz - f * g.X;
          const int ez = exz[nz];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int r = r0 + j;
            if (r >= 2 * d.pzh) break;
            float c[kDig];
#pragma unroll
            for (int l = 0; l < kDig; ++l) c[l] = lv[l][j];
            long long HO, LO;
            fold7(c, HO, LO);
            const bool im = r >= d.pzh;
            const int m = im ? r - d.pzh : r;
            double* sp_ = reinterpret_cast<double*>(&Zb[((size_t)f * g.pz + m) * g.X + x]) + (im ? 1 : 0);
            double* sm_ = reinterpret_cast<double*>(&Zb[((size_t)f * g.pz + m + d.pzh) * g.X + x]) + (im ? 1 : 0);
            const long long HE = __double_as_longlong(*sp_), LE = __double_as_longlong(*sm_);
            const int e = g.tcZE[r] + ez - 1022 - 64;
            const double vp = round_col(HE + HO, LE + LO, e, ez);
            const double vm = round_col(HE - HO, LE - LO, e, ez);
            *sp_ = vp;
            *sm_ = vm;
            if (!(im && x == 0)) {  // c2r ignores the imaginary part of the kx = 0 bin
              const int ep = (int)((__double_as_longlong(vp) >> 52) & 0x7FF);
              const int em = (int)((__double_as_longlong(vm) >> 52) & 0x7FF);
              if (ep) atomicMax(&exx[f * g.pz + m], ep);
              if (em) atomicMax(&exx[f * g.pz + m + d.pzh], em);
            }
          }
        }
      }
    }
    fence_before();
    __syncthreads();

    // ---- x stage in tiles of 128 columns n = f pz + m; K words: Re, Im of
    // Z[m][j] for the even j, then the odd j (Im of j = 0 unused)
    double* stage = reinterpret_cast<double*>(areg);
    const int KWx = d.KTx * 8, WE = d.KTxE * 8;
    for (int tile = 0; tile < t.ntile; ++tile) {
      const int c0 = tile * 128, nct = min(128, t.ncx - c0);
      for (int idx = tid; idx < 128 * KWx; idx += kT5Threads) {
        const int rest = idx >> 5, ng = rest & 15, wg = rest >> 4;
        const int nl = ng * 8 + (idx & 7), w = wg * 4 + ((idx >> 3) & 3), n = c0 + nl;
        const int j = w < WE ? (w < d.nxE ? d.Rx * w : -1) : (w - WE < d.nxO ? 2 * (w - WE) + 1 : -1);
        cpx v = {0.0, 0.0};
        int ex = 0;
        if (nl < nct) {
          if (j >= 0) v = Zb[(size_t)n * g.X + j];
          if (j == 0) v.im = 0.0;
          ex = exx[n] - 1022;
        }
        const int kt = w >> 3;
        uint32_t* dst = reinterpret_cast<uint32_t*>(areg + (size_t)kt * ablkx +
                                                    ((size_t)((nl >> 3) * 2 + ((w & 7) >> 2)) * 128) + (nl & 7) * 16 +
                                                    (w & 3) * 4);
        digits_pair_bf16(scaled56(v.re, ex), scaled56(v.im, ex), dst, (size_t)d.KTx * ablkx / 4);
      }
      fence_async_smem();
      __syncthreads();
      if (tid == 0) {
        fence_after();
        t5_mma_stage(tm, 0, a0, ablkx, d.KTx, bx0, t.NpX, 0, d.KTxE);
        t5_mma_stage(tm, kT5XO, a0, ablkx, d.KTx, bx0, t.NpX, d.KTxE, d.KTx);
        umma_commit(bar_mma);
      }
      ok = !__syncthreads_or(!mbar_wait(bar_mma, mph));
      mph ^= 1;
      if (!ok) break;
      fence_after();
      {
        const int nl = 32 * q + lane, n = c0 + nl;
        const int rows_x = ((d.pxh + kT5Groups - 1) / kT5Groups + 3) / 4 * 4;  // rows per group, 4 | rows_x
        const int ecol = nl < nct ? exx[n] : 0;
        for (int r0 = grp * rows_x; r0 < (grp + 1) * rows_x; r0 += 4) {
          if (r0 >= d.pxh) break;
          float lvE[kDig][4], lvO[kDig][4];
#pragma unroll
          for (int l = 0; l < kDig; ++l) {
            tmem_ld<4>(tm + ((uint32_t)(32 * q) << 16) + (uint32_t)(l * t.NpX + r0), lvE[l]);
            tmem_ld<4>(tm + ((uint32_t)(32 * q) << 16) + (uint32_t)(kT5XO + l * t.NpX + r0), lvO[l]);
          }
          tmem_wait_ld();
          if (nl < nct) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int xp = r0 + j;
              if (xp >= d.pxh) break;
              float cE[kDig], cO[kDig];
#pragma unroll
              for (int l = 0; l < kDig; ++l) {
                cE[l] = lvE[l][j];
                cO[l] = lvO[l][j];
              }
              long long HE, LE, HO, LO;
              fold7(cE, HE, LE);
              fold7(cO, HO, LO);
              const int e = g.tcXE[xp] + ecol - 1022 - 64;
              const double vp = round_col(HE + HO, LE + LO, e, ecol);
              const double vm = round_col(HE - HO, LE - LO, e, ecol);
              stage[(size_t)nl * t.stage_ld + xp] = vp;
              stage[(size_t)nl * t.stage_ld + xp + d.pxh] = vm;
              nonfinite |= !finite_bits(vp) || !finite_bits(vm);
            }
          }
        }
      }
      fence_before();
      __syncthreads();
      // write the tile out: consecutive threads, consecutive xp of one row m
      for (int idx = tid; idx < nct * g.px; idx += kT5Threads) {
        const int nl = idx / g.px, xp = idx - nl * g.px, n = c0 + nl;
        const int f = n / g.pz, m = n - f * g.pz;
        P[((size_t)f * g.Q + y) * plane + (size_t)m * g.px + xp] = stage[(size_t)nl * t.stage_ld + xp];
      }
      __syncthreads();
    }
    if (!ok) break;
    if (__syncthreads_or(nonfinite) && tid == 0 && a.status) atomicOr(&a.status[inst / a.sdiv], ST_NONFINITE);
    if (a.cfl_check) {
      // the plane's CFL maximum (channel/pass1.c:116-138) from the velocity
      // fields this CTA just wrote
      double mx = 0.0;
      const double* Pu = P + (size_t)y * plane;
      const size_t fs = (size_t)g.Q * plane;
      const double c2 = g.cfl2[y];
      for (int i = tid; i < g.pz * g.px; i += kT5Threads)
        mx = fmax(mx, fabs(Pu[i]) * g.cfl1 + fabs(Pu[fs + i]) * c2 + fabs(Pu[2 * fs + i]) * g.cfl3);
      red[tid] = mx;
      __syncthreads();
      for (int w = kT5Threads / 2; w > 0; w >>= 1) {
        if (tid < w) red[tid] = fmax(red[tid], red[tid + w]);
        __syncthreads();
      }
      if (tid == 0) {
        const double c = red[0] * g.dt;
        if (a.cflmax)
          atomicMax(reinterpret_cast<unsigned long long*>(&a.cflmax[inst / a.sdiv]),
                    (unsigned long long)__double_as_longlong(c));
        if (c >= 2.8) atomicOr(&a.status[inst / a.sdiv], ST_CFL);
      }
      __syncthreads();
    }
  }
  if (!ok && tid == 0) atomicExch(&g_tc5_error, 1);
  if (!ok) {
    // a wait expired: give the copy or the MMAs still in flight (bounded)
    // time to finish before the memory they write is released
    if (!tab_ok) mbar_wait(bar_tab, 0);
    else mbar_wait(bar_mma, mph ^ 1);
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tm), "r"(kT5Cols));
  }
}

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------

static int s_t5_sms = 0;

static int s_t5_optin = 0;

// both stages split radix-2 (even pz, px); a z-stage column per tensor-memory
// lane; the accumulators within the 512 tensor-memory columns (z: 7 levels
// of the padded rows; x: two sets of 7 below column 256 each)
bool phys_tc5_fits(const Grid& g, int nf, int optin) {
  if (g.pz % 2 || g.px % 2 || nf < 1) return false;
  const T5Dims t = t5_dims(g, nf);
  return t.ncz <= 128 && 7 * t.NpZ <= kT5Cols && 7 * t.NpX <= kT5XO && t5_smem_bytes(t) <= (size_t)optin;
}

// One CTA per SM: the request is at least half the shared memory of an SM,
// so no second CTA (which would wait for the first one's tensor memory)
// shares it.
cudaError_t launch_phys_inverse_tc5(const Grid& g, const PhysArgs& a, cudaStream_t st) {
  const T5Dims t = t5_dims(g, a.nfields);
  const long long items = (long long)a.ninst * g.Q;
  const int grid = (int)(items < s_t5_sms ? items : s_t5_sms);
  if (grid <= 0) return cudaSuccess;
  size_t sm = t5_smem_bytes(t);
  const size_t one_per_sm = (size_t)s_t5_optin / 2 + 1024;
  if (sm < one_per_sm) sm = one_per_sm;
  k_phys_inverse_tc5<<<grid, kT5Threads, sm, st>>>(g, a);
  return cudaGetLastError();
}

void prepare_phys_tc5(int optin) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&s_t5_sms, cudaDevAttrMultiProcessorCount, dev);
  s_t5_optin = optin;
  cudaFuncSetAttribute(k_phys_inverse_tc5, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

// the error word of the bounded waits: returns it and clears it
int tc5_take_error() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc5_error, sizeof(int)) != cudaSuccess) return -1;
  if (v) {
    const int zero = 0;
    cudaMemcpyToSymbol(g_tc5_error, &zero, sizeof(int));
  }
  return v;
}

}  // namespace chn
