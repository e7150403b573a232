// Shared-memory FFT building blocks for the padded x/z transforms.
//
// Transforms are unnormalised, exp(sign * 2 pi i jk/N).  A batch of nb
// transforms of length N lives in shared memory with element stride es and
// batch stride bs.  Each pass is a Stockham autosort radix-R step (output in
// natural order after the last pass); threads stride over (transform,
// butterfly) pairs and the caller separates passes with __syncthreads().
//
// The 3/2-padded transforms of this solver have a zero band in the middle
// third of the input (inverse) or an unneeded middle third of the output
// (forward).  Running the radix-3 pass first (inverse) or last (forward) at
// stride N/3 turns that band into the middle butterfly input (output), which
// the pass then skips.  N = 3*M with M = Nz/2 (z) or Nx/2 (x); M is split
// into radix 4, 2, 3 and 5 passes.
#pragma once

#include "chn_common.cuh"

namespace chn {

struct FftPlan {
  int n;           // length
  int np;          // number of passes
  int radix[12];   // radix of each pass in execution order
  bool r3first;    // the radix-3 pass that meets the 3/2-padding band is pass 0 (else the last pass)
};

__host__ __device__ inline int plan_factor(int m, int* out) {
  int k = 0;
  while (m > 1) {
    int f;
    if (m % 4 == 0) f = 4;
    else if (m % 2 == 0) f = 2;
    else if (m % 3 == 0) f = 3;
    else if (m % 5 == 0) f = 5;
    else f = m;  // generic odd radix (slow path)
    out[k++] = f;
    m /= f;
  }
  return k;
}

// lengths 3 * 2^i * 3^j need only radices 2, 3, 4
__host__ __device__ inline bool radix234_only(int n) {
  if (n % 3) return false;
  int m = n / 3;
  while (m % 2 == 0) m /= 2;
  while (m % 3 == 0) m /= 3;
  return m == 1;
}

// inverse plan: radix 3 first; forward plan: radix 3 last
__host__ __device__ inline FftPlan make_plan(int n, bool radix3_first) {
  FftPlan p;
  p.n = n;
  p.r3first = radix3_first;
  int f[12];
  int k = plan_factor(n / 3, f);
  p.np = k + 1;
  if (radix3_first) {
    p.radix[0] = 3;
    for (int i = 0; i < k; ++i) p.radix[i + 1] = f[i];
  } else {
    for (int i = 0; i < k; ++i) p.radix[i] = f[i];
    p.radix[k] = 3;
  }
  return p;
}

// twiddle W_N^e for sign s from a table of exp(-2 pi i k/N)
__device__ __forceinline__ cpx tw_get(const cpx* tw, int e, int N, int sign) {
  cpx w = tw[e % N];
  if (sign > 0) w.im = -w.im;
  return w;
}

template <int R>
__device__ __forceinline__ void dft_small(cpx* v, int sign, const cpx* tw, int N) {
  if (R == 2) {
    cpx a = v[0], b = v[1];
    v[0].re = a.re + b.re; v[0].im = a.im + b.im;
    v[1].re = a.re - b.re; v[1].im = a.im - b.im;
  } else if (R == 4) {
    const double s = (double)sign;
    double a0r = v[0].re + v[2].re, a0i = v[0].im + v[2].im;
    double a1r = v[0].re - v[2].re, a1i = v[0].im - v[2].im;
    double b0r = v[1].re + v[3].re, b0i = v[1].im + v[3].im;
    double b1r = v[1].re - v[3].re, b1i = v[1].im - v[3].im;
    v[0].re = a0r + b0r; v[0].im = a0i + b0i;
    v[2].re = a0r - b0r; v[2].im = a0i - b0i;
    v[1].re = a1r - s * b1i; v[1].im = a1i + s * b1r;
    v[3].re = a1r + s * b1i; v[3].im = a1i - s * b1r;
  } else if (R == 3) {
    // W_3 = -1/2 + i*h, h = sign * sin(2 pi/3)
    const double h = tw_get(tw, N / 3, N, sign).im;
    double sr = v[1].re + v[2].re, si = v[1].im + v[2].im;
    double dr = v[1].re - v[2].re, di = v[1].im - v[2].im;
    double mr = fma(-0.5, sr, v[0].re), mi = fma(-0.5, si, v[0].im);
    v[0].re = v[0].re + sr; v[0].im = v[0].im + si;
    v[1].re = fma(-h, di, mr); v[1].im = fma(h, dr, mi);
    v[2].re = fma(h, di, mr); v[2].im = fma(-h, dr, mi);
  } else {
    cpx t[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
      double ar = 0.0, ai = 0.0;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        cpx w = tw_get(tw, ((u * q) % R) * (N / R), N, sign);
        ar = fma(v[q].re, w.re, fma(-v[q].im, w.im, ar));
        ai = fma(v[q].re, w.im, fma(v[q].im, w.re, ai));
      }
      t[u].re = ar; t[u].im = ai;
    }
#pragma unroll
    for (int u = 0; u < R; ++u) v[u] = t[u];
  }
}

// One Stockham pass.  Ns = product of the radices already applied.
// zero_mid (radix 3 only): the input at r = 1 is known to be zero.
// skip_mid (radix 3 only): the output at r = 1 is not needed.
template <int R>
__device__ void stockham_pass(const cpx* __restrict__ in, cpx* __restrict__ out, int N, int Ns, int nb,
                              int es, int bs, const cpx* tw, int sign, bool zero_mid, bool skip_mid) {
  const int M = N / R;
  const int tot = nb * M;
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    const int b = t / M, j = t - b * M;
    const cpx* src = in + b * bs;
    cpx v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (R == 3 && r == 1 && zero_mid) { v[r].re = 0.0; v[r].im = 0.0; }
      else v[r] = src[(j + r * M) * es];
    }
    const int jm = j % Ns;
    if (Ns > 1 && jm != 0) {
      const int step = N / (Ns * R);
#pragma unroll
      for (int r = 1; r < R; ++r) {
        if (R == 3 && r == 1 && zero_mid) continue;
        v[r] = cmul(v[r], tw_get(tw, r * jm * step, N, sign));
      }
    }
    dft_small<R>(v, sign, tw, N);
    const int idxD = (j / Ns) * Ns * R + jm;
    cpx* dst = out + b * bs;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (R == 3 && r == 1 && skip_mid) continue;
      dst[(idxD + r * Ns) * es] = v[r];
    }
  }
}

// Run a full transform; data starts in buf0, result ends in the returned buffer.
// Callers must __syncthreads() before (data ready) and after (result ready).
// GENERAL = false compiles radices 2, 3 and 4 only (lengths 3 * 2^i * 3^j): the
// radix-5 and -7 butterflies more than double the registers of a kernel.
template <bool GENERAL = true>
__device__ inline cpx* fft_run(const FftPlan& p, cpx* buf0, cpx* buf1, int nb, int es, int bs,
                               const cpx* tw, int sign, bool prune) {
  cpx* in = buf0;
  cpx* out = buf1;
  int Ns = 1;
  for (int s = 0; s < p.np; ++s) {
    const int R = p.radix[s];
    // only the designated radix-3 pass meets the zero band; n/3 may hold
    // further factors of 3 (3Nz/2 = 72), whose passes are not pruned
    const bool zero_mid = prune && p.r3first && s == 0 && R == 3;
    const bool skip_mid = prune && !p.r3first && s == p.np - 1 && R == 3;
    switch (R) {
      case 2: stockham_pass<2>(in, out, p.n, Ns, nb, es, bs, tw, sign, false, false); break;
      case 3: stockham_pass<3>(in, out, p.n, Ns, nb, es, bs, tw, sign, zero_mid, skip_mid); break;
      case 4: stockham_pass<4>(in, out, p.n, Ns, nb, es, bs, tw, sign, false, false); break;
      case 5:
        if constexpr (GENERAL) stockham_pass<5>(in, out, p.n, Ns, nb, es, bs, tw, sign, false, false);
        break;
      case 7:
        if constexpr (GENERAL) stockham_pass<7>(in, out, p.n, Ns, nb, es, bs, tw, sign, false, false);
        break;
      default: break;  // sizes are validated on the host
    }
    Ns *= R;
    __syncthreads();
    cpx* t = in; in = out; out = t;
  }
  return in;
}

}  // namespace chn
