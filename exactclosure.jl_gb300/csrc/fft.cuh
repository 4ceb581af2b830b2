// Batched radix-2/3/4/8 Stockham FFTs over lines held in shared memory.
//
// Replaces the CUFFT/FFTW real-to-complex plan of the reference's Poisson
// solver (`poissonsolver`/`project!`, src/N.jl:202-307).  A CTA holds
// `nlines` lines of length L (line stride ls >= L, padded against bank
// conflicts); each pass reads R values per butterfly into registers,
// twiddles, transforms, synchronises and writes them back in place
// (autosort order).  Twiddles come from one table of W_n^m = exp(-2 pi i m/n),
// m < n; a length-L transform with L | n reads it with stride n/L.
#pragma once
#include "exc_common.cuh"

namespace exc {

constexpr int FFT_THREADS = 256;
constexpr int FFT_TILE = 4096;  // max complex values per CTA (nlines * L)
constexpr int FFT_MAXPASS = 12;

struct FftPlan {
  int L;             // transform length
  int npass;
  int radix[FFT_MAXPASS];
};

inline FftPlan make_plan(int L) {
  FftPlan p{};
  p.L = L;
  int m = L, a = 0, b = 0;
  while (m % 2 == 0) { m /= 2; ++a; }
  while (m % 3 == 0) { m /= 3; ++b; }
  int np = 0;
  while (a >= 3) { p.radix[np++] = 8; a -= 3; }
  if (a == 2) p.radix[np++] = 4;
  if (a == 1) p.radix[np++] = 2;
  while (b-- > 0) p.radix[np++] = 3;
  p.npass = np;
  return p;
}

// In-register DFT of size R (forward: exp(-2 pi i qr/R); INV: conjugate).
template <int R, bool INV, typename C> __device__ __forceinline__ void dft_small(C* v) {
  using T = decltype(v[0].x);
  if constexpr (R == 2) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (R == 3) {
    const T s3 = (T)0.86602540378443864676;  // sin(pi/3)
    C t1 = cadd(v[1], v[2]);
    C t2; t2.x = v[0].x - (T)0.5 * t1.x; t2.y = v[0].y - (T)0.5 * t1.y;
    C d = csub(v[1], v[2]);
    // forward: -i*s3*d ; inverse: +i*s3*d
    C t3; t3.x = s3 * d.x; t3.y = s3 * d.y;
    t3 = mul_mi<INV>(t3);
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  } else if constexpr (R == 4) {
    C t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    C t2 = cadd(v[1], v[3]), t3 = mul_mi<INV>(csub(v[1], v[3]));
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  } else if constexpr (R == 8) {
    const T r2 = (T)0.70710678118654752440;
    C a[4], b[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) { a[k] = cadd(v[k], v[k + 4]); b[k] = csub(v[k], v[k + 4]); }
    // b_k *= W8^k  (forward W8 = (1 - i)/sqrt2)
    {
      C x = b[1];
      C y;
      if (INV) { y.x = (x.x - x.y) * r2; y.y = (x.x + x.y) * r2; }
      else     { y.x = (x.x + x.y) * r2; y.y = (x.y - x.x) * r2; }
      b[1] = y;
      b[2] = mul_mi<INV>(b[2]);
      x = b[3];
      if (INV) { y.x = -(x.x + x.y) * r2; y.y = (x.x - x.y) * r2; }
      else     { y.x = (x.y - x.x) * r2; y.y = -(x.x + x.y) * r2; }
      b[3] = y;
    }
    dft_small<4, INV, C>(a);
    dft_small<4, INV, C>(b);
#pragma unroll
    for (int k = 0; k < 4; ++k) { v[2 * k] = a[k]; v[2 * k + 1] = b[k]; }
  }
}

// One Stockham pass of radix R over all lines of the CTA's tile.
template <int R, bool INV, typename C>
__device__ __forceinline__ void fft_pass(C* s, int ls, int nlines, int L, int Ns,
                                         const C* __restrict__ tw, int n) {
  constexpr int NB = (FFT_TILE / R + FFT_THREADS - 1) / FFT_THREADS;
  const int nb = L / R;
  const int total = nlines * nb;
  const int twmul = n / (Ns * R);
  C v[NB][R];
  int obase[NB];
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    int t = threadIdx.x + b * FFT_THREADS;
    obase[b] = -1;
    if (t < total) {
      int line = t / nb, j = t - line * nb;
      C* ln = s + line * ls;
      int k = j % Ns;
#pragma unroll
      for (int r = 0; r < R; ++r) v[b][r] = ln[j + r * nb];
      if (Ns > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          C w = __ldg(&tw[r * k * twmul]);
          v[b][r] = INV ? cmulc(v[b][r], w) : cmul(v[b][r], w);
        }
      }
      dft_small<R, INV, C>(v[b]);
      obase[b] = line * ls + (j / Ns) * Ns * R + k;
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    if (obase[b] >= 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) s[obase[b] + r * Ns] = v[b][r];
    }
  }
  __syncthreads();
}

// Full transform of every line in the tile (natural-order in and out).
template <bool INV, typename C>
__device__ void fft_lines(C* s, int ls, int nlines, const FftPlan& plan,
                          const C* __restrict__ tw, int n) {
  int Ns = 1;
  for (int p = 0; p < plan.npass; ++p) {
    int R = plan.radix[p];
    switch (R) {
      case 8: fft_pass<8, INV>(s, ls, nlines, plan.L, Ns, tw, n); break;
      case 4: fft_pass<4, INV>(s, ls, nlines, plan.L, Ns, tw, n); break;
      case 3: fft_pass<3, INV>(s, ls, nlines, plan.L, Ns, tw, n); break;
      default: fft_pass<2, INV>(s, ls, nlines, plan.L, Ns, tw, n); break;
    }
    Ns *= R;
  }
}

}  // namespace exc
