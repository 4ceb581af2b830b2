// Batched radix-2/3/4/5/8 (and prime radix 7/11/13/17) Stockham FFTs over lines
// held in shared memory.
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

// Threads per CTA: one radix-8 butterfly per thread per pass over a full tile.
template <typename C> constexpr int fft_threads() { return sizeof(C) == 16 ? 256 : 512; }
// Max complex values per CTA (nlines * L): 32 KB of data.
template <typename C> constexpr int fft_tile() { return 32768 / (int)sizeof(C); }
// Shared-memory lines are padded with one slot after every 8 elements
// (element e of a line at pe(e)), so the strided writes of the early
// Stockham passes (stride R complex) and the column moves spread over all
// banks; a line of L elements takes padded_len(L) slots.
__host__ __device__ __forceinline__ int pe(int e) { return e + (e >> 3); }
__host__ __device__ __forceinline__ int padded_len(int L) { return L + (L >> 3) + 1; }
// Pass sequence of a length-L transform: n8 radix-8 passes, then at most one
// radix-4 or radix-2 pass, then the radix-3, 5, 7, 11, 13 and 17 passes
// (L = 8^n8 4^n4 2^n2 3^n3 5^n5 7^n7 11^n11 13^n13 17^n17).
// The pass index math divides by nb = L/R and by Ns (the product of the
// earlier radices); both divisions use multiply-high reciprocals
// ceil(2^32/d), exact for every quotient here (dividends < 2^17, d <= 2^11;
// checked exhaustively), and 0 marks d == 1.
constexpr int FFT_MAX_PASSES = 12;
struct FftPlan {
  int L;
  int n8, n4, n2, n3, n5, n7, n11, n13, n17;
  unsigned rnb[FFT_MAX_PASSES], rns[FFT_MAX_PASSES];
  unsigned rL, rL1, rhalf, r2L;  // reciprocals of L, L + 1, L/2 + 1, 2L (row splits of the x passes)
};

inline unsigned fast_recip(unsigned d) { return d <= 1 ? 0u : (unsigned)((0x100000000ull + d - 1) / d); }
__device__ __forceinline__ unsigned fast_div(unsigned x, unsigned r) { return r ? __umulhi(x, r) : x; }

inline FftPlan make_plan(int L) {
  FftPlan p{};
  p.L = L;
  int m = L, a = 0, b = 0, c5 = 0, c7 = 0, c11 = 0, c13 = 0, c17 = 0;
  while (m % 2 == 0) { m /= 2; ++a; }
  while (m % 3 == 0) { m /= 3; ++b; }
  while (m % 5 == 0) { m /= 5; ++c5; }
  while (m % 7 == 0) { m /= 7; ++c7; }
  while (m % 11 == 0) { m /= 11; ++c11; }
  while (m % 13 == 0) { m /= 13; ++c13; }
  while (m % 17 == 0) { m /= 17; ++c17; }
  p.n8 = a / 3;
  p.n4 = (a % 3) == 2;
  p.n2 = (a % 3) == 1;
  p.n3 = b;
  p.n5 = c5;
  p.n7 = c7;
  p.n11 = c11;
  p.n13 = c13;
  p.n17 = c17;
  int radix[FFT_MAX_PASSES], np = 0;
  for (int q = 0; q < p.n8; ++q) radix[np++] = 8;
  if (p.n4) radix[np++] = 4;
  if (p.n2) radix[np++] = 2;
  for (int q = 0; q < p.n3; ++q) radix[np++] = 3;
  for (int q = 0; q < p.n5; ++q) radix[np++] = 5;
  for (int q = 0; q < p.n7; ++q) radix[np++] = 7;
  for (int q = 0; q < p.n11; ++q) radix[np++] = 11;
  for (int q = 0; q < p.n13; ++q) radix[np++] = 13;
  for (int q = 0; q < p.n17; ++q) radix[np++] = 17;
  int Ns = 1;
  for (int q = 0; q < np; ++q) {
    p.rnb[q] = fast_recip((unsigned)(L / radix[q]));
    p.rns[q] = fast_recip((unsigned)Ns);
    Ns *= radix[q];
  }
  p.rL = fast_recip((unsigned)L);
  p.rL1 = fast_recip((unsigned)L + 1);
  p.rhalf = fast_recip((unsigned)(L / 2 + 1));
  p.r2L = fast_recip((unsigned)(2 * L));
  return p;
}

// ---------------------------------------------------------------------------
// Compile-time roots of unity: cos and sin of 2 pi j / R by octant reduction
// and Taylor series on [0, pi/4] (terms to x^23: below 1e-17 there).
// ---------------------------------------------------------------------------
constexpr double kPiD = 3.14159265358979323846;
constexpr double taylor_sin(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int k = 1; k < 12; ++k) {
    term *= -x2 / (double)((2 * k) * (2 * k + 1));
    sum += term;
  }
  return sum;
}
constexpr double taylor_cos(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k < 12; ++k) {
    term *= -x2 / (double)((2 * k - 1) * (2 * k));
    sum += term;
  }
  return sum;
}
struct CosSin { double c, s; };
// angle 2 pi j / R = q pi/4 + theta, q the octant
constexpr CosSin cos_sin_2pi(int j, int R) {
  j %= R;
  if (j < 0) j += R;
  const int q = (8 * j) / R, r = 8 * j - q * R;
  if (q % 2 == 0) {
    const double t = kPiD * r / (4.0 * R);
    const double c = taylor_cos(t), s = taylor_sin(t);
    switch ((q / 2) & 3) {
      case 0: return {c, s};
      case 1: return {-s, c};
      case 2: return {-c, -s};
      default: return {s, -c};
    }
  }
  // odd octant: angle = p pi/2 - phi, p = (q + 1)/2, phi = pi/4 - theta
  const double f = kPiD * (R - r) / (4.0 * R);
  const double c = taylor_cos(f), s = taylor_sin(f);
  switch (((q + 1) / 2) & 3) {
    case 0: return {c, -s};
    case 1: return {s, c};
    case 2: return {-c, s};
    default: return {-s, -c};
  }
}

// cos and sin of 2 pi m / R for m < R, for indexing with unrolled loop
// counters (folded to immediates).
template <int R> struct RootTable { double c[R], s[R]; };
template <int R> constexpr RootTable<R> root_table() {
  RootTable<R> t{};
  for (int m = 0; m < R; ++m) {
    const CosSin w = cos_sin_2pi(m, R);
    t.c[m] = w.c;
    t.s[m] = w.s;
  }
  return t;
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
  } else if constexpr (R == 5) {
    // X1 = a1 - i b1, X4 = a1 + i b1, X2 = a2 - i b2, X3 = a2 + i b2 (forward)
    const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;  // cos(2 pi/5), cos(4 pi/5)
    const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;   // sin(2 pi/5), sin(4 pi/5)
    const C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    const C t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
    C a1, a2, b1, b2;
    a1.x = v[0].x + c1 * t1.x + c2 * t2.x; a1.y = v[0].y + c1 * t1.y + c2 * t2.y;
    a2.x = v[0].x + c2 * t1.x + c1 * t2.x; a2.y = v[0].y + c2 * t1.y + c1 * t2.y;
    b1.x = s1 * t3.x + s2 * t4.x; b1.y = s1 * t3.y + s2 * t4.y;
    b2.x = s2 * t3.x - s1 * t4.x; b2.y = s2 * t3.y - s1 * t4.y;
    const C ib1 = mul_mi<INV>(b1), ib2 = mul_mi<INV>(b2);
    v[0] = cadd(v[0], cadd(t1, t2));
    v[1] = cadd(a1, ib1);
    v[4] = csub(a1, ib1);
    v[2] = cadd(a2, ib2);
    v[3] = csub(a2, ib2);
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
  } else {
    // odd prime R >= 7 by pairs (j, R - j): with t_j = v_j + v_{R-j} and
    // d_j = v_j - v_{R-j}, X_k = a_k - i b_k and X_{R-k} = a_k + i b_k
    // (forward), a_k = v_0 + sum_j cos(2 pi jk/R) t_j, b_k = sum_j sin(2 pi jk/R) d_j
    static_assert(R % 2 == 1 && R >= 7, "radix");
    constexpr int H = (R - 1) / 2;
    constexpr RootTable<R> rt = root_table<R>();
    C t[H], d[H];
    C x0 = v[0];
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      t[j - 1] = cadd(v[j], v[R - j]);
      d[j - 1] = csub(v[j], v[R - j]);
      x0 = cadd(x0, t[j - 1]);
    }
    const C v0 = v[0];
#pragma unroll
    for (int k = 1; k <= H; ++k) {
      C a = v0, b;
      b.x = (T)0;
      b.y = (T)0;
#pragma unroll
      for (int j = 1; j <= H; ++j) {
        const T c = (T)rt.c[(j * k) % R], sn = (T)rt.s[(j * k) % R];
        a.x = fma(c, t[j - 1].x, a.x);
        a.y = fma(c, t[j - 1].y, a.y);
        b.x = fma(sn, d[j - 1].x, b.x);
        b.y = fma(sn, d[j - 1].y, b.y);
      }
      const C ib = mul_mi<INV>(b);
      v[k] = cadd(a, ib);
      v[R - k] = csub(a, ib);
    }
    v[0] = x0;
  }
}

// One Stockham pass of radix R over all lines of the CTA's tile.
template <int R, bool INV, typename C>
__device__ __forceinline__ void fft_pass(C* s, int ls, int nlines, int L, int Ns, unsigned rnb, unsigned rns,
                                         const C* __restrict__ tw, int n) {
  constexpr int NT = fft_threads<C>();
  constexpr int NB = (fft_tile<C>() / R + NT - 1) / NT;
  const int nb = L / R;
  const int total = nlines * nb;
  const int twmul = n / (Ns * R);
  C v[NB][R];
  int obase[NB], ebase[NB];
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    int t = threadIdx.x + b * NT;
    obase[b] = -1;
    if (t < total) {
      const int line = (int)fast_div((unsigned)t, rnb), j = t - line * nb;
      C* ln = s + line * ls;
      const int q = (int)fast_div((unsigned)j, rns);
      const int k = j - q * Ns;
#pragma unroll
      for (int r = 0; r < R; ++r) v[b][r] = ln[pe(j + r * nb)];
      if (Ns > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          C w = __ldg(&tw[r * k * twmul]);
          v[b][r] = INV ? cmulc(v[b][r], w) : cmul(v[b][r], w);
        }
      }
      dft_small<R, INV, C>(v[b]);
      obase[b] = line * ls;
      ebase[b] = q * Ns * R + k;
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    if (obase[b] >= 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) s[obase[b] + pe(ebase[b] + r * Ns)] = v[b][r];
    }
  }
  __syncthreads();
}

// Move a tile of `lines` columns x n rows (row stride `es` elements, columns
// contiguous in global memory) between global memory and line-major shared
// memory (line l, element e at s[l*ls + e]).  Full tiles of a power-of-two
// width use shifts for the index split and, for float2 elements, 16-byte
// accesses of column pairs; loops are unrolled so several accesses are in
// flight per thread.
template <bool LOAD, typename C>
__device__ __forceinline__ void tile_move(C* s, int ls, C* base, long long es, int lines, int W, int wlog, int n) {
  if (lines == W) {
    if constexpr (sizeof(C) == 8) {
      if (W >= 2) {
        const int hl = W >> 1, hlog = wlog - 1, tot = hl * n;
#pragma unroll 4
        for (int t = threadIdx.x; t < tot; t += blockDim.x) {
          const int e = t >> hlog, l2 = t & (hl - 1);
          float4* g = reinterpret_cast<float4*>(base + e * es + 2 * l2);
          C* a = s + (2 * l2) * ls + pe(e);
          if (LOAD) {
            const float4 v = *g;
            a[0].x = v.x; a[0].y = v.y;
            a[ls].x = v.z; a[ls].y = v.w;
          } else {
            *g = make_float4(a[0].x, a[0].y, a[ls].x, a[ls].y);
          }
        }
        return;
      }
    }
    const int tot = W * n;
#pragma unroll 4
    for (int t = threadIdx.x; t < tot; t += blockDim.x) {
      const int e = t >> wlog, l = t & (W - 1);
      if (LOAD) s[l * ls + pe(e)] = base[e * es + l];
      else base[e * es + l] = s[l * ls + pe(e)];
    }
    return;
  }
  for (int t = threadIdx.x; t < lines * n; t += blockDim.x) {
    const int e = t / lines, l = t - e * lines;
    if (LOAD) s[l * ls + pe(e)] = base[e * es + l];
    else base[e * es + l] = s[l * ls + pe(e)];
  }
}

// Asynchronous copy of a column tile (`lines` columns x n rows, row stride
// `es` elements) from global memory into line-major shared memory with
// cp.async: one 8-byte (FP32 complex) or 16-byte (FP64 complex) copy per
// element, consecutive threads on consecutive columns of a row, nothing held
// in registers.  The caller commits the group and waits for it (cp_wait)
// before a __syncthreads and the first read of the tile.
__device__ __forceinline__ void cp_async_elem(void* smem, const void* gmem, int bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  if (bytes == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory"); }

template <typename C>
__device__ __forceinline__ void tile_load_async(C* s, int ls, const C* base, long long es, int lines, int W,
                                                int wlog, int n) {
  if (lines == W) {
    const int tot = W * n;
#pragma unroll 4
    for (int t = threadIdx.x; t < tot; t += blockDim.x) {
      const int e = t >> wlog, l = t & (W - 1);
      cp_async_elem(s + l * ls + pe(e), base + e * es + l, (int)sizeof(C));
    }
    return;
  }
  for (int t = threadIdx.x; t < lines * n; t += blockDim.x) {
    const int e = t / lines, l = t - e * lines;
    cp_async_elem(s + l * ls + pe(e), base + e * es + l, (int)sizeof(C));
  }
}

// Full transform of every line in the tile (natural-order in and out).  One
// loop per radix keeps each pass body's registers separate.
template <bool INV, bool EXT, typename C>
__device__ void fft_lines(C* s, int ls, int nlines, const FftPlan& plan,
                          const C* __restrict__ tw, int n) {
  int Ns = 1, p = 0;
  const int L = plan.L;
  for (int q = 0; q < plan.n8; ++q, ++p) { fft_pass<8, INV>(s, ls, nlines, L, Ns, plan.rnb[p], plan.rns[p], tw, n); Ns *= 8; }
  if (plan.n4) { fft_pass<4, INV>(s, ls, nlines, L, Ns, plan.rnb[p], plan.rns[p], tw, n); Ns *= 4; ++p; }
  if (plan.n2) { fft_pass<2, INV>(s, ls, nlines, L, Ns, plan.rnb[p], plan.rns[p], tw, n); Ns *= 2; ++p; }
  for (int q = 0; q < plan.n3; ++q, ++p) { fft_pass<3, INV>(s, ls, nlines, L, Ns, plan.rnb[p], plan.rns[p], tw, n); Ns *= 3; }
  for (int q = 0; q < plan.n5; ++q, ++p) { fft_pass<5, INV>(s, ls, nlines, L, Ns, plan.rnb[p], plan.rns[p], tw, n); Ns *= 5; }
  if constexpr (!EXT) return;
  for (int q = 0; q < plan.n7; ++q, ++p) { fft_pass<7, INV>(s, ls, nlines, L, Ns, plan.rnb[p], plan.rns[p], tw, n); Ns *= 7; }
  for (int q = 0; q < plan.n11; ++q, ++p) { fft_pass<11, INV>(s, ls, nlines, L, Ns, plan.rnb[p], plan.rns[p], tw, n); Ns *= 11; }
  for (int q = 0; q < plan.n13; ++q, ++p) { fft_pass<13, INV>(s, ls, nlines, L, Ns, plan.rnb[p], plan.rns[p], tw, n); Ns *= 13; }
  for (int q = 0; q < plan.n17; ++q, ++p) { fft_pass<17, INV>(s, ls, nlines, L, Ns, plan.rnb[p], plan.rns[p], tw, n); Ns *= 17; }
}

}  // namespace exc
