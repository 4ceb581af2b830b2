// Register-resident two-level FFTs for the Poisson solver's passes.
//
// Replaces, for the grid sizes in `reg_split`, the Stockham shared-memory
// passes of fft.cuh (the CUFFT/FFTW plan of the reference's `poissonsolver` /
// `project!`, src/N.jl:202-307).  A line of length L = N1 N2 is transformed in
// two register levels with one shared-memory exchange between them
// (Cooley-Tukey with m = N2 m1 + m2, k = k1 + N1 k2):
//   level A: the thread of sub-line m2 holds x[N2 m1 + m2] (m1 < N1), does an
//            N1-point DFT and multiplies by W_L^(m2 k1);
//   level B: the thread of k1 gathers the N2 values of its k1 from shared
//            memory and does an N2-point DFT, giving X[k1 + N1 k2].
// The small DFTs run fully unrolled in registers (radix 2/3/4/5/8 butterflies
// and their compositions with compile-time twiddles).  The level twiddles
// W_L^(m2 k1) come from a table of L entries laid out [k1][m2], so a warp
// reads them coalesced or as a broadcast.
//
// Column passes (y and z): a tile is W consecutive kx columns (the lines),
// one warp row of W lines per element, so loads and stores go straight
// between global memory and registers, coalesced along kx.  x passes: a CTA
// takes RW rows; lanes run along the row, loads and stores are direct and
// coalesced as well.
#pragma once
#include "internal.cuh"

namespace exc {

// u * W_R^J (forward W_R = exp(-2 pi i / R); INV: conjugate root).
template <int R, int J, bool INV, typename C>
__device__ __forceinline__ C mul_root(C u) {
  using T = decltype(u.x);
  constexpr int j = J % R;
  if constexpr (j == 0) {
    return u;
  } else if constexpr (2 * j == R) {
    C r; r.x = -u.x; r.y = -u.y;
    return r;
  } else if constexpr (4 * j == R) {
    return mul_mi<INV>(u);
  } else if constexpr (4 * j == 3 * R) {
    return mul_mi<!INV>(u);
  } else {
    constexpr CosSin w = cos_sin_2pi(j, R);
    constexpr T c = (T)w.c;
    constexpr T s = INV ? (T)w.s : (T)-w.s;  // root = c + i s
    C r;
    r.x = fma(c, u.x, -s * u.y);
    r.y = fma(c, u.y, s * u.x);
    return r;
  }
}

// First factor A of a composed register DFT of size R = A * (R / A).
constexpr int reg_radix_a(int R) {
  return R == 16 ? 4 : (R % 8 == 0) ? 8 : (R % 4 == 0) ? 4 : (R % 2 == 0) ? 2 : (R % 3 == 0) ? 3 : 5;
}

template <int R, bool INV, typename C> __device__ __forceinline__ void dft_reg(C* v);

// R = A B in registers: A-point DFTs over stride-B subsequences, twiddles
// W_R^(b k1), B-point DFTs; natural order in and out.
template <int A, int B, bool INV, typename C>
struct ComposedDft {
  template <int b, int k>
  static __device__ __forceinline__ void twiddle_row(const C* u, C* t) {
    if constexpr (k < A) {
      t[b * A + k] = mul_root<A * B, b * k, INV>(u[k]);
      twiddle_row<b, k + 1>(u, t);
    }
  }
  template <int b>
  static __device__ __forceinline__ void first(const C* v, C* t) {
    if constexpr (b < B) {
      C u[A];
#pragma unroll
      for (int a = 0; a < A; ++a) u[a] = v[B * a + b];
      dft_reg<A, INV>(u);
      twiddle_row<b, 0>(u, t);
      first<b + 1>(v, t);
    }
  }
  static __device__ __forceinline__ void run(C* v) {
    C t[A * B];
    first<0>(v, t);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      C u[B];
#pragma unroll
      for (int b = 0; b < B; ++b) u[b] = t[b * A + k1];
      dft_reg<B, INV>(u);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = u[k2];
    }
  }
};

template <int R, bool INV, typename C>
__device__ __forceinline__ void dft_reg(C* v) {
  if constexpr (R == 1) {
  } else if constexpr (R == 2 || R == 3 || R == 4 || R == 5 || R == 8) {
    dft_small<R, INV, C>(v);
  } else {
    constexpr int A = reg_radix_a(R);
    ComposedDft<A, R / A, INV, C>::run(v);
  }
}

// ---------------------------------------------------------------------------
// Sizes: line length L -> N1 (N2 = L / N1), 0 when L has no register plan.
// ---------------------------------------------------------------------------
// N1 <= N2: level A (the loads) runs on N2 threads per line, the larger count.
constexpr int reg_split(int L) {
  switch (L) {
    case 16: return 4;
    case 24: return 4;
    case 32: return 4;
    case 48: return 6;
    case 64: return 8;
    case 96: return 8;
    case 128: return 8;
    case 192: return 12;
    case 256: return 16;
    case 384: return 16;
    case 512: return 16;
    case 1024: return 32;
    default: return 0;
  }
}

// Column tile geometry: W lines (kx columns) per tile, 128 bytes per element
// row; FP32 lines of 384 and more take 8 columns, so the CTA of a 24- or
// 32-point level stays at 192-256 threads (two CTAs per SM at 128 registers).
template <typename T, int N1, int N2>
struct ColGeom {
  static constexpr int L = N1 * N2;
  static constexpr int W = sizeof(T) == 4 ? (L >= 384 ? 8 : 16) : 8;
  static constexpr int NR = N1 > N2 ? N1 : N2;
  static constexpr int NT = W * NR;
  static constexpr size_t SMEM = (size_t)W * L * 2 * sizeof(T);
  // CTAs per SM the register cap aims at: the registers of NR complex values
  // plus about 40 of addressing and temporaries, at most 4
  static constexpr int REGS = (int)(2 * sizeof(T) / 4) * NR + 40;
  static constexpr int MINB0 = 65536 / (NT * REGS);
  static constexpr int MINB = MINB0 < 1 ? 1 : MINB0 > 4 ? 4 : MINB0;
  static constexpr int MINB_Z = MINB > 3 ? 3 : MINB;  // z pass: one more set of twiddles live
  // z pass: the tile's 1/(lambda N) entries (8 bytes each) are prefetched
  // into shared memory at kernel start when they fit in 32 KB
  static constexpr bool TABS = (size_t)W * L * 8 <= 32768;
  static constexpr size_t SMEM_Z = SMEM + (TABS ? (size_t)W * L * 8 : 0);
};

constexpr int pow2_floor(int x) {
  int p = 1;
  while (p * 2 <= x) p *= 2;
  return p;
}

// x-pass geometry: RW rows per CTA (a power of two, about 256 threads); the
// exchange buffer row of XS complex words holds [k1][m2] with m2 stride 1 and
// k1 stride N2 + 1 (odd: conflict-free level-B reads); XS = N2 (mod 16) so the
// rows of a half warp start on different banks.
template <typename T, int N1, int N2>
struct XGeom {
  static constexpr int L = N1 * N2;
  static constexpr int NR = N1 > N2 ? N1 : N2;
  static constexpr int RW = pow2_floor(256 / NR);
  static constexpr int NT = RW * NR;
  static constexpr int XS0 = N1 * (N2 + 1);
  static constexpr int XS = XS0 + (((N2 - XS0) % 16) + 16) % 16;
  static constexpr size_t SMEM = (size_t)RW * XS * 2 * sizeof(T);
  // FP32 divergence pass: the RW rows (one z plane when RW divides n) of
  // u_x, u_z, u_z(z-1) and RW + 1 rows of u_y are staged in shared memory by
  // 16-byte cp.async copies, which keep every load in flight without holding
  // registers; the exchange buffer reuses the staging area afterwards
  static constexpr int NX = 2 * L;
  static constexpr size_t STAGE_BYTES = (size_t)(4 * RW + 1) * NX * sizeof(T);
  static constexpr bool STAGE = sizeof(T) == 4 && NX % RW == 0 && STAGE_BYTES <= 100 * 1024;
  static constexpr size_t SMEM_DIV = STAGE && STAGE_BYTES > SMEM ? STAGE_BYTES : SMEM;
};

// ---------------------------------------------------------------------------
// Column pass along y (es = P, outer = z, outer_stride = n P) or z (es = n P,
// outer = y, outer_stride = P).  One tile of W kx columns per CTA:
// blockIdx.x = outer * ntx + tile column, blockIdx.z = slot.
// ---------------------------------------------------------------------------
template <typename T, int N1, int N2, bool INV>
__global__ void __launch_bounds__(ColGeom<T, N1, N2>::NT, ColGeom<T, N1, N2>::MINB)
rcols_kernel(cplx<T>* __restrict__ g, int nkx, int ntx, long long es, long long outer_stride,
             const cplx<T>* __restrict__ tl, SlotBatch sb) {
  using C = cplx<T>;
  using G = ColGeom<T, N1, N2>;
  constexpr int W = G::W;
  extern __shared__ unsigned char smem_raw[];
  C* xs = reinterpret_cast<C*>(smem_raw);
  if (sb.active && !sb.active[blockIdx.z]) return;
  g += blockIdx.z * sb.wstride;
  const int outer = blockIdx.x / ntx, kx0 = (blockIdx.x - outer * ntx) * W;
  const int lines = min(W, nkx - kx0);
  C* const base = g + outer * outer_stride + kx0;
  const int tid = threadIdx.x, line = tid % W;
  const bool lv = line < lines;
  if (tid < W * N2) {
    const int m2 = tid / W;
    const C* p = base + m2 * es + line;
    const long long step = N2 * es;
    C v[N1];
#pragma unroll
    for (int m1 = 0; m1 < N1; ++m1) v[m1] = lv ? p[m1 * step] : mk<T>(0, 0);
    dft_reg<N1, INV>(v);
#pragma unroll
    for (int k1 = 1; k1 < N1; ++k1) {
      const C w = __ldg(&tl[k1 * N2 + m2]);
      v[k1] = INV ? cmulc(v[k1], w) : cmul(v[k1], w);
    }
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) xs[(k1 * N2 + m2) * W + line] = v[k1];
  }
  __syncthreads();
  if (tid < W * N1) {
    const int k1 = tid / W;
    C v[N2];
#pragma unroll
    for (int m2 = 0; m2 < N2; ++m2) v[m2] = xs[(k1 * N2 + m2) * W + line];
    dft_reg<N2, INV>(v);
    if (lv) {
      C* q = base + k1 * es + line;
      const long long step = N1 * es;
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) q[k2 * step] = v[k2];
    }
  }
}

// z pass with the spectral divide of `project!` (src/N.jl:281-298): forward
// transform along z (levels A, B), multiply by 1/(lambda N) (zero for the mean
// mode), inverse from registers: N2-point inverse DFT over k2, twiddle
// W_L^(-k1 j1), exchange, N1-point inverse DFT over k1, giving y[j1 + N2 j2].
// `invlap` is the float64 table [kz][ky][kx] (FP32: (hi, lo) float pairs).
template <typename T, int N1, int N2>
__global__ void __launch_bounds__(ColGeom<T, N1, N2>::NT, ColGeom<T, N1, N2>::MINB_Z)
rzsolve_kernel(cplx<T>* __restrict__ g, int n, int nkx, int ntx, int P, const cplx<T>* __restrict__ tl,
               const double* __restrict__ invlap, SlotBatch sb) {
  using C = cplx<T>;
  using G = ColGeom<T, N1, N2>;
  constexpr int W = G::W, L = N1 * N2;
  extern __shared__ unsigned char smem_raw[];
  C* xs = reinterpret_cast<C*>(smem_raw);
  double* tab = reinterpret_cast<double*>(smem_raw + G::SMEM);  // [kz][line], 8-byte entries
  if (sb.active && !sb.active[blockIdx.z]) return;
  g += blockIdx.z * sb.wstride;
  const long long es = (long long)n * P;
  const int ky = blockIdx.x / ntx, kx0 = (blockIdx.x - ky * ntx) * W;
  const int lines = min(W, nkx - kx0);
  C* const base = g + (long long)ky * P + kx0;
  const int tid = threadIdx.x, line = tid % W;
  const bool lv = line < lines;
  if constexpr (G::TABS) {
    for (int t = tid; t < L * W; t += G::NT) {
      const int kz = t / W, l = t - kz * W;
      if (l < lines) cp_async_word(&tab[t], invlap + invlap_index(n, kz, ky, kx0 + l));
    }
    cp_async_commit();
  }
  if (tid < W * N2) {
    const int m2 = tid / W;
    const C* p = base + m2 * es + line;
    const long long step = N2 * es;
    C v[N1];
#pragma unroll
    for (int m1 = 0; m1 < N1; ++m1) v[m1] = lv ? p[m1 * step] : mk<T>(0, 0);
    dft_reg<N1, false>(v);
#pragma unroll
    for (int k1 = 1; k1 < N1; ++k1) v[k1] = cmul(v[k1], __ldg(&tl[k1 * N2 + m2]));
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) xs[(k1 * N2 + m2) * W + line] = v[k1];
  }
  if constexpr (G::TABS) cp_async_wait_all();
  __syncthreads();
  C v[N2];
  const int k1 = tid / W;
  const bool actb = tid < W * N1;
  if (actb) {
#pragma unroll
    for (int m2 = 0; m2 < N2; ++m2) v[m2] = xs[(k1 * N2 + m2) * W + line];
    dft_reg<N2, false>(v);
    // divide: mode (kz, ky, kx) with kz = k1 + N1 k2 (folded table)
    if (lv) {
      const int kx = kx0 + line;
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) {
        const int kz = k1 + N1 * k2;
        const long long mi = G::TABS ? (long long)kz * W + line : invlap_index(n, kz, ky, kx);
        const double* src_f = G::TABS ? tab : invlap;
        if constexpr (sizeof(T) == 4) {
          // float64 factor as hi + lo floats: v (hi + lo) with one FMA keeps
          // the factor's float64 precision up to the final float rounding
          const float2 f = reinterpret_cast<const float2*>(src_f)[mi];
          v[k2].x = fmaf(v[k2].x, f.x, v[k2].x * f.y);
          v[k2].y = fmaf(v[k2].y, f.x, v[k2].y * f.y);
        } else {
          const double f = src_f[mi];
          v[k2].x = (T)((double)v[k2].x * f);
          v[k2].y = (T)((double)v[k2].y * f);
        }
      }
    }
    dft_reg<N2, true>(v);
#pragma unroll
    for (int j1 = 1; j1 < N2; ++j1) v[j1] = cmulc(v[j1], __ldg(&tl[k1 * N2 + j1]));
  }
  __syncthreads();  // level-B reads of xs are complete
  if (actb) {
#pragma unroll
    for (int j1 = 0; j1 < N2; ++j1) xs[(j1 * N1 + k1) * W + line] = v[j1];
  }
  __syncthreads();
  if (tid < W * N2) {
    const int j1 = tid / W;
    C y[N1];
#pragma unroll
    for (int k = 0; k < N1; ++k) y[k] = xs[(j1 * N1 + k) * W + line];
    dft_reg<N1, true>(y);
    if (lv) {
      C* q = base + j1 * es + line;
      const long long step = N2 * es;
#pragma unroll
      for (int j2 = 0; j2 < N1; ++j2) q[j2 * step] = y[j2];
    }
  }
}

// ---------------------------------------------------------------------------
// Pipelined column passes (FP32 grids whose tile and divide table fit twice
// in shared memory).  Persistent CTAs walk the tiles t = blockIdx.x,
// blockIdx.x + gridDim.x, ...; a tile's W lines arrive in a staging buffer by
// 16-byte cp.async copies issued while the previous tile is transformed, so
// the HBM reads overlap the DFTs instead of alternating with them (two CTAs
// per SM).  Same arithmetic as rcols_kernel / rzsolve_kernel, term for term.
// ---------------------------------------------------------------------------
template <typename T, int N1, int N2>
struct PipeGeom {
  using CG = ColGeom<T, N1, N2>;
  static constexpr int L = N1 * N2, W = CG::W;
  static constexpr int CPL = 16 / (int)(2 * sizeof(T));  // complex words per 16-byte piece
  static constexpr int PW = W / CPL;                      // pieces per line row
  // exchange rows padded by 64 bytes when a tile row is 64 bytes wide: a
  // warp's four row groups then alternate between the two halves of the
  // banks (two wavefronts) instead of sharing the same 16 banks
  // (the y passes; measured slower in the z pass, which keeps the dense rows)
  static constexpr int PADC = (W * 2 * (int)sizeof(T) == 64) ? 64 / (2 * (int)sizeof(T)) : 0;
  static constexpr int RS1 = N2 * W + PADC;  // y pass exchange: row k1 of [m2][line]
  static constexpr int XSC = N1 * RS1;       // y pass exchange size, complex words
  static constexpr size_t SMEM_COLS = ((size_t)XSC + (size_t)W * L) * 2 * sizeof(T);
  // z pass exchange rows: level B reads rows k1 (stride RZ1), the last level
  // reads rows j1 (stride RZ2); PZ1, PZ2 pad them (complex words).  Unpadded,
  // a warp's four row groups share banks (4-way conflicts), yet 64-byte pads
  // measured slower at 512^3 FP32 (step 16.98 ms unpadded; 17.04, 17.18 and
  // 17.17 ms padding the first, the second and both): the pass is bound by
  // its instruction stream, not by these conflicts.
  static constexpr int PZ1 = 0, PZ2 = 0;
  static constexpr int RZ1 = N2 * W + PZ1, RZ2 = N1 * W + PZ2;
  static constexpr int XZ = (N1 * RZ1 > N2 * RZ2 ? N1 * RZ1 : N2 * RZ2);  // exchange size, complex words
  static constexpr size_t SMEM_Z = ((size_t)XZ + (size_t)W * L) * 2 * sizeof(T) + (size_t)W * L * 8;
  static constexpr bool OK = sizeof(T) == 4 && CG::TABS && SMEM_Z <= 110 * 1024;
};

// Stage the W lines of tile (outer, kx0) -- rows r = 0..L-1 at base + r es --
// into stg[r][line]; pieces past the padded row (column >= P) are skipped.
template <typename T, int N1, int N2>
__device__ __forceinline__ void stage_tile(cplx<T>* stg, const cplx<T>* base, long long es, int kx0, int P, int tid,
                                           int nthreads) {
  using Gp = PipeGeom<T, N1, N2>;
  constexpr int W = Gp::W, CPL = Gp::CPL, PW = Gp::PW, L = Gp::L;
  for (int q = tid; q < L * PW; q += nthreads) {
    const int r = q / PW, j = q - r * PW;
    if (kx0 + j * CPL < P) cp_async_16(stg + r * W + j * CPL, base + r * es + j * CPL);
  }
}

template <typename T, int N1, int N2, bool INV>
__global__ void __launch_bounds__(ColGeom<T, N1, N2>::NT, 3)
rcols_pipe_kernel(cplx<T>* __restrict__ g, int nkx, int ntx, int ntiles, int P, long long es, long long outer_stride,
                  const cplx<T>* __restrict__ tl, SlotBatch sb) {
  using C = cplx<T>;
  using G = ColGeom<T, N1, N2>;
  using Gp = PipeGeom<T, N1, N2>;
  constexpr int W = G::W, RS1 = Gp::RS1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* xs = reinterpret_cast<C*>(smem_raw);
  C* stg = xs + Gp::XSC;
  if (sb.active && !sb.active[blockIdx.z]) return;
  g += blockIdx.z * sb.wstride;
  const int tid = threadIdx.x, line = tid % W;
  auto prefetch = [&](int t) {
    const int outer = t / ntx, kx0 = (t - outer * ntx) * W;
    stage_tile<T, N1, N2>(stg, g + outer * outer_stride + kx0, es, kx0, P, tid, G::NT);
    cp_async_commit();
  };
  int t = blockIdx.x;
  if (t < ntiles) prefetch(t);
  for (; t < ntiles; t += gridDim.x) {
    const int outer = t / ntx, kx0 = (t - outer * ntx) * W;
    const int lines = min(W, nkx - kx0);
    const bool lv = line < lines;
    cp_async_wait_all();
    __syncthreads();  // the tile is staged; the previous tile's xs reads are done
    if (tid < W * N2) {
      const int m2 = tid / W;
      C v[N1];
#pragma unroll
      for (int m1 = 0; m1 < N1; ++m1) v[m1] = stg[(N2 * m1 + m2) * W + line];
      dft_reg<N1, INV>(v);
#pragma unroll
      for (int k1 = 1; k1 < N1; ++k1) {
        const C w = __ldg(&tl[k1 * N2 + m2]);
        v[k1] = INV ? cmulc(v[k1], w) : cmul(v[k1], w);
      }
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1) xs[k1 * RS1 + m2 * W + line] = v[k1];
    }
    __syncthreads();  // stg consumed, xs complete
    if (t + (int)gridDim.x < ntiles) prefetch(t + gridDim.x);
    if (tid < W * N1) {
      const int k1 = tid / W;
      C v[N2];
#pragma unroll
      for (int m2 = 0; m2 < N2; ++m2) v[m2] = xs[k1 * RS1 + m2 * W + line];
      dft_reg<N2, INV>(v);
      if (lv) {
        C* q = g + outer * outer_stride + kx0 + k1 * es + line;
        const long long step = N1 * es;
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) q[k2 * step] = v[k2];
      }
    }
  }
}

template <typename T, int N1, int N2>
__global__ void __launch_bounds__(ColGeom<T, N1, N2>::NT, 2)
rzsolve_pipe_kernel(cplx<T>* __restrict__ g, int n, int nkx, int ntx, int ntiles, int P,
                    const cplx<T>* __restrict__ tl, const double* __restrict__ invlap, SlotBatch sb) {
  using C = cplx<T>;
  using G = ColGeom<T, N1, N2>;
  using Gp = PipeGeom<T, N1, N2>;
  constexpr int W = G::W, L = N1 * N2, RS1 = Gp::RZ1, RS2 = Gp::RZ2;
  static_assert(G::TABS, "the pipelined z pass stages the divide table");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* xs = reinterpret_cast<C*>(smem_raw);
  C* stg = xs + Gp::XZ;
  double* tab = reinterpret_cast<double*>(stg + W * L);  // [kz][line]
  if (sb.active && !sb.active[blockIdx.z]) return;
  g += blockIdx.z * sb.wstride;
  const long long es = (long long)n * P;
  const int tid = threadIdx.x, line = tid % W;
  auto prefetch_cols = [&](int t) {
    const int ky = t / ntx, kx0 = (t - ky * ntx) * W;
    stage_tile<T, N1, N2>(stg, g + (long long)ky * P + kx0, es, kx0, P, tid, G::NT);
    cp_async_commit();
  };
  auto prefetch_tab = [&](int t) {
    const int ky = t / ntx, kx0 = (t - ky * ntx) * W;
    const int lines = min(W, nkx - kx0);
    for (int q = tid; q < L * W; q += G::NT) {
      const int kz = q / W, l = q - kz * W;
      if (l < lines) cp_async_word(&tab[q], invlap + invlap_index(n, kz, ky, kx0 + l));
    }
    cp_async_commit();
  };
  int t = blockIdx.x;
  if (t < ntiles) {
    prefetch_cols(t);
    prefetch_tab(t);
  }
  for (; t < ntiles; t += gridDim.x) {
    const int ky = t / ntx, kx0 = (t - ky * ntx) * W;
    const int lines = min(W, nkx - kx0);
    const bool lv = line < lines;
    C* const base = g + (long long)ky * P + kx0;
    cp_async_wait_all();
    __syncthreads();  // tile and table staged; the previous tile's xs reads are done
    if (tid < W * N2) {
      const int m2 = tid / W;
      C v[N1];
#pragma unroll
      for (int m1 = 0; m1 < N1; ++m1) v[m1] = stg[(N2 * m1 + m2) * W + line];
      dft_reg<N1, false>(v);
#pragma unroll
      for (int k1 = 1; k1 < N1; ++k1) v[k1] = cmul(v[k1], __ldg(&tl[k1 * N2 + m2]));
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1) xs[k1 * RS1 + m2 * W + line] = v[k1];
    }
    __syncthreads();  // stg consumed, xs complete
    if (t + (int)gridDim.x < ntiles) prefetch_cols(t + gridDim.x);
    C v[N2];
    const int k1 = tid / W;
    const bool actb = tid < W * N1;
    if (actb) {
#pragma unroll
      for (int m2 = 0; m2 < N2; ++m2) v[m2] = xs[k1 * RS1 + m2 * W + line];
      dft_reg<N2, false>(v);
      if (lv) {
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) {
          const int kz = k1 + N1 * k2;
          if constexpr (sizeof(T) == 4) {
            const float2 f = reinterpret_cast<const float2*>(tab)[kz * W + line];
            v[k2].x = fmaf(v[k2].x, f.x, v[k2].x * f.y);
            v[k2].y = fmaf(v[k2].y, f.x, v[k2].y * f.y);
          } else {
            const double f = tab[kz * W + line];
            v[k2].x = (T)((double)v[k2].x * f);
            v[k2].y = (T)((double)v[k2].y * f);
          }
        }
      }
      dft_reg<N2, true>(v);
#pragma unroll
      for (int j1 = 1; j1 < N2; ++j1) v[j1] = cmulc(v[j1], __ldg(&tl[k1 * N2 + j1]));
    }
    __syncthreads();  // level-B reads of xs and of the table are complete
    if (t + (int)gridDim.x < ntiles) prefetch_tab(t + gridDim.x);
    if (actb) {
#pragma unroll
      for (int j1 = 0; j1 < N2; ++j1) xs[j1 * RS2 + k1 * W + line] = v[j1];
    }
    __syncthreads();
    if (tid < W * N2) {
      const int j1 = tid / W;
      C y[N1];
#pragma unroll
      for (int k = 0; k < N1; ++k) y[k] = xs[j1 * RS2 + k * W + line];
      dft_reg<N1, true>(y);
      if (lv) {
        C* q = base + j1 * es + line;
        const long long step = N2 * es;
#pragma unroll
        for (int j2 = 0; j2 < N1; ++j2) q[j2 * step] = y[j2];
      }
    }
  }
}

// Persistent CTAs per slot of a pipelined column pass: the CTAs resident at
// once (per_sm on each of the 152 SMs) shared among the slots.
inline int pipe_ctas(int ntiles, int nslots, int per_sm) {
  const int per = (per_sm * 152 + nslots - 1) / nslots;
  return ntiles < per ? ntiles : per;
}

// ---------------------------------------------------------------------------
// x pass, real -> half complex (L = n/2 complex points z_m = x_2m + i x_2m+1
// per row, then X_k = (Z_k + conj Z_{L-k})/2 - (i/2) W_n^k (Z_k - conj Z_{L-k}),
// k = 0..L).  With DIV the row is d = div(u) (src/N.jl:222-238) computed on
// the fly.  blockIdx.x = row block, blockIdx.y = slot.
// ---------------------------------------------------------------------------
template <typename T, int N1, int N2, bool DIV, bool STAGE = false>
__global__ void __launch_bounds__(XGeom<T, N1, N2>::NT)
rr2c_kernel(const T* __restrict__ src, T inv_h, cplx<T>* __restrict__ out, int P, const cplx<T>* __restrict__ tw,
            const cplx<T>* __restrict__ tl, SlotBatch sb) {
  using C = cplx<T>;
  using T2 = C;
  using G = XGeom<T, N1, N2>;
  constexpr int L = N1 * N2, n = 2 * L, RW = G::RW, XS = G::XS;
  extern __shared__ unsigned char smem_raw[];
  C* xs = reinterpret_cast<C*>(smem_raw);
  const int slot = blockIdx.y;
  if (sb.active && !sb.active[slot]) return;
  src += slot * sb.ustride;
  out += slot * sb.wstride;
  constexpr long long nn = (long long)n * n, N = nn * n;
  const long long row0 = (long long)blockIdx.x * RW;
  const int tid = threadIdx.x;
  if constexpr (STAGE) {
    // rows row0 .. row0 + RW - 1: one z plane, y = y0 .. y0 + RW - 1
    static_assert(DIV && G::STAGE, "staging is the FP32 divergence pass");
    T* const sux = reinterpret_cast<T*>(smem_raw);
    T* const suy = sux + RW * n;            // rows y0 - 1 .. y0 + RW - 1
    T* const suz = suy + (RW + 1) * n;
    T* const szm = suz + RW * n;            // u_z of plane z - 1
    const int z = (int)(row0 / n), y0 = (int)(row0 - (long long)z * n);
    const int zm = z == 0 ? n - 1 : z - 1;
    const T* gx = src + row0 * n;
    const T* gy = src + N + row0 * n;
    const T* gz = src + 2 * N + row0 * n;
    const T* gzm = src + 2 * N + ((long long)zm * n + y0) * n;
    constexpr int PR = RW * n / 4;  // 16-byte pieces of RW rows
    for (int t = tid; t < PR; t += G::NT) {
      cp_async_16(sux + 4 * t, gx + 4 * t);
      cp_async_16(suy + n + 4 * t, gy + 4 * t);
      cp_async_16(suz + 4 * t, gz + 4 * t);
      cp_async_16(szm + 4 * t, gzm + 4 * t);
    }
    const T* gyd = src + N + ((long long)z * n + (y0 == 0 ? n - 1 : y0 - 1)) * n;
    for (int t = tid; t < n / 4; t += G::NT) cp_async_16(suy + 4 * t, gyd + 4 * t);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
  }
  C v[N1];
  const int line = tid / N2, m2 = tid - line * N2;
  if (tid < RW * N2) {
    const long long row = row0 + line;
    if (STAGE) {
      const T* ux = reinterpret_cast<const T*>(smem_raw) + line * n;
      const T* uy = ux + RW * n;          // row y - 1 of the staged u_y
      const T* uz = uy + (RW + 1) * n;
      const T* uzm = uz + RW * n;
      const T2* ux2 = reinterpret_cast<const T2*>(ux);
      const T2* uy2 = reinterpret_cast<const T2*>(uy + n);
      const T2* uyd = reinterpret_cast<const T2*>(uy);
      const T2* uz2 = reinterpret_cast<const T2*>(uz);
      const T2* uzd = reinterpret_cast<const T2*>(uzm);
#pragma unroll
      for (int m1 = 0; m1 < N1; ++m1) {
        const int m = m2 + N2 * m1;
        const int xm = (m == 0) ? n - 1 : 2 * m - 1;
        const T2 a0 = ux2[m], b0 = uy2[m], b1 = uyd[m], c0 = uz2[m], c1 = uzd[m];
        const T uxm = ux[xm];
        v[m1].x = ((a0.x - uxm) + (b0.x - b1.x) + (c0.x - c1.x)) * inv_h;
        v[m1].y = ((a0.y - a0.x) + (b0.y - b1.y) + (c0.y - c1.y)) * inv_h;
      }
    } else if (row < nn) {
      const long long base = row * n;
      if constexpr (!DIV) {
        const T2* s2 = reinterpret_cast<const T2*>(src + base);
#pragma unroll
        for (int m1 = 0; m1 < N1; ++m1) v[m1] = s2[m2 + N2 * m1];
      } else {
        const int z = (int)(row / n), y = (int)(row - (long long)z * n);
        const long long rowy = (long long)z * n + (y == 0 ? n - 1 : y - 1);
        const long long rowz = (long long)(z == 0 ? n - 1 : z - 1) * n + y;
        const T* ux = src;
        const T* uy = src + N;
        const T* uz = src + 2 * N;
        const T2* ux2 = reinterpret_cast<const T2*>(ux + base);
        const T2* uy2 = reinterpret_cast<const T2*>(uy + base);
        const T2* uyd = reinterpret_cast<const T2*>(uy + rowy * n);
        const T2* uz2 = reinterpret_cast<const T2*>(uz + base);
        const T2* uzd = reinterpret_cast<const T2*>(uz + rowz * n);
#pragma unroll
        for (int m1 = 0; m1 < N1; ++m1) {
          const int m = m2 + N2 * m1;
          const int xm = (m == 0) ? n - 1 : 2 * m - 1;
          const T2 a0 = ux2[m], b0 = uy2[m], b1 = uyd[m], c0 = uz2[m], c1 = uzd[m];
          const T uxm = ux[base + xm];
          v[m1].x = ((a0.x - uxm) + (b0.x - b1.x) + (c0.x - c1.x)) * inv_h;
          v[m1].y = ((a0.y - a0.x) + (b0.y - b1.y) + (c0.y - c1.y)) * inv_h;
        }
      }
    } else {
#pragma unroll
      for (int m1 = 0; m1 < N1; ++m1) v[m1] = mk<T>(0, 0);
    }
    dft_reg<N1, false>(v);
#pragma unroll
    for (int k1 = 1; k1 < N1; ++k1) v[k1] = cmul(v[k1], __ldg(&tl[k1 * N2 + m2]));
  }
  if constexpr (STAGE) __syncthreads();  // the staged rows are read; xs reuses them
  if (tid < RW * N2) {
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) xs[line * XS + k1 * (N2 + 1) + m2] = v[k1];
  }
  __syncthreads();
  const int lb = tid / N1, k1 = tid - lb * N1;
  const bool actb = tid < RW * N1;
  C z[N2];
  if (actb) {
#pragma unroll
    for (int m2 = 0; m2 < N2; ++m2) z[m2] = xs[lb * XS + k1 * (N2 + 1) + m2];
    dft_reg<N2, false>(z);
  }
  __syncthreads();
  if (actb) {
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) xs[lb * XS + k1 + N1 * k2] = z[k2];
  }
  __syncthreads();
  const long long row = row0 + lb;
  if (actb && row < nn) {
    C* o = out + row * P;
    const C* zr = xs + lb * XS;
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
      const int k = k1 + N1 * k2;
      const C zk = z[k2];
      const C zc = cconj(zr[k == 0 ? 0 : L - k]);
      const C e = cadd(zk, zc), d = csub(zk, zc);
      const C wo = cmul(d, __ldg(&tw[k]));
      C X;
      X.x = (T)0.5 * (e.x + wo.y);
      X.y = (T)0.5 * (e.y - wo.x);
      o[k] = X;
    }
    if (k1 == 0) {
      // k = L (Nyquist) from Z_0
      const C zk = z[0], zc = cconj(z[0]);
      const C e = cadd(zk, zc), d = csub(zk, zc);
      const C wo = cmul(d, __ldg(&tw[L]));
      C X;
      X.x = (T)0.5 * (e.x + wo.y);
      X.y = (T)0.5 * (e.y - wo.x);
      o[L] = X;
    }
  }
}

// ---------------------------------------------------------------------------
// x pass, half complex -> real, in place (row pitch P complex = 2P reals):
//   Z_k = (X_k + conj X_{L-k}) + i W_n^-k (X_k - conj X_{L-k}), k < L,
//   z = IDFT_L(Z) (unnormalised), x_2m = Re z_m, x_2m+1 = Im z_m.
// Every load of a row precedes the barrier, every store follows it.
// ---------------------------------------------------------------------------
template <typename T, int N1, int N2>
__global__ void __launch_bounds__(XGeom<T, N1, N2>::NT)
rc2r_kernel(cplx<T>* __restrict__ g, int P, const cplx<T>* __restrict__ tw, const cplx<T>* __restrict__ tl,
            SlotBatch sb) {
  using C = cplx<T>;
  using G = XGeom<T, N1, N2>;
  constexpr int L = N1 * N2, n = 2 * L, RW = G::RW, XS = G::XS;
  extern __shared__ unsigned char smem_raw[];
  C* xs = reinterpret_cast<C*>(smem_raw);
  if (sb.active && !sb.active[blockIdx.y]) return;
  g += blockIdx.y * sb.wstride;
  constexpr long long nn = (long long)n * n;
  const long long row0 = (long long)blockIdx.x * RW;
  const int tid = threadIdx.x;
  if (tid < RW * N2) {
    const int line = tid / N2, m2 = tid - line * N2;
    const long long row = row0 + line;
    C v[N1];
    if (row < nn) {
      const C* x = g + row * P;
#pragma unroll
      for (int m1 = 0; m1 < N1; ++m1) {
        const int k = m2 + N2 * m1;
        const C xa = x[k], xb = x[L - k];
        const C e = cadd(xa, cconj(xb));
        const C o = cmulc(csub(xa, cconj(xb)), __ldg(&tw[k]));
        v[m1].x = e.x - o.y;
        v[m1].y = e.y + o.x;
      }
    } else {
#pragma unroll
      for (int m1 = 0; m1 < N1; ++m1) v[m1] = mk<T>(0, 0);
    }
    dft_reg<N1, true>(v);
#pragma unroll
    for (int k1 = 1; k1 < N1; ++k1) v[k1] = cmulc(v[k1], __ldg(&tl[k1 * N2 + m2]));
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) xs[line * XS + k1 * (N2 + 1) + m2] = v[k1];
  }
  __syncthreads();
  const int lb = tid / N1, k1 = tid - lb * N1;
  const long long row = row0 + lb;
  if (tid < RW * N1 && row < nn) {
    C z[N2];
#pragma unroll
    for (int m2 = 0; m2 < N2; ++m2) z[m2] = xs[lb * XS + k1 * (N2 + 1) + m2];
    dft_reg<N2, true>(z);
    C* r = g + row * P;  // reals x_2m, x_2m+1 = complex slot m of the row
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) r[k1 + N1 * k2] = z[k2];
  }
}

// One-size launcher; instantiated per grid in the two translation units.
template <typename T, int NN>
struct RegSolve {
  static constexpr int A1 = reg_split(NN), A2 = NN / (A1 ? A1 : 1);
  static constexpr int H = NN / 2;
  static constexpr int B1 = reg_split(H), B2 = H / (B1 ? B1 : 1);
  using CG = ColGeom<T, A1, A2>;
  using XG = XGeom<T, B1, B2>;
  using C_t = cplx<T>;

  static cudaError_t configure() {
    cudaError_t e = cudaSuccess;
    auto set = [&](const void* f, size_t sh) {
      if (e == cudaSuccess && sh > 48 * 1024)
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
    };
    set((const void*)rcols_kernel<T, A1, A2, false>, CG::SMEM);
    set((const void*)rcols_kernel<T, A1, A2, true>, CG::SMEM);
    set((const void*)rzsolve_kernel<T, A1, A2>, CG::SMEM_Z);
    set((const void*)rr2c_kernel<T, B1, B2, true>, XG::SMEM);
    if constexpr (XG::STAGE) set((const void*)rr2c_kernel<T, B1, B2, true, true>, XG::SMEM_DIV);
    set((const void*)rr2c_kernel<T, B1, B2, false>, XG::SMEM);
    set((const void*)rc2r_kernel<T, B1, B2>, XG::SMEM);
    if constexpr (PipeGeom<T, A1, A2>::OK) {
      set((const void*)rcols_pipe_kernel<T, A1, A2, false>, PipeGeom<T, A1, A2>::SMEM_COLS);
      set((const void*)rcols_pipe_kernel<T, A1, A2, true>, PipeGeom<T, A1, A2>::SMEM_COLS);
      set((const void*)rzsolve_pipe_kernel<T, A1, A2>, PipeGeom<T, A1, A2>::SMEM_Z);
    }
    return e;
  }

  // y forward, z solve, y inverse on the spectral array g (pitch P)
  static void columns(C_t* g, int nkx, int P, const C_t* tln, const double* invlap, cudaStream_t st,
                      const SlotBatch& sb, int ns) {
    constexpr int n = NN;
    const int ntx = (nkx + CG::W - 1) / CG::W;
    const int ntiles = ntx * n;
    if constexpr (PipeGeom<T, A1, A2>::OK) {
      using Gp = PipeGeom<T, A1, A2>;
      const dim3 gy((unsigned)pipe_ctas(ntiles, ns, 3), 1, ns), gz((unsigned)pipe_ctas(ntiles, ns, 4), 1, ns);
      rcols_pipe_kernel<T, A1, A2, false><<<gy, CG::NT, Gp::SMEM_COLS, st>>>(g, nkx, ntx, ntiles, P, P,
                                                                             (long long)n * P, tln, sb);
      rzsolve_pipe_kernel<T, A1, A2><<<gz, CG::NT, Gp::SMEM_Z, st>>>(g, n, nkx, ntx, ntiles, P, tln, invlap, sb);
      rcols_pipe_kernel<T, A1, A2, true><<<gy, CG::NT, Gp::SMEM_COLS, st>>>(g, nkx, ntx, ntiles, P, P,
                                                                            (long long)n * P, tln, sb);
    } else {
      const dim3 gc((unsigned)ntiles, 1, ns);
      rcols_kernel<T, A1, A2, false><<<gc, CG::NT, CG::SMEM, st>>>(g, nkx, ntx, P, (long long)n * P, tln, sb);
      rzsolve_kernel<T, A1, A2><<<gc, CG::NT, CG::SMEM_Z, st>>>(g, n, nkx, ntx, P, tln, invlap, sb);
      rcols_kernel<T, A1, A2, true><<<gc, CG::NT, CG::SMEM, st>>>(g, nkx, ntx, P, (long long)n * P, tln, sb);
    }
  }

  static cudaError_t solve(exc_poisson* ps, const T* src, bool vec, cudaStream_t st, const SlotBatch& sb, int ns) {
    using C = cplx<T>;
    constexpr int n = NN;
    const int P = ps->P, nkx = n / 2 + 1;
    C* g = reinterpret_cast<C*>(ps->work);
    const C* tw = reinterpret_cast<const C*>(ps->tw);
    const C* tln = reinterpret_cast<const C*>(ps->twl_n);
    const C* tlh = reinterpret_cast<const C*>(ps->twl_h);
    const long long nn = (long long)n * n;
    const dim3 gx((unsigned)((nn + XG::RW - 1) / XG::RW), ns);
    bool staged = false;
    if constexpr (XG::STAGE) {
      // 16-byte copies need a 16-byte aligned field (slot strides 3 n^3 words keep it)
      if (vec && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
        rr2c_kernel<T, B1, B2, true, true><<<gx, XG::NT, XG::SMEM_DIV, st>>>(src, (T)(1.0 / ps->h), g, P, tw, tlh, sb);
        staged = true;
      }
    }
    if (staged) {
    } else if (vec)
      rr2c_kernel<T, B1, B2, true><<<gx, XG::NT, XG::SMEM, st>>>(src, (T)(1.0 / ps->h), g, P, tw, tlh, sb);
    else
      rr2c_kernel<T, B1, B2, false><<<gx, XG::NT, XG::SMEM, st>>>(src, (T)1, g, P, tw, tlh, sb);
    columns(g, nkx, P, tln, ps->invlap, st, sb, ns);
    rc2r_kernel<T, B1, B2><<<gx, XG::NT, XG::SMEM, st>>>(g, P, tw, tlh, sb);
    return cudaGetLastError();
  }
};

}  // namespace exc
