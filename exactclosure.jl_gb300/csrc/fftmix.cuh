// FP64 Poisson solve by mixed-precision iterative refinement.
//
// The FP64 pressure solve of `project!` (src/N.jl:256-307) computes p with
// L_h p = d, d = div(u), on the GPU's FP64 pipe, which on GB300 retires about
// two operations per clock per SM: the FFT passes of a 512^3 solve are bound
// by it.  This solve instead runs the FFTs in FP32 (register-resident passes
// of fftreg.cuh, bound by HBM) and recovers FP64 accuracy by refinement with
// residuals formed in FP64:
//
//   q1 = S32(d),       r1 = d  - L_h q1
//   q2 = S32(r1),      r2 = r1 - L_h q2
//   q3 = S32(r2),      p  = (q1 + q2) + q3
//
// where S32 is the FP32 spectral solve (relative error about 1e-7) and L_h
// the 7-point staggered Laplacian, (sum of the 6 neighbours - 6 p) / h^2,
// whose eigenvalues are the spectral solver's -4/h^2 sum sin^2(pi k/n).  Each
// correction shrinks the error by about the FP32 solve's relative error, so
// after two corrections p agrees with the FP64 FFT solve to FP64 rounding
// (about 1e-15 relative for smooth and for white-noise right-hand sides).
// The corrections q1, q2 are kept as FP32 fields and p is written once, by
// the last pass; the stencil sums of L_h q_k are
// formed from FP32 values by error-free extraction (stencil7_f32) on the
// FP32 pipe and rounded once to FP64, more accurate than the six FP64
// additions they replace; each residual then costs three FP64 operations
// per cell instead of seven.  The divergence is formed once in FP64
// (unscaled by 1/h: the FP32 solves carry the factor 1/h in their
// 1/(lambda N) table) and the first residual replaces it; the pressure's
// mean (the solution's free constant, which the FP32 solves leave at their
// rounding level) is measured during the last residual pass and removed in
// the last accumulation, so p has zero mean like the reference's -- unless
// the owner reads p only through its gradient (mix_zero_mean false: the case
// stepper), where the constant changes nothing.
//
// Included by fftreg_f32.cu only: the FP32 column kernels it launches must be
// the instantiations of that translation unit, whose shared-memory opt-ins
// RegSolve<float, N>::configure sets.
#pragma once
#include "fftreg.cuh"

namespace exc {

enum { MIX_DIV = 0, MIX_SCAL = 1, MIX_RES = 2, MIX_RES_MEAN = 3 };
enum { MIX_Q = 0, MIX_FIN = 1, MIX_FIN_MEAN = 2 };

// Conversions between the FP64 fields and the FP32 transforms on the integer
// pipe (the FP64 pipe, about two operations per clock per SM on GB300, is the
// solve's bottleneck), by moving the IEEE 754 binary64/binary32 fields:
// exponent rebiased by 1023 - 127 = 896, mantissa shifted by 29 bits.
//
// FP64 -> FP32 truncates the mantissa (the refinement needs about seven
// digits from each FP32 solve, not a rounded input); magnitudes below the
// smallest normal float become a signed zero, above the largest float an
// infinity, NaN stays NaN.
__device__ __forceinline__ float f64_to_f32_trunc(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned a = hi & 0x7FFFFFFFu, sign = hi & 0x80000000u;
  const unsigned t = a - 0x38000000u;  // exponent field minus 896 (in bits 30..20)
  unsigned f = (__funnelshift_l(lo, t, 3) & 0x7FFFFFFFu) | sign;
  if (a < 0x38100000u) f = sign;  // below 2^-126 (and zero)
  if (a >= 0x47F00000u) f = sign | 0x7F800000u | ((a > 0x7FF00000u || (a == 0x7FF00000u && lo)) ? 0x400000u : 0u);
  return __uint_as_float(f);
}

// FP32 -> FP64, exact for normal numbers, zeros, infinities and NaN (float
// subnormals, below 1.2e-38, become a signed zero).
__device__ __forceinline__ double f32_to_f64(float v) {
  const unsigned b = __float_as_uint(v);
  const unsigned a = b & 0x7FFFFFFFu, sign = b & 0x80000000u;
  unsigned hi = ((a >> 3) + (a >= 0x7F800000u ? 0x70000000u : 0x38000000u)) | sign;
  unsigned lo = b << 29;
  if (a < 0x00800000u) { hi = sign; lo = 0u; }
  return __hiloint2double((int)hi, (int)lo);
}

// The FP32 value the conversion above puts into p: float subnormals become a
// signed zero, so the correction kept for the next residual is the one added.
__device__ __forceinline__ float f32_flush(float v) {
  const unsigned b = __float_as_uint(v);
  return (b & 0x7F800000u) ? v : __uint_as_float(b & 0x80000000u);
}

// One level of error-free extraction (ExtractScalar of Rump, Ogita and Oishi,
// "Accurate floating-point summation part I: faithful rounding", SIAM J. Sci.
// Comput. 31(1), 2008): for a power of two sigma and |t| <= sigma / 2, hi =
// fl(fl(sigma + t) - sigma) is exact (Sterbenz) and a multiple of u sigma (u =
// 2^-24), and t - hi is exact with |t - hi| <= u sigma; t becomes t - hi.
__device__ __forceinline__ float extract_hi(float sigma, float& t) {
  const float hi = __fsub_rn(__fadd_rn(sigma, t), sigma);
  t = __fsub_rn(t, hi);
  return hi;
}

// (n0 + ... + n5) - 6 c of FP32 values, rounded once to FP64.  The eight
// terms (the neighbours, -4c, -2c) have |t| <= M < 2^(E+1); with sigma1 =
// 2^(E+5) every partial sum of the extracted parts is a multiple of u sigma1
// below sigma1 (sum |t| <= 8M < sigma1 / 2), so their FP32 sum h1 is exact;
// the remainders (|t| <= u sigma1) go through a second level at sigma2 =
// 2^-19 sigma1 (exact h2, a multiple of 2^(E-38)), and the last remainders
// (|t| <= 2^(E-38)) are summed in FP32, an error below 2^(E-58).  h1 + h2
// spans 43 bits and is exact in FP64; adding the last sum rounds once.  The
// six FP64 additions this replaces err by up to about 2^(E-48).
__device__ __forceinline__ double stencil7_f32(float n0, float n1, float n2, float n3, float n4, float n5,
                                               float c) {
  float t[8] = {n0, n1, n2, n3, n4, n5, -4.0f * c, -2.0f * c};
  unsigned mb = 0u;
#pragma unroll
  for (int i = 0; i < 8; ++i) mb = max(mb, __float_as_uint(t[i]) & 0x7FFFFFFFu);
  // biased exponent of the largest term (0: zero or subnormal), capped so
  // sigma1 stays finite; sigma2 at least the smallest normal float
  const unsigned e1 = min((mb >> 23) + 5u, 254u);
  const float s1 = __uint_as_float(e1 << 23);
  const float s2 = __uint_as_float((e1 > 20u ? e1 - 19u : 1u) << 23);
  float h1 = 0.0f, h2 = 0.0f, l2 = 0.0f;
#pragma unroll
  for (int i = 0; i < 8; ++i) h1 = __fadd_rn(h1, extract_hi(s1, t[i]));
#pragma unroll
  for (int i = 0; i < 8; ++i) h2 = __fadd_rn(h2, extract_hi(s2, t[i]));
#pragma unroll
  for (int i = 0; i < 8; ++i) l2 = __fadd_rn(l2, t[i]);
  return (f32_to_f64(h1) + f32_to_f64(h2)) + f32_to_f64(l2);
}

template <typename C>
__device__ __forceinline__ C to_f32c(double a, double b) {
  C r;
  r.x = f64_to_f32_trunc(a);
  r.y = f64_to_f32_trunc(b);
  return r;
}

// x pass, FP64 input -> FP32 half spectrum (the rr2c_kernel transform):
//   MIX_DIV:  d' = h div(u) from the FP64 vector u, stored, transformed;
//   MIX_SCAL: d' = h (d - mean d) from a scalar FP64 right-hand side (its
//             mean, the part no pressure can balance, is removed first so the
//             FP32 residual solves do not carry it), stored, transformed;
//   MIX_RES:  r' = r'_prev - (sum of neighbours of q - 6 q) / h with the
//             previous residual r'_prev in d (the divergence at first) and
//             the last FP32 correction q (n^3 floats), transformed; stored
//             back to d when `store` is set;
//   MIX_RES_MEAN: as MIX_RES, and the CTA's sum of the pressure so far,
//             q1 + q2 (qp = q1, q = q2), goes to part[blockIdx.x].
template <int N1, int N2, int MODE>
__global__ void __launch_bounds__(XGeom<float, N1, N2>::NT)
mr2c_kernel(const double* __restrict__ src, double h, double* __restrict__ d, const double* __restrict__ p, int P,
            double inv_h, cplx<float>* __restrict__ out, const cplx<float>* __restrict__ tw,
            const cplx<float>* __restrict__ tl, double* __restrict__ part, const float* __restrict__ q,
            const float* __restrict__ qp, int store) {
  using C = cplx<float>;
  using G = XGeom<float, N1, N2>;
  constexpr int L = N1 * N2, n = 2 * L, RW = G::RW, XS = G::XS;
  extern __shared__ unsigned char smem_raw[];
  C* xs = reinterpret_cast<C*>(smem_raw);
  constexpr long long nn = (long long)n * n, N = nn * n;
  const long long row0 = (long long)blockIdx.x * RW;
  const int tid = threadIdx.x;
  const int line = tid / N2, m2 = tid - line * N2;
  double psum = 0.0;
  C v[N1];
  if (tid < RW * N2) {
    const long long row = row0 + line;
    if (row < nn) {
      const int z = (int)(row / n), y = (int)(row - (long long)z * n);
      const long long base = row * n;
      if constexpr (MODE == MIX_DIV) {
        const long long rowy = (long long)z * n + wrap_dn(y, n);
        const long long rowz = (long long)wrap_dn(z, n) * n + y;
        const double* ux = src;
        const double2* ux2 = reinterpret_cast<const double2*>(src + base);
        const double2* uy2 = reinterpret_cast<const double2*>(src + N + base);
        const double2* uyd = reinterpret_cast<const double2*>(src + N + rowy * n);
        const double2* uz2 = reinterpret_cast<const double2*>(src + 2 * N + base);
        const double2* uzd = reinterpret_cast<const double2*>(src + 2 * N + rowz * n);
        double2* d2 = reinterpret_cast<double2*>(d + base);
#pragma unroll
        for (int m1 = 0; m1 < N1; ++m1) {
          const int m = m2 + N2 * m1;
          const int xm = (m == 0) ? n - 1 : 2 * m - 1;
          const double2 a0 = ux2[m], b0 = uy2[m], b1 = uyd[m], c0 = uz2[m], c1 = uzd[m];
          const double uxm = ux[base + xm];
          double2 dv;
          dv.x = (a0.x - uxm) + (b0.x - b1.x) + (c0.x - c1.x);
          dv.y = (a0.y - a0.x) + (b0.y - b1.y) + (c0.y - c1.y);
          d2[m] = dv;
          v[m1] = to_f32c<C>(dv.x, dv.y);
        }
      } else if constexpr (MODE == MIX_SCAL) {
        const double2* s2 = reinterpret_cast<const double2*>(src + base);
        double2* d2 = reinterpret_cast<double2*>(d + base);
        const double dm = part[0];
#pragma unroll
        for (int m1 = 0; m1 < N1; ++m1) {
          const int m = m2 + N2 * m1;
          double2 dv = s2[m];
          dv.x = (dv.x - dm) * h;
          dv.y = (dv.y - dm) * h;
          d2[m] = dv;
          v[m1] = to_f32c<C>(dv.x, dv.y);
        }
      } else {
        const float* qr = q + base;
        const float2* qc2 = reinterpret_cast<const float2*>(qr);
        const float2* qym = reinterpret_cast<const float2*>(q + ((long long)z * n + wrap_dn(y, n)) * n);
        const float2* qyp = reinterpret_cast<const float2*>(q + ((long long)z * n + wrap_up(y, n)) * n);
        const float2* qzm = reinterpret_cast<const float2*>(q + ((long long)wrap_dn(z, n) * n + y) * n);
        const float2* qzp = reinterpret_cast<const float2*>(q + ((long long)wrap_up(z, n) * n + y) * n);
        double2* d2 = reinterpret_cast<double2*>(d + base);
        const float2* const qp2 = reinterpret_cast<const float2*>(qp + base);
#pragma unroll
        for (int m1 = 0; m1 < N1; ++m1) {
          const int m = m2 + N2 * m1;
          const float2 qc = qc2[m];
          const float qxm = qr[m == 0 ? n - 1 : 2 * m - 1];
          const float qxp = qr[m == L - 1 ? 0 : 2 * m + 2];
          const float2 a = qym[m], b = qyp[m], c = qzm[m], e = qzp[m];
          double2 rv = d2[m];
          // neighbours of x = 2m: qxm and 2m + 1; of x = 2m + 1: 2m and qxp
          rv.x = fma(-inv_h, stencil7_f32(qxm, qc.y, a.x, b.x, c.x, e.x, qc.x), rv.x);
          rv.y = fma(-inv_h, stencil7_f32(qc.x, qxp, a.y, b.y, c.y, e.y, qc.y), rv.y);
          if (store) d2[m] = rv;
          if constexpr (MODE == MIX_RES_MEAN) {
            const float2 pa = qp2[m];
            psum += (f32_to_f64(pa.x) + f32_to_f64(qc.x)) + (f32_to_f64(pa.y) + f32_to_f64(qc.y));
          }
          v[m1] = to_f32c<C>(rv.x, rv.y);
        }
      }
    } else {
#pragma unroll
      for (int m1 = 0; m1 < N1; ++m1) v[m1] = mk<float>(0, 0);
    }
    dft_reg<N1, false>(v);
#pragma unroll
    for (int k1 = 1; k1 < N1; ++k1) v[k1] = cmul(v[k1], __ldg(&tl[k1 * N2 + m2]));
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) xs[line * XS + k1 * (N2 + 1) + m2] = v[k1];
  }
  __syncthreads();
  const int lb = tid / N1, k1 = tid - lb * N1;
  const bool actb = tid < RW * N1;
  C zz[N2];
  if (actb) {
#pragma unroll
    for (int q = 0; q < N2; ++q) zz[q] = xs[lb * XS + k1 * (N2 + 1) + q];
    dft_reg<N2, false>(zz);
  }
  __syncthreads();
  if (actb) {
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) xs[lb * XS + k1 + N1 * k2] = zz[k2];
  }
  __syncthreads();
  const long long row = row0 + lb;
  if (actb && row < nn) {
    C* o = out + row * P;
    const C* zr = xs + lb * XS;
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
      const int k = k1 + N1 * k2;
      const C zk = zz[k2];
      const C zc = cconj(zr[k == 0 ? 0 : L - k]);
      const C e = cadd(zk, zc), dd = csub(zk, zc);
      const C wo = cmul(dd, __ldg(&tw[k]));
      C X;
      X.x = 0.5f * (e.x + wo.y);
      X.y = 0.5f * (e.y - wo.x);
      o[k] = X;
    }
    if (k1 == 0) {
      const C zk = zz[0], zc = cconj(zz[0]);
      const C e = cadd(zk, zc), dd = csub(zk, zc);
      const C wo = cmul(dd, __ldg(&tw[L]));
      C X;
      X.x = 0.5f * (e.x + wo.y);
      X.y = 0.5f * (e.y - wo.x);
      o[L] = X;
    }
  }
  if constexpr (MODE == MIX_RES_MEAN) {
    // fixed-order block sum of p (deterministic for a fixed launch shape)
    __shared__ double red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) psum += __shfl_down_sync(0xffffffffu, psum, o);
    const int warp = tid >> 5, lane = tid & 31;
    if (lane == 0) red[warp] = psum;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
      part[blockIdx.x] = s;
    }
  }
}

// x pass, FP32 half spectrum -> reals c (the rc2r_kernel transform):
//   MIX_Q:        c to q (n^3 floats; a correction kept for the residual and
//                 the final sum);
//   MIX_FIN:      the FP64 pressure p (row pitch 2P) = (q1 + q2) + c;
//   MIX_FIN_MEAN: p = ((q1 + q2) - mean) + c.
// Summed in this order, p has the bits of accumulating each correction into
// an FP64 p as it arrives, without the FP64 field's reads and writes between.
template <int N1, int N2, int MODE>
__global__ void __launch_bounds__(XGeom<float, N1, N2>::NT)
mc2r_kernel(const cplx<float>* __restrict__ g, int P, const cplx<float>* __restrict__ tw,
            const cplx<float>* __restrict__ tl, double* __restrict__ p, const double* __restrict__ mean,
            float* __restrict__ q, const float* __restrict__ q1, const float* __restrict__ q2) {
  using C = cplx<float>;
  using G = XGeom<float, N1, N2>;
  constexpr int L = N1 * N2, n = 2 * L, RW = G::RW, XS = G::XS;
  extern __shared__ unsigned char smem_raw[];
  C* xs = reinterpret_cast<C*>(smem_raw);
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
      for (int m1 = 0; m1 < N1; ++m1) v[m1] = mk<float>(0, 0);
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
    C zz[N2];
#pragma unroll
    for (int q = 0; q < N2; ++q) zz[q] = xs[lb * XS + k1 * (N2 + 1) + q];
    dft_reg<N2, true>(zz);
    if constexpr (MODE == MIX_Q) {
      float2* const qo = reinterpret_cast<float2*>(q + row * n);
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2)
        qo[k1 + N1 * k2] = make_float2(f32_flush(zz[k2].x), f32_flush(zz[k2].y));
    } else {
      double2* const r = reinterpret_cast<double2*>(p + row * 2LL * P);
      const float2* const a1 = reinterpret_cast<const float2*>(q1 + row * n);
      const float2* const a2 = reinterpret_cast<const float2*>(q2 + row * n);
      double mu = 0.0;
      if constexpr (MODE == MIX_FIN_MEAN) mu = *mean;
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) {
        const int m = k1 + N1 * k2;
        const float2 b1 = a1[m], b2 = a2[m];
        const double sx = f32_to_f64(b1.x) + f32_to_f64(b2.x), sy = f32_to_f64(b1.y) + f32_to_f64(b2.y);
        double2 o;
        if constexpr (MODE == MIX_FIN) {
          o.x = sx + f32_to_f64(zz[k2].x);
          o.y = sy + f32_to_f64(zz[k2].y);
        } else {
          o.x = (sx - mu) + f32_to_f64(zz[k2].x);
          o.y = (sy - mu) + f32_to_f64(zz[k2].y);
        }
        r[m] = o;
      }
    }
  }
}

// Per-CTA sums of a dense field (the scalar right-hand side's mean), fixed order.
__global__ void mix_sum_kernel(const double* __restrict__ src, long long count, double* __restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < count; i += 256LL * gridDim.x) s += src[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Mean of p from the per-CTA sums, in a fixed order.
__global__ void mix_mean_kernel(const double* __restrict__ part, int nparts, double invN, double* __restrict__ mean) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < nparts; i += 256) s += part[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *mean = red[0] * invN;
}

template <int NN>
struct MixSolve {
  using RS = RegSolve<float, NN>;
  static constexpr int A1 = RS::A1, A2 = RS::A2, B1 = RS::B1, B2 = RS::B2;
  using CG = typename RS::CG;
  using XG = typename RS::XG;
  static constexpr long long NPARTS = ((long long)NN * NN + XG::RW - 1) / XG::RW;
  static constexpr int SUM_CTAS = 1024;  // mix_sum_kernel grid
  // doubles of `part`: the CTA sums of the last residual pass (NPARTS) and
  // the mean of p after them, or the scalar right-hand side's mean and its
  // SUM_CTAS partial sums
  static constexpr long long PART_WORDS = (NPARTS > SUM_CTAS ? NPARTS : SUM_CTAS) + 2;

  static cudaError_t configure() {
    cudaError_t e = cudaSuccess;
    auto set = [&](const void* f, size_t sh) {
      if (e == cudaSuccess && sh > 48 * 1024)
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
    };
    set((const void*)mr2c_kernel<B1, B2, MIX_DIV>, XG::SMEM);
    set((const void*)mr2c_kernel<B1, B2, MIX_SCAL>, XG::SMEM);
    set((const void*)mr2c_kernel<B1, B2, MIX_RES>, XG::SMEM);
    set((const void*)mr2c_kernel<B1, B2, MIX_RES_MEAN>, XG::SMEM);
    set((const void*)mc2r_kernel<B1, B2, MIX_Q>, XG::SMEM);
    set((const void*)mc2r_kernel<B1, B2, MIX_FIN>, XG::SMEM);
    set((const void*)mc2r_kernel<B1, B2, MIX_FIN_MEAN>, XG::SMEM);
    return e;
  }

  static cudaError_t solve(exc_poisson* ps, const double* src, bool vec, cudaStream_t st) {
    using C = cplx<float>;
    constexpr int n = NN;
    exc_poisson* sp = ps->mix;
    const int P = ps->P, nkx = n / 2 + 1;
    C* g = reinterpret_cast<C*>(sp->work);
    const C* tw = reinterpret_cast<const C*>(sp->tw);
    const C* tln = reinterpret_cast<const C*>(sp->twl_n);
    const C* tlh = reinterpret_cast<const C*>(sp->twl_h);
    double* p = reinterpret_cast<double*>(ps->work);
    double* d = ps->mix_d;
    double* part = ps->mix_part;
    double* mean = part + NPARTS;
    const double h = ps->h, inv_h = 1.0 / ps->h;
    const unsigned gx = (unsigned)NPARTS;
    const SlotBatch one;
    auto columns = [&]() { RS::columns(g, nkx, P, tln, sp->invlap, st, one, 1); };
    float* const q1 = ps->mix_q;
    float* const q2 = ps->mix_q2;
    if (vec) {
      mr2c_kernel<B1, B2, MIX_DIV><<<gx, XG::NT, XG::SMEM, st>>>(src, h, d, p, P, inv_h, g, tw, tlh, part, q1, q1, 0);
    } else {
      // mean of d into part[0] (partials in part[1 .. SUM_CTAS])
      mix_sum_kernel<<<SUM_CTAS, 256, 0, st>>>(src, (long long)n * n * n, part + 1);
      mix_mean_kernel<<<1, 256, 0, st>>>(part + 1, SUM_CTAS, 1.0 / ((double)n * n * n), part);
      mr2c_kernel<B1, B2, MIX_SCAL><<<gx, XG::NT, XG::SMEM, st>>>(src, h, d, p, P, inv_h, g, tw, tlh, part, q1, q1,
                                                                  0);
    }
    columns();
    mc2r_kernel<B1, B2, MIX_Q><<<gx, XG::NT, XG::SMEM, st>>>(g, P, tw, tlh, p, mean, q1, nullptr, nullptr);
    mr2c_kernel<B1, B2, MIX_RES><<<gx, XG::NT, XG::SMEM, st>>>(src, h, d, p, P, inv_h, g, tw, tlh, part, q1, q1, 1);
    columns();
    mc2r_kernel<B1, B2, MIX_Q><<<gx, XG::NT, XG::SMEM, st>>>(g, P, tw, tlh, p, mean, q2, nullptr, nullptr);
    if (ps->mix_zero_mean) {
      mr2c_kernel<B1, B2, MIX_RES_MEAN><<<gx, XG::NT, XG::SMEM, st>>>(src, h, d, p, P, inv_h, g, tw, tlh, part, q2,
                                                                      q1, 0);
      mix_mean_kernel<<<1, 256, 0, st>>>(part, (int)NPARTS, 1.0 / ((double)n * n * n), mean);
      columns();
      mc2r_kernel<B1, B2, MIX_FIN_MEAN><<<gx, XG::NT, XG::SMEM, st>>>(g, P, tw, tlh, p, mean, nullptr, q1, q2);
    } else {
      mr2c_kernel<B1, B2, MIX_RES><<<gx, XG::NT, XG::SMEM, st>>>(src, h, d, p, P, inv_h, g, tw, tlh, part, q2, q1,
                                                                 0);
      columns();
      mc2r_kernel<B1, B2, MIX_FIN><<<gx, XG::NT, XG::SMEM, st>>>(g, P, tw, tlh, p, mean, nullptr, q1, q2);
    }
    return cudaGetLastError();
  }
};

}  // namespace exc
