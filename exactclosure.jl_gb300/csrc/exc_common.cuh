// Common types and helpers of libexc (GB300 / sm_103a).
//
// Field layout (the reference's column-major Field, src/N.jl:29 and :45): a
// scalar field is n^3 contiguous words, x fastest; a vector field is three
// such arrays, component slowest.  The spectral work array is
// [n][n][P] complex with P = pad8(n/2 + 1) (the rfft half axis is x, like
// FFTW's first-dimension halving in src/N.jl:207-217); its real view holds
// the pressure as [n][n][2P] words after the inverse transform.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

#include "../../include/exc.h"

namespace exc {

template <typename T> struct cplx_t;
template <> struct cplx_t<double> { using type = double2; };
template <> struct cplx_t<float> { using type = float2; };
template <typename T> using cplx = typename cplx_t<T>::type;

template <typename T> __host__ __device__ __forceinline__ cplx<T> mk(T a, T b) { cplx<T> r; r.x = a; r.y = b; return r; }
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
// a * b
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = fma(a.x, b.x, -a.y * b.y);
  r.y = fma(a.x, b.y, a.y * b.x);
  return r;
}
// a * conj(b)
template <typename C> __host__ __device__ __forceinline__ C cmulc(C a, C b) {
  C r;
  r.x = fma(a.x, b.x, a.y * b.y);
  r.y = fma(a.y, b.x, -a.x * b.y);
  return r;
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) { C r; r.x = a.x; r.y = -a.y; return r; }
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename C> __host__ __device__ __forceinline__ C mul_mi(C a) {
  C r;
  if (INV) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; }
  return r;
}

__host__ __device__ __forceinline__ int pad8(int m) { return (m + 7) & ~7; }
__host__ __device__ __forceinline__ int spec_pitch(int n) { return pad8(n / 2 + 1); }

// Division of a linear index by a grid extent with a multiply-high
// reciprocal m = ceil(2^64 / d): x / d exactly for every x < 2^64 / d, which
// covers every index here.  Built once per thread (one 64-bit division), it
// replaces the per-element 64-bit divisions of grid-stride index splits.
// Constants of the FP64 RHS sweep's shifted stress form, w = sq u - qs
// (sq = sqrt(1/(4h)), qs = rho/2, rho = (4 visc/h) sq): one definition for
// the sweep and for the RK stage kernel that stores the next stage state in
// that form, so both produce the same bits.
struct Fp64Shift {
  double sq, rho, qs;
};
__device__ __forceinline__ Fp64Shift fp64_shift(double inv_h, double visc) {
  const double kd = 0.25 * inv_h;
  const double rv = 4.0 * visc * inv_h;
  const double sq = sqrt(kd);
  const double rho = rv * sq;
  return {sq, rho, 0.5 * rho};
}

struct IdxDiv {
  unsigned long long m;
  long long d;
  __host__ __device__ __forceinline__ explicit IdxDiv(long long d_)
      : m(d_ > 1 ? ~0ull / (unsigned long long)d_ + 1 : 0ull), d(d_) {}
  __device__ __forceinline__ long long div(long long x) const {
    return m ? (long long)__umul64hi((unsigned long long)x, m) : x;
  }
};

// Asynchronous global -> shared copy of one 4- or 8-byte word (cp.async);
// completion is waited for with cp_async_wait_all before a barrier.
template <typename T>
__device__ __forceinline__ void cp_async_word(T* smem, const T* gmem) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "word copies only");
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
// Asynchronous 16-byte global -> shared copy (both addresses 16-byte aligned).
template <typename T>
__device__ __forceinline__ void cp_async_16(T* smem, const T* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Periodic neighbour index along one axis.
__device__ __forceinline__ int wrap_up(int i, int n) { return (i + 1 == n) ? 0 : i + 1; }
__device__ __forceinline__ int wrap_dn(int i, int n) { return (i == 0) ? n - 1 : i - 1; }

// A batch of same-size solves laid out slot after slot (serving form).  The
// slot index comes from a grid dimension; inactive slots return at once.
struct SlotBatch {
  long long ustride = 0;          // words between slots of a vector field (3 n^3)
  long long wstride = 0;          // complex words between slots of the spectral work array
  const int* active = nullptr;    // per-slot flag, null = all active
  const void* visc = nullptr;     // per-slot viscosity (field word type), null = scalar argument
};

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Grid sizes the FFT supports: n = 2^a 3^b 5^c 7^d 11^e 13^f 17^g with a >= 1,
// 4 <= n <= 1024.
inline bool fft_size_ok(int n) {
  if (n < 4 || n > 1024 || (n & 1)) return false;
  int m = n;
  while (m % 2 == 0) m /= 2;
  while (m % 3 == 0) m /= 3;
  for (int f : {5, 7, 11, 13, 17})
    while (m % f == 0) m /= f;
  return m == 1;
}

}  // namespace exc

#define EXC_CHECK_CUDA(call)                               \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) { exc::set_last_error(cudaGetErrorString(e_)); return EXC_ERR_CUDA; } \
  } while (0)

namespace exc {
void set_last_error(const char* msg);

// |x| as its magnitude bits: for non-negative IEEE values the unsigned
// integer order is the numeric order, and NaN patterns sort above infinity,
// so maxima of magnitudes run exactly on the integer pipe.
template <typename T> struct MagBits;
template <> struct MagBits<double> { using type = unsigned long long; using vec = double2; };
template <> struct MagBits<float> { using type = unsigned; using vec = float4; };
__device__ __forceinline__ unsigned long long mag_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ unsigned mag_bits(float x) { return __float_as_uint(x) & 0x7FFFFFFFu; }
template <typename T> __device__ __forceinline__ T from_mag_bits(typename MagBits<T>::type b);
template <> __device__ __forceinline__ double from_mag_bits<double>(unsigned long long b) {
  return __longlong_as_double((long long)b);
}
template <> __device__ __forceinline__ float from_mag_bits<float>(unsigned b) { return __uint_as_float(b); }
}
