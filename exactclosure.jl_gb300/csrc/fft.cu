// FFT Poisson solver: R2C along x, complex passes along y and z with the
// spectral divide of `project!` (src/N.jl:272-298) fused between the forward
// and inverse z transforms, then C2R along x back into the work array.
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace exc {

// ---------------------------------------------------------------------------
// x pass, real -> half complex.  A CTA transforms `rows` x-lines of n reals as
// complex lines of length n/2 (z_m = x_2m + i x_2m+1) and untangles them:
//   X_k = (Z_k + conj Z_{n/2-k})/2 - (i/2) W_n^k (Z_k - conj Z_{n/2-k}).
// With DIV the input line is d = div(u) (src/N.jl:222-238) computed on the fly.
// ---------------------------------------------------------------------------
template <typename T, bool DIV, bool EXT = false>
__global__ void __launch_bounds__(fft_threads<cplx<T>>(), 3)
r2c_x_kernel(const T* __restrict__ src, int n, T inv_h, cplx<T>* __restrict__ out, int P,
             const cplx<T>* __restrict__ tw, FftPlan plan, int rows_per_cta, SlotBatch sb) {
  using C = cplx<T>;
  extern __shared__ unsigned char smem_raw[];
  C* s = reinterpret_cast<C*>(smem_raw);
  const int slot = blockIdx.y;
  if (sb.active && !sb.active[slot]) return;
  src += slot * sb.ustride;
  out += slot * sb.wstride;
  const int N2 = n / 2;
  const int ls = padded_len(N2);
  const long long nn = (long long)n * n;
  const long long N = nn * n;
  const long long row0 = (long long)blockIdx.x * rows_per_cta;
  const int rows = (int)min((long long)rows_per_cta, nn - row0);
  // load
  for (int t = threadIdx.x; t < rows * N2; t += blockDim.x) {
    const int r = (int)fast_div((unsigned)t, plan.rL), m = t - r * N2;
    long long row = row0 + r;
    long long base = row * n;
    T a, b;
    if (!DIV) {
      a = src[base + 2 * m];
      b = src[base + 2 * m + 1];
    } else {
      const int z = (int)fast_div((unsigned)row, plan.r2L), y = (int)row - z * n;  // row < n^2 <= 2^20
      long long rowy = (long long)z * n + (y == 0 ? n - 1 : y - 1);
      long long rowz = (long long)(z == 0 ? n - 1 : z - 1) * n + y;
      const T* ux = src;
      const T* uy = src + N;
      const T* uz = src + 2 * N;
      int x0 = 2 * m, x1 = 2 * m + 1;
      int xm = (x0 == 0) ? n - 1 : x0 - 1;
      a = ((ux[base + x0] - ux[base + xm]) + (uy[base + x0] - uy[rowy * n + x0]) +
           (uz[base + x0] - uz[rowz * n + x0])) * inv_h;
      b = ((ux[base + x1] - ux[base + x0]) + (uy[base + x1] - uy[rowy * n + x1]) +
           (uz[base + x1] - uz[rowz * n + x1])) * inv_h;
    }
    s[r * ls + pe(m)] = mk<T>(a, b);
  }
  __syncthreads();
  fft_lines<false, EXT>(s, ls, rows, plan, tw, n);
  // untangle and store k = 0..N2
  for (int t = threadIdx.x; t < rows * (N2 + 1); t += blockDim.x) {
    const int r = (int)fast_div((unsigned)t, plan.rL1), k = t - r * (N2 + 1);
    C zk = s[r * ls + pe(k == N2 ? 0 : k)];
    C zc = cconj(s[r * ls + pe(k == 0 ? 0 : N2 - k)]);
    C e = cadd(zk, zc);
    C o = csub(zk, zc);
    C w = tw[k];                  // W_n^k, k <= n/2 < n
    C wo = cmul(o, w);            // W^k (Z_k - conj Z_{N2-k})
    // X = e/2 - i/2 * wo
    C X;
    X.x = (T)0.5 * (e.x + wo.y);
    X.y = (T)0.5 * (e.y - wo.x);
    out[(row0 + r) * P + k] = X;
  }
}

// ---------------------------------------------------------------------------
// Column passes along y (elem_stride = P, outer = z) or z (elem_stride = n P,
// outer = y).  A tile is `W` consecutive kx columns of one outer index; tile
// id = outer * ntx + kx tile.  The CTAs are persistent: each walks the tiles
// id = blockIdx.x, + gridDim.x, ... with two shared-memory tile buffers; the
// next tile's cp.async copies are issued before the current tile is
// transformed, so HBM traffic continues while the shared-memory passes run.
// ---------------------------------------------------------------------------
struct ColTiles {
  int nkx, W, wlog, ntx, ntiles;  // ntiles = ntx * n < 2^17
  long long outer_stride;
  __device__ __forceinline__ int lines(int id) const {
    return min(W, nkx - (id % ntx) * W);
  }
  __device__ __forceinline__ long long offset(int id) const {
    const int outer = id / ntx;
    return (long long)outer * outer_stride + (id - outer * ntx) * W;
  }
};

__device__ __forceinline__ ColTiles col_tiles(int n, int nkx, int W, long long outer_stride) {
  ColTiles t;
  t.nkx = nkx;
  t.W = W;
  t.wlog = 31 - __clz(W);
  t.ntx = (nkx + W - 1) / W;
  t.ntiles = t.ntx * n;
  t.outer_stride = outer_stride;
  return t;
}

// Shared memory: two buffers of W lines of stride n + 1.  A CTA takes the
// tiles blockIdx.x and blockIdx.x + gridDim.x; the second tile's copies are
// in flight while the first is transformed.
template <typename T, bool INV, bool EXT = false>
__global__ void __launch_bounds__(fft_threads<cplx<T>>(), 3)
cols_kernel(cplx<T>* __restrict__ g, int n, int nkx, int W, long long elem_stride,
            long long outer_stride, const cplx<T>* __restrict__ tw, FftPlan plan, SlotBatch sb) {
  using C = cplx<T>;
  extern __shared__ unsigned char smem_raw[];
  C* const buf0 = reinterpret_cast<C*>(smem_raw);
  C* const buf1 = buf0 + W * padded_len(n);
  if (sb.active && !sb.active[blockIdx.z]) return;
  g += blockIdx.z * sb.wstride;
  const int ls = padded_len(n);
  const ColTiles ct = col_tiles(n, nkx, W, outer_stride);
  const int a = blockIdx.x, b = blockIdx.x + gridDim.x;
  if (a >= ct.ntiles) return;
  const bool two = b < ct.ntiles;
  tile_load_async(buf0, ls, g + ct.offset(a), elem_stride, ct.lines(a), W, ct.wlog, n);
  cp_commit();
  if (two) tile_load_async(buf1, ls, g + ct.offset(b), elem_stride, ct.lines(b), W, ct.wlog, n);
  cp_commit();
  cp_wait<1>();
  __syncthreads();
  fft_lines<INV, EXT>(buf0, ls, ct.lines(a), plan, tw, n);
  tile_move<false>(buf0, ls, g + ct.offset(a), elem_stride, ct.lines(a), W, ct.wlog, n);
  if (!two) return;
  cp_wait<0>();
  __syncthreads();
  fft_lines<INV, EXT>(buf1, ls, ct.lines(b), plan, tw, n);
  tile_move<false>(buf1, ls, g + ct.offset(b), elem_stride, ct.lines(b), W, ct.wlog, n);
}

// 1/d in float64 for d in (0, 3] (a sum of three sin^2): a single-precision
// estimate refined by two Newton-Raphson steps r <- r + r(1 - d r), each of
// which squares the relative error (6e-8 -> 4e-15 -> below the float64 ulp).
__device__ __forceinline__ double recip_f64(double d) {
  double r = (double)__frcp_rn((float)d);
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  e = fma(-d, r, 1.0);
  return fma(r, e, r);
}

// ---------------------------------------------------------------------------
// z pass with the spectral divide: forward FFT along z, multiply by
// 1/(lambda N) with lambda = -4/h^2 sum_d sin^2(pi k_d/n) (src/N.jl:281-291)
// and the mean mode set to zero (src/N.jl:298), inverse FFT along z.  The
// divide is computed in float64 for every precision.
// ---------------------------------------------------------------------------
// z forward transform, divide and inverse of one tile in shared memory.
template <typename T, bool EXT>
__device__ __forceinline__ void zsolve_tile(cplx<T>* s, int ls, int lines, int wlog, int n, int nkx, int kx0, int ky,
                                            const cplx<T>* __restrict__ tw, const FftPlan& plan,
                                            const double* __restrict__ sin2, double coef,
                                            const double* __restrict__ invlap) {
  using C = cplx<T>;
  fft_lines<false, EXT>(s, ls, lines, plan, tw, n);
  const double sy = sin2[ky];
  const bool pow2 = lines == (1 << wlog);
  for (int t = threadIdx.x; t < lines * n; t += blockDim.x) {
    const int kz = pow2 ? t >> wlog : t / lines, l = t - kz * lines;
    int kx = kx0 + l;
    C v = s[l * ls + pe(kz)];
    const long long mi = invlap_index(n, kz, ky, kx);
    if (sizeof(T) == 4 && invlap) {
      // FP32 form: the float64 factor 1/(lambda N) stored as hi + lo floats;
      // v (hi + lo) with one FMA keeps the factor's float64 precision up to
      // the final float rounding, without FP64-pipe work
      const float2 f2 = reinterpret_cast<const float2*>(invlap)[mi];
      v.x = (T)fmaf((float)v.x, f2.x, (float)v.x * f2.y);
      v.y = (T)fmaf((float)v.y, f2.x, (float)v.y * f2.y);
    } else {
      double f;
      if (invlap) {
        // precomputed 1/(lambda N), one float64 per mode ([kz][ky][kx])
        f = invlap[mi];
      } else {
        double den = sin2[kx] + sy + sin2[kz];
        f = (kx == 0 && ky == 0 && kz == 0) ? 0.0 : coef * recip_f64(den);
      }
      v.x = (T)((double)v.x * f);
      v.y = (T)((double)v.y * f);
    }
    s[l * ls + pe(kz)] = v;
  }
  __syncthreads();
  fft_lines<true, EXT>(s, ls, lines, plan, tw, n);
}

// Two tiles per CTA, as in cols_kernel.
template <typename T, bool EXT = false>
__global__ void __launch_bounds__(fft_threads<cplx<T>>(), 3)
zsolve_kernel(cplx<T>* __restrict__ g, int n, int nkx, int W, int P, const cplx<T>* __restrict__ tw,
              FftPlan plan, const double* __restrict__ sin2, double coef, const double* __restrict__ invlap,
              SlotBatch sb) {
  using C = cplx<T>;
  extern __shared__ unsigned char smem_raw[];
  C* const buf0 = reinterpret_cast<C*>(smem_raw);
  C* const buf1 = buf0 + W * padded_len(n);
  if (sb.active && !sb.active[blockIdx.z]) return;
  g += blockIdx.z * sb.wstride;
  const int ls = padded_len(n);
  const long long es = (long long)n * P;
  const ColTiles ct = col_tiles(n, nkx, W, P);
  const int a = blockIdx.x, b = blockIdx.x + gridDim.x;
  if (a >= ct.ntiles) return;
  const bool two = b < ct.ntiles;
  tile_load_async(buf0, ls, g + ct.offset(a), es, ct.lines(a), W, ct.wlog, n);
  cp_commit();
  if (two) tile_load_async(buf1, ls, g + ct.offset(b), es, ct.lines(b), W, ct.wlog, n);
  cp_commit();
  cp_wait<1>();
  __syncthreads();
  {
    const int ky = a / ct.ntx;
    zsolve_tile<T, EXT>(buf0, ls, ct.lines(a), ct.wlog, n, nkx, (a - ky * ct.ntx) * W, ky, tw, plan, sin2, coef, invlap);
    tile_move<false>(buf0, ls, g + ct.offset(a), es, ct.lines(a), W, ct.wlog, n);
  }
  if (!two) return;
  cp_wait<0>();
  __syncthreads();
  const int ky = b / ct.ntx;
  zsolve_tile<T, EXT>(buf1, ls, ct.lines(b), ct.wlog, n, nkx, (b - ky * ct.ntx) * W, ky, tw, plan, sin2, coef, invlap);
  tile_move<false>(buf1, ls, g + ct.offset(b), es, ct.lines(b), W, ct.wlog, n);
}

// ---------------------------------------------------------------------------
// x pass, half complex -> real, in place (row pitch P complex = 2P reals):
//   Z_k = (X_k + conj X_{N2-k}) + i W_n^-k (X_k - conj X_{N2-k}),
//   z = IDFT_{N2}(Z) (unnormalised), x_2m = Re z_m, x_2m+1 = Im z_m.
// ---------------------------------------------------------------------------
template <typename T, bool EXT = false>
__global__ void __launch_bounds__(fft_threads<cplx<T>>(), 3)
c2r_x_kernel(cplx<T>* __restrict__ g, int n, int P, const cplx<T>* __restrict__ tw, FftPlan plan,
             int rows_per_cta, SlotBatch sb) {
  using C = cplx<T>;
  extern __shared__ unsigned char smem_raw[];
  C* s = reinterpret_cast<C*>(smem_raw);
  if (sb.active && !sb.active[blockIdx.y]) return;
  g += blockIdx.y * sb.wstride;
  const int N2 = n / 2;
  const int ls = padded_len(N2);
  const long long nn = (long long)n * n;
  const long long row0 = (long long)blockIdx.x * rows_per_cta;
  const int rows = (int)min((long long)rows_per_cta, nn - row0);
  for (int t = threadIdx.x; t < rows * (N2 + 1); t += blockDim.x) {
    const int r = (int)fast_div((unsigned)t, plan.rL1), k = t - r * (N2 + 1);
    s[r * ls + pe(k)] = g[(row0 + r) * P + k];
  }
  __syncthreads();
  // pairs (k, N2-k) handled by one thread, so the tangle is in place
  const int half = N2 / 2 + 1;
  for (int t = threadIdx.x; t < rows * half; t += blockDim.x) {
    const int r = (int)fast_div((unsigned)t, plan.rhalf), k = t - r * half;
    int k2 = N2 - k;
    C xa = s[r * ls + pe(k)], xb = s[r * ls + pe(k2)];
    C wa = tw[k], wb = tw[k2];
    // Z_k
    C e = cadd(xa, cconj(xb));
    C o = cmulc(csub(xa, cconj(xb)), wa);  // W^-k (X_k - conj X_k2)
    C za; za.x = e.x - o.y; za.y = e.y + o.x;
    // Z_k2
    C e2 = cadd(xb, cconj(xa));
    C o2 = cmulc(csub(xb, cconj(xa)), wb);
    C zb; zb.x = e2.x - o2.y; zb.y = e2.y + o2.x;
    if (k < N2) s[r * ls + pe(k)] = za;
    if (k2 < N2 && k2 != k) s[r * ls + pe(k2)] = zb;
  }
  __syncthreads();
  fft_lines<true, EXT>(s, ls, rows, plan, tw, n);
  T* gr = reinterpret_cast<T*>(g);
  for (int t = threadIdx.x; t < rows * N2; t += blockDim.x) {
    const int r = (int)fast_div((unsigned)t, plan.rL), m = t - r * N2;
    C z = s[r * ls + pe(m)];
    T* row = gr + (row0 + r) * (2LL * P);
    row[2 * m] = z.x;
    row[2 * m + 1] = z.y;
  }
}

template <typename T>
__global__ void copy_pitched_kernel(const T* __restrict__ src, int pitch, T* __restrict__ dst, int n) {
  long long N = (long long)n * n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    long long row = i / n;
    int x = (int)(i - row * n);
    dst[i] = src[row * pitch + x];
  }
}

// In place: each float64 factor f of the 1/(lambda N) table becomes the
// float pair (hi, lo) with hi = fl32(f), lo = fl32(f - hi) (FP32 solvers).
__global__ void invlap_split_kernel(long long tot, double* __restrict__ t) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < tot; g += (long long)gridDim.x * blockDim.x) {
    const double f = t[g];
    const float hi = (float)f;
    const float lo = (float)(f - (double)hi);
    reinterpret_cast<float2*>(t)[g] = make_float2(hi, lo);
  }
}

// 1/(lambda N) for kz, ky <= n/2 and kx <= n/2 ([kz][ky][kx], invlap_index),
// 0 for the mean mode; sin2 is mirrored (sin2[n-k] == sin2[k]), so these
// entries are the factors of every mode.
__global__ void invlap_kernel(int n, const double* __restrict__ sin2, double coef, double* __restrict__ out) {
  const int nkx = n / 2 + 1;
  const long long tot = (long long)nkx * nkx * nkx;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < tot; g += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(g % nkx);
    const long long r = g / nkx;
    const int ky = (int)(r % nkx), kz = (int)(r / nkx);
    out[g] = (kx == 0 && ky == 0 && kz == 0) ? 0.0 : coef / (sin2[kx] + sin2[ky] + sin2[kz]);
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static int col_width(int n, int tile) {
  int w = 1;
  while (w * 2 * n <= tile && w < 64) w *= 2;
  return w;
}

// CTAs of a column pass: two tiles each.
static inline unsigned column_ctas(long long ntiles) { return (unsigned)((ntiles + 1) / 2); }

// Launch geometry of the passes: columns per CTA of the y/z passes and rows
// per CTA of the x passes, from the solver's tuned values (autotuner) when
// set and legal for the tile, else the largest that fills the 32 KB tile.
template <typename C>
static void geometry(const exc_poisson* ps, int& W, int& rows) {
  const int n = ps->n, N2 = n / 2;
  const long long nn = (long long)n * n;
  const int wmax = col_width(n, fft_tile<C>());
  W = (ps->col_w > 0 && ps->col_w <= wmax) ? ps->col_w : wmax;
  const int rmax = fft_tile<C>() / (N2 + 1);
  rows = (ps->x_rows > 0 && ps->x_rows <= rmax) ? ps->x_rows : rmax;
  if (rows > nn) rows = (int)nn;
}

// Stockham passes with radix 7/11/13/17 are separate kernel instantiations
// (EXT): their larger butterflies would otherwise cost every size registers.
static bool plan_ext(const FftPlan& p) { return p.n7 || p.n11 || p.n13 || p.n17; }

template <typename T, bool EXT>
static cudaError_t stockham_solve(exc_poisson* ps, const T* src, bool src_is_vector, cudaStream_t st,
                                  const SlotBatch& sb, int nslots) {
  using C = cplx<T>;
  const int n = ps->n, P = ps->P, N2 = n / 2, nkx = N2 + 1;
  C* g = reinterpret_cast<C*>(ps->work);
  const C* tw = reinterpret_cast<const C*>(ps->tw);
  const long long nn = (long long)n * n;
  int W, rows;
  geometry<C>(ps, W, rows);
  // x forward
  size_t shx = (size_t)rows * padded_len(N2) * sizeof(C);
  dim3 gx((unsigned)((nn + rows - 1) / rows), nslots);
  if (src_is_vector)
    r2c_x_kernel<T, true, EXT><<<gx, fft_threads<C>(), shx, st>>>(src, n, (T)(1.0 / ps->h), g, P, tw, ps->plan_h, rows, sb);
  else
    r2c_x_kernel<T, false, EXT><<<gx, fft_threads<C>(), shx, st>>>(src, n, (T)1, g, P, tw, ps->plan_h, rows, sb);
  // y forward
  const long long ntiles = (long long)((nkx + W - 1) / W) * n;
  size_t shc = 2 * (size_t)W * padded_len(n) * sizeof(C);
  dim3 gc(column_ctas(ntiles), 1, nslots);
  cols_kernel<T, false, EXT><<<gc, fft_threads<C>(), shc, st>>>(g, n, nkx, W, P, (long long)n * P, tw, ps->plan_n, sb);
  // z forward + divide + inverse; coef = 1/(lambda N) numerator: -h^2/(4 N)
  double coef = -ps->h * ps->h / (4.0 * (double)n * (double)n * (double)n);
  zsolve_kernel<T, EXT><<<gc, fft_threads<C>(), shc, st>>>(g, n, nkx, W, P, tw, ps->plan_n, ps->sin2, coef, ps->invlap, sb);
  // y inverse
  cols_kernel<T, true, EXT><<<gc, fft_threads<C>(), shc, st>>>(g, n, nkx, W, P, (long long)n * P, tw, ps->plan_n, sb);
  // x inverse (in place)
  c2r_x_kernel<T, EXT><<<gx, fft_threads<C>(), shx, st>>>(g, n, P, tw, ps->plan_h, rows, sb);
  return cudaGetLastError();
}

template <typename T>
cudaError_t poisson_solve_inplace(exc_poisson* ps, const T* src, bool src_is_vector, cudaStream_t st,
                                  const SlotBatch& sb, int nslots) {
  if constexpr (sizeof(T) == 8) {
    if (ps->engine == 0 && ps->mix && nslots == 1 && !sb.active)
      return fftmix_solve(ps, reinterpret_cast<const double*>(src), src_is_vector, st);
  }
  if (ps->engine != 1 && ps->twl_n && ps->twl_h && ps->invlap)
    return fftreg_solve(ps, src, src_is_vector, st, sb, nslots);
  if (plan_ext(ps->plan_n) || plan_ext(ps->plan_h))
    return stockham_solve<T, true>(ps, src, src_is_vector, st, sb, nslots);
  return stockham_solve<T, false>(ps, src, src_is_vector, st, sb, nslots);
}

// Plain 3-D real transforms on the work array (no divide): forward leaves the
// half spectrum [n][n][P]; inverse (unnormalised) leaves reals at pitch 2P.
template <typename T, bool EXT>
static cudaError_t fft3d_forward_t(exc_poisson* ps, const T* src, cudaStream_t st) {
  using C = cplx<T>;
  const int n = ps->n, P = ps->P, N2 = n / 2, nkx = N2 + 1;
  C* g = reinterpret_cast<C*>(ps->work);
  const C* tw = reinterpret_cast<const C*>(ps->tw);
  const long long nn = (long long)n * n;
  int W, rows;
  geometry<C>(ps, W, rows);
  const SlotBatch one;
  size_t shx = (size_t)rows * padded_len(N2) * sizeof(C);
  int gx = (int)((nn + rows - 1) / rows);
  r2c_x_kernel<T, false, EXT><<<gx, fft_threads<C>(), shx, st>>>(src, n, (T)1, g, P, tw, ps->plan_h, rows, one);
  const long long ntiles = (long long)((nkx + W - 1) / W) * n;
  size_t shc = 2 * (size_t)W * padded_len(n) * sizeof(C);
  dim3 gc(column_ctas(ntiles));
  cols_kernel<T, false, EXT><<<gc, fft_threads<C>(), shc, st>>>(g, n, nkx, W, P, (long long)n * P, tw, ps->plan_n, one);
  cols_kernel<T, false, EXT><<<gc, fft_threads<C>(), shc, st>>>(g, n, nkx, W, (long long)n * P, P, tw, ps->plan_n, one);
  return cudaGetLastError();
}

template <typename T, bool EXT>
static cudaError_t fft3d_inverse_t(exc_poisson* ps, cudaStream_t st) {
  using C = cplx<T>;
  const int n = ps->n, P = ps->P, N2 = n / 2, nkx = N2 + 1;
  C* g = reinterpret_cast<C*>(ps->work);
  const C* tw = reinterpret_cast<const C*>(ps->tw);
  const long long nn = (long long)n * n;
  int W, rows;
  geometry<C>(ps, W, rows);
  const SlotBatch one;
  const long long ntiles = (long long)((nkx + W - 1) / W) * n;
  size_t shc = 2 * (size_t)W * padded_len(n) * sizeof(C);
  dim3 gc(column_ctas(ntiles));
  cols_kernel<T, true, EXT><<<gc, fft_threads<C>(), shc, st>>>(g, n, nkx, W, (long long)n * P, P, tw, ps->plan_n, one);
  cols_kernel<T, true, EXT><<<gc, fft_threads<C>(), shc, st>>>(g, n, nkx, W, P, (long long)n * P, tw, ps->plan_n, one);
  size_t shx = (size_t)rows * padded_len(N2) * sizeof(C);
  int gx = (int)((nn + rows - 1) / rows);
  c2r_x_kernel<T, EXT><<<gx, fft_threads<C>(), shx, st>>>(g, n, P, tw, ps->plan_h, rows, one);
  return cudaGetLastError();
}

template <typename T>
cudaError_t fft3d_forward(exc_poisson* ps, const T* src, cudaStream_t st) {
  return plan_ext(ps->plan_n) || plan_ext(ps->plan_h) ? fft3d_forward_t<T, true>(ps, src, st)
                                                      : fft3d_forward_t<T, false>(ps, src, st);
}

template <typename T>
cudaError_t fft3d_inverse(exc_poisson* ps, cudaStream_t st) {
  return plan_ext(ps->plan_n) || plan_ext(ps->plan_h) ? fft3d_inverse_t<T, true>(ps, st)
                                                      : fft3d_inverse_t<T, false>(ps, st);
}

template cudaError_t fft3d_forward<double>(exc_poisson*, const double*, cudaStream_t);
template cudaError_t fft3d_forward<float>(exc_poisson*, const float*, cudaStream_t);
template cudaError_t fft3d_inverse<double>(exc_poisson*, cudaStream_t);
template cudaError_t fft3d_inverse<float>(exc_poisson*, cudaStream_t);

template <typename T>
cudaError_t copy_pressure(const exc_poisson* ps, T* p, cudaStream_t st) {
  long long N = (long long)ps->n * ps->n * ps->n;
  int blocks = (int)std::min<long long>((N + 255) / 256, 152LL * 16);
  copy_pitched_kernel<T><<<blocks, 256, 0, st>>>(reinterpret_cast<const T*>(ps->work), 2 * ps->P, p, ps->n);
  return cudaGetLastError();
}

template cudaError_t poisson_solve_inplace<double>(exc_poisson*, const double*, bool, cudaStream_t, const SlotBatch&,
                                                   int);
template cudaError_t poisson_solve_inplace<float>(exc_poisson*, const float*, bool, cudaStream_t, const SlotBatch&,
                                                  int);
template cudaError_t copy_pressure<double>(const exc_poisson*, double*, cudaStream_t);
template cudaError_t copy_pressure<float>(const exc_poisson*, float*, cudaStream_t);

template <typename T, bool EXT>
static cudaError_t configure_fft_t() {
  using C = cplx<T>;
  // a tile of fft_tile elements in padded lines: at most 9/8 of it plus a slot per line
  int maxsh = (int)(fft_tile<C>() * 9 / 8 + 1024) * (int)sizeof(C);
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(r2c_x_kernel<T, true, EXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsh)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(r2c_x_kernel<T, false, EXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsh)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(cols_kernel<T, false, EXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * maxsh)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(cols_kernel<T, true, EXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * maxsh)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(zsolve_kernel<T, EXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * maxsh)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(c2r_x_kernel<T, EXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsh)) != cudaSuccess) return e;
  return cudaSuccess;
}

cudaError_t configure_fft() {
  cudaError_t e = configure_fft_t<double, false>();
  if (e == cudaSuccess) e = configure_fft_t<float, false>();
  if (e == cudaSuccess) e = configure_fft_t<double, true>();
  if (e == cudaSuccess) e = configure_fft_t<float, true>();
  if (e == cudaSuccess) e = configure_fftreg_f64();
  if (e == cudaSuccess) e = configure_fftreg_f32();
  if (e == cudaSuccess) e = configure_fftmix();
  return e;
}

// Level twiddles of a length-L register plan with first factor N1:
// tl[k1 N2 + m2] = W_L^(m2 k1), from long double.
template <typename C>
static std::vector<C> level_table(int L, int N1) {
  const int N2 = L / N1;
  std::vector<C> t((size_t)L);
  const long double pi_l = 3.141592653589793238462643383279502884L;
  for (int k1 = 0; k1 < N1; ++k1)
    for (int m2 = 0; m2 < N2; ++m2) {
      const long double a = -2.0L * pi_l * (long double)((m2 * k1) % L) / (long double)L;
      C w;
      w.x = (decltype(w.x))cosl(a);
      w.y = (decltype(w.y))sinl(a);
      t[(size_t)k1 * N2 + m2] = w;
    }
  return t;
}

template <typename C>
static int alloc_level_tables(exc_poisson* ps) {
  const int n = ps->n;
  const std::vector<C> tn = level_table<C>(n, reg_split_host(n));
  const std::vector<C> th = level_table<C>(n / 2, reg_split_host(n / 2));
  if (cudaMalloc(&ps->twl_n, tn.size() * sizeof(C)) != cudaSuccess ||
      cudaMalloc(&ps->twl_h, th.size() * sizeof(C)) != cudaSuccess) {
    set_last_error("out of device memory (poisson level twiddles)");
    return EXC_ERR_OOM;
  }
  cudaMemcpy(ps->twl_n, tn.data(), tn.size() * sizeof(C), cudaMemcpyHostToDevice);
  cudaMemcpy(ps->twl_h, th.data(), th.size() * sizeof(C), cudaMemcpyHostToDevice);
  return EXC_OK;
}

int poisson_init(exc_poisson* ps, int precision, int n, double l, void* work) {
  if (!fft_size_ok(n)) { set_last_error("grid size must be 2^a 3^b 5^c 7^d 11^e 13^f 17^g, a >= 1, 4 <= n <= 1024"); return EXC_ERR_SHAPE; }
  if (!(l > 0)) { set_last_error("domain size must be positive"); return EXC_ERR_ARG; }
  if (precision != EXC_F64 && precision != EXC_F32) { set_last_error("bad precision"); return EXC_ERR_ARG; }
  ps->precision = precision;
  ps->n = n;
  ps->l = l;
  ps->h = l / n;
  ps->P = spec_pitch(n);
  ps->plan_n = make_plan(n);
  ps->plan_h = make_plan(n / 2);
  size_t csz = precision == EXC_F64 ? sizeof(double2) : sizeof(float2);
  int crc = configure_device();
  if (crc) return crc;
  // twiddles W_n^m and sin^2 table, from long double on the host
  std::vector<double2> twd(n);
  std::vector<float2> twf(n);
  std::vector<double> s2(n);
  const long double pi_l = 3.141592653589793238462643383279502884L;
  for (int m = 0; m < n; ++m) {
    long double a = -2.0L * pi_l * (long double)m / (long double)n;
    double c = (double)cosl(a), s = (double)sinl(a);
    twd[m] = make_double2(c, s);
    twf[m] = make_float2((float)cosl(a), (float)sinl(a));
    long double sn = sinl(pi_l * (long double)std::min(m, n - m) / (long double)n);
    s2[m] = (double)(sn * sn);  // mirrored: s2[n - m] == s2[m]
  }
  if (cudaMalloc(&ps->tw, n * csz) != cudaSuccess || cudaMalloc(&ps->sin2, n * sizeof(double)) != cudaSuccess) {
    set_last_error("out of device memory (poisson tables)");
    poisson_free(ps);
    return EXC_ERR_OOM;
  }
  cudaMemcpy(ps->tw, precision == EXC_F64 ? (const void*)twd.data() : (const void*)twf.data(), n * csz,
             cudaMemcpyHostToDevice);
  cudaMemcpy(ps->sin2, s2.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  {
    // 1/(lambda N) per mode with ky, kz folded to <= n/2 (lambda is even in
    // each wavenumber), from an exact float64 division
    const size_t tb = (size_t)(n / 2 + 1) * (n / 2 + 1) * (n / 2 + 1) * sizeof(double);
    if (cudaMalloc(&ps->invlap, tb) != cudaSuccess) {
      set_last_error("out of device memory (poisson inverse symbol)");
      poisson_free(ps);
      return EXC_ERR_OOM;
    }
    const double coef = -ps->h * ps->h / (4.0 * (double)n * (double)n * (double)n);
    const long long tot = (long long)(n / 2 + 1) * (n / 2 + 1) * (n / 2 + 1);
    invlap_kernel<<<(int)std::min<long long>((tot + 255) / 256, 152LL * 32), 256>>>(n, ps->sin2, coef, ps->invlap);
    if (precision == EXC_F32)
      invlap_split_kernel<<<(int)std::min<long long>((tot + 255) / 256, 152LL * 32), 256>>>(tot, ps->invlap);
  }
  if (fftreg_supported(n, precision)) {
    const int rc = precision == EXC_F64 ? alloc_level_tables<double2>(ps) : alloc_level_tables<float2>(ps);
    if (rc) { poisson_free(ps); return rc; }
  }
  if (precision == EXC_F64 && !work && fftmix_supported(n)) {
    // the mixed-precision solve's FP32 inner solver, with the factor 1/h of
    // the unscaled FP64 divergence folded into its divide table
    ps->mix = new exc_poisson;
    int rc = poisson_init(ps->mix, EXC_F32, n, l, nullptr);
    if (rc) { poisson_free(ps); return rc; }
    const long long tot = (long long)(n / 2 + 1) * (n / 2 + 1) * (n / 2 + 1);
    const double coef_mix = -ps->h / (4.0 * (double)n * (double)n * (double)n);
    const int blocks = (int)std::min<long long>((tot + 255) / 256, 152LL * 32);
    invlap_kernel<<<blocks, 256>>>(n, ps->mix->sin2, coef_mix, ps->mix->invlap);
    invlap_split_kernel<<<blocks, 256>>>(tot, ps->mix->invlap);
    if (cudaMalloc(&ps->mix_d, (size_t)n * n * n * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&ps->mix_q, (size_t)n * n * n * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&ps->mix_q2, (size_t)n * n * n * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&ps->mix_part, (size_t)fftmix_part_words(n) * sizeof(double)) != cudaSuccess) {
      set_last_error("out of device memory (mixed-precision poisson buffers)");
      poisson_free(ps);
      return EXC_ERR_OOM;
    }
  }
  size_t wbytes = (size_t)n * n * ps->P * csz;
  if (work) {
    ps->work = work;
    ps->external_work = true;
  } else {
    if (cudaMalloc(&ps->work, wbytes) != cudaSuccess) {
      set_last_error("out of device memory (poisson work array)");
      poisson_free(ps);
      return EXC_ERR_OOM;
    }
    cudaMemset(ps->work, 0, wbytes);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); poisson_free(ps); return EXC_ERR_CUDA; }
  return EXC_OK;
}

void poisson_free(exc_poisson* ps) {
  if (ps->mix) {
    poisson_free(ps->mix);
    delete ps->mix;
    ps->mix = nullptr;
  }
  if (ps->mix_d) cudaFree(ps->mix_d);
  if (ps->mix_q) cudaFree(ps->mix_q);
  if (ps->mix_q2) cudaFree(ps->mix_q2);
  if (ps->mix_part) cudaFree(ps->mix_part);
  ps->mix_d = ps->mix_part = nullptr;
  ps->mix_q = ps->mix_q2 = nullptr;
  if (ps->tw) cudaFree(ps->tw);
  if (ps->sin2) cudaFree(ps->sin2);
  if (ps->invlap) cudaFree(ps->invlap);
  ps->invlap = nullptr;
  if (ps->twl_n) cudaFree(ps->twl_n);
  if (ps->twl_h) cudaFree(ps->twl_h);
  ps->twl_n = ps->twl_h = nullptr;
  if (ps->work && !ps->external_work) cudaFree(ps->work);
  ps->tw = nullptr;
  ps->sin2 = nullptr;
  ps->work = nullptr;
}

}  // namespace exc
