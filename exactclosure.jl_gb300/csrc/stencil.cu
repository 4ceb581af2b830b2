// Staggered-grid stencils: the convection-diffusion RHS, divergence,
// pressure gradient and explicit tensor divergences (src/N.jl:94-254).
#include <type_traits>

#include "internal.cuh"

namespace exc {

// ---------------------------------------------------------------------------
// Simple per-cell kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cell_of(long long g, int n, int& x, int& y, int& z) {
  const IdxDiv dn(n);
  const long long r = dn.div(g);
  x = (int)(g - r * n);
  z = (int)dn.div(r);
  y = (int)(r - (long long)z * n);
}

// The 6 stress components materialised (src/N.jl:94-118).
template <typename T>
__global__ void stress_kernel(int n, T h, T visc, const T* __restrict__ u, T* __restrict__ s6) {
  const long long N = (long long)n * n * n;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    cell_of(g, n, x, y, z);
    int c[3] = {x, y, z};
    const int comps[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {2, 0}};
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      int i = comps[m][0], j = comps[m][1];
      auto idx = [&](int d, int s) {
        int cc[3] = {c[0], c[1], c[2]};
        cc[d] = (cc[d] + s + n) % n;
        return ((long long)cc[2] * n + cc[1]) * n + cc[0];
      };
      int off = (i != j);
      T uir = u[i * N + idx(j, off)], uil = u[i * N + idx(j, off - 1)];
      T ujr = u[j * N + idx(i, off)], ujl = u[j * N + idx(i, off - 1)];
      T etaj_ui = (uir + uil) / 2, etai_uj = (ujr + ujl) / 2;
      T dj_ui = (uir - uil) / h, di_uj = (ujr - ujl) / h;
      s6[m * N + g] = etaj_ui * etai_uj - visc * (dj_ui + di_uj);
    }
  }
}

// du_i = doadd*du_i - sum_j delta_j s_ij with an explicit tensor (src/N.jl:120-200).
template <typename T>
__global__ void tensordiv_kernel(int n, T h, int nsym, const T* __restrict__ s, T* __restrict__ du, int doadd) {
  const long long N = (long long)n * n * n;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    cell_of(g, n, x, y, z);
    int c[3] = {x, y, z};
    auto nb = [&](int d, int sgn) {
      int cc[3] = {c[0], c[1], c[2]};
      cc[d] = (cc[d] + sgn + n) % n;
      return ((long long)cc[2] * n + cc[1]) * n + cc[0];
    };
    for (int i = 0; i < 3; ++i) {
      T acc = doadd ? du[i * N + g] : (T)0;
      for (int j = 0; j < 3; ++j) {
        int m;
        if (nsym == 9) m = 3 * j + i;  // s11,s21,s31,s12,... (src/N.jl:181)
        else {
          if (i == j) m = i;
          else {
            int a = i < j ? i : j, b = i < j ? j : i;
            m = (a == 0 && b == 1) ? 3 : (a == 1 && b == 2) ? 4 : 5;
          }
        }
        const T* sc = s + (long long)m * N;
        if (i == j) acc -= (sc[nb(j, 1)] - sc[g]) / h;
        else acc -= (sc[g] - sc[nb(j, -1)]) / h;
      }
      du[i * N + g] = acc;
    }
  }
}

template <typename T>
__global__ void divergence_kernel(int n, T h, const T* __restrict__ u, T* __restrict__ d) {
  const long long N = (long long)n * n * n;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    cell_of(g, n, x, y, z);
    long long gx = g - x + wrap_dn(x, n);
    long long gy = ((long long)z * n + wrap_dn(y, n)) * n + x;
    long long gz = ((long long)wrap_dn(z, n) * n + y) * n + x;
    d[g] = (u[g] - u[gx]) / h + (u[N + g] - u[N + gy]) / h + (u[2 * N + g] - u[2 * N + gz]) / h;
  }
}

// u_i -= (p[I+e_i] - p[I]) / h, p at row pitch ppitch (src/N.jl:240-254).
template <typename T>
__global__ void gradient_kernel(int n, T inv_h, T* __restrict__ u, const T* __restrict__ p, int ppitch) {
  const long long N = (long long)n * n * n;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    cell_of(g, n, x, y, z);
    long long row = (long long)z * n + y;
    T pc = p[row * ppitch + x];
    T px = p[row * ppitch + wrap_up(x, n)];
    T py = p[((long long)z * n + wrap_up(y, n)) * ppitch + x];
    T pz = p[((long long)wrap_up(z, n) * n + y) * ppitch + x];
    u[g] -= (px - pc) * inv_h;
    u[N + g] -= (py - pc) * inv_h;
    u[2 * N + g] -= (pz - pc) * inv_h;
  }
}

// The same update for even n, two cells of a row per thread (vector loads
// and stores, one 32-bit division per thread): the expressions of
// gradient_kernel, so the results are bit-identical.
template <typename T>
__global__ void gradient2_kernel(int n, T inv_h, T* __restrict__ u, const T* __restrict__ p, int ppitch) {
  using V2 = typename std::conditional<sizeof(T) == 8, double2, float2>::type;
  const long long N = (long long)n * n * n;
  const int hx = n >> 1;
  const long long total = N >> 1;
  // total < 2^31 (launch condition): 32-bit index arithmetic
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const unsigned r32 = (unsigned)t / (unsigned)hx;
    const long long row = r32;
    const int x = 2 * (int)((unsigned)t - r32 * (unsigned)hx);
    const int z = (int)(r32 / (unsigned)n), y = (int)(r32 - (unsigned)z * (unsigned)n);
    const T* const pr = p + row * ppitch;
    const V2 pc = *reinterpret_cast<const V2*>(pr + x);
    const T pn = pr[x + 2 == n ? 0 : x + 2];
    const V2 py = *reinterpret_cast<const V2*>(p + ((long long)z * n + wrap_up(y, n)) * ppitch + x);
    const V2 pz = *reinterpret_cast<const V2*>(p + ((long long)wrap_up(z, n) * n + y) * ppitch + x);
    const long long g = row * n + x;
    V2* const u0 = reinterpret_cast<V2*>(u + g);
    V2* const u1 = reinterpret_cast<V2*>(u + N + g);
    V2* const u2 = reinterpret_cast<V2*>(u + 2 * N + g);
    V2 a = *u0, b = *u1, c = *u2;
    a.x -= (pc.y - pc.x) * inv_h;
    a.y -= (pn - pc.y) * inv_h;
    b.x -= (py.x - pc.x) * inv_h;
    b.y -= (py.y - pc.y) * inv_h;
    c.x -= (pz.x - pc.x) * inv_h;
    c.y -= (pz.y - pc.y) * inv_h;
    *u0 = a;
    *u1 = b;
    *u2 = c;
  }
}

static inline int grid_for(long long N, int threads) {
  long long b = (N + threads - 1) / threads;
  return (int)(b < 152LL * 32 ? b : 152LL * 32);
}

template <typename T>
cudaError_t launch_stress(int n, T h, T visc, const T* u, T* s6, cudaStream_t st) {
  long long N = (long long)n * n * n;
  stress_kernel<T><<<grid_for(N, 256), 256, 0, st>>>(n, h, visc, u, s6);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_tensordiv(int n, T h, int nsym, const T* s, T* du, bool doadd, cudaStream_t st) {
  long long N = (long long)n * n * n;
  tensordiv_kernel<T><<<grid_for(N, 256), 256, 0, st>>>(n, h, nsym, s, du, doadd ? 1 : 0);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_divergence(int n, T h, const T* u, T* d, cudaStream_t st) {
  long long N = (long long)n * n * n;
  divergence_kernel<T><<<grid_for(N, 256), 256, 0, st>>>(n, h, u, d);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_gradient(int n, T h, T* u, const T* p, int ppitch, cudaStream_t st) {
  long long N = (long long)n * n * n;
  const bool vec = n % 2 == 0 && ppitch % 2 == 0 && N / 2 < (1LL << 31) && (reinterpret_cast<uintptr_t>(u) % (2 * sizeof(T))) == 0 &&
                   (reinterpret_cast<uintptr_t>(p) % (2 * sizeof(T))) == 0;
  if (vec)
    gradient2_kernel<T><<<grid_for(N / 2, 256), 256, 0, st>>>(n, (T)(1.0 / (double)h), u, p, ppitch);
  else
    gradient_kernel<T><<<grid_for(N, 256), 256, 0, st>>>(n, (T)(1.0 / (double)h), u, p, ppitch);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// max |x|: per-block maxima into `partial`, then one block folds them
// (deterministic; no atomics).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void maxabs_partial_kernel(size_t count, const T* __restrict__ x, double* __restrict__ partial) {
  // the maximum of |x| is taken on the magnitude bits (unsigned integer order
  // equals the order of non-negative IEEE values, and NaN patterns sort above
  // infinity, so a NaN propagates): exact, on the integer pipe, and with
  // 16-byte loads when the array allows them
  using B = typename MagBits<T>::type;
  __shared__ B red[32];
  B m = 0;
  constexpr int E = 16 / (int)sizeof(T);
  const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x, nth = (size_t)gridDim.x * blockDim.x;
  size_t done = 0;
  if ((reinterpret_cast<uintptr_t>(x) & 15) == 0) {
    using V = typename MagBits<T>::vec;
    const V* xv = reinterpret_cast<const V*>(x);
    const size_t nv = count / E;
#pragma unroll 4
    for (size_t i = tid; i < nv; i += nth) {
      const V v = xv[i];
      const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
      for (int k = 0; k < E; ++k) m = max(m, mag_bits(e[k]));
    }
    done = nv * E;
  }
  for (size_t i = done + tid; i < count; i += nth) m = max(m, mag_bits(x[i]));
  for (int o = 16; o > 0; o >>= 1) m = max(m, (B)__shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : (B)0;
    for (int o = 16; o > 0; o >>= 1) m = max(m, (B)__shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) partial[blockIdx.x] = (double)from_mag_bits<T>(m);
  }
}

__global__ void maxabs_final_kernel(int np, const double* __restrict__ partial, double* __restrict__ out) {
  __shared__ double red[32];
  double m = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    double v = partial[i];
    m = (v > m || v != v) ? v : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_xor_sync(0xffffffffu, m, o);
    m = (w > m || w != w) ? w : m;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      double w = __shfl_xor_sync(0xffffffffu, m, o);
      m = (w > m || w != w) ? w : m;
    }
    if (threadIdx.x == 0) *out = m;
  }
}

template <typename T>
cudaError_t launch_max_abs(size_t count, const T* x, double* out_dev, double* partial, int npartial,
                           cudaStream_t st) {
  int blocks = (int)std::min<size_t>((count + 255) / 256, (size_t)npartial);
  if (blocks < 1) blocks = 1;
  maxabs_partial_kernel<T><<<blocks, 256, 0, st>>>(count, x, partial);
  maxabs_final_kernel<<<1, 1024, 0, st>>>(blocks, partial, out_dev);
  return cudaGetLastError();
}

#define INST(T)                                                                                   \
  template cudaError_t launch_stress<T>(int, T, T, const T*, T*, cudaStream_t);                   \
  template cudaError_t launch_tensordiv<T>(int, T, int, const T*, T*, bool, cudaStream_t);        \
  template cudaError_t launch_divergence<T>(int, T, const T*, T*, cudaStream_t);                  \
  template cudaError_t launch_gradient<T>(int, T, T*, const T*, int, cudaStream_t);               \
  template cudaError_t launch_max_abs<T>(size_t, const T*, double*, double*, int, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace exc
