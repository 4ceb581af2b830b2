// Pointwise field kernels: RK4 stage combination, the projected-RHS update
// k = rhs - grad p, the counter-based normal generator, FP64 reductions and
// the deterministic shell histogram used by `randomfield` and `spectrum`.
#include "internal.cuh"
#include "fields.cuh"

namespace exc {

static inline int grid_for(long long N, int threads = 256) {
  long long b = (N + threads - 1) / threads;
  return (int)(b < 152LL * 32 ? b : 152LL * 32);
}

// ---------------------------------------------------------------------------
// k = rhs - grad p in place (rhs <- k), p read at pitch 2P from the Poisson
// work array (`pressuregradient!`, src/N.jl:240-254), then the RK4 stage
// combination of the tableau of `rk4_timestep!` (src/Burgers.jl:120-142):
//   s = 0: xfin = x0 + dt/6 k;  xs = x0 + dt/2 k
//   s = 1: xfin += dt/3 k;      xs = x0 + dt/2 k
//   s = 2: xfin += dt/3 k;      xs = x0 + dt k
//   s = 3: xfin += dt/6 k
// ---------------------------------------------------------------------------
// With STORE_K the projected k is written back (the LES closures filter it);
// without, k is consumed here and the write is skipped.
template <typename T, bool GRAD, bool STORE_K = true>
__global__ void rk_stage_kernel(int n, T inv_h, T* __restrict__ k, const T* __restrict__ p, int ppitch,
                                const T* __restrict__ x0, T* __restrict__ xs, T* __restrict__ xfin, int stage,
                                const double* __restrict__ dtp, SlotBatch sb) {
  const long long N = (long long)n * n * n;
  const int slot = blockIdx.y;  // batch of same-size solves (serving form)
  if (sb.active && !sb.active[slot]) return;
  k += slot * sb.ustride;
  x0 += slot * sb.ustride;
  xs += slot * sb.ustride;
  xfin += slot * sb.ustride;
  if (GRAD) p += slot * 2 * sb.wstride;
  const double dt = dtp[slot];
  const T cf = (T)((stage == 0 || stage == 3) ? dt / 6.0 : dt / 3.0);
  const T cs = (T)(stage == 2 ? dt : 0.5 * dt);
  const IdxDiv dn(n);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
    T k0 = k[g], k1 = k[N + g], k2 = k[2 * N + g];
    if (GRAD) {
      const long long r = dn.div(g);
      int x = (int)(g - r * n);
      int z = (int)dn.div(r);
      int y = (int)(r - (long long)z * n);
      T pc = p[r * ppitch + x];
      T px = p[r * ppitch + wrap_up(x, n)];
      T py = p[((long long)z * n + wrap_up(y, n)) * ppitch + x];
      T pz = p[((long long)wrap_up(z, n) * n + y) * ppitch + x];
      k0 -= (px - pc) * inv_h;
      k1 -= (py - pc) * inv_h;
      k2 -= (pz - pc) * inv_h;
      if (STORE_K) {
        k[g] = k0;
        k[N + g] = k1;
        k[2 * N + g] = k2;
      }
    }
    T a0 = 0, a1 = 0, a2 = 0;  // x0 is not read at stage 3
    if (stage < 3) {
      a0 = x0[g];
      a1 = x0[N + g];
      a2 = x0[2 * N + g];
    }
    if (stage == 0) {
      xfin[g] = a0 + cf * k0;
      xfin[N + g] = a1 + cf * k1;
      xfin[2 * N + g] = a2 + cf * k2;
    } else {
      xfin[g] += cf * k0;
      xfin[N + g] += cf * k1;
      xfin[2 * N + g] += cf * k2;
    }
    if (stage < 3) {
      xs[g] = a0 + cs * k0;
      xs[N + g] = a1 + cs * k1;
      xs[2 * N + g] = a2 + cs * k2;
    }
  }
}

// FP32 form of rk_stage_kernel with GRAD for n % 4 == 0: four consecutive
// x cells per thread with 16-byte loads and stores (same arithmetic per
// element, so the results are bitwise those of the scalar kernel).
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

template <bool STORE_K>
__global__ void rk_stage4_kernel(int n, float inv_h, float* __restrict__ k, const float* __restrict__ p, int ppitch,
                                 const float* __restrict__ x0, float* __restrict__ xs, float* __restrict__ xfin,
                                 int stage, const double* __restrict__ dtp, SlotBatch sb) {
  const long long N = (long long)n * n * n;
  const int slot = blockIdx.y;
  if (sb.active && !sb.active[slot]) return;
  k += slot * sb.ustride;
  x0 += slot * sb.ustride;
  xs += slot * sb.ustride;
  xfin += slot * sb.ustride;
  p += slot * 2 * sb.wstride;
  const double dt = dtp[slot];
  const float cf = (float)((stage == 0 || stage == 3) ? dt / 6.0 : dt / 3.0);
  const float cs = (float)(stage == 2 ? dt : 0.5 * dt);
  const IdxDiv dn(n);
  const long long Q = N / 4;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < Q; q += (long long)gridDim.x * blockDim.x) {
    const long long g = 4 * q;
    const long long r = dn.div(g);
    const int x = (int)(g - r * n);
    const int z = (int)dn.div(r);
    const int y = (int)(r - (long long)z * n);
    float4 k0 = ld4(k + g), k1 = ld4(k + N + g), k2 = ld4(k + 2 * N + g);
    const float* prow = p + r * ppitch;
    const float4 pc = ld4(prow + x);
    const float pn = prow[x + 4 == n ? 0 : x + 4];
    const float4 py = ld4(p + ((long long)z * n + wrap_up(y, n)) * ppitch + x);
    const float4 pz = ld4(p + ((long long)wrap_up(z, n) * n + y) * ppitch + x);
    k0.x -= (pc.y - pc.x) * inv_h; k0.y -= (pc.z - pc.y) * inv_h;
    k0.z -= (pc.w - pc.z) * inv_h; k0.w -= (pn - pc.w) * inv_h;
    k1.x -= (py.x - pc.x) * inv_h; k1.y -= (py.y - pc.y) * inv_h;
    k1.z -= (py.z - pc.z) * inv_h; k1.w -= (py.w - pc.w) * inv_h;
    k2.x -= (pz.x - pc.x) * inv_h; k2.y -= (pz.y - pc.y) * inv_h;
    k2.z -= (pz.z - pc.z) * inv_h; k2.w -= (pz.w - pc.w) * inv_h;
    if (STORE_K) {
      st4(k + g, k0);
      st4(k + N + g, k1);
      st4(k + 2 * N + g, k2);
    }
    const float4 kk[3] = {k0, k1, k2};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float4 kc = kk[c];
      const float4 a = stage < 3 ? ld4(x0 + c * N + g) : make_float4(0.f, 0.f, 0.f, 0.f);  // unused at stage 3
      float4 f;
      if (stage == 0) {
        f = make_float4(a.x + cf * kc.x, a.y + cf * kc.y, a.z + cf * kc.z, a.w + cf * kc.w);
      } else {
        f = ld4(xfin + c * N + g);
        f.x += cf * kc.x; f.y += cf * kc.y; f.z += cf * kc.z; f.w += cf * kc.w;
      }
      st4(xfin + c * N + g, f);
      if (stage < 3) st4(xs + c * N + g, make_float4(a.x + cs * kc.x, a.y + cs * kc.y, a.z + cs * kc.z, a.w + cs * kc.w));
    }
  }
}

// FP64 form: two consecutive x cells per thread with 16-byte accesses (same
// arithmetic per element as the scalar kernel).
__device__ __forceinline__ double2 ld2(const double* p) { return *reinterpret_cast<const double2*>(p); }
__device__ __forceinline__ void st2(double* p, double2 v) { *reinterpret_cast<double2*>(p) = v; }

// WOUT: the stage state goes out in the RHS sweep's shifted form w = sq x -
// qs (fp64_shift of inv_h and wvisc), the only form its one reader, the next
// RHS sweep, needs: the same bits as the sweep shifting the plain state.
template <bool STORE_K, bool WOUT = false>
__global__ void rk_stage2_kernel(int n, double inv_h, double* __restrict__ k, const double* __restrict__ p, int ppitch,
                                 const double* __restrict__ x0, double* __restrict__ xs, double* __restrict__ xfin,
                                 int stage, const double* __restrict__ dtp, SlotBatch sb, double wvisc = 0.0) {
  const long long N = (long long)n * n * n;
  const int slot = blockIdx.y;
  if (sb.active && !sb.active[slot]) return;
  k += slot * sb.ustride;
  x0 += slot * sb.ustride;
  xs += slot * sb.ustride;
  xfin += slot * sb.ustride;
  p += slot * 2 * sb.wstride;
  const double dt = dtp[slot];
  const double cf = (stage == 0 || stage == 3) ? dt / 6.0 : dt / 3.0;
  const double cs = stage == 2 ? dt : 0.5 * dt;
  const Fp64Shift fs = fp64_shift(inv_h, wvisc);
  const IdxDiv dn(n);
  const long long Q = N / 2;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < Q; q += (long long)gridDim.x * blockDim.x) {
    const long long g = 2 * q;
    const long long r = dn.div(g);
    const int x = (int)(g - r * n);
    const int z = (int)dn.div(r);
    const int y = (int)(r - (long long)z * n);
    double2 k0 = ld2(k + g), k1 = ld2(k + N + g), k2 = ld2(k + 2 * N + g);
    const double* prow = p + r * ppitch;
    const double2 pc = ld2(prow + x);
    const double pn = prow[x + 2 == n ? 0 : x + 2];
    const double2 py = ld2(p + ((long long)z * n + wrap_up(y, n)) * ppitch + x);
    const double2 pz = ld2(p + ((long long)wrap_up(z, n) * n + y) * ppitch + x);
    k0.x -= (pc.y - pc.x) * inv_h; k0.y -= (pn - pc.y) * inv_h;
    k1.x -= (py.x - pc.x) * inv_h; k1.y -= (py.y - pc.y) * inv_h;
    k2.x -= (pz.x - pc.x) * inv_h; k2.y -= (pz.y - pc.y) * inv_h;
    if (STORE_K) {
      st2(k + g, k0);
      st2(k + N + g, k1);
      st2(k + 2 * N + g, k2);
    }
    const double2 kk[3] = {k0, k1, k2};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double2 kc = kk[c];
      const double2 a = stage < 3 ? ld2(x0 + c * N + g) : make_double2(0.0, 0.0);  // unused at stage 3
      double2 f;
      if (stage == 0) {
        f = make_double2(a.x + cf * kc.x, a.y + cf * kc.y);
      } else {
        f = ld2(xfin + c * N + g);
        f.x += cf * kc.x;
        f.y += cf * kc.y;
      }
      st2(xfin + c * N + g, f);
      if (stage < 3) {
        double2 v = make_double2(fma(cs, kc.x, a.x), fma(cs, kc.y, a.y));
        if (WOUT) v = make_double2(fma(fs.sq, v.x, -fs.qs), fma(fs.sq, v.y, -fs.qs));
        st2(xs + c * N + g, v);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// RK stage that also forms the transverse box sums of the LES filters (the
// first pass of filter_vector_box, tb_kernel) of k and of the stage output:
// a CTA owns one coarse column (Jz, Jy) of ratio C0 (C0^2 fine rows of n
// cells) and walks it in chunks of XC cells per row; after the RK arithmetic
// of rk_stage4_kernel / rk_stage2_kernel (same expressions, V cells per
// thread), k and the stage output of the chunk sit in shared memory and are
// summed over the C0 x C0 transverse boxes in tb_kernel's order, so the sums
// are bit-identical to tb_kernel's on the stored fields.  k itself is not
// stored.  tbs (sums of xs, stages 0-2) may be null.
// ---------------------------------------------------------------------------
template <typename T, int C0>
__global__ void __launch_bounds__(256)
rk_stage_sums_kernel(int n, T inv_h, const T* __restrict__ k, const T* __restrict__ p, int ppitch,
                     const T* __restrict__ x0, T* __restrict__ xs, T* __restrict__ xfin, int stage,
                     const double* __restrict__ dtp, T* __restrict__ tbk, T* __restrict__ tbs) {
  constexpr int V = 16 / (int)sizeof(T);
  constexpr int ROWS = C0 * C0;
  constexpr int LANES = 256 / ROWS;
  constexpr int XC = LANES * V;
  constexpr int JC = XC / C0;  // coarse x cells per chunk
  static_assert(ROWS <= 256 && XC % C0 == 0, "chunk must hold whole coarse cells");
  __shared__ __align__(16) T sk[3][ROWS][XC];
  __shared__ __align__(16) T ss[3][ROWS][XC];
  const int m = n / C0;
  const long long N = (long long)n * n * n;
  const long long Mt = (long long)n * m * m;
  const int Jy = blockIdx.x % m, Jz = blockIdx.x / m;
  const int tid = threadIdx.x, r = tid / LANES, lane = tid - r * LANES;
  const int z = C0 * Jz + r / C0, y = C0 * Jy + r % C0;
  const double dt = dtp[0];
  const T cf = (T)((stage == 0 || stage == 3) ? dt / 6.0 : dt / 3.0);
  const T cs = (T)(stage == 2 ? dt : 0.5 * dt);
  const long long rowbase = ((long long)z * n + y) * n;
  const T* prow = p + ((long long)z * n + y) * ppitch;
  const T* prowy = p + ((long long)z * n + wrap_up(y, n)) * ppitch;
  const T* prowz = p + ((long long)wrap_up(z, n) * n + y) * ppitch;
  const bool sums_s = tbs != nullptr && stage < 3;
  for (int xc = 0; xc < n; xc += XC) {
    const int x = xc + V * lane;
    const long long g = rowbase + x;
    T kk[3][V], pc[V], py[V], pz[V];
#pragma unroll
    for (int i = 0; i < V; ++i) {
      kk[0][i] = k[g + i];
      kk[1][i] = k[N + g + i];
      kk[2][i] = k[2 * N + g + i];
      pc[i] = prow[x + i];
      py[i] = prowy[x + i];
      pz[i] = prowz[x + i];
    }
    const T pn = prow[x + V == n ? 0 : x + V];
#pragma unroll
    for (int i = 0; i < V; ++i) {
      kk[0][i] -= ((i + 1 < V ? pc[i + 1] : pn) - pc[i]) * inv_h;
      kk[1][i] -= (py[i] - pc[i]) * inv_h;
      kk[2][i] -= (pz[i] - pc[i]) * inv_h;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T a[V], f[V];
#pragma unroll
      for (int i = 0; i < V; ++i) a[i] = stage < 3 ? x0[c * N + g + i] : (T)0;  // x0 unused at stage 3
#pragma unroll
      for (int i = 0; i < V; ++i) f[i] = stage == 0 ? a[i] + cf * kk[c][i] : xfin[c * N + g + i] + cf * kk[c][i];
#pragma unroll
      for (int i = 0; i < V; ++i) xfin[c * N + g + i] = f[i];
      if (stage < 3) {
#pragma unroll
        for (int i = 0; i < V; ++i) {
          const T sv = a[i] + cs * kk[c][i];
          xs[c * N + g + i] = sv;
          ss[c][r][V * lane + i] = sv;
        }
      }
#pragma unroll
      for (int i = 0; i < V; ++i) sk[c][r][V * lane + i] = kk[c][i];
    }
    __syncthreads();
    // box sums of the chunk: component 0 over the C0^2 rows at each x;
    // component 1 over (dz, dx) for each dy; component 2 over (dy, dx) for
    // each dz (tb_kernel's orders)
    for (int q = 0; q < (sums_s ? 2 : 1); ++q) {
      const T(*src)[ROWS][XC] = q == 0 ? sk : ss;
      T* const out = q == 0 ? tbk : tbs;
      for (int o = tid; o < 3 * XC; o += 256) {
        const int c = o / XC, i = o - c * XC;
        T acc = (T)0;
        if (c == 0) {
#pragma unroll 4
          for (int rr = 0; rr < ROWS; ++rr) acc += src[0][rr][i];
          out[((long long)Jz * m + Jy) * n + xc + i] = acc;
        } else if (c == 1) {
          const int ddy = i / JC, jx = i - ddy * JC;
          for (int ddz = 0; ddz < C0; ++ddz)
#pragma unroll
            for (int dx = 0; dx < C0; ++dx) acc += src[1][ddz * C0 + ddy][C0 * jx + dx];
          out[Mt + ((long long)Jz * n + C0 * Jy + ddy) * m + xc / C0 + jx] = acc;
        } else {
          const int ddz = i / JC, jx = i - ddz * JC;
          for (int ddy = 0; ddy < C0; ++ddy)
#pragma unroll
            for (int dx = 0; dx < C0; ++dx) acc += src[2][ddz * C0 + ddy][C0 * jx + dx];
          out[2 * Mt + ((long long)(C0 * Jz + ddz) * m + Jy) * m + xc / C0 + jx] = acc;
        }
      }
    }
    __syncthreads();
  }
}

template <typename T>
cudaError_t launch_rk_stage_sums(int n, int c0, T h, const T* k, const T* p, int ppitch, const T* x0, T* xs, T* xfin,
                                 int stage, const double* dtp, T* tbk, T* tbs, cudaStream_t st) {
  const int xcw = rk_sums_chunk<T>(c0);
  if (!xcw || n % xcw != 0 || n % c0 != 0) return cudaErrorInvalidValue;
  const int m = n / c0;
  const T ih = (T)(1.0 / (double)h);
  const dim3 grid((unsigned)(m * m));
  switch (c0) {
    case 2: rk_stage_sums_kernel<T, 2><<<grid, 256, 0, st>>>(n, ih, k, p, ppitch, x0, xs, xfin, stage, dtp, tbk, tbs); break;
    case 4: rk_stage_sums_kernel<T, 4><<<grid, 256, 0, st>>>(n, ih, k, p, ppitch, x0, xs, xfin, stage, dtp, tbk, tbs); break;
    default: rk_stage_sums_kernel<T, 8><<<grid, 256, 0, st>>>(n, ih, k, p, ppitch, x0, xs, xfin, stage, dtp, tbk, tbs); break;
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_rk_stage(int n, T h, T* k, const T* p, int ppitch, const T* x0, T* xs, T* xfin, int stage,
                            const double* dtp, cudaStream_t st, const SlotBatch& sb, int nslots, bool store_k,
                            bool shifted_out, double visc) {
  if (shifted_out && (!p || !rk_writes_shifted<T>(n))) return cudaErrorInvalidValue;
  long long N = (long long)n * n * n;
  dim3 grid(nslots > 1 ? std::min(grid_for(N), 152 * 8) : grid_for(N), nslots);
  if constexpr (sizeof(T) == 4) {
    if (p && n % 4 == 0) {
      dim3 g4(nslots > 1 ? std::min(grid_for(N / 4), 152 * 8) : grid_for(N / 4), nslots);
      const float ih = (float)(1.0 / (double)h);
      if (store_k)
        rk_stage4_kernel<true><<<g4, 256, 0, st>>>(n, ih, (float*)k, (const float*)p, ppitch, (const float*)x0,
                                                   (float*)xs, (float*)xfin, stage, dtp, sb);
      else
        rk_stage4_kernel<false><<<g4, 256, 0, st>>>(n, ih, (float*)k, (const float*)p, ppitch, (const float*)x0,
                                                    (float*)xs, (float*)xfin, stage, dtp, sb);
      return cudaGetLastError();
    }
  } else {
    if (p && n % 2 == 0) {
      dim3 g2(nslots > 1 ? std::min(grid_for(N / 2), 152 * 8) : grid_for(N / 2), nslots);
      const double ih = 1.0 / (double)h;
      if (shifted_out && store_k)
        rk_stage2_kernel<true, true><<<g2, 256, 0, st>>>(n, ih, (double*)k, (const double*)p, ppitch,
                                                         (const double*)x0, (double*)xs, (double*)xfin, stage, dtp, sb,
                                                         visc);
      else if (shifted_out)
        rk_stage2_kernel<false, true><<<g2, 256, 0, st>>>(n, ih, (double*)k, (const double*)p, ppitch,
                                                          (const double*)x0, (double*)xs, (double*)xfin, stage, dtp, sb,
                                                          visc);
      else if (store_k)
        rk_stage2_kernel<true><<<g2, 256, 0, st>>>(n, ih, (double*)k, (const double*)p, ppitch, (const double*)x0,
                                                   (double*)xs, (double*)xfin, stage, dtp, sb);
      else
        rk_stage2_kernel<false><<<g2, 256, 0, st>>>(n, ih, (double*)k, (const double*)p, ppitch, (const double*)x0,
                                                    (double*)xs, (double*)xfin, stage, dtp, sb);
      return cudaGetLastError();
    }
  }
  if (p && store_k)
    rk_stage_kernel<T, true><<<grid, 256, 0, st>>>(n, (T)(1.0 / (double)h), k, p, ppitch, x0, xs, xfin, stage, dtp, sb);
  else if (p)
    rk_stage_kernel<T, true, false><<<grid, 256, 0, st>>>(n, (T)(1.0 / (double)h), k, p, ppitch, x0, xs, xfin, stage,
                                                          dtp, sb);
  else
    rk_stage_kernel<T, false><<<grid, 256, 0, st>>>(n, (T)0, k, nullptr, 0, x0, xs, xfin, stage, dtp, sb);
  return cudaGetLastError();
}

// a = a + b * scale (elementwise, count words)
template <typename T>
__global__ void axpy_kernel(long long count, T* __restrict__ a, const T* __restrict__ b, T scale) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    a[i] += scale * b[i];
}
template <typename T>
cudaError_t launch_axpy(long long count, T* a, const T* b, T scale, cudaStream_t st) {
  axpy_kernel<T><<<grid_for(count), 256, 0, st>>>(count, a, b, scale);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// dt = min(cfl*h/umax, cfl*h^2/visc/6) (`propose_timestep`, src/N.jl:348-356),
// or the fixed dt; flags a non-finite umax; advances the clock.
// ---------------------------------------------------------------------------
__global__ void set_dt_kernel(const double* __restrict__ umax, double h, double visc, double cfl, double fixed,
                              double* __restrict__ dt, double* __restrict__ clock, int* __restrict__ flag) {
  double m = *umax;
  double d;
  if (fixed > 0) d = fixed;
  else {
    double dt_adv = cfl * h / m;
    double dt_visc = cfl * h * h / visc / 6.0;
    d = dt_adv < dt_visc ? dt_adv : dt_visc;
  }
  if (!(m < 1e300)) { *flag = 1; d = 0.0; }
  *dt = d;
  *clock += d;
}
cudaError_t launch_set_dt(const double* umax, double h, double visc, double cfl, double fixed, double* dt,
                          double* clock, int* flag, cudaStream_t st) {
  set_dt_kernel<<<1, 1, 0, st>>>(umax, h, visc, cfl, fixed, dt, clock, flag);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Counter-based normals: splitmix64 of seed*phi + 2m (+1) -> two uniforms in
// (0,1) -> Box-Muller.  The oracle evaluates the same formula.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long splitmix(unsigned long long x) {
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
// The FP32 form draws the same counters with 24-bit uniforms and FP32
// Box-Muller (the FP64 pipe is the slow one on this part): each normal
// differs from the FP64 draw by about 1e-7 relative, below the form's own
// rounding; the FP64 path keeps the oracle's formula exactly.
template <typename T>
__global__ void normal_kernel(long long count, unsigned long long seed, T* __restrict__ out) {
  const unsigned long long base = seed * 0x9E3779B97F4A7C15ull;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    unsigned long long m = (unsigned long long)i;
    unsigned long long z1 = splitmix(base + 2ull * m);
    unsigned long long z2 = splitmix(base + 2ull * m + 1ull);
    if constexpr (sizeof(T) == 4) {
      const float u1 = ((float)(unsigned)(z1 >> 40) + 0.5f) * 0x1.0p-24f;
      const float u2 = ((float)(unsigned)(z2 >> 40) + 0.5f) * 0x1.0p-24f;
      out[i] = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
    } else {
      double u1 = ((double)(z1 >> 11) + 0.5) * 0x1.0p-53;
      double u2 = ((double)(z2 >> 11) + 0.5) * 0x1.0p-53;
      out[i] = (T)(sqrt(-2.0 * log(u1)) * cospi(2.0 * u2));
    }
  }
}
template <typename T>
cudaError_t launch_normals(long long count, unsigned long long seed, T* out, cudaStream_t st) {
  normal_kernel<T><<<grid_for(count), 256, 0, st>>>(count, seed, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Deterministic FP64 reductions.  Fixed grid; per-block partials; one block
// folds them in index order.
// ---------------------------------------------------------------------------
constexpr int RED_BLOCKS = 304;

// sums[0] = sum (a-b)^2, sums[1] = sum b^2 over count words (b may be null: sum a^2)
template <typename T>
__global__ void sqdiff_partial_kernel(long long count, const T* __restrict__ a, const T* __restrict__ b,
                                      double* __restrict__ part) {
  __shared__ double r0[256], r1[256];
  double s0 = 0, s1 = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    double av = (double)a[i];
    double bv = b ? (double)b[i] : 0.0;
    double d = av - bv;
    s0 += d * d;
    s1 += bv * bv;
  }
  r0[threadIdx.x] = s0;
  r1[threadIdx.x] = s1;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) { r0[threadIdx.x] += r0[threadIdx.x + o]; r1[threadIdx.x] += r1[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = r0[0]; part[2 * blockIdx.x + 1] = r1[0]; }
}
__global__ void fold_pairs_kernel(int nb, const double* __restrict__ part, double* __restrict__ out) {
  if (threadIdx.x == 0) {
    double s0 = 0, s1 = 0;
    for (int b = 0; b < nb; ++b) { s0 += part[2 * b]; s1 += part[2 * b + 1]; }
    out[0] = s0;
    out[1] = s1;
  }
}
// sum_ij (delta_j u_i)^2 over all cells (forward differences, FP64): the
// discrete dissipation of the viscous term -visc delta_j(delta_j u_i +
// delta_i u_j) of `stress` (src/N.jl:106-118) for a divergence-free u.
template <typename T>
__global__ void gradsq_partial_kernel(int n, const T* __restrict__ u, double* __restrict__ part) {
  __shared__ double r0[256];
  const long long N = (long long)n * n * n;
  double s = 0;
  const IdxDiv dn(n);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
    const long long r = dn.div(g);
    int x = (int)(g - r * n);
    int z = (int)dn.div(r);
    int y = (int)(r - (long long)z * n);
    long long nb[3] = {g - x + wrap_up(x, n), ((long long)z * n + wrap_up(y, n)) * n + x,
                       ((long long)wrap_up(z, n) * n + y) * n + x};
    for (int i = 0; i < 3; ++i) {
      double c = (double)u[i * N + g];
      for (int j = 0; j < 3; ++j) {
        double d = (double)u[i * N + nb[j]] - c;
        s += d * d;
      }
    }
  }
  r0[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) r0[threadIdx.x] += r0[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = r0[0]; part[2 * blockIdx.x + 1] = 0.0; }
}
template <typename T>
cudaError_t launch_gradsq(int n, const T* u, double* part, double* out, cudaStream_t st) {
  gradsq_partial_kernel<T><<<RED_BLOCKS, 256, 0, st>>>(n, u, part);
  fold_pairs_kernel<<<1, 32, 0, st>>>(RED_BLOCKS, part, out);
  return cudaGetLastError();
}
template cudaError_t launch_gradsq<double>(int, const double*, double*, double*, cudaStream_t);
template cudaError_t launch_gradsq<float>(int, const float*, double*, double*, cudaStream_t);

template <typename T>
cudaError_t launch_sqdiff(long long count, const T* a, const T* b, double* part, double* out, cudaStream_t st) {
  sqdiff_partial_kernel<T><<<RED_BLOCKS, 256, 0, st>>>(count, a, b, part);
  fold_pairs_kernel<<<1, 32, 0, st>>>(RED_BLOCKS, part, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Shell histogram on the rfft half grid: e = scale * sum_c |F_c|^2 / 2 with
// the conjugate weight 2 for kx = 1..n/2-1 (src/N.jl:443, 534-543), binned by
// shell k = isqrt(kx^2+ky^2+kz^2) (src/N.jl:375-392).  Lanes of a warp add in
// lane order into the warp's shared row, warps fold in order, blocks fold in
// order: bit-reproducible.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int isqrt_ll(long long v) {
  long long r = (long long)sqrt((double)v);
  while (r * r > v) --r;
  while ((r + 1) * (r + 1) <= v) ++r;
  return (int)r;
}
__device__ __forceinline__ int wavenum(int i, int n) { return i <= (n - 1) / 2 ? i : i - n; }

template <typename T>
__global__ void shell_partial_kernel(int n, int P, int ncomp, const cplx<T>* __restrict__ spec, long long cstride,
                                     double scale, int nshell, double* __restrict__ part) {
  extern __shared__ double acc[];  // [8][nshell]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < 8 * nshell; i += blockDim.x) acc[i] = 0.0;
  __syncthreads();
  const int nkx = n / 2 + 1;
  const long long total = (long long)n * n * nkx;
  double* my = acc + warp * nshell;
  for (long long base = (long long)blockIdx.x * blockDim.x + warp * 32; base < total;
       base += (long long)gridDim.x * blockDim.x) {
    long long g = base + lane;
    int sh = -1;
    double e = 0.0;
    if (g < total) {
      long long r = g / nkx;
      int kx = (int)(g - r * nkx);
      int kz = (int)(r / n);
      int ky = (int)(r - (long long)kz * n);
      long long off = r * P + kx;
      for (int c = 0; c < ncomp; ++c) {
        cplx<T> v = spec[c * cstride + off];
        e += ((double)v.x * v.x + (double)v.y * v.y);
      }
      double w = (kx >= 1 && kx <= n / 2 - 1) ? 2.0 : 1.0;
      e *= 0.5 * scale * w;
      int a = wavenum(ky, n), b = wavenum(kz, n);
      long long kk = (long long)kx * kx + (long long)a * a + (long long)b * b;
      sh = isqrt_ll(kk);
      if (sh >= nshell) sh = -1;
    }
    for (int l = 0; l < 32; ++l) {
      if (lane == l && sh >= 0) my[sh] += e;
      __syncwarp();
    }
  }
  __syncthreads();
  for (int s = threadIdx.x; s < nshell; s += blockDim.x) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += acc[w * nshell + s];
    part[(long long)blockIdx.x * nshell + s] = t;
  }
}
__global__ void shell_fold_kernel(int nb, int nshell, const double* __restrict__ part, double* __restrict__ out) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nshell; s += gridDim.x * blockDim.x) {
    double t = 0.0;
    for (int b = 0; b < nb; ++b) t += part[(long long)b * nshell + s];
    out[s] = t;
  }
}
template <typename T>
cudaError_t launch_shell_energy(int n, int P, int ncomp, const cplx<T>* spec, long long cstride, double scale,
                                int nshell, double* part, int nblocks, double* out, cudaStream_t st) {
  size_t sh = (size_t)8 * nshell * sizeof(double);
  shell_partial_kernel<T><<<nblocks, 256, sh, st>>>(n, P, ncomp, spec, cstride, scale, nshell, part);
  shell_fold_kernel<<<(nshell + 255) / 256, 256, 0, st>>>(nblocks, nshell, part, out);
  return cudaGetLastError();
}

cudaError_t configure_fields() {
  cudaError_t e = cudaFuncSetAttribute(shell_partial_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 80 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(shell_partial_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 80 * 1024);
  return e;
}

// Multiply every mode of shell k (k <= kdiag) by factor[k] (src/N.jl:441-449).
template <typename T>
__global__ void shell_scale_kernel(int n, int P, int ncomp, cplx<T>* __restrict__ spec, long long cstride,
                                   int nshell, const double* __restrict__ factor) {
  const int nkx = n / 2 + 1;
  const long long total = (long long)n * n * nkx;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total; g += (long long)gridDim.x * blockDim.x) {
    long long r = g / nkx;
    int kx = (int)(g - r * nkx);
    int kz = (int)(r / n);
    int ky = (int)(r - (long long)kz * n);
    int a = wavenum(ky, n), b = wavenum(kz, n);
    long long kk = (long long)kx * kx + (long long)a * a + (long long)b * b;
    int sh = isqrt_ll(kk);
    if (sh >= nshell) continue;
    double f = factor[sh];
    long long off = r * P + kx;
    for (int c = 0; c < ncomp; ++c) {
      cplx<T> v = spec[c * cstride + off];
      v.x = (T)((double)v.x * f);
      v.y = (T)((double)v.y * f);
      spec[c * cstride + off] = v;
    }
  }
}
template <typename T>
cudaError_t launch_shell_scale(int n, int P, int ncomp, cplx<T>* spec, long long cstride, int nshell,
                               const double* factor, cudaStream_t st) {
  long long total = (long long)n * n * (n / 2 + 1);
  shell_scale_kernel<T><<<grid_for(total), 256, 0, st>>>(n, P, ncomp, spec, cstride, nshell, factor);
  return cudaGetLastError();
}

// Host-side shell factors sqrt(E0/Eshell) with E0 = energy * profile(k) / sum
// of profiles (src/N.jl:436-451); computed on the device to avoid a sync.
// Shell profile: `peak_profile` k^4 exp(-2 (k/k0)^2) (src/N.jl:366) or the
// power law (k > 0) k^p of `dnsaid_project` (src/N.jl:1245).
__device__ __forceinline__ double shell_profile(int profile, double param, int k) {
  if (profile == 1) return k > 0 ? pow((double)k, param) : 0.0;
  const double q = k / param;
  return (double)k * k * (double)k * k * exp(-2.0 * q * q);
}

// One CTA: the profiles in parallel, their total in shell order by one thread.
__global__ void shell_factor_kernel(int nshell, int profile, double param, double energy,
                                    const double* __restrict__ eshell, double* __restrict__ factor) {
  extern __shared__ double sprof[];  // nshell profiles, then the total
  for (int k = threadIdx.x; k < nshell; k += blockDim.x) sprof[k] = shell_profile(profile, param, k);
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int k = 0; k < nshell; ++k) tot += sprof[k];
    sprof[nshell] = tot;
  }
  __syncthreads();
  const double tot = sprof[nshell];
  for (int k = threadIdx.x; k < nshell; k += blockDim.x) {
    const double e0 = energy * sprof[k] / tot;
    const double es = eshell[k];
    factor[k] = es > 0 ? sqrt(e0 / es) : 1.0;
  }
}
cudaError_t launch_shell_factor(int nshell, int profile, double param, double energy, const double* eshell,
                                double* factor, cudaStream_t st) {
  shell_factor_kernel<<<1, 256, (size_t)(nshell + 1) * sizeof(double), st>>>(nshell, profile, param, energy, eshell,
                                                                             factor);
  return cudaGetLastError();
}

// dense (n^3) <- pitched real view (row pitch `pitch` words), scaled
template <typename T>
__global__ void unpitch_kernel(int n, const T* __restrict__ src, int pitch, T* __restrict__ dst, T scale) {
  long long N = (long long)n * n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    long long row = i / n;
    int x = (int)(i - row * n);
    dst[i] = src[row * pitch + x] * scale;
  }
}
template <typename T>
cudaError_t launch_unpitch(int n, const T* src, int pitch, T* dst, T scale, cudaStream_t st) {
  long long N = (long long)n * n * n;
  unpitch_kernel<T><<<grid_for(N), 256, 0, st>>>(n, src, pitch, dst, scale);
  return cudaGetLastError();
}

// precision conversion
template <typename A, typename B>
__global__ void convert_kernel(long long count, const A* __restrict__ a, B* __restrict__ b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    b[i] = (B)a[i];
}
template <typename A, typename B>
cudaError_t launch_convert(long long count, const A* a, B* b, cudaStream_t st) {
  convert_kernel<A, B><<<grid_for(count), 256, 0, st>>>(count, a, b);
  return cudaGetLastError();
}

#define INST(T)                                                                                                 \
  template cudaError_t launch_rk_stage_sums<T>(int, int, T, const T*, const T*, int, const T*, T*, T*, int,     \
                                               const double*, T*, T*, cudaStream_t);                           \
  template cudaError_t launch_rk_stage<T>(int, T, T*, const T*, int, const T*, T*, T*, int, const double*,      \
                                          cudaStream_t, const SlotBatch&, int, bool, bool, double);                                                        \
  template cudaError_t launch_axpy<T>(long long, T*, const T*, T, cudaStream_t);                                \
  template cudaError_t launch_normals<T>(long long, unsigned long long, T*, cudaStream_t);                      \
  template cudaError_t launch_sqdiff<T>(long long, const T*, const T*, double*, double*, cudaStream_t);         \
  template cudaError_t launch_shell_energy<T>(int, int, int, const cplx<T>*, long long, double, int, double*,   \
                                              int, double*, cudaStream_t);                                      \
  template cudaError_t launch_shell_scale<T>(int, int, int, cplx<T>*, long long, int, const double*,            \
                                             cudaStream_t);                                                     \
  template cudaError_t launch_unpitch<T>(int, const T*, int, T*, T, cudaStream_t);
INST(double)
INST(float)
#undef INST
template cudaError_t launch_convert<double, float>(long long, const double*, float*, cudaStream_t);
template cudaError_t launch_convert<float, double>(long long, const float*, double*, cudaStream_t);
template cudaError_t launch_convert<double, double>(long long, const double*, double*, cudaStream_t);

}  // namespace exc
