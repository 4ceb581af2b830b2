// Discrete filters and coarse-graining (src/N.jl:592-698, 999-1135): the
// separable filter-and-sample operator of `lazycoarsegrain(lazyfilter(.))`
// materialised on the LES grid, for velocities (volume or face average) and
// for the closure fluxes r = sigma(u) + p I evaluated on the fly.
#include <vector>

#include "internal.cuh"
#include "filter.cuh"

namespace exc {

// Coarse sample `ib` along one axis = sum_t w_t f[(c*ib + o_t) mod n].
// Odd c reproduces the reference's sample point c*Ib - !stag*div(c,2)
// (1-based, src/N.jl:686-698) and its `tophat`; even c (the reference asserts
// odd ratios, src/N.jl:593) averages the piecewise-constant fine field over
// the coarse cell extent: trapezoid [1/2,1,..,1,1/2]/c on a face axis, box of
// the c fine cells on a centre axis, mean of the two straddling fine centres
// for a centre point sample.  An optional odd Gaussian FDelta is convolved in
// (`get_kernels`, src/N.jl:1008-1020).
Taps1D build_taps(int c, bool stag, bool point, const double* fdelta, int nfd) {
  std::vector<int> o;
  std::vector<double> w;
  int a = c / 2;
  if (stag) {
    int base = c - 1;
    if (point) { o = {base}; w = {1.0}; }
    else if (c % 2 == 1) { for (int k = -a; k <= a; ++k) { o.push_back(base + k); w.push_back(1.0 / c); } }
    else {
      for (int k = -a; k <= a; ++k) { o.push_back(base + k); w.push_back(1.0 / c); }
      w.front() = 0.5 / c;
      w.back() = 0.5 / c;
    }
  } else {
    if (point) {
      if (c % 2 == 1) { o = {a}; w = {1.0}; }
      else { o = {a - 1, a}; w = {0.5, 0.5}; }
    } else {
      for (int k = 0; k < c; ++k) { o.push_back(k); w.push_back(1.0 / c); }
    }
  }
  if (fdelta && nfd > 1) {
    int R = nfd / 2;
    int lo = o.front() - R, hi = o.back() + R;
    std::vector<double> acc(hi - lo + 1, 0.0);
    for (size_t t = 0; t < o.size(); ++t)
      for (int r = -R; r <= R; ++r) acc[o[t] + r - lo] += w[t] * fdelta[r + R];
    o.clear();
    w.clear();
    for (int k = lo; k <= hi; ++k) { o.push_back(k); w.push_back(acc[k - lo]); }
  }
  Taps1D t{};
  t.cnt = (int)o.size();
  for (int k = 0; k < t.cnt && k < MAX_TAPS; ++k) { t.off[k] = o[k]; t.w[k] = w[k]; }
  if (t.cnt > MAX_TAPS) t.cnt = -1;  // rejected by callers
  return t;
}

// ---------------------------------------------------------------------------
// Sources
// ---------------------------------------------------------------------------
template <typename T>
struct FieldSrc {
  const T* f;
  int n;
  __device__ __forceinline__ double operator()(int x, int y, int z) const {
    return (double)f[((long long)z * n + y) * n + x];
  }
};

// Launch the filter of one flux component with compile-time (i, j).
template <typename T, int I, int J>
static void launch_flux_filter(const T* u, const T* p, int n, T inv_h, T visc, int c, const Taps3& taps, T* out,
                               long long M, cudaStream_t st);

template <typename T>
static void launch_flux_filter_rt(int i, int j, const T* u, const T* p, int n, T inv_h, T visc, int c,
                                  const Taps3& taps, T* out, long long M, cudaStream_t st) {
#define EXC_FLUX(I, J) \
  if (i == I && j == J) return launch_flux_filter<T, I, J>(u, p, n, inv_h, visc, c, taps, out, M, st);
  EXC_FLUX(0, 0) EXC_FLUX(0, 1) EXC_FLUX(0, 2)
  EXC_FLUX(1, 0) EXC_FLUX(1, 1) EXC_FLUX(1, 2)
  EXC_FLUX(2, 0) EXC_FLUX(2, 1) EXC_FLUX(2, 2)
#undef EXC_FLUX
}

// One thread per coarse cell: separable sum over the three tap lists.
template <typename T, typename Src>
__global__ void filter_kernel(Src src, int n, int c, Taps3 taps, T* __restrict__ out) {
  const int m = n / c;
  const long long M = (long long)m * m * m;
  const IdxDiv dm(m);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < M; g += (long long)gridDim.x * blockDim.x) {
    const long long r = dm.div(g);
    int ix = (int)(g - r * m);
    int iz = (int)dm.div(r);
    int iy = (int)(r - (long long)iz * m);
    double acc = 0.0;
    // tap offsets stay within (-n, 2n): wrap by comparison
    auto wrapc = [n](int q) { return q < 0 ? q + n : (q >= n ? q - n : q); };
    for (int tz = 0; tz < taps.a[2].cnt; ++tz) {
      const int z = wrapc(c * iz + taps.a[2].off[tz]);
      double az = 0.0;
      for (int ty = 0; ty < taps.a[1].cnt; ++ty) {
        const int y = wrapc(c * iy + taps.a[1].off[ty]);
        double ay = 0.0;
        for (int tx = 0; tx < taps.a[0].cnt; ++tx) {
          const int x = wrapc(c * ix + taps.a[0].off[tx]);
          ay += taps.a[0].w[tx] * src(x, y, z);
        }
        az += taps.a[1].w[ty] * ay;
      }
      acc += taps.a[2].w[tz] * az;
    }
    out[g] = (T)acc;
  }
}

static inline int grid_for(long long M) {
  long long b = (M + 255) / 256;
  return (int)(b < 152LL * 32 ? b : 152LL * 32);
}

// Filter of one closure-flux component r_ij = sigma_ij(u) + delta_ij p with
// compile-time (I, J).  The flux splits into an advective product and a
// viscous difference,
//   r = a b / 4 - (visc / h) d + delta_ij p,
//   a = u_i(x + o e_j) + u_i(x + (o - 1) e_j),  b = the same for u_j along i,
//   d = [u_i(x + o e_j) - u_i(x + (o - 1) e_j)] + [the same for u_j along i],
// o = (i != j); the taps sum a b, d and p separately and the three sums are
// combined once per coarse cell.  That is 8 FP64 operations per fine cell off
// the diagonal and 5 on it (the diagonal has a = b and d = 2 d_i), against 12
// for summing r itself; the results differ from summing r only by rounding.
template <typename T, int I, int J, bool P>
__global__ void __launch_bounds__(256, 2) flux_filter_kernel(const T* __restrict__ u, const T* __restrict__ p, int n,
                                                          int c, double vh, Taps3 taps, T* __restrict__ out) {
  const int m = n / c;
  const long long M = (long long)m * m * m, N = (long long)n * n * n;
  const IdxDiv dm(m);
  const T* __restrict__ ui = u + I * N;
  const T* __restrict__ uj = u + J * N;
  constexpr int o = (I != J);
  auto wrapc = [n](int q) { return q < 0 ? q + n : (q >= n ? q - n : q); };
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < M; g += (long long)gridDim.x * blockDim.x) {
    const long long r = dm.div(g);
    const int ix = (int)(g - r * m);
    const int iz = (int)dm.div(r);
    const int iy = (int)(r - (long long)iz * m);
    double sab = 0.0, sd = 0.0, sp = 0.0;
    for (int tz = 0; tz < taps.a[2].cnt; ++tz) {
      const int z = wrapc(c * iz + taps.a[2].off[tz]);
      double zab = 0.0, zd = 0.0, zp = 0.0;
      for (int ty = 0; ty < taps.a[1].cnt; ++ty) {
        const int y = wrapc(c * iy + taps.a[1].off[ty]);
        // the rows of u_i and u_j at (y, z) and their neighbours along j and i
        auto row = [&](int axis, int s) -> long long {
          const int yy = axis == 1 ? wrapc(y + s) : y, zz = axis == 2 ? wrapc(z + s) : z;
          return ((long long)zz * n + yy) * n;
        };
        const long long ri_r = row(J, o), ri_l = row(J, o - 1);
        const long long rj_r = row(I, o), rj_l = row(I, o - 1);
        const long long rc = ((long long)z * n + y) * n;
        double yab = 0.0, yd = 0.0, yp = 0.0;
        for (int tx = 0; tx < taps.a[0].cnt; ++tx) {
          const int x = wrapc(c * ix + taps.a[0].off[tx]);
          const int xi_r = J == 0 ? wrapc(x + o) : x, xi_l = J == 0 ? wrapc(x + o - 1) : x;
          const double w = taps.a[0].w[tx];
          const T air = ui[ri_r + xi_r], ail = ui[ri_l + xi_l];
          if constexpr (I == J) {
            const T a = air + ail, d = air - ail;
            yab = fma(w, (double)(a * a), yab);
            yd = fma(w, (double)d, yd);
          } else {
            const int xj_r = I == 0 ? wrapc(x + o) : x, xj_l = I == 0 ? wrapc(x + o - 1) : x;
            const T ajr = uj[rj_r + xj_r], ajl = uj[rj_l + xj_l];
            const T a = air + ail, b = ajr + ajl, d = (air + ajr) - (ail + ajl);
            yab = fma(w, (double)(a * b), yab);
            yd = fma(w, (double)d, yd);
          }
          if constexpr (P) yp = fma(w, (double)p[rc + x], yp);
        }
        const double wy = taps.a[1].w[ty];
        zab = fma(wy, yab, zab);
        zd = fma(wy, yd, zd);
        if constexpr (P) zp = fma(wy, yp, zp);
      }
      const double wz = taps.a[2].w[tz];
      sab = fma(wz, zab, sab);
      sd = fma(wz, zd, sd);
      if constexpr (P) sp = fma(wz, zp, sp);
    }
    // the diagonal's d is half the viscous difference
    const double k = I == J ? 2.0 * vh : vh;
    out[g] = (T)(fma(0.25, sab, -k * sd) + sp);
  }
}

template <typename T, int I, int J>
static void launch_flux_filter(const T* u, const T* p, int n, T inv_h, T visc, int c, const Taps3& taps, T* out,
                               long long M, cudaStream_t st) {
  const double vh = (double)visc * (double)inv_h;
  if (I == J && p)
    flux_filter_kernel<T, I, J, true><<<grid_for(M), 256, 0, st>>>(u, p, n, c, vh, taps, out);
  else
    flux_filter_kernel<T, I, J, false><<<grid_for(M), 256, 0, st>>>(u, p, n, c, vh, taps, out);
}

int make_taps3(int c, const bool stag[3], const bool point[3], const double* fdelta, int nfd, Taps3* out) {
  for (int d = 0; d < 3; ++d) {
    out->a[d] = build_taps(c, stag[d], point[d], fdelta, nfd);
    if (out->a[d].cnt < 0) { set_last_error("filter stencil longer than MAX_TAPS"); return EXC_ERR_ARG; }
  }
  return EXC_OK;
}

template <typename T>
int filter_vector(int n, int c, int kind, const double* fdelta, int nfd, const T* u, T* ub, cudaStream_t st) {
  const long long N = (long long)n * n * n;
  const int m = n / c;
  const long long M = (long long)m * m * m;
  for (int i = 0; i < 3; ++i) {
    bool stag[3] = {i == 0, i == 1, i == 2};
    bool point[3] = {false, false, false};
    if (kind == EXC_FILTER_FACE) point[i] = true;
    Taps3 taps;
    int rc = make_taps3(c, stag, point, fdelta, nfd, &taps);
    if (rc) return rc;
    FieldSrc<T> src{u + i * N, n};
    filter_kernel<T><<<grid_for(M), 256, 0, st>>>(src, n, c, taps, ub + i * M);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

// rDHi: component (i, j) = r_ij filtered with GDHi[j] (point along j, volume
// elsewhere), sampled at the LES centre (i == j) or edge (i, j)
// (src/N.jl:1038-1073); output order s11,s21,s31,s12,... (src/N.jl:181).
template <typename T>
int closure_flux(int n, int c, double l, double visc, const double* fdelta, int nfd, const T* u, const T* p,
                 T* r9, cudaStream_t st) {
  const int m = n / c;
  const long long M = (long long)m * m * m;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) {
      bool stag[3], point[3];
      for (int d = 0; d < 3; ++d) {
        stag[d] = (i != j) && (d == i || d == j);
        point[d] = (d == j);
      }
      Taps3 taps;
      int rc = make_taps3(c, stag, point, fdelta, nfd, &taps);
      if (rc) return rc;
      launch_flux_filter_rt<T>(i, j, u, p, n, (T)(1.0 / (l / n)), (T)visc, c, taps, r9 + (long long)(3 * j + i) * M, M,
                               st);
    }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

// Surface-filtered flux of the paper's face-average driver (dns_aid_surface,
// src/NavierStokes.jl:368-369): component (i, j) = r_ij point-sampled along i
// (the face of the velocity u_i it updates) and boxed along the other two
// axes (Turbulox's surfacefilter!(firu, ru, c, true)); with `line`, the
// off-diagonal components are point-sampled along j too and boxed along the
// third axis only (linefilter!), the diagonal unchanged.  Sampled at the LES
// centre (i == j) or edge (i, j); order s11,s21,s31,s12,... like rDHi.
template <typename T>
int surface_flux(int n, int c, double l, double visc, const double* fdelta, int nfd, const T* u, const T* p,
                 T* r9, bool line, cudaStream_t st) {
  const int m = n / c;
  const long long M = (long long)m * m * m;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) {
      bool stag[3], point[3];
      for (int d = 0; d < 3; ++d) {
        stag[d] = (i != j) && (d == i || d == j);
        point[d] = (d == i) || (line && d == j);
      }
      Taps3 taps;
      int rc = make_taps3(c, stag, point, fdelta, nfd, &taps);
      if (rc) return rc;
      launch_flux_filter_rt<T>(i, j, u, p, n, (T)(1.0 / (l / n)), (T)visc, c, taps, r9 + (long long)(3 * j + i) * M, M,
                               st);
    }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

// sigmaDH (src/N.jl:1088-1115): volume filter GDH of each stress component,
// sampled at LES centres/edges; order s11,s22,s33,s12,s23,s31.  With p the
// total flux r = sigma + p I is filtered (the paper driver's volume-filtered
// flux, src/NavierStokes.jl:199).
template <typename T>
int filtered_stress(int n, int c, double l, double visc, const double* fdelta, int nfd, const T* u, T* s6,
                    cudaStream_t st, const T* p) {
  const int m = n / c;
  const long long M = (long long)m * m * m;
  const int comps[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {2, 0}};
  for (int k = 0; k < 6; ++k) {
    int i = comps[k][0], j = comps[k][1];
    bool stag[3], point[3] = {false, false, false};
    for (int d = 0; d < 3; ++d) stag[d] = (i != j) && (d == i || d == j);
    Taps3 taps;
    int rc = make_taps3(c, stag, point, fdelta, nfd, &taps);
    if (rc) return rc;
    launch_flux_filter_rt<T>(i, j, u, p, n, (T)(1.0 / (l / n)), (T)visc, c, taps, s6 + (long long)k * M,
                             M, st);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

// ---------------------------------------------------------------------------
// Two-stage box filter of a vector field (volume or face average without a
// Gaussian), the form the case stepper uses every stage.  Stage 1 reads each
// fine value once, coalesced: for component i it sums the c x c fine cells of
// each coarse transverse cell at every fine position along axis i,
//   tb_0[(Jz m + Jy) n + x], tb_1[(Jz n + y) m + Jx], tb_2[(z m + Jy) m + Jx].
// Stage 2 applies the own-axis taps of build_taps (trapezoid/box or face
// point sample) and the transverse weight 1/c^2.  Both stages sum in a fixed
// order, so the result is bit-reproducible.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void tb_kernel(const T* __restrict__ f3, int n, int c, T* __restrict__ tb3) {
  const int comp = blockIdx.y;
  const int m = n / c;
  const long long N = (long long)n * n * n;
  const long long Mt = (long long)n * m * m;
  const T* __restrict__ f = f3 + comp * N;
  T* __restrict__ tb = tb3 + comp * Mt;
  const IdxDiv dn(n), dm(m);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < Mt; g += (long long)gridDim.x * blockDim.x) {
    T acc = (T)0;
    if (comp == 0) {
      const long long r = dn.div(g);
      const int x = (int)(g - r * n);
      const int Jz = (int)dm.div(r), Jy = (int)(r - (long long)Jz * m);
      const T* p = f + ((long long)(c * Jz) * n + c * Jy) * n + x;
      for (int dz = 0; dz < c; ++dz)
        for (int dy = 0; dy < c; ++dy) acc += p[((long long)dz * n + dy) * n];
    } else if (comp == 1) {
      const long long r = dm.div(g);
      const int Jx = (int)(g - r * m);
      const int Jz = (int)dn.div(r), y = (int)(r - (long long)Jz * n);
      const T* p = f + ((long long)(c * Jz) * n + y) * n + c * Jx;
      for (int dz = 0; dz < c; ++dz)
        for (int dx = 0; dx < c; ++dx) acc += p[(long long)dz * n * n + dx];
    } else {
      const long long r = dm.div(g);
      const int Jx = (int)(g - r * m);
      const int z = (int)dm.div(r), Jy = (int)(r - (long long)z * m);
      const T* p = f + ((long long)z * n + c * Jy) * n + c * Jx;
      for (int dy = 0; dy < c; ++dy)
        for (int dx = 0; dx < c; ++dx) acc += p[(long long)dy * n + dx];
    }
    tb[g] = acc;
  }
}

template <typename T>
__global__ void oa_kernel(const T* __restrict__ tb3, int n, int c, Taps1D taps, double scale, T* __restrict__ out3) {
  const int comp = blockIdx.y;
  const int m = n / c;
  const long long M = (long long)m * m * m;
  const long long Mt = (long long)n * m * m;
  const T* __restrict__ tb = tb3 + comp * Mt;
  const IdxDiv dm(m);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < M; g += (long long)gridDim.x * blockDim.x) {
    const long long r = dm.div(g);
    const int ix = (int)(g - r * m);
    const int iz = (int)dm.div(r), iy = (int)(r - (long long)iz * m);
    const int own = comp == 0 ? ix : (comp == 1 ? iy : iz);
    // accumulate in the field's word type (FP32 form: no FP64-pipe work)
    T acc = (T)0;
    for (int t = 0; t < taps.cnt; ++t) {
      int fi = c * own + taps.off[t];
      fi = fi >= n ? fi - n : (fi < 0 ? fi + n : fi);
      long long idx;
      if (comp == 0) idx = ((long long)iz * m + iy) * n + fi;
      else if (comp == 1) idx = ((long long)iz * n + fi) * m + ix;
      else idx = ((long long)fi * m + iy) * m + ix;
      acc += (T)taps.w[t] * tb[idx];
    }
    out3[comp * M + g] = acc * (T)scale;
  }
}

// Transverse sums of ratio cf * r from those of ratio cf: an r x r block of
// the cf-sums (block order a, b; each cf-sum in its own fixed order), so a
// case with several LES reads the fine field once per filtered quantity.
template <typename T>
__global__ void tb_coarsen_kernel(const T* __restrict__ tf3, int n, int cf, int r, T* __restrict__ tt3) {
  const int comp = blockIdx.y;
  const int mf = n / cf, mt = mf / r;
  const long long Mtf = (long long)n * mf * mf;
  const long long Mtt = (long long)n * mt * mt;
  const T* __restrict__ tf = tf3 + comp * Mtf;
  T* __restrict__ tt = tt3 + comp * Mtt;
  const IdxDiv dn(n), dmt(mt);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < Mtt; g += (long long)gridDim.x * blockDim.x) {
    T acc = (T)0;
    if (comp == 0) {  // [(Kz mt + Ky) n + x]
      const long long q = dn.div(g);
      const int x = (int)(g - q * n);
      const int Kz = (int)dmt.div(q), Ky = (int)(q - (long long)Kz * mt);
      for (int a = 0; a < r; ++a)
        for (int b = 0; b < r; ++b) acc += tf[((long long)(r * Kz + a) * mf + r * Ky + b) * n + x];
    } else if (comp == 1) {  // [(Kz n + y) mt + Kx]
      const long long q = dmt.div(g);
      const int Kx = (int)(g - q * mt);
      const int Kz = (int)dn.div(q), y = (int)(q - (long long)Kz * n);
      for (int a = 0; a < r; ++a)
        for (int b = 0; b < r; ++b) acc += tf[((long long)(r * Kz + a) * n + y) * mf + r * Kx + b];
    } else {  // [(z mt + Ky) mt + Kx]
      const long long q = dmt.div(g);
      const int Kx = (int)(g - q * mt);
      const int z = (int)dmt.div(q), Ky = (int)(q - (long long)z * mt);
      for (int a = 0; a < r; ++a)
        for (int b = 0; b < r; ++b) acc += tf[((long long)z * mf + r * Ky + a) * mf + r * Kx + b];
    }
    tt[g] = acc;
  }
}

template <typename T>
cudaError_t box_tb(int n, int c, const T* u, T* tb, cudaStream_t st) {
  const int m = n / c;
  const long long Mt = (long long)n * m * m;
  tb_kernel<T><<<dim3(grid_for(Mt), 3), 256, 0, st>>>(u, n, c, tb);
  return cudaGetLastError();
}

template <typename T>
cudaError_t box_tb_coarsen(int n, int cf, int ct, const T* tbf, T* tbt, cudaStream_t st) {
  const int mt = n / ct;
  const long long Mtt = (long long)n * mt * mt;
  tb_coarsen_kernel<T><<<dim3(grid_for(Mtt), 3), 256, 0, st>>>(tbf, n, cf, ct / cf, tbt);
  return cudaGetLastError();
}

template <typename T>
cudaError_t box_oa(int n, int c, int kind, const T* tb, T* ub, cudaStream_t st) {
  const int m = n / c;
  const long long M = (long long)m * m * m;
  Taps1D taps = build_taps(c, true, kind == EXC_FILTER_FACE, nullptr, 0);
  // the transverse box weight 1/c is applied once per axis here; the own-axis
  // taps already carry their 1/c
  const double scale = 1.0 / ((double)c * c);
  oa_kernel<T><<<dim3(grid_for(M), 3), 256, 0, st>>>(tb, n, c, taps, scale, ub);
  return cudaGetLastError();
}

template <typename T>
cudaError_t filter_vector_box(int n, int c, int kind, const T* u, T* ub, T* tb, cudaStream_t st) {
  cudaError_t e = box_tb<T>(n, c, u, tb, st);
  if (e == cudaSuccess) e = box_oa<T>(n, c, kind, tb, ub, st);
  return e;
}

// Stress of the fine-grid filtered velocity, uf = lazyfilter(u, GDH) on the
// DNS grid (centred box of odd width c, composed with FDelta), at fine cell
// (x, y, z): the field that `step_ΔHπ_classic!` (src/N.jl:1137-1162) samples
// at the LES centres and edges.  Each uf value is evaluated on the fly.
// sigma_ij of the fine-filtered velocity GDH u at fine cell (x, y, z); the
// components (I, J) are compile-time and every index wraps by comparison (tap
// offsets stay within (-n, 2n)).
template <typename T, int I, int J>
struct FineFilteredStressSrc {
  const T* u;
  int n;
  T inv_h, visc;
  Taps1D ft;  // centred fine-filter taps (same along every axis)
  __device__ __forceinline__ int wrap(int q) const { return q < 0 ? q + n : (q >= n ? q - n : q); }
  __device__ __forceinline__ double uf(int comp, int x, int y, int z) const {
    const long long N = (long long)n * n * n;
    const T* f = u + comp * N;
    double acc = 0.0;
    for (int tz = 0; tz < ft.cnt; ++tz) {
      const int zz = wrap(z + ft.off[tz]);
      double az = 0.0;
      for (int ty = 0; ty < ft.cnt; ++ty) {
        const T* row = f + ((long long)zz * n + wrap(y + ft.off[ty])) * n;
        double ay = 0.0;
        for (int tx = 0; tx < ft.cnt; ++tx) ay += ft.w[tx] * (double)row[wrap(x + ft.off[tx])];
        az += ft.w[ty] * ay;
      }
      acc += ft.w[tz] * az;
    }
    return acc;
  }
  template <int A>
  __device__ __forceinline__ double uf_at(int comp, int x, int y, int z, int s) const {
    if (A == 0) x = wrap(x + s);
    if (A == 1) y = wrap(y + s);
    if (A == 2) z = wrap(z + s);
    return uf(comp, x, y, z);
  }
  __device__ __forceinline__ double operator()(int x, int y, int z) const {
    constexpr int off = (I != J);
    const double uir = uf_at<J>(I, x, y, z, off), uil = uf_at<J>(I, x, y, z, off - 1);
    // on the diagonal the two pairs are the same filtered values
    const double ujr = I == J ? uir : uf_at<I>(J, x, y, z, off);
    const double ujl = I == J ? uil : uf_at<I>(J, x, y, z, off - 1);
    const double etaj_ui = (uir + uil) / 2, etai_uj = (ujr + ujl) / 2;
    const double dj_ui = (uir - uil) * (double)inv_h, di_uj = (ujr - ujl) * (double)inv_h;
    return etaj_ui * etai_uj - (double)visc * (dj_ui + di_uj);
  }
};

template <typename T, int I, int J>
static void launch_classic(const T* u, int n, T inv_h, T visc, const Taps1D& ft, int c, const Taps3& taps, T* out,
                           long long M, cudaStream_t st) {
  FineFilteredStressSrc<T, I, J> src{u, n, inv_h, visc, ft};
  filter_kernel<T><<<grid_for(M), 256, 0, st>>>(src, n, c, taps, out);
}

// sigma2 of `step_ΔHπ_classic!`: `lazytensorcoarsegrain(g_les,
// stresstensor(lazyfilter(u, GDH)))` (src/N.jl:1117-1135, 1143-1145); order
// s11, s22, s33, s12, s23, s31.  Odd ratios only (the reference's top hat).
template <typename T>
int classic_stress(int n, int c, double l, double visc, const double* fdelta, int nfd, const T* u, T* s6,
                   cudaStream_t st) {
  if (c % 2 == 0) { set_last_error("the classic closure's fine-grid filter needs an odd ratio"); return EXC_ERR_RATIO; }
  const int m = n / c;
  const long long M = (long long)m * m * m;
  Taps1D ft = build_taps(c, false, false, fdelta, nfd);
  if (ft.cnt < 0) { set_last_error("filter stencil longer than MAX_TAPS"); return EXC_ERR_ARG; }
  for (int k = 0; k < ft.cnt; ++k) ft.off[k] -= c / 2;  // centre the box on the fine cell
  const int comps[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {2, 0}};
  for (int k = 0; k < 6; ++k) {
    const int i = comps[k][0], j = comps[k][1];
    bool stag[3], point[3] = {true, true, true};
    for (int d = 0; d < 3; ++d) stag[d] = (i != j) && (d == i || d == j);
    Taps3 taps;
    int rc = make_taps3(c, stag, point, nullptr, 0, &taps);
    if (rc) return rc;
    const T inv_h = (T)(1.0 / (l / n));
    T* out = s6 + (long long)k * M;
#define EXC_CLASSIC(I, J) \
  if (i == I && j == J) launch_classic<T, I, J>(u, n, inv_h, (T)visc, ft, c, taps, out, M, st);
    EXC_CLASSIC(0, 0) EXC_CLASSIC(1, 1) EXC_CLASSIC(2, 2) EXC_CLASSIC(0, 1) EXC_CLASSIC(1, 2) EXC_CLASSIC(2, 0)
#undef EXC_CLASSIC
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

#define INST(T)                                                                                          \
  template int classic_stress<T>(int, int, double, double, const double*, int, const T*, T*, cudaStream_t); \
  template cudaError_t filter_vector_box<T>(int, int, int, const T*, T*, T*, cudaStream_t);              \
  template cudaError_t box_tb<T>(int, int, const T*, T*, cudaStream_t);                                  \
  template cudaError_t box_tb_coarsen<T>(int, int, int, const T*, T*, cudaStream_t);                     \
  template cudaError_t box_oa<T>(int, int, int, const T*, T*, cudaStream_t);                             \
  template int filter_vector<T>(int, int, int, const double*, int, const T*, T*, cudaStream_t);          \
  template int surface_flux<T>(int, int, double, double, const double*, int, const T*, const T*, T*, bool, \
                               cudaStream_t);                                                             \
  template int closure_flux<T>(int, int, double, double, const double*, int, const T*, const T*, T*,     \
                               cudaStream_t);                                                            \
  template int filtered_stress<T>(int, int, double, double, const double*, int, const T*, T*, cudaStream_t, const T*);
INST(double)
INST(float)
#undef INST

}  // namespace exc
