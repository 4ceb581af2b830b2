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

// r_ij = sigma_ij(u) + delta_ij p at fine cell (x, y, z) (src/N.jl:106-118, 1022-1036)
template <typename T>
struct FluxSrc {
  const T* u;
  const T* p;  // may be null: sigma only
  int n;
  int i, j;
  T h, visc;
  __device__ __forceinline__ long long at(int x, int y, int z) const { return ((long long)z * n + y) * n + x; }
  __device__ __forceinline__ double operator()(int x, int y, int z) const {
    const long long N = (long long)n * n * n;
    int c[3] = {x, y, z};
    int off = (i != j);
    int cr[3] = {c[0], c[1], c[2]}, cl[3] = {c[0], c[1], c[2]};
    cr[j] = (cr[j] + off) % n;
    cl[j] = (cl[j] + off - 1 + n) % n;
    T uir = u[i * N + at(cr[0], cr[1], cr[2])], uil = u[i * N + at(cl[0], cl[1], cl[2])];
    int dr[3] = {c[0], c[1], c[2]}, dl[3] = {c[0], c[1], c[2]};
    dr[i] = (dr[i] + off) % n;
    dl[i] = (dl[i] + off - 1 + n) % n;
    T ujr = u[j * N + at(dr[0], dr[1], dr[2])], ujl = u[j * N + at(dl[0], dl[1], dl[2])];
    T etaj_ui = (uir + uil) / 2, etai_uj = (ujr + ujl) / 2;
    T dj_ui = (uir - uil) / h, di_uj = (ujr - ujl) / h;
    T s = etaj_ui * etai_uj - visc * (dj_ui + di_uj);
    if (i == j && p) s += p[at(x, y, z)];
    return (double)s;
  }
};

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
    for (int tz = 0; tz < taps.a[2].cnt; ++tz) {
      int z = c * iz + taps.a[2].off[tz];
      z = ((z % n) + n) % n;
      double az = 0.0;
      for (int ty = 0; ty < taps.a[1].cnt; ++ty) {
        int y = c * iy + taps.a[1].off[ty];
        y = ((y % n) + n) % n;
        double ay = 0.0;
        for (int tx = 0; tx < taps.a[0].cnt; ++tx) {
          int x = c * ix + taps.a[0].off[tx];
          x = ((x % n) + n) % n;
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
      FluxSrc<T> src{u, p, n, i, j, (T)(l / n), (T)visc};
      filter_kernel<T><<<grid_for(M), 256, 0, st>>>(src, n, c, taps, r9 + (long long)(3 * j + i) * M);
    }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

// sigmaDH (src/N.jl:1088-1115): volume filter GDH of each stress component,
// sampled at LES centres/edges; order s11,s22,s33,s12,s23,s31.
template <typename T>
int filtered_stress(int n, int c, double l, double visc, const double* fdelta, int nfd, const T* u, T* s6,
                    cudaStream_t st) {
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
    FluxSrc<T> src{u, nullptr, n, i, j, (T)(l / n), (T)visc};
    filter_kernel<T><<<grid_for(M), 256, 0, st>>>(src, n, c, taps, s6 + (long long)k * M);
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
template <typename T>
struct FineFilteredStressSrc {
  const T* u;
  int n, i, j;
  T h, visc;
  Taps1D ft;  // centred fine-filter taps (same along every axis)
  __device__ __forceinline__ double uf(int comp, int x, int y, int z) const {
    const long long N = (long long)n * n * n;
    const T* f = u + comp * N;
    double acc = 0.0;
    for (int tz = 0; tz < ft.cnt; ++tz) {
      int zz = z + ft.off[tz];
      zz = ((zz % n) + n) % n;
      double az = 0.0;
      for (int ty = 0; ty < ft.cnt; ++ty) {
        int yy = y + ft.off[ty];
        yy = ((yy % n) + n) % n;
        double ay = 0.0;
        for (int tx = 0; tx < ft.cnt; ++tx) {
          int xx = x + ft.off[tx];
          xx = ((xx % n) + n) % n;
          ay += ft.w[tx] * (double)f[((long long)zz * n + yy) * n + xx];
        }
        az += ft.w[ty] * ay;
      }
      acc += ft.w[tz] * az;
    }
    return acc;
  }
  __device__ __forceinline__ double operator()(int x, int y, int z) const {
    const int c[3] = {x, y, z};
    const int off = (i != j);
    int cr[3] = {c[0], c[1], c[2]}, cl[3] = {c[0], c[1], c[2]};
    cr[j] = (cr[j] + off) % n;
    cl[j] = (cl[j] + off - 1 + n) % n;
    int dr[3] = {c[0], c[1], c[2]}, dl[3] = {c[0], c[1], c[2]};
    dr[i] = (dr[i] + off) % n;
    dl[i] = (dl[i] + off - 1 + n) % n;
    const double uir = uf(i, cr[0], cr[1], cr[2]), uil = uf(i, cl[0], cl[1], cl[2]);
    const double ujr = uf(j, dr[0], dr[1], dr[2]), ujl = uf(j, dl[0], dl[1], dl[2]);
    const double etaj_ui = (uir + uil) / 2, etai_uj = (ujr + ujl) / 2;
    const double dj_ui = (uir - uil) / (double)h, di_uj = (ujr - ujl) / (double)h;
    return etaj_ui * etai_uj - (double)visc * (dj_ui + di_uj);
  }
};

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
    FineFilteredStressSrc<T> src{u, n, i, j, (T)(l / n), (T)visc, ft};
    filter_kernel<T><<<grid_for(M), 256, 0, st>>>(src, n, c, taps, s6 + (long long)k * M);
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
  template int closure_flux<T>(int, int, double, double, const double*, int, const T*, const T*, T*,     \
                               cudaStream_t);                                                            \
  template int filtered_stress<T>(int, int, double, double, const double*, int, const T*, T*, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace exc
