// Separable filter stencils (see filter.cu).
#pragma once
#include "exc_common.cuh"

namespace exc {

constexpr int MAX_TAPS = 40;

struct Taps1D {
  int cnt;
  int off[MAX_TAPS];
  double w[MAX_TAPS];
};
struct Taps3 {
  Taps1D a[3];  // x, y, z
};

Taps1D build_taps(int c, bool stag, bool point, const double* fdelta, int nfd);
int make_taps3(int c, const bool stag[3], const bool point[3], const double* fdelta, int nfd, Taps3* out);

template <typename T>
int filter_vector(int n, int c, int kind, const double* fdelta, int nfd, const T* u, T* ub, cudaStream_t st);
// Box-only volume/face filter in two coalesced passes; tb: 3 n (n/c)^2 words
// of scratch.
template <typename T>
cudaError_t filter_vector_box(int n, int c, int kind, const T* u, T* ub, T* tb, cudaStream_t st);
// Its passes: transverse c x c sums of the fine field (tb), the same sums of
// ratio ct = r cf from those of ratio cf, and the own-axis taps into ub.
template <typename T>
cudaError_t box_tb(int n, int c, const T* u, T* tb, cudaStream_t st);
template <typename T>
cudaError_t box_tb_coarsen(int n, int cf, int ct, const T* tbf, T* tbt, cudaStream_t st);
template <typename T>
cudaError_t box_oa(int n, int c, int kind, const T* tb, T* ub, cudaStream_t st);
template <typename T>
int closure_flux(int n, int c, double l, double visc, const double* fdelta, int nfd, const T* u, const T* p,
                 T* r9, cudaStream_t st);
template <typename T>
int surface_flux(int n, int c, double l, double visc, const double* fdelta, int nfd, const T* u, const T* p,
                 T* r9, bool line, cudaStream_t st);
template <typename T>
int classic_stress(int n, int c, double l, double visc, const double* fdelta, int nfd, const T* u, T* s6,
                   cudaStream_t st);
template <typename T>
int filtered_stress(int n, int c, double l, double visc, const double* fdelta, int nfd, const T* u, T* s6,
                    cudaStream_t st,
                    const T* p = nullptr);

}  // namespace exc
