// Learned closure: a 3-D convolutional net on the LES grid (periodic 3x3x3
// kernels, channels 3 -> 32 -> 32 -> 3, GELU after the first two layers),
// trained on (filtered velocity, exact closure) pairs and used inside an LES.
// No counterpart in the reference (its closures are the exact and classic
// ones, src/N.jl:1137-1226).
//
// Activations are channel-last BF16 ([voxel][channel], channels padded to 16
// or 32, outputs to 8); pre-activations are kept in FP32 for the backward
// pass.  Forward and input-gradient convolutions are implicit GEMMs on the
// tensor cores, BF16 inputs with FP32 accumulation: on 64^3 grids with 32
// input channels tcgen05.mma with tensor-memory accumulators (conv_umma_kernel),
// otherwise mma.sync m16n8k16 with the taps' input rows and the weights staged
// in shared memory.  Weight gradients are FP32 reductions with fixed-order
// partials.  Adam keeps FP32 master weights and moments and refreshes the BF16
// copies.
#include <cuda.h>  // CUtensorMap

#include <cmath>
#include <cstring>
#include <vector>

#include <mutex>

#include "internal.cuh"
#include "fields.cuh"

#include <cuda_bf16.h>

namespace exc {

constexpr int NET_TAPS = 27;
constexpr int CONV_M = 64;  // voxels per CTA
constexpr int CONV_THREADS = 128;

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad_f(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}
// GELU(x) and GELU'(x) with one erf: the same values as gelu_f and gelu_grad_f
__device__ __forceinline__ void gelu_and_grad(float x, float& g, float& d) {
  const float e = erff(x * 0.70710678118654752f);
  g = 0.5f * x * (1.0f + e);
  d = 0.5f * (1.0f + e) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__device__ __forceinline__ unsigned ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const unsigned*>(p); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Divisors of the voxel index split (multiply-high reciprocals, built once per
// thread).
struct VoxDiv {
  IdxDiv N, nn, n;
  __device__ __forceinline__ explicit VoxDiv(int n_)
      : N((long long)n_ * n_ * n_), nn((long long)n_ * n_), n(n_) {}
};

// Periodic neighbour of voxel v (linear, x fastest) on an n^3 grid per sample.
__device__ __forceinline__ long long neighbour(long long v, int n, int dz, int dy, int dx, const VoxDiv& dv) {
  const long long nn = (long long)n * n, N = nn * n;
  const long long b = dv.N.div(v);
  long long r = v - b * N;
  int z = (int)dv.nn.div(r);
  r -= (long long)z * nn;
  int y = (int)dv.n.div(r), x = (int)(r - (long long)y * n);
  z += dz; y += dy; x += dx;
  z = z < 0 ? z + n : (z >= n ? z - n : z);
  y = y < 0 ? y + n : (y >= n ? y - n : y);
  x = x < 0 ? x + n : (x >= n ? x - n : x);
  return b * N + ((long long)z * n + y) * n + x;
}

// ---------------------------------------------------------------------------
// Implicit-GEMM convolution on the tensor cores:
//   out[v][co] = bias[co] + sum_{tap, ci} in[v + tap][ci] * Wt[tap][co][ci]
// KP: input channels (multiple of 16), NP: output channels (multiple of 8).
// EPI 0: store GELU(pre) (BF16) and, unless dg is null (inference), GELU'(pre)
// (BF16) into dg for the backward pass;  EPI 1: store out (FP32);
// EPI 2: input gradient: multiply by GELU'(pre) read from dg, store BF16.
// ---------------------------------------------------------------------------
template <int KP, int NP, int EPI>
__global__ void __launch_bounds__(CONV_THREADS)
conv_mma_kernel(long long V, int n, const __nv_bfloat16* __restrict__ in, const __nv_bfloat16* __restrict__ Wt,
                const float* __restrict__ bias, float* __restrict__ pre_out, __nv_bfloat16* __restrict__ act_out,
                __nv_bfloat16* __restrict__ dg, int nout_valid) {
  constexpr int AS = KP + 8;  // padded row stride (bf16) against bank conflicts
  __shared__ __align__(16) __nv_bfloat16 sA[CONV_M * AS];
  __shared__ __align__(16) __nv_bfloat16 sW[NP * AS];
  const long long v0 = (long long)blockIdx.x * CONV_M;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3;
  float acc[NP / 8][4];
#pragma unroll
  for (int j = 0; j < NP / 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
  const VoxDiv dv(n);
  for (int tap = 0; tap < NET_TAPS; ++tap) {
    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    __syncthreads();
    // stage the tap's input rows (16-byte chunks) and weights
    constexpr int CH = KP / 8;  // 8 bf16 per 16-byte chunk
    for (int t = threadIdx.x; t < CONV_M * CH; t += CONV_THREADS) {
      const int r = t / CH, c = t - r * CH;
      const long long v = v0 + r;
      uint4 val = make_uint4(0, 0, 0, 0);
      if (v < V) val = *reinterpret_cast<const uint4*>(in + neighbour(v, n, dz, dy, dx, dv) * KP + c * 8);
      *reinterpret_cast<uint4*>(sA + r * AS + c * 8) = val;
    }
    for (int t = threadIdx.x; t < NP * CH; t += CONV_THREADS) {
      const int r = t / CH, c = t - r * CH;
      *reinterpret_cast<uint4*>(sW + r * AS + c * 8) =
          *reinterpret_cast<const uint4*>(Wt + ((long long)tap * NP + r) * KP + c * 8);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < KP; kk += 16) {
      unsigned a[4];
      const __nv_bfloat16* ar = sA + (warp * 16 + gid) * AS + kk + tig * 2;
      a[0] = ld32(ar);
      a[1] = ld32(ar + 8 * AS);
      a[2] = ld32(ar + 8);
      a[3] = ld32(ar + 8 * AS + 8);
#pragma unroll
      for (int j = 0; j < NP / 8; ++j) {
        const __nv_bfloat16* br = sW + (j * 8 + gid) * AS + kk + tig * 2;
        mma_bf16(acc[j], a, ld32(br), ld32(br + 8));
      }
    }
  }
  // epilogue: C fragment rows gid / gid + 8, columns tig*2 + {0, 1}
#pragma unroll
  for (int j = 0; j < NP / 8; ++j)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long v = v0 + warp * 16 + gid + h * 8;
      if (v >= V) continue;
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int co = j * 8 + tig * 2 + e;
        float x = acc[j][h * 2 + e];
        if (EPI == 0) {
          x += bias[co];
          if (dg) {
            float gx, dx;
            gelu_and_grad(x, gx, dx);
            act_out[v * NP + co] = __float2bfloat16(gx);
            dg[v * NP + co] = __float2bfloat16(dx);
          } else {
            act_out[v * NP + co] = __float2bfloat16(gelu_f(x));
          }
        } else if (EPI == 1) {
          x += bias[co];
          pre_out[v * NP + co] = co < nout_valid ? x : 0.f;
        } else {
          act_out[v * NP + co] = __float2bfloat16(x * __bfloat162float(dg[v * NP + co]));
        }
      }
    }
}

// ---------------------------------------------------------------------------
// The same convolution with the input staged once per CTA: a CTA owns a
// 4 x 4 x 4 voxel block of one sample and loads its 6 x 6 x 6 halo tile
// (all input channels) into shared memory once; the 27 taps then read their
// shifted rows from the tile, and the weights arrive one 3 x 3 tap plane
// (9 taps) at a time.  Used when n % 4 == 0.
// ---------------------------------------------------------------------------
constexpr int TB = 4;            // block edge (voxels)
constexpr int TH = TB + 2;       // halo tile edge
constexpr int TVOX = TH * TH * TH;

template <int KP, int NP, int EPI>
__global__ void __launch_bounds__(CONV_THREADS)
conv_tile_kernel(int n, const __nv_bfloat16* __restrict__ in, const __nv_bfloat16* __restrict__ Wt,
                 const float* __restrict__ bias, float* __restrict__ pre_out, __nv_bfloat16* __restrict__ act_out,
                 __nv_bfloat16* __restrict__ dg, int nout_valid) {
  constexpr int AS = KP + 8;  // padded row stride (bf16) against bank conflicts
  constexpr int CH = KP / 8;  // 16-byte chunks per voxel row
  __shared__ __align__(16) __nv_bfloat16 sT[TVOX * AS];
  __shared__ __align__(16) __nv_bfloat16 sW[9 * NP * AS];
  const int nb = n / TB;
  const long long N = (long long)n * n * n;
  int blk = blockIdx.x;
  const int bxb = blk % nb; blk /= nb;
  const int byb = blk % nb; blk /= nb;
  const int bzb = blk % nb;
  const int b = blk / nb;
  const int x0 = bxb * TB, y0 = byb * TB, z0 = bzb * TB;
  const __nv_bfloat16* inb = in + (long long)b * N * KP;
  // halo tile
  for (int t = threadIdx.x; t < TVOX * CH; t += CONV_THREADS) {
    const int vox = t / CH, c = t - vox * CH;
    const int tx = vox % TH, ty = (vox / TH) % TH, tz = vox / (TH * TH);
    int gx = x0 - 1 + tx, gy = y0 - 1 + ty, gz = z0 - 1 + tz;
    gx = gx < 0 ? gx + n : (gx >= n ? gx - n : gx);
    gy = gy < 0 ? gy + n : (gy >= n ? gy - n : gy);
    gz = gz < 0 ? gz + n : (gz >= n ? gz - n : gz);
    const long long gv = ((long long)gz * n + gy) * n + gx;
    *reinterpret_cast<uint4*>(sT + vox * AS + c * 8) = *reinterpret_cast<const uint4*>(inb + gv * KP + c * 8);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3;
  // the two output rows of this lane: voxels r0 = warp*16 + gid and r0 + 8
  const int r0 = warp * 16 + gid, r1 = r0 + 8;
  const int l0x = r0 % TB, l0y = (r0 / TB) % TB, l0z = r0 / (TB * TB);
  const int l1x = r1 % TB, l1y = (r1 / TB) % TB, l1z = r1 / (TB * TB);
  float acc[NP / 8][4];
#pragma unroll
  for (int j = 0; j < NP / 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
  for (int dzp = 0; dzp < 3; ++dzp) {
    __syncthreads();
    for (int t = threadIdx.x; t < 9 * NP * CH; t += CONV_THREADS) {
      const int row = t / CH, c = t - row * CH;  // row = tap9 * NP + co
      *reinterpret_cast<uint4*>(sW + row * AS + c * 8) =
          *reinterpret_cast<const uint4*>(Wt + ((long long)(dzp * 9) * NP + row) * KP + c * 8);
    }
    __syncthreads();
#pragma unroll 1
    for (int t9 = 0; t9 < 9; ++t9) {
      const int dy = t9 / 3, dx = t9 - dy * 3;  // offsets + 1
      const __nv_bfloat16* a0r = sT + (((l0z + dzp) * TH + (l0y + dy)) * TH + (l0x + dx)) * AS;
      const __nv_bfloat16* a1r = sT + (((l1z + dzp) * TH + (l1y + dy)) * TH + (l1x + dx)) * AS;
#pragma unroll
      for (int kk = 0; kk < KP; kk += 16) {
        unsigned a[4];
        a[0] = ld32(a0r + kk + tig * 2);
        a[1] = ld32(a1r + kk + tig * 2);
        a[2] = ld32(a0r + kk + 8 + tig * 2);
        a[3] = ld32(a1r + kk + 8 + tig * 2);
#pragma unroll
        for (int j = 0; j < NP / 8; ++j) {
          const __nv_bfloat16* br = sW + (t9 * NP + j * 8 + gid) * AS + kk + tig * 2;
          mma_bf16(acc[j], a, ld32(br), ld32(br + 8));
        }
      }
    }
  }
#pragma unroll
  for (int j = 0; j < NP / 8; ++j)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int lx = h ? l1x : l0x, ly = h ? l1y : l0y, lz = h ? l1z : l0z;
      const long long v = (long long)b * N + ((long long)(z0 + lz) * n + (y0 + ly)) * n + (x0 + lx);
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int co = j * 8 + tig * 2 + e;
        float x = acc[j][h * 2 + e];
        if (EPI == 0) {
          x += bias[co];
          if (dg) {
            float gx, dx;
            gelu_and_grad(x, gx, dx);
            act_out[v * NP + co] = __float2bfloat16(gx);
            dg[v * NP + co] = __float2bfloat16(dx);
          } else {
            act_out[v * NP + co] = __float2bfloat16(gelu_f(x));
          }
        } else if (EPI == 1) {
          x += bias[co];
          pre_out[v * NP + co] = co < nout_valid ? x : 0.f;
        } else {
          act_out[v * NP + co] = __float2bfloat16(x * __bfloat162float(dg[v * NP + co]));
        }
      }
    }
}

// ---------------------------------------------------------------------------
// Convolution with the weights resident in shared memory (grids n % 8 == 0):
// a persistent CTA of 8 warps loads all 27 taps of the weights once, then
// walks 8 x 8 x 4 voxel blocks (x, y, z) of the batch; each block's
// 10 x 10 x 6 halo (all input channels) arrives by 16-byte cp.async into one
// of two buffers while the other is consumed.  Warp w computes the 32 voxels
// of slice z = w / 2, rows y = 4 (w % 2) .. + 3, as two 16-voxel m-tiles
// (m = x + 8 y'), so it keeps 2 x NP / 8 independent accumulators; A
// fragments by ldmatrix from the halo rows, B fragments by ldmatrix from the
// weight rows ([tap][co][ci]); rows are padded to an odd number of 16-byte
// units, so the 8 rows of an ldmatrix fall in distinct banks.  Same epilogues
// as conv_tile_kernel.
// ---------------------------------------------------------------------------
constexpr int CR_WARPS = 8, CR_THREADS = 32 * CR_WARPS;
constexpr int CR_BV = 256;  // block 8 x 8 x 4 voxels
constexpr int CR_HX = 10, CR_HY = 10, CR_HZ = 6, CR_HALO = CR_HX * CR_HY * CR_HZ;

template <int KP, int NP>
constexpr size_t conv_res_smem() {
  return ((size_t)NET_TAPS * NP * (KP + 8) + 2 * (size_t)CR_HALO * (KP + 8)) * sizeof(__nv_bfloat16);
}
template <int KP, int NP>
constexpr int conv_res_per_sm() {
  return (int)((227 * 1024) / (conv_res_smem<KP, NP>() + 1024)) < 4 ? (int)((227 * 1024) / (conv_res_smem<KP, NP>() + 1024)) : 4;
}

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

template <int KP, int NP, int EPI>
__global__ void __launch_bounds__(CR_THREADS)
conv_res_kernel(int batch, int n, const __nv_bfloat16* __restrict__ in, const __nv_bfloat16* __restrict__ Wt,
                const float* __restrict__ bias, float* __restrict__ pre_out, __nv_bfloat16* __restrict__ act_out,
                __nv_bfloat16* __restrict__ dg, int nout_valid) {
  constexpr int AS = KP + 8, NTL = NP / 8;
  static_assert(NTL % 2 == 0, "B fragments load two n-tiles at a time");
  extern __shared__ __align__(16) unsigned char cr_smem[];
  __nv_bfloat16* const sW = reinterpret_cast<__nv_bfloat16*>(cr_smem);
  __nv_bfloat16* const sT0 = sW + NET_TAPS * NP * AS;
  for (int t = threadIdx.x; t < NET_TAPS * NP * (KP / 8); t += CR_THREADS) {
    const int row = t / (KP / 8), c = t - row * (KP / 8);
    cp_async_16(sW + row * AS + c * 8, Wt + (long long)row * KP + c * 8);
  }
  cp_async_commit();
  const int nbx = n / 8, nby = n / 8, nbz = n / 4;
  const long long nb3 = (long long)nbx * nby * nbz;
  const long long nblk = (long long)batch * nb3;
  const long long N = (long long)n * n * n;
  auto origin = [&](long long b, long long& s, int& x0, int& y0, int& z0) {
    s = b / nb3;
    const long long r = b - s * nb3;
    z0 = 4 * (int)(r / ((long long)nbx * nby));
    y0 = 8 * (int)((r / nbx) % nby);
    x0 = 8 * (int)(r % nbx);
  };
  auto load_block = [&](long long b, int buf) {
    long long s;
    int x0, y0, z0;
    origin(b, s, x0, y0, z0);
    const __nv_bfloat16* ins = in + s * N * KP;
    __nv_bfloat16* const sT = sT0 + buf * CR_HALO * AS;
    for (int t = threadIdx.x; t < CR_HALO * (KP / 8); t += CR_THREADS) {
      const int h = t / (KP / 8), c = t - h * (KP / 8);
      const int hz = h / (CR_HX * CR_HY), hy = (h / CR_HX) % CR_HY, hx = h % CR_HX;
      int x = x0 - 1 + hx, y = y0 - 1 + hy, z = z0 - 1 + hz;
      x = x < 0 ? x + n : (x >= n ? x - n : x);
      y = y < 0 ? y + n : (y >= n ? y - n : y);
      z = z < 0 ? z + n : (z >= n ? z - n : z);
      cp_async_16(sT + h * AS + c * 8, ins + (((long long)z * n + y) * n + x) * KP + c * 8);
    }
    cp_async_commit();
  };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3, mat = lane >> 3, lr = lane & 7;
  // this lane's ldmatrix rows: A voxel m = lr + 8 (mat & 1) of m-tile t:
  // x = m % 8, y = 4 (warp % 2) + 2 t + m / 8, z = warp / 2
  const int am = lr + 8 * (mat & 1);
  const int wz = warp >> 1, wy = 4 * (warp & 1);
  const int ah = (am & 7) + CR_HX * (wy + (am >> 3)) + CR_HX * CR_HY * wz;  // halo row of m-tile 0, tap offsets 0
  const int ak = 8 * (mat >> 1);
  long long b = blockIdx.x;
  int buf = 0;
  if (b < nblk) load_block(b, 0);
  for (; b < nblk; b += gridDim.x, buf ^= 1) {
    const long long nxt = b + gridDim.x;
    if (nxt < nblk) {
      load_block(nxt, buf ^ 1);
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    } else {
      cp_async_wait_all();
    }
    __syncthreads();
    const __nv_bfloat16* T = sT0 + buf * CR_HALO * AS;
    float acc[2][NTL][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int j = 0; j < NTL; ++j) acc[mt][j][0] = acc[mt][j][1] = acc[mt][j][2] = acc[mt][j][3] = 0.f;
#pragma unroll 1
    for (int dz = 0; dz < 3; ++dz)
#pragma unroll
      for (int t9 = 0; t9 < 9; ++t9) {
        const int tap = dz * 9 + t9, dy = t9 / 3, dx = t9 - dy * 3;
        const __nv_bfloat16* arow = T + (ah + dx + CR_HX * dy + CR_HX * CR_HY * dz) * AS + ak;
#pragma unroll
        for (int kk = 0; kk < KP; kk += 16) {
          unsigned a0[4], a1[4];
          ldsm_x4(a0, arow + kk);
          ldsm_x4(a1, arow + 2 * CR_HX * AS + kk);  // m-tile 1: two rows further in y
#pragma unroll
          for (int p = 0; p < NTL / 2; ++p) {
            unsigned r[4];
            ldsm_x4(r, sW + (tap * NP + 16 * p + 8 * (mat >> 1) + lr) * AS + kk + 8 * (mat & 1));
            mma_bf16(acc[0][2 * p], a0, r[0], r[1]);
            mma_bf16(acc[0][2 * p + 1], a0, r[2], r[3]);
            mma_bf16(acc[1][2 * p], a1, r[0], r[1]);
            mma_bf16(acc[1][2 * p + 1], a1, r[2], r[3]);
          }
        }
      }
    long long s;
    int x0, y0, z0;
    origin(b, s, x0, y0, z0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int mt = q >> 1, h2 = q & 1;
      const int m = gid + 8 * h2;
      const long long v = s * N + ((long long)(z0 + wz) * n + (y0 + wy + 2 * mt + (m >> 3))) * n + (x0 + (m & 7));
#pragma unroll
      for (int j = 0; j < NTL; ++j) {
        const int co = j * 8 + tig * 2;
        float x0v = acc[mt][j][h2 * 2], x1v = acc[mt][j][h2 * 2 + 1];
        if (EPI == 0) {
          x0v += bias[co];
          x1v += bias[co + 1];
          if (dg) {
            float g0, d0, g1, d1;
            gelu_and_grad(x0v, g0, d0);
            gelu_and_grad(x1v, g1, d1);
            *reinterpret_cast<__nv_bfloat162*>(act_out + v * NP + co) =
                __halves2bfloat162(__float2bfloat16(g0), __float2bfloat16(g1));
            *reinterpret_cast<__nv_bfloat162*>(dg + v * NP + co) =
                __halves2bfloat162(__float2bfloat16(d0), __float2bfloat16(d1));
          } else {
            *reinterpret_cast<__nv_bfloat162*>(act_out + v * NP + co) =
                __halves2bfloat162(__float2bfloat16(gelu_f(x0v)), __float2bfloat16(gelu_f(x1v)));
          }
        } else if (EPI == 1) {
          x0v += bias[co];
          x1v += bias[co + 1];
          *reinterpret_cast<float2*>(pre_out + v * NP + co) =
              make_float2(co < nout_valid ? x0v : 0.f, co + 1 < nout_valid ? x1v : 0.f);
        } else {
          const float2 dd = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(dg + v * NP + co));
          *reinterpret_cast<__nv_bfloat162*>(act_out + v * NP + co) =
              __halves2bfloat162(__float2bfloat16(x0v * dd.x), __float2bfloat16(x1v * dd.y));
        }
      }
    }
    __syncthreads();  // this buffer is refilled by the next iteration's prefetch
  }
}

// ---------------------------------------------------------------------------
// The convolution on the fifth-generation tensor cores (tcgen05), for 64^3
// grids with 32 input channels: tcgen05.mma kind::f16 (BF16 operands in
// shared memory, FP32 accumulators in tensor memory).
//
// The x taps ride on the N side of the product.  For the nine (dy, dz) tap
// pairs, one instruction multiplies M = 128 voxels (two consecutive output
// rows of 64, the input rows shifted by (dy, dz)) by all three dx taps'
// weights at once, N = 3 NP columns (dx, co), K = 16 input channels:
//   D[v][dx][co] = sum_{dy, dz, ci} in[v + (dy - 1, dz - 1)][ci] W[dx, dy, dz][co][ci],
// and the epilogue forms out[x][co] = D[x - 1][0][co] + D[x][1][co] + D[x + 1][2][co]
// with x periodic along the row.  Input rows therefore need no x halo: a
// block of 4 output rows reads 3 planes x 6 rows of 64 voxels, stored
// [plane][KP/8][row][x][8 channels], so 128 consecutive voxels (two rows) of
// one channel chunk form the A operand (8-row groups 128 bytes apart, chunks
// 6 KB apart, no swizzle).  Weights sit as [dy, dz][KP/8][dx, co][8].  A block
// takes 2 tiles x 9 (dy, dz) x KP/16 instructions.
//
// A persistent CTA keeps the weights resident and walks blocks (sample, z,
// 4 rows) with warp-specialised roles and mbarrier hand-offs only:
//   warp 1 (loads): waits until the halo buffer is free, then fetches the
//     block's rows by TMA (cp.async.bulk.tensor, one 6-row box per plane and
//     chunk, single rows where y wraps), completing on the buffer's mbarrier;
//   warp 0 (products): one lane waits for the halo and for a free accumulator
//     set, issues the block's instructions and commits them twice (halo
//     buffer free, accumulators full);
//   warps 2-17 (epilogue): wait for the accumulators, read them with
//     tcgen05.ld (warp w reads sub-partition w % 4: output voxel m of an
//     M = 128 tile sits in lane m), exchange the ends of their 32 voxels with
//     the warp holding the other half of the row (shared memory, a two-warp
//     mbarrier), release the set, combine the x taps (shuffles within the
//     warp), apply bias / GELU / GELU' and store.
// Two halo buffers and two accumulator sets let loads, products and epilogue
// of consecutive blocks overlap.  Every wait is bounded; a wait that gives up
// records a fault flag (read by exc_device_faults), every role stops, the
// copies and products in flight are waited for (bounded) and the tensor
// memory is freed.
// ---------------------------------------------------------------------------
constexpr int CU_N = 64;    // grid edge this kernel serves (the row is 64 voxels)
constexpr int CU_ROWS = 4;  // output rows per block: two M = 128 tiles
constexpr int CU_HY = CU_ROWS + 2, CU_HZ = 3;
constexpr int CU_EPI_WARPS = 16;
constexpr int CU_THREADS = 32 * (2 + CU_EPI_WARPS);
constexpr int CU_KP = 32, CU_KC = CU_KP / 8;  // input channels (chunks of 8)

// Tensor maps of one input tensor viewed as (8 channels, 64 x, rows) per
// channel chunk: 6-row and 1-row boxes.
struct HaloMaps {
  CUtensorMap rows6[CU_KC];
  CUtensorMap row1[CU_KC];
};

__device__ int g_learned_fault = 0;
// Wait drill (exc_debug_wait_drill bit 1): the load warp issues no copy at
// all, so the products and the epilogue wait for data that never comes; every
// wait then gives up after CU_DRILL_POLLS polls with nothing in flight.
__device__ int g_learned_drill = 0;
constexpr int CU_POLLS = 1 << 20, CU_DRILL_POLLS = 64;

constexpr int cu_row_bytes = CU_N * 16;  // one row of one chunk
constexpr int cu_halo_bytes = CU_HZ * CU_KC * CU_HY * cu_row_bytes;
template <int NP> __host__ __device__ constexpr int cu_w_bytes() { return NET_TAPS * CU_KP * NP * 2; }
template <int NP> __host__ __device__ constexpr int cu_xch_bytes() { return 2 * CU_EPI_WARPS * 2 * (NP / 2) * 4; }
template <int NP> __host__ __device__ constexpr size_t conv_umma_smem() {
  return 2 * (size_t)cu_halo_bytes + cu_w_bytes<NP>() + cu_xch_bytes<NP>() + 24 * 8 + 16;
}
// tensor-memory columns: two accumulator sets of two tiles x 3 NP
template <int NP> __host__ __device__ constexpr unsigned cu_tmem_cols() { return 2 * 2 * 3 * NP <= 256 ? 256u : 512u; }

__device__ __forceinline__ unsigned cu_smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle: start, leading (K direction)
// and stride (M/N direction, 8-row groups) byte offsets, descriptor version 1.
__device__ __forceinline__ unsigned long long umma_sdesc(unsigned saddr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((saddr >> 4) & 0x3FFF) | ((unsigned long long)((lbo >> 4) & 0x3FFF) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr unsigned umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}
__device__ __forceinline__ void umma_bf16(unsigned dt, unsigned long long ad, unsigned long long bd, unsigned idesc,
                                          unsigned acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(cu_smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ bool cu_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(cu_smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait for the phase of `parity` to complete
__device__ __forceinline__ bool cu_wait(unsigned long long* bar, unsigned parity, int limit = CU_POLLS) {
  for (int polls = 0; polls < limit; ++polls)
    if (cu_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void cu_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(cu_smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void cu_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(cu_smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cu_tma_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                          unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
          cu_smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(cu_smem_u32(bar))
      : "memory");
}
// 32 lanes x 32 bit x NC columns of tensor memory into registers (no wait)
template <int NC>
__device__ __forceinline__ void tmem_ld_nowait(unsigned taddr, unsigned (&r)[NC]) {
  static_assert(NC == 8 || NC == 16, "8 or 16 columns");
  if constexpr (NC == 16) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
  } else {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
  }
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

template <int NP, int EPI>
__global__ void __launch_bounds__(CU_THREADS, 1)
conv_umma_kernel(int batch, const __grid_constant__ HaloMaps maps, const __nv_bfloat16* __restrict__ Wt,
                 const float* __restrict__ bias, float* __restrict__ pre_out, __nv_bfloat16* __restrict__ act_out,
                 __nv_bfloat16* __restrict__ dg, int nout_valid) {
  constexpr int n = CU_N, KP = CU_KP, KC = CU_KC, NT = 3 * NP, NH = NP / 2;
  constexpr int HB = cu_halo_bytes, WB = cu_w_bytes<NP>();
  constexpr unsigned TCOLS = cu_tmem_cols<NP>();
  constexpr unsigned IDESC = umma_idesc_bf16(128, NT);
  constexpr int CHUNK = CU_HY * cu_row_bytes;  // one plane's rows of one chunk (the A operand's K stride)
  extern __shared__ __align__(1024) unsigned char cu_smem[];
  unsigned char* const sH = cu_smem;  // two halo buffers
  unsigned char* const sW = cu_smem + 2 * HB;
  float* const xch = reinterpret_cast<float*>(cu_smem + 2 * HB + WB);  // [block parity][warp][2][NH]
  unsigned long long* const bars = reinterpret_cast<unsigned long long*>(cu_smem + 2 * HB + WB + cu_xch_bytes<NP>());
  unsigned long long* const hfull = bars;       // [2] halo landed (TMA bytes)
  unsigned long long* const hempty = bars + 2;  // [2] halo read by the products (commit)
  unsigned long long* const afull = bars + 4;   // [2] accumulators written (commit)
  unsigned long long* const aempty = bars + 6;  // [2] accumulators read (16 epilogue warps)
  unsigned long long* const xbar = bars + 8;    // [8 warp pairs][2] edge exchange (2 warps)
  unsigned* const s_tmem = reinterpret_cast<unsigned*>(bars + 24);
  volatile int* const s_abort = reinterpret_cast<volatile int*>(s_tmem + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr long long N = (long long)n * n * n;
  constexpr int RG = n / CU_ROWS;  // row groups per z
  const long long nblk = (long long)batch * n * RG;
  const int nb = blockIdx.x < nblk ? (int)((nblk - 1 - blockIdx.x) / gridDim.x) + 1 : 0;
  auto origin = [&](long long b, long long& s, int& z0, int& y0) {
    s = b / (n * RG);
    const int r = (int)(b - s * (n * RG));
    z0 = r / RG;
    y0 = CU_ROWS * (r - (r / RG) * RG);
  };
  auto fault = [&]() {
    atomicExch(&g_learned_fault, 1);
    *s_abort = 1;
  };
  const bool drill = g_learned_drill != 0;
  const int polls = drill ? CU_DRILL_POLLS : CU_POLLS;

  // weights: tap (dx, dy, dz) = dz 9 + dy 3 + dx -> [dy, dz][chunk][dx NP + co][8]
  for (int t = tid; t < NET_TAPS * NP * KC; t += CU_THREADS) {
    const int c = t % KC, row = t / KC, tap = row / NP, co = row - tap * NP;
    const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3, g = dy * 3 + dz;
    cp_async_16(reinterpret_cast<__nv_bfloat16*>(sW + ((g * KC + c) * NT + dx * NP + co) * 16),
                Wt + (long long)row * KP + c * 8);
  }
  cp_async_commit();
  if (tid == 0) {
    for (int k = 0; k < 24; ++k)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(cu_smem_u32(&bars[k])),
                   "r"(k < 6 ? 1 : (k < 8 ? CU_EPI_WARPS : 2))
                   : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    *s_abort = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(cu_smem_u32(s_tmem)),
                 "r"(TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  cp_async_wait_all();
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // weights -> tensor-core reads
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *s_tmem;

  if (warp == 1) {
    // ---- loads ----
    int i = 0;
    for (; i < nb && !drill; ++i) {
      const int buf = i & 1;
      if (i >= 2 && !__all_sync(0xffffffffu, cu_wait(&hempty[buf], (unsigned)(((i - 2) >> 1) & 1), polls))) {
        if (lane == 0) fault();
        break;
      }
      if (*s_abort) break;
      long long s;
      int z0, y0;
      origin(blockIdx.x + (long long)i * gridDim.x, s, z0, y0);
      if (lane == 0) cu_expect_tx(&hfull[buf], (unsigned)HB);
      __syncwarp();
      if (lane < KC * CU_HZ) {
        const int c = lane / CU_HZ, hz = lane - c * CU_HZ;
        int zz = z0 - 1 + hz;
        zz = zz < 0 ? zz + n : (zz >= n ? zz - n : zz);
        const int rbase = (int)(s * n * n) + zz * n;  // row index of (y = 0, zz, s)
        unsigned char* const dst = sH + buf * HB + (hz * KC + c) * CHUNK;
        if (y0 >= 1 && y0 + CU_ROWS < n) {
          cu_tma_3d(dst, &maps.rows6[c], 0, 0, rbase + y0 - 1, &hfull[buf]);
        } else {
          for (int hy = 0; hy < CU_HY; ++hy) {
            int y = y0 - 1 + hy;
            y = y < 0 ? y + n : (y >= n ? y - n : y);
            cu_tma_3d(dst + hy * cu_row_bytes, &maps.row1[c], 0, 0, rbase + y, &hfull[buf]);
          }
        }
      }
    }
    // copies in flight: the last two issued batches land (bounded)
    for (int j = i - 2; j < i; ++j)
      if (j >= 0 && !__all_sync(0xffffffffu, cu_wait(&hfull[j & 1], (unsigned)((j >> 1) & 1), polls)) && lane == 0) fault();
  } else if (warp == 0) {
    // ---- products ----
    if (lane == 0) {
      const unsigned long long bd0 = umma_sdesc(cu_smem_u32(sW), NT * 16, 128);
      int i = 0;
      for (; i < nb; ++i) {
        const int buf = i & 1;
        if (!cu_wait(&hfull[buf], (unsigned)((i >> 1) & 1), polls) ||
            (i >= 2 && !cu_wait(&aempty[buf], (unsigned)(((i - 2) >> 1) & 1), polls))) {
          fault();
          break;
        }
        if (*s_abort) break;
        tc_fence_after();
        // the start address (/16) is the descriptor's low field: an operand
        // at a byte offset is the base descriptor plus offset / 16
        const unsigned long long ad0 = umma_sdesc(cu_smem_u32(sH + buf * HB), CHUNK, 128);
#pragma unroll
        for (int t = 0; t < 2; ++t)
#pragma unroll
          for (int g = 0; g < 9; ++g)
#pragma unroll
            for (int kk = 0; kk < KP / 16; ++kk) {
              const int dy = g / 3, dz = g % 3;
              const unsigned aoff = (unsigned)(((dz * KC + 2 * kk) * CHUNK + (2 * t + dy) * cu_row_bytes) >> 4);
              const unsigned boff = (unsigned)((g * KC + kk * 2) * NT);
              umma_bf16(tmem + (unsigned)((buf * 2 + t) * NT), ad0 + aoff, bd0 + boff, IDESC, (g | kk) != 0);
            }
        umma_commit(&hempty[buf]);
        umma_commit(&afull[buf]);
      }
      // products in flight complete (bounded)
      if (i > 0 && !cu_wait(&afull[(i - 1) & 1], (unsigned)(((i - 1) >> 1) & 1), polls)) fault();
    }
    __syncwarp();
  } else {
    // ---- epilogue ----
    // sub-partition q (lanes 32q..), tile et (rows 2 et, 2 et + 1), channel
    // half eh; the partner warp (w ^ 1, sub-partition q ^ 1) holds the other
    // 32 voxels of the same row
    const int q = warp & 3, k = (warp - 2) >> 2, et = k & 1, eh = k >> 1;
    const int erow = 2 * et + (q >> 1), x = 32 * (q & 1) + lane, cb = eh * NH;
    float bb[NH];
#pragma unroll
    for (int j = 0; j < NH; ++j) bb[j] = (EPI == 2) ? 0.f : __ldg(bias + cb + j);
    for (int i = 0; i < nb; ++i) {
      const int set = i & 1;
      if (!__all_sync(0xffffffffu, cu_wait(&afull[set], (unsigned)((i >> 1) & 1), polls))) {
        if (lane == 0) fault();
        break;
      }
      if (*s_abort) break;
      tc_fence_after();
      const unsigned ta = tmem + ((unsigned)(32 * q) << 16) + (unsigned)((set * 2 + et) * NT + cb);
      unsigned d0[NH], d1[NH], d2[NH];
      tmem_ld_nowait<NH>(ta, d0);
      tmem_ld_nowait<NH>(ta + NP, d1);
      tmem_ld_nowait<NH>(ta + 2 * NP, d2);
      tmem_wait_ld();
      // ends of the 32 voxels go to the partner warp (buffers alternate with
      // the block; the pair's mbarrier, two arrivals, orders writes and reads)
      float* const mine = xch + ((i & 1) * CU_EPI_WARPS + (warp - 2)) * 2 * NH;
      const float* const other = xch + ((i & 1) * CU_EPI_WARPS + ((warp ^ 1) - 2)) * 2 * NH;
      if (lane == 31) {
#pragma unroll
        for (int j = 0; j < NH; ++j) mine[j] = __uint_as_float(d0[j]);
      }
      if (lane == 0) {
#pragma unroll
        for (int j = 0; j < NH; ++j) mine[NH + j] = __uint_as_float(d2[j]);
      }
      __syncwarp();
      unsigned long long* const xb = &xbar[((warp - 2) >> 1) * 2 + (i & 1)];
      if (lane == 0) cu_arrive(xb);
      if (!__all_sync(0xffffffffu, cu_wait(xb, (unsigned)((i >> 1) & 1), polls))) {
        if (lane == 0) fault();
        break;
      }
      float f[NH];
#pragma unroll
      for (int j = 0; j < NH; ++j) {
        // D[x - 1][0] from the lane below, D[x + 1][2] from the lane above
        float lo = __uint_as_float(__shfl_up_sync(0xffffffffu, d0[j], 1));
        float hi = __uint_as_float(__shfl_down_sync(0xffffffffu, d2[j], 1));
        if (lane == 0) lo = other[j];
        if (lane == 31) hi = other[NH + j];
        f[j] = lo + __uint_as_float(d1[j]) + hi;
      }
      // the accumulator set and this block's exchange buffer are released:
      // both are rewritten two blocks later, after every warp's release
      tc_fence_before();
      __syncwarp();
      if (lane == 0) cu_arrive(&aempty[set]);
      long long s;
      int z0, y0;
      origin(blockIdx.x + (long long)i * gridDim.x, s, z0, y0);
      const long long g = s * N + ((long long)z0 * n + (y0 + erow)) * n + x;
      if (EPI == 0 || EPI == 1) {
#pragma unroll
        for (int j = 0; j < NH; j += 4) {
          float4 v;
          v.x = f[j] + bb[j];
          v.y = f[j + 1] + bb[j + 1];
          v.z = f[j + 2] + bb[j + 2];
          v.w = f[j + 3] + bb[j + 3];
          if (EPI == 1) {
            const int co = cb + j;
            v.x = co < nout_valid ? v.x : 0.f;
            v.y = co + 1 < nout_valid ? v.y : 0.f;
            v.z = co + 2 < nout_valid ? v.z : 0.f;
            v.w = co + 3 < nout_valid ? v.w : 0.f;
          }
          if (EPI == 1) {
            *reinterpret_cast<float4*>(pre_out + g * NP + cb + j) = v;
          } else if (dg) {
            float ga, da, gb, db, gc, dc, gd, dd;
            gelu_and_grad(v.x, ga, da);
            gelu_and_grad(v.y, gb, db);
            gelu_and_grad(v.z, gc, dc);
            gelu_and_grad(v.w, gd, dd);
            __nv_bfloat162 h0 = __halves2bfloat162(__float2bfloat16(ga), __float2bfloat16(gb));
            __nv_bfloat162 h1 = __halves2bfloat162(__float2bfloat16(gc), __float2bfloat16(gd));
            uint2 pk;
            pk.x = *reinterpret_cast<unsigned*>(&h0);
            pk.y = *reinterpret_cast<unsigned*>(&h1);
            *reinterpret_cast<uint2*>(act_out + g * NP + cb + j) = pk;
            h0 = __halves2bfloat162(__float2bfloat16(da), __float2bfloat16(db));
            h1 = __halves2bfloat162(__float2bfloat16(dc), __float2bfloat16(dd));
            pk.x = *reinterpret_cast<unsigned*>(&h0);
            pk.y = *reinterpret_cast<unsigned*>(&h1);
            *reinterpret_cast<uint2*>(dg + g * NP + cb + j) = pk;
          } else {
            __nv_bfloat162 h0 = __halves2bfloat162(__float2bfloat16(gelu_f(v.x)), __float2bfloat16(gelu_f(v.y)));
            __nv_bfloat162 h1 = __halves2bfloat162(__float2bfloat16(gelu_f(v.z)), __float2bfloat16(gelu_f(v.w)));
            uint2 pk;
            pk.x = *reinterpret_cast<unsigned*>(&h0);
            pk.y = *reinterpret_cast<unsigned*>(&h1);
            *reinterpret_cast<uint2*>(act_out + g * NP + cb + j) = pk;
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < NH; j += 4) {
          const uint2 dq = *reinterpret_cast<const uint2*>(dg + g * NP + cb + j);
          const float2 pa = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&dq.x));
          const float2 pb = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&dq.y));
          __nv_bfloat162 h0 = __halves2bfloat162(__float2bfloat16(f[j] * pa.x), __float2bfloat16(f[j + 1] * pa.y));
          __nv_bfloat162 h1 = __halves2bfloat162(__float2bfloat16(f[j + 2] * pb.x), __float2bfloat16(f[j + 3] * pb.y));
          uint2 pk;
          pk.x = *reinterpret_cast<unsigned*>(&h0);
          pk.y = *reinterpret_cast<unsigned*>(&h1);
          *reinterpret_cast<uint2*>(act_out + g * NP + cb + j) = pk;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TCOLS) : "memory");
  }
}

// Tiled tensor map encoder (defined with the RHS sweep).
bool encode_tiled_map(CUtensorMap* map, CUtensorMapDataType dt, unsigned rank, const void* base,
                      const cuuint64_t* dims, const cuuint64_t* strides, const cuuint32_t* box);

// The maps of a [batch][64^3][32] BF16 tensor; false when they cannot be made.
static bool halo_maps(const __nv_bfloat16* in, int batch, HaloMaps* m) {
  if ((reinterpret_cast<uintptr_t>(in) & 15) != 0) return false;
  const cuuint64_t dims[3] = {8, (cuuint64_t)CU_N, (cuuint64_t)batch * CU_N * CU_N};
  const cuuint64_t strides[2] = {(cuuint64_t)CU_KP * 2, (cuuint64_t)CU_N * CU_KP * 2};
  const cuuint32_t box6[3] = {8, (cuuint32_t)CU_N, (cuuint32_t)CU_HY}, box1[3] = {8, (cuuint32_t)CU_N, 1};
  for (int c = 0; c < CU_KC; ++c) {
    if (!encode_tiled_map(&m->rows6[c], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, in + c * 8, dims, strides, box6) ||
        !encode_tiled_map(&m->row1[c], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, in + c * 8, dims, strides, box1))
      return false;
  }
  return true;
}

// Engine 0: the tcgen05 kernel on 64^3 grids for 32 input channels (with 16
// the weight-resident mma.sync kernel measured faster: its epilogue, not the
// products, bounds both), else the mma.sync forms; engine 1: the mma.sync
// forms only.
template <int KP, int NP, int EPI>
static void conv_launch(int engine, long long V, int n, const __nv_bfloat16* in, const __nv_bfloat16* W,
                        const float* bias, float* pre_out, __nv_bfloat16* act_out, __nv_bfloat16* dg,
                        int nout_valid, cudaStream_t st) {
  if constexpr (KP == CU_KP) {
    if (engine == 0 && n == CU_N) {
      const long long N = (long long)n * n * n;
      const int batch = (int)(V / N);
      HaloMaps maps;
      if (batch == 0) return;
      if (halo_maps(in, batch, &maps)) {
        const long long nblk = (long long)batch * n * (n / CU_ROWS);
        const long long ctas = std::min<long long>(nblk, 152);
        conv_umma_kernel<NP, EPI><<<(unsigned)ctas, CU_THREADS, conv_umma_smem<NP>(), st>>>(
            batch, maps, W, bias, pre_out, act_out, dg, nout_valid);
        return;
      }
    }
  }
  if (n % 8 == 0) {
    const long long N = (long long)n * n * n;
    const long long nblk = V / CR_BV;
    const long long ctas = std::min<long long>(nblk, (long long)conv_res_per_sm<KP, NP>() * 152);
    conv_res_kernel<KP, NP, EPI><<<(unsigned)ctas, CR_THREADS, conv_res_smem<KP, NP>(), st>>>(
        (int)(V / N), n, in, W, bias, pre_out, act_out, dg, nout_valid);
  } else if (n % TB == 0) {
    const long long N = (long long)n * n * n;
    const long long blocks = (V / N) * (N / (TB * TB * TB));
    conv_tile_kernel<KP, NP, EPI><<<(unsigned)blocks, CONV_THREADS, 0, st>>>(n, in, W, bias, pre_out, act_out,
                                                                          dg, nout_valid);
  } else {
    conv_mma_kernel<KP, NP, EPI><<<(unsigned)((V + CONV_M - 1) / CONV_M), CONV_THREADS, 0, st>>>(
        V, n, in, W, bias, pre_out, act_out, dg, nout_valid);
  }
}

// ---------------------------------------------------------------------------
// Weight gradient on the tensor cores: for one tap, the KP x NP matrix
//   dW[tap][ci][co] = sum_v in[v + tap][ci] g[v][co]
// is a GEMM with the voxels as the reduction axis (A = in_shifted^T, B = g).
// A CTA reduces one chunk of WG_CHUNK voxels for one tap: blocks of WG_VB
// voxels are staged transposed ([channel][voxel], BF16) so the mma fragments
// are 32-bit loads of voxel pairs; each warp owns KP*NP/(16*8*4) 16x8 output
// tiles.  Partials per (chunk, tap) are folded in a fixed order
// (wgrad_fold_kernel), so the result is deterministic.
// ---------------------------------------------------------------------------
constexpr int WG_CHUNK = 4096;
constexpr int WG_VB = 64;

template <int KP, int NP>
__global__ void __launch_bounds__(128)
wgrad_partial_kernel(long long V, int n, const __nv_bfloat16* __restrict__ in, const __nv_bfloat16* __restrict__ g,
                     float* __restrict__ part) {
  constexpr int VS = WG_VB + 8;  // padded voxel stride (bf16)
  constexpr int MT = KP / 16, NT = NP / 8, TILES = MT * NT, TPW = TILES / 4;
  static_assert(TILES % 4 == 0, "tiles must split over 4 warps");
  __shared__ __align__(16) __nv_bfloat16 sX[KP * VS];
  __shared__ __align__(16) __nv_bfloat16 sG[NP * VS];
  const int tap = blockIdx.y;
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  const long long c0 = (long long)blockIdx.x * WG_CHUNK;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const VoxDiv dv(n);
  float acc[TPW][4];
#pragma unroll
  for (int q = 0; q < TPW; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
  for (long long s0 = c0; s0 < c0 + WG_CHUNK && s0 < V; s0 += WG_VB) {
    __syncthreads();
    // stage transposed: 16-byte chunks of 8 channels of one voxel
    for (int t = threadIdx.x; t < WG_VB * (KP / 8); t += blockDim.x) {
      const int r = t / (KP / 8), c = t - r * (KP / 8);
      const long long v = s0 + r;
      uint4 val = make_uint4(0, 0, 0, 0);
      if (v < V) val = *reinterpret_cast<const uint4*>(in + neighbour(v, n, dz, dy, dx, dv) * KP + c * 8);
      const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&val);
#pragma unroll
      for (int i = 0; i < 8; ++i) sX[(c * 8 + i) * VS + r] = e[i];
    }
    for (int t = threadIdx.x; t < WG_VB * (NP / 8); t += blockDim.x) {
      const int r = t / (NP / 8), c = t - r * (NP / 8);
      const long long v = s0 + r;
      uint4 val = make_uint4(0, 0, 0, 0);
      if (v < V) val = *reinterpret_cast<const uint4*>(g + v * NP + c * 8);
      const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&val);
#pragma unroll
      for (int i = 0; i < 8; ++i) sG[(c * 8 + i) * VS + r] = e[i];
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < WG_VB; kk += 16) {
#pragma unroll
      for (int q = 0; q < TPW; ++q) {
        const int tile = warp * TPW + q;
        const int mt = tile / NT, nt = tile - mt * NT;
        const __nv_bfloat16* ar = sX + (mt * 16 + gid) * VS + kk + tig * 2;
        unsigned a[4];
        a[0] = ld32(ar);
        a[1] = ld32(ar + 8 * VS);
        a[2] = ld32(ar + 8);
        a[3] = ld32(ar + 8 * VS + 8);
        const __nv_bfloat16* br = sG + (nt * 8 + gid) * VS + kk + tig * 2;
        mma_bf16(acc[q], a, ld32(br), ld32(br + 8));
      }
    }
  }
  // C fragment: rows (ci) gid / gid + 8, columns (co) tig*2 + {0, 1}
  float* out = part + ((long long)blockIdx.x * NET_TAPS + tap) * (KP * NP);
#pragma unroll
  for (int q = 0; q < TPW; ++q) {
    const int tile = warp * TPW + q;
    const int mt = tile / NT, nt = tile - mt * NT;
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int ci = mt * 16 + gid + h * 8, co = nt * 8 + tig * 2 + e;
        out[ci * NP + co] = acc[q][h * 2 + e];
      }
  }
}

// ---------------------------------------------------------------------------
// Weight gradient over 8 x 2 x 4 voxel blocks (x, y, z), every tap in one
// CTA:
//   dW[tap][ci][co] = sum_v in[v + shift(tap)][ci] * g[v][co].
// A persistent CTA of 9 warps walks the blocks of the batch; each block's
// 10 x 4 x 6 halo of `in` and its 64 rows of `g` arrive by 16-byte cp.async
// into one of two buffers while the other is consumed, so both tensors are
// read once per block (the halo of `in` from L2).  Voxel rows in shared memory
// are padded to an odd number of 16-byte units, so the 8 rows of an ldmatrix
// (8 consecutive x) fall in distinct banks.  Warp w owns the three taps
// (dz, dy) = (w / 3 - 1, w % 3 - 1), dx = -1, 0, 1, and accumulates them over
// all of its blocks in registers; its A fragments (in^T, channels x voxels)
// and B fragments (g, voxels x channels) come from the [voxel][channel]
// layouts by ldmatrix.trans.  The partials of a CTA go to part[cta] and are
// folded in a fixed order (wgrad_fold_kernel).
// ---------------------------------------------------------------------------
constexpr int WT_WARPS = 9, WT_THREADS = 32 * WT_WARPS, WT_CTAS = 152;
constexpr int WT_BY = 4, WT_BV = 8 * WT_BY * 4;  // block 8 x WT_BY x 4 voxels
constexpr int WT_HX = 10, WT_HY = WT_BY + 2, WT_HZ = 6, WT_HALO = WT_HX * WT_HY * WT_HZ;

// shared memory of wgrad_tile_kernel: two buffers of the halo rows (stride
// KP + 8 halves) and of the g rows (stride NP + 8 halves)
template <int KP, int NP>
constexpr size_t wgrad_tile_smem() {
  return 2 * ((size_t)WT_HALO * (KP + 8) + WT_BV * (size_t)(NP + 8)) * sizeof(__nv_bfloat16);
}

__device__ __forceinline__ void ldsm_x4_trans(unsigned (&r)[4], const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

template <int KP, int NP>
__global__ void __launch_bounds__(WT_THREADS, 1)
wgrad_tile_kernel(int batch, int n, const __nv_bfloat16* __restrict__ in, const __nv_bfloat16* __restrict__ g,
                  float* __restrict__ part, double* __restrict__ bpart) {
  constexpr int MT = KP / 16, NTL = NP / 8, KS = KP + 8, NS = NP + 8;
  static_assert(NTL % 2 == 0, "B fragments load two n-tiles at a time");
  extern __shared__ __align__(16) unsigned char wt_smem[];
  __nv_bfloat16* const sX0 = reinterpret_cast<__nv_bfloat16*>(wt_smem);
  __nv_bfloat16* const sG0 = sX0 + 2 * WT_HALO * KS;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wdz = warp / 3, wdy = warp % 3;  // dz + 1, dy + 1 of this warp's taps
  const int nbx = n / 8, nby = n / WT_BY, nbz = n / 4;
  const long long nb3 = (long long)nbx * nby * nbz;
  const long long nblk = (long long)batch * nb3;
  const long long N = (long long)n * n * n;
  float acc[3][MT][NTL][4];
#pragma unroll
  for (int t = 0; t < 3; ++t)
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int q = 0; q < NTL; ++q) acc[t][m][q][0] = acc[t][m][q][1] = acc[t][m][q][2] = acc[t][m][q][3] = 0.f;
  // copies of block b into buffer buf: halo voxels (hx, hy, hz) at origin
  // (8 bx, WT_BY by, 4 bz) - 1 (periodic in the sample), KP / 8 pieces each;
  // g rows of the block voxels (v = x + 8 y + 8 WT_BY z), NP / 8 pieces each
  auto load_block = [&](long long b, int buf) {
    const long long s = b / nb3;
    const long long r = b - s * nb3;
    const int bz = (int)(r / ((long long)nbx * nby)), by = (int)((r / nbx) % nby), bx = (int)(r % nbx);
    const __nv_bfloat16* ins = in + s * N * KP;
    __nv_bfloat16* const sX = sX0 + buf * WT_HALO * KS;
    for (int t = threadIdx.x; t < WT_HALO * (KP / 8); t += WT_THREADS) {
      const int h = t / (KP / 8), c = t - h * (KP / 8);
      const int hz = h / (WT_HX * WT_HY), hy = (h / WT_HX) % WT_HY, hx = h % WT_HX;
      int x = 8 * bx - 1 + hx, y = WT_BY * by - 1 + hy, z = 4 * bz - 1 + hz;
      x = x < 0 ? x + n : (x >= n ? x - n : x);
      y = y < 0 ? y + n : (y >= n ? y - n : y);
      z = z < 0 ? z + n : (z >= n ? z - n : z);
      cp_async_16(sX + h * KS + c * 8, ins + (((long long)z * n + y) * n + x) * KP + c * 8);
    }
    const __nv_bfloat16* gs = g + s * N * NP;
    __nv_bfloat16* const sG = sG0 + buf * WT_BV * NS;
    for (int t = threadIdx.x; t < WT_BV * (NP / 8); t += WT_THREADS) {
      const int v = t / (NP / 8), c = t - v * (NP / 8);
      const int x = 8 * bx + (v & 7), y = WT_BY * by + ((v >> 3) % WT_BY), z = 4 * bz + v / (8 * WT_BY);
      cp_async_16(sG + v * NS + c * 8, gs + (((long long)z * n + y) * n + x) * NP + c * 8);
    }
    cp_async_commit();
  };
  // ldmatrix lane roles: matrix mat = lane / 8, row r = lane % 8
  const int mat = lane >> 3, lr = lane & 7;
  // bias gradient db[co] = sum_v g[v][co] from the same g rows: thread
  // t < 2 NP sums rows 32 (t / NP) .. + 31 of channel t % NP per block in
  // FP32 and the block sums in FP64, in the CTA's fixed block order
  const int bco = threadIdx.x % NP, bhalf = threadIdx.x / NP;
  double bsum = 0.0;
  long long b = blockIdx.x;
  int buf = 0;
  if (b < nblk) load_block(b, 0);
  for (; b < nblk; b += gridDim.x, buf ^= 1) {
    const long long nxt = b + gridDim.x;
    if (nxt < nblk) {
      load_block(nxt, buf ^ 1);
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    } else {
      cp_async_wait_all();
    }
    __syncthreads();
    const __nv_bfloat16* X = sX0 + buf * WT_HALO * KS;
    const __nv_bfloat16* G = sG0 + buf * WT_BV * NS;
    if (bhalf < 2) {
      float fs = 0.f;
#pragma unroll 8
      for (int v = (WT_BV / 2) * bhalf; v < (WT_BV / 2) * (bhalf + 1); ++v) fs += __bfloat162float(G[v * NS + bco]);
      bsum += (double)fs;
    }
#pragma unroll 2
    for (int ks = 0; ks < WT_BV / 16; ++ks) {
      // step ks: the 16 voxels x = 0..7, y = 2 (ks % (WT_BY / 2)) + {0, 1},
      // z = ks / (WT_BY / 2) (rows 16 ks .. 16 ks + 15 of the g block)
      const int kz = ks / (WT_BY / 2), ky0 = 2 * (ks % (WT_BY / 2));
      // B: voxels k = x + 8 y of the step; two n-tiles per ldmatrix.x4
      unsigned bf[NTL][2];
#pragma unroll
      for (int p = 0; p < NTL / 2; ++p) {
        const int k = lr + 8 * (mat & 1);
        unsigned r[4];
        ldsm_x4_trans(r, G + (16 * ks + k) * NS + 16 * p + 8 * (mat >> 1));
        bf[2 * p][0] = r[0];
        bf[2 * p][1] = r[1];
        bf[2 * p + 1][0] = r[2];
        bf[2 * p + 1][1] = r[3];
      }
      // A: in at the shifted voxel of each tap, channels 16 mt ..
      const int ka = lr + 8 * (mat >> 1);
      const int hy = ky0 + (ka >> 3) + wdy, hz = kz + wdz;
#pragma unroll
      for (int t = 0; t < 3; ++t) {
        const int h = (ka & 7) + t + WT_HX * hy + WT_HX * WT_HY * hz;
#pragma unroll
        for (int m = 0; m < MT; ++m) {
          unsigned a[4];
          ldsm_x4_trans(a, X + h * KS + 16 * m + 8 * (mat & 1));
#pragma unroll
          for (int q = 0; q < NTL; ++q) mma_bf16(acc[t][m][q], a, bf[q][0], bf[q][1]);
        }
      }
    }
    __syncthreads();  // this buffer is refilled by the next iteration's prefetch
  }
  if (bhalf < 2) bpart[((long long)blockIdx.x * 2 + bhalf) * NP + bco] = bsum;
  // C fragment: rows (ci) gid / gid + 8, columns (co) tig * 2 + {0, 1}
  const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    const int tap = wdz * 9 + wdy * 3 + t;
    float* out = part + ((long long)blockIdx.x * NET_TAPS + tap) * (KP * NP);
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int q = 0; q < NTL; ++q)
#pragma unroll
        for (int hh = 0; hh < 2; ++hh)
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const int ci = m * 16 + gid + hh * 8, co = q * 8 + tig * 2 + e;
            out[ci * NP + co] = acc[t][m][q][hh * 2 + e];
          }
  }
}

// ---------------------------------------------------------------------------
// Weight gradient on the tcgen05 tensor cores (64^3 grids, conv engine 0):
//   dW[tap][ci][co] = sum_v in[v + tap][ci] g[v][co]
// reduced over blocks of WU_RB = 2 output rows (64 voxels along x, rows y0,
// y0 + 1 at fixed z and sample).  For a block the A operand holds, for each
// dz, the window of four input rows y0 - 1 .. y0 + 2 at z + dz (TMA boxes of
// 8 channels x 64 voxels, 1 KB each; rows shared by the block's two output
// rows, so 12 rows per two output rows cross L2 instead of 18), laid out
// [dz][window row][channel chunk][x], and the B operand each output row of g
// with its two copies rotated by -dx for dx = -1, +1 (periodic along x, which
// a TMA box cannot wrap: the helper warps copy them in shared memory).  Both
// operands are MN-major (channels contiguous per voxel, as stored): for
// output row r the M = 128 rows of a product are (window rows r .. r + 3 of
// 128 / (4 KP) consecutive dz, input channel) at a uniform 1 KB chunk stride,
// and
//   D[(dz, w, ci)][(dx, co)] += sum_x in[x, y0 - 1 + r + w, z + dz][ci] g[x - dx, y0 + r][co]
// is the contribution to dW[tap (dx, dy = w - 1, dz)] (w = 3 lands on the
// next window or buffer and is not used).  N = 3 NP.  The CTA's whole dW stays
// in tensor memory over its blocks and is written once as the CTA's partial
// (folded by wgrad_fold_kernel in a fixed order).  Roles: warp 0 issues the
// products, warp 1 the copies, warps 2-5 rotate g, sum it for the bias
// gradient (FP32 per row segment, FP64 over rows, one partial per CTA) and, at
// the end, read the accumulators.  Three or four stages of buffers keep
// copies of later blocks in flight; every wait is bounded as in
// conv_umma_kernel (a wait that gives up records the fault, every role stops,
// copies and products in flight are waited for, the tensor memory is freed).
// ---------------------------------------------------------------------------
constexpr int WU_THREADS = 192;
constexpr int WU_RB = 2;  // output rows per block
struct WgMaps {
  CUtensorMap a[4];  // input rows, per 8-channel chunk
  CUtensorMap b[4];  // g rows, per 8-channel chunk
};
template <int KP> __host__ __device__ constexpr int wu_spg() { return 128 / KP; }  // window rows per product
template <int KP> __host__ __device__ constexpr int wu_groups() { return (3 * 4 * KP + 127) / 128; }
template <int KP> __host__ __device__ constexpr int wu_a_bytes() { return 3 * (WU_RB + 2) * (KP / 8) * 1024; }
template <int NP> __host__ __device__ constexpr int wu_b_bytes() { return WU_RB * 3 * (NP / 8) * 1024; }
template <int KP, int NP> __host__ __device__ constexpr int wu_stage_bytes() { return wu_a_bytes<KP>() + wu_b_bytes<NP>(); }
// stages of buffers that fit in 216 KB (at most four)
template <int KP, int NP> __host__ __device__ constexpr int wu_stages() {
  return 216 * 1024 / wu_stage_bytes<KP, NP>() >= 4 ? 4 : (216 * 1024 / wu_stage_bytes<KP, NP>() >= 3 ? 3 : 2);
}
template <int KP, int NP> __host__ __device__ constexpr size_t wgrad_umma_smem() {
  return 1024 + (size_t)wu_stages<KP, NP>() * wu_stage_bytes<KP, NP>() + 16 * 8;  // 1024: alignment slack
}
template <int KP, int NP> __host__ __device__ constexpr unsigned wu_tmem_cols() {
  return wu_groups<KP>() * 3 * NP <= 256 ? 256u : 512u;
}

template <int KP, int NP>
__global__ void __launch_bounds__(WU_THREADS, 1)
wgrad_umma_kernel(int batch, const __grid_constant__ WgMaps maps, float* __restrict__ part,
                  double* __restrict__ bpart) {
  constexpr int n = CU_N, KC = KP / 8, NC = NP / 8, SPG = wu_spg<KP>(), NG = wu_groups<KP>(), NT = 3 * NP;
  constexpr int AB = wu_a_bytes<KP>(), SB = wu_stage_bytes<KP, NP>(), NS = wu_stages<KP, NP>();
  constexpr int WR = WU_RB + 2;                     // window rows per dz
  constexpr int NA = 3 * WR * KC, NB = WU_RB * NC;  // copies per block
  constexpr int SEGS = 128 / NP, SL = CU_N / SEGS;  // bias sums: row segments per channel
  constexpr unsigned TCOLS = wu_tmem_cols<KP, NP>();
  // kind::f16, FP32 accumulator, BF16 A and B, both MN-major (bits 15, 16)
  constexpr unsigned IDESC = umma_idesc_bf16(128, NT) | (1u << 15) | (1u << 16);
  constexpr unsigned TX = (unsigned)(NA + NB) * 1024u;  // copy bytes per block
  static_assert(NP % 16 == 0 && NT <= 256 && KC <= 4 && NC <= 4 && SPG % WR == 0, "shape");
  static_assert(wgrad_umma_smem<KP, NP>() <= 232448, "shared memory");
  // the last product group reads 16 KB from its start: inside the stage
  static_assert((NG - 1) * SPG * KC * 1024 + (WU_RB - 1) * KC * 1024 + 16 * 1024 <= SB, "operand span");
  extern __shared__ unsigned char wu_raw[];
  unsigned char* const sm = wu_raw + ((1024u - (cu_smem_u32(wu_raw) & 1023u)) & 1023u);
  unsigned long long* const bars = reinterpret_cast<unsigned long long*>(sm + NS * SB);
  unsigned long long* const full = bars;            // [NS] copies landed (TMA bytes)
  unsigned long long* const rot = bars + NS;        // [NS] rotated copies written (4 helper warps)
  unsigned long long* const empty = bars + 2 * NS;  // [NS] products done with the stage (commit)
  unsigned long long* const done = bars + 3 * NS;   // every product done (commit)
  unsigned* const s_tmem = reinterpret_cast<unsigned*>(bars + 3 * NS + 1);
  volatile int* const s_abort = reinterpret_cast<volatile int*>(s_tmem + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long nblk = (long long)batch * n * (n / WU_RB);
  const int nb = blockIdx.x < nblk ? (int)((nblk - 1 - blockIdx.x) / gridDim.x) + 1 : 0;
  auto fault = [&]() {
    atomicExch(&g_learned_fault, 1);
    *s_abort = 1;
  };
  const bool drill = g_learned_drill != 0;
  const int polls = drill ? CU_DRILL_POLLS : CU_POLLS;
  double bsum = 0.0;  // helper threads: bias sum of their channel and row segment
  if (tid == 0) {
    for (int k = 0; k < 3 * NS + 1; ++k)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(cu_smem_u32(&bars[k])),
                   "r"(k >= NS && k < 2 * NS ? 4 : 1)
                   : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    *s_abort = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(cu_smem_u32(s_tmem)),
                 "r"(TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *s_tmem;

  if (warp == 1) {
    // ---- copies ----
    int i = 0;
    for (; i < nb && !drill; ++i) {
      const int buf = i % NS;
      if (i >= NS && !__all_sync(0xffffffffu, cu_wait(&empty[buf], (unsigned)((i / NS - 1) & 1), polls))) {
        if (lane == 0) fault();
        break;
      }
      if (*s_abort) break;
      const long long blk = blockIdx.x + (long long)i * gridDim.x;
      const int smp = (int)(blk / (n * (n / WU_RB))), r = (int)(blk - (long long)smp * n * (n / WU_RB));
      const int z = r / (n / WU_RB), y0 = WU_RB * (r - z * (n / WU_RB));
      unsigned char* const A = sm + buf * SB;
      unsigned char* const B = A + AB;
      if (lane == 0) cu_expect_tx(&full[buf], TX);
      __syncwarp();
      for (int j = lane; j < NA + NB; j += 32) {
        if (j < NA) {
          // window row w of dz (layout [dz][w][chunk])
          const int dz = j / (WR * KC), w = (j / KC) % WR, c = j % KC;
          int yy = y0 - 1 + w, zz = z + dz - 1;
          yy = yy < 0 ? yy + n : (yy >= n ? yy - n : yy);
          zz = zz < 0 ? zz + n : (zz >= n ? zz - n : zz);
          cu_tma_3d(A + j * 1024, &maps.a[c], 0, 0, (smp * n + zz) * n + yy, &full[buf]);
        } else {
          // the unrotated copy (dx = 0) of output row rr of g
          const int rr = (j - NA) / NC, c = (j - NA) % NC;
          cu_tma_3d(B + (rr * 3 * NC + NC + c) * 1024, &maps.b[c], 0, 0, (smp * n + z) * n + y0 + rr, &full[buf]);
        }
      }
    }
    // copies in flight: the last NS issued stages land (bounded)
    for (int j = i - NS; j < i; ++j)
      if (j >= 0 && !__all_sync(0xffffffffu, cu_wait(&full[j % NS], (unsigned)((j / NS) & 1), polls)) && lane == 0)
        fault();
  } else if (warp == 0) {
    // ---- products ----
    if (lane == 0) {
      int i = 0;
      for (; i < nb; ++i) {
        const int buf = i % NS;
        if (!cu_wait(&rot[buf], (unsigned)((i / NS) & 1), polls)) {
          fault();
          break;
        }
        if (*s_abort) break;
        tc_fence_after();
        // MN-major, no swizzle: 8-channel chunks 1 KB apart (stride byte
        // offset), 8-voxel groups 128 bytes apart (leading byte offset)
        const unsigned a0 = cu_smem_u32(sm + buf * SB), b0 = a0 + AB;
#pragma unroll
        for (int rr = 0; rr < WU_RB; ++rr)
#pragma unroll
          for (int gr = 0; gr < NG; ++gr)
#pragma unroll
            for (int kk = 0; kk < CU_N / 16; ++kk)
              umma_bf16(tmem + (unsigned)(gr * NT),
                        umma_sdesc(a0 + gr * SPG * KC * 1024 + rr * KC * 1024 + kk * 256, 128, 1024),
                        umma_sdesc(b0 + rr * 3 * NC * 1024 + kk * 256, 128, 1024), IDESC, (i | rr | kk) != 0);
        umma_commit(&empty[buf]);
      }
      if (i > 0) {
        umma_commit(done);
        if (!cu_wait(done, 0u, polls)) fault();
      }
    }
    __syncwarp();
  } else {
    // ---- rotations of g: dx = -1 (copy 0, g[x + 1]) and dx = +1 (copy 2, g[x - 1]) ----
    const int ht = tid - 64;
    const int bco = ht % NP, bseg = ht / NP;
    for (int i = 0; i < nb; ++i) {
      const int buf = i % NS;
      if (!__all_sync(0xffffffffu, cu_wait(&full[buf], (unsigned)((i / NS) & 1), polls))) {
        if (lane == 0) fault();
        break;
      }
      if (*s_abort) break;
      unsigned char* const B = sm + buf * SB + AB;
#pragma unroll
      for (int rr = 0; rr < WU_RB; ++rr) {
        unsigned char* const Br = B + rr * 3 * NC * 1024;
        const uint4* const src = reinterpret_cast<const uint4*>(Br + NC * 1024);
        {
          // bias gradient: channel bco over the row segment bseg
          const __nv_bfloat16* const gb =
              reinterpret_cast<const __nv_bfloat16*>(src) + (bco / 8) * CU_N * 8 + bco % 8;
          float fs = 0.f;
#pragma unroll 4
          for (int x = bseg * SL; x < (bseg + 1) * SL; ++x) fs += __bfloat162float(gb[x * 8]);
          bsum += (double)fs;
        }
        for (int p = ht; p < 2 * NC * CU_N; p += 128) {
          const int h = p / (NC * CU_N), rem = p - h * (NC * CU_N), c = rem / CU_N, x = rem % CU_N;
          const int xs = h == 0 ? (x + 1) % CU_N : (x + CU_N - 1) % CU_N;
          reinterpret_cast<uint4*>(Br + ((2 * h) * NC + c) * 1024)[x] = src[c * CU_N + xs];
        }
      }
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // generic writes -> tensor-core reads
      __syncwarp();
      if (lane == 0) cu_arrive(&rot[buf]);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  // ---- bias partial of this CTA: the segments of each channel in order (the
  // first stage's A buffer is free: no copy or product is in flight) ----
  double* const red = reinterpret_cast<double*>(sm);
  if (warp >= 2) red[(tid - 64) / NP * NP + (tid - 64) % NP] = bsum;
  __syncthreads();
  if (warp >= 2 && tid - 64 < NP && !*s_abort) {
    double b = 0.0;
    for (int sg = 0; sg < SEGS; ++sg) b += red[sg * NP + tid - 64];
    bpart[(long long)blockIdx.x * NP + tid - 64] = b;
  }
  // ---- partial of this CTA: accumulator row m = (dz, window row w, ci), column (dx, co) ----
  if (warp >= 2 && !*s_abort && nb > 0) {
    const int q = warp & 3, m = 32 * q + lane;
#pragma unroll 1
    for (int gr = 0; gr < NG; ++gr) {
      const int slot = m / KP, ci = m % KP;
      const int dzp = gr * (SPG / WR) + slot / WR, w = slot % WR;  // dz + 1, dy + 1 = w
#pragma unroll 1
      for (int c0 = 0; c0 < NT; c0 += 16) {
        unsigned r[16];
        tmem_ld_nowait<16>(tmem + ((unsigned)(32 * q) << 16) + (unsigned)(gr * NT + c0), r);
        tmem_wait_ld();
        if (dzp < 3 && w < 3) {
          const int t = c0 / NP, co0 = c0 - t * NP;
          float* const o =
              part + ((long long)blockIdx.x * NET_TAPS + dzp * 9 + w * 3 + t) * (KP * NP) + ci * NP + co0;
#pragma unroll
          for (int j = 0; j < 16; j += 4)
            *reinterpret_cast<float4*>(o + j) = make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]),
                                                            __uint_as_float(r[j + 2]), __uint_as_float(r[j + 3]));
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TCOLS) : "memory");
  }
}

// Row maps of a [batch][64^3][ch] BF16 tensor per 8-channel chunk (boxes of 8
// channels x 64 voxels); false when they cannot be made.
static bool wgrad_row_maps(const __nv_bfloat16* t, int ch, int batch, CUtensorMap* m) {
  if ((reinterpret_cast<uintptr_t>(t) & 15) != 0) return false;
  const cuuint64_t dims[3] = {8, (cuuint64_t)CU_N, (cuuint64_t)batch * CU_N * CU_N};
  const cuuint64_t strides[2] = {(cuuint64_t)ch * 2, (cuuint64_t)CU_N * ch * 2};
  const cuuint32_t box[3] = {8, (cuuint32_t)CU_N, 1};
  for (int c = 0; c < ch / 8; ++c)
    if (!encode_tiled_map(&m[c], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, t + c * 8, dims, strides, box)) return false;
  return true;
}

// fold partials over chunks; bias gradient from the g sums of tap 13 (centre)
template <int KP, int NP>
__global__ void wgrad_fold_kernel(int nchunk, const float* __restrict__ part, float* __restrict__ dW) {
  // four lanes per output: lane q sums chunks q, q + 4, ... in order, then
  // the four sums combine in a fixed order (deterministic)
  constexpr int PAIRS = KP * NP;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t >> 2, q = t & 3;
  double s = 0;
  if (i < NET_TAPS * PAIRS)
    for (int c = q; c < nchunk; c += 4) s += (double)part[(long long)c * NET_TAPS * PAIRS + i];
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  if (q == 0 && i < NET_TAPS * PAIRS) dW[i] = (float)s;
}

// Bias gradient db[co] = sum_v g[v][co]: BG_BLOCKS blocks, each thread one
// channel of 256/NP voxel lanes (coalesced rows of g), FP64 sums folded in a
// fixed order (block tree, then blocks in order), so the result is
// deterministic.
constexpr int BG_BLOCKS = 304;

template <int NP>
__global__ void __launch_bounds__(256) bgrad_partial_kernel(long long V, const __nv_bfloat16* __restrict__ g,
                                                            double* __restrict__ part) {
  constexpr int LANES = 256 / NP;
  __shared__ double red[256];
  const int co = threadIdx.x % NP, vl = threadIdx.x / NP;
  double s = 0;
  for (long long v = (long long)blockIdx.x * LANES + vl; v < V; v += (long long)gridDim.x * LANES)
    s += (double)__bfloat162float(g[v * NP + co]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = LANES / 2; o > 0; o >>= 1) {
    if (vl < o) red[threadIdx.x] += red[threadIdx.x + o * NP];
    __syncthreads();
  }
  if (vl == 0) part[(long long)blockIdx.x * NP + co] = red[threadIdx.x];
}

template <int NP>
__global__ void bgrad_fold_kernel(int nblk, const double* __restrict__ part, float* __restrict__ db) {
  // one warp per channel: lane l sums partials l, l + 32, ... in order, then
  // a fixed shuffle tree (deterministic)
  const int co = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (co >= NP) return;
  double s = 0;
  for (int b = lane; b < nblk; b += 32) s += part[(long long)b * NP + co];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) db[co] = (float)s;
}

// ---------------------------------------------------------------------------
// Packing, loss, Adam, weight layouts
// ---------------------------------------------------------------------------
// fields [b][3][n^3] (T) -> channel-last bf16 [b n^3][KP], scaled
template <typename T>
__global__ void pack_input_kernel(long long V, long long N, const T* __restrict__ f, double scale,
                                  __nv_bfloat16* __restrict__ out, int KP) {
  // one voxel row per thread, written as 16-byte pieces (KP % 8 == 0)
  const IdxDiv dN(N);
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const long long b = dN.div(v), r = v - b * N;
    __nv_bfloat16 row[8];
#pragma unroll
    for (int c = 0; c < 8; ++c)
      row[c] = __float2bfloat16(c < 3 ? (float)((double)f[(b * 3 + c) * N + r] * scale) : 0.f);
    uint4* o = reinterpret_cast<uint4*>(out + v * KP);
    o[0] = *reinterpret_cast<const uint4*>(row);
    for (int c = 1; c < KP / 8; ++c) o[c] = make_uint4(0, 0, 0, 0);
  }
}

constexpr int OUTP = 16;  // padded output channels

// net output [V][OUTP] (FP32, normalised) -> fields [b][3][n^3] (T) * scale
template <typename T>
__global__ void unpack_output_kernel(long long V, long long N, const float* __restrict__ o, double scale,
                                     T* __restrict__ f) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const long long b = v / N, r = v - b * N;
    for (int c = 0; c < 3; ++c) f[(b * 3 + c) * N + r] = (T)((double)o[v * OUTP + c] * scale);
  }
}

// g = 2 (out - target*tscale) / count (bf16, [V][OUTP]); per-block squared-error partials
template <typename T>
__global__ void loss_grad_kernel(long long V, long long N, const float* __restrict__ out, const T* __restrict__ tgt,
                                 double tscale, double inv_count, __nv_bfloat16* __restrict__ g,
                                 double* __restrict__ part) {
  __shared__ double red[256];
  double s = 0;
  const IdxDiv dN(N);
  const float gs = (float)(2.0 * inv_count);
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const long long b = dN.div(v), r = v - b * N;
    // the output row's first 4 words in one 16-byte load; the gradient row
    // (3 values, then zeros) in 16-byte pieces
    const float4 o4 = *reinterpret_cast<const float4*>(out + v * OUTP);
    const float oc[3] = {o4.x, o4.y, o4.z};
    __nv_bfloat16 row[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      float d = 0.f;
      if (c < 3) d = oc[c] - (float)((double)tgt[(b * 3 + c) * N + r] * tscale);
      if (c < 3) s += (double)d * d;
      row[c] = __float2bfloat16(gs * d);
    }
    uint4* gr = reinterpret_cast<uint4*>(g + v * OUTP);
    gr[0] = *reinterpret_cast<const uint4*>(row);
    gr[1] = make_uint4(0, 0, 0, 0);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Sum of np partials in a fixed order: one block of 256 threads, each thread
// a strided subset in order, then a fixed tree.
__global__ void __launch_bounds__(256) sum_kernel(int np, const double* __restrict__ part, double scale,
                                                  double* __restrict__ out) {
  __shared__ double red[256];
  double s = 0;
  for (int i = threadIdx.x; i < np; i += 256) s += part[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0] * scale;
}

// Adam (Kingma & Ba 2015): m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2;
// w -= lr mhat / (sqrt(vhat) + eps)
__global__ void adam_kernel(int count, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float c1, float c2, float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// master W[tap][KP][NP] (FP32, padded entries zero) -> forward
// Wt[tap][co][ci] and input-gradient Wb[tap][ci][co] = W[26 - tap][ci][co]
// (n = ci, k = co), both bf16
__global__ void refresh_weights_kernel(const float* __restrict__ W, int KP, int NP, __nv_bfloat16* __restrict__ Wt,
                                       __nv_bfloat16* __restrict__ Wb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int tot = NET_TAPS * KP * NP;
  if (i >= tot) return;
  {
    const int tap = i / (NP * KP), r = i - tap * NP * KP;
    const int co = r / KP, ci = r - co * KP;
    Wt[i] = __float2bfloat16(W[((long long)tap * KP + ci) * NP + co]);
  }
  {
    const int tap = i / (KP * NP), r = i - tap * KP * NP;
    const int ci = r / NP, co = r - ci * NP;
    Wb[i] = __float2bfloat16(W[((long long)(26 - tap) * KP + ci) * NP + co]);
  }
}

}  // namespace exc

// ---------------------------------------------------------------------------
// Host side: the network object and its C ABI
// ---------------------------------------------------------------------------
struct exc_net {
  // padded layer shapes: (KP, NP) = (16, 32), (32, 32), (32, 16)
  static constexpr int K1 = 16, N1 = 32, K2 = 32, N2 = 32, K3 = 32, N3 = exc::OUTP;
  static constexpr long long W1 = 27LL * K1 * N1, W2 = 27LL * K2 * N2, W3 = 27LL * K3 * N3;
  static constexpr long long NPARAM = W1 + N1 + W2 + N2 + W3 + N3;
  float* params = nullptr;  // [W1 b1 W2 b2 W3 b3], FP32 master, padded entries zero
  float* grads = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  __nv_bfloat16* wbf = nullptr;  // Wt1 Wb1 Wt2 Wb2 Wt3 Wb3
  int adam_t = 0;
  int conv_engine = 0;  // 0: tcgen05 convolutions on 64^3 grids; 1: mma.sync only
  double in_scale = 1.0, out_scale = 1.0;
  long long vcap = 0;  // voxel capacity of the workspace
  int ws_gen = 0;       // bumped whenever the workspace moves (captured graphs must re-capture)
  __nv_bfloat16 *x0 = nullptr, *a1 = nullptr, *a2 = nullptr, *g3 = nullptr, *gp2 = nullptr, *gp1 = nullptr;
  // GELU'(pre-activation) of the hidden layers (BF16), written by a training
  // forward pass for the backward pass
  __nv_bfloat16 *dg1 = nullptr, *dg2 = nullptr;
  float *out = nullptr, *wpart = nullptr;
  double* lpart = nullptr;  // loss partials + result
  float* W(int l) { return params + (l == 0 ? 0 : l == 1 ? W1 + N1 : W1 + N1 + W2 + N2); }
  float* B(int l) { return W(l) + (l == 0 ? W1 : l == 1 ? W2 : W3); }
  float* dW(int l) { return grads + (W(l) - params); }
  float* dB(int l) { return grads + (B(l) - params); }
  __nv_bfloat16* Wt(int l) { return wbf + (l == 0 ? 0 : l == 1 ? 2 * W1 : 2 * (W1 + W2)); }
  __nv_bfloat16* Wb(int l) { return Wt(l) + (l == 0 ? W1 : l == 1 ? W2 : W3); }
};

namespace exc {

static void free_workspace(exc_net* net) {
  void* ps[] = {net->x0, net->a1, net->a2, net->g3, net->gp2, net->gp1, net->dg1, net->dg2, net->out, net->wpart,
                net->lpart};
  for (void* p : ps)
    if (p) cudaFree(p);
  net->x0 = net->a1 = net->a2 = net->g3 = net->gp2 = net->gp1 = nullptr;
  net->dg1 = net->dg2 = nullptr;
  net->out = net->wpart = nullptr;
  net->lpart = nullptr;
  net->vcap = 0;
}

static int ensure_workspace(exc_net* net, long long V) {
  if (V <= net->vcap) return EXC_OK;
  cudaDeviceSynchronize();
  free_workspace(net);
  const long long nchunk = std::max<long long>((V + WG_CHUNK - 1) / WG_CHUNK, WT_CTAS);
  bool ok = cudaMalloc(&net->x0, V * exc_net::K1 * 2) == cudaSuccess &&
            cudaMalloc(&net->a1, V * exc_net::N1 * 2) == cudaSuccess &&
            cudaMalloc(&net->a2, V * exc_net::N2 * 2) == cudaSuccess &&
            cudaMalloc(&net->g3, V * exc_net::N3 * 2) == cudaSuccess &&
            cudaMalloc(&net->gp2, V * exc_net::N2 * 2) == cudaSuccess &&
            cudaMalloc(&net->gp1, V * exc_net::N1 * 2) == cudaSuccess &&
            cudaMalloc(&net->dg1, V * exc_net::N1 * 2) == cudaSuccess &&
            cudaMalloc(&net->dg2, V * exc_net::N2 * 2) == cudaSuccess &&
            cudaMalloc(&net->out, V * exc_net::N3 * 4) == cudaSuccess &&
            cudaMalloc(&net->wpart, nchunk * 27 * 32 * 32 * 4 + (long long)WT_CTAS * 2 * 32 * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&net->lpart, (1024 + 8) * sizeof(double)) == cudaSuccess;
  if (!ok) {
    free_workspace(net);
    set_last_error("out of device memory (network workspace)");
    return EXC_ERR_OOM;
  }
  net->vcap = V;
  net->ws_gen += 1;
  return EXC_OK;
}

int net_reserve(exc_net* net, long long V) { return ensure_workspace(net, V); }
int net_workspace_gen(const exc_net* net) { return net->ws_gen; }

static cudaError_t refresh(exc_net* net, cudaStream_t st) {
  const int ks[3] = {exc_net::K1, exc_net::K2, exc_net::K3}, ns[3] = {exc_net::N1, exc_net::N2, exc_net::N3};
  for (int l = 0; l < 3; ++l) {
    const int tot = 27 * ks[l] * ns[l];
    refresh_weights_kernel<<<(tot + 255) / 256, 256, 0, st>>>(net->W(l), ks[l], ns[l], net->Wt(l), net->Wb(l));
  }
  return cudaGetLastError();
}


// forward from the packed input x0; leaves a1, a2, out and, for training,
// the GELU derivatives dg1, dg2
static cudaError_t forward_packed(exc_net* net, long long V, int n, bool train, cudaStream_t st) {
  conv_launch<16, 32, 0>(net->conv_engine, V, n, net->x0, net->Wt(0), net->B(0), nullptr, net->a1,
                         train ? net->dg1 : nullptr, 32, st);
  conv_launch<32, 32, 0>(net->conv_engine, V, n, net->a1, net->Wt(1), net->B(1), nullptr, net->a2,
                         train ? net->dg2 : nullptr, 32, st);
  conv_launch<32, 16, 1>(net->conv_engine, V, n, net->a2, net->Wt(2), net->B(2), net->out, nullptr, nullptr, 3, st);
  return cudaGetLastError();
}

template <int KP, int NP>
static cudaError_t wgrad(exc_net* net, int l, long long V, int n, const __nv_bfloat16* in, const __nv_bfloat16* g,
                         cudaStream_t st) {
  int nchunk;
  const long long N = (long long)n * n * n;
  if (net->conv_engine == 0 && n == CU_N) {
    const int batch = (int)(V / N);
    WgMaps maps;
    if (batch > 0 && wgrad_row_maps(in, KP, batch, maps.a) && wgrad_row_maps(g, NP, batch, maps.b)) {
      nchunk = (int)std::min<long long>((long long)batch * n * (n / WU_RB), 152);
      // bias partials (one per CTA) after the weight partials
      double* bpart = reinterpret_cast<double*>(net->wpart + (size_t)WT_CTAS * NET_TAPS * 32 * 32);
      wgrad_umma_kernel<KP, NP><<<nchunk, WU_THREADS, wgrad_umma_smem<KP, NP>(), st>>>(batch, maps, net->wpart,
                                                                                       bpart);
      wgrad_fold_kernel<KP, NP><<<(4 * 27 * KP * NP + 255) / 256, 256, 0, st>>>(nchunk, net->wpart, net->dW(l));
      bgrad_fold_kernel<NP><<<1, 32 * NP, 0, st>>>(nchunk, bpart, net->dB(l));
      return cudaGetLastError();
    }
  }
  if (n % 8 == 0) {
    // all taps per CTA over 8 x 2 x 4 voxel blocks, one persistent CTA per
    // SM; the bias partials follow the weight partials in the buffer
    const long long nblk = V / WT_BV;
    nchunk = (int)std::min<long long>(nblk, WT_CTAS);
    double* bpart = reinterpret_cast<double*>(net->wpart + (size_t)WT_CTAS * NET_TAPS * 32 * 32);
    wgrad_tile_kernel<KP, NP><<<nchunk, WT_THREADS, wgrad_tile_smem<KP, NP>(), st>>>((int)(V / N), n, in, g,
                                                                                      net->wpart, bpart);
    wgrad_fold_kernel<KP, NP><<<(4 * 27 * KP * NP + 255) / 256, 256, 0, st>>>(nchunk, net->wpart, net->dW(l));
    bgrad_fold_kernel<NP><<<1, 32 * NP, 0, st>>>(2 * nchunk, bpart, net->dB(l));
    return cudaGetLastError();
  } else {
    nchunk = (int)((V + WG_CHUNK - 1) / WG_CHUNK);
    wgrad_partial_kernel<KP, NP><<<dim3(nchunk, 27), 128, 0, st>>>(V, n, in, g, net->wpart);
  }
  wgrad_fold_kernel<KP, NP><<<(4 * 27 * KP * NP + 255) / 256, 256, 0, st>>>(nchunk, net->wpart, net->dW(l));
  // the weight-gradient partials are folded by now: reuse their buffer
  double* bpart = reinterpret_cast<double*>(net->wpart);
  bgrad_partial_kernel<NP><<<BG_BLOCKS, 256, 0, st>>>(V, g, bpart);
  bgrad_fold_kernel<NP><<<1, 32 * NP, 0, st>>>(BG_BLOCKS, bpart, net->dB(l));
  return cudaGetLastError();
}

// loss, backward; gradients into net->grads, loss into lpart[1024]
template <typename T>
static cudaError_t backward(exc_net* net, long long V, int n, long long N, const T* target, cudaStream_t st) {
  const int lb = (int)std::min<long long>((V + 255) / 256, 1024);
  loss_grad_kernel<T><<<lb, 256, 0, st>>>(V, N, net->out, target, 1.0 / net->out_scale, 1.0 / (3.0 * (double)V),
                                          net->g3, net->lpart);
  sum_kernel<<<1, 256, 0, st>>>(lb, net->lpart, 1.0 / (3.0 * (double)V), net->lpart + 1024);
  cudaError_t e = wgrad<32, 16>(net, 2, V, n, net->a2, net->g3, st);
  // input gradient of layer 3 times GELU'(pre2)
  conv_launch<16, 32, 2>(net->conv_engine, V, n, net->g3, net->Wb(2), nullptr, nullptr, net->gp2, net->dg2, 32, st);
  if (e == cudaSuccess) e = wgrad<32, 32>(net, 1, V, n, net->a1, net->gp2, st);
  conv_launch<32, 32, 2>(net->conv_engine, V, n, net->gp2, net->Wb(1), nullptr, nullptr, net->gp1, net->dg1, 32, st);
  if (e == cudaSuccess) e = wgrad<16, 32>(net, 0, V, n, net->x0, net->gp1, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e;
}

template <typename T>
static int net_forward_t(exc_net* net, int batch, int n, const T* u, T* m, cudaStream_t st) {
  const long long N = (long long)n * n * n, V = batch * N;
  int rc = ensure_workspace(net, V);
  if (rc) return rc;
  const int gb = (int)std::min<long long>((V + 255) / 256, 152LL * 32);
  pack_input_kernel<T><<<gb, 256, 0, st>>>(V, N, u, 1.0 / net->in_scale, net->x0, exc_net::K1);
  cudaError_t e = forward_packed(net, V, n, false, st);
  if (e == cudaSuccess) {
    unpack_output_kernel<T><<<gb, 256, 0, st>>>(V, N, net->out, net->out_scale, m);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

template <typename T>
static int net_grad_t(exc_net* net, int batch, int n, const T* u, const T* m, cudaStream_t st) {
  const long long N = (long long)n * n * n, V = batch * N;
  int rc = ensure_workspace(net, V);
  if (rc) return rc;
  const int gb = (int)std::min<long long>((V + 255) / 256, 152LL * 32);
  pack_input_kernel<T><<<gb, 256, 0, st>>>(V, N, u, 1.0 / net->in_scale, net->x0, exc_net::K1);
  cudaError_t e = forward_packed(net, V, n, true, st);
  if (e == cudaSuccess) e = backward<T>(net, V, n, N, m, st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

// He-normal initial weights from the project's counter generator (host)
static double host_normal(uint64_t seed, uint64_t i) {
  auto sm = [](uint64_t x) {
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
  };
  const uint64_t base = seed * 0x9E3779B97F4A7C15ull;
  double u1 = ((double)(sm(base + 2 * i) >> 11) + 0.5) * 0x1.0p-53;
  double u2 = ((double)(sm(base + 2 * i + 1) >> 11) + 0.5) * 0x1.0p-53;
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
}

}  // namespace exc

using namespace exc;

namespace exc {

// Shared-memory opt-in of the weight-resident convolutions (before any
// stream capture).
template <int KP, int NP, int EPI>
static cudaError_t conv_res_attr() {
  return cudaFuncSetAttribute(conv_res_kernel<KP, NP, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)conv_res_smem<KP, NP>());
}
template <int NP, int EPI>
static cudaError_t conv_umma_attr() {
  return cudaFuncSetAttribute(conv_umma_kernel<NP, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)conv_umma_smem<NP>());
}
template <int KP, int NP>
static cudaError_t wgrad_umma_attr() {
  return cudaFuncSetAttribute(wgrad_umma_kernel<KP, NP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)wgrad_umma_smem<KP, NP>());
}
template <int KP, int NP>
static cudaError_t wgrad_tile_attr() {
  return cudaFuncSetAttribute(wgrad_tile_kernel<KP, NP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)wgrad_tile_smem<KP, NP>());
}
static int configure_learned() {
  static std::mutex mu;
  static bool done[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    set_last_error("no usable CUDA device");
    return EXC_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return EXC_OK;
  cudaError_t e = conv_res_attr<16, 32, 0>();
  if (e == cudaSuccess) e = wgrad_tile_attr<16, 32>();
  if (e == cudaSuccess) e = wgrad_tile_attr<32, 32>();
  if (e == cudaSuccess) e = wgrad_tile_attr<32, 16>();
  if (e == cudaSuccess) e = conv_res_attr<32, 32, 0>();
  if (e == cudaSuccess) e = conv_res_attr<32, 16, 1>();
  if (e == cudaSuccess) e = conv_res_attr<16, 32, 2>();
  if (e == cudaSuccess) e = conv_res_attr<32, 32, 2>();
  if (e == cudaSuccess) e = conv_umma_attr<32, 0>();
  if (e == cudaSuccess) e = conv_umma_attr<16, 1>();
  if (e == cudaSuccess) e = conv_umma_attr<32, 2>();
  if (e == cudaSuccess) e = wgrad_umma_attr<16, 32>();
  if (e == cudaSuccess) e = wgrad_umma_attr<32, 32>();
  if (e == cudaSuccess) e = wgrad_umma_attr<32, 16>();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  done[dev] = true;
  return EXC_OK;
}

// Read and clear the flag of a tensor-core wait that gave up.
int learned_set_drill(int on) {
  cudaError_t e = cudaMemcpyToSymbol(g_learned_drill, &on, sizeof(int));
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

int learned_fault_take(int* flag) {
  int v = 0, zero = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_learned_fault, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_learned_fault, &zero, sizeof(int));
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  *flag = v;
  return EXC_OK;
}

}  // namespace exc

extern "C" {

int exc_net_create(uint64_t seed, exc_net** out) {
  if (!out) { set_last_error("null argument"); return EXC_ERR_ARG; }
  *out = nullptr;
  int rc = configure_device();
  if (rc == EXC_OK) rc = configure_learned();
  if (rc) return rc;
  exc_net* net = new exc_net();
  const size_t pb = exc_net::NPARAM * sizeof(float);
  const size_t wb = 2 * (exc_net::W1 + exc_net::W2 + exc_net::W3) * sizeof(__nv_bfloat16);
  if (cudaMalloc(&net->params, pb) != cudaSuccess || cudaMalloc(&net->grads, pb) != cudaSuccess ||
      cudaMalloc(&net->adam_m, pb) != cudaSuccess || cudaMalloc(&net->adam_v, pb) != cudaSuccess ||
      cudaMalloc(&net->wbf, wb) != cudaSuccess) {
    exc_net_destroy(net);
    set_last_error("out of device memory (network)");
    return EXC_ERR_OOM;
  }
  std::vector<float> h(exc_net::NPARAM, 0.f);
  const int cin[3] = {3, 32, 32}, cout[3] = {32, 32, 3};
  const int ks[3] = {exc_net::K1, exc_net::K2, exc_net::K3}, ns[3] = {exc_net::N1, exc_net::N2, exc_net::N3};
  uint64_t ctr = 0;
  for (int l = 0; l < 3; ++l) {
    const double std_ = std::sqrt(2.0 / (27.0 * cin[l]));
    float* W = h.data() + (net->W(l) - net->params);
    for (int t = 0; t < 27; ++t)
      for (int ci = 0; ci < cin[l]; ++ci)
        for (int co = 0; co < cout[l]; ++co) W[((size_t)t * ks[l] + ci) * ns[l] + co] = (float)(std_ * host_normal(seed, ctr++));
  }
  cudaMemcpy(net->params, h.data(), pb, cudaMemcpyHostToDevice);
  cudaMemset(net->grads, 0, pb);
  cudaMemset(net->adam_m, 0, pb);
  cudaMemset(net->adam_v, 0, pb);
  cudaError_t e = refresh(net, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { exc_net_destroy(net); set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  *out = net;
  return EXC_OK;
}

int exc_net_set_conv_engine(exc_net* net, int engine) {
  if (!net || engine < 0 || engine > 1) { set_last_error("invalid network or convolution engine"); return EXC_ERR_ARG; }
  net->conv_engine = engine;
  return EXC_OK;
}

int exc_net_destroy(exc_net* net) {
  if (!net) return EXC_OK;
  cudaDeviceSynchronize();
  free_workspace(net);
  if (net->params) cudaFree(net->params);
  if (net->grads) cudaFree(net->grads);
  if (net->adam_m) cudaFree(net->adam_m);
  if (net->adam_v) cudaFree(net->adam_v);
  if (net->wbf) cudaFree(net->wbf);
  delete net;
  return EXC_OK;
}

int exc_net_param_count(void) { return (int)exc_net::NPARAM; }

int exc_net_set_scales(exc_net* net, double in_scale, double out_scale) {
  if (!net || !(in_scale > 0) || !(out_scale > 0)) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  net->in_scale = in_scale;
  net->out_scale = out_scale;
  return EXC_OK;
}

int exc_net_get_params(exc_net* net, float* host, int count) {
  if (!net || !host || count != (int)exc_net::NPARAM) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  cudaError_t e = cudaMemcpy(host, net->params, count * sizeof(float), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

int exc_net_set_params(exc_net* net, const float* host, int count) {
  if (!net || !host || count != (int)exc_net::NPARAM) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  cudaError_t e = cudaMemcpy(net->params, host, count * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = refresh(net, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  net->adam_t = 0;
  if (e == cudaSuccess) e = cudaMemset(net->adam_m, 0, exc_net::NPARAM * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(net->adam_v, 0, exc_net::NPARAM * sizeof(float));
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

int exc_net_forward(exc_net* net, int precision, int batch, int n, const void* u, void* m, void* stream) {
  if (!net || !u || !m || batch < 1 || n < 1) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == EXC_F64) return net_forward_t<double>(net, batch, n, (const double*)u, (double*)m, st);
  if (precision == EXC_F32) return net_forward_t<float>(net, batch, n, (const float*)u, (float*)m, st);
  set_last_error("bad precision");
  return EXC_ERR_ARG;
}

int exc_net_gradients(exc_net* net, int precision, int batch, int n, const void* u, const void* m, float* grad_host,
                      double* loss_host, void* stream) {
  if (!net || !u || !m || batch < 1 || n < 1) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  int rc = precision == EXC_F64 ? net_grad_t<double>(net, batch, n, (const double*)u, (const double*)m, st)
                                : net_grad_t<float>(net, batch, n, (const float*)u, (const float*)m, st);
  if (rc) return rc;
  cudaError_t e = cudaSuccess;
  if (grad_host) e = cudaMemcpyAsync(grad_host, net->grads, exc_net::NPARAM * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && loss_host) e = cudaMemcpyAsync(loss_host, net->lpart + 1024, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

int exc_net_train_step(exc_net* net, int precision, int batch, int n, const void* u, const void* m, double lr,
                       double* loss_host, void* stream) {
  int rc = exc_net_gradients(net, precision, batch, n, u, m, nullptr, nullptr, stream);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  net->adam_t += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)net->adam_t), c2 = 1.f - std::pow(b2, (float)net->adam_t);
  const int cnt = (int)exc_net::NPARAM;
  adam_kernel<<<(cnt + 255) / 256, 256, 0, st>>>(cnt, net->params, net->grads, net->adam_m, net->adam_v, (float)lr, b1,
                                                 b2, c1, c2, 1e-8f);
  cudaError_t e = refresh(net, st);
  if (e == cudaSuccess && loss_host) e = cudaMemcpyAsync(loss_host, net->lpart + 1024, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

}  // extern "C"
