// RHS sweep: du = doadd*du - div sigma(u) (`stresstensor` + `tensordivergence!`,
// src/N.jl:94-160), marching along z.
//
// A CTA of 32 x 8 threads owns a PTX x PTY column of cells (PTY = 8 NC, NC
// consecutive rows per thread) and walks ptz planes (4 to 32).  Three plane buffers of u
// with a one-cell x/y halo sit in shared memory: planes z and z+1 are read
// while plane z+2 streams in with cp.async; each thread evaluates the six
// stress components at its own cells (the edge stresses s13, s23 and the
// diagonal s33 of the next plane are kept in registers for the next plane),
// six warps evaluate the halo stresses lane-parallel (one task per warp), and
// the divergence is formed from shared memory and registers.  Every stress
// value is computed once (plus the x/y halo), copy offsets are computed once
// per thread, and global loads and stores are row-contiguous.
#include <cuda.h>  // CUtensorMap (the encoder is reached through the runtime's driver entry point)

#include <cstring>
#include <mutex>

#include "internal.cuh"

namespace exc {

// Set when a wait for a TMA plane gave up (the copy never completed): the
// sweep then ran on incomplete data; read and cleared by exc_device_faults.
__device__ int g_rhs_tma_fault = 0;
// Wait drill (exc_debug_wait_drill bit 0): tiles that would take their planes
// by TMA issue no copy at all, so their plane waits give up after
// RHS_DRILL_POLLS polls with nothing in flight (the sweep's output is then
// not valid); 0 in normal operation.
__device__ int g_rhs_drill = 0;
constexpr int RHS_POLLS = 1 << 20, RHS_DRILL_POLLS = 64;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// 3-D tiled TMA load of one box (x, y, z) of the tensor map into shared memory
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

constexpr int PTX = 32, NWARP = 8;
constexpr int PBX = PTX + 2;  // plane box with one-cell halo (box x = x - x0 + 1)
// u rows in shared memory: box x index xb sits at xb + SH<T>, so the 32
// interior cells start on a 16-byte boundary and arrive by 16-byte copies
template <typename T> constexpr int SH = 16 / (int)sizeof(T) - 1;
template <typename T> constexpr int UROW = ((SH<T> + PBX) + 16 / (int)sizeof(T) - 1) / (16 / (int)sizeof(T)) *
                                           (16 / (int)sizeof(T));
// NC cells per thread along y: a tile is PTY = 8 NC rows
template <int NC> constexpr int PTYT = NWARP * NC;
template <int NC> constexpr int PBYT = PTYT<NC> + 2;

// One component plane of a buffer: PBY rows of UROW words, padded to a
// multiple of 128 bytes (TMA destinations); u[c][row] is the row's pointer.
template <typename T, int NC>
struct CompPlane {
  static constexpr int WORDS = PBYT<NC> * UROW<T>;
  static constexpr int PADDED = (WORDS * (int)sizeof(T) + 127) / 128 * 128 / (int)sizeof(T);
  T r[PBYT<NC>][UROW<T>];
  T pad[PADDED > WORDS ? PADDED - WORDS : 128 / (int)sizeof(T)];
  __device__ __forceinline__ const T* operator[](int row) const { return r[row]; }
  __device__ __forceinline__ T* operator[](int row) { return r[row]; }
};

template <typename T, int NC>
struct PlaneSmem {
  CompPlane<T, NC> u[3][3];  // [plane buffer][component]
  T s[5][PBYT<NC>][PBX];     // s11, s22, s12, s13, s23 of the current plane
  unsigned long long bar[3];  // TMA completion of each plane buffer
};
// dynamic shared memory of rhs_kernel: the struct plus room to align it to
// 128 bytes
template <typename T, int NC>
constexpr size_t plane_smem_bytes() {
  return sizeof(PlaneSmem<T, NC>) + 128;
}

// Stress values.  FP32 form (SC false): 4 sigma of the velocities in shared
// memory, the divergence takes 1/(4h).  FP64 form (SC true): the planes in
// shared memory hold w = s u - q (s = sqrt(kd), kd = 1/(4h), rho = rv s, q =
// rho/2, rv = 4 visc/h) and the stresses are -kd 4 sigma up to a constant per
// component, which the divergence's differences cancel:
//   -kd 4 sigma_ii = -(w_i + w_i(-e_i))^2 - 4 rho w_i(-e_i) - rho^2,
//   -kd 4 sigma_ij = -(w_i + w_i(+e_j)) (w_j + w_j(+e_i)) - 2 rho (w_i + w_j) - rho^2,
// (expand 4 sigma_ii = (a + b)^2 - 2 rv (a - b), 4 sigma_ij = (a + b)(c + d)
// - rv ((b - a) + (d - c)) with a = (w_a + q) / s ...): 3 and 5 FP64
// operations instead of 4 and 7, and no scaling in the divergence -- the FP64
// pipe, about two operations per clock per SM, bounds this sweep.
// Diagonal: a at the cell, b its lower neighbour along i; cd = rv2 (FP32
// form) or -4 rho (FP64 form).
template <bool SC, typename T>
__device__ __forceinline__ T sdiag_of(T a, T b, T cd) {
  const T s = a + b;
  if constexpr (SC) {
    return fma(-s, s, cd * b);
  } else {
    const T d = a - b;
    return s * s - cd * d;
  }
}
// Off-diagonal: a = u_i, b = u_i(+e_j), c = u_j, d = u_j(+e_i); co = rv (FP32
// form) or -2 rho (FP64 form).
template <bool SC, typename T>
__device__ __forceinline__ T soff_of(T a, T b, T c, T d, T co) {
  if constexpr (SC) return fma(-(a + b), c + d, co * (a + c));
  else return (a + b) * (c + d) - co * ((b - a) + (d - c));
}
// sigma_ii at box (bx, by) of plane buffer b (uses u_i at the cell and at -e_i)
template <bool SC, typename T, int I, typename U>
__device__ __forceinline__ T sdiag(const U& u, int bx, int by, T cd) {
  bx += SH<T>;
  return sdiag_of<SC>(u[I][by][bx], I == 0 ? u[0][by][bx - 1] : u[1][by - 1][bx], cd);
}
// sigma_12 at box (bx, by): u1, u1(+y), u2, u2(+x)
template <bool SC, typename T, typename U>
__device__ __forceinline__ T s12(const U& u, int bx, int by, T co) {
  bx += SH<T>;
  return soff_of<SC>(u[0][by][bx], u[0][by + 1][bx], u[1][by][bx], u[1][by][bx + 1], co);
}
// sigma_13 at box (bx, by): u1, u1(+z) [next plane], u3, u3(+x)
template <bool SC, typename T, typename U>
__device__ __forceinline__ T s13(const U& uc, const U& un, int bx, int by, T co) {
  bx += SH<T>;
  return soff_of<SC>(uc[0][by][bx], un[0][by][bx], uc[2][by][bx], uc[2][by][bx + 1], co);
}
// sigma_23 at box (bx, by): u2, u2(+z) [next plane], u3, u3(+y)
template <bool SC, typename T, typename U>
__device__ __forceinline__ T s23(const U& uc, const U& un, int bx, int by, T co) {
  bx += SH<T>;
  return soff_of<SC>(uc[1][by][bx], un[1][by][bx], uc[2][by][bx], uc[2][by + 1][bx], co);
}
// sigma_33 between planes: u3 of the upper plane and of the lower plane
template <bool SC, typename T>
__device__ __forceinline__ T s33(T up, T lo, T cd) {
  return sdiag_of<SC>(up, lo, cd);
}

template <typename T, int NC, bool DOADD>
__global__ void __launch_bounds__(PTX * NWARP, sizeof(T) == 4 ? 4 : 3)
rhs_kernel(int n, T inv_h, T visc, const T* __restrict__ u, T* __restrict__ du, SlotBatch sb, int zblocks, int ptz,
           const __grid_constant__ CUtensorMap umap, int have_map, int pre_shifted) {
  constexpr int PTY = PTYT<NC>, PBY = PBYT<NC>;
  constexpr int CSTRIDE = (int)(sizeof(CompPlane<T, NC>) / sizeof(T));
  extern __shared__ __align__(128) unsigned char rhs_smem[];
  PlaneSmem<T, NC>& sm =
      *reinterpret_cast<PlaneSmem<T, NC>*>(rhs_smem + ((128u - (smem_u32(rhs_smem) & 127u)) & 127u));
  const long long N = (long long)n * n * n;
  // slot of a batch of same-size solves (serving form): blockIdx.z = slot * zblocks + zb
  const int slot = blockIdx.z / zblocks;
  const int zb = blockIdx.z - slot * zblocks;
  if (sb.active && !sb.active[slot]) return;
  u += slot * sb.ustride;
  du += slot * sb.ustride;
  if (sb.visc) visc = reinterpret_cast<const T*>(sb.visc)[slot];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int lane = tx, warp = ty;
  const int x0 = blockIdx.x * PTX, y0 = blockIdx.y * PTY, z0 = zb * ptz;
  // FP32: stresses kept as 4 sigma (rv = 4 visc / h), the divergence takes
  // 1/(4h).  FP64 (SC): shared memory holds w = s u - q, stresses are -kd 4
  // sigma up to constants (see sdiag_of / soff_of)
  constexpr bool SC = sizeof(T) == 8;
  const T kd = (T)0.25 * inv_h;
  const T rv = (T)4 * visc * inv_h;
  const Fp64Shift fs = fp64_shift((double)inv_h, (double)visc);
  const T sq = SC ? (T)fs.sq : (T)1;
  const T rho = (T)fs.rho;
  const T qs = (T)fs.qs;
  const T cd = SC ? (T)-4 * rho : (T)2 * rv;
  const T co = SC ? (T)-2 * rho : rv;
  auto wrap = [n](int g) { return g < 0 ? g + n : (g >= n ? g - n : g); };
  auto wrapm = [n](int g) { return ((g % n) + n) % n; };
  const bool big = n >= PBX;
  // asynchronous copy of plane gz (with halo) into buffer buf; the caller
  // commits and waits (cp_async_wait_all) before the __syncthreads that
  // publishes it.  Full x tiles of a grid whose rows are 16-byte multiples
  // copy each box row as NV + 2 aligned 16-byte pieces: the interior, the
  // piece ending at x0 - 1 (left halo in its last word) and the piece starting
  // at x0 + PTX (right halo in its first word).  Each thread's pieces are the
  // same in every plane: their offsets are computed once, and a plane adds
  // gz n^2.  Other tiles copy word by word.
  constexpr int VE = 16 / (int)sizeof(T), NV = PTX / VE;
  constexpr int NPIECE = 3 * PBY * (NV + 2);
  constexpr int NSLOT = (NPIECE + PTX * NWARP - 1) / (PTX * NWARP);
  const bool vec = big && x0 + PTX <= n && (n % VE) == 0 && (reinterpret_cast<uintptr_t>(u) & 15) == 0;
  const int tid = ty * PTX + tx;
  long long goff[NSLOT];
  int soff[NSLOT];
  if (vec) {
#pragma unroll
    for (int i = 0; i < NSLOT; ++i) {
      const int t = tid + i * PTX * NWARP;
      goff[i] = -1;
      soff[i] = 0;
      if (t < NPIECE) {
        const int c = t / (PBY * (NV + 2));
        const int rem = t - c * (PBY * (NV + 2));
        const int rr = rem / (NV + 2), j = rem - rr * (NV + 2);
        const int gy = wrap(y0 - 1 + rr);
        const int gx = j < NV ? x0 + j * VE : (j == NV ? wrap(x0 - VE) : wrap(x0 + PTX));
        const int bx0 = j < NV ? SH<T> + 1 + j * VE : (j == NV ? 0 : SH<T> + 1 + PTX);
        goff[i] = c * N + (long long)gy * n + gx;
        soff[i] = c * CSTRIDE + rr * UROW<T> + bx0;
      }
    }
  }
  const long long nn = (long long)n * n;
  // full tiles whose box (x0 - VE .. x0 - VE + UROW - 1, y0 - 1 .. y0 + PTY)
  // lies inside the grid take each component plane as one TMA box, completed
  // on the buffer's mbarrier; the others use the cp.async pieces
  const bool tma = vec && have_map && x0 >= VE && x0 - VE + UROW<T> <= n && y0 >= 1 && y0 + PTY + 1 <= n;
  unsigned parity = 0;  // bit b: phase of buffer b's mbarrier to wait for
  const bool drill = tma && g_rhs_drill != 0;
  const int poll_limit = drill ? RHS_DRILL_POLLS : RHS_POLLS;
  if (tma) {
    if (tid == 0) {
#pragma unroll
      for (int b = 0; b < 3; ++b) mbar_init(&sm.bar[b], 1);
      asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
  }
  auto load_plane = [&](int buf, int gz) {
    if (tma) {
      if (tid == 0 && !drill) {
        mbar_expect_tx(&sm.bar[buf], 3u * CompPlane<T, NC>::WORDS * sizeof(T));
#pragma unroll
        for (int c = 0; c < 3; ++c)
          tma_load_3d(&sm.u[buf][c].r[0][0], &umap, x0 - VE, y0 - 1, (slot * 3 + c) * n + gz, &sm.bar[buf]);
      }
      return;
    }
    if (vec) {
      T* const sb0 = &sm.u[buf][0].r[0][0];
      const T* const ub = u + gz * nn;
#pragma unroll
      for (int i = 0; i < NSLOT; ++i)
        if (goff[i] >= 0) cp_async_16(sb0 + soff[i], ub + goff[i]);
    } else {
      const long long pz = (long long)gz * n;
      for (int rr = ty; rr < PBY; rr += NWARP) {
        const int gy = big ? wrap(y0 - 1 + rr) : wrapm(y0 - 1 + rr);
        for (int bxx = tx; bxx < PBX; bxx += PTX) {
          const int gx = big ? wrap(x0 - 1 + bxx) : wrapm(x0 - 1 + bxx);
#pragma unroll
          for (int c = 0; c < 3; ++c)
            cp_async_word(&sm.u[buf][c][rr][bxx + SH<T>], u + c * N + (pz + gy) * n + gx);
        }
      }
    }
    cp_async_commit();
  };
  auto zwrap = [&](int z) { return big ? wrap(z) : wrapm(z); };
  const int bx = tx + 1;
  // prologue: planes z0-1 (buffer 0) and z0 (buffer 1) give s13, s23 of plane
  // z0-1 and s33 of plane z0 for this thread's cells
  // completion of the loads of buffer buf (its mbarrier phase, or every
  // cp.async of this thread); a TMA wait gives up after about 2^20 polls
  // (RHS_DRILL_POLLS in the wait drill), records the fault and goes on
  auto wait_plane = [&](int buf) {
    if (!tma) {
      cp_async_wait_all();
      return;
    }
    int polls = 0;
    while (!mbar_try_wait(&sm.bar[buf], (parity >> buf) & 1u)) {
      if (++polls > poll_limit) {
        if (tid == 0) atomicExch(&g_rhs_tma_fault, 1);
        break;
      }
    }
    parity ^= 1u << buf;
  };
  // FP64 form: w = s u - q in place over what this thread may touch of
  // buffer buf after its wait -- the whole plane for TMA tiles (the mbarrier
  // wait makes every copy visible to every waiting thread), else its own
  // 16-byte pieces or words; the barrier after the wait publishes the result
  auto shift_plane = [&](int buf) {
    if constexpr (SC) {
      if (pre_shifted) return;  // the field is stored in the shifted form already
      if (tma) {
        constexpr int HALF = PBY * UROW<T> / 2;  // 16-byte pairs per component plane
        static_assert(PBY * UROW<T> % 2 == 0, "component plane of whole pairs");
        for (int i = tid; i < 3 * HALF; i += PTX * NWARP) {
          const int c = i / HALF;
          double2* const p2 = reinterpret_cast<double2*>(&sm.u[buf][c].r[0][0]) + (i - c * HALF);
          double2 v = *p2;
          v.x = fma(sq, v.x, -qs);
          v.y = fma(sq, v.y, -qs);
          *p2 = v;
        }
      } else if (vec) {
        T* const sb0 = &sm.u[buf][0].r[0][0];
#pragma unroll
        for (int i = 0; i < NSLOT; ++i)
          if (goff[i] >= 0) {
            double2* const p2 = reinterpret_cast<double2*>(sb0 + soff[i]);
            double2 v = *p2;
            v.x = fma(sq, v.x, -qs);
            v.y = fma(sq, v.y, -qs);
            *p2 = v;
          }
      } else {
        for (int rr = ty; rr < PBY; rr += NWARP)
          for (int bxx = tx; bxx < PBX; bxx += PTX)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              T& w = sm.u[buf][c][rr][bxx + SH<T>];
              w = fma(sq, w, -qs);
            }
      }
    }
  };
  load_plane(0, zwrap(z0 - 1));
  load_plane(1, zwrap(z0));
  load_plane(2, zwrap(z0 + 1));
  wait_plane(0);
  wait_plane(1);
  wait_plane(2);
  shift_plane(0);
  shift_plane(1);
  shift_plane(2);
  __syncthreads();
  T s13_prev[NC], s23_prev[NC], s33_cur[NC];
#pragma unroll
  for (int i = 0; i < NC; ++i) {
    const int by = NC * ty + 1 + i;
    s13_prev[i] = s13<SC, T>(sm.u[0], sm.u[1], bx, by, co);
    s23_prev[i] = s23<SC, T>(sm.u[0], sm.u[1], bx, by, co);
    s33_cur[i] = s33<SC, T>(sm.u[1][2][by][bx + SH<T>], sm.u[0][2][by][bx + SH<T>], cd);
  }
  __syncthreads();  // buffer 0 is refilled by the first prefetch
  // buffers: cur = plane z, nxt = plane z + 1, pre = the free one
  int cur = 1, nxt = 2, pre = 0;
  const int gx = x0 + tx;
  T* const du1 = du;
  T* const du2 = du + N;
  T* const du3 = du + 2 * N;
  for (int kz = 0; kz < ptz; ++kz) {
    const int z = z0 + kz;
    if (z >= n) break;  // uniform across the CTA
    // plane z + 2 streams into the free buffer while plane z is processed
    // (its last reader finished before the previous iteration's barrier)
    if (kz + 1 < ptz && z + 1 < n) load_plane(pre, zwrap(z + 2));
    const auto& uc = sm.u[cur];
    const auto& un = sm.u[nxt];
    // own-cell stresses
    T v11[NC], v22[NC], v12[NC], v13[NC], v23[NC], v33n[NC];
#pragma unroll
    for (int i = 0; i < NC; ++i) {
      const int by = NC * ty + 1 + i;
      v11[i] = sdiag<SC, T, 0>(uc, bx, by, cd);
      v22[i] = sdiag<SC, T, 1>(uc, bx, by, cd);
      v12[i] = s12<SC, T>(uc, bx, by, co);
      v13[i] = s13<SC, T>(uc, un, bx, by, co);
      v23[i] = s23<SC, T>(uc, un, bx, by, co);
      v33n[i] = s33<SC, T>(un[2][by][bx + SH<T>], uc[2][by][bx + SH<T>], cd);
      // s22 is read from the row above and s23 from the row below: inside a
      // thread's rows they stay in registers
      sm.s[0][by][bx] = v11[i];
      if (i == 0) sm.s[1][by][bx] = v22[i];
      sm.s[2][by][bx] = v12[i];
      sm.s[3][by][bx] = v13[i];
      if (i == NC - 1) sm.s[4][by][bx] = v23[i];
    }
    // halo stresses, one task per warp: s12, s23 on the lower halo row, s22
    // on the upper halo row, s12 and s13 on the left halo column, s11 on the
    // right halo column
    if (warp == 0) {
      sm.s[2][0][lane + 1] = s12<SC, T>(uc, lane + 1, 0, co);
    } else if (warp == 1) {
      sm.s[4][0][lane + 1] = s23<SC, T>(uc, un, lane + 1, 0, co);
    } else if (warp == 2) {
      sm.s[1][PTY + 1][lane + 1] = sdiag<SC, T, 1>(uc, lane + 1, PTY + 1, cd);
    } else if (warp == 3) {
      for (int r = lane; r <= PTY; r += 32) sm.s[2][r][0] = s12<SC, T>(uc, 0, r, co);
    } else if (warp == 4) {
      for (int r = lane + 1; r <= PTY; r += 32) sm.s[3][r][0] = s13<SC, T>(uc, un, 0, r, co);
    } else if (warp == 5) {
      for (int r = lane + 1; r <= PTY; r += 32) sm.s[0][r][PTX + 1] = sdiag<SC, T, 0>(uc, PTX + 1, r, cd);
    }
    __syncthreads();
    if (gx < n) {
      const auto& S = sm.s;
#pragma unroll
      for (int i = 0; i < NC; ++i) {
        const int by = NC * ty + 1 + i;
        const int gy = y0 + by - 1;
        if (gy < n) {
          // a thread's cells are consecutive rows: the stresses of the row
          // below and above come from registers where the thread owns them
          const T s12_below = i > 0 ? v12[i > 0 ? i - 1 : 0] : S[2][by - 1][bx];
          const T s22_above = i < NC - 1 ? v22[i < NC - 1 ? i + 1 : 0] : S[1][by + 1][bx];
          const T s23_below = i > 0 ? v23[i > 0 ? i - 1 : 0] : S[4][by - 1][bx];
          const T d1 = (S[0][by][bx + 1] - v11[i]) + (v12[i] - s12_below) + (v13[i] - s13_prev[i]);
          const T d2 = (v12[i] - S[2][by][bx - 1]) + (s22_above - v22[i]) + (v23[i] - s23_prev[i]);
          const T d3 = (v13[i] - S[3][by][bx - 1]) + (v23[i] - s23_below) + (v33n[i] - s33_cur[i]);
          const long long g = ((long long)z * n + gy) * n + gx;
          if constexpr (SC) {  // the stresses carry -kd
            if (DOADD) {
              du1[g] += d1;
              du2[g] += d2;
              du3[g] += d3;
            } else {
              du1[g] = d1;
              du2[g] = d2;
              du3[g] = d3;
            }
          } else if (DOADD) {
            du1[g] -= kd * d1;
            du2[g] -= kd * d2;
            du3[g] -= kd * d3;
          } else {
            du1[g] = -kd * d1;
            du2[g] = -kd * d2;
            du3[g] = -kd * d3;
          }
        }
        s13_prev[i] = v13[i];
        s23_prev[i] = v23[i];
        s33_cur[i] = v33n[i];
      }
    }
    if (kz + 1 < ptz && z + 1 < n) {
      wait_plane(pre);
      shift_plane(pre);
    }
    __syncthreads();
    const int freed = cur;
    cur = nxt;
    nxt = pre;
    pre = freed;
  }
}

// ---------------------------------------------------------------------------
// FP32 sweep with 2 x 2 cells per thread (64 x 16 tiles, grids that are
// multiples of 64): each thread reads its u rows as aligned float pairs, takes
// the x and y neighbour stresses of its own cells from registers and stores
// float pairs, which halves the shared-memory and global instructions per
// cell.  Same stress and divergence arithmetic, in the same order, as
// rhs_kernel: the results are bit-identical.
// ---------------------------------------------------------------------------
constexpr int QX = 64, QY = 16, QBX = QX + 2, QBY = QY + 2;
constexpr int QROW = 72;  // box x b at b + 3: left piece [0, 4), interior [4, 68), right piece [68, 72)
constexpr int QPLANE = QBY * QROW;                 // words of one component plane
constexpr int QCOMP = (QPLANE + 31) / 32 * 32;     // padded to 128 bytes (TMA destinations)

struct QuadComp {
  float r[QBY][QROW];
  float pad[QCOMP - QPLANE];
};
struct QuadSmem {
  QuadComp u[3][3];      // [plane buffer][component]
  float s[5][QBY][QBX];  // s11, s22, s12, s13, s23 of the current plane
  unsigned long long bar[3];  // TMA completion of each plane buffer
};
// dynamic shared memory of rhs_quad_kernel: the struct plus room to align it
// to 128 bytes
constexpr size_t QUAD_SMEM = sizeof(QuadSmem) + 128;



__device__ __forceinline__ float qdiag(float a, float b, float rv2) {
  const float s = a + b, d = a - b;
  return s * s - rv2 * d;
}
__device__ __forceinline__ float qoff(float a, float b, float c, float d, float rv) {
  return (a + b) * (c + d) - rv * ((b - a) + (d - c));
}

template <bool DOADD>
__global__ void __launch_bounds__(256, 3)
rhs_quad_kernel(int n, float inv_h, float visc, const float* __restrict__ u, float* __restrict__ du, SlotBatch sb,
                int zblocks, int ptz, const __grid_constant__ CUtensorMap umap, int have_map) {
  extern __shared__ __align__(128) unsigned char quad_smem[];
  QuadSmem& sm = *reinterpret_cast<QuadSmem*>(quad_smem + ((128u - (smem_u32(quad_smem) & 127u)) & 127u));
  const long long N = (long long)n * n * n;
  const int slot = blockIdx.z / zblocks;
  const int zb = blockIdx.z - slot * zblocks;
  if (sb.active && !sb.active[slot]) return;
  u += slot * sb.ustride;
  du += slot * sb.ustride;
  if (sb.visc) visc = reinterpret_cast<const float*>(sb.visc)[slot];
  const int tx = threadIdx.x, ty = threadIdx.y, lane = tx, warp = ty;
  const int x0 = blockIdx.x * QX, y0 = blockIdx.y * QY, z0 = zb * ptz;
  const float kd = 0.25f * inv_h, rv = 4.0f * visc * inv_h, rv2 = 2.0f * rv;  // 4 sigma kept, as above
  auto wrap = [n](int g) { return g < 0 ? g + n : (g >= n ? g - n : g); };
  // 16-byte copy pieces of a plane: 18 pieces per box row (left, 16 interior,
  // right), offsets computed once
  constexpr int NPQ = 3 * QBY * 18, NSQ = (NPQ + 255) / 256;
  const int tid = ty * 32 + tx;
  long long goff[NSQ];
  int soff[NSQ];
#pragma unroll
  for (int i = 0; i < NSQ; ++i) {
    const int t = tid + i * 256;
    goff[i] = -1;
    soff[i] = 0;
    if (t < NPQ) {
      const int c = t / (QBY * 18), rem = t - c * (QBY * 18);
      const int rr = rem / 18, j = rem - rr * 18;
      const int gy = wrap(y0 - 1 + rr);
      const int gx = j == 0 ? wrap(x0 - 4) : (j == 17 ? wrap(x0 + QX) : x0 + 4 * (j - 1));
      goff[i] = c * N + (long long)gy * n + gx;
      soff[i] = c * QCOMP + rr * QROW + 4 * j;
    }
  }
  const long long nn = (long long)n * n;
  // tiles whose box (x0 - 4 .. x0 + 67, y0 - 1 .. y0 + 16) lies inside the
  // grid take each component plane as one TMA box, completed on the
  // buffer's mbarrier; the others (their halo wraps around the periodic
  // boundary) use the cp.async pieces
  const bool tma = have_map && x0 >= 4 && x0 + QX + 4 <= n && y0 >= 1 && y0 + QY + 1 <= n;
  unsigned parity = 0;  // bit b: phase of buffer b's mbarrier to wait for
  const bool drill = tma && g_rhs_drill != 0;
  const int poll_limit = drill ? RHS_DRILL_POLLS : RHS_POLLS;
  if (tma) {
    if (tid == 0) {
#pragma unroll
      for (int b = 0; b < 3; ++b) mbar_init(&sm.bar[b], 1);
      asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
  }
  auto load_plane = [&](int buf, int gz) {
    if (tma) {
      if (tid == 0 && !drill) {
        mbar_expect_tx(&sm.bar[buf], 3u * QPLANE * sizeof(float));
#pragma unroll
        for (int c = 0; c < 3; ++c)
          tma_load_3d(&sm.u[buf][c].r[0][0], &umap, x0 - 4, y0 - 1, (slot * 3 + c) * n + gz, &sm.bar[buf]);
      }
      return;
    }
    float* const s0 = &sm.u[buf][0].r[0][0];
    const float* const ub = u + gz * nn;
#pragma unroll
    for (int i = 0; i < NSQ; ++i)
      if (goff[i] >= 0) cp_async_16(s0 + soff[i], ub + goff[i]);
    cp_async_commit();
  };
  // completion of the loads of buffer buf (its mbarrier phase, or every
  // cp.async of this thread); a TMA wait gives up after about 2^20 polls
  // (RHS_DRILL_POLLS in the wait drill), records the fault and goes on
  auto wait_plane = [&](int buf) {
    if (!tma) {
      cp_async_wait_all();
      return;
    }
    int polls = 0;
    while (!mbar_try_wait(&sm.bar[buf], (parity >> buf) & 1u)) {
      if (++polls > poll_limit) {
        if (tid == 0) atomicExch(&g_rhs_tma_fault, 1);
        break;
      }
    }
    parity ^= 1u << buf;
  };
  // this thread: box columns c0 = 2 tx + 1, c0 + 1 and rows r0 = 2 ty + 1, r0 + 1
  const int c0 = 2 * tx + 1, r0 = 2 * ty + 1;
  const int sc = c0 + 3;  // smem column of c0 (even: float2 aligned)
  auto f2 = [&](const float* row) { return *reinterpret_cast<const float2*>(row + sc); };
  load_plane(0, wrap(z0 - 1));
  load_plane(1, wrap(z0));
  load_plane(2, wrap(z0 + 1));
  wait_plane(0);
  wait_plane(1);
  wait_plane(2);
  __syncthreads();
  float p13[2][2], p23[2][2], p33[2][2];  // [row j][col i]
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const auto& ua = sm.u[0];  // plane z0 - 1
    const auto& ub = sm.u[1];  // plane z0
    const int r = r0 + j;
    const float2 a1 = f2(ua[0].r[r]), b1 = f2(ub[0].r[r]), a3 = f2(ua[2].r[r]), a2 = f2(ua[1].r[r]), b2 = f2(ub[1].r[r]);
    const float a3r = ua[2].r[r][sc + 2];
    const float2 a3u = f2(ua[2].r[r + 1]);
    const float2 b3 = f2(ub[2].r[r]);
    p13[j][0] = qoff(a1.x, b1.x, a3.x, a3.y, rv);
    p13[j][1] = qoff(a1.y, b1.y, a3.y, a3r, rv);
    p23[j][0] = qoff(a2.x, b2.x, a3.x, a3u.x, rv);
    p23[j][1] = qoff(a2.y, b2.y, a3.y, a3u.y, rv);
    p33[j][0] = qdiag(b3.x, a3.x, rv2);
    p33[j][1] = qdiag(b3.y, a3.y, rv2);
  }
  __syncthreads();  // buffer 0 is refilled by the first prefetch
  int cur = 1, nxt = 2, pre = 0;
  const int gx = x0 + 2 * tx, gy = y0 + 2 * ty;
  float* const du1 = du;
  float* const du2 = du + N;
  float* const du3 = du + 2 * N;
  for (int kz = 0; kz < ptz; ++kz) {
    const int z = z0 + kz;
    if (z >= n) break;  // uniform across the CTA
    if (kz + 1 < ptz && z + 1 < n) load_plane(pre, wrap(z + 2));
    const auto& uc = sm.u[cur];
    const auto& un = sm.u[nxt];
    // register patch: u1 rows r0, r0+1, r0+2 and column c0-1; u2 rows r0-1,
    // r0, r0+1 and column c0+2; u3 rows r0, r0+1, r0+2 and column c0+2; the
    // next plane's u1, u2, u3 on the thread's rows
    float2 u1r[3], u2r[3], u3r[3], u1n[2], u2n[2], u3n[2];
    float u1l[2], u2r2[2], u3r2[2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      u1r[k] = f2(uc[0].r[r0 + k]);
      u2r[k] = f2(uc[1].r[r0 - 1 + k]);
      u3r[k] = f2(uc[2].r[r0 + k]);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      u1l[j] = uc[0].r[r0 + j][sc - 1];
      u2r2[j] = uc[1].r[r0 + j][sc + 2];
      u3r2[j] = uc[2].r[r0 + j][sc + 2];
      u1n[j] = f2(un[0].r[r0 + j]);
      u2n[j] = f2(un[1].r[r0 + j]);
      u3n[j] = f2(un[2].r[r0 + j]);
    }
    float v11[2][2], v22[2][2], v12[2][2], v13[2][2], v23[2][2], v33[2][2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const float2 a1 = u1r[j], a1u = u1r[j + 1];
      const float2 a2 = u2r[j + 1], a2d = u2r[j];
      const float2 a3 = u3r[j], a3u = u3r[j + 1];
      v11[j][0] = qdiag(a1.x, u1l[j], rv2);
      v11[j][1] = qdiag(a1.y, a1.x, rv2);
      v22[j][0] = qdiag(a2.x, a2d.x, rv2);
      v22[j][1] = qdiag(a2.y, a2d.y, rv2);
      v12[j][0] = qoff(a1.x, a1u.x, a2.x, a2.y, rv);
      v12[j][1] = qoff(a1.y, a1u.y, a2.y, u2r2[j], rv);
      v13[j][0] = qoff(a1.x, u1n[j].x, a3.x, a3.y, rv);
      v13[j][1] = qoff(a1.y, u1n[j].y, a3.y, u3r2[j], rv);
      v23[j][0] = qoff(a2.x, u2n[j].x, a3.x, a3u.x, rv);
      v23[j][1] = qoff(a2.y, u2n[j].y, a3.y, a3u.y, rv);
      v33[j][0] = qdiag(u3n[j].x, a3.x, rv2);
      v33[j][1] = qdiag(u3n[j].y, a3.y, rv2);
    }
    // stresses other threads read: s11 of column c0 (left neighbour), s12 of
    // column c0+1 and of row r0+1 (right neighbour, row above), s13 of column
    // c0+1, s22 of row r0 (row below), s23 of row r0+1 (row above)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      sm.s[0][r0 + j][c0] = v11[j][0];
      sm.s[3][r0 + j][c0 + 1] = v13[j][1];
    }
    sm.s[2][r0][c0 + 1] = v12[0][1];
    sm.s[2][r0 + 1][c0] = v12[1][0];
    sm.s[2][r0 + 1][c0 + 1] = v12[1][1];
    sm.s[1][r0][c0] = v22[0][0];
    sm.s[1][r0][c0 + 1] = v22[0][1];
    sm.s[4][r0 + 1][c0] = v23[1][0];
    sm.s[4][r0 + 1][c0 + 1] = v23[1][1];
    // halo stresses, one task per warp (box row 0, row QY+1, column 0,
    // column QX+1)
    if (warp == 0) {
      for (int c = lane + 1; c <= QX; c += 32)
        sm.s[2][0][c] = qoff(uc[0].r[0][c + 3], uc[0].r[1][c + 3], uc[1].r[0][c + 3], uc[1].r[0][c + 4], rv);
    } else if (warp == 1) {
      for (int c = lane + 1; c <= QX; c += 32)
        sm.s[4][0][c] = qoff(uc[1].r[0][c + 3], un[1].r[0][c + 3], uc[2].r[0][c + 3], uc[2].r[1][c + 3], rv);
    } else if (warp == 2) {
      for (int c = lane + 1; c <= QX; c += 32)
        sm.s[1][QY + 1][c] = qdiag(uc[1].r[QY + 1][c + 3], uc[1].r[QY][c + 3], rv2);
    } else if (warp == 3) {
      if (lane <= QY) sm.s[2][lane][0] = qoff(uc[0].r[lane][3], uc[0].r[lane + 1][3], uc[1].r[lane][3], uc[1].r[lane][4], rv);
    } else if (warp == 4) {
      if (lane < QY) {
        const int r = lane + 1;
        sm.s[3][r][0] = qoff(uc[0].r[r][3], un[0].r[r][3], uc[2].r[r][3], uc[2].r[r][4], rv);
      }
    } else if (warp == 5) {
      if (lane < QY) {
        const int r = lane + 1;
        sm.s[0][r][QX + 1] = qdiag(uc[0].r[r][QX + 4], uc[0].r[r][QX + 3], rv2);
      }
    }
    __syncthreads();
    const auto& S = sm.s;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int r = r0 + j;
      float d1[2], d2[2], d3[2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int c = c0 + i;
        const float s11_right = i == 0 ? v11[j][1] : S[0][r][c + 1];
        const float s12_below = j == 1 ? v12[0][i] : S[2][r - 1][c];
        const float s12_left = i == 1 ? v12[j][0] : S[2][r][c - 1];
        const float s22_above = j == 0 ? v22[1][i] : S[1][r + 1][c];
        const float s13_left = i == 1 ? v13[j][0] : S[3][r][c - 1];
        const float s23_below = j == 1 ? v23[0][i] : S[4][r - 1][c];
        d1[i] = (s11_right - v11[j][i]) + (v12[j][i] - s12_below) + (v13[j][i] - p13[j][i]);
        d2[i] = (v12[j][i] - s12_left) + (s22_above - v22[j][i]) + (v23[j][i] - p23[j][i]);
        d3[i] = (v13[j][i] - s13_left) + (v23[j][i] - s23_below) + (v33[j][i] - p33[j][i]);
        p13[j][i] = v13[j][i];
        p23[j][i] = v23[j][i];
        p33[j][i] = v33[j][i];
      }
      const long long g = ((long long)z * n + gy + j) * n + gx;
      float2* o1 = reinterpret_cast<float2*>(du1 + g);
      float2* o2 = reinterpret_cast<float2*>(du2 + g);
      float2* o3 = reinterpret_cast<float2*>(du3 + g);
      if (DOADD) {
        float2 a = *o1, b = *o2, c = *o3;
        a.x -= kd * d1[0]; a.y -= kd * d1[1];
        b.x -= kd * d2[0]; b.y -= kd * d2[1];
        c.x -= kd * d3[0]; c.y -= kd * d3[1];
        *o1 = a; *o2 = b; *o3 = c;
      } else {
        *o1 = make_float2(-kd * d1[0], -kd * d1[1]);
        *o2 = make_float2(-kd * d2[0], -kd * d2[1]);
        *o3 = make_float2(-kd * d3[0], -kd * d3[1]);
      }
    }
    if (kz + 1 < ptz && z + 1 < n) wait_plane(pre);
    __syncthreads();
    const int freed = cur;
    cur = nxt;
    nxt = pre;
    pre = freed;
  }
}

// Cells per thread along y: two (16-row tiles: the halo stresses are
// recomputed for fewer cells and adjacent rows share their u reads); four ran
// slower in FP32 (94 registers, two CTAs per SM).
template <typename T> constexpr int CYT = 2;

// The driver's tensor-map encoder, reached through the runtime (no link to
// the driver library); null when the driver does not provide it.
using TensorMapEncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                          const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                          CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                          CUtensorMapFloatOOBfill);
static TensorMapEncodeTiled tensor_map_encoder() {
  static std::once_flag once;
  static TensorMapEncodeTiled fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<TensorMapEncodeTiled>(p);
  });
  return fn;
}

// Tiled tensor map, no interleave or swizzle, 128-byte L2 promotion, zero
// fill; false when the encoder is unavailable or rejects the arguments.
bool encode_tiled_map(CUtensorMap* map, CUtensorMapDataType dt, unsigned rank, const void* base,
                      const cuuint64_t* dims, const cuuint64_t* strides, const cuuint32_t* box) {
  std::memset(map, 0, sizeof(*map));
  TensorMapEncodeTiled enc = tensor_map_encoder();
  if (!enc) return false;
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  return enc(map, dt, rank, const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor map of the vector fields of nslots solves as one 3-D tensor
// (x, y, (slot * 3 + component) * n + z) with boxes of bx x by x 1 words;
// false when it cannot be made (the sweep then copies with cp.async).
template <typename T>
static bool field_tensor_map(const T* u, int n, int nslots, const SlotBatch& sb, unsigned bx, unsigned by,
                             CUtensorMap* map) {
  std::memset(map, 0, sizeof(*map));
  const long long N = (long long)n * n * n;
  if (nslots > 1 && sb.ustride != 3 * N) return false;
  if ((reinterpret_cast<uintptr_t>(u) & 15) != 0 || (n * sizeof(T)) % 16 != 0) return false;
  TensorMapEncodeTiled enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)n, (cuuint64_t)n, (cuuint64_t)nslots * 3 * n};
  const cuuint64_t strides[2] = {(cuuint64_t)n * sizeof(T), (cuuint64_t)n * n * sizeof(T)};
  const cuuint32_t box[3] = {bx, by, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  return enc(map, sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
             const_cast<T*>(u), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <typename T>
cudaError_t launch_rhs(int n, T h, T visc, const T* u, T* du, bool doadd, cudaStream_t st, const SlotBatch& sb,
                       int nslots, bool pre_shifted) {
  constexpr int NC = CYT<T>;
  // planes per CTA (4 to 32): the fewest waves of resident CTAs (`per_sm`
  // per SM) times the planes each CTA walks plus one for its start (three
  // planes loaded, the previous plane's stresses), ties to more planes -- so
  // small grids and single solves still fill the GPU without a nearly empty
  // last wave.  The split changes no cell's arithmetic.
  auto zsplit = [&](long long columns, int per_sm, int& ptz, int& zblocks) {
    const long long slots = (long long)per_sm * 152;
    long long best = -1;
    for (int c = 32; c >= 4; --c) {
      const int zb = (n + c - 1) / c;
      const long long waves = (columns * zb * nslots + slots - 1) / slots;
      if (best < 0 || waves * (c + 1) < best) {
        best = waves * (c + 1);
        ptz = c;
        zblocks = zb;
      }
    }
    return columns * zblocks * nslots;
  };
  int ptz, zblocks;
  if constexpr (sizeof(T) == 4) {
    // grids of 64-multiples with 16-byte aligned fields and at least one full
    // wave of CTAs (three per SM): the 2 x 2 kernel
    if (n % QX == 0 && (reinterpret_cast<uintptr_t>(u) & 15) == 0 && (reinterpret_cast<uintptr_t>(du) & 15) == 0 &&
        zsplit((long long)(n / QX) * (n / QY), 3, ptz, zblocks) >= 3LL * 152) {
      dim3 gq(n / QX, n / QY, zblocks * nslots);
      const float ih = (float)(1.0 / (double)h);
      CUtensorMap map;
      const int have = field_tensor_map<float>((const float*)u, n, nslots, sb, QROW, QBY, &map) ? 1 : 0;
      if (doadd)
        rhs_quad_kernel<true><<<gq, dim3(32, 8), QUAD_SMEM, st>>>(n, ih, (float)visc, (const float*)u, (float*)du, sb,
                                                                  zblocks, ptz, map, have);
      else
        rhs_quad_kernel<false><<<gq, dim3(32, 8), QUAD_SMEM, st>>>(n, ih, (float)visc, (const float*)u, (float*)du, sb,
                                                                   zblocks, ptz, map, have);
      return cudaGetLastError();
    }
  }
  const int gxb = (n + PTX - 1) / PTX, gyb = (n + PTYT<NC> - 1) / PTYT<NC>;
  zsplit((long long)gxb * gyb, sizeof(T) == 4 ? 4 : 3, ptz, zblocks);
  dim3 grid(gxb, gyb, zblocks * nslots);
  const size_t sh = plane_smem_bytes<T, NC>();
  CUtensorMap map;
  const int have = field_tensor_map<T>(u, n, nslots, sb, UROW<T>, PBYT<NC>, &map) ? 1 : 0;
  if (doadd)
    rhs_kernel<T, NC, true><<<grid, dim3(PTX, NWARP), sh, st>>>(n, (T)(1.0 / (double)h), visc, u, du, sb, zblocks, ptz,
                                                                map, have, pre_shifted ? 1 : 0);
  else
    rhs_kernel<T, NC, false><<<grid, dim3(PTX, NWARP), sh, st>>>(n, (T)(1.0 / (double)h), visc, u, du, sb, zblocks,
                                                                 ptz, map, have, pre_shifted ? 1 : 0);
  return cudaGetLastError();
}

template <typename T>
static cudaError_t configure_rhs_t() {
  constexpr int NC = CYT<T>;
  const int sh = (int)plane_smem_bytes<T, NC>();
  cudaError_t e = cudaFuncSetAttribute(rhs_kernel<T, NC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sh);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(rhs_kernel<T, NC, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sh);
  return e;
}

cudaError_t configure_stencil() {
  cudaError_t e = configure_rhs_t<float>();
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(rhs_quad_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)QUAD_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(rhs_quad_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)QUAD_SMEM);
  if (e == cudaSuccess) e = configure_rhs_t<double>();
  return e;
}

template cudaError_t launch_rhs<double>(int, double, double, const double*, double*, bool, cudaStream_t,
                                        const SlotBatch&, int, bool);
template cudaError_t launch_rhs<float>(int, float, float, const float*, float*, bool, cudaStream_t, const SlotBatch&,
                                       int, bool);

}  // namespace exc

extern "C" int exc_debug_wait_drill(int flags) {
  if (flags < 0 || flags > 3) { exc::set_last_error("drill flags must be 0..3"); return EXC_ERR_ARG; }
  int rc = exc::configure_device();
  if (rc) return rc;
  const int rhs = flags & 1;
  cudaError_t e = cudaMemcpyToSymbol(exc::g_rhs_drill, &rhs, sizeof(int));
  if (e != cudaSuccess) { exc::set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return exc::learned_set_drill((flags >> 1) & 1);
}

extern "C" int exc_device_sync(void* stream, int* flags) {
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) { exc::set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  int f = 0;
  int rc = exc_device_faults(&f);
  if (rc) return rc;
  if (flags) *flags = f;
  if (f) {
    exc::set_last_error(f & 1 ? (f & 2 ? "device waits gave up (RHS sweep TMA plane, tensor-core convolution)"
                                       : "a device wait gave up (RHS sweep TMA plane)")
                              : "a device wait gave up (tensor-core convolution)");
    return EXC_ERR_TIMEOUT;
  }
  return EXC_OK;
}

extern "C" int exc_device_faults(int* flags) {
  if (!flags) { exc::set_last_error("null argument"); return EXC_ERR_ARG; }
  int v = 0, zero = 0, lf = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, exc::g_rhs_tma_fault, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(exc::g_rhs_tma_fault, &zero, sizeof(int));
  if (e != cudaSuccess) { exc::set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  const int rc = exc::learned_fault_take(&lf);
  if (rc) return rc;
  *flags = (v ? 1 : 0) | (lf ? 2 : 0);
  return EXC_OK;
}
