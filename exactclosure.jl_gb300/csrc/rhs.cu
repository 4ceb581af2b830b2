// RHS sweep: du = doadd*du - div sigma(u) (`stresstensor` + `tensordivergence!`,
// src/N.jl:94-160), marching along z.
//
// A CTA owns a TX x TY column of cells and walks TZ planes.  Three plane
// buffers of u with a one-cell x/y halo sit in shared memory: planes z and
// z+1 are read while plane z+2 streams in with cp.async; each thread
// evaluates the six stress components at its own cell (the edge stresses s13,
// s23 and the diagonal s33 of the next plane are kept in registers for the
// next plane), four warps evaluate the halo stresses lane-parallel, and the
// divergence is formed from shared memory and registers.  Every stress value
// is computed once (plus the x/y halo), index arithmetic is per plane, and
// global loads and stores are row-contiguous.  Stresses are kept divided by h.
#include "internal.cuh"

namespace exc {

constexpr int PTX = 32, PTY = 8, PTZ = 32;
constexpr int PBX = PTX + 2, PBY = PTY + 2;  // plane box with one-cell halo (box x = x - x0 + 1)
// u rows in shared memory: box x index xb sits at xb + SH<T>, so the 32
// interior cells start on a 16-byte boundary and arrive by 16-byte copies
template <typename T> constexpr int SH = 16 / (int)sizeof(T) - 1;
template <typename T> constexpr int UROW = ((SH<T> + PBX) + 16 / (int)sizeof(T) - 1) / (16 / (int)sizeof(T)) *
                                           (16 / (int)sizeof(T));

template <typename T>
struct PlaneSmem {
  __align__(16) T u[3][3][PBY][UROW<T>];
  T s[5][PBY][PBX];  // s11, s22, s12, s13, s23 of the current plane
};

// sigma_ii at box (bx, by) of plane buffer b (uses u_i at the cell and at -e_i)
template <typename T, int I>
__device__ __forceinline__ T sdiag(const T (&u)[3][PBY][UROW<T>], int bx, int by, T kd, T kv2) {
  bx += SH<T>;
  const T a = u[I][by][bx];
  const T b = I == 0 ? u[0][by][bx - 1] : u[1][by - 1][bx];
  const T s = a + b, d = a - b;
  return s * s * kd - kv2 * d;
}
// sigma_12 at box (bx, by): u1, u1(+y), u2, u2(+x)
template <typename T>
__device__ __forceinline__ T s12(const T (&u)[3][PBY][UROW<T>], int bx, int by, T kd, T kv) {
  bx += SH<T>;
  const T a = u[0][by][bx], b = u[0][by + 1][bx], c = u[1][by][bx], d = u[1][by][bx + 1];
  return (a + b) * (c + d) * kd - kv * ((b - a) + (d - c));
}
// sigma_13 at box (bx, by): u1, u1(+z) [next plane], u3, u3(+x)
template <typename T>
__device__ __forceinline__ T s13(const T (&uc)[3][PBY][UROW<T>], const T (&un)[3][PBY][UROW<T>], int bx, int by,
                                 T kd, T kv) {
  bx += SH<T>;
  const T a = uc[0][by][bx], b = un[0][by][bx], c = uc[2][by][bx], d = uc[2][by][bx + 1];
  return (a + b) * (c + d) * kd - kv * ((b - a) + (d - c));
}
// sigma_23 at box (bx, by): u2, u2(+z) [next plane], u3, u3(+y)
template <typename T>
__device__ __forceinline__ T s23(const T (&uc)[3][PBY][UROW<T>], const T (&un)[3][PBY][UROW<T>], int bx, int by,
                                 T kd, T kv) {
  bx += SH<T>;
  const T a = uc[1][by][bx], b = un[1][by][bx], c = uc[2][by][bx], d = uc[2][by + 1][bx];
  return (a + b) * (c + d) * kd - kv * ((b - a) + (d - c));
}
// sigma_33 between planes: u3 of the upper plane and of the lower plane
template <typename T>
__device__ __forceinline__ T s33(T up, T lo, T kd, T kv2) {
  const T s = up + lo, d = up - lo;
  return s * s * kd - kv2 * d;
}

template <typename T>
__global__ void __launch_bounds__(PTX * PTY)
rhs_kernel(int n, T inv_h, T visc, const T* __restrict__ u, T* __restrict__ du, int doadd, SlotBatch sb,
           int zblocks) {
  __shared__ PlaneSmem<T> sm;
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
  const int x0 = blockIdx.x * PTX, y0 = blockIdx.y * PTY, z0 = zb * PTZ;
  const T kd = (T)0.25 * inv_h;
  const T kv = visc * inv_h * inv_h;
  const T kv2 = (T)2 * kv;
  auto wrap = [n](int g) { return g < 0 ? g + n : (g >= n ? g - n : g); };
  auto wrapm = [n](int g) { return ((g % n) + n) % n; };
  // per-thread load offsets within a plane: rows ty and ty + 8, columns tx and tx + 32
  const bool big = n >= PBX;
  const int ra = big ? wrap(y0 - 1 + ty) : wrapm(y0 - 1 + ty);
  const int rb = big ? wrap(y0 - 1 + ty + PTY) : wrapm(y0 - 1 + ty + PTY);
  const int ca = big ? wrap(x0 - 1 + tx) : wrapm(x0 - 1 + tx);
  const int cb = big ? wrap(x0 - 1 + tx + PTX) : wrapm(x0 - 1 + tx + PTX);
  const bool xr = tx < PBX - PTX, yr = ty < PBY - PTY;
  // asynchronous copy of plane gz (with halo) into buffer buf; the caller
  // commits and waits (cp_async_wait_all) before the __syncthreads that
  // publishes it
  // full x tiles of a grid whose rows are 16-byte multiples take the row
  // interiors as 16-byte copies (VE words each) and the two halo cells as
  // words; other tiles copy word by word
  constexpr int VE = 16 / (int)sizeof(T), NV = PTX / VE;
  const bool vec = big && x0 + PTX <= n && (n % VE) == 0;
  const int cl = wrap(x0 - 1), cr = wrap(x0 + PTX);
  const int tid = ty * PTX + tx;
  auto load_plane = [&](int buf, int gz) {
    const long long pz = (long long)gz * n;
    if (vec) {
      for (int t = tid; t < 3 * PBY * (NV + 2); t += PTX * PTY) {
        const int c = t / (PBY * (NV + 2));
        const int rem = t - c * (PBY * (NV + 2));
        const int rr = rem / (NV + 2), j = rem - rr * (NV + 2);
        const int gy = wrap(y0 - 1 + rr);
        const T* row = u + c * N + (pz + gy) * n;
        T* srow = &sm.u[buf][c][rr][SH<T>];
        if (j < NV) cp_async_16(srow + 1 + j * VE, row + x0 + j * VE);
        else if (j == NV) cp_async_word(srow, row + cl);
        else cp_async_word(srow + PTX + 1, row + cr);
      }
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const T* p = u + c * N;
        const long long oa = (pz + ra) * n, ob = (pz + rb) * n;
        cp_async_word(&sm.u[buf][c][ty][tx + SH<T>], p + oa + ca);
        if (xr) cp_async_word(&sm.u[buf][c][ty][tx + PTX + SH<T>], p + oa + cb);
        if (yr) {
          cp_async_word(&sm.u[buf][c][ty + PTY][tx + SH<T>], p + ob + ca);
          if (xr) cp_async_word(&sm.u[buf][c][ty + PTY][tx + PTX + SH<T>], p + ob + cb);
        }
      }
    }
    cp_async_commit();
  };
  auto zwrap = [&](int z) { return big ? wrap(z) : wrapm(z); };
  const int bx = tx + 1, by = ty + 1;
  // prologue: planes z0-1 (buffer 0) and z0 (buffer 1) give s13, s23 of plane
  // z0-1 and s33 of plane z0 for this thread's cell
  load_plane(0, zwrap(z0 - 1));
  load_plane(1, zwrap(z0));
  load_plane(2, zwrap(z0 + 1));
  cp_async_wait_all();
  __syncthreads();
  T s13_prev = s13<T>(sm.u[0], sm.u[1], bx, by, kd, kv);
  T s23_prev = s23<T>(sm.u[0], sm.u[1], bx, by, kd, kv);
  T s33_cur = s33<T>(sm.u[1][2][by][bx + SH<T>], sm.u[0][2][by][bx + SH<T>], kd, kv2);
  __syncthreads();  // buffer 0 is refilled by the first prefetch
  // buffers: cur = plane z, nxt = plane z + 1, pre = the free one
  int cur = 1, nxt = 2, pre = 0;
  const int gx = x0 + tx, gy = y0 + ty;
  const bool inside = gx < n && gy < n;
  for (int kz = 0; kz < PTZ; ++kz) {
    const int z = z0 + kz;
    if (z >= n) break;  // uniform across the CTA
    // plane z + 2 streams into the free buffer while plane z is processed
    // (its last reader finished before the previous iteration's barrier)
    if (kz + 1 < PTZ && z + 1 < n) load_plane(pre, zwrap(z + 2));
    const auto& uc = sm.u[cur];
    const auto& un = sm.u[nxt];
    // own-cell stresses
    const T v11 = sdiag<T, 0>(uc, bx, by, kd, kv2);
    const T v22 = sdiag<T, 1>(uc, bx, by, kd, kv2);
    const T v12 = s12<T>(uc, bx, by, kd, kv);
    const T v13 = s13<T>(uc, un, bx, by, kd, kv);
    const T v23 = s23<T>(uc, un, bx, by, kd, kv);
    const T v33n = s33<T>(un[2][by][bx + SH<T>], uc[2][by][bx + SH<T>], kd, kv2);
    sm.s[0][by][bx] = v11;
    sm.s[1][by][bx] = v22;
    sm.s[2][by][bx] = v12;
    sm.s[3][by][bx] = v13;
    sm.s[4][by][bx] = v23;
    // halo stresses, lane-parallel: s12 on the lower row, s23 on the lower
    // row, s22 on the upper row, and the column halos (s12, s13 left; s11 right)
    if (warp == 0) {
      sm.s[2][0][lane + 1] = s12<T>(uc, lane + 1, 0, kd, kv);
    } else if (warp == 1) {
      sm.s[4][0][lane + 1] = s23<T>(uc, un, lane + 1, 0, kd, kv);
    } else if (warp == 2) {
      sm.s[1][PTY + 1][lane + 1] = sdiag<T, 1>(uc, lane + 1, PTY + 1, kd, kv2);
    } else if (warp == 3) {
      if (lane <= PTY) {
        sm.s[2][lane][0] = s12<T>(uc, 0, lane, kd, kv);
      } else if (lane <= 2 * PTY) {
        const int r = lane - PTY;
        sm.s[3][r][0] = s13<T>(uc, un, 0, r, kd, kv);
      } else if (lane <= 3 * PTY) {
        const int r = lane - 2 * PTY;
        sm.s[0][r][PTX + 1] = sdiag<T, 0>(uc, PTX + 1, r, kd, kv2);
      }
    }
    __syncthreads();
    if (inside) {
      const auto& S = sm.s;
      const T d1 = (S[0][by][bx + 1] - v11) + (v12 - S[2][by - 1][bx]) + (v13 - s13_prev);
      const T d2 = (v12 - S[2][by][bx - 1]) + (S[1][by + 1][bx] - v22) + (v23 - s23_prev);
      const T d3 = (v13 - S[3][by][bx - 1]) + (v23 - S[4][by - 1][bx]) + (v33n - s33_cur);
      const long long g = ((long long)z * n + gy) * n + gx;
      if (doadd) {
        du[g] -= d1;
        du[N + g] -= d2;
        du[2 * N + g] -= d3;
      } else {
        du[g] = -d1;
        du[N + g] = -d2;
        du[2 * N + g] = -d3;
      }
    }
    s13_prev = v13;
    s23_prev = v23;
    s33_cur = v33n;
    cp_async_wait_all();
    __syncthreads();
    const int freed = cur;
    cur = nxt;
    nxt = pre;
    pre = freed;
  }
}

template <typename T>
cudaError_t launch_rhs(int n, T h, T visc, const T* u, T* du, bool doadd, cudaStream_t st, const SlotBatch& sb,
                       int nslots) {
  const int zblocks = (n + PTZ - 1) / PTZ;
  dim3 grid((n + PTX - 1) / PTX, (n + PTY - 1) / PTY, zblocks * nslots);
  rhs_kernel<T><<<grid, dim3(PTX, PTY), 0, st>>>(n, (T)(1.0 / (double)h), visc, u, du, doadd ? 1 : 0, sb, zblocks);
  return cudaGetLastError();
}

cudaError_t configure_stencil() { return cudaSuccess; }

template cudaError_t launch_rhs<double>(int, double, double, const double*, double*, bool, cudaStream_t,
                                        const SlotBatch&, int);
template cudaError_t launch_rhs<float>(int, float, float, const float*, float*, bool, cudaStream_t, const SlotBatch&,
                                       int);

}  // namespace exc
