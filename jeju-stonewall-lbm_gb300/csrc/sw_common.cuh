// sw_common.cuh -- D3Q19 tables, device layout and storage policies shared by the kernels.
//
// Device layout (x fastest, one structure-of-arrays plane per population):
//   f[i][z][y][pitch]     i < 19, pitch = nx rounded up to 32 (128-byte rows for fp32)
//   flag[z][y][pitch]     uint8: 0 fluid, 1 stone (WALL), 2 ground (GROUND)
//   tiles[z][y][pitch/32] uint8 per 32-cell row segment (one warp): see TILE_*
// The reference keeps f[i][x][y][z] with z fastest (stonewall3d/lbm3d.py:293);
// sw_pack_* / sw_unpack_* convert at upload, download and checkpoint time only.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/stonewall.h"

namespace sw {

constexpr int Q = 19;
constexpr int SEG = 32;  // cells per row segment = one warp

// D3Q19 velocity set in the reference's order (lbm3d.py:20-24); the order is
// part of the checkpoint format, so it is kept exactly.
__host__ __device__ constexpr int CX(int i) {
  return (i == 1 || i == 7 || i == 9 || i == 11 || i == 13) ? 1
         : (i == 2 || i == 8 || i == 10 || i == 12 || i == 14) ? -1 : 0;
}
__host__ __device__ constexpr int CY(int i) {
  return (i == 3 || i == 7 || i == 10 || i == 15 || i == 17) ? 1
         : (i == 4 || i == 8 || i == 9 || i == 16 || i == 18) ? -1 : 0;
}
__host__ __device__ constexpr int CZ(int i) {
  return (i == 5 || i == 11 || i == 14 || i == 15 || i == 18) ? 1
         : (i == 6 || i == 12 || i == 13 || i == 16 || i == 17) ? -1 : 0;
}
// opposite direction (lbm3d.py:26): pairs (1,2), (3,4), ..., (17,18)
__host__ __device__ constexpr int OPP(int i) { return i == 0 ? 0 : ((i & 1) ? i + 1 : i - 1); }
// c_z mirrored (lbm3d.py:27)
__host__ __device__ constexpr int MIRZ(int i) {
  return i == 5 ? 6 : i == 6 ? 5 : i == 11 ? 13 : i == 13 ? 11 : i == 12 ? 14 : i == 14 ? 12
         : i == 15 ? 17 : i == 17 ? 15 : i == 16 ? 18 : i == 18 ? 16 : i;
}

// Lattice weights: float32 values of 1/3, 1/18, 1/36 as lbm3d.py:25 builds them.
template <typename R> __host__ __device__ constexpr R W(int i);
template <> __host__ __device__ constexpr float W<float>(int i) {
  return i == 0 ? (float)(1.0 / 3.0) : (i < 7 ? (float)(1.0 / 18.0) : (float)(1.0 / 36.0));
}
template <> __host__ __device__ constexpr double W<double>(int i) {
  return i == 0 ? 1.0 / 3.0 : (i < 7 ? 1.0 / 18.0 : 1.0 / 36.0);
}

// Tile kinds, one byte per 32-cell row segment.
enum : uint8_t {
  TILE_ALL_SOLID = 1,  // no fluid cell in the segment: nothing to do
  TILE_CHECK = 2,      // some cell, or some pull source of a fluid cell, is not fluid
  TILE_FORCE = 4,      // some pull source of a fluid cell is a stone: momentum exchange
};

// Fixed-point scale of the force accumulators: per-warp float64 partial sums
// are rounded to multiples of 2^-40 and added with 64-bit integer atomics, so
// the per-level totals do not depend on the order in which warps finish.
constexpr double FORCE_SCALE = 1099511627776.0;  // 2^40

// ---------------------------------------------------------------- storage policies
// R = arithmetic type of the collision, T = stored type.  The shifted 16-bit
// formats store g_i = f_i - w_i (the deviation from the rest state) to keep the
// significant bits where the signal is, and the step computes on g directly
// (kShift): ld / st move values of the compute domain (g when shifted, f
// otherwise); enc / dec convert full f values (init, layout transposes, macro).
template <int DT> struct Store;

template <> struct Store<SW_F32> {
  using T = float;
  using R = float;
  static constexpr bool kShift = false;
  template <int I> static __device__ __forceinline__ R ld(const T *p) { return __ldg(p); }
  template <int I> static __device__ __forceinline__ void st(T *p, R v) { __stcs(p, v); }
  template <int I> static __device__ __forceinline__ T enc(R v) { return v; }
  template <int I> static __device__ __forceinline__ R dec(T v) { return v; }
};
template <> struct Store<SW_F64> {
  using T = double;
  using R = double;
  static constexpr bool kShift = false;
  template <int I> static __device__ __forceinline__ R ld(const T *p) { return __ldg(p); }
  template <int I> static __device__ __forceinline__ void st(T *p, R v) { __stcs(p, v); }
  template <int I> static __device__ __forceinline__ T enc(R v) { return v; }
  template <int I> static __device__ __forceinline__ R dec(T v) { return v; }
};
template <> struct Store<SW_F16_SHIFT> {
  using T = __half;
  using R = float;
  static constexpr bool kShift = true;
  template <int I> static __device__ __forceinline__ R dec(T v) { return W<float>(I) + __half2float(v); }
  template <int I> static __device__ __forceinline__ T enc(R v) { return __float2half_rn(v - W<float>(I)); }
  template <int I> static __device__ __forceinline__ R ld(const T *p) { return __half2float(__ldg(p)); }
  template <int I> static __device__ __forceinline__ void st(T *p, R v) { __stcs(p, __float2half_rn(v)); }
  static __device__ __forceinline__ T from_shifted(R g) { return __float2half_rn(g); }
  static __device__ __forceinline__ R to_shifted(T v) { return __half2float(v); }
};
template <> struct Store<SW_BF16_SHIFT> {
  using T = __nv_bfloat16;
  using R = float;
  static constexpr bool kShift = true;
  template <int I> static __device__ __forceinline__ R dec(T v) { return W<float>(I) + __bfloat162float(v); }
  template <int I> static __device__ __forceinline__ T enc(R v) { return __float2bfloat16_rn(v - W<float>(I)); }
  template <int I> static __device__ __forceinline__ R ld(const T *p) { return __bfloat162float(__ldg(p)); }
  template <int I> static __device__ __forceinline__ void st(T *p, R v) { __stcs(p, __float2bfloat16_rn(v)); }
  static __device__ __forceinline__ T from_shifted(R g) { return __float2bfloat16_rn(g); }
  static __device__ __forceinline__ R to_shifted(T v) { return __bfloat162float(v); }
};

// lbm3d.py:33-36, same evaluation order.
template <typename R>
__device__ __forceinline__ R feq_i(R w, R cx, R cy, R cz, R rho, R ux, R uy, R uz) {
  R cu = R(3.0) * (cx * ux + cy * uy + cz * uz);
  return w * rho * (R(1.0) + cu + R(0.5) * cu * cu - R(1.5) * (ux * ux + uy * uy + uz * uz));
}

// Compile-time loop: calls f(std::integral_constant-like tag) for I = 0..N-1.
template <int I> struct Int { static constexpr int value = I; };
template <int I, int N, typename F> __device__ __forceinline__ void static_for(F &&f) {
  if constexpr (I < N) {
    f(Int<I>{});
    static_for<I + 1, N>(f);
  }
}

struct Geom {
  int nx, ny, nz, pitch;
  int nseg_x;            // pitch / 32
  long long plane;       // cells per population plane = nz * ny * pitch
};

inline int round_up(int a, int b) { return (a + b - 1) / b * b; }

}  // namespace sw
