// sw_aux.cu -- k_init, k_macro / k_accum, tile classification and layout transposes.
//
// This translation unit is compiled with --fmad=false: these kernels run once
// (or every few steps) and evaluate every expression in source order, so their
// float32 results equal the reference's operation sequence exactly (k_init for
// the same random stream, k_macro for the same f).
#include "sw_aux.cuh"

namespace sw {

// ---------------------------------------------------------------- random stream
// PCG hash (Jarzynski & Olano, JCGT 2020), used as rand_init(seed, offset) =
// pcg(seed + pcg(offset)) and randf(state) = (pcg(state) >> 8) / 2^24 -- the
// form of the wp.rand_init / wp.randf calls in lbm3d.py:48-52.
__device__ __forceinline__ uint32_t pcg_hash(uint32_t s) {
  uint32_t b = s * 747796405u + 2891336453u;
  uint32_t c = ((b >> ((b >> 28u) + 4u)) ^ b) * 277803737u;
  return (c >> 22u) ^ c;
}
__device__ __forceinline__ float randf(uint32_t &st) {
  st = pcg_hash(st);
  return (float)(st >> 8) * (1.0f / 16777216.0f);
}
// Standard normals by Box-Muller, in float (FP64 is slow on this part; the
// oracle's double-precision version agrees to float rounding).
__device__ __forceinline__ float gauss_pair(uint32_t &st, float *second) {
  const float u1 = 1.0f - randf(st);  // (0, 1]
  const float u2 = randf(st);
  const float r = sqrtf(-2.0f * logf(u1));
  float sn, cs;
  sincosf(6.2831853071795865f * u2, &sn, &cs);
  if (second) *second = r * sn;
  return r * cs;
}

// k_init, lbm3d.py:39-54.  One thread per cell of the padded grid.
template <int DT>
__global__ void k_init(Geom g, typename Store<DT>::T *f, const uint8_t *flag, const float *uin, float noise,
                       int seed, int noise_kind) {
  using S = Store<DT>;
  using R = typename S::R;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.plane) return;
  const int x = (int)(c % g.pitch);
  const long long row = c / g.pitch;
  const int y = (int)(row % g.ny), z = (int)(row / g.ny);
  if (x >= g.nx) return;
  R ux = R(0.0), uy = R(0.0), uz = R(0.0);
  if (flag[c] == 0) {
    const uint32_t off = ((uint32_t)x * 7919u + (uint32_t)y) * 7907u + (uint32_t)z;
    uint32_t st = pcg_hash((uint32_t)seed + pcg_hash(off));
    const R u0 = (R)uin[z];
    const R nz_ = (R)noise;
    if (noise_kind == SW_NOISE_UNIFORM) {
      ux = u0 * (R(1.0) + nz_ * (R(2.0) * (R)randf(st) - R(1.0)));
      uy = u0 * nz_ * (R(2.0) * (R)randf(st) - R(1.0));
      uz = u0 * nz_ * (R(2.0) * (R)randf(st) - R(1.0));
    } else {
      float g2 = 0.0f;
      const float g1 = gauss_pair(st, &g2);
      const float g3 = gauss_pair(st, nullptr);
      ux = u0 * (R(1.0) + nz_ * (R)g1);
      uy = u0 * nz_ * (R)g2;
      uz = u0 * nz_ * (R)g3;
    }
  }
  const size_t plane = (size_t)g.plane;
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    const R v = feq_i<R>(W<R>(i), R(CX(i)), R(CY(i)), R(CZ(i)), R(1.0), ux, uy, uz);
    f[(size_t)i * plane + c] = S::template enc<i>(v);
  });
}

// k_macro (lbm3d.py:158-182) with an optional fused k_accum (lbm3d.py:185-188) in double.
template <int DT>
__global__ void k_macro(Geom g, const typename Store<DT>::T *f, const uint8_t *flag, float *u, double *acc) {
  using S = Store<DT>;
  using R = typename S::R;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.plane) return;
  if ((int)(c % g.pitch) >= g.nx) return;
  const size_t P = (size_t)g.plane;
  R out[4];
  if (flag[c] != 0) {
    out[0] = R(1.0); out[1] = R(0.0); out[2] = R(0.0); out[3] = R(0.0);
  } else {
    R rho = R(0.0), mx = R(0.0), my = R(0.0), mz = R(0.0);
    static_for<0, Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      const R v = S::template dec<i>(f[(size_t)i * P + c]);
      rho += v;
      mx += v * R(CX(i));
      my += v * R(CY(i));
      mz += v * R(CZ(i));
    });
    out[0] = rho; out[1] = mx / rho; out[2] = my / rho; out[3] = mz / rho;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (u) u[k * P + c] = (float)out[k];
    if (acc) acc[k * P + c] += (double)out[k];
  }
}

__global__ void k_accum(Geom g, const float *u, double *acc) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= 4 * g.plane) return;
  if ((int)(c % g.pitch) >= g.nx) return;
  acc[c] += (double)u[c];
}

// Segment classification for the step kernel (see TILE_* in sw_common.cuh).
// Mirrors the pull-source mapping of the step (lbm3d.py:77-88).
__global__ void k_build_tiles(Geom g, const uint8_t *flag, uint8_t *tiles) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nseg = (long long)g.nseg_x * g.ny * g.nz;
  const long long seg = c >> 5;
  if (seg >= nseg) return;  // whole warps only (plane is a multiple of 32)
  const int lane = threadIdx.x & 31;
  const int x = (int)(c % g.pitch);
  const long long row = c / g.pitch;
  const int y = (int)(row % g.ny), z = (int)(row / g.ny);
  const bool live = x < g.nx;
  bool fluid = false, nonfluid_src = false, wall_src = false;
  if (live) {
    fluid = flag[c] == 0;
    if (fluid && x > 0) {  // inlet cells do not pull
      const int ym = (y == 0) ? g.ny - 1 : y - 1, yp = (y == g.ny - 1) ? 0 : y + 1;
      const int zp = (z == g.nz - 1) ? z : z + 1;
      const int xp = (x + 1 >= g.nx) ? x : x + 1;
      for (int i = 1; i < Q; ++i) {
        const int ex = CX(i), ey = CY(i), ez = CZ(i);
        if (ez == 1 && z == 0) { nonfluid_src = true; continue; }
        const int xs = ex == 1 ? x - 1 : (ex == -1 ? xp : x);
        const int ys = ey == 1 ? ym : (ey == -1 ? yp : y);
        const int zs = ez == 1 ? z - 1 : (ez == -1 ? zp : z);
        const uint8_t fs = flag[((long long)zs * g.ny + ys) * g.pitch + xs];
        if (fs != 0) nonfluid_src = true;
        if (fs == SW_WALL) wall_src = true;
      }
    }
  }
  const unsigned any_fluid = __ballot_sync(0xffffffffu, live && fluid);
  const unsigned any_check = __ballot_sync(0xffffffffu, live && (!fluid || nonfluid_src));
  const unsigned any_wall = __ballot_sync(0xffffffffu, live && fluid && wall_src);
  if (lane == 0)
    tiles[seg] = (uint8_t)((any_fluid ? 0 : TILE_ALL_SOLID) | (any_check ? TILE_CHECK : 0) |
                           (any_wall ? TILE_FORCE : 0));
}

// ---------------------------------------------------------------- x <-> z transposes
// Reference layout a[k][x][y][z] (z fastest) <-> device layout b[k][z][y][pitch].
// One block moves a 32 x 32 tile of the (x, z) plane of one (k, y).
template <typename A, typename B, typename Conv>
__global__ void k_ref_to_dev(Geom g, int nk, const A *a, B *b, Conv conv) {
  __shared__ A t[32][33];
  const int ky = blockIdx.x;             // k * ny + y
  const int k = ky / g.ny, y = ky % g.ny;
  const int x0 = blockIdx.y * 32, z0 = blockIdx.z * 32;
  const size_t aplane = (size_t)g.nx * g.ny * g.nz;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {   // r: x offset, threadIdx.x: z offset
    const int x = x0 + r, z = z0 + threadIdx.x;
    if (x < g.nx && z < g.nz) t[r][threadIdx.x] = a[k * aplane + ((size_t)x * g.ny + y) * g.nz + z];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {   // r: z offset, threadIdx.x: x offset
    const int z = z0 + r, x = x0 + threadIdx.x;
    if (x < g.pitch && z < g.nz) {
      const size_t o = (size_t)k * g.plane + ((size_t)z * g.ny + y) * g.pitch + x;
      if (x < g.nx) b[o] = conv(k, t[threadIdx.x][r]);
      else b[o] = conv.pad(k);
    }
  }
  (void)nk;
}

template <typename B, typename A, typename Conv>
__global__ void k_dev_to_ref(Geom g, int nk, const B *b, A *a, Conv conv) {
  __shared__ A t[32][33];
  const int ky = blockIdx.x;
  const int k = ky / g.ny, y = ky % g.ny;
  const int x0 = blockIdx.y * 32, z0 = blockIdx.z * 32;
  const size_t aplane = (size_t)g.nx * g.ny * g.nz;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {   // r: z offset, threadIdx.x: x offset
    const int z = z0 + r, x = x0 + threadIdx.x;
    if (x < g.nx && z < g.nz) t[r][threadIdx.x] = conv(k, b[(size_t)k * g.plane + ((size_t)z * g.ny + y) * g.pitch + x]);
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {   // r: x offset, threadIdx.x: z offset
    const int x = x0 + r, z = z0 + threadIdx.x;
    if (x < g.nx && z < g.nz) a[k * aplane + ((size_t)x * g.ny + y) * g.nz + z] = t[threadIdx.x][r];
  }
  (void)nk;
}

// Converters between a reference-layout value and the stored value of population k.
template <int DT, typename A> struct EncF {
  __device__ typename Store<DT>::T operator()(int k, A v) const { return enc_dyn(k, (typename Store<DT>::R)v); }
  __device__ typename Store<DT>::T pad(int k) const { return enc_dyn(k, W<typename Store<DT>::R>(k)); }
  static __device__ typename Store<DT>::T enc_dyn(int k, typename Store<DT>::R v) {
    typename Store<DT>::T out{};
    static_for<0, Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      if (k == i) out = Store<DT>::template enc<i>(v);
    });
    return out;
  }
};
template <int DT, typename A> struct DecF {
  __device__ A operator()(int k, typename Store<DT>::T v) const {
    A out{};
    static_for<0, Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      if (k == i) out = (A)Store<DT>::template dec<i>(v);
    });
    return out;
  }
};
template <typename A> struct Ident {
  __device__ A operator()(int, A v) const { return v; }
  __device__ A pad(int) const { return A(0); }
};

inline dim3 tgrid(const Geom &g, int nk, int xext) {
  return dim3((unsigned)(nk * g.ny), (unsigned)((xext + 31) / 32), (unsigned)((g.nz + 31) / 32));
}

template <int DT>
cudaError_t pack_f_t(const Geom &g, int ref_dtype, const void *ref, void *f, cudaStream_t s) {
  using T = typename Store<DT>::T;
  if (ref_dtype == SW_F32)
    k_ref_to_dev<<<tgrid(g, Q, g.pitch), dim3(32, 8), 0, s>>>(g, Q, (const float *)ref, (T *)f, EncF<DT, float>{});
  else
    k_ref_to_dev<<<tgrid(g, Q, g.pitch), dim3(32, 8), 0, s>>>(g, Q, (const double *)ref, (T *)f, EncF<DT, double>{});
  return cudaGetLastError();
}
template <int DT>
cudaError_t unpack_f_t(const Geom &g, int ref_dtype, const void *f, void *ref, cudaStream_t s) {
  using T = typename Store<DT>::T;
  if (ref_dtype == SW_F32)
    k_dev_to_ref<<<tgrid(g, Q, g.nx), dim3(32, 8), 0, s>>>(g, Q, (const T *)f, (float *)ref, DecF<DT, float>{});
  else
    k_dev_to_ref<<<tgrid(g, Q, g.nx), dim3(32, 8), 0, s>>>(g, Q, (const T *)f, (double *)ref, DecF<DT, double>{});
  return cudaGetLastError();
}

template <int DT>
cudaError_t init_t(const Geom &g, void *f, const uint8_t *flag, const float *uin, float noise, int seed, int kind,
                   cudaStream_t s) {
  const long long blocks = (g.plane + 255) / 256;
  k_init<DT><<<(unsigned)blocks, 256, 0, s>>>(g, (typename Store<DT>::T *)f, flag, uin, noise, seed, kind);
  return cudaGetLastError();
}
template <int DT>
cudaError_t macro_t(const Geom &g, const void *f, const uint8_t *flag, float *u, double *acc, cudaStream_t s) {
  const long long blocks = (g.plane + 255) / 256;
  k_macro<DT><<<(unsigned)blocks, 256, 0, s>>>(g, (const typename Store<DT>::T *)f, flag, u, acc);
  return cudaGetLastError();
}

#define SW_DISPATCH(dtype, CALL)                         \
  switch (dtype) {                                       \
    case SW_F32: { constexpr int DT = SW_F32; return CALL; } \
    case SW_F64: { constexpr int DT = SW_F64; return CALL; } \
    case SW_F16_SHIFT: { constexpr int DT = SW_F16_SHIFT; return CALL; } \
    case SW_BF16_SHIFT: { constexpr int DT = SW_BF16_SHIFT; return CALL; } \
    default: return cudaErrorInvalidValue;               \
  }

cudaError_t aux_init(const Geom &g, int dtype, void *f, const uint8_t *flag, const float *uin, float noise, int seed,
                     int kind, cudaStream_t s) {
  SW_DISPATCH(dtype, init_t<DT>(g, f, flag, uin, noise, seed, kind, s));
}
cudaError_t aux_macro(const Geom &g, int dtype, const void *f, const uint8_t *flag, float *u, double *acc,
                      cudaStream_t s) {
  SW_DISPATCH(dtype, macro_t<DT>(g, f, flag, u, acc, s));
}
cudaError_t aux_accum(const Geom &g, const float *u, double *acc, cudaStream_t s) {
  const long long blocks = (4 * g.plane + 255) / 256;
  k_accum<<<(unsigned)blocks, 256, 0, s>>>(g, u, acc);
  return cudaGetLastError();
}
cudaError_t aux_pack_f(const Geom &g, int dtype, int ref_dtype, const void *ref, void *f, cudaStream_t s) {
  SW_DISPATCH(dtype, pack_f_t<DT>(g, ref_dtype, ref, f, s));
}
cudaError_t aux_unpack_f(const Geom &g, int dtype, int ref_dtype, const void *f, void *ref, cudaStream_t s) {
  SW_DISPATCH(dtype, unpack_f_t<DT>(g, ref_dtype, f, ref, s));
}
cudaError_t aux_pack_flag(const Geom &g, const uint8_t *ref, uint8_t *flag, cudaStream_t s) {
  k_ref_to_dev<<<tgrid(g, 1, g.pitch), dim3(32, 8), 0, s>>>(g, 1, ref, flag, Ident<uint8_t>{});
  return cudaGetLastError();
}
cudaError_t aux_unpack_u(const Geom &g, const float *u, float *ref, cudaStream_t s) {
  k_dev_to_ref<<<tgrid(g, 4, g.nx), dim3(32, 8), 0, s>>>(g, 4, u, ref, Ident<float>{});
  return cudaGetLastError();
}
cudaError_t aux_unpack_acc(const Geom &g, const double *acc, double *ref, cudaStream_t s) {
  k_dev_to_ref<<<tgrid(g, 4, g.nx), dim3(32, 8), 0, s>>>(g, 4, acc, ref, Ident<double>{});
  return cudaGetLastError();
}
cudaError_t aux_build_tiles(const Geom &g, const uint8_t *flag, uint8_t *tiles, cudaStream_t s) {
  const long long blocks = (g.plane + 255) / 256;
  k_build_tiles<<<(unsigned)blocks, 256, 0, s>>>(g, flag, tiles);
  return cudaGetLastError();
}

__global__ void k_force_to_f64(const long long *fx, double *out, long long n) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = (double)fx[k] * (1.0 / FORCE_SCALE);
}
cudaError_t aux_force_to_f64(const long long *fx, double *out, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_force_to_f64<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(fx, out, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- wall-load coefficients
// lbm3d.py:396-407: per step t, Fx = sum_z F_x(z), Fz = sum_z F_z(z) and the
// overturning moment M = sum_z F_x(z) (z - 1/2) about the wall base, as
// Cd = Fx / (q A), Cl = Fz / (q A), Cm = M / (q A H), q A = U_H^2 / 2 * H ny.
// One warp per step: lanes over the levels (coalesced 16-byte rows), float64
// partial sums combined by an xor butterfly in a fixed order.
__global__ void k_coefficients(const long long *force, long long n_steps, int nz, double qa, double H,
                               double *coef) {
  const long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= n_steps) return;                                  // uniform across the warp
  const longlong2 *row = reinterpret_cast<const longlong2 *>(force + t * 2 * nz);
  double fx = 0.0, fz = 0.0, m = 0.0;
  for (int z = lane; z < nz; z += 32) {
    const longlong2 v = row[z];
    const double x = (double)v.x * (1.0 / FORCE_SCALE), y = (double)v.y * (1.0 / FORCE_SCALE);
    fx += x;
    fz += y;
    m += x * ((double)z - 0.5);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    fx += __shfl_xor_sync(0xffffffffu, fx, o);
    fz += __shfl_xor_sync(0xffffffffu, fz, o);
    m += __shfl_xor_sync(0xffffffffu, m, o);
  }
  if (lane == 0) {
    coef[t] = fx / qa;
    coef[n_steps + t] = fz / qa;
    coef[2 * n_steps + t] = m / (qa * H);
  }
}

// postprocess.py:65-82 over the steps t >= n_spin of the coefficient series:
// stats = mean Cd, max Cd, std Cd (about the mean, two passes), mean Cm, max Cm,
// mean Cl; NaN when no step is left.  One block; fixed reduction order.
constexpr int kStatThreads = 512;
__device__ __forceinline__ double block_sum(double v, double *sh) {
  const int tid = threadIdx.x;
  sh[tid] = v;
  __syncthreads();
  for (int s = kStatThreads / 2; s > 0; s >>= 1) {
    if (tid < s) sh[tid] += sh[tid + s];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}
__device__ __forceinline__ double block_max(double v, double *sh) {
  const int tid = threadIdx.x;
  sh[tid] = v;
  __syncthreads();
  for (int s = kStatThreads / 2; s > 0; s >>= 1) {
    if (tid < s) sh[tid] = fmax(sh[tid], sh[tid + s]);
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}
__global__ void __launch_bounds__(kStatThreads) k_coef_stats(const double *coef, long long n_steps, long long n_spin,
                                                            double *stats) {
  __shared__ double sh[kStatThreads];
  const double *cd = coef, *cl = coef + n_steps, *cm = coef + 2 * n_steps;
  const long long n = n_steps - n_spin;
  if (n <= 0) {
    if (threadIdx.x < 6) stats[threadIdx.x] = __longlong_as_double(0x7ff8000000000000ll);   // quiet NaN
    return;
  }
  double s_cd = 0.0, s_cm = 0.0, s_cl = 0.0, m_cd = -1.0 / 0.0, m_cm = -1.0 / 0.0;
  for (long long t = n_spin + threadIdx.x; t < n_steps; t += kStatThreads) {
    s_cd += cd[t];
    s_cm += cm[t];
    s_cl += cl[t];
    m_cd = fmax(m_cd, cd[t]);
    m_cm = fmax(m_cm, cm[t]);
  }
  const double mean_cd = block_sum(s_cd, sh) / (double)n;
  const double mean_cm = block_sum(s_cm, sh) / (double)n;
  const double mean_cl = block_sum(s_cl, sh) / (double)n;
  const double max_cd = block_max(m_cd, sh), max_cm = block_max(m_cm, sh);
  double s_dev = 0.0;
  for (long long t = n_spin + threadIdx.x; t < n_steps; t += kStatThreads) {
    const double d = cd[t] - mean_cd;
    s_dev += d * d;
  }
  const double var = block_sum(s_dev, sh) / (double)n;
  if (threadIdx.x == 0) {
    stats[0] = mean_cd;
    stats[1] = max_cd;
    stats[2] = sqrt(var);
    stats[3] = mean_cm;
    stats[4] = max_cm;
    stats[5] = mean_cl;
  }
}

cudaError_t aux_coefficients(const long long *force, long long n_steps, int nz, double qa, double H, double *coef,
                             cudaStream_t s) {
  if (n_steps <= 0) return cudaSuccess;
  const long long threads = n_steps * 32;
  k_coefficients<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(force, n_steps, nz, qa, H, coef);
  return cudaGetLastError();
}
cudaError_t aux_coef_stats(const double *coef, long long n_steps, long long n_spin, double *stats, cudaStream_t s) {
  k_coef_stats<<<1, kStatThreads, 0, s>>>(coef, n_steps, n_spin, stats);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- recirculation area
// export3d.py:169-184 on the every-2nd-cell mean field (lbm3d.py:412): the box
// of cells (2 (i0 + i), 2 j, 2 k), i < I, j < J, k < K, holds u_x of the time
// mean (sums / n_acc in float64, rounded to float) or 0.05 at non-fluid cells,
// divided by U_H in float; level k = 0 takes level 1's value; one 3-point box
// blur with edge clamping along i, then j, then k ((a + b) + c, then / 3, in
// float); the reverse-flow cells are those left below zero.  Built without FMA
// contraction (the file's --fmad=false) and with explicitly rounded operations,
// so the count equals the float32 NumPy restatement's.  Scratch layout
// [k][j][i].
struct RecircBox {
  int i0, I, J, K;
};
__global__ void k_recirc_gather(Geom g, RecircBox b, const double *acc, double n, const uint8_t *flag, float uh,
                                float *out) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)b.I * b.J * b.K) return;
  const int i = (int)(e % b.I), j = (int)((e / b.I) % b.J), k = (int)(e / ((long long)b.I * b.J));
  const int x = 2 * (b.i0 + i), y = 2 * j, z = 2 * (k == 0 ? 1 : k);
  const size_t c = ((size_t)z * g.ny + y) * g.pitch + x;
  const float v = flag[c] != 0 ? 0.05f : __double2float_rn(__ddiv_rn(acc[(size_t)g.plane + c], n));
  out[e] = __fdiv_rn(v, uh);
}
// AXIS 0: i, 1: j, 2: k.  With COUNT the result is not stored: each cell below
// zero adds one to *count (one atomic per warp).
template <int AXIS, bool COUNT>
__global__ void k_recirc_blur(RecircBox b, const float *in, float *out, unsigned long long *count) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)b.I * b.J * b.K;
  bool neg = false;
  if (e < n) {
    const int i = (int)(e % b.I), j = (int)((e / b.I) % b.J), k = (int)(e / ((long long)b.I * b.J));
    const int at = AXIS == 0 ? i : AXIS == 1 ? j : k;
    const int len = AXIS == 0 ? b.I : AXIS == 1 ? b.J : b.K;
    const long long step = AXIS == 0 ? 1 : AXIS == 1 ? (long long)b.I : (long long)b.I * b.J;
    const float lo = in[e - (at > 0 ? step : 0)], mid = in[e], hi = in[e + (at + 1 < len ? step : 0)];
    const float v = __fdiv_rn(__fadd_rn(__fadd_rn(lo, mid), hi), 3.0f);
    if (COUNT) neg = v < 0.0f;
    else out[e] = v;
  }
  if (COUNT) {
    const unsigned m = __ballot_sync(0xffffffffu, neg);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
  }
}
cudaError_t aux_recirc_count(const Geom &g, int i0, int I, int J, int K, const double *acc, long long n_acc,
                             const uint8_t *flag, float uh, float *scratch, long long *count, cudaStream_t s) {
  const RecircBox b{i0, I, J, K};
  const long long n = (long long)I * J * K;
  float *a = scratch, *t = scratch + n;
  unsigned long long *cnt = reinterpret_cast<unsigned long long *>(count);
  cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(*cnt), s);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  k_recirc_gather<<<blocks, 256, 0, s>>>(g, b, acc, (double)(n_acc > 0 ? n_acc : 1), flag, uh, a);
  k_recirc_blur<0, false><<<blocks, 256, 0, s>>>(b, a, t, nullptr);
  k_recirc_blur<1, false><<<blocks, 256, 0, s>>>(b, t, a, nullptr);
  k_recirc_blur<2, true><<<blocks, 256, 0, s>>>(b, a, nullptr, cnt);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- viewer payload
// k_slice_xz / k_slice_xy (lbm3d.py:191-200): the macro field u (device layout
// [4][nz][ny][pitch]) at y = y0 or z = z0, written in the reference layout
// out[c][x][z] / out[c][x][y].
__global__ void k_slice_xz(Geom g, const float *u, int y0, float *out) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 4ll * g.nx * g.nz) return;
  const int z = (int)(k % g.nz), x = (int)((k / g.nz) % g.nx), c = (int)(k / ((long long)g.nz * g.nx));
  out[k] = u[(size_t)c * g.plane + ((size_t)z * g.ny + y0) * g.pitch + x];
}
__global__ void k_slice_xy(Geom g, const float *u, int z0, float *out) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 4ll * g.nx * g.ny) return;
  const int y = (int)(k % g.ny), x = (int)((k / g.ny) % g.nx), c = (int)(k / ((long long)g.ny * g.nx));
  out[k] = u[(size_t)c * g.plane + ((size_t)z0 * g.ny + y) * g.pitch + x];
}

// Q-criterion at one cell (q_at, lbm3d.py:203-222): -1/2 A_ij A_ji of the
// central-difference velocity gradient, 0 next to any non-fluid cell; y
// periodic.  Float32 in the reference's evaluation order (this translation
// unit is compiled without multiply-add contraction).
__device__ float q_at(const Geom &g, const float *u, const uint8_t *flag, int x, int y, int z) {
  const int yp = (y + 1) % g.ny, ym = (y - 1 + g.ny) % g.ny;
  auto fl = [&](int xx, int yy, int zz) { return flag[((size_t)zz * g.ny + yy) * g.pitch + xx]; };
  if (fl(x, y, z) != 0 || fl(x + 1, y, z) != 0 || fl(x - 1, y, z) != 0 || fl(x, yp, z) != 0 || fl(x, ym, z) != 0 ||
      fl(x, y, z + 1) != 0 || fl(x, y, z - 1) != 0)
    return 0.0f;
  auto U = [&](int c, int xx, int yy, int zz) { return u[(size_t)c * g.plane + ((size_t)zz * g.ny + yy) * g.pitch + xx]; };
  const float a11 = 0.5f * (U(1, x + 1, y, z) - U(1, x - 1, y, z));
  const float a12 = 0.5f * (U(1, x, yp, z) - U(1, x, ym, z));
  const float a13 = 0.5f * (U(1, x, y, z + 1) - U(1, x, y, z - 1));
  const float a21 = 0.5f * (U(2, x + 1, y, z) - U(2, x - 1, y, z));
  const float a22 = 0.5f * (U(2, x, yp, z) - U(2, x, ym, z));
  const float a23 = 0.5f * (U(2, x, y, z + 1) - U(2, x, y, z - 1));
  const float a31 = 0.5f * (U(3, x + 1, y, z) - U(3, x - 1, y, z));
  const float a32 = 0.5f * (U(3, x, yp, z) - U(3, x, ym, z));
  const float a33 = 0.5f * (U(3, x, y, z + 1) - U(3, x, y, z - 1));
  return -0.5f * (a11 * a11 + a22 * a22 + a33 * a33 + 2.0f * (a12 * a21 + a13 * a31 + a23 * a32));
}

// k_qcoarse (lbm3d.py:225-238): max of max(Q, 0) over ds^3 blocks of the crop
// starting at (x0, 0, 0); out[i][j][k], one thread per output voxel.
__global__ void k_qcoarse(Geom g, const float *u, const uint8_t *flag, int x0, int ds, int di, int dj, int dk,
                          float *out) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= (long long)di * dj * dk) return;
  const int k = (int)(n % dk), j = (int)((n / dk) % dj), i = (int)(n / ((long long)dk * dj));
  float best = 0.0f;
  for (int a = 0; a < ds; ++a)
    for (int b = 0; b < ds; ++b)
      for (int c = 0; c < ds; ++c) {
        const int x = x0 + i * ds + a, y = j * ds + b, z = k * ds + c;
        if (x >= 1 && x < g.nx - 1 && z >= 1 && z < g.nz - 1) best = fmaxf(best, q_at(g, u, flag, x, y, z));
      }
  out[n] = best;
}

cudaError_t aux_slice_xz(const Geom &g, const float *u, int y0, float *out, cudaStream_t s) {
  const long long n = 4ll * g.nx * g.nz;
  k_slice_xz<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, u, y0, out);
  return cudaGetLastError();
}
cudaError_t aux_slice_xy(const Geom &g, const float *u, int z0, float *out, cudaStream_t s) {
  const long long n = 4ll * g.nx * g.ny;
  k_slice_xy<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, u, z0, out);
  return cudaGetLastError();
}
cudaError_t aux_qcoarse(const Geom &g, const float *u, const uint8_t *flag, int x0, int ds, int di, int dj, int dk,
                        float *out, cudaStream_t s) {
  const long long n = (long long)di * dj * dk;
  if (n == 0) return cudaSuccess;
  k_qcoarse<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(g, u, flag, x0, ds, di, dj, dk, out);
  return cudaGetLastError();
}

}  // namespace sw
