// sw_step.cuh -- the fused D3Q19 timestep (pull streaming + boundaries + bounce-back +
// momentum exchange + regularized BGK with Smagorinsky and the outlet sponge).
//
// Follows k_step of stonewall3d/lbm3d.py:57-155 term by term.  Differences in
// form, none in result beyond floating-point contraction:
//  * one warp = one 32-cell row segment along x; a byte per segment (tiles[])
//    says whether any pull source can be non-fluid.  Segments that cannot
//    (the bulk of the domain) skip the 19 neighbour flag loads of
//    lbm3d.py:88 and the force bookkeeping;
//  * products with a zero lattice component (v * 0, lbm3d.py:119-127, 153-154)
//    are skipped: for finite values they add +-0 and change nothing;
//  * the per-cell wall force is summed per warp in float64 (xor butterfly,
//    fixed order) and added to force[t][z] as 2^-40 fixed point with one
//    64-bit integer atomic per warp, so the totals are independent of warp
//    scheduling (the reference adds float32 atomics per cell, lbm3d.py:99-101).
#pragma once
#include "sw_common.cuh"

namespace sw {

struct StepParams {
  const void *fin;
  void *fout;
  const uint8_t *flag;
  const uint8_t *tiles;
  const float *uin;
  Geom g;
  double nu0, cs, nu_sponge;
  int x_sponge;
  long long *force;  // force row of this step: [nz][2], or nullptr
};

// Regularized-BGK collision of one cell from its 19 pulled populations fl[],
// lbm3d.py:103-155.  Writes f_out through `put(Int<i>, value)`.
template <typename R, typename Put>
__device__ __forceinline__ void collide(const R (&fl)[Q], int x, const Geom &g, R nu0, R cs, int x_sponge,
                                        R nu_sponge, Put &&put) {
  R rho = R(0.0), mx = R(0.0), my = R(0.0), mz = R(0.0);
  R pxx = R(0.0), pyy = R(0.0), pzz = R(0.0), pxy = R(0.0), pxz = R(0.0), pyz = R(0.0);
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ex = CX(i), ey = CY(i), ez = CZ(i);
    const R v = fl[i];
    rho += v;
    if constexpr (ex != 0) mx += (ex > 0 ? v : -v);
    if constexpr (ey != 0) my += (ey > 0 ? v : -v);
    if constexpr (ez != 0) mz += (ez > 0 ? v : -v);
    if constexpr (ex != 0) pxx += v;
    if constexpr (ey != 0) pyy += v;
    if constexpr (ez != 0) pzz += v;
    if constexpr (ex * ey != 0) pxy += (ex * ey > 0 ? v : -v);
    if constexpr (ex * ez != 0) pxz += (ex * ez > 0 ? v : -v);
    if constexpr (ey * ez != 0) pyz += (ey * ez > 0 ? v : -v);
  });
  const R ux = mx / rho, uy = my / rho, uz = mz / rho;
  const R third = rho / R(3.0);
  const R nxx = pxx - third - rho * ux * ux;
  const R nyy = pyy - third - rho * uy * uy;
  const R nzz = pzz - third - rho * uz * uz;
  const R nxy = pxy - rho * ux * uy;
  const R nxz = pxz - rho * ux * uz;
  const R nyz = pyz - rho * uy * uz;
  R nu = nu0;
  if (x > x_sponge) {
    const R s = R(x - x_sponge) / R(g.nx - x_sponge);
    nu = nu0 + nu_sponge * s * s;
  }
  const R tau0 = R(3.0) * nu + R(0.5);
  const R qn = sqrt(nxx * nxx + nyy * nyy + nzz * nzz + R(2.0) * (nxy * nxy + nxz * nxz + nyz * nyz));
  const R tau = R(0.5) * (tau0 + sqrt(tau0 * tau0 + R(18.0) * sqrt(R(2.0)) * cs * cs * qn / rho));
  const R keep = R(1.0) - R(1.0) / tau;
  const R usq = ux * ux + uy * uy + uz * uz;
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ex = CX(i), ey = CY(i), ez = CZ(i);
    constexpr R third_c = R(1.0) / R(3.0);
    constexpr R kx = R(ex * ex) - third_c, ky = R(ey * ey) - third_c, kz = R(ez * ez) - third_c;
    R off = R(0.0);
    if constexpr (ex * ey != 0) off += (ex * ey > 0 ? nxy : -nxy);
    if constexpr (ex * ez != 0) off += (ex * ez > 0 ? nxz : -nxz);
    if constexpr (ey * ez != 0) off += (ey * ez > 0 ? nyz : -nyz);
    const R qq = kx * nxx + ky * nyy + kz * nzz + R(2.0) * off;
    R cu = R(0.0);
    if constexpr (ex != 0) cu += (ex > 0 ? ux : -ux);
    if constexpr (ey != 0) cu += (ey > 0 ? uy : -uy);
    if constexpr (ez != 0) cu += (ez > 0 ? uz : -uz);
    cu = R(3.0) * cu;
    const R feq = W<R>(i) * rho * (R(1.0) + cu + R(0.5) * cu * cu - R(1.5) * usq);
    put(Int<i>{}, feq + keep * W<R>(i) * R(4.5) * qq);
  });
}

// One cell of the pull-scheme step.  CHECK selects the path with neighbour flag
// tests (segments next to stones, the ground or a fluid cell at z = 0).
template <int DT, bool CHECK>
__device__ __forceinline__ void step_cell(const StepParams &p, int x, int y, int z, typename Store<DT>::R &fxw,
                                          typename Store<DT>::R &fzw, int &hit) {
  using S = Store<DT>;
  using T = typename S::T;
  using R = typename S::R;
  const Geom &g = p.g;
  const T *__restrict__ fin = static_cast<const T *>(p.fin);
  T *__restrict__ fout = static_cast<T *>(p.fout);
  const size_t plane = (size_t)g.plane;
  const unsigned c = ((unsigned)z * g.ny + y) * g.pitch + x;
  if (CHECK && p.flag[c] != 0) return;                          // lbm3d.py:65-66
  if (x == 0) {                                                 // inlet, lbm3d.py:67-71
    const R u0 = (R)__ldg(p.uin + z);
    const R usq = u0 * u0;
    static_for<0, Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      constexpr int ex = CX(i);
      R cu = R(0.0);
      if constexpr (ex != 0) cu = (ex > 0 ? u0 : -u0);
      cu = R(3.0) * cu;
      const R v = W<R>(i) * R(1.0) * (R(1.0) + cu + R(0.5) * cu * cu - R(1.5) * usq);
      S::template st<i>(fout + (size_t)i * plane + c, v);
    });
    return;
  }
  // pull sources (lbm3d.py:77-86): periodic y, outlet copies column x, top mirrors z
  const int ym = (y == 0) ? g.ny - 1 : y - 1;    // source row of c_y = +1
  const int yp = (y == g.ny - 1) ? 0 : y + 1;    // source row of c_y = -1
  const bool top = (z == g.nz - 1);
  const int zp = top ? z : z + 1;                // source level of c_z = -1
  const int xp = (x + 1 >= g.nx) ? x : x + 1;    // source column of c_x = -1
  R fl[Q];
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ex = CX(i), ey = CY(i), ez = CZ(i);
    const int xs = ex == 1 ? x - 1 : (ex == -1 ? xp : x);
    const int ys = ey == 1 ? ym : (ey == -1 ? yp : y);
    const int zs = ez == 1 ? z - 1 : (ez == -1 ? zp : z);
    const unsigned src = ((unsigned)zs * g.ny + ys) * g.pitch + xs;
    bool pull = true;
    if constexpr (CHECK) {
      // a source below z = 0 (only for a fluid cell in the bottom plane, which
      // the reference never has) is treated as ground
      const uint8_t fs = (ez == 1 && z == 0) ? (uint8_t)SW_GROUND : __ldg(p.flag + src);
      if (fs != 0) {                                            // lbm3d.py:89-95
        pull = false;
        const R val = S::template ld<OPP(i)>(fin + (size_t)OPP(i) * plane + c);
        if (fs == SW_WALL) {
          const R fr = val - W<R>(i);
          if constexpr (ex != 0) fxw = fxw - R(2.0) * fr * R(ex);
          if constexpr (ez != 0) fzw = fzw - R(2.0) * fr * R(ez);
          hit = 1;
        }
        fl[i] = val;
      }
    }
    if (pull) {                                                 // lbm3d.py:97
      if constexpr (ez == -1) {
        if (top) fl[i] = S::template ld<MIRZ(i)>(fin + (size_t)MIRZ(i) * plane + src);
        else fl[i] = S::template ld<i>(fin + (size_t)i * plane + src);
      } else {
        fl[i] = S::template ld<i>(fin + (size_t)i * plane + src);
      }
    }
  });
  collide<R>(fl, x, g, (R)p.nu0, (R)p.cs, p.x_sponge, (R)p.nu_sponge, [&](auto I, R v) {
    constexpr int i = decltype(I)::value;
    S::template st<i>(fout + (size_t)i * plane + c, v);
  });
}

constexpr int STEP_THREADS = 256;
constexpr int STEP_WARPS = STEP_THREADS / 32;

template <int DT>
__global__ void __launch_bounds__(STEP_THREADS) k_step_pull(StepParams p) {
  using R = typename Store<DT>::R;
  const int seg = blockIdx.x * STEP_WARPS + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const Geom &g = p.g;
  if (seg >= g.nseg_x * g.ny * g.nz) return;
  const uint8_t kind = __ldg(p.tiles + seg);
  if (kind & TILE_ALL_SOLID) return;
  const int sx = seg % g.nseg_x;
  const int row = seg / g.nseg_x;
  const int y = row % g.ny, z = row / g.ny;
  const int x = sx * SEG + lane;
  R fxw = R(0.0), fzw = R(0.0);
  int hit = 0;
  if (!(kind & TILE_CHECK)) {
    if (x < g.nx) step_cell<DT, false>(p, x, y, z, fxw, fzw, hit);
    return;
  }
  if (x < g.nx) step_cell<DT, true>(p, x, y, z, fxw, fzw, hit);
  if ((kind & TILE_FORCE) && p.force != nullptr) {              // lbm3d.py:99-101
    double dx = (double)fxw, dz = (double)fzw;
    const unsigned any = __ballot_sync(0xffffffffu, hit);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      dx += __shfl_xor_sync(0xffffffffu, dx, o);
      dz += __shfl_xor_sync(0xffffffffu, dz, o);
    }
    if (lane == 0 && any) {
      atomicAdd(reinterpret_cast<unsigned long long *>(p.force + 2 * z),
                (unsigned long long)__double2ll_rn(dx * FORCE_SCALE));
      atomicAdd(reinterpret_cast<unsigned long long *>(p.force + 2 * z + 1),
                (unsigned long long)__double2ll_rn(dz * FORCE_SCALE));
    }
  }
}

template <int DT>
cudaError_t launch_step(const StepParams &p, cudaStream_t s) {
  const long long nseg = (long long)p.g.nseg_x * p.g.ny * p.g.nz;
  const long long blocks = (nseg + STEP_WARPS - 1) / STEP_WARPS;
  k_step_pull<DT><<<(unsigned)blocks, STEP_THREADS, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace sw
