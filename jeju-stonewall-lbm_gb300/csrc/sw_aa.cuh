// sw_aa.cuh -- the AA-pattern (in-place, one lattice) variant of the fused step.
//
// One lattice A instead of two.  Steps alternate between two kernels, always
// an odd step first; between an even step and the next odd one the state S
// (post-collision populations) sits in A in natural planes, A[k] = S_k, as
// after k_init or a checkpoint load.
//   odd  step: each cell pulls exactly as the two-lattice step does (same
//              sources, same bounce-back, same force), collides, and scatters
//              every new S_k to the slot(s) where the next even step will
//              find it:
//                (a) slot k of x + c_k (y periodic) when that cell is fluid,
//                (b) at the outlet, c_x = -1: slot k of (nx-1, y+c_y, z+c_z),
//                    the cell that copies column nx-1 there,
//                (c) at the top, c_z = +1: slot MIRZ(k) of (x+c_x, y+c_y, nz-1),
//                    and at the outlet also of (nx-1, y+c_y, nz-1),
//                (d) slot opp(k) of x itself when the pull of opp(k) bounces;
//   even step: each cell reads its 19 incoming values from its own slots,
//              collides, writes S_k to slot opp(k) of its own cell.
// Slot s lives in plane opp(s) (a fixed relabelling of the planes), so the
// even step's S_k lands in plane k: natural planes again.  With that
// labelling every slot the odd step reads (S_i of x - c_i is slot opp(i) of
// x - c_i, or slot i of x itself for a bounce-back) is written, if at all,
// only by the cell that reads it, so the step is race-free in place -- except
// the outlet copy (a cell at x = nx-1 takes c_x = -1 populations from its own
// column, slots other cells rewrite in the same step).  Those five
// populations of the outlet plane are copied to a ghost buffer before the odd
// step and read from there.  The plan is checked on the CPU
// (tests/aa_model.py) and against the two-lattice step on the GPU.
#pragma once
#include "sw_step.cuh"

namespace sw {

// ghost slot of a c_x = -1 population (2, 8, 10, 12, 14)
__host__ __device__ constexpr int GIDX(int j) {
  return j == 2 ? 0 : j == 8 ? 1 : j == 10 ? 2 : j == 12 ? 3 : j == 14 ? 4 : -1;
}
constexpr int kGhostPops = 5;

struct AAParams {
  const void *ghost;  // [5][nz][ny] stored values of the outlet plane, before the odd step
  void *ghost_w;      // same buffer, written by k_aa_ghost
};

// Outlet plane's c_x = -1 populations -> ghost.  One thread per (y, z).
template <int DT>
__global__ void k_aa_ghost(const __grid_constant__ StepParams p, AAParams a) {
  using T = typename Store<DT>::T;
  const int y = blockIdx.x * blockDim.x + threadIdx.x, z = blockIdx.y;
  const Geom &g = p.g;
  if (y >= g.ny) return;
  const int c = (z * g.ny + y) * g.pitch + (g.nx - 1);
  T *gw = static_cast<T *>(a.ghost_w);
  const size_t gp = (size_t)g.ny * g.nz;
  static_for<0, Q>([&](auto I) {
    constexpr int j = decltype(I)::value;
    if constexpr (GIDX(j) >= 0) gw[GIDX(j) * gp + (size_t)z * g.ny + y] = p.template in<T>(j)[c];
  });
}

// Decoded stored value in the compute domain (g for shifted formats, f otherwise).
template <int DT, int I>
__device__ __forceinline__ typename Store<DT>::R aa_ld(const typename Store<DT>::T *q) {
  using S = Store<DT>;
  if constexpr (S::kShift) return S::to_shifted(*q);       // g for the shifted formats
  else return *q;                                           // coherent loads: the lattice is written in place
}

template <int DT, bool CHECK, bool ACC>
__device__ __forceinline__ void aa_odd_cell(const StepParams &p, const AAParams &a, int x, int y, int z,
                                            typename Store<DT>::R &fxw, typename Store<DT>::R &fzw, int &hit) {
  using S = Store<DT>;
  using T = typename S::T;
  using R = typename S::R;
  const Geom &g = p.g;
  const int c = (z * g.ny + y) * g.pitch + x;
  if (CHECK && p.flag[c] != 0) return;
  const int row = g.pitch, lev = g.ny * g.pitch;
  const int off_ym = (y == 0) ? (g.ny - 1) * row : -row;        // row of y - 1 (periodic)
  const int off_yp = (y == g.ny - 1) ? -(g.ny - 1) * row : row; // row of y + 1 (periodic)
  const bool top = (z == g.nz - 1), outlet = (x == g.nx - 1);
  unsigned bounced = 0;
  R fl[Q];
  R u0 = R(0.0);
  if (x == 0) {                                                 // inlet: equilibrium, no pulls
    u0 = (R)__ldg(p.uin + z);
  } else {
    const int off_xp = outlet ? 0 : 1;
    const int off_zp = top ? 0 : lev;
    const T *ghost = static_cast<const T *>(a.ghost);
    const size_t gp = (size_t)g.ny * g.nz;
    static_for<0, Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      constexpr int ex = CX(i), ey = CY(i), ez = CZ(i);
      const int src = c + (ex == 1 ? -1 : ex == -1 ? off_xp : 0) + (ey == 1 ? off_ym : ey == -1 ? off_yp : 0) +
                      (ez == 1 ? -lev : ez == -1 ? off_zp : 0);
      bool pull = true;
      if constexpr (CHECK) {
        const uint8_t fs = (ez == 1 && z == 0) ? (uint8_t)SW_GROUND : __ldg(p.flag + src);
        if (fs != 0) {                                          // bounce-back: own cell's opposite population
          pull = false;
          bounced |= 1u << i;
          const R val = aa_ld<DT, OPP(i)>(p.template in<T>(OPP(i)) + c);
          if (fs == SW_WALL) {
            const R fr = S::kShift ? val : val - W<R>(i);
            if constexpr (ex != 0) fxw = fxw - R(2.0) * fr * R(ex);
            if constexpr (ez != 0) fzw = fzw - R(2.0) * fr * R(ez);
            hit = 1;
          }
          fl[i] = val;
        }
      }
      if (pull) {
        constexpr int jm = MIRZ(i);
        if constexpr (ex == -1) {
          if (outlet) {                                         // outlet copy: from the ghost
            const int ys = ey == 1 ? (y == 0 ? g.ny - 1 : y - 1) : ey == -1 ? (y == g.ny - 1 ? 0 : y + 1) : y;
            const int zs = ez == 1 ? z - 1 : (ez == -1 ? (top ? z : z + 1) : z);
            const size_t go = (size_t)zs * g.ny + ys;
            if (ez == -1 && top) fl[i] = S::template ld<jm>(ghost + GIDX(jm) * gp + go);
            else fl[i] = S::template ld<i>(ghost + GIDX(i) * gp + go);
          } else if (ez == -1 && top) {
            fl[i] = aa_ld<DT, jm>(p.template in<T>(jm) + src);
          } else {
            fl[i] = aa_ld<DT, i>(p.template in<T>(i) + src);
          }
        } else if constexpr (ez == -1) {
          if (top) fl[i] = aa_ld<DT, jm>(p.template in<T>(jm) + src);
          else fl[i] = aa_ld<DT, i>(p.template in<T>(i) + src);
        } else {
          fl[i] = aa_ld<DT, i>(p.template in<T>(i) + src);
        }
      }
    });
  }
  // scatter of S_k to the slots the next even step reads (physical planes: fout_pop).
  // A segment without the checked path has only fluid neighbours around its
  // pulling cells; an inlet cell does not pull, so its targets are checked.
  const bool chk = CHECK || x == 0;
  auto scatter = [&](auto I, R v) {
    constexpr int k = decltype(I)::value;
    constexpr int ex = CX(k), ey = CY(k), ez = CZ(k);
    T *pl = p.template out<T>(k);
    const int oy = ey == 1 ? off_yp : ey == -1 ? off_ym : 0;   // row of y + c_y
    if (CHECK && (bounced >> OPP(k)) & 1u)                      // (d)
      S::template st<k>(p.template out<T>(OPP(k)) + c, v);
    const int tx = x + ex, tz = z + ez;
    if (tx >= 0 && tx < g.nx && tz >= 0 && tz < g.nz) {          // (a)
      const int t = c + ex + oy + ez * lev;
      if (!chk || p.flag[t] == 0) S::template st<k>(pl + t, v);
    }
    if constexpr (ex == -1) {
      if (outlet && tz >= 0 && tz < g.nz) {                       // (b)
        const int t = c + oy + ez * lev;
        if (!chk || p.flag[t] == 0) S::template st<k>(pl + t, v);
      }
    }
    if constexpr (ez == 1) {
      if (top) {                                                  // (c)
        T *pm = p.template out<T>(MIRZ(k));
        if (tx >= 0 && tx < g.nx) {
          const int t = c + ex + oy;
          if (!chk || p.flag[t] == 0) S::template st<MIRZ(k)>(pm + t, v);
        }
        if (ex == -1 && outlet) {
          const int t = c + oy;
          if (!chk || p.flag[t] == 0) S::template st<MIRZ(k)>(pm + t, v);
        }
      }
    }
  };
  R rho, ux, uy, uz;
  if (x == 0) {
    const R usq = u0 * u0;
    static_for<0, Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      constexpr int ex = CX(i);
      R cu = R(0.0);
      if constexpr (ex != 0) cu = (ex > 0 ? u0 : -u0);
      cu = R(3.0) * cu;
      const R v = W<R>(i) * R(1.0) * (R(1.0) + cu + R(0.5) * cu * cu - R(1.5) * usq);
      scatter(I, S::kShift ? v - W<R>(i) : v);
    });
    rho = R(1.0); ux = u0; uy = R(0.0); uz = R(0.0);
  } else {
    const Phys<R> ph = phys<R>(p);
    collide<R, S::kShift>(fl, x, ph.nu0, ph.c18, p.x_sponge, ph.sponge_scale, ph.nu_sponge, rho, ux, uy, uz,
                          p.status, scatter);
  }
  if (ACC) {
    atomicAdd(p.accp(0) + c, (double)rho);
    atomicAdd(p.accp(1) + c, (double)ux);
    atomicAdd(p.accp(2) + c, (double)uy);
    atomicAdd(p.accp(3) + c, (double)uz);
  }
}

template <int DT, bool CHECK, bool ACC>
__device__ __forceinline__ void aa_even_cell(const StepParams &p, int x, int y, int z, typename Store<DT>::R &fxw,
                                             typename Store<DT>::R &fzw, int &hit) {
  using S = Store<DT>;
  using T = typename S::T;
  using R = typename S::R;
  const Geom &g = p.g;
  const int c = (z * g.ny + y) * g.pitch + x;
  if (CHECK && p.flag[c] != 0) return;
  R rho, ux, uy, uz;
  // own cell: incoming values in natural slots (fin_pop), results to opposite slots (fout_pop is permuted)
  auto put = [&](auto I, R v) {
    constexpr int k = decltype(I)::value;
    S::template st<k>(p.template out<T>(k) + c, v);
  };
  if (x == 0) {
    const R u0 = (R)__ldg(p.uin + z);
    const R usq = u0 * u0;
    static_for<0, Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      constexpr int ex = CX(i);
      R cu = R(0.0);
      if constexpr (ex != 0) cu = (ex > 0 ? u0 : -u0);
      cu = R(3.0) * cu;
      const R v = W<R>(i) * R(1.0) * (R(1.0) + cu + R(0.5) * cu * cu - R(1.5) * usq);
      put(I, S::kShift ? v - W<R>(i) : v);
    });
    rho = R(1.0); ux = u0; uy = R(0.0); uz = R(0.0);
  } else {
    R fl[Q];
    static_for<0, Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      fl[i] = aa_ld<DT, i>(p.template in<T>(i) + c);
    });
    if constexpr (CHECK) {                                      // momentum exchange (lbm3d.py:91-95)
      const int row = g.pitch, lev = g.ny * g.pitch;
      const int off_ym = (y == 0) ? (g.ny - 1) * row : -row;
      const int off_yp = (y == g.ny - 1) ? -(g.ny - 1) * row : row;
      const int off_xp = (x + 1 >= g.nx) ? 0 : 1;
      const int off_zp = (z == g.nz - 1) ? 0 : lev;
      static_for<0, Q>([&](auto I) {
        constexpr int i = decltype(I)::value;
        constexpr int ex = CX(i), ey = CY(i), ez = CZ(i);
        if constexpr (ex != 0 || ez != 0) {
          const int src = c + (ex == 1 ? -1 : ex == -1 ? off_xp : 0) + (ey == 1 ? off_ym : ey == -1 ? off_yp : 0) +
                          (ez == 1 ? -lev : ez == -1 ? off_zp : 0);
          const uint8_t fs = (ez == 1 && z == 0) ? (uint8_t)SW_GROUND : __ldg(p.flag + src);
          if (fs == SW_WALL) {                                  // fl[i] holds the bounced f_opp(i)(x)
            const R fr = S::kShift ? fl[i] : fl[i] - W<R>(i);
            if constexpr (ex != 0) fxw = fxw - R(2.0) * fr * R(ex);
            if constexpr (ez != 0) fzw = fzw - R(2.0) * fr * R(ez);
            hit = 1;
          }
        }
      });
    }
    const Phys<R> ph = phys<R>(p);
    collide<R, S::kShift>(fl, x, ph.nu0, ph.c18, p.x_sponge, ph.sponge_scale, ph.nu_sponge, rho, ux, uy, uz,
                          p.status, put);
  }
  if (ACC) {
    atomicAdd(p.accp(0) + c, (double)rho);
    atomicAdd(p.accp(1) + c, (double)ux);
    atomicAdd(p.accp(2) + c, (double)uy);
    atomicAdd(p.accp(3) + c, (double)uz);
  }
}

template <int DT, bool ODD, bool ACC, typename Cfg>
__global__ void __launch_bounds__(Cfg::THREADS, Cfg::MINB) k_step_aa(const __grid_constant__ StepParams p, AAParams a) {
  using R = typename Store<DT>::R;
  const Geom &g = p.g;
  const int y = blockIdx.y * Cfg::WY + threadIdx.y;
  if (y >= g.ny) return;
  const int z = blockIdx.z, lane = threadIdx.x;
  const int seg = (z * g.ny + y) * g.nseg_x + blockIdx.x;
  const uint8_t kind = __ldg(p.tiles + seg);
  if (kind & TILE_ALL_SOLID) return;
  const int x = blockIdx.x * SEG + lane;
  R fxw = R(0.0), fzw = R(0.0);
  int hit = 0;
  if (!(kind & TILE_CHECK)) {
    if (x < g.nx) {
      if (ODD) aa_odd_cell<DT, false, ACC>(p, a, x, y, z, fxw, fzw, hit);
      else aa_even_cell<DT, false, ACC>(p, x, y, z, fxw, fzw, hit);
    }
    return;
  }
  if (x < g.nx) {
    if (ODD) aa_odd_cell<DT, true, ACC>(p, a, x, y, z, fxw, fzw, hit);
    else aa_even_cell<DT, true, ACC>(p, x, y, z, fxw, fzw, hit);
  }
  if ((kind & TILE_FORCE) && p.force != nullptr) warp_force_add<R>(p, z, lane, fxw, fzw, hit);
}

// One AA step.  odd: reads natural planes, writes slot s to plane opp(s);
// even: reads slot s from plane opp(s), writes S_k to plane k.
template <int DT>
cudaError_t launch_aa(const StepParams &p_in, const AAParams &a, bool odd, cudaStream_t s) {
  using T = typename Store<DT>::T;
  if (p_in.g.nz > 65535 || (p_in.g.ny + 3) / 4 > 65535) return cudaErrorInvalidValue;
  StepParams p = p_in;
  set_plane_bases(p, sizeof(T));                    // fin == fout == the lattice: natural plane bases
  set_float_params(p);
  const size_t pb = (size_t)p.g.plane * sizeof(T);
  for (int i = 0; i < Q; ++i) {
    if (odd) p.fout_pop[i] = static_cast<char *>(p.fout) + (size_t)OPP(i) * pb;
    else p.fin_pop[i] = static_cast<const char *>(p.fin) + (size_t)OPP(i) * pb;
  }
  using C3 = StepCfg<4, 12>;
  using C0 = StepCfg<8, 4>;
  if (odd) {
    const dim3 gg((unsigned)((p.g.ny + 127) / 128), (unsigned)p.g.nz);
    k_aa_ghost<DT><<<gg, 128, 0, s>>>(p, a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  auto go = [&](auto cfg) -> cudaError_t {
    using Cfg = decltype(cfg);
    const dim3 grid((unsigned)p.g.nseg_x, (unsigned)((p.g.ny + Cfg::WY - 1) / Cfg::WY), (unsigned)p.g.nz);
    const dim3 block(32, Cfg::WY);
    if (odd) {
      if (p.acc) k_step_aa<DT, true, true, Cfg><<<grid, block, 0, s>>>(p, a);
      else k_step_aa<DT, true, false, Cfg><<<grid, block, 0, s>>>(p, a);
    } else {
      if (p.acc) k_step_aa<DT, false, true, Cfg><<<grid, block, 0, s>>>(p, a);
      else k_step_aa<DT, false, false, Cfg><<<grid, block, 0, s>>>(p, a);
    }
    return cudaGetLastError();
  };
  if constexpr (DT == SW_F64) return go(C0{});      // float64 registers: the wide, low-occupancy shape
  else return go(C3{});
}

}  // namespace sw
