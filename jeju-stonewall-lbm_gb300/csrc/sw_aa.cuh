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
  int tma = 1;        // 16-bit storage: stage the sources by TMA when the tensor maps can be made
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
  const int c = chk(p, (z * g.ny + y) * g.pitch + x);
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
      const int src = chk(p, c + (ex == 1 ? -1 : ex == -1 ? off_xp : 0) + (ey == 1 ? off_ym : ey == -1 ? off_yp : 0) +
                                 (ez == 1 ? -lev : ez == -1 ? off_zp : 0));
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
  const bool chk_t = CHECK || x == 0;
  auto scatter = [&](auto I, R v) {
    constexpr int k = decltype(I)::value;
    constexpr int ex = CX(k), ey = CY(k), ez = CZ(k);
    T *pl = p.template out<T>(k);
    const int oy = ey == 1 ? off_yp : ey == -1 ? off_ym : 0;   // row of y + c_y
    if (CHECK && (bounced >> OPP(k)) & 1u)                      // (d)
      S::template st<k>(p.template out<T>(OPP(k)) + c, v);
    const int tx = x + ex, tz = z + ez;
    if (tx >= 0 && tx < g.nx && tz >= 0 && tz < g.nz) {          // (a)
      const int t = chk(p, c + ex + oy + ez * lev);
      if (!chk_t || p.flag[t] == 0) S::template st<k>(pl + t, v);
    }
    if constexpr (ex == -1) {
      if (outlet && tz >= 0 && tz < g.nz) {                       // (b)
        const int t = chk(p, c + oy + ez * lev);
        if (!chk_t || p.flag[t] == 0) S::template st<k>(pl + t, v);
      }
    }
    if constexpr (ez == 1) {
      if (top) {                                                  // (c)
        T *pm = p.template out<T>(MIRZ(k));
        if (tx >= 0 && tx < g.nx) {
          const int t = chk(p, c + ex + oy);
          if (!chk_t || p.flag[t] == 0) S::template st<MIRZ(k)>(pm + t, v);
        }
        if (ex == -1 && outlet) {
          const int t = chk(p, c + oy);
          if (!chk_t || p.flag[t] == 0) S::template st<MIRZ(k)>(pm + t, v);
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
  const int c = chk(p, (z * g.ny + y) * g.pitch + x);
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
          const int src = chk(p, c + (ex == 1 ? -1 : ex == -1 ? off_xp : 0) +
                                     (ey == 1 ? off_ym : ey == -1 ? off_yp : 0) + (ez == 1 ? -lev : ez == -1 ? off_zp : 0));
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

// ---------------------------------------------------------------- two cells per thread (16-bit storage)
// The same plan with one 32-bit word carrying both cells of a pair, as the
// two-lattice pair kernel does; a warp covers two 32-cell segments of a row.
// Loads are coherent (plain) loads: the lattice is written in place.
template <int DT>
__device__ __forceinline__ uint32_t aa_word(const typename Store<DT>::T *q) {
  return *reinterpret_cast<const uint32_t *>(q);
}

// Even step, fast path: both cells read their 19 incoming values from their own
// slots (plane opp(i), fin_pop) and write S_k to plane k (fout_pop), packed.
template <int DT, bool ACC>
__device__ __forceinline__ void aa_pair_even_fast(const StepParams &p, int x0, int y, int z) {
  using T = typename Store<DT>::T;
  using PK = Pack16<DT>;
  const Geom &g = p.g;
  if (x0 >= g.nx) return;
  const bool has_b = x0 + 1 < g.nx;
  const int c = chk(p, (z * g.ny + y) * g.pitch + x0);
  f2 v[Q];
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    v[i].v = PK::both(aa_word<DT>(p.template in<T>(i) + c));
  });
  double2 acc_old[4];
  if (ACC) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      acc_old[k] = has_b ? *reinterpret_cast<const double2 *>(p.accp(k) + c) : make_double2(p.accp(k)[c], 0.0);
  }
  pair_collide_store<DT, ACC>(p, v, x0, c, z, x0 == 0, has_b, [&](int k) { return acc_old[k]; });
}

// The collision and scatter of an interior odd-step cell pair (see
// aa_pair_odd_interior), with the old float64 sums of the pair in acc_old.
// inlet (lane 0 of the first segment pair, cell x0 = 0): that cell does not
// pull (v holds its rest state) and scatters its inlet equilibrium
// (lbm3d.py:67-71) instead of its collision, to the targets that exist and
// are fluid (those in column 0 need not be: only cells of column 1 pull
// from column 0).
template <int DT, bool ACC>
__device__ __forceinline__ void aa_pair_collide_scatter(const StepParams &p, const f2 (&v)[Q], int x0, int c, int z,
                                                        int off_ym, int off_yp, int lev, int lane, bool inlet,
                                                        const double2 (&acc_old)[4]) {
  using S = Store<DT>;
  using T = typename S::T;
  using PK = Pack16<DT>;
  const Phys<float> ph = phys<float>(p);
  const float u0 = inlet ? __ldg(p.uin + z) : 0.0f;
  f2 rho, ux, uy, uz;
  collide2(v, x0, true, ph.nu0, ph.c18, p.x_sponge, ph.sponge_scale, ph.nu_sponge, rho, ux, uy, uz, p.status,
           [&](auto I, f2 o) {
             constexpr int k = decltype(I)::value;
             constexpr int ex = CX(k), ey = CY(k), ez = CZ(k);
             T *plane = p.template out<T>(k);
             const int t = c + (ey == 1 ? off_yp : ey == -1 ? off_ym : 0) + ez * lev;   // target row, column x0
             if (inlet) {                                              // the inlet cell's equilibrium
               float cu = 0.0f;
               if constexpr (ex != 0) cu = (ex > 0 ? u0 : -u0);
               cu = 3.0f * cu;
               const float w = W<float>(k) * 1.0f * (1.0f + cu + 0.5f * cu * cu - 1.5f * (u0 * u0));
               o.v.x = w - W<float>(k);
             }
             if constexpr (ex == 0) {
               const int tw = chk(p, t);
               if (!inlet || p.flag[tw] == 0) *reinterpret_cast<uint32_t *>(plane + tw) = PK::pack(o.v.x, o.v.y);
               else plane[tw + 1] = S::from_shifted(o.v.y);            // column 0's target is not fluid
             } else {
               // targets x0 + ex (first cell) and x0 + 1 + ex (second cell); lane L writes the
               // word holding its second target and lane L + 1's first
               const float nxt = __shfl_down_sync(0xffffffffu, o.v.x, 1);
               const int w = chk(p, t + (ex == 1 ? 2 : 0));
               if (lane < 31) *reinterpret_cast<uint32_t *>(plane + w) = PK::pack(o.v.y, nxt);
               else plane[w] = S::from_shifted(o.v.y);                 // the other half is the next warp's
               if (lane == 0 && !(inlet && ex == -1))                  // the previous warp's (none left of the inlet)
                 plane[chk(p, t + (ex == 1 ? 1 : -1))] = S::from_shifted(o.v.x);
             }
           });
  if (ACC) {
    const double2 v0 = acc_old[0], v1 = acc_old[1], v2 = acc_old[2], v3 = acc_old[3];
    const double ra = inlet ? 1.0 : (double)rho.v.x, xa = inlet ? (double)u0 : (double)ux.v.x;
    const double ya = inlet ? 0.0 : (double)uy.v.x, za = inlet ? 0.0 : (double)uz.v.x;
    *reinterpret_cast<double2 *>(p.accp(0) + c) = make_double2(v0.x + ra, v0.y + (double)rho.v.y);
    *reinterpret_cast<double2 *>(p.accp(1) + c) = make_double2(v1.x + xa, v1.y + (double)ux.v.y);
    *reinterpret_cast<double2 *>(p.accp(2) + c) = make_double2(v2.x + ya, v2.y + (double)uy.v.y);
    *reinterpret_cast<double2 *>(p.accp(3) + c) = make_double2(v3.x + za, v3.y + (double)uz.v.y);
  }
}

// Odd step, fast path of an interior segment pair (not the inlet or the outlet
// segment pair, not the top level; every pull source and scatter target is a
// fluid cell inside the lattice): pull as the two-lattice pair kernel does, then
// scatter S_k of both cells to slot k of x + c_k (fout_pop[k] = plane opp(k)).
// For c_x = +-1 the two targets straddle two aligned words: lane L writes the
// word that holds its second target and lane L + 1's first (one shuffle); the
// halves at the warp's edges, shared with the neighbouring warps, are 16-bit stores.
template <int DT, bool ACC>
__device__ __forceinline__ void aa_pair_odd_interior(const StepParams &p, int x0, int y, int z, int lane) {
  using S = Store<DT>;
  using T = typename S::T;
  using PK = Pack16<DT>;
  const Geom &g = p.g;
  const int c = chk(p, (z * g.ny + y) * g.pitch + x0);
  const int row = g.pitch, lev = g.ny * g.pitch;
  const int off_ym = (y == 0) ? (g.ny - 1) * row : -row;        // row of y - 1 (periodic)
  const int off_yp = (y == g.ny - 1) ? -(g.ny - 1) * row : row; // row of y + 1 (periodic)
  uint32_t P[Q];
  float edge[Q];
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ex = CX(i), ey = CY(i), ez = CZ(i);
    const T *plane = p.template in<T>(i);
    const int src = c + (ey == 1 ? off_ym : ey == -1 ? off_yp : 0) - ez * lev;
    P[i] = aa_word<DT>(plane + chk(p, src));
    if constexpr (ex == 1) edge[i] = lane == 0 ? S::to_shifted(plane[chk(p, src - 1)]) : 0.0f;
    if constexpr (ex == -1) edge[i] = lane == 31 ? S::to_shifted(plane[chk(p, src + 2)]) : 0.0f;
  });
  double2 acc_old[4];
  if (ACC) {
#pragma unroll
    for (int k = 0; k < 4; ++k) acc_old[k] = *reinterpret_cast<const double2 *>(p.accp(k) + c);
  }
  f2 v[Q];
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ex = CX(i);
    const float2 own = PK::both(P[i]);
    if constexpr (ex == 0) {
      v[i].v = own;
    } else if constexpr (ex == 1) {                                 // sources x0 - 1, x0
      const uint32_t prev = __shfl_up_sync(0xffffffffu, P[i], 1);
      v[i] = F2(lane == 0 ? edge[i] : PK::hi(prev), own.x);
    } else {                                                        // sources x0 + 1, x0 + 2
      const uint32_t next = __shfl_down_sync(0xffffffffu, P[i], 1);
      v[i] = F2(own.y, lane == 31 ? edge[i] : PK::lo(next));
    }
  });
  aa_pair_collide_scatter<DT, ACC>(p, v, x0, c, z, off_ym, off_yp, lev, lane, false, acc_old);
}

// Grid: (ceil(pitch / 64), ceil(ny / WY), nz); warp = two adjacent row segments.
template <int DT, bool ODD, bool ACC, typename Cfg>
__global__ void __launch_bounds__(Cfg::THREADS, Cfg::MINB)
    k_step_aa_pair(const __grid_constant__ StepParams p, AAParams a) {
  const Geom &g = p.g;
  const int y = blockIdx.y * Cfg::WY + threadIdx.y;
  if (y >= g.ny) return;
  const int z = blockIdx.z, lane = threadIdx.x, bx = blockIdx.x;
  const int sa = 2 * bx;
  const int seg = (z * g.ny + y) * g.nseg_x + sa;
  const uint8_t ka = __ldg(p.tiles + seg);
  const uint8_t kb = sa + 1 < g.nseg_x ? __ldg(p.tiles + seg + 1) : (uint8_t)TILE_ALL_SOLID;
  if (ka & kb & TILE_ALL_SOLID) return;
  const int x0s = 2 * SEG * bx, x0 = x0s + 2 * lane;
  if (!((ka | kb) & TILE_CHECK)) {
    if (!ODD) {
      aa_pair_even_fast<DT, ACC>(p, x0, y, z);
      return;
    }
    if (x0s > 0 && x0s + 2 * SEG < g.nx && z < g.nz - 1) {           // uniform across the warp
      aa_pair_odd_interior<DT, ACC>(p, x0, y, z, lane);
      return;
    }
    float fxw = 0.0f, fzw = 0.0f;                                    // inlet, outlet, top: per cell
    int hit = 0;
    if (x0 < g.nx) aa_odd_cell<DT, false, ACC>(p, a, x0, y, z, fxw, fzw, hit);
    if (x0 + 1 < g.nx) aa_odd_cell<DT, false, ACC>(p, a, x0 + 1, y, z, fxw, fzw, hit);
    return;
  }
  float fxw = 0.0f, fzw = 0.0f;
  int hit = 0;
  if (ODD) {
    if (x0 < g.nx) aa_odd_cell<DT, true, ACC>(p, a, x0, y, z, fxw, fzw, hit);
    if (x0 + 1 < g.nx) aa_odd_cell<DT, true, ACC>(p, a, x0 + 1, y, z, fxw, fzw, hit);
  } else {
    if (x0 < g.nx) aa_even_cell<DT, true, ACC>(p, x0, y, z, fxw, fzw, hit);
    if (x0 + 1 < g.nx) aa_even_cell<DT, true, ACC>(p, x0 + 1, y, z, fxw, fzw, hit);
  }
  if (((ka | kb) & TILE_FORCE) && p.force != nullptr) warp_force_add<float>(p, z, lane, fxw, fzw, hit);
}

// ---------------------------------------------------------------- TMA-staged 16-bit AA steps
// The AA steps with their sources staged in shared memory by TMA, as k_step_tma
// does for the two-lattice step (one item of 4 rows x 64 cells per block, all
// copies issued at the start, bounded waits).  Odd step: the boxes are the
// two-lattice step's (natural planes at the source rows and levels); a warp
// not in the outlet segment pair, not at the top level and not next to stones
// or the ground pulls from them and scatters as aa_pair_odd_interior does (the
// inlet cell of the first pair scatters its equilibrium); the other warps run
// the per-cell odd step.  Even step: box i is plane opp(i) -- slot i -- at
// the item's own rows and level; every warp collides from it as
// aa_pair_even_fast does, warps next to stones or the ground with the link
// masks of their cells (the stone links' force, cells that are not fluid left
// unwritten).  In place and race-free: every value a cell uses
// from a box is written in this step only by that cell, after its wait; the
// rest of a box (columns and rows of neighbouring items) may be read while
// its owners rewrite it, and is not used.

// Even step: the 19 own-slot boxes of item (x0, y0, z) and with ACC its sums.
template <bool ACC>
__device__ __forceinline__ void tma_issue_own(const CUtensorMap *map, const CUtensorMap *map_acc, int x0, int y0, int z,
                                              uint32_t st, uint32_t bar) {
  mbar_expect_tx(bar, Q * kTmaBoxBytes + (ACC ? kTmaAccBytes : 0));
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    tma_load_4d(st + i * kTmaBoxBytes, map, x0 - 8, y0, z, OPP(i), bar);
  });
  if constexpr (ACC) tma_load_4d(st + kTmaStageBytes, map_acc, x0, y0, z, 0, bar);
}

template <int DT, bool ODD, bool ACC>
__global__ void __launch_bounds__(128, 9)
    k_step_aa_tma(const __grid_constant__ CUtensorMap map, const __grid_constant__ CUtensorMap map1,
                  const __grid_constant__ CUtensorMap map_acc, const __grid_constant__ StepParams p, AAParams a) {
  using PK = Pack16<DT>;
  extern __shared__ __align__(128) uint8_t smem_raw[];
  __shared__ __align__(8) unsigned long long bar;
  uint8_t *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  const Geom &g = p.g;
  const int w = threadIdx.y, lane = threadIdx.x;
  const bool leader = w == 0 && lane == 0;
  const int bx = blockIdx.x, z = blockIdx.z;
  const int x0s = 2 * SEG * bx, y0 = blockIdx.y * 4, y = y0 + w, x0 = x0s + 2 * lane;
  const uint32_t st = smem_u32(smem);
  if (leader) {
    mbar_init(smem_u32(&bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (ODD) tma_issue<ACC>(&map, &map1, &map_acc, g, x0s, y0, z, st, smem_u32(&bar));
    else tma_issue_own<ACC>(&map, &map_acc, x0s, y0, z, st, smem_u32(&bar));
  }
  const int sa = 2 * bx;
  uint8_t ka = TILE_ALL_SOLID, kb = TILE_ALL_SOLID;
  if (y < g.ny) {
    const int seg = (z * g.ny + y) * g.nseg_x + sa;
    ka = __ldg(p.tiles + seg);
    kb = sa + 1 < g.nseg_x ? __ldg(p.tiles + seg + 1) : (uint8_t)TILE_ALL_SOLID;
  }
  __syncthreads();
  // even step next to stones or the ground: the link masks of the lane's cells
  // (which cells are fluid, which links come from stones), fetched during the copies
  const bool even_checked = !ODD && y < g.ny && !(ka & kb & TILE_ALL_SOLID) && ((ka | kb) & TILE_CHECK);
  uint32_t sm[2] = {1u, 1u}, wm[2] = {0u, 0u};
  if (even_checked) {
    cell_links(p, x0, y, z, sm[0], wm[0]);
    cell_links(p, x0 + 1, y, z, sm[1], wm[1]);
  }
  bool ok = mbar_wait(smem_u32(&bar), 0u, p.tma_poll_limit);
  if (ok && y < g.ny && !(ka & kb & TILE_ALL_SOLID)) {
    const int row = g.pitch, lev = g.ny * g.pitch;
    const int lane_word = 4 + lane;                                   // 32-bit word of elements 8 + 2 lane, + 1
    if (even_checked) {
      // The even step reads the cell's own slots, where the odd step already put the
      // bounce-back values (rule (d)); a link from a stone adds -2 (f - w) c of its
      // value to the wall force (lbm3d.py:91-101), cell x0 before x0 + 1, as
      // aa_even_cell adds them; cells that are not fluid are not stored.
      float fxw = 0.0f, fzw = 0.0f;
      int hit = 0;
      if (x0 < g.nx) {
        const bool has_b = x0 + 1 < g.nx;
        const int c = chk(p, (z * g.ny + y) * g.pitch + x0);
        f2 v[Q];
        static_for<0, Q>([&](auto I) {
          constexpr int i = decltype(I)::value;
          v[i].v = PK::both(reinterpret_cast<const uint32_t *>(smem + i * kTmaBoxBytes + w * kTmaRowBytes)[lane_word]);
        });
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          static_for<1, Q>([&](auto I) {
            constexpr int i = decltype(I)::value;
            constexpr int ex = CX(i), ez = CZ(i);
            if ((wm[h] >> i) & 1u) {
              const float fr = h ? v[i].v.y : v[i].v.x;
              if constexpr (ex != 0) fxw = fxw - 2.0f * fr * (float)ex;
              if constexpr (ez != 0) fzw = fzw - 2.0f * fr * (float)ez;
              hit = 1;
            }
          });
        }
        const uint32_t keep = pair_solid_cells(v, sm);
        if (keep != 0u) {
          const double2 *acc_box = reinterpret_cast<const double2 *>(smem + kTmaStageBytes) + w * 32 + lane;
          pair_collide_store<DT, ACC, true>(p, v, x0, c, z, x0 == 0, has_b,
                                            [&](int k) { return acc_box[k * 4 * 32]; }, keep);
        }
      }
      if (((ka | kb) & TILE_FORCE) && p.force != nullptr) warp_force_add<float>(p, z, lane, fxw, fzw, hit);
    } else if (!((ka | kb) & TILE_CHECK) && !ODD) {                   // even step: own slots, local
      if (x0 < g.nx) {
        const bool has_b = x0 + 1 < g.nx;
        const int c = chk(p, (z * g.ny + y) * g.pitch + x0);
        f2 v[Q];
        static_for<0, Q>([&](auto I) {
          constexpr int i = decltype(I)::value;
          v[i].v = PK::both(reinterpret_cast<const uint32_t *>(smem + i * kTmaBoxBytes + w * kTmaRowBytes)[lane_word]);
        });
        const double2 *acc_box = reinterpret_cast<const double2 *>(smem + kTmaStageBytes) + w * 32 + lane;
        pair_collide_store<DT, ACC>(p, v, x0, c, z, x0 == 0, has_b, [&](int k) { return acc_box[k * 4 * 32]; });
      }
    } else if (!((ka | kb) & TILE_CHECK) && x0s + 2 * SEG < g.nx && z < g.nz - 1) {   // odd: not the outlet or top
      const bool inlet = x0 == 0;                                     // lane 0 of the first pair
      const int c = chk(p, (z * g.ny + y) * g.pitch + x0);
      const int off_ym = (y == 0) ? (g.ny - 1) * row : -row;
      const int off_yp = (y == g.ny - 1) ? -(g.ny - 1) * row : row;
      f2 v[Q];
      static_for<0, Q>([&](auto I) {
        constexpr int i = decltype(I)::value;
        constexpr int ex = CX(i), ey = CY(i);
        const uint8_t *rowp = smem + i * kTmaBoxBytes + w * kTmaRowBytes;
        if constexpr (ey == 1) {
          if (y == 0) rowp = smem + Q * kTmaBoxBytes + wrap_slot(i) * kTmaWrapBytes;
        } else if constexpr (ey == -1) {
          if (y == g.ny - 1) rowp = smem + Q * kTmaBoxBytes + wrap_slot(i) * kTmaWrapBytes;
        }
        const uint32_t *r = reinterpret_cast<const uint32_t *>(rowp);
        const uint32_t own = r[lane_word];                            // cells x0, x0 + 1
        if constexpr (ex == 0) {
          v[i].v = PK::both(own);
        } else if constexpr (ex == 1) {                               // sources x0 - 1, x0
          v[i] = F2(PK::hi(r[lane_word - 1]), PK::lo(own));
        } else {                                                      // sources x0 + 1, x0 + 2
          v[i] = F2(PK::hi(own), PK::lo(r[lane_word + 1]));
        }
        if (inlet) v[i].v.x = 0.0f;                                   // the inlet cell does not pull
      });
      double2 acc_old[4];
      if (ACC) {
        const double2 *acc_box = reinterpret_cast<const double2 *>(smem + kTmaStageBytes) + w * 32 + lane;
#pragma unroll
        for (int k = 0; k < 4; ++k) acc_old[k] = acc_box[k * 4 * 32];
      }
      aa_pair_collide_scatter<DT, ACC>(p, v, x0, c, z, off_ym, off_yp, lev, lane, inlet, acc_old);
    } else {                                                          // per cell (from the lattice)
      float fxw = 0.0f, fzw = 0.0f;
      int hit = 0;
      if ((ka | kb) & TILE_CHECK) {                                   // odd step next to stones or the ground
        if (x0 < g.nx) aa_odd_cell<DT, true, ACC>(p, a, x0, y, z, fxw, fzw, hit);
        if (x0 + 1 < g.nx) aa_odd_cell<DT, true, ACC>(p, a, x0 + 1, y, z, fxw, fzw, hit);
        if (((ka | kb) & TILE_FORCE) && p.force != nullptr) warp_force_add<float>(p, z, lane, fxw, fzw, hit);
      } else {                                                        // odd: inlet, outlet, top
        if (x0 < g.nx) aa_odd_cell<DT, false, ACC>(p, a, x0, y, z, fxw, fzw, hit);
        if (x0 + 1 < g.nx) aa_odd_cell<DT, false, ACC>(p, a, x0 + 1, y, z, fxw, fzw, hit);
      }
    }
  }
  ok = __syncthreads_and(ok);
  if (!ok && leader) {                                                // a wait gave up: let the copies
    atomicAdd(&g_tma_timeouts, 1u);                                   // in flight land (normal bound)
    note_status(p, SW_STATUS_TIMEOUT);
    (void)mbar_wait(smem_u32(&bar), 0u);
  }
}

// The TMA-staged AA step on the lattice p.fin (== p.fout); cudaErrorNotSupported
// when the tensor maps cannot be made (the caller then runs k_step_aa_pair).
template <int DT, bool ODD, bool ACC>
cudaError_t launch_aa_tma(const StepParams &p, const AAParams &a, cudaStream_t s) {
  CUtensorMap map, map1, map_acc;
  if (!encode_lattice_map(&map, p.fin, p.g, 4) || !encode_lattice_map(&map1, p.fin, p.g, 1))
    return cudaErrorNotSupported;
  if (ACC) {
    if (!encode_acc_map(&map_acc, p.acc, p.g)) return cudaErrorNotSupported;
  } else {
    map_acc = map;                                                   // not read
  }
  constexpr int smem = tma_stage_bytes<ACC>() + 128;
  static_assert(smem <= 48 * 1024, "one stage fits the default shared memory of a block");
  const dim3 grid((unsigned)((p.g.nseg_x + 1) / 2), (unsigned)((p.g.ny + 3) / 4), (unsigned)p.g.nz);
  k_step_aa_tma<DT, ODD, ACC><<<grid, dim3(32, 4), smem, s>>>(map, map1, map_acc, p, a);
  return cudaGetLastError();
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
  if constexpr (is16(DT)) {                          // two cells per thread, sources staged by TMA
    if (a.tma) {
      cudaError_t e = odd ? (p.acc ? launch_aa_tma<DT, true, true>(p, a, s) : launch_aa_tma<DT, true, false>(p, a, s))
                        : (p.acc ? launch_aa_tma<DT, false, true>(p, a, s) : launch_aa_tma<DT, false, false>(p, a, s));
      if (e != cudaErrorNotSupported) return e;
    }
  }
  if constexpr (is16(DT)) {                          // no tensor maps: the same step from the lattice
    using Cfg = StepCfg<4, 8>;
    const dim3 grid((unsigned)((p.g.nseg_x + 1) / 2), (unsigned)((p.g.ny + Cfg::WY - 1) / Cfg::WY), (unsigned)p.g.nz);
    const dim3 block(32, Cfg::WY);
    if (odd) {
      if (p.acc) k_step_aa_pair<DT, true, true, Cfg><<<grid, block, 0, s>>>(p, a);
      else k_step_aa_pair<DT, true, false, Cfg><<<grid, block, 0, s>>>(p, a);
    } else {
      if (p.acc) k_step_aa_pair<DT, false, true, Cfg><<<grid, block, 0, s>>>(p, a);
      else k_step_aa_pair<DT, false, false, Cfg><<<grid, block, 0, s>>>(p, a);
    }
    return cudaGetLastError();
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
