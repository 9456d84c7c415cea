// sw_step.cuh -- the fused D3Q19 timestep (pull streaming + boundaries + bounce-back +
// momentum exchange + regularized BGK with Smagorinsky and the outlet sponge).
//
// Computes k_step of stonewall3d/lbm3d.py:57-155.  Same mathematics, arranged
// for the GPU:
//  * one warp = one 32-cell row segment along x; a byte per segment (tiles[])
//    says whether any pull source of its fluid cells can be non-fluid.
//    Segments that cannot (the bulk of the domain) skip the 19 neighbour flag
//    loads of lbm3d.py:88 and the force bookkeeping;
//  * the 18 moving populations are taken in opposite pairs (i, opp(i)):
//    s = f_i + f_opp, d = f_i - f_opp give rho, momentum m and the second
//    moment Pi with one add per term, and the regularized post-collision state
//      f_i = w_i [rho + 3 c_i.m + 4.5 Q_i:B],  B = m m / rho + (1 - 1/tau) Pi_neq,
//    Q_i = c_i c_i - I/3, is the reference's feq_i + (1 - 1/tau) w_i 4.5 Q_i:Pi_neq
//    (lbm3d.py:147-155) rewritten: both members of a pair share w (rho + 4.5 Q:B)
//    and differ in the sign of 3 w c.m.  Results agree with the reference's
//    expression order to float32 rounding (the parity tests bound it at 1e-5);
//  * one reciprocal of rho and one of tau replace the divisions;
//  * the per-cell wall force (float32, as lbm3d.py:91-95) is summed per warp in
//    float64 (xor butterfly, fixed order) and added to force[t][z] as 2^-40
//    fixed point with one 64-bit integer atomic per warp, so the totals do not
//    depend on warp scheduling (the reference adds float32 atomics per cell,
//    lbm3d.py:99-101);
//  * on accumulation steps (ACC) the cell's (rho, u) is added to the float64
//    running sums in the same pass: this is k_macro + k_accum (lbm3d.py:367-369)
//    of the new state, whose rho and m equal the pulled ones (the collision
//    conserves both).  Non-fluid cells are not touched; their sums are
//    n_acc * (1, 0, 0, 0) by definition and are filled in on download.
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
  double sponge_scale;  // 1 / (nx - x_sponge)
  // float copies for the float collision (set_float_params): rounded once on
  // the host instead of converted from double in every thread
  float nu0f, c18f, sponge_scalef, nu_spongef;
  int x_sponge;
  long long *force;  // force row of this step: [nz][2], or nullptr
  double *acc;       // float64 running sums [4][plane] (accumulation steps only)
  unsigned int *status;  // device status word (SW_STATUS_*), or nullptr: no checks
  int cfg;           // launch configuration (SW_STEP_CONFIGS)
  int tma_poll_limit;  // polls before a TMA-staged block gives up on a stage (set at launch)
  // per-population plane bases (fin + i * plane etc.), uniform across the grid,
  // so that every load and store needs only a 32-bit offset within a plane
  const void *fin_pop[Q];
  void *fout_pop[Q];
  double *acc_pop[4];

  // access used by the cell code (shared with the batched kernel's context)
  template <typename T> __device__ __forceinline__ const T *in(int pop) const {
    return static_cast<const T *>(fin_pop[pop]);
  }
  template <typename T> __device__ __forceinline__ T *out(int pop) const { return static_cast<T *>(fout_pop[pop]); }
  __device__ __forceinline__ double *accp(int k) const { return acc_pop[k]; }
};

// Fills the per-population bases from fin / fout / acc (host side).
inline void set_plane_bases(StepParams &p, size_t elem_bytes) {
  const size_t pb = (size_t)p.g.plane * elem_bytes;
  for (int i = 0; i < Q; ++i) {
    p.fin_pop[i] = static_cast<const char *>(p.fin) + i * pb;
    p.fout_pop[i] = static_cast<char *>(p.fout) + i * pb;
  }
  for (int k = 0; k < 4; ++k) p.acc_pop[k] = p.acc ? p.acc + (size_t)k * p.g.plane : nullptr;
}

// 18 sqrt(2) Cs^2 of the Smagorinsky time scale (lbm3d.py:144-146), evaluated
// in the order the float kernels evaluated it in-thread, so the rounded value
// is the same bits on the host and on the device.
__host__ __device__ inline float smag_c18f(float cs) {
  float c = 18.0f * sqrtf(2.0f);
  c = c * cs;
  return c * cs;
}

// The float copies of the physics parameters (host side, once per launch).
inline void set_float_params(StepParams &p) {
  p.nu0f = (float)p.nu0;
  p.c18f = smag_c18f((float)p.cs);
  p.sponge_scalef = (float)p.sponge_scale;
  p.nu_spongef = (float)p.nu_sponge;
}

// Physics parameters in the collision's arithmetic type R.
template <typename R> struct Phys {
  R nu0, c18, sponge_scale, nu_sponge;
};
template <typename R, typename Ctx> __device__ __forceinline__ Phys<R> phys(const Ctx &p) {
  if constexpr (sizeof(R) == 4) {
    return {p.nu0f, p.c18f, p.sponge_scalef, p.nu_spongef};
  } else {
    const R cs = p.cs;
    return {p.nu0, R(18.0) * sqrt(R(2.0)) * cs * cs, p.sponge_scale, p.nu_sponge};
  }
}

// ORs status bits into the lattice's status word (a rare branch: divergence or a time-out).
template <typename Ctx> __device__ __forceinline__ void note_status(const Ctx &p, unsigned int bits) {
  if (p.status != nullptr) atomicOr(p.status, bits);
}
// Element offset within a population plane (also the flag, tiles and sums
// planes).  The bounds-checked build (-DSW_CHECK, libstonewall_check.so) tests
// every computed offset against the plane and, outside it, reports
// SW_STATUS_BOUNDS and uses offset 0 instead; the normal build only passes it on.
template <typename Ctx> __device__ __forceinline__ int chk(const Ctx &p, int off) {
#ifdef SW_CHECK
  if ((unsigned long long)(long long)off >= (unsigned long long)p.g.plane) {
    note_status(p, SW_STATUS_BOUNDS);
    return 0;
  }
#endif
  return off;
}

// |v| <= largest finite value: false for infinities and NaN.
__device__ __forceinline__ bool finite_val(float v) { return fabsf(v) <= 3.402823466e38f; }
__device__ __forceinline__ bool finite_val(double v) { return fabs(v) <= 1.7976931348623157e308; }

// float: the hardware approximations (relative error about 2^-23, far below the
// 1e-5 parity bar); double: IEEE division and square root.
__device__ __forceinline__ float rcp(float v) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}
__device__ __forceinline__ double rcp(double v) { return 1.0 / v; }
__device__ __forceinline__ float fsqrt(float v) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}
__device__ __forceinline__ double fsqrt(double v) { return sqrt(v); }

// Regularized-BGK collision of one cell from its 19 pulled populations.
// Calls put(Int<i>, value) for every population and returns rho and u.
// SHIFT: f[] holds g_i = f_i - w_i and put() receives g_i.  Since sum_i w_i = 1,
// sum_i w_i c_i = 0 and sum_i w_i c_i c_i = I/3, the moments of g are rho - 1,
// m and Pi - I/3, so r0 = sum_i f[i] below is rho - 1 (shifted) or rho, and
// Pi_neq = P - r0/3 I - m m / rho holds in both cases.
// status: the lattice's status word (or nullptr).  A cell whose pulled density
// is not finite reports SW_STATUS_NONFINITE there, in a rare branch taken
// where rho is formed, so that no value stays live for the check.
template <typename R, bool SHIFT, typename Put>
__device__ __forceinline__ void collide(const R (&f)[Q], int x, R nu0, R cs2_18r2, int x_sponge, R sponge_scale,
                                        R nu_sponge, R &rho_out, R &ux_out, R &uy_out, R &uz_out, unsigned int *status,
                                        Put &&put) {
  // pair sums / differences, pair k = directions (2k+1, 2k+2), c(2k+2) = -c(2k+1)
  R s[9], d[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    s[k] = f[2 * k + 1] + f[2 * k + 2];
    d[k] = f[2 * k + 1] - f[2 * k + 2];
  }
  // pairs: 0 (1,0,0) 1 (0,1,0) 2 (0,0,1) 3 (1,1,0) 4 (1,-1,0) 5 (1,0,1) 6 (1,0,-1) 7 (0,1,1) 8 (0,1,-1)
  const R r0 = f[0] + (((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7])) + s[8]);
  const R rho = SHIFT ? r0 + R(1.0) : r0;
  if (!finite_val(r0) && status != nullptr) atomicOr(status, (unsigned int)SW_STATUS_NONFINITE);
  const R mx = (d[0] + d[3]) + (d[4] + d[5]) + d[6];
  const R my = (d[1] + d[3]) - d[4] + (d[7] + d[8]);
  const R mz = (d[2] + d[5]) - d[6] + (d[7] - d[8]);
  const R pxx = (s[0] + s[3]) + (s[4] + s[5]) + s[6];
  const R pyy = (s[1] + s[3]) + (s[4] + s[7]) + s[8];
  const R pzz = (s[2] + s[5]) + (s[6] + s[7]) + s[8];
  const R pxy = s[3] - s[4];
  const R pxz = s[5] - s[6];
  const R pyz = s[7] - s[8];
  const R inv = rcp(rho);
  const R ux = mx * inv, uy = my * inv, uz = mz * inv;
  const R third = r0 * R(1.0 / 3.0);
  // non-equilibrium stress (lbm3d.py:133-138)
  const R nxx = pxx - third - mx * ux;
  const R nyy = pyy - third - my * uy;
  const R nzz = pzz - third - mz * uz;
  const R nxy = pxy - mx * uy;
  const R nxz = pxz - mx * uz;
  const R nyz = pyz - my * uz;
  // sponge viscosity (lbm3d.py:140-143) and Smagorinsky time scale (lbm3d.py:144-147)
  R nu = nu0;
  if (x > x_sponge) {
    const R sp = R(x - x_sponge) * sponge_scale;
    nu = nu0 + nu_sponge * sp * sp;
  }
  const R tau0 = R(3.0) * nu + R(0.5);
  const R qn = fsqrt(nxx * nxx + nyy * nyy + nzz * nzz + R(2.0) * (nxy * nxy + nxz * nxz + nyz * nyz));
  const R tau = R(0.5) * (tau0 + fsqrt(tau0 * tau0 + cs2_18r2 * qn * inv));
  const R keep = R(1.0) - rcp(tau);
  // B = rho u u + keep Pi_neq and the pair terms of Q_i : B
  const R bxx = mx * ux + keep * nxx, byy = my * uy + keep * nyy, bzz = mz * uz + keep * nzz;
  const R bxy2 = R(2.0) * (mx * uy + keep * nxy);
  const R bxz2 = R(2.0) * (mx * uz + keep * nxz);
  const R byz2 = R(2.0) * (my * uz + keep * nyz);
  const R tr = (bxx + byy + bzz) * R(1.0 / 3.0);
  const R w0 = W<R>(0), w1 = W<R>(1), w2 = W<R>(7);
  put(Int<0>{}, w0 * (r0 - R(4.5) * tr));
  // f_(+-c) = w (r0 + 4.5 Q:B) +- 3 w c.m, as two fused multiply-adds per population
  const R wr1 = w1 * r0, wr2 = w2 * r0;
  auto pair = [&](auto I, R w, R wr, R qb, R cm) {
    constexpr int k = decltype(I)::value;
    const R base = fma(R(4.5) * w, qb, wr);
    put(Int<2 * k + 1>{}, fma(R(3.0) * w, cm, base));
    put(Int<2 * k + 2>{}, fma(R(-3.0) * w, cm, base));
  };
  pair(Int<0>{}, w1, wr1, bxx - tr, mx);
  pair(Int<1>{}, w1, wr1, byy - tr, my);
  pair(Int<2>{}, w1, wr1, bzz - tr, mz);
  const R exy = bxx + byy - tr, exz = bxx + bzz - tr, eyz = byy + bzz - tr;
  pair(Int<3>{}, w2, wr2, exy + bxy2, mx + my);
  pair(Int<4>{}, w2, wr2, exy - bxy2, mx - my);
  pair(Int<5>{}, w2, wr2, exz + bxz2, mx + mz);
  pair(Int<6>{}, w2, wr2, exz - bxz2, mx - mz);
  pair(Int<7>{}, w2, wr2, eyz + byz2, my + mz);
  pair(Int<8>{}, w2, wr2, eyz - byz2, my - mz);
  rho_out = rho;
  ux_out = ux;
  uy_out = uy;
  uz_out = uz;
}

// Launch configurations compiled in; the autotuner (stonewall/autotune.py)
// times them per storage type and grid and keeps the fastest.
//   WY   rows of a block (one 32-cell segment per warp): block = 32 x WY threads
//   MINB resident blocks per SM asked of the register allocator
template <int WY_, int MINB_> struct StepCfg {
  static constexpr int WY = WY_;
  static constexpr int MINB = MINB_;
  static constexpr int THREADS = 32 * WY_;
};
#define SW_STEP_CONFIGS(X) X(0, 8, 4) X(1, 8, 5) X(2, 4, 8) X(3, 4, 12)
// two cells per thread (16-bit storage only), see k_step_pair
#define SW_PAIR_CONFIGS(X) X(4, 4, 8) X(5, 4, 10) X(6, 8, 4) X(7, 8, 5)
// two cells per thread with TMA-staged sources (16-bit storage only), see sw_tma.cuh:
// (id, row-groups per block, stages, resident blocks asked of the register allocator).
// Shared memory holds a 2-stage block to 7 resident blocks (4 on accumulating
// steps), so 12 and 13 give the registers that residency leaves (72 and 128 per
// thread).  One item per block (one stage, no block barrier) leaves shared
// memory for more blocks: 10, 11 and 14-17 trade registers for residency
// (measured at 800x160x160: 16 fastest plain, 15 fastest accumulating).
#define SW_TMA_CONFIGS(X) X(8, 4, 2, 8) X(9, 2, 2, 8) X(10, 1, 1, 9) X(11, 1, 1, 7) X(12, 2, 2, 7) X(13, 4, 2, 4) \
  X(14, 1, 1, 12) X(15, 1, 1, 8) X(16, 1, 1, 10) X(17, 1, 1, 6)
constexpr int kStepConfigs = 18;

// Where the checked path of step_cell takes its inputs from, read from the
// lattice and the flags:
//   operator()  the pulled value of the link of population I, whose source is
//               element offset src of plane P (P = I, or its z mirror at the top);
//   self_solid  whether cell c itself is not fluid;
//   src_flag    the flag of link I's source (0 fluid, SW_WALL, SW_GROUND); a
//               source below z = 0 (only for a fluid cell in the bottom plane,
//               which the reference never has) is treated as ground;
//   bounce      the half-way bounce-back value of link I: the cell's own
//               population OPP(I) (lbm3d.py:89-95).
template <int DT> struct GlobalPull {
  using R = typename Store<DT>::R;
  using T = typename Store<DT>::T;
  template <int I, int P, typename Ctx>
  __device__ __forceinline__ R operator()(Int<I>, Int<P>, const Ctx &p, int src) const {
    return Store<DT>::template ld<P>(p.template in<T>(P) + src);
  }
  template <typename Ctx> __device__ __forceinline__ bool self_solid(const Ctx &p, int c) const {
    return p.flag[c] != 0;
  }
  template <int I, typename Ctx> __device__ __forceinline__ uint8_t src_flag(Int<I>, const Ctx &p, int src, int z) const {
    return (CZ(I) == 1 && z == 0) ? (uint8_t)SW_GROUND : __ldg(p.flag + src);
  }
  template <int I, typename Ctx> __device__ __forceinline__ R bounce(Int<I>, const Ctx &p, int c) const {
    return Store<DT>::template ld<OPP(I)>(p.template in<T>(OPP(I)) + c);
  }
};

// One cell of the pull-scheme step.  CHECK selects the path with neighbour flag
// tests (segments next to stones, the ground or a fluid cell at z = 0).
// Offsets within a population plane are 32-bit (grids below 2^31 cells).
template <int DT, bool CHECK, bool ACC, typename Ctx>
__device__ __forceinline__ void step_cell(const Ctx &p, int x, int y, int z, typename Store<DT>::R &fxw,
                                          typename Store<DT>::R &fzw, int &hit) {
  step_cell<DT, CHECK, ACC>(p, x, y, z, fxw, fzw, hit, GlobalPull<DT>{});
}

// The same with the checked path's inputs from `pull_val` (GlobalPull: the
// lattice and the flags).
template <int DT, bool CHECK, bool ACC, typename Ctx, typename Pull>
__device__ __forceinline__ void step_cell(const Ctx &p, int x, int y, int z, typename Store<DT>::R &fxw,
                                          typename Store<DT>::R &fzw, int &hit, const Pull &pull_val) {
  using S = Store<DT>;
  using T = typename S::T;
  using R = typename S::R;
  const Geom &g = p.g;
  const int c = chk(p, (z * g.ny + y) * g.pitch + x);
  auto out = [&](int pop) { return p.template out<T>(pop); };
  if (CHECK && pull_val.self_solid(p, c)) return;              // lbm3d.py:65-66
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
      S::template st<i>(out(i) + c, S::kShift ? v - W<R>(i) : v);
    });
    if (ACC) {
      atomicAdd(p.accp(0) + c, 1.0);
      atomicAdd(p.accp(1) + c, (double)u0);
    }
    return;
  }
  // pull sources (lbm3d.py:77-86) as element offsets from the cell:
  // periodic y, outlet copies column x, top mirrors z
  const int row = g.pitch, lev = g.ny * g.pitch;
  const int off_xm = c - 1;                                         // source of c_x = +1
  const int off_xp = (x + 1 >= g.nx) ? c : c + 1;                   // source of c_x = -1
  const int off_ym = (y == 0) ? (g.ny - 1) * row : -row;            // source row of c_y = +1
  const int off_yp = (y == g.ny - 1) ? -(g.ny - 1) * row : row;     // source row of c_y = -1
  const bool top = (z == g.nz - 1);
  const int off_zm = -lev;                                          // source level of c_z = +1
  const int off_zp = top ? 0 : lev;                                 // source level of c_z = -1
  // accumulation steps: the four running sums are read together with the
  // populations, so their latency overlaps (each cell is owned by one thread)
  double acc_old[4] = {0.0, 0.0, 0.0, 0.0};
  if (ACC) {
#pragma unroll
    for (int k = 0; k < 4; ++k) acc_old[k] = __ldcs(p.accp(k) + c);
  }
  R fl[Q];
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ex = CX(i), ey = CY(i), ez = CZ(i);
    const int src = chk(p, (ex == 1 ? off_xm : ex == -1 ? off_xp : c) + (ey == 1 ? off_ym : ey == -1 ? off_yp : 0) +
                               (ez == 1 ? off_zm : ez == -1 ? off_zp : 0));
    bool pull = true;
    if constexpr (CHECK) {
      const uint8_t fs = pull_val.src_flag(Int<i>{}, p, src, z);
      if (fs != 0) {                                            // lbm3d.py:89-95
        pull = false;
        const R val = pull_val.bounce(Int<i>{}, p, c);
        if (fs == SW_WALL) {
          const R fr = S::kShift ? val : val - W<R>(i);   // f - w, the rho = 1 background removed
          if constexpr (ex != 0) fxw = fxw - R(2.0) * fr * R(ex);
          if constexpr (ez != 0) fzw = fzw - R(2.0) * fr * R(ez);
          hit = 1;
        }
        fl[i] = val;
      }
    }
    if (pull) {                                                 // lbm3d.py:97
      if constexpr (ez == -1) {
        if (top) fl[i] = pull_val(Int<i>{}, Int<MIRZ(i)>{}, p, src);
        else fl[i] = pull_val(Int<i>{}, Int<i>{}, p, src);
      } else {
        fl[i] = pull_val(Int<i>{}, Int<i>{}, p, src);
      }
    }
  });
  R rho, ux, uy, uz;
  const Phys<R> ph = phys<R>(p);
  collide<R, S::kShift>(fl, x, ph.nu0, ph.c18, p.x_sponge, ph.sponge_scale, ph.nu_sponge, rho, ux, uy, uz, p.status,
                        [&](auto I, R v) {
                          constexpr int i = decltype(I)::value;
                          S::template st<i>(out(i) + c, v);
                        });
  if (ACC) {
    __stcs(p.accp(0) + c, acc_old[0] + (double)rho);
    __stcs(p.accp(1) + c, acc_old[1] + (double)ux);
    __stcs(p.accp(2) + c, acc_old[2] + (double)uy);
    __stcs(p.accp(3) + c, acc_old[3] + (double)uz);
  }
}

// Adds the warp's wall force (lbm3d.py:99-101): float64 xor-butterfly sum, then
// one 2^-40 fixed-point integer atomic per component.
template <typename R, typename Ctx>
__device__ __forceinline__ void warp_force_add(const Ctx &p, int z, int lane, R fxw, R fzw, int hit) {
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

// One warp, one 32-cell row segment (sx, y, z): fast path, checked path or nothing.
template <int DT, bool ACC, typename Ctx>
__device__ __forceinline__ void step_segment(const Ctx &p, int sx, int y, int z, int lane) {
  using R = typename Store<DT>::R;
  const Geom &g = p.g;
  const int seg = (z * g.ny + y) * g.nseg_x + sx;
  const uint8_t kind = __ldg(p.tiles + seg);
  if (kind & TILE_ALL_SOLID) return;
  const int x = sx * SEG + lane;
  R fxw = R(0.0), fzw = R(0.0);
  int hit = 0;
  if (!(kind & TILE_CHECK)) {
    if (x < g.nx) step_cell<DT, false, ACC>(p, x, y, z, fxw, fzw, hit);
    return;
  }
  if (x < g.nx) step_cell<DT, true, ACC>(p, x, y, z, fxw, fzw, hit);
  if ((kind & TILE_FORCE) && p.force != nullptr) warp_force_add<R>(p, z, lane, fxw, fzw, hit);
}

// Grid: (pitch / 32, ceil(ny / WY), nz); warp (threadIdx.y) = one row segment.
template <int DT, bool ACC, typename Cfg>
__global__ void __launch_bounds__(Cfg::THREADS, Cfg::MINB) k_step_pull(const __grid_constant__ StepParams p) {
  const int y = blockIdx.y * Cfg::WY + threadIdx.y;
  if (y >= p.g.ny) return;
  step_segment<DT, ACC>(p, blockIdx.x, y, (int)blockIdx.z, threadIdx.x);
}

// ---------------------------------------------------------------- packed two-cell collision
// Two cells per thread (the pair kernel) run the same collision; on sm_100+
// the FP32 arithmetic issues as two-wide packed instructions (FFMA2 / FADD2 /
// FMUL2 through __ffma2_rn / __fadd2_rn / __fmul2_rn), halving the issue slots
// of the collision.  Reciprocals and square roots stay per cell.  Same
// formulas as collide<float, true> (shifted storage).
struct f2 {
  float2 v;
};
__device__ __forceinline__ f2 F2(float a) { return {make_float2(a, a)}; }
__device__ __forceinline__ f2 F2(float a, float b) { return {make_float2(a, b)}; }
__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return {__fadd2_rn(a.v, b.v)}; }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return {__fmul2_rn(a.v, b.v)}; }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return {__ffma2_rn(b.v, make_float2(-1.0f, -1.0f), a.v)}; }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return {__ffma2_rn(a.v, b.v, c.v)}; }

// status: as collide; both densities are checked (the second only when has_b: past the row end it is padding).
template <typename Put>
__device__ __forceinline__ void collide2(const f2 (&f)[Q], int x0, bool has_b, float nu0, float cs2_18r2,
                                         int x_sponge, float sponge_scale, float nu_sponge, f2 &rho_out, f2 &ux_out,
                                         f2 &uy_out, f2 &uz_out, unsigned int *status, Put &&put) {
  f2 s[9], d[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    s[k] = f[2 * k + 1] + f[2 * k + 2];
    d[k] = f[2 * k + 1] - f[2 * k + 2];
  }
  const f2 r0 = f[0] + (((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7])) + s[8]);
  const f2 rho = r0 + F2(1.0f);
  if (!finite_val(fabsf(r0.v.x) + (has_b ? fabsf(r0.v.y) : 0.0f)) && status != nullptr)
    atomicOr(status, (unsigned int)SW_STATUS_NONFINITE);
  const f2 mx = (d[0] + d[3]) + (d[4] + d[5]) + d[6];
  const f2 my = (d[1] + d[3]) - d[4] + (d[7] + d[8]);
  const f2 mz = (d[2] + d[5]) - d[6] + (d[7] - d[8]);
  const f2 pxx = (s[0] + s[3]) + (s[4] + s[5]) + s[6];
  const f2 pyy = (s[1] + s[3]) + (s[4] + s[7]) + s[8];
  const f2 pzz = (s[2] + s[5]) + (s[6] + s[7]) + s[8];
  const f2 pxy = s[3] - s[4];
  const f2 pxz = s[5] - s[6];
  const f2 pyz = s[7] - s[8];
  const f2 inv = F2(rcp(rho.v.x), rcp(rho.v.y));
  const f2 ux = mx * inv, uy = my * inv, uz = mz * inv;
  const f2 nux = ux * F2(-1.0f), nuy = uy * F2(-1.0f), nuz = uz * F2(-1.0f);
  const f2 third = r0 * F2(1.0f / 3.0f);
  const f2 nxx = fma2(mx, nux, pxx - third);
  const f2 nyy = fma2(my, nuy, pyy - third);
  const f2 nzz = fma2(mz, nuz, pzz - third);
  const f2 nxy = fma2(mx, nuy, pxy);
  const f2 nxz = fma2(mx, nuz, pxz);
  const f2 nyz = fma2(my, nuz, pyz);
  float nua = nu0, nub = nu0;
  if (x0 > x_sponge) {
    const float sa = (float)(x0 - x_sponge) * sponge_scale;
    nua = nu0 + nu_sponge * sa * sa;
  }
  if (x0 + 1 > x_sponge) {
    const float sb = (float)(x0 + 1 - x_sponge) * sponge_scale;
    nub = nu0 + nu_sponge * sb * sb;
  }
  const f2 tau0 = fma2(F2(3.0f), F2(nua, nub), F2(0.5f));
  const f2 q1 = fma2(nzz, nzz, fma2(nyy, nyy, nxx * nxx));
  const f2 q2 = fma2(nyz, nyz, fma2(nxz, nxz, nxy * nxy));
  const f2 q = fma2(q2, F2(2.0f), q1);
  const f2 qn = F2(fsqrt(q.v.x), fsqrt(q.v.y));
  const f2 arg = fma2(tau0, tau0, (F2(cs2_18r2) * qn) * inv);
  const f2 tau = F2(0.5f) * (tau0 + F2(fsqrt(arg.v.x), fsqrt(arg.v.y)));
  const f2 keep = F2(1.0f) - F2(rcp(tau.v.x), rcp(tau.v.y));
  const f2 bxx = fma2(keep, nxx, mx * ux), byy = fma2(keep, nyy, my * uy), bzz = fma2(keep, nzz, mz * uz);
  const f2 bxy2 = F2(2.0f) * fma2(keep, nxy, mx * uy);
  const f2 bxz2 = F2(2.0f) * fma2(keep, nxz, mx * uz);
  const f2 byz2 = F2(2.0f) * fma2(keep, nyz, my * uz);
  const f2 tr = (bxx + byy + bzz) * F2(1.0f / 3.0f);
  const float w0 = W<float>(0), w1 = W<float>(1), w2 = W<float>(7);
  put(Int<0>{}, F2(w0) * fma2(tr, F2(-4.5f), r0));
  const f2 wr1 = F2(w1) * r0, wr2 = F2(w2) * r0;
  auto pair = [&](auto I, float w, f2 wr, f2 qb, f2 cm) {
    constexpr int k = decltype(I)::value;
    const f2 base = fma2(F2(4.5f * w), qb, wr);
    put(Int<2 * k + 1>{}, fma2(F2(3.0f * w), cm, base));
    put(Int<2 * k + 2>{}, fma2(F2(-3.0f * w), cm, base));
  };
  pair(Int<0>{}, w1, wr1, bxx - tr, mx);
  pair(Int<1>{}, w1, wr1, byy - tr, my);
  pair(Int<2>{}, w1, wr1, bzz - tr, mz);
  const f2 exy = bxx + byy - tr, exz = bxx + bzz - tr, eyz = byy + bzz - tr;
  pair(Int<3>{}, w2, wr2, exy + bxy2, mx + my);
  pair(Int<4>{}, w2, wr2, exy - bxy2, mx - my);
  pair(Int<5>{}, w2, wr2, exz + bxz2, mx + mz);
  pair(Int<6>{}, w2, wr2, exz - bxz2, mx - mz);
  pair(Int<7>{}, w2, wr2, eyz + byz2, my + mz);
  pair(Int<8>{}, w2, wr2, eyz - byz2, my - mz);
  rho_out = rho;
  ux_out = ux;
  uy_out = uy;
  uz_out = uz;
}

// ---------------------------------------------------------------- two cells per thread, 16-bit storage
// One 32-bit load carries the populations of cells x0 and x0 + 1 (x0 even); a
// warp covers 64 cells of a row.  Pulls along x take the neighbouring cell's
// half from the adjacent lane (warp shuffle); the first and last lane load the
// cell just outside the warp's 64 directly.  Outputs are packed two per 32-bit
// store.  Warps whose segments need flag tests take the same two-cell path with
// the link masks of their cells (pair_links_prefetch, pair_link).
template <int DT> struct Pack16;
template <> struct Pack16<SW_F16_SHIFT> {
  static __device__ __forceinline__ float2 both(uint32_t v) {
    __half2 h;
    *reinterpret_cast<uint32_t *>(&h) = v;
    return __half22float2(h);
  }
  static __device__ __forceinline__ float lo(uint32_t v) { return both(v).x; }
  static __device__ __forceinline__ float hi(uint32_t v) { return both(v).y; }
  static __device__ __forceinline__ float one(const __half *q) { return __half2float(__ldg(q)); }
  static __device__ __forceinline__ uint32_t pack(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
  }
};
template <> struct Pack16<SW_BF16_SHIFT> {
  static __device__ __forceinline__ float2 both(uint32_t v) {
    return make_float2(__uint_as_float(v << 16), __uint_as_float(v & 0xffff0000u));
  }
  static __device__ __forceinline__ float lo(uint32_t v) { return __uint_as_float(v << 16); }
  static __device__ __forceinline__ float hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }
  static __device__ __forceinline__ float one(const __nv_bfloat16 *q) { return __bfloat162float(__ldg(q)); }
  static __device__ __forceinline__ uint32_t pack(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
  }
};

// The link masks of one cell of the checked path, for the flags of its pull
// sources as step_cell maps them (lbm3d.py:77-95): bit i of `solid` is set when
// link i's source is not fluid, bit i of `wall` when it is a stone; bit 0 of
// `solid` marks a cell that is itself not fluid (or lies past the row end).
// The inlet column pulls nothing.  Every load is issued before any is used.
template <typename Ctx>
__device__ __forceinline__ void cell_links(const Ctx &p, int x, int y, int z, uint32_t &solid, uint32_t &wall) {
  const Geom &g = p.g;
  solid = 1u;
  wall = 0u;
  if (x >= g.nx) return;
  const int c = chk(p, (z * g.ny + y) * g.pitch + x);
  const uint8_t own = p.flag[c];
  if (x > 0) {
    const int row = g.pitch, lev = g.ny * g.pitch;
    const int off_xm = c - 1;
    const int off_xp = (x + 1 >= g.nx) ? c : c + 1;
    const int off_ym = (y == 0) ? (g.ny - 1) * row : -row;
    const int off_yp = (y == g.ny - 1) ? -(g.ny - 1) * row : row;
    const int off_zm = -lev;
    const int off_zp = (z == g.nz - 1) ? 0 : lev;
    uint8_t fs[Q];
    static_for<1, Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      constexpr int ex = CX(i), ey = CY(i), ez = CZ(i);
      if (ez == 1 && z == 0) {
        fs[i] = (uint8_t)SW_GROUND;
      } else {
        const int src = chk(p, (ex == 1 ? off_xm : ex == -1 ? off_xp : c) + (ey == 1 ? off_ym : ey == -1 ? off_yp : 0) +
                                   (ez == 1 ? off_zm : ez == -1 ? off_zp : 0));
        fs[i] = __ldg(p.flag + src);
      }
    });
    uint32_t sm = 0u, wm = 0u;
    static_for<1, Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      sm |= (fs[i] != 0 ? 1u : 0u) << i;
      wm |= (fs[i] == SW_WALL ? 1u : 0u) << i;
    });
    solid = sm;
    wall = wm;
  } else {
    solid = 0u;
  }
  if (own != 0) {
    solid = 1u;
    wall = 0u;
  }
}

// The checked path of a cell pair, first part: the link masks of cells x0 and
// x0 + 1 and the bounce-back pairs (the 32-bit pair of population OPP(i) at the
// pair's own offset) of the links that bounce in either cell.  The input
// lattice is not written during the step, so the TMA-staged step issues these
// loads before it waits for its copies and their latency overlaps the copies'.
template <int DT, typename Ctx>
__device__ __forceinline__ void pair_links_prefetch(const Ctx &p, int x0, int y, int z, uint32_t (&sm)[2],
                                                     uint32_t (&wm)[2], uint32_t (&bnc)[Q]) {
  using T = typename Store<DT>::T;
  const Geom &g = p.g;
  cell_links(p, x0, y, z, sm[0], wm[0]);
  cell_links(p, x0 + 1, y, z, sm[1], wm[1]);
  const uint32_t any = (sm[0] | sm[1]) & ~1u;                 // no link bit in a lane past the row end
  const int c = (z * g.ny + y) * g.pitch + x0;                // even: the pair is one aligned 32-bit word
  static_for<1, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    bnc[i] = ((any >> i) & 1u) ? __ldg(reinterpret_cast<const unsigned int *>(p.template in<T>(OPP(i)) + chk(p, c)))
                               : 0u;
  });
  bnc[0] = 0u;
}

// The checked path of a cell pair, second part, for link I once its pulled pair
// vi is built: where the link's source is not fluid the cell takes its own
// population OPP(I) (half-way bounce-back, lbm3d.py:89-95), and a stone's adds
// -2 (f - w) c to the wall force (lbm3d.py:99-101); cell x0 before x0 + 1.
template <int DT, int I>
__device__ __forceinline__ void pair_link(f2 &vi, const uint32_t (&sm)[2], const uint32_t (&wm)[2], uint32_t b,
                                          float &fxw, float &fzw, int &hit) {
  using PK = Pack16<DT>;
  constexpr int ex = CX(I), ez = CZ(I);
  const float2 own = PK::both(b);
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    if ((sm[h] >> I) & 1u) {
      const float val = h ? own.y : own.x;
      if (h) vi.v.y = val;
      else vi.v.x = val;
      if ((wm[h] >> I) & 1u) {
        if constexpr (ex != 0) fxw = fxw - 2.0f * val * (float)ex;
        if constexpr (ez != 0) fzw = fzw - 2.0f * val * (float)ez;
        hit = 1;
      }
    }
  }
}

// The checked path of a cell pair, last part: a cell that is not fluid (bit 0 of
// its mask; also a cell past the row end) gets the rest state g = 0, so that the
// pair's collision stays finite, and is not stored.  Returns the cells to store
// (bit 0: x0, bit 1: x0 + 1).
__device__ __forceinline__ uint32_t pair_solid_cells(f2 (&v)[Q], const uint32_t (&sm)[2]) {
  const bool sa = sm[0] & 1u, sb = sm[1] & 1u;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    if (sa) v[i].v.x = 0.0f;
    if (sb) v[i].v.y = 0.0f;
  }
  return (sa ? 0u : 1u) | (sb ? 0u : 2u);
}

// Collision of a cell pair and its stores.  Both cells of the pair are stored
// with one 32-bit store even when cell x0 + 1 lies past the row end: that
// half lands in the row's padding columns (x >= nx), which nothing reads.  The
// inlet cell (x0 == 0, lbm3d.py:67-71) is collided like the others and then
// overwritten by its equilibrium in a branch only its lane takes.
// has_b: cell x0 + 1 exists (x0 + 1 < nx).  acc_old(k): the old float64 sums
// of the pair for sum k (a double2; .y unused without has_b), called where
// they are added.  MASKED (the checked path): only the cells in `keep` (bit 0:
// x0, bit 1: x0 + 1) are stored and summed; the inlet cell only when kept.
template <int DT, bool ACC, bool MASKED = false, typename Ctx, typename AccOld>
__device__ __forceinline__ void pair_collide_store(const Ctx &p, const f2 (&v)[Q], int x0, int c, int z, bool inlet,
                                                   bool has_b, AccOld &&acc_old, uint32_t keep = 3u) {
  using S = Store<DT>;
  using T = typename S::T;
  using PK = Pack16<DT>;
  const Phys<float> ph = phys<float>(p);
  f2 rho, ux, uy, uz;
  if (MASKED) inlet = inlet && (keep & 1u);
  collide2(v, x0, has_b, ph.nu0, ph.c18, p.x_sponge, ph.sponge_scale, ph.nu_sponge, rho, ux, uy, uz,
           p.status, [&](auto I, f2 o) {
             constexpr int i = decltype(I)::value;
             if (!MASKED || keep == 3u)
               __stcs(reinterpret_cast<unsigned int *>(p.template out<T>(i) + c), PK::pack(o.v.x, o.v.y));
             else if (keep == 1u)
               __stcs(p.template out<T>(i) + c, S::from_shifted(o.v.x));
             else if (keep == 2u)
               __stcs(p.template out<T>(i) + c + 1, S::from_shifted(o.v.y));
           });
  float u0 = 0.0f;
  if (inlet) {
    u0 = __ldg(p.uin + z);
    const float usq = u0 * u0;
    static_for<0, Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      constexpr int ex = CX(i);
      float cu = 0.0f;
      if constexpr (ex != 0) cu = (ex > 0 ? u0 : -u0);
      cu = 3.0f * cu;
      const float w = W<float>(i) * 1.0f * (1.0f + cu + 0.5f * cu * cu - 1.5f * usq);
      __stcs(p.template out<T>(i) + c, S::from_shifted(w - W<float>(i)));
    });
  }
  if (ACC) {
    const double ra = inlet ? 1.0 : (double)rho.v.x, xa = inlet ? (double)u0 : (double)ux.v.x;
    const double ya = inlet ? 0.0 : (double)uy.v.x, za = inlet ? 0.0 : (double)uz.v.x;
    if (MASKED && keep != 3u) {                         // one cell of the pair (or none)
      if (keep == 1u) {
        __stcs(p.accp(0) + c, acc_old(0).x + ra);
        __stcs(p.accp(1) + c, acc_old(1).x + xa);
        __stcs(p.accp(2) + c, acc_old(2).x + ya);
        __stcs(p.accp(3) + c, acc_old(3).x + za);
      } else if (keep == 2u) {
        __stcs(p.accp(0) + c + 1, acc_old(0).y + (double)rho.v.y);
        __stcs(p.accp(1) + c + 1, acc_old(1).y + (double)ux.v.y);
        __stcs(p.accp(2) + c + 1, acc_old(2).y + (double)uy.v.y);
        __stcs(p.accp(3) + c + 1, acc_old(3).y + (double)uz.v.y);
      }
    } else if (has_b) {                                 // cells x0, x0 + 1: one 16-byte update per sum
      const double2 v0 = acc_old(0), v1 = acc_old(1), v2 = acc_old(2), v3 = acc_old(3);
      __stcs(reinterpret_cast<double2 *>(p.accp(0) + c), make_double2(v0.x + ra, v0.y + (double)rho.v.y));
      __stcs(reinterpret_cast<double2 *>(p.accp(1) + c), make_double2(v1.x + xa, v1.y + (double)ux.v.y));
      __stcs(reinterpret_cast<double2 *>(p.accp(2) + c), make_double2(v2.x + ya, v2.y + (double)uy.v.y));
      __stcs(reinterpret_cast<double2 *>(p.accp(3) + c), make_double2(v3.x + za, v3.y + (double)uz.v.y));
    } else {
      __stcs(p.accp(0) + c, acc_old(0).x + ra);
      __stcs(p.accp(1) + c, acc_old(1).x + xa);
      __stcs(p.accp(2) + c, acc_old(2).x + ya);
      __stcs(p.accp(3) + c, acc_old(3).x + za);
    }
  }
}

template <int DT, bool ACC, typename Ctx>
__device__ __forceinline__ void step_pair_fast(const Ctx &p, int x0, int y, int z, int lane) {
  using T = typename Store<DT>::T;
  using PK = Pack16<DT>;
  const Geom &g = p.g;
  const bool live = x0 < g.nx;        // cell x0 exists; the 32-bit pair lies inside the row
  const bool has_b = x0 + 1 < g.nx;   // cell x0 + 1 exists
  const bool has_r = x0 + 2 < g.nx;   // cell x0 + 2 exists (else the outlet copies x0 + 1)
  const bool inlet = x0 == 0;         // cell x0 is the inlet
  const int c = chk(p, (z * g.ny + y) * g.pitch + x0);
  auto in = [&](int pop) { return p.template in<T>(pop); };
  const int row = g.pitch, lev = g.ny * g.pitch;
  const int off_ym = (y == 0) ? (g.ny - 1) * row : -row;
  const int off_yp = (y == g.ny - 1) ? -(g.ny - 1) * row : row;
  const bool top = (z == g.nz - 1);
  const int off_zm = -lev;
  const int off_zp = top ? 0 : lev;
  // phase 1: every load in flight before the first shuffle consumes one
  uint32_t P[Q];
  float edge[Q];                                        // lane 0: cell x0 - 1, lane 31: cell x0 + 2
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ex = CX(i), ey = CY(i), ez = CZ(i);
    const int rowoff = (ey == 1 ? off_ym : ey == -1 ? off_yp : 0) + (ez == 1 ? off_zm : ez == -1 ? off_zp : 0);
    const T *plane = (ez == -1 && top) ? in(MIRZ(i)) : in(i);
    const int src = c + rowoff;                                       // source row, column x0
    P[i] = live ? __ldg(reinterpret_cast<const unsigned int *>(plane + chk(p, src))) : 0u;
    if constexpr (ex == 1) edge[i] = (lane == 0 && live && x0 > 0) ? PK::one(plane + chk(p, src - 1)) : 0.0f;
    if constexpr (ex == -1) edge[i] = (lane == 31 && live && has_r) ? PK::one(plane + chk(p, src + 2)) : 0.0f;
  });
  // accumulation steps: the sums of both cells, read with the populations
  double2 acc_old[4];
  if (ACC) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (live && has_b) acc_old[k] = __ldcs(reinterpret_cast<const double2 *>(p.accp(k) + c));
      else acc_old[k] = make_double2(live ? __ldcs(p.accp(k) + c) : 0.0, 0.0);
    }
  }
  // phase 2: pulls along x from the neighbouring lanes (outlet copies column x)
  f2 v[Q];
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ex = CX(i);
    const float2 own = PK::both(P[i]);
    if constexpr (ex == 0) {
      v[i].v = own;
    } else if constexpr (ex == 1) {                     // sources x0 - 1, x0
      const uint32_t prev = __shfl_up_sync(0xffffffffu, P[i], 1);
      v[i] = F2(lane == 0 ? edge[i] : PK::hi(prev), own.x);
    } else {                                            // sources x0 + 1, x0 + 2
      const uint32_t next = __shfl_down_sync(0xffffffffu, P[i], 1);
      const float right = lane == 31 ? edge[i] : PK::lo(next);
      v[i] = F2(has_b ? own.y : own.x, has_r ? right : own.y);
    }
  });
  if (!live) return;
  pair_collide_store<DT, ACC>(p, v, x0, c, z, inlet, has_b, [&](int k) { return acc_old[k]; });
}

// The checked two-cell step of a lane (segments next to stones or the ground):
// step_pair_fast's loads and pulls, then the link masks and bounce-back pairs
// of pair_links_prefetch replace the pulls of the links whose sources are not
// fluid, wall links add to fxw / fzw / hit, and cells that are not fluid are
// not stored; a source below z = 0 is not read.  (A separate copy: sharing one
// template with the fast path changed the fast path's code and slowed it.)
template <int DT, bool ACC, typename Ctx>
__device__ __forceinline__ void step_pair_links(const Ctx &p, int x0, int y, int z, int lane, const uint32_t (&sm)[2],
                                                const uint32_t (&wm)[2], const uint32_t (&bnc)[Q], float &fxw,
                                                float &fzw, int &hit) {
  using T = typename Store<DT>::T;
  using PK = Pack16<DT>;
  const Geom &g = p.g;
  const bool live = x0 < g.nx;        // cell x0 exists; the 32-bit pair lies inside the row
  const bool has_b = x0 + 1 < g.nx;   // cell x0 + 1 exists
  const bool has_r = x0 + 2 < g.nx;   // cell x0 + 2 exists (else the outlet copies x0 + 1)
  const bool inlet = x0 == 0;         // cell x0 is the inlet
  const int c0 = (z * g.ny + y) * g.pitch + x0;
  const int c = live ? chk(p, c0) : c0;                             // a lane past the row end uses no offset
  auto in = [&](int pop) { return p.template in<T>(pop); };
  const int row = g.pitch, lev = g.ny * g.pitch;
  const int off_ym = (y == 0) ? (g.ny - 1) * row : -row;
  const int off_yp = (y == g.ny - 1) ? -(g.ny - 1) * row : row;
  const bool top = (z == g.nz - 1);
  const int off_zm = -lev;
  const int off_zp = top ? 0 : lev;
  // phase 1: every load in flight before the first shuffle consumes one
  uint32_t P[Q];
  float edge[Q];                                        // lane 0: cell x0 - 1, lane 31: cell x0 + 2
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ex = CX(i), ey = CY(i), ez = CZ(i);
    const int rowoff = (ey == 1 ? off_ym : ey == -1 ? off_yp : 0) + (ez == 1 ? off_zm : ez == -1 ? off_zp : 0);
    const T *plane = (ez == -1 && top) ? in(MIRZ(i)) : in(i);
    const int src = c + rowoff;                                       // source row, column x0
    const bool ld = live && !(ez == 1 && z == 0);                     // (the ground below z = 0 bounces)
    P[i] = ld ? __ldg(reinterpret_cast<const unsigned int *>(plane + chk(p, src))) : 0u;
    if constexpr (ex == 1) edge[i] = (lane == 0 && ld && x0 > 0) ? PK::one(plane + chk(p, src - 1)) : 0.0f;
    if constexpr (ex == -1) edge[i] = (lane == 31 && ld && has_r) ? PK::one(plane + chk(p, src + 2)) : 0.0f;
  });
  // accumulation steps: the sums of both cells, read with the populations
  double2 acc_old[4];
  if (ACC) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (live && has_b) acc_old[k] = __ldcs(reinterpret_cast<const double2 *>(p.accp(k) + c));
      else acc_old[k] = make_double2(live ? __ldcs(p.accp(k) + c) : 0.0, 0.0);
    }
  }
  // phase 2: pulls along x from the neighbouring lanes (outlet copies column x)
  f2 v[Q];
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ex = CX(i);
    const float2 own = PK::both(P[i]);
    if constexpr (ex == 0) {
      v[i].v = own;
    } else if constexpr (ex == 1) {                     // sources x0 - 1, x0
      const uint32_t prev = __shfl_up_sync(0xffffffffu, P[i], 1);
      v[i] = F2(lane == 0 ? edge[i] : PK::hi(prev), own.x);
    } else {                                            // sources x0 + 1, x0 + 2
      const uint32_t next = __shfl_down_sync(0xffffffffu, P[i], 1);
      const float right = lane == 31 ? edge[i] : PK::lo(next);
      v[i] = F2(has_b ? own.y : own.x, has_r ? right : own.y);
    }
    if constexpr (i > 0) pair_link<DT, i>(v[i], sm, wm, bnc[i], fxw, fzw, hit);
  });
  if (!live) return;
  const uint32_t keep = pair_solid_cells(v, sm);
  if (keep == 0u) return;
  pair_collide_store<DT, ACC, true>(p, v, x0, c, z, inlet, has_b, [&](int k) { return acc_old[k]; }, keep);
}

// The checked path of a two-cell warp (segments next to stones or the ground).
// A separate function: inlined next to the fast path, its masks and bounce-back
// pairs would set the register allocation of the whole kernel and make the
// fast path spill.
template <int DT, bool ACC, typename Ctx>
__device__ __noinline__ void step_pair_checked(const Ctx &p, int x0, int y, int z, int lane, bool force) {
  float fxw = 0.0f, fzw = 0.0f;
  int hit = 0;
  uint32_t sm[2], wm[2], bnc[Q];
  pair_links_prefetch<DT>(p, x0, y, z, sm, wm, bnc);
  step_pair_links<DT, ACC>(p, x0, y, z, lane, sm, wm, bnc, fxw, fzw, hit);
  if (force && p.force != nullptr) warp_force_add<float>(p, z, lane, fxw, fzw, hit);
}

// One warp, the row segments 2 bx and 2 bx + 1 of (y, z).
template <int DT, bool ACC, typename Ctx>
__device__ __forceinline__ void step_pair_segment(const Ctx &p, int bx, int y, int z, int lane) {
  const Geom &g = p.g;
  const int sa = 2 * bx;
  const bool has_tb = sa + 1 < g.nseg_x;
  const int seg = (z * g.ny + y) * g.nseg_x + sa;
  const uint8_t ka = __ldg(p.tiles + seg);
  const uint8_t kb = has_tb ? __ldg(p.tiles + seg + 1) : (uint8_t)TILE_ALL_SOLID;
  if ((ka & kb & TILE_ALL_SOLID)) return;
  const int x0 = 2 * SEG * bx + 2 * lane;
  if (!((ka | kb) & TILE_CHECK)) {
    step_pair_fast<DT, ACC>(p, x0, y, z, lane);
    return;
  }
  step_pair_checked<DT, ACC>(p, x0, y, z, lane, (ka | kb) & TILE_FORCE);
}

// Grid: (ceil(pitch / 64), ceil(ny / WY), nz); warp = two adjacent row segments.
template <int DT, bool ACC, typename Cfg>
__global__ void __launch_bounds__(Cfg::THREADS, Cfg::MINB) k_step_pair(const __grid_constant__ StepParams p) {
  const int y = blockIdx.y * Cfg::WY + threadIdx.y;
  if (y >= p.g.ny) return;
  step_pair_segment<DT, ACC>(p, blockIdx.x, y, (int)blockIdx.z, threadIdx.x);
}

template <int DT, bool ACC, typename Cfg>
cudaError_t launch_cfg(const StepParams &p, cudaStream_t s) {
  const dim3 grid((unsigned)p.g.nseg_x, (unsigned)((p.g.ny + Cfg::WY - 1) / Cfg::WY), (unsigned)p.g.nz);
  const dim3 block(32, Cfg::WY);
  k_step_pull<DT, ACC, Cfg><<<grid, block, 0, s>>>(p);
  return cudaGetLastError();
}

template <int DT, bool ACC, typename Cfg>
cudaError_t launch_pair(const StepParams &p, cudaStream_t s) {
  const dim3 grid((unsigned)((p.g.nseg_x + 1) / 2), (unsigned)((p.g.ny + Cfg::WY - 1) / Cfg::WY), (unsigned)p.g.nz);
  const dim3 block(32, Cfg::WY);
  k_step_pair<DT, ACC, Cfg><<<grid, block, 0, s>>>(p);
  return cudaGetLastError();
}

constexpr bool is16(int dt) { return dt == SW_F16_SHIFT || dt == SW_BF16_SHIFT; }

// Whether configuration cfg exists for storage type dt.
inline bool step_config_valid(int dt, int cfg) {
  return (cfg >= 0 && cfg < 4) || (cfg >= 4 && cfg < kStepConfigs && is16(dt));
}
// Whether the persistent batched kernel has configuration cfg (not the TMA-staged ones).
inline bool batch_config_valid(int dt, int cfg) { return cfg < 8 && step_config_valid(dt, cfg); }

}  // namespace sw
#include "sw_tma.cuh"
namespace sw {

template <int DT>
cudaError_t launch_step(const StepParams &p_in, cudaStream_t s) {
  if (p_in.g.nz > 65535 || (p_in.g.ny + 3) / 4 > 65535) return cudaErrorInvalidValue;
  StepParams p = p_in;
  set_plane_bases(p, sizeof(typename Store<DT>::T));
  set_float_params(p);
  switch (p.cfg) {
#define SW_CASE(ID, WY, MINB)                                                                      \
  case ID:                                                                                         \
    return p.acc ? launch_cfg<DT, true, StepCfg<WY, MINB>>(p, s) : launch_cfg<DT, false, StepCfg<WY, MINB>>(p, s);
    SW_STEP_CONFIGS(SW_CASE)
#undef SW_CASE
#define SW_CASE(ID, WY, MINB)                                                                      \
  case ID:                                                                                         \
    if constexpr (is16(DT))                                                                        \
      return p.acc ? launch_pair<DT, true, StepCfg<WY, MINB>>(p, s)                               \
                   : launch_pair<DT, false, StepCfg<WY, MINB>>(p, s);                             \
    else                                                                                           \
      return cudaErrorNotSupported;
    SW_PAIR_CONFIGS(SW_CASE)
#undef SW_CASE
#define SW_CASE(ID, ITEMS, NSTAGE, MINB)                                                          \
  case ID:                                                                                         \
    if constexpr (is16(DT))                                                                        \
      return p.acc ? launch_tma<DT, true, TmaCfg<ITEMS, NSTAGE, MINB>>(p, s)                      \
                   : launch_tma<DT, false, TmaCfg<ITEMS, NSTAGE, MINB>>(p, s);                    \
    else                                                                                           \
      return cudaErrorNotSupported;
    SW_TMA_CONFIGS(SW_CASE)
#undef SW_CASE
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace sw
