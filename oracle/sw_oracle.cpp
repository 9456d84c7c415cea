// sw_oracle.cpp -- CPU oracle for the fused D3Q19 timestep.
//
// TEST INFRASTRUCTURE ONLY.  This file is a line-by-line CPU restatement of the
// reference's Warp kernels in stonewall3d/lbm3d.py.  Only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm load it,
// and only as the checker (or as the timed CPU baseline).  The product path
// (libstonewall.so) never links or calls it.
//
// Pinning: tests/golden/*.npz hold outputs of the reference's own kernel bodies
// (lbm3d.py k_init/k_step/k_macro/k_accum and its main() driver) executed in
// float32 by tests/golden/make_golden.py.  tests/test_oracle_golden.py checks
// this file against them bit-for-bit on the fields.  Warp itself (third-party,
// version unpinned in the reference, not installable here) is not reproduced:
// its RNG stream is restated below from the published PCG hash, and its GPU
// FMA-contraction choices are not modelled (this file is built with
// -ffp-contract=off so that it evaluates every expression in source order).
//
// Layout: the reference's own, C-contiguous with z fastest:
//   f[i][x][y][z]  (i < 19),  flag[x][y][z],  u[c][x][y][z]  (c < 4).
// Forces are accumulated in double per z level (the reference adds float32
// atomics into force[t][z][0..1], lbm3d.py:99-101; any summation order is a
// valid execution of that, this one is fixed: per x-plane partials summed in
// increasing x).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// D3Q19 velocity set, lbm3d.py:20-24 (order is part of the checkpoint format).
const int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
const int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
// lbm3d.py:26  (pairs (1,2), (3,4), ...)
const int OPP[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};
// lbm3d.py:27  (c_z -> -c_z)
const int MIRZ[19] = {0, 1, 2, 3, 4, 6, 5, 7, 8, 9, 10, 13, 14, 11, 12, 17, 18, 15, 16};

template <typename R> R weight(int i);
// lbm3d.py:25: float32 weights (double 1/3 etc. rounded to float32)
template <> float weight<float>(int i) {
  return i == 0 ? (float)(1.0 / 3.0) : (i < 7 ? (float)(1.0 / 18.0) : (float)(1.0 / 36.0));
}
template <> double weight<double>(int i) {
  return i == 0 ? 1.0 / 3.0 : (i < 7 ? 1.0 / 18.0 : 1.0 / 36.0);
}

// lbm3d.py:33-36
template <typename R>
inline R feq_i(R w, R cx, R cy, R cz, R rho, R ux, R uy, R uz) {
  R cu = R(3.0) * (cx * ux + cy * uy + cz * uz);
  return w * rho * (R(1.0) + cu + R(0.5) * cu * cu - R(1.5) * (ux * ux + uy * uy + uz * uz));
}

// Counter-based RNG used by k_init (lbm3d.py:48-52 calls Warp's
// wp.rand_init(seed, offset) and wp.randf(state)).  Restated from the published
// PCG hash (Jarzynski & Olano, "Hash Functions for GPU Rendering", JCGT 2020):
//   state0 = pcg(seed + pcg(offset)),  randf: state = pcg(state); (state >> 8) / 2^24.
inline uint32_t pcg_hash(uint32_t s) {
  uint32_t b = s * 747796405u + 2891336453u;
  uint32_t c = ((b >> ((b >> 28u) + 4u)) ^ b) * 277803737u;
  return (c >> 22u) ^ c;
}
inline float randf(uint32_t &st) {
  st = pcg_hash(st);
  return (float)(st >> 8) * (1.0f / 16777216.0f);
}
// Standard normal from two uniforms (Box-Muller, evaluated in double and rounded).
inline float gauss_pair(uint32_t &st, float *second) {
  double u1 = 1.0 - (double)randf(st);  // (0, 1]
  double u2 = (double)randf(st);
  double r = std::sqrt(-2.0 * std::log(u1));
  double a = 6.283185307179586 * u2;
  if (second) *second = (float)(r * std::sin(a));
  return (float)(r * std::cos(a));
}

struct Grid {
  int nx, ny, nz;
  size_t cells() const { return (size_t)nx * ny * nz; }
  size_t at(int x, int y, int z) const { return ((size_t)x * ny + y) * nz + z; }
};

// lbm3d.py:39-54.  noise_kind 0: uniform as the reference (u0*(1+noise*(2r-1)), ...);
// noise_kind 1: Gaussian (u0*(1+noise*g1), u0*noise*g2, u0*noise*g3).
template <typename R>
void init(R *f, const uint8_t *flag, const R *uin, Grid g, R noise, int seed, int noise_kind) {
  const size_t N = g.cells();
#pragma omp parallel for schedule(static)
  for (int x = 0; x < g.nx; ++x)
    for (int y = 0; y < g.ny; ++y)
      for (int z = 0; z < g.nz; ++z) {
        size_t c = g.at(x, y, z);
        R ux = R(0.0), uy = R(0.0), uz = R(0.0);
        if (flag[c] == 0) {
          uint32_t off = ((uint32_t)x * 7919u + (uint32_t)y) * 7907u + (uint32_t)z;
          uint32_t st = pcg_hash((uint32_t)seed + pcg_hash(off));
          R u0 = uin[z];
          if (noise_kind == 0) {
            ux = u0 * (R(1.0) + noise * (R(2.0) * (R)randf(st) - R(1.0)));
            uy = u0 * noise * (R(2.0) * (R)randf(st) - R(1.0));
            uz = u0 * noise * (R(2.0) * (R)randf(st) - R(1.0));
          } else {
            float g2 = 0.0f;
            float g1 = gauss_pair(st, &g2);
            float g3 = gauss_pair(st, nullptr);
            ux = u0 * (R(1.0) + noise * (R)g1);
            uy = u0 * noise * (R)g2;
            uz = u0 * noise * (R)g3;
          }
        }
        for (int i = 0; i < 19; ++i)
          f[(size_t)i * N + c] = feq_i<R>(weight<R>(i), (R)CX[i], (R)CY[i], (R)CZ[i], R(1.0), ux, uy, uz);
      }
}

// One cell of k_step, lbm3d.py:64-155, statement by statement.
template <typename R>
inline void step_cell(const R *fin, R *fout, const uint8_t *flag, const R *uin, Grid g, size_t N,
                      R nu0, R cs, int x_sponge, R nu_sponge, int x, int y, int z, double *fpart) {
  const size_t c = g.at(x, y, z);
  if (flag[c] != 0) return;                                       // :65-66
  if (x == 0) {                                                   // :67-71 inlet
    R u0 = uin[z];
    for (int i = 0; i < 19; ++i)
      fout[(size_t)i * N + c] = feq_i<R>(weight<R>(i), (R)CX[i], (R)CY[i], (R)CZ[i], R(1.0), u0, R(0.0), R(0.0));
    return;
  }
  R fl[19];
  R fxw = R(0.0), fzw = R(0.0);
  int hit = 0;
  for (int i = 0; i < 19; ++i) {                                  // :77-98
    int xs = x - CX[i];
    int ys = (y - CY[i] + g.ny) % g.ny;
    int zs = z - CZ[i];
    int j = i;
    if (xs >= g.nx) xs = x;                                       // outlet
    if (zs >= g.nz) { zs = z; j = MIRZ[i]; }                      // top
    R val;
    uint8_t fs = flag[g.at(xs, ys, zs)];
    if (fs != 0) {                                                // bounce-back
      val = fin[(size_t)OPP[i] * N + c];
      if (fs == 1) {                                              // momentum exchange
        R fr = val - weight<R>(i);
        fxw = fxw - R(2.0) * fr * (R)CX[i];
        fzw = fzw - R(2.0) * fr * (R)CZ[i];
        hit = 1;
      }
    } else {
      val = fin[(size_t)j * N + g.at(xs, ys, zs)];
    }
    fl[i] = val;
  }
  if (hit == 1) {                                                 // :99-101
    fpart[2 * z + 0] += (double)fxw;
    fpart[2 * z + 1] += (double)fzw;
  }
  R rho = R(0.0), mx = R(0.0), my = R(0.0), mz = R(0.0);         // :103-127
  R pxx = R(0.0), pyy = R(0.0), pzz = R(0.0), pxy = R(0.0), pxz = R(0.0), pyz = R(0.0);
  for (int i = 0; i < 19; ++i) {
    R v = fl[i];
    R ex = (R)CX[i], ey = (R)CY[i], ez = (R)CZ[i];
    rho += v;
    mx += v * ex;
    my += v * ey;
    mz += v * ez;
    pxx += v * ex * ex;
    pyy += v * ey * ey;
    pzz += v * ez * ez;
    pxy += v * ex * ey;
    pxz += v * ex * ez;
    pyz += v * ey * ez;
  }
  R ux = mx / rho, uy = my / rho, uz = mz / rho;                  // :128-138
  R third = rho / R(3.0);
  R nxx = pxx - third - rho * ux * ux;
  R nyy = pyy - third - rho * uy * uy;
  R nzz = pzz - third - rho * uz * uz;
  R nxy = pxy - rho * ux * uy;
  R nxz = pxz - rho * ux * uz;
  R nyz = pyz - rho * uy * uz;
  R nu = nu0;                                                     // :140-143 sponge
  if (x > x_sponge) {
    R s = (R)(x - x_sponge) / (R)(g.nx - x_sponge);
    nu = nu0 + nu_sponge * s * s;
  }
  R tau0 = R(3.0) * nu + R(0.5);                                  // :144-147 Smagorinsky
  R qn = std::sqrt(nxx * nxx + nyy * nyy + nzz * nzz + R(2.0) * (nxy * nxy + nxz * nxz + nyz * nyz));
  R tau = R(0.5) * (tau0 + std::sqrt(tau0 * tau0 + R(18.0) * std::sqrt(R(2.0)) * cs * cs * qn / rho));
  R keep = R(1.0) - R(1.0) / tau;
  for (int i = 0; i < 19; ++i) {                                  // :149-155 regularized write
    R ex = (R)CX[i], ey = (R)CY[i], ez = (R)CZ[i];
    R qq = ((ex * ex - R(1.0) / R(3.0)) * nxx + (ey * ey - R(1.0) / R(3.0)) * nyy +
            (ez * ez - R(1.0) / R(3.0)) * nzz + R(2.0) * (ex * ey * nxy + ex * ez * nxz + ey * ez * nyz));
    fout[(size_t)i * N + c] = feq_i<R>(weight<R>(i), ex, ey, ez, rho, ux, uy, uz) + keep * weight<R>(i) * R(4.5) * qq;
  }
}

template <typename R>
void step(const R *fin, R *fout, const uint8_t *flag, const R *uin, Grid g, R nu0, R cs, int x_sponge,
          R nu_sponge, double *force_row /* [nz][2], accumulated */) {
  const size_t N = g.cells();
  std::vector<double> part((size_t)g.nx * g.nz * 2, 0.0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int x = 0; x < g.nx; ++x) {
    double *fp = part.data() + (size_t)x * g.nz * 2;
    for (int y = 0; y < g.ny; ++y)
      for (int z = 0; z < g.nz; ++z)
        step_cell<R>(fin, fout, flag, uin, g, N, nu0, cs, x_sponge, nu_sponge, x, y, z, fp);
  }
  if (force_row)
    for (int x = 0; x < g.nx; ++x)
      for (int k = 0; k < 2 * g.nz; ++k) force_row[k] += part[(size_t)x * g.nz * 2 + k];
}

// lbm3d.py:158-182
template <typename R>
void macro(const R *f, const uint8_t *flag, Grid g, R *u) {
  const size_t N = g.cells();
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < (long long)N; ++c) {
    if (flag[c] != 0) {
      u[c] = R(1.0); u[N + c] = R(0.0); u[2 * N + c] = R(0.0); u[3 * N + c] = R(0.0);
      continue;
    }
    R rho = R(0.0), mx = R(0.0), my = R(0.0), mz = R(0.0);
    for (int i = 0; i < 19; ++i) {
      R v = f[(size_t)i * N + c];
      rho += v;
      mx += v * (R)CX[i];
      my += v * (R)CY[i];
      mz += v * (R)CZ[i];
    }
    u[c] = rho; u[N + c] = mx / rho; u[2 * N + c] = my / rho; u[3 * N + c] = mz / rho;
  }
}

}  // namespace

extern "C" {

int sw_oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void sw_oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// Tables as laid out in lbm3d.py:20-28 (c: [19][3]).
void sw_oracle_tables(int32_t *c, float *w, int32_t *opp, int32_t *mirz) {
  for (int i = 0; i < 19; ++i) {
    c[3 * i] = CX[i]; c[3 * i + 1] = CY[i]; c[3 * i + 2] = CZ[i];
    w[i] = weight<float>(i); opp[i] = OPP[i]; mirz[i] = MIRZ[i];
  }
}

void sw_oracle_init_f32(float *f, const uint8_t *flag, const float *uin, int nx, int ny, int nz,
                        float noise, int seed, int noise_kind) {
  init<float>(f, flag, uin, Grid{nx, ny, nz}, noise, seed, noise_kind);
}
void sw_oracle_init_f64(double *f, const uint8_t *flag, const double *uin, int nx, int ny, int nz,
                        double noise, int seed, int noise_kind) {
  init<double>(f, flag, uin, Grid{nx, ny, nz}, noise, seed, noise_kind);
}
void sw_oracle_step_f32(const float *fin, float *fout, const uint8_t *flag, const float *uin, int nx, int ny,
                        int nz, float nu0, float cs, int x_sponge, float nu_sponge, double *force_row) {
  step<float>(fin, fout, flag, uin, Grid{nx, ny, nz}, nu0, cs, x_sponge, nu_sponge, force_row);
}
void sw_oracle_step_f64(const double *fin, double *fout, const uint8_t *flag, const double *uin, int nx,
                        int ny, int nz, double nu0, double cs, int x_sponge, double nu_sponge,
                        double *force_row) {
  step<double>(fin, fout, flag, uin, Grid{nx, ny, nz}, nu0, cs, x_sponge, nu_sponge, force_row);
}
void sw_oracle_macro_f32(const float *f, const uint8_t *flag, int nx, int ny, int nz, float *u) {
  macro<float>(f, flag, Grid{nx, ny, nz}, u);
}
void sw_oracle_macro_f64(const double *f, const uint8_t *flag, int nx, int ny, int nz, double *u) {
  macro<double>(f, flag, Grid{nx, ny, nz}, u);
}
// lbm3d.py:185-188 (acc += u), accumulated here in double.
void sw_oracle_accum(const float *u, double *acc, long long n) {
#pragma omp parallel for schedule(static)
  for (long long k = 0; k < n; ++k) acc[k] += (double)u[k];
}

}  // extern "C"
