// sw_capi.cu -- the extern "C" entry points declared in include/stonewall.h.
//
// Every entry point validates its arguments, launches on the caller's stream
// and returns an SW_* status; nothing here allocates or synchronises.
#include <algorithm>
#include <cstddef>
#include <cstdio>

#include "sw_aa.cuh"
#include "sw_aux.cuh"
#include "sw_batch.cuh"
#include "sw_step.cuh"

namespace {

thread_local int g_last_cuda = 0;

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return SW_OK;
  g_last_cuda = (int)e;
  return SW_ERR_CUDA;
}

bool geom_ok(const sw_geom *g) {
  if (!g || g->nx <= 0 || g->ny <= 0 || g->nz <= 0) return false;
  if (g->pitch != sw::round_up(g->nx, sw::SEG)) return false;
  const long long cells = (long long)g->nz * g->ny * g->pitch;
  return cells < (1ll << 31);
}

sw::Geom to_geom(const sw_geom *g) {
  sw::Geom o;
  o.nx = g->nx;
  o.ny = g->ny;
  o.nz = g->nz;
  o.pitch = g->pitch;
  o.nseg_x = g->pitch / sw::SEG;
  o.plane = (long long)g->nz * g->ny * g->pitch;
  return o;
}

bool dtype_ok(int dt) { return dt == SW_F32 || dt == SW_F64 || dt == SW_F16_SHIFT || dt == SW_BF16_SHIFT; }
bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

cudaStream_t st(sw_stream s) { return reinterpret_cast<cudaStream_t>(s); }

// Clears the calling thread's last CUDA error before this library launches, so
// that the error read after the launch is the launch's own and not one an
// earlier, unrelated runtime call (in the caller or another library) left behind.
void clear_stale() { (void)cudaGetLastError(); }

}  // namespace

namespace sw {
// Records a CUDA error code for sw_last_cuda_error() and returns SW_ERR_CUDA
// (for entry points defined in other translation units).
int note_cuda_error(int cuda_error) { return cuda_status((cudaError_t)cuda_error); }
}  // namespace sw

extern "C" {

const char *sw_version(void) { return "stonewall-gb300 0.1 (sm_103a)"; }

const char *sw_status_string(int status) {
  switch (status) {
    case SW_OK: return "ok";
    case SW_ERR_BAD_ARG: return "bad argument";
    case SW_ERR_OOM: return "out of device memory";
    case SW_ERR_NONFINITE: return "non-finite state";
    case SW_ERR_TIMEOUT: return "device wait timed out";
    case SW_ERR_CUDA: return "CUDA error";
    case SW_ERR_UNSUPPORTED: return "unsupported";
    case SW_ERR_TOO_LARGE: return "grid larger than the fixed scratch of sw_step_noalloc";
    default: return "unknown status";
  }
}

int sw_last_cuda_error(void) { return g_last_cuda; }

int sw_geom_make(int32_t nx, int32_t ny, int32_t nz, sw_geom *out) {
  if (!out || nx <= 0 || ny <= 0 || nz <= 0) return SW_ERR_BAD_ARG;
  sw_geom g{nx, ny, nz, sw::round_up(nx, sw::SEG)};
  if (!geom_ok(&g)) return SW_ERR_BAD_ARG;
  *out = g;
  return SW_OK;
}

int64_t sw_cells_padded(const sw_geom *g) { return geom_ok(g) ? (int64_t)g->nz * g->ny * g->pitch : -1; }
int64_t sw_lattice_elems(const sw_geom *g) { return geom_ok(g) ? (int64_t)sw::Q * g->nz * g->ny * g->pitch : -1; }
int64_t sw_tile_count(const sw_geom *g) { return geom_ok(g) ? (int64_t)g->nz * g->ny * (g->pitch / sw::SEG) : -1; }

size_t sw_dtype_size(int dtype) {
  switch (dtype) {
    case SW_F32: return 4;
    case SW_F64: return 8;
    case SW_F16_SHIFT: return 2;
    case SW_BF16_SHIFT: return 2;
    default: return 0;
  }
}

int sw_pack_flag(const sw_geom *g, const uint8_t *flag_ref, uint8_t *flag, sw_stream s) {
  if (!geom_ok(g) || !flag_ref || !flag) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_pack_flag(to_geom(g), flag_ref, flag, st(s)));
}

int sw_pack_f(const sw_geom *g, int dtype, int ref_dtype, const void *f_ref, void *f, sw_stream s) {
  if (!geom_ok(g) || !dtype_ok(dtype) || (ref_dtype != SW_F32 && ref_dtype != SW_F64) || !f_ref || !f)
    return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_pack_f(to_geom(g), dtype, ref_dtype, f_ref, f, st(s)));
}

int sw_unpack_f(const sw_geom *g, int dtype, int ref_dtype, const void *f, void *f_ref, sw_stream s) {
  if (!geom_ok(g) || !dtype_ok(dtype) || (ref_dtype != SW_F32 && ref_dtype != SW_F64) || !f_ref || !f)
    return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_unpack_f(to_geom(g), dtype, ref_dtype, f, f_ref, st(s)));
}

int sw_unpack_u(const sw_geom *g, const float *u, float *u_ref, sw_stream s) {
  if (!geom_ok(g) || !u || !u_ref) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_unpack_u(to_geom(g), u, u_ref, st(s)));
}

int sw_unpack_acc(const sw_geom *g, const double *acc, double *acc_ref, sw_stream s) {
  if (!geom_ok(g) || !acc || !acc_ref) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_unpack_acc(to_geom(g), acc, acc_ref, st(s)));
}

int sw_build_tiles(const sw_geom *g, const uint8_t *flag, uint8_t *tiles, sw_stream s) {
  if (!geom_ok(g) || !flag || !tiles) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_build_tiles(to_geom(g), flag, tiles, st(s)));
}

int sw_init(const sw_geom *g, int dtype, void *f, const uint8_t *flag, const float *uin, float noise, int32_t seed,
            int32_t noise_kind, sw_stream s) {
  if (!geom_ok(g) || !dtype_ok(dtype) || !f || !flag || !uin || !aligned16(f)) return SW_ERR_BAD_ARG;
  if (noise_kind != SW_NOISE_UNIFORM && noise_kind != SW_NOISE_GAUSSIAN) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_init(to_geom(g), dtype, f, flag, uin, noise, seed, noise_kind, st(s)));
}

namespace {
// launch configurations used by sw_step and by sw_step_accum, per storage type
int g_step_cfg[4] = {0, 0, 0, 0};
int g_step_cfg_acc[4] = {0, 0, 0, 0};
// polls of a TMA-staged block on one stage before it gives up (sw_debug_tma_poll_limit)
int g_tma_poll_limit = 1 << 14;

void fill_physics(sw::StepParams &p, const sw_geom *g, double nu0, double cs, int32_t x_sponge, double nu_sponge) {
  p.nu0 = nu0;
  p.cs = cs;
  p.nu_sponge = nu_sponge;
  p.x_sponge = x_sponge;
  p.sponge_scale = (g->nx != x_sponge) ? 1.0 / (double)(g->nx - x_sponge) : 0.0;
}

int step_impl(const sw_geom *g, int dtype, const void *f_in, void *f_out, const uint8_t *flag, const uint8_t *tiles,
              const float *uin, double nu0, double cs, int32_t x_sponge, double nu_sponge, int64_t *force,
              int64_t t, double *acc, int cfg, uint32_t *status, sw_stream s) {
  if (!geom_ok(g) || !dtype_ok(dtype) || !f_in || !f_out || !flag || !tiles || !uin) return SW_ERR_BAD_ARG;
  if (cfg == -1) cfg = acc ? g_step_cfg_acc[dtype] : g_step_cfg[dtype];
  if (cfg < 0 || cfg >= sw::kStepConfigs) return SW_ERR_BAD_ARG;
  if (!sw::step_config_valid(dtype, cfg)) return SW_ERR_UNSUPPORTED;
  if (f_in == f_out || !aligned16(f_in) || !aligned16(f_out) || t < 0) return SW_ERR_BAD_ARG;
  if (status && ((uintptr_t)status & 3u)) return SW_ERR_BAD_ARG;
  sw::StepParams p;
  p.fin = f_in;
  p.fout = f_out;
  p.flag = flag;
  p.tiles = tiles;
  p.uin = uin;
  p.g = to_geom(g);
  fill_physics(p, g, nu0, cs, x_sponge, nu_sponge);
  p.force = force ? reinterpret_cast<long long *>(force) + (size_t)t * 2 * g->nz : nullptr;
  p.acc = acc;
  p.status = status;
  p.cfg = cfg;
  p.tma_poll_limit = g_tma_poll_limit;
  clear_stale();
  cudaError_t e;
  switch (dtype) {
    case SW_F32: e = sw::step_f32(p, st(s)); break;
    case SW_F64: e = sw::step_f64(p, st(s)); break;
    case SW_F16_SHIFT: e = sw::step_f16s(p, st(s)); break;
    default: e = sw::step_bf16s(p, st(s)); break;
  }
  if (e == cudaErrorNotSupported) return SW_ERR_UNSUPPORTED;   // e.g. no tensor-map encoder in the driver
  return cuda_status(e);
}
}  // namespace

int sw_step(const sw_geom *g, int dtype, const void *f_in, void *f_out, const uint8_t *flag, const uint8_t *tiles,
            const float *uin, double nu0, double cs, int32_t x_sponge, double nu_sponge, int64_t *force, int64_t t,
            sw_stream s) {
  return step_impl(g, dtype, f_in, f_out, flag, tiles, uin, nu0, cs, x_sponge, nu_sponge, force, t, nullptr,
                   dtype_ok(dtype) ? g_step_cfg[dtype] : 0, nullptr, s);
}

int sw_step_accum(const sw_geom *g, int dtype, const void *f_in, void *f_out, const uint8_t *flag,
                  const uint8_t *tiles, const float *uin, double nu0, double cs, int32_t x_sponge, double nu_sponge,
                  int64_t *force, int64_t t, double *acc, sw_stream s) {
  if (!acc) return SW_ERR_BAD_ARG;
  return step_impl(g, dtype, f_in, f_out, flag, tiles, uin, nu0, cs, x_sponge, nu_sponge, force, t, acc,
                   dtype_ok(dtype) ? g_step_cfg_acc[dtype] : 0, nullptr, s);
}

int sw_step_cfg(const sw_geom *g, int dtype, const void *f_in, void *f_out, const uint8_t *flag, const uint8_t *tiles,
                const float *uin, double nu0, double cs, int32_t x_sponge, double nu_sponge, int64_t *force,
                int64_t t, double *acc, int cfg, sw_stream s) {
  if (cfg < 0) return SW_ERR_BAD_ARG;
  return step_impl(g, dtype, f_in, f_out, flag, tiles, uin, nu0, cs, x_sponge, nu_sponge, force, t, acc, cfg,
                   nullptr, s);
}

int sw_step_checked(const sw_geom *g, int dtype, const void *f_in, void *f_out, const uint8_t *flag,
                    const uint8_t *tiles, const float *uin, double nu0, double cs, int32_t x_sponge,
                    double nu_sponge, int64_t *force, int64_t t, double *acc, int cfg, uint32_t *status,
                    sw_stream s) {
  if (cfg < -1) return SW_ERR_BAD_ARG;
  return step_impl(g, dtype, f_in, f_out, flag, tiles, uin, nu0, cs, x_sponge, nu_sponge, force, t, acc, cfg,
                   status, s);
}

int sw_status_error(uint32_t word) {
  if (word & SW_STATUS_TIMEOUT) return SW_ERR_TIMEOUT;
  if (word & SW_STATUS_NONFINITE) return SW_ERR_NONFINITE;
  return SW_OK;
}

// whether 16-bit AA steps stage their sources by TMA (sw_debug_aa_tma)
int g_aa_tma = 1;

int32_t sw_debug_aa_tma(int32_t on) {
  const int32_t old = g_aa_tma;
  if (on >= 0) g_aa_tma = on != 0;
  return old;
}

int32_t sw_debug_tma_poll_limit(int32_t polls) {
  const int32_t old = g_tma_poll_limit;
  if (polls >= 0) g_tma_poll_limit = polls;
  return old;
}

int sw_step_config_count(void) { return sw::kStepConfigs; }

int64_t sw_tma_timeouts(void) {
  const unsigned a = sw::tma_timeouts_f16s(), b = sw::tma_timeouts_bf16s();
  if (a == ~0u || b == ~0u) return -1;
  return (int64_t)a + (int64_t)b;
}

int sw_set_step_config(int dtype, int cfg) {
  if (!dtype_ok(dtype) || cfg < 0 || cfg >= sw::kStepConfigs) return SW_ERR_BAD_ARG;
  if (!sw::step_config_valid(dtype, cfg)) return SW_ERR_UNSUPPORTED;
  g_step_cfg[dtype] = cfg;
  return SW_OK;
}

int sw_get_step_config(int dtype) { return dtype_ok(dtype) ? g_step_cfg[dtype] : -1; }

int sw_set_step_config_accum(int dtype, int cfg) {
  if (!dtype_ok(dtype) || cfg < 0 || cfg >= sw::kStepConfigs) return SW_ERR_BAD_ARG;
  if (!sw::step_config_valid(dtype, cfg)) return SW_ERR_UNSUPPORTED;
  g_step_cfg_acc[dtype] = cfg;
  return SW_OK;
}

int sw_get_step_config_accum(int dtype) { return dtype_ok(dtype) ? g_step_cfg_acc[dtype] : -1; }

int sw_macro(const sw_geom *g, int dtype, const void *f, const uint8_t *flag, float *u, sw_stream s) {
  if (!geom_ok(g) || !dtype_ok(dtype) || !f || !flag || !u) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_macro(to_geom(g), dtype, f, flag, u, nullptr, st(s)));
}

int sw_accum(const sw_geom *g, const float *u, double *acc, sw_stream s) {
  if (!geom_ok(g) || !u || !acc) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_accum(to_geom(g), u, acc, st(s)));
}

int sw_macro_accum(const sw_geom *g, int dtype, const void *f, const uint8_t *flag, float *u, double *acc,
                   sw_stream s) {
  if (!geom_ok(g) || !dtype_ok(dtype) || !f || !flag || !acc) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_macro(to_geom(g), dtype, f, flag, u, acc, st(s)));
}

// The table layout the Python host mirrors (stonewall/batch.py).
static_assert(sizeof(sw_batch_entry) == 160 && offsetof(sw_batch_entry, status) == 144 &&
                  offsetof(sw_batch_entry, ghost) == 152 && offsetof(sw_batch_entry, t0) == 128,
              "sw_batch_entry layout");
static_assert(sizeof(sw_batch_header) == 32 && offsetof(sw_batch_header, next_item) == 16, "sw_batch_header layout");

int sw_batch_prepare(sw_batch_entry *entries, int32_t n, int dtype, int cfg, sw_batch_header *hdr) {
  if (!entries || n <= 0 || !hdr || !dtype_ok(dtype)) return SW_ERR_BAD_ARG;
  if (cfg < 0 || cfg >= sw::kStepConfigs) return SW_ERR_BAD_ARG;
  if (!sw::batch_config_valid(dtype, cfg)) return SW_ERR_UNSUPPORTED;
  int wy = 0;
  bool pair = false;
  if (!sw::config_shape(cfg, &wy, &pair)) return SW_ERR_UNSUPPORTED;
  long long item0 = 0;
  for (int i = 0; i < n; ++i) {
    sw_batch_entry &e = entries[i];
    if (e.ghost) return SW_ERR_UNSUPPORTED;                          // AA members: graph mode only
    if (!geom_ok(&e.geom) || !e.f[0] || !e.f[1] || e.f[0] == e.f[1] || !aligned16(e.f[0]) || !aligned16(e.f[1]))
      return SW_ERR_BAD_ARG;
    if (!e.flag || !e.tiles || !e.uin || e.cur0 < 0 || e.cur0 > 1 || e.t0 < 0) return SW_ERR_BAD_ARG;
    if (e.acc && e.acc_every <= 0) return SW_ERR_BAD_ARG;
    if (e.geom.nz > 65535) return SW_ERR_BAD_ARG;
    e.items = sw::batch_items(e.geom.nx, e.geom.ny, e.geom.nz, pair, wy);
    e.item0 = item0;
    item0 += e.items;
  }
  hdr->n = n;
  hdr->reserved = 0;
  hdr->total_items = item0;
  hdr->next_item = 0;
  hdr->done_blocks = 0;
  hdr->reserved2 = 0;
  return SW_OK;
}

int sw_batch_setup(int dtype, int cfg) {
  if (!dtype_ok(dtype) || cfg < 0 || cfg >= sw::kStepConfigs) return SW_ERR_BAD_ARG;
  if (!sw::batch_config_valid(dtype, cfg)) return SW_ERR_UNSUPPORTED;
  cudaError_t e;
  switch (dtype) {
    case SW_F32: e = sw::batch_f32(nullptr, nullptr, cfg, -1, nullptr); break;
    case SW_F64: e = sw::batch_f64(nullptr, nullptr, cfg, -1, nullptr); break;
    case SW_F16_SHIFT: e = sw::batch_f16s(nullptr, nullptr, cfg, -1, nullptr); break;
    default: e = sw::batch_bf16s(nullptr, nullptr, cfg, -1, nullptr); break;
  }
  return cuda_status(e);
}

int sw_batch_step(const sw_batch_header *hdr_dev, const sw_batch_entry *table_dev, int dtype, int cfg, int32_t k,
                  sw_stream s) {
  if (!hdr_dev || !table_dev || !dtype_ok(dtype) || k < 0) return SW_ERR_BAD_ARG;
  if (cfg < 0 || cfg >= sw::kStepConfigs) return SW_ERR_BAD_ARG;
  if (!sw::batch_config_valid(dtype, cfg)) return SW_ERR_UNSUPPORTED;
  clear_stale();
  cudaError_t e;
  switch (dtype) {
    case SW_F32: e = sw::batch_f32(hdr_dev, table_dev, cfg, k, st(s)); break;
    case SW_F64: e = sw::batch_f64(hdr_dev, table_dev, cfg, k, st(s)); break;
    case SW_F16_SHIFT: e = sw::batch_f16s(hdr_dev, table_dev, cfg, k, st(s)); break;
    default: e = sw::batch_bf16s(hdr_dev, table_dev, cfg, k, st(s)); break;
  }
  return cuda_status(e);
}

int64_t sw_aa_ghost_elems(const sw_geom *g) {
  return geom_ok(g) ? (int64_t)sw::kGhostPops * g->ny * g->nz : -1;
}

int sw_step_aa(const sw_geom *g, int dtype, void *f, int32_t odd, const uint8_t *flag, const uint8_t *tiles,
               const float *uin, double nu0, double cs, int32_t x_sponge, double nu_sponge, int64_t *force,
               int64_t t, double *acc, void *ghost, uint32_t *status, sw_stream s) {
  if (!geom_ok(g) || !dtype_ok(dtype) || !f || !flag || !tiles || !uin || !ghost || !aligned16(f) || t < 0)
    return SW_ERR_BAD_ARG;
  if (odd != 0 && odd != 1) return SW_ERR_BAD_ARG;
  if (status && ((uintptr_t)status & 3u)) return SW_ERR_BAD_ARG;
  sw::StepParams p;
  p.fin = f;
  p.fout = f;
  p.flag = flag;
  p.tiles = tiles;
  p.uin = uin;
  p.g = to_geom(g);
  fill_physics(p, g, nu0, cs, x_sponge, nu_sponge);
  p.force = force ? reinterpret_cast<long long *>(force) + (size_t)t * 2 * g->nz : nullptr;
  p.acc = acc;
  p.status = status;
  p.cfg = 0;
  p.tma_poll_limit = g_tma_poll_limit;
  sw::AAParams a{ghost, ghost, g_aa_tma};
  clear_stale();
  cudaError_t e;
  switch (dtype) {
    case SW_F32: e = sw::aa_f32(p, a, odd != 0, st(s)); break;
    case SW_F64: e = sw::aa_f64(p, a, odd != 0, st(s)); break;
    case SW_F16_SHIFT: e = sw::aa_f16s(p, a, odd != 0, st(s)); break;
    default: e = sw::aa_bf16s(p, a, odd != 0, st(s)); break;
  }
  return cuda_status(e);
}

int sw_force_to_f64(const int64_t *force, double *out, int64_t n, sw_stream s) {
  if (n < 0 || (n > 0 && (!force || !out))) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_force_to_f64(reinterpret_cast<const long long *>(force), out, n, st(s)));
}

int sw_coefficients(const int64_t *force, int64_t n_steps, int32_t nz, double UH, double H, int32_t ny, double *coef,
                    sw_stream s) {
  if (n_steps < 0 || nz <= 0 || ny <= 0 || !(UH > 0.0) || !(H > 0.0)) return SW_ERR_BAD_ARG;
  if (n_steps > 0 && (!force || !coef || ((uintptr_t)force & 15u))) return SW_ERR_BAD_ARG;
  const double qref = 0.5 * (UH * UH);
  const double qa = qref * (H * (double)ny);
  clear_stale();
  return cuda_status(sw::aux_coefficients(reinterpret_cast<const long long *>(force), n_steps, nz, qa, H, coef, st(s)));
}

int sw_coef_stats(const double *coef, int64_t n_steps, int64_t n_spin, double *stats, sw_stream s) {
  if (n_steps < 0 || n_spin < 0 || !stats || (n_steps > 0 && !coef)) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_coef_stats(coef, n_steps, n_spin, stats, st(s)));
}

// The box of the recirculation count (export3d.py:177-179 on the every-2nd-cell
// field): i from X0 / 2 to min(ceil(nx / 2), (X0 + 10 H) / 2), every j, k below
// min(ceil(nz / 2), H); false when it is empty or has fewer than two levels.
static bool recirc_box(const sw_geom *g, int32_t H, int32_t X0, int &i0, int &I, int &J, int &K) {
  if (!geom_ok(g) || H <= 0 || X0 < 0) return false;
  const long long nxd = (g->nx + 1) / 2, nzd = (g->nz + 1) / 2;
  const long long i1 = std::min(nxd, ((long long)X0 + 10ll * H) / 2);
  i0 = X0 / 2;
  I = (int)(i1 - i0);
  J = (g->ny + 1) / 2;
  K = (int)std::min(nzd, (long long)(2ll * H) / 2);
  return I > 0 && J > 0 && K >= 2;
}

int64_t sw_recirc_scratch_bytes(const sw_geom *g, int32_t H, int32_t X0) {
  int i0, I, J, K;
  if (!recirc_box(g, H, X0, i0, I, J, K)) return SW_ERR_BAD_ARG;
  return 2ll * I * J * K * (int64_t)sizeof(float);
}

int sw_recirc_count(const sw_geom *g, const double *acc, int64_t n_acc, const uint8_t *flag, int32_t H, int32_t X0,
                    double UH, void *scratch, int64_t scratch_bytes, int64_t *count, sw_stream s) {
  int i0, I, J, K;
  if (!recirc_box(g, H, X0, i0, I, J, K) || !acc || !flag || !scratch || !count || n_acc < 0 || !(UH > 0.0))
    return SW_ERR_BAD_ARG;
  if (scratch_bytes < 2ll * I * J * K * (int64_t)sizeof(float) || (reinterpret_cast<uintptr_t>(scratch) & 3u) ||
      (reinterpret_cast<uintptr_t>(count) & 7u))
    return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_recirc_count(to_geom(g), i0, I, J, K, acc, n_acc, flag, (float)UH,
                                          static_cast<float *>(scratch), reinterpret_cast<long long *>(count),
                                          st(s)));
}

int sw_slice_xz(const sw_geom *g, const float *u, int32_t y0, float *out, sw_stream s) {
  if (!geom_ok(g) || !u || !out || y0 < 0 || y0 >= g->ny) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_slice_xz(to_geom(g), u, y0, out, st(s)));
}

int sw_slice_xy(const sw_geom *g, const float *u, int32_t z0, float *out, sw_stream s) {
  if (!geom_ok(g) || !u || !out || z0 < 0 || z0 >= g->nz) return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_slice_xy(to_geom(g), u, z0, out, st(s)));
}

int sw_qcoarse(const sw_geom *g, const float *u, const uint8_t *flag, int32_t x0, int32_t ds, int32_t di,
               int32_t dj, int32_t dk, float *out, sw_stream s) {
  if (!geom_ok(g) || !u || !flag || !out || x0 < 0 || ds <= 0 || di < 0 || dj < 0 || dk < 0) return SW_ERR_BAD_ARG;
  // every cell a block visits, and its +-1 neighbours in x and z, lies inside the grid
  if ((long long)x0 + (long long)di * ds > g->nx || (long long)dj * ds > g->ny || (long long)dk * ds > g->nz)
    return SW_ERR_BAD_ARG;
  clear_stale();
  return cuda_status(sw::aux_qcoarse(to_geom(g), u, flag, x0, ds, di, dj, dk, out, st(s)));
}

}  // extern "C"
