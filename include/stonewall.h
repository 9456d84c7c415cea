/* stonewall.h -- C ABI of the GB300 (sm_103a) D3Q19 wall-wind solver.
 *
 * Drop-in for the Warp kernels of stonewall3d/lbm3d.py (Cat-yejun/jeju-stonewall-lbm).
 * Each entry point below replaces one `wp.launch(k_*, dim=..., inputs=[...])`
 * call of the reference; the citation beside it names the kernel and the call
 * site.  As in the reference, the caller owns every device buffer (the driver
 * allocates them, lbm3d.py:292-313) and the entry points only launch work on
 * the given stream; they return an SW_* status instead of raising.
 *
 * Device layout (x fastest; the reference's arrays are z fastest):
 *   f      [19][nz][ny][pitch] of the storage type (sw_dtype_size)
 *   flag   [nz][ny][pitch]     uint8, 0 fluid / 1 stone / 2 ground (lbm3d.py:30)
 *   tiles  [nz][ny][pitch/32]  uint8, derived from flag by sw_build_tiles
 *   u      [4][nz][ny][pitch]  float: rho, ux, uy, uz (lbm3d.py:158-182)
 *   acc    [4][nz][ny][pitch]  double time sums of u
 *   force  [n_t][nz][2]        int64, fixed point with 2^-40 units (SW_FORCE_SCALE):
 *                              x and z momentum-exchange force per height level
 *                              and step, as force[t][z][0..1] in lbm3d.py:99-101
 * pitch = nx rounded up to a multiple of 32 (sw_geom_make).  Cells with
 * x >= nx are padding: the step never reads them, and the 16-bit steps may
 * write don't-care values there (they store cells in aligned pairs).
 *
 * The D3Q19 tables that the reference passes as arrays (cx, cy, cz, w, opp,
 * mirz; lbm3d.py:20-28, 297-300) are compiled in, in the reference's order.
 * Nothing here allocates device memory or synchronises the device unless its
 * comment says so.
 */
#ifndef STONEWALL_H
#define STONEWALL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
enum {
  SW_OK = 0,
  SW_ERR_BAD_ARG = 1,     /* null pointer, bad extent, unknown dtype, inconsistent geometry */
  SW_ERR_OOM = 2,         /* reserved for callers that allocate (the library never does) */
  SW_ERR_NONFINITE = 3,   /* a diverged state (sw_status_error of SW_STATUS_NONFINITE) */
  SW_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
  SW_ERR_CUDA = 5,        /* a CUDA call failed; sw_last_cuda_error() has the code */
  SW_ERR_UNSUPPORTED = 6, /* valid request this build does not implement */
  SW_ERR_TOO_LARGE = 7    /* grid exceeds the fixed scratch of sw_step_noalloc */
};

/* Bits of a lattice's device status word (uint32_t in device memory).  The
 * checked step entry points (sw_step_checked, sw_step_aa, batch entries with a
 * status pointer) OR them in; the caller zeroes the word and reads it back
 * when it wants to know, e.g. once per run of steps.  The reference detects
 * divergence on the host, from the macro field every 5000 steps
 * (lbm3d.py:386-391); here every fluid cell of every step is covered. */
enum {
  SW_STATUS_NONFINITE = 1, /* some fluid cell had a non-finite density after pulling its populations */
  SW_STATUS_TIMEOUT = 2,   /* a block of the TMA-staged step gave up waiting for its copies: cells unwritten */
  SW_STATUS_BOUNDS = 4     /* bounds-checked build only (libstonewall_check.so): a computed element offset
                              fell outside its population plane; the access went to element 0 instead */
};

/* storage type of the distributions */
enum {
  SW_F32 = 0,        /* float32, as the reference (lbm3d.py:293-294) */
  SW_F64 = 1,        /* float64 storage and arithmetic (the precision oracle run) */
  SW_F16_SHIFT = 2,  /* binary16 holding f_i - w_i, float32 collision */
  SW_BF16_SHIFT = 3  /* bfloat16 holding f_i - w_i, float32 collision */
};

/* cell flags (lbm3d.py:30) */
enum { SW_FLUID = 0, SW_WALL = 1, SW_GROUND = 2 };

/* noise distributions of sw_init */
enum { SW_NOISE_UNIFORM = 0, SW_NOISE_GAUSSIAN = 1 };

#define SW_FORCE_SCALE 1099511627776.0 /* 2^40 fixed-point units per force unit */

typedef void *sw_stream; /* a cudaStream_t; NULL is the legacy default stream */

typedef struct sw_geom {
  int32_t nx, ny, nz; /* cells along x (wind), y (span, periodic), z (height) */
  int32_t pitch;      /* padded x extent of the device layout */
} sw_geom;

/* ---------------------------------------------------------------- library */
const char *sw_version(void);
const char *sw_status_string(int status);
/* cudaError_t of the last CUDA failure reported as SW_ERR_CUDA by this thread. */
int sw_last_cuda_error(void);

/* ---------------------------------------------------------------- geometry and sizes
 * Replaces the shape arithmetic of lbm3d.py:270, 283, 293-303. */
int sw_geom_make(int32_t nx, int32_t ny, int32_t nz, sw_geom *out);
int64_t sw_cells_padded(const sw_geom *g);   /* nz * ny * pitch */
int64_t sw_lattice_elems(const sw_geom *g);  /* 19 * nz * ny * pitch */
int64_t sw_tile_count(const sw_geom *g);     /* nz * ny * pitch / 32 */
size_t sw_dtype_size(int dtype);             /* bytes per stored population, 0 if unknown */

/* ---------------------------------------------------------------- layout conversion
 * The reference's host<->device copies (wp.array(flag) lbm3d.py:295, f0.assign
 * lbm3d.py:332, f0.numpy() lbm3d.py:345) use its z-fastest layout; these
 * device-to-device transposes convert to and from it.  ref_dtype is SW_F32 or
 * SW_F64 (the type of the reference-layout array). */
int sw_pack_flag(const sw_geom *g, const uint8_t *flag_ref, uint8_t *flag, sw_stream s);
int sw_pack_f(const sw_geom *g, int dtype, int ref_dtype, const void *f_ref, void *f, sw_stream s);
int sw_unpack_f(const sw_geom *g, int dtype, int ref_dtype, const void *f, void *f_ref, sw_stream s);
/* u / acc in the device layout -> [4][nx][ny][nz] float (u) or double (acc). */
int sw_unpack_u(const sw_geom *g, const float *u, float *u_ref, sw_stream s);
int sw_unpack_acc(const sw_geom *g, const double *acc, double *acc_ref, sw_stream s);

/* Classify every 32-cell row segment (fluid-only fast path, stone contact,
 * all solid).  Must be rerun whenever flag changes.  Has no reference
 * counterpart: it replaces the per-cell neighbour flag tests of
 * lbm3d.py:88-95 where they cannot fire. */
int sw_build_tiles(const sw_geom *g, const uint8_t *flag, uint8_t *tiles, sw_stream s);

/* ---------------------------------------------------------------- kernels */
/* k_init, lbm3d.py:39-54 (launched at lbm3d.py:340): equilibrium at rho = 1
 * with the inlet speed uin[z] perturbed per fluid cell; solids at rest.
 * noise_kind SW_NOISE_UNIFORM follows the reference (u0*(1+noise*(2r-1)), ...),
 * SW_NOISE_GAUSSIAN draws standard normals instead.  The random stream is a
 * PCG hash of (seed, cell) in the form rand_init(seed, (x*7919+y)*7907+z). */
int sw_init(const sw_geom *g, int dtype, void *f, const uint8_t *flag, const float *uin, float noise,
            int32_t seed, int32_t noise_kind, sw_stream s);

/* k_step, lbm3d.py:57-155 (launched at lbm3d.py:359-361): one fused timestep
 * f_in -> f_out: pull streaming (periodic y, outlet copy, free-slip top),
 * half-way bounce-back, momentum-exchange force into force[t][z][0..1] (added
 * atomically: the row must hold zero, or the partial sum to add to), regularized
 * BGK with the Smagorinsky time scale and the outlet sponge.  Non-fluid cells of
 * f_out are not written, as in the reference.  force may be NULL (no force). */
int sw_step(const sw_geom *g, int dtype, const void *f_in, void *f_out, const uint8_t *flag,
            const uint8_t *tiles, const float *uin, double nu0, double cs, int32_t x_sponge,
            double nu_sponge, int64_t *force, int64_t t, sw_stream s);

/* k_step followed by k_macro + k_accum of the new state (lbm3d.py:359-369 on an
 * accumulation step) in one pass: as sw_step, and (rho, ux, uy, uz) of every
 * fluid cell is added to acc (float64, [4][nz][ny][pitch]).  Non-fluid cells of
 * acc are not touched (their sums are n_acc * (1, 0, 0, 0) by definition). */
int sw_step_accum(const sw_geom *g, int dtype, const void *f_in, void *f_out, const uint8_t *flag,
                  const uint8_t *tiles, const float *uin, double nu0, double cs, int32_t x_sponge,
                  double nu_sponge, int64_t *force, int64_t t, double *acc, sw_stream s);

/* Launch configurations of the step (block shape and register budget, see
 * csrc/sw_step.cuh): 0-3 one cell per thread, 4-7 two cells per thread and
 * 8-10 two cells per thread with TMA-staged sources (csrc/sw_tma.cuh), the
 * last two groups for 16-bit storage only.  sw_step and sw_step_accum use the
 * configuration set for their storage type (process-wide, default 0);
 * stonewall/autotune.py times every configuration with sw_step_cfg and sets
 * the fastest.  No reference counterpart (Warp chooses its own launch shape). */
int sw_step_config_count(void);
/* Blocks of the TMA-staged configurations that gave up a bounded wait for
 * their copies since the last call (read and cleared; -1 if unreadable).  A
 * non-zero count means the steps they belonged to are not valid. */
int64_t sw_tma_timeouts(void);
int sw_set_step_config(int dtype, int cfg);
int sw_get_step_config(int dtype);
/* The same for sw_step_accum (accumulation steps move more data per cell and
 * may prefer another register budget). */
int sw_set_step_config_accum(int dtype, int cfg);
int sw_get_step_config_accum(int dtype);
/* sw_step (acc NULL) or sw_step_accum (acc non-NULL) with an explicit configuration. */
int sw_step_cfg(const sw_geom *g, int dtype, const void *f_in, void *f_out, const uint8_t *flag,
                const uint8_t *tiles, const float *uin, double nu0, double cs, int32_t x_sponge, double nu_sponge,
                int64_t *force, int64_t t, double *acc, int cfg, sw_stream s);
/* k_step with the failure checks of lbm3d.py:386-391 moved onto the device:
 * as sw_step_cfg, and every fluid cell whose pulled density is not finite, and
 * every TMA-staged block that gave up waiting, ORs SW_STATUS_NONFINITE /
 * SW_STATUS_TIMEOUT into *status (a device word the caller owns and clears;
 * NULL: no checks, as sw_step_cfg).  cfg -1 takes the configuration installed
 * for the storage type (sw_set_step_config, or ..._accum when acc is given). */
int sw_step_checked(const sw_geom *g, int dtype, const void *f_in, void *f_out, const uint8_t *flag,
                    const uint8_t *tiles, const float *uin, double nu0, double cs, int32_t x_sponge,
                    double nu_sponge, int64_t *force, int64_t t, double *acc, int cfg, uint32_t *status,
                    sw_stream s);
/* The error a status word read back from the device stands for: SW_OK (0),
 * SW_ERR_TIMEOUT (checked first: the cells of a timed-out block were not
 * written) or SW_ERR_NONFINITE. */
int sw_status_error(uint32_t word);
/* Test hook, no reference counterpart: the polls a TMA-staged block makes on
 * a stage's copies before it gives up (default 16384, microseconds apart).
 * With 0 every block of the next TMA-staged launches gives up at once, lets
 * the copies it issued land (that wait keeps its normal bound) and reports
 * SW_STATUS_TIMEOUT, which is how the time-out path is tested without a
 * device fault.  Returns the previous value; a negative argument only reads. */
int32_t sw_debug_tma_poll_limit(int32_t polls);

/* Test hook, no reference counterpart: 1 (the default) lets 16-bit AA steps
 * stage their sources by TMA, 0 runs the same steps with plain loads (the form
 * used when tensor maps cannot be made), so both stay tested.  Returns the
 * previous value; a negative argument only reads. */
int32_t sw_debug_aa_tma(int32_t on);

/* AA pattern: the same step on ONE lattice, updated in place (half the
 * memory of f_in + f_out).  No reference counterpart: the reference always
 * steps f0 into f1 (lbm3d.py:293-294, 362); this replaces that pair of
 * buffers with one.  Steps alternate odd / even, starting with odd.  Before an
 * odd step and after an even one the lattice holds the state in the usual
 * layout (plane k holds f_k, as after sw_init or sw_pack_f), so exports,
 * macros and checkpoints are taken after even steps; after an odd step the
 * lattice is in transit and can only be advanced by the even step.  ghost:
 * sw_aa_ghost_elems(g) stored values of scratch, written and read by the odd
 * step.  acc may be NULL (otherwise as sw_step_accum).  States, forces and
 * sums after every even step equal the two-lattice step's bit for bit.
 * status: as sw_step_checked (NULL: no checks). */
int64_t sw_aa_ghost_elems(const sw_geom *g);
int sw_step_aa(const sw_geom *g, int dtype, void *f, int32_t odd, const uint8_t *flag, const uint8_t *tiles,
               const float *uin, double nu0, double cs, int32_t x_sponge, double nu_sponge, int64_t *force,
               int64_t t, double *acc, void *ghost, uint32_t *status, sw_stream s);

/* k_macro, lbm3d.py:158-182 (lbm3d.py:367, 387): u = (rho, ux, uy, uz); solids -> (1, 0, 0, 0). */
int sw_macro(const sw_geom *g, int dtype, const void *f, const uint8_t *flag, float *u, sw_stream s);
/* k_accum, lbm3d.py:185-188 (lbm3d.py:369): acc += u, in double. */
int sw_accum(const sw_geom *g, const float *u, double *acc, sw_stream s);
/* k_macro followed by k_accum (lbm3d.py:367-369) in one pass; u may be NULL. */
int sw_macro_accum(const sw_geom *g, int dtype, const void *f, const uint8_t *flag, float *u, double *acc,
                   sw_stream s);

/* ---------------------------------------------------------------- batches
 * Many independent lattices (walls of different sizes) advanced by one
 * persistent launch per step.  No reference counterpart: the reference runs
 * one wall per process (run_all.sh:11-17 runs the cases one after another).
 * The caller keeps a table of entries in device memory; sw_batch_prepare
 * (host only) validates it and fills the work-item fields and the header.
 * The kernel reads table and header at run time, so a captured CUDA graph of
 * sw_batch_step launches serves any composition that fits: rewrite t0 /
 * steps_left / cur0 (and entries and header) between replays. */
typedef struct sw_batch_entry {
  sw_geom geom;          /* extents and pitch (sw_geom_make) */
  int64_t item0;         /* first work item of this lattice   (set by sw_batch_prepare) */
  int64_t items;         /* work items per step of this lattice (set by sw_batch_prepare) */
  void *f[2];            /* the two population buffers (device layout, the batch's storage type) */
  const uint8_t *flag;   /* device layout */
  const uint8_t *tiles;  /* sw_build_tiles */
  const float *uin;      /* [nz] */
  int64_t *force;        /* [n_total][nz][2] fixed point, row t0 + k is written; or NULL */
  double *acc;           /* [4][nz][ny][pitch] float64 sums, or NULL */
  double nu0, cs, nu_sponge;
  int32_t x_sponge;
  int32_t n_spin;        /* accumulate on steps t >= n_spin with (t - n_spin) % acc_every == 0 */
  int32_t acc_every;
  int32_t cur0;          /* buffer (0 or 1) holding the state at k = 0 */
  int64_t t0;            /* step index of launch k = 0 */
  int64_t steps_left;    /* launches with k >= steps_left leave the lattice untouched */
  uint32_t *status;      /* the lattice's device status word (SW_STATUS_*), or NULL: no checks */
  void *ghost;           /* NULL: the two-lattice pattern.  Otherwise an in-place AA member (graph mode
                          * only): f[0] == f[1] is its one lattice, ghost its sw_aa_ghost_elems buffer,
                          * and cur0 = 0 when its next step is odd, 1 when even */
} sw_batch_entry;

typedef struct sw_batch_header {
  int32_t n;             /* entries in the table */
  int32_t reserved;
  int64_t total_items;   /* sum of items (set by sw_batch_prepare) */
  /* work counters of a launch: zero before it (sw_batch_prepare sets them), used by the
   * kernel's blocks to take items in order, and zero again when the launch ends */
  uint64_t next_item;
  uint32_t done_blocks;
  uint32_t reserved2;
} sw_batch_header;

/* Host only: check entries[0..n) for storage type dtype and configuration cfg
 * and fill item0 / items and *hdr. */
int sw_batch_prepare(sw_batch_entry *entries, int32_t n, int dtype, int cfg, sw_batch_header *hdr);
/* Queries the device once for the persistent grid of (dtype, cfg); sw_batch_step
 * does the same on first use, so call this first when the launches are to be
 * captured in a CUDA graph. */
int sw_batch_setup(int dtype, int cfg);
/* Launch k of a batch step: every entry with k < steps_left advances from
 * buffer (cur0 + k) & 1 to the other one, as sw_step / sw_step_accum would. */
int sw_batch_step(const sw_batch_header *hdr_dev, const sw_batch_entry *table_dev, int dtype, int cfg, int32_t k,
                  sw_stream s);

/* The same batch as one CUDA graph of single-lattice launches: per entry a
 * chain of min(k_steps, steps_left) sw_step_checked launches (the storage
 * type's configurations from sw_set_step_config[_accum]; accumulating on the
 * entry's accumulation steps; checks into the entry's status word), the chains
 * parallel branches between a fork and a join, so lattices run concurrently
 * under the hardware block scheduler.  entries is a HOST table (item0 and
 * items are not used; no sw_batch_prepare needed), at most
 * SW_BATCH_MAX_ENTRIES long.  Each call captures the launches, updates the
 * handle's executable graph (instantiating anew only when the number of
 * lattices or launches changed) and launches it on s; the handle's two
 * executable graphs alternate, so a call may wait for the launch of the call
 * before last to finish.  Entries with a ghost buffer are in-place AA
 * members: their chains alternate sw_step_aa odd and even steps (odd first
 * when cur0 = 0).  One handle per device and host thread.  No reference
 * counterpart (see sw_batch_step). */
#define SW_BATCH_MAX_ENTRIES 256
typedef struct sw_batch_graph sw_batch_graph;
int sw_batch_graph_create(sw_batch_graph **out);
int sw_batch_graph_destroy(sw_batch_graph *g);
int sw_batch_graph_run(sw_batch_graph *g, const sw_batch_entry *entries, int32_t n, int dtype, int32_t k_steps,
                       sw_stream s);
/* step kernels in the graphs this handle has launched */
int64_t sw_batch_graph_launches(const sw_batch_graph *g);

/* force rows (fixed point) -> double, n values. */
int sw_force_to_f64(const int64_t *force, double *out, int64_t n, sw_stream s);

/* ---------------------------------------------------------------- wall loads on the device
 * The coefficient series of lbm3d.py:396-407 from the fixed-point force rows
 * force[n_steps][nz][2] (16-byte aligned): coef[0][t] = Cd = Fx / (q A),
 * coef[1][t] = Cl = Fz / (q A), coef[2][t] = Cm = M / (q A H), with Fx, Fz the
 * sums over the levels, M = sum_z F_x(z) (z - 1/2), q A = U_H^2 / 2 * H ny;
 * coef is [3][n_steps] doubles. */
int sw_coefficients(const int64_t *force, int64_t n_steps, int32_t nz, double UH, double H, int32_t ny, double *coef,
                    sw_stream s);
/* postprocess.py:65-82 on the device: over the steps t >= n_spin of a coefficient
 * series from sw_coefficients, stats[0..5] = mean Cd, max Cd, std Cd (about the
 * mean), mean Cm, max Cm, mean Cl (6 doubles, device memory; NaN with no step
 * left).  A solve's statistics then need 48 bytes downloaded, not its force series. */
int sw_coef_stats(const double *coef, int64_t n_steps, int64_t n_spin, double *stats, sw_stream s);

/* Recirculation area behind the wall (export3d.py:169-184; replaces the host
 * computation on the every-2nd-cell mean field of lbm3d.py:412).  On the cells
 * (2 i, 2 j, 2 k) with X0/2 <= i < min(ceil(nx/2), (X0 + 10 H)/2), every j,
 * k < min(ceil(nz/2), H): u_x of the time mean acc[1] / max(n_acc, 1) (acc: the
 * float64 sums [4][nz][ny][pitch] of sw_macro_accum / sw_step), 0.05 at
 * non-fluid cells, over U_H; level k = 0 copies level 1; one separable 3-point
 * box blur with edge clamping; *count (device int64) = the cells below zero.
 * The area in H^2 per unit wall length is count * 8 / (H^2 ny).  scratch:
 * sw_recirc_scratch_bytes() bytes of device memory (4-byte aligned);
 * sw_recirc_scratch_bytes returns SW_ERR_BAD_ARG when the box is empty or has
 * fewer than two levels. */
int64_t sw_recirc_scratch_bytes(const sw_geom *g, int32_t H, int32_t X0);
int sw_recirc_count(const sw_geom *g, const double *acc, int64_t n_acc, const uint8_t *flag, int32_t H, int32_t X0,
                    double UH, void *scratch, int64_t scratch_bytes, int64_t *count, sw_stream s);

/* ---------------------------------------------------------------- wall masks on the device
 * The per-cell work of the two stone-wall generators of the Python package
 * (stonewall/geometry.py); their random draws stay on the host, so a seed gives
 * the host generator's mask bit for bit.
 *
 * Ellipsoid packer (the BASELINE wall; no reference counterpart): candidate
 * stones drawn on the host in the generator's order, each with its cell range
 * x in [x0, x1), y in [y0, y1) (periodic, unwrapped), k in [k0, k1).  Cell
 * (x, y, k) is inside when, with a = (x + 1/2, y + 1/2, k - 1/2) - centre,
 * t_j = ((a_0 rot[j] + a_1 rot[3 + j]) + a_2 rot[6 + j]) / semi[j] and
 * (t_0^2 + t_1^2) + t_2^2 <= 1 (float64, in that order, no contraction). */
typedef struct sw_ellipsoid {
  double centre[3];
  double semi[3];
  double rot[9];                 /* rotation, row-major */
  int32_t x0, x1, y0, y1, k0, k1;
} sw_ellipsoid;
/* Bytes of the bitset of the wall box x in [X0, X0 + T), y in [0, ny),
 * k in [1, z_hi): bit ((x - X0) ny + y) (z_hi - 1) + (k - 1); -1 on bad sizes. */
int64_t sw_pack_box_bytes(int32_t T, int32_t ny, int32_t z_hi);
/* The packer's loop over cand[0..n) (device memory) in order, one block on s:
 * while state[0] (solid cells so far) < target - 1/2, count the cells the
 * candidate adds; accept it unless it adds none or state[0] + n_new > target
 * + n_new / 2; set its cells in box_bits (device, in/out).  state[1] receives
 * the candidates consumed.  Boxes above 200 KiB of bits: SW_ERR_TOO_LARGE. */
int sw_pack_ellipsoids(const sw_ellipsoid *cand, int32_t n, int32_t X0, int32_t T, int32_t ny, int32_t z_hi,
                       double target, uint32_t *box_bits, int64_t *state, sw_stream s);
/* Course-wall rasteriser, geometry.py:68-84: stone s (device array) marks cell
 * (x, y mod ny, k) of mask[nx][ny][nz] (device, uint8, reference layout; ORed
 * in) when (|x + 1/2 - xc| / a)^p + (|y + 1/2 - yc| / b)^p + (|k - 1/2 - zc| /
 * c)^p <= 1.  Cells whose sum is within 1e-12 of 1, where this GPU's pow and
 * the host's may round apart, are not decided: they are listed in amb
 * (device, 1 + 4 cap ints: count, then (stone, x, y, k) per cell) for the
 * host to decide with its own arithmetic. */
typedef struct sw_stone {
  double xc, yc, zc, a, b, c, p;
  int32_t x0, x1, y0, y1, k0, k1;
} sw_stone;
int sw_voxelize_stones(const sw_stone *stones, int32_t n, int32_t nx, int32_t ny, int32_t nz, uint8_t *mask,
                       int32_t *amb, int32_t cap, sw_stream s);

/* ---------------------------------------------------------------- viewer payload
 * From the macro field u of sw_macro (device layout [4][nz][ny][pitch]).
 * k_slice_xz, lbm3d.py:191-194 (lbm3d.py:372): out[4][nx][nz] = u at y = y0.
 * k_slice_xy, lbm3d.py:197-200 (lbm3d.py:373): out[4][nx][ny] = u at z = z0.
 * k_qcoarse, lbm3d.py:203-238 (lbm3d.py:316): out[di][dj][dk] = max(0, max
 * over the ds^3 block at (x0 + i ds, j ds, k ds) of the Q-criterion), Q taken
 * as 0 next to non-fluid cells and outside 1 <= x < nx-1, 1 <= z < nz-1.
 * Float32, evaluated in the reference's order without contraction. */
int sw_slice_xz(const sw_geom *g, const float *u, int32_t y0, float *out, sw_stream s);
int sw_slice_xy(const sw_geom *g, const float *u, int32_t z0, float *out, sw_stream s);
int sw_qcoarse(const sw_geom *g, const float *u, const uint8_t *flag, int32_t x0, int32_t ds, int32_t di,
               int32_t dj, int32_t dk, float *out, sw_stream s);

/* ---------------------------------------------------------------- step without allocation
 * No counterpart in the reference: an addition for callers that cannot
 * allocate device memory -- a host that only receives device pointers from an
 * allocator it does not own, or a loop that must not call cudaMalloc/cudaFree
 * because they can synchronise the device.  Same arguments and results as
 * sw_step minus `tiles`: the row-segment classes live in a fixed device array
 * of SW_NOALLOC_MAX_SEGMENTS bytes inside the library (every GPU that loads the
 * library holds it until the process exits), rebuilt from `flag` on each call.
 *   - grids with more than SW_NOALLOC_MAX_SEGMENTS segments (nz*ny*pitch/32,
 *     about 134 M cells) are rejected with SW_ERR_TOO_LARGE;
 *   - the entry point calls no allocating routine.  The array itself comes
 *     into existence with the library's device code on that device: at the
 *     first call per device under CUDA's default lazy module loading (or when
 *     the library loads, with CUDA_MODULE_LOADING=EAGER);
 *   - the first call on a device looks up the array's device address (once per
 *     device, with that device current) and caches it: make that first call
 *     before any stream capture.  cudaDeviceReset destroys the array with the
 *     context; the cached address is then stale, so do not call this entry
 *     point on a device after resetting it;
 *   - all calls on a device share the array: calls that overlap on the GPU
 *     (other streams, other host threads) race and must be serialised. */
#define SW_NOALLOC_MAX_SEGMENTS (1 << 22)
int sw_step_noalloc(const sw_geom *g, int dtype, const void *f_in, void *f_out, const uint8_t *flag,
                    const float *uin, double nu0, double cs, int32_t x_sponge, double nu_sponge, int64_t *force,
                    int64_t t, sw_stream s);

#ifdef __cplusplus
}
#endif
#endif /* STONEWALL_H */
