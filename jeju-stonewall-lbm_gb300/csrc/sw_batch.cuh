// sw_batch.cuh -- many lattices, one persistent launch per step.
//
// The lattices of a batch are described by a table in device memory
// (sw_batch_entry, include/stonewall.h): geometry, the two ping-pong buffers,
// flags, segment classes, inlet, force series, float64 sums, physics, and the
// per-lattice step counter t0 and remaining steps.  A step of the batch is one
// launch of k_step_batch with a grid of (SMs x resident blocks) that walks all
// work items of all lattices (an item = one block's rows of one lattice), so
// lattices of any size share the GPU in one launch.  The kernel reads the
// table at run time: a CUDA graph of K launches (k = 0..K-1) captured once
// serves any batch composition -- the host rewrites the table (and the header
// with the count) between replays to admit, advance and retire lattices.
//
// Each lattice's cells are computed by the same cell code as the single-lattice
// step; force rows use integer atomics and the sums are owned per cell, so a
// lattice's results do not depend on what else is in the batch.
#pragma once
#include "sw_step.cuh"

namespace sw {

// Cell-code context of one batched lattice: population planes at pop * plane.
struct BatchCtx {
  Geom g;
  const uint8_t *flag;
  const uint8_t *tiles;
  const float *uin;
  double nu0, cs, nu_sponge, sponge_scale;
  float nu0f, c18f, sponge_scalef, nu_spongef;   // as StepParams (set_float_params)
  int x_sponge;
  long long *force;
  unsigned int *status;     // the lattice's status word, or nullptr
  const void *fin_pop[Q];   // plane bases, filled once per lattice
  void *fout_pop[Q];
  double *acc_pop[4];
  template <typename T> __device__ __forceinline__ const T *in(int pop) const {
    return static_cast<const T *>(fin_pop[pop]);
  }
  template <typename T> __device__ __forceinline__ T *out(int pop) const { return static_cast<T *>(fout_pop[pop]); }
  __device__ __forceinline__ double *accp(int k) const { return acc_pop[k]; }
};

// Work items per step of one lattice (host and device): an item is one block's
// WY rows (y) of one x segment (a 64-cell pair segment for the 16-bit kernel)
// at one level z; items of a lattice are numbered with x fastest, then y, z.
__host__ __device__ inline long long batch_items(int nx, int ny, int nz, bool pair, int wy) {
  const int nseg_x = (nx + SEG - 1) / SEG;
  const int nbx = pair ? (nseg_x + 1) / 2 : nseg_x;
  return (long long)nbx * ((ny + wy - 1) / wy) * nz;
}

// The accumulating variant of an item (one step in acc_every of a lattice in
// its averaging phase) is a separate function: inlined next to the plain
// variant its extra live values (the four float64 sums) would set the
// register allocation of the whole loop and make the plain path spill.
template <int DT, bool PAIR>
__device__ __noinline__ void batch_item_acc(const BatchCtx &sc, int bx, int y, int z, int lane) {
  if constexpr (PAIR) step_pair_segment<DT, true>(sc, bx, y, z, lane);
  else step_segment<DT, true>(sc, bx, y, z, lane);
}

// Persistent blocks take the items in order from a work counter in the header,
// kGrab at a time: the items in flight at any moment form one compact window
// (a few levels of one lattice), so the z - 1 and z + 1 planes a level pulls
// from are still in L2 when their neighbours need them, and items that cost
// more (the checked path next to stones and the ground) go to whichever block
// is free, as the hardware block scheduler would hand them out.  (A static
// grid-stride assignment let blocks drift apart and re-read neighbour planes
// from DRAM.)  The block that finishes last zeroes the counters for the next
// launch.  A lattice has thousands of items, so consecutive items of a block
// mostly stay in one lattice and the block refills its context only when it
// crosses into another.  The context lives in shared memory (the single-lattice
// kernel reads the same values from the constant bank) and takes no registers
// across the item loop.
constexpr int kGrab = 2;
template <int DT, bool PAIR, typename Cfg>
__global__ void __launch_bounds__(Cfg::THREADS, Cfg::MINB)
    k_step_batch(const sw_batch_header *hdr, const sw_batch_entry *__restrict__ tab, int k) {
  __shared__ BatchCtx sc;
  __shared__ long long s_first, s_next, s_grab;
  __shared__ int s_run, s_acc, s_lat;
  sw_batch_header *hw = const_cast<sw_batch_header *>(hdr);       // the work counters
  const long long total = hdr->total_items;
  long long first = 0, next = 0;                                  // item range of the loaded lattice
  int nbx = 1, nyb = 1;
  const bool t0 = threadIdx.x == 0 && threadIdx.y == 0;
  for (;;) {
    if (t0)
      s_grab = (long long)atomicAdd(reinterpret_cast<unsigned long long *>(&hw->next_item), (unsigned long long)kGrab);
    __syncthreads();
    const long long grab = s_grab;
    __syncthreads();                                              // s_grab is rewritten by the next grab
    if (grab >= total) break;
    const long long grab_end = grab + kGrab < total ? grab + kGrab : total;
    for (long long item = grab; item < grab_end; ++item) {
      if (item >= next || item < first) {                         // uniform across the block
        __syncthreads();
        if (threadIdx.x == 0 && threadIdx.y == 0) {
          const int n = hdr->n;
          int lo = 0, hi = n - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tab[mid].item0 <= item) lo = mid;
            else hi = mid - 1;
          }
          const sw_batch_entry &e = tab[lo];
          s_lat = lo;
          s_first = e.item0;
          s_next = e.item0 + e.items;
          s_run = (long long)k < e.steps_left;
          sc.g.nx = e.geom.nx;
          sc.g.ny = e.geom.ny;
          sc.g.nz = e.geom.nz;
          sc.g.pitch = e.geom.pitch;
          sc.g.nseg_x = e.geom.pitch / SEG;
          sc.g.plane = (long long)e.geom.nz * e.geom.ny * e.geom.pitch;
          sc.flag = e.flag;
          sc.tiles = e.tiles;
          sc.uin = e.uin;
          sc.nu0 = e.nu0;
          sc.cs = e.cs;
          sc.nu_sponge = e.nu_sponge;
          sc.x_sponge = e.x_sponge;
          sc.sponge_scale = (e.geom.nx != e.x_sponge) ? 1.0 / (double)(e.geom.nx - e.x_sponge) : 0.0;
          sc.nu0f = (float)e.nu0;
          sc.c18f = smag_c18f((float)e.cs);
          sc.sponge_scalef = (float)sc.sponge_scale;
          sc.nu_spongef = (float)e.nu_sponge;
          sc.status = e.status;
          const long long t = e.t0 + k;
          sc.force = e.force ? reinterpret_cast<long long *>(e.force) + t * 2 * e.geom.nz : nullptr;
          s_acc = e.acc != nullptr && t >= e.n_spin && (t - e.n_spin) % e.acc_every == 0;
        }
        __syncthreads();
        {                                                           // plane bases, one per thread
          const sw_batch_entry &e = tab[s_lat];
          const int tid = threadIdx.y * 32 + threadIdx.x;
          const int cur = (e.cur0 + k) & 1;
          const size_t pb = (size_t)sc.g.plane * sizeof(typename Store<DT>::T);
          if (tid < Q) sc.fin_pop[tid] = static_cast<const char *>(e.f[cur]) + tid * pb;
          else if (tid < 2 * Q) sc.fout_pop[tid - Q] = static_cast<char *>(e.f[cur ^ 1]) + (tid - Q) * pb;
          else if (tid < 2 * Q + 4) sc.acc_pop[tid - 2 * Q] = e.acc ? e.acc + (size_t)(tid - 2 * Q) * sc.g.plane : nullptr;
        }
        __syncthreads();
        first = s_first;
        next = s_next;
        nbx = PAIR ? (sc.g.nseg_x + 1) / 2 : sc.g.nseg_x;
        nyb = (sc.g.ny + Cfg::WY - 1) / Cfg::WY;
      }
      const int local = (int)(item - first);
      const int bx = local % nbx;
      const int rest = local / nbx;
      const int yg = rest % nyb;
      const int z = rest / nyb;
      if (s_run) {
        const int y = yg * Cfg::WY + threadIdx.y;
        if (y < sc.g.ny) {
          if (s_acc) batch_item_acc<DT, PAIR>(sc, bx, y, z, threadIdx.x);
          else if constexpr (PAIR) step_pair_segment<DT, false>(sc, bx, y, z, threadIdx.x);
          else step_segment<DT, false>(sc, bx, y, z, threadIdx.x);
        }
      }
    }
  }
  if (t0) {                                                       // the last block out zeroes the counters
    __threadfence();
    if (atomicAdd(&hw->done_blocks, 1u) == gridDim.x - 1) {
      hw->next_item = 0;
      hw->done_blocks = 0;
      __threadfence();
    }
  }
}

template <int DT, bool PAIR, typename Cfg>
cudaError_t launch_batch_cfg(const sw_batch_header *hdr, const sw_batch_entry *tab, int k, cudaStream_t s) {
  static int grid = 0;                                             // SMs x resident blocks, per instantiation
  if (grid == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_batch<DT, PAIR, Cfg>, Cfg::THREADS, 0);
    if (e != cudaSuccess) return e;
    grid = sms * (per_sm > 0 ? per_sm : 1);
  }
  if (k < 0) return cudaSuccess;                                   // query only: grid size now cached
  k_step_batch<DT, PAIR, Cfg><<<grid, dim3(32, Cfg::WY), 0, s>>>(hdr, tab, k);
  return cudaGetLastError();
}

template <int DT>
cudaError_t launch_batch(const sw_batch_header *hdr, const sw_batch_entry *tab, int cfg, int k, cudaStream_t s) {
  switch (cfg) {
#define SW_CASE(ID, WY, MINB) \
  case ID: return launch_batch_cfg<DT, false, StepCfg<WY, MINB>>(hdr, tab, k, s);
    SW_STEP_CONFIGS(SW_CASE)
#undef SW_CASE
#define SW_CASE(ID, WY, MINB)                                                     \
  case ID:                                                                        \
    if constexpr (is16(DT)) return launch_batch_cfg<DT, true, StepCfg<WY, MINB>>(hdr, tab, k, s); \
    else return cudaErrorNotSupported;
    SW_PAIR_CONFIGS(SW_CASE)
#undef SW_CASE
    default:
      return cudaErrorInvalidValue;
  }
}

// (wy, pair) of a configuration, for sw_batch_prepare.
inline bool config_shape(int cfg, int *wy, bool *pair) {
  switch (cfg) {
#define SW_CASE(ID, WY, MINB) \
  case ID: *wy = WY; *pair = false; return true;
    SW_STEP_CONFIGS(SW_CASE)
#undef SW_CASE
#define SW_CASE(ID, WY, MINB) \
  case ID: *wy = WY; *pair = true; return true;
    SW_PAIR_CONFIGS(SW_CASE)
#undef SW_CASE
    default:
      return false;
  }
}

}  // namespace sw
