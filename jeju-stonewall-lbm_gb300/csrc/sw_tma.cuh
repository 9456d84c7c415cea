// sw_tma.cuh -- the 16-bit step with its pull sources staged in shared memory by TMA.
//
// Included by sw_step.cuh after the cell code it reuses (collide2, Pack16,
// the link masks of the checked path, warp_force_add).  Same cells, same arithmetic, same results as
// the two-cells-per-thread kernel (k_step_pair); what changes is how the 19
// pulled values reach the registers.  k_step_pair loads every population row
// with 32-bit loads and moves the x-shifted ones between lanes (shuffles plus
// per-lane edge loads), which costs more issue slots than the collision
// itself; here one thread per block describes, per population, the whole
// source tile of the block -- an 80-cell x WY-row box of one population plane
// at level z - c_z (the mirrored plane at the top), x from x0 - 8 -- to the
// tensor-memory accelerator, which copies it into shared memory and signals an
// mbarrier.  Warps then read their two cells' sources from the box row at the
// shifted offset (two aligned 32-bit shared loads and a byte permute for
// c_x = +-1, one load otherwise).
//
// Boxes start on 16-byte boundaries (x0 - 8 is a multiple of 8 halves); a box
// reaching outside the lattice reads zeros there: x < 0 only feeds the inlet
// cell (which does not pull), x >= nx only the outlet copy (handled by the
// same per-lane selects as k_step_pair), z < 0 only links from the ground
// below the bottom level (segments there take the checked path, which puts the
// bounce-back values in their place).  The periodic y wrap is not a box: the
// warp whose source row is -1 or ny reads a one-row box of row ny - 1 or 0
// loaded beside the stage.
//
// A block runs ITEMS consecutive y row-groups of one 64-cell x segment pair at
// one level, with NSTAGE stages in flight.  When ITEMS > NSTAGE the stages form a
// ring released by a block barrier per item; otherwise every item is issued at
// the start and the warps run without barriers.  Every wait on an mbarrier is
// bounded; on time-out the block records the event in g_tma_timeouts and the
// lattice's status word, waits (bounded) for its copies in flight and leaves.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>

namespace sw {

template <int ITEMS_, int NSTAGE_, int MINB_> struct TmaCfg {
  static constexpr int WY = 4;
  static constexpr int THREADS = 32 * WY;
  static constexpr int ITEMS = ITEMS_;
  static constexpr int NSTAGE = NSTAGE_;
  static constexpr int MINB = MINB_;
};

constexpr int kTmaBoxX = 80;                                 // halves per box row: 8 + 64 + 8
constexpr int kTmaRowBytes = kTmaBoxX * 2;                   // 160
constexpr int kTmaBoxBytes = kTmaRowBytes * 4;               // one population, WY = 4 rows: 640 (5 x 128)
constexpr int kTmaWrapBytes = 256;                           // one-row box (160 B) in a 128-aligned slot
constexpr int kTmaWrapSlots = 10;                            // the populations with c_y != 0
constexpr int kTmaStageBytes = Q * kTmaBoxBytes + kTmaWrapSlots * kTmaWrapBytes;
// accumulating steps also stage the float64 sums of the item: 64 cells x 4 rows x 4 sums
constexpr int kTmaAccBytes = 64 * 4 * 4 * 8;
template <bool ACC> constexpr int tma_stage_bytes() { return kTmaStageBytes + (ACC ? kTmaAccBytes : 0); }

// wrap slot of a population with c_y != 0 (3, 4, 7, 8, 9, 10, 15, 16, 17, 18)
__host__ __device__ constexpr int wrap_slot(int i) {
  return i == 3 ? 0 : i == 4 ? 1 : i == 7 ? 2 : i == 8 ? 3 : i == 9 ? 4 : i == 10 ? 5 : i == 15 ? 6 : i == 16 ? 7
       : i == 17 ? 8 : i == 18 ? 9 : -1;
}

// blocks that gave up waiting (must stay 0); one counter per translation unit
static __device__ unsigned int g_tma_timeouts;

// Reads and clears this translation unit's time-out counter (host).
static inline unsigned int tma_timeouts_take() {
  unsigned int v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_tma_timeouts, sizeof(v)) != cudaSuccess) return ~0u;
  if (v != 0 && cudaMemcpyToSymbol(g_tma_timeouts, &zero, sizeof(zero)) != cudaSuccess) return ~0u;
  return v;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded wait: `polls` polls with back-off (the default 2^14: a copy lands in
// microseconds, this gives up after milliseconds), then false.
constexpr int kTmaPolls = 1 << 14;
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int polls = kTmaPolls) {
  for (int k = 0; k < polls; ++k) {
    if (mbar_try_wait(bar, parity)) return true;
    if (k > 64) __nanosleep(64);
  }
  return false;
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}


// Issue the copies of item (x0, y0, z) into stage `st`, arriving on `bar` (one
// thread); with ACC also the item's float64 sums (map_acc) behind the boxes.
template <bool ACC>
__device__ __forceinline__ void tma_issue(const CUtensorMap *map, const CUtensorMap *map1, const CUtensorMap *map_acc,
                                          const Geom &g, int x0, int y0, int z, uint32_t st, uint32_t bar) {
  const bool top = z == g.nz - 1;
  const bool wrap_lo = y0 == 0;                  // source row -1 of the first warp (c_y = +1)
  const bool wrap_hi = y0 + 4 >= g.ny;           // source row ny of the warp at y = ny - 1 (c_y = -1)
  uint32_t bytes = Q * kTmaBoxBytes + (ACC ? kTmaAccBytes : 0);
  if (wrap_lo) bytes += 5 * kTmaRowBytes;
  if (wrap_hi) bytes += 5 * kTmaRowBytes;
  mbar_expect_tx(bar, bytes);
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ey = CY(i), ez = CZ(i);
    const int pop = (ez == -1 && top) ? MIRZ(i) : i;
    const int zl = (ez == -1 && top) ? z : z - ez;
    tma_load_4d(st + i * kTmaBoxBytes, map, x0 - 8, y0 - ey, zl, pop, bar);
    if constexpr (ey == 1) {
      if (wrap_lo) tma_load_4d(st + Q * kTmaBoxBytes + wrap_slot(i) * kTmaWrapBytes, map1, x0 - 8, g.ny - 1, zl, pop, bar);
    } else if constexpr (ey == -1) {
      if (wrap_hi) tma_load_4d(st + Q * kTmaBoxBytes + wrap_slot(i) * kTmaWrapBytes, map1, x0 - 8, 0, zl, pop, bar);
    }
  });
  if constexpr (ACC) tma_load_4d(st + kTmaStageBytes, map_acc, x0, y0, z, 0, bar);
}

// The pair-kernel two-cell step with the sources read from the staged boxes (st: the stage).
// INTERIOR: the warp's row is neither the inlet segment pair nor the last one
// (every lane's cells and right neighbour exist) nor a periodic edge row in y,
// so no lane needs the inlet, outlet or wrap selects (decided per warp and item).
// CHECKED: as step_pair_fast's (link masks and bounce-back pairs from
// pair_links_prefetch; the boxes read zeros below z = 0).
template <int DT, bool ACC, bool INTERIOR, bool CHECKED = false>
__device__ __forceinline__ void tma_pair_fast(const StepParams &p, const uint8_t *st, int x0, int y, int z, int w,
                                              int lane, const uint32_t (*sm)[2] = nullptr,
                                              const uint32_t (*wm)[2] = nullptr, const uint32_t (*bnc)[Q] = nullptr,
                                              float *fxw = nullptr, float *fzw = nullptr, int *hit = nullptr) {
  using PK = Pack16<DT>;
  const Geom &g = p.g;
  const bool live = INTERIOR || x0 < g.nx;
  const bool has_b = INTERIOR || x0 + 1 < g.nx;
  const bool has_r = INTERIOR || x0 + 2 < g.nx;
  const bool inlet = !INTERIOR && x0 == 0;
  const int c0 = (z * g.ny + y) * g.pitch + x0;
  const int c = live ? chk(p, c0) : c0;                             // a lane past the row end uses no offset
  const int lane_word = 4 + lane;                                     // 32-bit word of elements 8 + 2 lane, + 1
  f2 v[Q];
  static_for<0, Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int ex = CX(i), ey = CY(i);
    const uint8_t *rowp = st + i * kTmaBoxBytes + w * kTmaRowBytes;
    if constexpr (ey == 1 && !INTERIOR) {
      if (y == 0) rowp = st + Q * kTmaBoxBytes + wrap_slot(i) * kTmaWrapBytes;
    } else if constexpr (ey == -1 && !INTERIOR) {
      if (y == g.ny - 1) rowp = st + Q * kTmaBoxBytes + wrap_slot(i) * kTmaWrapBytes;
    }
    const uint32_t *row = reinterpret_cast<const uint32_t *>(rowp);
    const uint32_t own = row[lane_word];                               // cells x0, x0 + 1
    if constexpr (ex == 0) {
      v[i].v = PK::both(own);
    } else if constexpr (ex == 1) {                                   // sources x0 - 1, x0
      const uint32_t left = row[lane_word - 1];
      v[i] = F2(PK::hi(left), PK::lo(own));
    } else {                                                          // sources x0 + 1, x0 + 2 (outlet: x)
      const uint32_t right = row[lane_word + 1];
      const float2 o = PK::both(own);
      v[i] = F2(has_b ? o.y : o.x, has_r ? PK::lo(right) : o.y);
    }
    if constexpr (CHECKED && i > 0) pair_link<DT, i>(v[i], *sm, *wm, (*bnc)[i], *fxw, *fzw, *hit);
  });
  if (!live) return;
  // accumulating steps: the pair's old sums from the staged box [4 sums][4 rows][64 cells], read where added
  const double2 *acc_box = reinterpret_cast<const double2 *>(st + kTmaStageBytes) + w * 32 + lane;
  if constexpr (CHECKED) {
    const uint32_t keep = pair_solid_cells(v, *sm);
    if (keep == 0u) return;
    pair_collide_store<DT, ACC, true>(p, v, x0, c, z, inlet, has_b, [&](int k) { return acc_box[k * 4 * 32]; }, keep);
  } else {
    pair_collide_store<DT, ACC>(p, v, x0, c, z, inlet, has_b, [&](int k) { return acc_box[k * 4 * 32]; });
  }
}

// Grid: (ceil(pitch / 64), ceil(ceil(ny / 4) / ITEMS), nz); block = 4 warps, warp w = row y0 + w.
template <int DT, bool ACC, typename Cfg>
__global__ void __launch_bounds__(Cfg::THREADS, Cfg::MINB)
    k_step_tma(const __grid_constant__ CUtensorMap map, const __grid_constant__ CUtensorMap map1,
               const __grid_constant__ CUtensorMap map_acc, const __grid_constant__ StepParams p) {
  constexpr int kStage = tma_stage_bytes<ACC>();
  // With no more items than stages every item's copies are issued at the start
  // and no stage is reused: warps then run their items without block barriers.
  constexpr bool kRing = Cfg::ITEMS > Cfg::NSTAGE;
  static_assert(2 * Cfg::ITEMS <= 32, "one lane per tile byte of the block's items");
  extern __shared__ __align__(128) uint8_t smem_raw[];
  __shared__ __align__(8) unsigned long long bars[Cfg::NSTAGE];
  uint8_t *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);   // 128-byte aligned boxes
  const Geom &g = p.g;
  const int w = threadIdx.y, lane = threadIdx.x;
  const bool leader = w == 0 && lane == 0;
  const int bx = blockIdx.x, z = blockIdx.z;
  const int x0s = 2 * SEG * bx;                                        // first cell of the segment pair
  const int nyb = (g.ny + 3) / 4;
  const int yb0 = blockIdx.y * Cfg::ITEMS;
  const int n_items = min(Cfg::ITEMS, nyb - yb0);
  const uint32_t base = smem_u32(smem);
  if (leader) {
    for (int s = 0; s < Cfg::NSTAGE; ++s) mbar_init(smem_u32(&bars[s]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    for (int j = 0; j < Cfg::NSTAGE && j < n_items; ++j)
      tma_issue<ACC>(&map, &map1, &map_acc, g, x0s, (yb0 + j) * 4, z, base + j * kStage, smem_u32(&bars[j]));
  }
  // The segment classes of this warp's rows in all its items, fetched once up
  // front (lane j: segment 2 bx of item j, lane ITEMS + j: segment 2 bx + 1),
  // so their latency overlaps the first copies instead of following each wait.
  uint32_t kinds = TILE_ALL_SOLID;
  {
    const int j = lane < Cfg::ITEMS ? lane : lane - Cfg::ITEMS;
    const int sx = 2 * bx + (lane < Cfg::ITEMS ? 0 : 1);
    const int y = (yb0 + j) * 4 + w;
    if (lane < 2 * Cfg::ITEMS && j < n_items && y < g.ny && sx < g.nseg_x)
      kinds = __ldg(p.tiles + ((size_t)(z * g.ny + y) * g.nseg_x + sx));
  }
  __syncthreads();
  const int polls = p.tma_poll_limit;
  bool ok = true;
  int j = 0;
  for (; j < n_items; ++j) {
    const int s = j % Cfg::NSTAGE;
    const uint32_t st = base + s * kStage;
    const int y = (yb0 + j) * 4 + w;
    const uint8_t ka = (uint8_t)__shfl_sync(0xffffffffu, kinds, j);
    const uint8_t kb = (uint8_t)__shfl_sync(0xffffffffu, kinds, Cfg::ITEMS + j);
    const int x0 = x0s + 2 * lane;
    const bool work = y < g.ny && !(ka & kb & TILE_ALL_SOLID);
    const bool checked = work && ((ka | kb) & TILE_CHECK);          // uniform across the warp
    uint32_t sm[2], wm[2], bnc[Q];
    if (checked) pair_links_prefetch<DT>(p, x0, y, z, sm, wm, bnc);
    if (ok) ok = mbar_wait(smem_u32(&bars[s]), (uint32_t)((j / Cfg::NSTAGE) & 1), polls);
    if (ok && work) {
      if (!checked) {
        if (x0s > 0 && x0s + 2 * SEG < g.nx && y > 0 && y < g.ny - 1)     // uniform across the warp
          tma_pair_fast<DT, ACC, true>(p, smem + s * kStage, x0, y, z, w, lane);
        else
          tma_pair_fast<DT, ACC, false>(p, smem + s * kStage, x0, y, z, w, lane);
      } else {                                                        // next to stones / the ground
        float fxw = 0.0f, fzw = 0.0f;
        int hit = 0;
        tma_pair_fast<DT, ACC, false, true>(p, smem + s * kStage, x0, y, z, w, lane, &sm, &wm, &bnc, &fxw, &fzw, &hit);
        if (((ka | kb) & TILE_FORCE) && p.force != nullptr) warp_force_add<float>(p, z, lane, fxw, fzw, hit);
      }
    }
    if constexpr (kRing) {                                            // stages are reused: the block
      ok = __syncthreads_and(ok);                                     // barrier frees stage s
      if (!ok) break;
      if (leader && j + Cfg::NSTAGE < n_items)
        tma_issue<ACC>(&map, &map1, &map_acc, g, x0s, (yb0 + j + Cfg::NSTAGE) * 4, z, st, smem_u32(&bars[s]));
    }
  }
  if constexpr (!kRing) ok = __syncthreads_and(ok);                 // every item was issued at the start
  if (!ok && leader) {                                                // some wait gave up: let every copy
    atomicAdd(&g_tma_timeouts, 1u);                                   // in flight land (normal bound)
    note_status(p, SW_STATUS_TIMEOUT);
    if constexpr (kRing) {                                            // item j failed: j .. j+NSTAGE-1 issued
      for (int k = j; k < n_items && k < j + Cfg::NSTAGE; ++k)
        (void)mbar_wait(smem_u32(&bars[k % Cfg::NSTAGE]), (uint32_t)((k / Cfg::NSTAGE) & 1));
    } else {
      for (int k = 0; k < n_items; ++k) (void)mbar_wait(smem_u32(&bars[k]), 0u);
    }
  }
}

// ---------------------------------------------------------------- host side
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

// The lattice f (16-bit elements, [19][nz][ny][pitch]) as a 4-D tensor, boxes of 80 x rows x 1 x 1.
inline bool encode_lattice_map(CUtensorMap *m, const void *f, const Geom &g, int rows) {
  auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dim[4] = {(cuuint64_t)g.pitch, (cuuint64_t)g.ny, (cuuint64_t)g.nz, (cuuint64_t)Q};
  const cuuint64_t stride[3] = {(cuuint64_t)g.pitch * 2, (cuuint64_t)g.pitch * g.ny * 2, (cuuint64_t)g.plane * 2};
  const cuuint32_t box[4] = {(cuuint32_t)kTmaBoxX, (cuuint32_t)rows, 1, 1};
  const cuuint32_t estride[4] = {1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT16, 4, const_cast<void *>(f), dim, stride, box, estride,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The float64 sums acc ([4][nz][ny][pitch]) as a 4-D tensor, boxes of 64 cells x 4 rows x 1 level x 4 sums.
inline bool encode_acc_map(CUtensorMap *m, const double *acc, const Geom &g) {
  auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dim[4] = {(cuuint64_t)g.pitch, (cuuint64_t)g.ny, (cuuint64_t)g.nz, 4};
  const cuuint64_t stride[3] = {(cuuint64_t)g.pitch * 8, (cuuint64_t)g.pitch * g.ny * 8, (cuuint64_t)g.plane * 8};
  const cuuint32_t box[4] = {64, 4, 1, 4};
  const cuuint32_t estride[4] = {1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, const_cast<double *>(acc), dim, stride, box, estride,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int DT, bool ACC, typename Cfg>
cudaError_t launch_tma(const StepParams &p, cudaStream_t s) {
  CUtensorMap map, map1, map_acc;
  if (!encode_lattice_map(&map, p.fin, p.g, 4) || !encode_lattice_map(&map1, p.fin, p.g, 1))
    return cudaErrorNotSupported;
  if (ACC) {
    if (!encode_acc_map(&map_acc, p.acc, p.g)) return cudaErrorNotSupported;
  } else {
    map_acc = map;                                                   // not read
  }
  constexpr int smem = Cfg::NSTAGE * tma_stage_bytes<ACC>() + 128;   // + alignment slack
  static_assert(smem <= 227 * 1024, "stages exceed the shared memory of a block");
  if constexpr (smem > 48 * 1024) {                                  // beyond the default: opt in, once
    static bool opted = false;
    if (!opted) {
      const cudaError_t e = cudaFuncSetAttribute(k_step_tma<DT, ACC, Cfg>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 smem);
      if (e != cudaSuccess) return e;
      opted = true;
    }
  }
  const int nyb = (p.g.ny + 3) / 4;
  const dim3 grid((unsigned)((p.g.nseg_x + 1) / 2), (unsigned)((nyb + Cfg::ITEMS - 1) / Cfg::ITEMS), (unsigned)p.g.nz);
  k_step_tma<DT, ACC, Cfg><<<grid, dim3(32, 4), smem, s>>>(map, map1, map_acc, p);
  return cudaGetLastError();
}

}  // namespace sw
