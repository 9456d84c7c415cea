// sw_noalloc.cu -- sw_step_noalloc: the fused step for callers that cannot allocate device memory.
//
// sw_step needs a caller-provided `tiles` buffer (one byte per 32-cell row
// segment, built by sw_build_tiles).  Some callers cannot provide it: a host
// that only receives device pointers from an allocator it does not own, or a
// loop that must not call cudaMalloc / cudaFree because they can synchronise
// the device.  This entry point keeps that buffer in a file-scope device array
// of fixed size instead, so the caller passes only the inputs and outputs.
//
// The array (SW_NOALLOC_MAX_SEGMENTS bytes) exists on every GPU that loads the
// library's device code (at the first call there under lazy module loading),
// for the life of the process, or until cudaDeviceReset destroys the context:
// the address cached below is not re-queried after a reset.  Every call on a device shares it and
// rewrites the part its grid uses before reading it, so calls on one device
// that overlap in time on the GPU (different streams, or different host
// threads) race with each other and must be serialised by the caller.
#include <mutex>

#include "sw_aux.cuh"
#include "sw_step.cuh"

namespace {

constexpr int kMaxDevices = 64;

// Row-segment classes of the grid being stepped (see TILE_* in sw_common.cuh).
static __device__ __align__(256) uint8_t g_noalloc_tiles[SW_NOALLOC_MAX_SEGMENTS];

std::mutex g_mu;
uint8_t *g_tiles_ptr[kMaxDevices] = {};

// The array's device address on the current device.  In host code the symbol
// g_noalloc_tiles is only a host-side stand-in, so the address is looked up
// once per device with that device current, and cached.
int tiles_on_current_device(uint8_t **out, int *cuda_err) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) { *cuda_err = (int)e; return SW_ERR_CUDA; }
  if (dev < 0 || dev >= kMaxDevices) return SW_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_tiles_ptr[dev] == nullptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_tiles);
    if (e != cudaSuccess || p == nullptr) { *cuda_err = (int)e; return SW_ERR_CUDA; }
    g_tiles_ptr[dev] = static_cast<uint8_t *>(p);
  }
  *out = g_tiles_ptr[dev];
  return SW_OK;
}

}  // namespace

extern "C" int sw_step_noalloc(const sw_geom *g, int dtype, const void *f_in, void *f_out, const uint8_t *flag,
                               const float *uin, double nu0, double cs, int32_t x_sponge, double nu_sponge,
                               int64_t *force, int64_t t, sw_stream s) {
  if (!g || g->nx <= 0 || g->ny <= 0 || g->nz <= 0 || g->pitch != sw::round_up(g->nx, sw::SEG)) return SW_ERR_BAD_ARG;
  const long long nseg = (long long)g->nz * g->ny * (g->pitch / sw::SEG);
  if (nseg > (long long)SW_NOALLOC_MAX_SEGMENTS) return SW_ERR_TOO_LARGE;
  if (!f_in || !f_out || !flag || !uin || f_in == f_out || t < 0) return SW_ERR_BAD_ARG;
  if ((((uintptr_t)f_in) & 15u) || (((uintptr_t)f_out) & 15u)) return SW_ERR_BAD_ARG;
  if (dtype != SW_F32 && dtype != SW_F64 && dtype != SW_F16_SHIFT && dtype != SW_BF16_SHIFT) return SW_ERR_BAD_ARG;
  uint8_t *tiles = nullptr;
  int cuda_err = 0;
  const int st = tiles_on_current_device(&tiles, &cuda_err);
  if (st == SW_ERR_CUDA) return sw::note_cuda_error(cuda_err);  // visible through sw_last_cuda_error()
  if (st != SW_OK) return st;
  // classify this grid's segments into the shared array, then step with it
  const int rc = sw_build_tiles(g, flag, tiles, s);
  if (rc != SW_OK) return rc;
  return sw_step(g, dtype, f_in, f_out, flag, tiles, uin, nu0, cs, x_sponge, nu_sponge, force, t, s);
}
