// sw_geometry.cu -- stone-wall masks on the GPU.
//
// Two mask producers of the host package (stonewall/geometry.py) have their
// per-cell work here; the random draws, and every decision that depends on
// their order, stay on the host, so a seed gives the same mask as the host
// generator.
//
//  * k_pack_ellipsoids -- the ellipsoid packer's rejection loop.  The host
//    draws the candidates (centre, semi-axes, rotation, cell range) in the
//    generator's order; one block walks them in that order over a bitset of
//    the wall box in shared memory: count the cells a candidate would add,
//    accept it under the packer's rule, set its cells, stop at the target.
//    The inside test is the host generator's expression, evaluated in the
//    same order without contraction (this file is built with --fmad=false),
//    so every decision is the host's.
//  * k_voxelize_stones -- the course wall's rasteriser (geometry.py:68-84):
//    one block per superellipsoid stone over its cell range.  The inside test
//    raises to a real power, which this GPU's pow and the host's libm may
//    round differently in the last bits; cells whose sum lies within 1e-12 of
//    the surface are listed instead of decided, and the host decides them with
//    its own expression.
#include "sw_aux.cuh"

namespace sw {

// ---------------------------------------------------------------- ellipsoid packer
// Box cell (x, y, k) of the wall box x in [X0, X0 + T), y in [0, ny), k in [1, z_hi):
// bit ((x - X0) * ny + y) * nzb + (k - 1) of the box bitset, nzb = z_hi - 1.
__device__ __forceinline__ bool ellipsoid_inside(const sw_ellipsoid &e, int x, int y, int k) {
  const double dx = ((double)x + 0.5) - e.centre[0];
  const double dy = ((double)y + 0.5) - e.centre[1];
  const double dz = ((double)k - 0.5) - e.centre[2];
  // body-frame coordinates d_j = sum_i a_i R[i][j], then sum_j (d_j / semi_j)^2
  const double t0 = ((dx * e.rot[0] + dy * e.rot[3]) + dz * e.rot[6]) / e.semi[0];
  const double t1 = ((dx * e.rot[1] + dy * e.rot[4]) + dz * e.rot[7]) / e.semi[1];
  const double t2 = ((dx * e.rot[2] + dy * e.rot[5]) + dz * e.rot[8]) / e.semi[2];
  return ((t0 * t0 + t1 * t1) + t2 * t2) <= 1.0;
}

constexpr int kPackThreads = 1024;

__global__ void __launch_bounds__(kPackThreads)
    k_pack_ellipsoids(const sw_ellipsoid *cand, int n, int X0, int T, int ny, int z_hi, double target,
                      uint32_t *box_bits, long long *state) {
  extern __shared__ uint32_t box[];
  __shared__ long long red[kPackThreads / 32];
  const int nzb = z_hi - 1;
  const long long cells = (long long)T * ny * nzb;
  const int words = (int)((cells + 31) / 32);
  for (int w = threadIdx.x; w < words; w += kPackThreads) box[w] = box_bits[w];
  long long solid = state[0];
  int used = 0;
  __syncthreads();
  for (int c = 0; c < n; ++c) {
    if (!((double)solid < target - 0.5)) break;                  // the loop condition, before each try
    used = c + 1;
    const sw_ellipsoid &e = cand[c];
    const int lx = e.x1 - e.x0, ly = e.y1 - e.y0, lk = e.k1 - e.k0;
    if (lx <= 0 || lk <= 0 || ly <= 0) continue;
    const long long m = (long long)lx * ly * lk;
    // pass 1: cells inside the candidate that are not solid yet
    long long fresh = 0;
    for (long long i = threadIdx.x; i < m; i += kPackThreads) {
      const int k = e.k0 + (int)(i % lk);
      const long long r = i / lk;
      const int yy = e.y0 + (int)(r % ly);
      const int x = e.x0 + (int)(r / ly);
      if (x < X0 || x >= X0 + T || k < 1 || k >= z_hi) continue;  // outside the box: not part of the wall
      if (!ellipsoid_inside(e, x, yy, k)) continue;
      const int y = ((yy % ny) + ny) % ny;
      const long long b = ((long long)(x - X0) * ny + y) * nzb + (k - 1);
      fresh += !((box[b >> 5] >> (b & 31)) & 1u);
    }
    for (int o = 16; o > 0; o >>= 1) fresh += __shfl_xor_sync(0xffffffffu, fresh, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = fresh;
    __syncthreads();
    long long n_new = 0;
    for (int w = 0; w < kPackThreads / 32; ++w) n_new += red[w];  // the same order in every thread
    __syncthreads();                                              // red is rewritten by the next candidate
    if (n_new == 0 || (double)(solid + n_new) > target + 0.5 * (double)n_new) continue;
    // pass 2: accept, set the candidate's cells
    for (long long i = threadIdx.x; i < m; i += kPackThreads) {
      const int k = e.k0 + (int)(i % lk);
      const long long r = i / lk;
      const int yy = e.y0 + (int)(r % ly);
      const int x = e.x0 + (int)(r / ly);
      if (x < X0 || x >= X0 + T || k < 1 || k >= z_hi) continue;
      if (!ellipsoid_inside(e, x, yy, k)) continue;
      const int y = ((yy % ny) + ny) % ny;
      const long long b = ((long long)(x - X0) * ny + y) * nzb + (k - 1);
      atomicOr(&box[b >> 5], 1u << (b & 31));
    }
    solid += n_new;
    __syncthreads();
  }
  for (int w = threadIdx.x; w < words; w += kPackThreads) box_bits[w] = box[w];
  if (threadIdx.x == 0) {
    state[0] = solid;
    state[1] = used;
  }
}

long long pack_box_bytes(int T, int ny, int z_hi) {
  const long long cells = (long long)T * ny * (z_hi - 1);
  return (cells + 31) / 32 * 4;
}

cudaError_t launch_pack_ellipsoids(const sw_ellipsoid *cand, int n, int X0, int T, int ny, int z_hi, double target,
                                   uint32_t *box_bits, long long *state, cudaStream_t s) {
  const long long bytes = pack_box_bytes(T, ny, z_hi);
  static bool opted = false;
  if (!opted) {
    const cudaError_t e = cudaFuncSetAttribute(k_pack_ellipsoids, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)kPackBoxBytesMax);
    if (e != cudaSuccess) return e;
    opted = true;
  }
  k_pack_ellipsoids<<<1, kPackThreads, (size_t)bytes, s>>>(cand, n, X0, T, ny, z_hi, target, box_bits, state);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- course-wall rasteriser
// geometry.py:68-84: cell (x, y, k) with centre (x + 1/2, y + 1/2, k - 1/2) is
// stone s when |dx / a|^p + |dy / b|^p + |dz / c|^p <= 1 (left to right sums).
constexpr double kSurfaceBand = 1e-12;

__global__ void k_voxelize_stones(const sw_stone *stones, int nx, int ny, int nz, uint8_t *mask, int *amb,
                                  int cap) {
  const sw_stone &st = stones[blockIdx.x];
  const int lx = st.x1 - st.x0, ly = st.y1 - st.y0, lk = st.k1 - st.k0;
  if (lx <= 0 || ly <= 0 || lk <= 0) return;
  const long long m = (long long)lx * ly * lk;
  for (long long i = threadIdx.x; i < m; i += blockDim.x) {
    const int k = st.k0 + (int)(i % lk);
    const long long r = i / lk;
    const int yy = st.y0 + (int)(r % ly);
    const int x = st.x0 + (int)(r / ly);
    if (x < 0 || x >= nx || k < 0 || k >= nz) continue;              // ranges come clamped from the host
    const double X = (double)x + 0.5, Y = (double)yy + 0.5, K = (double)k - 0.5;
    const double v = (pow(fabs(X - st.xc) / st.a, st.p) + pow(fabs(Y - st.yc) / st.b, st.p)) +
                     pow(fabs(K - st.zc) / st.c, st.p);
    const int y = ((yy % ny) + ny) % ny;
    if (v <= 1.0 - kSurfaceBand) {
      mask[((size_t)x * ny + y) * nz + k] = 1;                     // the same value from every writer
    } else if (v <= 1.0 + kSurfaceBand) {                          // too close to call: the host decides
      const int j = atomicAdd(amb, 1);
      if (j < cap) {
        int *o = amb + 1 + 4 * j;
        o[0] = (int)blockIdx.x;
        o[1] = x;
        o[2] = yy;
        o[3] = k;
      }
    }
  }
}

cudaError_t launch_voxelize_stones(const sw_stone *stones, int n, int nx, int ny, int nz, uint8_t *mask, int *amb,
                                   int cap, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_voxelize_stones<<<n, 256, 0, s>>>(stones, nx, ny, nz, mask, amb, cap);
  return cudaGetLastError();
}

}  // namespace sw

extern "C" {

int sw_pack_ellipsoids(const sw_ellipsoid *cand, int32_t n, int32_t X0, int32_t T, int32_t ny, int32_t z_hi,
                       double target, uint32_t *box_bits, int64_t *state, sw_stream s) {
  if (n < 0 || (n > 0 && !cand) || !box_bits || !state || X0 < 0 || T <= 0 || ny <= 0 || z_hi < 2)
    return SW_ERR_BAD_ARG;
  if (sw::pack_box_bytes(T, ny, z_hi) > sw::kPackBoxBytesMax) return SW_ERR_TOO_LARGE;
  (void)cudaGetLastError();                                         // report this launch's error only
  const cudaError_t e = sw::launch_pack_ellipsoids(cand, n, X0, T, ny, z_hi, target, box_bits,
                                                   reinterpret_cast<long long *>(state),
                                                   reinterpret_cast<cudaStream_t>(s));
  return e == cudaSuccess ? SW_OK : sw::note_cuda_error((int)e);
}

int64_t sw_pack_box_bytes(int32_t T, int32_t ny, int32_t z_hi) {
  if (T <= 0 || ny <= 0 || z_hi < 2) return -1;
  return sw::pack_box_bytes(T, ny, z_hi);
}

int sw_voxelize_stones(const sw_stone *stones, int32_t n, int32_t nx, int32_t ny, int32_t nz, uint8_t *mask,
                       int32_t *amb, int32_t cap, sw_stream s) {
  if (n < 0 || (n > 0 && !stones) || !mask || !amb || cap < 0 || nx <= 0 || ny <= 0 || nz <= 0) return SW_ERR_BAD_ARG;
  (void)cudaGetLastError();
  const cudaError_t e = sw::launch_voxelize_stones(stones, n, nx, ny, nz, mask, amb, cap,
                                                   reinterpret_cast<cudaStream_t>(s));
  return e == cudaSuccess ? SW_OK : sw::note_cuda_error((int)e);
}

}  // extern "C"
