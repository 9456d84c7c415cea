// sw_aux.cuh -- host-side launchers of the kernels in sw_aux.cu and sw_step_*.cu.
#pragma once
#include "sw_common.cuh"

namespace sw {

struct StepParams;

cudaError_t aux_init(const Geom &g, int dtype, void *f, const uint8_t *flag, const float *uin, float noise, int seed,
                     int kind, cudaStream_t s);
cudaError_t aux_macro(const Geom &g, int dtype, const void *f, const uint8_t *flag, float *u, double *acc,
                      cudaStream_t s);
cudaError_t aux_accum(const Geom &g, const float *u, double *acc, cudaStream_t s);
cudaError_t aux_pack_f(const Geom &g, int dtype, int ref_dtype, const void *ref, void *f, cudaStream_t s);
cudaError_t aux_unpack_f(const Geom &g, int dtype, int ref_dtype, const void *f, void *ref, cudaStream_t s);
cudaError_t aux_pack_flag(const Geom &g, const uint8_t *ref, uint8_t *flag, cudaStream_t s);
cudaError_t aux_unpack_u(const Geom &g, const float *u, float *ref, cudaStream_t s);
cudaError_t aux_unpack_acc(const Geom &g, const double *acc, double *ref, cudaStream_t s);
cudaError_t aux_build_tiles(const Geom &g, const uint8_t *flag, uint8_t *tiles, cudaStream_t s);
cudaError_t aux_force_to_f64(const long long *fx, double *out, long long n, cudaStream_t s);
cudaError_t aux_coefficients(const long long *force, long long n_steps, int nz, double qa, double H, double *coef,
                             cudaStream_t s);
cudaError_t aux_coef_stats(const double *coef, long long n_steps, long long n_spin, double *stats, cudaStream_t s);
cudaError_t aux_recirc_count(const Geom &g, int i0, int I, int J, int K, const double *acc, long long n_acc,
                             const uint8_t *flag, float uh, float *scratch, long long *count, cudaStream_t s);
cudaError_t aux_slice_xz(const Geom &g, const float *u, int y0, float *out, cudaStream_t s);
cudaError_t aux_slice_xy(const Geom &g, const float *u, int z0, float *out, cudaStream_t s);
cudaError_t aux_qcoarse(const Geom &g, const float *u, const uint8_t *flag, int x0, int ds, int di, int dj, int dk,
                        float *out, cudaStream_t s);

int note_cuda_error(int cuda_error);  // sw_capi.cu
// largest wall box (bytes of its bitset) the ellipsoid packer holds in shared memory
constexpr long long kPackBoxBytesMax = 200 * 1024;
unsigned int tma_timeouts_f16s();      // read and clear the TMA wait time-outs of sw_step_f16s.cu
unsigned int tma_timeouts_bf16s();

// one launcher per storage type, each in its own translation unit (sw_step_<dtype>.cu)
cudaError_t step_f32(const StepParams &p, cudaStream_t s);
cudaError_t step_f64(const StepParams &p, cudaStream_t s);
cudaError_t step_f16s(const StepParams &p, cudaStream_t s);
cudaError_t step_bf16s(const StepParams &p, cudaStream_t s);
struct AAParams;
cudaError_t aa_f32(const StepParams &p, const AAParams &a, bool odd, cudaStream_t s);
cudaError_t aa_f64(const StepParams &p, const AAParams &a, bool odd, cudaStream_t s);
cudaError_t aa_f16s(const StepParams &p, const AAParams &a, bool odd, cudaStream_t s);
cudaError_t aa_bf16s(const StepParams &p, const AAParams &a, bool odd, cudaStream_t s);
cudaError_t batch_f32(const sw_batch_header *h, const sw_batch_entry *t, int cfg, int k, cudaStream_t s);
cudaError_t batch_f64(const sw_batch_header *h, const sw_batch_entry *t, int cfg, int k, cudaStream_t s);
cudaError_t batch_f16s(const sw_batch_header *h, const sw_batch_entry *t, int cfg, int k, cudaStream_t s);
cudaError_t batch_bf16s(const sw_batch_header *h, const sw_batch_entry *t, int cfg, int k, cudaStream_t s);

}  // namespace sw
