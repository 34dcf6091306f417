// kb_march.cu -- dispatch of the two HBM passes to the per-precision /
// per-flux instantiations (kb_march_f32_*.cu, kb_march_f64_*.cu).
#include "kb_kernels.cuh"

namespace kb {

#define KB_DECL(NAME)                                      \
  int moments_##NAME(DevState& s, cudaStream_t st);        \
  int march_##NAME(DevState& s, double dt, cudaStream_t st);
KB_DECL(f32_kfvs)
KB_DECL(f32_kcu)
KB_DECL(f32_ugks)
KB_DECL(f64_kfvs)
KB_DECL(f64_kcu)
KB_DECL(f64_ugks)
#undef KB_DECL

int launch_moments(DevState& s, cudaStream_t st) {
  if (s.prec == 0) {
    if (s.flux == FLUX_KFVS) return moments_f64_kfvs(s, st);
    if (s.flux == FLUX_KCU) return moments_f64_kcu(s, st);
    return moments_f64_ugks(s, st);
  }
  if (s.flux == FLUX_KFVS) return moments_f32_kfvs(s, st);
  if (s.flux == FLUX_KCU) return moments_f32_kcu(s, st);
  return moments_f32_ugks(s, st);
}

int launch_march(DevState& s, double dt, cudaStream_t st) {
  if (s.prec == 0) {
    if (s.flux == FLUX_KFVS) return march_f64_kfvs(s, dt, st);
    if (s.flux == FLUX_KCU) return march_f64_kcu(s, dt, st);
    return march_f64_ugks(s, dt, st);
  }
  if (s.flux == FLUX_KFVS) return march_f32_kfvs(s, dt, st);
  if (s.flux == FLUX_KCU) return march_f32_kcu(s, dt, st);
  return march_f32_ugks(s, dt, st);
}

}  // namespace kb
