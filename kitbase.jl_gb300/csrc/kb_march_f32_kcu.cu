// kb_march_f32_kcu.cu -- float x KCU instantiation of the two HBM passes.
#include "kb_march.cuh"

KB_MARCH_INSTANCE(float, kb::FLUX_KCU, f32_kcu)
