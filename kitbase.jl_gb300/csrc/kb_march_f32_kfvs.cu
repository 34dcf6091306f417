// kb_march_f32_kfvs.cu -- float x KFVS instantiation of the two HBM passes.
#include "kb_march.cuh"

KB_MARCH_INSTANCE(float, kb::FLUX_KFVS, f32_kfvs)
