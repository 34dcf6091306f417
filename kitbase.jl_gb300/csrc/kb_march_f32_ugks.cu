// kb_march_f32_ugks.cu -- float x UGKS instantiation of the two HBM passes.
#include "kb_march.cuh"

KB_MARCH_INSTANCE(float, kb::FLUX_UGKS, f32_ugks)
