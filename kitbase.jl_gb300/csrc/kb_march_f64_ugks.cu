// kb_march_f64_ugks.cu -- double x UGKS instantiation of the two HBM passes.
#include "kb_march.cuh"

KB_MARCH_INSTANCE(double, kb::FLUX_UGKS, f64_ugks)
