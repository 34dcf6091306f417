// kb_march_f64_kfvs.cu -- double x KFVS instantiation of the two HBM passes.
#include "kb_march.cuh"

KB_MARCH_INSTANCE(double, kb::FLUX_KFVS, f64_kfvs)
