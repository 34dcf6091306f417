// kb_march_f64_kcu.cu -- double x KCU instantiation of the two HBM passes.
#include "kb_march.cuh"

KB_MARCH_INSTANCE(double, kb::FLUX_KCU, f64_kcu)
