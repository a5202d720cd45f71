// FP32 instantiations of the compile-time-size passes.
#include "passes_ct.cuh"

GB_CT_DEFINE(float, f32)
GB_CT_DEFINE_PLANE()
