// FP64 instantiations of the compile-time-size passes.
#include "passes_ct.cuh"

GB_CT_DEFINE(double, f64)
