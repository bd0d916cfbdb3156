// FP32-bulk instantiation of the per-atom passes.
#define PASS_REAL float
#include "pass_inst.cuh"
