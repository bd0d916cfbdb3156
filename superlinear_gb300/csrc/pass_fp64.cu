// FP64 plain instantiation of the per-atom passes.
#define PASS_REAL double
#include "pass_inst.cuh"
