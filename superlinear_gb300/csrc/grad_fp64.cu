// FP64 plain instantiation of the parameter-gradient passes.
#define PASS_REAL double
#include "grad_inst.cuh"
