// FP32-bulk instantiation of the parameter-gradient passes.
#define PASS_REAL float
#include "grad_inst.cuh"
