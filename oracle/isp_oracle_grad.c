/*
 * isp_oracle_grad.c - FP64 differentiable forward and analytic gradient of the calibration
 * pipeline.  TEST INFRASTRUCTURE ONLY (the checker of the adjoint kernel).
 */
#include "isp_oracle.h"
