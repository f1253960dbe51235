// SQP, vector-Jacobian-product and evaluation kernels of the quaternion SRBD model
// (a unit of its own so that the models compile in parallel).
#include "sqp_ops.cuh"

MPXG_DEFINE_SQP_OPS(mpxg::ModelQuat13, quat13)
