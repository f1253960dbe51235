// SQP, vector-Jacobian-product and evaluation kernels of the biped SRBD model
// (a unit of its own so that the models compile in parallel).
#include "sqp_ops.cuh"

MPXG_DEFINE_SQP_OPS(mpxg::ModelBiped12, biped12)
