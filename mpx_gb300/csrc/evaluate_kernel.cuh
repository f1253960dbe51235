// Cost and constraint residuals of given trajectories: the quantities the
// reference prints between offline SQP iterations through
// optimizers.model_evaluator_helper(cost, dynamics, x0, X, U) -> (g, c)
// (mpx/utils/mpc_wrapper.py:419-423,452-465).  One thread per (instance,
// stage); rows past an instance's horizon are written as zeros.
#pragma once
#include "models.cuh"

namespace mpxg {

template <class M>
__global__ void evaluate_kernel(ModelConst mc, int batch, int n_max, const int* __restrict__ horizon,
                                const float* __restrict__ x0, const float* __restrict__ X,
                                const float* __restrict__ U, const float* __restrict__ ref,
                                const float* __restrict__ par, const float* __restrict__ w, float* __restrict__ g,
                                float* __restrict__ c) {
  constexpr int NX = M::NX, NU = M::NU;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)batch * (n_max + 1)) return;
  const int b = (int)(idx / (n_max + 1)), t = (int)(idx % (n_max + 1));
  const int N = horizon ? horizon[b] : n_max;
  float* co = c + idx * NX;
  if (N < 1 || N > n_max || t > N) {
    g[idx] = 0.0f;
#pragma unroll
    for (int i = 0; i < NX; ++i) co[i] = 0.0f;
    return;
  }
  const float* Xb = X + (size_t)b * (n_max + 1) * NX;
  const float* Ub = U + (size_t)b * n_max * NU;
  float xt[NX], ut[NU];
#pragma unroll
  for (int i = 0; i < NX; ++i) xt[i] = Xb[t * NX + i];
#pragma unroll
  for (int a = 0; a < NU; ++a) ut[a] = t < N ? Ub[t * NU + a] : 0.0f;
  const float l = stage_cost<M>(mc, xt, ut, ref + ((size_t)b * (n_max + 1) + t) * M::NREF, w + (size_t)b * 24, t == N);
  g[idx] = l;
  if (t == 0) {
#pragma unroll
    for (int i = 0; i < NX; ++i) co[i] = x0[(size_t)b * NX + i] - xt[i];
  } else {
    float xp[NX], up[NU], fx[NX];
#pragma unroll
    for (int i = 0; i < NX; ++i) xp[i] = Xb[(t - 1) * NX + i];
#pragma unroll
    for (int a = 0; a < NU; ++a) up[a] = Ub[(t - 1) * NU + a];
    M::template dynamics<float>(mc, xp, up, par + ((size_t)b * (n_max + 1) + t - 1) * M::NPAR, fx);
#pragma unroll
    for (int i = 0; i < NX; ++i) co[i] = fx[i] - xt[i];
  }
}

}  // namespace mpxg
