// Whole-body rigid-body terms, torque interface and model step
// (mpxg_wb_terms, mpxg_wb_interface, mpxg_wb_step; kernels in wb_kernel.cuh).
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/mpxg.h"
#include "internal.h"
#include "wb_kernel.cuh"

using namespace mpxg;

// ---------------------------------------------------------------- whole body
// The checks the whole-body kernel relies on (it indexes shared arrays by
// these fields without further bounds tests).
const char* mpxg::wb_model_check(const mpxg_wb_model* m) {
  using namespace mpxg::wb;
  if (!m) return "null model";
  if (m->nbody < 1 || m->nbody > MPXG_WB_MAX_BODY) return "nbody out of range 1..32";
  if (m->nv < 0 || m->nv > MPXG_WB_MAX_DOF) return "nv out of range 0..32";
  if (m->nq < 0 || m->nq > MPXG_WB_MAX_DOF + 4) return "nq out of range";
  if (m->n_contact < 0 || m->n_contact > MPXG_WB_MAX_CONTACT) return "n_contact out of range 0..8";
  int dof = 0, qp = 0;
  for (int b = 0; b < m->nbody; ++b) {
    const int jt = m->jnt_type[b];
    if (m->parent[b] < -1 || m->parent[b] >= b) return "bodies must be listed parents first";
    if (jt < 0 || jt > 3) return "unknown joint type";
    if (jt == 1 && (b != 0 || m->parent[b] != -1)) return "a free joint is allowed on the first body only";
    if (m->dof_adr[b] != dof || m->qpos_adr[b] != qp) return "dof / qpos addresses must be dense in body order";
    dof += ndof(jt);
    qp += nqpos(jt);
    if (!(m->mass[b] >= 0.0f)) return "negative mass";
  }
  if (dof != m->nv || qp != m->nq) return "nv / nq do not match the joints";
  for (int c = 0; c < m->n_contact; ++c)
    if (m->contact_point_body[c] < 0 || m->contact_point_body[c] >= m->nbody || m->contact_jac_body[c] < 0 ||
        m->contact_jac_body[c] >= m->nbody)
      return "contact body out of range";
  return nullptr;
}

// The smallest capacity the (checked) model fits.
template <int MODE>
static cudaError_t wb_launch(const mpxg_wb_model& m, int batch, const mpxg::wb::Args& a, cudaStream_t st) {
  using namespace mpxg::wb;
  if (m.nbody <= CapQuad::MB && m.nv <= CapQuad::MD && m.nq <= CapQuad::MD + 4 && 3 * m.n_contact <= CapQuad::MR)
    wb_kernel<MODE, CapQuad><<<(batch + CapQuad::NW - 1) / CapQuad::NW, 32 * CapQuad::NW, 0, st>>>(m, batch, a);
  else
    wb_kernel<MODE, CapAny><<<(batch + CapAny::NW - 1) / CapAny::NW, 32 * CapAny::NW, 0, st>>>(m, batch, a);
  return cudaGetLastError();
}

extern "C" {

mpxg_status mpxg_wb_terms(void* stream, const mpxg_wb_model* model, int batch, const float* qpos, const float* qvel,
                          float* M, float* bias, float* cpos, float* J, float* cvel) {
  using namespace mpxg::wb;
  if (const char* why = wb_model_check(model)) return lib_fail(MPXG_ERR_INVALID_ARG, std::string("mpxg_wb_terms: ") + why);
  if (batch < 0 || (batch > 0 && (!qpos || !qvel)))
    return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_wb_terms: bad batch or null state");
  if (batch == 0) return MPXG_OK;
  Args a{};
  a.qpos = qpos; a.qvel = qvel; a.M = M; a.bias = bias; a.cpos = cpos; a.J = J; a.cvel = cvel;
  a.sq = model->nq; a.sv = model->nv;
  cudaError_t e = wb_launch<MODE_TERMS>(*model, batch, a, (cudaStream_t)stream);
  return e == cudaSuccess ? MPXG_OK : lib_cuda_fail(e, "wb_kernel launch");
}

mpxg_status mpxg_wb_interface(void* stream, const mpxg_wb_model* model, int batch, const float* qpos,
                              const float* qvel, const float* grf, const float* foot_ref, const float* foot_ref_dot,
                              const int* contact, const float* Kp, const float* Kd, float* tau, float* J) {
  using namespace mpxg::wb;
  if (const char* why = wb_model_check(model))
    return lib_fail(MPXG_ERR_INVALID_ARG, std::string("mpxg_wb_interface: ") + why);
  if (model->jnt_type[0] != 1 || model->n_contact < 1 || model->nv != 6 + 3 * model->n_contact)
    return lib_fail(MPXG_ERR_INVALID_ARG,
                "mpxg_wb_interface: needs a free root and nv = 6 + 3 x contacts (one torque row per contact axis)");
  if (batch < 0 || (batch > 0 && (!qpos || !qvel || !grf || !foot_ref || !foot_ref_dot || !contact || !Kp || !Kd ||
                                  !tau)))
    return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_wb_interface: bad batch or null pointer");
  if (batch == 0) return MPXG_OK;
  Args a{};
  a.qpos = qpos; a.qvel = qvel; a.grf = grf; a.foot_ref = foot_ref; a.foot_ref_dot = foot_ref_dot;
  a.contact = contact; a.Kp = Kp; a.Kd = Kd; a.tau = tau; a.J = J;
  a.sq = model->nq; a.sv = model->nv;
  cudaError_t e = wb_launch<MODE_INTERFACE>(*model, batch, a, (cudaStream_t)stream);
  return e == cudaSuccess ? MPXG_OK : lib_cuda_fail(e, "wb_kernel launch");
}

mpxg_status mpxg_wb_step(void* stream, const mpxg_wb_model* model, int batch, float dt, float alpha, const float* x,
                         const float* u, const int* contact, float* x_next) {
  using namespace mpxg::wb;
  if (const char* why = wb_model_check(model)) return lib_fail(MPXG_ERR_INVALID_ARG, std::string("mpxg_wb_step: ") + why);
  const int nv = model->nv, nr = 3 * model->n_contact;
  if (model->jnt_type[0] != 1 || model->nq != nv + 1 || model->n_contact < 1 || nr > nv || nv + nr + 1 > 32)
    return lib_fail(MPXG_ERR_INVALID_ARG,
                "mpxg_wb_step: needs a free root, hinge or slide joints elsewhere, 3 x contacts <= nv and "
                "nv + 3 x contacts + 1 <= 32");
  if (batch < 0 || (batch > 0 && (!x || !u || !contact || !x_next)) || !(dt > 0.0f))
    return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_wb_step: bad batch, dt or null pointer");
  if (batch == 0) return MPXG_OK;
  Args a{};
  const int nx = model->nq + nv + 2 * nr;
  a.qpos = x; a.qvel = x + model->nq; a.sq = nx; a.sv = nx;
  a.u = u; a.contact = contact; a.x_next = x_next; a.dt = dt; a.alpha = alpha;
  cudaError_t e = wb_launch<MODE_STEP>(*model, batch, a, (cudaStream_t)stream);
  return e == cudaSuccess ? MPXG_OK : lib_cuda_fail(e, "wb_kernel launch");
}

}  // extern "C"
