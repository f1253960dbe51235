// Equality-constrained LQ solve of the large linearised problems
// (mpxg_lqr_eq_solve): tensor cores (lqr_eq_tc.cuh) and CUDA cores
// (lqr_eq_kernel.cuh).
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/mpxg.h"
#include "internal.h"
#include "lqr_eq_tc.cuh"

using namespace mpxg;

extern "C" {

size_t mpxg_lqr_eq_workspace_bytes(int batch, int N, int n) {
  if (batch < 0 || N < 1 || n < 1) return 0;
  return lqeq::lqr_eq_scratch_bytes(batch, N, n);
}

mpxg_status mpxg_lqr_eq_solve_method(void* stream, const mpxg_lq_eq_io* io, int method) {
  if (!io || io->batch < 0 || io->N < 1 || !io->A || !io->Bm || !io->c || !io->Q || !io->R || !io->M || !io->q ||
      !io->r || !io->C || !io->D || !io->e || !io->x0 || !io->K || !io->k || !io->Knu || !io->knu || !io->X ||
      !io->U || !io->lam || !io->nu || !io->workspace)
    return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_solve: bad arguments");
  if (method != 0 && method != 1) return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_solve: method is 0 or 1");
  if (method == 0 && (reinterpret_cast<uintptr_t>(io->workspace) & 15u) != 0)
    return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_solve: workspace must be 16-byte aligned");
  if (io->batch == 0) return MPXG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  const bool tcores = (method == 0);
  if (io->n == 72 && io->m == 30 && io->n_eq == 12)
    e = tcores ? lqeq::launch_lqr_eq_tc<72, 30, 12>(st, *io) : lqeq::launch_lqr_eq<72, 30, 12>(st, *io);
  else if (io->n == 16 && io->m == 8 && io->n_eq == 4)
    e = tcores ? lqeq::launch_lqr_eq_tc<16, 8, 4>(st, *io) : lqeq::launch_lqr_eq<16, 8, 4>(st, *io);
  else if (io->n == 8 && io->m == 5 && io->n_eq == 2)
    e = tcores ? lqeq::launch_lqr_eq_tc<8, 5, 2>(st, *io) : lqeq::launch_lqr_eq<8, 5, 2>(st, *io);
  else return lib_fail(MPXG_ERR_UNSUPPORTED, "mpxg_lqr_eq_solve: (n, m, n_eq) not built: (72,30,12) (16,8,4) (8,5,2)");
  return e == cudaSuccess ? MPXG_OK : lib_cuda_fail(e, "lqr_eq kernel launch");
}

mpxg_status mpxg_lqr_eq_solve(void* stream, const mpxg_lq_eq_io* io) { return mpxg_lqr_eq_solve_method(stream, io, 0); }

}  // extern "C"
