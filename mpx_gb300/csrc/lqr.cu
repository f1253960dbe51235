// Isolated time-varying LQR solve (mpxg_lqr_solve): sequential Riccati
// (lqr_kernels.cuh) and associative scan (lqr_scan.cuh).
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/mpxg.h"
#include "internal.h"
#include "lqr_kernels.cuh"

using namespace mpxg;

extern "C" {

size_t mpxg_lqr_workspace_bytes(int batch, int N, int n, int m, int method) {
  (void)m;
  (void)method;
  if (batch < 0 || N < 1 || n < 1) return 0;
  return lqr_scratch_bytes(batch, N, n);
}

mpxg_status mpxg_lqr_solve(void* stream, const mpxg_lq_io* io, int method) {
  return lqr_solve_host(stream, io, method, &lib_error());
}

}  // extern "C"
