// Equality-constrained time-varying LQR (mpxg_lqr_eq_solve) with the
// Riccati stage's dense products on the tensor cores.
//
// The recursion is the one of lqr_eq_kernel.cuh (stagewise Riccati with a
// Schur-complement control QP; D K = -C so P <- Q_xx + Q_ux'K + C'K_nu).  Per
// stage, three split-TF32 tcgen05 products with float32 accumulators in
// tensor memory carry ~90 % of the arithmetic:
//   alpha  D1 = P [A | B | c]                        (n x n)(n x (n+m+1))
//   beta   D2 = [A | B | c]' [P A | P B | P c + p]   ((n+m+1) x n)(n x (n+m+1))
//          -> Q_xx - Q, Q_ux - M', Q_uu - R, q_x - q, q_u - r in one product
//   gamma  D2[0:n, 0:n] += [Q_ux' | C'] [K ; K_nu]   (n x (m+p))((m+p) x n)
// and P = D2[0:n, 0:n] + Q, symmetrised.  The eliminations with Q_uu and S
// (column-parallel block Gauss-Jordan solves, shared with the CUDA-core
// kernel), the small products of the elimination and p stay on the CUDA
// cores.  The stage's cost blocks (M, R, Q) are added to the raw
// accumulators, and every stage input arrives by cp.async while the previous
// stage computes.  One 256-thread block per problem: thread 0 issues each
// product's MMAs and commits them to an mbarrier; the eight warps read the
// accumulators back (warp w: lanes 32 (w % 4) .., column groups w / 4, + 2).
//
// Shared memory (n = 72, m = 30, p = 12: ~219 KB) holds the operands in the
// slab layout of tc_tf32.cuh, each as a TF32 hi and lo copy:
//   region P: P (alpha's A operand), later [Q_ux' | C'] (gamma's A operand);
//   region F: [A | B | c] as rows (alpha's B operand and beta's A operand),
//             later the float32 P - Q before symmetrisation, and behind it
//             the next stage's raw inputs;
//   region G: [PA | PB | Pc + p] as rows (beta's B operand), later [K ; K_nu]
//             and the stage's Q;
//   then the column-major blocks and vectors of the elimination, M and R.
// The forward sweep and the costates are the CUDA-core code of
// lqr_eq_kernel.cuh over the same buffers.
#pragma once
#include "lqr_eq_kernel.cuh"
#include "tc_tf32.cuh"

namespace mpxg {
namespace lqeq {

constexpr int rup8(int v) { return (v + 7) / 8 * 8; }
constexpr int rup16(int v) { return (v + 15) / 16 * 16; }
constexpr uint32_t al128(uint32_t v) { return (v + 127u) / 128u * 128u; }
constexpr uint32_t umax(uint32_t a, uint32_t b) { return a > b ? a : b; }

template <int NX, int NU, int NE>
struct TcLay {
  static_assert(NX % 8 == 0 && NX <= 128, "state dimension: a multiple of 8, at most 128 (one M = 128 tile)");
  static_assert(NX + NU + 1 <= 128, "beta's rows (n + m + 1) must fit one M = 128 tile");
  // product shapes (M = 128 for all three)
  static constexpr int N1 = rup16(NX + NU + 1);  // alpha, beta
  static constexpr int N3 = rup16(NX);           // gamma
  static constexpr int K1 = NX;                  // alpha, beta
  static constexpr int K3 = rup8(NU + NE);       // gamma
  static constexpr int SL1 = K1 / 4, SL3 = K3 / 4;
  // slab strides (bytes): used rows x 16 + 16 (the extra 16 bytes spread a
  // column of lanes over all banks)
  static constexpr uint32_t SP = NX * 16 + 16, SF = rup8(NX + NU + 1) * 16 + 16, SG = SF;
  static constexpr uint32_t SH = NX * 16 + 16, SJ = NX * 16 + 16;
  // regions (bytes)
  static constexpr uint32_t OFF_BAR = 0;
  static constexpr uint32_t OFF_P = 128;
  static constexpr uint32_t BYTES_P = umax(2u * SL1 * SP, 2u * SL3 * SH);
  static constexpr uint32_t OFF_F = al128(OFF_P + BYTES_P);
  static constexpr uint32_t BYTES_F = umax(2u * SL1 * SF, (uint32_t)(NX * (NX + 1) * 4));
  static constexpr uint32_t OFF_G = al128(OFF_F + BYTES_F);
  static constexpr uint32_t BYTES_G = umax(2u * SL1 * SG, 2u * SL3 * SJ);
  static constexpr uint32_t OFF_S = al128(OFF_G + BYTES_G);
  // elimination blocks (floats from OFF_S), column-major, odd leading dims
  static constexpr int LU = NU + (NU % 2 == 0 ? 1 : 2), LE = NE + (NE % 2 == 0 ? 1 : 2);
  // ZW: the solution [Z | g | W] of Q_uu [Z | g | W] = [Q_ux | q_u | D'];
  // TS: D [Z | g | W]; KK: [K_nu | k_nu]
  static constexpr int NZW = NX + 1 + NE;
  static constexpr int QUU = 0, QUX = QUU + NU * LU, ZW = QUX + NX * LU, C = ZW + NZW * LU, D = C + NX * LE,
                       TS = D + NU * LE, KK = TS + NZW * LE, PIV = (KK + (NX + 1) * LE + 3) / 4 * 4,
                       V = PIV + 2 * kGjBlock * 32;
  static constexpr int VL = NX + 4;
  static constexpr int vq = V, vr = vq + VL, ve = vr + VL, vp = ve + VL, vqx = vp + VL, vqu = vqx + VL,
                       vkn = vqu + VL, vk = vkn + VL, vx = vk + VL, vu = vx + VL, vt = vu + VL, FLOATS = vt + VL;
  // the stage's M and R (row-major, copied asynchronously)
  static constexpr uint32_t OFF_MR = al128(OFF_S + (uint32_t)FLOATS * 4u);
  static constexpr uint32_t MR_BYTES = (uint32_t)(NX * NU + NU * NU) * 4u;
  // the stage's Q (row-major) sits in region G behind gamma's B operand
  static constexpr uint32_t OFF_QS = OFF_G + 2u * SL3 * SJ;
  static_assert(2u * SL3 * SJ + (uint32_t)(NX * NX) * 4u <= BYTES_G, "Q must fit region G behind [K ; K_nu]");
  // the next stage's raw A | B | c | C | D | q | r | e (each 16-byte
  // aligned), copied into region F behind the float32 P while the
  // elimination runs (region F is free between beta and gamma)
  static constexpr int r4(int v) { return (v + 3) / 4 * 4; }
  static constexpr int RA = 0, RB = RA + r4(NX * NX), RC = RB + r4(NX * NU), RCC = RC + r4(NX),
                       RD = RCC + r4(NE * NX), RQ = RD + r4(NE * NU), RR = RQ + r4(NX), RE = RR + r4(NU),
                       RAW_FLOATS = RE + r4(NE);
  static constexpr uint32_t OFF_RAW = OFF_F + al128((uint32_t)(NX * (NX + 1) * 4));
  static constexpr uint32_t RAW_BYTES = (uint32_t)RAW_FLOATS * 4u;
  static_assert(OFF_RAW + RAW_BYTES <= OFF_F + BYTES_F, "raw stage data must fit region F behind P");
  // asynchronous copies move 16-byte chunks: per-stage sizes must allow them
  static constexpr bool ASYNC_SIZES = (NX * NX * 4) % 16 == 0 && (NX * NU * 4) % 16 == 0 &&
                                      (NU * NU * 4) % 16 == 0 && (NX * 4) % 16 == 0;
  // + 2 KB: a 128-row operand read past the last buffer's used rows (their
  // accumulator rows are never read) stays inside the allocation
  static constexpr uint32_t BYTES = OFF_MR + MR_BYTES + 2048u;
  static_assert(BYTES <= 232448u, "227 KB of shared memory per block");
  // forward sweep staging (two stages of A | B | K | c | k) over regions F, G;
  // the costates' x staging (a warp's NX floats) over the elimination blocks
  static_assert(2u * FwdLay<NX, NU>::STG * 4u <= OFF_S - OFF_F, "forward staging must fit regions F and G");
  static_assert((kThreads / 32) * NX <= V, "costate staging must fit the elimination blocks");
};

template <int NX, int NU, int NE>
constexpr size_t tc_smem_bytes() { return TcLay<NX, NU, NE>::BYTES; }

// Bounded wait on the product mbarrier; every thread gets the same verdict.
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t& phase) {
  const bool ok = tc::mbar_wait(bar, phase & 1u, 1 << 22);
  ++phase;
  tc::fence_after_sync();
  return __syncthreads_and(ok ? 1 : 0) != 0;
}

// Generic-proxy shared writes (operands) and tensor-memory reads before this
// point are ordered before the MMAs thread 0 issues after it.
__device__ __forceinline__ void tc_handoff() {
  tc::fence_smem_to_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

// Asynchronous global -> shared copy of one stage block by the whole block
// (completion per thread through commit groups): 16-byte chunks when `vec`
// (16-byte aligned source and destination, size a multiple of 4 floats),
// else 4-byte copies.
__device__ __forceinline__ void copy_async(float* dst, const float* src, int floats, bool vec) {
  const uint32_t d = tc::smem_u32(dst);
  const char* g = reinterpret_cast<const char*>(src);
  if (vec && (floats & 3) == 0) {
    for (int off = threadIdx.x * 16; off < floats * 4; off += kThreads * 16)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d + off), "l"(g + off) : "memory");
  } else {
    for (int off = threadIdx.x * 4; off < floats * 4; off += kThreads * 4)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d + off), "l"(g + off) : "memory");
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_older() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int NX, int NU, int NE>
__global__ void __launch_bounds__(kThreads, 1) lqr_eq_tc_kernel(mpxg_lq_eq_io io, float* Pscr, bool async) {
  typedef TcLay<NX, NU, NE> L;
  constexpr int LU = L::LU, LE = L::LE;
  extern __shared__ __align__(1024) unsigned char smraw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw + L::OFF_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smraw + L::OFF_BAR + 8);
  unsigned char* Ph = smraw + L::OFF_P;
  unsigned char* Pl = Ph + L::SL1 * L::SP;
  unsigned char* Hh = smraw + L::OFF_P;
  unsigned char* Hl = Hh + L::SL3 * L::SH;
  unsigned char* Fh = smraw + L::OFF_F;
  unsigned char* Fl = Fh + L::SL1 * L::SF;
  float* Pst = reinterpret_cast<float*>(smraw + L::OFF_F);  // float32 P, row-major, stride NX + 1
  unsigned char* Gh = smraw + L::OFF_G;
  unsigned char* Gl = Gh + L::SL1 * L::SG;
  unsigned char* Jh = smraw + L::OFF_G;
  unsigned char* Jl = Jh + L::SL3 * L::SJ;
  float* s = reinterpret_cast<float*>(smraw + L::OFF_S);
  float *Quu = s + L::QUU, *Qux = s + L::QUX, *ZW = s + L::ZW, *sC = s + L::C, *sD = s + L::D, *TS = s + L::TS;
  float *KK = s + L::KK, *piv = s + L::PIV;
  float* sM = reinterpret_cast<float*>(smraw + L::OFF_MR);
  float* sR = sM + NX * NU;
  float* sQ = reinterpret_cast<float*>(smraw + L::OFF_QS);
  float* raw = reinterpret_cast<float*>(smraw + L::OFF_RAW);
  float *rawA = raw + L::RA, *rawB = raw + L::RB, *rawc = raw + L::RC, *rawC = raw + L::RCC, *rawD = raw + L::RD;
  float *rawq = raw + L::RQ, *rawr = raw + L::RR, *rawe = raw + L::RE;
  float *vq = s + L::vq, *vr = s + L::vr, *ve = s + L::ve, *vp = s + L::vp, *vqx = s + L::vqx, *vqu = s + L::vqu;
  float *vkn = s + L::vkn, *vk = s + L::vk, *vx = s + L::vx, *vu = s + L::vu;
  float* vt = s + L::vt;
  const int b = blockIdx.x, N = io.N, tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31, quarter = warp & 3, half = warp >> 2;
  const int row = 32 * quarter + lane;  // accumulator row this thread reads
  constexpr int NP = NX + 1;
  float* Ps = Pscr + (size_t)b * (N + 1) * NP * NX;
  const size_t sn = (size_t)b * N, sn1 = (size_t)b * (N + 1);

  // ---- tensor memory (D1: columns 0.., D2: columns 128..) and the mbarrier.
  // The allocation cannot wait on another block: ~219 KB of shared memory
  // keeps one block of this kernel per SM, 256 of the SM's 512 columns are
  // taken, and no other kernel of the library uses tensor memory.
  if (warp == 0) tc::tmem_alloc(tc::smem_u32(tslot), 256);
  if (tid == 0) {
    tc::mbar_init(tc::smem_u32(bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = *tslot;
  const uint32_t D1 = tm, D2 = tm + 128u, lrow = (uint32_t)(32 * quarter) << 16;
  const uint32_t barp = tc::smem_u32(bar);
  uint32_t phase = 0;
  bool ok = true;

  // Symmetrise the float32 P in Pst (+ the stage's Q, in shared memory, when
  // given; also symmetrised) into region P (TF32 hi / lo) and the workspace
  // row t; p from vp.
  constexpr int PIT = (NX * (NX / 4) + kThreads - 1) / kThreads;
  auto store_P = [&](int t, const float* Qt) {
    float* Pt = Ps + (size_t)t * NP * NX;
#pragma unroll
    for (int it = 0; it < PIT; ++it) {
      const int e = tid + kThreads * it;
      if (e < NX * (NX / 4)) {
        const int m = e % NX, k0 = 4 * (e / NX);  // lanes over rows: conflict-free column reads
        float v[4], h[4], l[4];
        float4 qr = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float qc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (Qt) {
          qr = *reinterpret_cast<const float4*>(Qt + m * NX + k0);
#pragma unroll
          for (int j = 0; j < 4; ++j) qc[j] = Qt[(k0 + j) * NX + m];
        }
        const float qrv[4] = {qr.x, qr.y, qr.z, qr.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          v[j] = 0.5f * ((Pst[m * (NX + 1) + k0 + j] + Pst[(k0 + j) * (NX + 1) + m]) + (qrv[j] + qc[j]));
          tc::split(v[j], &h[j], &l[j]);
        }
        const uint32_t o = tc::slab_off(m, k0, L::SP);
        *reinterpret_cast<float4*>(Ph + o) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4*>(Pl + o) = make_float4(l[0], l[1], l[2], l[3]);
        *reinterpret_cast<float4*>(Pt + m * NX + k0) = make_float4(v[0], v[1], v[2], v[3]);
      }
    }
    for (int i = tid; i < NX; i += kThreads) Pt[NX * NX + i] = vp[i];
  };

  // the raw stage-t data into region F (16-byte chunks when aligned)
  auto copy_raw = [&](int t) {
    copy_async(rawA, io.A + (sn + t) * NX * NX, NX * NX, async);
    copy_async(rawB, io.Bm + (sn + t) * NX * NU, NX * NU, async);
    copy_async(rawc, io.c + (sn + t) * NX, NX, async);
    copy_async(rawC, io.C + (sn + t) * NE * NX, NE * NX, async);
    copy_async(rawD, io.D + (sn + t) * NE * NU, NE * NU, async);
    copy_async(rawq, io.q + (sn1 + t) * NX, NX, async);
    copy_async(rawr, io.r + (sn + t) * NU, NU, async);
    copy_async(rawe, io.e + (sn + t) * NE, NE, async);
  };

  // L2 prefetch of one stage's matrices (128-byte lines over the block; only
  // with 16-byte aligned inputs, like the asynchronous copies)
  auto prefetch_stage = [&](int t) {
    if (!async) return;
    auto pf = [&](const float* base, int floats) {
      const char* c = reinterpret_cast<const char*>(base);
      for (int off = tid * 128; off < floats * 4; off += kThreads * 128)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(c + off));
    };
    pf(io.A + (sn + t) * NX * NX, NX * NX);
    pf(io.Bm + (sn + t) * NX * NU, NX * NU);
    pf(io.Q + (sn1 + t) * NX * NX, NX * NX);
    pf(io.M + (sn + t) * NX * NU, NX * NU);
    pf(io.R + (sn + t) * NU * NU, NU * NU);
    pf(io.C + (sn + t) * NE * NX, NE * NX);
    pf(io.D + (sn + t) * NE * NU, NE * NU);
  };

  // ---- terminal value function
  {
    const float* QN = io.Q + (sn1 + N) * NX * NX;
    for (int e = tid; e < NX * NX; e += kThreads) Pst[(e / NX) * (NX + 1) + e % NX] = __ldg(QN + e);
    load_vec<NX>(vp, io.q + (sn1 + N) * NX);
    if (N >= 1) {
      prefetch_stage(N - 1);
      copy_raw(N - 1);
    }
    cp_async_commit();
    __syncthreads();
    store_P(N, nullptr);
    __syncthreads();
  }

  for (int t = N - 1; t >= 0 && ok; --t) {
    if (t >= 1) prefetch_stage(t - 1);
    cp_async_wait_all();  // this stage's raw A | B | c (copied during the last one)
    __syncthreads();
    copy_async(sM, io.M + (sn + t) * NX * NU, NX * NU, async);
    copy_async(sR, io.R + (sn + t) * NU * NU, NU * NU, async);
    cp_async_commit();
    // ---- stage data: [A | B | c] as operand rows (element (n, k) = F[k][n])
    // from the raw copy, the equality blocks and the vectors
    {
      constexpr int NF = NX + NU + 1, FE = (NX / 4) * NF, FIT = (FE + kThreads - 1) / kThreads;
      float v[FIT][4];
#pragma unroll
      for (int it = 0; it < FIT; ++it) {
        const int e = tid + kThreads * it;
        const int k0 = 4 * (e / NF), n = e % NF;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int k = k0 + j;
          v[it][j] = e >= FE ? 0.0f : (n < NX ? rawA[k * NX + n] : (n < NX + NU ? rawB[k * NU + n - NX] : rawc[k]));
        }
      }
      // the equality blocks (column-major) and the vectors from the raw copy
      for (int e = tid; e < NE * NX; e += kThreads) sC[(e % NX) * LE + e / NX] = rawC[e];
      for (int e = tid; e < NE * NU; e += kThreads) sD[(e % NU) * LE + e / NU] = rawD[e];
      for (int i = tid; i < NX; i += kThreads) vq[i] = rawq[i];
      for (int i = tid; i < NU; i += kThreads) vr[i] = rawr[i];
      for (int i = tid; i < NE; i += kThreads) ve[i] = rawe[i];
      __syncthreads();  // the slabs overwrite the raw copy
#pragma unroll
      for (int it = 0; it < FIT; ++it) {
        const int e = tid + kThreads * it;
        if (e < FE) {
          const int k0 = 4 * (e / NF), n = e % NF;
          float h[4], l[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) tc::split(v[it][j], &h[j], &l[j]);
          const uint32_t o = tc::slab_off(n, k0, L::SF);
          *reinterpret_cast<float4*>(Fh + o) = make_float4(h[0], h[1], h[2], h[3]);
          *reinterpret_cast<float4*>(Fl + o) = make_float4(l[0], l[1], l[2], l[3]);
        }
      }
    }
    tc_handoff();
    // ---- alpha: D1 = P [A | B | c]
    if (tid == 0) {
      tc::issue_split_product(D1, tc::idesc_tf32(128, L::N1), tc::smem_u32(Ph), tc::smem_u32(Pl), L::SP,
                              tc::smem_u32(Fh), tc::smem_u32(Fl), L::SF, L::K1 / 8, false);
      tc::mma_commit(barp);
    }
    if (!(ok = tc_wait(barp, phase))) break;
    // ---- alpha's rows k < NX -> beta's B operand: (n, k) = D1[k][n], with
    // p added to column n + m (w = P c + p)
    if (32 * quarter < NX) {
      for (int g = half; g < L::N1 / 8; g += 2) {
        float v[8];
        tc::tmem_ld8(D1 + lrow + 8 * g, v);
        tc::tmem_ld_wait();
        if (row < NX) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int n = 8 * g + j;
            if (n < NX + NU + 1) {
              float h, l;
              tc::split(n == NX + NU ? v[j] + vp[row] : v[j], &h, &l);
              const uint32_t o = tc::slab_off(n, row, L::SG);
              *reinterpret_cast<float*>(Gh + o) = h;
              *reinterpret_cast<float*>(Gl + o) = l;
            }
          }
        }
      }
    }
    tc_handoff();
    // ---- beta: D2 = [A | B | c]' [PA | PB | w]
    if (tid == 0) {
      tc::issue_split_product(D2, tc::idesc_tf32(128, L::N1), tc::smem_u32(Fh), tc::smem_u32(Fl), L::SF,
                              tc::smem_u32(Gh), tc::smem_u32(Gl), L::SG, L::K1 / 8, false);
      tc::mma_commit(barp);
    }
    if (!(ok = tc_wait(barp, phase))) break;
    copy_async(sQ, io.Q + (sn1 + t) * NX * NX, NX * NX, async);  // region G is free until gamma's operands
    if (t >= 1) copy_raw(t - 1);  // region F is free until gamma's P
    cp_async_commit();
    // ---- Q-function blocks from D2: q_x = q + A'w (rows < n, column n + m),
    // and rows n .. n + m - 1: B'PA (-> Q_ux), B'PB (-> Q_uu), q_u = r + B'w
    {
      const bool has_x = 32 * quarter < NX;
      const bool has_u = (32 * quarter + 31 >= NX) && (32 * quarter < NX + NU);
      constexpr int gw = (NX + NU) / 8;  // column group holding column n + m
      for (int g = half; g <= gw; g += 2) {
        if (!(has_u || (has_x && g == gw))) continue;  // warp-uniform
        float v[8];
        tc::tmem_ld8(D2 + lrow + 8 * g, v);
        tc::tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int col = 8 * g + j;
          if (row < NX) {
            if (col == NX + NU) vqx[row] = vq[row] + v[j];
          } else if (row < NX + NU) {
            const int a = row - NX;
            if (col < NX) Qux[col * LU + a] = v[j];
            else if (col < NX + NU) Quu[(col - NX) * LU + a] = v[j];
            else if (col == NX + NU) vqu[a] = vr[a] + v[j];
          }
        }
      }
    }
    cp_async_wait_older();  // M and R have landed (Q may still be in flight)
    __syncthreads();
    // ---- elimination (CUDA cores), two column-parallel Gauss-Jordan solves:
    //   Q_uu [Z | g | W] = [Q_ux | q_u | D'];
    //   [S | T | h] = [D W | C - D Z | D g + e],  S [K_nu | -k_nu] = [T | h];
    //   Z += W K_nu (K = -Z), g += W k_nu (k = -g)
    // (the column loads finish Q_uu = R + B'PB and Q_ux = M' + B'PA, and put
    // Q_ux' into gamma's A operand in region P)
    gj_solve<NU, NU + L::NZW, kGjBlock>(piv, [&](int j, float* v) {
      if (j < NU) {
#pragma unroll
        for (int i = 0; i < NU; ++i) v[i] = Quu[j * LU + i] + sR[i * NU + j];
      } else if (j < NU + NX) {
        const int col = j - NU;
#pragma unroll
        for (int i = 0; i < NU; ++i) {
          const float qux = Qux[col * LU + i] + sM[col * NU + i];
          Qux[col * LU + i] = qux;
          v[i] = qux;
          float h, l;
          tc::split(qux, &h, &l);
          const uint32_t o = tc::slab_off(col, i, L::SH);
          *reinterpret_cast<float*>(Hh + o) = h;
          *reinterpret_cast<float*>(Hl + o) = l;
        }
      } else {
#pragma unroll
        for (int i = 0; i < NU; ++i) v[i] = j == NU + NX ? vqu[i] : sD[i * LE + (j - NU - NX - 1)];
      }
    }, [&](int j, const float* v) {
#pragma unroll
      for (int i = 0; i < NU; ++i) ZW[(j - NU) * LU + i] = v[i];
    });
    bmm<NE, NU, L::NZW, false, false, false>(TS, LE, sD, LE, ZW, LU, 1.0f, nullptr, 0);
    gj_solve<NE, NE + NX + 1>(piv, [&](int j, float* v) {
#pragma unroll
      for (int i = 0; i < NE; ++i)
        v[i] = j < NE ? TS[(NX + 1 + j) * LE + i]
                      : (j < NE + NX ? sC[(j - NE) * LE + i] - TS[(j - NE) * LE + i] : TS[NX * LE + i] + ve[i]);
    }, [&](int j, const float* v) {
      const float sg = (j == NE + NX) ? -1.0f : 1.0f;
#pragma unroll
      for (int i = 0; i < NE; ++i) KK[(j - NE) * LE + i] = sg * v[i];
    });
    bmm<NU, NE, NX + 1, false, false, false>(ZW, LU, ZW + (NX + 1) * LU, LU, KK, LE, 1.0f, ZW, LU);
    // ---- gains out; gamma's operands: [K ; K_nu] rows (region G) and the
    // C' / zero columns of [Q_ux' | C'] (region P)
    {
      float* Ko = io.K + (sn + t) * NU * NX;
      float* ko = io.k + (sn + t) * NU;
      float* Kno = io.Knu + (sn + t) * NE * NX;
      float* kno = io.knu + (sn + t) * NE;
      for (int e = tid; e < NU * NX; e += kThreads) Ko[e] = -ZW[(e % NX) * LU + e / NX];
      for (int e = tid; e < NE * NX; e += kThreads) Kno[e] = KK[(e % NX) * LE + e / NX];
      for (int a = tid; a < NU; a += kThreads) { vk[a] = -ZW[NX * LU + a]; ko[a] = -ZW[NX * LU + a]; }
      for (int j = tid; j < NE; j += kThreads) { vkn[j] = KK[NX * LE + j]; kno[j] = KK[NX * LE + j]; }
      for (int e = tid; e < (L::K3 / 4) * NX; e += kThreads) {
        const int k0 = 4 * (e / NX), n = e % NX;
        float h[4], l[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int k = k0 + j;
          const float v = k < NU ? -ZW[n * LU + k] : (k < NU + NE ? KK[n * LE + k - NU] : 0.0f);
          tc::split(v, &h[j], &l[j]);
        }
        const uint32_t o = tc::slab_off(n, k0, L::SJ);
        *reinterpret_cast<float4*>(Jh + o) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4*>(Jl + o) = make_float4(l[0], l[1], l[2], l[3]);
      }
      for (int e = tid; e < (L::K3 - NU) * NX; e += kThreads) {
        const int k = NU + e / NX, m = e % NX;
        float h, l;
        tc::split(k < NU + NE ? sC[m * LE + k - NU] : 0.0f, &h, &l);
        const uint32_t o = tc::slab_off(m, k, L::SH);
        *reinterpret_cast<float*>(Hh + o) = h;
        *reinterpret_cast<float*>(Hl + o) = l;
      }
    }
    __syncthreads();
    // p <- q_x + Q_ux' k + C' k_nu (CUDA cores; vt as temporary)
    bmv<NX, NU, true>(vt, Qux, LU, vk, 1.0f, vqx);
    bmv<NX, NE, true>(vp, sC, LE, vkn, 1.0f, vt);
    tc_handoff();
    // ---- gamma: D2[0:n, 0:n] += [Q_ux' | C'] [K ; K_nu]
    if (tid == 0) {
      tc::issue_split_product(D2, tc::idesc_tf32(128, L::N3), tc::smem_u32(Hh), tc::smem_u32(Hl), L::SH,
                              tc::smem_u32(Jh), tc::smem_u32(Jl), L::SJ, L::K3 / 8, true);
      tc::mma_commit(barp);
    }
    if (!(ok = tc_wait(barp, phase))) break;
    // ---- P - Q = D2[0:n, 0:n] into region F (float32), then + Q and
    // symmetrised
    if (32 * quarter < NX) {
      for (int g = half; g < NX / 8; g += 2) {
        float v[8];
        tc::tmem_ld8(D2 + lrow + 8 * g, v);
        tc::tmem_ld_wait();
        if (row < NX) {
#pragma unroll
          for (int j = 0; j < 8; ++j) Pst[row * (NX + 1) + 8 * g + j] = v[j];
        }
      }
    }
    cp_async_wait_all();
    __syncthreads();
    store_P(t, sQ);
    __syncthreads();
  }

  // ---- release tensor memory (after a failed wait, first give the MMAs in
  // flight a bounded time to finish, and let this thread's asynchronous
  // copies land before the block can exit)
  if (!ok) {
    tc::mbar_wait(barp, (phase - 1u) & 1u, 1 << 22);
    cp_async_wait_all();
    __syncthreads();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tm, 256);
  if (!ok) {  // reported as a non-finite solution
    const float nan = __int_as_float(0x7fc00000);
    for (int i = tid; i < (N + 1) * NX; i += kThreads) io.X[sn1 * NX + i] = nan;
    return;
  }

  // ---- forward sweep (staging over regions F and G) and costates (CUDA
  // cores, shared with lqr_eq_kernel)
  {
    float* fb = reinterpret_cast<float*>(smraw + L::OFF_F);
    forward_sweep<NX, NU>(io, b, fb, fb + FwdLay<NX, NU>::STG, vx, vu, vt);
  }
  __syncthreads();
  costates<NX, NE>(io, b, Ps, s);
}

template <int NX, int NU, int NE>
inline cudaError_t launch_lqr_eq_tc(cudaStream_t st, const mpxg_lq_eq_io& io) {
  const size_t smem = tc_smem_bytes<NX, NU, NE>();
  cudaError_t e = cudaFuncSetAttribute(lqr_eq_tc_kernel<NX, NU, NE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
  const bool async = TcLay<NX, NU, NE>::ASYNC_SIZES && al16(io.M) && al16(io.R) && al16(io.Q) && al16(io.A) &&
                     al16(io.Bm) && al16(io.c) && al16(io.C) && al16(io.D) && al16(io.q) && al16(io.r) &&
                     al16(io.e);
  lqr_eq_tc_kernel<NX, NU, NE><<<io.batch, kThreads, smem, st>>>(io, io.workspace, async);
  return cudaGetLastError();
}

}  // namespace lqeq
}  // namespace mpxg
