// Rigid-body terms of a floating-base kinematic tree and the whole-body torque
// interface of the SRBD controller (mpx/utils/mpc_utils.py:275-313), one warp
// per environment.
//
// The reference obtains these from MuJoCo XLA (mjx.fwd_position,
// mjx.fwd_velocity, mjx.jac; mpc_utils.py:279-298).  Here they are computed
// directly in world coordinates, with spatial vectors taken about one point o
// (the first body's origin), in four warp-synchronous passes:
//   1. forward kinematics level by level down the tree (lane = body);
//   2. the motion axis S_j = (omega; v at o) of every degree of freedom and
//      each body's spatial inertia about o (lane = body);
//   3. body velocities V_b = sum S_j qdot_j over the chain, accelerations at
//      qacc = 0 (gravity as a base acceleration, dS_j/dt = V ×m S_j for
//      axes fixed in a body), the bias force of each body
//      F_b = I_b A_b + V_b ×f (I_b V_b), and the subtree sums of the forces
//      and inertias (lane = body);
//   4. bias_j = S_j . F_subtree(body(j)) and the composite-rigid-body mass
//      matrix M_ij = S_i . (I_subtree(body(j)) S_j) for i in the chain of j
//      (lane = degree of freedom), plus armature on the diagonal.
// Contact points are geom positions; their translational Jacobian column j is
// v_j + omega_j × (p - o) when dof j moves the point's body.
#pragma once
#include <cuda_runtime.h>

#include "../../include/mpxg.h"

namespace mpxg {
namespace wb {

// Shared-memory capacities of the two instantiations: any model the ABI
// accepts, and models up to 16 bodies, 20 dofs and 4 contacts (a quadruped
// with a floating base and 12 joints), whose smaller per-warp footprint lets
// 27 environments share an SM (4096 in one wave on 152 SMs).
template <int MB_, int MD_, int MC_, int NW_, int MINB_>
struct Cap {
  static constexpr int MB = MB_, MD = MD_, MR = 3 * MC_, NW = NW_, MINB = MINB_;
};
using CapAny = Cap<MPXG_WB_MAX_BODY, MPXG_WB_MAX_DOF, MPXG_WB_MAX_CONTACT, 2, 1>;
using CapQuad = Cap<16, 20, 4, 3, 9>;

// The kernels are generic over the scalar T: float for every entry point;
// the whole-body SQP (wb_sqp.cu) also runs the step in double (defects and
// merit) and on a forward-mode dual number (its Jacobians).
template <class T>
struct ArgsT {
  const T *qpos, *qvel, *grf, *foot_ref, *foot_ref_dot, *Kp, *Kd, *u;
  const int* contact;
  T *M, *bias, *cpos, *J, *cvel, *tau, *x_next;
  int sq, sv;        // row strides of qpos and qvel (elements)
  T dt, alpha;       // the dynamics step
};
using Args = ArgsT<float>;

__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_t(double x) { return rsqrt(x); }
__device__ __forceinline__ float sqrt_t(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_t(double x) { return sqrt(x); }
__device__ __forceinline__ void sincos_t(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void sincos_t(double x, double* s, double* c) { sincos(x, s, c); }

enum { MODE_TERMS = 0, MODE_INTERFACE = 1, MODE_STEP = 2 };

template <class C, class T = float>
struct Warp {
  static constexpr int MB = C::MB, MD = C::MD, MR = C::MR;
  T quat[MB][4], R[MB][9], xp[MB][3];
  T S[MD][6];                 // per dof: (omega; linear velocity at o)
  T V[MB][6], F[MB][6], Fc[MB][6];
  T Ib[MB][10], Ic[MB][10];   // (m, h = m c, J_o upper triangle xx xy xz yy yz zz)
  T M[MD][MD + 1];
  T J[MD][MR + 1];
  T bias[MD], qpos[MD + 4], qvel[MD], w[MD];
  T cpos[MR], cvel[MR], a[MR], y[MR];
  int dof_body[MD], depth[MB], par[MB], jtyp[MB], dadr[MB];
  unsigned anc[MB];               // bit a set: a is b or an ancestor of b
};

__host__ __device__ __forceinline__ int ndof(int jt) { return jt == 1 ? 6 : (jt >= 2 ? 1 : 0); }
__host__ __device__ __forceinline__ int nqpos(int jt) { return jt == 1 ? 7 : (jt >= 2 ? 1 : 0); }

template <class A, class B, class T>
__device__ __forceinline__ void cross3(const A* a, const B* b, T* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
template <class A, class B, class T>
__device__ __forceinline__ void quat_mul(const A* a, const B* b, T* c) {  // c = a b, (w, x, y, z)
  c[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
  c[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
  c[2] = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
  c[3] = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
}
// a quaternion of (near) zero norm becomes the identity, as MuJoCo does
template <class T>
__device__ __forceinline__ void quat_normalize(T* q) {
  const T n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  if (!(n2 > 1e-30f)) {
    q[0] = T(1.0); q[1] = q[2] = q[3] = T(0.0);
    return;
  }
  const T s = rsqrt_t(n2);
#pragma unroll
  for (int i = 0; i < 4; ++i) q[i] *= s;
}
// rotation matrix (row-major, world from body) of a unit quaternion
template <class A, class T>
__device__ __forceinline__ void quat_mat(const A* q, T* R) {
  const T w = q[0], x = q[1], y = q[2], z = q[3];
  R[0] = T(1.0) - T(2.0) * (y * y + z * z); R[1] = T(2.0) * (x * y - w * z); R[2] = T(2.0) * (x * z + w * y);
  R[3] = T(2.0) * (x * y + w * z); R[4] = T(1.0) - T(2.0) * (x * x + z * z); R[5] = T(2.0) * (y * z - w * x);
  R[6] = T(2.0) * (x * z - w * y); R[7] = T(2.0) * (y * z + w * x); R[8] = T(1.0) - T(2.0) * (x * x + y * y);
}
template <class A, class B, class T>
__device__ __forceinline__ void mat_vec(const A* R, const B* v, T* o) {
#pragma unroll
  for (int i = 0; i < 3; ++i) o[i] = R[3 * i] * v[0] + R[3 * i + 1] * v[1] + R[3 * i + 2] * v[2];
}
// spatial inertia (m, h, J_o) times a motion (w; v): (J w + h × v; m v + w × h)
template <class T>
__device__ __forceinline__ void inert_mul(const T* I, const T* s, T* o) {
  const T m = I[0], h[3] = {I[1], I[2], I[3]};
  const T Jxx = I[4], Jxy = I[5], Jxz = I[6], Jyy = I[7], Jyz = I[8], Jzz = I[9];
  T hv[3], wh[3];
  cross3(h, s + 3, hv);
  cross3(s, h, wh);
  o[0] = Jxx * s[0] + Jxy * s[1] + Jxz * s[2] + hv[0];
  o[1] = Jxy * s[0] + Jyy * s[1] + Jyz * s[2] + hv[1];
  o[2] = Jxz * s[0] + Jyz * s[1] + Jzz * s[2] + hv[2];
#pragma unroll
  for (int i = 0; i < 3; ++i) o[3 + i] = m * s[3 + i] + wh[i];
}
// motion cross motion: (w; v) ×m (w2; v2) = (w × w2; w × v2 + v × w2)
template <class T>
__device__ __forceinline__ void crm(const T* a, const T* b, T* o) {
  T t[3];
  cross3(a, b, o);
  cross3(a, b + 3, o + 3);
  cross3(a + 3, b, t);
#pragma unroll
  for (int i = 0; i < 3; ++i) o[3 + i] += t[i];
}
// motion cross force: (w; v) ×f (n; f) = (w × n + v × f; w × f)
template <class T>
__device__ __forceinline__ void crf(const T* a, const T* f, T* o) {
  T t[3];
  cross3(a, f, o);
  cross3(a + 3, f + 3, t);
  cross3(a, f + 3, o + 3);
#pragma unroll
  for (int i = 0; i < 3; ++i) o[i] += t[i];
}
template <class T>
__device__ __forceinline__ T dot6(const T* a, const T* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3] + a[4] * b[4] + a[5] * b[5];
}

// Gauss-Jordan elimination of the first n pivots of a column-distributed
// matrix: lane c holds column c in col[0..N).  Without pivoting (the matrices
// here are symmetric positive definite); afterwards the columns right of the
// pivots hold the solutions.
template <int N, class T>
__device__ __forceinline__ void gj_lanes(T (&col)[N], int n) {
  const unsigned full = 0xffffffffu;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    if (k < n) {
      const T dk = __shfl_sync(full, col[k], k);
      const T yk = col[k] / dk;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        if (i < n && i != k) {
          const T gik = __shfl_sync(full, col[i], k);
          col[i] -= gik * yk;
        }
      }
      col[k] = yk;
    }
  }
}

// One step of the whole-body model (mpx/utils/models.py:39-117) from the
// terms already in shared memory (M, bias, J, contact points at x):
//   Y = M^-1 J, z = M^-1 (tau - bias), tau = [0 (6), u],
//   (J'Y) f = -J'z - 2 alpha J'qdot,   f masked by contact,
//   v+ = qdot + (z + Y f) dt,  p+ = p + v+ dt,  quat+ = quat * exp(w+ dt / 2),
//   q+ = q + dq+ dt;  x+ = [p+, quat+, q+, v+, contact points at x, f].
// Requires a free root, nq = nv + 1 and nv + 3 C + 1 <= 32 (host checks).
template <class C, class T>
__device__ __forceinline__ void step(const mpxg_wb_model& m, Warp<C, T>& s, const T* u, const int* contact, T dt,
                                     T alpha, T* xo, int lane) {
  constexpr int MD = C::MD, MR = C::MR;
  const int nv = m.nv, nq = m.nq, nc = m.n_contact, nr = 3 * nc;
  // [M | J | tau - bias], lane c holding column c
  T col[MD];
#pragma unroll
  for (int i = 0; i < MD; ++i) {
    T g = T(0.0);
    if (i < nv) {
      if (lane < nv)
        g = s.M[i][lane];
      else if (lane < nv + nr)
        g = s.J[i][lane - nv];
      else if (lane == nv + nr)
        g = (i >= 6 ? u[i - 6] : T(0.0)) - s.bias[i];
    }
    col[i] = g;
  }
  gj_lanes<MD>(col, nv);
  __syncwarp();
  // Y over the mass matrix's storage, z in w
  if (lane >= nv && lane < nv + nr) {
#pragma unroll
    for (int i = 0; i < MD; ++i)
      if (i < nv) s.M[i][lane - nv] = col[i];
  } else if (lane == nv + nr) {
#pragma unroll
    for (int i = 0; i < MD; ++i)
      if (i < nv) s.w[i] = col[i];
  }
  __syncwarp();
  // [J'Y | -J'z - 2 alpha J'qdot] over the contact rows
  T c2[MR];
#pragma unroll
  for (int r = 0; r < MR; ++r) {
    T g = T(0.0);
    if (r < nr) {
      if (lane < nr) {
        for (int i = 0; i < nv; ++i) g += s.J[i][r] * s.M[i][lane];
      } else if (lane == nr) {
        T jz = T(0.0), jv = T(0.0);
        for (int i = 0; i < nv; ++i) {
          jz += s.J[i][r] * s.w[i];
          jv += s.J[i][r] * s.qvel[i];
        }
        g = -jz - T(2.0) * alpha * jv;
      }
    }
    c2[r] = g;
  }
  gj_lanes<MR>(c2, nr);
  if (lane == nr) {
#pragma unroll
    for (int r = 0; r < MR; ++r)
      if (r < nr) s.y[r] = c2[r] * (T)contact[r / 3];
  }
  __syncwarp();
  // v+ (in the bias storage, no longer needed)
  if (lane < nv) {
    T acc = s.w[lane];
    for (int r = 0; r < nr; ++r) acc += s.M[lane][r] * s.y[r];
    s.bias[lane] = s.qvel[lane] + acc * dt;
  }
  __syncwarp();
  if (lane < 3) xo[lane] = s.qpos[lane] + s.bias[lane] * dt;
  if (lane == 3) {  // quat * exp(w dt / 2), w in the body frame, renormalised
    const T w0 = s.bias[3], w1 = s.bias[4], w2 = s.bias[5];
    const T n2 = w0 * w0 + w1 * w1 + w2 * w2;
    const T h = T(0.5) * dt;
    T ch, k;  // cos(h |w|) and sin(h |w|) / |w|
    if (n2 > T(1e-12)) {
      const T n = sqrt_t(n2);
      T sh;
      sincos_t(h * n, &sh, &ch);
      k = sh / n;
    } else {  // the series at a vanishing rate (smooth through |w| = 0)
      ch = T(1.0) - T(0.5) * h * h * n2;
      k = h * (T(1.0) - h * h * n2 / T(6.0));
    }
    const T qr[4] = {ch, w0 * k, w1 * k, w2 * k};
    T qn[4];
    quat_mul(s.qpos + 3, qr, qn);
    quat_normalize(qn);
#pragma unroll
    for (int i = 0; i < 4; ++i) xo[3 + i] = qn[i];
  }
  for (int j = lane; j < nq - 7; j += 32) xo[7 + j] = s.qpos[7 + j] + s.bias[6 + j] * dt;
  if (lane < nv) xo[nq + lane] = s.bias[lane];
  if (lane < nr) {
    xo[nq + nv + lane] = s.cpos[lane];
    xo[nq + nv + nr + lane] = s.y[lane];
  }
}

// Passes 1-4 of the header for the configuration already in s.qpos / s.qvel:
// kinematics, dof axes, inertias, velocities, bias forces, mass matrix,
// contact points, their Jacobians and velocities, all left in s.  Every lane
// of the warp takes part.
template <class C, class T>
__device__ __forceinline__ void rb_terms(const mpxg_wb_model& m, Warp<C, T>& s, int lane) {
  constexpr int MB = C::MB;
  const unsigned full = 0xffffffffu;
  const int nb = m.nbody, nv = m.nv, nc = m.n_contact, nr = 3 * nc;
  // the tree's indices in shared memory: the chain walks below read them at
  // lane-dependent positions
  if (lane < nb) {
    s.par[lane] = m.parent[lane];
    s.jtyp[lane] = m.jnt_type[lane];
    s.dadr[lane] = m.dof_adr[lane];
  }
  __syncwarp();
  int dep = 0;
  if (lane < nb) {
    unsigned mask = 0;
    int b = lane;
    for (int g = 0; g < MB && b >= 0; ++g) {
      mask |= 1u << b;
      b = s.par[b];
      ++dep;
    }
    s.anc[lane] = mask;
    s.depth[lane] = dep - 1;
    const int jt = s.jtyp[lane];
    for (int k = 0; k < ndof(jt); ++k) s.dof_body[s.dadr[lane] + k] = lane;
  }
  __syncwarp();
  // ---- 1. forward kinematics, one tree level per step
  const int maxd = __reduce_max_sync(full, lane < nb ? dep - 1 : 0);
  for (int d = 0; d <= maxd; ++d) {
    if (lane < nb && s.depth[lane] == d) {
      const int b = lane, p = s.par[b], jt = s.jtyp[b];
      T q[4], x[3];
      if (jt == 1) {
        const T* qp = s.qpos + m.qpos_adr[b];
        x[0] = qp[0]; x[1] = qp[1]; x[2] = qp[2];
        q[0] = qp[3]; q[1] = qp[4]; q[2] = qp[5]; q[3] = qp[6];
      } else {
        T pq[4] = {T(1.0), T(0.0), T(0.0), T(0.0)}, px[3] = {T(0.0), T(0.0), T(0.0)};
        T pR[9] = {T(1.0), T(0.0), T(0.0), T(0.0), T(1.0), T(0.0), T(0.0), T(0.0), T(1.0)};
        if (p >= 0) {
#pragma unroll
          for (int i = 0; i < 4; ++i) pq[i] = s.quat[p][i];
#pragma unroll
          for (int i = 0; i < 3; ++i) px[i] = s.xp[p][i];
#pragma unroll
          for (int i = 0; i < 9; ++i) pR[i] = s.R[p][i];
        }
        T bp[3];
        mat_vec(pR, m.body_pos[b], bp);
#pragma unroll
        for (int i = 0; i < 3; ++i) x[i] = px[i] + bp[i];
        quat_mul(pq, m.body_quat[b], q);
        if (jt >= 2) {
          T Rb[9], t[3];
          quat_mat(q, Rb);
          const T qj = s.qpos[m.qpos_adr[b]];
          if (jt == 2) {  // rotate about the axis through the anchor
            T anchor[3];
            mat_vec(Rb, m.jnt_pos[b], t);
#pragma unroll
            for (int i = 0; i < 3; ++i) anchor[i] = x[i] + t[i];
            T sh, ch;
            sincos_t(T(0.5) * qj, &sh, &ch);
            const T qa[4] = {ch, sh * m.jnt_axis[b][0], sh * m.jnt_axis[b][1], sh * m.jnt_axis[b][2]};
            T qn[4];
            quat_mul(q, qa, qn);
            quat_normalize(qn);
#pragma unroll
            for (int i = 0; i < 4; ++i) q[i] = qn[i];
            quat_mat(q, Rb);
            mat_vec(Rb, m.jnt_pos[b], t);
#pragma unroll
            for (int i = 0; i < 3; ++i) x[i] = anchor[i] - t[i];
          } else {  // slide along the axis
            mat_vec(Rb, m.jnt_axis[b], t);
#pragma unroll
            for (int i = 0; i < 3; ++i) x[i] += t[i] * qj;
          }
        }
      }
      quat_normalize(q);
#pragma unroll
      for (int i = 0; i < 4; ++i) s.quat[b][i] = q[i];
#pragma unroll
      for (int i = 0; i < 3; ++i) s.xp[b][i] = x[i];
      quat_mat(q, s.R[b]);
    }
    __syncwarp();
  }
  const T o[3] = {s.xp[0][0], s.xp[0][1], s.xp[0][2]};
  // ---- 2. dof axes and body inertias about o
  if (lane < nb) {
    const int b = lane, jt = s.jtyp[b], da = s.dadr[b];
    const T* R = s.R[b];
    const T* xb = s.xp[b];
    T c[3];
    mat_vec(R, m.com[b], c);
#pragma unroll
    for (int i = 0; i < 3; ++i) c[i] += xb[i] - o[i];
    // I_world = R I R'
    const float* Il = m.inertia[b];
    T RI[9], Iw[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) RI[3 * i + k] = R[3 * i] * Il[k] + R[3 * i + 1] * Il[3 + k] + R[3 * i + 2] * Il[6 + k];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) Iw[3 * i + k] = RI[3 * i] * R[3 * k] + RI[3 * i + 1] * R[3 * k + 1] + RI[3 * i + 2] * R[3 * k + 2];
    const T ms = m.mass[b], cc = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
    T* Ib = s.Ib[b];
    Ib[0] = ms;
    Ib[1] = ms * c[0]; Ib[2] = ms * c[1]; Ib[3] = ms * c[2];
    Ib[4] = Iw[0] + ms * (cc - c[0] * c[0]);
    Ib[5] = T(0.5) * (Iw[1] + Iw[3]) - ms * c[0] * c[1];
    Ib[6] = T(0.5) * (Iw[2] + Iw[6]) - ms * c[0] * c[2];
    Ib[7] = Iw[4] + ms * (cc - c[1] * c[1]);
    Ib[8] = T(0.5) * (Iw[5] + Iw[7]) - ms * c[1] * c[2];
    Ib[9] = Iw[8] + ms * (cc - c[2] * c[2]);
    T r[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) r[i] = o[i] - xb[i];
    if (jt == 1) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        T* St = s.S[da + k];
        St[0] = St[1] = St[2] = T(0.0);
        St[3] = k == 0 ? T(1.0) : T(0.0); St[4] = k == 1 ? T(1.0) : T(0.0); St[5] = k == 2 ? T(1.0) : T(0.0);
        T* Sr = s.S[da + 3 + k];
        Sr[0] = R[k]; Sr[1] = R[3 + k]; Sr[2] = R[6 + k];
        cross3(Sr, r, Sr + 3);
      }
    } else if (jt == 2) {
      T* Sj = s.S[da];
      T t[3];
      mat_vec(R, m.jnt_axis[b], Sj);
      mat_vec(R, m.jnt_pos[b], t);
      T ra[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) ra[i] = r[i] - t[i];  // o - anchor
      cross3(Sj, ra, Sj + 3);
    } else if (jt == 3) {
      T* Sj = s.S[da];
      Sj[0] = Sj[1] = Sj[2] = T(0.0);
      mat_vec(R, m.jnt_axis[b], Sj + 3);
    }
  }
  __syncwarp();
  // ---- 3. velocities
  if (lane < nb) {
    T Vb[6] = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)};
    int b = lane;
    for (int g = 0; g < MB && b >= 0; ++g, b = s.par[b]) {
      const int nd = ndof(s.jtyp[b]), da = s.dadr[b];
      for (int k = 0; k < nd; ++k) {
        const T qd = s.qvel[da + k];
#pragma unroll
        for (int i = 0; i < 6; ++i) Vb[i] += s.S[da + k][i] * qd;
      }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) s.V[lane][i] = Vb[i];
  }
  __syncwarp();
  // accelerations at qacc = 0 and the bias force of each body
  if (lane < nb) {
    T A[6] = {T(0.0), T(0.0), T(0.0), -m.gravity[0], -m.gravity[1], -m.gravity[2]};
    int b = lane;
    for (int g = 0; g < MB && b >= 0; ++g, b = s.par[b]) {
      const int jt = s.jtyp[b], nd = ndof(jt), da = s.dadr[b];
      // the free joint's translation axes are fixed in the world: no derivative
      for (int k = (jt == 1 ? 3 : 0); k < nd; ++k) {
        T t[6];
        crm(s.V[b], s.S[da + k], t);
        const T qd = s.qvel[da + k];
#pragma unroll
        for (int i = 0; i < 6; ++i) A[i] += t[i] * qd;
      }
    }
    T IA[6], IV[6], t[6];
    inert_mul(s.Ib[lane], A, IA);
    inert_mul(s.Ib[lane], s.V[lane], IV);
    crf(s.V[lane], IV, t);
#pragma unroll
    for (int i = 0; i < 6; ++i) s.F[lane][i] = IA[i] + t[i];
  }
  __syncwarp();
  // subtree sums
  if (lane < nb) {
    T Fc[6] = {T(0.0), T(0.0), T(0.0), T(0.0), T(0.0), T(0.0)}, Ic[10];
#pragma unroll
    for (int i = 0; i < 10; ++i) Ic[i] = T(0.0);
    for (int d = lane; d < nb; ++d) {
      if ((s.anc[d] >> lane) & 1u) {
#pragma unroll
        for (int i = 0; i < 6; ++i) Fc[i] += s.F[d][i];
#pragma unroll
        for (int i = 0; i < 10; ++i) Ic[i] += s.Ib[d][i];
      }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) s.Fc[lane][i] = Fc[i];
#pragma unroll
    for (int i = 0; i < 10; ++i) s.Ic[lane][i] = Ic[i];
  }
  // contact points
  if (lane < nc) {
    const int gb = m.contact_point_body[lane];
    T t[3];
    mat_vec(s.R[gb], m.contact_point_pos[lane], t);
#pragma unroll
    for (int i = 0; i < 3; ++i) s.cpos[3 * lane + i] = s.xp[gb][i] + t[i];
  }
  __syncwarp();
  // ---- 4. bias forces, mass matrix and contact Jacobians (lane = dof)
  if (lane < nv) {
    const int j = lane, bj = s.dof_body[j];
    s.bias[j] = dot6(s.S[j], s.Fc[bj]);
    T Fj[6];
    inert_mul(s.Ic[bj], s.S[j], Fj);
    for (int i = 0; i <= j; ++i) {
      const T v = ((s.anc[bj] >> s.dof_body[i]) & 1u) ? dot6(s.S[i], Fj) : T(0.0);
      s.M[i][j] = v;
      s.M[j][i] = v;
    }
    s.M[j][j] += m.armature[j];
    for (int c = 0; c < nc; ++c) {
      T jp[3] = {T(0.0), T(0.0), T(0.0)};
      if ((s.anc[m.contact_jac_body[c]] >> bj) & 1u) {
        T r[3], t[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) r[i] = s.cpos[3 * c + i] - o[i];
        cross3(s.S[j], r, t);
#pragma unroll
        for (int i = 0; i < 3; ++i) jp[i] = s.S[j][3 + i] + t[i];
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) s.J[j][3 * c + i] = jp[i];
    }
  }
  __syncwarp();
  if (lane < nr) {
    T v = T(0.0);
    for (int j = 0; j < nv; ++j) v += s.J[j][lane] * s.qvel[j];
    s.cvel[lane] = v;
  }
  __syncwarp();
}

// The model must have passed the host checks of mpxg_wb_terms (parents
// precede children, one joint per body, the free joint only on body 0, dof and
// qpos addresses dense in body order, contacts on existing bodies) and fit the
// capacity C: nbody <= MB, nv <= MD, nq <= MD + 4, 3 x contacts <= MR.
template <int MODE, class C, class T = float>
__global__ void __launch_bounds__(32 * C::NW, C::MINB) wb_kernel(const __grid_constant__ mpxg_wb_model m, int batch,
                                                                 ArgsT<T> a) {
  constexpr int MR = C::MR;
  __shared__ Warp<C, T> sw[C::NW];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int env = blockIdx.x * C::NW + wid;
  if (env >= batch) return;  // the whole warp leaves; no block-wide barrier follows
  Warp<C, T>& s = sw[wid];
  const int nq = m.nq, nv = m.nv, nc = m.n_contact, nr = 3 * nc;
  for (int i = lane; i < nq; i += 32) s.qpos[i] = a.qpos[(size_t)env * a.sq + i];
  if (lane < nv) s.qvel[lane] = a.qvel[(size_t)env * a.sv + lane];
  __syncwarp();
  rb_terms(m, s, lane);
  if constexpr (MODE == MODE_TERMS) {
    const size_t e = (size_t)env;
    if (a.M)
      for (int i = lane; i < nv * nv; i += 32) a.M[e * nv * nv + i] = s.M[i / nv][i % nv];
    if (a.bias && lane < nv) a.bias[e * nv + lane] = s.bias[lane];
    if (a.cpos && lane < nr) a.cpos[e * nr + lane] = s.cpos[lane];
    if (a.cvel && lane < nr) a.cvel[e * nr + lane] = s.cvel[lane];
    if (a.J)
      for (int i = lane; i < nv * nr; i += 32) a.J[e * nv * nr + i] = s.J[i / nr][i % nr];
    return;
  }
  const size_t e = (size_t)env;
  if constexpr (MODE == MODE_STEP) {
    const int nx = nq + nv + 2 * nr;
    step(m, s, a.u + e * (nv - 6), a.contact + e * nc, a.dt, a.alpha, a.x_next + e * nx, lane);
    return;
  }
  // ---- the interface (mpc_utils.py:300-311)
  if (lane < nr) {
    T v = T(0.0);
    for (int q = 0; q < nr; ++q)
      v += a.Kp[lane * nr + q] * (a.foot_ref[e * nr + q] - s.cpos[q]) +
           a.Kd[lane * nr + q] * (a.foot_ref_dot[e * nr + q] - s.cvel[q]);
    s.a[lane] = v;
  }
  __syncwarp();
  // y = (J'J)^-1 a by Gauss-Jordan on [J'J | a], lane c holding column c
  T col[MR];
#pragma unroll
  for (int i = 0; i < MR; ++i) {
    T g = T(0.0);
    if (i < nr) {
      if (lane < nr) {
        for (int j = 0; j < nv; ++j) g += s.J[j][i] * s.J[j][lane];
      } else if (lane == nr) {
        g = s.a[i];
      }
    }
    col[i] = g;
  }
  gj_lanes<MR>(col, nr);
  if (lane == nr) {
#pragma unroll
    for (int i = 0; i < MR; ++i)
      if (i < nr) s.y[i] = col[i];
  }
  __syncwarp();
  if (lane < nv) {  // w = pinv(J') a = J y
    T v = T(0.0);
    for (int r = 0; r < nr; ++r) v += s.J[lane][r] * s.y[r];
    s.w[lane] = v;
  }
  __syncwarp();
  if (lane >= 6 && lane < nv) {
    const int j = lane;
    T mw = T(0.0), jg = T(0.0);
    for (int i = 0; i < nv; ++i) mw += s.M[j][i] * s.w[i];
    for (int r = 0; r < nr; ++r) jg += s.J[j][r] * a.grf[e * nr + r];
    const T fb = s.bias[j] + mw, mpc = -jg;
    const T msk = (T)a.contact[e * nc + (j - 6) / 3];
    a.tau[e * (nv - 6) + (j - 6)] = mpc * msk + (T(1.0) - msk) * fb;
  }
  if (a.J)
    for (int i = lane; i < nv * nr; i += 32) a.J[e * nv * nr + i] = s.J[i / nr][i % nr];
}

}  // namespace wb
}  // namespace mpxg
