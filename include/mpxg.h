/*
 * mpxg.h — C ABI of the GB300-native batched primal-dual iLQR MPC solver.
 *
 * This is the drop-in boundary for the solve call of iit-DLSLab/mpx:
 *
 *   optimizers.mpc(cost, dynamics, hessian_approx, limited_memory,
 *                  reference, parameter, W, x0, X0, U0, V0) -> (X, U, V)
 *
 * bound with functools.partial and jax.jit(jax.vmap(...)) at
 * mpx/utils/mpc_wrapper_srbd.py:68,77,124-132 and
 * mpx/utils/mpc_wrapper.py:74,150-158,244,346-354.  Python callables cannot
 * cross a C ABI, so the (cost, dynamics, hessian_approx) triple is selected
 * by a compiled-in model id; `limited_memory` has no counterpart (accepted and
 * ignored by the Python layer).  Everything else maps one to one onto
 * mpxg_batch_io.
 *
 * Conventions
 *  - Every pointer in mpxg_batch_io / mpxg_lq_io is a DEVICE pointer on the
 *    current CUDA device; arrays are float32, row-major, padded to n_max.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *  - Solve calls are asynchronous on `stream`, allocate nothing and never
 *    synchronise the host; all device memory is allocated in mpxg_create.
 *  - A handle is used by one host thread at a time; handles are independent.
 *  - Solves of one handle may overlap on several streams.  Each warp claims
 *    a scratch slot for the length of its launch from a pool sized for the
 *    most warps that can be resident at once, and each solve takes its own
 *    work counter from a ring of 64 (a reused entry first waits for the
 *    solve that used it last).  Solves captured into CUDA graphs take their
 *    counters from a second ring of 64 without that wait: replays of more
 *    than 64 captured solves of one handle must not overlap.
 *  - Numerical trouble does not abort a batch: it is reported per instance in
 *    status[b] (bits MPXG_INST_*), as the reference reports it through NaNs
 *    (mpx/utils/mpc_wrapper.py:96,280).
 */
#ifndef MPXG_H
#define MPXG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  MPXG_OK = 0,
  MPXG_ERR_INVALID_ARG = 1,
  MPXG_ERR_OUT_OF_MEMORY = 2,
  MPXG_ERR_BUDGET = 3,       /* admission refused: device-memory budget exhausted */
  MPXG_ERR_CUDA = 4,
  MPXG_ERR_TIMEOUT = 5,      /* a bounded wait expired */
  MPXG_ERR_NUMERICAL = 6,
  MPXG_ERR_NOT_READY = 7,    /* polled result not finished yet */
  MPXG_ERR_UNSUPPORTED = 8
} mpxg_status;

/* Compiled-in models (the reference binds them with functools.partial). */
enum {
  MPXG_MODEL_SRBD_QUAT13 = 1,   /* mpx/utils/models.py:6-37 + objectives.py:7-75 */
  MPXG_MODEL_SRBD_RPY12 = 2,    /* same body, roll-pitch-yaw state */
  MPXG_MODEL_BIPED_WRENCH12 = 3,/* two rectangular feet, 6-D wrenches */
  MPXG_MODEL_GENERIC_LQ = 4     /* per-stage LQ data (mpxg_lqr_solve) */
};

/* Per-instance status bits. */
enum {
  MPXG_INST_NAN = 1,       /* non-finite result */
  MPXG_INST_NON_PD = 2,    /* a Q_uu pivot was not positive */
  MPXG_INST_LS_FAIL = 4,   /* line search took its smallest step */
  MPXG_INST_BAD_HORIZON = 8 /* horizon[b] outside 1..n_max: instance skipped */
};

/* Problem description: fixed for the life of a handle.
 * Replaces the functools.partial bindings of mpx/utils/mpc_wrapper_srbd.py:61-66
 * (n_contact, N, mass, inertia, inertia^-1, dt). */
typedef struct {
  int model;           /* MPXG_MODEL_* */
  int n, m;            /* state / control dimension (must match the model) */
  int n_contact;
  int n_max;           /* largest horizon N of any instance */
  int batch_max;       /* largest batch per mpxg_solve call */
  float dt, mass, gravity, mu;
  float barrier_alpha, barrier_sigma;   /* relaxed friction-cone barrier, objectives.py:7 */
  float foot_length, foot_width;        /* biped foot plates */
  int barrier_kind;    /* 0: penalty() of objectives.py:7-13; 1: C2 relaxed log barrier */
  int barrier_masked;  /* 1: barrier cost applied to stance legs only */
  float barrier_hess_scale;
  float inertia[9];    /* row-major */
  float inertia_inv[9];
  float cone_eps2;     /* smoothing of the friction cone's tangential norm,
                          c = mu fz - sqrt(fx^2 + fy^2 + cone_eps2) (N^2); 0 selects
                          the reference's 1e-2 (objectives.py:29) */
} mpxg_problem_desc;

/* SQP settings (the reference's solver constants are not in its tree). */
typedef struct {
  int sqp_iters;       /* SQP iterations per solve */
  int ls_max_trials;   /* merit line-search trials */
  float ls_beta, ls_eta, reg, rho0;
  float ls_skip_tol;   /* a predicted merit decrease below ls_skip_tol * (1 + |merit|)
                          takes the full step unsearched (1e-7 recommended: larger
                          values let Gauss-Newton steps cycle near convergence) */
  int compute_kkt;     /* 1: evaluate the KKT residual of the result */
  int warps_per_block; /* 0: default (4); at most 4 */
  int blocks_per_sm;   /* 0: default (tuned) */
  int team_warps;      /* 0 or 1: one warp per instance; 4 or 8: instances whose horizon is
                          at least team_min_horizon are solved by a block of 4 or 8 warps each,
                          the KKT step split over the horizon in as many chunks (time-parallel
                          Riccati and forward sweeps); the choice depends on the horizon only,
                          so a result does not depend on the rest of its batch */
  int team_min_horizon;
  int team_exact_last; /* nonzero: the team kernel takes its last SQP iteration's KKT step as one
                          sequential sweep over the whole horizon (the one-warp kernel's accuracy
                          for the returned duals, at the latency of one sequential sweep) */
} mpxg_solver_opts;

/* One batched solve.  Layout: x0 [B,n]; X,V [B,n_max+1,n]; U [B,n_max,m];
 * reference [B,n_max+1,ref_cols]; parameter [B,n_max+1,par_cols];
 * w [B,24] = diagonal of the reference's W [B,24,24] (mpc_wrapper_srbd.py:127);
 * K [B,n_max,m,n], k [B,n_max,m]: gains of the last SQP step (optional);
 * kkt [B,3] = (r_prim, r_dual, max) (optional); status [B] (optional).
 * X_in/U_in/V_in are the warm start (X0, U0, V0 of the reference) and may
 * alias X/U/V. */
typedef struct {
  int batch;
  const int* slot;         /* [B] pool row of instance b, or NULL: row b.  Every
                              per-instance array below is indexed by that row,
                              so a batch can be any subset of a resident pool */
  const int* horizon;      /* [pool] per-instance N (1..n_max) or NULL = n_max */
  const float* x0;
  const float* X_in;
  const float* U_in;
  const float* V_in;
  const float* reference;
  const float* parameter;
  const float* w;
  float* X;
  float* U;
  float* V;
  float* K;
  float* k;
  float* kkt;
  int* status;
  float* first;            /* optional [batch, m+4], indexed by batch entry b (not by slot):
                              first control U[0], kkt[3], status -- the per-tick result
                              a controller reads back.  Each row's status entry is written
                              last, after a system-scope fence, so `first` may point into
                              mapped host memory and a reader may take a row as complete
                              once its status entry changes */
} mpxg_batch_io;

typedef struct mpxg_handle mpxg_handle;

/* Create a solver handle; all device memory is allocated here.
 * Replaces the construction of `self._solve = jax.jit(jax.vmap(work))`
 * (mpx/utils/mpc_wrapper_srbd.py:68,77). */
mpxg_status mpxg_create(const mpxg_problem_desc* desc, const mpxg_solver_opts* opts, mpxg_handle** out);
void mpxg_destroy(mpxg_handle* h);

/* Launch geometry the handle uses for mpxg_solve (persistent grid of
 * num_sms * blocks_per_sm blocks of warps_per_block warps). */
mpxg_status mpxg_query_geometry(const mpxg_handle* h, int* warps_per_block, int* blocks_per_sm, int* num_sms);

/* Device bytes mpxg_create allocates for (desc, opts). */
size_t mpxg_workspace_bytes(const mpxg_problem_desc* desc, const mpxg_solver_opts* opts);

/* Batched solve: all instances in one persistent launch.
 * Replaces self._solve(reference, parameter, W, x0, X0, U0, V0)
 * (mpx/utils/mpc_wrapper_srbd.py:124-132). */
mpxg_status mpxg_solve(mpxg_handle* h, void* stream, const mpxg_batch_io* io);

/* The plain path: one launch per instance, no batching, no graph (the
 * comparator of the batched path).  Same inputs and outputs as mpxg_solve. */
mpxg_status mpxg_solve_plain(mpxg_handle* h, void* stream, const mpxg_batch_io* io);

/* Warm start for the next control tick: X,U,V shifted by `shift` rows with the
 * last row repeated, per instance horizon (mpx/utils/mpc_wrapper_srbd.py:135-137).
 * In place is allowed (Xo == X etc.).  slot [batch] (or NULL) maps batch
 * entries to pool rows as in mpxg_batch_io. */
mpxg_status mpxg_shift_warm_start(mpxg_handle* h, void* stream, int batch, const int* slot, const int* horizon,
                                  int shift, const float* X, const float* U, const float* V, float* Xo, float* Uo,
                                  float* Vo);

/* Gait timer of a batch (mpx/utils/mpc_utils.py:7-14), float32 without fused
 * multiply-add: leg_time [B, n_legs] updated in place, contact [B, n_legs]. */
/* Vector-Jacobian product of converged solutions (the differentiable solve;
 * the reference describes its solver as differentiable, README.md:26-27).
 * At the solution X, U (with the duals V, as returned by mpxg_solve) the
 * implicit-function theorem on the Gauss-Newton KKT system the solve factors
 * gives, for cotangents gX [B,n_max+1,n], gU [B,n_max,m] of a scalar loss:
 *   wX, wU, wL  the adjoint solution (H w + A'mu = g, A w = 0, dx_0 = 0;
 *               wL the costates of that system, [B,n_max+1,n])
 *   gx0 [B,n]   dLoss/dx0 = mu_0
 *   gref [B,n_max+1,12]  dLoss/dreference for the 12 tracked state columns
 *               (models with an identity tracking residual: roll-pitch-yaw
 *               quadruped, biped), = W * wX.
 * Any output pointer may be NULL.  Same handle, batch layout and slots as
 * mpxg_solve; K, k, kkt, first and V_in of mpxg_batch_io are ignored. */
typedef struct {
  mpxg_batch_io io;        /* x0, X_in (= X), U_in (= U), V_in, reference, parameter, w, horizon, slot, batch */
  const float* gX;
  const float* gU;
  float *wX, *wU, *wL, *gx0, *gref;
} mpxg_vjp_io;
mpxg_status mpxg_solve_vjp(mpxg_handle* h, void* stream, const mpxg_vjp_io* v);

/* Cost and constraint residuals of trajectories X [batch, n_max+1, n], U
 * [batch, n_max, m] with the handle's model (replaces
 * optimizers.model_evaluator_helper(cost, dynamics, x0, X, U) -> (g, c),
 * called at mpx/utils/mpc_wrapper.py:419-423,452-465):
 *   g [batch, n_max+1]     g[b,t] = l_t, the cost of stage t (terminal cost
 *                          at t = N; may be negative with the relaxed log
 *                          barrier), so sum(g) is the objective;
 *   c [batch, n_max+1, n]  c[b,0] = x0 - X[0], c[b,t] = f(X[t-1], U[t-1]) - X[t],
 *                          so sum(c^2) is the reference's constraint figure.
 * Rows past horizon[b] (n_max when horizon is NULL) are zero. */
mpxg_status mpxg_evaluate(mpxg_handle* h, void* stream, int batch, const int* horizon, const float* x0,
                          const float* X, const float* U, const float* reference, const float* parameter,
                          const float* w, float* g, float* c);

/* Opaque operand of the XLA custom call below. */
typedef struct {
  mpxg_problem_desc desc;
  mpxg_solver_opts opts;
  int batch;
  int reserved;
} mpxg_xla_opaque;

/* XLA custom-call target (status-returning custom-call signature: stream,
 * buffers, opaque, opaque_len, XlaCustomCallStatus*), so a JAX program can
 * keep the solve inside jax.jit as the reference does with
 * jax.jit(jax.vmap(optimizers.mpc ...)) (mpx/utils/mpc_wrapper_srbd.py:68,77).
 * buffers: reference, parameter, w (the diagonal [B,24] of W), x0, X0, U0, V0,
 * then the results X, U, V, in the reference's argument order.  All horizons
 * are desc.n_max.  The call allocates nothing: it uses the handle that
 * mpxg_xla_prepare made for (current device, opaque), and fails when there is
 * none.  Errors go to XlaCustomCallStatusSetFailure when the host process
 * exports it, and to mpxg_last_error(NULL). */
void mpxg_xla_solve(void* stream, void** buffers, const char* opaque, size_t opaque_len, void* status);
/* Creates (once) the handle of (current device, opaque) that the XLA targets
 * use, so that device memory is allocated when the program is built rather
 * than inside the custom call (where XLA may be capturing a command buffer).
 * Replaces the one-time jit compilation of the solve,
 * jax.jit(jax.vmap(partial(optimizers.mpc, ...))) (mpx/utils/mpc_wrapper_srbd.py:68,77).
 * Call it with each device the program runs on current. */
mpxg_status mpxg_xla_prepare(const char* opaque, size_t opaque_len);
/* XLA custom-call target of the backward pass (mpxg_solve_vjp): buffers
 * reference, parameter, w, x0, X, U, V (the solution), gX, gU (cotangents),
 * then the results gx0 [B,n] and gref [B,N+1,12].  Same opaque and prepared
 * handle as mpxg_xla_solve. */
void mpxg_xla_solve_vjp(void* stream, void** buffers, const char* opaque, size_t opaque_len, void* status);

mpxg_status mpxg_timer_run(void* stream, int batch, int n_legs, float duty_factor, float step_freq, float dt,
                           float* leg_time, int* contact);

/* SRBD reference generator (mpx/utils/mpc_utils.py:146-270, path with
 * use_terrain_estimator = False) for a batch.  Inputs [B,...]: t_timer [B,4],
 * x [B,13], foot [B,12], input [B,7], contact [B,4], liftoff [B,12] (in/out).
 * Outputs: reference [B,N+1,17], parameter [B,N+1,16], foot_ref_dot [B,N+1,12]
 * (row stride n_max+1 when n_max > N). */
mpxg_status mpxg_refgen_srbd(void* stream, int batch, int N, int n_max, float dt, const float* foot0,
                             float duty_factor, float step_freq, float step_height, float clearence_speed,
                             const float* t_timer, const float* x, const float* foot, const float* input,
                             const float* contact, float* liftoff, float* reference, float* parameter,
                             float* foot_ref_dot);

/* Whole-body reference generator (mpx/utils/mpc_utils.py:15-145,
 * reference_generator, with terrain_orientation when use_terrain_estimation)
 * for a batch of quadrupeds with 4 contact points.  Inputs [B,...]: t_timer
 * [B,4], x [B,13+2nj+24] (the whole-body state), foot [B,12], input [B,7],
 * contact [B,4], liftoff [B,12] (in/out); foot0 [12] and q0 [nj] are host
 * arrays, mass the robot's mass (the reference's qM[0]).  Outputs:
 * reference [B,N+1,13+nj+28] rows [p, quat, q0, dp, omega, feet, contact,
 * forces] and parameter [B,N+1,4] (the contact sequence). */
mpxg_status mpxg_refgen_wb(void* stream, int batch, int N, int n_joints, float dt, float mass, const float* foot0,
                           const float* q0, float duty_factor, float step_freq, float step_height,
                           float clearence_speed, int use_terrain_estimation, const float* t_timer, const float* x,
                           const float* foot, const float* input, const float* contact, float* liftoff,
                           float* reference, float* parameter);

/* Gait tables of the synthetic trot / walk workloads, one warp per batch
 * entry and a lane per stage (row slot[b] of every per-instance array, or
 * row b when slot is NULL):
 *   mode 0 (first tick): x0 as given, timers as given; the warm start is
 *          initialised (X = x0 at every stage, V = 0, U = `weight` split over
 *          the legs in stance at each stage);
 *   mode 1 (next tick):  x0 = X[b,0,:] + drift (X already shifted), drift
 *          ~ N(0, drift_std^2) from a counter-based hash of (seed, row, i);
 *          one gait-timer step of leg_time;
 *   mode 2 (next tick, measured state): x0 as given (e.g. copied from the
 *          host), one gait-timer step of leg_time, warm start kept.
 * Then for t = 0..horizon the contact flags from t+1 further timer steps (the
 * schedule rule of mpx/utils/mpc_utils.py:187-189), a CoM reference moving at
 * v_ref along x at constant `height` with zero attitude and rate, and feet at
 * `offsets` (legs x 3) from the CoM reference. */
typedef struct {
  int model, batch, n_max, mode;
  const int* slot;
  const int* horizon;
  float dt, duty_factor, step_freq, height, weight, drift_std;
  unsigned int seed;
  float offsets[12];
  float *x0, *X, *U, *V;
  const float* v_ref;
  float* leg_time;
  float *reference, *parameter;
} mpxg_gait_args;
mpxg_status mpxg_gait_tables(void* stream, const mpxg_gait_args* args);

/* Device work queue (continuous batching without a launch per batch): one
 * persistent SQP kernel on `stream` drains a queue that the host fills while
 * it runs.  `pool` describes the instances the queue may solve (as for
 * mpxg_solve, pool->batch rows, no slot map; pool->first is ignored): the
 * host updates a row's inputs, then mpxg_queue_push(row) publishes it; the
 * kernel solves it exactly as mpxg_solve's one-warp kernels would and flags
 * it done, and mpxg_queue_result copies its result row (m controls, the KKT
 * triple, the status) to the host.  The ring holds `capacity` tickets: a
 * push whose ring entry still holds an unfinished ticket returns
 * MPXG_ERR_NOT_READY.  Every wait of the kernel is bounded: a warp waiting
 * longer than idle_timeout_ns (1 ms .. 60 s, %globaltimer) for work gives up,
 * and the queue then reports MPXG_ERR_TIMEOUT (push, result, finish) instead
 * of hanging.  mpxg_queue_finish lets the kernel drain what was pushed,
 * waits for it, frees the queue and returns MPXG_ERR_TIMEOUT if a wait ran
 * out.  Stands in for the reference's one-call-per-tick loop
 * (mpx/utils/mpc_wrapper.py:297-365). */
typedef struct mpxg_queue mpxg_queue;
mpxg_status mpxg_queue_start(mpxg_handle* h, void* stream, const mpxg_batch_io* pool, int capacity,
                             long long idle_timeout_ns, mpxg_queue** out);
mpxg_status mpxg_queue_push(mpxg_queue* q, int row, long long* ticket);
mpxg_status mpxg_queue_result(mpxg_queue* q, long long ticket, float* row_out);
mpxg_status mpxg_queue_finish(mpxg_queue* q);

/* One persistent SQP launch over the batches of two handles of different
 * models, so that a mix of robot models takes a single solve launch (the
 * served stream's quadrupeds and bipeds; the reference serves one model per
 * optimizers.mpc call, mpx/utils/mpc_wrapper_srbd.py:124-132).  Built pairs
 * (a, b): (MPXG_MODEL_SRBD_RPY12, MPXG_MODEL_BIPED_WRENCH12) and
 * (MPXG_MODEL_SRBD_QUAT13, MPXG_MODEL_BIPED_WRENCH12); the handles must
 * share n_max and the device and stay alive while the mixed handle is used.
 * Each instance is solved by one warp with its own handle's model and
 * options, in the same order of operations as mpxg_solve's one-warp kernels
 * (the time-parallel team path is not used), so a result does not depend on
 * the mix it was solved in.  The queue serves the longest horizons of both
 * batches first when both carry horizons.  io_a / io_b as for mpxg_solve on
 * a / b (either batch may be 0).  The mixed handle owns its own scratch:
 * mpxg_mixed_create allocates, mpxg_solve_mixed does not. */
typedef struct mpxg_mixed mpxg_mixed;
mpxg_status mpxg_mixed_create(mpxg_handle* a, mpxg_handle* b, mpxg_mixed** out);
void mpxg_mixed_destroy(mpxg_mixed* mx);
mpxg_status mpxg_solve_mixed(mpxg_mixed* mx, void* stream, const mpxg_batch_io* io_a, const mpxg_batch_io* io_b);

/* Time-varying LQR in absolute coordinates for a batch (isolated KKT/LQR):
 * x_{t+1} = A_t x_t + B_t u_t + c_t, cost 1/2 x'Qx + x'Mu + 1/2 u'Ru + q'x + r'u,
 * terminal Q[N], q[N].  A [B,N,n,n], Bm [B,N,n,m], c [B,N,n], Q [B,N+1,n,n],
 * R [B,N,m,m], M [B,N,n,m], q [B,N+1,n], r [B,N,m], x0 [B,n].
 * Outputs K [B,N,m,n], k [B,N,m], X [B,N+1,n], U [B,N,m], lam [B,N+1,n]
 * (costates dV_t/dx_t).  `method`: 0 sequential Riccati (one block per
 * problem); 1 time-parallel associative scan of the value-function recursion
 * over 8 horizon chunks (one 8-warp block per problem).  Built sizes (n, m):
 * (24,12) (12,12) (8,4) (4,2).  Stands in for the LQR/KKT step of the absent
 * primal_dual_ilqr solver (parallel in time, README.md:23-24,29). */
typedef struct {
  int batch, N, n, m;
  const float *A, *Bm, *c, *Q, *R, *M, *q, *r, *x0;
  float *K, *k, *X, *U, *lam;
  float* workspace;  /* device, >= mpxg_lqr_workspace_bytes(batch, N, n, m, method) bytes */
} mpxg_lq_io;
size_t mpxg_lqr_workspace_bytes(int batch, int N, int n, int m, int method);
mpxg_status mpxg_lqr_solve(void* stream, const mpxg_lq_io* io, int method);

/* Equality-constrained time-varying LQR for a batch (the LQ/KKT step of
 * large linearised problems; stands in for the absent primal_dual_ilqr
 * solver's KKT solve, as mpxg_lqr_solve does):
 *   x_{t+1} = A x + B u + c,  C x + D u = e (n_eq rows),  cost as mpxg_lq_io.
 * A [B,N,n,n], Bm [B,N,n,m], c [B,N,n], Q [B,N+1,n,n], R [B,N,m,m],
 * M [B,N,n,m], q [B,N+1,n], r [B,N,m], C [B,N,n_eq,n], D [B,N,n_eq,m],
 * e [B,N,n_eq], x0 [B,n].  Outputs K [B,N,m,n], k [B,N,m], Knu [B,N,n_eq,n],
 * knu [B,N,n_eq] (u = K x + k, nu = Knu x + knu), X [B,N+1,n], U [B,N,m],
 * lam [B,N+1,n] (costates), nu [B,N,n_eq] (multipliers of C x + D u = e,
 * stationarity l_u + B'lam_{t+1} + D'nu = 0).  D must have full row rank and
 * R + B'P B be positive definite.  Built sizes (n, m, n_eq): (72,30,12)
 * (16,8,4) (8,5,2). */
typedef struct {
  int batch, N, n, m, n_eq;
  const float *A, *Bm, *c, *Q, *R, *M, *q, *r, *C, *D, *e, *x0;
  float *K, *k, *Knu, *knu, *X, *U, *lam, *nu;
  float* workspace;  /* device, >= mpxg_lqr_eq_workspace_bytes(batch, N, n) bytes, 16-byte aligned */
} mpxg_lq_eq_io;
size_t mpxg_lqr_eq_workspace_bytes(int batch, int N, int n);
mpxg_status mpxg_lqr_eq_solve(void* stream, const mpxg_lq_eq_io* io);
/* The same solve with the stage products' engine chosen: method 0 (what
 * mpxg_lqr_eq_solve runs) puts the Riccati stage's dense products on the
 * tensor cores (tcgen05, split-TF32: three TF32 MMAs per float32 product,
 * float32 accumulation in tensor memory); method 1 runs every product on
 * the CUDA cores in float32.  A product that does not finish within a
 * bounded wait leaves that problem's X non-finite. */
mpxg_status mpxg_lqr_eq_solve_method(void* stream, const mpxg_lq_eq_io* io, int method);

/* SQP iterations on the equality-constrained LQ problem of `lq` (config 4's
 * large linearised problems through the SQP path of optimizers.mpc,
 * mpx/utils/mpc_wrapper_srbd.py:124-132; solver module absent from the
 * reference tree).  Each iteration forms the step problem at the iterate
 * (defects c' = A x + B u + c - x+, gradients q' = Q x + M u + q,
 * r' = M'x + R u + r, constraint residuals e' = e - C x - D u, x0 - x_0),
 * solves it with mpxg_lqr_eq_solve_method (`method`) and takes the full step
 * (the problem is linear-quadratic: the Newton step is exact, and a second
 * iteration refines float32's rounding).  lq.X [B,N+1,n] and lq.U [B,N,m]
 * hold the starting iterate on entry and the result on return; lq.lam,
 * lq.nu, lq.K, lq.k, lq.Knu, lq.knu receive the multipliers and gains of
 * the last step; lq.workspace as for mpxg_lqr_eq_solve.  kkt (optional)
 * [B,3] = (primal residual, dual residual / (1 + max |gradient|), max) of
 * the result.  iters = 0 only evaluates kkt at the caller's X, U, lam, nu.
 * step: device workspace of
 * mpxg_lqr_eq_sqp_workspace_bytes(batch, N, n, m, n_eq) bytes. */
typedef struct {
  mpxg_lq_eq_io lq;
  int iters;
  int method;
  float* kkt;
  float* step;
} mpxg_lq_eq_sqp_io;
size_t mpxg_lqr_eq_sqp_workspace_bytes(int batch, int N, int n, int m, int n_eq);
mpxg_status mpxg_lqr_eq_sqp(void* stream, const mpxg_lq_eq_sqp_io* io);

/* Allocation-free batched solve.  No counterpart in the reference.  For
 * callers that cannot allocate device memory when they solve (a real-time
 * loop that forbids cudaMalloc after start-up, or a plugin host that hands
 * over only input and output buffers): no handle, same inputs and outputs as
 * mpxg_solve, scratch taken from a 64 MiB static device array that every GPU
 * loading this library holds until exit.  The array must hold one warp's
 * scratch per SM, else the call is rejected (MPXG_ERR_INVALID_ARG; on a
 * 152-SM GB300 n_max up to 141 for the roll-pitch-yaw quadruped, 135 for the
 * biped, 116 for the quaternion model).  All calls share that array: calls
 * that overlap on the GPU race, so serialise them on one stream.  The first call on a device looks up the
 * array's device address; make it before any stream capture.  That address is
 * kept for the life of the process, so after a cudaDeviceReset the entry point
 * must not be called again in that process.  warps_per_block is 0..4, as for
 * mpxg_create.  Errors are reported through mpxg_last_error(NULL). */
mpxg_status mpxg_solve_noalloc(const mpxg_problem_desc* desc, const mpxg_solver_opts* opts, void* stream,
                               const mpxg_batch_io* io);

/* ---------------------------------------------------------------- serving
 * A served MPC stream: each request is one control tick of a persistent
 * episode (a robot).  The server keeps every admitted episode's warm start
 * (X, U, V), gait timers, horizon and weights resident on the device in
 * per-model slot pools sized by a device-memory budget; a tick moves only the
 * batch's slot ids in and one result row out.  Requests submitted while
 * earlier batches run form the next batch, launched on the next of `streams`
 * CUDA streams (continuous batching): per batch, the warm-start shift and
 * gait tables of its episodes (cold start for new episodes and after a
 * non-finite result, the NaN fallback of mpx/utils/mpc_wrapper.py:79-98), one
 * persistent solve over their scattered slots, and one copy of the result
 * rows.  No counterpart in the reference, which solves one fixed batch per
 * call (mpx/utils/mpc_wrapper_srbd.py:91-141).
 * Single-threaded: one host thread drives a server. */
typedef struct {
  mpxg_problem_desc desc;   /* n_max and batch_max are set by the server */
  float duty_factor, step_freq, height;
  float offsets[12];        /* foot offsets from the CoM reference, per leg (x, y, z) */
  float phase0[4];          /* gait timer of each leg at phase 0 */
  float w[24];              /* diagonal cost weights */
} mpxg_served_model;

typedef struct {
  int n_models;
  const mpxg_served_model* models;
  int n_max;                /* longest horizon of any episode */
  size_t budget_bytes;      /* device memory for slots + solver scratch, split evenly over the models */
  int max_slots;            /* cap per model (0: as many as the budget allows) */
  int streams;              /* concurrent batches (CUDA streams) */
  float drift_std;          /* per-tick state drift N(0, drift_std^2) added on the device */
  unsigned int seed;
  mpxg_solver_opts opts;
  int mixed_launch;         /* nonzero (two models of a built mpxg_mixed pair): each step solves both
                               models' ticks in one mixed-model launch; its scratch comes off the budget */
} mpxg_server_desc;

typedef struct {
  long long ticket;
  int episode;
  int status;               /* MPXG_INST_* bits */
  float u0[12];             /* first control of the solution (m entries used) */
  float kkt[3];             /* r_prim, r_dual, max */
} mpxg_result;

typedef struct mpxg_server mpxg_server;

mpxg_status mpxg_server_create(const mpxg_server_desc* desc, mpxg_server** out);
void mpxg_server_destroy(mpxg_server* s);
/* Slots of model `model` (the number of episodes it can hold at once). */
int mpxg_server_capacity(const mpxg_server* s, int model);
/* Admit an episode: x0 [n] (host), horizon 1..n_max, forward speed v_ref,
 * gait phase offset.  Returns its id in *episode, or MPXG_ERR_BUDGET when the
 * model's slots are all taken.  Its first tick cold-starts on the device. */
mpxg_status mpxg_server_admit(mpxg_server* s, int model, const float* x0, int horizon, float v_ref, float phase,
                              int* episode);
/* Cold-start the episode's next tick (from a new x0 when x0 is not NULL). */
mpxg_status mpxg_server_reset(mpxg_server* s, int episode, const float* x0);
/* Free the episode's slot once its queued and running ticks are done. */
mpxg_status mpxg_server_release(mpxg_server* s, int episode);
/* Queue the episode's next control tick; *ticket identifies its result. */
mpxg_status mpxg_submit(mpxg_server* s, int episode, long long* ticket);
/* Queue the next tick of n episodes at once (tickets[i] for episodes[i]);
 * stops at the first failing episode and returns its status (tickets of the
 * queued ones are set). */
mpxg_status mpxg_submit_many(mpxg_server* s, const int* episodes, int n, long long* tickets);
/* Collect finished batches and launch queued ticks on free streams (one tick
 * per episode in flight at a time).  Never blocks; `block` != 0 waits for the
 * oldest running batch first.  *launched / *finished (may be NULL): ticks
 * launched / completed by this call. */
mpxg_status mpxg_server_step(mpxg_server* s, int block, int* launched, int* finished);
/* The result of `ticket` (MPXG_ERR_NOT_READY until its batch finished; a
 * result is returned once). */
mpxg_status mpxg_poll(mpxg_server* s, long long ticket, mpxg_result* result);
/* Results finished since the last call, up to `max`; *count set. */
mpxg_status mpxg_server_completed(mpxg_server* s, mpxg_result* results, int max, int* count);
/* Ticks queued, running; kernel launches issued so far. */
mpxg_status mpxg_server_stats(const mpxg_server* s, int* queued, int* running, long long* launches);
const char* mpxg_server_last_error(const mpxg_server* s);

/* ---------------------------------------------------------------- whole body
 * Rigid-body terms of a floating-base kinematic tree (an MJCF model parsed on
 * the host: mpx_gb300/mjcf.py) and the whole-body torque interface of the SRBD
 * controller (mpx/utils/mpc_utils.py:275-313, bound per environment at
 * mpx/utils/mpc_wrapper_srbd.py:73,80 and called by whole_body_run at
 * :153-154).  MuJoCo's conventions: qpos = [free joint position (3), unit
 * quaternion w,x,y,z (4), hinge / slide coordinates], qvel = [world linear
 * velocity of the free body's origin (3), its angular velocity in its own
 * frame (3), joint rates]; a hinge rotates its body about the joint axis
 * through the joint anchor.  Bodies are listed parents first. */
#define MPXG_WB_MAX_BODY 32
#define MPXG_WB_MAX_DOF 32
#define MPXG_WB_MAX_CONTACT 8
typedef struct {
  int nbody, nq, nv, n_contact;
  int parent[MPXG_WB_MAX_BODY];    /* -1 = attached to the world */
  int jnt_type[MPXG_WB_MAX_BODY];  /* 0 none (welded), 1 free (root only), 2 hinge, 3 slide */
  int qpos_adr[MPXG_WB_MAX_BODY], dof_adr[MPXG_WB_MAX_BODY];
  float body_pos[MPXG_WB_MAX_BODY][3], body_quat[MPXG_WB_MAX_BODY][4]; /* in the parent frame */
  float jnt_pos[MPXG_WB_MAX_BODY][3], jnt_axis[MPXG_WB_MAX_BODY][3];   /* in the body frame, axis unit */
  float mass[MPXG_WB_MAX_BODY], com[MPXG_WB_MAX_BODY][3];             /* com in the body frame */
  float inertia[MPXG_WB_MAX_BODY][9]; /* about the com, body frame, row-major */
  float armature[MPXG_WB_MAX_DOF];    /* added to the mass matrix diagonal */
  float gravity[3];
  /* contact point c: a point fixed in body contact_point_body[c] at
   * contact_point_pos[c] (the MJCF geom), differentiated as attached to
   * body contact_jac_body[c] (mjx.jac's body argument) */
  int contact_point_body[MPXG_WB_MAX_CONTACT], contact_jac_body[MPXG_WB_MAX_CONTACT];
  float contact_point_pos[MPXG_WB_MAX_CONTACT][3];
} mpxg_wb_model;

/* Per environment b (device arrays, row-major): qpos [B,nq], qvel [B,nv] ->
 *   M [B,nv,nv]      joint-space inertia with armature (mjx_data.qM),
 *   bias [B,nv]      Coriolis, centrifugal and gravity forces at qacc = 0
 *                    (mjx_data.qfrc_bias; passive forces excluded),
 *   cpos [B,3C]      contact point positions (geom_xpos of the contacts),
 *   J [B,nv,3C]      translational Jacobians of the contact points, column
 *                    block c = mjx.jac(..)[0] of contact c,
 *   cvel [B,3C]      J' qvel.
 * Any output may be NULL.  One warp per environment. */
mpxg_status mpxg_wb_terms(void* stream, const mpxg_wb_model* model, int batch, const float* qpos,
                          const float* qvel, float* M, float* bias, float* cpos, float* J, float* cvel);

/* The whole-body interface (mpc_utils.py:276-313) for a batch:
 *   a   = Kp (foot_ref - cpos) + Kd (foot_ref_dot - J' qvel)
 *   tau = (-(J grf))[6:] where contact, (bias + M pinv(J') a)[6:] elsewhere,
 * with the mask of joint i = contact[i / 3]; requires nv = 6 + 3C with a
 * free root.  grf, foot_ref, foot_ref_dot [B,3C]; contact [B,C] (int);
 * Kp, Kd [3C,3C] shared by all environments.  Outputs tau [B,nv-6] and, if
 * J is not NULL, J [B,nv,3C].  pinv(J') a is J (J'J)^-1 a (J' of full row
 * rank, which a leg away from a kinematic singularity gives). */
mpxg_status mpxg_wb_interface(void* stream, const mpxg_wb_model* model, int batch, const float* qpos,
                              const float* qvel, const float* grf, const float* foot_ref,
                              const float* foot_ref_dot, const int* contact, const float* Kp, const float* Kd,
                              float* tau, float* J);

/* One step of the whole-body MPC model of the reference's whole-body
 * configurations (quadruped_wb_dynamics, mpx/utils/models.py:39-117; bound at
 * config_aliengo.py:68, config_go2.py:69) for a batch:
 *   x [B, nq + nv + 6C] = [qpos, qvel, contact points, contact forces],
 *   u [B, nv - 6] joint torques, contact [B, C] (int, the reference's
 *   parameter[t, :C]) ->
 *   x_next [B, nq + nv + 6C] = [qpos+, qvel+, contact points at x, forces],
 * with forces f from (J'M^-1 J) f = -J'M^-1 (tau - bias) - 2 alpha J'qdot
 * (alpha = 25 in the reference), masked by contact, then
 * qvel+ = qvel + M^-1 (tau - bias + J f) dt and a semi-implicit Euler step of
 * qpos (the free joint's quaternion by its body-frame rate).  Requires a free
 * root, hinge or slide joints elsewhere, 3C <= nv and nv + 3C + 1 <= 32.  The
 * contact-point and force entries of x are not read. */
mpxg_status mpxg_wb_step(void* stream, const mpxg_wb_model* model, int batch, float dt, float alpha, const float* x,
                         const float* u, const int* contact, float* x_next);

/* SQP iterations of the whole-body MPC for a batch: the solve that
 * mpc_wrapper.py's wrappers run each tick (self._solve / self.work,
 * mpc_wrapper.py:150-158 and 346-354, built at :67 and :236 from
 * config_aliengo.py / config_go2.py: quadruped_wb_dynamics,
 * quadruped_wb_obj(True, ...), quadruped_wb_hessian_gn(True, ...)), standing
 * in for the absent optimizers.mpc as mpxg_solve does for the SRBD model.
 * x = [qpos, qvel, contact points (3C), contact forces (3C)] (nx = nq + nv +
 * 6C), u = joint torques (nj = nv - 6).  One iteration at (X, U, V):
 *   defects c_0 = x0 - X_0, c_{t+1} = f(X_t, U_t, contact_t) - X_{t+1}
 *     (f = mpxg_wb_step's model, evaluated in float64);
 *   Jacobians of f over qpos, qvel and u by forward-mode differentiation of
 *     the step in float32 (exact up to rounding; f does not read the point
 *     and force states);
 *   the cost's exact gradient and the reference's Gauss-Newton blocks
 *     (objectives.py:77-203), reg added to the control block;
 *   the step by a float32 Riccati sweep (one 256-thread block per instance);
 *   the merit line search of mpxg_solve (augmented-Lagrangian merit, rho
 *     raised to 2 G / |c|^2, Armijo with eta, steps beta^k for k <
 *     ls_max_trials evaluated together, the first accepted one taken), merit
 *     terms in float64;
 *   X += a dX, U += a dU, V += a (lam - V).
 * x0 [B,nx]; X [B,N+1,nx], U [B,N,nj], V [B,N+1,nx]: the warm start in, the
 * result out (float32); reference [B,N+1,13+nj+7C] (the whole-body reference
 * rows: p, quat, q, v, omega, foot positions, contact, forces); contact
 * [B,N+1,C] int (the dynamics' mask, parameter[t,:C]); W [B,12+3nj+6C] (the
 * diagonal of the reference's block-diagonal W).  Optional outputs: kkt
 * [B,3] (primal max |c|, dual residual / (1 + max |gradient|), their max) at
 * the result, status [B] (MPXG_INST_* bits).  iters = 0 only evaluates kkt.
 * Built size: nv = 18 with 4 contact points (nx = 61, nj = 12: the aliengo
 * and go2 configurations); the model must pass mpxg_wb_step's checks.
 * workspace: device, >= mpxg_wb_sqp_workspace_bytes(model, batch, N) bytes,
 * 256-byte aligned.  No allocation, no host synchronisation. */
typedef struct {
  const mpxg_wb_model* model; /* host pointer */
  int batch, N, iters;
  float dt, alpha;            /* step and Baumgarte gain (25 in the reference) */
  int swing_tracking;         /* quadruped_wb_obj's first argument (True in both configs) */
  float reg, rho0, ls_beta, ls_eta, ls_skip_tol;
  int ls_max_trials;          /* 1..8 */
  const float* x0;
  float *X, *U, *V;
  const float* reference;
  const int* contact;
  const float* W;
  float* kkt;
  int* status;
  void* workspace;
} mpxg_wb_sqp_io;
size_t mpxg_wb_sqp_workspace_bytes(const mpxg_wb_model* model, int batch, int N);
mpxg_status mpxg_wb_sqp(void* stream, const mpxg_wb_sqp_io* io);

/* Last error message of a handle (or of the library when h is NULL). */
const char* mpxg_last_error(const mpxg_handle* h);
const char* mpxg_status_string(int status);
int mpxg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MPXG_H */
