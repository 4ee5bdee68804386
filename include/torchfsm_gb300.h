/*
 * torchfsm_gb300 C ABI: Fourier-spectral ETD time stepping on one GB300 (sm_103a).
 *
 * Plain C: every argument is a pointer, an integer, a double or a stream
 * handle (cudaStream_t passed as void*). No C++ types or exceptions cross
 * this boundary. Every entry point returns an FSM_* status; the message of
 * the last failure on the calling host thread is read with fsm_last_error.
 *
 * Conventions
 *  - Spectral fields are "half spectra": the transform over all spatial axes,
 *    with the last axis kept for k = 0..n/2 only (the real-to-complex layout).
 *    A field of a mesh (n0, .., n_{d-1}) holds S = n0*..*n_{d-2}*(n_{d-1}/2+1)
 *    complex64 values, row-major; arrays are [batch][channel][S].
 *  - The forward transform is unnormalised and the inverse carries 1/(n0*..)
 *    (torch's "backward" norm), so half spectra equal the reference's
 *    torch.fft.fftn output restricted to the last axis' first n/2+1 entries.
 *  - Every buffer is allocated by the caller (device memory unless stated).
 *    A plan owns only its constant tables (coefficients, wavenumbers, masks,
 *    twiddles), is immutable after creation and may be used from several
 *    host threads on different streams; workspaces are per call.
 *  - All work is launched asynchronously on the given stream.
 *  - Mesh sizes: powers of two, 16..4096 points in 1D, 16..512 per axis in
 *    2D. Other programs/sizes return FSM_ERR_UNSUPPORTED.
 *
 * Reference interfaces replaced (torchfsm 0.0.4, paths in the torchfsm tree):
 *  fsm_plan_create   OperatorLike._build_integrator / register_mesh linear-coefficient
 *                    precompute: operator/_base.py:339-357, 441-526;
 *                    UnCachedSETDRK1..4.__init__ integrator/_stable_etdrk/_uncached.py:46-211;
 *                    ETDRK0..2.__init__ integrator/_etdrk.py:10-82
 *  fsm_integrate     OperatorLike.integrate step loop operator/_base.py:726-746 with
 *                    setdrk*_step integrator/_stable_etdrk/_setdrk_step.py:5-82, the
 *                    nonlinear closure operator/_base.py:375-403 and the recorder
 *                    traj_recorder.py:46-55
 *  fsm_rfftn/irfftn  FourierMesh.fft / ifft(...).real mesh.py:481-491
 */
#ifndef TORCHFSM_GB300_H
#define TORCHFSM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FSM_OK 0
#define FSM_ERR_INVALID 1      /* bad argument */
#define FSM_ERR_UNSUPPORTED 2  /* program or size without a fused kernel */
#define FSM_ERR_CUDA 3         /* a CUDA call failed */
#define FSM_ERR_OOM 4          /* device allocation failed */
#define FSM_ERR_NONFINITE 5    /* a result holds NaN or Inf (reserved: fsm_nonfinite_flags reports it per field) */
#define FSM_ERR_TIMEOUT 6      /* a bounded device wait ran out (reserved: no kernel here waits on a device flag) */

/* nonlinear term of the program (at most one, plus an optional explicit source) */
#define FSM_NL_NONE 0        /* linear, or explicit source only */
#define FSM_NL_CONVECTION 1  /* (u.grad)u, C == ndim (operator/generic/_convection.py:18-46) */
#define FSM_NL_VORTICITY 2   /* u.grad(w) with u from the streamfunction, 2D, C == 1
                                (operator/dedicated/_navier_stokes.py:27-46) */
#define FSM_NL_KS 3          /* 0.5 |grad phi|^2, C == 1 (operator/dedicated/_ks_convection.py:18-38) */
#define FSM_NL_LERAY 4       /* -grad p - (u.grad)u, C == ndim (operator/dedicated/_navier_stokes.py:231-254) */

/* program flags */
#define FSM_FLAG_REMOVE_MEAN 1 /* FSM_NL_KS: subtract the mean over the whole batch */

/* integrators (integrator/_etdrk.py, integrator/_stable_etdrk/) */
#define FSM_ETDRK0 0
#define FSM_ETDRK1 1
#define FSM_ETDRK2 2
#define FSM_SETDRK1 11
#define FSM_SETDRK2 12
#define FSM_SETDRK3 13
#define FSM_SETDRK4 14
/* explicit Runge-Kutta on the full right-hand side L u + N(u), fixed step
   (integrator/_rk.py:43-58 _rk_step; tableaus :82-255) */
#define FSM_RK_EULER 21
#define FSM_RK_MIDPOINT 22
#define FSM_RK_HEUN12 23
#define FSM_RK_RALSTON12 24
#define FSM_RK_BOGACKI_SHAMPINE23 25
#define FSM_RK4 26
#define FSM_RK4_38RULE 27
#define FSM_RK_DORPI45 28
#define FSM_RK_FEHLBERG45 29
#define FSM_RK_CASHKARP45 30
/* one evaluation of the right-hand side: a 1-step integrate overwrites the state with
   L u + N(u) (Operator.__call__, operator/_base.py:753-790) */
#define FSM_APPLY 40

typedef struct FsmPlan FsmPlan;

typedef struct FsmMeshDesc {
  int32_t ndim;      /* 1..3 */
  int32_t n[3];      /* points per axis */
  double length[3];  /* end - start per axis (mesh.py:185-191: f = fftfreq(n, length/n)) */
} FsmMeshDesc;

typedef struct FsmProgramDesc {
  int32_t n_channel;
  int32_t nonlinear;        /* FSM_NL_* */
  int32_t flags;            /* FSM_FLAG_* */
  int32_t integrator;       /* FSM_ETDRK* / FSM_SETDRK* / FSM_RK* */
  double nonlinear_coef;    /* scalar coefficient of the nonlinear term */
  const uint8_t* keep[3];   /* HOST: per axis, n[i] dealias keep flags in fftfreq order
                               (mesh.py:443-461); NULL keeps every mode */
  int32_t n_integration_points;  /* SETDRK contour points M (default 16) */
  double integration_radius;     /* SETDRK contour radius r (default 1.0) */
  const double* linear_coef;     /* DEVICE complex128 [lin_batch][lin_channel][S] (interleaved
                                    re, im); NULL means L = 0 */
  int32_t lin_batch;             /* 1 or the batch size */
  int32_t lin_channel;           /* 1 or n_channel */
  const void* source;            /* DEVICE complex64 [src_batch][n_channel][S], added to the
                                    nonlinear value of every stage; NULL for none */
  int32_t src_batch;             /* 1 or the batch size */
  int32_t table_batch;           /* entries of the coefficient tables along the batch (0: lin_batch);
                                    above 1, sample b uses entry b, whose time step can be changed with
                                    fsm_plan_set_batch_dt (one plan serving samples of different dt) */
} FsmProgramDesc;

/* Build a plan: validates the program, copies the wavenumbers, masks and
 * twiddles to the device and evaluates the exponential-integrator tables in
 * FP64 on the device (contour-integral mean over M points for SETDRK), then
 * rounds them to FP32. The linear coefficient buffer is read on `stream`
 * and may be freed once the stream has passed this call. */
int fsm_plan_create(const FsmMeshDesc* mesh, const FsmProgramDesc* program, double dt, void* stream,
                    FsmPlan** out);

/* Recompute the coefficient tables of batch entry b for time step dt
 * (plans with table_batch > 1): fsm_integrate then advances sample b with dt. Mutates the
 * plan: not to be called while work using the plan is in flight on another stream. The
 * serving engine does the same internally for each admitted request's table entry. No
 * counterpart in the reference (its integrator holds one dt,
 * integrator/_stable_etdrk/_uncached.py:180-211). */
int fsm_plan_set_batch_dt(FsmPlan* plan, int32_t b, double dt, void* stream);

/* Copy the coefficient tables of batch entry src to entry dst (a caller that compacts its
 * samples keeps each sample's dt). Same mutation rule as fsm_plan_set_batch_dt. */
int fsm_plan_move_batch(FsmPlan* plan, int32_t dst, int32_t src, void* stream);

/* Copy the plan's coefficient tables (complex64, [ntab][table_batch][lin_channel][S], the
 * scheme's order: SETDRK4 E - 1, E2 - 1, c1, c4, c5, c6) to the device buffer dst of
 * capacity_bytes; with dst == NULL only report ntab and the entries per table. The exponential
 * tables (E = exp(dt L), E2 = exp(dt L / 2); table 0 of every ETD scheme, table 1 of SETDRK3/4)
 * hold E - 1: the kernels form E u as u + (E - 1) u, which keeps E's FP32 rounding error from
 * compounding over the steps.
 * Inspection of UnCachedSETDRK*.__init__'s tables (integrator/_stable_etdrk/_uncached.py:180-211). */
int fsm_plan_tables(const FsmPlan* plan, void* dst, size_t capacity_bytes, int32_t* ntab, int64_t* entries,
                    void* stream);

/* Release a plan (synchronises the device first). */
int fsm_plan_destroy(FsmPlan* plan);

/* Bytes of device workspace fsm_integrate needs for `batch` samples and `steps` steps. */
int fsm_plan_workspace_bytes(const FsmPlan* plan, int32_t batch, int32_t steps, size_t* bytes);

/* Number of kernel launches fsm_integrate makes for `batch` samples and `steps` steps outside
 * stream capture (large batches run in parts, each with its own launches); batch 0 counts
 * one launch sequence (what a captured call makes). */
int fsm_plan_launch_count(const FsmPlan* plan, int32_t batch, int32_t steps, int64_t* launches);

/* Advance `state` (half spectra, [batch][C][S] complex64, in place) by `steps`
 * steps of dt. record_slot (HOST, steps+1 entries, or NULL): for step i
 * (0 = initial state, steps = final state) the frame index in `traj` to
 * write, or -1; traj is [batch][T][C][S] complex64 with T frames. */
int fsm_integrate(const FsmPlan* plan, int32_t batch, void* state, int32_t steps, const int32_t* record_slot,
                  void* traj, int32_t n_frames, void* workspace, size_t workspace_bytes, void* stream);

/* fsm_integrate without recording, with every kernel launch bracketed by CUDA
 * events on `stream`; blocks until the work is done. kernel_ms[4] and
 * kernel_launches[4] (HOST) receive the summed device time and the launch
 * count per kernel kind: 0 column pass, 1 row pass, 2 first column pass
 * (priming), 3 other (1D line, pointwise, batch means). Instrumentation for
 * benchmarks; not for production loops. */
int fsm_integrate_profiled(const FsmPlan* plan, int32_t batch, void* state, int32_t steps, void* workspace,
                           size_t workspace_bytes, void* stream, double* kernel_ms, int64_t* kernel_launches);

/* Size of the device scratch array behind fsm_integrate_static (32 MiB per GPU). */
#define FSM_STATIC_SCRATCH_BYTES (32u * 1024u * 1024u)

/* fsm_integrate (no recording) for callers that cannot allocate device memory:
 * code that may not call cudaMalloc or an allocating library after start-up
 * (host callbacks, allocation-free plugin hosts, real-time loops). Its scratch
 * is a fixed FSM_STATIC_SCRATCH_BYTES device array inside this library, held
 * by every GPU that loads it until the process exits; the caller still passes
 * the plan (created beforehand; plan creation allocates) and the state. Work
 * whose scratch would exceed the array (fsm_plan_workspace_bytes) is rejected
 * with FSM_ERR_INVALID. It runs one launch sequence on `stream` (never the
 * library's own streams of a split batch). The first call on a device looks up
 * the array's device address and must come before any stream capture on that device. With
 * CUDA's lazy module loading (the default), that first call, and the first launch of each
 * kernel a plan uses, load code and back the array, which can allocate: make one warm-up call
 * per device and plan at start-up, before the region that may not allocate; later calls
 * allocate nothing. The address is cached per device index for the life of the process:
 * cudaDeviceReset (or any reset of the primary context) is not supported after the first
 * call. All calls share the one array: calls that overlap on the GPU (other streams, other
 * threads) race and corrupt each other's results; serialise them. No
 * counterpart in the reference. */
int fsm_integrate_static(const FsmPlan* plan, int32_t batch, void* state, int32_t steps, void* stream);

/* Forward real transform over the plan's spatial axes: `count` real fields
 * [count][n0..] (float32) -> half spectra [count][S] (complex64). */
int fsm_rfftn(const FsmPlan* plan, int32_t count, const float* in, void* out, void* stream);

/* Inverse: half spectra [count][S] -> real fields [count][n0..] with 1/N; the
 * imaginary parts of self-conjugate modes are ignored (= ifftn(...).real).
 * `in` is used as scratch and is overwritten. */
int fsm_irfftn(const FsmPlan* plan, int32_t count, void* in, float* out, void* stream);

/* Write, for each of `count` half-spectrum fields, 1 into flags[i] if it holds
 * a NaN or Inf and 0 otherwise (device int32 array). */
int fsm_nonfinite_flags(const FsmPlan* plan, int32_t count, const void* fields, int32_t* flags, void* stream);

/* Elementwise kernels of the hand-written SETDRK4 adjoint (gradients of integrate; no
 * counterpart in the reference, which differentiates its loop with torch autograd,
 * operator/_base.py:731-735). All arrays are device arrays, launched on `stream`.
 * fsm_adj_accumulate: tbar[i] += Re(conj(x[i]) y[i]), i < n (x, y complex64, tbar float64).
 * fsm_adj_vjp_products: the physical-space products of the Convection vector-Jacobian
 *   product for `batch` samples of `points` grid points and nd = C channels: w_c = scale
 *   nbar_c, ubar_c = sum_c' w_c' g_c[c'] (g_c = d_c u, arrays [batch][C][points]),
 *   uw[i][b][c] = u_i w_c ([nd][batch][C][points]).
 * fsm_adj_vjp_combine: out = m (sub - i sum_i k_i suw[i]) over [batch_channels][points]
 *   half-spectrum points (sub, out complex64; suw [nd][batch_channels][points]; k_i and m
 *   float [points]). */
int fsm_adj_accumulate(int64_t n, const void* x, const void* y, double* tbar, void* stream);

/* One step of the discrete adjoint of the plan's SETDRK4 step for a Convection program
 * (integrator/_stable_etdrk/_setdrk_step.py:55-82 with operator/generic/_convection.py:43-46;
 * the reference gets it from torch autograd, operator/_base.py:731-735). The plan must be
 * SETDRK4, FSM_NL_CONVECTION with C == ndim, no source, and a real linear symbol (the tables
 * are read as real). u: DEVICE [batch][C][S] state at the start of the step; ubar_next:
 * cotangent of the state after it; ubar (output, may alias u or ubar_next): cotangent of u.
 * Cotangents are half spectra v with dLoss = Re sum_k conj(v_k) du_k over the full spectrum.
 * tbar (DEVICE float64 [6][batch][C][S], or NULL): tbar[t] += the cotangent of coefficient
 * table t (E, E2, c1, c4, c5, c6) per mode. The forward stages are recomputed with the plan's
 * own tables, so this is the exact adjoint of the forward the plan runs. Launches only (no
 * allocation, no synchronisation): it may be captured into a CUDA graph. */
int fsm_step_adjoint_workspace_bytes(const FsmPlan* plan, int32_t batch, size_t* bytes);
int fsm_step_adjoint(const FsmPlan* plan, int32_t batch, const void* u, const void* ubar_next, void* ubar,
                     double* tbar, void* workspace, size_t workspace_bytes, void* stream);
int fsm_adj_vjp_products(int32_t batch, int32_t nd, int64_t points, float scale, const float* nbar, const float* u,
                         const float* g0, const float* g1, const float* g2, float* ubar, float* uw, void* stream);
int fsm_adj_vjp_combine(int32_t batch_channels, int32_t nd, int64_t points, const void* sub, const void* suw,
                        const float* k0, const float* k1, const float* k2, const float* m, void* out, void* stream);

/* Serving engine: a slot pool of one plan advancing many independent solve requests together
 * (continuous batching). No counterpart in the reference, whose Operator.integrate
 * (operator/_base.py:676-751) solves one batch at a time with one dt; each request here is
 * that solve with its own batch, step count and dt.
 *
 * fsm_serve_create: `plan` built with table_batch >= capacity (a table entry per request, each with
 *   its own dt); `state` DEVICE complex64 [capacity][C][S]; `workspace` DEVICE of at least
 *   fsm_serve_workspace_bytes(plan, capacity, chunk) bytes (the integration's workspace and the
 *   slots' table entries); all work runs on `stream`. flags:
 *   FSM_SERVE_GRAPHS replays ticks of at most 64 steps as CUDA graphs (captured per
 *   (occupied slots, steps), step counts of such ticks rounded down to a power of two).
 *   tick_ms > 0 bounds a tick to about that much device time (from the measured time per step
 *   and slot); 0: ticks of up to `chunk` steps. The engine keeps the pointers; it allocates no
 *   device memory. Plans whose samples interact (KS with the batch-wide mean) are refused.
 * fsm_serve_submit: queue a request of `batch` samples: u0 DEVICE [batch][C][S] half spectra,
 *   read when the request is admitted; out DEVICE [batch][C][S], written when it leaves (u0 and
 *   out may be the same buffer). Both must stay valid until the request has left. Ids are the
 *   caller's and unique among pending requests.
 * fsm_serve_tick: if no tick is in flight, admit waiting requests in submission order while the
 *   head of the queue fits into the free slots (each admitted request's coefficient tables are
 *   computed once for its dt, in one table entry its samples share), then launch k steps of every
 *   occupied slot
 *   (k = the fewest remaining steps, at most chunk and the tick_ms bound). *steps_launched = k,
 *   0 when a tick is in flight or no slot is occupied.
 * fsm_serve_poll: complete the tick in flight once the device has finished it (wait != 0:
 *   block until then). Completed requests copy their slots to `out` (on the stream: the results
 *   are ready for work enqueued on it after this call) and leave; the remaining slots are
 *   compacted. Up to max_ids ids of completed requests are reported in done_ids (the rest at
 *   the next poll); *in_flight = 1 while a tick is still running.
 * fsm_serve_cancel: a waiting request is dropped (u0, out untouched); an active one leaves at
 *   once, or when the tick in flight completes, writing the state it reached to `out`; it is
 *   not reported by fsm_serve_poll.
 * fsm_serve_request_status: FSM_SERVE_WAITING / ACTIVE / DONE (completed, not yet reported) or
 *   FSM_SERVE_UNKNOWN, and the steps still to run.
 * fsm_serve_stats: up to n of {occupied slots, waiting requests, active requests, tick in
 *   flight, ticks, kernel launches, graph replays, slot-steps launched, completed, cancelled}.
 * fsm_serve_destroy: waits for the stream, releases the graphs and events.
 * One engine is used by one host thread at a time (calls are serialised by a lock); engines on
 * different streams run concurrently. */
typedef struct FsmServe FsmServe;
#define FSM_SERVE_GRAPHS 1
#define FSM_SERVE_UNKNOWN (-1)
#define FSM_SERVE_WAITING 0
#define FSM_SERVE_ACTIVE 1
#define FSM_SERVE_DONE 2
#define FSM_SERVE_NSTATS 10
int fsm_serve_workspace_bytes(const FsmPlan* plan, int32_t capacity, int32_t chunk, size_t* bytes);
int fsm_serve_create(FsmPlan* plan, int32_t capacity, int32_t chunk, void* state, void* workspace,
                     size_t workspace_bytes, int32_t flags, double tick_ms, void* stream, FsmServe** out);
int fsm_serve_submit(FsmServe* server, int64_t request_id, int32_t batch, int32_t steps, double dt, const void* u0,
                     void* out);
int fsm_serve_tick(FsmServe* server, int32_t* steps_launched);
int fsm_serve_poll(FsmServe* server, int32_t wait, int64_t* done_ids, int32_t max_ids, int32_t* n_done,
                   int32_t* in_flight);
int fsm_serve_cancel(FsmServe* server, int64_t request_id);
int fsm_serve_request_status(FsmServe* server, int64_t request_id, int32_t* status, int32_t* remaining);
int fsm_serve_stats(FsmServe* server, int64_t* stats, int32_t n);
int fsm_serve_destroy(FsmServe* server);

/* Serving groups: engines of different grid sizes (and PDEs) ticked together. No counterpart in
 * the reference (see the serving engine above).
 *
 * fsm_serve_group_create: 1 to 8 engines that share one stream and have no tick in flight. From
 *   then on they are ticked only through the group (fsm_serve_tick on a member is refused);
 *   requests are still submitted to, polled from (fsm_serve_poll reports the completed ids),
 *   cancelled at and queried from the members. tick_ms as in fsm_serve_create, measured per
 *   step and occupied slot over the whole group.
 * fsm_serve_group_tick: admit into every member, then advance every occupied slot of every
 *   member by the same k steps (the fewest remaining steps of any active request, at most the
 *   smallest member chunk and the tick_ms bound). When every member is a 1D line plan of 256 to
 *   4096 points and one nonlinear kind (KS or Burgers), the tick is ONE kernel launch over all
 *   of them. When every member is a SETDRK4 plan of a square 2D grid of 64, 128 or 256 points
 *   per axis and one nonlinear kind (Convection or VorticityConvection), each pass of the tick
 *   is one launch over all of them (a priming column pass, then a row and a column pass per
 *   stage). Otherwise the members are launched one after the other in the tick (lockstep).
 *   *steps_launched = k, 0 when a tick is in flight or no slot is occupied.
 * fsm_serve_group_poll: complete the group's tick once the device has finished it (wait != 0:
 *   block until then): every member's finished requests leave as in fsm_serve_poll;
 *   *in_flight = 1 while the tick is still running.
 * fsm_serve_group_stats: up to n of {ticks, kernel launches, tick in flight, one launch per tick
 *   (1D lines), one launch per pass (2D planes)}.
 * fsm_serve_group_destroy: waits for the stream, accounts a finished tick, releases the members
 *   (which may then be ticked alone or destroyed; destroying a member of a group is refused). */
typedef struct FsmServeGroup FsmServeGroup;
#define FSM_SERVE_GROUP_NSTATS 5
int fsm_serve_group_create(FsmServe* const* engines, int32_t count, double tick_ms, FsmServeGroup** out);
int fsm_serve_group_tick(FsmServeGroup* group, int32_t* steps_launched);
int fsm_serve_group_poll(FsmServeGroup* group, int32_t wait, int32_t* in_flight);
int fsm_serve_group_stats(FsmServeGroup* group, int64_t* stats, int32_t n);
int fsm_serve_group_destroy(FsmServeGroup* group);

/* Copy the message of the last failure on this host thread into buf. */
int fsm_last_error(char* buf, size_t len);

/* ABI version of this library. */
int fsm_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* TORCHFSM_GB300_H */
