/*
 * fluids2d_gb300 - C ABI of the GB300-native time-stepping path of Fluids2d.
 *
 * Plain pointers and sizes only. Every function returns 0 on success and a
 * non-zero code otherwise; f2d_last_error() gives the message of the last
 * failure on the calling thread. Arrays crossing the boundary use the
 * reference's layout: C-contiguous (ny+6, nx+6) float64 (int8 for masks and
 * stencil orders), halo width 3.
 *
 * Reference interfaces each entry point replaces are cited as
 * file:line of pvthinker/Fluids2d.
 */
#ifndef FLUIDS2D_GB300_H
#define FLUIDS2D_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define F2D_ABI_VERSION 1

/* models (param.py:1-2) the GPU path implements */
enum { F2D_MODEL_EULERPSI = 0, F2D_MODEL_RSW = 1, F2D_MODEL_QG = 2,
       F2D_MODEL_EULER = 3, F2D_MODEL_BOUSSINESQ = 4, F2D_MODEL_QGRSW = 5 };
/* flux methods (param.py:4, weno.py:338-343); CLASSIC is accepted for the
 * innerproduct only (param.py:5, the 4-point product of operators.py:86-90) */
enum { F2D_METHOD_WENO = 0, F2D_METHOD_UPWIND = 1, F2D_METHOD_CENTERED = 2,
       F2D_METHOD_CWENO = 3, F2D_METHOD_CLASSIC = 4 };
/* integrators (integrators.py:9-131): SSP-RK3, Euler forward,
 * energy-conserving RK3, leap-frog with Robert-Asselin filter */
enum { F2D_INTEG_RK3 = 0, F2D_INTEG_EF = 1, F2D_INTEG_ENRK3 = 2,
       F2D_INTEG_LFRA = 3 };
/* arithmetic of the stencils and of the multigrid cycle */
enum { F2D_PREC_FP64 = 0, F2D_PREC_FP32 = 1 };
/* param.noslip (noslip.py:18-34): None/False, True, or a list of sides */
enum { F2D_SLIP_FREE = 0, F2D_SLIP_NOSLIP = 1, F2D_SLIP_SIDES = 2 };
enum { F2D_SIDE_LEFT = 1, F2D_SIDE_RIGHT = 2, F2D_SIDE_BOTTOM = 4,
       F2D_SIDE_TOP = 8 };

/* The subset of fluids2d.Param (param.py:11-59) the stepping path reads. */
typedef struct f2d_params {
    int model;          /* F2D_MODEL_* */
    int nx, ny;         /* interior cells */
    int halowidth;      /* must be 3 */
    int xperiodic;      /* 0/1 */
    int yperiodic;      /* must be 0 */
    double Lx, Ly;
    double f0, beta, g, H;
    double cfl, dtmax, dt; /* dt > 0: fixed time step (model.py:72-74) */
    int compflux, vortexforce, innerproduct; /* F2D_METHOD_* */
    int maxorder;
    int noslip;         /* F2D_SLIP_* */
    int noslip_sides;   /* F2D_SIDE_* bits when noslip == F2D_SLIP_SIDES */
    int precision;      /* F2D_PREC_* */
    double poisson_tol; /* relative residual of the Poisson solve */
    int poisson_maxit;
    int integrator;     /* F2D_INTEG_* */
    double ragamma;     /* Robert-Asselin coefficient of LFRA (param.py:50) */
    int tracer;         /* 1: a passive tracer field "tracer" (param.py:57,
                           equations.py:217-226) */
    int reserved[3];
} f2d_params;

typedef struct f2d_model_s *f2d_model;

int f2d_abi_version(void);
const char *f2d_last_error(void);

/* Defaults of param.py:11-59 plus poisson_tol = 1e-12, maxit = 200. */
int f2d_params_default(f2d_params *p);

/* ---- host-side mesh construction (no GPU needed) ---------------------- */

/* set_order (meshes.py:146-186): stencil orders of a flattened mask. */
int f2d_set_order(const int8_t *msk, int64_t n, int64_t shift, int maxorder,
                  int8_t *order);

/* Mesh.finalize without the factorisations (meshes.py:34-37, 77-104;
 * noslip.py:4-36; elliptic.py:102-111, 198-203). Outputs are (ny+6, nx+6)
 * arrays; orders is 6 arrays back to back: oc.x, oc.y, ov.x, ov.y, ok.x,
 * ok.y; gv is the vertex index G of Poisson2D(mesh, "v"). Any output
 * pointer may be NULL. */
int f2d_mesh_build(const f2d_params *p, const int8_t *msk, int8_t *mskx,
                   int8_t *msky, int8_t *mskv, double *slipcoef,
                   int8_t *orders, int32_t *gv);

/* ---- flat-index sweeps on device arrays (weno.py:346-446) ------------- */
/* CompFlux[method](flx, U, q, o, s, i0, i1), weno.py:349-363 */
int f2d_compflux(int method, double *flx, const double *U, const double *q,
                 const int8_t *o, int64_t s, int64_t i0, int64_t i1,
                 void *stream);
/* VortexForce[method](du, V, q, o, s, s2, sign, i0, i1), weno.py:370-384 */
int f2d_vortexforce(int method, double *du, const double *V, const double *q,
                    const int8_t *o, int64_t s, int64_t s2, int sign,
                    int64_t i0, int64_t i1, void *stream);
/* InnerProduct[method](ke, U, q, o, s, i0, i1), weno.py:391-403 */
int f2d_innerproduct(int method, double *ke, const double *U, const double *q,
                     const int8_t *o, int64_t s, int64_t i0, int64_t i1,
                     void *stream);

/* ---- models ------------------------------------------------------------ */

/* Model(param) with the mask msk (meshes.py:18-52, model.py:14-24); msk may
 * be NULL for the default mask (meshes.py:70-75). Device buffers are owned
 * by the model. */
int f2d_model_create(const f2d_params *p, const int8_t *msk, f2d_model *out);
int f2d_model_destroy(f2d_model m);

/* Mesh.finalize after editing the mask (meshes.py:34-52). */
int f2d_model_set_mask(f2d_model m, const int8_t *msk);

/* Stream the model runs on (cudaStream_t as void*); NULL = its own. */
int f2d_model_set_stream(f2d_model m, void *stream);

/* State fields by the reference's names (states.py:7-17): "omega", "psi",
 * "vomega", "U.x", "U.y", "u.x", "u.y", "h", "ke", "p", "pv", "work", ...
 * Host arrays are (ny+6, nx+6) float64. set/get synchronise the stream. */
int f2d_field_set(f2d_model m, const char *name, const double *host);
int f2d_field_get(f2d_model m, const char *name, double *host);
/* Same, asynchronous on the model's stream (host memory should be pinned). */
int f2d_field_set_async(f2d_model m, const char *name, const double *host);
int f2d_field_get_async(f2d_model m, const char *name, double *host);
/* Device address, row pitch (elements) and element size of a field. */
int f2d_field_device(f2d_model m, const char *name, void **ptr,
                     int64_t *pitch, int *elem_size);
/* Names of the fields of the model, comma-separated. */
int f2d_field_names(f2d_model m, char *buf, size_t len);
/* A field as packed (ny+6, nx+6) float32, the history's dtype "f"
 * (io.py:12-33, 71): converted on the device, then copied to host. */
int f2d_field_get_f32(f2d_model m, const char *name, float *host);

/* Bulk diagnostics (diagnostics.py:39-57) on the device: f2d_bulk_record
 * appends {t, ke, ens, vort, angular} of the current state to a device ring
 * of 1000 records (no host synchronisation; models with ke and omega);
 * f2d_bulk_read copies the records out (5 doubles each) and empties it. */
int f2d_bulk_record(f2d_model m);
int f2d_bulk_read(f2d_model m, double *host, int capacity, int *nrec);

/* mesh.f, the vertex Coriolis term of the beta-plane (qg_inversion,
 * operators.py:186-191); (ny+6, nx+6) float64. */
int f2d_set_coriolis(f2d_model m, const double *f_vertices);

/* integrator.diag(state) (equations.py:80-84, 99-101, 150-155) */
int f2d_diag(f2d_model m);
/* qg_projection(mesh, s.u, s.h, s.pv, s.psi) (operators.py:176-183, the
 * anomaly=False form used to set a qgrsw initial state): the state's (u, h)
 * in place, pv and psi of the projection; qgrsw models only. */
int f2d_qg_projection(f2d_model m);
/* Model.step(n) with the current time step (model.py:67-69) */
int f2d_step(f2d_model m, int nsteps);
/* n iterations of the Model.run loop body: set_dt then step(1)
 * (model.py:45-51); the CFL time step is computed on the device. */
int f2d_run(f2d_model m, int nsteps);
/* The right-hand side alone, rhs(s, ds) of equations.py:73-157 (the
 * registry get_rhs_and_diag, equations.py:190-210, with the tracer equation
 * 217-226 and any forcing term 229-238): the tendency of the current state
 * (whose diagnostics must be current, as after f2d_diag) into the fields
 * "rhs.<var>" of every prognostic variable ("rhs.omega", "rhs.u.x",
 * "rhs.u.y", "rhs.h", "rhs.pv", "rhs.b", "rhs.tracer"), read with
 * f2d_field_get; the state is not changed (qgrsw: like the reference, the
 * projection leaves its pv and psi). The plug point that lets the
 * reference's own integrators (integrators.py:92-155) drive the GPU. */
int f2d_rhs(f2d_model m);
/* Stage k (1-based) of the integrator's step (integrators.py:92-155: rk3 and
 * enrk3 have 3 stages, ef and LFRA 1) with the current time step: the
 * stage's right-hand side and update, then diag; the last stage also
 * advances the time line (timeline.py:20-35). f2d_set_dt, then stages
 * 1..n, is one Model.run iteration; between stages the host may change the
 * forcing fields (f2d_forcing_set), which is how a forcing function that
 * depends on time or state runs. */
int f2d_stage(f2d_model m, int k);
/* Model.add_forcing (model.py:121-123, addforcingterm equations.py:229-238)
 * on the device: the forcing term of prognostic variable `name` ("omega",
 * "u.x", "u.y", "h", "pv", "b", "tracer"; a (ny+6, nx+6) float64 host
 * array), added to its tendency after the right-hand side in every stage of
 * step, run, f2d_stage and f2d_rhs until changed or cleared. In an
 * x-periodic domain the halo columns of the tendency of omega, pv, u, h, b
 * and the tracer take the forced value of their interior copy (give the
 * forcing periodic halo columns for the reference's result). The first call
 * allocates the forcing fields of all variables (zero) and drops the
 * recorded graphs. */
int f2d_forcing_set(f2d_model m, const char *name, const double *host);
/* All forcing terms back to zero (no reference counterpart). */
int f2d_forcing_clear(f2d_model m);
/* Model.set_dt (model.py:71-87) */
int f2d_set_dt(f2d_model m);
/* Time (timeline.py:4-35) */
int f2d_time_get(f2d_model m, double *t, double *dt, int64_t *ite);
int f2d_time_set(f2d_model m, double t, double dt, int64_t ite);

/* Poisson2D.solve(b, x) (elliptic.py:80-87) on the vertex operator
 * (which = 0) or the qg Helmholtz operator (which = 1, meshes.py:42-47):
 * only fluid points of x are written, then the halo fill. Host arrays.
 * *iters = CG iterations of the solve (FP32 form: summed over its
 * refinement rounds), *relres = final relative residual. */
int f2d_poisson_solve(f2d_model m, int which, const double *b, double *x,
                      int *iters, double *relres);

/* Wait for the model's stream; returns the device status (timeouts,
 * non-converged solves, non-finite values) as an error. */
int f2d_sync(f2d_model m);
/* Time `reps` launches of the fused right-hand-side + RK3-update kernel of
 * stage 1..3 on the model's stream with CUDA events (L2 flushed between
 * launches when flush_l2 != 0); *avg_ms = mean milliseconds per launch.
 * Repeated launches recompute the same output, so the state is unchanged.
 * No reference counterpart: the measurement hook of the benchmark. */
int f2d_time_stage(f2d_model m, int stage, int reps, int flush_l2,
                   double *avg_ms);
/* Autotuner of the multigrid schedule (tile rows 32/64, sweeps per leg 1/2,
 * and in the FP32 form the inner tolerance 1e-8 .. 1e-4): each candidate's
 * solve of the current state's right-hand side is captured as a graph and
 * timed over `reps` solves from the warm start 0.999 psi; the fastest that
 * reaches the tolerance is kept (the step graphs are re-captured). The state
 * is unchanged. Outputs may be NULL. Models with a vertex Poisson/Helmholtz
 * solve (eulerpsi, qg, qgrsw) and ensembles. */
int f2d_autotune(f2d_model m, int reps, int *tile_rows, int *sweeps, double *tol_in,
                 double *ms_per_solve);
/* Set the multigrid schedule directly (what f2d_autotune would pick):
 * tile rows 32 or 64, red-black sweeps per leg 1 or 2, and the inner
 * tolerance of the FP32 form's refinement rounds (0 < tol_in < 1; unused in
 * the FP64 form). Recorded graphs are dropped. No reference counterpart. */
int f2d_set_schedule(f2d_model m, int tile_rows, int sweeps, double tol_in);
/* Time `reps` launches of the Poisson solver's level-0 down kernel
 * (pre-smoothing + residual + restriction of the V-cycle, the solver's largest
 * share) on the current right-hand side, L2 flushed between launches when
 * flush_l2 != 0; *avg_ms = mean ms, *nodes = level-0 nodes, *elem_bytes = 4
 * or 8 (multigrid precision). Measurement hook of the benchmark; no
 * reference counterpart. The model must have solved once. */
int f2d_time_solver(f2d_model m, int reps, int flush_l2, double *avg_ms,
                    int64_t *nodes, int *elem_bytes);
/* Which level kernels the solver timed by f2d_time_solver runs: *pipelined =
 * 1 for the persistent TMA-staged FP32 kernels (k_mgp_down / k_mgp_up), 0
 * for the one-tile-per-block kernels (k_mg_down / k_mg_up: the FP64 form,
 * or level arrays outside the pipelined kernels' layout). Instrumentation,
 * no reference counterpart. The model must have solved once. */
int f2d_solver_pipelined(f2d_model m, int *pipelined);
/* Failure-detection test switch (no reference counterpart). enabled != 0:
 * every stage kernel, once its TMA tile has landed, also waits for a barrier
 * phase that nothing completes, gives up after limit_ms (0 < limit_ms <=
 * 1000) and records the TMA time-out status, which the next f2d_sync /
 * f2d_ensemble_sync reports; the stage's output is then not written.
 * enabled == 0 restores normal operation. Applies to every model and
 * ensemble of the process; synchronises the device. For tests only. */
int f2d_test_tma_wait(int enabled, double limit_ms);
/* Test hook (no reference counterpart): the library's integer-pipe
 * binary64 -> binary32 (round to nearest even) and binary32 -> binary64
 * conversions next to the hardware conversions, on the device, for host
 * inputs x64[n64] and x32[n32]; outputs sw32/hw32[n64], sw64/hw64[n32]. */
int f2d_test_conversions(const double *x64, int64_t n64, float *sw32, float *hw32,
                         const float *x32, int64_t n32, double *sw64, double *hw64);
/* Refinement rounds of the FP32 form's solves summed since creation (see
 * f2d_ensemble_refine_rounds). Instrumentation. */
int f2d_refine_rounds(f2d_model m, int64_t *rounds);
/* Counters: Poisson iterations summed over all solves since creation; the
 * kernels one time step launches outside the Poisson loops; the kernels one
 * Poisson iteration launches. No reference counterpart (instrumentation). */
int f2d_stats(f2d_model m, int64_t *poisson_iters,
              int64_t *launches_per_step, int64_t *launches_per_iter);

/* ---- batched ensembles ------------------------------------------------- */

/* No single counterpart in the reference: tools.run_twin_experiments
 * (tools.py:29-49) steps two models in lockstep; an ensemble advances
 * `count` independent eulerpsi or qg models with their own nx[b], ny[b] and
 * masks msks[b] (NULL entries: default mask) together, one kernel launch
 * per operation for all members, each member with its own CFL time step.
 * The common parameters (model, Lx, Ly, f0, beta, cfl, precision, Poisson
 * tolerance...) come from p; p->dt must be 0. */
typedef struct f2d_ensemble_s *f2d_ensemble;
int f2d_ensemble_create(const f2d_params *p, int count, const int *nx,
                        const int *ny, const int8_t *const *msks,
                        f2d_ensemble *out);
int f2d_ensemble_destroy(f2d_ensemble e);
int f2d_ensemble_set_stream(f2d_ensemble e, void *stream);
/* A field of ALL members at once, in the packed host layout: member b's
 * (ny_b+6, nx_b+6) float64 array at offset f2d_ensemble_packed_size-style
 * prefix sums (member order), one host<->device copy and one gather/scatter
 * kernel for the whole ensemble. async != 0: no stream synchronisation (the
 * host buffer must then be pinned and stay alive until f2d_ensemble_sync). */
int f2d_ensemble_fields_set(f2d_ensemble e, const char *name, const double *host,
                            int async);
int f2d_ensemble_fields_get(f2d_ensemble e, const char *name, double *host, int async);
/* Elements of the packed layout (sum over members of (ny+6)(nx+6)). */
int64_t f2d_ensemble_packed_size(f2d_ensemble e);
/* Fields of member b by the reference's names ("omega" or "pv", "psi",
 * "vomega" or "work", "U.x", "U.y"; "f" sets the qg vertex Coriolis term);
 * (ny[b]+6, nx[b]+6) float64 host arrays. */
int f2d_ensemble_field_set(f2d_ensemble e, int member, const char *name,
                           const double *host);
int f2d_ensemble_field_get(f2d_ensemble e, int member, const char *name,
                           double *host);
int f2d_ensemble_field_set_async(f2d_ensemble e, int member, const char *name,
                                 const double *host);
int f2d_ensemble_field_get_async(f2d_ensemble e, int member, const char *name,
                                 double *host);
/* integrator.diag of every member (equations.py:80-84, 99-101) */
int f2d_ensemble_diag(f2d_ensemble e);
/* The autotuner (see f2d_autotune) on the ensemble's batched solver. */
int f2d_ensemble_autotune(f2d_ensemble e, int reps, int *tile_rows, int *sweeps,
                          double *tol_in, double *ms_per_solve);
/* f2d_set_schedule for the ensemble's batched solver. */
int f2d_ensemble_set_schedule(f2d_ensemble e, int tile_rows, int sweeps, double tol_in);
/* n iterations of set_dt + step(1) for every member (model.py:45-51) */
int f2d_ensemble_run(f2d_ensemble e, int nsteps);
int f2d_ensemble_time_get(f2d_ensemble e, int member, double *t, double *dt,
                          int64_t *ite);
int f2d_ensemble_sync(f2d_ensemble e);
/* interior cells of all members, Poisson iterations summed over members,
 * iterations of the batched CG loop (each runs the body once for all
 * members still iterating), kernels per step outside the Poisson loops,
 * kernels per loop iteration (instrumentation) */
int f2d_ensemble_stats(f2d_ensemble e, int64_t *cells, int64_t *poisson_iters,
                       int64_t *loop_iters, int64_t *launches_per_step,
                       int64_t *launches_per_iter);
/* Refinement rounds of the FP32 form's Poisson solves (each an inner FP32
 * CG solve followed by an FP64 residual), summed over all solves and members
 * since creation; 0 in the FP64 form. Instrumentation, no reference
 * counterpart. */
int f2d_ensemble_refine_rounds(f2d_ensemble e, int64_t *rounds);
/* f2d_time_stage for the batched stage kernel of all members (measurement
 * hook of the benchmark; no reference counterpart). */
int f2d_ensemble_time_stage(f2d_ensemble e, int stage, int reps, int flush_l2,
                            double *avg_ms);
/* f2d_time_solver for the batched solver of all members. */
int f2d_ensemble_time_solver(f2d_ensemble e, int reps, int flush_l2, double *avg_ms,
                             int64_t *nodes, int *elem_bytes);
/* f2d_solver_pipelined for the batched solver of all members. */
int f2d_ensemble_solver_pipelined(f2d_ensemble e, int *pipelined);

/* ---- discrete adjoint (eulerpsi, closed basin, weno/upwind fluxes) ------ */

/* No counterpart in the reference (it has no differentiation); the forward
 * map is its RK3 step (integrators.py:92-107) of equations.py:73-86 with the
 * time step held fixed at dt. Runs nsteps steps from w0 and writes the final
 * vorticity to wT. w0 and wT are DEVICE FP64 arrays of (ny+6) x (nx+6)
 * points, rows contiguous. Keeps the vorticity every `every` steps as a
 * checkpoint for f2d_adjoint_backward. Leaves the model on a constant time
 * step dt. Stream-ordered on the model's stream (no synchronisation). */
int f2d_adjoint_forward(f2d_model m, const double *w0, double *wT, int nsteps,
                        double dt, int every);
/* Gradient pull-back of the last f2d_adjoint_forward: lam0 = (dwT/dw0)^T lamT
 * (device FP64 arrays as above). Recomputes each checkpoint segment while
 * recording the stage states, then runs the adjoint steps backwards: the
 * discrete adjoint of the WENO-Z flux divergence with its smoothness weights
 * differentiated exactly, of perpgrad and of the centre-to-vertex average,
 * and the same masked Poisson solve for the adjoint streamfunction. The
 * adjoint arithmetic is FP64 for either forward precision. Afterwards the
 * model holds the state at the end of the first segment. */
int f2d_adjoint_backward(f2d_model m, const double *lamT, double *lam0);

/* ---- allocation-free entry point ---------------------------------------- */

/* No counterpart in the reference. For callers that must not allocate
 * device memory (frameworks that route all device memory through their own
 * pool, loops where a cudaMalloc would synchronise the device):
 * Model.set_dt's CFL step computed from
 * caller-owned device arrays U.x, U.y of rows x cols points with row pitch
 * `pitch` (elements). Writes out[0] = max|U.x|, out[1] = max|U.y|,
 * out[2] = min(cfl / (out[0] + out[1] + 1e-99), dtmax) to the caller's device
 * buffer `out` on `stream`; calls no cudaMalloc/cudaFree.
 * Its reduction scratch is a fixed 128 KiB array inside the library, kept by
 * every GPU that loads the library until exit, so rows * pitch is limited to
 * 33,554,432 points (larger arrays are refused with an error). The first call
 * on each device looks up that array's device address (kept until exit, so
 * cudaDeviceReset after it is not supported); make that first call before
 * any stream capture. Calls share the array: calls that overlap on the GPU
 * race and give wrong results, so serialise them on one stream. A NaN in U
 * gives NaN in out, as numpy's max gives in the reference's set_dt. */
int f2d_cfl_dt_noalloc(const double *Ux, const double *Uy, int64_t rows,
                       int64_t cols, int64_t pitch, double cfl, double dtmax,
                       double *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FLUIDS2D_GB300_H */
