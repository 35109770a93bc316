/*
 * splash_gb300.h — C ABI of the GB300 (sm_103a) MUSCL time step of SPLASH.
 *
 * The reference exposes its solver only as header-only C++ classes
 * (Riemann_solvers/{HLLE_p,HLLC,HLLCplus}.hpp on top of physics/adiabatic.hpp
 * and MUSCL_base/MUSCL_base.hpp); it has no FFI.  Each entry point below
 * replaces one member of that class API, cited per function, so that a
 * C++ wrapper (include/splash_muscl.hpp), a ctypes binding or any other FFI
 * can drive the GPU solver with plain pointers and sizes.
 *
 * Conventions
 *   - Every function returns an int status: SPLASH_OK (0) or one of the
 *     SPLASH_E_* codes; splash_last_error() returns a message for the calling
 *     thread's most recent failure.
 *   - Conserved state arrays are row-major [n_faces][dim] float64 in the
 *     reference face order (the order of pmp's face iterator, i.e. the order
 *     test.cpp reads input/input.dat).  Renumbering to the internal
 *     space-filling-curve order happens inside the library.
 *   - A solver handle is driven by one host thread at a time (the reference
 *     object is not re-entrant either).  splash_do_step() is asynchronous on
 *     the solver's CUDA stream; every call that returns host data
 *     synchronises that stream.
 *   - Physics problems never abort: like the reference they latch the stop
 *     flag (MUSCL_base.hpp:17,232-235), readable with splash_stop_check()
 *     and, bit by bit, with splash_error_word().
 */
#ifndef SPLASH_GB300_H
#define SPLASH_GB300_H

#include <stddef.h>
#include <stdint.h>

/* Exported entry points; everything else in the library has hidden
 * visibility, so no internal C++ symbol can clash with a caller's. */
#if defined(__GNUC__)
#define SPLASH_API __attribute__((visibility("default")))
#else
#define SPLASH_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define SPLASH_OK 0
#define SPLASH_E_INVALID 1     /* bad argument (null pointer, size, enum) */
#define SPLASH_E_CUDA 2        /* CUDA runtime failure */
#define SPLASH_E_MESH 3        /* mesh violates a reference assumption */
#define SPLASH_E_NOMEM 4       /* host or device allocation failed */
#define SPLASH_E_UNSUPPORTED 5 /* combination not implemented */

/* ---- stop-flag bits (device error word) ------------------------------ */
#define SPLASH_STOP_NAN_FLUX 1u       /* MUSCL_base.hpp:264-268 */
#define SPLASH_STOP_NAN_WAVESPEED 2u  /* physics/adiabatic.hpp:671-676 */
#define SPLASH_STOP_WAVE_ORDER 4u     /* HLLE_p.hpp:50-55, HLLC.hpp:234-239, HLLCplus.hpp:169-174 */
#define SPLASH_STOP_NEG_EXTRA_DT 8u   /* physics/adiabatic.hpp:573-577 */

/* ---- enums ------------------------------------------------------------ */
typedef enum splash_mesh_kind {
  SPLASH_MESH_ICOSPHERE_HEX = 0, /* geometry/sph_gen.h:278-284 */
  SPLASH_MESH_QUAD_SPHERE = 1,   /* geometry/sph_gen.h:286-295 */
  SPLASH_MESH_ICOSPHERE = 2      /* geometry/sph_gen.h:267-276 */
} splash_mesh_kind;

typedef enum splash_solver_kind {
  SPLASH_SOLVER_HLLE_P = 1,   /* MUSCL_HLLE_p   Riemann_solvers/HLLE_p.hpp:6-59 */
  SPLASH_SOLVER_HLLC = 2,     /* MUSCL_HLLC     Riemann_solvers/HLLC.hpp:6-122 */
  SPLASH_SOLVER_HLLCPLUS = 3, /* MUSCL_HLLCplus Riemann_solvers/HLLCplus.hpp:6-177 */
  SPLASH_SOLVER_HLLE = 4      /* MUSCL_HLLE     Riemann_solvers/HLLE.hpp:6-62, isothermal, dim 4 */
} splash_solver_kind;

typedef enum splash_precision {
  SPLASH_PREC_FP64 = 0, /* the reference method in FP64 */
  SPLASH_PREC_MIXED = 1 /* FP32 reconstruction + Riemann, FP64 state/accumulation */
} splash_precision;

/* Mesh description.  If `vertices` is NULL the mesh is generated from
 * (kind, level) exactly as the reference generators number it; otherwise
 * the caller supplies a closed polygonal sphere mesh in its own order. */
typedef struct splash_mesh_desc {
  int kind;  /* splash_mesh_kind, used when vertices == NULL */
  int level; /* subdivision level, used when vertices == NULL */
  int n_vertices;
  const double* vertices; /* [n_vertices][3] */
  int n_faces;
  const int* face_offsets;  /* [n_faces + 1] CSR offsets into face_vertices */
  const int* face_vertices; /* corner ids, counter-clockwise seen from outside */
} splash_mesh_desc;

/* The keys the adiabatic constructor reads from input/parameters.json
 * (physics/adiabatic.hpp:59-68). */
typedef struct splash_params {
  double accretion_rate;
  double e_acc;
  double omega_acc_abs;
  double tilt_angle;
  double acc_width;
  double alpha;
  int friction_on;
} splash_params;

typedef struct splash_solver splash_solver;
typedef struct splash_geometry splash_geometry;

/* ---- library ---------------------------------------------------------- */
/* Message of the calling thread's last failure ("" if none). */
SPLASH_API const char* splash_last_error(void);
/* Library version string. */
SPLASH_API const char* splash_version(void);

/* ---- solver lifetime ---------------------------------------------------- */
/* Replaces the constructors MUSCL_HLLE_p / MUSCL_HLLC / MUSCL_HLLCplus
 * (Riemann_solvers/HLLE_p.hpp:11-13, HLLC.hpp:11-13, HLLCplus.hpp:11-13)
 * with the adiabatic and base constructors they chain to
 * (physics/adiabatic.hpp:18-91, MUSCL_base/MUSCL_base.hpp:20-95,
 * geometry/MUSCL_geometry.hpp:43-225).  `U_in` is [n_faces][dim] in the
 * reference face order; `params` replaces the parameters.json read.
 * `device` selects the CUDA device; `threads` sizes host-side helpers
 * (geometry precompute) only, 0 = all cores.  The adiabatic solvers need
 * dim 5 and the isothermal SPLASH_SOLVER_HLLE (MUSCL_HLLE, HLLE.hpp:11-13,
 * physics/isothermal.hpp:13-40) dim 4; other combinations are rejected with
 * SPLASH_E_UNSUPPORTED (the reference prints "check dim", latches stop_check
 * and, for the adiabatic solvers, then indexes past the state vector,
 * physics/adiabatic.hpp:26-30, Riemann_solvers/HLLC.hpp:208).  The
 * isothermal solver ignores omega_ns, accretion_on and params (its
 * constructor takes none of them).  Its reference path reads
 * and writes a fifth state field and an uninitialised limiter variable
 * (MUSCL_base.hpp:203, 324, 368-370; isothermal.hpp:272, 307); the GPU path
 * is the defined form: no fifth field, CFL sound speed a = 1, etha_minus =
 * H_minus / BM_dist. */
SPLASH_API int splash_create(const splash_mesh_desc* mesh, const double* U_in, int dim, double gam,
                  double omega_ns, int accretion_on, const splash_params* params,
                  int solver_kind, int precision, int device, int threads,
                  splash_solver** out);
SPLASH_API int splash_destroy(splash_solver* s);

/* ---- the hot path ------------------------------------------------------ */
/* Replaces MUSCL_base::do_step(double dt0) (MUSCL_base.hpp:97-225): one RK2
 * midpoint step with dt = min(dt0, 0.1 h0 / max_vel, extra_dt_constr()).
 * Asynchronous: enqueues one CUDA-graph replay on the solver's stream. */
SPLASH_API int splash_do_step(splash_solver* s, double dt0);
/* `n` consecutive do_step(dt0) calls without returning to the host. */
SPLASH_API int splash_do_steps(splash_solver* s, int n, double dt0);
/* Blocks until all enqueued steps have finished. */
SPLASH_API int splash_synchronize(splash_solver* s);

/* The cudaStream_t the solver launches on (as void*), so a caller can
 * order its own work or record CUDA events against the step. */
SPLASH_API int splash_stream(splash_solver* s, void** stream);
/* Runs `reps` un-captured steps with CUDA events between the step's phases
 * and returns the mean device time per phase in milliseconds:
 * ms[0] dt reduction (FP64 path; on the mixed path the stage-1 edge
 * launch clips dt itself and ms[0] is an empty slot); FP64 path: ms[1]
 * reconstruct (stage 1),
 * ms[2] flux+update (stage 1), ms[3] reconstruct (stage 2), ms[4]
 * flux+update (stage 2); mixed path: ms[1] edge (reconstruction + Riemann
 * flux, stage 1), ms[2] update (stage 1), ms[3] edge (stage 2), ms[4] update
 * (stage 2).  The steps advance the state like do_step(dt0). */
SPLASH_API int splash_kernel_times(splash_solver* s, int reps, double dt0, double ms[5]);
/* Mean device ms of every launch of one step over `reps` un-captured steps,
 * with a CUDA event between consecutive launches (which serialises the
 * step's programmatic overlap, so the sum exceeds the captured step's time).
 * Five slots on either path: mixed, the dt clip (an empty slot: the
 * stage-1 edge launch clips dt itself, so a mixed step is four launches),
 * edge (reconstruction + Riemann flux, stage 1), update (stage 1), edge
 * (stage 2), update (stage 2); FP64, dt reduction, reconstruct,
 * flux+update, reconstruct, flux+update.  Writes min(cap, *count) values;
 * *count = 5.
 * The steps advance the state like do_step(dt0). */
SPLASH_API int splash_launch_times(splash_solver* s, int reps, double dt0, double* ms, int cap, int* count);
/* Device bytes held by the solver: out[0] geometry, out[1] state + scratch. */
SPLASH_API int splash_memory(splash_solver* s, int64_t out[2]);

/* ---- accessors ---------------------------------------------------------- */
SPLASH_API int splash_time(splash_solver* s, double* t);               /* MUSCL_base.hpp:227-230 */
SPLASH_API int splash_stop_check(splash_solver* s, int* stop);         /* MUSCL_base.hpp:232-235 */
SPLASH_API int splash_error_word(splash_solver* s, uint32_t* bits);    /* SPLASH_STOP_* bits */
SPLASH_API int splash_last_dt(splash_solver* s, double* dt);           /* the clipped dt of the last step */
SPLASH_API int splash_steps(splash_solver* s, int64_t* steps);         /* MUSCL_base::steps */
SPLASH_API int splash_n_faces(splash_solver* s, int* n_faces);
SPLASH_API int splash_dim(splash_solver* s, int* dim);
/* [n_faces][dim] conserved state, reference order (MUSCL_base::U). */
/* State transfers: when the device can access pageable host memory (a
 * coherent CPU-GPU link, cudaDevAttrPageableMemoryAccess) the state moves
 * between the caller's array and the device planes in one kernel, without
 * a staging copy; otherwise through a pinned staging buffer.  Setting the
 * environment variable SPLASH_STAGED_TRANSFERS before splash_create forces
 * the staging path.  Both are synchronous and give identical states. */
SPLASH_API int splash_get_state(splash_solver* s, double* U);
SPLASH_API int splash_set_state(splash_solver* s, const double* U);
/* set_state(U_in), n do_step(dt0) calls and get_state(U_out) as one call
 * with one synchronisation, at the end (either state pointer may be NULL;
 * U_in may equal U_out): for a coupling code that owns the state in host
 * memory and hands it over every step.  The same states as the three calls.
 * No counterpart in the reference (its state stays in the solver object). */
SPLASH_API int splash_do_steps_host(splash_solver* s, const double* U_in, int n, double dt0, double* U_out);
/* Per-step diagnostics of MUSCL_base.hpp:187-214 for the current state:
 * out[0] = sum Sigma*A, out[1..3] = sum l*A, out[4] = sum E*A. */
SPLASH_API int splash_diagnostics(splash_solver* s, double out[5]);
/* Internal (space-filling-curve) position -> reference face id, [n_faces]. */
SPLASH_API int splash_get_permutation(splash_solver* s, int* internal_to_ref);
/* The solver's unit face centres fc/|fc| ([n_faces][3]) and face areas
 * ([n_faces]) in reference face order (MUSCL_geometry.hpp:1069-1077 writes the
 * same centres); either pointer may be NULL.  No counterpart member in the
 * reference: an accessor so that a caller can build initial states without
 * a second geometry build. */
SPLASH_API int splash_face_geometry(splash_solver* s, double* unit_centres, double* area);

/* ---- writers (physics/adiabatic.hpp:101-348) ---------------------------- */
/* Each appends one line "t  v0 v1 ... " to `path` with the reference's
 * default stream formatting (6 significant digits). */
SPLASH_API int splash_write_t_rho(splash_solver* s, const char* path);     /* adiabatic.hpp:101-111 */
SPLASH_API int splash_write_t_p(splash_solver* s, const char* path);       /* adiabatic.hpp:113-133 */
SPLASH_API int splash_write_t_curl(splash_solver* s, const char* path);    /* adiabatic.hpp:135-177 */
SPLASH_API int splash_write_t_omega_z(splash_solver* s, const char* path); /* adiabatic.hpp:195-226 */
/* three files, Lx/Ly/Lz (adiabatic.hpp:179-193) */
SPLASH_API int splash_write_t_L(splash_solver* s, const char* path_x, const char* path_y,
                     const char* path_z);
/* out[4] = flux towards observers at 0, 45, 90, 180 deg (adiabatic.hpp:228-333) */
SPLASH_API int splash_get_light_curves(splash_solver* s, double out[4]);
/* [n_faces] lines of dim values (adiabatic.hpp:335-348) */
SPLASH_API int splash_write_final_state(splash_solver* s, const char* path);

/* ---- geometry (host, reference numbering) ------------------------------ */
/* Builds the reference geometry (geometry/MUSCL_geometry.hpp:43-575) for a
 * mesh description; used by the drop-in classes' geometry writers
 * (MUSCL_geometry.hpp:1069-1117) and by the test-suite. */
SPLASH_API int splash_geometry_build(const splash_mesh_desc* mesh, int threads, splash_geometry** out);
SPLASH_API int splash_geometry_free(splash_geometry* g);
/* sizes[0..3] = n_vertices, n_faces, n_slots, max_slots;
 * scalars[0..1] = h0, round_diff */
SPLASH_API int splash_geometry_info(const splash_geometry* g, int64_t sizes[4], double scalars[2]);
/* Copies the named array into dst (capacity `bytes`).  Names: vertices,
 * face_off, face_vtx, nbr_off, nbr, nbr_edge, face_centers, normals, area,
 * edge_normals, bm_dist, h_plus, h_minus, ff_plus, ff_minus, beta_plus,
 * beta_minus, unit_face_centers (fc/|fc|), and hilbert_order (internal
 * position -> reference face id, the numbering splash_create uses).  *written receives the byte count
 * (may be NULL). */
SPLASH_API int splash_geometry_get(const splash_geometry* g, const char* name, void* dst, size_t bytes,
                        size_t* written);

/* ---- ensembles -------------------------------------------------------------
 * Many independent solvers (different meshes, parameters and states, each
 * with its own CFL dt) advanced together: one do_step of the ensemble is one
 * CUDA-graph replay whose launches cover every member.  No counterpart in the
 * reference, which runs one solver per process; each member computes exactly
 * what splash_create/splash_do_step with SPLASH_PREC_MIXED would.  Members on
 * the same mesh share its geometry on the device. */
typedef struct splash_member {
  int mesh_kind;        /* splash_mesh_kind */
  int level;            /* subdivision level */
  const double* U_in;   /* [n_faces][dim] conserved state, reference face order;
                           dim = 4 for SPLASH_SOLVER_HLLE (isothermal, no source:
                           accretion_on and params are ignored), else 5 */
  double gam;
  double omega_ns;
  int accretion_on;
  splash_params params;
  int solver_kind;      /* splash_solver_kind */
} splash_member;

typedef struct splash_ensemble splash_ensemble;

/* Builds the ensemble (FP32/FP64 mixed precision).  With `autotune` != 0 the
 * schedule is picked by timing every candidate for a few steps on the
 * ensemble itself (the state is restored afterwards): the member order of
 * the face and edge tiles (member order, largest first, round-robin) and
 * either five launches per step (per-member dt, edge and update of each
 * stage) with 32-, 64- or 128-thread edge blocks, or one persistent
 * cooperative launch per do_steps call that runs all its steps with grid
 * barriers between the phases. */
SPLASH_API int splash_ensemble_create(const splash_member* members, int n, int device, int autotune,
                           splash_ensemble** out);
SPLASH_API int splash_ensemble_destroy(splash_ensemble* e);
/* n steps of every member: member i advances by min(dt0, its CFL clip).
 * One graph replay per step, or one (the persistent schedule) for all n. */
SPLASH_API int splash_ensemble_do_steps(splash_ensemble* e, int n, double dt0);
/* Waits for the ensemble's stream; SPLASH_E_CUDA if a grid barrier of the
 * persistent launch timed out (its bounded wait, about 0.25 s). */
SPLASH_API int splash_ensemble_synchronize(splash_ensemble* e);
/* Sets the schedule: tile order 0..2 and edge_block 32, 64 or 128 threads
 * (five launches per step), or 0 for the persistent launch. */
SPLASH_API int splash_ensemble_set_schedule(splash_ensemble* e, int order, int edge_block);
SPLASH_API int splash_ensemble_stream(splash_ensemble* e, void** stream);
SPLASH_API int splash_ensemble_get_state(splash_ensemble* e, int member, double* U);
/* out = {t, dt of the last step, max_vel, extra_dt}; err = stop bits */
SPLASH_API int splash_ensemble_member_info(splash_ensemble* e, int member, double out[4], uint32_t* err);
/* The chosen schedule: tile order (0 member order, 1 largest first, 2
 * round-robin) and the threads per block of the reconstruction + edge-flux
 * launch (0: the persistent launch); and the autotuner's ms per step of
 * each candidate: [order*3 + {32,64,128}-thread blocks] for five launches
 * per step, [9 + order] for the persistent launch (0 where not timed). */
SPLASH_API int splash_ensemble_schedule(splash_ensemble* e, int* order, int* recon_width, double trial_ms[12]);
SPLASH_API int splash_ensemble_size(splash_ensemble* e, int* n_members, int64_t* total_faces);

/* ---- allocation-free CFL clip --------------------------------------------
 * No counterpart in the reference: an addition for callers that cannot
 * allocate device memory when they need the time step (a coupling code that
 * owns all device memory through its own pool, or code about to capture its
 * stream into a CUDA graph).  Computes, on the CURRENT CUDA device and on
 * `stream` (NULL = the default stream), the dt that an FP64 adiabatic
 * (dim 5) solver's do_step(dt0) would use for a conserved state already on
 * the device (a mixed-precision solver clips from FP32 candidates, within
 * ~1e-7 relative of this value; dim-4 isothermal states are not accepted):
 *   U            [n_faces][5] conserved state (device)
 *   unit_centres [n_faces][3] unit face centres, fc/|fc| (device)
 *   area         [n_faces] face areas (device)
 *   h0           minimum edge arc length (splash_geometry_info scalars[0])
 *   out          9 doubles (device): dt, max_vel, extra_dt, stop (1.0 when
 *                extra_dt_constr was negative), then the sums of
 *                Sigma*A, l_x*A, l_y*A, l_z*A, E*A.  dt, max_vel and
 *                extra_dt equal the solver's bit for bit; the sums are
 *                reduced in another order and agree to rounding.
 * It allocates nothing: the reduction's partial records live in a static
 * 1 MiB __device__ array inside the library (held by every GPU that loads
 * it until exit), so n_faces is limited to 4,194,304 (larger sizes return
 * SPLASH_E_INVALID).  The first call on a device looks up that array's
 * device address; make it before any stream capture (calls outside a
 * capture look it up again, calls inside one reuse the last).  All calls
 * share the array: calls that overlap on the GPU race.  Asynchronous on
 * `stream`. */
SPLASH_API int splash_cfl_dt_noalloc(const double* U, const double* unit_centres, const double* area,
                          int n_faces, double gam, double omega_ns, double alpha, double h0,
                          double dt0, double* out, void* stream);

/* ---- tangent-linear model and discrete adjoint of N FP64 do_step calls --
 * No counterpart in the reference (it has no derivative code).  The
 * differentiated map is U0 (and theta) -> the state after n_steps FP64
 * do_step(dt0) calls, with theta = {accretion_rate, tilt_angle,
 * omega_acc_abs} (the splash_params fields of the same names; the other
 * parameters, mesh, solver kind, gam and omega_ns come from `base`).  The
 * dt schedule of the forward run is frozen: the CFL clip is a min() and its
 * derivative is taken on the branch the forward took, so dt does not depend
 * on the state (splash_adjoint_info reports the steps the clip shortened).
 * Limiter kinks, Riemann wave-speed sides, HLLC+ switches and the density
 * and pressure floors likewise reuse the forward's branch choices.
 *
 * An adjoint object borrows the geometry of `base` (an FP64 solver, which
 * must outlive it) and owns its own state.  The forward run keeps the state
 * every `checkpoint_every` steps; the backward run recomputes each interval
 * from its checkpoint (the tape of one interval: checkpoint_every *
 * (20 + 42 * max_slots) * 8 bytes per face, 4.5 GB for icosphere_hex(6) at
 * 50 steps) and sweeps it in reverse.  States and adjoints are [n_faces][5] in reference face
 * order; every call is synchronous. */
typedef struct splash_adjoint splash_adjoint;

SPLASH_API int splash_adjoint_create(splash_solver* base, int checkpoint_every, splash_adjoint** out);
SPLASH_API int splash_adjoint_destroy(splash_adjoint* a);
/* Runs n_steps from U0 with theta (NULL: base's parameters); keeps the
 * checkpoints and the dt schedule; U_final may be NULL. */
SPLASH_API int splash_adjoint_forward(splash_adjoint* a, const double* U0, const double* theta, int n_steps,
                                      double dt0, double* U_final);
/* Given lambda_final = dLoss/dU_final of the last forward run, writes
 * grad_U0 = dLoss/dU0 ([n_faces][5]) and grad_theta[3] = dLoss/dtheta
 * (either may be NULL). */
SPLASH_API int splash_adjoint_backward(splash_adjoint* a, const double* lambda_final, double* grad_U0,
                                       double* grad_theta);
/* forward + loss = 1/2 sum_n area_n (Sigma_final_n - sigma_target_n)^2 +
 * backward (area from the base solver's geometry, reference order). */
SPLASH_API int splash_adjoint_run(splash_adjoint* a, const double* U0, const double* theta, int n_steps,
                                  double dt0, const double* sigma_target, double* loss, double* grad_U0,
                                  double* grad_theta);
/* Tangent-linear run: U_final and its directional derivative dU_final
 * along (dU0, dtheta) (NULL directions are zero).  The values are
 * bit-identical to the FP64 forward run. */
SPLASH_API int splash_tlm_run(splash_adjoint* a, const double* U0, const double* theta, const double* dU0,
                              const double* dtheta, int n_steps, double dt0, double* U_final,
                              double* dU_final);
/* Validation of the derivatives: the FP64 forward of n_steps steps from U0
 * and theta on the dt schedule of the last splash_adjoint_forward (which
 * must have run at least n_steps steps), with every branch decision of the
 * step (limiter cases and min/max arguments, Riemann-solver sides,
 * wave-speed fallbacks, floors) taped per face and launch:
 *   mode 1  record the decisions (the run is the plain FP64 forward);
 *   mode 0  replay the last recording: the branch-frozen map that the
 *           adjoint and the TLM differentiate; count = replayed decisions
 *           the run's own values would have taken the other way.  Where a
 *           replayed branch leads a formula out of its domain (the limiter
 *           switch's (1 - r)^0.1 on 0 < r < 1) the run returns NaN states;
 *   mode 2  the plain forward, compared with the recording; count = the
 *           (face, launch) evaluations whose branch path departs from the
 *           recorded one: the kink crossings between the two points.
 * The recording holds 64 bytes per face per launch (1 + 4 n_steps launches:
 * 10.5 GB for icosphere_hex(6) and 1000 steps).  count may be NULL.
 * Returns SPLASH_E_UNSUPPORTED if a face makes more decisions in one launch
 * than its tape slice holds (480).  No counterpart in the reference. */
SPLASH_API int splash_adjoint_branch_tape(splash_adjoint* a, const double* U0, const double* theta, int n_steps,
                                          int mode, double* U_final, int64_t* count);
/* out[8]: steps of the last forward, steps whose dt the CFL clip shortened,
 * min dt, max dt, forward ms, backward ms, last TLM ms (CUDA events), device
 * bytes held. */
SPLASH_API int splash_adjoint_info(splash_adjoint* a, double out[8]);
SPLASH_API int splash_adjoint_error_word(splash_adjoint* a, unsigned* err);
/* The dt of every step of the last forward run (n >= n_steps). */
SPLASH_API int splash_adjoint_dt_schedule(splash_adjoint* a, double* dts, int n);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* SPLASH_GB300_H */
