/*
 * mfree_gb300 -- C ABI of the GB300 (sm_103a) explicit meshless time step.
 *
 * This is the drop-in boundary for the reference's step loop: the caller builds
 * bodies of particles, registers the reference's action callbacks by id, optional
 * Dirichlet boundary conditions and contact boundaries, and steps.  Plain pointers
 * and sizes only; the context owns all device memory, the caller owns every host
 * buffer.  One context per host thread; calls on one context are not reentrant.
 * Every function returns an mf_status (0 = ok, < 0 = error); mf_last_error() gives
 * the message of the last failure on a context.
 *
 * Reference interfaces replaced (paths within the reference's src/):
 *   body<T>::body(particles, n, simulation_data, dt, bc)    body.h:216-217,228-233
 *   body<T>::add_action(void (*)(body<T>&))                  body.h:219-221
 *   body<T>::step()                                          body.h:223-225
 *   body<T>::set_boundary / update_boundary                  body.h:153-166,178
 *   boundary_conditions<T>::add_boundary_condition           boundary_conditions.h:32-34
 *   contact_apply_body_to_boundary(master, slave)            contact.h:36-80
 *   convex_hull(particles, n)                                convex_hull.h:62-95
 *   the step loop of main()                                  mfree_iwf.cpp:84-97
 */
#ifndef MFREE_GB300_H
#define MFREE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MF_API __attribute__((visibility("default")))
#else
#define MF_API
#endif

typedef struct mf_ctx mf_ctx;
typedef int32_t mf_status;

enum {
	MF_OK = 0,
	MF_ERR_ARG = -1,           /* invalid argument */
	MF_ERR_CUDA = -2,          /* CUDA runtime error (message in mf_last_error) */
	MF_ERR_NBH_OVERFLOW = -3,  /* neighbour count reached the capacity (the reference's assert, grid.h:167) */
	MF_ERR_NONFINITE = -4,     /* NaN/Inf in the state (the reference traps FE_INVALID|FE_OVERFLOW, mfree_iwf.cpp:40) */
	MF_ERR_TIMEOUT = -5,       /* a bounded device wait gave up */
	MF_ERR_PIPELINE = -6,      /* an action list the fused kernels do not implement */
	MF_ERR_GRID = -7,          /* num_cell >= n (grid.h:114) or a particle outside the grid */
	MF_ERR_STATE = -8,         /* call not valid in the context's current state */
	MF_ERR_NO_DEVICE = -9,     /* no CUDA device */
	MF_ERR_SINGULAR = -10,     /* singular corrector matrix (precomp_shape_functions.h:45) */
	MF_ERR_NO_NEIGHBOR = -11,  /* a particle without neighbours (grid.h:168) */
	MF_ERR_CAPACITY = -12,     /* a size beyond a documented maximum */
	MF_ERR_BODY_FAILED = -13   /* with per-body masking: some bodies failed and are frozen, the
	                              others stepped on (which: mf_get_failed) */
};

/* Method families (the reference's particle types). */
typedef enum {
	MF_METHOD_UL = 1,      /* particle_monaghan: updated-Lagrangian Gray-Monaghan SPH, grid rebuilt per stage */
	MF_METHOD_TL = 2,      /* particle_tl: total-Lagrangian SPH, fixed neighbours, Randles-Libersky correction */
	MF_METHOD_TL_WEAK = 3, /* particle_tl_weak: weak-form TL with RKPM shape functions and Gauss points */
	MF_METHOD_COROT = 4,   /* particle_corotational: TL neighbours, plain SPH weights, per-particle rotation */
	MF_METHOD_POTENTIAL = 5, /* particle_potential: TL neighbours, symmetric Randles-Libersky weights, elastic-potential
	                           pair forces */
	MF_METHOD_UL_WEAK = 6   /* particle_ul_weak: weak-form UL with stress points (mf_set_stress_points), per-stage
	                           neighbour ellipses from Manhattan candidates and RKPM shape functions */
} mf_method;

/* Arithmetic forms. */
typedef enum {
	MF_PREC_FP64_STRICT = 0, /* FP64, no FMA contraction: the reference-parity form */
	MF_PREC_FP64 = 1,        /* FP64 with FMA contraction */
	MF_PREC_MIXED = 2        /* FP32 pair sums and per-row algebra over float-float position and velocity
	                            differences (float-float where a sum sets a stress rate, as in the weak UL
	                            stress points); FP64 position/velocity RK4 state */
} mf_precision;

/* Action callbacks of the reference, by id (body<T>::add_action). */
typedef enum {
	MF_RIEMANN_UPDATE_INTEGRATION_WEIGHTS = 1,     /* riemann_integration.h:28-33 */
	MF_MATERIAL_EOS = 2,                           /* material.h:56-64 */
	MF_CORRECTORS_MGHN_ARTIFICIAL_STRESS = 3,      /* correctors.h:43-81 */
	MF_DERIVE_STRESS_MONAGHAN = 4,                 /* derivatives.h:378-443 */
	MF_DERIVE_VELOCITY = 5,                        /* derivatives.h:32-66 */
	MF_CORRECTORS_MGHN_ARTIFICIAL_VISCOSITY = 6,   /* correctors.h:83-137 */
	MF_CORRECTORS_XSPH = 7,                        /* correctors.h:139-169 */
	MF_MATERIAL_STRESS_RATE_JAUMANN = 8,           /* material.h:95-100 */
	MF_CONTMECH_CONTINUITY = 9,                    /* cont_mech.h:122-126 */
	MF_CONTMECH_MOMENTUM_UL = 10,                  /* cont_mech.h:32-49 */
	MF_CONTMECH_ADVECTION = 11,                    /* cont_mech.h:134-142 */
	MF_DERIVE_DISPLACEMENT = 12,                   /* derivatives.h:101-149 */
	MF_MATERIAL_COMPUTE_STRESS_GREEN_STVENANT = 13,/* material.h:155-161 */
	MF_CONTMECH_CAUCHY_TO_NOMINAL = 14,            /* cont_mech.h:213-218 */
	MF_DERIVE_STRESS_TL = 15,                      /* derivatives.h:331-376 */
	MF_CONTMECH_MOMENTUM_TL = 16,                  /* cont_mech.h:70-87 */
	MF_DERIVE_VELOCITY_TL = 17,                    /* derivatives.h:483-519 */
	MF_CONTMECH_VELOCITY_GRADIENT_TL = 18,         /* cont_mech.h:188-203 */
	MF_DERIVE_DISPLACEMENT_WEAK = 19,              /* derivatives.h:152-200 */
	MF_DERIVE_VELOCITY_TL_WEAK = 20,               /* derivatives.h:445-481 */
	MF_CONTMECH_VELOCITY_GRADIENT_TL_GP = 21,      /* cont_mech.h:171-186 */
	MF_CONTMECH_CONTINUITY_GP = 22,                /* cont_mech.h:128-132 */
	MF_MATERIAL_EOS_GP = 23,                       /* material.h:46-54 */
	MF_MATERIAL_STRESS_RATE_JAUMANN_GP = 24,       /* material.h:86-93 */
	MF_CONTMECH_CAUCHY_TO_NOMINAL_GP = 25,         /* cont_mech.h:206-211 */
	MF_DERIVE_STRESS_WEAK_TL = 26,                 /* derivatives.h:260-294 */
	MF_CONTMECH_MOMENTUM_TL_WEAK = 27,             /* cont_mech.h:89-106 */
	MF_COROTATIONAL_ANISOTROPY_TENSOR = 28,        /* corotational.h:32-84 */
	MF_DERIVE_DISPLACEMENT_COROTATIONAL = 29,      /* derivatives.h:202-258 */
	MF_MATERIAL_COMPUTE_STRESS_CAUCHY_GREEN = 30,  /* material.h:102-130 */
	MF_DERIVE_STRESS_COROTATIONAL = 31,            /* derivatives.h:521-588 */
	MF_GODUNOV_CONTINUITY = 32,                    /* godunov.h:144-187 (MF_METHOD_UL) */
	MF_GODUNOV_MOMENTUM = 33,                      /* godunov.h:86-142 (MF_METHOD_UL) */
	MF_POTENTIAL_COMP_ELASTIC_POTENTIAL = 34,      /* potential.h:32-83 (MF_METHOD_POTENTIAL) */
	MF_RIEMANN_UPDATE_INTEGRATION_WEIGHTS_GP = 35, /* riemann_integration.h:21-26 (MF_METHOD_UL_WEAK) */
	MF_DERIVE_STRESS_WEAK_UL = 36,                 /* derivatives.h:296-329 */
	MF_DERIVE_VELOCITY_WEAK = 37,                  /* derivatives.h:68-99 */
	MF_CONTMECH_MOMENTUM_UL_WEAK = 38,             /* cont_mech.h:51-68 */
	MF_INTERPOLATION_INTERPOLATE_VELOCITY = 39,    /* interpolation.h:32-59 */
	MF_CONTMECH_ADVECTION_GP = 40                  /* cont_mech.h:144-152 */
} mf_action;

/* Boundary-condition kinds (boundary_conditions<T> functors). */
typedef enum {
	MF_BC_PULL = 1,    /* x = X + v*t, y = Y, vx = v, vy = 0, vx_t = vy_t = 0 (tensile.cpp:20-42); TL-type bodies,
	                      at the start of every derivative evaluation */
	MF_BC_VELOCITY = 2 /* x_t = v, y_t = 0, vx = v, vy = 0, vx_t = vy_t = 0 (tensile.cpp:44-66); UL bodies, after
	                      every step (rk4.h:105) */
} mf_bc_kind;

typedef struct mf_config {
	int32_t method;      /* mf_method; every body of a context uses it */
	int32_t precision;   /* mf_precision */
	int32_t device;      /* CUDA device ordinal */
	uint32_t max_nbh;    /* neighbour capacity per particle; the reference's MAX_NBH is 200 (0 = 200) */
	double nbh_eps;      /* absolute epsilon of the predicate r^2 <= 4h^2 + eps (the reference: 1e-6) */
	double nbh_h;        /* TL / TL_WEAK: the h given to the set-up neighbour search (neighbor_search.h:116) */
	int32_t contact;     /* 1: after every step, penalty contact between bodies of a group (mfree_iwf.cpp:91-97) */
	int32_t graph;       /* 1: capture one step as a CUDA graph and replay it (not while timing is on) */
} mf_config;

/* simulation_data (simulation_data.h:25-99) */
typedef struct mf_sim_data {
	double nu, E, rho0;                          /* physical_constants */
	double mghn_wdeltap, mghn_corr_exp, mghn_eps;/* constants_monaghan */
	double artvisc_alpha, artvisc_beta, artvisc_eta; /* constants_artificial_viscosity */
	double xsph_eps;
	int32_t do_smooth;                           /* correctors_smooth_vel after each TL_WEAK step */
	int32_t reserved;
} mf_sim_data;

/* Initial particle state, host SoA of n doubles each (particle.h:42-47).
 * X, Y may be NULL for MF_METHOD_UL (they are then copies of x, y). */
typedef struct mf_particles {
	const double *x, *y, *X, *Y, *m, *rho, *h, *quad_weight, *vx, *vy, *Sxx, *Sxy, *Syy;
} mf_particles;

/* Output state, host SoA; any pointer may be NULL to skip that field. */
typedef struct mf_state {
	double *x, *y, *vx, *vy, *rho, *Sxx, *Sxy, *Syy, *fcx, *fcy;
} mf_state;

/* Context lifetime. */
MF_API mf_status mf_create(const mf_config* cfg, mf_ctx** out);
MF_API void mf_destroy(mf_ctx* ctx);
MF_API const char* mf_last_error(const mf_ctx* ctx);
MF_API const char* mf_status_string(mf_status s);

/* A body: n particles, its simulation_data and time step (body.h:228-233).
 * group: bodies with the same group are one simulation (contact only within a group). */
MF_API mf_status mf_add_body(mf_ctx* ctx, const mf_particles* p, uint32_t n, const mf_sim_data* sd, double dt,
                             int32_t group, int32_t* body_id);
/* Append an action to a body's action list (body.h:219-221). */
MF_API mf_status mf_add_action(mf_ctx* ctx, int32_t body, int32_t action);
/* Dirichlet condition on particles idx[0..k) (boundary_conditions.h:32-34). */
MF_API mf_status mf_add_boundary_condition(mf_ctx* ctx, int32_t body, const uint32_t* idx, uint32_t k, int32_t kind,
                                           double value);
/* Contact boundary: particle indices of the body's outline, in tour order (body.h:178, boundary.h:37-48). */
MF_API mf_status mf_set_boundary(mf_ctx* ctx, int32_t body, const uint32_t* idx, uint32_t nb);
/* MF_METHOD_TL_WEAK: the body's particles are the nodes of element_map_rectangle(ex, ey)
 * ((ex+1)*(ey+1) particles, ex+1 per row) with 2x2 Gauss points per element, whose h
 * and rho are gp_h and gp_rho (gauss_int, tensile.cpp:776-795). */
MF_API mf_status mf_set_gauss_mesh(mf_ctx* ctx, int32_t body, uint32_t ex, uint32_t ey, double gp_h, double gp_rho);
/* Weak-form shape functions of a MF_METHOD_TL_WEAK body (mf_set_elements). */
enum {
	MF_SHAPE_RKPM = 0,   /* RKPM on neighbourhoods of radius config.nbh_h (tensile.cpp:797-801) */
	MF_SHAPE_ELEMENT = 1 /* the elements' own bilinear functions: each Gauss point sees its element's four
	                        nodes (the *_fem set-ups: tensile.cpp:585-601, rotation.cpp:425-440, rings.cpp:742-790) */
};
/* MF_METHOD_TL_WEAK on an explicit element map (element.h: ll, lr, tr, tl particle indices of
 * the body per element, quads[4 e + k]): order x order Gauss points per element (order 1 or
 * 2; gauss_int::update_gauss_points, gauss_integration.h:47-123) placed on the particles'
 * reference positions X, with h = gp_h and rho = gp_rho (both positive) unless
 * mf_set_gauss_points gives them; `shape` is MF_SHAPE_RKPM or MF_SHAPE_ELEMENT.  Replaces mf_set_gauss_mesh. */
MF_API mf_status mf_set_elements(mf_ctx* ctx, int32_t body, const uint32_t* quads, uint32_t n_elem, uint32_t order,
                                 int32_t shape, double gp_h, double gp_rho);
/* The Gauss points' current position, h and rho as the set-up left them (e.g. moved with
 * their body after update_gauss_points, rings.cpp:1003-1013), n = order^2 * n_elem, point
 * order^2 e + (i order + j) for abscissae i (xi) and j (eta).  A point's displacement from
 * its place on X enters the displacement gradient (derivatives.h:296-345). */
MF_API mf_status mf_set_gauss_points(mf_ctx* ctx, int32_t body, const double* x, const double* y, const double* h,
                                     const double* rho, uint32_t n);

/* MF_METHOD_UL_WEAK: the body's stress points (the quad_points of body<particle_ul_weak>,
 * body.h:216-217), n of them, with the particles' field layout (X, Y may be NULL).  Their
 * candidate particles are found at the first step, as find_neighbors(particles, np,
 * stress_points, ns, config.nbh_h, distance_manhattan) does (neighbor_search.h:84-113);
 * the particles' own candidates likewise (:150-180).  Replaces body<T>(..., stress_points,
 * ns) (tensile.cpp:711). */
MF_API mf_status mf_set_stress_points(mf_ctx* ctx, int32_t body, const mf_particles* stress_points, uint32_t n);
/* Convex hull (monotone chain, collinear points kept) of n points: the reference's
 * set-up for contact boundaries (convex_hull.h:62-95).  out_idx holds n entries. */
MF_API mf_status mf_convex_hull(const double* x, const double* y, uint32_t n, uint32_t* out_idx, uint32_t* out_n);

/* Advance every body by nsteps RK4 steps in the reference driver's order: all bodies
 * step, boundaries are updated, then contact between ordered body pairs. */
MF_API mf_status mf_step(mf_ctx* ctx, int32_t nsteps);
/* Block until all queued work is done; returns the first device error. */
MF_API mf_status mf_synchronize(mf_ctx* ctx);

/* State access (device -> caller-owned host buffers, synchronous). */
MF_API mf_status mf_get_state(mf_ctx* ctx, int32_t body, const mf_state* out);
/* Overwrite a body's state (x, y, vx, vy, rho, Sxx, Sxy, Syy; NULL fields kept). */
MF_API mf_status mf_set_state(mf_ctx* ctx, int32_t body, const mf_particles* p);
/* All bodies at once: one row per particle of the context, the bodies' rows
 * concatenated in id order (one transfer per field instead of one per body and field;
 * for ensembles of hundreds of bodies). */
MF_API mf_status mf_get_state_all(mf_ctx* ctx, const mf_state* out);
MF_API mf_status mf_set_state_all(mf_ctx* ctx, const mf_particles* p);
/* The same transfers stream-ordered (strong forms): each returns once its work is
 * queued behind the steps already issued; host buffers (pinned, for the copies to run
 * asynchronously) are valid / reusable after mf_synchronize.  Per field, the
 * device->host copies run on one copy stream and the host->device copies on another;
 * a set waits, field by field, for an earlier get of the same field, so that a get and
 * a set of the same host arrays are ordered while the two directions of the host link
 * overlap.  No counterpart in the reference (its state lives in host memory). */
MF_API mf_status mf_get_state_all_async(mf_ctx* ctx, const mf_state* out);
MF_API mf_status mf_set_state_all_async(mf_ctx* ctx, const mf_particles* p);
MF_API mf_status mf_get_time(mf_ctx* ctx, int32_t body, double* t);
MF_API mf_status mf_num_particles(mf_ctx* ctx, int32_t body, uint32_t* n);
/* The stress the method evaluates at a body's current state, per particle.  TL (strong
 * form): the nominal stress P = J F^-1 sigma that derive_stress_tl consumes
 * (cont_mech.h:154-169), evaluated on the current state -- the reference keeps TL
 * stresses in per-stage particle copies only, and its state's Sxx, Sxy, Syy stay at
 * their initial values; UL: the state's S (Pxy = Pyx = Sxy).  Other methods return
 * MF_ERR_STATE. */
MF_API mf_status mf_get_stress(mf_ctx* ctx, int32_t body, double* Pxx, double* Pxy, double* Pyx, double* Pyy);
/* The weak forms' Gauss-point (TL) or stress-point (UL) state (rho, Sxx, Sxy, Syy;
 * NULL fields skipped), the bodies' points concatenated in id order; *n_out = number of
 * points (all NULL: only the count).  The particles' own S is not evolved by these
 * forms. */
/* Per-body failure words of an updated-Lagrangian context (0: running; otherwise the
 * bits of what failed it: 1 neighbour capacity, 2 no neighbour, 4 cell grid, 8
 * non-finite state).  Bodies fail alone only with the option "mask_failed" set
 * (mf_set_option): then a NaN, a neighbour overflow or a grid error in one body freezes
 * that body -- its rows leave the grid and the pair pass -- while the others step on
 * unchanged, and mf_step returns MF_ERR_BODY_FAILED instead of failing the whole step.
 * The reference aborts the process instead (assert, grid.h:167-168).  No counterpart
 * in the reference. */
MF_API mf_status mf_get_failed(mf_ctx* ctx, uint32_t* flags, uint32_t n_bodies);
MF_API mf_status mf_get_gauss_state(mf_ctx* ctx, double* rho, double* Sxx, double* Sxy, double* Syy, uint32_t cap,
                                    uint32_t* n_out);

/* Neighbour lists of a body's current state, as particle indices within the body:
 * for MF_METHOD_UL those of the next first-stage grid (grid.h:117-177), for TL the
 * fixed set-up lists.  counts[n]; idx holds up to cap entries; *total = sum(counts). */
MF_API mf_status mf_get_neighbors(mf_ctx* ctx, int32_t body, uint32_t* counts, uint32_t* idx, uint64_t cap,
                                  uint64_t* total);

/* Instrumentation: CUDA-event timing of the kernels, per kernel class. */
MF_API mf_status mf_set_timing(mf_ctx* ctx, int32_t enable);
/* kind: 0 = UL pair, 1 = TL pass A, 2 = TL pass B, 3 = contact, 4 = grid build, 5 = weak (Gauss) pass.
 * Returns the summed event time in ms, the launch count and rows processed. */
MF_API mf_status mf_kernel_stats(mf_ctx* ctx, int32_t kind, double* total_ms, uint64_t* launches, uint64_t* rows);
/* Number of kernel launches issued by this context since creation. */
MF_API mf_status mf_launch_count(mf_ctx* ctx, uint64_t* launches);
/* Autotuner: times the candidate launch shapes of the hot kernels (rows per block,
 * plain or persistent pair kernel, rows per work chunk) for trial_steps steps each on
 * a snapshot of the state, restores the state, and keeps the fastest.  Results are
 * cached per process by (method, precision, particle-count bucket, h bucket).  report (may be
 * NULL) receives a one-line summary. */
MF_API mf_status mf_autotune(mf_ctx* ctx, int32_t trial_steps, char* report, uint32_t report_len);
/* Per-step monitor: after every step each body's [mean vx, mean vy, max von Mises
 * stress, sum of |contact force|] is written on the device into a ring of `capacity`
 * rows (0 disables).  mf_get_monitor copies the min(steps, capacity) rows written,
 * row-major [row][body][4] floats (row = step % capacity), and their count. */
MF_API mf_status mf_set_monitor(mf_ctx* ctx, uint32_t capacity);
MF_API mf_status mf_get_monitor(mf_ctx* ctx, float* out, uint32_t* rows);
/* Tuning options (no counterpart in the reference).  Keys:
 *   "tl_tiles"        0 (default) / 1: the mixed TL passes gather neighbours from global
 *                     memory / stage each 128-row tile's neighbours in shared memory
 *                     (bit-identical results; the tiles are built at set-up, so set 1
 *                     before the first step)
 *   "ul_split"        1 (default) / 4 / 8: threads per row of the mixed UL pair pass
 *                     (plain grid; partial sums added across the row's threads, so the
 *                     pair sums change order); mf_autotune tries all three
 *   "async_steps"     0 (default) / 1: mf_step queues the steps and returns without
 *                     reading the device status word (no host synchronization per
 *                     call); errors -- and, with "mask_failed", failed bodies -- are
 *                     reported by the next mf_synchronize instead
 *   "contact_overlap" 1 (default) / 0: mixed total-Lagrangian bodies with contact run
 *                     the contact query of the positions a step ends with at the start
 *                     of the next step, beside stage 0's pass A on a second stream (the
 *                     pass reads no contact force), instead of at the end of the step:
 *                     bit-identical results.  Every call that reads the state or the
 *                     forces, replaces the state, dumps or tunes runs a pending query
 *                     first; off while the monitor or per-kernel timing is on.  Work a
 *                     caller enqueues on mf_get_stream between steps does not see the
 *                     forces of the last step until such a call.
 * read-only, through mf_get_option:
 *   "tl_tiles_built"  1 when the halo tiles exist (mixed TL, after the first step)
 *   "tl_halo_max"     the largest tile halo, in rows
 *   "weak_gauss_points", "weak_gp_entries", "weak_particle_entries"
 *                     MF_METHOD_TL_WEAK after the first step: the Gauss points, and the
 *                     entries of their lists and of the particles' transposed lists */
MF_API mf_status mf_set_option(mf_ctx* ctx, const char* key, int64_t value);
MF_API mf_status mf_get_option(mf_ctx* ctx, const char* key, int64_t* value);
/* ---------------------------------------------------------------------------
 * State output.  VTK files in the reference's legacy ASCII layout (vtk_writer_write,
 * vtk_writer.h:27-127: points, vertex cells, h, density, Sxx, Sxy, Syy, velocity;
 * "%f" text), and binary checkpoints that restore a context's state exactly (UL and TL
 * bodies: positions, velocities, density, stress, contact forces and clocks, in the
 * context's own precision).  mf_dump_async snapshots the state on the device behind
 * the steps already issued and writes the file from a host thread, so stepping can go
 * on; one dump is in flight at a time, mf_dump_wait returns its status.
 * ------------------------------------------------------------------------- */
enum { MF_DUMP_VTK = 0, MF_DUMP_CHECKPOINT = 1 };

typedef struct mf_vtk_body {
	uint32_t n;
	uint32_t reserved;
	const double *x, *y, *h, *rho, *Sxx, *Sxy, *Syy, *vx, *vy;
} mf_vtk_body;

/* Host-only writer: the bodies' particles in order into one file. */
MF_API mf_status mf_vtk_write(const char* path, const mf_vtk_body* bodies, uint32_t n_bodies);
MF_API mf_status mf_dump_async(mf_ctx* ctx, const char* path, int32_t kind);
MF_API mf_status mf_dump_wait(mf_ctx* ctx);
MF_API mf_status mf_write_vtk(mf_ctx* ctx, const char* path);         /* dump + wait */
MF_API mf_status mf_checkpoint_save(mf_ctx* ctx, const char* path);   /* dump + wait */
MF_API mf_status mf_checkpoint_load(mf_ctx* ctx, const char* path);
/* The context's CUDA stream (cudaStream_t), for callers that order their own work on it. */
MF_API mf_status mf_get_stream(mf_ctx* ctx, void** stream);

/* ---------------------------------------------------------------------------
 * Allocation-free UL step.  No counterpart in the reference: it exists for callers
 * that must not allocate device memory after start-up (applications that reserve all
 * GPU memory in their own pools, plug-ins that must not trigger the implicit device
 * synchronisation of cudaMalloc/cudaFree).
 * The caller passes device pointers to one body's particle arrays, updated in place;
 * all scratch of the step lives in one fixed array inside the library, sized for at
 * most MF_NOALLOC_MAX_PARTICLES particles (larger n returns MF_ERR_CAPACITY).  Every
 * call on a device shares that array: calls that overlap on the GPU race, so
 * serialise them.  The first call on a device looks up the array's address; make it
 * before any stream capture begins.  Form: FP64 strict, the reference predicate
 * epsilon 1e-6 and capacity 200; no contact, no boundary conditions.
 * ------------------------------------------------------------------------- */
#define MF_NOALLOC_MAX_PARTICLES 16384u

typedef struct mf_device_body {
	uint32_t n;
	uint32_t reserved;
	double *x, *y, *vx, *vy, *rho, *Sxx, *Sxy, *Syy;   /* device arrays, read and updated */
	const double *m, *h, *quad_weight;                  /* device arrays, read */
} mf_device_body;

/* nsteps RK4 steps of the updated-Lagrangian pipeline given by actions[0..n_actions)
 * (an ascending subsequence of the rings_monaghan list), on `stream` (a cudaStream_t,
 * NULL = default stream) of the current device; returns after the stream is idle. */
MF_API mf_status mf_ul_step_noalloc(const mf_device_body* body, const mf_sim_data* sd, double dt,
                                    const int32_t* actions, uint32_t n_actions, int32_t nsteps, void* stream);

/* ---------------------------------------------------------------------------
 * MLP surrogate.  No counterpart in the reference: an ensemble of `members` fully
 * connected ReLU networks (the last layer linear) with BF16 weights and activations,
 * FP32 accumulation and FP32 Adam master weights, trained on the device on solver
 * outputs.  Parameters of one member, as get/set_params exchange them: for each layer
 * l, W_l [dims[l+1]][dims[l]] row-major, then b_l [dims[l+1]].  Pointers to sample
 * arrays may be host or device memory.
 * ------------------------------------------------------------------------- */
#define MF_MLP_MAX_LAYERS 8
#define MF_MLP_MAX_WIDTH 512

typedef struct mf_mlp mf_mlp;

typedef struct mf_mlp_config {
	int32_t members;                      /* ensemble size, 1..64 */
	int32_t n_layers;                     /* weight layers, 1..MF_MLP_MAX_LAYERS */
	int32_t dims[MF_MLP_MAX_LAYERS + 1];  /* widths, input first, each 1..MF_MLP_MAX_WIDTH */
	int32_t max_batch;                    /* rows per pass: the training minibatch and the inference chunk */
	int32_t device;
	uint64_t seed;                        /* weight initialisation and minibatch sampling */
} mf_mlp_config;

MF_API mf_status mf_mlp_create(const mf_mlp_config* cfg, mf_mlp** model);
MF_API void mf_mlp_destroy(mf_mlp* model);
MF_API const char* mf_mlp_last_error(const mf_mlp* model);
MF_API mf_status mf_mlp_num_params(const mf_mlp* model, uint64_t* n);  /* per member */
MF_API mf_status mf_mlp_get_params(mf_mlp* model, int32_t member, float* params);
MF_API mf_status mf_mlp_set_params(mf_mlp* model, int32_t member, const float* params);
/* Gradients of the mean squared error (over batch x dims[L]) of every member on its own
 * batch x [members][batch][dims[0]] against y [members][batch][dims[L]]; loss (may be
 * NULL) receives [members].  mf_mlp_get_grads then returns one member's gradients in
 * the parameter layout.  batch <= max_batch. */
MF_API mf_status mf_mlp_gradients(mf_mlp* model, const float* x, const float* y, int32_t batch, float* loss);
MF_API mf_status mf_mlp_get_grads(mf_mlp* model, int32_t member, float* grads);
/* Training set x [n][dims[0]], y [n][dims[L]] (copied to the device). */
MF_API mf_status mf_mlp_set_data(mf_mlp* model, const float* x, const float* y, int32_t n);
/* `steps` Adam steps on minibatches of max_batch rows, each member drawing its own
 * rows with replacement; learning rate cosine-annealed from lr0 to lr1 over the call.
 * loss_history (may be NULL) receives [steps][members] minibatch losses. */
MF_API mf_status mf_mlp_train(mf_mlp* model, int32_t steps, float lr0, float lr1, float* loss_history);
/* Every member's outputs y [members][n][dims[L]] for x [n][dims[0]]. */
MF_API mf_status mf_mlp_predict(mf_mlp* model, const float* x, int32_t n, float* y);
MF_API mf_status mf_mlp_launch_count(const mf_mlp* model, uint64_t* launches);
MF_API mf_status mf_mlp_get_stream(const mf_mlp* model, void** stream);
/* Options: "tcgen05" (1: the forward products with K a multiple of 64 and N <= 256 run
 * on Blackwell's tcgen05 tensor cores with TMEM accumulators and TMA-staged operands,
 * the default on compute capability 10.x; 0: the mma.sync kernels). */
MF_API mf_status mf_mlp_set_option(mf_mlp* model, const char* key, int64_t value);
MF_API mf_status mf_mlp_get_option(const mf_mlp* model, const char* key, int64_t* value);

#ifdef __cplusplus
}
#endif

#endif
