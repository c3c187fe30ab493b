/*
 * vfvm_gb300.h -- C ABI of the GB300-native assembly + Newton library.
 *
 * This is the boundary a VoronoiFVM.jl shim binds with `ccall`.  Each entry
 * point replaces one piece of the reference's
 * hot path (paths relative to the VoronoiFVM.jl project):
 *
 *   vfvm_create            SystemState(sys) + update_grid_edgewise!
 *                          (src/vfvm_state.jl:99-157, src/vfvm_system.jl:690-755)
 *   vfvm_init_dirichlet    _initialize_dirichlet! (src/vfvm_system.jl:947-1003)
 *   vfvm_assemble          eval_and_assemble / evaluate_residual_and_jacobian
 *                          (src/vfvm_assembly.jl:520-643, src/vfvm_solver.jl:224-260)
 *   vfvm_pattern           the sparsity pattern of state.matrix after flush!
 *   vfvm_solve             solve_step! (src/vfvm_solver.jl:13-222) with the linear
 *                          solve of _solve_linear! (src/vfvm_linsolve.jl:6-61)
 *                          replaced by device Krylov
 *   vfvm_evolve            solve_transient! (src/vfvm_solver.jl:267-537)
 *   vfvm_set_params        replacing physics data between solves (the `data`
 *                          kwarg of solve!, src/vfvm_solver.jl:551-581)
 *
 * Conventions
 *   - all host arrays are caller-owned; the context owns its device buffers;
 *   - solution/residual vectors are the reference's dense solution layout
 *     (nspec x nnodes, column-major: dof = inode*nspec + ispec, 0-based,
 *     src/vfvm_system.jl:808-811);
 *   - grid index arrays are 0-based, region numbers are 1-based as in the
 *     reference;
 *   - return value: VFVM_OK or one of the error codes below, which map to the
 *     reference's exceptions (src/vfvm_logging_exceptions.jl:6-29).
 */
#ifndef VFVM_GB300_H
#define VFVM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define VFVM_OK 0
#define VFVM_ERR_CONVERGENCE 1  /* ConvergenceError (src/vfvm_solver.jl:196-198) */
#define VFVM_ERR_ASSEMBLY 2     /* AssemblyError: NaN assembled (src/vfvm_assembly.jl:10-12) */
#define VFVM_ERR_LINEAR 3       /* LinearSolverError: Krylov breakdown / no convergence */
#define VFVM_ERR_TIMEOUT 4      /* a bounded device wait expired */
#define VFVM_ERR_INPUT 5        /* bad argument (sizes, ids, indices) */
#define VFVM_ERR_CUDA 6         /* CUDA runtime error */
#define VFVM_ERR_EMBEDDING 7    /* step size fell below its minimum in vfvm_evolve */
#define VFVM_ERR_NOALLOC_LIMIT 8 /* system larger than the fixed work memory of a no-allocation entry point */

/* physics registry: device functors standing in for the Julia callbacks */
#define VFVM_PHYS_EX105 1             /* Example105 nonlinear Poisson 1D;     params: eps */
#define VFVM_PHYS_EX106 2             /* Example106 porous medium (u^m);      params: m */
#define VFVM_PHYS_EX110 3             /* Example110 two-species RD;           params: eps1, eps2 */
#define VFVM_PHYS_EX160 4             /* Example160 sedan drift-diffusion;    params: eps, z, V */
#define VFVM_PHYS_EX207 5             /* Example207 nonlinear Poisson 2D;     params: eps */
#define VFVM_PHYS_EX301 6             /* Example301 Laplace 3D with source */
#define VFVM_PHYS_EX440 7             /* Example440 Dirichlet + influx;       params: influx */
#define VFVM_PHYS_LAPLACE_DIRICHLET 8 /* test030 Laplace, u=0 (region 1), u=1 (region 2) */
#define VFVM_PHYS_NLPOISSON 11        /* -div grad u + u^3 = 1, u = 0 on the boundary */
#define VFVM_PHYS_POROUS 12           /* u_t - div grad u^2 = 0 */
#define VFVM_PHYS_BIPOLAR 13          /* bipolar drift-diffusion (psi,n,p);  params: lambda2,mu_n,mu_p,tau_n,tau_p,doping,V */
#define VFVM_PHYS_RD2 14              /* two-species reaction-diffusion;    params: D1, D2, k */
#define VFVM_PHYS_KAPPA_EXP 15        /* -div kappa grad u + exp(u) = f;     params: f; node data: kappa */
#define VFVM_PHYS_SURFACE_HEAT 16     /* heat equation + conducting surface layer (bflux, bstorage, bsource,
                                         breaction on boundary region breg; cf. Example311);
                                         params: eps, eps_s, c_s, k, q0, breg */
#define VFVM_PHYS_BOUNDARY_SPECIES 17 /* bulk species 1 and a boundary species 2 living on boundary region
                                         breg (examples/Example230_BoundaryFlux.jl): species 1
                                         -d u'' + k u = c; species 2 -d_b v'' + k_b(s) v = c_b(s) along
                                         breg (bflux, breaction, bsource) or, enabled as a bulk species
                                         of a 1D grid, in the bulk; s = the second coordinate on the
                                         boundary, the first in the bulk; k_b = kmax, c_b = 0 for
                                         s <= 1/2, else k_b = 0, c_b = cmax;
                                         params: d, k, c, d_b, kmax, cmax, breg */
#define VFVM_PHYS_EDGE_REACTION 18    /* u_t - div grad u = 1, u = 0 on boundary regions 1-6, the source as a
                                         node reaction (mode 0) or an edge reaction -h^2/(2 dim) (mode 1) or
                                         -(x_K - x_L)^2/2 (mode 2) (examples/DevEx002_EdgeReaction.jl);
                                         params: mode, dim */
#define VFVM_PHYS_JOULE_HEAT 19       /* potential phi and temperature T with Joule heating as an edge
                                         reaction (the callbacks of examples/Example206_JouleHeat.jl);
                                         params: kappa0, alpha, T0, lambda, c */
#define VFVM_PHYS_EX161 20            /* Example161 bipolar drift-diffusion in quasi-Fermi potentials (phi_n,
                                         phi_p, psi), doping per cell region 1/2/3, bias ramp in time on
                                         boundary region 2; params: Cn, Cp, Ca, En, Ep, mu_n, mu_p, lambda,
                                         tPrecond, tRamp, tExt, Vprecond, VExt, DirichletVal */
#define VFVM_PHYS_TESTFUNCTION 21     /* the Laplace system of TestFunctionFactory (flux u_K - u_L, storage u);
                                         Dirichlet values through the legacy boundary data */
#define VFVM_PHYS_EX430 22            /* Example430 (runh): flux (1+p)(u_K^2 - u_L^2), reaction p u^5, u = 0 on
                                         boundary region 1, u = p on region 3; p has parameter derivatives;
                                         params: p */
#define VFVM_PHYS_OUTFLOW 23          /* pressure + transported concentration with an outflow boundary (the
                                         reference's pluto-examples/outflow.jl: Darcy flux, Scharfetter-Gummel
                                         transport, boutflow on region G_out);
                                         params: k, v_in, c_in, D, G_in, G_out */
#define VFVM_PHYS_EX210 24            /* Example210 two-species linear reaction-diffusion with a Gaussian source,
                                         storage u, no-flux boundary; params: eps, k */
#define VFVM_PHYS_EX102 25            /* Example102 stationary convection-diffusion, velocity v along the first
                                         coordinate; params: D, v, flux (0 exponential, 1 upwind, 2 central) */
#define VFVM_PHYS_EX107 26            /* Example107 nonlinear storage (eps + u)^(1/m), flux u_K - u_L;
                                         params: m, eps */
#define VFVM_PHYS_EX115 27            /* Example115 heterogeneous catalysis: bulk species A, B, boundary species
                                         C on region iCat (mass-action breaction, bstorage);
                                         params: D_A, D_B, kp_AC, km_AC, kp_BC, km_BC, S, iCat */
#define VFVM_PHYS_EX215 28            /* Example215 two species, flux eps, storage u, boundary reaction
                                         k (u1 - u2) on boundary region 2; params: eps, k */
#define VFVM_PHYS_EX220 29            /* Example220 bulk species 1, 2 and boundary species 3 on region 2
                                         (breaction, bstorage), Gaussian source; params: k, eps */
#define VFVM_PHYS_EX203 30            /* Example203 -div grad u = f (flux u_K - u_L, constant source f), for the
                                         coordinate systems; params: f */

/* linear solver / preconditioner / precision selectors */
#define VFVM_KRYLOV_BICGSTAB 0
#define VFVM_KRYLOV_GMRES 1    /* restarted GMRES(gmres_restart), left-preconditioned (KrylovJL_GMRES in
                                  examples/DevEx004_EquationBlock3D.jl:187); single-system solves only:
                                  it runs on the persistent engine (VFVM_ENGINE_GRAPH, multi-region
                                  systems and batched solves return VFVM_ERR_INPUT) */
#define VFVM_GMRES_MAX_RESTART 32
#define VFVM_PRECON_JACOBI 0   /* (block-)Jacobi: inverse of the nspec x nspec diagonal blocks */
#define VFVM_PRECON_ILU0 1     /* ILU(0) in multicolour order */
#define VFVM_PRECON_BLOCK_ILU0 2 /* ILU(0) restricted to each CTA's node range (block-Jacobi with ILU0
                                    blocks; exact ILU0 when one CTA solves the system) */
#define VFVM_PRECISION_FP64 0  /* FP64 Jacobian and FP64 Krylov */
#define VFVM_PRECISION_MIXED 1 /* FP64 residual/update, FP32 Jacobian + FP32 Krylov (Newton refines) */

typedef struct vfvm_ctx vfvm_ctx;

typedef struct vfvm_grid {
  int32_t dim, nnodes, ncells, nbfaces;
  const double* coord;         /* dim x nnodes, column-major */
  const int32_t* cellnodes;    /* (dim+1) x ncells, column-major, 0-based */
  const int32_t* cellregions;  /* ncells, 1-based */
  const int32_t* bfacenodes;   /* dim x nbfaces, column-major, 0-based */
  const int32_t* bfaceregions; /* nbfaces, 1-based */
  int32_t coordsystem;         /* VFVM_COORD_*: the form factors (src/vfvm_formfactors.jl:12-332) */
} vfvm_grid;

/* coordinate systems (ExtendableGrids' CoordinateSystem, set by circular_symmetric! /
   spherical_symmetric!): the node volumes and edge factors of the symmetric body */
#define VFVM_COORD_CARTESIAN 0   /* any dimension */
#define VFVM_COORD_POLAR1D 1     /* 1D, r: a disk or ring (circular_symmetric! on a 1D grid) */
#define VFVM_COORD_SPHERICAL1D 2 /* 1D, r: a ball or shell (spherical_symmetric!) */
#define VFVM_COORD_CYLINDRICAL2D 3 /* 2D, (r, z): a cylinder (circular_symmetric! on a 2D grid) */

typedef struct vfvm_physics_desc {
  int32_t physics_id;
  int32_t nparams;
  const double* params;
  int32_t nnodedata;           /* values per node */
  const double* nodedata;      /* nnodes x nnodedata, node-major */
  int32_t nbregions;           /* legacy boundary data (boundary_dirichlet!(sys, ...)): */
  const double* bfactors;      /* nspec x nbregions, column-major; 1e30 marks Dirichlet */
  const double* bvalues;       /* nspec x nbregions */
  /* Species restricted to regions (enable_species!(sys, ispec, regions) and
   * enable_boundary_species!(sys, ispec, bregions), src/vfvm_system.jl:433-513).
   * Both counts 0: every species lives on every node (the default here).
   * Otherwise region_species (nspec x ncellregions_species, column-major) is
   * nonzero where species ispec is enabled in cell region ireg, bregion_species
   * (nspec x nbregions_species) where it is enabled on boundary region ibreg.  A
   * node carries a species when a cell of an enabled region or a boundary face
   * of an enabled boundary region contains it.  The unknowns stay dense (nspec
   * per node, the reference's DenseSystem): node, edge, boundary-node and
   * boundary-edge terms assemble the rows and columns of the species of their
   * region or node only (src/vfvm_assemblydata.jl:245-470), the other dofs get
   * F += U - Uold with a unit diagonal (src/vfvm_system.jl:1012-1026) and are
   * set to 0 before each Newton solve (:1030-1042).  The values on the enabled
   * dofs are those of the reference's sparse unknown storage as well.  Systems
   * with restricted species assemble with the node-centric kernel and run on
   * single-system solves (batched solves return VFVM_ERR_INPUT). */
  int32_t ncellregions_species;
  const int32_t* region_species;
  int32_t nbregions_species;
  const int32_t* bregion_species;
} vfvm_physics_desc;

/* SolverControl subset (src/vfvm_solvercontrol.jl:13-270) plus device solver settings. */
typedef struct vfvm_control {
  double abstol, reltol;       /* Newton update-norm tolerances */
  int32_t maxiters;
  double tol_round, tol_mono;
  double damp_initial, damp_growth;
  int32_t max_round;
  int32_t is_linear;           /* one Newton step (System(...; is_linear=true)) */
  int32_t updatecontrol;       /* 1: norm = max|update| (reference default); 0: norm = max|F|
                                  over the rows without a Dirichlet penalty, taken before the update */
  double reltol_linear, abstol_linear;
  int32_t maxiters_linear;
  int32_t krylov;              /* VFVM_KRYLOV_* */
  int32_t precon;              /* VFVM_PRECON_* */
  int32_t precision;           /* VFVM_PRECISION_* */
  int32_t gmres_restart;       /* GMRES: Krylov basis size before a restart, 1..VFVM_GMRES_MAX_RESTART */
  /* time / embedding step control (solve_transient!) */
  double dt, dt_min, dt_max, dt_grow, dt_decrease;
  double dp, dp_min, dp_max, dp_grow, dp_decrease;
  double du_opt, du_max_factor;
  int32_t num_final_steps, force_first_step, handle_exceptions, store_all;
  int32_t engine;              /* VFVM_ENGINE_*: how the device Newton loop is driven */
  int32_t team_ctas;           /* batched solves: CTAs per system (0 = default) */
  int32_t coarse;              /* coarse-grid correction stage of the preconditioner: about this many
                                  coarse unknowns (aggregates x nspec, at most VFVM_COARSE_MAX); 0 = off */
  int32_t batch_krylov_tail;   /* batched solves on the sweep engine: a Newton step's BiCGStab loop ends
                                  for all systems once at most this many are still iterating and they are
                                  at most a tenth of the systems that entered the loop; those take their
                                  current iterate as the (inexact) Newton update, judged by the same FP64
                                  residual.  0 = off (each system iterates to its own tolerance or
                                  maxiters_linear) */
} vfvm_control;

#define VFVM_COARSE_MAX 208

#define VFVM_ENGINE_GRAPH 0      /* CUDA graph of kernels with conditional WHILE nodes */
#define VFVM_ENGINE_PERSISTENT 1 /* one persistent cooperative launch per solve (or per fixed-step run) */
#define VFVM_ENGINE_AUTO 2       /* persistent for small systems (<= 16384 unknowns), graph otherwise */

/* NewtonSolverHistory (src/vfvm_history.jl:10-37), accumulated over a call. */
typedef struct vfvm_history {
  int32_t nnewton;             /* Newton iterations */
  int32_t nlin;                /* Krylov iterations */
  int32_t nsteps;              /* accepted time/embedding steps (vfvm_evolve) */
  int32_t status;
  double updatenorm;           /* last update norm */
  double resnorm;              /* max|F| over non-Dirichlet rows at the last Newton iteration */
  double time_ms, tasm_ms, tlinsolve_ms;
} vfvm_history;

/* Fill *c with the reference defaults (src/vfvm_solvercontrol.jl:30-257) and the
 * device solver defaults (BiCGStab, ILU0, FP64, abstol_linear = 0: the Krylov
 * tolerance is relative to the preconditioned right hand side). */
void vfvm_control_default(vfvm_control* c);

/* Create a context on the current CUDA device: tables, form factors, matrix
 * pattern, work buffers.  Returns NULL on failure with *status set. */
vfvm_ctx* vfvm_create(const vfvm_grid* grid, const vfvm_physics_desc* phys, int* status);
void vfvm_destroy(vfvm_ctx* ctx);

/* Test-function integrals (integrate(system, T, U) and its implicit Euler form,
 * src/vfvm_testfunctions.jl:125-380) of host arrays T (nnodes), U and Uold
 * (nspec x nnodes; Uold NULL: U), physics evaluated at (time, lambda) (the
 * reference uses 0 and 1).  out = 6 x nspec, per species: the flux term
 * sum fac flux (T_K - T_L), the reaction, source, storage(U) and storage(Uold)
 * terms sum fac f T_K, and the edge-reaction term sum fac r (T_K + T_L).
 * integrate(system, T, U) = flux + reaction - source + edge reaction; the
 * implicit Euler form adds (storage - old storage) / tstep. */
int vfvm_integrate(vfvm_ctx* ctx, const double* T, const double* U, const double* Uold, double time, double lambda,
                   double* out);

/* Parameter derivatives of the residual (the reference's dudp, accumulated by
 * asm_param in src/vfvm_assembly.jl:116-120, 194-198, 232-236, 403-405,
 * 434-436, 497-501) at the host array U: dudp = npd x nspec x nnodes (host),
 * the derivatives with respect to the first npd physics parameters, those the
 * physics differentiates (*npd = 0: none; dudp may be NULL to ask for npd). */
int vfvm_parameter_derivatives(vfvm_ctx* ctx, const double* U, double time, double tstep, double lambda,
                               double* dudp, int32_t* npd);

/* The ODE/DAE form (src/vfvm_diffeq_interface.jl:10-112): the right hand side
 * is -F and its Jacobian -J of vfvm_assemble at tstep = INFINITY; the mass
 * matrix is the storage Jacobian at U = 0 (storage and bstorage with their
 * node factors).  vals: its values in the scalar pattern of vfvm_pattern. */
int vfvm_mass_matrix(vfvm_ctx* ctx, double* vals);

/* sizes: out[0]=nspec, out[1]=nnodes, out[2]=nedges, out[3]=nnz of the scalar
 * pattern, out[4]=number of matrix blocks, out[5]=ncolors of the ILU0 ordering */
int vfvm_info(vfvm_ctx* ctx, int64_t out[8]);

/* Scalar CSR pattern of the Jacobian (rowptr: n+1, colind: nnz), rows/cols in dof order. */
int vfvm_pattern(vfvm_ctx* ctx, int64_t* rowptr, int32_t* colind);

/* Node volumes (sum of node factors over regions) and the per-edge form
 * factors (edge list oriented low -> high node index). */
int vfvm_geometry(vfvm_ctx* ctx, double* nodevolumes, double* edgefactors, int32_t* edgenodes);

/* Replace the physics parameter block (the `data` of the reference). */
int vfvm_set_params(vfvm_ctx* ctx, const double* params, int32_t nparams);

/* Replace the per-node physics data (nnodes x nnodedata values, node-major). */
int vfvm_set_nodedata(vfvm_ctx* ctx, const double* nodedata, int32_t nnodedata);

/* _initialize_dirichlet!: overwrite Dirichlet values in U (host array, n values). */
int vfvm_init_dirichlet(vfvm_ctx* ctx, double* U, double time, double lambda);

/* eval_and_assemble at U (Uold for storage terms; tstep = INFINITY is stationary).
 * F (n values) and Jvals (nnz values in vfvm_pattern order) are optional outputs. */
int vfvm_assemble(vfvm_ctx* ctx, const double* U, const double* Uold, double time, double tstep,
                  double lambda, double* F, double* Jvals);

/* solve_step!: one damped Newton solve from inival (also the old time step
 * solution for storage terms) at (time, tstep, lambda); result in U. */
int vfvm_solve(vfvm_ctx* ctx, const vfvm_control* control, const double* inival, double* U,
               double time, double tstep, double lambda, vfvm_history* hist);

/* solve_transient!: implicit Euler (transient != 0) or parameter embedding over
 * lambdas[0..nlambdas-1].  Stores up to max_store solutions (n values each) in
 * U_store and their times in t_store; *nstored receives the count. */
int vfvm_evolve(vfvm_ctx* ctx, const vfvm_control* control, const double* inival,
                const double* lambdas, int32_t nlambdas, int32_t transient, double time,
                double* U_store, double* t_store, int32_t max_store, int32_t* nstored,
                vfvm_history* hist);

/* solve_transient! with the step-size control on the device: the same
 * arguments and results as vfvm_evolve (lambdas must increase strictly;
 * max_store >= 1), but the step loop -- tentative step, Newton, the solution
 * change, accept / reject / grow (src/vfvm_solver.jl:350-513) -- runs as one
 * launch of a CUDA graph whose controller kernel decides every step on the
 * device; stored solutions are copied to the host once, at the end.  Uses the
 * graph engine with BiCGStab (GMRES: VFVM_ERR_INPUT); at most 262144 tentative
 * steps per call (then VFVM_ERR_EMBEDDING).  *host_syncs (optional)
 * receives the number of host synchronisations of the call (independent of the
 * number of steps). */
int vfvm_evolve_device(vfvm_ctx* ctx, const vfvm_control* control, const double* inival, const double* lambdas,
                       int32_t nlambdas, int32_t transient, double time, double* U_store, double* t_store,
                       int32_t max_store, int32_t* nstored, vfvm_history* hist, int32_t* host_syncs);

/* Device-resident variants: U_dev / inival_dev are device pointers (n doubles).
 * These run the same device loop without host<->device copies; the stream is
 * the context's stream (vfvm_stream). */
int vfvm_solve_device(vfvm_ctx* ctx, const vfvm_control* control, const double* inival_dev,
                      double* U_dev, double time, double tstep, double lambda, vfvm_history* hist);
int vfvm_evolve_fixed_device(vfvm_ctx* ctx, const vfvm_control* control, double* U_dev,
                             double t0, double dt, int32_t nsteps, vfvm_history* hist);
/* One assembly launch on device buffers (U_dev, Uold_dev, F_dev: n doubles); the
 * Jacobian goes to the context's block matrix (FP64, or FP32 with
 * VFVM_PRECISION_MIXED).  Enqueued on the context stream, not synchronised. */
int vfvm_assemble_device(vfvm_ctx* ctx, const double* U_dev, const double* Uold_dev, double time,
                         double tstep, double lambda, double* F_dev, int32_t precision);
void* vfvm_stream(vfvm_ctx* ctx);

/* Batched solves: many systems of one physics, uneven grids and parameters,
 * solved together in one persistent cooperative launch (a group of CTAs per
 * system, largest systems first).  The reference solves such sweeps with one
 * SystemState per thread (examples/Example440_ParallelState.jl:36-45); this is
 * the device counterpart.  Unknowns are packed system after system
 * (vfvm_batch_offsets gives the ninst+1 dof offsets). */
typedef struct vfvm_batch vfvm_batch;
vfvm_batch* vfvm_batch_create(int32_t ninst, const vfvm_grid* grids, const vfvm_physics_desc* phys, int* status);
void vfvm_batch_destroy(vfvm_batch* batch);
int vfvm_batch_offsets(vfvm_batch* batch, int64_t* offsets);
/* Replace system `inst`'s parameters and/or node data (NULL keeps them).  When
 * every grid passed to vfvm_batch_create used the same arrays, the systems share
 * one set of device grid tables. */
int vfvm_batch_set_instance(vfvm_batch* batch, int32_t inst, const double* params, int32_t nparams,
                            const double* nodedata, int32_t nnodedata);
/* Replace every system's parameters and/or node data (NULL keeps them) from
 * DEVICE arrays: params_dev = ninst x nparams (system-major), nodedata_dev = the
 * systems' nnodes_i x nnodedata blocks (node-major) one after another in system
 * order.  Device-to-device copies on the batch stream after the work already
 * queued on the legacy default stream (the stream frameworks write inputs on);
 * returns once they are complete.  The many-systems form of the reference's
 * new physics `data` between solves (src/vfvm_solver.jl:578-581). */
int vfvm_batch_load_device(vfvm_batch* batch, const double* params_dev, int32_t nparams,
                           const double* nodedata_dev, int32_t nnodedata);
/* out[0] = systems, out[1] = packed unknowns, out[2] = CTAs per system chosen
 * by vfvm_batch_tune (0: not tuned), out[3] = 1 if the last solve ran as a
 * captured CUDA graph, out[4] = engine of the last solve (0: persistent CTA
 * teams, one cooperative launch; 1: sweep engine, whole-GPU kernels over all
 * systems), out[5] = 1 if all systems share one grid, out[6] = kernels the
 * last solve launched (counted from the graph's loop iterations).  Shared-grid
 * batches with ILU0 (and no legacy boundary data) use the sweep engine unless
 * control->engine is VFVM_ENGINE_PERSISTENT. */
int vfvm_batch_info(vfvm_batch* batch, int64_t out[7]);
/* One stationary solve (tstep = INFINITY) or implicit Euler step of every
 * system from inival; hist (optional) receives one record per system. */
int vfvm_batch_solve(vfvm_batch* batch, const vfvm_control* control, const double* inival, double* U, double time,
                     double tstep, double lambda, vfvm_history* hist);
int vfvm_batch_solve_device(vfvm_batch* batch, const vfvm_control* control, const double* inival_dev, double* U_dev,
                            double time, double tstep, double lambda, vfvm_history* hist);
/* Guarded start for a proposed initial value (e.g. a learned prediction):
 * every system runs Newton from guess_dev for as long as each iteration reduces
 * the FP64 residual max-norm; where an iteration does not (or Newton fails
 * otherwise: NaN, no convergence) it restarts with plain Newton from
 * inival_dev.  Convergence is judged by the same FP64 residual test as
 * vfvm_batch_solve_device.  There is no counterpart in the reference, whose
 * solve() (src/vfvm_solver.jl:551-668) always starts from inival.
 * from_guess (optional, one per system) = 1 where the result came from the
 * guess; the Newton and Krylov counts in hist include abandoned iterations. */
int vfvm_batch_solve_guarded_device(vfvm_batch* batch, const vfvm_control* control, const double* guess_dev,
                                    const double* inival_dev, double* U_dev, double time, double tstep,
                                    double lambda, vfvm_history* hist, int32_t* from_guess);
/* Autotuner: times the batch from inival_dev (device) for each candidate -- CTAs
 * per system on the CTA-team engine, blocks per system on the sweep engine --
 * keeps the fastest for later solves of this batch and reports it in
 * *best_ctas; times_ms[k] = -1 for candidates that do not fit.  Returns
 * VFVM_ERR_INPUT for a control batched solves do not run (GMRES) or when no
 * candidate fits, and the solve's status when none converged; the previous
 * setting is kept in both cases. */
int vfvm_batch_tune(vfvm_batch* batch, const vfvm_control* control, const double* inival_dev, int32_t* best_ctas,
                    float* times_ms, int32_t ncand, const int32_t* candidates);

/* Device linear solve A x = b for a square CSR matrix: the reference's
 * linear-solver plug point (control.method_linear, src/vfvm_solvercontrol.jl:106,
 * called from _solve_linear!, src/vfvm_linsolve.jl:6-61), served by
 * Jacobi-preconditioned BiCGStab in one persistent cooperative launch.
 * rowptr (n+1), colind (nnz, 0-based), vals (nnz), b (n), x (n) are device
 * pointers; x receives the solution (initial guess 0).  Stops when the
 * preconditioned residual is below max(abstol, reltol * its initial value) or
 * after maxiters iterations.  The structure is validated on the device first
 * (VFVM_ERR_INPUT for bad row pointers, columns or a missing diagonal).
 * Allocates its work memory per call; runs on the legacy default stream. */
int vfvm_linsolve_csr(int32_t n, int64_t nnz, const int32_t* rowptr, const int32_t* colind,
                      const double* vals, const double* b, double* x, double reltol, double abstol,
                      int32_t maxiters, int32_t* iters, double* resnorm);

/* Same solve without any device allocation, for callers that cannot call
 * cudaMalloc where they solve (device memory owned by a framework's own pool,
 * allocation forbidden in the calling region, fixed pre-reserved buffers).
 * There is no counterpart in the reference.  The caller passes the matrix,
 * b and x as for vfvm_linsolve_csr; the work vectors live in a fixed
 * file-scope device array (about 7.7 MB, held by every GPU that loads the
 * library until exit), which limits n to VFVM_NOALLOC_MAX_ROWS rows: larger
 * systems return VFVM_ERR_NOALLOC_LIMIT.  Every call looks up the array's
 * address in the current CUDA context (no allocation); the first call in a
 * context also loads the library's device code there, so make that first call
 * before any stream capture.  All calls share the array: calls that overlap on
 * the GPU race on it and must be serialised by the caller. */
#define VFVM_NOALLOC_MAX_ROWS 131072
int vfvm_linsolve_csr_noalloc(int32_t n, int64_t nnz, const int32_t* rowptr, const int32_t* colind,
                              const double* vals, const double* b, double* x, double reltol, double abstol,
                              int32_t maxiters, int32_t* iters, double* resnorm);

/* Self-check of the bounded device waits behind VFVM_ERR_TIMEOUT (the
 * reference maps solver failures to exceptions, src/vfvm_logging_exceptions.jl:6-29;
 * a device wait that never ends has no counterpart there).  Runs the team
 * barrier of the persistent solvers in `ctas` CTAs told to expect one CTA more,
 * so every wait must give up after its spin limit (about a second): on return
 * *wait_status is VFVM_ERR_TIMEOUT when the limit worked, *ms (optional) the
 * kernel's duration.  The CUDA context stays usable; nothing traps or faults. */
int vfvm_check_bounded_wait(int32_t ctas, int32_t* wait_status, float* ms);

/* ---- learned initial iterate: a small multilayer perceptron ----
 * There is no counterpart in the reference: the network predicts a coarse
 * initial iterate for solve() (src/vfvm_solver.jl:551-668, argument inival),
 * and every solve started from it is still judged by the FP64 residual of the
 * Newton loop (src/vfvm_solver.jl:43-198).
 * Layers: sizes[0] inputs -> sizes[1] -> ... -> sizes[nlayers] outputs, ReLU on
 * hidden layers, linear output.  Operands BF16, accumulation FP32 (tensor-core
 * MMA), FP32 master weights, Adam (beta1 0.9, beta2 0.999, eps 1e-8), loss =
 * mean squared error.  X, T, Y are device pointers to row-major FP32 arrays of
 * batch rows; batch <= max_batch.  Calls are serial per network. */
typedef struct vfvm_mlp vfvm_mlp;
vfvm_mlp* vfvm_mlp_create(int32_t nlayers, const int32_t* sizes, int32_t max_batch, uint64_t seed, int* status);
void vfvm_mlp_destroy(vfvm_mlp* net);
/* number of parameters: sum over layers of sizes[l]*sizes[l+1] + sizes[l+1] */
int vfvm_mlp_nparams(vfvm_mlp* net, int64_t* n);
/* host copy of the parameters in the order W0 (sizes[0] x sizes[1], row-major),
 * b0, W1, b1, ...: out != NULL reads them, in != NULL replaces them */
int vfvm_mlp_params(vfvm_mlp* net, float* out, const float* in);
/* Y = net(X) */
int vfvm_mlp_forward(vfvm_mlp* net, int32_t batch, const float* X, float* Y);
/* gradients of the loss against T (host array in vfvm_mlp_params order) and the loss */
int vfvm_mlp_gradients(vfvm_mlp* net, int32_t batch, const float* X, const float* T, float* grads, float* loss);
/* one Adam step with learning rate lr; loss (optional) before the step */
int vfvm_mlp_train_step(vfvm_mlp* net, int32_t batch, const float* X, const float* T, float lr, float* loss);
/* fine = s_b * (scale * (bilinear prolongation of coarse) + shift) for batch
 * coarse fields (nc x nc nodes, x fastest, FP32) onto nested fine grids
 * ((nc-1)*ratio+1 nodes per side, FP64, the node order of simplexgrid);
 * instance b reads coarse + b*coarse_stride and writes fine + b*fine_stride;
 * s_b = inst_scale[b] (device array of batch values; NULL: 1).  Device
 * pointers, enqueued on stream (NULL: the legacy default stream). */
int vfvm_prolong_bilinear(int32_t batch, int32_t nc, int32_t ratio, const float* coarse, int64_t coarse_stride,
                          double scale, double shift, const double* inst_scale, double* fine, int64_t fine_stride,
                          void* stream);

/* Network input features on the device: for batch positive node fields on
 * nested square grids ((nc-1)*ratio+1 nodes per side, FP64, the node order of
 * simplexgrid), X[b] = the mean of log(field) over the (2*half+1)^2 fine nodes
 * around each node of the nc x nc coarse subgrid (clipped at the boundary;
 * half = 0: the node's own value), then extra[b] (NULL: 0).  X is FP32, batch
 * rows of nc*nc + 1 values.  Device pointers, enqueued on stream (NULL: the
 * legacy default stream). */
int vfvm_coarse_log_features(int32_t batch, int32_t nc, int32_t ratio, int32_t half, const double* field,
                             int64_t field_stride, const double* extra, float* X, void* stream);

#ifdef __cplusplus
}
#endif
#endif
