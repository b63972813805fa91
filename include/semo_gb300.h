/*
 * semo_gb300.h -- C-ABI of the GB300 (sm_103a) pressure-correction hot path.
 *
 * Drop-in for SEMO's per-outer-iteration hot path: owner/neighbour face
 * lists go in (OpenFOAM polyMesh order, as SEMO loads them), the assembled
 * pressure-correction system comes out as an RCM-reordered CSR matrix plus
 * right-hand side, and the solution vector of the AMG-preconditioned Krylov
 * solve comes out in the caller's cell order.  The momentum equation that
 * precedes it in each outer iteration (one matrix, three right-hand sides)
 * is assembled and solved the same way.
 *
 * Conventions
 *  - plain pointers and sizes; no CUDA or torch types.  Host pointers unless a
 *    function says otherwise.  The caller owns every array it passes; the
 *    context owns all device memory.
 *  - every call returns a semo_status; semo_last_error() gives the message.
 *  - calls on one context are synchronous at return and not re-entrant; one
 *    context drives one GPU through one CUDA stream.
 *  - cell indices at the boundary are the caller's (original) numbering;
 *    only the *_rcm getters expose the reordered numbering.
 */
#ifndef SEMO_GB300_H
#define SEMO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SEMO_OK = 0,
    SEMO_ERR_ARGUMENT = 1,       /* null pointer, bad size, bad enum */
    SEMO_ERR_MESH = 2,           /* malformed face lists, non-positive volume, singular LSQ */
    SEMO_ERR_CUDA = 3,           /* CUDA runtime failure (message has the CUDA error) */
    SEMO_ERR_OUT_OF_MEMORY = 4,
    SEMO_ERR_NOT_CONVERGED = 5,  /* Krylov hit max_iter above tol (solution still returned) */
    SEMO_ERR_NAN = 6,            /* NaN/Inf in inputs or in a residual */
    SEMO_ERR_BREAKDOWN = 7,      /* Krylov breakdown (p.Ap <= 0 or rho == 0) */
    SEMO_ERR_STATE = 8,          /* call out of order (e.g. solve before assemble) */
    SEMO_ERR_NO_DEVICE = 9       /* no CUDA device / extension built for another arch */
} semo_status;

typedef enum {
    SEMO_PREC_FP64 = 0,          /* AMG hierarchy, V-cycle and Krylov all FP64 */
    SEMO_PREC_MIXED = 1          /* FP32 AMG hierarchy + V-cycle inside FP64 CG */
} semo_precision;

typedef enum {
    SEMO_BC_ZERO_GRADIENT = 0,
    SEMO_BC_FIXED_VALUE = 1,
    SEMO_BC_NO_SLIP = 2,         /* velocity only */
    SEMO_BC_SLIP = 3             /* velocity only */
} semo_bc;

typedef enum {
    SEMO_EQ_PRESSURE = 0,        /* calcPressureEq's system */
    SEMO_EQ_MOMENTUM = 1,        /* calcMomentumEqs' matrix with its three right-hand sides */
    SEMO_EQ_VOF = 2,             /* calcVolfracEq's system */
    SEMO_EQ_COUPLED = 3          /* calcCompCoupledEq's 5x5 block system */
} semo_eq;

typedef struct semo_ctx semo_ctx;

typedef struct {
    int device;                  /* CUDA ordinal */
    int precision;               /* semo_precision */
    double tol;                  /* relative residual ||b-Ax||/||b|| (FP64), default 1e-8 */
    int max_iter;                /* Krylov iteration cap, default 500 */
    /* smoothed aggregation (AMGCL smoothed_aggregation semantics) */
    double eps_strong;           /* strength threshold, halved per level; default 0.03 (AMGCL: 0.08) */
    int coarse_enough;           /* direct solve at or below this size; default 64 */
    int max_levels;              /* default 24, at most 64 */
    int cheb_degree;             /* Chebyshev pre/post smoothing degree; default 2 */
    int reuse_hierarchy;         /* keep the pressure AMG hierarchy when the assembled matrix is bit-identical
                                    to the one it was built from (same hierarchy, same result); default 1 */
    /* momentum solve (BiCGStab, Jacobi preconditioner, per right-hand side) */
    double mom_tol;              /* relative residual, default 1e-9 (SEMO's momentum tolerance) */
    int mom_max_iter;            /* default 1000 */
    int overlap_setup;           /* semo_outer_iteration assembles the pressure matrix (which depends only on
                                    geometry, dt and the densities) and builds its hierarchy on a second stream
                                    while the momentum pass runs; same results bit for bit; default 1 */
    int smoother;                /* AMG smoother: 0 Chebyshev (degree cheb_degree, default), 1 multicolour
                                    Gauss-Seidel (a forward sweep before the coarse correction, a backward one
                                    after; colours from a deterministic Jones-Plassmann colouring of each
                                    level; AMGCL's relaxation/gauss_seidel.hpp family) */
} semo_params;

/* Physics of one outer iteration (calcMomentumEqs / calcPressureEq inputs). */
typedef struct {
    double dt;                   /* controls.timeStep */
    double rho[2];               /* phase densities; phase 0 is the volume fraction VF */
    double gravity[3];           /* controls.gravityAcceleration */
    int use_gravity;             /* compute the gravity body-force source */
    double urf_p;                /* controls.prePreURF */
    double urf_u;                /* controls.preVelURF */
    double p_min, p_max, u_min, u_max, v_min, v_max, w_min, w_max;  /* controls.min/max clamps */
    double mu[2];                /* phase viscosities (species[].mu), laminar */
    double urf_mom;              /* controls.momVelURF */
    double urf_vof;              /* controls.vofVofURF */
    double sigma;                /* species[0].sigma, surface tension; 0 (default) leaves out the curvature,
                                    the source and the face-velocity terms (calcSourceSurfaceTension,
                                    calcInterpolVelSurfTens) */
} semo_physics;

typedef struct {
    int iterations;
    double rel_residual;         /* FP64 ||b-Ax||/||b|| of the returned solution */
    int levels;
    int coarse_size;
    double operator_complexity;
    double setup_ms, solve_ms;   /* device time of AMG setup and Krylov iterations */
} semo_solve_info;

/* Fill *p with defaults. */
void semo_params_default(semo_params* p);
void semo_physics_default(semo_physics* p);

/* Context lifetime.  Replaces: nothing (SEMO has no solver handle; its
   solveAMGCL builds everything per call, src/solvers/solveAMGCL.cpp:179). */
semo_status semo_ctx_create(semo_ctx** out, const semo_params* prm);
semo_status semo_ctx_destroy(semo_ctx* ctx);
const char* semo_last_error(const semo_ctx* ctx);
/* The cudaStream_t the context launches on, as an opaque pointer (for timing). */
void* semo_stream(semo_ctx* ctx);

/* Mesh ingestion, OpenFOAM polyMesh arrays.  Computes the geometry on the
   GPU (src/mesh/geometric.cpp:792-1500 semantics), the vertex stencil
   (geometric.cpp:1781-1845), the LSQ normal-matrix inverses
   (src/math/gradient.cpp:246-453), the RCM order (src/math/RCM.cpp:34-218)
   and the CSR pattern with face->slot maps (src/mesh/build.cpp:1319-1424).
   Replaces: SEMO_Mesh_Load::OpenFoam post-load sequence
   (src/load/loadOpenFoam.cpp:356-374) + SEMO_Mesh_Geometric::init +
   SEMO_Utility_Math::initLeastSquare. */
semo_status semo_mesh_upload(semo_ctx* ctx, int n_points, const double* points /*3*n_points*/,
                             int n_faces, int n_internal, int n_cells,
                             const int32_t* face_ptr /*n_faces+1*/, const int32_t* face_pts,
                             const int32_t* owner /*n_faces*/, const int32_t* neighbour /*n_internal*/,
                             int n_patches, const int32_t* patch_start, const int32_t* patch_size);

/* OpenFOAM polyMesh directories (ASCII points, faces, owner, neighbour,
   boundary), read as SEMO_Mesh_Load::OpenFoam reads them
   (src/load/loadOpenFoam.cpp:16-350: coordinates parsed to long double and
   rounded to double, faces "n(p0 ... )", the neighbour list ending at ')' or
   a negative label, patches "name { nFaces N; startFace S; }").  These two
   need no context and no GPU; on failure semo_foam_last_error() gives the
   message (per thread).
   semo_foam_sizes: out6 = points, faces, internal faces, cells, face-point
   entries, patches.
   semo_foam_read: fills caller arrays of those sizes (points 3 per point,
   face_ptr n_faces+1); patch_names n_patches x 64 chars, NUL-terminated. */
semo_status semo_foam_sizes(const char* dir, int64_t* out6);
semo_status semo_foam_read(const char* dir, double* points, int32_t* face_ptr, int32_t* face_pts, int32_t* owner,
                           int32_t* neighbour, int32_t* patch_start, int32_t* patch_size, char* patch_names);
const char* semo_foam_last_error(void);

/* Read an OpenFOAM polyMesh directory and upload it (semo_mesh_upload on the
   arrays read).  Replaces: SEMO_Mesh_Load::OpenFoam (src/load/load.h:58,
   src/load/loadOpenFoam.cpp:8-383) with its post-load sequence. */
semo_status semo_mesh_load_foam(semo_ctx* ctx, const char* dir);

/* RCM permutation, bit-exact with SEMO_Utility_Math::lib_RCM
   (src/math/RCM.cpp:199-201): perm[r] = original cell at RCM position r
   (cells[r].RCM), iperm[c] = RCM position of original cell c (cells[c].invRCM). */
semo_status semo_rcm(semo_ctx* ctx, int32_t* perm, int32_t* iperm);

/* Boundary conditions and physics.  bc_type is n_patches x 3 (pressure,
   velocity, volume fraction: semo_bc); bc_value is n_patches x 5 (p, u, v, w,
   vf).  Replaces: boundary.type / boundary.var and controls fields read by
   src/solvers/reconIncom.cpp:501-1035 and src/solvers/eqPressure.cpp. */
semo_status semo_set_physics(semo_ctx* ctx, const semo_physics* phys,
                             const int32_t* bc_type, const double* bc_value);

/* Cell fields in the caller's cell order (host pointers, n_cells each). */
semo_status semo_set_fields(semo_ctx* ctx, const double* P, const double* U, const double* V,
                            const double* W, const double* VF);
semo_status semo_get_fields(semo_ctx* ctx, double* P, double* U, double* V, double* W);

/* One pressure-correction pass: EOS, face values, gravity source, stencil
   min/max, five LSQ gradients, face-loop assembly, AMG-Krylov solve, two
   Gauss-Green sweeps of grad p' and the P/U/V/W update.  Returns SEMO's
   ||dprim||/||prim|| in *norm.  Replaces: SEMO_Solvers_Builder::calcPressureEq
   (src/solvers/build.h:150-154, src/solvers/eqPressure.cpp:8-942) together
   with the setIncomValuesLeftRightFace / calcSourceGravity calls before it
   (src/solvers/pressureBased.cpp:139-141, :211). */
semo_status semo_pressure_pass(semo_ctx* ctx, double* norm, semo_solve_info* info);

/* Old (n-1) and second-old (n-2) velocities for the BDF2 time term of the
   momentum equation, caller's cell order (host pointers, n_cells each).  All
   NULL clears them: the momentum pass then uses the current velocity for both,
   as SEMO does on the first time step (src/solvers/pressureBased.cpp:33-52).
   Replaces: cell.var[oldU/oldV/oldW] and cell.var[Qm[0..2]]. */
semo_status semo_set_old_velocity(semo_ctx* ctx, const double* oldU, const double* oldV, const double* oldW,
                                  const double* old2U, const double* old2V, const double* old2W);

/* One momentum pass: cell viscosity, face values, stencil min/max of P, U, V,
   W, five LSQ gradients, BDF2 + upwind convection + over-relaxed diffusion
   assembly of one matrix with three right-hand sides (x, y, z), the three
   solves, and U,V,W += urf_mom x with the clamps.  Returns SEMO's
   ||dU||/||U|| in *norm; info points to 3 entries (x, y, z), or NULL.
   Replaces: SEMO_Solvers_Builder::calcCellTransport (src/solvers/transport.cpp:
   9-98) + calcMomentumEqs (src/solvers/build.h:135-139, src/solvers/
   eqMomentum.cpp:9-1122) and its 3-RHS solveAMGCL call (src/solvers/build.h:
   233-239, src/solvers/solveAMGCL.cpp:1116-1271), with Jacobi-preconditioned
   BiCGStab instead of AMGCL's aggregation/ILU0 FGMRES. */
semo_status semo_momentum_pass(semo_ctx* ctx, double* norm, semo_solve_info* info);

/* Momentum assembly only. */
semo_status semo_assemble_momentum(semo_ctx* ctx);

/* The assembled momentum system in SEMO's own layout, as solveAMGCL's COO to
   CSR conversion leaves it (src/solvers/solveAMGCL.cpp:1129-1172): caller's
   cell numbering, each row's entries in COO order (diagonal first, then one
   entry per internal face in face order), off-diagonals with |a| < DBL_MIN
   left out as calcMomentumEqs leaves them out (eqMomentum.cpp:699-711).  ptr
   is n_cells+1, col/val nnz, b 3*n_cells (x, y, z planes).  *nnz gets the
   entry count; every output may be NULL (call with NULLs to size). */
semo_status semo_get_momentum_system(semo_ctx* ctx, int32_t* ptr, int32_t* col, double* val, double* b,
                                     int64_t* nnz);

/* Solve the assembled momentum system; x is 3*n_cells (x, y, z planes) in
   the caller's cell order; info points to 3 entries or NULL. */
semo_status semo_solve_momentum(semo_ctx* ctx, double* x, semo_solve_info* info);

/* One outer iteration of the pressure-based solver with one pressure
   correction (src/solvers/pressureBased.cpp:200-213, iterPreMax = 1): the
   momentum pass, then the pressure pass on the updated velocity.  norms[0]
   momentum, norms[1] pressure; info points to 4 entries (momentum x, y, z,
   pressure) or NULL. */
semo_status semo_outer_iteration(semo_ctx* ctx, double* norms, semo_solve_info* info);

/* Old (n-1) and second-old (n-2) volume fraction for the BDF2 term of the
   volume-fraction equation, caller's cell order; both NULL clears them (the
   current VF is used for both).  Replaces: cell.var[oldVF[0]] and
   cell.var[Qm[3]] (src/solvers/pressureBased.cpp:33-67). */
semo_status semo_set_old_vf(semo_ctx* ctx, const double* oldVF, const double* old2VF);

/* One volume-fraction sub-iteration: zero-order face values, LSQ gradients,
   MSTACS face reconstruction of VF, BDF2 + upwind convection assembly with
   the Rhie-Chow face velocity, the solve, VF += urf_vof x clamped to [0, 1].
   Returns SEMO's sqrt(sum x^2) in *norm.  The gravity source is the one of
   the time step: computed once after fields or physics are set, as SEMO
   computes it once per time step.  Replaces:
   setIncomValuesLeftRightFaceWithVfMSTACS (src/solvers/reconIncom.cpp:345-429,
   src/solvers/NVD.cpp:1098-1790) + calcVolfracEq (src/solvers/build.h,
   src/solvers/eqVolfrac.cpp:9-795) with its solveAMGCL("volume_fraction")
   (src/solvers/solveAMGCL.cpp:862-884), with Jacobi-preconditioned BiCGStab. */
semo_status semo_vof_pass(semo_ctx* ctx, double* norm, semo_solve_info* info);

/* Volume-fraction assembly only. */
semo_status semo_assemble_vof(semo_ctx* ctx);

/* Curvature and surface-tension source from the current fields (needs
   phys.sigma != 0).  The passes compute it themselves with the gravity
   source, once per change of fields or physics, as SEMO does once per time
   step before its outer loop (src/solvers/pressureBased.cpp:142); every face
   velocity then takes calcInterpolVelSurfTens' terms
   (src/solvers/surfaceNormalVelocity.cpp:190-221) and the momentum right-hand
   side the source (src/solvers/eqMomentum.cpp:320-322).  Replaces:
   SEMO_Solvers_Builder::calcSourceSurfaceTension
   (src/solvers/source/surfaceTension.cpp:7-120) with calcCurvature
   (src/solvers/source/curvature.cpp). */
semo_status semo_source_surface_tension(semo_ctx* ctx);
/* Its results in the caller's cell order: kappa (controls.kappa), ls
   (controls.LS, the re-initialised level set) and src, 4 per cell
   (controls.sourceSurfaceTension[0..3]: sigma kappa grad VF, and its dot
   product with U).  Any pointer may be null. */
semo_status semo_get_surface_tension(semo_ctx* ctx, double* kappa, double* ls, double* src);

/* The assembled volume-fraction system in SEMO's layout (as
   semo_get_momentum_system; b is n_cells). */
semo_status semo_get_vof_system(semo_ctx* ctx, int32_t* ptr, int32_t* col, double* val, double* b, int64_t* nnz);

/* Solve the assembled volume-fraction system; x in the caller's cell order. */
semo_status semo_solve_vof(semo_ctx* ctx, double* x, semo_solve_info* info);

/* Assembly only (steps up to the face loop of calcPressureEq).  After it, the
   system can be read out or solved. */
semo_status semo_assemble_pressure(semo_ctx* ctx);

/* The assembled system in RCM order: ptr (n_cells+1), col (nnz), val (nnz),
   b (n_cells).  In-row order is SEMO's (diagonal first, then faces in face
   order, src/solvers/solveAMGCL.cpp:206-251).  nnz = n_cells + 2*n_internal. */
semo_status semo_get_system_rcm(semo_ctx* ctx, int32_t* ptr, int32_t* col, double* val, double* b);

/* Any assembled system in RCM order on the mesh's CSR pattern (the pattern
   semo_get_system_rcm gives, nnz = n_cells + 2*n_internal entries, diagonal
   first in each row, then faces in face order): eq is a semo_eq; val holds
   nnz values (25 per entry, row-major 5x5 blocks, for SEMO_EQ_COUPLED) with
   0.0 where SEMO leaves an entry out of the momentum or volume-fraction
   matrix; b holds 1 plane of n_cells (pressure, volume fraction), 3
   (momentum x, y, z) or 5 (coupled p, u, v, w, T).  Any output may be NULL.
   Replaces: the (A_rows, A_cols, A_vals, B) each calc*Eq hands solveAMGCL
   (src/solvers/eqPressure.cpp:677, eqMomentum.cpp:1017, eqVolfrac.cpp:766),
   reordered by lib_RCM. */
semo_status semo_get_system_rcm_eq(semo_ctx* ctx, int eq, int32_t* ptr, int32_t* col, double* val, double* b);

/* Intermediates of the last assembly, in the caller's cell order, for
   checking: name is one of "grad_P","grad_U","grad_V","grad_W","grad_VF"
   (3*n_cells, xyz interleaved), "minmax_uvw" (6*n_cells), "minmax_vf",
   "minmax_p" (2*n_cells), "rho", "mu", "VF" (n_cells), "src_grav" (4*n_cells),
   "face_UnF" (n_faces, face order), "face_VF_LR" (2*n_faces: the
   reconstructed left/right face VF of the last VOF assembly, interleaved),
   "geometry:<name>". */
semo_status semo_get_array(semo_ctx* ctx, const char* name, double* out, int64_t count);

/* Solve the assembled pressure system; x in the caller's cell order. */
semo_status semo_solve_pressure(semo_ctx* ctx, double* x, semo_solve_info* info);

/* Solve a caller-supplied scalar system given as SEMO's COO triple (first
   n entries are the diagonals, as calcPressureEq builds them).  x is in/out
   (initial guess in, solution out).  Replaces: SEMO_Solvers_Builder::solveAMGCL
   for B_n = 1 (src/solvers/build.h:225-231, src/solvers/solveAMGCL.cpp:179-1108),
   with smoothed-aggregation AMG + CG instead of AMGCL's IDR(s). */
semo_status semo_solve_coo(semo_ctx* ctx, int n, int64_t nnz, const int32_t* rows, const int32_t* cols,
                           const double* vals, const double* b, double* x, semo_solve_info* info);

/* Solve a caller-supplied scalar system (B_n = 1, SEMO's COO triple) for
   nrhs = 1, 2 or 3 right-hand sides b[j*n + i] by the momentum and volume-
   fraction solver: Jacobi-preconditioned BiCGStab to params.mom_tol, batched
   when nrhs = 3 (the matrix is read once per product for all three).  x is
   nrhs*n, in/out: the initial guess in (zeros, as SEMO passes resiVar, or
   any guess, from which the correction is solved), the solutions out.  Each
   row needs a non-zero diagonal entry (the preconditioner reads the row's
   first one).  info points to nrhs entries or NULL.  Replaces, with
   BiCGStab instead of AMGCL's aggregation/ILU0 FGMRES:
   SEMO_Solvers_Builder::solveAMGCL's three-right-hand-side overload
   (src/solvers/build.h:233-239, src/solvers/solveAMGCL.cpp:1116-1271) that
   calcMomentumEqs calls (src/solvers/eqMomentum.cpp:1017), with nrhs = 3;
   solveAMGCL("volume_fraction", mesh, 1, ...) (src/solvers/solveAMGCL.cpp:
   862-937) that calcVolfracEq calls (src/solvers/eqVolfrac.cpp:766), with
   nrhs = 1 (a non-symmetric matrix, which semo_solve_coo's CG does not take). */
semo_status semo_solve_coo_multi(semo_ctx* ctx, int nrhs, int n, int64_t nnz, const int32_t* rows,
                                 const int32_t* cols, const double* vals, const double* b, double* x,
                                 semo_solve_info* info);

/* Optional per-cell source s (caller's order) added to the pressure RHS as
   b_i += s_i * V_i after assembly; NULL clears it.  No reference counterpart
   (used by the adjoint check of the pressure solve). */
semo_status semo_set_source(semo_ctx* ctx, const double* s);

/* Discrete adjoint of the pressure solve + face-flux residual: given
   dJ/dx (caller's order), returns lambda = A^-T dJ/dx and dJ/ds for a per-cell
   source s entering as b_i += s_i * V_i.  No reference counterpart (SEMO has
   no adjoint). */
semo_status semo_vjp_source(semo_ctx* ctx, const double* dJ_dx, double* lambda, double* dJ_ds,
                            semo_solve_info* info);

/* Discrete adjoint of the pressure-correction equation with respect to the
   cell fields: given dJ/dx for the solution x of the assembled pressure
   system (caller's order), solves A^T lambda = dJ/dx on the forward solve's
   AMG hierarchy and returns the vector-Jacobian products
   dJ/dphi = lambda^T db/dphi for phi = U, V, W, P, where b is the face-flux
   right-hand side of calcPressureEq (src/solvers/eqPressure.cpp:246-673:
   the skew-corrected, stencil-limited face velocity and the Rhie-Chow
   pressure terms of src/solvers/surfaceNormalVelocity.cpp:100-187, the
   boundary-face rules) at the context's current fields; the matrix depends
   only on geometry, dt and the densities, so this is the whole gradient of
   J through the solve.  At a clamped face reconstruction the derivative
   goes to the stencil cell holding the limit.  The face gradients are
   recomputed from the cell fields, not kept from the forward pass.  Needs a
   forward solve (semo_pressure_pass, or semo_assemble_pressure and
   semo_solve_pressure).  Any output pointer may be NULL.  No reference
   counterpart (SEMO has no adjoint). */
semo_status semo_vjp_fields(semo_ctx* ctx, const double* dJ_dx, double* lambda, double* dJ_dU, double* dJ_dV,
                            double* dJ_dW, double* dJ_dP, semo_solve_info* info);

/* Measurement hooks (no reference counterpart).  With profiling on, the
   named stages are bracketed by CUDA events on the stream that runs them
   (the pressure setup's on its own stream when it is built beside the
   momentum pass): assembly "face_values","gravity","stencil" (LSQ gradients
   and limits of all five fields),"stencil_uvw" (their U, V, W part, when P
   and VF are unchanged since the last full pass),"surface_tension";
   pressure "pface","pbface","pcell","amg_setup" (with "setup_aggregate",
   "setup_prolong","setup_galerkin","setup_level","setup_coarse",
   "setup_cycle"),"pcg","vcycle","gauss_green","update"; momentum "mface",
   "mbface","mcell","msolve","mupdate"; volume fraction "mstacs","vface",
   "vsolve","vupdate"; coupled "cgrad","cface","ccell","csolve","cupdate".  semo_stage_time returns the summed device time and
   number of timed calls since the last semo_reset_stats. */
void semo_set_profiling(semo_ctx* ctx, int on);
semo_status semo_stage_time(semo_ctx* ctx, const char* stage, double* total_ms, int64_t* calls);
semo_status semo_reset_stats(semo_ctx* ctx);
/* Device time of one y = A x launch on the last pressure hierarchy (after a
   pressure solve), averaged over reps launches on the context's stream:
   which 0 is the finest level's operator in the layout and precision the
   V-cycle applies it, 1 the FP64 outer operator of the Krylov loop.  The
   result vectors are the solver's scratch.  No reference counterpart. */
semo_status semo_time_spmv(semo_ctx* ctx, int which, int reps, double* ms_per_launch);
/* Sizes of the last pressure hierarchy: 6 values per level (rows, nnz of A,
   nnz of the prolongator P, nnz of the restriction R, layout of A in the
   V-cycle: 2 SELL-32 with 16-bit column offsets, 1 SELL-32, 0 CSR, -1 the
   coarsest level's direct solve; bytes per value), at most max_levels
   levels written; *levels gets the level count.  No reference counterpart. */
semo_status semo_hierarchy_levels(semo_ctx* ctx, int64_t* out, int max_levels, int* levels);
/* Kernel launches made by this library in this process so far. */
int64_t semo_kernel_launches(void);
/* Allocation-free relative residual ||b - A x|| / ||b|| of a CSR system
   already in device memory (ptr, col, val, x, b are device pointers).  No
   reference counterpart: it is for callers that cannot call cudaMalloc --
   code that runs inside a memory arena or pool it manages itself, under a
   strict device-memory budget, or in a loop that must not synchronise the
   device through allocation calls.  It allocates nothing: its only scratch
   (one pair of partial sums per 32 rows) is a fixed 1 MiB array in the
   library's static device memory, held by every GPU that loads the library
   until the process exits.  Writes {||r||/||b||, ||r||, ||b||} to out3
   (device, 3 doubles) asynchronously on `stream` (a cudaStream_t, NULL for
   the default stream).  Rows above SEMO_STATIC_MAX_ROWS are rejected with
   SEMO_ERR_ARGUMENT.  Each call made outside stream capture looks up the
   array's device address again (so a re-created context is followed); a call
   made during capture reuses the last address found on that device and gets
   SEMO_ERR_STATE if there is none, so make the first call on each device
   before any stream capture.  An error already pending from the caller's own
   work is left pending and reported as SEMO_ERR_CUDA before any launch.
   Every call shares the array: calls that overlap on a GPU race, so callers
   serialise their calls on each GPU. */
#define SEMO_STATIC_MAX_ROWS 2097152
semo_status semo_residual_norm_static(const int32_t* ptr, const int32_t* col, const double* val, int n,
                                      const double* x, const double* b, double* out3, void* stream);

/* ---------------------------------------------------------------------------
   Compressible coupled system: one ideal-gas species, five unknowns per cell
   (p, u, v, w, T), 5x5 blocks on the cell's scalar pattern.  Replaces
   calcCompCoupledEq (src/solvers/build.h:210-214,
   src/solvers/compressible/coupled.cpp:8-2711) with the face and EOS
   helpers it calls (src/solvers/flux.cpp:924-949 M_func/pre_func,
   src/solvers/eos.cpp:310-437 calcCellEOSMF, :805-844 eosIdeal) and its
   solveAMGCL("coupled", mesh, B_n, ...) (src/solvers/solveAMGCL.cpp:
   179-251, 485-520).  The reference's body of calcCompCoupledEq is commented
   out; the formulas are those of its last live state, with zero-order face
   values.  Boundary types per patch (p, u, T) use SEMO_BC_* codes.
   --------------------------------------------------------------------------- */
typedef struct {
    double cv, gamma;            /* species cv [J/(kg K)] and gamma; cp = gamma cv */
    double mu;                   /* dynamic viscosity */
    double dt, dt_old, dt_old2;  /* controls.timeStep, oldTimeStep, old2TimeStep (bounded BDF2) */
    double gravity[3];           /* controls.gravityAcceleration */
    double urf;                  /* update relaxation of p, U, T (controls.momVelURF) */
    double limits[10];           /* (min, max) clamps of P, U, V, W, T after the update */
} semo_coupled_physics;

/* Physics and per-patch boundary conditions: bc_type n_patches x 3
   (p, u, T), bc_value n_patches x 5 (p, u, v, w, T). */
semo_status semo_set_coupled_physics(semo_ctx* ctx, const semo_coupled_physics* phys, const int32_t* bc_type,
                                     const double* bc_value);

/* Cell fields in the caller's order; old / old2 are the primitives at steps
   n-1 and n-2 as 5 planes (P, U, V, W, T) of n_cells, or NULL for "same as
   the current fields". */
semo_status semo_set_coupled_fields(semo_ctx* ctx, const double* P, const double* U, const double* V,
                                    const double* W, const double* T, const double* old, const double* old2);

/* Current primitives (after semo_coupled_pass) in the caller's order. */
semo_status semo_get_coupled_fields(semo_ctx* ctx, double* P, double* U, double* V, double* W, double* T);

/* Assembly only: 5x5 blocks and the field-split right-hand side on the GPU. */
semo_status semo_assemble_coupled(semo_ctx* ctx);

/* The assembled system in the caller's order: ptr/col as the scalar pattern
   (row i: diagonal, then one entry per internal face of i in face order),
   val 25 per entry, row-major (equation a = p, u, v, w, T; variable b),
   b field-split: b[a * n_cells + i].  Blocks are kept whole: an entry the
   reference would drop as |v| < DBL_MIN is stored as it is. */
semo_status semo_get_coupled_system(semo_ctx* ctx, int32_t* ptr, int32_t* col, double* val, double* b,
                                    int64_t* nnz);

/* Solve the assembled system to params.tol (FP64 relative residual); x
   field-split in the caller's order.  BiCGStab preconditioned by an AMG
   V-cycle on a pressure equation formed from the blocks, followed by the
   inverses of the 5x5 diagonal blocks; mixed precision multiplies by an
   FP32 copy of the matrix and runs the preconditioner in FP32 inside FP64
   defect correction. */
semo_status semo_solve_coupled(semo_ctx* ctx, double* x, semo_solve_info* info);

/* One calcCompCoupledEq: EOS, gradients, assembly, solve, update and the
   reference's norm sqrt(sum dx^2) / sqrt(sum prim^2) / 5. */
semo_status semo_coupled_pass(semo_ctx* ctx, double* norm, semo_solve_info* info);

/* Mesh counts: out[0..6) = cells, faces, internal faces, boundary faces,
   vertex-stencil entries, matrix nonzeros. */
semo_status semo_mesh_info(semo_ctx* ctx, int64_t* out6);

#ifdef __cplusplus
}
#endif
#endif
