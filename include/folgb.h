/*
 * folgb.h — C ABI of the GB300 finite-element weighted-residual library.
 *
 * Drop-in boundary for folax's FE loss / solver hot path.  Every entry point
 * takes plain pointers and sizes; device arrays are caller-owned, work is
 * ordered on the caller's CUDA stream, and status is returned as an int
 * (never thrown).  Per-call entry points allocate nothing: scratch memory is
 * the caller-provided workspace whose size folgb_workspace_bytes() reports.
 * Mesh tables are built once per mesh by folgb_plan_create() (the analogue of
 * the reference's FiniteElementLoss.Initialize and of an XLA FFI "State").
 *
 * Reference interfaces replaced (paths inside the folax project):
 *   fol/loss_functions/fe_loss.py           FiniteElementLoss
 *   fol/loss_functions/thermal.py, mechanical.py, mechanical_neohooke_AD.py,
 *   mechanical_neohooke.py, mechanical_saint_venant.py, transient_thermal.py
 *   fol/solvers/fe_solver.py                FiniteElementSolver.LinearSolve
 *   fol/loss_functions/ffi_functions/kr_small_displacement_element.cc
 *                                           (XLA FFI handler precedent)
 */
#ifndef FOLGB_H
#define FOLGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (kr_small_displacement_element.cc:56,220-222 returns
 *      ffi::Error::InvalidArgument / Internal; these are the C equivalents) */
enum {
  FOLGB_OK = 0,
  FOLGB_ERR_INVALID_ARGUMENT = 1,
  FOLGB_ERR_NONPOSITIVE_DETJ = 2, /* an element Jacobian determinant <= 0    */
  FOLGB_ERR_NAN = 3,              /* a non-finite energy / residual / norm   */
  FOLGB_ERR_NOT_CONVERGED = 4,    /* PCG hit maxiter above tolerance         */
  FOLGB_ERR_CUDA = 5,             /* a CUDA runtime call failed              */
  FOLGB_ERR_WORKSPACE = 6,        /* workspace NULL or smaller than required */
  FOLGB_ERR_NO_PATTERN = 7,       /* plan built without the CSR tables       */
  FOLGB_ERR_TOO_LARGE = 8,        /* problem exceeds a fixed-size scratch    */
  FOLGB_ERR_TIMEOUT = 9           /* a bounded device-side wait gave up      */
};
/* Device status words (the device_status arguments) collect 1 << code for
 * the codes found on the device.  1 << FOLGB_ERR_TIMEOUT means a kernel
 * stopped early after a bounded wait gave up: every output of that launch
 * (losses, gradients, records) is invalid and must not be used; callers that
 * consume results without reading the status word accept that risk. */

/* element types (fol/geometries/__init__.py:18-21) */
enum { FOLGB_QUAD4 = 0, FOLGB_HEX8 = 1, FOLGB_TET4 = 2 };
/* element physics */
enum {
  FOLGB_THERMAL = 0,  /* thermal.py:28-49                 */
  FOLGB_ELASTIC = 1,  /* mechanical.py:98-117             */
  FOLGB_NEOHOOKE = 2, /* mechanical_neohooke_AD.py:254-293 */
  FOLGB_SAINT_VENANT = 3, /* mechanical_saint_venant.py:263-296 */
  FOLGB_TRANSIENT_THERMAL = 4, /* transient_thermal.py:43-78: implicit Euler;
                                  the control is the current temperature
                                  field, the dofs the next one */
  FOLGB_NEOHOOKE_SPLIT = 5 /* mechanical_neohooke.py:243-275: neo-Hooke with a
                              volumetric-isochoric split, kappa and mu from
                              the Young's modulus control */
};
/* control layout: nodal values gathered by connectivity (fe_loss.py:160), or
 * one value per element used as de = value * 1 (partition of unity). */
enum { FOLGB_CONTROL_NODAL = 0, FOLGB_CONTROL_ELEMENT = 1 };
/* Neo-Hookean shear convention of the FE residual/tangent: REFERENCE doubles
 * the shear entries of S_voigt as constitutive_material_models/utils.py:45-56
 * does; CONSISTENT uses the true S (residual = energy gradient). */
enum { FOLGB_SHEAR_REFERENCE = 0, FOLGB_SHEAR_CONSISTENT = 1 };

typedef struct folgb_physics {
  int32_t element_type;   /* FOLGB_QUAD4 / HEX8 / TET4                         */
  int32_t physics;        /* FOLGB_THERMAL / ELASTIC / NEOHOOKE / SAINT_VENANT /
                             TRANSIENT_THERMAL / NEOHOOKE_SPLIT                 */
  int32_t num_gp;         /* Gauss order 1..3 ("num_gp", fe_loss.py:68-83)     */
  int32_t control_layout; /* FOLGB_CONTROL_NODAL / ELEMENT                     */
  int32_t shear_mode;     /* FOLGB_SHEAR_REFERENCE / CONSISTENT                */
  int32_t kernel_variant; /* 0: fastest kernel for the element (sum-factorised
                             hex8 2x2x2 elasticity, variant set by
                             folgb_autotune); 1: the generic Gauss loop;
                             2 + v: sum-factorised variant v (0..17) */
  double young_modulus;   /* material_dict young_modulus (elastic D scale)     */
  double poisson_ratio;   /* material_dict poisson_ratio                       */
  double body_force[3];   /* loss_settings "body_foce" (mechanical.py:27)      */
  double beta, c;         /* thermal conductivity nonlinearity (thermal.py:22) */
  double loss_exponent;   /* loss_function_exponent (fe_loss.py:117-120)       */
  /* transient thermal only (transient_thermal.py:20-41): rho * cp, the time
   * step, and material_dict "beta" (K = k0 (1 + material_beta T^c), c above);
   * the nodal k0 field is set with folgb_plan_set_nodal_field (default 1) */
  double rho_cp, time_step, material_beta;
} folgb_physics;

typedef struct folgb_plan folgb_plan;

/* Builds the per-mesh tables on the host and uploads them to the current
 * device.  conn (num_elements x nodes_per_element, row-major) and xyz
 * (num_nodes x 3) are HOST arrays in the reference's layout
 * (Mesh.GetElementsNodes / GetNodesCoordinates, mesh.py:150-169);
 * dirichlet_dofs/values are the reference's dirichlet_indices/values
 * (fe_loss.py:34-55, global dof = ndof*node + component).  build_csr != 0 also
 * builds the fixed CSR pattern and the element-to-nonzero map.
 * Replaces FiniteElementLoss.Initialize (fe_loss.py:57-122). */
int folgb_plan_create(folgb_plan** plan, const folgb_physics* phys,
                      const int64_t* conn, int64_t num_elements,
                      const double* xyz, int64_t num_nodes,
                      const int64_t* dirichlet_dofs, const double* dirichlet_values,
                      int64_t num_dirichlet, int32_t build_csr);
int folgb_plan_destroy(folgb_plan* plan);

/* Sizes of the plan: dofs per node, total dofs, CSR rows and nonzeros (nnz 0
 * when the plan has no CSR tables). */
int folgb_plan_info(const folgb_plan* plan, int64_t* ndof_per_node, int64_t* total_dofs,
                    int64_t* csr_rows, int64_t* csr_nnz);

/* Kernel paths the plan's mesh allows (bit flags): FOLGB_FEATURE_TILES, tile
 * tables of the tile-local hex8 kernels; FOLGB_FEATURE_UNIFORM_BOX, every
 * hexahedron is the same axis-aligned box (exactly, in fp32 coordinates), with
 * linear elasticity, element controls and no body force, so the box kernels
 * (hex8 variants 20-22) apply: the element matrix in the Walsh-Hadamard basis
 * of the nodal values is eight 3 x 3 blocks; FOLGB_FEATURE_BOX_GRID, such a
 * mesh numbered as the box mesh generator numbers it (nodes x fastest, then y,
 * then z), so the one-launch grid kernels (variants 23-24, loss exponent 1)
 * apply (a call whose dloss_ddofs is host memory runs the box kernel and the
 * gather instead: they write the gradients over the host link faster);
 * FOLGB_FEATURE_TET_PATCHES, a tet mesh whose consecutive groups of 6 elements
 * each span at most 8 nodes (the 6-tet split of hexahedra), so the loss +
 * adjoint of 3-component mechanics sums each group's node results before the
 * gather (one record per group node instead of one per element node; kernel
 * variant 1, the generic per-element loop, turns it off).  No counterpart in
 * the reference (a query of this library's specialisations). */
enum { FOLGB_FEATURE_TILES = 1, FOLGB_FEATURE_UNIFORM_BOX = 2, FOLGB_FEATURE_BOX_GRID = 4,
       FOLGB_FEATURE_TET_PATCHES = 8 };
int folgb_plan_features(const folgb_plan* plan, int32_t* features);

/* Sets the Dirichlet values used by the in-kernel GetFullDofVector, scaled by
 * load_increment (ApplyDirichletBCOnDofVector, fe_loss.py:186-189). values is a
 * HOST array in the order given to folgb_plan_create. */
int folgb_plan_set_dirichlet_values(folgb_plan* plan, const double* values, double load_increment);

/* Sets the plan's nodal material field (HOST, num_nodes doubles): the
 * transient-thermal conductivity k0 (material_dict "k0",
 * transient_thermal.py:24-33).  Other physics ignore it. */
int folgb_plan_set_nodal_field(folgb_plan* plan, const double* values);

/* Operation ids for folgb_workspace_bytes. */
enum { FOLGB_OP_LOSS_ADJOINT = 0, FOLGB_OP_ASSEMBLE = 1, FOLGB_OP_PCG = 2,
       FOLGB_OP_PLAIN = 3, FOLGB_OP_KRYLOV64 = 4 };
size_t folgb_workspace_bytes(const folgb_plan* plan, int32_t op, int32_t batch);

/* Fused FE loss + adjoint for a batch of instances on one mesh.
 * Replaces FiniteElementLoss.ComputeBatchLoss (fe_loss.py:250-262) and the
 * reverse-mode pass jax.grad takes through it, plus the material sensitivity
 * (fe_response.py:434-526 semantics for the loss).
 *   dofs    [batch][total_dofs] full DOF vectors (interleaved, ndof*node+c);
 *           when apply_dirichlet != 0 the plan's Dirichlet values replace the
 *           Dirichlet entries first (GetFullDofVector, fe_loss.py:91-100).
 *   control [batch][N or E] (stride 0 broadcasts one field to every instance)
 *   losses  [batch] per-instance loss L_b = (sum_e energy_e)^p
 *   dloss_ddofs    [batch][total_dofs] d(mean_b L_b)/d dofs, 0 at Dirichlet dofs
 *   dloss_dcontrol [batch][N or E]     d(mean_b L_b)/d control (true
 *                  derivative of the loss value)
 * Either gradient pointer may be NULL.  device_status (may be NULL) receives
 * FOLGB_ERR_NONPOSITIVE_DETJ / FOLGB_ERR_NAN found on the device (it is only
 * ever raised, never cleared, by the kernels). */
int folgb_loss_adjoint(const folgb_plan* plan, int32_t batch,
                       const float* control, int64_t control_stride,
                       const float* dofs, int64_t dofs_stride, int32_t apply_dirichlet,
                       float* losses, float* dloss_ddofs, float* dloss_dcontrol,
                       int32_t* device_status, void* workspace, size_t workspace_bytes,
                       void* stream);

/* Same values as folgb_loss_adjoint, computed the plain way: a forward pass
 * that materialises every element matrix Se in HBM (as the reference's
 * ComputeElement does, mechanical.py:112-117) and a separate backward pass
 * re = Se ue - Fe with its deterministic scatter.  Speed-up denominator. */
int folgb_loss_adjoint_plain(const folgb_plan* plan, int32_t batch,
                             const float* control, int64_t control_stride,
                             const float* dofs, int64_t dofs_stride, int32_t apply_dirichlet,
                             float* losses, float* dloss_ddofs, float* dloss_dcontrol,
                             int32_t* device_status, void* workspace, size_t workspace_bytes,
                             void* stream);

/* folgb_loss_adjoint for callers that cannot allocate device memory when they
 * evaluate the loss (a framework custom call with no scratch-buffer slot, a
 * fixed memory budget, code running inside an allocator hook).  No
 * counterpart in the reference.  Same arguments and results as
 * folgb_loss_adjoint minus the workspace: the scratch is a fixed 48 MiB array
 * inside the library's device image (enough for 64^3 hex8 elasticity, batch
 * 1: the size folgb_workspace_bytes(plan, FOLGB_OP_LOSS_ADJOINT, batch)
 * reports must fit).  Larger problems return FOLGB_ERR_TOO_LARGE.  The array
 * is committed on a device when the first plan is created there
 * (folgb_plan_create looks up its address), and held until exit; create
 * plans before any stream capture.  A call made under another CUDA context
 * than the one the address was found in (after cudaDeviceReset) looks it up
 * again.  The array is shared by all calls on a device, so calls that overlap
 * on the GPU race; order them on one stream.  Calls no allocator. */
int folgb_loss_adjoint_noalloc(const folgb_plan* plan, int32_t batch,
                               const float* control, int64_t control_stride,
                               const float* dofs, int64_t dofs_stride, int32_t apply_dirichlet,
                               float* losses, float* dloss_ddofs, float* dloss_dcontrol,
                               int32_t* device_status, void* stream);

/* Autotuner (no counterpart in the reference): times every kernel variant of
 * the plan's fused loss + adjoint on the caller's inputs (elements per block
 * and accumulation scheme of the sum-factorised hex8 kernel; plans with one
 * variant are a no-op) and keeps the fastest in the plan.  Arguments as
 * folgb_loss_adjoint with apply_dirichlet = 1; repeats timed calls per variant
 * (<= 0: 5).  *chosen gets the variant index, ms_per_variant[v] (may be NULL)
 * the mean time of variant v.  Synchronises the stream. */
int folgb_autotune(folgb_plan* plan, int32_t batch, const float* control, int64_t control_stride,
                   const float* dofs, int64_t dofs_stride, float* losses, float* dloss_ddofs,
                   float* dloss_dcontrol, void* workspace, size_t workspace_bytes, int32_t repeats,
                   void* stream, int32_t* chosen, float* ms_per_variant, int32_t max_variants);

/* folgb_autotune with the L2 cold before every timed call, as it is inside a
 * training step where other work runs between loss evaluations: the caller's
 * device buffer flush_buffer (flush_bytes, larger than the L2 cache, e.g.
 * 256 MiB on GB300) is overwritten before each timed call, outside its timing.
 * No counterpart in the reference. */
int folgb_autotune_flushed(folgb_plan* plan, int32_t batch, const float* control, int64_t control_stride,
                           const float* dofs, int64_t dofs_stride, float* losses, float* dloss_ddofs,
                           float* dloss_dcontrol, void* workspace, size_t workspace_bytes, int32_t repeats,
                           void* stream, int32_t* chosen, float* ms_per_variant, int32_t max_variants,
                           void* flush_buffer, size_t flush_bytes);

/* Copies the plan's CSR pattern (canonical: sorted column indices, one entry
 * per connected dof pair, the pattern scipy.sparse.csr_array builds from the
 * reference's BCOO, fe_solver.py:71-72) into device arrays indptr[rows+1],
 * indices[nnz]. */
int folgb_csr_pattern(const folgb_plan* plan, int32_t* indptr, int32_t* indices, void* stream);

/* ComputeJacobianMatrixAndResidualVector (fe_loss.py:264-318): BC-applied
 * residual [total_dofs] and Jacobian values [nnz] in the plan's CSR pattern,
 * assembled by a deterministic segmented reduction over the element-to-nonzero
 * map (no float atomics).  dofs must already hold the Dirichlet values.
 * transpose != 0 assembles the transposed element matrices (fe_loss.py:222-230).
 * csr_values or residual may be NULL to skip that output.  inv_diag (may be
 * NULL) receives 1/diag for the Jacobi preconditioner. */
int folgb_assemble(const folgb_plan* plan, const float* control, const float* dofs,
                   int32_t transpose, float* residual, float* csr_values, float* inv_diag,
                   int32_t* device_status, void* workspace, size_t workspace_bytes,
                   void* stream);

/* Jacobi-preconditioned CG on the plan's CSR (x0 = 0), replacing
 * FiniteElementSolver.LinearSolve (fe_solver.py:60-78) for symmetric positive
 * definite systems.  Matrix and Krylov vectors FP32, inner products, norms and
 * the iterate FP64; reliable updates recompute the true residual b - A x in
 * FP64, and convergence (||b - A x|| <= rtol ||rhs||) is judged on it.
 * The call returns after the solve: it runs folgb_krylov_async and reads its
 * report (while kernel tracing is on, a host-driven loop that reads the
 * device flags every check_every iterations instead).  Returns
 * FOLGB_ERR_NOT_CONVERGED at maxiter (x holds the last iterate).
 * iterations / rel_residual may be NULL. */
int folgb_pcg(const folgb_plan* plan, const float* csr_values, const float* inv_diag,
              const float* rhs, float* x, double rtol, int32_t maxiter, int32_t check_every,
              int32_t* iterations, double* rel_residual,
              void* workspace, size_t workspace_bytes, void* stream);

/* Jacobi-preconditioned BiCGSTAB with the same precision scheme, for
 * nonsymmetric or indefinite systems: the reference's default linear solver
 * (jax.scipy.sparse.linalg.bicgstab, fe_solver.py:60-67).  Same arguments and
 * workspace as folgb_pcg. */
int folgb_bicgstab(const folgb_plan* plan, const float* csr_values, const float* inv_diag,
                   const float* rhs, float* x, double rtol, int32_t maxiter, int32_t check_every,
                   int32_t* iterations, double* rel_residual,
                   void* workspace, size_t workspace_bytes, void* stream);

/* Either solver with the Krylov vectors in fp32 (vector_bits 32: the same as
 * folgb_pcg / folgb_bicgstab, workspace FOLGB_OP_PCG) or fp64 (vector_bits
 * 64, workspace FOLGB_OP_KRYLOV64).  The matrix, preconditioner and rhs stay
 * fp32.  fp64 vectors keep BiCGSTAB convergent on the indefinite,
 * ill-conditioned Neo-Hookean tangents where fp32 recurrences diverge (the
 * reference runs the same solver in fp32 JAX by default).  method:
 * FOLGB_KRYLOV_CG or FOLGB_KRYLOV_BICGSTAB. */
enum { FOLGB_KRYLOV_CG = 0, FOLGB_KRYLOV_BICGSTAB = 1 };
int folgb_krylov(const folgb_plan* plan, int32_t method, int32_t vector_bits,
                 const float* csr_values, const float* inv_diag, const float* rhs, float* x,
                 double rtol, int32_t maxiter, int32_t check_every, int32_t* iterations,
                 double* rel_residual, void* workspace, size_t workspace_bytes, void* stream);

/* Engine of large CG solves (no counterpart in the reference):
 * FOLGB_KRYLOV_ENGINE_GRID (default) runs a fp32-vector CG on more than
 * 16,384 dofs as one cooperative launch (every block resident, grid
 * barriers with bounded waits between the phases of an iteration, the
 * iteration's vector update fused into it); FOLGB_KRYLOV_ENGINE_KERNELS
 * runs the loop of SpMV and update kernels (what kernel tracing always uses).
 * Process-wide; both give the same iterates up to the order of fp32
 * rounding in the reductions. */
enum { FOLGB_KRYLOV_ENGINE_GRID = 0, FOLGB_KRYLOV_ENGINE_KERNELS = 1 };
int folgb_krylov_set_engine(int32_t engine);

/* Stream-ordered folgb_krylov, for callers that must not block (an XLA FFI
 * LinearSolve handler on XLA's stream; fe_solver.py:60-78 is the reference
 * call, kr_small_displacement_element.cc:315-337 the handler precedent, whose
 * handlers enqueue their work on the given stream and return an error code).
 * Enqueues the whole solve on `stream` and returns: no host synchronisation,
 * no allocation.  The outcome goes to caller DEVICE buffers (any may be
 * NULL): *d_iterations, *d_rel_residual (true residual of the fp64 iterate)
 * and *d_status (FOLGB_OK, FOLGB_ERR_NOT_CONVERGED, FOLGB_ERR_NAN, or
 * FOLGB_ERR_TIMEOUT when a grid barrier of the grid engine gave up).  The
 * return value reports argument and launch errors only.
 * The solve runs as an instantiated CUDA graph (init, a WHILE node over
 * chunks of check_every iterations with the true-residual check, the fp32
 * copy of x, the report), built on the first call with a given set of
 * buffers, method, precision, rtol, maxiter and check_every and cached in the
 * plan (the 8 most recent sets); later calls with the same arguments launch
 * the cached graph.  On a stream that is being captured the same nodes are
 * added to the caller's graph instead.  Workspace as folgb_krylov; calls that
 * share a workspace must be ordered on one stream. */
int folgb_krylov_async(const folgb_plan* plan, int32_t method, int32_t vector_bits,
                       const float* csr_values, const float* inv_diag, const float* rhs, float* x,
                       double rtol, int32_t maxiter, int32_t check_every, int32_t* d_iterations,
                       double* d_rel_residual, int32_t* d_status, void* workspace,
                       size_t workspace_bytes, void* stream);

/* ---- device-resident Newton-Raphson with load stepping --------------------
 * FiniteElementNonLinearResidualBasedSolver.Solve
 * (fol/solvers/fe_nonlinear_residual_based_solver.py:76-170) as ONE CUDA
 * graph launched once: a WHILE node over Newton iterations, each [the
 * load-scaled Dirichlet values written into dofs at the start of a load step
 * (ApplyDirichletBCOnDofVector, fe_loss.py:186-189, with the plan's Dirichlet
 * values), residual + CSR tangent assembly (folgb_assemble), |r| and
 * rhs = -r, the Krylov solve of folgb_krylov (itself a nested WHILE node),
 * |du|, the convergence test, dofs += du].  Convergence as the reference:
 * |r| < abs_tol or |du| < rel_tol or max_iterations, the converged
 * iteration's update not applied; a non-finite |r| stops the solve with
 * FOLGB_ERR_NAN (the reference raises, :122-136).  Norms are fp64.  No host
 * synchronisation until the end; the call then waits for the stream. */
typedef struct folgb_newton_settings {
  int32_t load_steps;       /* nonlinear_solver_settings "load_incr"  */
  int32_t max_iterations;   /* "maxiter" per load step                */
  double abs_tol, rel_tol;  /* "abs_tol" on |r|, "rel_tol" on |du|    */
  int32_t krylov_method;    /* FOLGB_KRYLOV_CG / FOLGB_KRYLOV_BICGSTAB */
  int32_t vector_bits;      /* 32 or 64 (folgb_krylov)                */
  double krylov_rtol;       /* linear_solver_settings "tol"           */
  int32_t krylov_maxiter, check_every;
  /* Globalisation (no counterpart in the reference, whose Newton takes full
   * steps): 0 full steps; 1 backtracking line search on the element energy
   * (the plan's loss with exponent 1): the step t du, t = 1, 1/2, 1/4, ...
   * is taken once E(u + t du) <= E(u) + 1e-4 t (r . du) + 2e-6 |E(u)| and is
   * finite (no inverted element), at most line_search_max_halvings halvings
   * (then the solve stops with FOLGB_ERR_NOT_CONVERGED); a step whose
   * predicted decrease -(r . du) is below 1e-6 |E(u)| (the energy's fp32
   * resolution) is taken whole; a Newton step that is not a descent
   * direction (r . du >= 0: an indefinite tangent) or that the Krylov solve
   * left non-finite is replaced by the Jacobi-preconditioned steepest descent
   * step -D^-1 r.  Valid where the residual is the energy gradient:
   * neo-Hooke with FOLGB_SHEAR_CONSISTENT, no body force. */
  int32_t line_search, line_search_max_halvings;
} folgb_newton_settings;
typedef struct folgb_newton_info {
  int32_t newton_iterations;   /* over all load steps                 */
  int64_t krylov_iterations;   /* sum over the Newton iterations      */
  double last_res_norm, last_delta_norm;
  int32_t krylov_failures;     /* linear solves that ended non-finite / broke down */
  int32_t status;              /* FOLGB_OK, FOLGB_ERR_NAN, or FOLGB_ERR_NOT_CONVERGED
                                  (a line search that found no acceptable step) */
  int32_t line_search_halvings; /* over all Newton iterations           */
} folgb_newton_info;
size_t folgb_newton_workspace_bytes(const folgb_plan* plan, const folgb_newton_settings* settings);
/* dofs [total_dofs] (device): the initial guess in, the solution out.
 * history (HOST, may be NULL): 4 doubles per Newton iteration, at most
 * load_steps * max_iterations rows: (load step, iteration, |r|, |du|).
 * Needs a plan with the CSR tables; the caller's stream must not be capturing. */
int folgb_newton(const folgb_plan* plan, const float* control, float* dofs, const folgb_newton_settings* settings,
                 folgb_newton_info* info, double* history, int32_t* device_status, void* workspace,
                 size_t workspace_bytes, void* stream);

/* y = A x on the plan's CSR (FP32). */
int folgb_spmv(const folgb_plan* plan, const float* csr_values, const float* x, float* y,
               void* stream);

/* Adam update of a parameter array in place (optax.adam as used by the
 * reference's training loop, deep_network.py:100,141; tests/integration/
 * test_thermal_2D.py:58-59).  step_counter is a device int incremented by
 * the kernel, so the launch can be replayed inside a CUDA graph. */
int folgb_adam_step(float* params, const float* grads, float* m, float* v, int64_t n,
                    int32_t* step_counter, float lr, float beta1, float beta2, float eps,
                    void* stream);

/* ---- many instances with uneven meshes in one launch ------------------- */
typedef struct folgb_batch_plan folgb_batch_plan;

/* Builds one plan over num_instances meshes of one element type and physics,
 * concatenated (HOST arrays): element_offsets[num_instances+1] into conn
 * (rows of nodes_per_element LOCAL node ids) and node_offsets[num_instances+1]
 * into xyz.  Dirichlet dofs are GLOBAL dofs of the concatenated dof vector.
 * The reference batches only one mesh (fe_loss.py:250-262); this has no
 * counterpart there. */
int folgb_batch_plan_create(folgb_batch_plan** plan, const folgb_physics* phys,
                            int32_t num_instances, const int64_t* element_offsets,
                            const int64_t* node_offsets, const int64_t* conn, const double* xyz,
                            const int64_t* dirichlet_dofs, const double* dirichlet_values,
                            int64_t num_dirichlet, int32_t elements_per_tile);
int folgb_batch_plan_destroy(folgb_batch_plan* plan);
size_t folgb_batch_workspace_bytes(const folgb_batch_plan* plan);

/* Fused loss + adjoint over every instance in one persistent launch (plus one
 * deterministic gather launch).  losses[num_instances]; gradients are of
 * mean_i L_i.  dofs/control/gradients are concatenated over instances. */
int folgb_batch_loss_adjoint(const folgb_batch_plan* plan, const float* control,
                             const float* dofs, int32_t apply_dirichlet, float* losses,
                             float* dloss_ddofs, float* dloss_dcontrol, int32_t* device_status,
                             void* workspace, size_t workspace_bytes, void* stream);

/* Autotuner of the batched launch: times folgb_batch_loss_adjoint with 256,
 * 512, 1024, 2048 and 4096 elements per tile on the caller's inputs (2
 * warm-up and `repeats` timed calls each; flush_buffer, if not NULL, is
 * overwritten before every timed call, outside its timing) and keeps the
 * fastest in the plan: *chosen_tile, and ms_per_candidate[k] for the first
 * max_candidates sizes.  The workspace is that of folgb_batch_workspace_bytes
 * (it covers every tile size).  Synchronises the stream.  No counterpart in
 * the reference. */
int folgb_batch_autotune(folgb_batch_plan* plan, const float* control, const float* dofs,
                         int32_t apply_dirichlet, float* losses, float* dloss_ddofs,
                         float* dloss_dcontrol, int32_t* device_status, void* workspace,
                         size_t workspace_bytes, int32_t repeats, void* flush_buffer, size_t flush_bytes,
                         void* stream, int32_t* chosen_tile, float* ms_per_candidate,
                         int32_t max_candidates);

/* ---- adjoint sensitivities of an integral response ------------------------
 * FiniteElementResponse (fol/responses/fe_response.py:17-526) for thermal and
 * linear-elastic plans: J = sum_e sum_gp w detJ f(d_gp, u_gp) with d_gp, u_gp
 * the control and dofs interpolated at the Gauss point (:92-120) and f a
 * polynomial, sum_k coeff_k * d^control_power_k * prod_i u_i^dof_power_k[i]
 * (the host parses the reference's response formula string into monomials).
 * Any output may be NULL:
 *   value        device scalar J (ComputeValue, :208-225);
 *   adjoint_rhs  -(dJ/du) with zeros on Dirichlet dofs
 *                (ComputeAdjointJacobianMatrixAndRHSVector, :244-283; the
 *                matrix is folgb_assemble with transpose = 1);
 *   dcontrol     dJ/dcontrol + adjoint . dR/dcontrol
 *                (ComputeAdjointNodalControlDerivatives, :486-526);
 *   dxyz         [3 N] dJ/dx + adjoint . dR/dx
 *                (ComputeAdjointNodalShapeDerivatives, :365-406).
 * dcontrol and dxyz need the adjoint dofs (the AdjointFiniteElementSolver
 * solution).  dofs and adjoint are used as given (no Dirichlet overwrite).
 * Neo-Hookean plans return FOLGB_ERR_INVALID_ARGUMENT. */
typedef struct {
  double coeff;
  int32_t control_power;
  int32_t dof_power[3];
} folgb_monomial;
enum { FOLGB_MAX_MONOMIALS = 16 };
size_t folgb_response_workspace_bytes(const folgb_plan* plan);
int folgb_response(const folgb_plan* plan, int32_t num_monomials, const folgb_monomial* monomials,
                   const float* control, const float* dofs, const float* adjoint, float* value,
                   float* adjoint_rhs, float* dcontrol, float* dxyz, void* workspace,
                   size_t workspace_bytes, void* stream);

/* ---- nodal Fourier control ----------------------------------------------
 * FourierControl (fol/controls/fourier_control.py:14-59) on the device: the
 * map from Fourier coefficients to the nodal material field that precedes the
 * loss in a FOL training step, and its vector-Jacobian product.  Replaces
 * FourierControl.ComputeControlledVariables (:49-59) and the jax.grad of the
 * loss with respect to the coefficients through it.
 * Coefficients: [batch][1 + nx*ny*nz], the constant term first, then
 * meshgrid(x_freqs, y_freqs, z_freqs, indexing="ij") flattened row-major
 * (:44-45); scaled as coeffs * (scale_max - scale_min) + scale_min (:51-52).
 * xyz: node coordinates (HOST, num_nodes x 3, doubles). */
typedef struct folgb_fourier folgb_fourier;
int folgb_fourier_create(folgb_fourier** control, const double* x_freqs, int32_t nx,
                         const double* y_freqs, int32_t ny, const double* z_freqs, int32_t nz,
                         const double* xyz, int64_t num_nodes, double min_value, double max_value,
                         double beta, double scale_min, double scale_max);
int folgb_fourier_destroy(folgb_fourier* control);
/* values[b][n] = (max - min) * sigmoid(beta * (K_b(x_n) - 0.5)) + min. */
int folgb_fourier_forward(const folgb_fourier* control, int32_t batch, const float* coeffs,
                          float* values, void* stream);
size_t folgb_fourier_workspace_bytes(const folgb_fourier* control, int32_t batch);
/* dcoeffs[b][q] = sum_n dvalues[b][n] * d values[b][n] / d coeffs[b][q]
 * (deterministic: per-block partials summed in a fixed order). */
int folgb_fourier_backward(const folgb_fourier* control, int32_t batch, const float* coeffs,
                           const float* dvalues, float* dcoeffs, void* workspace,
                           size_t workspace_bytes, void* stream);

/* ---- opt-in kernel tracing ------------------------------------------------
 * CUDA events recorded on the launching stream around every kernel of the
 * entry points above, summed per kernel id.  The reference's only tracing is
 * wall-clock decorators (fol/tools/decoration_functions.py:7-32), which time
 * dispatch, not the device; this has no other counterpart there.
 * folgb_trace_read synchronises on the recorded events. */
enum {
  FOLGB_KERNEL_ELEM_LOSS = 0, FOLGB_KERNEL_GATHER = 1, FOLGB_KERNEL_ELEM_MATRIX = 2,
  FOLGB_KERNEL_PAIR_REDUCE = 3, FOLGB_KERNEL_PLAIN_BACKWARD = 4, FOLGB_KERNEL_ELEM_RESIDUAL = 5,
  FOLGB_KERNEL_PCG_SPMV = 6, FOLGB_KERNEL_PCG_UPDATE = 7, FOLGB_KERNEL_BATCH_LOSS = 8,
  FOLGB_KERNEL_HEX8_FUSED = 9
};
/* Self-test of the bounded device-side wait (no counterpart in the
 * reference): launches one block that waits on a shared-memory mbarrier whose
 * announced copy never comes; the wait gives up after its poll limit (well
 * under a second) and ORs 1 << FOLGB_ERR_TIMEOUT into device_status (device
 * int).  Shows that a lost copy cannot hang a kernel. */
int folgb_selftest_bounded_wait(int32_t* device_status, void* stream);

/* FP32 throughput probe (no counterpart in the reference): launches
 * blocks_per_sm x (SM count) blocks of 256 threads, each thread running
 * `iterations` x 8 packed-pair fused multiply-adds (independent chains), on
 * `stream`; *flops_per_launch gets the flop count (2 per FMA).  Time it with
 * events on the stream to measure the GPU's FP32 peak.  sink: any device
 * float (never written in practice). */
int folgb_fp32_peak_probe(float* sink, int32_t blocks_per_sm, int32_t iterations, double* flops_per_launch,
                          void* stream);

int folgb_trace_enable(int32_t on);
int folgb_trace_reset(void);
int folgb_trace_read(int32_t kernel_id, int64_t* launches, double* total_ms);

#ifdef __cplusplus
}
#endif
#endif /* FOLGB_H */
