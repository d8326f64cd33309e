/*
 * nsfv1_gb300.h -- C ABI of the GB300-native FV1 incompressible Navier-Stokes
 * assembly and Newton path (drop-in for the NavierStokesFV1 element disc of
 * UG4 plugin_NavierStokes).
 *
 * Conventions
 *  - Every function returns an int status (NSFV1_OK on success); the text of
 *    the last error of a handle is returned by nsfv1_last_error(). No C++
 *    exception crosses this boundary (the reference throws UG_THROW).
 *  - Pointers documented as "device" are CUDA device pointers owned by the
 *    caller; "host" pointers are read during the call only. Streams are
 *    cudaStream_t passed as void* (NULL = legacy default stream).
 *  - One handle = one element disc; calls on one handle are not re-entrant
 *    (the reference's disc is not re-entrant either, navier_stokes_fv1.cpp:259).
 *  - Element-local layouts (the reference's LocalVector / LocalMatrix,
 *    navier_stokes_fv1.h:128-140, fct-major):
 *      local vector  u[fct * nsh + sh]
 *      local matrix  J[((f1 * nsh + s1) * b + f2) * nsh + s2]
 *    Global layouts: vector U[node * b + fct]; matrix block CSR with b x b
 *    row-major blocks, rows sorted by column, b = dim + 1.
 *  - Element type ids are ugcore ReferenceObjectID values.
 */
#ifndef NSFV1_GB300_H
#define NSFV1_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define NSFV1_OK                0
#define NSFV1_ERR_ARGUMENT      1   /* bad argument or unknown name (reference: UG_THROW)      */
#define NSFV1_ERR_STATE         2   /* missing setup (e.g. no stabilisation, no mesh)           */
#define NSFV1_ERR_CUDA          3   /* CUDA runtime error                                       */
#define NSFV1_ERR_NOT_CONVERGED 4   /* Newton reached max iterations                            */
#define NSFV1_ERR_BREAKDOWN     5   /* Krylov breakdown (rho = 0, omega = 0, singular block)    */
#define NSFV1_ERR_NONFINITE     6   /* NaN / Inf in a defect or update                          */
#define NSFV1_ERR_GEOMETRY      7   /* upwind ray found no element side (reference: UG_THROW)   */
#define NSFV1_ERR_TIMEOUT       8   /* a bounded device wait ran out                            */

/* element types (ugcore ReferenceObjectID) */
#define NSFV1_TRIANGLE       2
#define NSFV1_QUADRILATERAL  3
#define NSFV1_TETRAHEDRON    4
#define NSFV1_PRISM          6
#define NSFV1_HEXAHEDRON     8

/* Jacobian value precision */
#define NSFV1_F64 0
#define NSFV1_F32 1

/* linear solvers of the Newton loop */
#define NSFV1_BICGSTAB 0
#define NSFV1_GMRES    1

typedef struct nsfv1_disc nsfv1_disc;

/* ---- element disc: construction and parameters ------------------------- */

/* NavierStokesFV1(fcts, subsets) + init(): dim+1 P1 functions, density 1
 * (navier_stokes_fv1.cpp:45-87); dim is 2 or 3. */
int nsfv1_create(int dim, nsfv1_disc** out);
int nsfv1_destroy(nsfv1_disc* h);
/* text of the last error on this handle (never NULL) */
const char* nsfv1_last_error(const nsfv1_disc* h);
/* disc_type() == "fv1" (navier_stokes_fv1.h:241) */
const char* nsfv1_disc_type(const nsfv1_disc* h);

/* NavierStokesBase::set_kinematic_viscosity(number) (navier_stokes_base.cpp:72-77) */
int nsfv1_set_kinematic_viscosity(nsfv1_disc* h, double nu);
/* IncompressibleNavierStokesBase::set_density(number) (incompressible_navier_stokes_base.cpp:93-98) */
int nsfv1_set_density(nsfv1_disc* h, double rho);
/* NavierStokesBase::set_source(std::vector<number>) (navier_stokes_base.cpp:91-97); n == dim */
int nsfv1_set_source(nsfv1_disc* h, const double* f, int n);
/* NavierStokesBase::set_exact_jacobian(number) (navier_stokes_base.h:194-196); 0 = fixpoint */
int nsfv1_set_exact_jacobian(nsfv1_disc* h, double factor);
/* set_stokes / set_laplace / set_peclet_blend (incompressible_navier_stokes_base.h:206-225) */
int nsfv1_set_stokes(nsfv1_disc* h, int on);
int nsfv1_set_laplace(nsfv1_disc* h, int on);
int nsfv1_set_peclet_blend(nsfv1_disc* h, int on);
/* NavierStokesFV1::set_upwind(const std::string&) (navier_stokes_fv1.h:213-215,
 * ids of CreateNavierStokesUpwind, upwind_interface.cpp:43-62): "no", "full",
 * "skewed", "lps" / "linearprofileskewed", "pos" / "positive" (case-insensitive,
 * trimmed). The object is shared with a stabilisation that has no upwind yet.
 * The positive upwind (upwind.cpp:643-786) has shapes at the other integration
 * points of an element, which selects the non-diagonal FIELDS / FLOW branches
 * (stabilization.cpp:244-403, 589-771); its element path needs a device
 * workspace of 12 KB per thread for hexahedra at 64 threads per SM (120 MB on
 * 152 SMs), allocated with the mesh or at the first device use after this call. A singular ip-ip system of
 * that branch gives NSFV1_ERR_BREAKDOWN ("Could not compute inverse."). The
 * regular upwind ("reg") is not provided. */
int nsfv1_set_upwind(nsfv1_disc* h, const char* name);
/* NavierStokesFV1::set_stabilization(name[, diffLength]) (navier_stokes_fv1.h:190-199,
 * CreateNavierStokesStabilization stabilization.cpp:46-57, set_diffusion_length
 * stabilization.cpp:86-100): "fields", "flow" (+ "without" for
 * NavierStokesFV1WithoutStabilization); diff_length "raw" (NULL), "fivepoint", "cor". */
int nsfv1_set_stabilization(nsfv1_disc* h, const char* name, const char* diff_length);
/* NavierStokesFV1::set_pac_upwind(bool) (navier_stokes_fv1.h:217-225): with on != 0
 * the stabilisation takes the convection's upwind object and its stabilised
 * velocity becomes the convective upwind velocity (PAC), in the defect and in
 * the Jacobian (navier_stokes_fv1.cpp:382-384, 398-427, 477-518); needs an
 * upwind and a stabilisation set before (NSFV1_ERR_STATE with the reference's
 * texts otherwise). on == 0 changes nothing, as in the reference; a later
 * nsfv1_set_upwind ends PAC. (The reference's convection keeps its old
 * stabilisation object if set_stabilization follows; here PAC uses the current
 * stabilisation.) */
int nsfv1_set_pac_upwind(nsfv1_disc* h, int on);
/* INavierStokesFV1Stabilization::set_upwind with an upwind object of its own
 * (stabilization.h:91-95, registered at register_fv1.cpp:246-249); ids as for
 * nsfv1_set_upwind. */
int nsfv1_set_stabilization_upwind(nsfv1_disc* h, const char* name);

/* ---- mesh, sparsity pattern, colouring ---------------------------------- */

/* Sets the element mesh (one element type; host arrays): coords[n_nodes*dim],
 * conn[n_elems*nsh] (ugcore corner order). Builds the block-CSR pattern (all
 * node pairs sharing an element; the sparsity of the reference's assembled
 * matrix) and a greedy element colouring, and uploads them.
 * Replaces prepare_setting / prep_elem_loop (navier_stokes_fv1.cpp:89-199)
 * plus ugcore's DoF distribution and matrix-pattern setup. */
int nsfv1_set_mesh(nsfv1_disc* h, int elem_type, int64_t n_nodes, const double* coords, int64_t n_elems, const int32_t* conn);
int nsfv1_pattern_info(const nsfv1_disc* h, int64_t* n_rows, int64_t* nnz_blocks, int* block_size, int* n_colors);
/* Host-only form of the same pattern / colouring build (no handle, no GPU):
 * call with row_ptr == NULL to get *nnz_blocks and *n_colors, then again with
 * row_ptr[n_nodes+1], col_idx[nnz_blocks], elem_color[n_elems] (each may be NULL). */
int nsfv1_mesh_pattern(int elem_type, int64_t n_nodes, int64_t n_elems, const int32_t* conn, int64_t* nnz_blocks,
                       int* n_colors, int32_t* row_ptr, int32_t* col_idx, int32_t* elem_color);
/* host copies of the pattern (row_ptr[n_rows+1], col_idx[nnz_blocks]) and colouring */
int nsfv1_get_pattern(const nsfv1_disc* h, int32_t* row_ptr, int32_t* col_idx);
int nsfv1_get_coloring(const nsfv1_disc* h, int32_t* elem_color);
/* device pointers of the pattern, owned by the handle (valid until the next set_mesh/destroy) */
int nsfv1_device_pattern(const nsfv1_disc* h, const int32_t** row_ptr, const int32_t** col_idx);
/* Dirichlet rows (host arrays): dofs[k] = node * b + fct, value g_k.
 * Defect row = u - g, Jacobian row = identity (the reference's core
 * DirichletBoundary semantics, bnd/wall_impl.h:57-69). */
int nsfv1_set_dirichlet(nsfv1_disc* h, int64_t n, const int32_t* dofs, const double* values);

/* ---- boundary-condition element discs (host arrays) ---------------------- */

/* ugcore's DirichletBoundary::add, for single unknowns: appends Dirichlet rows
 * (dofs[k] = node * b + fct, value g_k) to the handle's, a later value of the same
 * unknown replacing an earlier one (nsfv1_set_dirichlet replaces them all). */
int nsfv1_add_dirichlet(nsfv1_disc* h, int64_t n, const int32_t* dofs, const double* values);

/* NavierStokesWall::add(subsets) (incompressible/bnd/wall_impl.h:57-69): every
 * velocity component of the given nodes is a Dirichlet row with value 0.
 * Rows accumulate with earlier nsfv1_add_wall / nsfv1_add_inflow calls (a later
 * value of the same unknown wins); nsfv1_set_dirichlet replaces them all. */
int nsfv1_add_wall(nsfv1_disc* h, int64_t n_nodes, const int32_t* nodes);
/* NavierStokesInflowFV1::add(velocity, subsets) (incompressible/fv1/bnd/
 * inflow_fv1_impl.h:57-82) for a constant inflow velocity vel[dim] on the given
 * boundary sides (n_sides x side_nco node ids; 2D: edges of 2 nodes, 3D:
 * triangles of 3 or quadrilaterals of 4 nodes, in the element's side order):
 *  - Dirichlet rows velocity = vel at every node of the sides (the reference's
 *    DirichletBoundary on the velocity functions);
 *  - the Neumann flux of the continuity equation (the reference's
 *    NeumannBoundaryFV1 on the pressure function with the same vector data):
 *    the continuity defect of each side corner gets + vel . n_bf, n_bf the
 *    outward, area-weighted normal of that corner's part of the side in the
 *    FV1 dual mesh ({corner, edge midpoints, side centre}); scaled by dt in
 *    the implicit-Euler defect, like every right-hand side.
 * A side must belong to exactly one element (NSFV1_ERR_ARGUMENT otherwise). */
int nsfv1_add_inflow(nsfv1_disc* h, int64_t n_sides, int side_nco, const int32_t* side_nodes, const double* vel);
/* NavierStokesNoNormalStressOutflowFV1::add(subsets) (incompressible/fv1/bnd/
 * no_normal_stress_outflow_fv1.cpp:343-504) on the given boundary sides (as for
 * nsfv1_add_inflow): every corner's part of a side (the FV1 boundary face, with
 * its outward area-weighted normal n and the P1 shapes and gradients at its
 * integration point) adds to the corner's rows
 *  - momentum: the viscous flux -nu rho ((grad u + grad u^T) n) without its
 *    component along n (v - (v.n) n with the area-weighted n, as the reference
 *    computes it), and the outgoing convective flux max(rho u.n, 0) u (not with
 *    the Stokes option);
 *  - continuity: rho u.n;
 * and the Jacobian: the viscous and continuity terms exactly, the convective one
 * with the flux frozen, as the reference's add_jac_A_elem does. Part of every
 * defect / Jacobian assembly (dt-scaled when transient) until
 * nsfv1_clear_boundary. Sides accumulate over calls. */
int nsfv1_add_outflow(nsfv1_disc* h, int64_t n_sides, int side_nco, const int32_t* side_nodes);
/* removes every Dirichlet row and inflow flux */
int nsfv1_clear_boundary(nsfv1_disc* h);

/* ---- assembly (device pointers) ----------------------------------------- */

/* Global defect d = A(u) - F (stationary, u_old == NULL) or
 * d = M(u) - M(u_old) + dt (A(u) - F) (implicit Euler), FP64, with Dirichlet rows.
 * Replaces the element loop over prep_elem + add_def_A_elem + add_def_M_elem +
 * add_rhs_elem (navier_stokes_fv1.cpp:208-248, 597-869) and the scatter. */
int nsfv1_assemble_defect(nsfv1_disc* h, const double* u, const double* u_old, double dt, double* d, void* stream);
/* Global Jacobian values J = dA/du (or M + dt dA/du) in the handle's block CSR,
 * vals[nnz_blocks * b * b] of double (NSFV1_F64) or float (NSFV1_F32; for 3D
 * meshes 16-byte aligned: each 4-float block row is one vector reduction).
 * Replaces the element loop over add_jac_A_elem + add_jac_M_elem
 * (navier_stokes_fv1.cpp:250-595, 781-808) and the matrix insertion. */
int nsfv1_assemble_jacobian(nsfv1_disc* h, const double* u, const double* u_old, double dt, void* vals, int prec, void* stream);
/* Defect and Jacobian at the same state (both outputs of the two calls above) in
 * one pass over the elements: the per-SCVF geometry, upwind shapes and
 * stabilisation feed both, where the reference evaluates them in each of
 * add_def_A_elem and add_jac_A_elem (navier_stokes_fv1.cpp:296-309, 645-659).
 * NSFV1_F64: the same results as nsfv1_assemble_defect + nsfv1_assemble_jacobian.
 * NSFV1_F32: the FP64 defect and the FP32 Jacobian of nsfv1_assemble_jacobian,
 * colour by colour (vals 16-byte aligned for 3D meshes); the same results as the
 * two calls. */
int nsfv1_assemble_defect_jacobian(nsfv1_disc* h, const double* u, const double* u_old, double dt, double* d, void* vals, int prec,
                                   void* stream);
/* The reference's per-element callbacks, batched over n independent elements
 * (device arrays): corners[n][nsh][dim], u/u_old[n][b*nsh] (local layout);
 * outputs (each may be NULL) defA, defM, rhs [n][b*nsh] and jacA, jacM
 * [n][(b*nsh)^2]: add_def_A_elem, add_def_M_elem, add_rhs_elem, add_jac_A_elem,
 * add_jac_M_elem (navier_stokes_fv1.cpp:250-869), each output zeroed first. */
int nsfv1_elem_batch(nsfv1_disc* h, int elem_type, int64_t n, const double* corners, const double* u, const double* u_old,
                     double dt, double* defA, double* jacA, double* defM, double* jacM, double* rhs, void* stream);

/* ---- data exports ---------------------------------------------------------
 * NavierStokesFV1's data exports (navier_stokes_fv1.cpp:894-1491, registered per
 * element type at :1573-1577): ex_nodal_velocity, ex_velocity_grad,
 * ex_velocity_ip (the stabilised velocity), ex_nodal_pressure, ex_pressure_grad,
 * for n elements at once (device arrays; layouts as nsfv1_elem_batch):
 *   points  ip_kind NSFV1_IPS_SCVF: the SCVF integration points (the exports'
 *           FV1 branch, nip = number of SCVFs); NSFV1_IPS_SCV: the SCV ips = the
 *           corners (nip = corners); NSFV1_IPS_GIVEN: nip (1..64) local points
 *           local_ips[nip][dim] (a HOST array), the exports' general branch;
 *   values  [n][nip][vs], vs = dim, dim*dim (row d1: d u_d1 / d x_d2), dim, 1, dim;
 *   derivs  [n][nip][dim+1][corners][vs] (may be NULL): the derivative of each
 *           value w.r.t. the element's unknowns (function, corner), as the
 *           reference fills its vvvDeriv: entries it leaves alone are zero, and
 *           where it assigns a scalar to a vector entry every component holds it.
 * Both outputs are overwritten (the reference adds the nodal velocity into the
 * caller's array). As in the reference, the velocity gradient's general branch
 * is taken in local (reference-element) coordinates, while the pressure
 * gradient's is mapped with J^-T at the point. The call waits for its stream. */
#define NSFV1_EX_VELOCITY       0
#define NSFV1_EX_VELOCITY_GRAD  1
#define NSFV1_EX_VELOCITY_IP    2
#define NSFV1_EX_PRESSURE       3
#define NSFV1_EX_PRESSURE_GRAD  4
#define NSFV1_IPS_SCVF          0
#define NSFV1_IPS_SCV           1
#define NSFV1_IPS_GIVEN         2
int nsfv1_export(nsfv1_disc* h, int which, int elem_type, int64_t n, const double* corners, const double* u, const double* u_old, double dt,
                 int ip_kind, int nip, const double* local_ips, double* values, double* derivs, void* stream);

/* ---- post-processing (incompressible/navier_stokes_tools.h) ----------------
 * vorticityFV1 (:387-525): vort[n_nodes] = sum over the node's SCVs of |SCV| times
 * the curl d u_y/dx - d u_x/dy of the P1 velocity at the corner, divided by the
 * summed |SCV| (the first two velocity components, also in 3D, as the reference's
 * formula takes them); u[n_nodes * b] on the device. Deterministic (element
 * colours in order). The call waits for its stream. */
int nsfv1_vorticity(nsfv1_disc* h, const double* u, double* vort, void* stream);
/* The value of function fct (0..dim; dim = pressure) of the P1 solution u at n
 * global points points[n][dim] (device arrays): the first element in mesh order
 * containing the point, interpolated with the P1 shapes there; NaN outside the
 * mesh. The point evaluation of DrivenCavityEvalAtPoints / DrivenCavityLinesEval
 * (:540-729). The call waits for its stream. */
int nsfv1_eval_points(nsfv1_disc* h, const double* u, int64_t n, const double* points, int fct, double* values, void* stream);

/* The same callbacks with HOST arrays (same layouts): the library stages them
 * through device memory it allocates for the call and returns when the outputs
 * are on the host. For host-side element loops such as a ugcore IElemDisc
 * adapter (navier_stokes_fv1.cpp:1553-1579 registers the reference's). */
int nsfv1_elem_batch_host(nsfv1_disc* h, int elem_type, int64_t n, const double* corners, const double* u, const double* u_old,
                          double dt, double* defA, double* jacA, double* defM, double* jacM, double* rhs);


/* ---- linear algebra on the handle's pattern (device pointers) ------------ */

/* y = J x with J in the handle's block CSR (prec as above; x, y FP64) */
int nsfv1_bsr_mv(nsfv1_disc* h, const void* vals, int prec, const double* x, double* y, void* stream);

/* The FP64 vector x[n] as float pairs xs[2n] (xs[2i] the leading 24 bits of
 * x[i], xs[2i+1] the next 24; device arrays), the operand of
 * nsfv1_bsr_mv_split. */
int nsfv1_split_vector(int64_t n, const double* x, float* xs, void* stream);
/* y = J x for FP32 values and x given split by nsfv1_split_vector (xs 8-byte
 * aligned): the result of nsfv1_bsr_mv with NSFV1_F32, bit for bit, without
 * splitting x once per matrix block (the form the Newton loop's BiCGStab
 * applies: its update kernels write the split of every vector they produce). */
int nsfv1_bsr_mv_split(nsfv1_disc* h, const float* vals, const float* xs, double* y, void* stream);

/* Point-block Jacobi preconditioner of a Jacobian on the handle's pattern
 * (the preconditioner of the Newton loop's linear solves): inverts every
 * b x b diagonal block of vals (prec NSFV1_F64 / NSFV1_F32) in FP64 into
 * scratch owned by the handle (allocated on first use, nNodes*b*b doubles)
 * and returns z = D^-1 r (device vectors). NSFV1_ERR_BREAKDOWN on a singular
 * block. Replaces the core's block-Jacobi preconditioner step of the
 * reference's linear solver. */
int nsfv1_block_jacobi(nsfv1_disc* h, const void* vals, int prec, const double* r, double* z, void* stream);

/* Largest mesh (nodes) that nsfv1_block_jacobi_noalloc accepts. */
#define NSFV1_NOALLOC_MAX_NODES 32768

/* The same preconditioner as nsfv1_block_jacobi, allocating nothing: for
 * callers whose device memory is all handed out by their own pool allocator,
 * so that a cudaMalloc from inside a library would fail or fragment that pool.
 * No counterpart in the reference (its CPU preconditioner allocates freely).
 * The scratch is a fixed 4 MiB device array inside the library, shared by all
 * calls; meshes above NSFV1_NOALLOC_MAX_NODES nodes are rejected with
 * NSFV1_ERR_ARGUMENT. The first call on a device looks the array up with
 * cudaGetSymbolAddress and should come before any stream capture. Like
 * nsfv1_block_jacobi, every call waits for its stream to finish: it reads the
 * singular-block flag back to the host (NSFV1_ERR_BREAKDOWN). Calls that
 * overlap on the GPU race on the shared array and must be serialised. */
int nsfv1_block_jacobi_noalloc(nsfv1_disc* h, const void* vals, int prec, const double* r, double* z, void* stream);

/* ---- Newton solve (the plain method and the FP32-Jacobian mode) ---------- */

typedef struct {
    double rtol;            /* relative defect reduction (e.g. 1e-8)                      */
    double atol;            /* absolute defect floor (0 to disable)                       */
    int max_iter;           /* Newton iterations                                          */
    double lin_rtol;        /* relative residual reduction of the linear solve            */
    int lin_max_iter;       /* linear iterations per Newton step                          */
    int line_search_steps;  /* backtracking halvings (0 = full steps)                     */
    int jacobian_prec;      /* NSFV1_F64 (plain method) or NSFV1_F32: Jacobian and its    */
                            /* block inverses stored in FP32, Krylov vectors FP64         */
    int linear_solver;      /* NSFV1_BICGSTAB or NSFV1_GMRES                              */
    int gmres_restart;      /* GMRES restart length (<= 64)                               */
} nsfv1_newton_params;

typedef struct {
    int iterations;
    int linear_iterations;
    double initial_defect;  /* ||d(u0)||_2 */
    double final_defect;    /* ||d(u)||_2  */
    int status;             /* NSFV1_OK, NSFV1_ERR_NOT_CONVERGED, ...                      */
} nsfv1_newton_result;

/* Newton from the given device vector u (overwritten with the solution): the
 * Dirichlet values are set into u, then d = defect(u); loop { J(u) du = d
 * (point-block-Jacobi preconditioned BiCGStab / GMRES in the Jacobian's
 * precision); u -= lambda du with backtracking on ||d||_2 } until
 * ||d|| <= rtol ||d0|| (ugcore's Newton, restated). Defect, norms, update and
 * line search are FP64. u_old/dt as in nsfv1_assemble_defect. */
int nsfv1_newton_solve(nsfv1_disc* h, double* u, const double* u_old, double dt, const nsfv1_newton_params* p,
                       nsfv1_newton_result* r, void* stream);

/* The Newton loop's linear solver on a given system (the core's linear solver
 * applied to an assembled Jacobian): J x = rhs on the handle's pattern, J =
 * vals of precision p->jacobian_prec, rhs and x FP64 device vectors, x = 0
 * start; point-block-Jacobi right-preconditioned BiCGStab or GMRES(m)
 * (p->linear_solver, p->gmres_restart) to p->lin_rtol relative residual in at
 * most p->lin_max_iter iterations. Out (host, each may be NULL): iterations,
 * the final relative residual and the BiCGStab restarts (a zero (r0, v) or
 * rho, a zero omega or a non-finite coefficient makes the current residual the
 * new shadow vector; after 20 restarts the solve stops with the last iterate).
 * NSFV1_ERR_BREAKDOWN: a singular diagonal block or a non-finite residual;
 * NSFV1_ERR_NOT_CONVERGED: the tolerance was not reached. */
int nsfv1_linear_solve(nsfv1_disc* h, const void* vals, const double* rhs, double* x, const nsfv1_newton_params* p, int* iterations,
                       double* relres, int* restarts, void* stream);

/* ---- many independent instances (batched cavities) ------------------------ */

/* Per-element kinematic viscosity (host array [n_elems]), replacing the
 * constant of nsfv1_set_kinematic_viscosity; NULL returns to the constant.
 * (The reference takes any CplUserData viscosity, navier_stokes_fv1.cpp:109-114.) */
int nsfv1_set_elem_viscosity(nsfv1_disc* h, const double* nu);
/* Declares the mesh as n_inst independent instances: node ranges
 * [node_offsets[i], node_offsets[i+1]) (host array [n_inst+1], from 0 to
 * n_nodes); no element may span two instances. */
int nsfv1_set_instances(nsfv1_disc* h, int n_inst, const int32_t* node_offsets);

/* Declares every instance a structured square grid of cells[i] x cells[i]
 * quadrilaterals (lexicographic nodes, ugcore corner order) and builds the
 * geometric multigrid hierarchy used as the GMRES preconditioner of
 * nsfv1_newton_solve_batched: vertex-nested coarse levels down to 4 cells per
 * side (rediscretised Jacobians at the injected state, bilinear prolongation,
 * restriction = its transpose, damped point-block Jacobi smoothing). */
int nsfv1_set_instance_grids(nsfv1_disc* h, const int32_t* cells);

typedef struct {
    int cluster_size;    /* CTAs per thread-block cluster working on one instance (1..16; 0 = 4)   */
    int max_clusters;    /* upper bound on concurrently resident clusters (0 = as many as fit)     */
    int mg_levels;       /* 0: point-block Jacobi only; otherwise the multigrid V-cycle (if built)  */
    int smooth_steps;    /* V-cycle pre/post smoothing sweeps (0 = 2)                               */
    int coarse_steps;    /* sweeps on the coarsest level (0 = 20)                                   */
    double smooth_omega; /* damping of the smoother (0 = 0.7)                                       */
    int defect_reference;/* 0: rtol relative to each instance's initial iterate; 1: relative to the   */
                         /*    defect of the zero iterate (Dirichlet values, 0 elsewhere)             */
    int zero_fallback;   /* with defect_reference 1: an instance whose initial defect exceeds the     */
                         /*    zero iterate's restarts from the zero iterate                          */
    double forcing_max;  /* > 0: Eisenstat-Walker linear tolerance per instance and step, within     */
                         /*    [p->lin_rtol, forcing_max]; 0: p->lin_rtol throughout                   */
    int graph;           /* 1: each step's fixed device work (Jacobians on all levels, block         */
                         /*    inverses, the GMRES launch) replays one captured CUDA graph            */
    int tail_clusters;   /* 1: while active instances x cluster_size leave SMs idle, the step uses    */
                         /*    clusters of 2x, 4x ... (at most 16 CTAs) for the remaining instances   */
} nsfv1_batch_options;

/* Newton on every instance at once (each to its own ||d_i|| <= rtol ||d_i,0||):
 * one assembly pass over all unconverged instances per step, then ONE
 * persistent launch of a cluster-per-instance restarted GMRES (right
 * point-block Jacobi, restart p->gmres_restart <= 32) over the unconverged
 * instances, then a per-instance backtracking line search. results[n_inst]
 * receives each instance's iterations, linear iterations, defects and status. */
int nsfv1_newton_solve_batched(nsfv1_disc* h, double* u, const double* u_old, double dt, const nsfv1_newton_params* p,
                               const nsfv1_batch_options* opt, nsfv1_newton_result* results, void* stream);

/* ---- learned warm start: coordinate MLP on the tensor cores --------------- *
 * (no reference counterpart: the reference starts Newton from the caller's
 * iterate). Features [sin, cos](pi k x), [sin, cos](pi k y), k = 1..16; four
 * FiLM-conditioned SiLU layers of width 256; head 256 -> 3 predicting
 * (u/lid, v/lid, p/lid^2). BF16 GEMM operands, FP32 accumulation (tcgen05),
 * FP32 master weights and Adam. Points come in contiguous slots (one
 * conditioning each): slot_ptr[n_slots+1] on the host, from 0 to n_points. */
typedef struct nsfv1_mlp nsfv1_mlp;
typedef struct {
    int max_points;      /* point capacity of one forward / training batch */
    int max_slots;       /* slots (instances) per batch */
} nsfv1_mlp_config;
typedef struct {
    int64_t n_train;     /* training instances, all on one mesh */
    int64_t n_nodes;     /* nodes of that mesh */
    const float* coords; /* device [n_nodes x 2] */
    const float* targets;/* device [n_train x n_nodes x 3], normalised (nsfv1_mlp_targets) */
    const float* cond;   /* device [n_train x 2], nsfv1_mlp_condition of each instance */
} nsfv1_mlp_dataset;
typedef struct {
    int steps;           /* Adam steps */
    int slots;           /* instances per minibatch */
    int points_per_slot; /* nodes drawn per instance */
    float lr, lr_final;  /* cosine schedule from lr to lr_final */
    uint64_t seed;
    int64_t step_offset; /* first step index of the sampler (to continue a run) */
} nsfv1_mlp_train_params;

int nsfv1_mlp_create(const nsfv1_mlp_config* cfg, nsfv1_mlp** out);
void nsfv1_mlp_destroy(nsfv1_mlp* m);
const char* nsfv1_mlp_last_error(const nsfv1_mlp* m);
int64_t nsfv1_mlp_num_params(const nsfv1_mlp* m);
/* conditioning of one cavity: c = ((ln Re - ln 100) / ln 10, (lid - 1.25) / 0.75) */
void nsfv1_mlp_condition(double re, double lid, float* c2);
int nsfv1_mlp_init(nsfv1_mlp* m, uint64_t seed);
int nsfv1_mlp_get_params(nsfv1_mlp* m, float* host, int64_t n);
int nsfv1_mlp_set_params(nsfv1_mlp* m, const float* host, int64_t n);
/* out[n x 3] (device) = network output at xy[n x 2] (device); cond host [n_slots x 2] */
int nsfv1_mlp_forward(nsfv1_mlp* m, int64_t n_points, const float* xy, int n_slots, const int32_t* slot_ptr, const float* cond,
                      float* out, void* stream);
/* loss (host) and the gradient of every parameter (device [num_params]) against target[n x 3] (device) */
int nsfv1_mlp_loss_grad(nsfv1_mlp* m, int64_t n_points, const float* xy, int n_slots, const int32_t* slot_ptr, const float* cond,
                        const float* target, double* loss, float* grad, void* stream);
/* Adam training on minibatches drawn on the device; loss_history[steps] (host) may be NULL */
int nsfv1_mlp_train(nsfv1_mlp* m, const nsfv1_mlp_dataset* data, const nsfv1_mlp_train_params* tp, float* loss_history, void* stream);
/* normalised targets of n_instances solutions on one mesh: u device [n_instances x n_nodes x 3] (FP64), lid device [n_instances] */
int nsfv1_mlp_targets(int64_t n_instances, int64_t n_nodes, const double* u, const double* lid, float* targets, void* stream);
/* Newton initial iterate: u[n x 3] (device, FP64) = (lid out_0, lid out_1, lid^2 out_2); cond, lid host per slot */
int nsfv1_mlp_predict(nsfv1_mlp* m, int64_t n_points, const float* xy, int n_slots, const int32_t* slot_ptr, const float* cond,
                      const float* lid, double* u, void* stream);
/* the tensor-core GEMM itself: C[splits][M][N] (FP32) = A[M x K] * B[N x K]^T over K
 * chunks (BF16 row-major operands; M % 128 == 0, K % 64 == 0, N = 64, 128 or a multiple of 256) */
int nsfv1_gemm_bf16(int M, int N, int K, const void* A, const void* B, float* C, int splits, void* stream);
/* the number of K chunks nsfv1_gemm_bf16 uses for K and a requested split count */
int nsfv1_gemm_bf16_splits(int K, int splits);

/* CTA size of the assembly colour launches (32, 64, 96 or 128; default 32):
 * the element kernels use up to 255 registers per thread, so small CTAs
 * spread each colour evenly over the SMs. (No reference counterpart.) */
int nsfv1_set_assembly_threads(nsfv1_disc* h, int threads);
int nsfv1_get_assembly_threads(const nsfv1_disc* h);
/* Assembly autotuner: times one defect + Jacobian assembly at u (device) for
 * every candidate CTA size, in precision prec (nsfv1_assemble_defect_jacobian),
 * and keeps the fastest;
 * ms[n_candidates] (host, may be NULL) receives the second pass's times. */
int nsfv1_assembly_autotune(nsfv1_disc* h, const double* u, int prec, const int* candidates, int n_candidates, double* ms, void* stream);

/* Timing of the last batched solve: out[0] Newton steps, out[1] device ms of the
 * steps' fixed work (Jacobians, block inverses, GMRES), out[2] device ms of the
 * line searches, out[3] wall ms of the whole call; further entries 0. */
int nsfv1_batch_stats(const nsfv1_disc* h, double* out, int n);

/* Autotuner of the batched solve: times one Newton step from u (u is not
 * changed) for every candidate cluster size (CTAs per instance) and writes the
 * fastest into opt->cluster_size; ms[n_candidates] (host, may be NULL)
 * receives each candidate's time of the second of two passes. */
int nsfv1_batch_autotune(nsfv1_disc* h, const double* u, const double* u_old, double dt, const nsfv1_newton_params* p,
                         nsfv1_batch_options* opt, const int* candidates, int n_candidates, double* ms, void* stream);

/* reference-element tables used by the kernels (for the table-consistency test):
 * edges[2*nedge], sides[4*nside] (unused slots -1), side_nco[nside], edge_face[2*nedge] */
int nsfv1_ref_tables(int elem_type, int* nco, int* nedge, int* edges, int* nside, int* side_nco, int* sides, int* edge_face);

#ifdef __cplusplus
}
#endif

#endif /* NSFV1_GB300_H */
