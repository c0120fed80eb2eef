/*
 * llfem_gb300.h — C-ABI of the GB300 operator-assembly + iterative-solve library.
 *
 * This is the drop-in boundary behind LowLevelFEM.jl's own Julia API for its
 * assembly/solve hot path.  Every entry point is `extern "C"`, takes plain
 * pointers and sizes, returns an int status (LLF_OK == 0, negative on error)
 * and leaves a message readable through llf_last_error().  No entry point
 * throws, aborts, or falls back to host computation: when the CUDA runtime or
 * a device is missing, calls that need the GPU return LLF_ERR_CUDA.
 *
 * Conventions kept from the reference (LowLevelFEM.jl v1.13.31):
 *   - node tags are dense and 1-based (src/multifield.jl:1602-1611);
 *   - DoF numbering is interleaved, dof = (node-1)*pdim + comp (1-based,
 *     src/general.jl:5245-5247); internally 0-based, 1-based at copy-out;
 *   - matrices leave the library as SparseMatrixCSC{Float64,Int64} arrays:
 *     1-based Int64 colptr (n+1) and rowval (nnz), Float64 nzval, rows sorted
 *     within each column, exact zeros removed as dropzeros! does
 *     (src/linear.jl:323-324);
 *   - element node tables (connectivity) are element-major, npe entries per
 *     element, in the element family's node order (gmsh order for the tables
 *     the caller uploads, this library's order for its built-in tables).
 *
 * Objects (opaque, all device-resident):
 *   llf_ctx      one CUDA device + one stream + last-error text; not thread
 *                safe — use one context per host thread / Julia task.
 *   llf_mesh     node coordinates, connectivity, node->element adjacency,
 *                quadrature + shape tables, per-element material index.
 *   llf_pattern  structural CSC pattern of a mesh for pdim components per
 *                node (node-level adjacency expanded to DoFs).
 *   llf_matrix   values on a pattern (structural nzval) plus, after
 *                assembly, the stored (dropzeros'ed) form.
 */
#ifndef LLFEM_GB300_H
#define LLFEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define LLF_OK                  0
#define LLF_ERR_ARG            -1   /* bad argument (null pointer, size, enum)   */
#define LLF_ERR_CUDA           -2   /* CUDA runtime error or no device           */
#define LLF_ERR_MESH           -3   /* bad connectivity / non-positive Jacobian  */
#define LLF_ERR_NOT_CONVERGED  -4   /* iterative solve hit maxiter               */
#define LLF_ERR_STATE          -5   /* object used with a mismatched partner     */
#define LLF_ERR_UNSUPPORTED    -6   /* element family/order/problem not built    */
#define LLF_ERR_LIMIT          -7   /* a documented size limit was exceeded      */
#define LLF_ERR_NUMERIC        -8   /* NaN/Inf in input, or singular pivot      */

/* ---- element families (values equal gmsh's first-order type numbers) ---- */
#define LLF_LINE  1
#define LLF_TRI   2
#define LLF_QUAD  3
#define LLF_TET   4
#define LLF_HEX   5

/* ---- problem types (Problem.type of src/general.jl:478-632) ------------- */
#define LLF_SOLID                  0   /* :Solid,   dim 3, pdim 3 */
#define LLF_PLANE_STRESS           1   /* :PlaneStress, dim 2, pdim 2 */
#define LLF_PLANE_STRAIN           2   /* :PlaneStrain, dim 2, pdim 2 */
#define LLF_HEAT_CONDUCTION        3   /* :HeatConduction, dim 3, pdim 1 */
#define LLF_PLANE_HEAT_CONDUCTION  4   /* :PlaneHeatConduction, dim 2, pdim 1 */

/* ---- arithmetic forms ---------------------------------------------------- */
#define LLF_FP64   0   /* plain form: every operation in IEEE FP64, fixed order */
#define LLF_FP32Q  1   /* precision form: FP32 quadrature, FP64 accumulation    */
#define LLF_TF32X3 2   /* tensor-core form: element contraction on the tensor
                          cores with split TF32 operands (hi*hi + hi*lo + lo*hi),
                          FP32 accumulation, FP64 global accumulation */

/* ---- weak-form DSL bilinear forms (src/multifield.jl:4385-4931) -------- */
#define LLF_FORM_SYMGRAD_D_SYMGRAD 0  /* ∫(SymGrad(P)⋅D⋅SymGrad(P)), isotropic D: c1 = lambda, c2 = mu */
#define LLF_FORM_GRAD_K_GRAD       1  /* ∫(Grad(P)⋅k⋅Grad(P)), scalar P: c1 = k */
#define LLF_FORM_ID_C_ID           2  /* ∫(Id(P)⋅c⋅Id(P)): c1 = c */

/* ---- hyperelastic laws for the Total Lagrangian kernels ----------------- */
#define LLF_LAW_CONSTANT_C     0   /* params: 36 values, 6x6 Voigt tangent, column-major */
#define LLF_LAW_NEOHOOKE_COMP  1   /* params: mu, lambda; psi = mu/2(I1-3) - mu lnJ + lambda/2 (lnJ)^2 */
#define LLF_LAW_SVK            2   /* params: mu, lambda; psi = lambda/2 tr(E)^2 + mu E:E */

/* ---- preconditioners for llf_pcg ---------------------------------------- */
#define LLF_PRECOND_NONE     0   /* IterativeSolvers Identity() (src/linear.jl:3711) */
#define LLF_PRECOND_JACOBI   1
#define LLF_PRECOND_BJACOBI  2   /* pdim x pdim node-block Jacobi */
#define LLF_PRECOND_IC0      3   /* node-block IC(0) in multicolour order (llf_pcg, llf_pcg_batched) */

typedef struct llf_ctx     llf_ctx;
typedef struct llf_mesh    llf_mesh;
typedef struct llf_pattern llf_pattern;
typedef struct llf_matrix  llf_matrix;

/* ======================================================================== */
/* Library / context                                                        */
/* ======================================================================== */

/* Version string of the shared library. */
const char *llf_version(void);

/* Create a context on CUDA device `device` with its own non-blocking stream.
 * Replaces nothing in the reference (Julia has no device); the Julia shim
 * creates one per task. */
int llf_ctx_create(int device, llf_ctx **out);
int llf_ctx_destroy(llf_ctx *ctx);

/* Message of the last failing call on this context ("" after success).
 * Plays the role of the reference's error("...") text (e.g. src/linear.jl:185). */
const char *llf_last_error(const llf_ctx *ctx);

/* Synchronise the context's stream (all queued work finished). */
int llf_ctx_sync(llf_ctx *ctx);

/* The stream the context launches on, as a cudaStream_t cast to void*. */
int llf_ctx_stream(llf_ctx *ctx, void **stream);

/* Tracing (no counterpart in the reference, which times with @time).
 * Every kernel launch of the context is counted; with profiling enabled,
 * CUDA events bracket each launch on the context stream and the report
 * holds per-kernel launch counts and summed device milliseconds as JSON
 * {"kernel": {"launches": n, "ms": t}, ...}.  report writes at most len
 * bytes (NUL-terminated) and returns the full length through *needed. */
int llf_profile_enable(llf_ctx *ctx, int on);
int llf_profile_reset(llf_ctx *ctx);
int llf_profile_report(llf_ctx *ctx, char *buf, int64_t len, int64_t *needed);
int llf_launch_count(llf_ctx *ctx, int64_t *launches);
/* Device allocations the context has made since it was created (every
 * stream-ordered allocation of an entry point counts once).  A diagnostic
 * counter with no reference counterpart: a caller can check that a call
 * allocated nothing by reading it before and after. */
int llf_alloc_count(llf_ctx *ctx, int64_t *allocs);

/* ======================================================================== */
/* Built-in quadrature and shape tables (host only, no GPU needed)          */
/* ======================================================================== */

/* Quadrature rule exact to degree 2*order+1 and Lagrange shape tables of one
 * element family/order, standing in for gmsh's
 *   getIntegrationPoints(et, "Gauss"*(2*order+1))   (src/linear.jl:235)
 *   getBasisFunctions(et, ip, "Lagrange"/"GradLagrange") (src/linear.jl:238).
 * Two-phase: call with null arrays to obtain *nip and *npe, then again with
 * arrays of size xi[3*nip], w[nip], N[nip*npe], dN[3*nip*npe],
 * node_ref[3*npe].  N[q*npe+a] = N_a(xi_q); dN[(q*npe+a)*3+j] = dN_a/dxi_j.
 * Reference elements follow gmsh: [-1,1]^d for quads/hexes, the unit
 * simplex for triangles/tetrahedra. */
int llf_builtin_rule(int family, int order, int *nip, int *npe,
                     double *xi, double *w, double *N, double *dN,
                     double *node_ref);

/* Reference gradients of the built-in basis at the element's own nodes,
 * dNn[(k*npe+l)*3+j] = dN_l/dxi_j at node k (npe*npe*3 values) — the table
 * ∇ evaluates at element nodes (gmsh getBasisFunctions at the element's
 * local node coordinates, src/nabla.jl:124-126). */
int llf_builtin_node_gradients(int family, int order, double *dNn);

/* ======================================================================== */
/* Mesh                                                                     */
/* ======================================================================== */

/* Upload a mesh: xyz[3*non] (x,y,z per node; z ignored when dim==2),
 * conn[npe*nel] 1-based node tags, element-major.  The built-in tables of
 * (family, order) are attached; llf_tables_upload replaces them.
 * Replaces the gmsh queries getNodes / getElementsByType of
 * src/linear.jl:241 and src/multifield.jl:1612-1648. */
int llf_mesh_upload(llf_ctx *ctx, int dim, int64_t non, const double *xyz,
                    int64_t nel, int npe, const int64_t *conn,
                    int family, int order, llf_mesh **out);

/* Overwrite the coordinates (and, if conn != NULL, the connectivity, which
 * must describe the same adjacency) of an uploaded mesh; used when node
 * positions move but the pattern is reused. */
int llf_mesh_update(llf_ctx *ctx, llf_mesh *mesh, const double *xyz,
                    const int64_t *conn);

/* Per-element material index (0..nmat-1) or -1 for "not in any material
 * group" (such elements contribute nothing, as elements outside every
 * Material physical group do in src/linear.jl:211-232).  NULL = all 0. */
int llf_mesh_set_materials(llf_ctx *ctx, llf_mesh *mesh,
                           const int32_t *elem_mat);

/* Replace the quadrature/shape tables with caller-supplied ones (e.g. gmsh's
 * own getIntegrationPoints / getBasisFunctions output), same layout as
 * llf_builtin_rule.  N may be NULL when only gradients are needed. */
int llf_tables_upload(llf_ctx *ctx, llf_mesh *mesh, int nip, const double *w,
                      const double *N, const double *dN);

int llf_mesh_destroy(llf_ctx *ctx, llf_mesh *mesh);

/* ======================================================================== */
/* CSC pattern                                                              */
/* ======================================================================== */

/* Structural CSC pattern for pdim components per node: node adjacency
 * through shared elements, rows sorted per column, components expanded —
 * build_csc_pattern of src/multifield.jl:2083-2250.  *nnz_out receives the
 * structural nnz. */
int llf_pattern_build(llf_ctx *ctx, llf_mesh *mesh, int pdim,
                      int64_t *nnz_out, llf_pattern **out);

/* Copy the structural pattern to host arrays: colptr[n+1], rowval[nnz],
 * both 1-based Int64. */
int llf_pattern_copy(llf_ctx *ctx, const llf_pattern *pat, int64_t *colptr,
                     int64_t *rowval);

int llf_pattern_info(const llf_pattern *pat, int64_t *ndof, int64_t *nnz,
                     int *pdim);

int llf_pattern_destroy(llf_ctx *ctx, llf_pattern *pat);

/* ======================================================================== */
/* Assembly                                                                 */
/* ======================================================================== */
/* All assembly calls create a new device matrix on the pattern, fill the
 * structural values, then apply dropzeros!.  Material arrays hold one value
 * per material index (nmat entries). `form` is LLF_FP64 or LLF_FP32Q.
 *
 * Stored layouts.  A pattern keeps the stored (dropzeros'ed) column layout
 * of its last assembly of each operator and form (stiffness, mass, heat; a
 * few at a time).  The next such assembly on the pattern writes its stored
 * CSC straight from the gather into that layout and checks every column's
 * non-zero count; if a count differs, the assembly counts and compacts the
 * usual way and keeps the new layout.  The arrays returned are the same
 * either way.  A matrix assembled into a kept layout holds the stored CSC
 * only; its structural values (the solvers' format) are expanded from it on
 * the first call that needs them (llf_pcg*, llf_matrix_spmv,
 * llf_matrix_copy_structural, llf_matrix_axpby, llf_heat_fdm, or
 * llf_matrix_prepare), except llf_pcg_noalloc, which refuses such a matrix.
 * LLF_STORED_LAYOUT=0 in the environment turns the reuse off.  Not used for
 * lumped mass matrices, nor for assemblies that accumulate into a matrix. */

/* K = sum_e sum_q B^T D B b detJ w — stiffnessMatrix / stiffnessMatrixSolid,
 * src/linear.jl:70-87, :154-188, :190-330.  ptype LLF_SOLID,
 * LLF_PLANE_STRESS (b = thickness) or LLF_PLANE_STRAIN (b = 1). */
int llf_assemble_stiffness(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat,
                           int ptype, const double *E, const double *nu,
                           int nmat, double thickness, int form,
                           llf_matrix **out);

/* Tune the launch schedule of llf_assemble_stiffness for this mesh and
 * pattern (the reference leaves its threaded assembly's element chunk size
 * to an automatic choice, src/multifield.jl:2645, :3029-3033): the element
 * kernels' CTAs per SM, the gather's degree-class threshold and warps per
 * CTA, chosen one knob at a time from timed assemblies (best of `trials`
 * each, after a warm one).  No choice changes a result bit, and every
 * candidate's stored CSC is checked against the first one's.  The choice is
 * kept on the pattern and reused for every pattern of the same shape
 * (family, order, nodes per element, DoFs per node, operator, form, log2
 * of the element count) in this process, and across processes when the
 * environment variable LLF_TUNE_FILE names a file.  report (may be NULL)
 * receives a JSON text of the candidates and their times; *needed its
 * length. */
int llf_autotune_stiffness(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int ptype,
                           const double *E, const double *nu, int nmat, double thickness,
                           int form, int trials, char *report, int64_t report_len,
                           int64_t *needed);

/* stiffnessMatrix straight into the host arrays of a
 * SparseMatrixCSC{Float64,Int64} — the same result, bit for bit, as
 * llf_assemble_stiffness followed by llf_matrix_copy_csc, in one call whose
 * device-to-host copy of each column slab overlaps the gather and
 * compaction of the next (the copy is the largest cost of the pair).
 * rowval and nzval hold `capacity` entries, at least the pattern's
 * structural nnz (llf_pattern_info); *nnz receives the stored count (the
 * Julia side resize!s the arrays to it).  colptr[ndof+1].  Page-locked host
 * arrays let the copies run asynchronously. */
int llf_assemble_stiffness_csc(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat,
                               int ptype, const double *E, const double *nu,
                               int nmat, double thickness, int form,
                               int64_t capacity, int64_t *colptr,
                               int64_t *rowval, double *nzval, int64_t *nnz);

/* stiffnessMatrix as values against a pattern the caller already holds
 * (no counterpart in the reference; its stiffnessMatrix returns a fresh
 * SparseMatrixCSC each call).  The same assembly and column-slab copies as
 * llf_assemble_stiffness_csc, but rowval, which the pattern fixes up to
 * the entries dropzeros! removes, is not copied: colptr[ndof+1] (1-based)
 * and nzval[capacity >= structural nnz] receive the stored CSC, and
 * keep[(structural nnz + 31)/32] one bit per structural entry (bit k of
 * word k/32: entry k of llf_pattern_copy's rowval is stored).  The stored
 * rowval is the structural rowval filtered by keep (llf_rowval_from_keep);
 * a caller that re-assembles the same operator keeps its previous rowval
 * while the keep bits do not change, so each call moves about half the
 * bytes of llf_assemble_stiffness_csc.  *keep_changed (may be NULL)
 * receives 0 when the bits equal those of the previous values call on the
 * same pattern (compared on the device), else 1. */
int llf_assemble_stiffness_values(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat,
                                  int ptype, const double *E, const double *nu,
                                  int nmat, double thickness, int form,
                                  int64_t capacity, int64_t *colptr, double *nzval,
                                  uint32_t *keep, int64_t *nnz, int *keep_changed);

/* Host only: the stored rowval from the structural rowval and the keep bits
 * of llf_assemble_stiffness_values; returns the stored count (or a negative
 * status). */
int64_t llf_rowval_from_keep(int64_t nnz_structural, const int64_t *rowval_structural,
                             const uint32_t *keep, int64_t *rowval);

/* M = rho b sum H^T H detJ w, consistent (lumped == 0) or row-sum lumped —
 * massMatrix / massMatrixSolid, src/linear.jl:1843-2004. */
int llf_assemble_mass(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat,
                      int ptype, const double *rho, int nmat,
                      double thickness, int lumped, int form,
                      llf_matrix **out);

/* K_T = sum grad N^T grad N k b detJ w — heatConductionMatrix /
 * heatCondMatrixSolid, src/heat.jl:28-137 (b = thickness in 2D and 3D). */
int llf_assemble_heat(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat,
                      int ptype, const double *k, int nmat, double thickness,
                      int form, llf_matrix **out);

/* Follower-load tangent of traction loads on faces of a 3D body —
 * externalTangentFollower, src/nonlinear.jl:3053-3258: per face point, with
 * F_q interpolated from F_nodal[9*non] (column-major 3x3 per node), tg = F_q t
 * and g = grad N_b on the face (Jacobian [t1 t2 n], n the unit normal),
 *   K[(a,i),(b,j)] += N_a (Jgp F^-T ((F^-1[:,j].g) tg - (F^-1[:,j].tg) g
 *                     + (g.F^-1 tg) e_j))_i |t1 x t2| w,
 * triplets in element order, sparse, dropzeros!.  Traction per boundary
 * element t_elem[3*nel_b] or at its nodes t_elem_nodal[3*npe*nel_b]
 * (exactly one non-NULL).  The matrix is unsymmetric and lives on the
 * volume pattern. */
int llf_follower_tangent(llf_ctx *ctx, llf_pattern *pat, llf_mesh *bmesh,
                         const double *F_nodal, const double *t_elem,
                         const double *t_elem_nodal, llf_matrix **out);

/* Weak-form DSL bilinear term ∫(a(P)⋅coef⋅b(P); csc_matrix) —
 * src/multifield.jl:5280-5346 with assemble_operator, :2630-.  The three
 * forms above run on the assembly kernels with the coefficients as given
 * (b = 1; per material index, nmat entries).  accumulate NULL: a new matrix
 * with dropzeros!.  accumulate = a matrix on the same pattern (csc_matrix):
 * the assembly adds into its values in element order, keeps the full
 * structural pattern, and the result is returned in *out (accumulate itself
 * is left unchanged). */
int llf_assemble_form(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int form_kind,
                      const double *c1, const double *c2, int nmat,
                      const llf_matrix *accumulate, int form, llf_matrix **out);

/* build_csc_pattern, src/multifield.jl:2083-2250: a matrix on the pattern
 * holding structural zeros, whose stored form keeps every entry. */
int llf_matrix_zero_pattern(llf_ctx *ctx, llf_pattern *pat, llf_matrix **out);

/* Boundary support matrix C = sum H^T diag(k) H Ja w over the elements of
 * `bmesh` (dimension dim-1, node tags of the pattern's volume mesh), Ja as in
 * llf_load_vector — elasticSupportMatrix, src/linear.jl:2859-3005 (k = kx,
 * ky, kz), and heatConvectionMatrix, src/heat.jl:562-567 (pdim 1, k = h).
 * Exactly one of k_elem[pdim*nel_b] (one constant per boundary element) and
 * k_elem_nodal[pdim*npe*nel_b] (values at every element's nodes,
 * interpolated at the points) is non-NULL.  Several support groups go in one
 * call as one element list in group order, which sums them in the order of
 * the reference's single sparse() call.  The matrix lives on the volume
 * pattern, so it adds to the stiffness or conduction matrix with
 * llf_matrix_axpby. */
int llf_assemble_support(llf_ctx *ctx, llf_pattern *pat, llf_mesh *bmesh,
                         const double *k_elem, const double *k_elem_nodal,
                         double thickness, llf_matrix **out);

/* Total Lagrangian material tangent K_mat = sum B(F)^T C B(F) detJ0 w —
 * materialTangentMatrix, src/nonlinear.jl:2083-2268.  Felem[9*npe*nel] holds
 * the elementwise nodal deformation gradient, column-major 3x3 per element
 * node (the TensorField layout of src/nonlinear.jl:2183-2199).  `law` and
 * params[] as LLF_LAW_*; for LLF_LAW_CONSTANT_C, params is the 6x6 matrix. */
int llf_tl_material_tangent(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat,
                            const double *Felem, int law,
                            const double *params, int nparams,
                            llf_matrix **out);

/* Consistent Newton tangent K_mat + K_geo in one pass from the elementwise
 * nodal F: at every point S and the tangent come from the same C = F^T F, so
 * the matrix is the exact derivative of llf_tl_internal_force.  Replaces the
 * user-level sum materialTangentMatrix(F) + initialStressMatrix(C) of the
 * reference's Newton loops (src/nonlinear.jl:2083-2595), which interpolates
 * the nodal C = F^T F instead. */
int llf_tl_tangent(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat,
                   const double *Felem, int law, const double *params,
                   int nparams, llf_matrix **out);

/* llf_tl_tangent with a choice of arithmetic: LLF_FP64 (the call above) or
 * LLF_TF32X3 — the element matrices as one dense GEMM per element,
 * [B; G]^T diag(w D, w S (x) I) [B; G] with 15 rows per point, on the
 * tensor cores (tcgen05, split TF32 products, FP32 accumulation in tensor
 * memory), then summed in FP64.  Meant for high-order elements (order >= 3),
 * where the contraction is dense.  The tile operands are formed in FP32 and
 * summed in FP32, so values agree with the FP64 form to about 1e-5 of the
 * largest entry for a well-conditioned F (less as det F approaches 0). */
int llf_tl_tangent_form(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat,
                        const double *Felem, int law, const double *params,
                        int nparams, int form, llf_matrix **out);

/* Geometric (initial-stress) stiffness K_geo[a i, b i] = sum grad Na^T S
 * grad Nb detJ0 w, identity component block — initialStressMatrix,
 * src/nonlinear.jl:2417-2595.  Exactly one of Selem (elementwise nodal PK2
 * stress, 9*npe*nel) or Celem (elementwise nodal right Cauchy-Green tensor,
 * with `law`) is non-NULL. */
int llf_tl_initial_stress(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat,
                          const double *Selem, const double *Celem, int law,
                          const double *params, int nparams,
                          llf_matrix **out);

/* Internal force f_int[a i] = sum P_iJ dNa/dX_J detJ0 w, P = F S —
 * internalForceVector, src/nonlinear.jl:2738-2910.  Exactly one of Pelem
 * (elementwise nodal first Piola-Kirchhoff stress) or Felem (with `law`) is
 * non-NULL.  f_int[3*non] is a host array, overwritten. */
int llf_tl_internal_force(llf_ctx *ctx, llf_mesh *mesh, const double *Pelem,
                          const double *Felem, int law, const double *params,
                          int nparams, double *f_int);

/* Elementwise nodal gradient of a nodal vector field, T[i,j] = du_i/dX_j,
 * column-major 3x3 per element node (9*npe*nel) — the :vector_grad branch of
 * ∇ / u∘∇, src/nabla.jl:77-311 and src/operators.jl:2875-2881.  u[pdim*non]
 * interleaved; with add_identity != 0 the result is F = I + u∘∇. */
int llf_grad_elementwise(llf_ctx *ctx, llf_mesh *mesh, const double *u,
                         int add_identity, double *out);

/* Consistent nodal load of boundary elements: f += sum H^T t Ja w over the
 * elements of `bmesh` (a mesh of dimension dim-1 embedded in dim), with t a
 * constant pdim-vector (t_const) or nodal values t_nodal[pdim*non_b] per
 * boundary-mesh node (NULL to use t_const).  Ja is the line/area measure
 * (times thickness for 2D problems) — loadVector, src/linear.jl:3088-3434,
 * Ja at :3378-3407.  Node tags of bmesh index the volume mesh's nodes;
 * f[pdim*non] is a host array accumulated into. */
int llf_load_vector(llf_ctx *ctx, llf_mesh *bmesh, int problem_dim, int pdim,
                    const double *t_const, const double *t_nodal,
                    double thickness, double *f, int64_t ndof);

/* Follower traction loads of a 3D body — loadVector(problem, loads; F),
 * src/linear.jl:3333-3372: the traction at a face point is F_q t (F_q
 * interpolated from F_nodal[9*non], column-major 3x3 per node), integrated
 * on the reference face.  t_const[3] or t_nodal[3*non]; f[3*non] host,
 * accumulated into. */
int llf_load_vector_follower(llf_ctx *ctx, llf_mesh *bmesh, const double *F_nodal,
                             const double *t_const, const double *t_nodal,
                             double *f, int64_t ndof);

/* elementsToNodes, src/general.jl:5519-5640: nodal[ncomp*non] = the mean of
 * the element-node values elem_values[ncomp*npe*nel] of every node (summed
 * in element order, times 1/count); nodes in no element get 0. */
int llf_elements_to_nodes(llf_ctx *ctx, llf_mesh *mesh, int ncomp,
                          const double *elem_values, double *nodal);

/* ======================================================================== */
/* Matrices                                                                 */
/* ======================================================================== */

/* Stored nnz after dropzeros!. */
int llf_matrix_nnz(llf_ctx *ctx, const llf_matrix *m, int64_t *nnz);

/* Copy the stored CSC to host: colptr[n+1], rowval[nnz] (1-based Int64),
 * nzval[nnz]. Any pointer may be NULL to skip that array. */
int llf_matrix_copy_csc(llf_ctx *ctx, const llf_matrix *m, int64_t *colptr,
                        int64_t *rowval, double *nzval);

/* Make the matrix's structural values resident: expands them from the
 * stored CSC when its assembly wrote the stored CSC only (allocates the
 * structural array), else does nothing.  Call it before llf_pcg_noalloc on
 * a matrix assembled into a kept stored layout. */
int llf_matrix_prepare(llf_ctx *ctx, llf_matrix *m);

/* Structural values (length = structural nnz of the pattern) to host.  For
 * a matrix assembled into a kept stored layout they are expanded from its
 * stored CSC first; the entries dropzeros! removed then read +0.0. */
int llf_matrix_copy_structural(llf_ctx *ctx, const llf_matrix *m,
                               double *nzval);

/* Device matrix from host structural values nzval[nnz of pat], in the
 * pattern's CSC order; the stored form is then built with dropzeros!.  Lets
 * a host-side SystemMatrix (e.g. after applyElasticSupport!) re-enter the
 * device solve (SystemMatrix(A, model), src/general.jl:762-771). */
int llf_matrix_from_structural(llf_ctx *ctx, llf_pattern *pat, const double *nzval,
                               llf_matrix **out);

/* C = a*A + b*B on the same pattern, then dropzeros! — SystemMatrix +/-
 * of src/operators.jl:2421-2486 (Kmat + Kgeo, K - Kext).  A lumped
 * (diagonal) operand adds on the diagonal; two lumped operands give a
 * lumped result. */
int llf_matrix_axpby(llf_ctx *ctx, double a, const llf_matrix *A, double b,
                     const llf_matrix *B, llf_matrix **out);

/* y = A x with host vectors of length n. */
int llf_matrix_spmv(llf_ctx *ctx, const llf_matrix *m, const double *x,
                    double *y);

int llf_matrix_destroy(llf_ctx *ctx, llf_matrix *m);

/* ======================================================================== */
/* Solve                                                                    */
/* ======================================================================== */

/* Condensed Dirichlet solve by preconditioned CG — the iterative branch of
 * solveDisplacement / solveTemperature / solveField (src/linear.jl:3711-3743,
 * :3801-3834; src/heat.jl:1020-1084; src/poisson.jl:1432-1546):
 *   fixed[i] != 0 marks constrained DoFs, whose prescribed values are taken
 *   from x on entry (applyBoundaryConditions!, src/linear.jl:3505-3563);
 *   f_kin = A[:,fixed] x[fixed]; x[free] solves
 *   A[free,free] x[free] = b[free] - f_kin[free]
 * with IterativeSolvers.cg's recurrence and stopping rule
 * (||r|| <= reltol ||b_free - f_kin_free||, x0 = 0 on the free DoFs).
 * All vectors are host arrays of length n.  *iters and *relres report the
 * iteration count and final relative residual; LLF_ERR_NOT_CONVERGED is
 * returned (x still holds the last iterate) when maxiter is reached. */
int llf_pcg(llf_ctx *ctx, const llf_matrix *m, const double *b, double *x,
            const uint8_t *fixed, int precond, double reltol, int64_t maxiter,
            int64_t *iters, double *relres);

/* Transient heat conduction by the theta-method — FDM(K, C, q, bc, T0, n,
 * dt; ϑ), src/heat.jl:1466-1616.  K (conduction, with any convection added)
 * and C (capacity, consistent or lumped) on the same pattern.  q[ndof*q_steps]
 * (q_steps 1 or nsteps, column-major), T[ndof*nsteps] host: on entry column
 * 0 is the initial state and the fixed entries of every column hold the
 * prescribed values (applyBoundaryConditions!); on return every column holds
 * the state at t = i*dt.  theta == 0 with a lumped C takes the reference's
 * explicit update; otherwise every step solves
 *   (C + ϑ dt K)_ff T_f^{n+1} = ((C - (1-ϑ) dt K) T^n + dt q^{n+ϑ})_f
 *                               - (C + ϑ dt K)_fc T_c^{n+1}
 * by PCG to reltol (the reference uses one LU factorisation), starting from
 * T^n, with the preconditioner built once.  *iters_total sums the PCG
 * iterations.  A non-positive diag(C) on a free DoF is an error, as in the
 * reference. */
int llf_heat_fdm(llf_ctx *ctx, const llf_matrix *K, const llf_matrix *C,
                 const double *q, int q_steps, double *T, const uint8_t *fixed,
                 int64_t nsteps, double dt, double theta, int precond,
                 double reltol, int64_t maxiter, int64_t *iters_total);

/* Largest system (DoFs) llf_pcg_noalloc accepts. */
#define LLF_NOALLOC_MAX_DOFS 131072

/* Allocation-free variant of llf_pcg (no counterpart in the reference).
 *
 * For callers that cannot allocate device memory once they are running:
 * code inside a host framework that has already reserved the GPU's memory
 * for its own pool, real-time or control loops that forbid allocation (and
 * its latency and fragmentation) after start-up, and solvers embedded in a
 * process whose device-memory budget is fixed in advance.  Such a caller
 * passes device pointers it already owns — right-hand side d_b, the initial
 * and prescribed values d_x (overwritten with the solution) and the mask
 * d_fixed, each of the matrix's DoF count — and the call allocates nothing:
 * no cudaMalloc, cudaMallocAsync or cudaFree, no library allocator.  The CG
 * work vectors live in one fixed array compiled into the library
 * (about 8.7 MB for LLF_NOALLOC_MAX_DOFS = 131072 unknowns), which every GPU
 * that loads the library holds until the process exits.
 *
 * Same algorithm and results as llf_pcg (IterativeSolvers.cg recurrence and
 * stopping rule, Dirichlet masking) with the preconditioners none, Jacobi
 * and block Jacobi; IC(0) is not available here (its factor and colouring
 * need memory sized by the matrix) and is refused with LLF_ERR_UNSUPPORTED.
 * Systems above LLF_NOALLOC_MAX_DOFS are rejected with LLF_ERR_LIMIT.  The
 * first call on a device looks up the array's device address for that
 * device, with that device made current for the lookup and the caller's
 * current device restored afterwards (make that first call before any
 * stream capture).  The address is kept for the life of the process: a
 * cudaDeviceReset, or any other teardown of the device's primary context,
 * invalidates it, so do not call this entry point after one.  All calls
 * share the one array and it keeps the previous call's contents; each call
 * clears on its own stream what has to start at zero (the count of
 * unconverged systems and the three arrival counters of the chunk
 * reductions: the product's u.c for alpha, the update's residual norm and
 * z.r after a sweep preconditioner)
 * and writes every other work vector before reading it.  Calls whose work
 * overlaps on the GPU (two contexts or threads at once) race on the array:
 * serialise them.  The matrix's structural values must be resident (see
 * llf_matrix_prepare); a matrix that holds its stored CSC only is refused
 * with LLF_ERR_STATE. */
int llf_pcg_noalloc(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
                    const uint8_t *d_fixed, int precond, double reltol, int64_t maxiter,
                    int64_t *iters, double *relres);

/* Batched form of llf_pcg for a block-diagonal matrix of nseg independent
 * systems (for example many meshes assembled together as one mesh with one
 * material per instance): system g owns DoFs [seg_off[g], seg_off[g+1]).
 * Every system runs its own CG — own scalars and stopping test, exactly as a
 * separate llf_pcg call would — inside the same kernel launches, replayed
 * from a captured CUDA graph.  iters[nseg] and relres[nseg] are per system.
 * Replaces a loop of solveField calls (src/poisson.jl:1432-1546). */
int llf_pcg_batched(llf_ctx *ctx, const llf_matrix *m, const double *b, double *x,
                    const uint8_t *fixed, int nseg, const int64_t *seg_off,
                    int precond, double reltol, int64_t maxiter, int64_t *iters,
                    double *relres);

/* Mixed-precision form of llf_pcg_batched (nseg = 1: a single system),
 * replacing the same cg(K.A[free,free], ...) call (src/linear.jl:3827-3828).
 * The iterations run in FP32: an FP32 copy of the matrix values, FP32
 * vectors and products, the preconditioner (Jacobi, block Jacobi or IC(0))
 * applied into FP32.  The solution is accumulated in FP64 and the residual
 * is replaced by the true residual b - A x of the FP64 matrix whenever the
 * FP32 one has fallen 100-fold since the last replacement, at the
 * tolerance and at maxiter; a system stops only when that true FP64
 * residual meets ||r|| <= reltol ||r0||, so relres[] is an FP64 residual.
 * iters[] counts FP32 products.  Each system runs its own CG, and its
 * result is the same alone and in a batch. */
int llf_pcg_mixed(llf_ctx *ctx, const llf_matrix *m, const double *b, double *x,
                  const uint8_t *fixed, int nseg, const int64_t *seg_off,
                  int precond, double reltol, int64_t maxiter, int64_t *iters,
                  double *relres);

/* ======================================================================== */
/* Serving                                                                  */
/* ======================================================================== */
/* A request server for steady heat-conduction solves — the serving form of
 * solveTemperature(problem; heatFlux, temperatureConstraint)
 * (src/heat.jl:1068-1084): each request carries its own mesh, conductivity,
 * right-hand side, prescribed temperatures and tolerance.  nworkers threads,
 * each with its own context and stream, take queued requests in arrival
 * order as soon as a worker is free and the request's device-memory
 * estimate fits in mem_budget_bytes; requests in flight overlap on the GPU.
 * Results are the same as a lone solve of the request (deterministic
 * kernels). */
typedef struct llf_server llf_server;

int llf_server_create(int device, int nworkers, int64_t mem_budget_bytes,
                      llf_server **out);

/* The continuous-batching form of the same server.  nprep preparation
 * threads (each with its own context) take requests in arrival order as the
 * memory budget allows, upload the mesh, build the pattern, assemble K and
 * run the first CG steps.  One engine thread then runs the CG iterations of
 * every prepared request together: the requests occupy slots (at most
 * max_systems) of a device-resident table, and one captured CUDA graph of 16
 * iterations is replayed over the table; between replays converged requests
 * are retired (result to the host, memory released) and newly prepared ones
 * admitted, so requests that arrive while others iterate join the next
 * replay.  Preconditioners: none, Jacobi, block Jacobi (IC(0) is refused per
 * request).  Each result equals that of a lone llf_pcg solve of the request
 * bit for bit.  Submission, waiting, statistics and destruction are the
 * calls below. */
int llf_server_create_batched(int device, int nprep, int max_systems,
                              int64_t mem_budget_bytes, llf_server **out);

/* Copy one request into the server; *ticket identifies it. x0[non] holds the
 * prescribed temperatures on fixed[non] != 0 (other entries ignored); rhs
 * (may be NULL = 0) the nodal heat loads.  maxiter <= 0 means 20*non. */
int llf_server_submit_heat(llf_server *s, int dim, int64_t non,
                           const double *xyz, int64_t nel, int npe,
                           const int64_t *conn, int family, int order,
                           double k, double thickness, const double *rhs,
                           const double *x0, const uint8_t *fixed,
                           int precond, double reltol, int64_t maxiter,
                           int64_t *ticket);

/* Wait up to timeout_s (< 0: no limit) for a ticket and take its result:
 * solution x[non], CG iterations and relative residual, latency from
 * submission to result and the worker's service time; err receives the
 * error text of a failed request.  Returns LLF_ERR_STATE on timeout or an
 * unknown ticket, otherwise the request's own status. */
int llf_server_wait(llf_server *s, int64_t ticket, double timeout_s, double *x,
                    int64_t *iters, double *relres, double *latency_s,
                    double *service_s, char *err, int64_t errlen);

int llf_server_stats(llf_server *s, int64_t *queued, int64_t *served,
                     int64_t *bytes_in_use, int64_t *peak_bytes);

/* Where a continuous-batching server's time went (no reference
 * counterpart; a diagnostic): seconds summed over the preparation threads,
 * the engine's replays, its retirements and its idle waits, the replay
 * count and the mean number of requests admitted per replay. */
int llf_server_timing(llf_server *s, double *prep_s, double *step_s, double *collect_s,
                      double *idle_s, int64_t *replays, double *mean_admitted);

/* Drains the queue, joins the workers and frees the server. */
int llf_server_destroy(llf_server *s);

#ifdef __cplusplus
}
#endif

#endif /* LLFEM_GB300_H */
