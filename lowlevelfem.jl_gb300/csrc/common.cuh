// Internal declarations shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <functional>
#include <string>
#include <vector>

#include "../../include/llfem_gb300.h"

// ---------------------------------------------------------------- status
// Bits a kernel may set in the context's device status word.  Kernels never
// trap; the host reads the word after the operation and turns a set bit into
// an error return.
enum : unsigned {
  ST_BAD_NODE = 1u << 0,      // connectivity entry outside 1..non
  ST_BAD_JACOBIAN = 1u << 1,  // non-positive Jacobian determinant
  ST_CAPACITY = 1u << 2,      // per-node candidate list exceeds its buffer
  ST_NONFINITE = 1u << 3,     // NaN/Inf in an input array
  ST_PATTERN = 1u << 4,       // an element pair found no pattern slot
  ST_BREAKDOWN = 1u << 5,     // CG breakdown (u.Au <= 0 or not finite)
  ST_TIMEOUT = 1u << 6,       // a bounded wait on the tensor cores gave up
};

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

// Per-kernel tracing: every launch site opens a KernelScope; launches are
// always counted, and with profiling enabled a pair of CUDA events brackets
// the launch on the context's stream (durations resolved lazily).
struct ProfPending {
  const char *name;
  cudaEvent_t a, b;
};
struct ProfAcc {
  double ms = 0.0;
  long long launches = 0;
};

struct llf_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  unsigned *d_status = nullptr;   // device status word
  unsigned *h_status = nullptr;   // pinned host mirror
  int num_sms = 0;
  bool profiling = false;
  long long launches = 0;
  long long allocs = 0;           // device allocations made through the context
  std::vector<ProfPending> pending;
  std::vector<std::pair<std::string, ProfAcc>> prof;
};

void prof_resolve(llf_ctx *ctx);

struct KernelScope {
  llf_ctx *ctx;
  ProfPending rec{};
  bool on = false;
  KernelScope(llf_ctx *c, const char *name) : ctx(c) {
    ctx->launches++;
    if (ctx->profiling) {
      rec.name = name;
      if (cudaEventCreate(&rec.a) == cudaSuccess && cudaEventCreate(&rec.b) == cudaSuccess) {
        cudaEventRecord(rec.a, ctx->stream);
        on = true;
      }
    }
  }
  ~KernelScope() {
    if (on) {
      cudaEventRecord(rec.b, ctx->stream);
      ctx->pending.push_back(rec);
      if (ctx->pending.size() > 4096) prof_resolve(ctx);
    }
  }
};

struct llf_mesh {
  int dim = 0, family = 0, order = 0, npe = 0;
  int64_t non = 0, nel = 0;
  double *d_xyz = nullptr;      // 3*non
  int32_t *d_conn = nullptr;    // npe*nel, 0-based node index
  int32_t *d_emat = nullptr;    // nel material index, -1 = skip (nullptr: all 0)
  // tables
  int nip = 0;
  double *d_w = nullptr;        // nip
  double *d_N = nullptr;        // nip*npe
  double *d_dN = nullptr;       // nip*npe*3
  double *d_dNn = nullptr;      // npe*npe*3 gradients at the element nodes
  std::vector<double> h_w, h_N, h_dN;  // host copies (FP32 tables derive from these)
  float *d_wf = nullptr, *d_Nf = nullptr, *d_dNf = nullptr;
  int tables_version = 0;
  int conn_version = 0;           // bumped when llf_mesh_update changes the connectivity
  int geo_version = 0;            // bumped by every coordinate, connectivity or material upload
  // affine geometry of the elements (assemble.cu), kept for the geometry
  // version and tables it was computed from: per element the flag and
  // J^-1, det (k_affine_geometry), and whether every element in use is affine
  uint8_t *d_aflag = nullptr;
  double *d_ageo = nullptr;
  int geo_cached = -1, geo_cached_tables = -1;
  bool geo_all_affine = false;
  // affine-element tables (built-in rules, whose node coordinates are known;
  // null after llf_tables_upload): reference node coordinates [npe*3] and,
  // per upper-triangle node pair (a <= b, a-major), R_ab [9] and Mref_ab
  double *d_nref = nullptr, *d_Rp = nullptr, *d_Mp = nullptr;
  float *d_Rpf = nullptr, *d_Mpf = nullptr;  // the same tables rounded to FP32
};

struct llf_pattern {
  llf_mesh *mesh = nullptr;
  int pdim = 0;
  int64_t ndof = 0;       // pdim*non
  int64_t nnzb = 0;       // node-level blocks
  int64_t nnz = 0;        // structural DoF-level nnz = pdim^2 * nnzb
  // node->element adjacency (elements with material >= 0), sorted by element
  int64_t *d_n2e_ptr = nullptr;   // non+1
  int2 *d_n2e = nullptr;          // (element, local index)
  int max_n2e = 0;
  // node-level CSC
  int64_t *d_nptr = nullptr;      // non+1
  int32_t *d_nadj = nullptr;      // nnzb (0-based node index, sorted per column)
  int32_t *d_diagpos = nullptr;   // non: position of the node itself in its column
  int max_deg = 0;                // largest number of row nodes of a column node
  // DoF-level colptr (0-based)
  int64_t *d_colptr = nullptr;    // ndof+1
  // element-to-column map: for column node B, element k of its list and local
  // node a, the position of node conn[e][a] in B's row-node list,
  // d_pos[(n2e_ptr[B] + k) * npe + a] (0xffff: not in the pattern)
  uint16_t *d_pos = nullptr;
  // bit 15 of a d_pos entry marks the first block of its row position in the
  // column's element order (assemble.cu, set by the first gather)
  bool pos_first = false;
  int conn_version = 0;           // mesh connectivity the pattern was built from
  void *ic_coloring = nullptr;    // node colouring of the IC(0) preconditioner (ic0.cu), on first use
  // the gather's column nodes in two degree classes (assemble.cu, on first
  // use): d_gather_nodes holds the nodes of degree <= gather_md_low, then
  // the others; each class runs with a buffer sized for its own degrees
  int32_t *d_gather_nodes = nullptr;
  int64_t gather_n_low = 0;
  int gather_md_low = 0;
  bool gather_split_done = false;
  // launch schedule of this pattern's assemblies (autotune.cu picks it;
  // every choice gives the same bits): element kernels' CTAs per SM
  // (0: as many as fit), the gather's degree-class threshold in percent of
  // the largest degree (0: one class) and its warps per CTA
  struct Tune {
    int elem_cap = 0;
    int gather_thr = 70;
    int gather_wpb = 4;
    bool from_tuner = false;
  } tune;
  // per column slab of the to-host assembly: one past the largest element
  // index that a node of this or an earlier slab touches (assemble.cu)
  std::vector<int64_t> slab_elem_end;
  // keep bits of the last values-only assembly on this pattern (assemble.cu):
  // the next one reports whether its bits differ
  unsigned *d_keep_prev = nullptr;
  // stored layouts of recent assemblies on this pattern (assemble.cu), one
  // per operator and arithmetic form: the 0-based start of every stored
  // (dropzeros'ed) column.  The next assembly of the same operator and form
  // writes its stored CSC straight from the gather into this layout and
  // checks every column's count; a column whose count differs sends the
  // assembly through the counting compaction instead.
  struct StoredLayout {
    int kind = -1, form = -1;
    int64_t total = 0;
    int64_t *d_ptr0 = nullptr;   // ndof + 1
    uint64_t used = 0;
  };
  StoredLayout layouts[4];
  uint64_t layout_clock = 0;
};

// The stored layout an assembly's gather writes into (assemble.cu).  When
// a column's count differs, the gather is run again the usual way: the
// structural values go to *nz_slot (allocated then) and the column counts
// to cnt_fallback, and fell_back is set.
struct StoredSpec {
  const int64_t *ptr0 = nullptr;   // 0-based stored column starts, ndof + 1
  int64_t *rowval_s = nullptr;     // 1-based rows, total entries
  double *nzval_s = nullptr;
  unsigned *mismatch = nullptr;    // device: set when a column's stored count differs
  double **nz_slot = nullptr;
  int64_t *cnt_fallback = nullptr;
  bool fell_back = false;
};

struct llf_matrix {
  llf_pattern *pat = nullptr;
  // structural values (pattern->nnz).  An assembly that wrote its stored
  // CSC straight into a kept layout leaves them to matrix_ensure_nz, which
  // expands them from the stored CSC on the first use that needs them.
  double *d_nz = nullptr;
  bool diagonal_only = false;     // lumped mass: values live on the diagonal
  bool keep_pattern = false;      // stored form keeps every structural entry (no dropzeros!)
  double *d_diag = nullptr;       // ndof (diagonal_only)
  // stored (dropzeros'ed) form, SparseMatrixCSC arrays, 1-based
  int64_t nnz_s = 0;
  int64_t *d_colptr_s = nullptr;  // ndof+1
  int64_t *d_rowval_s = nullptr;  // nnz_s
  double *d_nzval_s = nullptr;    // nnz_s
};

// ---------------------------------------------------------------- helpers
#define LLF_CUDA_TRY(ctx, expr)                                            \
  do {                                                                     \
    cudaError_t _e = (expr);                                               \
    if (_e != cudaSuccess) {                                               \
      return llf_fail((ctx), LLF_ERR_CUDA,                                 \
                      std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    }                                                                      \
  } while (0)

int llf_fail(llf_ctx *ctx, int code, const std::string &msg);
int llf_ok(llf_ctx *ctx);

// Read and clear the device status word (synchronises the stream).
int llf_check_status(llf_ctx *ctx, const char *what);

template <class T>
cudaError_t dalloc(llf_ctx *ctx, T **p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  ctx->allocs++;
  return cudaMallocAsync((void **)p, count * sizeof(T), ctx->stream);
}
template <class T>
void dfree(llf_ctx *ctx, T *&p) {
  if (p) cudaFreeAsync((void *)p, ctx->stream);
  p = nullptr;
}

// ---------------------------------------------------------------- kernels
// scan.cu
cudaError_t exclusive_scan_i64(llf_ctx *ctx, const int64_t *in, int64_t *out,
                               int64_t n, int64_t *total_host);

cudaError_t exclusive_scan_i64_dev(llf_ctx *ctx, const int64_t *in, int64_t *out, int64_t n, int64_t *d_total);

// pattern.cu
int pattern_build_impl(llf_ctx *ctx, llf_mesh *mesh, int pdim, llf_pattern *pat);
int mesh_convert_conn(llf_ctx *ctx, llf_mesh *mesh, const int64_t *d_conn64);
// Replace the connectivity by d_conn64 (1-based); *changed tells whether any
// entry differs from the current one.
int mesh_update_conn(llf_ctx *ctx, llf_mesh *mesh, const int64_t *d_conn64, bool *changed);
int check_finite(llf_ctx *ctx, const double *d, int64_t n);
// node -> (element, local index) lists sorted by element (elements with emat < 0 skipped)
int build_n2e(llf_ctx *ctx, const int32_t *conn, const int32_t *emat, int64_t nel, int npe,
              int64_t non, int64_t **ptr, int2 **list, int *max_len);

// assemble.cu
// Receives the complete element matrices of an assembly in place of the
// whole-pattern gather (FP64 or FP32 element matrices, cs values per column).
// elems(e0, e1) launches the element kernel on elements [e0, e1); the sink
// calls it so that each element range is ready before the slabs that use it.
using ElemLauncher = std::function<int(int64_t, int64_t)>;
struct GatherSink {
  virtual int gather(llf_ctx *ctx, llf_pattern *pat, const double *Kf, int64_t cs, bool blockval,
                     const ElemLauncher &elems) = 0;
  virtual int gather(llf_ctx *ctx, llf_pattern *pat, const float *Kf, int64_t cs, bool blockval,
                     const ElemLauncher &elems) = 0;
  virtual ~GatherSink() {}
};
// init (device, structural values of the pattern, or null): the assembly adds
// into these values instead of starting from zero (the DSL's csc_matrix).
// sink (or null): takes the element matrices; m is then neither gathered
// nor finalised.
int assemble_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int kind,
                  int ptype, const double *c1, const double *c2, int nmat,
                  int form, int lumped, llf_matrix *m, const double *init = nullptr,
                  GatherSink *sink = nullptr);
// stiffness straight to host CSC arrays, column slabs copied out while the
// next slab is gathered and compacted (assemble.cu)
int assemble_to_host_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int kind, const double *c1,
                          const double *c2, int nmat, int form, int64_t capacity, int64_t *colptr,
                          int64_t *rowval, double *nzval, int64_t *nnz, unsigned *keep = nullptr,
                          int *keep_changed = nullptr);
// autotune.cu: the tuned schedule for a pattern's shape, if one is known
// (in this process, or in the file LLF_TUNE_FILE names); applied at the
// pattern's first assembly
void tune_lookup(llf_pattern *pat, int kind, int form);
void tune_reset_split(llf_ctx *ctx, llf_pattern *pat);
int autotune_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int kind, int ptype, const double *c1,
                  const double *c2, int nmat, int form, int trials, std::string *report);
// dropzeros -> stored form; counts (non-zeros per DoF column) may come from
// the gather, else they are counted here
int matrix_finalize(llf_ctx *ctx, llf_matrix *m, int64_t *counts, int64_t **ptr0_out = nullptr);
// frees the pattern's stored layouts (assemble.cu)
void pattern_free_layouts(llf_ctx *ctx, llf_pattern *pat);
// The structural values of m, expanded from its stored CSC if the assembly
// left them out (assemble.cu): the stored entries at their structural
// positions, +0.0 at the others.  Allocates; a no-op when they exist.
int matrix_ensure_nz(llf_ctx *ctx, const llf_matrix *m);
// assemble_fp32.cu: precision form (FP32 quadrature, FP64 accumulation) into nz
// aflag/ageo: per-element affine flag and invJ/det (null: quadrature form
// only); all_affine: every element in use is affine, so the quadrature
// kernel is not launched
int assemble_fp32_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int kind,
                       const double *d_c1, const double *d_c2, const uint8_t *aflag,
                       const double *ageo, double *nz, int64_t *cnt, const double *init = nullptr,
                       GatherSink *sink = nullptr, StoredSpec *spec = nullptr, bool all_affine = false);
// Element-ordered column-node gather of whole element matrices laid out as
// Kf[element][column node][row node][block] (blockval: pdim x pdim blocks,
// entry (i,j) at i*pdim+j; otherwise one scalar per node pair placed on the
// component diagonal).  Column (e, b) starts at Kf + (e*npe + b)*colstride
// (colstride >= npe*block size, in elements).  Writes the structural values
// and, if cnt != NULL, the non-zero count of every DoF column.
// With spec, the gather writes the stored CSC into spec's layout instead
// (and no structural values), checking every column's count against it; see
// StoredSpec for a count that differs.
int gather_full(llf_ctx *ctx, llf_pattern *pat, const double *Kf, int64_t colstride, bool blockval,
                double *nz, int64_t *cnt, const double *init = nullptr, StoredSpec *spec = nullptr);
int gather_full32(llf_ctx *ctx, llf_pattern *pat, const float *Kf, int64_t colstride, bool blockval,
                  double *nz, int64_t *cnt, const double *init = nullptr, StoredSpec *spec = nullptr);
// The same gather for another element set on the pattern's nodes (e.g.
// boundary faces): its node -> element lists, element-to-column map and npe.
int gather_full_ext(llf_ctx *ctx, llf_pattern *pat, const int64_t *n2e_ptr, const int2 *n2e, const uint16_t *pos,
                    int npe, const double *Kf, int64_t colstride, bool blockval, double *nz, int64_t *cnt);
// Element-to-column map of an element set (conn, npe, node lists) into the
// pattern's node CSC; *pos allocated (n2e_total * npe entries).
int row_positions(llf_ctx *ctx, const llf_pattern *pat, const int32_t *conn, int npe, const int64_t *n2e_ptr,
                  const int2 *n2e, int64_t n2e_total, uint16_t **pos);
// elasticSupportMatrix / heatConvectionMatrix on the volume pattern (field.cu)
int support_impl(llf_ctx *ctx, llf_pattern *pat, llf_mesh *bmesh, const double *d_ke, const double *d_ken,
                 double thickness, llf_matrix *m);
// Element-matrix block stride (values per node block): an FP32 3x3 block is
// padded to 12 floats so that it is three 16-byte stores and loads.
__host__ __device__ constexpr int kf_bstride(int P, bool blockval, int tsize) {
  return !blockval ? 1 : (tsize == 4 && P == 3 ? 12 : P * P);
}
// Element-matrix column stride (elements of `tsize` bytes) padded to 16 bytes,
// so that every column can be fetched by one bulk copy.
inline int64_t kf_colstride(int npe, int bs, int tsize) {
  const int64_t bytes = ((int64_t)npe * bs * tsize + 15) / 16 * 16;
  return bytes / tsize;
}
// field.cu: f[node*pdim+i] += fe[e][a][i] of every element of the node, in element order.
int node_gather(llf_ctx *ctx, const int32_t *conn, int64_t nel, int npe, int64_t non, int pdim,
                const double *fe, double *f);
int matrix_axpby_impl(llf_ctx *ctx, double a, const llf_matrix *A, double b,
                      const llf_matrix *B, llf_matrix *C);

// solve.cu
int spmv_impl(llf_ctx *ctx, const llf_matrix *m, const double *d_x, double *d_y);
int pcg_impl(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
             const uint8_t *d_fixed, int precond, double reltol,
             int64_t maxiter, int64_t *iters, double *relres);
int pcg_noalloc_impl(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
                     const uint8_t *d_fixed, int precond, double reltol, int64_t maxiter,
                     int64_t *iters, double *relres);
int heat_fdm_impl(llf_ctx *ctx, const llf_matrix *K, const llf_matrix *C, const double *d_q, int nq, double *d_T,
                  const uint8_t *d_fixed, int64_t nsteps, double dt, double theta, int precond, double reltol,
                  int64_t maxiter, int64_t *iters_total);
// mixed: FP32 iterations with FP64 reliable updates (solve.cu, pcg_mixed_core)
int pcg_batched_impl(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
                     const uint8_t *d_fixed, int nseg, const int64_t *seg_off, int precond,
                     double reltol, int64_t maxiter, int64_t *iters, double *relres, bool mixed = false);

// ic0.cu: multicolour node-block IC(0)
struct Ic0Factor {
  int ncolors = 0;
  std::vector<int64_t> color_ptr;   // host: colour c = nodes [color_ptr[c], color_ptr[c+1]) of d_nodes
  const int16_t *d_color = nullptr; // per node (owned by the pattern)
  const int32_t *d_nodes = nullptr; // nodes sorted by colour (owned by the pattern)
  // during the factorisation, in FP64 or (fp32) FP32:
  void *Lrow = nullptr;             // L_jk with node j's list  (nnzb * P * P)
  void *Lcol = nullptr;             // L_jk with node k's list  (nnzb * P * P)
  void *Ldinv = nullptr;            // L_jj^-1 per node          (non * P * P)
  bool fp32 = false;
  double shift = 0.0;               // diagonal shift the factorisation needed
  // FP32 factor for the solves, indexed by a node's position t in d_nodes
  // (colour order): the earlier neighbours fk[fptr[t]..] with blocks Lf
  // (L_jk), the later neighbours bk[bptr[t]..] with blocks Lb (L_kj),
  // L_jj^-1 (Ldf) and the node's system (segc); the index arrays belong to
  // the pattern's colouring
  const int64_t *fptr = nullptr, *bptr = nullptr;
  const int32_t *fk = nullptr, *bk = nullptr;
  float *Lf = nullptr, *Lb = nullptr, *Ldf = nullptr;
  int32_t *segc = nullptr;
};
// seg_nodes: first node of each independent system (+ node count), d_node_seg:
// system of every node; a system's colouring and factor do not depend on the
// others, so a batched system preconditions exactly as it would alone.
int ic0_factor(llf_ctx *ctx, const llf_matrix *m, const uint8_t *d_fixed, const std::vector<int64_t> &seg_nodes,
               const int32_t *d_node_seg, Ic0Factor *f);
void ic0_release(llf_ctx *ctx, Ic0Factor *f);
void ic0_coloring_free(llf_ctx *ctx, llf_pattern *pat);

// tl.cu
int tl_material_tangent_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat,
                             const double *d_F, int law, const double *params,
                             int nparams, llf_matrix *m);
int tl_tangent_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, const double *d_F, int law,
                    const double *params, int nparams, llf_matrix *m);
int tl_tangent_tc_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, const double *d_F, int law,
                       const double *params, int nparams, llf_matrix *m);
int tl_initial_stress_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat,
                           const double *d_S, const double *d_C, int law,
                           const double *params, int nparams, llf_matrix *m);
int tl_internal_force_impl(llf_ctx *ctx, llf_mesh *mesh, const double *d_P,
                           const double *d_F, int law, const double *params,
                           int nparams, double *d_f);
int grad_elementwise_impl(llf_ctx *ctx, llf_mesh *mesh, const double *d_u,
                          int add_identity, double *d_out);
int load_vector_impl(llf_ctx *ctx, llf_mesh *bmesh, int problem_dim, int pdim,
                     const double *t_const, const double *d_tn,
                     double thickness, const double *d_Fn, double *d_f, int64_t ndof);
// externalTangentFollower on the volume pattern (field.cu)
int follower_tangent_impl(llf_ctx *ctx, llf_pattern *pat, llf_mesh *bmesh, const double *d_Fn,
                          const double *d_te, const double *d_ten, llf_matrix *m);
// elementsToNodes of ncomp values per element node (field.cu)
int elements_to_nodes_impl(llf_ctx *ctx, llf_mesh *mesh, int ncomp, const double *d_ev, double *d_nv);

// kinds of element operators
enum { KIND_ELASTIC = 0, KIND_HEAT = 1, KIND_MASS = 2, KIND_TLMAT = 3, KIND_TLGEO = 4 };

inline int ptype_dim(int ptype) {
  return (ptype == LLF_SOLID || ptype == LLF_HEAT_CONDUCTION) ? 3 : 2;
}
