// gfe_internal.h -- shared definitions of libgfe (not part of the public ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/gfe.h"

#include <nvtx3/nvToolsExt.h>

namespace gfe {

// Makes ctx's device current for one ABI call and restores the caller's device after it.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// NVTX range over one ABI call (visible in nsys / ncu range filters; no cost without a tool)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// ---- errors -------------------------------------------------------------------------------
int set_error(int code, const char* fmt, ...);
void clear_error();
const char* g_last_error_ptr();

#define GFE_CUDA_TRY(expr)                                                                 \
  do {                                                                                     \
    cudaError_t e_ = (expr);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return ::gfe::set_error(e_ == cudaErrorMemoryAllocation ? GFE_ERR_OUT_OF_MEMORY      \
                                                              : GFE_ERR_CUDA,              \
                              "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_),      \
                              __FILE__, __LINE__);                                         \
  } while (0)

#define GFE_TRY(expr)            \
  do {                           \
    int s_ = (expr);             \
    if (s_ != GFE_OK) return s_; \
  } while (0)

// Device-side error word: kernels write the first failure code and an index.
struct DevError {
  int code;
  int pad;
  long long index;
};

// ---- device buffers -----------------------------------------------------------------------
// A growable device allocation. With an owner context it comes from the context's
// stream-ordered memory pool (cudaMallocAsync / cudaFreeAsync on the context's stream), so
// buffers created and released every step are recycled without device synchronisation.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  gfe_ctx* owner = nullptr;
  DevBuf() = default;
  explicit DevBuf(gfe_ctx* o) : owner(o) {}
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf();
  int reserve(size_t nbytes);  // keeps contents only if no growth is needed
  void release();
  template <class T>
  T* as() const { return static_cast<T*>(ptr); }
};

// ---- context ------------------------------------------------------------------------------
struct ScratchSlot;
struct FcgLoopCache;  // the flexible CG's device loop and multigrid hierarchy (gfe_solve.cu)
void fcg_cache_release(gfe_ctx* ctx);

}  // namespace gfe

namespace gfe {
// Optional per-kernel timing: CUDA events recorded on the context's stream around the
// launches of a kernel class, summed when the stream is next synchronised by the library.
struct KernelTimer {
  bool enabled = false;
  std::vector<cudaEvent_t> pool;
  std::vector<int> kinds;  // kind of each (begin, end) pair in use
  size_t used = 0;
  double total_ms[8] = {0};
  long long count[8] = {0};
};
}  // namespace gfe

struct gfe_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  // a second stream for host-to-device copies that overlap work on `stream` (created on first
  // use), with the events that order it against `stream`
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_fork = nullptr, copy_join = nullptr;
  cudaMemPool_t pool = nullptr;  // stream-ordered pool of this context's device buffers
  int num_sms = 0;
  long long launches = 0;
  gfe::DevError* d_err = nullptr;  // device error word
  // named scratch buffers reused across calls
  gfe::DevBuf scratch[18];
  // Dirichlet values (device) of the assembly call in progress; the row gathers of a
  // matrix-and-vector assembly add the lift b_i -= K_ij u_D_j when set
  const double* lift_uD = nullptr;
  int64_t lift_ndiri = 0;
  // pinned staging for small device->host reads
  void* h_pinned = nullptr;
  // the device error word copied into h_pinned + kStagedErrorOffset ahead of a wait, for the
  // check that follows it (stage_device_error)
  bool err_staged = false;
  gfe::KernelTimer timer;
  // CUDA graph of one chunk of CG iterations, reused while its launch parameters match
  cudaGraphExec_t cg_exec = nullptr;
  uint64_t cg_key = 0;
  // limit of the first wait of the bounded mbarrier waits in the lattice SpMV (ns); 0 makes
  // that wait give up at once (gfe_ctx_set_wait_limit, for tests of the timeout path)
  unsigned long long first_wait_ns = 1000000000ull;
  bool q2tab_valid = false;  // scratch[SCR_Q2TAB] holds the tensor-core Q2 E table
  // the flexible CG's device loop graph and its multigrid hierarchy, kept while the buffers
  // they were built on stay the same
  gfe::FcgLoopCache* fcg_cache = nullptr;
};

struct gfe_matrix {
  gfe_ctx* ctx = nullptr;
  int64_t nrows = 0, ncols = 0, nnz = 0;
  int32_t nd = 0;   // local rows per cell
  int32_t ndc = 0;  // local columns per cell (rectangular blocks); 0 means nd
  int64_t ncells = 0;
  int cols_per_cell() const { return ndc > 0 ? ndc : nd; }
  // optional local coupling mask (nd x cols_per_cell(), column-major, nonzero keeps): the
  // (local row, local column) pairs a multi-field weak form leaves untouched get no entry
  gfe::DevBuf lmask;
  bool has_lmask = false;
  // CSR pattern and values (0-based, int32 indices)
  gfe::DevBuf rowptr, colval, val;
  // cell ids the pattern was built from (device copies)
  gfe::DevBuf cell_rows, cell_cols;
  // the column ids are the row ids (square cells given the same array): cell_cols stays empty
  bool cols_alias = false;
  // values not yet zeroed (the closed-form Cartesian pattern defers it: the class-sum
  // assembly writes every entry); ensure_values zeroes them before any other use
  bool val_pending = false;
  // the values are the class-sum kernel's on cubic cells, unchanged since: the entries of
  // the face classes (neighbours along one axis) are exact zeros, which the FP64 lattice
  // residual skips
  bool zf_values = false;
  const int32_t* col_ids() const {
    return cols_alias ? cell_rows.as<int32_t>() : cell_cols.as<int32_t>();
  }
  // row -> (cell*nd + local row) references, sorted by cell: the row-gather assembly lists
  gfe::DevBuf ref_ptr, refs;
  // position of every (reference, local column) in its row's column list, cols_per_cell()
  // entries per reference (uint8 when every row has <= 255 entries, else uint16); 0xff /
  // 0xffff marks a skipped (negative) id
  gfe::DevBuf refpos;
  int pos_bytes = 1;
  int max_width = 0;
  int64_t nrefs = 0;
  // solver plan (sliced ELL copy with 32-row slices), built lazily
  bool plan_valid = false;
  int64_t nslices = 0, sell_nnz = 0;
  gfe::DevBuf sell_ptr, sell_col, sell_val64, sell_val32, dinv64, dinv32;
  // diagonal (DIA) FP32 copy, built when all column offsets c - r fall in <= 32 values
  bool dia_checked = false, dia_valid = false;
  int dia_ndiag = 0;
  int32_t dia_off[32] = {0};
  gfe::DevBuf dia_val32;
  // matrix-free FP32 form of a uniform Cartesian Q1 diffusion matrix (3-D) whose rows are the
  // interior nodes in node order: per-cell kappa in FP32 plus the reference stiffness. The
  // fused assembly attaches it and checks the row numbering on the device (mf_flag); any
  // other change of the values drops it. 0 none, 1 numbering check pending, 2 valid.
  int mf_state = 0;
  int64_t mf_n[3] = {0, 0, 0};
  // the pattern is the closed form of a 3-D Cartesian Q1 grid of cart_n cells whose rows and
  // columns are the interior nodes in node order (set by the problem-aware symbolic loop
  // after its device check of the ids)
  bool cart_lattice = false;
  int64_t cart_n[3] = {0, 0, 0};
  // p-multigrid data of a 3-D Q2 matrix on a Cartesian grid (nodes possibly jittered) whose
  // vertex dofs are the interior vertices in node order (gfe_pmg.cu): the Q2 node lattice
  // -> free dof map and the coarse Q1 lattice operator (kappa in FP32, the reference
  // stiffness of the uniform grid). 0 none, 1 check pending, 2 valid.
  int pmg_state = 0;
  int64_t pmg_n[3] = {0, 0, 0};
  float pmg_K[64] = {0};
  gfe::DevBuf pmg_node, pmg_kap32, pmg_flag;
  // two-level data of a vector P2 elasticity matrix on a simplexified Cartesian box
  // (gfe_pmg.cu): the box and the Lame coefficients (2 per tet, or 2 constants) from which
  // the P1 coarse operator is assembled. 0 none, 2 attached.
  int p2mg_state = 0;
  int64_t p2mg_part[3] = {0, 0, 0};
  double p2mg_dom[6] = {0, 0, 0, 0, 0, 0};
  int p2mg_coef_kind = 0;
  gfe::DevBuf p2mg_lame;
  // ref_ptr / refs / refpos of the closed-form pattern not written yet (ensure_row_refs)
  bool refs_pending = false;
  // a pattern built by the general symbolic loop was checked once against the closed form
  // of a problem's grid (cartesian_ids_match): the same ids give the same pattern
  bool cart_checked = false;
  float mf_K[64] = {0};
  gfe::DevBuf mf_kap32, mf_flag;
};

namespace gfe {

// scratch slot ids in gfe_ctx::scratch
enum ScratchId {
  SCR_TMP0 = 0,
  SCR_TMP1,
  SCR_TMP2,
  SCR_TMP3,
  SCR_CELLIDS,
  SCR_COEF,
  SCR_SRC,
  SCR_CELLMAT,
  SCR_CELLVEC,
  SCR_COORDS,
  SCR_CELLNODES,
  SCR_VEC_B,
  SCR_VEC_X,
  SCR_SOLVER,
  SCR_SOLVER2,
  SCR_REDUCE,
  SCR_DIRI,
  SCR_Q2TAB,  // the tensor-core Q2 kernel's E table (built once per context)
  SCR_COUNT
};
static_assert(SCR_COUNT <= 18, "scratch slots");

// The class-sum numeric assembly of 3-D uniform Cartesian Q1 diffusion into the closed-form
// lattice pattern (gfe_assemble_lattice.cu); *done is false when the problem is not one it
// covers (the caller then runs the generic row gather).
int assemble_cartesian_q1_lattice(gfe_ctx* ctx, gfe_matrix* A, const gfe_problem* p,
                                  const double* d_coef, int src_kind, const double* d_src,
                                  const double* Kref, const double* mref, double* d_b,
                                  bool* done);

// p-multigrid for 3-D Q2 (gfe_pmg.cu): attached by the Q2 assembly, used by the flexible CG
// with GFE_PC_MG when the matrix has no Q1 lattice form.
int attach_q2_pmg(gfe_ctx* ctx, gfe_matrix* A, const gfe_problem* p, const double* d_coef);
struct Q2PMG;
// two-level P2 -> P1 preconditioner of vector P2 elasticity (gfe_pmg.cu)
int attach_p2_pmg(gfe_ctx* ctx, gfe_matrix* A, const gfe_problem* p, const double* d_coef);
struct P2PMG;
int p2mg_create(gfe_ctx* ctx, gfe_matrix* A, P2PMG** out);
int p2mg_apply(P2PMG* pm, const float* r, float* z, const int* done);
// one cycle launched on the context's stream without a graph of its own (direct, or inside a
// caller's capture)
int p2mg_record(P2PMG* pm, const float* r, float* z, const int* done);
void p2mg_destroy(P2PMG* pm);
int pmg_ready(gfe_ctx* ctx, gfe_matrix* A, bool* ok);
int pmg_create(gfe_ctx* ctx, gfe_matrix* A, Q2PMG** out);
int pmg_apply(Q2PMG* pmg, const float* r, float* z, const int* done);
int pmg_record(Q2PMG* pmg, const float* r, float* z, const int* done);
void pmg_destroy(Q2PMG* pmg);
// Whether A's cell ids are the interior-node numbering of an (n0, n1, n2) Cartesian Q1 grid
// with every boundary node Dirichlet (device check); the pattern is then the closed form.
int cartesian_ids_match(gfe_ctx* ctx, gfe_matrix* A, int64_t n0, int64_t n1, int64_t n2,
                        bool* ok);
// Writes the row references and positions of a closed-form Cartesian pattern if they are
// still pending (every row gather over a matrix calls it first).
int ensure_row_refs(gfe_ctx* ctx, gfe_matrix* A);

// pointer classification
bool is_device_ptr(const void* p);
// Returns a device view of `n` bytes at `p`: `p` itself if it is device memory, else an
// async H2D copy into scratch slot `slot`.
int device_view(gfe_ctx* ctx, const void* p, size_t n, int slot, const void** out);
// Copies n bytes from device memory `src` to `dst` (host or device) and waits if host.
int copy_out(gfe_ctx* ctx, void* dst, const void* src, size_t n);
// Reads and resets the device error word; returns its code (GFE_OK if none).
int check_device_error(gfe_ctx* ctx, const char* where);
// Issues the copy of the device error word into pinned staging, to be read after the caller's
// next wait by check_staged_error (no device work may come between the two).
constexpr size_t kStagedErrorOffset = 2048;
int stage_device_error(gfe_ctx* ctx);
// check_device_error from the staged copy, without a wait of its own (or with one when
// nothing was staged)
int check_staged_error(gfe_ctx* ctx, const char* where);
// zeroes A's values when their zeroing was deferred (val_pending)
int ensure_values(gfe_ctx* ctx, gfe_matrix* A);

inline unsigned grid_for(int64_t n, int block, int64_t cap = 1 << 30) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

// ---- kernel launch wrappers implemented in the .cu files ----------------------------------
// exclusive scan of n int64 counts (in) to out[0..n] (out[n] = total). in/out device.
int scan_exclusive_i64(gfe_ctx* ctx, const int64_t* in, int64_t* out, int64_t n);
int scan_exclusive_i32_to_i64(gfe_ctx* ctx, const int32_t* in, int64_t* out, int64_t n);
int narrow_i64_to_i32(gfe_ctx* ctx, const int64_t* in, int32_t* out, int64_t n);

// pattern (gfe_pattern.cu)
int build_refs(gfe_ctx* ctx, gfe_matrix* A);
int build_pattern(gfe_ctx* ctx, gfe_matrix* A);
// The pattern of Q1 cells of an n0 x n1 x n2 Cartesian grid numbered by interior nodes, in
// closed form after a device check of the ids; *done false (nothing changed) when the ids
// are not that numbering.
// host_ids: ids still in host memory (A->cell_rows reserved, not yet filled); they are copied
// into A->cell_rows on the context's copy stream while the closed-form row pointers and
// columns are built, or on the main stream when the closed form does not apply.
int build_pattern_cartesian(gfe_ctx* ctx, gfe_matrix* A, int64_t n0, int64_t n1, int64_t n2,
                            bool* done, const int32_t* host_ids = nullptr);

// assembly (gfe_assemble.cu)
int assemble_cellmats(gfe_ctx* ctx, gfe_matrix* A, const double* d_cellmats);
int assemble_cellvecs(gfe_ctx* ctx, int64_t ncells, int nd, const int32_t* d_rows,
                      const double* d_cellvecs, int64_t nrows, double* d_b);
int assemble_problem(gfe_ctx* ctx, const gfe_problem* p, gfe_matrix* A, double* d_b);

// tensor-core Q2 cell integrals (gfe_q2_tc.cu); tabs (device) and htabs (host) hold the same
// FP64 reference tables w | phi2 | dphi1 | B
int launch_q2_cells_tc(gfe_ctx* ctx, int64_t ncells, const int32_t* cell_vertices,
                       const double* coords, const double* tabs, const double* htabs,
                       int coef_kind, const double* coef, int src_kind, const double* src,
                       float* K, float* bvec);
// tensor-core P2 elasticity cells of affine tets (gfe_p2_tc.cu): K tile-major FP32
// (K[((cell/16)*900 + li + lj*30)*16 + cell%16], room for whole 16-cell tiles), b entry-major
// FP64 (b[li*ncells + cell]); hGref the host reference integrals
int launch_p2_cells_tc(gfe_ctx* ctx, int64_t ncells, const double* coords,
                       const int32_t* tet_vertices, int coef_kind, const double* coef,
                       const double* f, const double* mref, const double* hGref, float* K,
                       double* bvec);

// learned block preconditioner (gfe_learned.cu); `skip` (device int, may be null) makes the
// kernels return at once when non-zero
int learned_apply(gfe_ctx* ctx, gfe_learned_pc* pc, const float* d_r, float* d_z,
                  const int* skip = nullptr);
int64_t learned_ndofs(const gfe_learned_pc* pc);
// z = base + M(r) (base may be null), e.g. a learned smoothing step x + M(b - A x); `timed`
// false inside a captured V-cycle (the graph launch is timed as a whole)
int learned_apply_into(gfe_ctx* ctx, gfe_learned_pc* pc, const float* d_r, const float* base,
                       float* d_z, const int* skip, bool timed);
// (the solve's last wait brings the device error word along: check_staged_error follows)
int solve_fcg(gfe_ctx* ctx, gfe_matrix* A, gfe_learned_pc* pc, const gfe_solver_opts* o,
              const double* d_b, double* d_x, gfe_solve_report* rep);

// solver (gfe_solve.cu)
int build_solver_plan(gfe_ctx* ctx, gfe_matrix* A);
int build_dia(gfe_ctx* ctx, gfe_matrix* A);
int solve(gfe_ctx* ctx, gfe_matrix* A, const gfe_solver_opts* o, const double* d_b,
          double* d_x, gfe_solve_report* rep);
int spmv64(gfe_ctx* ctx, gfe_matrix* A, const double* d_x, double* d_y);

// kernel timing (gfe_host.cpp): begin/end bracket one launch of kernel class `kind`;
// flush folds finished pairs into the totals (call after a stream synchronisation).
void timer_begin(gfe_ctx* ctx, int kind);
void timer_end(gfe_ctx* ctx);
// drops the last n (begin, end) pairs (launches that turned out to be no-ops)
void timer_drop_last(gfe_ctx* ctx, int n);
int timer_flush(gfe_ctx* ctx);
void timer_release(gfe_ctx* ctx);

// host set-up (gfe_host.cpp)
int tensor_quadrature(int D, int degree, std::vector<double>& x, std::vector<double>& w);
void q1_unit_stiffness_classes(double W[8]);
void q1_shapes(int D, int nq, const double* qx, std::vector<double>& phi,
               std::vector<double>& dphi);
void q2_node_lattice(int D, int* idx);
void q2_shapes(int D, int nq, const double* qx, std::vector<double>& phi,
               std::vector<double>& dphi);
// geometric multigrid V-cycle on the lattice operator (gfe_mg.cu)
struct LatticeQ1Op;
struct LatticeMG;
int mg_create(gfe_ctx* ctx, const LatticeQ1Op& fine, LatticeMG** out);
// Re-forms the coarse kappa and D^-1 of a hierarchy from its fine kappa (same array and
// dimensions as at creation, new values)
int mg_refresh(LatticeMG* mg, const LatticeQ1Op& fine);
// A dot product of the V-cycle's result z that the cycle's last kernel reduces (the flexible
// CG's beta, v = q = A p and den = p.q): *out = -(z . v) / *den, 0 when *den is 0. partials
// holds one entry per block of the fine level's sweep (at most twice LatticeQ1Op::blocks).
struct MgDot {
  const float* v = nullptr;
  double* partials = nullptr;
  unsigned* ticket = nullptr;
  const double* den = nullptr;
  double* out = nullptr;
};
int mg_apply(LatticeMG* mg, const float* r, float* z, const int* done,
             const MgDot* dot = nullptr);
// Records one V-cycle (b = r, result in z) on the context's stream without capturing it (for
// a caller that captures a larger cycle around it).
int mg_record(LatticeMG* mg, const float* r, float* z, const int* done,
              const MgDot* dot = nullptr);
// Whether the cycle's last kernel forms an MgDot: not when the fine level runs inside the
// one-block coarse kernel or with the learned smoother.
bool mg_fuses_dot(const LatticeMG* mg);
// Makes the learned block preconditioner the fine level's smoother of the V-cycle (pre:
// x = M(b); post: x += M(b - A x)); the coarser levels keep damped Jacobi.
int mg_set_learned(LatticeMG* mg, gfe_learned_pc* pc);
void mg_destroy(LatticeMG* mg);
// Jacobi-preconditioned FP64 BiCGStab from x = 0 (gfe_bicgstab.cu)
int bicgstab(gfe_ctx* ctx, gfe_matrix* A, const double* dinv, const double* d_b, double* d_x,
             double rtol, int maxit, int* iterations);
// quasilinear diffusion residual + Jacobian (gfe_nonlinear.cu)
int assemble_quasilinear(gfe_ctx* ctx, const gfe_problem* p, gfe_matrix* A, double* d_b);
// simplexified boxes and P2 tets (gfe_simplex.cpp)
extern const int kHexTets[6][4];
extern const int kTetEdges[6][2];
int tet_quadrature(int degree, std::vector<double>& x, std::vector<double>& w);
void p2tet_shapes(int nq, const double* qx, double* phi, double* dphi);
int elasticity_p2_tables(const double* h, int degree, std::vector<double>& tab);
int p2tet_reference_integrals(int degree, std::vector<double>& G, std::vector<double>& m);
// matrix-free FP32 operator attached by the Cartesian Q1 assembly (gfe_solve.cu)
int attach_lattice_operator(gfe_ctx* ctx, gfe_matrix* A, const gfe_problem* p,
                            const double* d_coef, const double* Kref);
// P2 tet elasticity assembly (gfe_elasticity.cu)
int assemble_p2_elasticity(gfe_ctx* ctx, const gfe_problem* p, gfe_matrix* A, double* d_b);

}  // namespace gfe
