// evr_internal.h -- shared declarations of the GB300 H.psi library (host tables,
// device context, kernel launchers).  Not part of the public ABI (include/evr_gpu.h).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/evr_gpu.h"

namespace evr {

constexpr int kMaxD = 24;      // modes (positions of a term and modes of a problem)
// G(Q) table: point-major, the D(D+1)/2 symmetric entries of a point padded to a multiple
// of four (16-byte rows in FP32, 32-byte in FP64) so that a point's row loads as vectors
__host__ __device__ constexpr int g_table_stride(int D) { return (D * (D + 1) / 2 + 3) & ~3; }
constexpr int kMaxN1 = 24;     // largest 1-D nq (and nb)
constexpr int kMaxNb0 = 4;     // electronic states
// default size (grid points x vectors of an item) below which a term runs in the general
// kernel instead of the slab kernel (evr_autotune re-chooses it)
constexpr int kSmallTermPoints = 2048;
// weighted reduction: rows of at most this many entries are summed by one thread per
// (row, vector), longer ones (the low basis functions, shared by many terms) by a CTA
constexpr int kCsrShortRow = 64;

// ---------------------------------------------------------------------------
// Host-side tables (built once by evr_setup.cpp)
// ---------------------------------------------------------------------------
struct Basis1D {
  int nb = 0, nq = 0;
  std::vector<double> x, w;           // scaled grid, weights (wrho)
  std::vector<double> d0b, d1b, d2b;  // nq x nb column-major
  std::vector<double> bgw;            // nb x nq = d0b^T diag(w)
  std::vector<double> d1gg, d2gg;     // nq x nq
};

// Per-term description used by the device kernels.  Offsets are in elements.
// The modes of a term are stored in a permuted order (perm[p] = reference mode of
// position p) that puts the mode with the most grid points last: the slab kernel walks
// the term grid one slab (fixed last-mode point) at a time.  Term-local basis and grid
// indices on the device (map, CSR, V and G grids) follow the permuted order, first
// position fastest.
struct TermDesc {
  int64_t off_nb;        // offset of the term in the term-basis space (sum_nb order)
  int64_t off_nq;        // offset of the term grid
  int32_t NB, NQ;        // prod nb_i, prod nq_i
  int32_t nb[kMaxD];
  int32_t nq[kMaxD];
  int32_t perm[kMaxD];
  int32_t m_d0b[kMaxD];  // offsets of the 1-D matrices in the flat matrix pool
  int32_t m_bgw[kMaxD];
  int32_t m_d1[kMaxD];
  int32_t m_d2[kMaxD];
  int32_t m_x[kMaxD];
  // last-position (slab) mode: d1.d0b, d2.d0b (grid <- basis) and bgw.d1, bgw.d2
  // (basis <- grid), padded like the others
  int32_t m_x1L, m_x2L, m_e1L, m_e2L;
  int32_t msz;           // elements of the term's 1-D matrices staged in shared memory
  int32_t D;             // positions of the term (its modes minus the dropped 1-point ones)
  int32_t g0off, goff;   // offsets of the problem's G0 (Dp*Dp) and g (Dp^3) in the coefficient arrays
  int32_t Dp;            // modes of the term's problem (strides of G0, g; G-table slots per point)
  double weight;         // Smolyak weight times the factors of the dropped 1-point modes
  double vshift;         // constant added to V_aa: second derivatives of dropped modes (type 1)
};

// elements of one staged matrix block: rows padded to 4, times the columns
__host__ __device__ inline int mat_block(int rows, int cols) { return ((rows + 3) & ~3) * cols; }
// shared-memory elements of a term's matrices (d0b, bgw, d1, d2 per position, and the
// last position's d1.d0b, bgw.d1, bgw.d2), in the order the kernels stage them
__host__ __device__ inline int term_matrix_elems(const TermDesc& T, int D) {
  int s = 0;
  for (int p = 0; p < D; ++p)
    s += mat_block(T.nq[p], T.nb[p]) + mat_block(T.nb[p], T.nq[p]) + 2 * mat_block(T.nq[p], T.nq[p]);
  const int L = D - 1;
  s += mat_block(T.nq[L], T.nb[L]) + 2 * mat_block(T.nb[L], T.nq[L]);
  return s;
}

// One unit of work of the H.psi kernel: one term, a tile of vectors.
struct WorkItem {
  int32_t term;
  int32_t v0;
  int32_t vt;            // vectors in the tile
  int32_t smem;          // general kernel: 1 buffers in shared memory, 0 in the CTA's global buffer;
                         // slab kernel: 1 partially transformed tensor in the CTA's global buffer,
                         // 2 in shared memory too, 3 W and the ping-pong tensors in global,
                         // 4 as 3 plus the staged term grid (FP32 type 10)
};

struct HostProblem {
  int kind = 0, D = 0, nb0 = 1, LG = 0, LB = 0, keo_type = 10;
  bool symmetric = true;                  // every 1-D basis has nq == nb (operator symmetric)
  std::vector<std::vector<Basis1D>> bas;  // [mode][level]
  std::vector<std::vector<int>> ltab;     // l(n), 1-based n
  std::vector<int> term_l;                // n_terms x D
  std::vector<double> weight;
  std::vector<TermDesc> terms;
  std::vector<TermDesc> termsT;           // same terms, matrix offsets of the transposed operator
  int64_t Np = 0, sum_nb = 0, sum_nq = 0, max_nq = 0, max_nb = 0;
  std::vector<int> packed;                // Np x D
  std::vector<int> map;                   // sum_nb (packed index or -1), reference term-local order
  std::vector<int> map_perm;              // same, term-local order of the permuted modes (device)
  std::vector<int64_t> grid_perm;         // device grid point -> reference grid point (sum_nq)
  std::vector<double> mat_pool;           // all 1-D matrices
  // CSR of the transposed map over N = Np*nb0 rows: sources in the term-basis
  // output buffer (off_nb*nb0 + a*NB + iB) and their Smolyak weight
  std::vector<int64_t> csr_ptr;
  std::vector<int64_t> csr_src;
  std::vector<double> csr_w;
  // operator
  std::vector<double> mono_coef;
  std::vector<int> mono_idx, mono_elec;
  std::vector<double> G0, g;              // D*D, D*D*D
  std::vector<double> e0diag;             // zero-order diagonal (preconditioner), N
  double flop_per_hpsi = 0.0;
};

// Builds every host table from the public description; returns EVR_OK or an error
// with a message in `err`.
int build_host_problem(const evr_problem_desc* d, HostProblem& P, std::string& err);

// Device copy of the problem and the buffers of the H.psi pipeline.
struct DeviceProblem {
  TermDesc* terms = nullptr;
  TermDesc* termsT = nullptr;
  double* mats = nullptr;
  float* mats32 = nullptr;
  double* vgrid = nullptr;          // sum_nq * nb0^2
  float* vgrid32 = nullptr;
  int* map = nullptr;               // sum_nb
  int64_t* csr_ptr = nullptr;
  int64_t* csr_src = nullptr;
  double* csr_w = nullptr;
  int64_t* csr_long = nullptr;      // rows with more than kCsrShortRow entries
  int64_t n_long = 0;
  double* G0 = nullptr;
  double* g = nullptr;
  float* G0_32 = nullptr;           // FP32 copies of G0 and g (FP32 H.psi)
  float* g32 = nullptr;
  double* mono_coef = nullptr;
  int* mono_idx = nullptr;
  int* mono_elec = nullptr;
  double* e0diag = nullptr;
};

// Work decomposition of one (nvec, precision) pair.
struct ItemSet {
  int nvec = 0, prec = 0;
  WorkItem* items = nullptr;       // general kernel
  int n_items = 0;
  WorkItem* items_slab = nullptr;  // slab kernel
  int n_slab = 0;
  WorkItem* items_small = nullptr;  // general kernel as small CTAs (small terms)
  int n_small = 0;
  std::vector<WorkItem> h_items, h_slab, h_small;  // host copies (filtered launches of batches)
};

struct Workspace {
  std::vector<ItemSet> sets;        // cached decompositions
  int* counter = nullptr;
  void* slab = nullptr;             // per-CTA global scratch
  size_t slab_per_cta_bytes = 0;
  int cap = 0;                      // vector capacity of ht/ht2/xin/xout
  void* ht = nullptr;               // term-basis output (sum_nb*nb0 x cap)
  void* ht2 = nullptr;              // second output for the symmetrised operator
  double* xin = nullptr;            // interleaved copies (layout conversions)
  double* xout = nullptr;
  int grid = 0, smem_bytes = 0;             // general kernel
  int grid_small = 0, smem_small_bytes = 0; // general kernel as small CTAs
  // slab kernel, per precision (index EVR_PREC_FP64 / EVR_PREC_FP32): grid, dynamic shared
  // memory and global tensor per CTA
  int grid_slab[2] = {0, 0}, smem_slab_bytes[2] = {0, 0};
  size_t slab_slab_bytes[2] = {0, 0};
  WorkItem* f_items = nullptr;              // filtered item lists (terms of active problems)
  WorkItem* f_slab = nullptr;
  WorkItem* f_small = nullptr;
  size_t f_cap = 0;
};

// operator forms
enum OpForm { OP_H = 0, OP_HT = 1, OP_HSYM = 2 };

// Grid operator of one H.psi call: potential vw*V(Q) + mw*mu(Q) (mu: the dipole table of
// evr_set_dipole; mw = -E for a field E) and the kinetic part when keo != 0.  The default
// is the plain H.  mu_dev, when set, is a device scalar read in place of mw (a field
// value that changes between replays of a captured launch sequence).
struct OpExtras {
  double vw = 1.0, mw = 0.0;
  int keo = 1;
  const double* mu_dev = nullptr;
};

// Stage buffers of the grid-wide single-term path (evr_stages.cu).
struct StageBuffers {
  void* buf = nullptr;
  size_t elems = 0;   // elements per buffer (FP64), Smax * nb0 * kMaxBlock
  int64_t smax = 0;   // largest intermediate tensor of one vector and state
};

}  // namespace evr

struct evr_ctx {
  int device = 0;
  bool host_only = false;           // created with device < 0: tables only
  int op_form = 0;                  // EVR_OP_H, EVR_OP_HT or EVR_OP_HSYM
  bool capturing = false;           // inside a stream capture: no event records
  bool use_slab = true;             // slab kernel for the terms that fit (evr_set_kernel_path)
  bool slab_all = false;            // path 2: small terms too (no small-term routing)
  bool use_tc = false;              // FP32 slab-kernel contractions on the tensor cores (evr_set_tensor_cores;
                                    // off by default: slower than the CUDA cores at these sizes, see evr_autotune)
  int tc_min_km = 64;               // contractions with K*M below this stay on the CUDA cores
  bool use_stages = true;           // grid-wide stage path for single-term problems
  bool gfly = false;                // G(Q) from the linear model per point instead of a table
  int vt_cap_slab = 32, vt_cap_items = 32;  // widest vector tile of an item (evr_autotune)
  // terms with fewer grid points x vectors run in the general kernel, as small CTAs when
  // their buffers fit one
  int slab_min_points = evr::kSmallTermPoints;
  int64_t ws_gen = 0;               // bumped whenever workspace buffers are freed (captured graphs)
  std::vector<unsigned char> term_active;  // batches: terms to run (empty = all)
  int n_sys = 1;                    // problems stacked in this context (evr_create_batch)
  cudaStream_t stream = nullptr;
  evr::HostProblem hp;
  evr::DeviceProblem dp;
  evr::Workspace ws;
  int num_sms = 0;
  std::string err;
  int64_t last_kernels = 0, last_items = 0;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // around the items kernel and the reduction
  double* dp_ggrid = nullptr;      // symmetric G(Q) on the grid (type 10 with g != 0)
  float* dp_ggrid32 = nullptr;
  double* dp_jgrid = nullptr;      // (Jac, sqrt(rho/Jac)) per grid point (evr_set_jacobian), or none
  float* dp_jgrid32 = nullptr;
  double* dp_mugrid = nullptr;     // dipole mu(Q) on the grid (sum_nq * nb0^2), evr_set_dipole
  float* dp_mugrid32 = nullptr;
  double mu_max = 0.0;             // max over grid points of the row-sum norm of mu
  evr::StageBuffers stg;
  evr::OpExtras field;             // grid-operator extras of evr_hpsi_* / Davidson / Chebyshev (evr_set_field)
  void* oc = nullptr;              // optimal-control state (evr_control.cu)
  void* batch = nullptr;           // stacked problems (evr_batch.cu)
  // host staging for the host-pointer entry points
  double* pinned = nullptr;
  size_t pinned_bytes = 0;
};

namespace evr {
// kernels (evr_kernels.cu)
int upload_problem(evr_ctx* c);
void free_problem(evr_ctx* c);
int ensure_workspace(evr_ctx* c, int nvec, int prec);
void free_workspace(evr_ctx* c);
// H.psi (op = OP_H), H^T.psi or (H+H^T)/2.psi on interleaved device blocks (ld >= nvec),
// nvec <= kMaxBlock per call; returns a status.
constexpr int kMaxBlock = 64;
int hpsi_interleaved(evr_ctx* c, const double* x, int64_t ldx, double* y, int64_t ldy, int nvec, int prec,
                     cudaStream_t s, int op = OP_H, const OpExtras* ex = nullptr);
// any nvec: splits into blocks of kMaxBlock vectors
// FP64 H.psi with caller-provided scratch (no allocation); see evr_hpsi_noalloc
int hpsi_scratch(evr_ctx* c, const double* x, int64_t ldx, double* y, int64_t ldy, int nvec, unsigned char* scratch,
                 size_t scratch_bytes, cudaStream_t s);
int hpsi_blocks(evr_ctx* c, const double* x, int64_t ldx, double* y, int64_t ldy, int nvec, int prec,
                cudaStream_t s, int op = OP_H, const OpExtras* ex = nullptr);
// grid-wide path for problems of one term (evr_stages.cu); nvec <= kMaxBlock
bool stages_apply(const evr_ctx* c);
int hpsi_stages(evr_ctx* c, const double* x, int64_t ldx, double* y, int64_t ldy, int nvec, int prec,
                cudaStream_t s, int op, const OpExtras& ex);
void free_stages(evr_ctx* c);
void free_control(evr_ctx* c);
void free_batch_info(evr_ctx* c);
// weighted CSR reduction of the term-basis output(s) into y (evr_kernels.cu)
int upload_long_rows(evr_ctx* c);
int upload_coeffs32(evr_ctx* c);
int reduce_terms(evr_ctx* c, int prec, const void* ht, const void* ht2, int nvec, double scale, double* y,
                 int64_t ldy, cudaStream_t s);
// evaluates monomials (device arrays) on every term grid into out (sum_nq * nb0^2) and
// returns the largest row-sum norm over the points in *maxnorm
int eval_grid_monomials(evr_ctx* c, int n_mono, const double* coef, const int* idx, const int* elec, double* out,
                        double* maxnorm);
// Chebyshev series of exp(-i r x) on [-1, 1]: c_0 = J_0(r), c_k = 2 J_k(r), k <= K, with K the
// first order after which every |c_k| < tol (evr_propagate.cu); returns false when too long
bool cheby_series(double r, double tol, std::vector<double>& coef);
int transpose_to_interleaved(const double* in, int64_t ld_in, double* out, int64_t ld_out, int64_t N, int nvec,
                             cudaStream_t s);
int transpose_from_interleaved(const double* in, int64_t ld_in, double* out, int64_t ld_out, int64_t N, int nvec,
                               cudaStream_t s);
int set_error(evr_ctx* c, int code, const std::string& msg);
// Grid values given in the reference's point order (layout EVR_VGRID_TERMS: term-major with
// (a,b) blocks per term; EVR_VGRID_REF: (iq, a, b) over the whole grid) -> the device's
// table order, FP64 and FP32; with_shift adds each term's constant of dropped 1-point
// modes on the diagonal (the V table holds it, the dipole table does not).
void grid_values_to_device(const HostProblem& P, const double* v, int layout, bool with_shift,
                           std::vector<double>& dev, std::vector<float>& dev32);
// reads (and clears) the flag the term kernels raise when an item would exceed its buffers
int check_item_bounds(evr_ctx* c);
void clear_item_sets(evr_ctx* c);
int cuda_check(evr_ctx* c, cudaError_t e, const char* what);
}  // namespace evr
