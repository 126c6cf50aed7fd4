// evr_batch.cu -- many independent problems in one context: stacked H.psi and a lock-step
// batched Davidson.
//
// evr_create_batch stacks n problems (any D and level, the same number of electronic
// states and KEO form) into one term table: the terms of problem s keep their own 1-D
// matrices, grids, G0 and g (at the offsets g0off/goff of each term), and their packed
// functions occupy rows offsets[s] .. offsets[s+1]-1 of a stacked vector.  H is then block
// diagonal, and one H.psi launch of the term kernels (one persistent item queue) applies
// H_s to the rows of every problem in every column at once.  G(Q) is evaluated per point
// from the linear model instead of a table (a table for 256 problems up to D=6, L=8 would
// take 160 GB).
//
// evr_batch_davidson runs sub_propagation_Davidson (sub_module_Davidson.f90:54-748, as in
// evr_davidson.cu) for every problem at once: all problems share the subspace size, so the
// per-problem projections and Ritz combinations are segmented products over row chunks
// of the stack (partial Grams summed per problem in a fixed order), the small projected
// eigenproblems are solved by a batched Jacobi kernel (one CTA per problem), and the H.psi
// of the new directions of all problems is one call.  Mixed precision: an FP32 phase as in
// evr_davidson, then the FP64 iteration continued from its Ritz vectors.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <numeric>
#include <vector>

#include "evr_internal.h"

using namespace evr;

namespace {

constexpr int kBT = 256;

// ---------------------------------------------------------------------------------------
// device kernels
// ---------------------------------------------------------------------------------------

// V table of the terms [t0, t1) from one problem's monomials (positions -> reference modes)
__global__ void batch_vgrid_kernel(const TermDesc* __restrict__ terms, int t0, int t1, const double* __restrict__ mats,
                                   int64_t q0, int64_t q1, int nb0, int n_mono, const double* __restrict__ coef,
                                   const int* __restrict__ midx, const int* __restrict__ melec,
                                   double* __restrict__ vgrid) {
  for (int64_t gq = q0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; gq < q1;
       gq += (int64_t)gridDim.x * blockDim.x) {
    int lo = t0, hi = t1 - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (terms[mid].off_nq <= gq) lo = mid; else hi = mid - 1;
    }
    const TermDesc& T = terms[lo];
    const int64_t q = gq - T.off_nq;
    const int NQ = T.NQ, D = T.D;
    double Q[kMaxD];  // dropped 1-point modes sit at Q = 0
    for (int d = 0; d < kMaxD; ++d) Q[d] = 0.0;
    int64_t r = q;
    for (int d = 0; d < D; ++d) {
      Q[T.perm[d]] = mats[T.m_x[d] + (int)(r % T.nq[d])];
      r /= T.nq[d];
    }
    double* V = vgrid + T.off_nq * nb0 * nb0;
    for (int ab = 0; ab < nb0 * nb0; ++ab) V[(int64_t)ab * NQ + q] = ab % (nb0 + 1) == 0 ? T.vshift : 0.0;
    for (int m = 0; m < n_mono; ++m) {
      double v = coef[m];
      for (int k = 0; k < 4; ++k) {
        const int i = midx[4 * m + k];
        if (i >= 0) v *= Q[i];
      }
      V[(int64_t)(melec[2 * m] + nb0 * melec[2 * m + 1]) * NQ + q] += v;
    }
  }
}

__global__ void batch_to_float(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// Eigen-decomposition of one symmetric n x n matrix per CTA (n <= 64) by cyclic Jacobi
// with the round-robin ordering: each round rotates n/2 disjoint pairs at once (angles
// from the matrix before the round, so the round is A <- R^T A R with R a product of
// commuting plane rotations).  A pair is rotated unless |a_pq| <= tol sqrt(|a_pp a_qq|)
// (relative to its own diagonal, so very large diagonal entries -- the flagged empty
// directions -- do not hide the others); at most max_sweeps sweeps, stopping after a
// sweep without rotations.  Eigenvalues ascending into W, eigenvectors as the columns of
// V (column-major, ld ldv).  The sweep flag is reset only after every thread has read it
// (a barrier on both sides), so all threads leave the sweep loop together.
__global__ void batched_jacobi_kernel(const double* __restrict__ A, int lda, int64_t sa, int n,
                                      double* __restrict__ W, int64_t sw, double* __restrict__ V, int ldv, int64_t sv,
                                      int max_sweeps, double tol, int* __restrict__ err) {
  extern __shared__ double sm[];
  const int np = (n + 1) & ~1;
  double* a = sm;             // np x np, a[i + np*j]
  double* v = sm + np * np;   // np x np
  __shared__ double c_[32], s_[32];
  __shared__ int p_[32], q_[32];
  __shared__ int s_rot;
  const double* Ab = A + blockIdx.x * sa;
  for (int e = threadIdx.x; e < np * np; e += blockDim.x) {
    const int i = e % np, j = e / np;
    a[e] = (i < n && j < n) ? 0.5 * (Ab[i + (int64_t)lda * j] + Ab[j + (int64_t)lda * i]) : 0.0;
    v[e] = i == j ? 1.0 : 0.0;
  }
  __syncthreads();
  const int npair = np / 2;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    __syncthreads();  // every thread has read the previous sweep's flag
    if (threadIdx.x == 0) s_rot = 0;
    __syncthreads();
    for (int r = 0; r < np - 1; ++r) {
      if (threadIdx.x < npair) {
        const int k = threadIdx.x;
        auto player = [&](int pos) { return pos == 0 ? 0 : ((pos - 1 + r) % (np - 1)) + 1; };
        int p = player(k), q = player(np - 1 - k);
        if (p > q) { const int t = p; p = q; q = t; }
        const double apq = a[p + np * q];
        double c = 1.0, s = 0.0;
        if (fabs(apq) > 1e-300 && fabs(apq) > tol * sqrt(fabs(a[p + np * p] * a[q + np * q]))) {
          s_rot = 1;
          const double tau = (a[q + np * q] - a[p + np * p]) / (2.0 * apq);
          const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
          c = 1.0 / sqrt(1.0 + t * t);
          s = t * c;
        }
        c_[k] = c; s_[k] = s; p_[k] = p; q_[k] = q;
      }
      __syncthreads();
      // rows p, q: a_pj <- c a_pj - s a_qj, a_qj <- s a_pj + c a_qj
      for (int e = threadIdx.x; e < npair * np; e += blockDim.x) {
        const int k = e / np, j = e % np;
        const int p = p_[k], q = q_[k];
        const double c = c_[k], s = s_[k];
        const double x = a[p + np * j], y = a[q + np * j];
        a[p + np * j] = c * x - s * y;
        a[q + np * j] = s * x + c * y;
      }
      __syncthreads();
      // columns p, q of A and V
      for (int e = threadIdx.x; e < npair * np; e += blockDim.x) {
        const int k = e / np, i = e % np;
        const int p = p_[k], q = q_[k];
        const double c = c_[k], s = s_[k];
        const double x = a[i + np * p], y = a[i + np * q];
        a[i + np * p] = c * x - s * y;
        a[i + np * q] = s * x + c * y;
        const double vx = v[i + np * p], vy = v[i + np * q];
        v[i + np * p] = c * vx - s * vy;
        v[i + np * q] = s * vx + c * vy;
      }
      __syncthreads();
    }
    const int rot = s_rot;
    if (!rot) break;
  }
  // ascending order of the n real eigenvalues (the padding index, if any, is np - 1 = n
  // and stays decoupled)
  __shared__ int ord[64];
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) ord[i] = i;
    for (int i = 1; i < n; ++i) {
      const int t = ord[i];
      const double x = a[t + np * t];
      int j = i - 1;
      while (j >= 0 && a[ord[j] + np * ord[j]] > x) { ord[j + 1] = ord[j]; --j; }
      ord[j + 1] = t;
    }
  }
  __syncthreads();
  double* Wb = W + blockIdx.x * sw;
  double* Vb = V + blockIdx.x * sv;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e % n, j = e / n;
    const int oj = ord[j];
    if (oj < 0 || oj >= n) {  // cannot happen with a consistent sort: flag it, skip the access
      atomicOr(err, 1);
      continue;
    }
    Vb[i + (int64_t)ldv * j] = v[i + np * oj];
  }
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const int oj = ord[j];
    if (oj >= 0 && oj < n) Wb[j] = a[oj + np * oj];
  }
}

// Segmented products over the stacked rows.  The rows of every problem are cut into
// chunks (crow[c] .. crow[c+1]-1, never across a problem boundary; chunk c belongs to
// problem cq[c] and the chunks of problem q are cb[q] .. cb[q+1]-1).  Row g of a stacked
// block X with leading dimension ldx holds X[g*ldx + 0 .. n-1] (the column-major layout of
// cuBLAS with the roles of rows and columns swapped).

// partial Gram of one chunk: part[c] (na x nb, column-major) = sum_rows A_g^T B_g; a
// thread owns a 4 x 4 tile of the result and groups of threads take interleaved rows,
// summed in a fixed order at the end (no atomics: the sums are reproducible)
constexpr int kSegRows = 32;
__global__ void __launch_bounds__(256) seg_gram_kernel(const double* __restrict__ A, int lda,
                                                       const double* __restrict__ B, int ldb, int na, int nb,
                                                       const int64_t* __restrict__ crow, double* __restrict__ part) {
  __shared__ double sm[2 * kSegRows * 64];
  double* sA = sm;
  double* sB = sm + kSegRows * 64;
  const int tI = (na + 3) / 4, tJ = (nb + 3) / 4, nt = tI * tJ;
  const int PA = 4 * tI, PB = 4 * tJ;
  const int G = blockDim.x / nt;
  const int tid = threadIdx.x;
  const int g = tid / nt, w = tid % nt, ti = w % tI, tj = w / tI;
  const bool act = g < G;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  const int64_t rb = crow[blockIdx.x], re = crow[blockIdx.x + 1];
  for (int64_t r0 = rb; r0 < re; r0 += kSegRows) {
    const int nr = (int)(re - r0 < kSegRows ? re - r0 : kSegRows);
    __syncthreads();
    for (int e = tid; e < nr * PA; e += blockDim.x) {
      const int r = e / PA, i = e % PA;
      sA[e] = i < na ? A[(r0 + r) * lda + i] : 0.0;
    }
    for (int e = tid; e < nr * PB; e += blockDim.x) {
      const int r = e / PB, j = e % PB;
      sB[e] = j < nb ? B[(r0 + r) * ldb + j] : 0.0;
    }
    __syncthreads();
    if (act)
      for (int r = g; r < nr; r += G) {
        double x[4], y[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          x[a] = sA[r * PA + 4 * ti + a];
          y[a] = sB[r * PB + 4 * tj + a];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] = fma(x[a], y[b], acc[a][b]);
      }
  }
  __syncthreads();
  // G * nt * 16 <= 16 * blockDim.x = 4096 doubles: the tiles reuse sA and sB
  if (act) {
    double* red = sm + (size_t)(g * nt + w) * 16;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) red[a * 4 + b] = acc[a][b];
  }
  __syncthreads();
  double* out = part + (int64_t)blockIdx.x * na * nb;
  for (int e = tid; e < na * nb; e += blockDim.x) {
    const int i = e % na, j = e / na;
    const int ww = i / 4 + tI * (j / 4), k = (i % 4) * 4 + j % 4;
    double sum = 0.0;
    for (int gg = 0; gg < G; ++gg) sum += sm[(size_t)(gg * nt + ww) * 16 + k];
    out[e] = sum;
  }
}

// C_q (ld ldc, at C + q*cstride) = sum of its chunks' partial Grams + beta C_q
__global__ void seg_gram_reduce_kernel(const double* __restrict__ part, const int* __restrict__ cb, int na, int nb,
                                       double* __restrict__ C, int ldc, int64_t cstride, double beta) {
  const int q = blockIdx.x;
  double* Cq = C + q * cstride;
  const int c0 = cb[q], c1 = cb[q + 1];
  for (int e = threadIdx.x; e < na * nb; e += blockDim.x) {
    const int i = e % na, j = e / na;
    double sum = 0.0;
    for (int c = c0; c < c1; ++c) sum += part[(int64_t)c * na * nb + e];
    double* dst = Cq + i + (int64_t)ldc * j;
    *dst = beta == 0.0 ? sum : sum + beta * *dst;
  }
}

// Y_g (k entries) = alpha X_g (n entries) Mat_q + beta Y_g for the rows g of one chunk;
// Mat_q (n x k, column-major, ld ldm) at Mat + q*mstride.  Mat_q and a tile of rows sit
// in shared memory; a thread forms 4 consecutive entries of one row.
__global__ void __launch_bounds__(256) seg_combine_kernel(const double* __restrict__ X, int ldx, int n,
                                                          const double* __restrict__ Mat, int ldm, int64_t mstride,
                                                          int k, double* __restrict__ Y, int ldy, double alpha,
                                                          double beta, const int64_t* __restrict__ crow,
                                                          const int* __restrict__ cq) {
  extern __shared__ double dsm[];
  const int kq = (k + 3) / 4, PK = 4 * kq;
  const int TR = min(64, (int)blockDim.x / kq);
  double* sM = dsm;            // n x PK, row i = row i of Mat_q
  double* sX = dsm + n * PK;   // TR x n
  const double* Mq = Mat + cq[blockIdx.x] * mstride;
  for (int e = threadIdx.x; e < n * PK; e += blockDim.x) {
    const int i = e / PK, j = e % PK;
    sM[e] = j < k ? Mq[i + (int64_t)ldm * j] : 0.0;
  }
  const int64_t rb = crow[blockIdx.x], re = crow[blockIdx.x + 1];
  const int r = threadIdx.x / kq, c = threadIdx.x % kq;
  for (int64_t r0 = rb; r0 < re; r0 += TR) {
    const int nr = (int)(re - r0 < TR ? re - r0 : TR);
    __syncthreads();
    for (int e = threadIdx.x; e < nr * n; e += blockDim.x) sX[e] = X[(r0 + e / n) * ldx + e % n];
    __syncthreads();
    if (r < nr) {
      double acc[4] = {0.0, 0.0, 0.0, 0.0};
      for (int i = 0; i < n; ++i) {
        const double x = sX[r * n + i];
        const double* m = sM + i * PK + 4 * c;
#pragma unroll
        for (int a = 0; a < 4; ++a) acc[a] = fma(x, m[a], acc[a]);
      }
      double* y = Y + (r0 + r) * ldy + 4 * c;
#pragma unroll
      for (int a = 0; a < 4; ++a)
        if (4 * c + a < k) y[a] = beta == 0.0 ? alpha * acc[a] : alpha * acc[a] + beta * y[a];
    }
  }
}

// mirror the new columns of every projected matrix into its rows and, for dropped
// (zero) columns, put a large diagonal so that they never enter the lowest Ritz pairs
__global__ void batch_mirror_kernel(double* __restrict__ Hs, int ldh, int64_t sh, int n0, int n1,
                                    const unsigned char* __restrict__ dead, int mcols) {
  double* H = Hs + blockIdx.x * sh;
  const unsigned char* dd = dead + (int64_t)blockIdx.x * mcols;
  for (int e = threadIdx.x; e < n1 * (n1 - n0); e += blockDim.x) {
    const int i = e % n1, j = n0 + e / n1;
    if (i < n0) H[j + (int64_t)ldh * i] = H[i + (int64_t)ldh * j];
  }
  __syncthreads();
  for (int j = n0 + threadIdx.x; j < n1; j += blockDim.x)
    if (dd[j]) {
      for (int i = 0; i < n1; ++i) {
        H[i + (int64_t)ldh * j] = 0.0;
        H[j + (int64_t)ldh * i] = 0.0;
      }
    }
  __syncthreads();
  for (int j = n0 + threadIdx.x; j < n1; j += blockDim.x)
    if (dd[j]) H[j + (int64_t)ldh * j] = 1e30;
}

// R[r, j] = HX[r, j] - E[sys(r), j] X[r, j], j < k; and |R_j|^2 per problem (atomics: the
// norms only steer the iteration)
__global__ void batch_residual_kernel(const double* __restrict__ X, const double* __restrict__ HX, int ldx,
                                      const double* __restrict__ E, int lde, const int* __restrict__ sys, int k,
                                      int64_t N, double* __restrict__ R, double* __restrict__ nrm) {
  const int64_t total = N * k;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / k;
    const int j = (int)(e - r * k);
    const int s = __ldg(sys + r);
    const double val = HX[r * ldx + j] - __ldg(E + (int64_t)s * lde + j) * X[r * ldx + j];
    R[r * ldx + j] = val;
    atomicAdd(nrm + (int64_t)s * k + j, val * val);
  }
}

// T[r, j] = R[r, sel[sys, j]] / (E[sys, sel] - e0[r]) (diagonal preconditioner, floored)
__global__ void batch_precondition_kernel(const double* __restrict__ R, int ldr, const int* __restrict__ sel, int ns,
                                          const double* __restrict__ E, int lde, const double* __restrict__ e0,
                                          const int* __restrict__ sys, int64_t N, double* __restrict__ T, int ldt,
                                          double floor_) {
  const int64_t total = N * ns;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / ns;
    const int j = (int)(e - r * ns);
    const int s = __ldg(sys + r);
    const int l = __ldg(sel + s * ns + j);
    double den = __ldg(E + (int64_t)s * lde + l) - __ldg(e0 + r);
    if (fabs(den) < floor_) den = den < 0 ? -floor_ : floor_;
    T[r * ldt + j] = R[r * ldr + l] / den;
  }
}

// rows of the problems that are not active: zero (their new directions and H.psi columns)
__global__ void batch_zero_rows_kernel(double* __restrict__ X, int ldx, int c0, int ncol, const int* __restrict__ sys,
                                       const unsigned char* __restrict__ active, int64_t N) {
  const int64_t total = N * ncol;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / ncol;
    if (!active[__ldg(sys + r)]) X[r * ldx + c0 + (int)(e - r * ncol)] = 0.0;
  }
}

// transform of the symmetric orthonormalisation: M[:, j] = U[:, j]/sqrt(lambda_j) for
// lambda_j > thr * lambda_max, else 0 (column j dropped)
__global__ void batch_lowdin_kernel(const double* __restrict__ U, const double* __restrict__ lam, int ns,
                                    double* __restrict__ Mt, int ldm, int64_t smt, unsigned char* __restrict__ dead,
                                    int mcols, int col0, double thr) {
  const double* Ub = U + blockIdx.x * (int64_t)ns * ns;
  const double* lb = lam + blockIdx.x * (int64_t)ns;
  double* Mb = Mt + blockIdx.x * smt;
  const double lmax = fmax(lb[ns - 1], 1e-300);
  for (int e = threadIdx.x; e < ns * ns; e += blockDim.x) {
    const int i = e % ns, j = e / ns;
    const bool ok = lb[j] > thr * lmax && lb[j] > 1e-280;
    Mb[i + (int64_t)ldm * j] = ok ? Ub[i + (int64_t)ns * j] / sqrt(lb[j]) : 0.0;
  }
  for (int j = threadIdx.x; j < ns; j += blockDim.x) {
    const bool ok = lb[j] > thr * lmax && lb[j] > 1e-280;
    dead[(int64_t)blockIdx.x * mcols + col0 + j] = ok ? 0 : 1;
  }
}

// a projected matrix of Ritz pairs: diag(E_s) in the leading k x k block
__global__ void batch_diag_kernel(double* __restrict__ Hs, int ldh, int64_t sh, const double* __restrict__ E,
                                  int lde, int k) {
  double* H = Hs + blockIdx.x * sh;
  for (int e = threadIdx.x; e < ldh * ldh; e += blockDim.x) H[e] = 0.0;
  __syncthreads();
  for (int j = threadIdx.x; j < k; j += blockDim.x) H[j + (int64_t)ldh * j] = E[(int64_t)blockIdx.x * lde + j];
}

struct DBuf {
  void* p = nullptr;
  ~DBuf() {
    if (p) cudaFree(p);
  }
  bool alloc(size_t bytes) { return cudaMalloc(&p, std::max<size_t>(bytes, 8)) != cudaSuccess; }
  double* d() const { return (double*)p; }
};

}  // namespace

// ---------------------------------------------------------------------------------------
// batch context
// ---------------------------------------------------------------------------------------
namespace evr {
struct BatchInfo {
  std::vector<int64_t> off;  // n_sys + 1 packed offsets
  std::vector<HostProblem> sub;
  std::vector<int> term_sys; // term -> problem
  int* sys_d = nullptr;      // row -> problem (nb0 == 1)
};
}  // namespace evr

static void free_batch(evr_ctx* c) {
  BatchInfo* b = (BatchInfo*)c->batch;
  if (!b) return;
  if (b->sys_d) cudaFree(b->sys_d);
  delete b;
  c->batch = nullptr;
}

namespace evr {
void free_batch_info(evr_ctx* c) { free_batch(c); }
}  // namespace evr

#define EVR_CU(call, what)                 \
  do {                                     \
    int _rc = cuda_check(c, (call), what); \
    if (_rc != EVR_OK) return _rc;         \
  } while (0)

static int merge_problems(evr_ctx* c, std::vector<HostProblem>& sub, std::string& err) {
  HostProblem& P = c->hp;
  P = HostProblem();
  const HostProblem& P0 = sub[0];
  P.kind = P0.kind;
  P.nb0 = P0.nb0;
  P.keo_type = P0.keo_type;
  P.symmetric = true;
  int Dmax = 0;
  for (const HostProblem& Q : sub) {
    if (Q.nb0 != P.nb0) { err = "batched problems need the same number of electronic states"; return EVR_EINVAL; }
    if (Q.keo_type != P.keo_type) { err = "batched problems need the same KEO type"; return EVR_EINVAL; }
    Dmax = std::max(Dmax, Q.D);
    P.symmetric = P.symmetric && Q.symmetric;
  }
  P.D = Dmax;
  int64_t np_off = 0, nb_off = 0, nq_off = 0;
  size_t pool_off = 0, g0_off = 0, g_off = 0;
  std::vector<int64_t> np_of(sub.size());
  for (size_t s = 0; s < sub.size(); ++s) {
    const HostProblem& Q = sub[s];
    np_of[s] = np_off;
    if (pool_off + Q.mat_pool.size() > (size_t)INT32_MAX || g_off + Q.g.size() > (size_t)INT32_MAX) {
      err = "batch too large for 32-bit table offsets";
      return EVR_EINVAL;
    }
    P.mat_pool.insert(P.mat_pool.end(), Q.mat_pool.begin(), Q.mat_pool.end());
    P.G0.insert(P.G0.end(), Q.G0.begin(), Q.G0.end());
    P.g.insert(P.g.end(), Q.g.begin(), Q.g.end());
    auto shift = [&](TermDesc T) {
      T.off_nb += nb_off;
      T.off_nq += nq_off;
      for (int p = 0; p < Q.D; ++p) {
        T.m_d0b[p] += (int)pool_off;
        T.m_bgw[p] += (int)pool_off;
        T.m_d1[p] += (int)pool_off;
        T.m_d2[p] += (int)pool_off;
        T.m_x[p] += (int)pool_off;
      }
      T.m_x1L += (int)pool_off;
      T.m_x2L += (int)pool_off;
      T.m_e1L += (int)pool_off;
      T.m_e2L += (int)pool_off;
      T.g0off = (int)g0_off;
      T.goff = (int)g_off;
      return T;
    };
    for (size_t t = 0; t < Q.terms.size(); ++t) {
      P.terms.push_back(shift(Q.terms[t]));
      P.termsT.push_back(shift(Q.termsT[t]));
      P.weight.push_back(Q.weight[t]);
    }
    for (int v : Q.map_perm) P.map_perm.push_back(v >= 0 ? (int)(v + np_off) : -1);
    for (int v : Q.map) P.map.push_back(v >= 0 ? (int)(v + np_off) : -1);
    np_off += Q.Np;
    nb_off += Q.sum_nb;
    nq_off += Q.sum_nq;
    pool_off += Q.mat_pool.size();
    g0_off += Q.G0.size();
    g_off += Q.g.size();
    P.max_nq = std::max(P.max_nq, Q.max_nq);
    P.max_nb = std::max(P.max_nb, Q.max_nb);
    P.flop_per_hpsi += Q.flop_per_hpsi;
  }
  if (np_off * P.nb0 >= INT32_MAX) { err = "batch too large (packed index beyond 32 bits)"; return EVR_EINVAL; }
  P.Np = np_off;
  P.sum_nb = nb_off;
  P.sum_nq = nq_off;
  const int nb0 = P.nb0;
  const int64_t N = P.Np * nb0;
  // CSR over the stacked rows (a * Np + packed), sources shifted with the term offsets
  P.csr_ptr.assign((size_t)N + 1, 0);
  for (int a = 0; a < nb0; ++a)
    for (size_t s = 0; s < sub.size(); ++s) {
      const HostProblem& Q = sub[s];
      for (int64_t k = 0; k < Q.Np; ++k) {
        const int64_t lr = a * Q.Np + k, gr = a * P.Np + np_of[s] + k;
        P.csr_ptr[(size_t)gr + 1] = Q.csr_ptr[(size_t)lr + 1] - Q.csr_ptr[(size_t)lr];
      }
    }
  for (int64_t r = 0; r < N; ++r) P.csr_ptr[(size_t)r + 1] += P.csr_ptr[(size_t)r];
  P.csr_src.resize((size_t)P.csr_ptr[(size_t)N]);
  P.csr_w.resize((size_t)P.csr_ptr[(size_t)N]);
  P.e0diag.assign((size_t)N, 0.0);
  int64_t nbo = 0;
  for (size_t s = 0; s < sub.size(); ++s) {
    const HostProblem& Q = sub[s];
    for (int a = 0; a < nb0; ++a)
      for (int64_t k = 0; k < Q.Np; ++k) {
        const int64_t lr = a * Q.Np + k, gr = a * P.Np + np_of[s] + k;
        int64_t o = P.csr_ptr[(size_t)gr];
        for (int64_t e = Q.csr_ptr[(size_t)lr]; e < Q.csr_ptr[(size_t)lr + 1]; ++e, ++o) {
          // local source off_nb*nb0 + a*NB + iB -> shift off_nb by the problem's offset
          P.csr_src[(size_t)o] = Q.csr_src[(size_t)e] + nbo * nb0;
          P.csr_w[(size_t)o] = Q.csr_w[(size_t)e];
        }
        P.e0diag[(size_t)gr] = Q.e0diag[(size_t)lr];
      }
    nbo += Q.sum_nb;
  }
  return EVR_OK;
}

static int upload_batch(evr_ctx* c) {
  HostProblem& P = c->hp;
  DeviceProblem& d = c->dp;
  BatchInfo* b = (BatchInfo*)c->batch;
  auto up = [&](void** dst, const void* src, size_t bytes) -> int {
    EVR_CU(cudaMalloc(dst, std::max<size_t>(bytes, 8)), "cudaMalloc");
    if (bytes) EVR_CU(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice), "cudaMemcpy");
    return EVR_OK;
  };
  int rc;
  if ((rc = up((void**)&d.terms, P.terms.data(), P.terms.size() * sizeof(TermDesc)))) return rc;
  if ((rc = up((void**)&d.termsT, P.termsT.data(), P.termsT.size() * sizeof(TermDesc)))) return rc;
  if ((rc = up((void**)&d.mats, P.mat_pool.data(), P.mat_pool.size() * sizeof(double)))) return rc;
  if ((rc = up((void**)&d.map, P.map_perm.data(), P.map_perm.size() * sizeof(int)))) return rc;
  if ((rc = up((void**)&d.csr_ptr, P.csr_ptr.data(), P.csr_ptr.size() * sizeof(int64_t)))) return rc;
  if ((rc = up((void**)&d.csr_src, P.csr_src.data(), P.csr_src.size() * sizeof(int64_t)))) return rc;
  if ((rc = up((void**)&d.csr_w, P.csr_w.data(), P.csr_w.size() * sizeof(double)))) return rc;
  if ((rc = upload_long_rows(c))) return rc;
  if ((rc = up((void**)&d.G0, P.G0.data(), P.G0.size() * sizeof(double)))) return rc;
  if ((rc = up((void**)&d.g, P.g.data(), P.g.size() * sizeof(double)))) return rc;
  if ((rc = upload_coeffs32(c))) return rc;
  if ((rc = up((void**)&d.e0diag, P.e0diag.data(), P.e0diag.size() * sizeof(double)))) return rc;
  const int nb0 = P.nb0;
  const int64_t nv = P.sum_nq * nb0 * nb0;
  EVR_CU(cudaMalloc((void**)&d.vgrid, nv * sizeof(double)), "cudaMalloc vgrid");
  // V per problem from its own monomials
  int64_t t0 = 0, q0 = 0;
  for (const HostProblem& Q : b->sub) {
    const int nm = (int)Q.mono_coef.size();
    double* dc = nullptr;
    int *di = nullptr, *de = nullptr;
    if ((rc = up((void**)&dc, Q.mono_coef.data(), nm * sizeof(double))) ||
        (rc = up((void**)&di, Q.mono_idx.data(), Q.mono_idx.size() * sizeof(int))) ||
        (rc = up((void**)&de, Q.mono_elec.data(), Q.mono_elec.size() * sizeof(int))))
      return rc;
    const int64_t t1 = t0 + (int64_t)Q.terms.size(), q1 = q0 + Q.sum_nq;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((Q.sum_nq + 255) / 256, c->num_sms * 8));
    batch_vgrid_kernel<<<blocks, 256, 0, c->stream>>>(d.terms, (int)t0, (int)t1, d.mats, q0, q1, nb0, nm, dc, di, de,
                                                       d.vgrid);
    EVR_CU(cudaGetLastError(), "batch_vgrid_kernel");
    EVR_CU(cudaStreamSynchronize(c->stream), "batch V");
    cudaFree(dc);
    cudaFree(di);
    cudaFree(de);
    t0 = t1;
    q0 = q1;
  }
  EVR_CU(cudaMalloc((void**)&d.mats32, P.mat_pool.size() * sizeof(float) + 16), "cudaMalloc mats32");
  EVR_CU(cudaMalloc((void**)&d.vgrid32, nv * sizeof(float)), "cudaMalloc vgrid32");
  batch_to_float<<<c->num_sms * 4, 256, 0, c->stream>>>(d.mats, d.mats32, (int64_t)P.mat_pool.size());
  batch_to_float<<<c->num_sms * 8, 256, 0, c->stream>>>(d.vgrid, d.vgrid32, nv);
  EVR_CU(cudaGetLastError(), "batch_to_float");
  // row -> problem
  if (nb0 == 1) {
    std::vector<int> sys((size_t)P.Np);
    for (size_t s = 0; s + 1 < b->off.size(); ++s)
      for (int64_t k = b->off[s]; k < b->off[s + 1]; ++k) sys[(size_t)k] = (int)s;
    if ((rc = up((void**)&b->sys_d, sys.data(), sys.size() * sizeof(int)))) return rc;
  }
  EVR_CU(cudaStreamSynchronize(c->stream), "batch set-up");
  return EVR_OK;
}

extern "C" {

int evr_create_batch(evr_ctx** out, const evr_problem_desc* descs, int n_sys, int device) {
  if (!out) return EVR_EINVAL;
  *out = nullptr;
  evr_ctx* c = new (std::nothrow) evr_ctx();
  if (!c) return EVR_ENOMEM;
  *out = c;
  if (!descs || n_sys < 1) return set_error(c, EVR_EINVAL, "evr_create_batch: no problems");
  c->device = device;
  BatchInfo* b = new BatchInfo();
  c->batch = b;
  b->sub.resize(n_sys);
  b->off.assign(n_sys + 1, 0);
  {
    // the problems' host tables are independent: built on up to 16 host threads, each
    // taking the next problem; errors are reported for the first failing problem in order
    std::vector<int> rcs(n_sys, EVR_OK);
    std::vector<std::string> errs(n_sys);
    std::atomic<int> next{0};
    auto work = [&]() {
      for (int s = next.fetch_add(1); s < n_sys; s = next.fetch_add(1))
        rcs[s] = build_host_problem(&descs[s], b->sub[s], errs[s]);
    };
    const int nthr = std::max(1, std::min({n_sys, 16, (int)std::thread::hardware_concurrency()}));
    std::vector<std::thread> pool;
    for (int i = 1; i < nthr; ++i) pool.emplace_back(work);
    work();
    for (std::thread& t : pool) t.join();
    for (int s = 0; s < n_sys; ++s)
      if (rcs[s]) return set_error(c, rcs[s], "evr_create_batch: problem " + std::to_string(s) + ": " + errs[s]);
  }
  for (int s = 0; s < n_sys; ++s) {
    b->off[s + 1] = b->off[s] + b->sub[s].Np;
    b->term_sys.insert(b->term_sys.end(), b->sub[s].terms.size(), s);
  }
  std::string err;
  int rc = merge_problems(c, b->sub, err);
  if (rc) return set_error(c, rc, "evr_create_batch: " + err);
  c->n_sys = n_sys;
  c->gfly = false;
  for (const HostProblem& Q : b->sub)
    if (Q.keo_type == 10)
      for (double v : Q.g) c->gfly |= (v != 0.0);
  c->use_stages = false;
  if (device < 0) {
    c->host_only = true;
    return EVR_OK;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device >= ndev) {
    (void)cudaGetLastError();
    return set_error(c, EVR_EDEVICE, "no CUDA device " + std::to_string(device));
  }
  EVR_CU(cudaSetDevice(device), "cudaSetDevice");
  EVR_CU(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device), "attr");
  EVR_CU(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  for (auto& e : c->ev) EVR_CU(cudaEventCreate(&e), "cudaEventCreate");
  return upload_batch(c);
}

int evr_batch_offsets(const evr_ctx* c, int64_t* offsets) {
  if (!c || !offsets) return EVR_EINVAL;
  const BatchInfo* b = (const BatchInfo*)c->batch;
  if (!b) {
    offsets[0] = 0;
    offsets[1] = c->hp.Np;
    return EVR_OK;
  }
  std::copy(b->off.begin(), b->off.end(), offsets);
  return EVR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// batched Davidson
// ---------------------------------------------------------------------------------------
namespace {

struct BatchDavidson {
  evr_ctx* c;
  cudaStream_t s;
  int nsys = 0, M = 0, nkeep = 0, bmax = 0, op = OP_H, nch = 0;
  int64_t N = 0;
  std::vector<int64_t> off;
  const int* sys_d = nullptr;
  DBuf Pt, HPt, X, HX, R, T, Tt, Hs, Wv, Ev, Cm, Gm, Um, Lm, Mt, nrm, sel, dead, actv;
  DBuf crow, cq, cb, part;  // row chunks of the segmented products and their partial Grams
  DBuf errf;                // consistency flag of the batched Jacobi kernel
  std::vector<unsigned char> active;      // problems still iterating
  const std::vector<int>* term_sys = nullptr;
  int64_t sh = 0;  // stride of one projected matrix (M*M)

  int fail(int code, const std::string& m) { return set_error(c, code, "evr_batch_davidson: " + m); }

  int init() {
    if (M > 64 || bmax > 64) return fail(EVR_EINVAL, "subspace larger than 64");
    sh = (int64_t)M * M;
    // row chunks: about four per SM over the whole stack, none across a problem boundary
    const int64_t rc = std::max<int64_t>(256, (N + 4 * c->num_sms - 1) / (4 * c->num_sms));
    std::vector<int64_t> hrow;
    std::vector<int> hq, hb(nsys + 1);
    for (int q = 0; q < nsys; ++q) {
      hb[q] = (int)hrow.size();
      for (int64_t r = off[q]; r < off[q + 1]; r += rc) {
        hrow.push_back(r);
        hq.push_back(q);
      }
    }
    nch = (int)hrow.size();
    hb[nsys] = nch;
    hrow.push_back(N);
    if (crow.alloc(hrow.size() * sizeof(int64_t)) || cq.alloc(hq.size() * sizeof(int)) ||
        cb.alloc(hb.size() * sizeof(int)) || part.alloc((size_t)nch * M * M * 8) || errf.alloc(sizeof(int)))
      return fail(EVR_ENOMEM, "device allocation");
    if (cudaMemsetAsync(errf.p, 0, sizeof(int), s)) return fail(EVR_EDEVICE, "memset");
    if (cudaMemcpyAsync(crow.p, hrow.data(), hrow.size() * sizeof(int64_t), cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(cq.p, hq.data(), hq.size() * sizeof(int), cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(cb.p, hb.data(), hb.size() * sizeof(int), cudaMemcpyHostToDevice, s) ||
        cudaStreamSynchronize(s))
      return fail(EVR_EDEVICE, "chunk upload");
    if (cudaFuncSetAttribute(seg_combine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 64 * 64 * 8) !=
        cudaSuccess)
      return fail(EVR_EDEVICE, "combine attribute");
    const size_t nm = (size_t)N * M;
    if (Pt.alloc(nm * 8) || HPt.alloc(nm * 8) || X.alloc((size_t)N * nkeep * 8) || HX.alloc((size_t)N * nkeep * 8) ||
        R.alloc((size_t)N * nkeep * 8) || T.alloc((size_t)N * bmax * 8) || Tt.alloc((size_t)N * bmax * 8) ||
        Hs.alloc((size_t)nsys * sh * 8) || Wv.alloc((size_t)nsys * sh * 8) || Ev.alloc((size_t)nsys * M * 8) ||
        Cm.alloc((size_t)nsys * M * bmax * 8) || Gm.alloc((size_t)nsys * bmax * bmax * 8) ||
        Um.alloc((size_t)nsys * bmax * bmax * 8) || Lm.alloc((size_t)nsys * bmax * 8) ||
        Mt.alloc((size_t)nsys * bmax * bmax * 8) || nrm.alloc((size_t)nsys * nkeep * 8) ||
        sel.alloc((size_t)nsys * bmax * sizeof(int)) || dead.alloc((size_t)nsys * M) || actv.alloc((size_t)nsys))
      return fail(EVR_ENOMEM, "device allocation");
    if (cudaMemsetAsync(dead.p, 0, (size_t)nsys * M, s)) return fail(EVR_EDEVICE, "memset");
    const int np = ((std::max(M, bmax) + 1) & ~1);
    if (cudaFuncSetAttribute(batched_jacobi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(2 * np * np * sizeof(double))) != cudaSuccess)
      return fail(EVR_EDEVICE, "jacobi attribute");
    return EVR_OK;
  }

  // C_q (na x nb, ld ldc, at C + q*cstride) = A_q^T B_q + beta C_q over the rows of problem q
  int gram(const double* A, int lda, const double* B, int ldb, int na, int nb, double* C, int ldc, int64_t cstride,
           double beta = 0.0) {
    if (na < 1 || nb < 1 || na > 64 || nb > 64) return fail(EVR_EINVAL, "gram size");
    seg_gram_kernel<<<nch, kBT, 0, s>>>(A, lda, B, ldb, na, nb, (const int64_t*)crow.p, part.d());
    seg_gram_reduce_kernel<<<nsys, kBT, 0, s>>>(part.d(), (const int*)cb.p, na, nb, C, ldc, cstride, beta);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? EVR_OK : fail(EVR_EDEVICE, std::string("gram launch: ") + cudaGetErrorString(e));
  }
  // Y_q (rows x k, ld ldy) = alpha X_q (rows x n, ld ldx) Mat_q (n x k, ld ldm, at Mat + q*mstride) + beta Y_q
  int combine(const double* Xb, int ldx, int n, const double* Mat, int ldm, int64_t mstride, int k, double* Y, int ldy,
              double alpha, double beta) {
    if (n < 1 || k < 1 || n > 64 || k > 64) return fail(EVR_EINVAL, "combine size");
    const int kq = (k + 3) / 4, tr = std::min(64, kBT / kq);
    const size_t smem = (size_t)(n * 4 * kq + tr * n) * sizeof(double);
    seg_combine_kernel<<<nch, kBT, smem, s>>>(Xb, ldx, n, Mat, ldm, mstride, k, Y, ldy, alpha, beta,
                                              (const int64_t*)crow.p, (const int*)cq.p);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? EVR_OK : fail(EVR_EDEVICE, std::string("combine launch: ") + cudaGetErrorString(e));
  }

  // H.psi of n columns for the active problems only (the others' rows come out zero)
  int hop(double* x, int ldx, double* y, int ldy, int n, int prec, int64_t& c64, int64_t& c32) {
    int na = 0;
    for (unsigned char a : active) na += a;
    if (na == 0) return EVR_OK;
    const bool all = na == nsys;
    if (!all) {
      c->term_active.resize(term_sys->size());
      for (size_t t = 0; t < term_sys->size(); ++t) c->term_active[t] = active[(*term_sys)[t]];
    }
    int rc = hpsi_blocks(c, x, ldx, y, ldy, n, prec, s, op);
    c->term_active.clear();
    if (rc) return rc;
    if (!all) {
      if (cudaMemcpyAsync(actv.p, active.data(), nsys, cudaMemcpyHostToDevice, s)) return fail(EVR_EDEVICE, "copy");
      batch_zero_rows_kernel<<<c->num_sms * 8, kBT, 0, s>>>(y, ldy, 0, n, sys_d, (const unsigned char*)actv.p, N);
      if (cudaStreamSynchronize(s)) return fail(EVR_EDEVICE, "sync");
    }
    (prec == EVR_PREC_FP32 ? c32 : c64) += (int64_t)n * na * (op == OP_HSYM ? 2 : 1);
    return EVR_OK;
  }

  int jacobi(const double* A, int lda, int64_t sa, int n, double* W, int64_t sw, double* V, int ldv, int64_t sv) {
    const int np = (n + 1) & ~1;
    batched_jacobi_kernel<<<nsys, kBT, 2 * np * np * sizeof(double), s>>>(A, lda, sa, n, W, sw, V, ldv, sv, 40, 1e-15,
                                                                         (int*)errf.p);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? EVR_OK : fail(EVR_EDEVICE, std::string("jacobi launch: ") + cudaGetErrorString(e));
  }

  // orthonormalise the ns columns of T against Pt(:, 0:n1) and among themselves, append
  // them to Pt(:, n1:n1+ns); dropped directions become zero columns flagged in `dead`
  int orthonormalize(int ns, int n1) {
    for (int pass = 0; pass < 2; ++pass) {
      if (n1 > 0) {
        int rc = gram(Pt.d(), M, T.d(), bmax, n1, ns, Cm.d(), M, (int64_t)M * bmax);
        if (rc) return rc;
        rc = combine(Pt.d(), M, n1, Cm.d(), M, (int64_t)M * bmax, ns, T.d(), bmax, -1.0, 1.0);
        if (rc) return rc;
      }
    }
    int rc = gram(T.d(), bmax, T.d(), bmax, ns, ns, Gm.d(), ns, (int64_t)ns * ns);
    if (rc) return rc;
    if ((rc = jacobi(Gm.d(), ns, (int64_t)ns * ns, ns, Lm.d(), ns, Um.d(), ns, (int64_t)ns * ns))) return rc;
    batch_lowdin_kernel<<<nsys, kBT, 0, s>>>(Um.d(), Lm.d(), ns, Mt.d(), bmax, (int64_t)bmax * bmax,
                                             (unsigned char*)dead.p, M, n1, 1e-12);
    if ((rc = combine(T.d(), bmax, ns, Mt.d(), bmax, (int64_t)bmax * bmax, ns, Tt.d(), bmax, 1.0, 0.0))) return rc;
    if (cudaMemcpy2DAsync(Pt.d() + n1, sizeof(double) * M, Tt.d(), sizeof(double) * bmax, sizeof(double) * ns, N,
                          cudaMemcpyDeviceToDevice, s))
      return fail(EVR_EDEVICE, "append");
    return EVR_OK;
  }

  // projected matrices, new columns n0..n1 (all columns carry an H.psi of one precision)
  int rayleigh_ritz(int n0, int n1) {
    int rc = gram(Pt.d(), M, HPt.d() + n0, M, n1, n1 - n0, Hs.d() + (int64_t)M * n0, M, sh);
    if (rc) return rc;
    batch_mirror_kernel<<<nsys, kBT, 0, s>>>(Hs.d(), M, sh, n0, n1, (const unsigned char*)dead.p, M);
    return jacobi(Hs.d(), M, sh, n1, Ev.d(), M, Wv.d(), M, sh);
  }
};

}  // namespace

extern "C" int evr_batch_davidson(evr_ctx* c, const evr_davidson_opts* o, double* eig, int64_t* info) {
  if (!c || !o || !eig) return EVR_EINVAL;
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  BatchInfo* bi = (BatchInfo*)c->batch;
  if (!bi) return set_error(c, EVR_EINVAL, "evr_batch_davidson: not a batch context (evr_create_batch)");
  if (c->hp.nb0 != 1) return set_error(c, EVR_EINVAL, "evr_batch_davidson: one electronic state per problem");
  if (o->prec != EVR_PREC_FP64 && o->prec != EVR_PREC_FP32) return set_error(c, EVR_EINVAL, "unknown precision");
  const int nsys = c->n_sys;
  const int nlev = o->n_levels;
  int64_t nmin = INT64_MAX;
  for (int q = 0; q < nsys; ++q) nmin = std::min(nmin, bi->off[q + 1] - bi->off[q]);
  const int b = std::min(std::max(o->block, 1), 32);
  if (nlev < 1 || nlev > nmin) return set_error(c, EVR_EINVAL, "evr_batch_davidson: n_levels out of range");
  if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, EVR_EDEVICE, "cudaSetDevice");
  BatchDavidson d;
  d.c = c;
  d.s = c->stream;
  d.nsys = nsys;
  d.N = c->hp.Np;
  d.off = bi->off;
  d.sys_d = bi->sys_d;
  d.term_sys = &bi->term_sys;
  d.active.assign(nsys, 1);
  d.bmax = b;
  d.nkeep = (int)std::min<int64_t>(nmin, nlev + b);
  d.M = (int)std::min<int64_t>(std::min<int64_t>(nmin, 64), std::max(o->max_dim, d.nkeep + b));
  if (d.M < d.nkeep + 1) return set_error(c, EVR_EINVAL, "evr_batch_davidson: subspace too small for the smallest problem");
  d.op = (o->sym > 0 || (o->sym < 0 && !c->hp.symmetric)) ? OP_HSYM : OP_H;
  int rc = d.init();
  if (rc) return rc;
  const int M = d.M;
  cudaStream_t s = d.s;
  const int64_t N = d.N;

  // initial space: unit vectors on the lowest zero-order energies of every problem
  int n1 = 0, n0 = 0;
  {
    const int ninit = std::min(std::min(std::max(nlev, b), M - b), b);
    std::vector<double> h((size_t)N * b, 0.0);
    for (int q = 0; q < nsys; ++q) {
      const int64_t r0 = bi->off[q], nr = bi->off[q + 1] - r0;
      std::vector<int64_t> idx(nr);
      std::iota(idx.begin(), idx.end(), 0);
      const int m = (int)std::min<int64_t>(ninit, nr);
      std::partial_sort(idx.begin(), idx.begin() + m, idx.end(),
                        [&](int64_t a, int64_t bb) { return c->hp.e0diag[r0 + a] < c->hp.e0diag[r0 + bb]; });
      for (int j = 0; j < m; ++j) h[(size_t)(r0 + idx[j]) * b + j] = 1.0;
    }
    if (cudaMemcpyAsync(d.T.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s))
      return set_error(c, EVR_EDEVICE, "init copy");
    if ((rc = d.orthonormalize(ninit, 0))) return rc;
    n1 = ninit;
  }
  int prec = o->prec;
  int64_t c64 = 0, c32 = 0;
  std::vector<double> Eh((size_t)nsys * M), Eold((size_t)nsys * nlev, 1e300), rn((size_t)nsys * d.nkeep);
  // FP32 phase of the mixed form, per problem: best residual so far, iterations without
  // halving it, and whether the problem has reached its FP32 floor (it then waits, taking
  // no H.psi, until every problem has)
  std::vector<double> best_q(nsys, 1e300);
  std::vector<int> stall_q(nsys, 0);
  std::vector<unsigned char> floor_q(nsys, 0);
  int it = 0, it32 = 0;
  bool converged = false;
  for (it = 0; it < o->max_it; ++it) {
    if ((rc = d.hop(d.Pt.d() + n0, M, d.HPt.d() + n0, M, n1 - n0, prec, c64, c32))) return rc;
    if ((rc = d.rayleigh_ritz(n0, n1))) return rc;
    n0 = n1;
    const int k = std::min(d.nkeep, n1);
    // Ritz vectors and their H.psi
    if ((rc = d.combine(d.Pt.d(), M, n1, d.Wv.d(), M, d.sh, k, d.X.d(), d.nkeep, 1.0, 0.0))) return rc;
    if ((rc = d.combine(d.HPt.d(), M, n1, d.Wv.d(), M, d.sh, k, d.HX.d(), d.nkeep, 1.0, 0.0))) return rc;
    if (cudaMemsetAsync(d.nrm.p, 0, sizeof(double) * nsys * k, s)) return set_error(c, EVR_EDEVICE, "memset");
    batch_residual_kernel<<<c->num_sms * 8, kBT, 0, s>>>(d.X.d(), d.HX.d(), d.nkeep, d.Ev.d(), M, d.sys_d, k, N,
                                                         d.R.d(), d.nrm.d());
    int jerr = 0;
    if (cudaMemcpyAsync(rn.data(), d.nrm.p, sizeof(double) * nsys * k, cudaMemcpyDeviceToHost, s) ||
        cudaMemcpyAsync(Eh.data(), d.Ev.p, sizeof(double) * nsys * M, cudaMemcpyDeviceToHost, s) ||
        cudaMemcpyAsync(&jerr, d.errf.p, sizeof(int), cudaMemcpyDeviceToHost, s) || cudaStreamSynchronize(s))
      return set_error(c, EVR_EDEVICE, "evr_batch_davidson: residual norms");
    if (jerr) return set_error(c, EVR_EDEVICE, "evr_batch_davidson: inconsistent eigenvalue order in the Jacobi kernel");
    const int nt = std::min(nlev, k);
    std::vector<double> rq(nsys, 0.0);
    std::vector<std::vector<int>> todo(nsys);
    size_t most = 0;
    for (int q = 0; q < nsys; ++q) {
      for (int j = 0; j < nt; ++j) {
        const double r = std::sqrt(rn[(size_t)q * k + j]);
        const double e = Eh[(size_t)q * M + j];
        const double de = std::fabs(e - Eold[(size_t)q * nlev + j]);
        Eold[(size_t)q * nlev + j] = e;
        rq[q] = std::max(rq[q], r);
        if (!(r < o->conv_resi && de < o->conv_ene)) todo[q].push_back(j);
      }
      most = std::max(most, todo[q].size());
    }
    // problems with nothing left to do stop taking H.psi (their new columns are empty)
    for (int q = 0; q < nsys; ++q) d.active[q] = (nt < nlev || !todo[q].empty()) ? 1 : 0;
    if (nt == nlev && most == 0 && prec == EVR_PREC_FP64) {
      converged = true;
      break;
    }
    if (prec == EVR_PREC_FP32) {
      // Each problem runs its FP32 phase until its largest residual reaches 1e-4 of its
      // level energies, stops halving for two iterations, or meets the tolerance; it then
      // waits (no H.psi, empty new columns) while the others go on.  When every problem has
      // reached its floor the whole batch continues as the FP64 iteration from the Ritz
      // vectors (in lock step a mixed refinement would recompute the Ritz vectors' H.psi
      // in FP64 after every subspace restart, as many FP64 H.psi as the plain solve).
      ++it32;
      bool all_floor = nt == nlev;
      for (int q = 0; q < nsys && nt == nlev; ++q) {
        if (floor_q[q]) continue;
        const double hs = std::max(std::fabs(Eh[(size_t)q * M]), std::fabs(Eh[(size_t)q * M + nt - 1]));
        if (rq[q] < 0.5 * best_q[q]) {
          best_q[q] = rq[q];
          stall_q[q] = 0;
        } else {
          ++stall_q[q];
        }
        if (rq[q] < std::max(o->conv_resi, 1e-4 * hs) || stall_q[q] >= 2 || todo[q].empty()) floor_q[q] = 1;
        all_floor = all_floor && floor_q[q];
      }
      // a cap on the FP32 phase: half of the iteration budget
      if (all_floor || it32 >= std::max(2, o->max_it / 2)) {
        const int kr = std::min(k, nlev);
        if (cudaMemcpy2DAsync(d.Pt.p, sizeof(double) * M, d.X.p, sizeof(double) * d.nkeep, sizeof(double) * kr, N,
                              cudaMemcpyDeviceToDevice, s) ||
            cudaMemsetAsync(d.dead.p, 0, (size_t)nsys * M, s))
          return set_error(c, EVR_EDEVICE, "restart copy");
        prec = EVR_PREC_FP64;
        n1 = kr;
        n0 = 0;
        std::fill(Eold.begin(), Eold.end(), 1e300);
        std::fill(d.active.begin(), d.active.end(), 1);  // every problem continues in FP64
        continue;
      }
      for (int q = 0; q < nsys; ++q)
        if (floor_q[q]) d.active[q] = 0;  // waits for the others at its FP32 floor
    }
    // new directions: per problem its lowest unconverged levels, filled up with its other
    // levels so that every problem adds the same number of columns
    int ns = (int)std::min<size_t>(std::max<size_t>(most, 1), (size_t)d.bmax);
    if (nt < nlev) ns = std::min(d.bmax, nt);
    std::vector<int> selh((size_t)nsys * ns);
    for (int q = 0; q < nsys; ++q) {
      std::vector<int> lst = todo[q];
      if (nt < nlev) {
        lst.clear();
        for (int j = 0; j < nt; ++j) lst.push_back(j);
      }
      for (int j = 0; j < nt && (int)lst.size() < ns; ++j)
        if (std::find(lst.begin(), lst.end(), j) == lst.end()) lst.push_back(j);
      for (int j = 0; j < ns; ++j) selh[(size_t)q * ns + j] = lst[(size_t)j % lst.size()];
    }
    if (cudaMemcpyAsync(d.sel.p, selh.data(), selh.size() * sizeof(int), cudaMemcpyHostToDevice, s))
      return set_error(c, EVR_EDEVICE, "copy");
    batch_precondition_kernel<<<c->num_sms * 8, kBT, 0, s>>>(d.R.d(), d.nkeep, (const int*)d.sel.p, ns, d.Ev.d(), M,
                                                             c->dp.e0diag, d.sys_d, N, d.T.d(), d.bmax, 1e-6);
    // converged problems add empty directions (flagged and ignored by the projections)
    if (cudaMemcpyAsync(d.actv.p, d.active.data(), nsys, cudaMemcpyHostToDevice, s))
      return set_error(c, EVR_EDEVICE, "copy");
    batch_zero_rows_kernel<<<c->num_sms * 8, kBT, 0, s>>>(d.T.d(), d.bmax, 0, ns, d.sys_d,
                                                          (const unsigned char*)d.actv.p, N);
    if (n1 + ns > M) {
      if (cudaMemcpy2DAsync(d.Pt.p, sizeof(double) * M, d.X.p, sizeof(double) * d.nkeep, sizeof(double) * k, N,
                            cudaMemcpyDeviceToDevice, s) ||
          cudaMemcpy2DAsync(d.HPt.p, sizeof(double) * M, d.HX.p, sizeof(double) * d.nkeep, sizeof(double) * k, N,
                            cudaMemcpyDeviceToDevice, s) ||
          cudaMemsetAsync(d.dead.p, 0, (size_t)nsys * M, s))
        return set_error(c, EVR_EDEVICE, "restart copy");
      batch_diag_kernel<<<nsys, kBT, 0, s>>>(d.Hs.d(), M, d.sh, d.Ev.d(), M, k);
      n1 = n0 = k;
    }
    if ((rc = d.orthonormalize(ns, n1))) return rc;
    n1 += ns;
  }
  const int k = std::min(d.nkeep, n1);
  for (int q = 0; q < nsys; ++q)
    for (int j = 0; j < nlev; ++j) eig[(size_t)q * nlev + j] = j < k ? Eh[(size_t)q * M + j] : NAN;
  if (info) {
    info[0] = it;
    info[1] = c64;
    info[2] = c32;
    info[3] = converged ? 1 : 0;
  }
  if (cudaStreamSynchronize(s)) return set_error(c, EVR_EDEVICE, "sync");
  if ((rc = check_item_bounds(c))) return rc;
  return converged ? EVR_OK : set_error(c, EVR_ENOCONV, "evr_batch_davidson: not converged in max_it iterations");
}
