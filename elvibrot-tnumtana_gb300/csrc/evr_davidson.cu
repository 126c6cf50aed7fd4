// evr_davidson.cu -- block Davidson on the GPU for the lowest levels of H.
//
// Follows sub_propagation_Davidson (Source_ElVibRot/sub_propagation/sub_module_Davidson.f90:54-748):
//   H.psi of the new vectors (sub_MakeHPsi_Davidson :880-1024) -> projected matrix
//   (sub_MakeH_Davidson :1028-1143, symmetrised as sub_hermitic_H) -> dense eigensolve
//   (diagonalization type 3, here a parallel Jacobi kernel on the device) -> residuals
//   g_j = sum_i (H psi_i - E_j psi_i) V_ij (MakeResidual_Davidson :1214-1288) and the
//   convergence tests on |dE| and |g| (:407-449) -> new vectors from the residuals with a
//   diagonal preconditioner (NewVec_type 4, :1424-1445, with the separable harmonic
//   energies as the diagonal) -> two classical Gram-Schmidt passes (:1513-1529) ->
//   restart from the Ritz vectors when the subspace is full (:491-595).
// Everything stays on the device in FP64; the vector blocks use the library's
// interleaved layout (row k of the N x ld block holds component k of every vector).  The
// projections, combinations and the projected eigenproblem are the hand-written,
// deterministic kernels of evr_dense.cuh (no BLAS or LAPACK library).
//
// Mixed precision (prec = EVR_PREC_FP32): the iteration first runs with FP32 contractions
// in H.psi.  When the residuals reach the FP32 floor (or stop decreasing) the subspace is
// collapsed to the n_levels Ritz vectors and only those get an FP64 H.psi.  The iteration
// then goes on with FP32 H.psi for the new directions, while every projected-matrix entry
// that pairs a new direction with one of the FP64 columns is taken from the FP64 side,
// <H psi_exact | t> (H, or (H + H^T)/2, is symmetric): the FP32 error then enters only
// through the components of the Ritz vectors along the new directions, which are of the
// size of the residual at the switch, so the residuals and eigenvalues converge below the
// FP32 floor to the FP64 operator's.  A restart keeps the Ritz vectors and their H.psi as
// FP64 columns; a stall of the refinement recomputes them in FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "evr_dense.cuh"
#include "evr_internal.h"

using namespace evr;

namespace {

struct DevBuf {
  double* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(double)); }
};

// R[k, j] = HX[k, j] - E[j] X[k, j] for j < nt (interleaved, ld = ldk)
__global__ void residual_kernel(const double* __restrict__ X, const double* __restrict__ HX, int64_t ldk,
                                const double* __restrict__ E, int nt, int64_t N, double* __restrict__ R, int64_t ldr) {
  const int64_t total = N * nt;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / nt;
    const int j = (int)(i - r * nt);
    R[r * ldr + j] = HX[r * ldk + j] - E[j] * X[r * ldk + j];
  }
}

// T[k, s] = R[k, sel[s]] / (E[sel[s]] - d[k]) with the denominator kept away from zero
__global__ void precondition_kernel(const double* __restrict__ R, int64_t ldr, const int* __restrict__ sel,
                                    const double* __restrict__ E, const double* __restrict__ d, int ns, int64_t N,
                                    double* __restrict__ T, int64_t ldt, double floor_) {
  const int64_t total = N * ns;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / ns;
    const int s = (int)(i - r * ns);
    const int j = sel[s];
    double den = E[j] - d[r];
    if (fabs(den) < floor_) den = den < 0 ? -floor_ : floor_;
    T[r * ldt + s] = R[r * ldr + j] / den;
  }
}

// Jacobi eigen-decomposition of a small symmetric matrix (host, column-major), ascending.
void small_eigh(int n, std::vector<double> a, std::vector<double>& val, std::vector<double>& vec) {
  vec.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) vec[i + (size_t)n * i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int q = 0; q < n; ++q)
      for (int p = 0; p < n; ++p) {
        tot += a[p + (size_t)n * q] * a[p + (size_t)n * q];
        if (p != q) off += a[p + (size_t)n * q] * a[p + (size_t)n * q];
      }
    if (off <= 1e-30 * tot) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[p + (size_t)n * q];
        if (apq == 0.0) continue;
        const double theta = (a[q + (size_t)n * q] - a[p + (size_t)n * p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < n; ++k) {
          const double x = a[k + (size_t)n * p], y = a[k + (size_t)n * q];
          a[k + (size_t)n * p] = cs * x - sn * y;
          a[k + (size_t)n * q] = sn * x + cs * y;
        }
        for (int k = 0; k < n; ++k) {
          const double x = a[p + (size_t)n * k], y = a[q + (size_t)n * k];
          a[p + (size_t)n * k] = cs * x - sn * y;
          a[q + (size_t)n * k] = sn * x + cs * y;
        }
        for (int k = 0; k < n; ++k) {
          const double x = vec[k + (size_t)n * p], y = vec[k + (size_t)n * q];
          vec[k + (size_t)n * p] = cs * x - sn * y;
          vec[k + (size_t)n * q] = sn * x + cs * y;
        }
      }
  }
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::sort(idx.begin(), idx.end(), [&](int i, int j) { return a[i + (size_t)n * i] < a[j + (size_t)n * j]; });
  val.resize(n);
  std::vector<double> v2((size_t)n * n);
  for (int k = 0; k < n; ++k) {
    val[k] = a[idx[k] + (size_t)n * idx[k]];
    for (int i = 0; i < n; ++i) v2[i + (size_t)n * k] = vec[i + (size_t)n * idx[k]];
  }
  vec.swap(v2);
}

struct Davidson {
  evr_ctx* c;
  cudaStream_t s;
  int64_t N = 0;
  int M = 0;        // max subspace (columns of Pt/HPt)
  int nkeep = 0;    // Ritz vectors kept at a restart
  int bmax = 0;     // new vectors per iteration
  int op = OP_H;
  DevBuf Pt, HPt, X, HX, R, T, Hs, Hw, V, E, C, W, nrm, Tt;
  DevBuf part, wa, wv;   // partial sums of the row chunks; Jacobi working matrices
  int* sel_d = nullptr;
  int* word_d = nullptr;
  int64_t rows_per_chunk = 0;
  int nchunk = 0, jgrid = 0;
  std::string err;

  ~Davidson() {
    if (sel_d) cudaFree(sel_d);
    if (word_d) cudaFree(word_d);
  }

  int fail(int code, const std::string& m) { return set_error(c, code, "evr_davidson: " + m); }

  int init() {
    if (M > dense::kMaxEig) return fail(EVR_EINVAL, "subspace larger than 512 vectors (max_dim)");
    const size_t nm = (size_t)N * M;
    // row chunks of the projections: about two per SM, at least 256 rows each
    rows_per_chunk = std::max<int64_t>(256, (N + 2 * c->num_sms - 1) / (2 * c->num_sms));
    nchunk = (int)((N + rows_per_chunk - 1) / rows_per_chunk);
    const int np = (M + 1) & ~1;
    if (Pt.alloc(nm) || HPt.alloc(nm) || X.alloc((size_t)N * nkeep) || HX.alloc((size_t)N * nkeep) ||
        R.alloc((size_t)N * nkeep) || T.alloc((size_t)N * bmax) || Tt.alloc((size_t)N * bmax) ||
        Hs.alloc((size_t)M * M) || Hw.alloc((size_t)M * M) || V.alloc((size_t)M * M) || E.alloc(M) ||
        C.alloc((size_t)M * bmax) || W.alloc((size_t)bmax * bmax) || nrm.alloc(M) ||
        part.alloc((size_t)nchunk * std::max<int64_t>((int64_t)M * M, nkeep)) || wa.alloc((size_t)np * np) ||
        wv.alloc((size_t)np * np))
      return fail(EVR_ENOMEM, "device allocation");
    if (cudaMalloc(&sel_d, sizeof(int) * bmax) || cudaMalloc(&word_d, sizeof(int) * np))
      return fail(EVR_ENOMEM, "device allocation");
    int coop = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device) != cudaSuccess || !coop)
      return fail(EVR_EDEVICE, "cooperative launch not supported");
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dense::jacobi_coop_kernel, 256, 0) != cudaSuccess ||
        per_sm < 1)
      return fail(EVR_EDEVICE, "Jacobi kernel occupancy");
    jgrid = std::min(32, c->num_sms * per_sm);
    return EVR_OK;
  }

  // C(na x nb) = sum_r A[r, i] * B[r, j] over the N rows of interleaved blocks (+ beta C)
  int gram(const double* A, int lda, const double* B, int ldb, int na, int nb, double* Cm, int ldc, double beta = 0.0) {
    if (na < 1 || nb < 1) return EVR_OK;
    const int tiles = ((na + dense::kTile - 1) / dense::kTile) * ((nb + dense::kTile - 1) / dense::kTile);
    dense::gram_part_kernel<<<dim3(nchunk, tiles), 256, 0, s>>>(A, lda, B, ldb, na, nb, N, rows_per_chunk, part.p);
    dense::gram_reduce_kernel<<<std::min(1024, (na * nb + 255) / 256), 256, 0, s>>>(part.p, nchunk, na, nb, Cm, ldc,
                                                                                   beta);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? EVR_OK : fail(EVR_EDEVICE, std::string("gram: ") + cudaGetErrorString(e));
  }

  // Y(:, 0:k) = alpha * X_block(:, 0:n) * Mat(n x k) + beta * Y   (interleaved blocks)
  int combine(const double* Xb, int ldx, int n, const double* Mat, int ldm, int k, double* Y, int ldy, double alpha,
              double beta) {
    if (k < 1) return EVR_OK;
    dense::combine_kernel<<<dim3((unsigned)((N + 63) / 64), (unsigned)((k + 31) / 32)), 256, 0, s>>>(
        Xb, ldx, n, Mat, ldm, k, Y, ldy, alpha, beta, N);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? EVR_OK : fail(EVR_EDEVICE, std::string("combine: ") + cudaGetErrorString(e));
  }

  // squared norms of the k columns of an interleaved block into out[0..k)
  int colnorm2(const double* Xb, int ldx, int k, double* out) {
    dense::colnorm_part_kernel<<<dim3(nchunk, (k + 31) / 32), dim3(32, 8), 0, s>>>(Xb, ldx, k, N, rows_per_chunk,
                                                                                    part.p);
    dense::gram_reduce_kernel<<<1, 256, 0, s>>>(part.p, nchunk, k, 1, out, k, 0.0);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? EVR_OK : fail(EVR_EDEVICE, std::string("column norms: ") + cudaGetErrorString(e));
  }

  // eigenvalues (ascending) and eigenvectors of the symmetric part of A (n x n, ld M)
  int eigh(const double* A, int n, double* Wv, double* Vm) {
    int nn = n, lda = M, ldv = M, sweeps = 40;
    double tol = 1e-15;
    double* wap = wa.p;
    double* wvp = wv.p;
    int* wop = word_d;
    void* args[] = {(void*)&A, &lda, &nn, &Wv, &Vm, &ldv, &wap, &wvp, &wop, &sweeps, &tol};
    const cudaError_t e =
        cudaLaunchCooperativeKernel((const void*)dense::jacobi_coop_kernel, dim3(jgrid), dim3(256), args, 0, s);
    return e == cudaSuccess ? EVR_OK : fail(EVR_EDEVICE, std::string("Jacobi launch: ") + cudaGetErrorString(e));
  }

  int hop(const double* x, int ldx, double* y, int ldy, int n, int prec, int64_t& cnt64, int64_t& cnt32) {
    int rc = hpsi_blocks(c, x, ldx, y, ldy, n, prec, s, op);
    if (rc) return rc;
    (prec == EVR_PREC_FP32 ? cnt32 : cnt64) += n * (op == OP_HSYM ? 2 : 1);
    return EVR_OK;
  }

  // Orthonormalise the ns vectors of the interleaved block Tb (ld = bmax) against the
  // first n1 columns of Pt (two classical Gram-Schmidt passes) and among themselves
  // (symmetric orthonormalisation of their Gram matrix, dropping dependent directions);
  // the accepted vectors are written to Pt columns n1.. and their count returned in `added`.
  int orthonormalize(double* Tb, int ns, int n1, int& added) {
    added = 0;
    std::vector<double> G((size_t)ns * ns), val, vec;
    for (int pass = 0; pass < 2; ++pass) {
      if (n1 > 0) {
        int rc = gram(Pt.p, M, Tb, bmax, n1, ns, C.p, M);  // C = Psi^T T   (n1 x ns)
        if (rc) return rc;
        rc = combine(Pt.p, M, n1, C.p, M, ns, Tb, bmax, -1.0, 1.0);  // T -= Psi C
        if (rc) return rc;
      }
      int rc = gram(Tb, bmax, Tb, bmax, ns, ns, W.p, bmax);
      if (rc) return rc;
      std::vector<double> Wh((size_t)bmax * ns);
      if (cudaMemcpyAsync(Wh.data(), W.p, sizeof(double) * bmax * ns, cudaMemcpyDeviceToHost, s) ||
          cudaStreamSynchronize(s))
        return fail(EVR_EDEVICE, "copy gram");
      for (int j = 0; j < ns; ++j)
        for (int i = 0; i < ns; ++i) G[i + (size_t)ns * j] = Wh[i + (size_t)bmax * j];
      small_eigh(ns, G, val, vec);
      const double vmax = std::max(val.back(), 1e-300);
      // keep directions with relative weight above 1e-12 (the reference drops |psi|^2 < 1e-10)
      std::vector<int> keep;
      for (int k = ns - 1; k >= 0; --k)
        if (val[k] > 1e-12 * vmax && val[k] > 1e-280) keep.push_back(k);
      const int nk = (int)keep.size();
      if (nk == 0) return EVR_OK;
      std::vector<double> Mh((size_t)bmax * nk, 0.0);  // T_new = T U_k / sqrt(lambda_k)
      for (int j = 0; j < nk; ++j)
        for (int i = 0; i < ns; ++i) Mh[i + (size_t)bmax * j] = vec[i + (size_t)ns * keep[j]] / std::sqrt(val[keep[j]]);
      if (cudaMemcpyAsync(W.p, Mh.data(), sizeof(double) * bmax * nk, cudaMemcpyHostToDevice, s))
        return fail(EVR_EDEVICE, "copy");
      rc = combine(Tb, bmax, ns, W.p, bmax, nk, Tt.p, bmax, 1.0, 0.0);
      if (rc) return rc;
      if (cudaMemcpyAsync(Tb, Tt.p, sizeof(double) * N * bmax, cudaMemcpyDeviceToDevice, s))
        return fail(EVR_EDEVICE, "copy");
      ns = nk;
    }
    if (n1 + ns > M) ns = M - n1;
    if (cudaMemcpy2DAsync(Pt.p + n1, sizeof(double) * M, Tb, sizeof(double) * bmax, sizeof(double) * ns, N,
                          cudaMemcpyDeviceToDevice, s))
      return fail(EVR_EDEVICE, "append");
    added = ns;
    return EVR_OK;
  }

  // Projected matrix rows/cols n0..n1, eigen-decomposition of the leading n1 x n1 block.
  // Columns 0..ke-1 carry an FP64 H.psi: their rows of the new block are <H psi_i|psi_j>.
  int rayleigh_ritz(int n0, int n1, std::vector<double>& Eh, int ke = 0) {
    int rc = gram(Pt.p, M, HPt.p + n0, M, n1, n1 - n0, Hs.p + (size_t)M * n0, M);  // Hs(0:n1, n0:n1)
    if (rc) return rc;
    const int kx = std::min(ke, n0);
    if (kx > 0 && (rc = gram(HPt.p, M, Pt.p + n0, M, kx, n1 - n0, Hs.p + (size_t)M * n0, M))) return rc;
    // mirror the new columns into the new rows: Hs(n0:n1, 0:n0) = Hs(0:n0, n0:n1)^T
    if (n0 > 0) dense::mirror_kernel<<<64, 256, 0, s>>>(Hs.p, M, n0, n1);
    // eigenpairs of the symmetric part (sub_hermitic_H), eigenvectors into Hw
    if ((rc = eigh(Hs.p, n1, E.p, Hw.p))) return rc;
    Eh.resize(n1);
    if (cudaMemcpyAsync(Eh.data(), E.p, sizeof(double) * n1, cudaMemcpyDeviceToHost, s) || cudaStreamSynchronize(s))
      return fail(EVR_EDEVICE, "copy eigenvalues");
    return EVR_OK;
  }
};

}  // namespace

extern "C" int evr_davidson(evr_ctx* c, const evr_davidson_opts* o, const double* guess, double* eig, double* vec,
                            int64_t* info) {
  if (!c || !o || !eig) return EVR_EINVAL;
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  const int64_t N = c->hp.Np * c->hp.nb0;
  const int nlev = o->n_levels;
  int b = std::min(std::max(o->block, 1), kMaxBlock);
  if (nlev < 1 || nlev > N) return set_error(c, EVR_EINVAL, "evr_davidson: n_levels out of range");
  if (o->prec != EVR_PREC_FP64 && o->prec != EVR_PREC_FP32) return set_error(c, EVR_EINVAL, "unknown precision");
  if (o->n_guess < 0 || (o->n_guess > 0 && !guess)) return set_error(c, EVR_EINVAL, "guess");
  if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, EVR_EDEVICE, "cudaSetDevice");
  Davidson d;
  d.c = c;
  d.s = c->stream;
  d.N = N;
  d.bmax = b;
  d.nkeep = (int)std::min<int64_t>(N, nlev + b);
  d.M = (int)std::min<int64_t>(N, std::max(o->max_dim, d.nkeep + b));
  d.op = (o->sym > 0 || (o->sym < 0 && !c->hp.symmetric)) ? OP_HSYM : OP_H;
  int rc = d.init();
  if (rc) return rc;
  const int M = d.M;
  cudaStream_t s = d.s;

  // ---- initial space: guess vectors (ReadWP0_Davidson :752-878), or unit vectors on the
  // lowest zero-order energies; added in chunks of bmax vectors
  int n1 = 0, n0 = 0, added = 0;
  {
    const int ninit = o->n_guess > 0 ? std::min(o->n_guess, M - d.bmax)
                                     : (int)std::min<int64_t>(N, std::min(std::max(nlev, b), M - d.bmax));
    std::vector<int> idx;
    if (o->n_guess == 0) {
      idx.resize(N);
      std::iota(idx.begin(), idx.end(), 0);
      const std::vector<double>& e0 = c->hp.e0diag;
      std::partial_sort(idx.begin(), idx.begin() + ninit, idx.end(), [&](int a, int bb) { return e0[a] < e0[bb]; });
    }
    DevBuf g;
    if (o->n_guess > 0 && g.alloc((size_t)N * d.bmax)) return set_error(c, EVR_ENOMEM, "guess");
    const double one = 1.0;
    for (int j0 = 0; j0 < ninit; j0 += d.bmax) {
      const int nc = std::min(d.bmax, ninit - j0);
      if (o->n_guess > 0) {
        if (cudaMemcpyAsync(g.p, guess + (size_t)j0 * N, sizeof(double) * N * nc, cudaMemcpyHostToDevice, s))
          return set_error(c, EVR_EDEVICE, "guess copy");
        if ((rc = transpose_to_interleaved(g.p, N, d.T.p, d.bmax, N, nc, s))) return set_error(c, rc, "transpose");
      } else {
        if (cudaMemsetAsync(d.T.p, 0, sizeof(double) * N * d.bmax, s)) return set_error(c, EVR_EDEVICE, "memset");
        for (int j = 0; j < nc; ++j)
          if (cudaMemcpyAsync(d.T.p + (size_t)idx[j0 + j] * d.bmax + j, &one, sizeof(double), cudaMemcpyHostToDevice,
                              s))
            return set_error(c, EVR_EDEVICE, "init");
      }
      if (cudaStreamSynchronize(s)) return set_error(c, EVR_EDEVICE, "sync");
      if ((rc = d.orthonormalize(d.T.p, nc, n1, added))) return rc;
      n1 += added;
    }
    if (n1 == 0) return set_error(c, EVR_EINVAL, "evr_davidson: empty initial space");
  }
  // grow the start space to nlev vectors with preconditioned residual blocks if needed
  int prec = o->prec;
  int64_t cnt64 = 0, cnt32 = 0;
  std::vector<double> Eh, Eold(nlev, 1e300), rnorm(d.nkeep, 0.0);
  double best_r = 1e300;
  int stall = 0, it = 0;
  bool converged = false;
  bool refine = false;  // mixed precision after the switch: FP64 columns 0..ke-1, FP32 H.psi for the others
  int ke = 0;
  for (it = 0; it < o->max_it; ++it) {
    // H.psi of the new vectors (FP64 for the columns a switch or refresh marked exact)
    if (refine && n0 < ke) {
      if ((rc = d.hop(d.Pt.p + n0, M, d.HPt.p + n0, M, ke - n0, EVR_PREC_FP64, cnt64, cnt32))) return rc;
      if (n1 > ke && (rc = d.hop(d.Pt.p + ke, M, d.HPt.p + ke, M, n1 - ke, EVR_PREC_FP32, cnt64, cnt32))) return rc;
    } else if ((rc = d.hop(d.Pt.p + n0, M, d.HPt.p + n0, M, n1 - n0, prec, cnt64, cnt32))) {
      return rc;
    }
    if ((rc = d.rayleigh_ritz(n0, n1, Eh, refine ? ke : 0))) return rc;
    n0 = n1;
    const int k = std::min(d.nkeep, n1);
    // Ritz vectors and H applied to them
    if ((rc = d.combine(d.Pt.p, M, n1, d.Hw.p, M, k, d.X.p, d.nkeep, 1.0, 0.0))) return rc;
    if ((rc = d.combine(d.HPt.p, M, n1, d.Hw.p, M, k, d.HX.p, d.nkeep, 1.0, 0.0))) return rc;
    residual_kernel<<<c->num_sms * 8, 256, 0, s>>>(d.X.p, d.HX.p, d.nkeep, d.E.p, k, N, d.R.p, d.nkeep);
    if ((rc = d.colnorm2(d.R.p, d.nkeep, k, d.nrm.p))) return rc;
    if (cudaMemcpyAsync(rnorm.data(), d.nrm.p, sizeof(double) * k, cudaMemcpyDeviceToHost, s) ||
        cudaStreamSynchronize(s))
      return set_error(c, EVR_EDEVICE, "evr_davidson: residual norms");
    const int nt = std::min(nlev, k);
    double rmax = 0.0, demax = 0.0;
    std::vector<int> todo;
    for (int j = 0; j < nt; ++j) {
      rnorm[j] = std::sqrt(rnorm[j]);
      const double de = std::fabs(Eh[j] - Eold[j]);
      rmax = std::max(rmax, rnorm[j]);
      demax = std::max(demax, de);
      if (!(rnorm[j] < o->conv_resi && de < o->conv_ene)) todo.push_back(j);
    }
    for (int j = 0; j < nt; ++j) Eold[j] = Eh[j];
    if (nt == nlev && todo.empty()) {
      if (prec == EVR_PREC_FP64 || refine) {
        converged = true;
        break;
      }
    }
    // FP32 phase -> refinement: residual floor of the FP32 operator reached or stalled;
    // in the refinement a stall recomputes the Ritz vectors' H.psi in FP64
    if (prec == EVR_PREC_FP32) {
      // the refinement converges at the rate of the FP64 iteration, so the FP32 phase ends
      // early: at a residual of 1e-4 of the level energies or when it stops halving
      const double hscale = std::max(std::fabs(Eh.front()), std::fabs(Eh.back()));
      const bool floor_hit = !refine && rmax < std::max(o->conv_resi, 1e-4 * hscale);
      if (rmax < (refine ? 0.7 : 0.5) * best_r) { best_r = rmax; stall = 0; } else ++stall;
      if (floor_hit || stall >= (refine ? 3 : 1) || (!refine && todo.empty())) {
        // restart on the lowest n_levels Ritz vectors, H.psi of those in FP64
        const int kr = std::min(k, nlev);
        if (cudaMemcpy2DAsync(d.Pt.p, sizeof(double) * M, d.X.p, sizeof(double) * d.nkeep, sizeof(double) * kr, N,
                              cudaMemcpyDeviceToDevice, s))
          return set_error(c, EVR_EDEVICE, "restart copy");
        refine = true;
        ke = kr;
        n1 = kr;
        n0 = 0;
        std::fill(Eold.begin(), Eold.end(), 1e300);
        best_r = 1e300;
        stall = 0;
        continue;
      }
    }
    // new vectors: preconditioned residuals of the lowest unconverged targets; while the
    // subspace holds fewer than nlev Ritz pairs every target contributes
    if (nt < nlev) {
      todo.clear();
      for (int j = 0; j < nt; ++j)
        if (rnorm[j] > 1e-14 * std::max(1.0, std::fabs(Eh[j]))) todo.push_back(j);
    }
    if ((int)todo.size() > d.bmax) todo.resize(d.bmax);
    const int ns = (int)todo.size();
    if (ns == 0) break;
    if (cudaMemcpyAsync(d.sel_d, todo.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s))
      return set_error(c, EVR_EDEVICE, "copy");
    precondition_kernel<<<c->num_sms * 8, 256, 0, s>>>(d.R.p, d.nkeep, d.sel_d, d.E.p, c->dp.e0diag, ns, N, d.T.p,
                                                       d.bmax, 1e-3 * std::max(1e-300, std::fabs(Eh[0])) + 1e-12);
    // restart when the subspace would overflow.  In the refinement the restart is a refresh:
    // the Ritz vectors' H.psi combines FP32 columns, so it is recomputed in FP64 before the
    // kept columns serve as exact ones (the FP64 side of the mixed products)
    if (n1 + ns > M && refine) {
      const int kr = std::min(k, nlev);
      if (cudaMemcpy2DAsync(d.Pt.p, sizeof(double) * M, d.X.p, sizeof(double) * d.nkeep, sizeof(double) * kr, N,
                            cudaMemcpyDeviceToDevice, s))
        return set_error(c, EVR_EDEVICE, "restart copy");
      ke = kr;
      n1 = kr;
      n0 = 0;
      continue;
    }
    if (n1 + ns > M) {
      if (cudaMemcpy2DAsync(d.Pt.p, sizeof(double) * M, d.X.p, sizeof(double) * d.nkeep, sizeof(double) * k, N,
                            cudaMemcpyDeviceToDevice, s) ||
          cudaMemcpy2DAsync(d.HPt.p, sizeof(double) * M, d.HX.p, sizeof(double) * d.nkeep, sizeof(double) * k, N,
                            cudaMemcpyDeviceToDevice, s))
        return set_error(c, EVR_EDEVICE, "restart copy");
      // projected matrix of the Ritz basis is diag(E)
      if (cudaMemsetAsync(d.Hs.p, 0, sizeof(double) * M * M, s)) return set_error(c, EVR_EDEVICE, "memset");
      for (int j = 0; j < k; ++j)
        if (cudaMemcpyAsync(d.Hs.p + j + (size_t)M * j, &Eh[j], sizeof(double), cudaMemcpyHostToDevice, s))
          return set_error(c, EVR_EDEVICE, "copy");
      if (cudaStreamSynchronize(s)) return set_error(c, EVR_EDEVICE, "sync");
      n1 = n0 = k;
      ke = k;  // Ritz vectors and their H.psi: FP64 columns of the refinement
    }
    if ((rc = d.orthonormalize(d.T.p, ns, n1, added))) return rc;
    if (added == 0) break;  // no new direction: converged as far as the operator allows
    n1 += added;
  }
  // results
  const int k = std::min(d.nkeep, n1);
  for (int j = 0; j < nlev; ++j) eig[j] = j < (int)Eh.size() ? Eh[j] : NAN;
  if (vec) {
    const int nv = std::min(nlev, k);
    DevBuf out;
    if (out.alloc((size_t)N * nv)) return set_error(c, EVR_ENOMEM, "output");
    if ((rc = transpose_from_interleaved(d.X.p, d.nkeep, out.p, N, N, nv, s))) return set_error(c, rc, "transpose");
    if (cudaMemcpyAsync(vec, out.p, sizeof(double) * N * nv, cudaMemcpyDeviceToHost, s) || cudaStreamSynchronize(s))
      return set_error(c, EVR_EDEVICE, "copy vectors");
  }
  if (info) {
    info[0] = it;
    info[1] = cnt64;
    info[2] = cnt32;
    info[3] = converged ? 1 : 0;
  }
  if (cudaStreamSynchronize(s)) return set_error(c, EVR_EDEVICE, "sync");
  if ((rc = check_item_bounds(c))) return rc;
  return converged ? EVR_OK : set_error(c, EVR_ENOCONV, "evr_davidson: not converged in max_it iterations");
}
