// evr_lanczos.cu -- restarted Lanczos on the GPU for the lowest levels (the ARPACK path).
//
// Replaces sub_propagation_Arpack_Sym
// (Source_ElVibRot/sub_propagation/sub_module_Arpack.f90:680-1139).  The reference drives
// ARPACK's dsaupd/dseupd by reverse communication, one OpPsi per request
// (sub_OpV1_TO_V2_Arpack :605-676), with which = 'SM', nev = nb_diago, ncv = 2*nev + 10
// (at most N), tol = 0 (machine precision), exact shifts (ishfts = 1), mode 1 and
// maxitr = min(max_diago, max_it), then reports |H v - E v| / |E| for every converged
// level (:1010-1020).  ARPACK (arpack-ng; not part of the reference's tree, and off in its
// default build: makefile ARPACK = 0) is the implicitly restarted Lanczos method with exact
// shifts (Sorensen 1992; Lehoucq and Sorensen 1996): after a restart the basis spans the
// Krylov space started from the kept Ritz vectors.  The thick restart of Wu and Simon
// (2000), used here, builds the same space directly: the k Ritz vectors of lowest value and
// the last Lanczos vector are kept, the projected matrix becomes diag(theta) bordered by
// the couplings beta*y_m, and Lanczos steps extend the basis to ncv vectors.  Every step
// re-orthogonalises the new vector against the whole basis twice (classical Gram-Schmidt,
// the role of ARPACK's DGKS correction) and takes the projected column from those
// coefficients.  Convergence is ARPACK's test (dsconv): the Ritz bound |beta y_m,i| below
// tol * max(eps^(2/3), |theta_i|), with tol = machine epsilon when 0 is given.  'SM'
// (smallest magnitude) selects the lowest levels of the positive spectra this path is
// used for; the routine targets the lowest (smallest algebraic) levels.
// The H.psi of a step is one vector (as ARPACK's reverse communication); the projections
// and combinations are the deterministic kernels of evr_dense.cuh; the projected matrix
// (at most 512) is diagonalised on the host by Jacobi rotations (evr_krylov.h).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <vector>

#include "evr_dense.cuh"
#include "evr_internal.h"
#include "evr_krylov.h"

using namespace evr;

namespace {

struct LBuf {
  double* p = nullptr;
  ~LBuf() {
    if (p) cudaFree(p);
  }
  bool alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(double)) == cudaSuccess; }
};

// Y[r*ldy + j] = X[r*ldx + j] * sc  (one column)
__global__ void lanczos_scale_col(const double* __restrict__ X, int64_t ldx, double* __restrict__ Y, int64_t ldy,
                                  double sc, int64_t N) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x)
    Y[r * ldy] = X[r * ldx] * sc;
}

// R[r, j] = HX[r, j] - E[j] X[r, j]
__global__ void lanczos_residual(const double* __restrict__ X, const double* __restrict__ HX,
                                 const double* __restrict__ E, int k, int64_t N, double* __restrict__ R) {
  const int64_t total = N * k;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    R[i] = HX[i] - E[i % k] * X[i];
}

struct Lanczos {
  evr_ctx* c = nullptr;
  cudaStream_t s = nullptr;
  int64_t N = 0;
  int64_t rows_per_chunk = 0;
  int nchunk = 0, grid = 0;
  LBuf part;

  int fail(int code, const std::string& m) { return set_error(c, code, "evr_lanczos: " + m); }
  int check(const char* what) {
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? EVR_OK : fail(EVR_EDEVICE, std::string(what) + ": " + cudaGetErrorString(e));
  }
  int init(int kmax) {
    rows_per_chunk = std::max<int64_t>(256, (N + 2 * c->num_sms - 1) / (2 * c->num_sms));
    nchunk = (int)((N + rows_per_chunk - 1) / rows_per_chunk);
    grid = c->num_sms * 8;
    if (!part.alloc((size_t)nchunk * kmax * kmax)) return fail(EVR_ENOMEM, "device allocation");
    return EVR_OK;
  }
  int gram(const double* A, int lda, const double* B, int ldb, int na, int nb, double* Cm, int ldc) {
    const int tiles = ((na + dense::kTile - 1) / dense::kTile) * ((nb + dense::kTile - 1) / dense::kTile);
    dense::gram_part_kernel<<<dim3(nchunk, tiles), 256, 0, s>>>(A, lda, B, ldb, na, nb, N, rows_per_chunk, part.p);
    dense::gram_reduce_kernel<<<std::min(1024, (na * nb + 255) / 256), 256, 0, s>>>(part.p, nchunk, na, nb, Cm, ldc,
                                                                                   0.0);
    return check("gram");
  }
  // Y(:, 0:k) = alpha X(:, 0:n) Mat(n x k) + beta Y
  int combine(const double* X, int ldx, int n, const double* Mat, int ldm, int k, double* Y, int ldy, double alpha,
              double beta) {
    dense::combine_kernel<<<dim3((unsigned)((N + 63) / 64), (unsigned)((k + 31) / 32)), 256, 0, s>>>(
        X, ldx, n, Mat, ldm, k, Y, ldy, alpha, beta, N);
    return check("combine");
  }
  int colnorm2(const double* X, int ldx, int k, double* out) {
    dense::colnorm_part_kernel<<<dim3(nchunk, (k + 31) / 32), dim3(32, 8), 0, s>>>(X, ldx, k, N, rows_per_chunk,
                                                                                    part.p);
    dense::gram_reduce_kernel<<<1, 256, 0, s>>>(part.p, nchunk, k, 1, out, k, 0.0);
    return check("column norms");
  }
  int to_host(const double* d, size_t n, double* h) {
    if (cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return fail(EVR_EDEVICE, "copy to host");
    return EVR_OK;
  }
  int to_dev(const double* h, size_t n, double* d) {
    if (cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess)
      return fail(EVR_EDEVICE, "copy to device");
    return EVR_OK;
  }
};

}  // namespace

extern "C" int evr_lanczos(evr_ctx* c, const evr_lanczos_opts* o, const double* v0, double* eig, double* vec,
                           double* rel_resid, int64_t* info) {
  if (!c || !o || !eig) return EVR_EINVAL;
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  const int64_t N = c->hp.Np * c->hp.nb0;
  const int nev = o->nev;
  if (nev < 1 || nev >= N) return set_error(c, EVR_EINVAL, "evr_lanczos: nev must be in [1, N)");
  int m = o->ncv > 0 ? o->ncv : 2 * nev + 10;
  m = (int)std::min<int64_t>(m, N);
  if (m <= nev) return set_error(c, EVR_EINVAL, "evr_lanczos: ncv must exceed nev (and N)");
  if (m > dense::kMaxEig) return set_error(c, EVR_EINVAL, "evr_lanczos: ncv above 512");
  if (o->max_restarts < 1) return set_error(c, EVR_EINVAL, "evr_lanczos: max_restarts below 1");
  if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, EVR_EDEVICE, "cudaSetDevice");
  const int op = (o->sym > 0 || (o->sym < 0 && !c->hp.symmetric)) ? OP_HSYM : OP_H;
  const double eps = 2.220446049250313e-16;
  const double tol = o->tol > 0.0 ? o->tol : eps;
  const double eps23 = std::pow(eps, 2.0 / 3.0);

  Lanczos L;
  L.c = c;
  L.s = c->stream;
  L.N = N;
  int rc = L.init(m + 1);
  if (rc) return rc;
  cudaStream_t s = L.s;
  const int ldv = m + 1;
  LBuf V, W, h, nrm, Y, X, HX, Ed;
  if (!V.alloc((size_t)N * ldv) || !W.alloc((size_t)N) || !h.alloc(m + 1) || !nrm.alloc(std::max(nev, 1)) ||
      !Y.alloc((size_t)m * m) || !X.alloc((size_t)N * m) || !HX.alloc((size_t)N * nev) || !Ed.alloc(nev))
    return L.fail(EVR_ENOMEM, "device allocation");
  if (cudaMemsetAsync(V.p, 0, sizeof(double) * (size_t)N * ldv, s) != cudaSuccess)
    return L.fail(EVR_EDEVICE, "memset");

  // ---- start vector (the reference's resid: ReadWP0_Arpack, or ARPACK's random one)
  {
    std::vector<double> q(N);
    if (v0) {
      std::copy(v0, v0 + N, q.begin());
    } else {
      std::mt19937_64 gen(o->seed);
      for (double& x : q) x = (double)(gen() >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    }
    double nn = 0.0;
    for (double x : q) nn += x * x;
    if (!(nn > 0.0)) return set_error(c, EVR_EINVAL, "evr_lanczos: zero start vector");
    for (double& x : q) x /= std::sqrt(nn);
    // column 0 of V (interleaved, ld = m+1): through W and a strided copy
    if ((rc = L.to_dev(q.data(), N, W.p))) return rc;
    lanczos_scale_col<<<L.grid, 256, 0, s>>>(W.p, 1, V.p, ldv, 1.0, N);
    if ((rc = L.check("start vector"))) return rc;
  }

  std::vector<double> T((size_t)m * m, 0.0);  // projected matrix (column-major), upper part filled
  std::vector<double> theta, Yh, hcol(m + 1), hc2(m + 1);
  int64_t nh = 0;
  int k = 0, restarts = 0, nconv = 0;
  double beta_last = 0.0;
  while (true) {
    // ---- extend the basis from k to m vectors
    for (int j = k; j < m; ++j) {
      if ((rc = hpsi_blocks(c, V.p + j, ldv, W.p, 1, 1, EVR_PREC_FP64, s, op))) return rc;
      nh += op == OP_HSYM ? 2 : 1;
      // w -= V h twice; the projected column j is the sum of the two passes' coefficients
      std::fill(hcol.begin(), hcol.end(), 0.0);
      for (int pass = 0; pass < 2; ++pass) {
        if ((rc = L.gram(V.p, ldv, W.p, 1, j + 1, 1, h.p, j + 1))) return rc;
        if ((rc = L.combine(V.p, ldv, j + 1, h.p, j + 1, 1, W.p, 1, -1.0, 1.0))) return rc;
        if ((rc = L.to_host(h.p, j + 1, hc2.data()))) return rc;
        for (int i = 0; i <= j; ++i) hcol[i] += hc2[i];
      }
      for (int i = 0; i <= j; ++i) T[i + (size_t)m * j] = hcol[i];
      if ((rc = L.colnorm2(W.p, 1, 1, nrm.p))) return rc;
      double b2 = 0.0;
      if ((rc = L.to_host(nrm.p, 1, &b2))) return rc;
      // with j + 1 == N the basis spans the whole space and w is rounding error: the
      // coupling is zero and the Ritz pairs are exact (ncv = min(N, 2 nev + 10) reaches N
      // on small problems, as in the reference)
      const double beta = j + 1 == N ? 0.0 : std::sqrt(std::max(b2, 0.0));
      beta_last = beta;
      if (j + 1 < m) T[j + (size_t)m * (j + 1)] = beta;  // coupling of v_j and v_(j+1)
      if (!(beta > 0.0)) {  // invariant subspace: the basis cannot grow
        if (j + 1 == m) break;  // full basis: the Ritz pairs are exact (all levels pass the test)
        return L.fail(EVR_ENOCONV, "Lanczos breakdown (invariant subspace of size " + std::to_string(j + 1) + ")");
      }
      lanczos_scale_col<<<L.grid, 256, 0, s>>>(W.p, 1, V.p + (j + 1), ldv, 1.0 / beta, N);
      if ((rc = L.check("next Lanczos vector"))) return rc;
    }
    // ---- Ritz pairs of the projected matrix (symmetric part of the computed columns)
    std::vector<double> A((size_t)m * m);
    for (int j = 0; j < m; ++j)
      for (int i = 0; i <= j; ++i) A[i + (size_t)m * j] = A[j + (size_t)m * i] = T[i + (size_t)m * j];
    if (!sym_eig_jacobi(m, A, theta, Yh)) return L.fail(EVR_ENOCONV, "projected eigenproblem");
    std::vector<int> ord(m);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return theta[a] < theta[b]; });
    std::vector<double> th(m), Ys((size_t)m * m);
    for (int j = 0; j < m; ++j) {
      th[j] = theta[ord[j]];
      for (int i = 0; i < m; ++i) Ys[i + (size_t)m * j] = Yh[i + (size_t)m * ord[j]];
    }
    nconv = 0;
    for (int i = 0; i < nev; ++i)
      if (std::fabs(beta_last * Ys[(m - 1) + (size_t)m * i]) <= tol * std::max(eps23, std::fabs(th[i]))) ++nconv;
    ++restarts;
    const bool done = nconv == nev || restarts >= o->max_restarts;
    // ---- thick restart (or the final Ritz vectors): X = V Y(:, 0:kk)
    const int kk = done ? nev : std::min(m - 1, nev + std::max(1, std::min(nconv, (m - nev) / 2)));
    if ((rc = L.to_dev(Ys.data(), (size_t)m * kk, Y.p))) return rc;
    if ((rc = L.combine(V.p, ldv, m, Y.p, m, kk, X.p, kk, 1.0, 0.0))) return rc;
    if (done) {
      if (eig)
        for (int i = 0; i < nev; ++i) eig[i] = th[i];
      break;
    }
    // V(:, 0:kk) = X; V(:, kk) = v_m; T = diag(theta) bordered by beta y_(m-1, i)
    for (int i = 0; i < kk; ++i) {
      lanczos_scale_col<<<L.grid, 256, 0, s>>>(X.p + i, kk, V.p + i, ldv, 1.0, N);
    }
    lanczos_scale_col<<<L.grid, 256, 0, s>>>(V.p + m, ldv, V.p + kk, ldv, 1.0, N);
    if ((rc = L.check("restart"))) return rc;
    std::fill(T.begin(), T.end(), 0.0);
    for (int i = 0; i < kk; ++i) {
      T[i + (size_t)m * i] = th[i];
      T[i + (size_t)m * kk] = beta_last * Ys[(m - 1) + (size_t)m * i];
    }
    k = kk;
    // the extension recomputes column kk from the re-orthogonalisation coefficients
  }

  // ---- |H x - E x| / |E| of every level (the reference's d(j,2)), and the vectors
  if ((rc = hpsi_blocks(c, X.p, nev, HX.p, nev, nev, EVR_PREC_FP64, s, op))) return rc;
  nh += (int64_t)nev * (op == OP_HSYM ? 2 : 1);
  if ((rc = L.to_dev(eig, nev, Ed.p))) return rc;
  lanczos_residual<<<L.grid, 256, 0, s>>>(X.p, HX.p, Ed.p, nev, N, HX.p);
  if ((rc = L.check("residual"))) return rc;
  if ((rc = L.colnorm2(HX.p, nev, nev, nrm.p))) return rc;
  std::vector<double> r2(nev);
  if ((rc = L.to_host(nrm.p, nev, r2.data()))) return rc;
  if (rel_resid)
    for (int i = 0; i < nev; ++i) rel_resid[i] = std::sqrt(std::max(r2[i], 0.0)) / std::max(std::fabs(eig[i]), 1e-300);
  if (vec) {
    if ((rc = transpose_from_interleaved(X.p, nev, HX.p, N, N, nev, s))) return rc;
    if (cudaMemcpyAsync(vec, HX.p, sizeof(double) * (size_t)N * nev, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return L.fail(EVR_EDEVICE, "copy of the vectors");
  }
  if (info) {
    info[0] = restarts;
    info[1] = nh;
    info[2] = nconv;
    info[3] = m;
  }
  return nconv == nev ? EVR_OK : set_error(c, EVR_ENOCONV, "evr_lanczos: " + std::to_string(nconv) + " of " +
                                                                 std::to_string(nev) + " levels converged");
}
