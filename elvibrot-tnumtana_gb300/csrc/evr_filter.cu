// evr_filter.cu -- Gaussian filter diagonalisation on the GPU.
//
// Replaces sub_GaussianFilterDiagonalization
// (Source_ElVibRot/sub_propagation/sub_module_Filter.f90:70-520): L Gaussian filters spread
// over an energy window are applied to start vectors as Chebyshev series of the scaled
// operator, the filtered vectors are orthonormalised and H is diagonalised in their span.
//   * scaling (:155-170): Hmin/Hmax widened by 1 % of the range, E0 = centre, Esc = half
//     range; window LambdaMin = max(Hmin, E0_filter - W/2), LambdaMax = LambdaMin + W;
//   * filter coefficients f(n, l) of exp(-((x - El)/sigma)^2), sigma = W/Esc/L, by the
//     Gauss-Chebyshev rule of gauss_chebyWeight with the weight factor (1-x^2)^(-1/4)
//     sqrt(2/pi) and the kernel damping factor KDF (:300-345, :2538-2579); the series
//     length grown by 10 % from the central window cell's estimate until the tail of the
//     central filter's coefficients is below 1e-8 or it exceeds max_order (:199-283);
//   * the recursion T_0 = q, T_1 = Hs q, T_n = 2 Hs T_(n-1) - T_(n-2) (sub_chebychev_
//     recursion :2221-2298) with z_l += f(n, l) T_n fused into the recurrence kernel, so
//     only three recursion vectors are held (the reference stores every T_n);
//   * sub_Lowdin (S = <z_i|z_j> of the normalised z, eigenvectors in decreasing eigenvalue
//     order, normalised combinations) then sub_Schmidt, here as a QR by the Cholesky factor
//     of the (nearly unit) overlap of the Lowdin vectors, the same span and order;
//   * the vectors with overlap eigenvalue above 1e-9 span the subspace; H_ij = <z_i|H z_j>,
//     non_hermitic = max|H - H^T|/2, H symmetrised (sub_hermitic_H), eigenvalues ascending,
//     residual norms of g_j = sum_i (H z_i - E_j z_i) V_ij (:405-470).
// The reference stops the program after this first diagonalisation; here the call returns
// the Ritz pairs, their residuals and the window counts.  Several start vectors (nstart)
// run in the same H.psi launches, L filtered vectors each.  The projections are the
// deterministic chunked Gram and combination kernels of the Davidson (evr_dense.cuh); the
// small symmetric eigenproblems (at most 512) are solved on the host by Jacobi rotations.
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

struct FBuf {
  double* p = nullptr;
  ~FBuf() {
    if (p) cudaFree(p);
  }
  bool alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(double)) == cudaSuccess; }
};

// Nodes and weights of gauss_chebyWeight (Source_Lib/sub_communf90/sub_math/sub_integration.f90:195-214)
void gauss_cheby_weight(int n, std::vector<double>& x, std::vector<double>& w) {
  const double pi = 3.14159265358979323846, step = pi / n;
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < n; ++i) {
    x[i] = std::cos(-0.5 * step + (i + 1) * step);
    w[i] = step * std::sqrt(1.0 - x[i] * x[i]);
  }
}

// kernel damping factor of coefficient j (1-based) of a series of nb terms
double kdf(int j, int nb) {
  if (j < 2) return 1.0;
  const double pi = 3.14159265358979323846;
  const double r0 = pi / (nb - 1), r = pi * (j - 1) / (nb - 1);
  return (std::cos(r) * (nb - j) + std::sin(r) * std::sin(r0) / std::cos(r0)) / (nb - 1);
}

// f[n + nb*l], n < nb: the Gaussian filters centred at the scaled energies c[l]
std::vector<double> cheby_coefficients(const std::vector<double>& c, double sigma, int nb) {
  std::vector<double> x, w;
  gauss_cheby_weight(nb, x, w);
  const double pi = 3.14159265358979323846;
  std::vector<double> f((size_t)nb * c.size(), 0.0), wfl(nb), p0(nb), p1(nb), p2(nb), sqw(nb);
  for (int k = 0; k < nb; ++k) sqw[k] = 1.0 / std::sqrt(std::sqrt(1.0 - x[k] * x[k])) * std::sqrt(2.0 / pi);
  for (size_t l = 0; l < c.size(); ++l) {
    for (int k = 0; k < nb; ++k) {
      const double d = (x[k] - c[l]) / sigma;
      wfl[k] = std::exp(-d * d) * w[k];
      p0[k] = 1.0;
      p1[k] = x[k];
    }
    double s = 0.0;
    for (int k = 0; k < nb; ++k) s += wfl[k] * p0[k] * sqw[k] / std::sqrt(2.0);
    f[nb * l] = s;
    if (nb > 1) {
      s = 0.0;
      for (int k = 0; k < nb; ++k) s += wfl[k] * p1[k] * sqw[k];
      f[1 + nb * l] = s * kdf(2, nb);
    }
    for (int j = 3; j <= nb; ++j) {
      s = 0.0;
      for (int k = 0; k < nb; ++k) {
        p2[k] = 2.0 * x[k] * p1[k] - p0[k];
        s += wfl[k] * p2[k] * sqw[k];
      }
      f[(j - 1) + nb * l] = s * kdf(j, nb);
      p0.swap(p1);
      p1.swap(p2);
    }
  }
  return f;
}

// Z[r, s*L + l] = f[l] * Q[r, s]
__global__ void filter_init(const double* __restrict__ Q, double* __restrict__ Z, const double* __restrict__ f0,
                            int ns, int L, int64_t N) {
  const int64_t total = N * ns;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / ns;
    const int s = (int)(i - r * ns);
    const double q = Q[i];
    double* z = Z + r * ((int64_t)ns * L) + (int64_t)s * L;
    for (int l = 0; l < L; ++l) z[l] = f0[l] * q;
  }
}

// Tn = (HT - E0 T)/Esc (first) or 2 (HT - E0 T)/Esc - Tp, and Z[r, s*L + l] += fn[l] Tn[r, s]
__global__ void filter_step(const double* __restrict__ Tp, const double* __restrict__ T, const double* __restrict__ HT,
                            double* __restrict__ Tn, double* __restrict__ Z, const double* __restrict__ fn, int ns,
                            int L, int64_t N, double E0, double inv_esc, int first) {
  const int64_t total = N * ns;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    double t = (HT[i] - E0 * T[i]) * inv_esc;
    if (!first) t = 2.0 * t - Tp[i];
    Tn[i] = t;
    const int64_t r = i / ns;
    const int s = (int)(i - r * ns);
    double* z = Z + r * ((int64_t)ns * L) + (int64_t)s * L;
    for (int l = 0; l < L; ++l) z[l] = fma(fn[l], t, z[l]);
  }
}

// X[r, j] *= sc[j]
__global__ void filter_scale(double* __restrict__ X, int k, int64_t N, const double* __restrict__ sc) {
  const int64_t total = N * k;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    X[i] *= sc[i % k];
}

// R[r, j] = HX[r, j] - E[j] X[r, j]
__global__ void filter_residual(const double* __restrict__ X, const double* __restrict__ HX, const double* __restrict__ E,
                                int k, int64_t N, double* __restrict__ R) {
  const int64_t total = N * k;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    R[i] = HX[i] - E[i % k] * X[i];
}

struct Filter {
  evr_ctx* c = nullptr;
  cudaStream_t s = nullptr;
  int64_t N = 0;
  int64_t rows_per_chunk = 0;
  int nchunk = 0, grid = 0;
  FBuf part;
  std::string err;

  int fail(int code, const std::string& m) { return set_error(c, code, "evr_filter_diag: " + m); }
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
  // C (na x nb, ld ldc) = A^T B over the N rows of interleaved blocks
  int gram(const double* A, int lda, const double* B, int ldb, int na, int nb, double* Cm, int ldc) {
    const int tiles = ((na + dense::kTile - 1) / dense::kTile) * ((nb + dense::kTile - 1) / dense::kTile);
    dense::gram_part_kernel<<<dim3(nchunk, tiles), 256, 0, s>>>(A, lda, B, ldb, na, nb, N, rows_per_chunk, part.p);
    dense::gram_reduce_kernel<<<std::min(1024, (na * nb + 255) / 256), 256, 0, s>>>(part.p, nchunk, na, nb, Cm, ldc,
                                                                                   0.0);
    return check("gram");
  }
  // Y(:, 0:k) = X(:, 0:n) Mat(n x k)
  int combine(const double* X, int ldx, int n, const double* Mat, int ldm, int k, double* Y, int ldy) {
    dense::combine_kernel<<<dim3((unsigned)((N + 63) / 64), (unsigned)((k + 31) / 32)), 256, 0, s>>>(
        X, ldx, n, Mat, ldm, k, Y, ldy, 1.0, 0.0, N);
    return check("combine");
  }
  int colnorm2(const double* X, int ldx, int k, double* out) {
    dense::colnorm_part_kernel<<<dim3(nchunk, (k + 31) / 32), dim3(32, 8), 0, s>>>(X, ldx, k, N, rows_per_chunk,
                                                                                    part.p);
    dense::gram_reduce_kernel<<<1, 256, 0, s>>>(part.p, nchunk, k, 1, out, k, 0.0);
    return check("column norms");
  }
  // device matrix (n x m, ld n) to the host
  int to_host(const double* d, size_t n, std::vector<double>& h) {
    h.resize(n);
    if (cudaMemcpyAsync(h.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return fail(EVR_EDEVICE, "copy to host");
    return EVR_OK;
  }
  int to_dev(const std::vector<double>& h, double* d) {
    if (cudaMemcpyAsync(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess)
      return fail(EVR_EDEVICE, "copy to device");
    return EVR_OK;
  }
  // normalises the k columns of X (interleaved, ld k); inverse norms through `sc`
  int normalise(double* X, int k, double* sc) {
    int rc = colnorm2(X, k, k, sc);
    std::vector<double> h;
    if (rc || (rc = to_host(sc, k, h))) return rc;
    for (double& v : h) v = v > 0.0 ? 1.0 / std::sqrt(v) : 0.0;
    if ((rc = to_dev(h, sc))) return rc;
    filter_scale<<<grid, 256, 0, s>>>(X, k, N, sc);
    return check("scale");
  }
};

}  // namespace

extern "C" int evr_filter_diag(evr_ctx* c, const evr_filter_opts* o, const double* q0, double* eig, double* resid,
                               double* vec, int* n_out, double* window, int64_t* info) {
  if (!c || !o || !eig || !n_out) return EVR_EINVAL;
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  const int L = o->n_filters, ns = std::max(o->nstart, 1), K = L * ns;
  const int64_t N = c->hp.Np * c->hp.nb0;
  if (L < 2) return set_error(c, EVR_EINVAL, "evr_filter_diag: n_filters must be at least 2");
  if (K > dense::kMaxEig || K > N) return set_error(c, EVR_EINVAL, "evr_filter_diag: n_filters * nstart above 512 or N");
  if (ns > kMaxBlock) return set_error(c, EVR_EINVAL, "evr_filter_diag: more than 64 start vectors");
  if (!(o->hmax > o->hmin) || !(o->width > 0.0)) return set_error(c, EVR_EINVAL, "evr_filter_diag: bounds or width");
  if (o->max_order < 4) return set_error(c, EVR_EINVAL, "evr_filter_diag: max_order below 4");
  if (o->prec != EVR_PREC_FP64 && o->prec != EVR_PREC_FP32) return set_error(c, EVR_EINVAL, "unknown precision");
  if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, EVR_EDEVICE, "cudaSetDevice");
  const int op = c->op_form == EVR_OP_HT ? OP_HT : (c->op_form == EVR_OP_HSYM ? OP_HSYM : OP_H);

  // ---- scaling, window, filters, series length (:155-345)
  const double pi = 3.14159265358979323846;
  const double d = o->hmax - o->hmin;
  const double lo = o->hmin - 0.01 * d, hi = o->hmax + 0.01 * d;
  const double E0 = lo + 0.5 * (hi - lo), Esc = 0.5 * (hi - lo);
  const double dlam = o->width / (L - 1);
  const double lmin = std::max(o->hmin, o->e0 - 0.5 * o->width), lmax = lmin + o->width;
  const double sigma = o->width / Esc / L;
  const double el = (o->e0 - E0) / Esc;
  const double a = std::max(-1.0, std::min(1.0, el - dlam / Esc / 2.0));
  const double b = std::max(-1.0, std::min(1.0, el + dlam / Esc / 2.0));
  const double nq0 = pi / std::fabs(std::acos(b) - std::acos(a)) / 3.0;
  if (!(nq0 < 1e6)) return set_error(c, EVR_EINVAL, "evr_filter_diag: window cell too narrow (series above 1e6 terms)");
  int nb = std::max(4, (int)nq0);
  while (true) {  // the reference's nb*11/10 does not grow nb below 10: grow by one there
    nb = std::max(nb * 11 / 10, nb + 1);
    const std::vector<double> fc = cheby_coefficients({el}, sigma, nb);
    const double ferr = (std::fabs(fc[nb - 4]) + std::fabs(fc[nb - 3]) + std::fabs(fc[nb - 2]) + std::fabs(fc[nb - 1])) / 3.0;
    if (ferr < 1e-8 || nb > o->max_order) break;
  }
  std::vector<double> centres(L);
  for (int l = 0; l < L; ++l) centres[l] = ((lmin + l * dlam) - E0) / Esc;
  const std::vector<double> f = cheby_coefficients(centres, sigma, nb);  // f[n + nb*l]
  std::vector<double> frows((size_t)nb * L);  // row n: the L coefficients of order n
  for (int n = 0; n < nb; ++n)
    for (int l = 0; l < L; ++l) frows[(size_t)n * L + l] = f[n + (size_t)nb * l];

  Filter F;
  F.c = c;
  F.s = c->stream;
  F.N = N;
  int rc = F.init(K);
  if (rc) return rc;
  cudaStream_t s = F.s;
  FBuf T0, T1, T2, HT, Z, Z2, HZ, X, HX, fr, sc, Cm;
  if (!T0.alloc((size_t)N * ns) || !T1.alloc((size_t)N * ns) || !T2.alloc((size_t)N * ns) ||
      !HT.alloc((size_t)N * ns) || !Z.alloc((size_t)N * K) || !Z2.alloc((size_t)N * K) || !HZ.alloc((size_t)N * K) ||
      !X.alloc((size_t)N * K) || !HX.alloc((size_t)N * K) || !fr.alloc(frows.size()) || !sc.alloc(K) ||
      !Cm.alloc((size_t)K * K))
    return F.fail(EVR_ENOMEM, "device allocation");
  if ((rc = F.to_dev(frows, fr.p))) return rc;

  // ---- start vectors: the caller's (N x ns column-major) or seeded random, normalised
  {
    std::vector<double> q((size_t)N * ns);
    if (q0) {
      for (int64_t r = 0; r < N; ++r)
        for (int j = 0; j < ns; ++j) q[(size_t)r * ns + j] = q0[(size_t)j * N + r];
    } else {
      std::mt19937_64 gen(o->seed);
      for (double& v : q) v = (double)(gen() >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    }
    for (int j = 0; j < ns; ++j) {
      double nn = 0.0;
      for (int64_t r = 0; r < N; ++r) nn += q[(size_t)r * ns + j] * q[(size_t)r * ns + j];
      if (!(nn > 0.0)) return set_error(c, EVR_EINVAL, "evr_filter_diag: zero start vector");
      const double inv = 1.0 / std::sqrt(nn);
      for (int64_t r = 0; r < N; ++r) q[(size_t)r * ns + j] *= inv;
    }
    if ((rc = F.to_dev(q, T0.p))) return rc;
  }
  int64_t nh = 0;
  // ---- Chebyshev recursion with the filtered sums
  filter_init<<<F.grid, 256, 0, s>>>(T0.p, Z.p, fr.p, ns, L, N);
  if ((rc = F.check("filter_init"))) return rc;
  double *tp = T0.p, *tc = T0.p, *tn = T1.p, *spare = T2.p;
  for (int n = 1; n < nb; ++n) {
    if ((rc = hpsi_blocks(c, tc, ns, HT.p, ns, ns, o->prec, s, op))) return rc;
    nh += ns;
    filter_step<<<F.grid, 256, 0, s>>>(tp, tc, HT.p, tn, Z.p, fr.p + (size_t)n * L, ns, L, N, E0, 1.0 / Esc, n == 1);
    if ((rc = F.check("filter_step"))) return rc;
    // rotate: (prev, cur) <- (cur, next); the buffer of the old prev takes the next one
    double* old_prev = (n == 1) ? spare : tp;
    tp = tc;
    tc = tn;
    tn = old_prev;
  }

  // ---- sub_Lowdin: normalise, S, eigenvectors in decreasing order, combine, normalise
  if ((rc = F.normalise(Z.p, K, sc.p))) return rc;
  if ((rc = F.gram(Z.p, K, Z.p, K, K, K, Cm.p, K))) return rc;
  std::vector<double> S, sv, V;
  if ((rc = F.to_host(Cm.p, (size_t)K * K, S))) return rc;
  for (int j = 0; j < K; ++j)
    for (int i = 0; i < j; ++i) S[i + (size_t)K * j] = S[j + (size_t)K * i] = 0.5 * (S[i + (size_t)K * j] + S[j + (size_t)K * i]);
  if (!sym_eig_jacobi(K, S, sv, V)) return F.fail(EVR_ENOCONV, "overlap eigenproblem");
  std::vector<int> ord(K);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int i, int j) { return sv[i] > sv[j]; });
  std::vector<double> Vs((size_t)K * K);
  for (int j = 0; j < K; ++j)
    for (int i = 0; i < K; ++i) Vs[i + (size_t)K * j] = V[i + (size_t)K * ord[j]];
  if ((rc = F.to_dev(Vs, Cm.p))) return rc;
  if ((rc = F.combine(Z.p, K, K, Cm.p, K, K, Z2.p, K))) return rc;
  if ((rc = F.normalise(Z2.p, K, sc.p))) return rc;
  int keep = 0;
  for (int j = 0; j < K; ++j)
    if (std::fabs(sv[ord[j]]) > 1e-9) ++keep;
  if (keep < 1) return F.fail(EVR_ENOCONV, "no filtered vector above the overlap threshold");
  // ---- sub_Schmidt on the kept vectors: Z3 = Z2 R^-1 with S2 = R^T R (Cholesky), twice
  for (int pass = 0; pass < 2; ++pass) {
    if ((rc = F.gram(Z2.p, K, Z2.p, K, keep, keep, Cm.p, keep))) return rc;
    std::vector<double> S2;
    if ((rc = F.to_host(Cm.p, (size_t)keep * keep, S2))) return rc;
    std::vector<double> R((size_t)keep * keep, 0.0);  // upper triangular, column-major
    for (int j = 0; j < keep; ++j) {
      for (int i = 0; i <= j; ++i) {
        double v = S2[i + (size_t)keep * j];
        for (int k = 0; k < i; ++k) v -= R[k + (size_t)keep * i] * R[k + (size_t)keep * j];
        if (i == j) {
          if (!(v > 0.0)) return F.fail(EVR_ENOCONV, "filtered vectors linearly dependent");
          R[i + (size_t)keep * j] = std::sqrt(v);
        } else {
          R[i + (size_t)keep * j] = v / R[i + (size_t)keep * i];
        }
      }
    }
    std::vector<double> Ri((size_t)keep * keep, 0.0);  // R^-1 (upper triangular)
    for (int j = 0; j < keep; ++j) {
      Ri[j + (size_t)keep * j] = 1.0 / R[j + (size_t)keep * j];
      for (int i = j - 1; i >= 0; --i) {
        double v = 0.0;
        for (int k = i + 1; k <= j; ++k) v += R[i + (size_t)keep * k] * Ri[k + (size_t)keep * j];
        Ri[i + (size_t)keep * j] = -v / R[i + (size_t)keep * i];
      }
    }
    if ((rc = F.to_dev(Ri, Cm.p))) return rc;
    if ((rc = F.combine(Z2.p, K, keep, Cm.p, keep, keep, Z.p, K))) return rc;
    std::swap(Z.p, Z2.p);
  }
  // ---- Rayleigh-Ritz in the span of the kept vectors (now in Z2)
  if ((rc = hpsi_blocks(c, Z2.p, K, HZ.p, K, keep, o->prec, s, op))) return rc;
  nh += keep;
  if ((rc = F.gram(Z2.p, K, HZ.p, K, keep, keep, Cm.p, keep))) return rc;
  std::vector<double> Hm;
  if ((rc = F.to_host(Cm.p, (size_t)keep * keep, Hm))) return rc;
  double nonh = 0.0;
  for (int j = 0; j < keep; ++j)
    for (int i = 0; i < keep; ++i) nonh = std::max(nonh, 0.5 * std::fabs(Hm[i + (size_t)keep * j] - Hm[j + (size_t)keep * i]));
  for (int j = 0; j < keep; ++j)
    for (int i = 0; i < j; ++i) Hm[i + (size_t)keep * j] = Hm[j + (size_t)keep * i] = 0.5 * (Hm[i + (size_t)keep * j] + Hm[j + (size_t)keep * i]);
  std::vector<double> ev, U;
  if (!sym_eig_jacobi(keep, Hm, ev, U)) return F.fail(EVR_ENOCONV, "projected eigenproblem");
  std::vector<int> eo(keep);
  std::iota(eo.begin(), eo.end(), 0);
  std::stable_sort(eo.begin(), eo.end(), [&](int i, int j) { return ev[i] < ev[j]; });
  std::vector<double> Us((size_t)keep * keep), es(keep);
  for (int j = 0; j < keep; ++j) {
    es[j] = ev[eo[j]];
    for (int i = 0; i < keep; ++i) Us[i + (size_t)keep * j] = U[i + (size_t)keep * eo[j]];
  }
  if ((rc = F.to_dev(Us, Cm.p))) return rc;
  if ((rc = F.combine(Z2.p, K, keep, Cm.p, keep, keep, X.p, keep))) return rc;
  if ((rc = F.combine(HZ.p, K, keep, Cm.p, keep, keep, HX.p, keep))) return rc;
  if ((rc = F.to_dev(es, sc.p))) return rc;
  filter_residual<<<F.grid, 256, 0, s>>>(X.p, HX.p, sc.p, keep, N, HZ.p);
  if ((rc = F.check("residual"))) return rc;
  if ((rc = F.colnorm2(HZ.p, keep, keep, sc.p))) return rc;
  std::vector<double> r2;
  if ((rc = F.to_host(sc.p, keep, r2))) return rc;

  const double epsi = std::max(o->conv_resi, nonh);
  int inwin = 0, convwin = 0;
  for (int j = 0; j < keep; ++j) {
    eig[j] = es[j];
    const double rn = std::sqrt(std::max(r2[j], 0.0));
    if (resid) resid[j] = rn;
    const bool in = es[j] >= lmin && es[j] <= lmax;
    inwin += in;
    convwin += in && rn < epsi;
  }
  if (vec) {
    FBuf Xc;
    if (!Xc.alloc((size_t)N * keep)) return F.fail(EVR_ENOMEM, "device allocation");
    if ((rc = transpose_from_interleaved(X.p, keep, Xc.p, N, N, keep, s))) return rc;
    if (cudaMemcpyAsync(vec, Xc.p, (size_t)N * keep * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return F.fail(EVR_EDEVICE, "copy of the vectors");
  }
  *n_out = keep;
  if (window) {
    window[0] = lmin;
    window[1] = lmax;
    window[2] = nonh;
  }
  if (info) {
    info[0] = nb;
    info[1] = nh;
    info[2] = keep;
    info[3] = inwin;
    info[4] = convwin;
  }
  return EVR_OK;
}
