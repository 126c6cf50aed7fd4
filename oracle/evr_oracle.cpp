// evr_oracle.cpp -- CPU oracle for the ElVibRot-TnumTana H.psi hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, loop for loop, the reference's
// Fortran algorithm for OpPsi on Smolyak (SG4) and direct-product bases so that
// the CUDA library can be checked against it.  Only tests/, the smoke check of
// __graft_entry__.py and the cpu_baseline leg of bench.py load it; the product
// library never links, loads or calls it.
//
// Parity pins (tests/test_oracle_golden.py):
//   * Gauss-Hermite nodes/weights against Internal_data/HermQuadra/herm<n>.txt
//   * 6-D Henon-Heiles SG4 spectrum against Working_tests/MPI_tests/6D_Davidson_S0/benchmark
//   * 12-D pyrazine SG4 autocorrelation against Working_tests/MPI_tests/12D_propagation_S0/benchmark
//
// Every function cites the reference file:line it restates (paths relative to
// the reference project root).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <vector>
#include <string>
#include <unordered_map>
#include <algorithm>
#include <omp.h>

namespace {

typedef long double LD;

// ---------------------------------------------------------------------------
// 1-D Gauss-Hermite rule.  The reference reads x (column 2) and w*exp(x^2)
// (column 4) from Internal_data/HermQuadra/herm<nq>.txt
// (Source_ElVibRot/sub_Basis/sub_quadra_herm.f90:322-343).  The oracle computes
// the same rule from the Jacobi matrix of the Hermite polynomials (eigenvalues
// by Sturm bisection, Newton polish, weights from the Christoffel function),
// all in long double; the golden test checks it against the tables.
// ---------------------------------------------------------------------------
static int sturm_count(int n, const std::vector<LD>& off2, LD x) {
  // number of eigenvalues of the symmetric tridiagonal (0 diag, off) below x
  int cnt = 0;
  LD q = -x;  // d_1 - x with d = 0
  if (q < 0) cnt++;
  for (int k = 1; k < n; ++k) {
    LD qq = (q == 0) ? 1e-300L : q;
    q = -x - off2[k - 1] / qq;
    if (q < 0) cnt++;
  }
  return cnt;
}

// orthonormal Hermite functions phi_k(x) = H_k(x) e^{-x^2/2} / sqrt(2^k k! sqrt(pi))
static void herm_functions(int n, LD x, std::vector<LD>& phi) {
  phi.assign(n, 0.0L);
  LD e = expl(-0.5L * x * x);
  LD p0 = e / sqrtl(sqrtl(3.14159265358979323846264338327950288L));
  phi[0] = p0;
  if (n > 1) phi[1] = sqrtl(2.0L) * x * p0;
  for (int k = 2; k < n; ++k)
    phi[k] = sqrtl(2.0L / k) * x * phi[k - 1] - sqrtl((LD)(k - 1) / k) * phi[k - 2];
}

static void gauss_hermite(int n, std::vector<double>& x, std::vector<double>& wexp) {
  x.assign(n, 0.0);
  wexp.assign(n, 0.0);
  if (n == 1) {
    x[0] = 0.0;
    wexp[0] = (double)sqrtl(3.14159265358979323846264338327950288L);
    return;
  }
  std::vector<LD> off2(n - 1);
  for (int k = 1; k < n; ++k) off2[k - 1] = (LD)k / 2.0L;
  LD bound = sqrtl(2.0L * n + 2.0L) + 1.0L;
  std::vector<LD> phi;
  for (int i = 0; i < n; ++i) {
    LD lo = -bound, hi = bound;
    for (int it = 0; it < 200; ++it) {  // i-th eigenvalue: count(<mid) > i
      LD mid = 0.5L * (lo + hi);
      if (sturm_count(n, off2, mid) > i) hi = mid; else lo = mid;
    }
    LD xi = 0.5L * (lo + hi);
    // Newton polish on phi_n(x) = 0 using phi_n' = sqrt(2n) phi_{n-1} - x phi_n
    for (int it = 0; it < 3; ++it) {
      herm_functions(n + 1, xi, phi);
      LD f = phi[n], fp = sqrtl(2.0L * n) * phi[n - 1] - xi * phi[n];
      if (fp != 0) xi -= f / fp;
    }
    herm_functions(n, xi, phi);
    LD s = 0;
    for (int k = 0; k < n; ++k) s += phi[k] * phi[k];
    x[i] = (double)xi;
    wexp[i] = (double)(1.0L / s);
  }
  // exact symmetry of the rule
  for (int i = 0; i < n / 2; ++i) {
    double a = 0.5 * (x[n - 1 - i] - x[i]);
    x[i] = -a; x[n - 1 - i] = a;
    double w = 0.5 * (wexp[i] + wexp[n - 1 - i]);
    wexp[i] = w; wexp[n - 1 - i] = w;
  }
  if (n % 2) x[n / 2] = 0.0;
}

// ---------------------------------------------------------------------------
// Normalised Hermite polynomial and its exp(-x^2/2) derivatives.
// Restates poly_Hermite (Source_Lib/sub_communf90/sub_math/sub_polyortho.f90:830-878)
// and d0d1d2poly_Hermite_exp (same file :1060-1131).
// ---------------------------------------------------------------------------
static double poly_hermite(double x, int l) {
  const double pi = 3.14159265358979323846;
  double norme = std::sqrt(pi);
  if (l == 0) return 1.0 / std::sqrt(norme);
  if (l == 1) { norme *= 2.0; return 2.0 * x / std::sqrt(norme); }
  double pl2 = 1.0, pl1 = 2.0 * x, pl0 = 0.0;
  norme *= 2.0;
  for (int i = 2; i <= l; ++i) {
    norme *= 2.0 * (double)i;
    pl0 = 2.0 * (x * pl1 - (double)(i - 1) * pl2);
    pl2 = pl1; pl1 = pl0;
  }
  return pl0 / std::sqrt(norme);
}

static void hermite_exp(double x, int l, double& d0, double& d1, double& d2) {
  d0 = poly_hermite(x, l);
  if (l == 0) { d1 = 0.0; d2 = 0.0; }
  else if (l == 1) { d1 = std::sqrt(2.0) * poly_hermite(x, 0); d2 = 0.0; }
  else {
    d1 = std::sqrt(2.0 * (double)l) * poly_hermite(x, l - 1);
    d2 = 2.0 * (x * d1 - d0 * (double)l);
  }
  double pexp = std::exp(-0.5 * x * x);
  d2 = (d2 - 2.0 * x * d1 + (x * x - 1.0) * d0) * pexp;
  d1 = (d1 - x * d0) * pexp;
  d0 = d0 * pexp;
}

// ---------------------------------------------------------------------------
// Cyclic Jacobi eigen-solver for a small symmetric matrix (column-major).
// Stands in for the reference's diagonalization(...,3,-1) call used by
// sub_dnGB_TO_dnGG (Source_ElVibRot/sub_Basis/sub_module_basis.f90:2254); the
// eigenvectors are returned sorted by DECREASING eigenvalue as sort=-1 asks.
// ---------------------------------------------------------------------------
static void jacobi_eig(int n, std::vector<double> a, std::vector<double>& val, std::vector<double>& vec) {
  vec.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) vec[i + (size_t)n * i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int q = 0; q < n; ++q) for (int p = 0; p < q; ++p) off += a[p + (size_t)n * q] * a[p + (size_t)n * q];
    if (off < 1e-300) break;
    for (int p = 0; p < n - 1; ++p) for (int q = p + 1; q < n; ++q) {
      double apq = a[p + (size_t)n * q];
      if (std::fabs(apq) < 1e-300) continue;
      double app = a[p + (size_t)n * p], aqq = a[q + (size_t)n * q];
      double theta = (aqq - app) / (2.0 * apq);
      double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
      double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
      for (int k = 0; k < n; ++k) {  // columns p,q
        double akp = a[k + (size_t)n * p], akq = a[k + (size_t)n * q];
        a[k + (size_t)n * p] = c * akp - s * akq;
        a[k + (size_t)n * q] = s * akp + c * akq;
      }
      for (int k = 0; k < n; ++k) {  // rows p,q
        double apk = a[p + (size_t)n * k], aqk = a[q + (size_t)n * k];
        a[p + (size_t)n * k] = c * apk - s * aqk;
        a[q + (size_t)n * k] = s * apk + c * aqk;
      }
      for (int k = 0; k < n; ++k) {
        double vkp = vec[k + (size_t)n * p], vkq = vec[k + (size_t)n * q];
        vec[k + (size_t)n * p] = c * vkp - s * vkq;
        vec[k + (size_t)n * q] = s * vkp + c * vkq;
      }
    }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int i, int j) { return a[i + (size_t)n * i] > a[j + (size_t)n * j]; });
  val.assign(n, 0.0);
  std::vector<double> v2((size_t)n * n);
  for (int k = 0; k < n; ++k) {
    val[k] = a[idx[k] + (size_t)n * idx[k]];
    for (int i = 0; i < n; ++i) v2[i + (size_t)n * k] = vec[i + (size_t)n * idx[k]];
  }
  vec.swap(v2);
}

// ---------------------------------------------------------------------------
// One primitive HO basis at one Smolyak level (tab_basisPrimSG(L,ib)).
// Matrices are column-major as in the Fortran: d0b(nq,nb), bgw(nb,nq), gg(nq,nq).
// ---------------------------------------------------------------------------
struct Basis1D {
  int nb = 0, nq = 0;
  std::vector<double> x, w;          // scaled grid and weights (wrho = w, rho = 1)
  std::vector<double> d0b, d1b, d2b; // dnRGB%d0,d1,d2 (nq x nb)
  std::vector<double> bgw;           // dnRBGwrho%d0 (nb x nq)
  std::vector<double> d1gg, d2gg;    // dnRGG%d1, dnRGG%d2 (nq x nq)
};

// construct_primitive_basis (Source_ElVibRot/sub_Basis/sub_module_basis.f90:391-782):
// sub_quadra_hermite (sub_quadra_herm.f90:208-411), sub_scale_basis (:1540-1638),
// sub_dnGB_TO_dnGG (:2195-2460, pseudo-inverse through the eigenpairs of
// d0b.d0b^T), sub_dnGB_TO_dnBG (:2062-2160).
static void build_basis(Basis1D& b, int nb, int nq, double scaleQ, double Q0) {
  b.nb = nb; b.nq = nq;
  gauss_hermite(nq, b.x, b.w);
  b.d0b.assign((size_t)nq * nb, 0.0); b.d1b = b.d0b; b.d2b = b.d0b;
  for (int k = 0; k < nq; ++k)
    for (int i = 0; i < nb; ++i)
      hermite_exp(b.x[k], i, b.d0b[k + (size_t)nq * i], b.d1b[k + (size_t)nq * i], b.d2b[k + (size_t)nq * i]);
  // scaling
  if (!(Q0 == 0.0 && scaleQ == 1.0)) {
    double sq = std::sqrt(scaleQ);
    for (int k = 0; k < nq; ++k) { b.x[k] = Q0 + b.x[k] / scaleQ; b.w[k] = b.w[k] * (1.0 / scaleQ); }
    for (auto& v : b.d0b) v *= sq;
    for (auto& v : b.d1b) v *= sq * scaleQ;
    for (auto& v : b.d2b) v *= sq * scaleQ * scaleQ;
  }
  // pseudo-inverse of d0b: P = d0b^T . (sum_{k<=nb} v_k v_k^T / lambda_k)
  std::vector<double> m((size_t)nq * nq, 0.0);
  for (int i = 0; i < nq; ++i) for (int j = 0; j < nq; ++j) {
    double s = 0.0;
    for (int k = 0; k < nb; ++k) s += b.d0b[i + (size_t)nq * k] * b.d0b[j + (size_t)nq * k];
    m[i + (size_t)nq * j] = s;
  }
  std::vector<double> val, vec;
  jacobi_eig(nq, m, val, vec);
  std::vector<double> t((size_t)nq * nq, 0.0);  // d0bxd0bT(:,i) = VecP(:,i)/valP(i), i<=nb
  for (int i = 0; i < nb; ++i) for (int r = 0; r < nq; ++r) t[r + (size_t)nq * i] = vec[r + (size_t)nq * i] / val[i];
  std::vector<double> inv((size_t)nq * nq, 0.0);  // matmul(d0bxd0bT, transpose(VecP))
  for (int r = 0; r < nq; ++r) for (int c = 0; c < nq; ++c) {
    double s = 0.0;
    for (int k = 0; k < nq; ++k) s += t[r + (size_t)nq * k] * vec[c + (size_t)nq * k];
    inv[r + (size_t)nq * c] = s;
  }
  std::vector<double> pinv((size_t)nb * nq, 0.0);  // matmul(dnRBG%d0, inv): (nb x nq)
  for (int r = 0; r < nb; ++r) for (int c = 0; c < nq; ++c) {
    double s = 0.0;
    for (int k = 0; k < nq; ++k) s += b.d0b[k + (size_t)nq * r] * inv[k + (size_t)nq * c];
    pinv[r + (size_t)nb * c] = s;
  }
  b.d1gg.assign((size_t)nq * nq, 0.0); b.d2gg = b.d1gg;
  for (int r = 0; r < nq; ++r) for (int c = 0; c < nq; ++c) {
    double s1 = 0.0, s2 = 0.0;
    for (int k = 0; k < nb; ++k) {
      s1 += b.d1b[r + (size_t)nq * k] * pinv[k + (size_t)nb * c];
      s2 += b.d2b[r + (size_t)nq * k] * pinv[k + (size_t)nb * c];
    }
    b.d1gg[r + (size_t)nq * c] = s1; b.d2gg[r + (size_t)nq * c] = s2;
  }
  b.bgw.assign((size_t)nb * nq, 0.0);
  for (int i = 0; i < nb; ++i) for (int k = 0; k < nq; ++k) b.bgw[i + (size_t)nb * k] = b.d0b[k + (size_t)nq * i] * b.w[k];
}

// ---------------------------------------------------------------------------
// Problem: basis tables, Smolyak terms, packed basis, map, operator data.
// ---------------------------------------------------------------------------
struct Monomial { double coef; int idx[4]; int ib0, jb0; };

struct Problem {
  int kind = 0;  // 0 = SG4, 1 = DP
  int D = 0, nb0 = 1, LG = 0, LB = 0;
  std::vector<std::vector<Basis1D>> bas;   // bas[mode][level]
  std::vector<std::vector<int>> ltab;      // l(n) for 1-based n, per mode
  std::vector<int> terms;                  // nterm x D levels
  std::vector<double> weight;
  std::vector<long long> off_nb, off_nq;   // prefix offsets (exclusive)
  std::vector<int> nb_t, nq_t;
  std::vector<int> packed;                 // Np x D (1-based n)
  std::vector<int> map;                    // sum_nb, 0-based packed index or -1
  long long Np = 0, sum_nb = 0, sum_nq = 0;
  // operator
  std::vector<Monomial> mono;
  int keo_type = 10;
  std::vector<double> G0, g;               // D*D, D*D*D
  std::vector<double> vgrid;               // sum_nq * nb0 * nb0
  bool vgrid_done = false;
  // field coupling (fcn_field, sub_module_propa_march.f90:1494-1503: (H - E Dip) WP):
  // grid operator vw*V + mw*mu, kinetic part when keo != 0
  std::vector<Monomial> dip;
  std::vector<double> mugrid;
  double vw = 1.0, mw = 0.0;
  int keo = 1;
  // type 10 with a general Tnum metric (get_d0GG, sub_OpPsi_SG4.f90:2717-2728): per grid
  // point (whole-grid order, off_nq[t] + iq) the Jacobian and sqRhoOVERJac = sqrt(rho/Jac),
  // and optionally G(Q) itself (D*D per point, column-major); empty: Jac = rho = 1 and
  // G = G0 + g.Q
  std::vector<double> jac, sqrho, ggrid;
};

// Get_n_FROM_Basis_L_TO_n, L_TO_n_type 0, expo 1 (sub_module_Basis_LTO_n.f90:443-447)
static inline int n_of_L(int A, int B, int L) { return A + B * L; }

// Smolyak terms: type -5 nDindex (first index fastest, ADD_ONE_TO_nDindex_type5m,
// Source_Lib/sub_nDindex/sub_module_nDindex.f90:2463-2517) with Lmin<=sum(l)<=Lmax,
// Lmin = max(0,Lmax-D+1) (sub_quadra_SparseBasis.f90:994-995).
static void smolyak_terms(int D, int Lmax, std::vector<int>& out) {
  int Lmin = std::max(0, Lmax - D + 1);
  std::vector<int> l(D, 0);
  out.clear();
  while (true) {
    int s = 0; for (int v : l) s += v;
    if (s >= Lmin && s <= Lmax) out.insert(out.end(), l.begin(), l.end());
    // odometer, first index fastest, skipping sums above Lmax
    int i = 0;
    while (i < D) {
      l[i]++;
      int s2 = 0; for (int v : l) s2 += v;
      if (l[i] <= Lmax && s2 <= Lmax) break;
      l[i] = 0; i++;
    }
    if (i == D) break;
  }
}

// calc_Weight_OF_SRep (Source_ElVibRot/sub_Basis/sub_module_param_SGType2.f90:754-803)
static double binomial(int n, int k) {
  double r = 1.0;
  for (int i = 1; i <= k; ++i) r = r * (double)(n - k + i) / (double)i;
  return std::round(r);
}

static Problem* create(int kind, int D, int nb0, int LG, int LB, const int* Aq, const int* Bq,
                       const int* Ab, const int* Bb, const int* nq_dp, const int* nb_dp,
                       const double* scaleQ, const double* Q0) {
  Problem* P = new Problem();
  P->kind = kind; P->D = D; P->nb0 = nb0; P->LG = LG; P->LB = LB;
  P->bas.resize(D); P->ltab.resize(D);
  if (kind == 0) {
    // tab_basisPrimSG(L,ib), L = 0..LG, nb = nb(L), nq = nq(L)
    // (sub_quadra_SparseBasis.f90:1037-1105)
    for (int d = 0; d < D; ++d) {
      P->bas[d].resize(LG + 1);
      for (int L = 0; L <= LG; ++L)
        build_basis(P->bas[d][L], n_of_L(Ab[d], Bb[d], L), n_of_L(Aq[d], Bq[d], L), scaleQ[d], Q0[d]);
      // tab_i_TO_l: Tab_L(1:nb(L)) = L, L = LG..0 (sub_module_basis.f90:701-705)
      int nbmax = n_of_L(Ab[d], Bb[d], LG);
      P->ltab[d].assign(nbmax + 1, 0);
      for (int L = LG; L >= 0; --L) {
        int nb = n_of_L(Ab[d], Bb[d], L);
        for (int n = 1; n <= nb; ++n) P->ltab[d][n] = L;
      }
    }
    smolyak_terms(D, LG, P->terms);
  } else {
    for (int d = 0; d < D; ++d) {
      P->bas[d].resize(1);
      build_basis(P->bas[d][0], nb_dp[d], nq_dp[d], scaleQ[d], Q0[d]);
      P->ltab[d].assign(nb_dp[d] + 1, 0);
    }
    P->terms.assign(D, 0);
  }
  int nterm = (int)(P->terms.size() / D);
  P->weight.resize(nterm); P->nb_t.resize(nterm); P->nq_t.resize(nterm);
  P->off_nb.resize(nterm + 1); P->off_nq.resize(nterm + 1);
  P->off_nb[0] = 0; P->off_nq[0] = 0;
  for (int t = 0; t < nterm; ++t) {
    int s = 0; long long nb = 1, nq = 1;
    for (int d = 0; d < D; ++d) {
      int l = P->terms[(size_t)t * D + d]; s += l;
      nb *= P->bas[d][l].nb; nq *= P->bas[d][l].nq;
    }
    if (kind == 0) {
      int dl = LG - s;
      P->weight[t] = (dl < 0 || dl > D - 1) ? 0.0 : ((dl % 2 == 0) ? binomial(D - 1, dl) : -binomial(D - 1, dl));
    } else P->weight[t] = 1.0;
    P->nb_t[t] = (int)nb; P->nq_t[t] = (int)nq;
    P->off_nb[t + 1] = P->off_nb[t] + nb; P->off_nq[t + 1] = P->off_nq[t] + nq;
  }
  P->sum_nb = P->off_nb[nterm]; P->sum_nq = P->off_nq[nterm];

  // packed basis
  std::unordered_map<std::string, int> index;
  std::vector<int> nbmax(D);
  for (int d = 0; d < D; ++d) nbmax[d] = (int)P->ltab[d].size() - 1;
  // key of a 1-based tuple: its bytes, exact for any number of modes and sizes
  auto key = [&](const int* n) { return std::string((const char*)n, sizeof(int) * (size_t)D); };
  std::vector<int> n(D, 1);
  if (kind == 0) {
    // type 5 nDindB, last index fastest, sum_i l(n_i) <= LB
    // (ADD_ONE_TO_nDindex_type5p, sub_module_nDindex.f90:2396-2462)
    while (true) {
      int s = 0; for (int d = 0; d < D; ++d) s += P->ltab[d][n[d]];
      if (s <= LB) { index[key(n.data())] = (int)(P->packed.size() / D); P->packed.insert(P->packed.end(), n.begin(), n.end()); }
      int i = D - 1;
      while (i >= 0) {
        n[i]++;
        int s2 = 0; bool ok = n[i] <= nbmax[i];
        if (ok) { for (int d = 0; d < D; ++d) s2 += P->ltab[d][n[d]]; ok = s2 <= LB; }
        if (ok) break;
        n[i] = 1; i--;
      }
      if (i < 0) break;
    }
  } else {
    // direct product: first mode fastest
    while (true) {
      index[key(n.data())] = (int)(P->packed.size() / D);
      P->packed.insert(P->packed.end(), n.begin(), n.end());
      int i = 0;
      while (i < D) { n[i]++; if (n[i] <= nbmax[i]) break; n[i] = 1; i++; }
      if (i == D) break;
    }
  }
  P->Np = (long long)(P->packed.size() / D);

  // map: Set_tables_FOR_SmolyakRepBasis_TO_tabPackedBasis
  // (sub_Basis_SG4/sub_module_basis_BtoG_GtoB_SG4.f90:625-949): local tuples first mode
  // fastest (ADD_ONE_TO_nDval_m1), excluded when sum l(ib) > LB.
  P->map.assign(P->sum_nb, -1);
  for (int t = 0; t < nterm; ++t) {
    std::vector<int> nbl(D), ib(D, 1);
    for (int d = 0; d < D; ++d) nbl[d] = P->bas[d][P->terms[(size_t)t * D + d]].nb;
    for (long long iB = 0; iB < P->nb_t[t]; ++iB) {
      int s = 0; for (int d = 0; d < D; ++d) s += P->ltab[d][ib[d]];
      if (kind == 1 || s <= LB) {
        auto it = index.find(key(ib.data()));
        if (it != index.end()) P->map[P->off_nb[t] + iB] = it->second;
      }
      for (int d = 0; d < D; ++d) { ib[d]++; if (ib[d] <= nbl[d]) break; ib[d] = 1; }
    }
  }
  P->G0.assign((size_t)D * D, 0.0);
  for (int d = 0; d < D; ++d) P->G0[d + (size_t)D * d] = 1.0;
  P->g.assign((size_t)D * D * D, 0.0);
  return P;
}

// grid point coordinates: Rec_Qact_SG4_with_Tab_iq (sub_module_basis.f90:4131), local
// point order first mode fastest.
static void term_point_Q(const Problem* P, int t, long long iq, double* Q) {
  for (int d = 0; d < P->D; ++d) {
    const Basis1D& b = P->bas[d][P->terms[(size_t)t * P->D + d]];
    Q[d] = b.x[iq % b.nq]; iq /= b.nq;
  }
}

static void fill_grid(Problem* P, const std::vector<Monomial>& mono, std::vector<double>& grid) {
  int nterm = (int)P->weight.size(), D = P->D, nb0 = P->nb0;
  grid.assign((size_t)P->sum_nq * nb0 * nb0, 0.0);
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nterm; ++t) {
    std::vector<double> Q(D);
    long long NQ = P->nq_t[t];
    double* Vt = &grid[(size_t)P->off_nq[t] * nb0 * nb0];
    for (long long iq = 0; iq < NQ; ++iq) {
      term_point_Q(P, t, iq, Q.data());
      for (const Monomial& m : mono) {
        double v = m.coef;
        for (int k = 0; k < 4; ++k) if (m.idx[k] >= 0) v *= Q[m.idx[k]];
        Vt[iq + NQ * (m.ib0 + (long long)nb0 * m.jb0)] += v;
      }
    }
  }
}

// grid operator tables: V, and the dipole when the field term is on
static void fill_vgrid(Problem* P) {
  fill_grid(P, P->mono, P->vgrid);
  if (!P->dip.empty()) fill_grid(P, P->dip, P->mugrid);
  else P->mugrid.clear();
  P->vgrid_done = true;
}

// BDP_TO_GDP_OF_SmolyakRep (sub_module_basis_BtoG_GtoB_SG4.f90:2385-2496) for one
// electronic component: modes i = 1..D, RTempG(iq,:,ib) = d0b . RTempB(iq,:,ib).
static void bdp_to_gdp(const Problem* P, int t, std::vector<double>& R) {
  int D = P->D;
  long long nnb = P->nb_t[t], nnq = 1;
  std::vector<double> out;
  for (int i = 0; i < D; ++i) {
    const Basis1D& b = P->bas[i][P->terms[(size_t)t * D + i]];
    int nb2 = b.nb, nq2 = b.nq;
    nnb /= nb2;
    out.assign((size_t)nnq * nq2 * nnb, 0.0);
    for (long long ib = 0; ib < nnb; ++ib)
      for (long long iq = 0; iq < nnq; ++iq)
        for (int q = 0; q < nq2; ++q) {
          double s = 0.0;
          for (int k = 0; k < nb2; ++k) s += b.d0b[q + (size_t)nq2 * k] * R[iq + nnq * (k + (long long)nb2 * ib)];
          out[iq + nnq * (q + (long long)nq2 * ib)] = s;
        }
    R.swap(out);
    nnq *= nq2;
  }
}

// GDP_TO_BDP_OF_SmolyakRep (same file :2497-2581): RTempB(ib,:,iq) = dnRBGwrho . RTempG(ib,:,iq).
static void gdp_to_bdp(const Problem* P, int t, std::vector<double>& R) {
  int D = P->D;
  long long nnq = P->nq_t[t], nnb = 1;
  std::vector<double> out;
  for (int i = 0; i < D; ++i) {
    const Basis1D& b = P->bas[i][P->terms[(size_t)t * D + i]];
    int nb2 = b.nb, nq2 = b.nq;
    nnq /= nq2;
    out.assign((size_t)nnb * nb2 * nnq, 0.0);
    for (long long iq = 0; iq < nnq; ++iq)
      for (long long ib = 0; ib < nnb; ++ib)
        for (int k = 0; k < nb2; ++k) {
          double s = 0.0;
          for (int q = 0; q < nq2; ++q) s += b.bgw[k + (size_t)nb2 * q] * R[ib + nnb * (q + (long long)nq2 * iq)];
          out[ib + nnb * (k + (long long)nb2 * iq)] = s;
        }
    R.swap(out);
    nnb *= nb2;
  }
}

// DerivOp_TO_RDP_OF_SmolaykRep (same file :2690-2795): apply dnRGG%d1 along mode i
// (order 1) or dnRGG%d2 (order 2) in place.
static void deriv_mode(const Problem* P, int t, int mode, int order, double* R) {
  int D = P->D;
  long long nnq1 = 1, nnq3 = P->nq_t[t];
  for (int i = 0; i < D; ++i) {
    const Basis1D& b = P->bas[i][P->terms[(size_t)t * D + i]];
    int nq2 = b.nq;
    nnq3 /= nq2;
    if (i == mode) {
      const std::vector<double>& M = (order == 1) ? b.d1gg : b.d2gg;
      std::vector<double> col(nq2);
      for (long long i3 = 0; i3 < nnq3; ++i3)
        for (long long i1 = 0; i1 < nnq1; ++i1) {
          for (int q = 0; q < nq2; ++q) col[q] = R[i1 + nnq1 * (q + (long long)nq2 * i3)];
          for (int q = 0; q < nq2; ++q) {
            double s = 0.0;
            for (int k = 0; k < nq2; ++k) s += M[q + (size_t)nq2 * k] * col[k];
            R[i1 + nnq1 * (q + (long long)nq2 * i3)] = s;
          }
        }
    }
    nnq1 *= nq2;
  }
}

// sub_TabOpPsi_OF_ONEDP_FOR_SGtype4 (Source_ElVibRot/sub_Operator/sub_OpPsi_SG4.f90:1354-1668),
// type 1 (:1490-1546) and type 10 (:1548-1650), for one term and one vector; psi_t on
// entry holds the gathered basis coefficients (nb0 blocks of NB_t), on exit H.psi_t.
static void term_oppsi(const Problem* P, int t, std::vector<double>& psi_t) {
  int D = P->D, nb0 = P->nb0;
  long long NB = P->nb_t[t], NQ = P->nq_t[t];
  std::vector<std::vector<double>> G(nb0);
  for (int a = 0; a < nb0; ++a) {
    G[a].assign(psi_t.begin() + a * NB, psi_t.begin() + (a + 1) * NB);
    bdp_to_gdp(P, t, G[a]);
  }
  const double* V = &P->vgrid[(size_t)P->off_nq[t] * nb0 * nb0];
  std::vector<double> Vf;  // vw*V + mw*mu with a field term
  if (P->vw != 1.0 || P->mw != 0.0) {
    const size_t n = (size_t)NQ * nb0 * nb0;
    Vf.assign(V, V + n);
    const double* M = P->mugrid.empty() ? nullptr : &P->mugrid[(size_t)P->off_nq[t] * nb0 * nb0];
    for (size_t i = 0; i < n; ++i) Vf[i] = P->vw * Vf[i] + (M ? P->mw * M[i] : 0.0);
    V = Vf.data();
  }
  std::vector<std::vector<double>> H(nb0, std::vector<double>(NQ, 0.0));
  if (!P->keo) {
    for (int a = 0; a < nb0; ++a)
      for (int b = 0; b < nb0; ++b)
        for (long long iq = 0; iq < NQ; ++iq) H[a][iq] += V[iq + NQ * (a + (long long)nb0 * b)] * G[b][iq];
  } else if (P->keo_type == 10) {
    std::vector<double> Q(D);
    std::vector<double> PsiRj((size_t)NQ * D), PsiRi(NQ), OpPsiR(NQ);
    std::vector<double> Gq((size_t)NQ * D * D);
    const long long q0 = P->off_nq[t];
    for (long long iq = 0; iq < NQ; ++iq) {  // G(Q) = G0 + sum_k g_ijk Q_k, or the host's G(Q)
      term_point_Q(P, t, iq, Q.data());
      for (int i = 0; i < D; ++i) for (int j = 0; j < D; ++j) {
        double s;
        if (!P->ggrid.empty()) {
          s = P->ggrid[(size_t)(q0 + iq) * D * D + j + (size_t)D * i];
        } else {
          s = P->G0[i + (size_t)D * j];
          for (int k = 0; k < D; ++k) s += P->g[i + (size_t)D * (j + (size_t)D * k)] * Q[k];
        }
        Gq[iq + NQ * (j + (size_t)D * i)] = s;  // GGiq(iq,j,i)
      }
    }
    // Jac and sqRhoOVERJac of the points (1 when not given)
    std::vector<double> Jq(NQ, 1.0), Sq(NQ, 1.0);
    if (!P->jac.empty())
      for (long long iq = 0; iq < NQ; ++iq) {
        Jq[iq] = P->jac[(size_t)(q0 + iq)];
        Sq[iq] = P->sqrho[(size_t)(q0 + iq)];
      }
    for (int a = 0; a < nb0; ++a) {
      std::vector<double> VPsi(NQ, 0.0);
      for (int b = 0; b < nb0; ++b)
        for (long long iq = 0; iq < NQ; ++iq) VPsi[iq] += V[iq + NQ * (a + (long long)nb0 * b)] * G[b][iq];
      // psi * sqRhoOVERJac (:1581), then its derivatives (:1587-1595)
      for (int j = 0; j < D; ++j) {
        for (long long iq = 0; iq < NQ; ++iq) PsiRj[(size_t)NQ * j + iq] = G[a][iq] * Sq[iq];
        deriv_mode(P, t, j, 1, &PsiRj[(size_t)NQ * j]);
      }
      std::fill(OpPsiR.begin(), OpPsiR.end(), 0.0);
      for (int i = 0; i < D; ++i) {  // d_i (Jac sum_j G_ji d_j) (:1599-1614)
        std::fill(PsiRi.begin(), PsiRi.end(), 0.0);
        for (int j = 0; j < D; ++j)
          for (long long iq = 0; iq < NQ; ++iq) PsiRi[iq] += Gq[iq + NQ * (j + (size_t)D * i)] * PsiRj[iq + NQ * j];
        for (long long iq = 0; iq < NQ; ++iq) PsiRi[iq] *= Jq[iq];
        deriv_mode(P, t, i, 1, PsiRi.data());
        for (long long iq = 0; iq < NQ; ++iq) OpPsiR[iq] += PsiRi[iq];
      }
      // -1/2 OpPsiR / (Jac sqRhoOVERJac) + VPsi (:1618)
      for (long long iq = 0; iq < NQ; ++iq) H[a][iq] = -0.5 * OpPsiR[iq] / (Jq[iq] * Sq[iq]) + VPsi[iq];
    }
  } else {
    // type 1: V term (0,0), then F2 terms: (i,i) with dnRGG%d2, (i<j) with d1 d1;
    // Gcte: F2(i,i) = -G(i,i)/2, F2(i,j) = -G(i,j) (i<j), diagonal in the electronic index.
    for (int a = 0; a < nb0; ++a)
      for (int b = 0; b < nb0; ++b)
        for (long long iq = 0; iq < NQ; ++iq) H[a][iq] += V[iq + NQ * (a + (long long)nb0 * b)] * G[b][iq];
    std::vector<double> ch(NQ);
    for (int i = 0; i < D; ++i)
      for (int j = i; j < D; ++j) {
        double f = (i == j) ? -0.5 * P->G0[i + (size_t)D * i] : -P->G0[i + (size_t)D * j];
        if (f == 0.0) continue;  // grid_zero
        for (int a = 0; a < nb0; ++a) {
          std::copy(G[a].begin(), G[a].end(), ch.begin());
          if (i == j) deriv_mode(P, t, i, 2, ch.data());
          else { deriv_mode(P, t, i, 1, ch.data()); deriv_mode(P, t, j, 1, ch.data()); }
          for (long long iq = 0; iq < NQ; ++iq) H[a][iq] += f * ch[iq];
        }
      }
  }
  for (int a = 0; a < nb0; ++a) {
    gdp_to_bdp(P, t, H[a]);
    std::copy(H[a].begin(), H[a].end(), psi_t.begin() + a * NB);
  }
}

}  // namespace

extern "C" {

void* or_create(int kind, int D, int nb0, int LG, int LB, const int* Aq, const int* Bq, const int* Ab,
                const int* Bb, const int* nq_dp, const int* nb_dp, const double* scaleQ, const double* Q0) {
  if (D < 1 || D > 32 || nb0 < 1) return nullptr;
  return create(kind, D, nb0, LG, LB, Aq, Bq, Ab, Bb, nq_dp, nb_dp, scaleQ, Q0);
}

void or_destroy(void* h) { delete (Problem*)h; }

// out: Np, nterm, sum_nb, sum_nq, max_nb_t, max_nq_t
void or_sizes(void* h, long long* out) {
  Problem* P = (Problem*)h;
  out[0] = P->Np; out[1] = (long long)P->weight.size(); out[2] = P->sum_nb; out[3] = P->sum_nq;
  out[4] = *std::max_element(P->nb_t.begin(), P->nb_t.end());
  out[5] = *std::max_element(P->nq_t.begin(), P->nq_t.end());
}

void or_tables(void* h, int* term_l, double* weight, int* map, int* packed) {
  Problem* P = (Problem*)h;
  if (term_l) std::copy(P->terms.begin(), P->terms.end(), term_l);
  if (weight) std::copy(P->weight.begin(), P->weight.end(), weight);
  if (map) std::copy(P->map.begin(), P->map.end(), map);
  if (packed) std::copy(P->packed.begin(), P->packed.end(), packed);
}

// 1-D tables of (mode, level); arrays sized by the caller (>= nq*nq each).
int or_basis(void* h, int mode, int level, int* nbq, double* x, double* w, double* d0b, double* d1b,
             double* d2b, double* bgw, double* d1gg, double* d2gg) {
  Problem* P = (Problem*)h;
  if (mode < 0 || mode >= P->D || level < 0 || level >= (int)P->bas[mode].size()) return -1;
  const Basis1D& b = P->bas[mode][level];
  nbq[0] = b.nb; nbq[1] = b.nq;
  if (x) std::copy(b.x.begin(), b.x.end(), x);
  if (w) std::copy(b.w.begin(), b.w.end(), w);
  if (d0b) std::copy(b.d0b.begin(), b.d0b.end(), d0b);
  if (d1b) std::copy(b.d1b.begin(), b.d1b.end(), d1b);
  if (d2b) std::copy(b.d2b.begin(), b.d2b.end(), d2b);
  if (bgw) std::copy(b.bgw.begin(), b.bgw.end(), bgw);
  if (d1gg) std::copy(b.d1gg.begin(), b.d1gg.end(), d1gg);
  if (d2gg) std::copy(b.d2gg.begin(), b.d2gg.end(), d2gg);
  return 0;
}

void or_gauss_hermite(int n, double* x, double* wexp) {
  std::vector<double> xx, ww;
  gauss_hermite(n, xx, ww);
  std::copy(xx.begin(), xx.end(), x);
  std::copy(ww.begin(), ww.end(), wexp);
}

// V = sum_m coef_m prod_k Q[idx_m[k]] on the electronic element (ib0, jb0).
int or_set_potential(void* h, int n_mono, const double* coef, const int* idx, const int* elec) {
  Problem* P = (Problem*)h;
  P->mono.resize(n_mono);
  for (int m = 0; m < n_mono; ++m) {
    P->mono[m].coef = coef[m];
    for (int k = 0; k < 4; ++k) P->mono[m].idx[k] = idx[4 * m + k];
    P->mono[m].ib0 = elec ? elec[2 * m] : 0; P->mono[m].jb0 = elec ? elec[2 * m + 1] : 0;
    for (int k = 0; k < 4; ++k) if (P->mono[m].idx[k] >= P->D) return -1;
    if (P->mono[m].ib0 >= P->nb0 || P->mono[m].jb0 >= P->nb0) return -1;
  }
  P->vgrid_done = false;
  return 0;
}

// KEO: type 10 with G(Q) = G0 + sum_k g[i,j,k] Q_k (column-major g(i,j,k)); type 1 with
// constant G0.
int or_set_keo(void* h, int type, const double* G0, const double* g) {
  Problem* P = (Problem*)h;
  if (type != 1 && type != 10) return -1;
  P->keo_type = type;
  int D = P->D;
  if (G0) P->G0.assign(G0, G0 + (size_t)D * D);
  if (g) P->g.assign(g, g + (size_t)D * D * D); else P->g.assign((size_t)D * D * D, 0.0);
  return 0;
}

// Dipole operator mu(Q) (the para_Dip of sub_Opt_control, sub_control.f90:290), monomials
// like the potential, and the field term of later or_hpsi calls: vw*V + mw*mu, kinetic
// part when keo != 0 (H - E mu: vw = 1, mw = -E, keo = 1).
int or_set_dipole(void* h, int n_mono, const double* coef, const int* idx, const int* elec) {
  Problem* P = (Problem*)h;
  P->dip.resize(n_mono);
  for (int m = 0; m < n_mono; ++m) {
    P->dip[m].coef = coef[m];
    for (int k = 0; k < 4; ++k) P->dip[m].idx[k] = idx[4 * m + k];
    P->dip[m].ib0 = elec ? elec[2 * m] : 0; P->dip[m].jb0 = elec ? elec[2 * m + 1] : 0;
    for (int k = 0; k < 4; ++k) if (P->dip[m].idx[k] >= P->D) return -1;
    if (P->dip[m].ib0 >= P->nb0 || P->dip[m].jb0 >= P->nb0) return -1;
  }
  P->vgrid_done = false;
  return 0;
}

// The Tnum side of a type-10 operator as grid values (get_d0GG per point,
// sub_OpPsi_SG4.f90:2717-2728), whole-grid order: jac and rho (sum_nq each; null: 1), and
// G (sum_nq x D x D, column-major per point; null: G0 + g.Q).  sqRhoOVERJac = sqrt(rho/jac).
int or_set_metric(void* h, const double* jac, const double* rho, const double* G) {
  Problem* P = (Problem*)h;
  const size_t n = (size_t)P->sum_nq;
  if (jac && rho) {
    P->jac.assign(jac, jac + n);
    P->sqrho.resize(n);
    for (size_t i = 0; i < n; ++i) {
      if (!(jac[i] > 0.0) || !(rho[i] > 0.0)) return -1;
      P->sqrho[i] = std::sqrt(rho[i] / jac[i]);
    }
  } else {
    P->jac.clear();
    P->sqrho.clear();
  }
  if (G) P->ggrid.assign(G, G + n * P->D * P->D);
  else P->ggrid.clear();
  return 0;
}

int or_set_field(void* h, double vw, double mw, int keo) {
  Problem* P = (Problem*)h;
  P->vw = vw; P->mw = mw; P->keo = keo ? 1 : 0;
  return 0;
}

int or_vgrid(void* h, double* v) {
  Problem* P = (Problem*)h;
  if (!P->vgrid_done) fill_vgrid(P);
  std::copy(P->vgrid.begin(), P->vgrid.end(), v);
  return 0;
}

// sub_TabOpPsi_FOR_SGtype4 (sub_OpPsi_SG4.f90:678-979): OpPsi = 0, then for every term
// (OpenMP static schedule as the reference :833) gather (tabPackedBasis_TO_tabR_AT_iG,
// BtoG_GtoB_SG4.f90:1176-1246), operator on the term, weighted scatter-add
// (tabR_AT_iG_TO_tabPackedBasis :1250-1289).  psi/hpsi: nvec columns of length Np*nb0
// with leading dimensions ld/ldh.  Per-thread accumulators replace the OMP ATOMIC and
// are summed in thread order.
int or_hpsi(void* h, const double* psi, long long ld, double* hpsi, long long ldh, int nvec, int nthreads) {
  Problem* P = (Problem*)h;
  if (!P->vgrid_done) fill_vgrid(P);
  int nterm = (int)P->weight.size(), nb0 = P->nb0;
  long long Np = P->Np, N = Np * nb0;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  std::vector<std::vector<double>> acc(nthreads);
#pragma omp parallel num_threads(nthreads)
  {
    int th = omp_get_thread_num();
    acc[th].assign((size_t)N * nvec, 0.0);
    std::vector<double> psi_t;
#pragma omp for schedule(static)
    for (int t = 0; t < nterm; ++t) {
      long long NB = P->nb_t[t];
      const int* mp = &P->map[P->off_nb[t]];
      for (int v = 0; v < nvec; ++v) {
        psi_t.assign((size_t)NB * nb0, 0.0);
        for (int a = 0; a < nb0; ++a)
          for (long long iB = 0; iB < NB; ++iB)
            if (mp[iB] >= 0) psi_t[iB + NB * a] = psi[(size_t)v * ld + mp[iB] + Np * a];
        term_oppsi(P, t, psi_t);
        double wt = P->weight[t];
        double* out = &acc[th][(size_t)v * N];
        for (int a = 0; a < nb0; ++a)
          for (long long iB = 0; iB < NB; ++iB)
            if (mp[iB] >= 0) out[mp[iB] + Np * a] += wt * psi_t[iB + NB * a];
      }
    }
  }
  for (int v = 0; v < nvec; ++v)
    for (long long k = 0; k < N; ++k) {
      double s = 0.0;
      for (int th = 0; th < nthreads; ++th) s += acc[th][(size_t)v * N + k];
      hpsi[(size_t)v * ldh + k] = s;
    }
  return 0;
}

}  // extern "C"
