// evr_setup.cpp -- host-side construction of the tables the H.psi kernels consume.
//
// It produces, from the few numbers of evr_problem_desc, what the reference builds in
//   construct_primitive_basis  (Source_ElVibRot/sub_Basis/sub_module_basis.f90:391-782)
//   RecSparseGrid_ForDP_type4  (Source_ElVibRot/sub_Basis/sub_quadra_SparseBasis.f90:924-1435)
//   Set_tables_FOR_SmolyakRepBasis_TO_tabPackedBasis
//                              (Source_ElVibRot/sub_Basis/sub_Basis_SG4/sub_module_basis_BtoG_GtoB_SG4.f90:625-949)
// laid out for the device: one flat pool of 1-D matrices, one TermDesc per Smolyak
// term, the packed<-term map and its CSR transpose for the deterministic weighted
// reduction that replaces the reference's OMP ATOMIC scatter (BtoG_GtoB_SG4.f90:1283).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <unordered_map>

#include "evr_internal.h"

namespace evr {
namespace {

typedef long double LD;
const LD kPiL = 3.14159265358979323846264338327950288L;

// Orthonormal Hermite functions phi_k(x), k < n, by their three-term recurrence.
void hermite_functions(int n, LD x, LD* phi) {
  phi[0] = expl(-0.5L * x * x) / sqrtl(sqrtl(kPiL));
  if (n > 1) phi[1] = sqrtl(2.0L) * x * phi[0];
  for (int k = 2; k < n; ++k) phi[k] = sqrtl(2.0L / k) * x * phi[k - 1] - sqrtl((LD)(k - 1) / k) * phi[k - 2];
}

// Eigenvalues of the symmetric tridiagonal Jacobi matrix of the Hermite weight
// (zero diagonal, off-diagonal sqrt(k/2)) by the implicit-shift QL iteration.
void tridiag_eigenvalues(int n, std::vector<LD>& d) {
  std::vector<LD> e(n, 0.0L);
  d.assign(n, 0.0L);
  for (int k = 1; k < n; ++k) e[k - 1] = sqrtl((LD)k / 2.0L);
  for (int l = 0; l < n; ++l) {
    for (int iter = 0; iter < 200; ++iter) {
      int m = l;
      for (; m < n - 1; ++m) {
        LD dd = fabsl(d[m]) + fabsl(d[m + 1]);
        if (fabsl(e[m]) <= 1e-30L * (dd + 1.0L)) break;
      }
      if (m == l) break;
      LD g = (d[l + 1] - d[l]) / (2.0L * e[l]);
      LD r = hypotl(g, 1.0L);
      g = d[m] - d[l] + e[l] / (g + (g >= 0 ? fabsl(r) : -fabsl(r)));
      LD s = 1.0L, c = 1.0L, p = 0.0L;
      int i = m - 1;
      for (; i >= l; --i) {
        LD f = s * e[i], b = c * e[i];
        r = hypotl(f, g);
        e[i + 1] = r;
        if (r == 0.0L) { d[i + 1] -= p; e[m] = 0.0L; break; }
        s = f / r; c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0L * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
      }
      if (r == 0.0L && i >= l) continue;
      d[l] -= p; e[l] = g; e[m] = 0.0L;
    }
  }
  std::sort(d.begin(), d.end());
}

// Gauss-Hermite nodes x_i and w_i*exp(x_i^2): the two columns the reference reads from
// Internal_data/HermQuadra/herm<nq>.txt (sub_quadra_herm.f90:322-343).
void gauss_hermite(int n, std::vector<double>& x, std::vector<double>& wexp) {
  x.assign(n, 0.0); wexp.assign(n, 0.0);
  if (n == 1) { wexp[0] = (double)sqrtl(kPiL); return; }
  std::vector<LD> d;
  tridiag_eigenvalues(n, d);
  std::vector<LD> phi(n + 1);
  for (int i = 0; i < n; ++i) {
    LD xi = d[i];
    for (int it = 0; it < 4; ++it) {  // Newton on phi_n, phi_n' = sqrt(2n) phi_{n-1} - x phi_n
      hermite_functions(n + 1, xi, phi.data());
      LD fp = sqrtl(2.0L * n) * phi[n - 1] - xi * phi[n];
      if (fp != 0.0L) xi -= phi[n] / fp;
    }
    hermite_functions(n, xi, phi.data());
    LD s = 0.0L;
    for (int k = 0; k < n; ++k) s += phi[k] * phi[k];
    x[i] = (double)xi;
    wexp[i] = (double)(1.0L / s);
  }
  for (int i = 0; i < n / 2; ++i) {  // symmetric rule
    double a = 0.5 * (x[n - 1 - i] - x[i]), w = 0.5 * (wexp[i] + wexp[n - 1 - i]);
    x[i] = -a; x[n - 1 - i] = a; wexp[i] = w; wexp[n - 1 - i] = w;
  }
  if (n % 2) x[n / 2] = 0.0;
}

// Solve the small SPD system A X = B (A nb x nb, B nb x m, column-major) in long double.
bool spd_solve(int nb, std::vector<LD> A, std::vector<LD>& B, int m) {
  // Cholesky A = L L^T
  for (int j = 0; j < nb; ++j) {
    LD s = A[j + (size_t)nb * j];
    for (int k = 0; k < j; ++k) s -= A[j + (size_t)nb * k] * A[j + (size_t)nb * k];
    if (s <= 0.0L) return false;
    LD ljj = sqrtl(s);
    A[j + (size_t)nb * j] = ljj;
    for (int i = j + 1; i < nb; ++i) {
      LD t = A[i + (size_t)nb * j];
      for (int k = 0; k < j; ++k) t -= A[i + (size_t)nb * k] * A[j + (size_t)nb * k];
      A[i + (size_t)nb * j] = t / ljj;
    }
  }
  for (int c = 0; c < m; ++c) {
    LD* b = &B[(size_t)nb * c];
    for (int i = 0; i < nb; ++i) {
      LD t = b[i];
      for (int k = 0; k < i; ++k) t -= A[i + (size_t)nb * k] * b[k];
      b[i] = t / A[i + (size_t)nb * i];
    }
    for (int i = nb - 1; i >= 0; --i) {
      LD t = b[i];
      for (int k = i + 1; k < nb; ++k) t -= A[k + (size_t)nb * i] * b[k];
      b[i] = t / A[i + (size_t)nb * i];
    }
  }
  return true;
}

bool finish_basis(Basis1D& b);

// One HO primitive basis ("HO"/"Hm", type 20) on its Gauss-Hermite grid, scaled as in
// sub_scale_basis (sub_module_basis.f90:1540-1638); grid derivative matrices through the
// pseudo-inverse of d0b (sub_dnGB_TO_dnGG, :2195-2460), here formed as
// (d0b^T d0b)^-1 d0b^T, which is the same operator as the reference's eigen-expansion.
bool build_basis(Basis1D& b, int nb, int nq, double scaleQ, double Q0) {
  if (nb < 1 || nq < nb || nq > kMaxN1) return false;
  b.nb = nb; b.nq = nq;
  gauss_hermite(nq, b.x, b.w);
  std::vector<LD> phi(nb + 2);
  b.d0b.assign((size_t)nq * nb, 0.0); b.d1b = b.d0b; b.d2b = b.d0b;
  const LD s = scaleQ, sq = sqrtl(s);
  for (int q = 0; q < nq; ++q) {
    LD x = b.x[q];
    hermite_functions(nb + 1, x, phi.data());
    for (int k = 0; k < nb; ++k) {
      LD d0 = phi[k];
      LD d1 = sqrtl((LD)k / 2.0L) * (k > 0 ? phi[k - 1] : 0.0L) - sqrtl((LD)(k + 1) / 2.0L) * phi[k + 1];
      LD d2 = (x * x - (LD)(2 * k + 1)) * phi[k];
      b.d0b[q + (size_t)nq * k] = (double)(d0 * sq);
      b.d1b[q + (size_t)nq * k] = (double)(d1 * sq * s);
      b.d2b[q + (size_t)nq * k] = (double)(d2 * sq * s * s);
    }
  }
  for (int q = 0; q < nq; ++q) { b.x[q] = Q0 + b.x[q] / scaleQ; b.w[q] = b.w[q] * (1.0 / scaleQ); }
  return finish_basis(b);
}

// A primitive basis given by the host as tables on its grid (the reference's tables after
// construct_primitive_basis and sub_scale_basis, sub_module_basis.f90:391-782, 1540-1638):
// x, w (nq), d0b, d1b, d2b (nq x nb, column-major); the grid derivative matrices and the
// weighted transpose follow as for the built bases.
bool basis_from_tables(Basis1D& b, const evr_basis1d& t) {
  const int nq = t.nq, nb = t.nb;
  if (nb < 1 || nq < nb || nq > kMaxN1 || !t.x || !t.w || !t.d0b || !t.d1b || !t.d2b) return false;
  b.nb = nb; b.nq = nq;
  b.x.assign(t.x, t.x + nq);
  b.w.assign(t.w, t.w + nq);
  const size_t n = (size_t)nq * nb;
  b.d0b.assign(t.d0b, t.d0b + n);
  b.d1b.assign(t.d1b, t.d1b + n);
  b.d2b.assign(t.d2b, t.d2b + n);
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(b.d0b[i]) || !std::isfinite(b.d1b[i]) || !std::isfinite(b.d2b[i])) return false;
  for (int q = 0; q < nq; ++q)
    if (!std::isfinite(b.x[q]) || !(b.w[q] > 0.0)) return false;
  return finish_basis(b);
}

// Grid derivative matrices through the pseudo-inverse of d0b (sub_dnGB_TO_dnGG,
// sub_module_basis.f90:2195-2460), P = (d0b^T d0b)^-1 d0b^T, and bgw = d0b^T diag(w).
bool finish_basis(Basis1D& b) {
  const int nb = b.nb, nq = b.nq;
  std::vector<LD> A((size_t)nb * nb), P((size_t)nb * nq);
  for (int i = 0; i < nb; ++i) for (int j = 0; j < nb; ++j) {
    LD t = 0.0L;
    for (int q = 0; q < nq; ++q) t += (LD)b.d0b[q + (size_t)nq * i] * b.d0b[q + (size_t)nq * j];
    A[i + (size_t)nb * j] = t;
  }
  for (int q = 0; q < nq; ++q) for (int i = 0; i < nb; ++i) P[i + (size_t)nb * q] = b.d0b[q + (size_t)nq * i];
  if (!spd_solve(nb, A, P, nq)) return false;
  b.d1gg.assign((size_t)nq * nq, 0.0); b.d2gg = b.d1gg;
  for (int r = 0; r < nq; ++r) for (int c = 0; c < nq; ++c) {
    LD t1 = 0.0L, t2 = 0.0L;
    for (int k = 0; k < nb; ++k) {
      t1 += (LD)b.d1b[r + (size_t)nq * k] * P[k + (size_t)nb * c];
      t2 += (LD)b.d2b[r + (size_t)nq * k] * P[k + (size_t)nb * c];
    }
    b.d1gg[r + (size_t)nq * c] = (double)t1; b.d2gg[r + (size_t)nq * c] = (double)t2;
  }
  b.bgw.assign((size_t)nb * nq, 0.0);
  for (int k = 0; k < nb; ++k) for (int q = 0; q < nq; ++q) b.bgw[k + (size_t)nb * q] = b.d0b[q + (size_t)nq * k] * b.w[q];
  return true;
}

double binom(int n, int k) {
  double r = 1.0;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return std::round(r);
}

// All level tuples with Lmin <= sum <= Lmax (Lmin = max(0, Lmax-D+1),
// sub_quadra_SparseBasis.f90:994-995), in the reference's nDind_SmolyakRep order:
// first index fastest (nDindex type -5).
void smolyak_terms(int D, int Lmax, std::vector<int>& out) {
  const int Lmin = std::max(0, Lmax - D + 1);
  std::vector<std::vector<int>> all;
  std::vector<int> cur(D, 0);
  // depth-first over modes, remaining budget
  std::vector<int> stack_budget;
  struct Rec {
    static void go(int d, int D, int budget, std::vector<int>& cur, std::vector<std::vector<int>>& all) {
      if (d == D) { all.push_back(cur); return; }
      for (int l = 0; l <= budget; ++l) { cur[d] = l; go(d + 1, D, budget - l, cur, all); }
      cur[d] = 0;
    }
  };
  Rec::go(0, D, Lmax, cur, all);
  std::vector<std::vector<int>> keep;
  for (auto& t : all) {
    int s = std::accumulate(t.begin(), t.end(), 0);
    if (s >= Lmin) keep.push_back(t);
  }
  // colexicographic order = last index most significant
  std::sort(keep.begin(), keep.end(), [D](const std::vector<int>& a, const std::vector<int>& b) {
    for (int i = D - 1; i >= 0; --i) if (a[i] != b[i]) return a[i] < b[i];
    return false;
  });
  out.clear();
  for (auto& t : keep) out.insert(out.end(), t.begin(), t.end());
}

}  // namespace

// Drops the positions of 1-point modes from every SG4 term: nq = nb = 1 with the grid node
// at 0 and a zero first derivative (the level-0 modes of L_TO_nq_A = 1 rules).  Such a mode
// multiplies the term's operator by d0b*bgw (folded into the term weight), its first
// derivatives vanish (type 10 and the off-diagonal type-1 terms), and its second
// derivative adds the constant -1/2 G0_ii d2gg to V_aa (type 1, `vshift`).  Term-local
// indices do not change (the dropped factors have size 1), so the map and the grids stay.
// The position with the most grid points stays last (a term of 1-point modes only keeps it).
static void compact_trivial_modes(HostProblem& P) {
  const int D = P.D;
  for (size_t t = 0; t < P.terms.size(); ++t) {
    TermDesc& T = P.terms[t];
    TermDesc& TT = P.termsT[t];
    T.Dp = TT.Dp = D;
    T.vshift = TT.vshift = 0.0;
    if (P.kind != EVR_BASIS_SG4) continue;
    int keep[kMaxD], nk = 0;
    double scale = 1.0, shift = 0.0;
    for (int p = 0; p < D; ++p) {
      const int i = T.perm[p];
      const Basis1D& b = P.bas[i][P.term_l[t * D + i]];
      const bool trivial = b.nq == 1 && b.nb == 1 && b.x[0] == 0.0 &&
                           std::fabs(b.d1gg[0]) <= 1e-14 * std::max(1.0, std::fabs(b.d2gg[0]));
      if (trivial && !(p == D - 1 && nk == 0)) {
        scale *= b.d0b[0] * b.bgw[0];
        if (P.keo_type == 1) shift += -0.5 * P.G0[i + (size_t)D * i] * b.d2gg[0];
      } else {
        keep[nk++] = p;
      }
    }
    if (nk == D) continue;
    auto squeeze = [&](TermDesc& X) {
      const TermDesc Y = X;
      for (int k = 0; k < kMaxD; ++k) {
        const bool on = k < nk;
        const int p = on ? keep[k] : 0;
        X.nb[k] = on ? Y.nb[p] : 0;
        X.nq[k] = on ? Y.nq[p] : 0;
        X.perm[k] = on ? Y.perm[p] : 0;
        X.m_d0b[k] = on ? Y.m_d0b[p] : 0;
        X.m_bgw[k] = on ? Y.m_bgw[p] : 0;
        X.m_d1[k] = on ? Y.m_d1[p] : 0;
        X.m_d2[k] = on ? Y.m_d2[p] : 0;
        X.m_x[k] = on ? Y.m_x[p] : 0;
      }
      X.D = nk;
      X.msz = term_matrix_elems(X, nk);
      X.weight = Y.weight * scale;
      X.vshift = shift;
    };
    squeeze(T);
    squeeze(TT);
  }
}

int build_host_problem(const evr_problem_desc* d, HostProblem& P, std::string& err) {
  if (!d) { err = "null problem description"; return EVR_EINVAL; }
  const int D = d->D;
  if (D < 1 || D > kMaxD) { err = "D must be in 1..24"; return EVR_EINVAL; }
  if (d->nb0 < 1 || d->nb0 > kMaxNb0) { err = "nb0 must be in 1..4"; return EVR_EINVAL; }
  if (d->kind != EVR_BASIS_SG4 && d->kind != EVR_BASIS_DP) { err = "unknown basis kind"; return EVR_EINVAL; }
  if (d->keo_type != 1 && d->keo_type != 10) { err = "keo_type must be 1 or 10"; return EVR_EINVAL; }
  P = HostProblem();
  P.kind = d->kind; P.D = D; P.nb0 = d->nb0; P.keo_type = d->keo_type;
  P.bas.resize(D); P.ltab.resize(D);
  std::vector<int> nbmax(D);
  if (d->kind == EVR_BASIS_SG4) {
    if (!d->Aq || !d->Bq || !d->Ab || !d->Bb) { err = "SG4 needs Aq, Bq, Ab, Bb"; return EVR_EINVAL; }
    if (d->LG < 0 || d->LB < 0 || d->LB > d->LG) { err = "need 0 <= LB <= LG"; return EVR_EINVAL; }
    P.LG = d->LG; P.LB = d->LB;
    for (int i = 0; i < D; ++i) {
      P.bas[i].resize(P.LG + 1);
      for (int L = 0; L <= P.LG; ++L) {
        int nq = d->Aq[i] + d->Bq[i] * L, nb = d->Ab[i] + d->Bb[i] * L;
        double s = d->scaleQ ? d->scaleQ[i] : 1.0, q0 = d->Q0 ? d->Q0[i] : 0.0;
        if (d->bases) {  // the host's tables of (mode i, level L)
          const evr_basis1d& t = d->bases[(size_t)i * (d->LG + 1) + L];
          if (t.nq != nq || t.nb != nb) {
            err = "host basis table of mode " + std::to_string(i) + " level " + std::to_string(L) +
                  " has nq, nb = " + std::to_string(t.nq) + ", " + std::to_string(t.nb) + "; the level rules give " +
                  std::to_string(nq) + ", " + std::to_string(nb);
            return EVR_EINVAL;
          }
          if (!basis_from_tables(P.bas[i][L], t)) {
            err = "invalid host basis table (null or non-finite arrays, non-positive weights, or a singular basis) "
                  "at mode " + std::to_string(i) + " level " + std::to_string(L);
            return EVR_EINVAL;
          }
          continue;
        }
        if (!(s > 0.0) || !build_basis(P.bas[i][L], nb, nq, s, q0)) {
          err = "invalid 1-D basis (need 1 <= nb <= nq <= 24, scaleQ > 0) at mode " + std::to_string(i);
          return EVR_EINVAL;
        }
      }
      // l(n) = min{L : nb(L) >= n}  (Tab_L, sub_module_basis.f90:701-705)
      nbmax[i] = P.bas[i][P.LG].nb;
      P.ltab[i].assign(nbmax[i] + 1, 0);
      for (int n = 1; n <= nbmax[i]; ++n) {
        int L = 0;
        while (P.bas[i][L].nb < n) ++L;
        P.ltab[i][n] = L;
      }
    }
    smolyak_terms(D, P.LG, P.term_l);
  } else {
    if (!d->nq_dp || !d->nb_dp) { err = "DP needs nq_dp and nb_dp"; return EVR_EINVAL; }
    for (int i = 0; i < D; ++i) {
      P.bas[i].resize(1);
      double s = d->scaleQ ? d->scaleQ[i] : 1.0, q0 = d->Q0 ? d->Q0[i] : 0.0;
      if (d->bases) {
        const evr_basis1d& t = d->bases[i];
        if (t.nq != d->nq_dp[i] || t.nb != d->nb_dp[i] || !basis_from_tables(P.bas[i][0], t)) {
          err = "invalid host basis table at mode " + std::to_string(i) +
                " (sizes must equal nq_dp, nb_dp; finite arrays, positive weights, a regular basis)";
          return EVR_EINVAL;
        }
      } else if (!(s > 0.0) || !build_basis(P.bas[i][0], d->nb_dp[i], d->nq_dp[i], s, q0)) {
        err = "invalid 1-D basis (need 1 <= nb <= nq <= 24, scaleQ > 0) at mode " + std::to_string(i);
        return EVR_EINVAL;
      }
      nbmax[i] = d->nb_dp[i];
      P.ltab[i].assign(nbmax[i] + 1, 0);
    }
    P.term_l.assign(D, 0);
  }

  // matrix pool
  // matrices of H and of its transpose: H^T applies (d0b^T w)^T = w d0b on the way to the
  // grid, d1gg^T / d2gg^T on the grid and d0b^T on the way back
  std::vector<std::vector<int>> off_d0(D), off_bgw(D), off_d1(D), off_d2(D), off_x(D);
  std::vector<std::vector<int>> offT_in(D), offT_out(D), offT_d1(D), offT_d2(D);
  // slab-mode products: d1.d0b, d2.d0b (nq x nb), bgw.d1, bgw.d2 (nb x nq), and the
  // transposed operator's counterparts
  std::vector<std::vector<int>> off_x1(D), off_x2(D), off_e1(D), off_e2(D);
  std::vector<std::vector<int>> offT_x1(D), offT_x2(D), offT_e1(D), offT_e2(D);
  auto transpose = [](const std::vector<double>& a, int r, int cc) {
    std::vector<double> t((size_t)r * cc);
    for (int i = 0; i < r; ++i) for (int j = 0; j < cc; ++j) t[j + (size_t)cc * i] = a[i + (size_t)r * j];
    return t;
  };
  // (r x k) . (k x c), column-major, accumulated in long double
  auto matmul = [](const std::vector<double>& a, const std::vector<double>& b, int r, int k, int c) {
    std::vector<double> o((size_t)r * c);
    for (int i = 0; i < r; ++i)
      for (int j = 0; j < c; ++j) {
        long double s = 0.0L;
        for (int m = 0; m < k; ++m) s += (long double)a[i + (size_t)r * m] * b[m + (size_t)k * j];
        o[i + (size_t)r * j] = (double)s;
      }
    return o;
  };
  P.symmetric = true;
  for (int i = 0; i < D; ++i) {
    int nl = (int)P.bas[i].size();
    off_d0[i].resize(nl); off_bgw[i].resize(nl); off_d1[i].resize(nl); off_d2[i].resize(nl); off_x[i].resize(nl);
    offT_in[i].resize(nl); offT_out[i].resize(nl); offT_d1[i].resize(nl); offT_d2[i].resize(nl);
    off_x1[i].resize(nl); off_x2[i].resize(nl); off_e1[i].resize(nl); off_e2[i].resize(nl);
    offT_x1[i].resize(nl); offT_x2[i].resize(nl); offT_e1[i].resize(nl); offT_e2[i].resize(nl);
    for (int L = 0; L < nl; ++L) {
      const Basis1D& b = P.bas[i][L];
      if (b.nq != b.nb) P.symmetric = false;
      // column-major rows x cols matrix stored with its columns padded to a multiple of 4
      // rows, each block starting on a 32-byte boundary (16-byte vector loads in FP32/FP64)
      auto put = [&](const std::vector<double>& v, int rows, int cols) {
        const int ld = (rows + 3) & ~3;
        int o = (int)P.mat_pool.size();
        for (int cc = 0; cc < cols; ++cc) {
          P.mat_pool.insert(P.mat_pool.end(), v.begin() + (size_t)rows * cc, v.begin() + (size_t)rows * (cc + 1));
          for (int r = rows; r < ld; ++r) P.mat_pool.push_back(0.0);
        }
        while (P.mat_pool.size() % 4) P.mat_pool.push_back(0.0);
        return o;
      };
      off_d0[i][L] = put(b.d0b, b.nq, b.nb); off_bgw[i][L] = put(b.bgw, b.nb, b.nq);
      off_d1[i][L] = put(b.d1gg, b.nq, b.nq); off_d2[i][L] = put(b.d2gg, b.nq, b.nq);
      off_x[i][L] = put(b.x, b.nq, 1);
      offT_in[i][L] = put(transpose(b.bgw, b.nb, b.nq), b.nq, b.nb);   // nq x nb
      offT_out[i][L] = put(transpose(b.d0b, b.nq, b.nb), b.nb, b.nq);  // nb x nq
      offT_d1[i][L] = put(transpose(b.d1gg, b.nq, b.nq), b.nq, b.nq);
      offT_d2[i][L] = put(transpose(b.d2gg, b.nq, b.nq), b.nq, b.nq);
      const std::vector<double> wd0b = transpose(b.bgw, b.nb, b.nq);  // w.d0b (nq x nb)
      const std::vector<double> d1T = transpose(b.d1gg, b.nq, b.nq), d2T = transpose(b.d2gg, b.nq, b.nq);
      const std::vector<double> d0bT = transpose(b.d0b, b.nq, b.nb);
      off_x1[i][L] = put(matmul(b.d1gg, b.d0b, b.nq, b.nq, b.nb), b.nq, b.nb);
      off_x2[i][L] = put(matmul(b.d2gg, b.d0b, b.nq, b.nq, b.nb), b.nq, b.nb);
      off_e1[i][L] = put(matmul(b.bgw, b.d1gg, b.nb, b.nq, b.nq), b.nb, b.nq);
      off_e2[i][L] = put(matmul(b.bgw, b.d2gg, b.nb, b.nq, b.nq), b.nb, b.nq);
      offT_x1[i][L] = put(matmul(d1T, wd0b, b.nq, b.nq, b.nb), b.nq, b.nb);
      offT_x2[i][L] = put(matmul(d2T, wd0b, b.nq, b.nq, b.nb), b.nq, b.nb);
      offT_e1[i][L] = put(matmul(d0bT, d1T, b.nb, b.nq, b.nq), b.nb, b.nq);
      offT_e2[i][L] = put(matmul(d0bT, d2T, b.nb, b.nq, b.nq), b.nb, b.nq);
    }
  }

  // terms
  const int nterm = (int)(P.term_l.size() / D);
  P.terms.resize(nterm); P.weight.resize(nterm);
  int64_t onb = 0, onq = 0;
  std::vector<std::vector<int>> perms(nterm);
  for (int t = 0; t < nterm; ++t) {
    TermDesc& T = P.terms[t];
    std::memset(&T, 0, sizeof(T));
    int64_t NB = 1, NQ = 1;
    int s = 0;
    // mode order: every mode but the one with the most grid points (the last such), then it
    int slab = 0;
    for (int i = 0; i < D; ++i)
      if (P.bas[i][P.term_l[(size_t)t * D + i]].nq >= P.bas[slab][P.term_l[(size_t)t * D + slab]].nq) slab = i;
    std::vector<int>& pm = perms[t];
    for (int i = 0; i < D; ++i)
      if (i != slab) pm.push_back(i);
    pm.push_back(slab);
    for (int p = 0; p < D; ++p) {
      const int i = pm[p];
      int L = P.term_l[(size_t)t * D + i];
      s += L;
      const Basis1D& b = P.bas[i][L];
      T.perm[p] = i;
      T.nb[p] = b.nb; T.nq[p] = b.nq;
      T.m_d0b[p] = off_d0[i][L]; T.m_bgw[p] = off_bgw[i][L]; T.m_d1[p] = off_d1[i][L];
      T.m_d2[p] = off_d2[i][L]; T.m_x[p] = off_x[i][L];
      NB *= b.nb; NQ *= b.nq;
    }
    {
      const int L = P.term_l[(size_t)t * D + slab];
      T.m_x1L = off_x1[slab][L]; T.m_x2L = off_x2[slab][L]; T.m_e1L = off_e1[slab][L]; T.m_e2L = off_e2[slab][L];
      T.msz = term_matrix_elems(T, D);
      T.D = D;
    }
    if (NB > (1 << 30) || NQ > (1 << 30)) { err = "term too large"; return EVR_EINVAL; }
    T.NB = (int32_t)NB; T.NQ = (int32_t)NQ; T.off_nb = onb; T.off_nq = onq;
    if (P.kind == EVR_BASIS_SG4) {
      int dl = P.LG - s;  // calc_Weight_OF_SRep (sub_module_param_SGType2.f90:784-803)
      T.weight = (dl < 0 || dl > D - 1) ? 0.0 : ((dl % 2) ? -binom(D - 1, dl) : binom(D - 1, dl));
    } else T.weight = 1.0;
    P.weight[t] = T.weight;
    onb += NB; onq += NQ;
    P.max_nq = std::max<int64_t>(P.max_nq, NQ); P.max_nb = std::max<int64_t>(P.max_nb, NB);
  }
  P.sum_nb = onb; P.sum_nq = onq;
  P.termsT = P.terms;
  for (int t = 0; t < nterm; ++t) {
    TermDesc& T = P.termsT[t];
    for (int p = 0; p < D; ++p) {
      const int i = perms[t][p];
      int L = P.term_l[(size_t)t * D + i];
      T.m_d0b[p] = offT_in[i][L]; T.m_bgw[p] = offT_out[i][L]; T.m_d1[p] = offT_d1[i][L]; T.m_d2[p] = offT_d2[i][L];
    }
    const int i = perms[t][D - 1];
    const int L = P.term_l[(size_t)t * D + i];
    T.m_x1L = offT_x1[i][L]; T.m_x2L = offT_x2[i][L]; T.m_e1L = offT_e1[i][L]; T.m_e2L = offT_e2[i][L];
  }

  // packed basis: SG4 -> all n with sum l(n_i) <= LB, last index fastest
  // (nDindB type 5, ADD_ONE_TO_nDindex_type5p, Source_Lib/sub_nDindex/sub_module_nDindex.f90:2396);
  // DP -> full product, first index fastest.
  // tuple keys: one byte per mode (n_i <= nb <= 24), exact for any number of modes
  auto key_of = [&](const int* n) {
    std::string k((size_t)D, '\0');
    for (int i = 0; i < D; ++i) k[(size_t)i] = (char)(unsigned char)n[i];
    return k;
  };
  std::unordered_map<std::string, int> rank;
  std::vector<int> n(D, 1);
  if (P.kind == EVR_BASIS_SG4) {
    struct Rec {
      static void go(int i, int D, int budget, std::vector<int>& n, const HostProblem& P,
                     const std::vector<int>& nbmax, std::vector<int>& out) {
        if (i == D) { out.insert(out.end(), n.begin(), n.end()); return; }
        for (int v = 1; v <= nbmax[i]; ++v) {
          int l = P.ltab[i][v];
          if (l > budget) break;  // l(n) is non-decreasing in n
          n[i] = v;
          go(i + 1, D, budget - l, n, P, nbmax, out);
        }
        n[i] = 1;
      }
    };
    Rec::go(0, D, P.LB, n, P, nbmax, P.packed);
  } else {
    int64_t tot = 1;
    for (int i = 0; i < D; ++i) tot *= nbmax[i];
    P.packed.resize((size_t)tot * D);
    for (int64_t k = 0; k < tot; ++k) {
      int64_t r = k;
      for (int i = 0; i < D; ++i) { P.packed[(size_t)k * D + i] = (int)(r % nbmax[i]) + 1; r /= nbmax[i]; }
    }
  }
  P.Np = (int64_t)(P.packed.size() / D);
  if (P.Np * P.nb0 >= (int64_t)1 << 31) { err = "packed basis too large"; return EVR_EINVAL; }
  rank.reserve((size_t)P.Np * 2);
  for (int64_t k = 0; k < P.Np; ++k) rank[key_of(&P.packed[(size_t)k * D])] = (int)k;

  // map: term-local tuples, first mode fastest; excluded when sum l > LB.  map keeps the
  // reference's term-local order, map_perm the device's (permuted modes, first fastest);
  // grid_perm sends a device grid point to the reference's point of the same term.
  P.map.assign((size_t)P.sum_nb, -1);
  P.map_perm.assign((size_t)P.sum_nb, -1);
  P.grid_perm.assign((size_t)P.sum_nq, 0);
  for (int t = 0; t < nterm; ++t) {
    const TermDesc& T = P.terms[t];
    std::vector<int> nbo(D), nqo(D);
    for (int i = 0; i < D; ++i) {
      const Basis1D& b = P.bas[i][P.term_l[(size_t)t * D + i]];
      nbo[i] = b.nb; nqo[i] = b.nq;
    }
    std::vector<int64_t> sb(D), sq(D);  // strides of the reference modes in the device order
    int64_t acc_b = 1, acc_q = 1;
    for (int p = 0; p < D; ++p) { sb[T.perm[p]] = acc_b; sq[T.perm[p]] = acc_q; acc_b *= T.nb[p]; acc_q *= T.nq[p]; }
    std::vector<int> ib(D, 1);
    for (int64_t iB = 0; iB < T.NB; ++iB) {
      int s = 0;
      int64_t iBp = 0;
      for (int i = 0; i < D; ++i) { s += P.ltab[i][ib[i]]; iBp += (int64_t)(ib[i] - 1) * sb[i]; }
      if (P.kind == EVR_BASIS_DP || s <= P.LB) {
        auto it = rank.find(key_of(ib.data()));
        if (it != rank.end()) {
          P.map[(size_t)T.off_nb + iB] = it->second;
          P.map_perm[(size_t)T.off_nb + iBp] = it->second;
        }
      }
      for (int i = 0; i < D; ++i) { if (++ib[i] <= nbo[i]) break; ib[i] = 1; }
    }
    std::vector<int> iq(D, 0);
    for (int64_t q = 0; q < T.NQ; ++q) {
      int64_t qp = 0;
      for (int i = 0; i < D; ++i) qp += (int64_t)iq[i] * sq[i];
      P.grid_perm[(size_t)T.off_nq + qp] = T.off_nq + q;
      for (int i = 0; i < D; ++i) { if (++iq[i] < nqo[i]) break; iq[i] = 0; }
    }
  }

  const int nb0 = P.nb0;
  // operator
  P.mono_coef.assign(d->mono_coef, d->mono_coef + d->n_mono);
  P.mono_idx.assign(d->mono_idx, d->mono_idx + 4 * (size_t)d->n_mono);
  if (d->mono_elec) P.mono_elec.assign(d->mono_elec, d->mono_elec + 2 * (size_t)d->n_mono);
  else P.mono_elec.assign(2 * (size_t)d->n_mono, 0);
  for (int m = 0; m < d->n_mono; ++m) {
    for (int k = 0; k < 4; ++k)
      if (P.mono_idx[4 * m + k] >= D || P.mono_idx[4 * m + k] < -1) { err = "monomial mode index out of range"; return EVR_EINVAL; }
    if (P.mono_elec[2 * m] < 0 || P.mono_elec[2 * m] >= nb0 || P.mono_elec[2 * m + 1] < 0 || P.mono_elec[2 * m + 1] >= nb0) {
      err = "monomial electronic index out of range"; return EVR_EINVAL;
    }
  }
  P.G0.assign((size_t)D * D, 0.0);
  if (d->G0) P.G0.assign(d->G0, d->G0 + (size_t)D * D);
  else for (int i = 0; i < D; ++i) P.G0[i + (size_t)D * i] = 1.0;
  P.g.assign((size_t)D * D * D, 0.0);
  if (d->g) P.g.assign(d->g, d->g + (size_t)D * D * D);

  // algorithmic FLOP of one H.psi on one real vector: contraction chain B->G and G->B,
  // 2D first-derivative passes (type 10) or D second-derivative passes (type 1),
  // pointwise G/V terms.
  double fl = 0.0;
  for (int t = 0; t < nterm; ++t) {
    const TermDesc& T = P.terms[t];
    double c = 0.0, a = 1.0;
    for (int i = 0; i < D; ++i) {
      double rest = 1.0;
      for (int j = i + 1; j < D; ++j) rest *= T.nb[j];
      c += a * T.nq[i] * T.nb[i] * rest;
      a *= T.nq[i];
    }
    double bg = 2.0 * c * nb0;                      // B->G and G->B, FMA counted as 2 FLOP below
    double der = 0.0;
    for (int i = 0; i < D; ++i) der += (double)T.NQ * T.nq[i];
    der *= (P.keo_type == 10 ? 2.0 : 1.0) * nb0;
    double pw = (P.keo_type == 10 ? (double)D * D + D : 0.0) * T.NQ * nb0 + (double)nb0 * nb0 * T.NQ;
    fl += 2.0 * (bg + der + pw);
  }
  P.flop_per_hpsi = fl;

  compact_trivial_modes(P);

  // CSR transpose over N = Np*nb0 rows, sources in the term-basis output buffer
  const int64_t N = P.Np * nb0;
  std::vector<int64_t> cnt(N + 1, 0);
  for (int t = 0; t < nterm; ++t) {
    const TermDesc& T = P.terms[t];
    if (T.weight == 0.0) continue;
    for (int64_t iB = 0; iB < T.NB; ++iB) {
      int k = P.map_perm[(size_t)T.off_nb + iB];
      if (k < 0) continue;
      for (int a = 0; a < nb0; ++a) cnt[k + P.Np * a + 1]++;
    }
  }
  for (int64_t k = 0; k < N; ++k) cnt[k + 1] += cnt[k];
  P.csr_ptr = cnt;
  P.csr_src.resize((size_t)cnt[N]); P.csr_w.resize((size_t)cnt[N]);
  std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
  for (int t = 0; t < nterm; ++t) {  // term order = the reference's summation order
    const TermDesc& T = P.terms[t];
    if (T.weight == 0.0) continue;
    for (int a = 0; a < nb0; ++a)
      for (int64_t iB = 0; iB < T.NB; ++iB) {
        int k = P.map_perm[(size_t)T.off_nb + iB];
        if (k < 0) continue;
        int64_t row = k + P.Np * a, pos = fill[row]++;
        P.csr_src[pos] = T.off_nb * nb0 + (int64_t)a * T.NB + iB;
        P.csr_w[pos] = T.weight;
      }
  }

  // zero-order diagonal for the Davidson preconditioner: separable harmonic energies
  // E0(n) = sum_i G0_ii scaleQ_i^2 (n_i - 1/2) plus the constant part of V_aa.
  P.e0diag.assign((size_t)N, 0.0);
  std::vector<double> vconst(nb0, 0.0);
  for (int m = 0; m < d->n_mono; ++m)
    if (P.mono_idx[4 * m] < 0 && P.mono_elec[2 * m] == P.mono_elec[2 * m + 1]) vconst[P.mono_elec[2 * m]] += P.mono_coef[m];
  // With host tables (any primitive basis) the diagonal is that of the separable part of H
  // on the largest basis of each mode: -1/2 G0_ii <n|d2|n> plus <n|V_i|n> for the monomials
  // of mode i alone, both by the mode's own quadrature.
  std::vector<std::vector<double>> e1(D);
  if (d->bases)
    for (int i = 0; i < D; ++i) {
      const Basis1D& b = P.bas[i].back();
      e1[i].assign(b.nb + 1, 0.0);
      for (int n = 0; n < b.nb; ++n) {
        double t = 0.0, v = 0.0;
        for (int q = 0; q < b.nq; ++q) {
          const double f = b.d0b[q + (size_t)b.nq * n];
          t += b.w[q] * f * b.d2b[q + (size_t)b.nq * n];
          double vq = 0.0;
          for (int m = 0; m < d->n_mono; ++m) {
            if (P.mono_elec[2 * m] != 0 || P.mono_elec[2 * m + 1] != 0) continue;
            bool alone = P.mono_idx[4 * m] >= 0;
            double term = P.mono_coef[m];
            for (int r = 0; r < 4 && alone; ++r) {
              const int ix = P.mono_idx[4 * m + r];
              if (ix < 0) continue;
              if (ix != i) alone = false;
              else term *= b.x[q];
            }
            if (alone) vq += term;
          }
          v += b.w[q] * f * f * vq;
        }
        e1[i][n + 1] = -0.5 * P.G0[i + (size_t)D * i] * t + v;
      }
    }
  for (int64_t k = 0; k < P.Np; ++k) {
    double e = 0.0;
    for (int i = 0; i < D; ++i) {
      const int n = P.packed[(size_t)k * D + i];
      if (d->bases) {
        e += e1[i][n];
      } else {
        double s = d->scaleQ ? d->scaleQ[i] : 1.0;
        e += P.G0[i + (size_t)D * i] * s * s * (n - 0.5);
      }
    }
    for (int a = 0; a < nb0; ++a) P.e0diag[k + P.Np * a] = e + vconst[a];
  }

  return EVR_OK;
}

}  // namespace evr
