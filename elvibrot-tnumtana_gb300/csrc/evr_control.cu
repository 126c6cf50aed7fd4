// evr_control.cu -- field coupling and the optimal-control gradient.
//
// Field: H(t) = H0 - E(t) mu with the dipole mu(Q) evaluated on the grid like V (the
// para_Dip operators of sub_Opt_control, Source_ElVibRot/sub_propagation/sub_control.f90:290,
// applied in fcn_field / march_noD_field, sub_module_propa_march.f90:1434-1514, 1635-1844).
// The field is piecewise constant, E_n on step n, so a step is exp(-i (H0 - E_n mu) dt),
// expanded in Chebyshev polynomials exactly like march_cheby (:4142-4434) with fixed
// bounds [Emin - Fmax*mu_max, Emax + Fmax*mu_max] for every step.
//
// Objective J = |<target|psi(T)>|^2 (calc_fidelity, sub_control.f90:1007-1050).  The gradient
// dJ/dE_n is the exact derivative of the discrete propagator (reverse mode through the
// Chebyshev recurrence).  For one step, out = sum_k s_k phi_k with s_k = exp(-i Ebar dt) c_k,
// phi_0 = psi, phi_1 = A psi, phi_{k+1} = 2 A phi_k + phi_{k-1}, A = -i Hs, Hs = (H_n - Ebar)/Esc.
// For f = <chi|out> the adjoint vectors (Clenshaw order) are
//   G_K = conj(s_K) chi,  G_k = conj(s_k) chi + 2 A^+ G_{k+1} + G_{k+2},
//   G_0 = conj(s_0) chi + A^+ G_1 + G_2           (A^+ = i Hs^T),
// G_0 = U_n^+ chi is the target propagated back one step, and with dHs/dE_n = -mu/Esc
//   df/dE_n = (i/Esc) [ <G_1|mu phi_0> + 2 sum_{k=1}^{K-1} <G_{k+1}|mu phi_k> ],
//   dJ/dE_n = 2 Re( conj(c) df/dE_n ),  c = <target|psi(T)>,  chi_N = target.
// States are kept every S steps (S = ceil(sqrt(nsteps)) by default); the backward pass
// recomputes one segment of states at a time from its checkpoint and, for each step, the
// phi_k of that step, so memory is O(sqrt(nsteps) + K) vectors and the work about three
// forward passes.  The reference itself updates the field with the continuous-time
// direction of build_field (:955-975), E_new = -Im(<psi|chi><chi|mu|psi>)/alpha; the same
// quantity, -2 Im(<psi(t_n)|chi(t_n)><chi(t_n)|mu|psi(t_n)>) = dJ/dE(t_n), is returned at the
// step boundaries for comparison.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "evr_internal.h"

using namespace evr;

namespace {

constexpr int kT = 256;

int grid_blocks(const evr_ctx* c, int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + kT - 1) / kT, (int64_t)c->num_sms * 4));
}

// A complex vector is N (re, im) pairs; pair k of a vector with stride ld is at p[k*ld].
// phi1 = -i Hs psi, acc = c0 psi + c1 phi1
__global__ void oc_first(const double* __restrict__ psi, int64_t lp, const double* __restrict__ H, int64_t lh,
                         double* __restrict__ phi1, int64_t l1, double* __restrict__ acc, double Eb, double inv,
                         double c0, double c1, int64_t N) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x) {
    const double pr = psi[k * lp], pi = psi[k * lp + 1];
    const double hr = (H[k * lh] - Eb * pr) * inv, hi = (H[k * lh + 1] - Eb * pi) * inv;
    phi1[k * l1] = hi;
    phi1[k * l1 + 1] = -hr;
    acc[2 * k] = fma(c1, hi, c0 * pr);
    acc[2 * k + 1] = fma(c1, -hr, c0 * pi);
  }
}

// next = prev - 2i Hs cur, acc += c next (next may alias prev)
__global__ void oc_step(const double* prev, int64_t lp, const double* __restrict__ cur, int64_t lc,
                        const double* __restrict__ H, int64_t lh, double* next, int64_t ln, double* __restrict__ acc,
                        double Eb, double inv, double c, int64_t N) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x) {
    const double hr = (H[k * lh] - Eb * cur[k * lc]) * inv, hi = (H[k * lh + 1] - Eb * cur[k * lc + 1]) * inv;
    const double nr = prev[k * lp] + 2.0 * hi, ni = prev[k * lp + 1] - 2.0 * hr;
    next[k * ln] = nr;
    next[k * ln + 1] = ni;
    acc[2 * k] = fma(c, nr, acc[2 * k]);
    acc[2 * k + 1] = fma(c, ni, acc[2 * k + 1]);
  }
}

// out = (cs - i sn) * in
__global__ void oc_phase(const double* __restrict__ in, int64_t li, double* __restrict__ out, int64_t lo, double cs,
                         double sn, int64_t N) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x) {
    const double a = in[k * li], b = in[k * li + 1];
    out[k * lo] = a * cs + b * sn;
    out[k * lo + 1] = b * cs - a * sn;
  }
}

// Gk = ck chi + f i Hs G1 + G2 (HG = H applied to G1; HG == nullptr means G1 = 0)
__global__ void oc_clenshaw(double* __restrict__ Gk, int64_t lk, const double* __restrict__ chi,
                            const double* __restrict__ HG, int64_t lh, const double* __restrict__ G1, int64_t l1,
                            const double* __restrict__ G2, int64_t l2, double ck, double f, double Eb, double inv,
                            int64_t N) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x) {
    double r = ck * chi[2 * k], i = ck * chi[2 * k + 1];
    if (HG) {
      const double hr = (HG[k * lh] - Eb * G1[k * l1]) * inv, hi = (HG[k * lh + 1] - Eb * G1[k * l1 + 1]) * inv;
      r = fma(-f, hi, r);  // f * i * (hr + i hi) = f (-hi + i hr)
      i = fma(f, hr, i);
    }
    if (G2) {
      r += G2[k * l2];
      i += G2[k * l2 + 1];
    }
    Gk[k * lk] = r;
    Gk[k * lk + 1] = i;
  }
}

// partial[(j*nblk + blk)*2 + {0,1}] = sum over this block's pairs of conj(a_j) b_j, for the
// vector pairs a_j = A + j*sa (stride la), b_j = B + j*sb (stride lb), j = blockIdx.y;
// fixed block count and order, so the sums are deterministic
constexpr int kDotBlocks = 64;
__global__ void oc_dots(const double* __restrict__ A, int64_t la, int64_t sa, const double* __restrict__ B, int64_t lb,
                        int64_t sb, int64_t N, double* __restrict__ partial) {
  const int j = blockIdx.y;
  const double* a = A + j * sa;
  const double* b = B + j * sb;
  double sr = 0.0, si = 0.0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x) {
    const double ar = a[k * la], ai = a[k * la + 1], br = b[k * lb], bi = b[k * lb + 1];
    sr = fma(ar, br, fma(ai, bi, sr));
    si = fma(ar, bi, fma(-ai, br, si));
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  __shared__ double red[2][kT / 32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[0][w] = sr;
    red[1][w] = si;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0, i = 0.0;
    for (int q = 0; q < kT / 32; ++q) {
      r += red[0][q];
      i += red[1][q];
    }
    partial[((int64_t)j * gridDim.x + blockIdx.x) * 2] = r;
    partial[((int64_t)j * gridDim.x + blockIdx.x) * 2 + 1] = i;
  }
}

// out[2j..] = sum_blk partial[j][blk]; then, when wsum != nullptr, wsum[0..1] =
// scale_i * (out_0 + 2 sum_{j>0} out_j) with scale_i = i / Esc  (the step's df/dE)
__global__ void oc_dots_final(const double* __restrict__ partial, int nblk, int nj, double* __restrict__ out,
                              double* __restrict__ wsum, double invEsc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double tr = 0.0, ti = 0.0;
  for (int j = 0; j < nj; ++j) {
    double r = 0.0, i = 0.0;
    for (int b = 0; b < nblk; ++b) {
      r += partial[((int64_t)j * nblk + b) * 2];
      i += partial[((int64_t)j * nblk + b) * 2 + 1];
    }
    if (out) {
      out[2 * j] = r;
      out[2 * j + 1] = i;
    }
    const double w = j == 0 ? 1.0 : 2.0;
    tr = fma(w, r, tr);
    ti = fma(w, i, ti);
  }
  if (wsum) {  // (i/Esc)(tr + i ti) = (-ti + i tr)/Esc
    wsum[0] = -ti * invEsc;
    wsum[1] = tr * invEsc;
  }
}

// ref = -2 Im(s1 s2) with s1 = <psi|chi>, s2 = <chi|mu psi>
__global__ void oc_ref(const double* __restrict__ s1, const double* __restrict__ s2, double* __restrict__ ref) {
  if (threadIdx.x == 0 && blockIdx.x == 0) ref[0] = -2.0 * (s1[0] * s2[1] + s1[1] * s2[0]);
}

// mw = -field[*step], ++*step: the field of the next step, read from device memory so that
// a captured step graph can be replayed for every step
__global__ void oc_next_field(const double* __restrict__ field, int* __restrict__ step, double* __restrict__ mw) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    mw[0] = -field[step[0]];
    step[0] += 1;
  }
}

__global__ void oc_set_step(int* __restrict__ step, int v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) step[0] = v;
}

__global__ void to_float(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

struct Dev {
  double* p = nullptr;
  size_t n = 0;
};

struct OCState {
  evr_oc_opts o{};
  int S = 1, K = 0, prec = EVR_PREC_FP64;
  int64_t N = 0;
  double Eb = 0, Esc = 1, cs = 1, sn = 0;
  std::vector<double> coef, field;
  double ovl[2] = {0, 0};
  int64_t fwd_cols = 0;
  bool have_forward = false;
  // device
  std::vector<double*> bufs;
  // field in device memory and the captured step graphs (forward step; backward step)
  double* d_field = nullptr;
  double* d_mw = nullptr;
  int* d_step = nullptr;
  double *pin = nullptr, *pn = nullptr;
  cudaGraphExec_t exF = nullptr, exB = nullptr;
  int64_t gen = -1;  // workspace generation the graphs were captured with
  double *target = nullptr, *cp = nullptr, *seg = nullptr, *Phi = nullptr, *MPhi = nullptr, *G = nullptr,
         *Hb = nullptr, *acc = nullptr, *ring = nullptr, *chi = nullptr, *chip = nullptr, *partial = nullptr,
         *dres = nullptr, *gc = nullptr, *ref = nullptr, *tmp = nullptr;
  int ncp = 0;
};

void oc_free(evr_ctx* c) {
  OCState* o = (OCState*)c->oc;
  if (!o) return;
  if (o->exF) cudaGraphExecDestroy(o->exF);
  if (o->exB) cudaGraphExecDestroy(o->exB);
  if (o->d_step) cudaFree(o->d_step);
  for (double* p : o->bufs)
    if (p) cudaFree(p);
  delete o;
  c->oc = nullptr;
}

int oc_alloc(evr_ctx* c, OCState* o, double** p, size_t n) {
  if (cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(double)) != cudaSuccess) {
    (void)cudaGetLastError();
    *p = nullptr;
    return set_error(c, EVR_ENOMEM, "optimal control: device allocation");
  }
  o->bufs.push_back(*p);
  return EVR_OK;
}

// one propagation step: psi_out = U_n psi_in (may alias); with Phi != nullptr the phi_k
// (k = 0..K) are kept at Phi + 2k (stride ldP); returns a status
int fwd_step(evr_ctx* c, OCState* o, const double* psi_in, int64_t lpi, double* psi_out, int64_t lpo, double E,
             double* Phi, int64_t ldP, const double* mu_dev = nullptr) {
  const int64_t N = o->N;
  cudaStream_t s = c->stream;
  OpExtras ex;
  ex.mw = -E;
  ex.mu_dev = mu_dev;
  const int gb = grid_blocks(c, N);
  const int K = o->K;
  const double inv = 1.0 / o->Esc;
  // phi_k locations
  auto loc = [&](int k, double*& p, int64_t& l) {
    if (Phi) {
      p = Phi + 2 * k;
      l = ldP;
    } else {
      p = o->ring + 2 * N * (k % 3);
      l = 2;
    }
  };
  double* p0;
  int64_t l0;
  loc(0, p0, l0);
  if (p0 != psi_in) {
    const cudaError_t e = cudaMemcpy2DAsync(p0, l0 * sizeof(double), psi_in, lpi * sizeof(double),
                                            2 * sizeof(double), N, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_check(c, e, "optimal control: copy");
  }
  int rc = hpsi_interleaved(c, p0, l0, o->Hb, 2, 2, o->prec, s, OP_H, &ex);
  if (rc) return rc;
  double* p1;
  int64_t l1;
  loc(1, p1, l1);
  oc_first<<<gb, kT, 0, s>>>(p0, l0, o->Hb, 2, p1, l1, o->acc, o->Eb, inv, o->coef[0], o->coef[1], N);
  for (int k = 1; k < K; ++k) {
    double *pc, *pp, *pn;
    int64_t lc, lp, ln;
    loc(k, pc, lc);
    loc(k - 1, pp, lp);
    loc(k + 1, pn, ln);
    if ((rc = hpsi_interleaved(c, pc, lc, o->Hb, 2, 2, o->prec, s, OP_H, &ex))) return rc;
    oc_step<<<gb, kT, 0, s>>>(pp, lp, pc, lc, o->Hb, 2, pn, ln, o->acc, o->Eb, inv, o->coef[k + 1], N);
  }
  oc_phase<<<gb, kT, 0, s>>>(o->acc, 2, psi_out, lpo, o->cs, o->sn, N);
  return cuda_check(c, cudaGetLastError(), "optimal control: step kernels");
}

// <a|b> for one pair of complex vectors into out[0..1] (device)
int dot1(evr_ctx* c, OCState* o, const double* a, int64_t la, const double* b, int64_t lb, double* out) {
  const int nb = std::min<int64_t>(kDotBlocks, (o->N + kT - 1) / kT);
  oc_dots<<<dim3(nb, 1), kT, 0, c->stream>>>(a, la, 0, b, lb, 0, o->N, o->partial);
  oc_dots_final<<<1, 32, 0, c->stream>>>(o->partial, nb, 1, out, nullptr, 0.0);
  return cuda_check(c, cudaGetLastError(), "optimal control: dot");
}

// Captures the launch sequence of body() on the context's stream into an executable graph.
template <typename F>
int capture(evr_ctx* c, F&& body, cudaGraphExec_t* exec) {
  cudaStream_t s = c->stream;
  c->capturing = true;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    c->capturing = false;
    (void)cudaGetLastError();
    return EVR_EDEVICE;
  }
  const int rc = body();
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(s, &g);
  c->capturing = false;
  if (rc || ce != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    (void)cudaGetLastError();
    return rc ? rc : EVR_EDEVICE;
  }
  const cudaError_t ie = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) {
    (void)cudaGetLastError();
    *exec = nullptr;
    return EVR_EDEVICE;
  }
  return EVR_OK;
}

// graphs hold the workspace's device pointers: drop them when the workspace changed
void check_graphs(evr_ctx* c, OCState* o) {
  if (o->gen == c->ws_gen) return;
  if (o->exF) cudaGraphExecDestroy(o->exF);
  if (o->exB) cudaGraphExecDestroy(o->exB);
  o->exF = o->exB = nullptr;
  o->gen = c->ws_gen;
}

}  // namespace

namespace evr {
void free_control(evr_ctx* c) { oc_free(c); }

// The FP64 and FP32 dipole tables, both or neither: a failed allocation frees the other,
// so a context never holds one without the other.
int alloc_dipole_tables(evr_ctx* c, size_t n) {
  if (c->dp_mugrid && c->dp_mugrid32) return EVR_OK;
  cudaError_t e = cudaSuccess;
  if (!c->dp_mugrid) e = cudaMalloc((void**)&c->dp_mugrid, n * sizeof(double));
  if (e == cudaSuccess && !c->dp_mugrid32) e = cudaMalloc((void**)&c->dp_mugrid32, n * sizeof(float));
  if (e != cudaSuccess) {
    if (c->dp_mugrid) cudaFree(c->dp_mugrid);
    if (c->dp_mugrid32) cudaFree(c->dp_mugrid32);
    c->dp_mugrid = nullptr;
    c->dp_mugrid32 = nullptr;
  }
  return cuda_check(c, e, "cudaMalloc dipole");
}
}  // namespace evr

extern "C" {

int evr_set_dipole(evr_ctx* c, int n_mono, const double* coef, const int* idx, const int* elec) {
  if (!c) return EVR_EINVAL;
  if (c->batch) return set_error(c, EVR_EINVAL, "evr_set_dipole: not for batched contexts");
  const HostProblem& P = c->hp;
  if (n_mono < 0 || (n_mono > 0 && (!coef || !idx || !elec)))
    return set_error(c, EVR_EINVAL, "evr_set_dipole: n_mono < 0 or null arrays");
  for (int m = 0; m < n_mono; ++m) {
    for (int k = 0; k < 4; ++k)
      if (idx[4 * m + k] < -1 || idx[4 * m + k] >= P.D)
        return set_error(c, EVR_EINVAL, "evr_set_dipole: mode index out of range");
    if (elec[2 * m] < 0 || elec[2 * m] >= P.nb0 || elec[2 * m + 1] < 0 || elec[2 * m + 1] >= P.nb0)
      return set_error(c, EVR_EINVAL, "evr_set_dipole: electronic index out of range");
  }
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  int rc = cuda_check(c, cudaSetDevice(c->device), "cudaSetDevice");
  if (rc) return rc;
  cudaStream_t s = c->stream;
  const size_t n = (size_t)P.sum_nq * P.nb0 * P.nb0;
  if ((rc = alloc_dipole_tables(c, n))) return rc;
  double* dcoef = nullptr;
  int *didx = nullptr, *delec = nullptr;
  const int nm = std::max(n_mono, 1);
  if ((rc = cuda_check(c, cudaMalloc((void**)&dcoef, nm * sizeof(double)), "cudaMalloc"))) return rc;
  if ((rc = cuda_check(c, cudaMalloc((void**)&didx, 4 * nm * sizeof(int)), "cudaMalloc"))) {
    cudaFree(dcoef);
    return rc;
  }
  if ((rc = cuda_check(c, cudaMalloc((void**)&delec, 2 * nm * sizeof(int)), "cudaMalloc"))) {
    cudaFree(dcoef);
    cudaFree(didx);
    return rc;
  }
  if (n_mono > 0) {
    cudaMemcpyAsync(dcoef, coef, n_mono * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(didx, idx, 4 * n_mono * sizeof(int), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(delec, elec, 2 * n_mono * sizeof(int), cudaMemcpyHostToDevice, s);
  }
  rc = eval_grid_monomials(c, n_mono, dcoef, didx, delec, c->dp_mugrid, &c->mu_max);
  if (!rc) {
    to_float<<<c->num_sms * 8, kT, 0, s>>>(c->dp_mugrid, c->dp_mugrid32, (int64_t)n);
    rc = cuda_check(c, cudaStreamSynchronize(s), "evr_set_dipole");
  }
  cudaFree(dcoef);
  cudaFree(didx);
  cudaFree(delec);
  return rc;
}

int evr_set_dipole_grid(evr_ctx* c, const double* mu, int layout) {
  if (!c) return EVR_EINVAL;
  if (!mu || (layout != EVR_VGRID_TERMS && layout != EVR_VGRID_REF))
    return set_error(c, EVR_EINVAL, "evr_set_dipole_grid: null values or unknown layout");
  if (c->batch) return set_error(c, EVR_EINVAL, "evr_set_dipole_grid: not for batched contexts");
  {
    const int64_t n = c->hp.sum_nq * c->hp.nb0 * c->hp.nb0;
    for (int64_t i = 0; i < n; ++i)
      if (!std::isfinite(mu[i]))
        return set_error(c, EVR_EINVAL, "evr_set_dipole_grid: value " + std::to_string(i) + " is not finite");
  }
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  int rc = cuda_check(c, cudaSetDevice(c->device), "cudaSetDevice");
  if (rc) return rc;
  const HostProblem& P = c->hp;
  std::vector<double> dev;
  std::vector<float> dev32;
  grid_values_to_device(P, mu, layout, false, dev, dev32);
  const size_t n = dev.size();
  // largest row-sum norm sum_b |mu_ab(q)| over the grid points, as evr_set_dipole computes it
  const int nb0 = P.nb0;
  double mmax = 0.0;
  for (const TermDesc& T : P.terms)
    for (int64_t q = 0; q < T.NQ; ++q)
      for (int a = 0; a < nb0; ++a) {
        double r = 0.0;
        for (int b = 0; b < nb0; ++b) r += std::fabs(dev[(size_t)T.off_nq * nb0 * nb0 + (size_t)(a + nb0 * b) * T.NQ + q]);
        mmax = std::max(mmax, r);
      }
  if ((rc = cuda_check(c, cudaDeviceSynchronize(), "sync before dipole update"))) return rc;
  oc_free(c);  // a forward state propagated with the old dipole would mix two operators
  if ((rc = alloc_dipole_tables(c, n))) return rc;
  cudaStream_t s = c->stream;
  if ((rc = cuda_check(c, cudaMemcpyAsync(c->dp_mugrid, dev.data(), n * sizeof(double), cudaMemcpyHostToDevice, s),
                       "copy dipole")) ||
      (rc = cuda_check(c, cudaMemcpyAsync(c->dp_mugrid32, dev32.data(), n * sizeof(float), cudaMemcpyHostToDevice, s),
                       "copy dipole")) ||
      (rc = cuda_check(c, cudaStreamSynchronize(s), "evr_set_dipole_grid")))
    return rc;
  c->mu_max = mmax;
  return EVR_OK;
}

int evr_set_field(evr_ctx* c, double vw, double mw, int keo) {
  if (!c) return EVR_EINVAL;
  if ((mw != 0.0 || vw != 1.0) && !c->dp_mugrid && !c->host_only)
    return set_error(c, EVR_EINVAL, "evr_set_field: no dipole (call evr_set_dipole first)");
  c->field.vw = vw;
  c->field.mw = mw;
  c->field.keo = keo ? 1 : 0;
  c->field.mu_dev = nullptr;
  return EVR_OK;
}

int evr_oc_forward(evr_ctx* c, const evr_oc_opts* opts, const double* field, const double* psi0, const double* target,
                   double* out3, double* psiT, int64_t* info) {
  if (!c) return EVR_EINVAL;
  if (!opts || !field || !psi0 || !target || opts->nsteps < 1 || !(opts->dt > 0.0) || !(opts->emax > opts->emin) ||
      !(opts->poly_tol > 0.0) || opts->checkpoint < 0)
    return set_error(c, EVR_EINVAL, "evr_oc_forward: bad arguments (nsteps >= 1, dt > 0, emax > emin, poly_tol > 0)");
  if (opts->prec != EVR_PREC_FP64 && opts->prec != EVR_PREC_FP32)
    return set_error(c, EVR_EINVAL, "evr_oc_forward: unknown precision");
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  if (!c->dp_mugrid) return set_error(c, EVR_EINVAL, "evr_oc_forward: no dipole (call evr_set_dipole first)");
  int rc = cuda_check(c, cudaSetDevice(c->device), "cudaSetDevice");
  if (rc) return rc;
  cudaStream_t s = c->stream;
  oc_free(c);
  OCState* o = new OCState();
  c->oc = o;
  o->o = *opts;
  o->prec = opts->prec;
  const int nst = opts->nsteps;
  o->field.assign(field, field + nst);
  o->N = c->hp.Np * c->hp.nb0;
  const int64_t N = o->N;
  double fmax = 0.0;
  for (double e : o->field) fmax = std::max(fmax, std::fabs(e));
  const double w = fmax * c->mu_max;
  const double emin = opts->emin - w, emax = opts->emax + w;
  o->Eb = 0.5 * (emin + emax);
  o->Esc = 0.5 * (emax - emin);
  if (!cheby_series(o->Esc * opts->dt, opts->poly_tol, o->coef)) {
    oc_free(c);
    return set_error(c, EVR_EINVAL, "evr_oc_forward: series too long (dt * spectral width too large)");
  }
  o->K = (int)o->coef.size() - 1;
  const double th = o->Eb * opts->dt;
  o->cs = std::cos(th);
  o->sn = std::sin(th);
  o->S = opts->checkpoint > 0 ? opts->checkpoint : (int)std::ceil(std::sqrt((double)nst));
  o->S = std::max(1, std::min(o->S, nst));
  o->ncp = nst / o->S + 1;
  const int K = o->K;
  const size_t v2 = (size_t)2 * N;
  if ((rc = oc_alloc(c, o, &o->target, v2)) || (rc = oc_alloc(c, o, &o->cp, v2 * o->ncp)) ||
      (rc = oc_alloc(c, o, &o->Hb, v2)) || (rc = oc_alloc(c, o, &o->acc, v2)) ||
      (rc = oc_alloc(c, o, &o->ring, 3 * v2)) || (rc = oc_alloc(c, o, &o->partial, (size_t)2 * kDotBlocks * (K + 2))) ||
      (rc = oc_alloc(c, o, &o->dres, (size_t)2 * (K + 6))) || (rc = oc_alloc(c, o, &o->tmp, v2)) ||
      (rc = oc_alloc(c, o, &o->d_field, (size_t)nst)) || (rc = oc_alloc(c, o, &o->d_mw, 1)) ||
      (rc = oc_alloc(c, o, &o->pin, v2)) || (rc = oc_alloc(c, o, &o->pn, v2)) ||
      (rc = cuda_check(c, cudaMalloc((void**)&o->d_step, sizeof(int)), "cudaMalloc"))) {
    oc_free(c);
    return rc;
  }
  cudaMemcpyAsync(o->cp, psi0, v2 * sizeof(double), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(o->target, target, v2 * sizeof(double), cudaMemcpyHostToDevice, s);
  if ((rc = cuda_check(c, cudaGetLastError(), "evr_oc_forward: upload"))) return rc;
  cudaMemcpyAsync(o->d_field, o->field.data(), nst * sizeof(double), cudaMemcpyHostToDevice, s);
  // psi lives in tmp; every S steps it is copied to the next checkpoint.  The first step
  // runs eagerly (it also sets up every work decomposition), the others replay its graph.
  o->gen = c->ws_gen;
  oc_set_step<<<1, 1, 0, s>>>(o->d_step, 0);
  cudaMemcpyAsync(o->tmp, o->cp, v2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
  auto stepF = [&]() -> int {
    oc_next_field<<<1, 1, 0, s>>>(o->d_field, o->d_step, o->d_mw);
    return fwd_step(c, o, o->tmp, 2, o->tmp, 2, 0.0, nullptr, 0, o->d_mw);
  };
  for (int n = 1; n <= nst; ++n) {
    if (n == 2 && !o->exF && capture(c, stepF, &o->exF) != EVR_OK) o->exF = nullptr;
    if (n >= 2 && o->exF) {
      if ((rc = cuda_check(c, cudaGraphLaunch(o->exF, s), "evr_oc_forward: graph launch"))) return rc;
    } else if ((rc = stepF())) {
      return rc;
    }
    if (n % o->S == 0)
      cudaMemcpyAsync(o->cp + v2 * (n / o->S), o->tmp, v2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
  }
  // overlap with the target, norms of psi(T) and psi(0)
  if ((rc = dot1(c, o, o->target, 2, o->tmp, 2, o->dres))) return rc;
  if ((rc = dot1(c, o, o->tmp, 2, o->tmp, 2, o->dres + 2))) return rc;
  if ((rc = dot1(c, o, o->cp, 2, o->cp, 2, o->dres + 4))) return rc;
  double h[6];
  if ((rc = cuda_check(c, cudaMemcpyAsync(h, o->dres, 6 * sizeof(double), cudaMemcpyDeviceToHost, s), "copy")))
    return rc;
  if (psiT && (rc = cuda_check(c, cudaMemcpyAsync(psiT, o->tmp, v2 * sizeof(double), cudaMemcpyDeviceToHost, s),
                               "copy psi(T)")))
    return rc;
  if ((rc = cuda_check(c, cudaStreamSynchronize(s), "evr_oc_forward"))) return rc;
  // a spectrum outside the bounds makes the series diverge: the norm then grows without
  // limit (the type-10 operator with nq > nb is not symmetric, so small drifts are normal)
  if (!(h[2] <= 2.0 * h[4] + 1e-300)) {
    o->have_forward = false;
    return set_error(c, EVR_ENOCONV, "evr_oc_forward: |psi(T)|^2 = " + std::to_string(h[2]) + " from " +
                                         std::to_string(h[4]) + " (spectrum outside [emin, emax]?)");
  }
  o->ovl[0] = h[0];
  o->ovl[1] = h[1];
  o->fwd_cols = (int64_t)nst * K * 2;
  o->have_forward = true;
  if (out3) {
    out3[0] = h[0] * h[0] + h[1] * h[1];
    out3[1] = h[0];
    out3[2] = h[1];
  }
  if (info) {
    info[0] = K;
    info[1] = o->fwd_cols;
    info[2] = o->ncp;
  }
  return EVR_OK;
}

int evr_oc_backward(evr_ctx* c, double* grad, double* ref, int64_t* info) {
  if (!c) return EVR_EINVAL;
  OCState* o = (OCState*)c->oc;
  if (!o || !o->have_forward) return set_error(c, EVR_EINVAL, "evr_oc_backward: no evr_oc_forward before");
  if (!grad) return set_error(c, EVR_EINVAL, "evr_oc_backward: null gradient array");
  int rc = cuda_check(c, cudaSetDevice(c->device), "cudaSetDevice");
  if (rc) return rc;
  cudaStream_t s = c->stream;
  const int64_t N = o->N;
  const int K = o->K, S = o->S, nst = o->o.nsteps;
  const size_t v2 = (size_t)2 * N;
  const int64_t ldP = 2 * (K + 2), ldG = 2 * (K + 2);
  if (!o->ref) {  // allocated last: any earlier failure leaves it null
    if ((rc = oc_alloc(c, o, &o->seg, v2 * (S + 1))) || (rc = oc_alloc(c, o, &o->Phi, (size_t)N * ldP)) ||
        (rc = oc_alloc(c, o, &o->MPhi, (size_t)N * ldP)) || (rc = oc_alloc(c, o, &o->G, (size_t)N * ldG)) ||
        (rc = oc_alloc(c, o, &o->chi, v2)) || (rc = oc_alloc(c, o, &o->chip, v2)) ||
        (rc = oc_alloc(c, o, &o->gc, (size_t)2 * (nst + 1))) || (rc = oc_alloc(c, o, &o->ref, (size_t)(nst + 1)) ))
      return rc;
  }
  const int gb = grid_blocks(c, N);
  const double inv = 1.0 / o->Esc;
  OpExtras mu_only;
  mu_only.vw = 0.0;
  mu_only.mw = 1.0;
  mu_only.keo = 0;
  int64_t cols = 0;
  cudaMemcpyAsync(o->chi, o->target, v2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
  // G_{K+1} = 0
  cudaMemset2DAsync(o->G + 2 * (K + 1), ldG * sizeof(double), 0, 2 * sizeof(double), N, s);
  const int nseg = (nst + S - 1) / S;
  const int ndb = (int)std::min<int64_t>(kDotBlocks, (N + kT - 1) / kT);
  double* s12 = o->dres + 2 * (K + 1);  // two complex scalars for the boundary gradient (dres holds 2(K+4))
  check_graphs(c, o);
  OpExtras exT;  // H^T - E_n mu with E_n from device memory
  exT.mu_dev = o->d_mw;
  double* gslot = o->dres + 2 * (K + 3);   // df/dE of the step (2 doubles)
  double* rslot = o->dres + 2 * (K + 3) + 2;  // boundary gradient of the step (dres holds 2(K+6))
  // one backward step: psi_{n-1} in pin, psi_n in pn, the step's field index in d_step
  auto stepB = [&]() -> int {
    int r;
    oc_next_field<<<1, 1, 0, s>>>(o->d_field, o->d_step, o->d_mw);
    // phi_0..phi_K of the step (phi_K is produced but not needed) and psi_n beside them
    if ((r = fwd_step(c, o, o->pin, 2, o->tmp, 2, 0.0, o->Phi, ldP, o->d_mw))) return r;
    cudaMemcpy2DAsync(o->Phi + 2 * (K + 1), ldP * sizeof(double), o->pn, 2 * sizeof(double), 2 * sizeof(double), N,
                      cudaMemcpyDeviceToDevice, s);
    // mu phi_k (k < K) and mu psi_n: columns 0..2K-1 and 2K+2..2K+3; phi_K's columns ride along
    if ((r = hpsi_blocks(c, o->Phi, ldP, o->MPhi, ldP, (int)ldP, o->prec, s, OP_H, &mu_only))) return r;
    // boundary gradient at t_n: -2 Im(<psi_n|chi_n><chi_n|mu psi_n>)
    if ((r = dot1(c, o, o->pn, 2, o->chi, 2, s12))) return r;
    if ((r = dot1(c, o, o->chi, 2, o->MPhi + 2 * (K + 1), ldP, s12 + 2))) return r;
    oc_ref<<<1, 32, 0, s>>>(s12, s12 + 2, rslot);
    // adjoint recurrence with chi' = exp(+i Ebar dt) chi
    oc_phase<<<gb, kT, 0, s>>>(o->chi, 2, o->chip, 2, o->cs, -o->sn, N);
    oc_clenshaw<<<gb, kT, 0, s>>>(o->G + 2 * K, ldG, o->chip, nullptr, 0, nullptr, 0, nullptr, 0, o->coef[K], 0.0,
                                  o->Eb, inv, N);
    for (int k = K - 1; k >= 0; --k) {
      const double* G1 = o->G + 2 * (k + 1);
      if ((r = hpsi_interleaved(c, G1, ldG, o->Hb, 2, 2, o->prec, s, OP_HT, &exT))) return r;
      oc_clenshaw<<<gb, kT, 0, s>>>(o->G + 2 * k, ldG, o->chip, o->Hb, 2, G1, ldG, o->G + 2 * (k + 2), ldG,
                                    o->coef[k], k == 0 ? 1.0 : 2.0, o->Eb, inv, N);
    }
    // df/dE_n = (i/Esc) sum_k w_k <G_{k+1}|mu phi_k>
    oc_dots<<<dim3(ndb, K), kT, 0, s>>>(o->G + 2, ldG, 2, o->MPhi, ldP, 2, N, o->partial);
    oc_dots_final<<<1, 32, 0, s>>>(o->partial, ndb, K, nullptr, gslot, inv);
    // chi_{n-1} = G_0
    cudaMemcpy2DAsync(o->chi, 2 * sizeof(double), o->G, ldG * sizeof(double), 2 * sizeof(double), N,
                      cudaMemcpyDeviceToDevice, s);
    return cuda_check(c, cudaGetLastError(), "evr_oc_backward: step kernels");
  };
  auto stepF = [&]() -> int {
    oc_next_field<<<1, 1, 0, s>>>(o->d_field, o->d_step, o->d_mw);
    return fwd_step(c, o, o->tmp, 2, o->tmp, 2, 0.0, nullptr, 0, o->d_mw);
  };
  bool first = true;
  for (int sg = nseg - 1; sg >= 0; --sg) {
    const int n0 = sg * S, n1 = std::min(n0 + S, nst);
    // states psi_{n0..n1} of the segment, by the forward step (graph when available)
    cudaMemcpyAsync(o->seg, o->cp + v2 * sg, v2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(o->tmp, o->cp + v2 * sg, v2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
    oc_set_step<<<1, 1, 0, s>>>(o->d_step, n0);
    for (int n = n0 + 1; n <= n1; ++n) {
      if (o->exF) {
        if ((rc = cuda_check(c, cudaGraphLaunch(o->exF, s), "evr_oc_backward: graph launch"))) return rc;
      } else if ((rc = stepF())) {
        return rc;
      }
      cudaMemcpyAsync(o->seg + v2 * (n - n0), o->tmp, v2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
      cols += 2 * K;
    }
    for (int n = n1; n > n0; --n) {
      cudaMemcpyAsync(o->pin, o->seg + v2 * (n - 1 - n0), v2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
      cudaMemcpyAsync(o->pn, o->seg + v2 * (n - n0), v2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
      oc_set_step<<<1, 1, 0, s>>>(o->d_step, n - 1);
      if (!first && !o->exB && capture(c, stepB, &o->exB) != EVR_OK) o->exB = nullptr;
      if (!first && o->exB) {
        if ((rc = cuda_check(c, cudaGraphLaunch(o->exB, s), "evr_oc_backward: graph launch"))) return rc;
      } else if ((rc = stepB())) {
        return rc;
      }
      first = false;
      cudaMemcpyAsync(o->gc + 2 * n, gslot, 2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
      cudaMemcpyAsync(o->ref + n, rslot, sizeof(double), cudaMemcpyDeviceToDevice, s);
      cols += 4 * K + ldP;
      if ((rc = cuda_check(c, cudaGetLastError(), "evr_oc_backward: step"))) return rc;
    }
  }
  // boundary gradient at t = 0
  {
    const double* psi0 = o->cp;
    cudaMemcpy2DAsync(o->Phi + 2 * (K + 1), ldP * sizeof(double), psi0, 2 * sizeof(double), 2 * sizeof(double), N,
                      cudaMemcpyDeviceToDevice, s);
    if ((rc = hpsi_interleaved(c, o->Phi + 2 * (K + 1), ldP, o->MPhi + 2 * (K + 1), ldP, 2, o->prec, s, OP_H,
                               &mu_only)))
      return rc;
    cols += 2;
    if ((rc = dot1(c, o, psi0, 2, o->chi, 2, s12))) return rc;
    if ((rc = dot1(c, o, o->chi, 2, o->MPhi + 2 * (K + 1), ldP, s12 + 2))) return rc;
    oc_ref<<<1, 32, 0, s>>>(s12, s12 + 2, o->ref);
  }
  std::vector<double> gch((size_t)2 * (nst + 1)), refh((size_t)nst + 1);
  cudaMemcpyAsync(gch.data(), o->gc, gch.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(refh.data(), o->ref, refh.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
  if ((rc = cuda_check(c, cudaStreamSynchronize(s), "evr_oc_backward"))) return rc;
  // dJ/dE_n = 2 Re(conj(c) df/dE_n)
  for (int n = 1; n <= nst; ++n)
    grad[n - 1] = 2.0 * (o->ovl[0] * gch[2 * n] + o->ovl[1] * gch[2 * n + 1]);
  if (ref) std::copy(refh.begin(), refh.end(), ref);
  if (info) {
    info[0] = cols;
    info[1] = o->ncp;
    info[2] = S;
  }
  return EVR_OK;
}

}  // extern "C"
