// evr_propagate.cu -- Chebyshev and short-iterative-Lanczos propagation of complex wave packets on the GPU.
//
// Restates march_cheby (Source_ElVibRot/sub_propagation/sub_module_propa_march.f90:4142-4434):
//   psi(t+dt) = exp(-i E0 dt) sum_k c_k phi_k,  phi_k = (-i)^k T_k(Hs) psi(t),
//   Hs = (H - E0)/Esc, E0 = (Emin+Emax)/2, Esc = (Emax-Emin)/2, r = Esc*dt,
//   c_0 = J_0(r), c_k = 2 J_k(r) (cof :5734-5757), and the recurrence
//   phi_{k+1} = phi_{k-1} - 2i Hs phi_k (:4296-4335).
// A complex packet is two real vectors (the split of sub_OpPsi.f90:392-407), so npsi
// packets are one interleaved block of 2*npsi columns for the H.psi kernels.
// The series length is fixed per call from the Bessel coefficients (|c_k| < poly_tol for
// every later order; |phi_k| <= |psi| when the spectrum lies in [Emin, Emax]), so one
// time step is a fixed launch sequence: it is captured once in a CUDA graph and replayed
// for every step, with the autocorrelation <psi0|psi(t_n)> and |psi|^2 written to device
// arrays and copied back at the end.  A norm moving by more than 1e-6 relative (1e-3 with
// FP32 contractions) signals a
// spectrum outside [Emin, Emax] (the reference retries with a larger Hmax, :4355-4362);
// the call then returns EVR_ENOCONV with the step where it happened.
#include <algorithm>
#include <cmath>
#include <vector>

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

// Bessel functions J_0..J_n(r) by Miller's backward recurrence normalised with
// J_0 + 2 sum J_2k = 1 (the role of mmbsjn, Source_Lib/sub_communf90/sub_math/sub_polyortho.f90:1781).
std::vector<double> bessel_j(int n, double r) {
  std::vector<double> j(n + 1, 0.0);
  if (r == 0.0) { j[0] = 1.0; return j; }
  const int start = std::max(n, (int)r) + 30 + (int)(2.0 * std::sqrt((double)std::max(n, (int)r) + 30.0));
  std::vector<long double> t(start + 2, 0.0L);
  t[start + 1] = 0.0L;
  t[start] = 1e-300L;
  long double norm = 0.0L;
  for (int k = start; k >= 1; --k) {
    t[k - 1] = (2.0L * k / r) * t[k] - t[k + 1];
    if (fabsl(t[k - 1]) > 1e250L) {  // rescale
      for (int m = k - 1; m <= start + 1; ++m) t[m] *= 1e-250L;
    }
  }
  norm = t[0];
  for (int k = 2; k <= start; k += 2) norm += 2.0L * t[k];
  for (int k = 0; k <= n; ++k) j[k] = (double)(t[k] / norm);
  return j;
}

// phi1 = -i Hs psi ; acc = c0 psi + c1 phi1
__global__ void cheby_first(const double* __restrict__ psi, const double* __restrict__ Hpsi, double* __restrict__ phi1,
                            double* __restrict__ acc, double E0, double invEsc, double c0, double c1, int64_t n2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = 2 * i;  // (re, im) pair
    const double hr = (Hpsi[e] - E0 * psi[e]) * invEsc, hi = (Hpsi[e + 1] - E0 * psi[e + 1]) * invEsc;
    const double pr = hi, pi = -hr;
    phi1[e] = pr;
    phi1[e + 1] = pi;
    acc[e] = c0 * psi[e] + c1 * pr;
    acc[e + 1] = c0 * psi[e + 1] + c1 * pi;
  }
}

// next = prev - 2i Hs cur ; acc += c next   (next may alias prev)
__global__ void cheby_step(const double* prev, const double* __restrict__ cur, const double* __restrict__ Hcur,
                           double* next, double* __restrict__ acc, double E0, double invEsc, double c, int64_t n2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = 2 * i;
    const double hr = (Hcur[e] - E0 * cur[e]) * invEsc, hi = (Hcur[e + 1] - E0 * cur[e + 1]) * invEsc;
    const double nr = prev[e] + 2.0 * hi, ni = prev[e + 1] - 2.0 * hr;
    next[e] = nr;
    next[e + 1] = ni;
    acc[e] = fma(c, nr, acc[e]);
    acc[e + 1] = fma(c, ni, acc[e + 1]);
  }
}

// psi = exp(-i theta) acc
__global__ void cheby_phase(const double* __restrict__ acc, double* __restrict__ psi, double cs, double sn, int64_t n2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = 2 * i;
    const double a = acc[e], b = acc[e + 1];
    psi[e] = a * cs + b * sn;
    psi[e + 1] = b * cs - a * sn;
  }
}

// per packet p: out[3p..] += (<psi0|psi>.re, <psi0|psi>.im, |psi|^2); block reduction with
// warp shuffles, one atomic per block and packet
__global__ void cheby_overlap(const double* __restrict__ psi0, const double* __restrict__ psi, int64_t N, int npsi,
                              double* __restrict__ out) {
  const int p = blockIdx.y;
  double sr = 0.0, si = 0.0, sn = 0.0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = k * 2 * npsi + 2 * p;
    const double a0 = psi0[e], b0 = psi0[e + 1], a = psi[e], b = psi[e + 1];
    sr = fma(a0, a, fma(b0, b, sr));
    si = fma(a0, b, fma(-b0, a, si));
    sn = fma(a, a, fma(b, b, sn));
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
    sn += __shfl_down_sync(0xffffffffu, sn, o);
  }
  __shared__ double red[3][32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { red[0][w] = sr; red[1][w] = si; red[2][w] = sn; }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    sr = l < nw ? red[0][l] : 0.0;
    si = l < nw ? red[1][l] : 0.0;
    sn = l < nw ? red[2][l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      sr += __shfl_down_sync(0xffffffffu, sr, o);
      si += __shfl_down_sync(0xffffffffu, si, o);
      sn += __shfl_down_sync(0xffffffffu, sn, o);
    }
    if (l == 0) {
      atomicAdd(out + 3 * p, sr);
      atomicAdd(out + 3 * p + 1, si);
      atomicAdd(out + 3 * p + 2, sn);
    }
  }
}

}  // namespace

namespace evr {
bool cheby_series(double r, double tol, std::vector<double>& coef) {
  int K = std::max(2, (int)std::ceil(r) + 8);
  std::vector<double> J;
  while (true) {
    J = bessel_j(K + 20, r);
    int last = 0;
    for (int k = 0; k <= K + 20; ++k)
      if ((k == 0 ? 1.0 : 2.0) * std::fabs(J[k]) >= tol) last = k;
    if (last + 1 < K) { K = std::max(2, last + 1); break; }
    K = 2 * K;
    if (K > 200000) return false;
  }
  J = bessel_j(K, r);
  coef.assign(K + 1, 0.0);
  for (int k = 0; k <= K; ++k) coef[k] = (k == 0 ? 1.0 : 2.0) * J[k];
  return true;
}
}  // namespace evr

extern "C" int evr_cheby_propagate(evr_ctx* c, const double* psi0, int npsi, double dt, int nsteps, double emin,
                                   double emax, double poly_tol, int prec, double* autocorr, double* psi_out,
                                   int64_t* info) {
  if (!c) return EVR_EINVAL;
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  if (!psi0 || npsi < 1 || 2 * npsi > kMaxBlock || nsteps < 0 || !(emax > emin) || !(poly_tol > 0.0) || !(dt > 0.0))
    return set_error(c, EVR_EINVAL, "evr_cheby_propagate: bad arguments (1 <= npsi <= 32, emax > emin, dt > 0)");
  if (prec != EVR_PREC_FP64 && prec != EVR_PREC_FP32) return set_error(c, EVR_EINVAL, "unknown precision");
  if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, EVR_EDEVICE, "cudaSetDevice");
  const int64_t N = c->hp.Np * c->hp.nb0;
  const int ncol = 2 * npsi;
  const double E0 = 0.5 * (emin + emax), Esc = 0.5 * (emax - emin), r = Esc * dt;
  // series length from the Bessel coefficients
  std::vector<double> coef;
  if (!cheby_series(r, poly_tol, coef))
    return set_error(c, EVR_EINVAL, "evr_cheby_propagate: series too long (dt*dE too large)");
  const int K = (int)coef.size() - 1;

  cudaStream_t s = c->stream;
  DevBuf d0, dpsi, dH, b0, b1, b2, dacc, dac;
  const size_t ne = (size_t)N * ncol;
  if (d0.alloc(ne) || dpsi.alloc(ne) || dH.alloc(ne) || b0.alloc(ne) || b1.alloc(ne) || b2.alloc(ne) ||
      dacc.alloc(ne) || dac.alloc((size_t)3 * npsi * (nsteps + 1)))
    return set_error(c, EVR_ENOMEM, "evr_cheby_propagate: device allocation");
  // host packets (npsi x N complex) -> interleaved N x 2npsi
  {
    std::vector<double> h(ne);
    for (int p = 0; p < npsi; ++p)
      for (int64_t k = 0; k < N; ++k) {
        h[k * ncol + 2 * p] = psi0[((size_t)p * N + k) * 2];
        h[k * ncol + 2 * p + 1] = psi0[((size_t)p * N + k) * 2 + 1];
      }
    if (cudaMemcpyAsync(d0.p, h.data(), sizeof(double) * ne, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(dpsi.p, d0.p, sizeof(double) * ne, cudaMemcpyDeviceToDevice, s) ||
        cudaMemsetAsync(dac.p, 0, sizeof(double) * 3 * npsi * (nsteps + 1), s) || cudaStreamSynchronize(s))
      return set_error(c, EVR_EDEVICE, "evr_cheby_propagate: upload");
  }
  int rc = ensure_workspace(c, ncol, prec);
  if (rc) return rc;
  const int gb = c->num_sms * 4;
  const int64_t n2 = N * npsi;
  dim3 og((unsigned)std::min<int64_t>((N + 255) / 256, 1024), (unsigned)npsi);
  cheby_overlap<<<og, 256, 0, s>>>(d0.p, dpsi.p, N, npsi, dac.p);
  const double invEsc = 1.0 / Esc, th = E0 * dt, cs = std::cos(th), sn = std::sin(th);

  // one time step as a launch sequence; `slot` selects the autocorrelation entry
  auto record_step = [&](int slot) -> int {
    int e;
    if ((e = hpsi_interleaved(c, dpsi.p, ncol, dH.p, ncol, ncol, prec, s, OP_H))) return e;
    cheby_first<<<gb, 256, 0, s>>>(dpsi.p, dH.p, b1.p, dacc.p, E0, invEsc, coef[0], coef[1], n2);
    double* prev = dpsi.p;  // phi_0
    double* cur = b1.p;     // phi_1
    double* spare[2] = {b0.p, b2.p};
    int sp = 0;
    for (int k = 1; k < K; ++k) {
      if ((e = hpsi_interleaved(c, cur, ncol, dH.p, ncol, ncol, prec, s, OP_H))) return e;
      double* next = (k == 1) ? spare[sp] : prev;  // phi_0 (= psi) must survive the first update
      if (k == 1) sp ^= 1;
      cheby_step<<<gb, 256, 0, s>>>(prev, cur, dH.p, next, dacc.p, E0, invEsc, coef[k + 1], n2);
      prev = cur;
      cur = next;
    }
    cheby_phase<<<gb, 256, 0, s>>>(dacc.p, dpsi.p, cs, sn, n2);
    cheby_overlap<<<og, 256, 0, s>>>(d0.p, dpsi.p, N, npsi, dac.p + (size_t)3 * npsi * slot);
    return cudaGetLastError() == cudaSuccess ? EVR_OK : EVR_EDEVICE;
  };
  // the step reads psi and writes psi; b0/b1/b2 rotate inside.  The first step runs
  // eagerly (it also checks the launch sequence), the others replay a captured graph
  // whose autocorrelation slot is advanced by a device-side offset copy.
  if (nsteps > 0 && (rc = record_step(1))) return set_error(c, rc, "evr_cheby_propagate: step");
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  DevBuf slotbuf;  // the graph writes its overlap into slotbuf, copied to dac after each replay
  if (nsteps > 1) {
    if (slotbuf.alloc(3 * npsi)) return set_error(c, EVR_ENOMEM, "slot");
    c->capturing = true;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      c->capturing = false;
      return set_error(c, EVR_EDEVICE, "evr_cheby_propagate: begin capture");
    }
    int e = EVR_OK;
    {
      int saved_rc = EVR_OK;
      // record with the overlap going to slotbuf (zeroed inside the graph)
      if (cudaMemsetAsync(slotbuf.p, 0, sizeof(double) * 3 * npsi, s) != cudaSuccess) saved_rc = EVR_EDEVICE;
      if (!saved_rc) {
        if ((saved_rc = hpsi_interleaved(c, dpsi.p, ncol, dH.p, ncol, ncol, prec, s, OP_H)) == EVR_OK) {
          cheby_first<<<gb, 256, 0, s>>>(dpsi.p, dH.p, b1.p, dacc.p, E0, invEsc, coef[0], coef[1], n2);
          double* prev = dpsi.p;
          double* cur = b1.p;
          for (int k = 1; k < K && !saved_rc; ++k) {
            saved_rc = hpsi_interleaved(c, cur, ncol, dH.p, ncol, ncol, prec, s, OP_H);
            double* next = (k == 1) ? b0.p : prev;
            cheby_step<<<gb, 256, 0, s>>>(prev, cur, dH.p, next, dacc.p, E0, invEsc, coef[k + 1], n2);
            prev = cur;
            cur = next;
          }
          cheby_phase<<<gb, 256, 0, s>>>(dacc.p, dpsi.p, cs, sn, n2);
          cheby_overlap<<<og, 256, 0, s>>>(d0.p, dpsi.p, N, npsi, slotbuf.p);
        }
      }
      e = saved_rc;
    }
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    c->capturing = false;
    if (e || ce != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return set_error(c, e ? e : EVR_EDEVICE, "evr_cheby_propagate: capture");
    }
    if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
      cudaGraphDestroy(graph);
      return set_error(c, EVR_EDEVICE, "evr_cheby_propagate: instantiate");
    }
    for (int st = 2; st <= nsteps; ++st) {
      if (cudaGraphLaunch(exec, s) != cudaSuccess ||
          cudaMemcpyAsync(dac.p + (size_t)3 * npsi * st, slotbuf.p, sizeof(double) * 3 * npsi,
                          cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        return set_error(c, EVR_EDEVICE, "evr_cheby_propagate: graph launch");
      }
    }
  }
  std::vector<double> ac((size_t)3 * npsi * (nsteps + 1));
  cudaError_t ce = cudaMemcpyAsync(ac.data(), dac.p, sizeof(double) * ac.size(), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (ce != cudaSuccess) return set_error(c, EVR_EDEVICE, "evr_cheby_propagate: results");
  int bad_step = -1;
  for (int st = 0; st <= nsteps && bad_step < 0; ++st)
    for (int p = 0; p < npsi; ++p) {
      const double n0 = ac[3 * p + 2], nn = ac[(size_t)3 * npsi * st + 3 * p + 2];
      // FP32 contractions move the norm by ~1e-6 per step; divergence grows it without bound
      const double ntol = prec == EVR_PREC_FP32 ? 1e-3 : 1e-6;
      if (!(std::fabs(nn - n0) <= ntol * n0 + 1e-300)) { bad_step = st; break; }
    }
  if (autocorr)
    for (int st = 0; st <= nsteps; ++st)
      for (int p = 0; p < npsi; ++p) {
        autocorr[((size_t)st * npsi + p) * 2] = ac[(size_t)3 * npsi * st + 3 * p];
        autocorr[((size_t)st * npsi + p) * 2 + 1] = ac[(size_t)3 * npsi * st + 3 * p + 1];
      }
  if (psi_out) {
    std::vector<double> h(ne);
    if (cudaMemcpy(h.data(), dpsi.p, sizeof(double) * ne, cudaMemcpyDeviceToHost) != cudaSuccess)
      return set_error(c, EVR_EDEVICE, "evr_cheby_propagate: copy psi");
    for (int p = 0; p < npsi; ++p)
      for (int64_t k = 0; k < N; ++k) {
        psi_out[((size_t)p * N + k) * 2] = h[k * ncol + 2 * p];
        psi_out[((size_t)p * N + k) * 2 + 1] = h[k * ncol + 2 * p + 1];
      }
  }
  if (info) {
    info[0] = K;
    info[1] = (int64_t)nsteps * K * ncol;
    info[2] = bad_step;
  }
  if (bad_step >= 0)
    return set_error(c, EVR_ENOCONV, "evr_cheby_propagate: norm not conserved from step " + std::to_string(bad_step) +
                                         " (spectrum outside [emin, emax]?)");
  return EVR_OK;
}

// ---------------------------------------------------------------------------------------
// Short-iterative-Lanczos propagation (march_SIL, sub_module_propa_march.f90:2899-3100).
// Per time step and packet: q_1 = psi/|psi|, E0 = <q_1|H q_1>; Lanczos on H - E0 with
// alpha_k = Re<q_k|w>, w = (H - E0) q_k - beta_{k-1} q_{k-1}; after each alpha the
// propagator column u = exp(-i T_k dt) e_1 of the Lanczos matrix T_k (UPsi_spec :3101) is
// formed on the host, and the space stops growing when |u_k| < poly_tol (or at npoly);
// psi(t+dt) = |psi| exp(-i E0 dt) sum_k u_k q_k.  The packets of a call share the H.psi
// launches (one interleaved block of 2*npsi columns); their Lanczos scalars are separate,
// and a packet whose space is complete only idles until the last one is.  The scalars
// come to the host after every H.psi (one small copy), so a step is not a fixed launch
// sequence and is not captured as a graph.
#include "evr_krylov.h"

namespace {

constexpr int kMaxPackets = evr::kMaxBlock / 2;

struct PacketCoef {
  double x[kMaxPackets];
  double y[kMaxPackets];
  double z[kMaxPackets];
};

// w -= x_p q + y_p qprev (qprev may be null); element i of the block is packet i % npsi
__global__ void sil_residual(const double* __restrict__ q, const double* __restrict__ qprev, double* __restrict__ w,
                             PacketCoef cf, int npsi, int64_t n2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(i % npsi);
    const int64_t e = 2 * i;
    double wr = w[e] - cf.x[p] * q[e], wi = w[e + 1] - cf.x[p] * q[e + 1];
    if (qprev) {
      wr -= cf.y[p] * qprev[e];
      wi -= cf.y[p] * qprev[e + 1];
    }
    w[e] = wr;
    w[e + 1] = wi;
  }
}

// out = x_p * in
__global__ void sil_scale(const double* __restrict__ in, double* __restrict__ out, PacketCoef cf, int npsi, int64_t n2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(i % npsi);
    out[2 * i] = cf.x[p] * in[2 * i];
    out[2 * i + 1] = cf.x[p] * in[2 * i + 1];
  }
}

// acc (= when first, else +=) (x_p + i y_p) q
__global__ void sil_accumulate(const double* __restrict__ q, double* __restrict__ acc, PacketCoef cf, int npsi,
                               int64_t n2, int first) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(i % npsi);
    const int64_t e = 2 * i;
    const double a = q[e], b = q[e + 1];
    const double r = cf.x[p] * a - cf.y[p] * b, m = cf.x[p] * b + cf.y[p] * a;
    acc[e] = first ? r : acc[e] + r;
    acc[e + 1] = first ? m : acc[e + 1] + m;
  }
}

struct DevVecs {
  std::vector<double*> v;
  ~DevVecs() {
    for (double* p : v)
      if (p) cudaFree(p);
  }
};

}  // namespace

extern "C" int evr_sil_propagate(evr_ctx* c, const double* psi0, int npsi, double dt, int nsteps, int npoly,
                                 double poly_tol, int prec, double* autocorr, double* psi_out, int64_t* info) {
  if (!c) return EVR_EINVAL;
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  if (c->batch) return set_error(c, EVR_EINVAL, "evr_sil_propagate: not for batched contexts");
  if (!psi0 || npsi < 1 || npsi > kMaxPackets || nsteps < 0 || npoly < 1 || npoly > 256 || !(poly_tol > 0.0) ||
      !(dt > 0.0))
    return set_error(c, EVR_EINVAL, "evr_sil_propagate: bad arguments (1 <= npsi <= 32, 1 <= npoly <= 256, dt > 0, "
                                    "poly_tol > 0)");
  if (prec != EVR_PREC_FP64 && prec != EVR_PREC_FP32) return set_error(c, EVR_EINVAL, "unknown precision");
  if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, EVR_EDEVICE, "cudaSetDevice");
  const int64_t N = c->hp.Np * c->hp.nb0;
  const int ncol = 2 * npsi;
  const size_t ne = (size_t)N * ncol;
  const int64_t n2 = N * npsi;
  cudaStream_t s = c->stream;
  DevBuf d0, dpsi, dw, dred, dac;
  if (d0.alloc(ne) || dpsi.alloc(ne) || dw.alloc(ne) || dred.alloc((size_t)3 * npsi) ||
      dac.alloc((size_t)3 * npsi * (nsteps + 1)))
    return set_error(c, EVR_ENOMEM, "evr_sil_propagate: device allocation");
  {
    std::vector<double> h(ne);
    for (int p = 0; p < npsi; ++p)
      for (int64_t k = 0; k < N; ++k) {
        h[k * ncol + 2 * p] = psi0[((size_t)p * N + k) * 2];
        h[k * ncol + 2 * p + 1] = psi0[((size_t)p * N + k) * 2 + 1];
      }
    if (cudaMemcpyAsync(d0.p, h.data(), sizeof(double) * ne, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(dpsi.p, d0.p, sizeof(double) * ne, cudaMemcpyDeviceToDevice, s) ||
        cudaMemsetAsync(dac.p, 0, sizeof(double) * 3 * npsi * (nsteps + 1), s) || cudaStreamSynchronize(s))
      return set_error(c, EVR_EDEVICE, "evr_sil_propagate: upload");
  }
  int rc = ensure_workspace(c, ncol, prec);
  if (rc) return rc;
  const int gb = c->num_sms * 4;
  dim3 og((unsigned)std::min<int64_t>((N + 255) / 256, 1024), (unsigned)npsi);
  // <a|b> per packet -> host (re, im, |b|^2)
  std::vector<double> red((size_t)3 * npsi);
  auto overlap = [&](const double* a, const double* b, double* out_dev) -> int {
    double* o = out_dev ? out_dev : dred.p;
    if (!out_dev && cudaMemsetAsync(dred.p, 0, sizeof(double) * 3 * npsi, s) != cudaSuccess) return EVR_EDEVICE;
    cheby_overlap<<<og, 256, 0, s>>>(a, b, N, npsi, o);
    if (out_dev) return cudaGetLastError() == cudaSuccess ? EVR_OK : EVR_EDEVICE;
    if (cudaMemcpyAsync(red.data(), dred.p, sizeof(double) * 3 * npsi, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return EVR_EDEVICE;
    return EVR_OK;
  };
  if ((rc = overlap(d0.p, dpsi.p, dac.p))) return set_error(c, rc, "evr_sil_propagate: overlap");
  DevVecs Q;  // Krylov vectors, allocated as the space grows, kept across steps
  auto krylov = [&](int k) -> double* {
    while ((int)Q.v.size() <= k) {
      double* p = nullptr;
      if (cudaMalloc((void**)&p, sizeof(double) * ne) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
      }
      Q.v.push_back(p);
    }
    return Q.v[k];
  };
  const int op = c->op_form;
  int64_t n_hpsi = 0;
  int max_dim = 0;
  std::vector<double> nrm(npsi), E0(npsi);
  std::vector<std::vector<double>> alpha(npsi), beta(npsi), u_re(npsi), u_im(npsi);
  std::vector<int> dim(npsi);
  for (int st = 1; st <= nsteps; ++st) {
    PacketCoef cf{};
    if ((rc = overlap(dpsi.p, dpsi.p, nullptr))) return set_error(c, rc, "evr_sil_propagate: norm");
    for (int p = 0; p < npsi; ++p) {
      nrm[p] = std::sqrt(red[3 * p + 2]);
      cf.x[p] = nrm[p] > 0.0 ? 1.0 / nrm[p] : 0.0;
      alpha[p].clear();
      beta[p].clear();
      dim[p] = 0;
    }
    double* q0 = krylov(0);
    if (!q0) return set_error(c, EVR_ENOMEM, "evr_sil_propagate: Krylov vectors");
    sil_scale<<<gb, 256, 0, s>>>(dpsi.p, q0, cf, npsi, n2);
    int active = npsi;
    for (int k = 0; k < npoly && active > 0; ++k) {
      double* qk = Q.v[k];
      if ((rc = hpsi_interleaved(c, qk, ncol, dw.p, ncol, ncol, prec, s, op)))
        return set_error(c, rc, "evr_sil_propagate: H.psi");
      ++n_hpsi;
      if (k == 0) {
        if ((rc = overlap(qk, dw.p, nullptr))) return set_error(c, rc, "evr_sil_propagate: E0");
        for (int p = 0; p < npsi; ++p) E0[p] = red[3 * p];
      }
      PacketCoef r{};
      for (int p = 0; p < npsi; ++p) {  // a complete packet's columns are zero from here on
        r.x[p] = E0[p];
        r.y[p] = (k > 0 && (size_t)k <= beta[p].size()) ? beta[p][k - 1] : 0.0;
      }
      sil_residual<<<gb, 256, 0, s>>>(qk, k > 0 ? Q.v[k - 1] : nullptr, dw.p, r, npsi, n2);
      if ((rc = overlap(qk, dw.p, nullptr))) return set_error(c, rc, "evr_sil_propagate: alpha");
      PacketCoef a{}, sc{};
      for (int p = 0; p < npsi; ++p) {
        if (dim[p]) continue;  // complete: the packet idles
        alpha[p].push_back(red[3 * p]);
        const int n = k + 1;
        u_re[p].assign(n, 0.0);
        u_im[p].assign(n, 0.0);
        if (!krylov_propagator_column(n, alpha[p].data(), beta[p].data(), dt, u_re[p].data(), u_im[p].data()))
          return set_error(c, EVR_ENOCONV, "evr_sil_propagate: Lanczos matrix eigen-decomposition");
        if (std::hypot(u_re[p][k], u_im[p][k]) < poly_tol || k == npoly - 1 || nrm[p] == 0.0) {
          dim[p] = n;
          --active;
        }
        a.x[p] = alpha[p][k];
      }
      if (active == 0) break;
      sil_residual<<<gb, 256, 0, s>>>(qk, nullptr, dw.p, a, npsi, n2);
      if ((rc = overlap(dw.p, dw.p, nullptr))) return set_error(c, rc, "evr_sil_propagate: beta");
      double* qn = krylov(k + 1);
      if (!qn) return set_error(c, EVR_ENOMEM, "evr_sil_propagate: Krylov vectors");
      for (int p = 0; p < npsi; ++p) {
        if (dim[p]) continue;
        const double b = std::sqrt(red[3 * p + 2]);
        double tmax = std::fabs(E0[p]);
        for (double x : alpha[p]) tmax = std::max(tmax, std::fabs(x));
        for (double x : beta[p]) tmax = std::max(tmax, x);
        if (!(b > 1e-13 * std::max(tmax, 1e-300))) {  // invariant subspace: the space is complete
          dim[p] = k + 1;
          --active;
          continue;
        }
        beta[p].push_back(b);
        sc.x[p] = 1.0 / b;
      }
      sil_scale<<<gb, 256, 0, s>>>(dw.p, qn, sc, npsi, n2);
    }
    // psi = |psi| exp(-i E0 dt) sum_k u_k q_k
    int kmax = 0;
    for (int p = 0; p < npsi; ++p) kmax = std::max(kmax, dim[p]);
    max_dim = std::max(max_dim, kmax);
    for (int k = 0; k < kmax; ++k) {
      PacketCoef u{};
      for (int p = 0; p < npsi; ++p) {
        if (k >= dim[p]) continue;
        const double cs = std::cos(E0[p] * dt), sn = -std::sin(E0[p] * dt);
        u.x[p] = nrm[p] * (cs * u_re[p][k] - sn * u_im[p][k]);
        u.y[p] = nrm[p] * (cs * u_im[p][k] + sn * u_re[p][k]);
      }
      sil_accumulate<<<gb, 256, 0, s>>>(Q.v[k], dpsi.p, u, npsi, n2, k == 0);
    }
    if ((rc = overlap(d0.p, dpsi.p, dac.p + (size_t)3 * npsi * st))) return set_error(c, rc, "evr_sil_propagate: overlap");
  }
  std::vector<double> ac((size_t)3 * npsi * (nsteps + 1));
  if (cudaMemcpyAsync(ac.data(), dac.p, sizeof(double) * ac.size(), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return set_error(c, EVR_EDEVICE, "evr_sil_propagate: results");
  int bad_step = -1;
  const double ntol = prec == EVR_PREC_FP32 ? 1e-3 : 1e-6;
  for (int st = 0; st <= nsteps && bad_step < 0; ++st)
    for (int p = 0; p < npsi; ++p) {
      const double n0 = ac[3 * p + 2], nn = ac[(size_t)3 * npsi * st + 3 * p + 2];
      if (!(std::fabs(nn - n0) <= ntol * n0 + 1e-300)) { bad_step = st; break; }
    }
  if (autocorr)
    for (int st = 0; st <= nsteps; ++st)
      for (int p = 0; p < npsi; ++p) {
        autocorr[((size_t)st * npsi + p) * 2] = ac[(size_t)3 * npsi * st + 3 * p];
        autocorr[((size_t)st * npsi + p) * 2 + 1] = ac[(size_t)3 * npsi * st + 3 * p + 1];
      }
  if (psi_out) {
    std::vector<double> h(ne);
    if (cudaMemcpy(h.data(), dpsi.p, sizeof(double) * ne, cudaMemcpyDeviceToHost) != cudaSuccess)
      return set_error(c, EVR_EDEVICE, "evr_sil_propagate: copy psi");
    for (int p = 0; p < npsi; ++p)
      for (int64_t k = 0; k < N; ++k) {
        psi_out[((size_t)p * N + k) * 2] = h[k * ncol + 2 * p];
        psi_out[((size_t)p * N + k) * 2 + 1] = h[k * ncol + 2 * p + 1];
      }
  }
  if (info) {
    info[0] = max_dim;
    info[1] = n_hpsi * ncol;
    info[2] = bad_step;
  }
  if (bad_step >= 0)
    return set_error(c, EVR_ENOCONV, "evr_sil_propagate: norm not conserved from step " + std::to_string(bad_step));
  return EVR_OK;
}
