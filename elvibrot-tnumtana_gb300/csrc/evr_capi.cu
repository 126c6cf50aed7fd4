// evr_capi.cu -- the C ABI of include/evr_gpu.h: context life cycle, table read-back,
// H.psi entry points.  Davidson and Chebyshev drivers live in evr_davidson.cu and
// evr_propagate.cu.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "evr_internal.h"

using namespace evr;

#define EVR_CU(call, what)                              \
  do {                                                  \
    int _rc = cuda_check(c, (call), what);              \
    if (_rc != EVR_OK) return _rc;                      \
  } while (0)

namespace evr {

void grid_values_to_device(const HostProblem& P, const double* v, int layout, bool with_shift,
                           std::vector<double>& dev, std::vector<float>& dev32) {
  const int nb2 = P.nb0 * P.nb0;
  const size_t n = (size_t)P.sum_nq * nb2;
  dev.assign(n, 0.0);
  dev32.assign(n, 0.0f);
  for (const TermDesc& T : P.terms)
    for (int ab = 0; ab < nb2; ++ab) {
      const double shift = with_shift && ab % (P.nb0 + 1) == 0 ? T.vshift : 0.0;
      for (int64_t qp = 0; qp < T.NQ; ++qp) {
        const int64_t q = P.grid_perm[(size_t)T.off_nq + qp] - T.off_nq;
        const size_t src = layout == EVR_VGRID_TERMS ? (size_t)T.off_nq * nb2 + (size_t)ab * T.NQ + q
                                                     : (size_t)(T.off_nq + q) + (size_t)P.sum_nq * ab;
        const size_t dst = (size_t)T.off_nq * nb2 + (size_t)ab * T.NQ + qp;
        dev[dst] = v[src] + shift;
        dev32[dst] = (float)dev[dst];
      }
    }
}

}  // namespace evr

extern "C" {

int evr_create(evr_ctx** out, const evr_problem_desc* desc, int device) {
  if (!out) return EVR_EINVAL;
  *out = nullptr;
  evr_ctx* c = new (std::nothrow) evr_ctx();
  if (!c) return EVR_ENOMEM;
  c->device = device;
  if (device < 0) {  // host-only context: tables are built and can be read back, no device work
    *out = c;
    c->host_only = true;
    return build_host_problem(desc, c->hp, c->err);
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    (void)cudaGetLastError();
    c->err = "no CUDA device " + std::to_string(device);
    *out = c;
    return EVR_EDEVICE;
  }
  *out = c;
  EVR_CU(cudaSetDevice(device), "cudaSetDevice");
  EVR_CU(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device), "attr");
  EVR_CU(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  for (auto& e : c->ev) EVR_CU(cudaEventCreate(&e), "cudaEventCreate");
  int rc = build_host_problem(desc, c->hp, c->err);
  if (rc) return rc;
  rc = upload_problem(c);
  return rc;
}

int evr_destroy(evr_ctx* c) {
  if (!c) return EVR_OK;
  if (c->host_only) {
    free_batch_info(c);
    delete c;
    return EVR_OK;
  }
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_control(c);
  free_batch_info(c);
  free_workspace(c);
  free_problem(c);
  if (c->pinned) cudaFreeHost(c->pinned);
  if (c->stream) cudaStreamDestroy(c->stream);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  delete c;
  return EVR_OK;
}

const char* evr_last_error(const evr_ctx* c) { return c ? c->err.c_str() : "null context"; }

int evr_sizes(const evr_ctx* c, evr_sizes_t* o) {
  if (!c || !o) return EVR_EINVAL;
  const HostProblem& P = c->hp;
  o->Np = P.Np;
  o->N = P.Np * P.nb0;
  o->n_terms = (int64_t)P.terms.size();
  o->sum_nb = P.sum_nb;
  o->sum_nq = P.sum_nq;
  o->max_nq_term = P.max_nq;
  o->flop_per_hpsi = P.flop_per_hpsi;
  return EVR_OK;
}

int evr_get_tables(const evr_ctx* c, int* term_l, double* weight, int* map, int* packed) {
  if (!c) return EVR_EINVAL;
  const HostProblem& P = c->hp;
  if (term_l) std::copy(P.term_l.begin(), P.term_l.end(), term_l);
  if (weight) std::copy(P.weight.begin(), P.weight.end(), weight);
  if (map) std::copy(P.map.begin(), P.map.end(), map);
  if (packed) std::copy(P.packed.begin(), P.packed.end(), packed);
  return EVR_OK;
}

int evr_get_basis(const evr_ctx* c, int mode, int level, int* nb_nq, double* x, double* w, double* d0b, double* d1b,
                  double* d2b, double* bgw, double* d1gg, double* d2gg) {
  if (!c || mode < 0 || mode >= (int)c->hp.bas.size() || level < 0 || level >= (int)c->hp.bas[mode].size() ||
      !nb_nq)
    return EVR_EINVAL;
  const Basis1D& b = c->hp.bas[mode][level];
  nb_nq[0] = b.nb;
  nb_nq[1] = b.nq;
  auto cp = [](const std::vector<double>& v, double* d) {
    if (d) std::copy(v.begin(), v.end(), d);
  };
  cp(b.x, x); cp(b.w, w); cp(b.d0b, d0b); cp(b.d1b, d1b); cp(b.d2b, d2b); cp(b.bgw, bgw); cp(b.d1gg, d1gg);
  cp(b.d2gg, d2gg);
  return EVR_OK;
}

int evr_get_vgrid(const evr_ctx* c0, double* v) {
  evr_ctx* c = const_cast<evr_ctx*>(c0);
  if (!c || !v) return EVR_EINVAL;
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  if (c->batch) return set_error(c, EVR_EINVAL, "evr_get_vgrid: not for batched contexts");
  EVR_CU(cudaSetDevice(c->device), "cudaSetDevice");
  const HostProblem& P = c->hp;
  const int nb2 = P.nb0 * P.nb0;
  const size_t n = (size_t)P.sum_nq * nb2;
  std::vector<double> dev(n);
  EVR_CU(cudaMemcpyAsync(dev.data(), c->dp.vgrid, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
         "copy vgrid");
  EVR_CU(cudaStreamSynchronize(c->stream), "sync");
  // device grid points follow each term's permuted mode order: back to the reference order;
  // the device table holds V plus the constant of the term's dropped 1-point modes
  for (const TermDesc& T : P.terms)
    for (int ab = 0; ab < nb2; ++ab) {
      const double shift = ab % (P.nb0 + 1) == 0 ? T.vshift : 0.0;
      for (int64_t qp = 0; qp < T.NQ; ++qp) {
        const int64_t q = P.grid_perm[(size_t)T.off_nq + qp] - T.off_nq;
        v[(size_t)T.off_nq * nb2 + (size_t)ab * T.NQ + q] = dev[(size_t)T.off_nq * nb2 + (size_t)ab * T.NQ + qp] - shift;
      }
    }
  return EVR_OK;
}

// Replaces the device V table (and its FP32 copy) with caller-supplied grid values: the
// inverse of evr_get_vgrid's mapping, done on the host and uploaded with plain copies.
int evr_set_vgrid(evr_ctx* c, const double* v, int layout) {
  if (!c) return EVR_EINVAL;
  if (!v || (layout != EVR_VGRID_TERMS && layout != EVR_VGRID_REF))
    return set_error(c, EVR_EINVAL, "evr_set_vgrid: null values or unknown layout");
  {
    const int64_t n = c->hp.sum_nq * c->hp.nb0 * c->hp.nb0;
    for (int64_t i = 0; i < n; ++i)
      if (!std::isfinite(v[i]))
        return set_error(c, EVR_EINVAL, "evr_set_vgrid: value " + std::to_string(i) + " is not finite");
  }
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  if (c->batch) return set_error(c, EVR_EINVAL, "evr_set_vgrid: not for batched contexts");
  EVR_CU(cudaSetDevice(c->device), "cudaSetDevice");
  std::vector<double> dev;
  std::vector<float> dev32;
  grid_values_to_device(c->hp, v, layout, true, dev, dev32);
  const size_t n = dev.size();
  // an H.psi still reading the old table may run on a caller's stream: wait for the device
  EVR_CU(cudaDeviceSynchronize(), "sync before vgrid update");
  free_control(c);  // a forward state of the old operator (see evr_set_ggrid)
  EVR_CU(cudaMemcpyAsync(c->dp.vgrid, dev.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream),
         "copy vgrid");
  EVR_CU(cudaMemcpyAsync(c->dp.vgrid32, dev32.data(), n * sizeof(float), cudaMemcpyHostToDevice, c->stream),
         "copy vgrid32");
  EVR_CU(cudaStreamSynchronize(c->stream), "sync");
  return EVR_OK;
}

// Replaces (or creates) the per-point G(Q) table of a type-10 context with host values.
// The rows follow grid_eval_kernel's layout: per device grid point one row of
// g_table_stride(D) entries, (i, j >= i) over the term's positions in its permuted order.
int evr_set_ggrid(evr_ctx* c, const double* G) {
  if (!c) return EVR_EINVAL;
  if (!G) return set_error(c, EVR_EINVAL, "evr_set_ggrid: null values");
  if (c->batch) return set_error(c, EVR_EINVAL, "evr_set_ggrid: not for batched contexts");
  const HostProblem& P = c->hp;
  if (P.keo_type != 10) return set_error(c, EVR_EINVAL, "evr_set_ggrid: the KEO of the context is not type 10");
  const int D = P.D, stride = g_table_stride(D);
  for (int64_t i = 0; i < P.sum_nq * D * D; ++i)
    if (!std::isfinite(G[i]))
      return set_error(c, EVR_EINVAL, "evr_set_ggrid: value " + std::to_string(i) + " is not finite");
  for (int64_t iq = 0; iq < P.sum_nq; ++iq) {  // the matrices must be symmetric
    const double* Gq = G + (size_t)iq * D * D;
    for (int i = 0; i < D; ++i)
      for (int j = i + 1; j < D; ++j) {
        const double a = Gq[i + (size_t)D * j], b = Gq[j + (size_t)D * i];
        if (!(std::fabs(a - b) <= 1e-12 * std::max(1.0, std::max(std::fabs(a), std::fabs(b)))))
          return set_error(c, EVR_EINVAL, "evr_set_ggrid: G(Q) is not symmetric at grid point " +
                                              std::to_string(iq) + " (entries " + std::to_string(i) + ", " +
                                              std::to_string(j) + ")");
      }
  }
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  EVR_CU(cudaSetDevice(c->device), "cudaSetDevice");
  const size_t ng = (size_t)P.sum_nq * stride;
  std::vector<double> dev(ng, 0.0);
  std::vector<float> dev32(ng, 0.0f);
  for (const TermDesc& T : P.terms)
    for (int64_t qp = 0; qp < T.NQ; ++qp) {
      const int64_t iq = P.grid_perm[(size_t)T.off_nq + qp];  // the reference's point
      const double* Gq = G + (size_t)iq * D * D;
      const size_t row = (size_t)(T.off_nq + qp) * stride;
      int e = 0;
      for (int i = 0; i < T.D; ++i)
        for (int j = i; j < T.D; ++j, ++e) {
          const int oi = T.perm[i], oj = T.perm[j];
          dev[row + e] = 0.5 * (Gq[oi + (size_t)D * oj] + Gq[oj + (size_t)D * oi]);
          dev32[row + e] = (float)dev[row + e];
        }
    }
  // an H.psi still reading the old table may run on a caller's stream: wait for the device
  EVR_CU(cudaDeviceSynchronize(), "sync before G table update");
  // an optimal-control forward state was propagated with the old operator: a gradient
  // would mix the two, so it is discarded (evr_oc_backward then asks for a new forward)
  free_control(c);
  if (!c->dp_ggrid || !c->dp_ggrid32) {  // a context made with constant G gets its table now
    cudaError_t e = cudaSuccess;
    if (!c->dp_ggrid) e = cudaMalloc((void**)&c->dp_ggrid, ng * sizeof(double));
    if (e == cudaSuccess && !c->dp_ggrid32) e = cudaMalloc((void**)&c->dp_ggrid32, ng * sizeof(float));
    if (e != cudaSuccess) {
      if (c->dp_ggrid) cudaFree(c->dp_ggrid);
      if (c->dp_ggrid32) cudaFree(c->dp_ggrid32);
      c->dp_ggrid = nullptr;
      c->dp_ggrid32 = nullptr;
      EVR_CU(e, "cudaMalloc G table");
    }
    // launch sequences captured with the constant G (optimal-control graphs) read no
    // table: drop them so that they are recaptured with it
    ++c->ws_gen;
  }
  EVR_CU(cudaMemcpyAsync(c->dp_ggrid, dev.data(), ng * sizeof(double), cudaMemcpyHostToDevice, c->stream),
         "copy G table");
  EVR_CU(cudaMemcpyAsync(c->dp_ggrid32, dev32.data(), ng * sizeof(float), cudaMemcpyHostToDevice, c->stream),
         "copy G table (FP32)");
  EVR_CU(cudaStreamSynchronize(c->stream), "sync");
  return EVR_OK;
}

// Jacobian and rho of a type-10 operator per grid point (the reference's point order):
// stored as (Jac, sqrt(rho/Jac)) rows in the device's point order, FP64 and FP32.  Null
// arrays remove the table (Jac = rho = 1).
int evr_set_jacobian(evr_ctx* c, const double* jac, const double* rho) {
  if (!c) return EVR_EINVAL;
  if (c->batch) return set_error(c, EVR_EINVAL, "evr_set_jacobian: not for batched contexts");
  const HostProblem& P = c->hp;
  if (P.keo_type != 10) return set_error(c, EVR_EINVAL, "evr_set_jacobian: the KEO of the context is not type 10");
  if ((jac == nullptr) != (rho == nullptr))
    return set_error(c, EVR_EINVAL, "evr_set_jacobian: give both Jac and rho, or neither");
  if (jac)
    for (int64_t iq = 0; iq < P.sum_nq; ++iq)
      if (!(jac[iq] > 0.0) || !(rho[iq] > 0.0) || !std::isfinite(jac[iq]) || !std::isfinite(rho[iq]))
        return set_error(c, EVR_EINVAL, "evr_set_jacobian: Jac and rho must be positive and finite (grid point " +
                                            std::to_string(iq) + ")");
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  EVR_CU(cudaSetDevice(c->device), "cudaSetDevice");
  EVR_CU(cudaDeviceSynchronize(), "sync before Jacobian update");
  free_control(c);  // a forward state of the old operator (see evr_set_ggrid)
  if (!jac) {
    if (c->dp_jgrid) cudaFree(c->dp_jgrid);
    if (c->dp_jgrid32) cudaFree(c->dp_jgrid32);
    c->dp_jgrid = nullptr;
    c->dp_jgrid32 = nullptr;
    clear_item_sets(c);
    free_stages(c);
    return EVR_OK;
  }
  const size_t n = (size_t)P.sum_nq * 2;
  std::vector<double> dev(n);
  std::vector<float> dev32(n);
  for (const TermDesc& T : P.terms)
    for (int64_t qp = 0; qp < T.NQ; ++qp) {
      const int64_t iq = P.grid_perm[(size_t)T.off_nq + qp];
      const size_t r = (size_t)(T.off_nq + qp) * 2;
      dev[r] = jac[iq];
      dev[r + 1] = std::sqrt(rho[iq] / jac[iq]);
      dev32[r] = (float)dev[r];
      dev32[r + 1] = (float)dev[r + 1];
    }
  if (!c->dp_jgrid) {
    cudaError_t e = cudaMalloc((void**)&c->dp_jgrid, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->dp_jgrid32, n * sizeof(float));
    if (e != cudaSuccess) {
      if (c->dp_jgrid) cudaFree(c->dp_jgrid);
      c->dp_jgrid = nullptr;
      c->dp_jgrid32 = nullptr;
      EVR_CU(e, "cudaMalloc Jacobian table");
    }
    clear_item_sets(c);  // every term moves to the general kernel
    free_stages(c);
  }
  EVR_CU(cudaMemcpyAsync(c->dp_jgrid, dev.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream),
         "copy Jacobian table");
  EVR_CU(cudaMemcpyAsync(c->dp_jgrid32, dev32.data(), n * sizeof(float), cudaMemcpyHostToDevice, c->stream),
         "copy Jacobian table (FP32)");
  EVR_CU(cudaStreamSynchronize(c->stream), "sync");
  return EVR_OK;
}

int evr_set_kernel_path(evr_ctx* c, int path) {
  if (!c) return EVR_EINVAL;
  if (path < 0 || path > 2) return set_error(c, EVR_EINVAL, "evr_set_kernel_path: 0, 1 or 2");
  const bool slab = path >= 1, stages = path == 1, all = path == 2;
  if (c->use_slab != slab || c->use_stages != stages || c->slab_all != all) {
    c->use_slab = slab;
    c->use_stages = stages;
    c->slab_all = all;
    if (!c->host_only) {
      cudaSetDevice(c->device);
      cudaStreamSynchronize(c->stream);
      free_workspace(c);  // work decompositions depend on the path
    }
  }
  return EVR_OK;
}

int evr_set_tensor_cores(evr_ctx* c, int on, int min_km) {
  if (!c) return EVR_EINVAL;
  if (min_km < 0) return set_error(c, EVR_EINVAL, "evr_set_tensor_cores: min_km < 0");
  const bool tc = on != 0;
  if (c->use_tc != tc || c->tc_min_km != min_km) {
    c->use_tc = tc;
    c->tc_min_km = min_km;
    if (!c->host_only) {
      cudaSetDevice(c->device);
      cudaStreamSynchronize(c->stream);
      clear_item_sets(c);  // FP32 work decompositions depend on the shared memory left
    }
  }
  return EVR_OK;
}

int evr_set_operator(evr_ctx* c, int form) {
  if (!c) return EVR_EINVAL;
  if (form != EVR_OP_H && form != EVR_OP_HT && form != EVR_OP_HSYM) return set_error(c, EVR_EINVAL, "operator form");
  c->op_form = form;
  return EVR_OK;
}

int evr_hpsi_device(evr_ctx* c, const double* psi, int64_t ld_psi, double* hpsi, int64_t ld_hpsi, int nvec, int layout,
                    int prec, void* stream) {
  if (!c) return EVR_EINVAL;
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  if (!psi || !hpsi || nvec < 1) return set_error(c, EVR_EINVAL, "evr_hpsi_device: null pointer or nvec < 1");
  if (prec != EVR_PREC_FP64 && prec != EVR_PREC_FP32) return set_error(c, EVR_EINVAL, "unknown precision");
  const int64_t N = c->hp.Np * c->hp.nb0;
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
  EVR_CU(cudaSetDevice(c->device), "cudaSetDevice");
  if (layout == EVR_LAYOUT_INTERLEAVED) {
    if (ld_psi < nvec || ld_hpsi < nvec) return set_error(c, EVR_EINVAL, "interleaved ld < nvec");
    return hpsi_blocks(c, psi, ld_psi, hpsi, ld_hpsi, nvec, prec, s, c->op_form);
  }
  if (layout != EVR_LAYOUT_COLMAJOR) return set_error(c, EVR_EINVAL, "unknown layout");
  if (ld_psi < N || ld_hpsi < N) return set_error(c, EVR_EINVAL, "column-major ld < N");
  int64_t kernels = 0;
  for (int v0 = 0; v0 < nvec; v0 += kMaxBlock) {
    const int nb = std::min(kMaxBlock, nvec - v0);
    int rc = ensure_workspace(c, nb, prec);
    if (rc) return rc;
    double* xin = c->ws.xin;
    double* xout = c->ws.xout;
    if ((rc = transpose_to_interleaved(psi + v0 * ld_psi, ld_psi, xin, nb, N, nb, s)))
      return set_error(c, rc, "transpose");
    if ((rc = hpsi_interleaved(c, xin, nb, xout, nb, nb, prec, s, c->op_form))) return rc;
    if ((rc = transpose_from_interleaved(xout, nb, hpsi + v0 * ld_hpsi, ld_hpsi, N, nb, s)))
      return set_error(c, rc, "transpose");
    kernels += c->last_kernels + 2;
  }
  c->last_kernels = kernels;
  return EVR_OK;
}

int evr_hpsi_host(evr_ctx* c, const double* psi, int64_t ld_psi, double* hpsi, int64_t ld_hpsi, int nvec, int layout,
                  int prec) {
  if (!c) return EVR_EINVAL;
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  if (!psi || !hpsi || nvec < 1) return set_error(c, EVR_EINVAL, "evr_hpsi_host: null pointer or nvec < 1");
  if (prec != EVR_PREC_FP64 && prec != EVR_PREC_FP32) return set_error(c, EVR_EINVAL, "unknown precision");
  if (layout != EVR_LAYOUT_INTERLEAVED && layout != EVR_LAYOUT_COLMAJOR) return set_error(c, EVR_EINVAL, "layout");
  const int64_t N = c->hp.Np * c->hp.nb0;
  if (layout == EVR_LAYOUT_INTERLEAVED && (ld_psi < nvec || ld_hpsi < nvec))
    return set_error(c, EVR_EINVAL, "interleaved ld < nvec");
  if (layout == EVR_LAYOUT_COLMAJOR && (ld_psi < N || ld_hpsi < N)) return set_error(c, EVR_EINVAL, "column-major ld < N");
  EVR_CU(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t s = c->stream;
  int64_t kernels = 0;
  for (int v0 = 0; v0 < nvec; v0 += kMaxBlock) {
    const int nb = std::min(kMaxBlock, nvec - v0);
    int rc = ensure_workspace(c, nb, prec);
    if (rc) return rc;
    double* xin = c->ws.xin;
    double* xout = c->ws.xout;
    if (layout == EVR_LAYOUT_INTERLEAVED) {
      EVR_CU(cudaMemcpy2DAsync(xin, nb * sizeof(double), psi + v0, ld_psi * sizeof(double), nb * sizeof(double), N,
                               cudaMemcpyHostToDevice, s), "H2D");
      if ((rc = hpsi_interleaved(c, xin, nb, xout, nb, nb, prec, s, c->op_form))) return rc;
      EVR_CU(cudaMemcpy2DAsync(hpsi + v0, ld_hpsi * sizeof(double), xout, nb * sizeof(double), nb * sizeof(double), N,
                               cudaMemcpyDeviceToHost, s), "D2H");
      kernels += c->last_kernels;
    } else {
      // column-major staging in xout, transposed on the device into xin
      EVR_CU(cudaMemcpy2DAsync(xout, N * sizeof(double), psi + v0 * ld_psi, ld_psi * sizeof(double),
                               N * sizeof(double), nb, cudaMemcpyHostToDevice, s), "H2D");
      if ((rc = transpose_to_interleaved(xout, N, xin, nb, N, nb, s))) return set_error(c, rc, "transpose");
      if ((rc = hpsi_interleaved(c, xin, nb, xout, nb, nb, prec, s, c->op_form))) return rc;
      kernels += c->last_kernels + 2;
      if ((rc = transpose_from_interleaved(xout, nb, xin, N, N, nb, s))) return set_error(c, rc, "transpose");
      EVR_CU(cudaMemcpy2DAsync(hpsi + v0 * ld_hpsi, ld_hpsi * sizeof(double), xin, N * sizeof(double),
                               N * sizeof(double), nb, cudaMemcpyDeviceToHost, s), "D2H");
    }
  }
  c->last_kernels = kernels;
  EVR_CU(cudaStreamSynchronize(s), "evr_hpsi_host");
  return check_item_bounds(c);
}


int evr_last_kernel_ms(evr_ctx* c, float* items_ms, float* reduce_ms) {
  if (!c || c->host_only) return EVR_EINVAL;
  EVR_CU(cudaEventSynchronize(c->ev[2]), "event sync");
  float a = 0.f, b = 0.f;
  EVR_CU(cudaEventElapsedTime(&a, c->ev[0], c->ev[1]), "event time");
  EVR_CU(cudaEventElapsedTime(&b, c->ev[1], c->ev[2]), "event time");
  if (items_ms) *items_ms = a;
  if (reduce_ms) *reduce_ms = b;
  return EVR_OK;
}

int evr_last_launch_count(const evr_ctx* c, int64_t* kernels, int64_t* items) {
  if (!c) return EVR_EINVAL;
  if (kernels) *kernels = c->last_kernels;
  if (items) *items = c->last_items;
  return EVR_OK;
}

}  // extern "C"
