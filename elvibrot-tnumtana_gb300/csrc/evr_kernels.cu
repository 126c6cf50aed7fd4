// evr_kernels.cu -- sm_103a kernels of the SG4 / direct-product H.psi path.
//
// One persistent kernel runs the whole per-term pipeline of the reference's
// sub_TabOpPsi_OF_ONEDP_FOR_SGtype4 (Source_ElVibRot/sub_Operator/sub_OpPsi_SG4.f90:1354-1668)
// for a (term, vector tile) work item per CTA:
//   gather psi_packed -> term basis   (tabPackedBasis_TO_tabR_AT_iG, BtoG_GtoB_SG4.f90:1176-1246)
//   B->G, modes 1..D with d0b         (BDP_TO_GDP_OF_SmolyakRep, :2385-2496)      [fused with the gather]
//   V.psi on the grid                 (:1566-1576)
//   KEO type 10: D first derivatives, G(Q) combination, D derivatives accumulated
//                                     (:1578-1628, DerivOp_TO_RDP_OF_SmolaykRep :2690-2795)
//   KEO type 1: F2 d2 / d1 d1 terms   (:1490-1546)
//   G->B, modes 1..D with d0b^T w     (GDP_TO_BDP_OF_SmolyakRep, :2497-2581)
// The weighted scatter-add of the reference (tabR_AT_iG_TO_tabPackedBasis, :1250-1289,
// OMP ATOMIC) becomes a deterministic CSR gather-reduce over the transposed map.
//
// Work buffers of an item live in shared memory when they fit, otherwise in a per-CTA
// slab of global memory (L2-resident for the CTAs in flight).  Every stage is a small
// dense contraction along one mode, executed by the whole CTA with one output fibre
// (M values) per thread and the 1-D matrix read through the read-only cache.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "evr_internal.h"
#include "evr_kernels_impl.cuh"

namespace evr {

using namespace kern;

namespace {

// y[k*ldy + v] = scale * sum_{e in row k} w_e * (ht[src_e*ldh + v] (+ ht2[...]))   (FP64 accumulation)
// The first short_blocks CTAs take the rows of at most kCsrShortRow entries, one thread per
// (row, vector) summing its row in order.  The others take the long rows of the list (the
// low basis functions, which every term's basis holds: at D=12 L=6 the first row has
// 18,564 entries), one CTA per row: thread (g, l) sums the entries g, g + ng, ... of vector
// v0 + l, and the ng partial sums of each vector are added in a fixed pairwise tree.  Both
// orders are fixed, so the result is the same run to run.
template <typename T>
__global__ void __launch_bounds__(256) csr_reduce_kernel(const int64_t* __restrict__ ptr,
                                                         const int64_t* __restrict__ src,
                                                         const double* __restrict__ wt, const T* __restrict__ ht,
                                                         const T* __restrict__ ht2, int64_t ldh, double scale,
                                                         double* __restrict__ y, int64_t ldy, int64_t N, int nvec,
                                                         const int64_t* __restrict__ long_rows, int64_t n_long,
                                                         int short_blocks) {
  if ((int)blockIdx.x < short_blocks) {
    const int64_t total = N * nvec;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)short_blocks * blockDim.x) {
      const int64_t k = idx / nvec;
      const int v = (int)(idx - k * nvec);
      const int64_t e0 = __ldg(ptr + k), e1 = __ldg(ptr + k + 1);
      if (e1 - e0 > kCsrShortRow) continue;  // a long row: the CTAs below
      double s = 0.0;
      if (ht2) {
        for (int64_t e = e0; e < e1; ++e) {
          const int64_t o = __ldg(src + e) * ldh + v;
          s = fma(__ldg(wt + e), (double)ht[o] + (double)ht2[o], s);
        }
      } else {
        for (int64_t e = e0; e < e1; ++e) s = fma(__ldg(wt + e), (double)ht[__ldg(src + e) * ldh + v], s);
      }
      y[k * ldy + v] = scale * s;
    }
    return;
  }
  __shared__ double part[256];
  const int vc = nvec < 32 ? nvec : 32;         // vector lanes
  const int ng = (int)blockDim.x / vc;          // entry groups
  const int g = (int)threadIdx.x / vc, l = (int)threadIdx.x - g * vc;
  const bool on = g < ng;
  const int nlb = (int)gridDim.x - short_blocks;
  for (int64_t li = (int64_t)blockIdx.x - short_blocks; li < n_long; li += nlb) {
    const int64_t k = __ldg(long_rows + li);
    const int64_t e0 = __ldg(ptr + k), e1 = __ldg(ptr + k + 1);
    for (int v0 = 0; v0 < nvec; v0 += vc) {
      const int v = v0 + l;
      double s = 0.0;
      if (on && v < nvec) {
        if (ht2) {
          for (int64_t e = e0 + g; e < e1; e += ng) {
            const int64_t o = __ldg(src + e) * ldh + v;
            s = fma(__ldg(wt + e), (double)ht[o] + (double)ht2[o], s);
          }
        } else {
          for (int64_t e = e0 + g; e < e1; e += ng) s = fma(__ldg(wt + e), (double)ht[__ldg(src + e) * ldh + v], s);
        }
      }
      part[threadIdx.x] = s;
      __syncthreads();
      for (int h = 1; h < ng; h <<= 1) {
        if (on && (g & (2 * h - 1)) == 0 && g + h < ng) part[threadIdx.x] += part[threadIdx.x + h * vc];
        __syncthreads();
      }
      if (g == 0 && v < nvec) y[k * ldy + v] = scale * part[l];
      __syncthreads();
    }
  }
}

// launch of csr_reduce_kernel: the short-row CTAs (at most 16 per SM) and one CTA per long
// row up to 8 per SM
template <typename T>
static cudaError_t launch_csr_reduce(const evr_ctx* c, const T* ht, const T* ht2, int64_t ldh, double scale,
                                     double* y, int64_t ldy, int nvec, cudaStream_t s) {
  const int64_t N = c->hp.Np * c->hp.nb0;
  const int sb = (int)std::max<int64_t>(1, std::min<int64_t>((N * nvec + 255) / 256, (int64_t)c->num_sms * 16));
  const int lb = (int)std::min<int64_t>(c->dp.n_long, (int64_t)c->num_sms * 8);
  csr_reduce_kernel<T><<<sb + lb, 256, 0, s>>>(c->dp.csr_ptr, c->dp.csr_src, c->dp.csr_w, ht, ht2, ldh, scale, y, ldy,
                                               N, nvec, c->dp.csr_long, c->dp.n_long, sb);
  return cudaGetLastError();
}

// grid tables: V_ab(Q) from monomials (plus the term's constant of dropped 1-point modes on
// the diagonal when with_shift) and the symmetric G(Q) = G0 + sum_k g_ijk Q_k over the
// term's positions; the dropped modes sit at Q = 0
__global__ void grid_eval_kernel(const TermDesc* __restrict__ terms, int n_terms, const double* __restrict__ mats,
                                 int64_t sum_nq, int D, int nb0, int n_mono, const double* __restrict__ coef,
                                 const int* __restrict__ midx, const int* __restrict__ melec, const double* __restrict__ G0,
                                 const double* __restrict__ g, double* __restrict__ vgrid, double* __restrict__ ggrid,
                                 int with_shift) {
  for (int64_t gq = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; gq < sum_nq;
       gq += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = n_terms - 1;  // last term with off_nq <= gq
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (terms[mid].off_nq <= gq) lo = mid; else hi = mid - 1;
    }
    const TermDesc& T = terms[lo];
    int64_t q = gq - T.off_nq;
    const int NQ = T.NQ;
    double Q[kMaxD];  // coordinates in the reference's mode order
    for (int d = 0; d < kMaxD; ++d) Q[d] = 0.0;
    int64_t r = q;
    for (int d = 0; d < T.D; ++d) {
      Q[T.perm[d]] = mats[T.m_x[d] + (int)(r % T.nq[d])];
      r /= T.nq[d];
    }
    double* V = vgrid + T.off_nq * nb0 * nb0;
    for (int ab = 0; ab < nb0 * nb0; ++ab)
      V[(int64_t)ab * NQ + q] = (with_shift && ab % (nb0 + 1) == 0) ? T.vshift : 0.0;
    for (int m = 0; m < n_mono; ++m) {
      double v = coef[m];
      for (int k = 0; k < 4; ++k) {
        int i = midx[4 * m + k];
        if (i >= 0) v *= Q[i];
      }
      V[(int64_t)(melec[2 * m] + nb0 * melec[2 * m + 1]) * NQ + q] += v;
    }
    if (ggrid) {
      double* Gp = ggrid + (T.off_nq + q) * g_table_stride(D);
      int c = 0;
      for (int i = 0; i < T.D; ++i)  // (i, j) positions of the term's mode order
        for (int j = i; j < T.D; ++j) {
          const int oi = T.perm[i], oj = T.perm[j];
          double s = G0[oi + D * oj];
          for (int k = 0; k < D; ++k) s += g[oi + D * (oj + D * k)] * Q[k];
          Gp[c] = s;
          ++c;
        }
    }
  }
}

__global__ void to_float_kernel(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// out[v*ld_out + k] <-> in[k*ld_in + v] tiled transposes
__global__ void transpose_kernel(const double* __restrict__ in, int64_t ld_in, double* __restrict__ out,
                                 int64_t ld_out, int64_t rows, int64_t cols) {
  // in: rows x cols with row stride ld_in (in[r*ld_in + c]); out[c*ld_out + r]
  __shared__ double tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int64_t r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[i][threadIdx.x] = in[r * ld_in + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int64_t c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[c * ld_out + r] = tile[threadIdx.x][i];
  }
}

template <typename T>
size_t footprint_elems(const HostProblem& P, const TermDesc& Tm, int vt) {
  int ny = (P.keo_type == 10) ? Tm.D : 1;
  return (size_t)(2 * P.nb0 + ny) * (size_t)Tm.NQ * (size_t)vt;
}

template <typename T>
void* dev_alloc(size_t n, int& rc) {
  void* p = nullptr;
  if (n == 0) n = 1;
  if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) { rc = EVR_ENOMEM; return nullptr; }
  return p;
}

}  // namespace

int set_error(evr_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_check(evr_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return EVR_OK;
  (void)cudaGetLastError();
  return set_error(c, e == cudaErrorMemoryAllocation ? EVR_ENOMEM : EVR_EDEVICE,
                   std::string(what) + ": " + cudaGetErrorString(e));
}

#define EVR_CU(call, what)                              \
  do {                                                  \
    int _rc = cuda_check(c, (call), what);              \
    if (_rc != EVR_OK) return _rc;                      \
  } while (0)

template <typename V>
static int upload(evr_ctx* c, V** dst, const std::vector<V>& src) {
  size_t n = std::max<size_t>(src.size(), 1);
  EVR_CU(cudaMalloc((void**)dst, n * sizeof(V)), "cudaMalloc");
  if (!src.empty()) EVR_CU(cudaMemcpy(*dst, src.data(), src.size() * sizeof(V), cudaMemcpyHostToDevice), "cudaMemcpy");
  return EVR_OK;
}

int upload_problem(evr_ctx* c) {
  HostProblem& P = c->hp;
  DeviceProblem& d = c->dp;
  int rc;
  if ((rc = upload(c, &d.terms, P.terms))) return rc;
  if ((rc = upload(c, &d.termsT, P.termsT))) return rc;
  if ((rc = upload(c, &d.mats, P.mat_pool))) return rc;
  if ((rc = upload(c, &d.map, P.map_perm))) return rc;
  if ((rc = upload(c, &d.csr_ptr, P.csr_ptr))) return rc;
  if ((rc = upload(c, &d.csr_src, P.csr_src))) return rc;
  if ((rc = upload(c, &d.csr_w, P.csr_w))) return rc;
  if ((rc = upload_long_rows(c))) return rc;
  if ((rc = upload(c, &d.G0, P.G0))) return rc;
  if ((rc = upload(c, &d.g, P.g))) return rc;
  if ((rc = upload_coeffs32(c))) return rc;
  if ((rc = upload(c, &d.mono_coef, P.mono_coef))) return rc;
  if ((rc = upload(c, &d.mono_idx, P.mono_idx))) return rc;
  if ((rc = upload(c, &d.mono_elec, P.mono_elec))) return rc;
  if ((rc = upload(c, &d.e0diag, P.e0diag))) return rc;
  const int nb0 = P.nb0, D = P.D;
  bool g_nonzero = false;
  for (double v : P.g) g_nonzero |= (v != 0.0);
  const int64_t nv = P.sum_nq * nb0 * nb0;
  EVR_CU(cudaMalloc((void**)&d.vgrid, nv * sizeof(double)), "cudaMalloc vgrid");
  double* gg = nullptr;
  if (P.keo_type == 10 && g_nonzero) {
    const size_t ng = (size_t)P.sum_nq * g_table_stride(D);
    EVR_CU(cudaMalloc((void**)&gg, ng * sizeof(double)), "cudaMalloc ggrid");
    EVR_CU(cudaMemsetAsync(gg, 0, ng * sizeof(double), c->stream), "memset ggrid");  // row padding
  }
  c->dp_ggrid = gg;
  grid_eval_kernel<<<c->num_sms * 8, 256, 0, c->stream>>>(d.terms, (int)P.terms.size(), d.mats, P.sum_nq, D, nb0,
                                                          (int)P.mono_coef.size(), d.mono_coef, d.mono_idx,
                                                          d.mono_elec, d.G0, d.g, d.vgrid, gg, 1);
  EVR_CU(cudaGetLastError(), "grid_eval_kernel");
  // FP32 copies for the mixed-precision contractions
  EVR_CU(cudaMalloc((void**)&d.mats32, P.mat_pool.size() * sizeof(float) + 16), "cudaMalloc mats32");
  EVR_CU(cudaMalloc((void**)&d.vgrid32, nv * sizeof(float)), "cudaMalloc vgrid32");
  to_float_kernel<<<c->num_sms * 4, 256, 0, c->stream>>>(d.mats, d.mats32, (int64_t)P.mat_pool.size());
  to_float_kernel<<<c->num_sms * 8, 256, 0, c->stream>>>(d.vgrid, d.vgrid32, nv);
  if (gg) {
    const int64_t ng = P.sum_nq * g_table_stride(D);
    EVR_CU(cudaMalloc((void**)&c->dp_ggrid32, ng * sizeof(float)), "cudaMalloc ggrid32");
    to_float_kernel<<<c->num_sms * 8, 256, 0, c->stream>>>(gg, c->dp_ggrid32, ng);
  }
  EVR_CU(cudaGetLastError(), "to_float_kernel");
  EVR_CU(cudaStreamSynchronize(c->stream), "grid set-up");
  return EVR_OK;
}

// FP32 copies of G0 and of the linear G model's g_ijk (read per grid point by FP32 H.psi)
int upload_coeffs32(evr_ctx* c) {
  DeviceProblem& d = c->dp;
  const std::vector<double>* src[2] = {&c->hp.G0, &c->hp.g};
  float** dst[2] = {&d.G0_32, &d.g32};
  for (int a = 0; a < 2; ++a) {
    std::vector<float> f(src[a]->begin(), src[a]->end());
    if (*dst[a]) cudaFree(*dst[a]);
    *dst[a] = nullptr;
    EVR_CU(cudaMalloc((void**)dst[a], std::max<size_t>(f.size(), 1) * sizeof(float)), "cudaMalloc");
    if (!f.empty()) EVR_CU(cudaMemcpy(*dst[a], f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy");
  }
  return EVR_OK;
}

// the rows of the weighted reduction with more than kCsrShortRow entries, on the device
int upload_long_rows(evr_ctx* c) {
  const std::vector<int64_t>& ptr = c->hp.csr_ptr;
  std::vector<int64_t> rows;
  for (size_t k = 0; k + 1 < ptr.size(); ++k)
    if (ptr[k + 1] - ptr[k] > kCsrShortRow) rows.push_back((int64_t)k);
  DeviceProblem& d = c->dp;
  if (d.csr_long) cudaFree(d.csr_long);
  d.csr_long = nullptr;
  d.n_long = 0;
  EVR_CU(cudaMalloc((void**)&d.csr_long, std::max<size_t>(rows.size(), 1) * sizeof(int64_t)), "cudaMalloc");
  if (!rows.empty())
    EVR_CU(cudaMemcpy(d.csr_long, rows.data(), rows.size() * sizeof(int64_t), cudaMemcpyHostToDevice), "cudaMemcpy");
  d.n_long = (int64_t)rows.size();
  return EVR_OK;
}

void free_problem(evr_ctx* c) {
  DeviceProblem& d = c->dp;
  void* ptrs[] = {d.terms, d.termsT, d.mats, d.mats32, d.vgrid, d.vgrid32, d.map, d.csr_ptr, d.csr_src, d.csr_w,
                  d.csr_long, d.G0_32, d.g32,
                  d.G0, d.g, d.mono_coef, d.mono_idx, d.mono_elec, d.e0diag, c->dp_ggrid, c->dp_ggrid32,
                  c->dp_mugrid, c->dp_mugrid32, c->dp_jgrid, c->dp_jgrid32};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  d = DeviceProblem();
  c->dp_ggrid = nullptr;
  c->dp_ggrid32 = nullptr;
  c->dp_jgrid = nullptr;
  c->dp_jgrid32 = nullptr;
  c->dp_mugrid = nullptr;
  c->dp_mugrid32 = nullptr;
}

void free_workspace(evr_ctx* c) {
  Workspace& w = c->ws;
  for (ItemSet& s : w.sets) {
    if (s.items) cudaFree(s.items);
    if (s.items_slab) cudaFree(s.items_slab);
    if (s.items_small) cudaFree(s.items_small);
  }
  void* ptrs[] = {w.counter, w.slab, w.ht, w.ht2, w.xin, w.xout, w.f_items, w.f_slab, w.f_small};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  w = Workspace();
  free_stages(c);
  ++c->ws_gen;
}

// bytes the FP32 slab kernel keeps for the tensor-core contractions (their shared block,
// placed 16-byte aligned at the end of the dynamic shared memory)
static size_t tc_reserve_bytes() { return (sizeof(tc::TcSmem) + 15) & ~(size_t)15; }

// Dynamic shared memory of the term kernels: the slab kernel's CTAs (slab_ctas per SM, per
// precision) and the general kernel's two CTAs per SM share the SM's shared memory, each
// CTA also holding its static block and the per-block reservation.  slab_bytes[p] for
// p = EVR_PREC_FP64, EVR_PREC_FP32.
int term_kernel_smem(evr_ctx* c, int* items_bytes, int* slab_bytes, int* small_bytes) {
  int optin = 0, per_sm = 0, reserved = 0;
  EVR_CU(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device), "attr");
  EVR_CU(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device), "attr");
  if (cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, c->device) != cudaSuccess) {
    (void)cudaGetLastError();
    reserved = 1024;
  }
  int st_slab = 0, st_items = 0, v = 0;
  EVR_CU((slab_kernel_static_smem<float, false, false>(&v)), "attr"); st_slab = std::max(st_slab, v);
  EVR_CU((slab_kernel_static_smem<float, true, false>(&v)), "attr"); st_slab = std::max(st_slab, v);
  EVR_CU((slab_kernel_static_smem<float, false, true>(&v)), "attr"); st_slab = std::max(st_slab, v);
  EVR_CU((slab_kernel_static_smem<float, true, true>(&v)), "attr"); st_slab = std::max(st_slab, v);
  EVR_CU((slab_kernel_static_smem<double, false, false>(&v)), "attr"); st_slab = std::max(st_slab, v);
  EVR_CU((slab_kernel_static_smem<double, true, false>(&v)), "attr"); st_slab = std::max(st_slab, v);
  EVR_CU((items_kernel_static_smem<float, false>(&v)), "attr"); st_items = std::max(st_items, v);
  EVR_CU((items_kernel_static_smem<float, true>(&v)), "attr"); st_items = std::max(st_items, v);
  EVR_CU((items_kernel_static_smem<double, false>(&v)), "attr"); st_items = std::max(st_items, v);
  EVR_CU((items_kernel_static_smem<double, true>(&v)), "attr"); st_items = std::max(st_items, v);
  // multiples of 256 bytes below the limits
  slab_bytes[EVR_PREC_FP64] = (std::min(optin - st_slab, per_sm / slab_ctas<double>() - reserved - st_slab)) & ~255;
  slab_bytes[EVR_PREC_FP32] = (std::min(optin - st_slab, per_sm / slab_ctas<float>() - reserved - st_slab)) & ~255;
  *items_bytes = (std::min(optin - st_items, per_sm / kItemsCtas - reserved - st_items)) & ~255;
  if (small_bytes) *small_bytes = (std::min(optin - st_items, per_sm / kSmallCtas - reserved - st_items)) & ~255;
  return EVR_OK;
}

// elements of shared memory the slab kernel needs for a term and a vector tile
static size_t slab_need_elems(const HostProblem& P, const TermDesc& Tm, int vt, bool fp32) {
  const int L = Tm.D - 1;  // the term's own mode count (stacked problems differ)
  const size_t ss = (size_t)(Tm.NQ / Tm.nq[L]) * vt, tsz = ss * Tm.nb[L];
  // type 10: the first derivatives, and d_L psi in FP32 (fused extraction)
  const size_t ny = (P.keo_type == 10) ? (size_t)L + (fp32 ? 1 : 0) : 1;
  return std::max(2 * tsz, tsz + (2 + ny) * ss);
}

// W-in-global mode of the slab kernel: shared memory holds only the slab arrays, the
// global buffer Tg, W and one ping-pong tensor (3 tensors of NQs*nb_L*vt)
static size_t slab_wg_smem_elems(const HostProblem& P, const TermDesc& Tm, int vt, bool fp32) {
  const int L = Tm.D - 1;
  const size_t ss = (size_t)(Tm.NQ / Tm.nq[L]) * vt;
  return (2 + ((P.keo_type == 10) ? (size_t)L + (fp32 ? 1 : 0) : 1)) * ss;
}
static size_t slab_wg_global_elems(const TermDesc& Tm, int vt) {
  const int L = Tm.D - 1;
  return 3 * (size_t)(Tm.NQ / Tm.nq[L]) * vt * Tm.nb[L];
}
// grid-staged mode (FP32 type 10): the W-in-global tensors and the staged term grid (psi
// and d_L psi on all NQ points)
static size_t slab_staged_global_elems(const TermDesc& Tm, int vt) {
  return slab_wg_global_elems(Tm, vt) + 2 * (size_t)Tm.NQ * vt;
}

// Work decomposition for a block of nvec vectors.  Terms whose slab pipeline fits the
// shared memory of one CTA (one electronic state) go to the slab kernel, with the widest
// vector tile that fits; the others go to the general kernel, in shared memory when
// their buffers fit, else in the CTA's global slab.  Items are ordered by decreasing
// cost.  Buffers are sized once for kMaxBlock vectors in FP64.
int ensure_workspace(evr_ctx* c, int nvec, int prec) {
  Workspace& w = c->ws;
  if (nvec < 1 || nvec > kMaxBlock) return set_error(c, EVR_EINVAL, "block of more than 64 vectors");
  const HostProblem& P = c->hp;
  int rc = EVR_OK;
  if (!w.counter) {
    // general kernel: kItemsCtas CTAs per SM; slab kernel: slab_ctas<T>() CTAs per SM
    if ((rc = term_kernel_smem(c, &w.smem_bytes, w.smem_slab_bytes, &w.smem_small_bytes))) return rc;
    w.grid = c->num_sms * kItemsCtas;
    w.grid_small = c->num_sms * kSmallCtas;
    w.grid_slab[EVR_PREC_FP64] = c->num_sms * slab_ctas<double>();
    w.grid_slab[EVR_PREC_FP32] = c->num_sms * slab_ctas<float>();
    size_t slab = 0;  // general kernel: FP64 buffers of the terms that run from global memory
    for (const TermDesc& Tm : P.terms) {
      size_t fp1 = footprint_elems<double>(P, Tm, 1) * sizeof(double);
      slab = std::max(slab, fp1);
    }
    w.slab_per_cta_bytes = slab;
    // the slab kernel keeps its partially transformed tensor (at most half of its shared
    // memory) in global memory; terms in the W-in-global mode (FP64 terms whose slab
    // pipeline does not fit shared memory) need three such tensors there
    const int s64 = w.smem_slab_bytes[EVR_PREC_FP64], s32 = w.smem_slab_bytes[EVR_PREC_FP32];
    size_t sb64 = (size_t)(s64 / 2 + 256), sb32 = (size_t)(s32 / 2 + 256);
    if (P.nb0 == 1)
      for (const TermDesc& Tm : P.terms) {
        if (Tm.weight == 0.0) continue;
        const size_t mats = (size_t)((Tm.msz + 3) & ~3) * sizeof(double);
        if (slab_need_elems(P, Tm, 1, false) * sizeof(double) + mats <= (size_t)s64) continue;
        if (slab_wg_smem_elems(P, Tm, 1, false) * sizeof(double) + mats > (size_t)s64) continue;
        sb64 = std::max(sb64, slab_wg_global_elems(Tm, 1) * sizeof(double));
      }
    // FP32 terms run in the W-in-global or grid-staged mode when it allows a wider vector
    // tile (below): room for tiles of 4 vectors, at most 8 MB per CTA
    if (P.nb0 == 1)
      for (const TermDesc& Tm : P.terms)
        if (Tm.weight != 0.0)
          sb32 = std::max(sb32, std::min<size_t>(slab_staged_global_elems(Tm, 4) * sizeof(float), 8u << 20));
    w.slab_slab_bytes[EVR_PREC_FP64] = (sb64 + 255) & ~(size_t)255;
    w.slab_slab_bytes[EVR_PREC_FP32] = (sb32 + 255) & ~(size_t)255;
    const size_t total = std::max({slab * w.grid, w.slab_slab_bytes[EVR_PREC_FP64] * w.grid_slab[EVR_PREC_FP64],
                                   w.slab_slab_bytes[EVR_PREC_FP32] * w.grid_slab[EVR_PREC_FP32]});
    w.counter = (int*)dev_alloc<int>(4, rc);  // item counters of both kernels, item-bounds flag
    if (rc) return set_error(c, rc, "workspace allocation (counter)");
    EVR_CU(cudaMemset(w.counter, 0, 4 * sizeof(int)), "memset counter");
    w.slab = dev_alloc<unsigned char>(total, rc);
    if (rc) return set_error(c, rc, "workspace allocation (slab)");
    w.cap = kMaxBlock;
    w.ht = dev_alloc<double>((size_t)P.sum_nb * P.nb0 * w.cap, rc);
    if (rc) return set_error(c, rc, "workspace allocation (term-basis output)");
    const size_t xe = (size_t)P.Np * P.nb0 * w.cap;
    w.xin = (double*)dev_alloc<double>(xe, rc);
    if (rc) return set_error(c, rc, "workspace allocation (xin)");
    w.xout = (double*)dev_alloc<double>(xe, rc);
    if (rc) return set_error(c, rc, "workspace allocation (xout)");
    EVR_CU((set_term_kernel_smem<float, false>(w.smem_bytes, s32)), "attr");
    EVR_CU((set_term_kernel_smem<double, false>(w.smem_bytes, s64)), "attr");
    EVR_CU((set_term_kernel_smem<float, true>(w.smem_bytes, s32)), "attr");
    EVR_CU((set_term_kernel_smem<double, true>(w.smem_bytes, s64)), "attr");
  }
  for (const ItemSet& s : w.sets)
    if (s.nvec == nvec && s.prec == prec) return EVR_OK;
  const size_t esz = prec == EVR_PREC_FP32 ? sizeof(float) : sizeof(double);
  const bool f32 = prec == EVR_PREC_FP32;
  // a Jacobian table runs every term in the general kernel (the slab kernel folds the
  // streamed position's derivatives into its basis transforms, which a point factor between
  // derivative and transform would break)
  const bool slab_ok = P.nb0 == 1 && c->use_slab && !c->dp_jgrid;
  // shared memory of a slab-kernel item: the FP32 tensor-core contractions keep their
  // operand tiles at the end of the block
  const int pi = f32 ? EVR_PREC_FP32 : EVR_PREC_FP64;
  const size_t slab_smem = (size_t)w.smem_slab_bytes[pi] - (f32 && c->use_tc ? tc_reserve_bytes() : 0);
  const size_t slab_glob = w.slab_slab_bytes[pi];
  std::vector<WorkItem> items, sitems, titems;
  for (int t = 0; t < (int)P.terms.size(); ++t) {
    const TermDesc& Tm = P.terms[t];
    if (Tm.weight == 0.0) continue;
    const size_t mats = (size_t)((Tm.msz + 3) & ~3) * esz;  // staged 1-D matrices
    if (mats > (size_t)w.smem_bytes) return set_error(c, EVR_EINVAL, "1-D matrices exceed shared memory");
    const bool small = !c->slab_all && (int64_t)Tm.NQ * std::min(nvec, c->vt_cap_slab) < c->slab_min_points;
    if (small) {
      // the general kernel as small CTAs when the term's buffers and matrices fit one
      const size_t fp1 = footprint_elems<double>(P, Tm, 1) * esz;
      if (fp1 + mats <= (size_t)w.smem_small_bytes) {
        int vt = 1;
        while (vt * 2 <= nvec && vt * 2 <= c->vt_cap_items && fp1 * (size_t)(vt * 2) + mats <= (size_t)w.smem_small_bytes)
          vt *= 2;
        for (int v0 = 0; v0 < nvec; v0 += vt) titems.push_back(WorkItem{t, v0, std::min(vt, nvec - v0), 1});
        continue;
      }
    }
    // W-in-global tile (shared memory holds only the slab arrays)
    auto wg_fits = [&](int v) {
      return slab_wg_smem_elems(P, Tm, v, f32) * esz + mats <= slab_smem &&
             slab_wg_global_elems(Tm, v) * esz <= slab_glob;
    };
    if (f32 && slab_ok && !small && wg_fits(1)) {
      // FP32 is bound by the instructions per grid point, not by the L2 traffic of W: the
      // W-in-global mode wins where it allows at least twice the tile of the shared-memory mode
      int v3 = 1, v1 = 0;
      while (v3 * 2 <= nvec && v3 * 2 <= c->vt_cap_slab && wg_fits(v3 * 2)) v3 *= 2;
      if (slab_need_elems(P, Tm, 1, f32) * esz + mats <= slab_smem) {
        v1 = 1;
        while (v1 * 2 <= nvec && v1 * 2 <= c->vt_cap_slab &&
               slab_need_elems(P, Tm, v1 * 2, f32) * esz + mats <= slab_smem)
          v1 *= 2;
      }
      // type 10: the grid-staged variant (the streamed position's transforms as two
      // contractions instead of a sweep over Tg and W per grid slab) where its buffer allows
      int v4 = 0;
      if (P.keo_type == 10) {
        auto st_fits = [&](int v) {
          return slab_wg_smem_elems(P, Tm, v, f32) * esz + mats <= slab_smem &&
                 slab_staged_global_elems(Tm, v) * esz <= slab_glob;
        };
        if (st_fits(1)) {
          v4 = 1;
          while (v4 * 2 <= nvec && v4 * 2 <= c->vt_cap_slab && st_fits(v4 * 2)) v4 *= 2;
        }
      }
      if (v4 >= 2 * v1 && v4 * 2 >= v3) {
        for (int v0 = 0; v0 < nvec; v0 += v4) sitems.push_back(WorkItem{t, v0, std::min(v4, nvec - v0), 4});
        continue;
      }
      if (v3 >= 2 * v1) {
        for (int v0 = 0; v0 < nvec; v0 += v3) sitems.push_back(WorkItem{t, v0, std::min(v3, nvec - v0), 3});
        continue;
      }
    }
    if (slab_ok && !small && slab_need_elems(P, Tm, 1, f32) * esz + mats <= slab_smem) {
      // FP32: the partially transformed tensor also in shared memory when a tile of
      // min(4, nvec) vectors fits (its per-slab re-reads then stay on the SM); FP64 keeps it
      // in the L2-resident global buffer, the FP64 pipe being the bound there
      const int L = Tm.D - 1;
      auto tg_elems = [&](int v) { return (size_t)(Tm.NQ / Tm.nq[L]) * v * Tm.nb[L]; };
      auto fits = [&](int v, bool tg) {
        return (slab_need_elems(P, Tm, v, f32) + (tg ? tg_elems(v) : 0)) * esz + mats <= slab_smem;
      };
      const bool tg = prec == EVR_PREC_FP32 && fits(std::min(4, nvec), true);
      int vt = 1;
      while (vt * 2 <= nvec && vt * 2 <= c->vt_cap_slab && fits(vt * 2, tg)) vt *= 2;
      for (int v0 = 0; v0 < nvec; v0 += vt) sitems.push_back(WorkItem{t, v0, std::min(vt, nvec - v0), tg ? 2 : 1});
      continue;
    }
    // W in global memory: the slab pipeline with only the slab arrays in shared memory
    if (slab_ok && !small && wg_fits(1)) {
      int vt = 1;
      while (vt * 2 <= nvec && vt * 2 <= c->vt_cap_slab && wg_fits(vt * 2)) vt *= 2;
      for (int v0 = 0; v0 < nvec; v0 += vt) sitems.push_back(WorkItem{t, v0, std::min(vt, nvec - v0), 3});
      continue;
    }
    int vt = 1;
    const size_t fp1 = footprint_elems<double>(P, Tm, 1) * esz;
    const bool in_smem = fp1 + mats <= (size_t)w.smem_bytes;
    if (in_smem)
      while (vt * 2 <= nvec && vt * 2 <= c->vt_cap_items && fp1 * (size_t)(vt * 2) + mats <= (size_t)w.smem_bytes)
        vt *= 2;
    for (int v0 = 0; v0 < nvec; v0 += vt) items.push_back(WorkItem{t, v0, std::min(vt, nvec - v0), in_smem ? 1 : 0});
  }
  auto by_cost = [&](const WorkItem& a, const WorkItem& b) {
    return (int64_t)P.terms[a.term].NQ * a.vt > (int64_t)P.terms[b.term].NQ * b.vt;
  };
  std::stable_sort(items.begin(), items.end(), by_cost);
  std::stable_sort(sitems.begin(), sitems.end(), by_cost);
  std::stable_sort(titems.begin(), titems.end(), by_cost);
  ItemSet s;
  s.nvec = nvec;
  s.prec = prec;
  s.n_items = (int)items.size();
  s.n_slab = (int)sitems.size();
  s.n_small = (int)titems.size();
  s.items = (WorkItem*)dev_alloc<WorkItem>(items.size(), rc);
  if (rc) return set_error(c, rc, "workspace allocation (items)");
  s.items_slab = (WorkItem*)dev_alloc<WorkItem>(sitems.size(), rc);
  if (rc) {
    cudaFree(s.items);
    return set_error(c, rc, "workspace allocation (items)");
  }
  s.items_small = (WorkItem*)dev_alloc<WorkItem>(titems.size(), rc);
  if (rc) {
    cudaFree(s.items);
    cudaFree(s.items_slab);
    return set_error(c, rc, "workspace allocation (items)");
  }
  if (!items.empty())
    EVR_CU(cudaMemcpy(s.items, items.data(), items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice), "items");
  if (!sitems.empty())
    EVR_CU(cudaMemcpy(s.items_slab, sitems.data(), sitems.size() * sizeof(WorkItem), cudaMemcpyHostToDevice),
           "items");
  if (!titems.empty())
    EVR_CU(cudaMemcpy(s.items_small, titems.data(), titems.size() * sizeof(WorkItem), cudaMemcpyHostToDevice),
           "items");
  s.h_items = items;
  s.h_slab = sitems;
  s.h_small = titems;
  w.sets.push_back(s);
  return EVR_OK;
}

template <typename T>
static int launch_items(evr_ctx* c, const ItemSet& set, const TermDesc* terms, int vtrans, T* ht, const double* x,
                        int64_t ldx, int nvec, cudaStream_t s, const OpExtras& ex) {
  const HostProblem& P = c->hp;
  Workspace& w = c->ws;
  ItemParams<T> p;
  const bool f32 = sizeof(T) == 4;
  p.terms = terms;
  p.mats = f32 ? (const T*)c->dp.mats32 : (const T*)c->dp.mats;
  p.vgrid = f32 ? (const T*)c->dp.vgrid32 : (const T*)c->dp.vgrid;
  p.ggrid = f32 ? (const T*)c->dp_ggrid32 : (const T*)c->dp_ggrid;
  p.G0 = c->dp.G0;
  p.map = c->dp.map;
  p.counter = w.counter;
  p.slab = (T*)w.slab;
  p.x = x;
  p.ldx = ldx;
  p.ht = ht;
  p.ldh = nvec;
  p.Np = P.Np;
  p.D = P.D;
  p.nb0 = P.nb0;
  p.keo_type = P.keo_type;
  p.vtrans = vtrans;
  p.implicit_nvec = 0;
  p.has_offdiag = 0;
  if (P.keo_type == 1) {
    if (c->batch) {
      p.has_offdiag = 1;  // stacked problems: the kernels skip the zero F2 pairs term by term
    } else {
      for (int i = 0; i < P.D; ++i)
        for (int j = i + 1; j < P.D; ++j) p.has_offdiag |= (P.G0[i + (size_t)P.D * j] != 0.0);
    }
  }
  set_plain(p);
  p.jgrid = f32 ? (const T*)c->dp_jgrid32 : (const T*)c->dp_jgrid;
  p.keo_on = ex.keo;
  p.gco = c->dp.g;
  p.G0t = f32 ? (const T*)c->dp.G0_32 : (const T*)c->dp.G0;
  p.gcot = f32 ? (const T*)c->dp.g32 : (const T*)c->dp.g;
  p.gfly = c->gfly ? 1 : 0;
  p.err = w.counter + 2;
  if (ex.mw != 0.0 || ex.vw != 1.0 || ex.mu_dev) {
    if (!c->dp_mugrid) return set_error(c, EVR_EINVAL, "field term without a dipole (evr_set_dipole)");
    p.mugrid = f32 ? (const T*)c->dp_mugrid32 : (const T*)c->dp_mugrid;
    p.vw = (T)ex.vw;
    p.mw = (T)ex.mw;
    p.mu_dev = ex.mu_dev;
  }
  EVR_CU(cudaMemsetAsync(w.counter, 0, 2 * sizeof(int), s), "memset counter");
  if (set.n_slab > 0) {
    ItemParams<T> ps = p;
    ps.items = set.items_slab;
    ps.n_items = set.n_slab;
    ps.counter = w.counter + 1;
    const int pi = sizeof(T) == 4 ? EVR_PREC_FP32 : EVR_PREC_FP64;
    const int sgrid = w.grid_slab[pi], ssmem = w.smem_slab_bytes[pi];
    ps.slab_per_cta = (int64_t)(w.slab_slab_bytes[pi] / sizeof(T));
    ps.smem_elems = (int64_t)(ssmem / sizeof(T));
    if (f32 && c->use_tc) {
      ps.use_tc = 1;
      ps.tc_off = (int)(((size_t)ssmem - tc_reserve_bytes()) & ~(size_t)15);
      ps.tc_min_km = c->tc_min_km;
      ps.smem_elems = (int64_t)(ps.tc_off / sizeof(T));
    }
    cudaError_t le;
    if constexpr (sizeof(T) == 4) {
      if (ps.use_tc)
        le = p.gfly ? launch_slab_kernel<T, true, true>(sgrid, ssmem, s, ps)
                    : launch_slab_kernel<T, false, true>(sgrid, ssmem, s, ps);
      else
        le = p.gfly ? launch_slab_kernel<T, true, false>(sgrid, ssmem, s, ps)
                    : launch_slab_kernel<T, false, false>(sgrid, ssmem, s, ps);
    } else {
      le = p.gfly ? launch_slab_kernel<T, true, false>(sgrid, ssmem, s, ps)
                  : launch_slab_kernel<T, false, false>(sgrid, ssmem, s, ps);
    }
    EVR_CU(le, "hpsi_slab_kernel launch");
  }
  if (set.n_items > 0) {
    ItemParams<T> pi = p;
    pi.items = set.items;
    pi.n_items = set.n_items;
    pi.slab_per_cta = (int64_t)(w.slab_per_cta_bytes / sizeof(T));
    pi.smem_elems = (int64_t)(w.smem_bytes / sizeof(T));
    EVR_CU((p.gfly ? launch_items_kernel<T, true>(w.grid, w.smem_bytes, s, pi)
                   : launch_items_kernel<T, false>(w.grid, w.smem_bytes, s, pi)),
           "hpsi_items_kernel launch");
  }
  if (set.n_small > 0) {
    // small terms: the general kernel as kSmallCtas CTAs of kSmallThreads per SM, every
    // item in shared memory (no global buffer)
    ItemParams<T> pt = p;
    pt.items = set.items_small;
    pt.n_items = set.n_small;
    pt.counter = w.counter + 3;
    pt.slab = nullptr;
    pt.slab_per_cta = 0;
    pt.smem_elems = (int64_t)(w.smem_small_bytes / sizeof(T));
    EVR_CU(cudaMemsetAsync(w.counter + 3, 0, sizeof(int), s), "memset counter");
    EVR_CU((p.gfly ? launch_items_kernel<T, true>(w.grid_small, w.smem_small_bytes, s, pt, kSmallThreads)
                   : launch_items_kernel<T, false>(w.grid_small, w.smem_small_bytes, s, pt, kSmallThreads)),
           "hpsi_items_kernel launch (small CTAs)");
  }
  return EVR_OK;
}

template <typename T>
static int run_items(evr_ctx* c, const ItemSet& set, const double* x, int64_t ldx, double* y, int64_t ldy, int nvec,
                     cudaStream_t s, int op, const OpExtras& ex) {
  const HostProblem& P = c->hp;
  Workspace& w = c->ws;
  if (op == OP_HSYM && !w.ht2) {
    int rc = EVR_OK;
    w.ht2 = dev_alloc<double>((size_t)P.sum_nb * P.nb0 * w.cap, rc);
    if (rc) return set_error(c, rc, "workspace allocation (second term-basis output)");
  }
  int rc;
  if (!c->capturing) EVR_CU(cudaEventRecord(c->ev[0], s), "event");
  if (op == OP_H || op == OP_HSYM)
    if ((rc = launch_items<T>(c, set, c->dp.terms, 0, (T*)w.ht, x, ldx, nvec, s, ex))) return rc;
  if (op == OP_HT || op == OP_HSYM)
    if ((rc = launch_items<T>(c, set, c->dp.termsT, 1, (T*)(op == OP_HT ? w.ht : w.ht2), x, ldx, nvec, s, ex)))
      return rc;
  if (!c->capturing) EVR_CU(cudaEventRecord(c->ev[1], s), "event");
  EVR_CU(launch_csr_reduce<T>(c, (const T*)w.ht, op == OP_HSYM ? (const T*)w.ht2 : nullptr, nvec,
                               op == OP_HSYM ? 0.5 : 1.0, y, ldy, nvec, s),
         "csr_reduce_kernel launch");
  if (!c->capturing) EVR_CU(cudaEventRecord(c->ev[2], s), "event");
  const int per_op = (set.n_slab > 0 ? 1 : 0) + (set.n_items > 0 ? 1 : 0) + (set.n_small > 0 ? 1 : 0);
  c->last_kernels = per_op * (op == OP_HSYM ? 2 : 1) + 1;
  c->last_items = (int64_t)(set.n_items + set.n_slab + set.n_small) * (op == OP_HSYM ? 2 : 1);
  return EVR_OK;
}

int hpsi_interleaved(evr_ctx* c, const double* x, int64_t ldx, double* y, int64_t ldy, int nvec, int prec,
                     cudaStream_t s, int op, const OpExtras* ex) {
  const OpExtras& e = ex ? *ex : c->field;
  int rc = ensure_workspace(c, nvec, prec);
  if (rc) return rc;
  if (stages_apply(c)) return hpsi_stages(c, x, ldx, y, ldy, nvec, prec, s, op, e);
  const ItemSet* set = nullptr;
  for (const ItemSet& it : c->ws.sets)
    if (it.nvec == nvec && it.prec == prec) set = &it;
  if (!set) return set_error(c, EVR_EINVAL, "no work decomposition");
  ItemSet cp;
  cp.nvec = set->nvec;
  cp.prec = set->prec;
  cp.items = set->items;
  cp.n_items = set->n_items;
  cp.items_slab = set->items_slab;
  cp.n_slab = set->n_slab;
  cp.items_small = set->items_small;
  cp.n_small = set->n_small;
  if (!c->term_active.empty()) {
    // batches: only the terms of the active problems (host-synchronous, not for capture)
    if (c->capturing) return set_error(c, EVR_EINVAL, "filtered H.psi inside a stream capture");
    Workspace& w = c->ws;
    const size_t need = std::max({set->h_items.size(), set->h_slab.size(), set->h_small.size()});
    if (w.f_cap < need) {
      if (w.f_items) cudaFree(w.f_items);
      if (w.f_slab) cudaFree(w.f_slab);
      if (w.f_small) cudaFree(w.f_small);
      w.f_items = w.f_slab = w.f_small = nullptr;
      w.f_cap = 0;
      EVR_CU(cudaMalloc((void**)&w.f_items, need * sizeof(WorkItem)), "cudaMalloc items");
      EVR_CU(cudaMalloc((void**)&w.f_slab, need * sizeof(WorkItem)), "cudaMalloc items");
      EVR_CU(cudaMalloc((void**)&w.f_small, need * sizeof(WorkItem)), "cudaMalloc items");
      w.f_cap = need;
    }
    std::vector<WorkItem> fi, fs, ft;
    for (const WorkItem& it : set->h_items)
      if (c->term_active[it.term]) fi.push_back(it);
    for (const WorkItem& it : set->h_slab)
      if (c->term_active[it.term]) fs.push_back(it);
    for (const WorkItem& it : set->h_small)
      if (c->term_active[it.term]) ft.push_back(it);
    EVR_CU(cudaStreamSynchronize(s), "sync");  // the previous launch may still read the lists
    if (!fi.empty()) EVR_CU(cudaMemcpy(w.f_items, fi.data(), fi.size() * sizeof(WorkItem), cudaMemcpyHostToDevice), "items");
    if (!fs.empty()) EVR_CU(cudaMemcpy(w.f_slab, fs.data(), fs.size() * sizeof(WorkItem), cudaMemcpyHostToDevice), "items");
    if (!ft.empty()) EVR_CU(cudaMemcpy(w.f_small, ft.data(), ft.size() * sizeof(WorkItem), cudaMemcpyHostToDevice), "items");
    cp.items = w.f_items;
    cp.n_items = (int)fi.size();
    cp.items_slab = w.f_slab;
    cp.n_slab = (int)fs.size();
    cp.items_small = w.f_small;
    cp.n_small = (int)ft.size();
  }
  if (prec == EVR_PREC_FP32) return run_items<float>(c, cp, x, ldx, y, ldy, nvec, s, op, e);
  return run_items<double>(c, cp, x, ldx, y, ldy, nvec, s, op, e);
}

int hpsi_blocks(evr_ctx* c, const double* x, int64_t ldx, double* y, int64_t ldy, int nvec, int prec, cudaStream_t s,
                int op, const OpExtras* ex) {
  int64_t k = 0, items = 0;
  for (int v0 = 0; v0 < nvec; v0 += kMaxBlock) {
    const int nb = std::min(kMaxBlock, nvec - v0);
    int rc = hpsi_interleaved(c, x + v0, ldx, y + v0, ldy, nb, prec, s, op, ex);
    if (rc) return rc;
    k += c->last_kernels;
    items += c->last_items;
  }
  c->last_kernels = k;
  c->last_items = items;
  return EVR_OK;
}

int transpose_to_interleaved(const double* in, int64_t ld_in, double* out, int64_t ld_out, int64_t N, int nvec,
                             cudaStream_t s) {
  // in: column-major N x nvec (in[v*ld_in + k]) == row-major nvec x N
  dim3 blk(32, 8), grd((unsigned)((N + 31) / 32), (unsigned)((nvec + 31) / 32));
  transpose_kernel<<<grd, blk, 0, s>>>(in, ld_in, out, ld_out, nvec, N);
  return cudaGetLastError() == cudaSuccess ? EVR_OK : EVR_EDEVICE;
}

int transpose_from_interleaved(const double* in, int64_t ld_in, double* out, int64_t ld_out, int64_t N, int nvec,
                               cudaStream_t s) {
  dim3 blk(32, 8), grd((unsigned)((nvec + 31) / 32), (unsigned)((N + 31) / 32));
  transpose_kernel<<<grd, blk, 0, s>>>(in, ld_in, out, ld_out, N, nvec);
  return cudaGetLastError() == cudaSuccess ? EVR_OK : EVR_EDEVICE;
}

// drops the cached work decompositions (they depend on the tile caps)
void clear_item_sets(evr_ctx* c) {
  for (ItemSet& st : c->ws.sets) {
    if (st.items) cudaFree(st.items);
    if (st.items_slab) cudaFree(st.items_slab);
    if (st.items_small) cudaFree(st.items_small);
  }
  c->ws.sets.clear();
  ++c->ws_gen;
}

int check_item_bounds(evr_ctx* c) {
  if (!c->ws.counter) return EVR_OK;
  int flag = 0;
  EVR_CU(cudaMemcpyAsync(&flag, c->ws.counter + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "flag");
  EVR_CU(cudaStreamSynchronize(c->stream), "flag");
  if (!flag) return EVR_OK;
  EVR_CU(cudaMemsetAsync(c->ws.counter + 2, 0, sizeof(int), c->stream), "flag");
  if (flag == 2)
    return set_error(c, EVR_ETIMEDOUT, "a tensor-core contraction's bounded wait ran out (result invalid)");
  return set_error(c, EVR_EDEVICE, "a work item exceeded its buffers and was skipped (internal sizing error)");
}

int reduce_terms(evr_ctx* c, int prec, const void* ht, const void* ht2, int nvec, double scale, double* y,
                 int64_t ldy, cudaStream_t s) {
  const cudaError_t e = prec == EVR_PREC_FP32
                            ? launch_csr_reduce<float>(c, (const float*)ht, (const float*)ht2, nvec, scale, y, ldy, nvec, s)
                            : launch_csr_reduce<double>(c, (const double*)ht, (const double*)ht2, nvec, scale, y, ldy,
                                                        nvec, s);
  return cuda_check(c, e, "csr_reduce_kernel launch");
}

namespace {
// largest row-sum norm sum_b |m_ab(q)| over the grid points (non-negative doubles order
// like their bit patterns, so the maximum is an integer atomicMax)
__global__ void rownorm_max_kernel(const double* __restrict__ m, int64_t n, int nb0, unsigned long long* out) {
  double best = 0.0;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    for (int a = 0; a < nb0; ++a) {
      double r = 0.0;
      for (int b = 0; b < nb0; ++b) r += fabs(m[(int64_t)(a + nb0 * b) * n + q]);
      best = fmax(best, r);
    }
  atomicMax(out, (unsigned long long)__double_as_longlong(best));
}
}  // namespace

int eval_grid_monomials(evr_ctx* c, int n_mono, const double* coef, const int* idx, const int* elec, double* out,
                        double* maxnorm) {
  const HostProblem& P = c->hp;
  grid_eval_kernel<<<c->num_sms * 8, 256, 0, c->stream>>>(c->dp.terms, (int)P.terms.size(), c->dp.mats, P.sum_nq,
                                                          P.D, P.nb0, n_mono, coef, idx, elec, c->dp.G0, c->dp.g,
                                                          out, nullptr, 0);
  EVR_CU(cudaGetLastError(), "grid_eval_kernel");
  if (maxnorm) {
    unsigned long long* d = nullptr;
    EVR_CU(cudaMalloc((void**)&d, sizeof(unsigned long long)), "cudaMalloc");
    cudaMemsetAsync(d, 0, sizeof(unsigned long long), c->stream);
    // the V table of term t starts at off_nq*nb0^2, with (a,b) blocks of NQ_t points; the
    // norm scan runs per term
    for (const TermDesc& Tm : P.terms)
      rownorm_max_kernel<<<std::max(1, std::min(c->num_sms * 4, (Tm.NQ + 255) / 256)), 256, 0, c->stream>>>(
          out + Tm.off_nq * P.nb0 * P.nb0, Tm.NQ, P.nb0, d);
    unsigned long long h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    EVR_CU(e, "dipole norm");
    double v;
    memcpy(&v, &h, sizeof(v));
    *maxnorm = v;
  }
  return EVR_OK;
}

// H.psi (FP64, the reference's operator H) on interleaved device blocks with all scratch
// memory supplied by the caller: [item counter (256 B)][term-basis output][per-CTA
// buffers].  Allocates nothing; every term runs one vector per item from the global
// buffers.  Returns EVR_EINVAL when the scratch is too small, and EVR_EDEVICE when the
// kernel skipped an item that would have exceeded its buffers (the flag is read back
// after the launches, so the call returns once the H.psi has completed).
int hpsi_scratch(evr_ctx* c, const double* x, int64_t ldx, double* y, int64_t ldy, int nvec, unsigned char* scratch,
                 size_t scratch_bytes, cudaStream_t s) {
  const HostProblem& P = c->hp;
  // the general kernel's shared memory of the regular path, so that two CTAs are resident
  // per SM and every CTA of the grid gets its per-CTA buffer in the first wave
  int smem_items = 0, smem_slab[2] = {0, 0};
  int rc0 = term_kernel_smem(c, &smem_items, smem_slab, nullptr);
  if (rc0) return rc0;
  // the same attribute values as ensure_workspace sets, so neither path lowers the other's
  EVR_CU((set_term_kernel_smem<double, false>(smem_items, smem_slab[EVR_PREC_FP64])), "attr");
  int per_sm = 0;
  EVR_CU((occupancy_items_kernel<double, false>(&per_sm, smem_items)), "occupancy");
  const int grid = c->num_sms * std::max(1, std::min(per_sm, kItemsCtas));
  size_t slab = 0, msz = 0;
  for (const TermDesc& Tm : P.terms) {
    slab = std::max(slab, footprint_elems<double>(P, Tm, 1));
    msz = std::max(msz, (size_t)((Tm.msz + 3) & ~3));
  }
  const size_t ht_bytes = ((size_t)P.sum_nb * P.nb0 * nvec * sizeof(double) + 255) & ~(size_t)255;
  const size_t slab_bytes = slab * sizeof(double);
  const size_t need = 256 + ht_bytes + slab_bytes * grid;
  if (need > scratch_bytes)
    return set_error(c, EVR_EINVAL, "evr_hpsi_noalloc: problem needs " + std::to_string(need) +
                                        " bytes of scratch, the static buffer holds " + std::to_string(scratch_bytes));
  const size_t smem = msz * sizeof(double);
  if (smem > (size_t)smem_items) return set_error(c, EVR_EINVAL, "evr_hpsi_noalloc: 1-D matrices too large");
  if (c->gfly || c->batch) return set_error(c, EVR_EINVAL, "evr_hpsi_noalloc: not for batched contexts");
  int* counter = reinterpret_cast<int*>(scratch);
  double* ht = reinterpret_cast<double*>(scratch + 256);
  double* slabp = reinterpret_cast<double*>(scratch + 256 + ht_bytes);
  ItemParams<double> p;
  p.terms = c->dp.terms;
  p.mats = c->dp.mats;
  p.vgrid = c->dp.vgrid;
  p.ggrid = c->dp_ggrid;
  p.G0 = c->dp.G0;
  p.map = c->dp.map;
  p.items = nullptr;
  p.n_items = (int)P.terms.size() * nvec;
  p.counter = counter;
  p.slab = slabp;
  p.slab_per_cta = (int64_t)slab;
  p.smem_elems = (int64_t)(smem_items / sizeof(double));
  p.err = counter + 2;
  p.x = x;
  p.ldx = ldx;
  p.ht = ht;
  p.ldh = nvec;
  p.Np = P.Np;
  p.D = P.D;
  p.nb0 = P.nb0;
  p.keo_type = P.keo_type;
  p.vtrans = 0;
  set_plain(p);
  p.G0t = c->dp.G0;  // constant G (no G table); the no-alloc path has no G model
  p.jgrid = c->dp_jgrid;
  p.implicit_nvec = nvec;
  p.has_offdiag = 0;
  if (P.keo_type == 1)
    for (int i = 0; i < P.D; ++i)
      for (int j = i + 1; j < P.D; ++j) p.has_offdiag |= (P.G0[i + (size_t)P.D * j] != 0.0);
  EVR_CU(cudaMemsetAsync(counter, 0, 4 * sizeof(int), s), "memset counter");  // the buffer keeps old contents
  EVR_CU((launch_items_kernel<double, false>(grid, smem_items, s, p)), "hpsi_items_kernel launch");
  EVR_CU(launch_csr_reduce<double>(c, ht, nullptr, nvec, 1.0, y, ldy, nvec, s), "csr_reduce_kernel launch");
  // the kernel's buffer-check flag: a plain copy into a host int (no allocation)
  int flag = 0;
  EVR_CU(cudaMemcpyAsync(&flag, counter + 2, sizeof(int), cudaMemcpyDeviceToHost, s), "flag");
  EVR_CU(cudaStreamSynchronize(s), "flag");
  if (flag) return set_error(c, EVR_EDEVICE, "evr_hpsi_noalloc: a work item exceeded its buffers and was skipped");
  return EVR_OK;
}

}  // namespace evr

namespace {
__global__ void autotune_fill(double* x, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = 1.0 / (1.0 + (double)((i * 2654435761u) % 1000));
}
}  // namespace

// Autotuner of the work decomposition: the widest vector tile an item of the slab kernel
// and of the general kernel may take (2..32), and the size (grid points x tile) below which
// a term runs in the general kernel's smaller CTAs.  Each candidate is timed with the
// events around the term kernels (second of two H.psi calls on a fixed block), one
// parameter at a time: slab cap, general cap, threshold.
extern "C" int evr_autotune(evr_ctx* c, int nvec, int prec, int* caps, double* best_ms) {
  using namespace evr;
  if (!c) return EVR_EINVAL;
  if (c->host_only) return set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  if (nvec < 1 || nvec > kMaxBlock) return set_error(c, EVR_EINVAL, "evr_autotune: 1 <= nvec <= 64");
  if (prec != EVR_PREC_FP64 && prec != EVR_PREC_FP32) return set_error(c, EVR_EINVAL, "unknown precision");
  EVR_CU(cudaSetDevice(c->device), "cudaSetDevice");
  const int64_t N = c->hp.Np * c->hp.nb0;
  double* x = nullptr;
  double* y = nullptr;
  EVR_CU(cudaMalloc((void**)&x, sizeof(double) * N * nvec), "cudaMalloc");
  if (cudaMalloc((void**)&y, sizeof(double) * N * nvec) != cudaSuccess) {
    cudaFree(x);
    (void)cudaGetLastError();
    return set_error(c, EVR_ENOMEM, "evr_autotune: allocation");
  }
  autotune_fill<<<c->num_sms * 4, 256, 0, c->stream>>>(x, N * nvec);
  auto time_it = [&](double& ms) -> int {
    clear_item_sets(c);
    float best = 1e30f;
    for (int r = 0; r < 2; ++r) {
      int rc = hpsi_interleaved(c, x, nvec, y, nvec, nvec, prec, c->stream, OP_H);
      if (rc) return rc;
      float a = 0.f;
      EVR_CU(cudaEventSynchronize(c->ev[2]), "event sync");
      EVR_CU(cudaEventElapsedTime(&a, c->ev[0], c->ev[1]), "event time");
      if (r > 0) best = a;
    }
    ms = best;
    return check_item_bounds(c);
  };
  const int cands[] = {32, 16, 8, 4, 2};
  int rc = EVR_OK;
  double best = 1e300;
  int bs = c->vt_cap_slab, bi = c->vt_cap_items;
  c->vt_cap_items = 32;
  for (int cap : cands) {
    c->vt_cap_slab = cap;
    double ms;
    if ((rc = time_it(ms))) break;
    if (ms < best) { best = ms; bs = cap; }
  }
  if (!rc) {
    c->vt_cap_slab = bs;
    for (int cap : cands) {
      c->vt_cap_items = cap;
      double ms;
      if ((rc = time_it(ms))) break;
      if (ms < best) { best = ms; bi = cap; }
    }
  }
  // small terms (grid points x tile below a threshold) in the general kernel's CTAs
  int bm = c->slab_min_points;
  if (!rc) {
    c->vt_cap_items = bi;
    const int thr[] = {0, 1024, kSmallTermPoints, 4096, 16384};
    for (int t : thr) {
      c->slab_min_points = t;
      double ms;
      if ((rc = time_it(ms))) break;
      if (ms < best) { best = ms; bm = t; }
    }
  }
  c->vt_cap_slab = bs;
  c->vt_cap_items = bi;
  c->slab_min_points = bm;
  // FP32: the slab kernel's contractions on the CUDA cores or on the tensor cores (above a
  // size K*M); the decomposition changes with the shared memory the tensor-core block takes
  if (!rc && prec == EVR_PREC_FP32) {
    bool btc = c->use_tc;
    int bkm = c->tc_min_km;
    const int kms[] = {64, 160, 288};
    for (int on = 0; on < 2 && !rc; ++on)
      for (int km : kms) {
        c->use_tc = on != 0;
        c->tc_min_km = km;
        double ms;
        if ((rc = time_it(ms))) break;
        if (ms < best) {
          best = ms;
          btc = c->use_tc;
          bkm = km;
        }
        if (!on) break;  // the threshold does not matter with the tensor cores off
      }
    c->use_tc = btc;
    c->tc_min_km = bkm;
  }
  clear_item_sets(c);
  cudaFree(x);
  cudaFree(y);
  if (rc) return rc;
  if (caps) {
    caps[0] = bs;
    caps[1] = bi;
    caps[2] = bm;
    caps[3] = c->use_tc ? c->tc_min_km : -1;
  }
  if (best_ms) *best_ms = best;
  return EVR_OK;
}
