// evr_stages.cu -- grid-wide H.psi for problems of a single term (direct-product bases).
//
// A direct-product basis is one term: the term-per-CTA kernels would run the whole
// operator on one CTA per vector tile.  Here every stage of the same algebra
// (sub_OpPsi_WITH_MemGrid_BGG_Hamil10, Source_ElVibRot/sub_Operator/sub_OpPsi.f90:1528-1794:
// B->G mode by mode, V(Q) and the type-10 / type-1 kinetic terms on the grid, G->B mode by
// mode) is one launch spread over all SMs:
//   b2g_first   gather from the packed block + B->G of position 0
//   contract    B->G of positions 1..D-1; later G->B of positions 0..D-1 (the last one
//               writes the term-basis output that the CSR reduction turns into H.psi)
//   grid        per grid point: Acc = (vw V + mw mu) psi_G, the first derivatives
//               y_j = d1_j psi_G along every position and Z_i = sum_j G_ij(Q) y_j (type 10),
//               or the F2 d2 diagonal terms and Z_i = sum_{j>i} F2_ij y_j (type 1)
//   div         per grid point: Acc += alpha sum_i d1_i Z_i (alpha = -1/2 for type 10)
// A thread owns one output fibre segment of a contraction (8 rows) or one grid point;
// tensors stay in global memory (L2-resident at direct-product sizes: 24^3 points x 64
// vectors x 8 B = 7 MB).  Element (a, k, b) of state e and vector v of a tensor lives at
// e*cs + (a + A*(k + K*b))*V + v, V = vectors of the call.
#include <algorithm>
#include <vector>

#include "evr_internal.h"

namespace evr {

namespace {

constexpr int kStageThreads = 256;
constexpr int kMG = 8;  // output rows per thread in the contractions

// out(a, m, b) = sum_k d0b[m, k] x(map[k + K*b]), position 0 of the term, all states
template <typename T>
__global__ void __launch_bounds__(kStageThreads) stg_b2g_first(const double* __restrict__ x, int64_t ldx,
                                                                const int* __restrict__ map, int64_t Np, int nb0,
                                                                int K, int M, int B, int V,
                                                                const T* __restrict__ mat, T* __restrict__ out,
                                                                int64_t cs) {
  const int ngrp = (M + kMG - 1) / kMG;
  const int total = nb0 * ngrp * B * V;
  const int ldm = (M + 3) & ~3;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    int r = t;
    const int v = r % V;
    r /= V;
    const int b = r % B;
    r /= B;
    const int g = r % ngrp;
    const int e = r / ngrp;
    const int m0 = g * kMG;
    T acc[kMG];
#pragma unroll
    for (int mm = 0; mm < kMG; ++mm) acc[mm] = T(0);
    for (int k = 0; k < K; ++k) {
      const int pk = __ldg(map + k + K * b);
      const T xk = pk >= 0 ? (T)__ldg(x + (pk + Np * e) * ldx + v) : T(0);
      const T* mk = mat + ldm * k + m0;
#pragma unroll
      for (int mm = 0; mm < kMG; ++mm)
        if (m0 + mm < M) acc[mm] = fma(__ldg(mk + mm), xk, acc[mm]);
    }
    T* op = out + e * cs + ((int64_t)M * b + m0) * V + v;
#pragma unroll
    for (int mm = 0; mm < kMG; ++mm)
      if (m0 + mm < M) op[(int64_t)mm * V] = acc[mm];
  }
}

// out(a, m, b) (+)= alpha sum_k mat[m, k] in(a, k, b), all states
template <typename T>
__global__ void __launch_bounds__(kStageThreads) stg_contract(const T* __restrict__ in, int64_t ics,
                                                               T* __restrict__ out, int64_t ocs, int nb0, int A,
                                                               int K, int M, int B, int V,
                                                               const T* __restrict__ mat, T alpha, int acc) {
  const int ngrp = (M + kMG - 1) / kMG;
  const int AV = A * V;
  const int total = nb0 * ngrp * B * AV;
  const int ldm = (M + 3) & ~3;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    int r = t;
    const int av = r % AV;  // (a, v) with v fastest: consecutive threads, consecutive addresses
    r /= AV;
    const int b = r % B;
    r /= B;
    const int g = r % ngrp;
    const int e = r / ngrp;
    const int m0 = g * kMG;
    T s[kMG];
#pragma unroll
    for (int mm = 0; mm < kMG; ++mm) s[mm] = T(0);
    const T* ip = in + e * ics + (int64_t)K * b * AV + av;
    for (int k = 0; k < K; ++k) {
      const T xk = ip[(int64_t)k * AV];
      const T* mk = mat + ldm * k + m0;
#pragma unroll
      for (int mm = 0; mm < kMG; ++mm)
        if (m0 + mm < M) s[mm] = fma(__ldg(mk + mm), xk, s[mm]);
    }
    T* op = out + e * ocs + ((int64_t)M * b + m0) * AV + av;
#pragma unroll
    for (int mm = 0; mm < kMG; ++mm)
      if (m0 + mm < M) {
        T val = alpha * s[mm];
        if (acc) val += op[(int64_t)mm * AV];
        op[(int64_t)mm * AV] = val;
      }
  }
}

struct GridArgs {
  int D, nb0, NQ, V, keo_on, keo_type, vtrans, has_offdiag;
  int nq[kMaxD], stride[kMaxD];
  int d1[kMaxD], d2[kMaxD];  // matrix offsets in the pool
  int perm[kMaxD];
};

// sum_k mat[qi + ldm*k] * src[(q + (k - qi)*stride)*V]: the 1-D matrix row of a point
// applied along one position
template <typename T>
__device__ __forceinline__ T along(const T* __restrict__ mat, int ldm, int n, int qi, const T* __restrict__ src,
                                   int64_t step) {
  T s = T(0);
  const T* p = src - (int64_t)qi * step;
  for (int k = 0; k < n; ++k) s = fma(__ldg(mat + qi + ldm * k), p[(int64_t)k * step], s);
  return s;
}

// Acc = (vw V + mw mu) psi_G; type 10: Z_i = sum_j G_ij(Q) d1_j psi_G; type 1: Acc += sum_i
// F2_ii d2_i psi_G and Z_i = sum_{j>i} F2_ij d1_j psi_G (F2 = -G0/2 diagonal, -G0 off-diagonal)
template <typename T, int DM>
__global__ void __launch_bounds__(kStageThreads) stg_grid(GridArgs ga, const T* __restrict__ g, T* __restrict__ Acc,
                                                           T* __restrict__ Z, int64_t cs, const T* __restrict__ mats,
                                                           const T* __restrict__ vgrid, const T* __restrict__ mugrid,
                                                           T vw, T mw, const double* __restrict__ mu_dev,
                                                           const T* __restrict__ ggrid,
                                                           const double* __restrict__ G0) {
  const int D = ga.D, nb0 = ga.nb0, NQ = ga.NQ, V = ga.V;
  const int total = NQ * V;
  if (mu_dev) mw = (T)__ldg(mu_dev);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int q = t / V;
    const int64_t pt = (int64_t)q * V + (t - q * V);
    int qi[DM];
    {
      int r = q;
#pragma unroll
      for (int j = 0; j < DM; ++j)
        if (j < D) {
          qi[j] = r % ga.nq[j];
          r /= ga.nq[j];
        }
    }
    T gv[kMaxNb0];
#pragma unroll
    for (int e = 0; e < kMaxNb0; ++e) gv[e] = e < nb0 ? g[e * cs + pt] : T(0);
    for (int a = 0; a < nb0; ++a) {
      T s = T(0);
      for (int b = 0; b < nb0; ++b) {
        const int ab = ga.vtrans ? (b + nb0 * a) : (a + nb0 * b);
        T vab = __ldg(vgrid + (int64_t)ab * NQ + q);
        if (mugrid) vab = fma(mw, __ldg(mugrid + (int64_t)ab * NQ + q), vw * vab);
        s = fma(vab, gv[b], s);
      }
      if (ga.keo_on && ga.keo_type == 1) {
#pragma unroll
        for (int i = 0; i < DM; ++i)
          if (i < D) {
            const T f = (T)(-0.5 * __ldg(G0 + ga.perm[i] + D * ga.perm[i]));
            if (f != T(0)) {
              const int n = ga.nq[i];
              s = fma(f, along(mats + ga.d2[i], (n + 3) & ~3, n, qi[i], g + a * cs + pt, (int64_t)ga.stride[i] * V),
                      s);
            }
          }
      }
      Acc[a * cs + pt] = s;
    }
    if (!ga.keo_on || (ga.keo_type == 1 && !ga.has_offdiag)) continue;
    for (int e = 0; e < nb0; ++e) {
      T y[DM], z[DM];
#pragma unroll
      for (int j = 0; j < DM; ++j) {
        z[j] = T(0);
        if (j < D) {
          const int n = ga.nq[j];
          y[j] = along(mats + ga.d1[j], (n + 3) & ~3, n, qi[j], g + e * cs + pt, (int64_t)ga.stride[j] * V);
        } else {
          y[j] = T(0);
        }
      }
      if (ga.keo_type == 10) {
        if (ggrid) {
          const T* Gp = ggrid + (int64_t)q * g_table_stride(D);
          int c = 0;
#pragma unroll
          for (int i = 0; i < DM; ++i) {
            if (i >= D) break;
#pragma unroll
            for (int j = i; j < DM; ++j) {
              if (j >= D) break;
              const T gij = __ldg(Gp + c);
              ++c;
              z[i] = fma(gij, y[j], z[i]);
              if (j != i) z[j] = fma(gij, y[i], z[j]);
            }
          }
        } else {
#pragma unroll
          for (int i = 0; i < DM; ++i) {
            if (i >= D) break;
#pragma unroll
            for (int j = 0; j < DM; ++j) {
              if (j >= D) break;
              z[i] = fma((T)__ldg(G0 + ga.perm[i] + D * ga.perm[j]), y[j], z[i]);
            }
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < DM; ++i) {
          if (i >= D) break;
#pragma unroll
          for (int j = i + 1; j < DM; ++j) {
            if (j >= D) break;
            z[i] = fma((T)(-__ldg(G0 + ga.perm[i] + D * ga.perm[j])), y[j], z[i]);
          }
        }
      }
#pragma unroll
      for (int i = 0; i < DM; ++i)
        if (i < D) Z[(int64_t)(i * nb0 + e) * cs + pt] = z[i];
    }
  }
}

// Acc += alpha sum_i d1_i Z_i
template <typename T, int DM>
__global__ void __launch_bounds__(kStageThreads) stg_div(GridArgs ga, const T* __restrict__ Z, T* __restrict__ Acc,
                                                          int64_t cs, const T* __restrict__ mats, T alpha) {
  const int D = ga.D, nb0 = ga.nb0, V = ga.V;
  const int total = ga.NQ * V;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int q = t / V;
    const int64_t pt = (int64_t)q * V + (t - q * V);
    int qi[DM];
    {
      int r = q;
#pragma unroll
      for (int j = 0; j < DM; ++j)
        if (j < D) {
          qi[j] = r % ga.nq[j];
          r /= ga.nq[j];
        }
    }
    for (int e = 0; e < nb0; ++e) {
      T s = T(0);
#pragma unroll
      for (int i = 0; i < DM; ++i)
        if (i < D) {
          const int n = ga.nq[i];
          s += along(mats + ga.d1[i], (n + 3) & ~3, n, qi[i], Z + (int64_t)(i * nb0 + e) * cs + pt,
                     (int64_t)ga.stride[i] * V);
        }
      Acc[e * cs + pt] = fma(alpha, s, Acc[e * cs + pt]);
    }
  }
}

template <typename T, int DM>
void launch_grid(const GridArgs& ga, int blocks, cudaStream_t s, const T* g, T* Acc, T* Z, int64_t cs,
                 const T* mats, const T* vgrid, const T* mugrid, T vw, T mw, const double* mu_dev, const T* ggrid,
                 const double* G0) {
  stg_grid<T, DM><<<blocks, kStageThreads, 0, s>>>(ga, g, Acc, Z, cs, mats, vgrid, mugrid, vw, mw, mu_dev, ggrid, G0);
}

template <typename T, int DM>
void launch_div(const GridArgs& ga, int blocks, cudaStream_t s, const T* Z, T* Acc, int64_t cs, const T* mats,
                T alpha) {
  stg_div<T, DM><<<blocks, kStageThreads, 0, s>>>(ga, Z, Acc, cs, mats, alpha);
}

int blocks_for(const evr_ctx* c, int64_t threads) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((threads + kStageThreads - 1) / kStageThreads,
                                                     (int64_t)c->num_sms * 8));
}

// one operator (terms or transposed terms) into ht; returns launches or < 0 on error
template <typename T>
int stage_chain(evr_ctx* c, const TermDesc& Tm, bool transposed, const double* x, int64_t ldx, T* ht, int nvec,
                cudaStream_t s, const OpExtras& ex, int& launches) {
  const HostProblem& P = c->hp;
  const bool f32 = sizeof(T) == 4;
  const T* mats = f32 ? (const T*)c->dp.mats32 : (const T*)c->dp.mats;
  const int D = P.D, nb0 = P.nb0, V = nvec;
  const int64_t cs = c->stg.smax * V;
  T* base = (T*)c->stg.buf;
  const size_t per = c->stg.elems;  // elements per buffer at FP64 size; FP32 uses the same offsets
  T* buf[2] = {base, base + per};
  T* Acc = base + 2 * per;
  T* Z = base + 3 * per;
  // B->G
  int cur = (D % 2) ? 0 : 1;  // so that position D-1 ends in buf[0]
  {
    const int K = Tm.nb[0], M = Tm.nq[0], B = Tm.NB / Tm.nb[0];
    const int64_t th = (int64_t)nb0 * ((M + kMG - 1) / kMG) * B * V;
    stg_b2g_first<T><<<blocks_for(c, th), kStageThreads, 0, s>>>(x, ldx, c->dp.map + Tm.off_nb, P.Np, nb0, K, M, B,
                                                                   V, mats + Tm.m_d0b[0], buf[cur], cs);
    ++launches;
    int A = M, Brest = B;
    for (int i = 1; i < D; ++i) {
      Brest /= Tm.nb[i];
      const int Ki = Tm.nb[i], Mi = Tm.nq[i];
      const int64_t thi = (int64_t)nb0 * ((Mi + kMG - 1) / kMG) * Brest * A * V;
      stg_contract<T><<<blocks_for(c, thi), kStageThreads, 0, s>>>(buf[cur], cs, buf[cur ^ 1], cs, nb0, A, Ki, Mi,
                                                                     Brest, V, mats + Tm.m_d0b[i], T(1), 0);
      ++launches;
      cur ^= 1;
      A *= Mi;
    }
  }
  const T* g = buf[cur];
  // grid stage
  GridArgs ga;
  ga.D = D;
  ga.nb0 = nb0;
  ga.NQ = Tm.NQ;
  ga.V = V;
  ga.keo_on = ex.keo;
  ga.keo_type = P.keo_type;
  ga.vtrans = transposed ? 1 : 0;
  ga.has_offdiag = 0;
  if (P.keo_type == 1)
    for (int i = 0; i < D; ++i)
      for (int j = i + 1; j < D; ++j) ga.has_offdiag |= (P.G0[i + (size_t)D * j] != 0.0);
  int st = 1;
  for (int i = 0; i < kMaxD; ++i) {
    ga.nq[i] = i < D ? Tm.nq[i] : 1;
    ga.stride[i] = st;
    if (i < D) st *= Tm.nq[i];
    ga.d1[i] = i < D ? Tm.m_d1[i] : 0;
    ga.d2[i] = i < D ? Tm.m_d2[i] : 0;
    ga.perm[i] = i < D ? Tm.perm[i] : 0;
  }
  const T* vgrid = f32 ? (const T*)c->dp.vgrid32 : (const T*)c->dp.vgrid;
  const T* mugrid = nullptr;
  if (ex.mw != 0.0 || ex.vw != 1.0 || ex.mu_dev) {
    if (!c->dp_mugrid) return -set_error(c, EVR_EINVAL, "field term without a dipole (evr_set_dipole)");
    mugrid = f32 ? (const T*)c->dp_mugrid32 : (const T*)c->dp_mugrid;
  }
  const T* ggrid = f32 ? (const T*)c->dp_ggrid32 : (const T*)c->dp_ggrid;
  vgrid += Tm.off_nq * nb0 * nb0;
  if (mugrid) mugrid += Tm.off_nq * nb0 * nb0;
  if (ggrid) ggrid += Tm.off_nq * g_table_stride(D);
  const int gb = blocks_for(c, (int64_t)Tm.NQ * V);
  const T vw = (T)ex.vw, mw = (T)ex.mw;
  if (D <= 4) launch_grid<T, 4>(ga, gb, s, g, Acc, Z, cs, mats, vgrid, mugrid, vw, mw, ex.mu_dev, ggrid, c->dp.G0);
  else if (D <= 8) launch_grid<T, 8>(ga, gb, s, g, Acc, Z, cs, mats, vgrid, mugrid, vw, mw, ex.mu_dev, ggrid, c->dp.G0);
  else launch_grid<T, 16>(ga, gb, s, g, Acc, Z, cs, mats, vgrid, mugrid, vw, mw, ex.mu_dev, ggrid, c->dp.G0);
  ++launches;
  const bool div = ex.keo && (P.keo_type == 10 || ga.has_offdiag);
  if (div) {
    const T alpha = P.keo_type == 10 ? T(-0.5) : T(1);
    if (D <= 4) launch_div<T, 4>(ga, gb, s, Z, Acc, cs, mats, alpha);
    else if (D <= 8) launch_div<T, 8>(ga, gb, s, Z, Acc, cs, mats, alpha);
    else launch_div<T, 16>(ga, gb, s, Z, Acc, cs, mats, alpha);
    ++launches;
  }
  // G->B, the last position into the term-basis output
  {
    const T* src = Acc;
    int nxt = 0;
    int A = 1, Brest = Tm.NQ;
    for (int i = 0; i < D; ++i) {
      Brest /= Tm.nq[i];
      const int Ki = Tm.nq[i], Mi = Tm.nb[i];
      const int64_t thi = (int64_t)nb0 * ((Mi + kMG - 1) / kMG) * Brest * A * V;
      T* dst;
      int64_t ocs;
      if (i == D - 1) {
        dst = ht + Tm.off_nb * nb0 * V;
        ocs = (int64_t)Tm.NB * V;
      } else {
        dst = buf[nxt];
        ocs = cs;
      }
      stg_contract<T><<<blocks_for(c, thi), kStageThreads, 0, s>>>(src, cs, dst, ocs, nb0, A, Ki, Mi, Brest, V,
                                                                     mats + Tm.m_bgw[i], T(1), 0);
      ++launches;
      src = dst;
      nxt ^= 1;
      A *= Mi;
    }
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -set_error(c, EVR_EDEVICE, "stage kernel launch");
}

}  // namespace

// largest intermediate tensor (one vector, one state) of the B->G and G->B chains
static int64_t stage_smax(const HostProblem& P) {
  const TermDesc& Tm = P.terms[0];
  int64_t smax = std::max<int64_t>(Tm.NQ, Tm.NB);
  for (int i = 0; i < P.D; ++i) {
    int64_t sb = 1, sg = 1;  // after B->G of positions <= i, and after G->B of positions <= i
    for (int j = 0; j < P.D; ++j) {
      sb *= j <= i ? Tm.nq[j] : Tm.nb[j];
      sg *= j <= i ? Tm.nb[j] : Tm.nq[j];
    }
    smax = std::max(smax, std::max(sb, sg));
  }
  return smax;
}

// Single-term problems whose stage tensors index in 32 bits (thread counts of a stage
// are at most smax * states * 64 vectors * 3 row groups).
bool stages_apply(const evr_ctx* c) {
  // (the stage kernels' per-point arrays hold up to 16 positions; larger direct products
  // run in the term kernels)
  if (!(c->use_stages && c->use_slab && !c->dp_jgrid && c->hp.terms.size() == 1 && c->hp.terms[0].weight != 0.0 &&
        c->hp.terms[0].D <= 16))
    return false;
  const int64_t smax = stage_smax(c->hp);
  return smax * c->hp.nb0 * kMaxBlock * 3 < ((int64_t)1 << 31);
}

void free_stages(evr_ctx* c) {
  if (c->stg.buf) cudaFree(c->stg.buf);
  c->stg = StageBuffers();
}

static int ensure_stages(evr_ctx* c) {
  if (c->stg.buf) return EVR_OK;
  const HostProblem& P = c->hp;
  const int64_t smax = stage_smax(P);
  const size_t per = (size_t)smax * P.nb0 * kMaxBlock;
  const size_t nbuf = 3 + (size_t)P.D;  // two ping-pong tensors, Acc, D divergence inputs
  void* p = nullptr;
  if (cudaMalloc(&p, nbuf * per * sizeof(double)) != cudaSuccess) {
    (void)cudaGetLastError();
    return set_error(c, EVR_ENOMEM, "stage buffers");
  }
  c->stg.buf = p;
  c->stg.elems = per;
  c->stg.smax = smax;
  return EVR_OK;
}

int hpsi_stages(evr_ctx* c, const double* x, int64_t ldx, double* y, int64_t ldy, int nvec, int prec,
                cudaStream_t s, int op, const OpExtras& ex) {
  int rc = ensure_stages(c);
  if (rc) return rc;
  Workspace& w = c->ws;
  const HostProblem& P = c->hp;
  if (op == OP_HSYM && !w.ht2) {
    if (cudaMalloc(&w.ht2, (size_t)P.sum_nb * P.nb0 * w.cap * sizeof(double)) != cudaSuccess) {
      (void)cudaGetLastError();
      w.ht2 = nullptr;
      return set_error(c, EVR_ENOMEM, "workspace allocation (second term-basis output)");
    }
  }
  if (!c->capturing) {
    rc = cuda_check(c, cudaEventRecord(c->ev[0], s), "event");
    if (rc) return rc;
  }
  int launches = 0;
  for (int pass = 0; pass < 2; ++pass) {
    const bool tr = pass == 1;
    if (tr && op == OP_H) continue;
    if (!tr && op == OP_HT) continue;
    const TermDesc& Tm = tr ? P.termsT[0] : P.terms[0];
    void* out = (op == OP_HSYM && tr) ? w.ht2 : w.ht;
    int r = prec == EVR_PREC_FP32
                ? stage_chain<float>(c, Tm, tr, x, ldx, (float*)out, nvec, s, ex, launches)
                : stage_chain<double>(c, Tm, tr, x, ldx, (double*)out, nvec, s, ex, launches);
    if (r < 0) return -r;
  }
  if (!c->capturing) {
    rc = cuda_check(c, cudaEventRecord(c->ev[1], s), "event");
    if (rc) return rc;
  }
  rc = reduce_terms(c, prec, w.ht, op == OP_HSYM ? w.ht2 : nullptr, nvec, op == OP_HSYM ? 0.5 : 1.0, y, ldy, s);
  if (rc) return rc;
  if (!c->capturing) {
    rc = cuda_check(c, cudaEventRecord(c->ev[2], s), "event");
    if (rc) return rc;
  }
  c->last_kernels = launches + 1;
  c->last_items = 0;
  return EVR_OK;
}

}  // namespace evr
