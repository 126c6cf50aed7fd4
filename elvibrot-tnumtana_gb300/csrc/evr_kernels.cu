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

namespace evr {

namespace {

constexpr int kThreads = 256;

template <typename T>
struct ItemParams {
  const TermDesc* terms;
  const T* mats;
  const T* vgrid;
  const T* ggrid;          // SoA symmetric G per term grid point, or nullptr (G constant)
  const double* G0;        // D*D (used when ggrid == nullptr)
  const int* map;
  const WorkItem* items;
  int n_items;
  int* counter;
  T* slab;
  int64_t slab_per_cta;
  const double* x;         // interleaved input (FP64)
  int64_t ldx;
  T* ht;                   // term-basis output
  int64_t ldh;
  int64_t Np;
  int D, nb0, keo_type;
  int has_offdiag;         // type 1 with off-diagonal F2 terms
  int vtrans;              // 1: V_ab read as V_ba (transposed operator)
  int implicit_nvec;       // > 0: items are implicit, item = term * implicit_nvec + vector, one
                           // vector each, buffers in the global slab (items == nullptr)
  // grid operator extras: pot = vw*V + mw*mu when mugrid != nullptr (mw read from mu_dev
  // when that is set); keo_on = 0 drops the kinetic part
  const T* mugrid;
  T vw, mw;
  const double* mu_dev;
  int keo_on;
};

// plain H: no dipole term, kinetic part on
template <typename T>
void set_plain(ItemParams<T>& p) {
  p.mugrid = nullptr;
  p.vw = T(1);
  p.mw = T(0);
  p.mu_dev = nullptr;
  p.keo_on = 1;
}

constexpr int kSlabThreads = 512;

// out(a, m, b, v) = alpha * sum_k mat[m + M*k] * in(a, k, b, v)  (+ out if acc)
// element (a, k, b, v) of a tensor with vector stride ld lives at ((a + A*(k + K*b))*ld + v).
// four consecutive matrix coefficients (staged in shared memory) in one 16-byte load
__device__ __forceinline__ void load4(const float* p, float& a, float& b, float& c, float& d) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  a = v.x; b = v.y; c = v.z; d = v.w;
}
__device__ __forceinline__ void load4(const double* p, double& a, double& b, double& c, double& d) {
  const double2 u = reinterpret_cast<const double2*>(p)[0];
  const double2 w = reinterpret_cast<const double2*>(p)[1];
  a = u.x; b = u.y; c = w.x; d = w.y;
}

// acc[m] += mat[m + ldm*k] * xk for m < M; the matrix columns are padded to ldm = 4*ceil(M/4)
template <typename T, int MAXM>
__device__ __forceinline__ void fma_column(T (&accv)[MAXM], const T* __restrict__ mk, T xk, int M) {
#pragma unroll
  for (int m4 = 0; m4 < MAXM; m4 += 4)
    if (m4 < M) {
      T c0, c1, c2, c3;
      load4(mk + m4, c0, c1, c2, c3);
      accv[m4] = fma(c0, xk, accv[m4]);
      accv[m4 + 1] = fma(c1, xk, accv[m4 + 1]);
      accv[m4 + 2] = fma(c2, xk, accv[m4 + 2]);
      accv[m4 + 3] = fma(c3, xk, accv[m4 + 3]);
    }
}

// Division by a loop-invariant divisor d >= 1 for 0 <= n < 2^31 with one multiply-high:
// q = (umulhi(m, n) + n) >> l, l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1.
struct FastDiv {
  uint32_t d, m, l;
  __device__ __forceinline__ explicit FastDiv(uint32_t dd) : d(dd), l(0) {
    while ((1u << l) < d) ++l;
    m = (uint32_t)((((uint64_t)1 << 32) * (((uint64_t)1 << l) - d)) / d + 1);
  }
  __device__ __forceinline__ uint32_t div(uint32_t n) const { return (__umulhi(m, n) + n) >> l; }
};

// Matrix-stationary contraction: a thread owns MG consecutive output rows m0.. of the 1-D
// matrix (held in registers) and one (a, v) lane, and walks the B dimension; each step
// loads the K inputs of one fibre and issues MG*K FMAs.  Lanes are (a, v, row group);
// when there are fewer lanes than threads the B dimension is split among them.
template <typename T, int MAXK, int MG>
__device__ __forceinline__ void contract_ms(const T* __restrict__ in, int64_t ldi, T* __restrict__ out, int64_t ldo,
                                            int A, int K, int M, int B, int Vt, const T* __restrict__ mat, T alpha,
                                            bool acc) {
  const int ldm = (M + 3) & ~3;
  const int nmg = (M + MG - 1) / MG;
  const int AV = A * Vt;
  const int lanes = AV * nmg;
  const int nthr = blockDim.x;
  int nbg = nthr / lanes;  // B groups when lanes < threads
  if (nbg < 1) nbg = 1;
  if (nbg > B) nbg = B;
  const int tasks = lanes * nbg;
  const FastDiv dvt((uint32_t)Vt), dlanes((uint32_t)lanes), dav((uint32_t)AV);
  const int64_t istr = (int64_t)A * ldi, ostr = (int64_t)A * ldo;
  for (int task = threadIdx.x; task < tasks; task += nthr) {
    const int bg = (int)dlanes.div((uint32_t)task);
    const int lane = task - bg * lanes;
    const int mg = (int)dav.div((uint32_t)lane);
    const int av = lane - mg * AV;
    const int a = (int)dvt.div((uint32_t)av);
    const int v = av - a * Vt;
    const int m0 = mg * MG;
    T strip[MG][MAXK];
#pragma unroll
    for (int mm = 0; mm < MG; ++mm)
#pragma unroll
      for (int k = 0; k < MAXK; ++k)
        strip[mm][k] = (k < K && m0 + mm < M) ? mat[(m0 + mm) + ldm * k] : T(0);
    const T* ip = in + (int64_t)a * ldi + v + (int64_t)bg * K * istr;
    T* op = out + (int64_t)a * ldo + v + (int64_t)m0 * ostr + (int64_t)bg * M * ostr;
    const int64_t istep = (int64_t)nbg * K * istr, ostep = (int64_t)nbg * M * ostr;
    for (int b = bg; b < B; b += nbg, ip += istep, op += ostep) {
      T x[MAXK];
#pragma unroll
      for (int k = 0; k < MAXK; ++k) x[k] = (k < K) ? ip[k * istr] : T(0);
#pragma unroll
      for (int mm = 0; mm < MG; ++mm) {
        T s = T(0);
#pragma unroll
        for (int k = 0; k < MAXK; ++k) s = fma(strip[mm][k], x[k], s);
        if (m0 + mm < M) {
          T val = alpha * s;
          if (acc) val += op[mm * ostr];
          op[mm * ostr] = val;
        }
      }
    }
  }
}

// Loads of a fibre are issued four at a time so that each thread keeps several memory
// requests in flight before the FMAs that consume them; in FP32 a thread carries two
// columns so that every matrix load feeds eight FMAs.
template <typename T, int MAXM, int COLS>
__device__ __forceinline__ void contract_m(const T* __restrict__ in, int64_t ldi, T* __restrict__ out, int64_t ldo,
                                           int A, int K, int M, int B, int Vt, const T* __restrict__ mat, T alpha,
                                           bool acc) {
  const int ncol = A * B * Vt;
  const int ldm = (M + 3) & ~3;
  const FastDiv dv((uint32_t)Vt), da((uint32_t)A);
  const int64_t istr = (int64_t)A * ldi, ostr = (int64_t)A * ldo;
  for (int col0 = threadIdx.x; col0 < ncol; col0 += COLS * blockDim.x) {
    const T* ip[COLS];
    T* op[COLS];
    bool on[COLS];
#pragma unroll
    for (int c = 0; c < COLS; ++c) {
      const int col = col0 + c * blockDim.x;
      on[c] = col < ncol;
      const int cc = on[c] ? col : col0;
      const int r = (int)dv.div((uint32_t)cc);
      const int v = cc - r * Vt;
      const int b = (int)da.div((uint32_t)r);
      const int a = r - b * A;
      ip[c] = in + (int64_t)(a + (int64_t)A * K * b) * ldi + v;
      op[c] = out + (int64_t)(a + (int64_t)A * M * b) * ldo + v;
    }
    T accv[COLS][MAXM];
#pragma unroll
    for (int c = 0; c < COLS; ++c)
#pragma unroll
      for (int m = 0; m < MAXM; ++m) accv[c][m] = T(0);
    for (int k0 = 0; k0 < K; k0 += 4) {
      T x[COLS][4];
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int c = 0; c < COLS; ++c) x[c][j] = (k0 + j < K) ? ip[c][(k0 + j) * istr] : T(0);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (k0 + j < K) {
          const T* mk = mat + ldm * (k0 + j);
#pragma unroll
          for (int m4 = 0; m4 < MAXM; m4 += 4)
            if (m4 < M) {
              T c0, c1, c2, c3;
              load4(mk + m4, c0, c1, c2, c3);
#pragma unroll
              for (int c = 0; c < COLS; ++c) {
                accv[c][m4] = fma(c0, x[c][j], accv[c][m4]);
                accv[c][m4 + 1] = fma(c1, x[c][j], accv[c][m4 + 1]);
                accv[c][m4 + 2] = fma(c2, x[c][j], accv[c][m4 + 2]);
                accv[c][m4 + 3] = fma(c3, x[c][j], accv[c][m4 + 3]);
              }
            }
        }
      }
    }
#pragma unroll
    for (int c = 0; c < COLS; ++c)
      if (on[c])
#pragma unroll
        for (int m = 0; m < MAXM; ++m)
          if (m < M) {
            T val = alpha * accv[c][m];
            if (acc) val += op[c][m * ostr];
            op[c][m * ostr] = val;
          }
  }
}

template <typename T>
__device__ __forceinline__ void contract(const T* in, int64_t ldi, T* out, int64_t ldo, int A, int K, int M, int B,
                                         int Vt, const T* mat, T alpha, bool acc) {
  if constexpr (sizeof(T) == 4) {  // FP32: two columns per thread, matrix coefficients from shared memory
    if (M <= 4) contract_m<T, 4, 2>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else if (M <= 8) contract_m<T, 8, 2>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else if (M <= 12) contract_m<T, 12, 2>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else if (M <= 16) contract_m<T, 16, 2>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else if (M <= 20) contract_m<T, 20, 2>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else contract_m<T, 24, 2>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
  } else {  // FP64: matrix strip in registers (register budget MG*MAXK <= 24 doubles)
    if (K <= 4) contract_ms<T, 4, 4>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else if (K <= 8) contract_ms<T, 8, 2>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else if (K <= 16) contract_ms<T, 16, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else contract_ms<T, 24, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
  }
}

// First B->G mode fused with the gather from the packed vector block:
// in(k, b, v) = x[(map[off_nb + k + K*b] + Np*e) * ldx + v0 + v]  (0 when excluded)
template <typename T, int MAXM>
__device__ __forceinline__ void gather_contract_m(const double* __restrict__ x, int64_t ldx, const int* __restrict__ mp,
                                                  int64_t eoff, T* __restrict__ out, int K, int M, int B, int Vt,
                                                  const T* __restrict__ mat) {
  const int ncol = B * Vt;
  const int ldm = (M + 3) & ~3;
  const FastDiv dv((uint32_t)Vt);
  for (int col = threadIdx.x; col < ncol; col += blockDim.x) {
    const int b = (int)dv.div((uint32_t)col);
    const int v = col - b * Vt;
    T accv[MAXM];
#pragma unroll
    for (int m = 0; m < MAXM; ++m) accv[m] = T(0);
    for (int k0 = 0; k0 < K; k0 += 4) {
      int pk[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) pk[j] = (k0 + j < K) ? __ldg(mp + k0 + j + K * b) : -1;
      T xv[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) xv[j] = (pk[j] >= 0) ? (T)__ldg(x + (pk[j] + eoff) * ldx + v) : T(0);
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (k0 + j < K) fma_column<T, MAXM>(accv, mat + ldm * (k0 + j), xv[j], M);
    }
    T* op = out + (int64_t)M * b * Vt + v;
#pragma unroll
    for (int m = 0; m < MAXM; ++m)
      if (m < M) op[(int64_t)m * Vt] = accv[m];
  }
}

template <typename T>
__device__ __forceinline__ void gather_contract(const double* x, int64_t ldx, const int* mp, int64_t eoff, T* out,
                                                int K, int M, int B, int Vt, const T* mat) {
  if (M <= 4) gather_contract_m<T, 4>(x, ldx, mp, eoff, out, K, M, B, Vt, mat);
  else if (M <= 8) gather_contract_m<T, 8>(x, ldx, mp, eoff, out, K, M, B, Vt, mat);
  else if (M <= 12) gather_contract_m<T, 12>(x, ldx, mp, eoff, out, K, M, B, Vt, mat);
  else if (M <= 16) gather_contract_m<T, 16>(x, ldx, mp, eoff, out, K, M, B, Vt, mat);
  else if (M <= 20) gather_contract_m<T, 20>(x, ldx, mp, eoff, out, K, M, B, Vt, mat);
  else gather_contract_m<T, 24>(x, ldx, mp, eoff, out, K, M, B, Vt, mat);
}

// Copies the item's 1-D matrices from the global pool into shared memory (the layout of
// term_matrix_elems) and points the shared TermDesc's offsets at the copies, so that every
// contraction reads its coefficients from shared memory instead of a small, easily evicted
// L1.
struct StageBlocks {
  int src[4 * kMaxD + 3], dst[4 * kMaxD + 3], n[4 * kMaxD + 3];
  int count;
};

template <typename T>
__device__ __forceinline__ void stage_matrices(TermDesc& Tm, int D, const T* __restrict__ pool, T* msm,
                                               StageBlocks& sb) {
  if (threadIdx.x == 0) {
    int o = 0, c = 0;
    auto add = [&](int32_t& off, int n) {
      sb.src[c] = off;
      sb.dst[c] = o;
      sb.n[c] = n;
      off = o;
      o += n;
      ++c;
    };
    for (int q = 0; q < D; ++q) {
      add(Tm.m_d0b[q], mat_block(Tm.nq[q], Tm.nb[q]));
      add(Tm.m_bgw[q], mat_block(Tm.nb[q], Tm.nq[q]));
      add(Tm.m_d1[q], mat_block(Tm.nq[q], Tm.nq[q]));
      add(Tm.m_d2[q], mat_block(Tm.nq[q], Tm.nq[q]));
    }
    const int L = D - 1;
    add(Tm.m_x1L, mat_block(Tm.nq[L], Tm.nb[L]));
    add(Tm.m_e1L, mat_block(Tm.nb[L], Tm.nq[L]));
    add(Tm.m_e2L, mat_block(Tm.nb[L], Tm.nq[L]));
    sb.count = c;
  }
  __syncthreads();
  for (int b = 0; b < sb.count; ++b) {
    const T* src = pool + sb.src[b];
    T* dst = msm + sb.dst[b];
    for (int i = threadIdx.x; i < sb.n[b]; i += blockDim.x) dst[i] = __ldg(src + i);
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 2) hpsi_items_kernel(ItemParams<T> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ TermDesc s_term;
  __shared__ StageBlocks s_blocks;
  const int D = p.D, nb0 = p.nb0;
  while (true) {
    if (threadIdx.x == 0) s_item = atomicAdd(p.counter, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= p.n_items) break;
    WorkItem w;
    if (p.implicit_nvec > 0) {
      w.term = it / p.implicit_nvec;
      w.v0 = it - w.term * p.implicit_nvec;
      w.vt = 1;
      w.smem = 0;
    } else {
      w = p.items[it];
    }
    {
      const int* src = reinterpret_cast<const int*>(p.terms + w.term);
      int* dst = reinterpret_cast<int*>(&s_term);
      for (int i = threadIdx.x; i < (int)(sizeof(TermDesc) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    T* const mb = reinterpret_cast<T*>(smem_raw);
    stage_matrices<T>(s_term, D, p.mats, mb, s_blocks);
    const TermDesc& Tm = s_term;
    const int NQ = Tm.NQ, NB = Tm.NB, Vt = w.vt;
    const int mpad = (Tm.msz + 3) & ~3;
    T* buf = w.smem ? reinterpret_cast<T*>(smem_raw) + mpad : p.slab + (int64_t)blockIdx.x * p.slab_per_cta;
    const int64_t stride = (int64_t)NQ * Vt;
    T* X0 = buf;                     // psi on the grid, nb0 components
    T* X1 = buf + nb0 * stride;      // H.psi accumulator, nb0 components
    T* Y = buf + 2 * nb0 * stride;   // derivative arrays

    // ---- gather + B->G (modes 0..D-1), ping-pong between X0[e] and X1[e]
    for (int e = 0; e < nb0; ++e) {
      T* A0 = X0 + e * stride;
      T* A1 = X1 + e * stride;
      T* cur = (D % 2) ? A0 : A1;   // so that the chain ends in A0
      int nb_rest = NB / Tm.nb[0];
      gather_contract<T>(p.x + w.v0, p.ldx, p.map + Tm.off_nb, p.Np * e, cur, Tm.nb[0], Tm.nq[0], nb_rest, Vt,
                         mb + Tm.m_d0b[0]);
      __syncthreads();
      int A = Tm.nq[0];
      for (int i = 1; i < D; ++i) {
        nb_rest /= Tm.nb[i];
        T* nxt = (cur == A0) ? A1 : A0;
        contract<T>(cur, Vt, nxt, Vt, A, Tm.nb[i], Tm.nq[i], nb_rest, Vt, mb + Tm.m_d0b[i], T(1), false);
        __syncthreads();
        cur = nxt;
        A *= Tm.nq[i];
      }
    }

    // ---- V.psi: X1[a] = sum_b V_ab X0[b]   (V -> vw V + mw mu with a dipole term)
    {
      const T* Vt_ = p.vgrid + Tm.off_nq * nb0 * nb0;
      const T* Mu_ = p.mugrid ? p.mugrid + Tm.off_nq * nb0 * nb0 : nullptr;
      const T mw = p.mu_dev ? (T)__ldg(p.mu_dev) : p.mw;
      const int64_t n = stride;
      for (int64_t idx = threadIdx.x; idx < n; idx += blockDim.x) {
        const int q = (int)(idx / Vt);
        for (int a = 0; a < nb0; ++a) {
          T s = T(0);
          for (int b = 0; b < nb0; ++b) {
            const int ab = p.vtrans ? (b + nb0 * a) : (a + nb0 * b);
            T vab = __ldg(Vt_ + (int64_t)ab * NQ + q);
            if (Mu_) vab = fma(mw, __ldg(Mu_ + (int64_t)ab * NQ + q), p.vw * vab);
            s = fma(vab, X0[b * stride + idx], s);
          }
          X1[a * stride + idx] = s;
        }
      }
      __syncthreads();
    }

    // ---- KEO
    if (!p.keo_on) {
    } else if (p.keo_type == 10) {
      for (int e = 0; e < nb0; ++e) {
        const T* P0 = X0 + e * stride;
        T* Acc = X1 + e * stride;
        int A = 1, Bq = NQ;
        for (int j = 0; j < D; ++j) {  // Y[j] = d1_j . psi_G
          Bq /= Tm.nq[j];
          contract<T>(P0, Vt, Y + j * stride, Vt, A, Tm.nq[j], Tm.nq[j], Bq, Vt, mb + Tm.m_d1[j], T(1), false);
          A *= Tm.nq[j];
        }
        __syncthreads();
        // Y[i] <- sum_j G_ij(q) Y[j]
        const int nG = D * (D + 1) / 2;
        for (int64_t idx = threadIdx.x; idx < stride; idx += blockDim.x) {
          const int q = (int)(idx / Vt);
          T y[kMaxD], z[kMaxD];
#pragma unroll
          for (int j = 0; j < kMaxD; ++j) { y[j] = (j < D) ? Y[j * stride + idx] : T(0); z[j] = T(0); }
          if (p.ggrid) {
            const T* Gp = p.ggrid + Tm.off_nq * nG + q;
            int c = 0;
#pragma unroll
            for (int i = 0; i < kMaxD; ++i) {
              if (i >= D) break;
#pragma unroll
              for (int j = i; j < kMaxD; ++j) {
                if (j >= D) break;
                const T gij = __ldg(Gp + (int64_t)c * NQ);
                ++c;
                z[i] = fma(gij, y[j], z[i]);
                if (j != i) z[j] = fma(gij, y[i], z[j]);
              }
            }
          } else {
#pragma unroll
            for (int i = 0; i < kMaxD; ++i) {
              if (i >= D) break;
#pragma unroll
              for (int j = 0; j < kMaxD; ++j) {
                if (j >= D) break;
                z[i] = fma((T)__ldg(p.G0 + Tm.perm[i] + D * Tm.perm[j]), y[j], z[i]);
              }
            }
          }
#pragma unroll
          for (int i = 0; i < kMaxD; ++i)
            if (i < D) Y[i * stride + idx] = z[i];
        }
        __syncthreads();
        A = 1; Bq = NQ;
        for (int i = 0; i < D; ++i) {  // Acc += -1/2 d1_i . Y[i]; same-fibre updates per mode
          Bq /= Tm.nq[i];
          contract<T>(Y + i * stride, Vt, Acc, Vt, A, Tm.nq[i], Tm.nq[i], Bq, Vt, mb + Tm.m_d1[i], T(-0.5), true);
          __syncthreads();
          A *= Tm.nq[i];
        }
      }
    } else {
      // type 1: Acc += F2_ii d2_i psi + sum_{i<j} F2_ij d1_i d1_j psi, F2 = -G0/2 (diag), -G0 (off)
      for (int e = 0; e < nb0; ++e) {
        const T* P0 = X0 + e * stride;
        T* Acc = X1 + e * stride;
        int A = 1, Bq = NQ;
        for (int i = 0; i < D; ++i) {
          Bq /= Tm.nq[i];
          const T f = (T)(-0.5 * __ldg(p.G0 + Tm.perm[i] + D * Tm.perm[i]));
          if (f != T(0))
            contract<T>(P0, Vt, Acc, Vt, A, Tm.nq[i], Tm.nq[i], Bq, Vt, mb + Tm.m_d2[i], f, true);
          __syncthreads();
          A *= Tm.nq[i];
        }
        if (p.has_offdiag) {
          int Ai = 1;
          for (int i = 0; i < D; ++i) {
            const int Bi = NQ / (Ai * Tm.nq[i]);
            int Aj = Ai * Tm.nq[i];
            for (int j = i + 1; j < D; ++j) {
              const int Bj = NQ / (Aj * Tm.nq[j]);
              const T f = (T)(-__ldg(p.G0 + Tm.perm[i] + D * Tm.perm[j]));
              if (f != T(0)) {
                contract<T>(P0, Vt, Y, Vt, Ai, Tm.nq[i], Tm.nq[i], Bi, Vt, mb + Tm.m_d1[i], T(1), false);
                __syncthreads();
                contract<T>(Y, Vt, Acc, Vt, Aj, Tm.nq[j], Tm.nq[j], Bj, Vt, mb + Tm.m_d1[j], f, true);
                __syncthreads();
              }
              Aj *= Tm.nq[j];
            }
            Ai *= Tm.nq[i];
          }
        }
      }
    }

    // ---- G->B (modes 0..D-1) with d0b^T w; the last mode writes the term-basis output
    for (int e = 0; e < nb0; ++e) {
      T* A0 = X1 + e * stride;
      T* A1 = X0 + e * stride;
      T* cur = A0;
      int A = 1, Bq = NQ;
      for (int i = 0; i < D; ++i) {
        Bq /= Tm.nq[i];
        if (i == D - 1) {
          T* dst = p.ht + (Tm.off_nb * nb0 + (int64_t)e * NB) * p.ldh + w.v0;
          contract<T>(cur, Vt, dst, p.ldh, A, Tm.nq[i], Tm.nb[i], Bq, Vt, mb + Tm.m_bgw[i], T(1), false);
        } else {
          T* nxt = (cur == A0) ? A1 : A0;
          contract<T>(cur, Vt, nxt, Vt, A, Tm.nq[i], Tm.nb[i], Bq, Vt, mb + Tm.m_bgw[i], T(1), false);
          cur = nxt;
        }
        __syncthreads();
        A *= Tm.nb[i];
      }
    }
  }
}

// P[a] = sum_{k < nL} X[ldx*k] * Tg[a + ss*k]  for a < ss  (one grid slab of the streamed
// position: row q of its grid<-basis matrix applied to the partially transformed tensor)
template <typename T>
__device__ __forceinline__ void slab_extract(const T* __restrict__ Tg, int64_t ss, int nL, const T* __restrict__ X,
                                             int ldx, T* __restrict__ P) {
  for (int64_t a = threadIdx.x; a < ss; a += blockDim.x) {
    T s = T(0);
    for (int k0 = 0; k0 < nL; k0 += 8) {
      T t[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) t[j] = (k0 + j < nL) ? Tg[a + ss * (k0 + j)] : T(0);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (k0 + j < nL) s = fma(X[ldx * (k0 + j)], t[j], s);
    }
    P[a] = s;
  }
}

// W[a + ss*k] += c1*O[k]*A1[a] + c2*E[k]*A2[a]  for k < nL (A2 may be null): the slab's
// image under G->B of the streamed position
template <typename T, int MAXL>
__device__ __forceinline__ void slab_accumulate_m(T* __restrict__ W, int64_t ss, int nL, const T* __restrict__ O,
                                                  const T* __restrict__ A1, T c1, const T* __restrict__ E,
                                                  const T* __restrict__ A2, T c2) {
  T o[MAXL], e[MAXL];  // the slab's column of both matrices, in registers
#pragma unroll
  for (int k = 0; k < MAXL; ++k) {
    o[k] = k < nL ? c1 * O[k] : T(0);
    e[k] = (A2 && k < nL) ? c2 * E[k] : T(0);
  }
  for (int64_t a = threadIdx.x; a < ss; a += blockDim.x) {
    const T u = A1[a];
    const T z = A2 ? A2[a] : T(0);
#pragma unroll
    for (int k = 0; k < MAXL; ++k)
      if (k < nL) W[a + ss * k] = fma(e[k], z, fma(o[k], u, W[a + ss * k]));
  }
}

template <typename T>
__device__ __forceinline__ void slab_accumulate(T* W, int64_t ss, int nL, const T* O, const T* A1, T c1, const T* E,
                                                const T* A2, T c2) {
  if (nL <= 8) slab_accumulate_m<T, 8>(W, ss, nL, O, A1, c1, E, A2, c2);
  else if (nL <= 16) slab_accumulate_m<T, 16>(W, ss, nL, O, A1, c1, E, A2, c2);
  else slab_accumulate_m<T, 24>(W, ss, nL, O, A1, c1, E, A2, c2);
}

// Phi_i = sum_j G_ij(Q) y_j on one slab, in place: y_j = Y[j] (j < L) and P (j = L).
// One thread per grid point: G(Q) (symmetric pairs, from the grid table or the constant
// G0) is read once and applied to the Vt vectors of the tile.
template <typename T, int DM>
__device__ __forceinline__ void slab_pointwise_G(const ItemParams<T>& p, const TermDesc& Tm, T* Y, T* P, int64_t ss,
                                                 int Vt, int q, int NQs, int nG) {
  const int D = p.D, L = D - 1;
  // registers hold the point's G for the vector loop when it is small (FP32, D <= 8)
  constexpr bool kCache = sizeof(T) == 4 && DM <= 8;
  constexpr int kG = kCache ? DM * (DM + 1) / 2 : 1;
  for (int pt = threadIdx.x; pt < NQs; pt += blockDim.x) {
    T G[kG];
    const T* Gp = p.ggrid ? p.ggrid + Tm.off_nq * nG + (int64_t)q * NQs + pt : nullptr;
    // packed slot of (i, j), i <= j < D, in the table's order
    auto slot = [D](int i, int j) { return i * D - i * (i - 1) / 2 + (j - i); };
    auto gload = [&](int i, int j) -> T {
      if (i >= D || j >= D) return T(0);
      return Gp ? __ldg(Gp + (int64_t)slot(i, j) * Tm.NQ) : (T)__ldg(p.G0 + Tm.perm[i] + D * Tm.perm[j]);
    };
    if constexpr (kCache) {
#pragma unroll
      for (int i = 0; i < DM; ++i)
#pragma unroll
        for (int j = i; j < DM; ++j) G[i * DM - i * (i - 1) / 2 + (j - i)] = gload(i, j);
    }
    for (int v = 0; v < Vt; ++v) {
      const int64_t a = (int64_t)pt * Vt + v;
      T y[DM], z[DM];
#pragma unroll
      for (int j = 0; j < DM; ++j) {
        y[j] = (j < L) ? Y[j * ss + a] : ((j == L) ? P[a] : T(0));
        z[j] = T(0);
      }
#pragma unroll
      for (int i = 0; i < DM; ++i)
#pragma unroll
        for (int j = i; j < DM; ++j) {
          T gij;
          if constexpr (kCache) gij = G[i * DM - i * (i - 1) / 2 + (j - i)];
          else gij = gload(i, j);
          z[i] = fma(gij, y[j], z[i]);
          if (j != i) z[j] = fma(gij, y[i], z[j]);
        }
#pragma unroll
      for (int i = 0; i < DM; ++i) {
        if (i < L) Y[i * ss + a] = z[i];
        else if (i == L) P[a] = z[i];
      }
    }
  }
}

// Slab-streaming pipeline for one (term, vector tile) item, one electronic state.  Positions
// 0..L-1 of the term's mode order are transformed whole, position L = D-1 is streamed:
//   A: gather + B->G over positions 0..L-1 (shared-memory ping-pong) -> Tg (global, L2)
//   B: for each grid point q of position L: extract the grid slab P = d0b_L[q,:].Tg, apply V,
//      the derivatives along positions < L and the G(Q) combination on the slab in shared
//      memory (d_L psi comes from (d1.d0b)_L[q,:].Tg), and accumulate the slab's image under
//      G->B of position L into W (shared memory):
//      W[:,k] += bgw_L[k,q] Acc - 1/2 (bgw.d1)_L[k,q] Phi_L        (type 10)
//      W[:,k] += bgw_L[k,q] Acc + F2_LL (bgw.d2)_L[k,q] P           (type 1)
//   C: G->B over positions 0..L-1 of W (shared-memory ping-pong), the last one into the
//      term-basis output.
// The algebra is that of sub_TabOpPsi_OF_ONEDP_FOR_SGtype4 (sub_OpPsi_SG4.f90:1490-1650)
// with the last mode's B->G, derivative and G->B matrices multiplied together.
template <typename T>
__global__ void __launch_bounds__(kSlabThreads, 1) hpsi_slab_kernel(ItemParams<T> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ TermDesc s_term;
  __shared__ StageBlocks s_blocks;
  const int D = p.D, L = D - 1;
  while (true) {
    if (threadIdx.x == 0) s_item = atomicAdd(p.counter, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= p.n_items) break;
    const WorkItem w = p.items[it];
    {
      const int* src = reinterpret_cast<const int*>(p.terms + w.term);
      int* dst = reinterpret_cast<int*>(&s_term);
      for (int i = threadIdx.x; i < (int)(sizeof(TermDesc) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    T* const mb = reinterpret_cast<T*>(smem_raw);
    stage_matrices<T>(s_term, D, p.mats, mb, s_blocks);
    const TermDesc& Tm = s_term;
    const int Vt = w.vt;
    const int gL = Tm.nq[L], nL = Tm.nb[L];
    const int NQs = Tm.NQ / gL;
    const int64_t ss = (int64_t)NQs * Vt;  // one slab array
    const int64_t tsz = ss * nL;           // T and W
    T* sm = reinterpret_cast<T*>(smem_raw) + ((Tm.msz + 3) & ~3);
    T* Tg = p.slab + (int64_t)blockIdx.x * p.slab_per_cta;

    // ---- A: gather + B->G over positions 0..L-1
    if (L == 0) {
      for (int64_t i = threadIdx.x; i < (int64_t)nL * Vt; i += blockDim.x) {
        const int v = (int)(i % Vt), k = (int)(i / Vt);
        const int pk = __ldg(p.map + Tm.off_nb + k);
        Tg[i] = pk >= 0 ? (T)__ldg(p.x + (int64_t)pk * p.ldx + w.v0 + v) : T(0);
      }
    } else {
      T* b0 = sm;
      T* b1 = sm + tsz;
      int nb_rest = Tm.NB / Tm.nb[0];
      T* cur = (L == 1) ? Tg : b0;
      gather_contract<T>(p.x + w.v0, p.ldx, p.map + Tm.off_nb, 0, cur, Tm.nb[0], Tm.nq[0], nb_rest, Vt,
                         mb + Tm.m_d0b[0]);
      __syncthreads();
      int A = Tm.nq[0];
      for (int i = 1; i < L; ++i) {
        nb_rest /= Tm.nb[i];
        T* nxt = (i == L - 1) ? Tg : (cur == b0 ? b1 : b0);
        contract<T>(cur, Vt, nxt, Vt, A, Tm.nb[i], Tm.nq[i], nb_rest, Vt, mb + Tm.m_d0b[i], T(1), false);
        __syncthreads();
        cur = nxt;
        A *= Tm.nq[i];
      }
    }
    __syncthreads();

    // ---- B: stream the grid slabs of position L
    T* W = sm;
    T* Acc = sm + tsz;
    T* P = Acc + ss;
    T* Y = P + ss;
    for (int64_t i = threadIdx.x; i < tsz; i += blockDim.x) W[i] = T(0);
    const int ldx0 = (gL + 3) & ~3, ldo = (nL + 3) & ~3;
    const T* X0 = mb + Tm.m_d0b[L];
    const T* OUT = mb + Tm.m_bgw[L];
    const int nG = D * (D + 1) / 2;
    for (int q = 0; q < gL; ++q) {
      __syncthreads();
      slab_extract<T>(Tg, ss, nL, X0 + q, ldx0, P);
      __syncthreads();
      const T* Vq = p.vgrid + Tm.off_nq + (int64_t)q * NQs;
      if (p.mugrid) {
        const T* Mq = p.mugrid + Tm.off_nq + (int64_t)q * NQs;
        const T mw = p.mu_dev ? (T)__ldg(p.mu_dev) : p.mw;
        for (int64_t a = threadIdx.x; a < ss; a += blockDim.x)
          Acc[a] = fma(mw, __ldg(Mq + a / Vt), p.vw * __ldg(Vq + a / Vt)) * P[a];
      } else {
        for (int64_t a = threadIdx.x; a < ss; a += blockDim.x) Acc[a] = __ldg(Vq + a / Vt) * P[a];
      }
      if (!p.keo_on) {
        __syncthreads();
        slab_accumulate<T>(W, ss, nL, OUT + (int64_t)ldo * q, Acc, T(1), nullptr, nullptr, T(0));
      } else if (p.keo_type == 10) {
        int A = 1, Bq = NQs;
        for (int j = 0; j < L; ++j) {  // Y[j] = d1_j P
          Bq /= Tm.nq[j];
          contract<T>(P, Vt, Y + j * ss, Vt, A, Tm.nq[j], Tm.nq[j], Bq, Vt, mb + Tm.m_d1[j], T(1), false);
          A *= Tm.nq[j];
        }
        __syncthreads();
        slab_extract<T>(Tg, ss, nL, mb + Tm.m_x1L + q, ldx0, P);  // P <- d_L psi on the slab
        __syncthreads();
        // Phi_i = sum_j G_ij(Q) y_j, in place (Y[i] for i < L, P for i = L)
        if (D <= 4) slab_pointwise_G<T, 4>(p, Tm, Y, P, ss, Vt, q, NQs, nG);
        else if (D <= 6) slab_pointwise_G<T, 6>(p, Tm, Y, P, ss, Vt, q, NQs, nG);
        else if (D <= 8) slab_pointwise_G<T, 8>(p, Tm, Y, P, ss, Vt, q, NQs, nG);
        else if (D <= 12) slab_pointwise_G<T, 12>(p, Tm, Y, P, ss, Vt, q, NQs, nG);
        else slab_pointwise_G<T, 16>(p, Tm, Y, P, ss, Vt, q, NQs, nG);
        __syncthreads();
        A = 1;
        Bq = NQs;
        for (int i = 0; i < L; ++i) {  // Acc += -1/2 d1_i Phi_i
          Bq /= Tm.nq[i];
          contract<T>(Y + i * ss, Vt, Acc, Vt, A, Tm.nq[i], Tm.nq[i], Bq, Vt, mb + Tm.m_d1[i], T(-0.5), true);
          __syncthreads();
          A *= Tm.nq[i];
        }
        slab_accumulate<T>(W, ss, nL, OUT + (int64_t)ldo * q, Acc, T(1), mb + Tm.m_e1L + (int64_t)ldo * q, P,
                           T(-0.5));
      } else {
        __syncthreads();
        int A = 1, Bq = NQs;
        for (int i = 0; i < L; ++i) {  // Acc += F2_ii d2_i P
          Bq /= Tm.nq[i];
          const T f = (T)(-0.5 * __ldg(p.G0 + Tm.perm[i] + D * Tm.perm[i]));
          if (f != T(0))
            contract<T>(P, Vt, Acc, Vt, A, Tm.nq[i], Tm.nq[i], Bq, Vt, mb + Tm.m_d2[i], f, true);
          __syncthreads();
          A *= Tm.nq[i];
        }
        if (p.has_offdiag) {
          int Ai = 1;
          for (int i = 0; i < L; ++i) {
            const int Bi = NQs / (Ai * Tm.nq[i]);
            int Aj = Ai * Tm.nq[i];
            for (int j = i + 1; j < L; ++j) {
              const int Bj = NQs / (Aj * Tm.nq[j]);
              const T f = (T)(-__ldg(p.G0 + Tm.perm[i] + D * Tm.perm[j]));
              if (f != T(0)) {
                contract<T>(P, Vt, Y, Vt, Ai, Tm.nq[i], Tm.nq[i], Bi, Vt, mb + Tm.m_d1[i], T(1), false);
                __syncthreads();
                contract<T>(Y, Vt, Acc, Vt, Aj, Tm.nq[j], Tm.nq[j], Bj, Vt, mb + Tm.m_d1[j], f, true);
                __syncthreads();
              }
              Aj *= Tm.nq[j];
            }
            Ai *= Tm.nq[i];
          }
        }
        const T fLL = (T)(-0.5 * __ldg(p.G0 + Tm.perm[L] + D * Tm.perm[L]));
        slab_accumulate<T>(W, ss, nL, OUT + (int64_t)ldo * q, Acc, T(1), mb + Tm.m_e2L + (int64_t)ldo * q, P,
                           fLL);
        if (p.has_offdiag) {  // F2_iL d1_i d_L: d_L through (bgw.d1)_L on the way back
          int Ai = 1;
          for (int i = 0; i < L; ++i) {
            const int Bi = NQs / (Ai * Tm.nq[i]);
            const T f = (T)(-__ldg(p.G0 + Tm.perm[i] + D * Tm.perm[L]));
            if (f != T(0)) {
              __syncthreads();
              contract<T>(P, Vt, Y, Vt, Ai, Tm.nq[i], Tm.nq[i], Bi, Vt, mb + Tm.m_d1[i], T(1), false);
              __syncthreads();
              slab_accumulate<T>(W, ss, nL, mb + Tm.m_e1L + (int64_t)ldo * q, Y, f, nullptr, nullptr, T(0));
            }
            Ai *= Tm.nq[i];
          }
        }
      }
    }
    __syncthreads();

    // ---- C: G->B over positions 0..L-1 of W, the last one into the term-basis output
    T* dst = p.ht + Tm.off_nb * p.ldh + w.v0;
    if (L == 0) {
      for (int64_t i = threadIdx.x; i < (int64_t)nL * Vt; i += blockDim.x) {
        const int v = (int)(i % Vt), k = (int)(i / Vt);
        dst[(int64_t)k * p.ldh + v] = W[i];
      }
    } else {
      T* b0 = W;
      T* b1 = sm + tsz;
      T* cur = b0;
      int A = 1, Bq = NQs;
      for (int i = 0; i < L; ++i) {
        Bq /= Tm.nq[i];
        const int Bt = Bq * nL;
        if (i == L - 1) {
          contract<T>(cur, Vt, dst, p.ldh, A, Tm.nq[i], Tm.nb[i], Bt, Vt, mb + Tm.m_bgw[i], T(1), false);
        } else {
          T* nxt = (cur == b0) ? b1 : b0;
          contract<T>(cur, Vt, nxt, Vt, A, Tm.nq[i], Tm.nb[i], Bt, Vt, mb + Tm.m_bgw[i], T(1), false);
          cur = nxt;
        }
        __syncthreads();
        A *= Tm.nb[i];
      }
    }
  }
}

// y[k*ldy + v] = scale * sum_{e in row k} w_e * (ht[src_e*ldh + v] (+ ht2[...]))   (FP64 accumulation)
template <typename T>
__global__ void csr_reduce_kernel(const int64_t* __restrict__ ptr, const int64_t* __restrict__ src,
                                  const double* __restrict__ wt, const T* __restrict__ ht, const T* __restrict__ ht2,
                                  int64_t ldh, double scale, double* __restrict__ y, int64_t ldy, int64_t N,
                                  int nvec) {
  const int64_t total = N * nvec;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = idx / nvec;
    const int v = (int)(idx - k * nvec);
    double s = 0.0;
    const int64_t e1 = __ldg(ptr + k + 1);
    if (ht2) {
      for (int64_t e = __ldg(ptr + k); e < e1; ++e) {
        const int64_t o = __ldg(src + e) * ldh + v;
        s = fma(__ldg(wt + e), (double)ht[o] + (double)ht2[o], s);
      }
    } else {
      for (int64_t e = __ldg(ptr + k); e < e1; ++e) s = fma(__ldg(wt + e), (double)ht[__ldg(src + e) * ldh + v], s);
    }
    y[k * ldy + v] = scale * s;
  }
}

// grid tables: V_ab(Q) from monomials and the symmetric G(Q) = G0 + sum_k g_ijk Q_k
__global__ void grid_eval_kernel(const TermDesc* __restrict__ terms, int n_terms, const double* __restrict__ mats,
                                 int64_t sum_nq, int D, int nb0, int n_mono, const double* __restrict__ coef,
                                 const int* __restrict__ midx, const int* __restrict__ melec, const double* __restrict__ G0,
                                 const double* __restrict__ g, double* __restrict__ vgrid, double* __restrict__ ggrid) {
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
    int64_t r = q;
    for (int d = 0; d < D; ++d) {
      Q[T.perm[d]] = mats[T.m_x[d] + (int)(r % T.nq[d])];
      r /= T.nq[d];
    }
    double* V = vgrid + T.off_nq * nb0 * nb0;
    for (int ab = 0; ab < nb0 * nb0; ++ab) V[(int64_t)ab * NQ + q] = 0.0;
    for (int m = 0; m < n_mono; ++m) {
      double v = coef[m];
      for (int k = 0; k < 4; ++k) {
        int i = midx[4 * m + k];
        if (i >= 0) v *= Q[i];
      }
      V[(int64_t)(melec[2 * m] + nb0 * melec[2 * m + 1]) * NQ + q] += v;
    }
    if (ggrid) {
      const int nG = D * (D + 1) / 2;
      double* Gp = ggrid + T.off_nq * nG + q;
      int c = 0;
      for (int i = 0; i < D; ++i)  // (i, j) positions of the term's mode order
        for (int j = i; j < D; ++j) {
          const int oi = T.perm[i], oj = T.perm[j];
          double s = G0[oi + D * oj];
          for (int k = 0; k < D; ++k) s += g[oi + D * (oj + D * k)] * Q[k];
          Gp[(int64_t)c * NQ] = s;
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
  int ny = (P.keo_type == 10) ? P.D : 1;
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
  if ((rc = upload(c, &d.G0, P.G0))) return rc;
  if ((rc = upload(c, &d.g, P.g))) return rc;
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
    EVR_CU(cudaMalloc((void**)&gg, P.sum_nq * (D * (D + 1) / 2) * sizeof(double)), "cudaMalloc ggrid");
  }
  c->dp_ggrid = gg;
  grid_eval_kernel<<<c->num_sms * 8, 256, 0, c->stream>>>(d.terms, (int)P.terms.size(), d.mats, P.sum_nq, D, nb0,
                                                          (int)P.mono_coef.size(), d.mono_coef, d.mono_idx,
                                                          d.mono_elec, d.G0, d.g, d.vgrid, gg);
  EVR_CU(cudaGetLastError(), "grid_eval_kernel");
  // FP32 copies for the mixed-precision contractions
  EVR_CU(cudaMalloc((void**)&d.mats32, P.mat_pool.size() * sizeof(float) + 16), "cudaMalloc mats32");
  EVR_CU(cudaMalloc((void**)&d.vgrid32, nv * sizeof(float)), "cudaMalloc vgrid32");
  to_float_kernel<<<c->num_sms * 4, 256, 0, c->stream>>>(d.mats, d.mats32, (int64_t)P.mat_pool.size());
  to_float_kernel<<<c->num_sms * 8, 256, 0, c->stream>>>(d.vgrid, d.vgrid32, nv);
  if (gg) {
    const int64_t ng = P.sum_nq * (D * (D + 1) / 2);
    EVR_CU(cudaMalloc((void**)&c->dp_ggrid32, ng * sizeof(float)), "cudaMalloc ggrid32");
    to_float_kernel<<<c->num_sms * 8, 256, 0, c->stream>>>(gg, c->dp_ggrid32, ng);
  }
  EVR_CU(cudaGetLastError(), "to_float_kernel");
  EVR_CU(cudaStreamSynchronize(c->stream), "grid set-up");
  return EVR_OK;
}

void free_problem(evr_ctx* c) {
  DeviceProblem& d = c->dp;
  void* ptrs[] = {d.terms, d.termsT, d.mats, d.mats32, d.vgrid, d.vgrid32, d.map, d.csr_ptr, d.csr_src, d.csr_w,
                  d.G0, d.g, d.mono_coef, d.mono_idx, d.mono_elec, d.e0diag, c->dp_ggrid, c->dp_ggrid32,
                  c->dp_mugrid, c->dp_mugrid32};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  d = DeviceProblem();
  c->dp_ggrid = nullptr;
  c->dp_ggrid32 = nullptr;
  c->dp_mugrid = nullptr;
  c->dp_mugrid32 = nullptr;
}

void free_workspace(evr_ctx* c) {
  Workspace& w = c->ws;
  for (ItemSet& s : w.sets) {
    if (s.items) cudaFree(s.items);
    if (s.items_slab) cudaFree(s.items_slab);
  }
  void* ptrs[] = {w.counter, w.slab, w.ht, w.ht2, w.xin, w.xout};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  w = Workspace();
  free_stages(c);
}

// elements of shared memory the slab kernel needs for a term and a vector tile
static size_t slab_need_elems(const HostProblem& P, const TermDesc& Tm, int vt) {
  const int L = P.D - 1;
  const size_t ss = (size_t)(Tm.NQ / Tm.nq[L]) * vt, tsz = ss * Tm.nb[L];
  const size_t ny = (P.keo_type == 10) ? (size_t)L : 1;
  return std::max(2 * tsz, tsz + (2 + ny) * ss);
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
    int optin = 0;
    EVR_CU(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device), "attr");
    w.smem_bytes = std::min(optin, 228 * 1024 / 2) - 2048;   // general kernel: 2 CTAs per SM
    w.smem_slab_bytes = optin - 2048;                         // slab kernel: 1 CTA per SM
    w.grid = c->num_sms * 2;
    w.grid_slab = c->num_sms;
    size_t slab = 0;  // general kernel: FP64 buffers of the terms that run from global memory
    for (const TermDesc& Tm : P.terms) {
      size_t fp1 = footprint_elems<double>(P, Tm, 1) * sizeof(double);
      slab = std::max(slab, fp1);
    }
    w.slab_per_cta_bytes = slab;
    // the slab kernel keeps its partially transformed tensor (at most half of its shared
    // memory) in global memory
    w.slab_slab_bytes = (size_t)(w.smem_slab_bytes / 2 + 256) & ~(size_t)255;
    const size_t total = std::max(slab * w.grid, w.slab_slab_bytes * w.grid_slab);
    w.counter = (int*)dev_alloc<int>(2, rc);
    if (rc) return set_error(c, rc, "workspace allocation (counter)");
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
    EVR_CU(cudaFuncSetAttribute(hpsi_items_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                w.smem_bytes), "attr");
    EVR_CU(cudaFuncSetAttribute(hpsi_items_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                w.smem_bytes), "attr");
    EVR_CU(cudaFuncSetAttribute(hpsi_slab_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                w.smem_slab_bytes), "attr");
    EVR_CU(cudaFuncSetAttribute(hpsi_slab_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                w.smem_slab_bytes), "attr");
  }
  for (const ItemSet& s : w.sets)
    if (s.nvec == nvec && s.prec == prec) return EVR_OK;
  const size_t esz = prec == EVR_PREC_FP32 ? sizeof(float) : sizeof(double);
  const bool slab_ok = P.nb0 == 1 && c->use_slab;
  std::vector<WorkItem> items, sitems;
  for (int t = 0; t < (int)P.terms.size(); ++t) {
    const TermDesc& Tm = P.terms[t];
    if (Tm.weight == 0.0) continue;
    const size_t mats = (size_t)((Tm.msz + 3) & ~3) * esz;  // staged 1-D matrices
    if (mats > (size_t)w.smem_bytes) return set_error(c, EVR_EINVAL, "1-D matrices exceed shared memory");
    if (slab_ok && slab_need_elems(P, Tm, 1) * esz + mats <= (size_t)w.smem_slab_bytes) {
      int vt = 1;
      while (vt * 2 <= nvec && vt * 2 <= 32 &&
             slab_need_elems(P, Tm, vt * 2) * esz + mats <= (size_t)w.smem_slab_bytes)
        vt *= 2;
      for (int v0 = 0; v0 < nvec; v0 += vt) sitems.push_back(WorkItem{t, v0, std::min(vt, nvec - v0), 1});
      continue;
    }
    int vt = 1;
    const size_t fp1 = footprint_elems<double>(P, Tm, 1) * esz;
    const bool in_smem = fp1 + mats <= (size_t)w.smem_bytes;
    if (in_smem)
      while (vt * 2 <= nvec && vt * 2 <= 32 && fp1 * (size_t)(vt * 2) + mats <= (size_t)w.smem_bytes) vt *= 2;
    for (int v0 = 0; v0 < nvec; v0 += vt) items.push_back(WorkItem{t, v0, std::min(vt, nvec - v0), in_smem ? 1 : 0});
  }
  auto by_cost = [&](const WorkItem& a, const WorkItem& b) {
    return (int64_t)P.terms[a.term].NQ * a.vt > (int64_t)P.terms[b.term].NQ * b.vt;
  };
  std::stable_sort(items.begin(), items.end(), by_cost);
  std::stable_sort(sitems.begin(), sitems.end(), by_cost);
  ItemSet s;
  s.nvec = nvec;
  s.prec = prec;
  s.n_items = (int)items.size();
  s.n_slab = (int)sitems.size();
  s.items = (WorkItem*)dev_alloc<WorkItem>(items.size(), rc);
  if (rc) return set_error(c, rc, "workspace allocation (items)");
  s.items_slab = (WorkItem*)dev_alloc<WorkItem>(sitems.size(), rc);
  if (rc) return set_error(c, rc, "workspace allocation (items)");
  if (!items.empty())
    EVR_CU(cudaMemcpy(s.items, items.data(), items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice), "items");
  if (!sitems.empty())
    EVR_CU(cudaMemcpy(s.items_slab, sitems.data(), sitems.size() * sizeof(WorkItem), cudaMemcpyHostToDevice),
           "items");
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
  if (P.keo_type == 1)
    for (int i = 0; i < P.D; ++i)
      for (int j = i + 1; j < P.D; ++j) p.has_offdiag |= (P.G0[i + (size_t)P.D * j] != 0.0);
  set_plain(p);
  p.keo_on = ex.keo;
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
    ps.slab_per_cta = (int64_t)(w.slab_slab_bytes / sizeof(T));
    hpsi_slab_kernel<T><<<w.grid_slab, kSlabThreads, w.smem_slab_bytes, s>>>(ps);
    EVR_CU(cudaGetLastError(), "hpsi_slab_kernel launch");
  }
  if (set.n_items > 0) {
    p.items = set.items;
    p.n_items = set.n_items;
    p.slab_per_cta = (int64_t)(w.slab_per_cta_bytes / sizeof(T));
    hpsi_items_kernel<T><<<w.grid, kThreads, w.smem_bytes, s>>>(p);
    EVR_CU(cudaGetLastError(), "hpsi_items_kernel launch");
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
  const int64_t N = P.Np * P.nb0;
  int rblocks = (int)std::min<int64_t>((N * nvec + 255) / 256, (int64_t)c->num_sms * 16);
  csr_reduce_kernel<T><<<rblocks, 256, 0, s>>>(c->dp.csr_ptr, c->dp.csr_src, c->dp.csr_w, (const T*)w.ht,
                                                op == OP_HSYM ? (const T*)w.ht2 : nullptr, nvec,
                                                op == OP_HSYM ? 0.5 : 1.0, y, ldy, N, nvec);
  EVR_CU(cudaGetLastError(), "csr_reduce_kernel launch");
  if (!c->capturing) EVR_CU(cudaEventRecord(c->ev[2], s), "event");
  const int per_op = (set.n_slab > 0 ? 1 : 0) + (set.n_items > 0 ? 1 : 0);
  c->last_kernels = per_op * (op == OP_HSYM ? 2 : 1) + 1;
  c->last_items = (int64_t)(set.n_items + set.n_slab) * (op == OP_HSYM ? 2 : 1);
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
  const ItemSet cp = *set;
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

int reduce_terms(evr_ctx* c, int prec, const void* ht, const void* ht2, int nvec, double scale, double* y,
                 int64_t ldy, cudaStream_t s) {
  const int64_t N = c->hp.Np * c->hp.nb0;
  const int rblocks = (int)std::min<int64_t>((N * nvec + 255) / 256, (int64_t)c->num_sms * 16);
  if (prec == EVR_PREC_FP32)
    csr_reduce_kernel<float><<<rblocks, 256, 0, s>>>(c->dp.csr_ptr, c->dp.csr_src, c->dp.csr_w, (const float*)ht,
                                                      (const float*)ht2, nvec, scale, y, ldy, N, nvec);
  else
    csr_reduce_kernel<double><<<rblocks, 256, 0, s>>>(c->dp.csr_ptr, c->dp.csr_src, c->dp.csr_w, (const double*)ht,
                                                       (const double*)ht2, nvec, scale, y, ldy, N, nvec);
  return cuda_check(c, cudaGetLastError(), "csr_reduce_kernel launch");
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
                                                          out, nullptr);
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
// buffers.  Returns EVR_EINVAL when the scratch is too small.
int hpsi_scratch(evr_ctx* c, const double* x, int64_t ldx, double* y, int64_t ldy, int nvec, unsigned char* scratch,
                 size_t scratch_bytes, cudaStream_t s) {
  const HostProblem& P = c->hp;
  const int grid = c->num_sms * 2;
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
  int optin = 0;
  EVR_CU(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device), "attr");
  if (smem > (size_t)optin / 2) return set_error(c, EVR_EINVAL, "evr_hpsi_noalloc: 1-D matrices too large");
  EVR_CU(cudaFuncSetAttribute(hpsi_items_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin / 2),
         "attr");
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
  p.implicit_nvec = nvec;
  p.has_offdiag = 0;
  if (P.keo_type == 1)
    for (int i = 0; i < P.D; ++i)
      for (int j = i + 1; j < P.D; ++j) p.has_offdiag |= (P.G0[i + (size_t)P.D * j] != 0.0);
  EVR_CU(cudaMemsetAsync(counter, 0, sizeof(int), s), "memset counter");  // the buffer keeps old contents
  hpsi_items_kernel<double><<<grid, kThreads, optin / 2, s>>>(p);
  EVR_CU(cudaGetLastError(), "hpsi_items_kernel launch");
  const int64_t N = P.Np * P.nb0;
  int rblocks = (int)std::min<int64_t>((N * nvec + 255) / 256, (int64_t)c->num_sms * 16);
  csr_reduce_kernel<double><<<rblocks, 256, 0, s>>>(c->dp.csr_ptr, c->dp.csr_src, c->dp.csr_w, ht, nullptr, nvec,
                                                     1.0, y, ldy, N, nvec);
  EVR_CU(cudaGetLastError(), "csr_reduce_kernel launch");
  return EVR_OK;
}

}  // namespace evr
