// evr_kernels_impl.cuh -- device code of the term kernels (general and slab-streaming),
// shared by the translation units that instantiate them (evr_kern_<type><gfly>.cu, one
// per precision and G-source variant, compiled in parallel) and by the host code of
// evr_kernels.cu, which only needs the parameter block and the launchers.
#pragma once
#include <algorithm>
#include <cstdio>

#include "evr_internal.h"
#include "evr_tc.cuh"

namespace evr {
namespace kern {

// general (items) kernel: resident CTAs per SM and threads of one (four CTAs of 128 threads
// measured 1 % slower in FP64 at D=6 L=8)
constexpr int kItemsCtas = 2;
constexpr int kThreads = 512 / kItemsCtas;
// the same kernel for small terms: eight CTAs of 64 threads per SM, each with an eighth of
// the shared memory.  Its launch bounds cap a thread at 128 registers, so eight such CTAs
// fit the register file; a small term then keeps two warps busy instead of eight, and
// eight terms share an SM instead of two (D=12 L=6, two vectors, every term below 2048
// points: 2.30 ms per FP64 H.psi against 4.60 ms through the slab kernel and 2.85 ms in
// 256-thread CTAs; FP32 0.78, 2.89 and 1.59 ms)
constexpr int kSmallCtas = 8;
constexpr int kSmallThreads = 64;

template <typename T>
struct ItemParams {
  const TermDesc* terms;
  const T* mats;
  const T* vgrid;
  const T* ggrid;          // symmetric G per grid point (rows of g_table_stride(D)), or nullptr
  const T* jgrid;          // type 10 with a Jacobian: (Jac, sqrt(rho/Jac)) per grid point, or nullptr
                           // (general kernel only; the host routes such contexts there)
  const double* G0;        // D*D per problem, at the term's g0off (used when ggrid == nullptr)
  const double* gco;       // g_ijk per problem at the term's goff: G(Q) = G0 + g.Q evaluated per point
                           // (problems without a G table: gfly != 0)
  const T* G0t;            // G0 and g_ijk in T, read per grid point (no FP64 conversions in FP32)
  const T* gcot;
  int gfly;
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
  // buffer bounds of an item, checked before it runs: elements of T in the dynamic shared
  // memory and in the per-CTA global buffer; an item that would exceed them is skipped
  // and flagged in *err (a host-side sizing error, reported by the host entry points)
  int64_t smem_elems;
  int* err;
  // FP32 slab kernel: mode contractions on the tensor cores (evr_tc.cuh) when use_tc, with
  // their shared-memory block at byte tc_off of the dynamic shared memory (after the
  // smem_elems the items may use); contractions with K*M < tc_min_km stay on the CUDA cores
  int use_tc, tc_off, tc_min_km;
};

// plain H: no dipole term, kinetic part on
template <typename T>
void set_plain(ItemParams<T>& p) {
  p.mugrid = nullptr;
  p.gco = nullptr;
  p.G0t = nullptr;
  p.gcot = nullptr;
  p.gfly = 0;
  p.vw = T(1);
  p.mw = T(0);
  p.mu_dev = nullptr;
  p.keo_on = 1;
  p.use_tc = 0;
  p.tc_off = 0;
  p.tc_min_km = 0;
  p.jgrid = nullptr;
}

// Resident slab-kernel CTAs per SM, and the threads of one: two CTAs of 256 threads, each
// with half of the SM's shared memory, overlap one CTA's barriers and shared-memory waits
// with the other's FMAs.  Measured on the D=6 L=8 launch: FP64 712 ms with one CTA of 512
// threads, 628 ms with two, 606 ms with four of 128 threads -- but with four most FP64 terms
// no longer fit and run in the general kernel from global buffers (55 GB of DRAM traffic
// per D=6 L=6 launch against 1.9 GB with two); FP32 114, 112 and 154 ms.  FP32 with one
// CTA of 1024 threads, 64 registers and one fibre per thread measured 5 % slower.
template <typename T>
constexpr int slab_ctas() { return 2; }
template <typename T>
constexpr int slab_threads() { return 512 / slab_ctas<T>(); }

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
      // FP64: no FMA for the rows past M (the FP64 pipe is the bound); FP32 keeps the
      // unconditional group of four (fewer predicates, the padded rows are discarded)
      constexpr bool kExact = sizeof(T) == 8;
      accv[m4] = fma(c0, xk, accv[m4]);
      if (!kExact || m4 + 1 < M) accv[m4 + 1] = fma(c1, xk, accv[m4 + 1]);
      if (!kExact || m4 + 2 < M) accv[m4 + 2] = fma(c2, xk, accv[m4 + 2]);
      if (!kExact || m4 + 3 < M) accv[m4 + 3] = fma(c3, xk, accv[m4 + 3]);
    }
}

// Division by a loop-invariant divisor d >= 1 for 0 <= n < 2^31 with one multiply-high:
// q = (umulhi(m, n) + n) >> l, l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1.
// Division by a run-time constant d (1 <= d <= 2^31) as a multiply-high and a shift.  The
// magic number costs a 64-bit division, so the kernels build the divisors of a work item
// once (the prefix products of its grid and basis sizes and the vector tile) in shared
// memory and pass them to the contractions.
struct FastDiv {
  uint32_t d, m, l;
  static __device__ __forceinline__ FastDiv make(uint32_t dd) {
    FastDiv f;
    f.d = dd;
    f.l = 0;
    while ((1u << f.l) < dd) ++f.l;
    f.m = (uint32_t)((((uint64_t)1 << 32) * (((uint64_t)1 << f.l) - dd)) / dd + 1);
    return f;
  }
  __device__ __forceinline__ uint32_t div(uint32_t n) const { return (__umulhi(m, n) + n) >> l; }
};

// divisors of one work item: fq[j] = prod_{k<j} nq_k, fb[j] = prod_{k<j} nb_k (j <= D) and
// the vector tile; filled by threads 0..D+1, read after the next barrier
struct ItemDivs {
  FastDiv fq[kMaxD + 1], fb[kMaxD + 1], fv;
};
__device__ __forceinline__ void fill_item_divs(ItemDivs& dv, const TermDesc& Tm, int vt) {
  const int t = threadIdx.x, D = Tm.D;
  if (t <= D) {
    uint32_t pq = 1, pb = 1;
    for (int k = 0; k < t; ++k) {
      pq *= (uint32_t)Tm.nq[k];
      pb *= (uint32_t)Tm.nb[k];
    }
    dv.fq[t] = FastDiv::make(pq);
    dv.fb[t] = FastDiv::make(pb);
  } else if (t == D + 1) {
    dv.fv = FastDiv::make((uint32_t)vt);
  }
}

// The packed G(Q) row of one point (the D(D+1)/2 entries of i <= j < D, i-major) into
// registers with 16-byte loads; the row is padded to a multiple of four entries and
// 16-byte aligned (g_table_stride).  For D == DM the row order is the register order.
template <typename T, int KG>
__device__ __forceinline__ void load_g_row(const T* __restrict__ gp, T (&G)[KG]) {
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int c = 0; c < KG; c += 4) {
      const float4 u = __ldg(reinterpret_cast<const float4*>(gp + c));
      G[c] = u.x;
      if (c + 1 < KG) G[c + 1] = u.y;
      if (c + 2 < KG) G[c + 2] = u.z;
      if (c + 3 < KG) G[c + 3] = u.w;
    }
  } else {
#pragma unroll
    for (int c = 0; c < KG; c += 2) {
      const double2 u = __ldg(reinterpret_cast<const double2*>(gp + c));
      G[c] = u.x;
      if (c + 1 < KG) G[c + 1] = u.y;
    }
  }
}

// Matrix-stationary contraction: a thread owns MG consecutive output rows m0.. of the 1-D
// matrix (held in registers) and one (a, v) lane, and walks the B dimension; each step
// loads the K inputs of one fibre and issues MG*K FMAs.  Lanes are (a, v, row group);
// when there are fewer lanes than threads the B dimension is split among them.
template <typename T, int MAXK, int MG>
__device__ __forceinline__ void contract_ms(const T* __restrict__ in, int64_t ldi, T* __restrict__ out, int64_t ldo,
                                            const FastDiv& da, int K, int M, int B, const FastDiv& dvt,
                                            const T* __restrict__ mat, T alpha, bool acc) {
  const int A = (int)da.d, Vt = (int)dvt.d;
  const int ldm = (M + 3) & ~3;
  const int nmg = (M + MG - 1) / MG;
  const int AV = A * Vt;
  const int lanes = AV * nmg;
  const int nthr = blockDim.x;
  int nbg = nthr / lanes;  // B groups when lanes < threads
  if (nbg < 1) nbg = 1;
  if (nbg > B) nbg = B;
  const int tasks = lanes * nbg;
  const int64_t istr = (int64_t)A * ldi, ostr = (int64_t)A * ldo;
  for (int task = threadIdx.x; task < tasks; task += nthr) {
    // task = v + Vt (a + A (mg + nmg bg))
    const int t1 = (int)dvt.div((uint32_t)task);
    const int v = task - t1 * Vt;
    const int t2 = (int)da.div((uint32_t)t1);
    const int a = t1 - t2 * A;
    const int bg = nmg == 1 ? t2 : t2 / nmg;
    const int mg = t2 - bg * nmg;
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
        for (int k = 0; k < MAXK; ++k)
          if (k < K) s = fma(strip[mm][k], x[k], s);
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
                                           const FastDiv& da, int K, int M, int B, const FastDiv& dv,
                                           const T* __restrict__ mat, T alpha, bool acc) {
  const int A = (int)da.d, Vt = (int)dv.d;
  const int ncol = A * B * Vt;
  const int ldm = (M + 3) & ~3;
  // strides along the contracted and produced index: 32-bit (a tensor of one item holds
  // fewer than 2^31 elements), so the per-load address arithmetic stays 32-bit
  const int istr = (int)(A * ldi), ostr = (int)(A * ldo);
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
__device__ __forceinline__ void contract(const T* in, int64_t ldi, T* out, int64_t ldo, const FastDiv& A, int K, int M,
                                         int B, const FastDiv& Vt, const T* mat, T alpha, bool acc) {
  if constexpr (sizeof(T) == 4) {  // FP32: two columns per thread, matrix coefficients from shared memory
    // four fibres per thread for M <= 12 measured 9 % slower, and a thread walking a chunk of
    // four fibres along B (one index decode per chunk) 14 % slower
    constexpr int C = 2;
    if (M <= 4) contract_m<T, 4, C>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else if (M <= 8) contract_m<T, 8, C>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else if (M <= 12) contract_m<T, 12, C>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else if (M <= 16) contract_m<T, 16, C>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else if (M <= 20) contract_m<T, 20, C>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
    else contract_m<T, 24, C>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
  } else {
    // FP64: one output row per thread with the row's coefficients in registers, in buckets
    // of odd lengths (the 1-D sizes 2l+1 and 2l+3 run without padded FMAs; an even K pads
    // one): the FP64 pipe is the bound, so padded FMAs cost time one for one
    switch ((K >> 1) + 1) {  // bucket 2j-1 >= K: j = K/2 + 1
      case 1: contract_ms<T, 1, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      case 2: contract_ms<T, 3, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      case 3: contract_ms<T, 5, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      case 4: contract_ms<T, 7, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      case 5: contract_ms<T, 9, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      case 6: contract_ms<T, 11, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      case 7: contract_ms<T, 13, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      case 8: contract_ms<T, 15, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      case 9: contract_ms<T, 17, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      case 10: contract_ms<T, 19, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      case 11: contract_ms<T, 21, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      case 12: contract_ms<T, 23, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
      default: contract_ms<T, 24, 1>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc); break;
    }
  }
}

// contract() or, for FP32 with a tensor-core state, the tcgen05 contraction (K <= 24,
// M <= 32, K*M at least the state's threshold).  CTA-wide either way.
template <typename T>
__device__ __forceinline__ void contract_x(tc::TcState* ts, const T* in, int64_t ldi, T* out, int64_t ldo,
                                           const FastDiv& A, int K, int M, int B, const FastDiv& Vt, const T* mat,
                                           T alpha, bool acc) {
  if constexpr (sizeof(T) == 4) {
    // after a lost wait (error flagged) the CTA finishes on the CUDA cores
    if (ts && K <= tc::kMaxKp && M <= tc::kMaxNp && K * M >= ts->min_km && !ts->sm->failed) {
      tc::contract_tc(*ts, in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
      return;
    }
    contract<T>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
  } else {
    contract<T>(in, ldi, out, ldo, A, K, M, B, Vt, mat, alpha, acc);
  }
}

// First B->G mode fused with the gather from the packed vector block:
// in(k, b, v) = x[(map[off_nb + k + K*b] + Np*e) * ldx + v0 + v]  (0 when excluded)
template <typename T, int MAXM>
__device__ __forceinline__ void gather_contract_m(const double* __restrict__ x, int64_t ldx, const int* __restrict__ mp,
                                                  int64_t eoff, T* __restrict__ out, int K, int M, int B,
                                                  const FastDiv& dv, const T* __restrict__ mat) {
  const int Vt = (int)dv.d;
  const int ncol = B * Vt;
  const int ldm = (M + 3) & ~3;
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
                                                int K, int M, int B, const FastDiv& Vt, const T* mat) {
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

// Coordinates of a term grid point: positions 0..npos-1 from the index r (first position
// fastest), the others left to the caller.
template <typename T, int DM>
__device__ __forceinline__ void point_coords(const ItemParams<T>& p, const TermDesc& Tm, int r, int npos,
                                             T (&xq)[DM]) {
#pragma unroll
  for (int k = 0; k < DM; ++k)
    if (k < npos) {
      const int n = Tm.nq[k];
      const int i = r % n;
      r /= n;
      xq[k] = p.mats[Tm.m_x[k] + i];
    } else {
      xq[k] = T(0);
    }
}

// G_ij(Q) = G0_ij + sum_k g_ijk Q_k at a point with coordinates xq (positions i, j, k of the
// term's mode order), for problems without a G table.  Evaluated in T from the T copies
// of G0 and g: in FP32 H.psi the model then costs D FP32 FMAs per entry and no FP64
// instruction (the GB300 FP64 pipe, and its conversions, issue at a small fraction of the
// FP32 rate; FP64 arithmetic here dominated the FP32 batched H.psi)
template <typename T, int DM>
__device__ __forceinline__ T g_model(const ItemParams<T>& p, const TermDesc& Tm, const T (&xq)[DM], int i, int j) {
  const int D = Tm.D, Dp = Tm.Dp, oi = Tm.perm[i], oj = Tm.perm[j];
  T s = __ldg(p.G0t + Tm.g0off + oi + Dp * oj);
  const T* gp = p.gcot + Tm.goff + oi + Dp * oj;
#pragma unroll
  for (int k = 0; k < DM; ++k)  // dropped 1-point modes sit at Q = 0
    if (k < D) s = fma(__ldg(gp + Dp * Dp * Tm.perm[k]), xq[k], s);
  return s;
}

// Phi_i = sum_j G_ij(Q) y_j for terms of more than 8 active positions (rare: levels above 8
// in more than 8 modes, or modes whose level-0 grid has several points), at points
// r0 .. r0+npts-1 of the term grid: y_j = Y[j*ys + pt*Vt + v] for j < D-1 and last[pt*Vt + v]
// for j = D-1, in place; with jac, Phi_i is multiplied by jac[2*(r0+pt)].  Runtime loops
// over the positions and the point's G (table row, G0 or the linear model) in a per-thread
// array: one out-of-line copy per kernel instead of unrolled loops of every width.
template <typename T, bool GFLY>
__device__ __noinline__ void pointwise_G_wide(const ItemParams<T>& p, const TermDesc& Tm, T* Y, int64_t ys, T* last,
                                              int Vt, int npts, int64_t r0, const T* jac) {
  const int D = Tm.D, L = D - 1;
  const int nG = g_table_stride(Tm.Dp);
  const int nch = max(1, min(Vt, (int)blockDim.x / max(npts, 1)));
  for (int task = threadIdx.x; task < npts * nch; task += blockDim.x) {
    const int pt = task / nch, ch = task - pt * nch;
    const int64_t r = r0 + pt;
    T G[kMaxD * (kMaxD + 1) / 2];
    if (GFLY) {  // the linear model in T, as g_model
      T xq[kMaxD];
      int rr = (int)r;
      for (int k = 0; k < D; ++k) {
        const int n = Tm.nq[k];
        const int i = rr % n;
        rr /= n;
        xq[k] = p.mats[Tm.m_x[k] + i];
      }
      int s = 0;
      for (int i = 0; i < D; ++i)
        for (int j = i; j < D; ++j, ++s) {
          const int oi = Tm.perm[i], oj = Tm.perm[j];
          T g = __ldg(p.G0t + Tm.g0off + oi + Tm.Dp * oj);
          const T* gp = p.gcot + Tm.goff + oi + Tm.Dp * oj;
          for (int k = 0; k < D; ++k) g = fma(__ldg(gp + Tm.Dp * Tm.Dp * Tm.perm[k]), xq[k], g);
          G[s] = g;
        }
    } else if (p.ggrid) {
      const T* Gp = p.ggrid + (Tm.off_nq + r) * nG;
      for (int s = 0; s < D * (D + 1) / 2; ++s) G[s] = __ldg(Gp + s);
    } else {
      int s = 0;
      for (int i = 0; i < D; ++i)
        for (int j = i; j < D; ++j, ++s) G[s] = __ldg(p.G0t + Tm.g0off + Tm.perm[i] + Tm.Dp * Tm.perm[j]);
    }
    const T jq = jac ? jac[2 * r] : T(1);
    for (int v = ch; v < Vt; v += nch) {
      const int64_t a = (int64_t)pt * Vt + v;
      T y[kMaxD], z[kMaxD];
      for (int j = 0; j < D; ++j) {
        y[j] = j < L ? Y[j * ys + a] : last[a];
        z[j] = T(0);
      }
      int s = 0;
      for (int i = 0; i < D; ++i)
        for (int j = i; j < D; ++j, ++s) {
          z[i] = fma(G[s], y[j], z[i]);
          if (j != i) z[j] = fma(G[s], y[i], z[j]);
        }
      for (int i = 0; i < D; ++i) {
        if (i < L) Y[i * ys + a] = jq * z[i];
        else last[a] = jq * z[i];
      }
    }
  }
}

// Y[i] <- sum_j G_ij(Q) Y[j] on the whole term grid (general kernel).  A thread owns a grid
// point and a residue class of the tile's vectors (several classes per point when the
// grid has fewer points than the CTA has threads); G(Q) is held in registers for D <= 6
// (FP64) or 8 (FP32) and applied to the thread's vectors.
template <typename T, int DM, bool GFLY>
__device__ __forceinline__ void items_pointwise_G(const ItemParams<T>& p, const TermDesc& Tm, T* Y, int64_t stride,
                                                  int Vt, int NQ) {
  // with a Jacobian table the combination is Jac(Q) sum_j G_ij(Q) Y_j (sub_OpPsi_SG4.f90:1599-1606)
  const T* Jp = p.jgrid ? p.jgrid + 2 * Tm.off_nq : nullptr;
  const int D = Tm.D;
  const int nG = g_table_stride(Tm.Dp);  // table row of a point (the problem's slots, padded)
  constexpr bool kCache = DM <= (sizeof(T) == 4 ? 8 : 6);
  constexpr int kG = kCache ? DM * (DM + 1) / 2 : 1;
  const int nch = max(1, min(Vt, (int)blockDim.x / max(NQ, 1)));
  auto slot = [D](int i, int j) { return i * D - i * (i - 1) / 2 + (j - i); };
  for (int task = threadIdx.x; task < NQ * nch; task += blockDim.x) {
    const int q = task / nch, ch = task - q * nch;
    const T* Gp = p.ggrid ? p.ggrid + (Tm.off_nq + q) * nG : nullptr;
    T xq[DM];
    if constexpr (GFLY) point_coords<T, DM>(p, Tm, q, D, xq);
    auto gget = [&](int i, int j) -> T {
      if (i >= D || j >= D) return T(0);
      if constexpr (GFLY) return g_model<T, DM>(p, Tm, xq, i, j);
      return Gp ? __ldg(Gp + slot(i, j)) : __ldg(p.G0t + Tm.g0off + Tm.perm[i] + Tm.Dp * Tm.perm[j]);
    };
    T G[kG];
    if constexpr (kCache) {
      if (!GFLY && Gp && D == DM) {
        load_g_row<T, kG>(Gp, G);
      } else {
#pragma unroll
        for (int i = 0; i < DM; ++i)
#pragma unroll
          for (int j = i; j < DM; ++j) G[i * DM - i * (i - 1) / 2 + (j - i)] = gget(i, j);
      }
    }
    // the thread's vectors ch, ch + nch, ... in an order rotated by the point, so that the
    // lanes of a warp (neighbouring points, Vt elements apart) fall in different banks
    const int cnt = (Vt - ch + nch - 1) / nch;
    int jv = cnt > 0 ? q % cnt : 0;
    for (int iv = 0; iv < cnt; ++iv) {
      const int v = ch + nch * jv;
      jv = (jv + 1 == cnt) ? 0 : jv + 1;
      const int64_t idx = (int64_t)q * Vt + v;
      T y[DM], z[DM];
#pragma unroll
      for (int j = 0; j < DM; ++j) {
        y[j] = (j < D) ? Y[j * stride + idx] : T(0);
        z[j] = T(0);
      }
#pragma unroll
      for (int i = 0; i < DM; ++i)
#pragma unroll
        for (int j = i; j < DM; ++j) {
          T gij;
          if constexpr (kCache) gij = G[i * DM - i * (i - 1) / 2 + (j - i)];
          else gij = gget(i, j);
          z[i] = fma(gij, y[j], z[i]);
          if (j != i) z[j] = fma(gij, y[i], z[j]);
        }
      const T jq = Jp ? Jp[2 * q] : T(1);
#pragma unroll
      for (int i = 0; i < DM; ++i)
        if (i < D) Y[i * stride + idx] = jq * z[i];
    }
  }
}

// Pointwise factors of a type-10 operator with a Jacobian (sub_OpPsi_SG4.f90:1581, :1618):
// X[q, v] *= sqRhoOVERJac(q) before the derivatives; for the transposed operator
// 1/(Jac sqRhoOVERJac) comes first instead
template <typename T>
__device__ __forceinline__ void items_jac_pre(const ItemParams<T>& p, const TermDesc& Tm, T* X, int Vt, int NQ) {
  const T* Jp = p.jgrid + 2 * Tm.off_nq;
  for (int64_t idx = threadIdx.x; idx < (int64_t)NQ * Vt; idx += blockDim.x) {
    const int q = (int)(idx / Vt);
    const T j = Jp[2 * q], sq = Jp[2 * q + 1];
    X[idx] *= p.vtrans ? T(1) / (j * sq) : sq;
  }
}
// Acc += -1/2 K / (Jac sqRhoOVERJac) (transposed operator: -1/2 K sqRhoOVERJac)
template <typename T>
__device__ __forceinline__ void items_jac_post(const ItemParams<T>& p, const TermDesc& Tm, const T* K, T* Acc, int Vt,
                                               int NQ) {
  const T* Jp = p.jgrid + 2 * Tm.off_nq;
  for (int64_t idx = threadIdx.x; idx < (int64_t)NQ * Vt; idx += blockDim.x) {
    const int q = (int)(idx / Vt);
    const T j = Jp[2 * q], sq = Jp[2 * q + 1];
    Acc[idx] = fma(T(-0.5) * K[idx], p.vtrans ? sq : T(1) / (j * sq), Acc[idx]);
  }
}

template <typename T, bool GFLY>
__global__ void __launch_bounds__(kThreads, kItemsCtas) hpsi_items_kernel(ItemParams<T> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ TermDesc s_term;
  __shared__ StageBlocks s_blocks;
  __shared__ ItemDivs s_div;
  const int nb0 = p.nb0;
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
    const int D = s_term.D;
    {
      const int64_t need = (int64_t)(2 * nb0 + (p.keo_type == 10 ? D : 1)) * s_term.NQ * w.vt;
      const int64_t mp = (s_term.msz + 3) & ~3;
      if (mp > p.smem_elems || (w.smem ? mp + need > p.smem_elems : need > p.slab_per_cta)) {
        if (threadIdx.x == 0) atomicExch(p.err, 1);
        continue;
      }
    }
    T* const mb = reinterpret_cast<T*>(smem_raw);
    fill_item_divs(s_div, s_term, w.vt);  // visible after the barriers of stage_matrices
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
      gather_contract<T>(p.x + w.v0, p.ldx, p.map + Tm.off_nb, p.Np * e, cur, Tm.nb[0], Tm.nq[0], nb_rest, s_div.fv,
                         mb + Tm.m_d0b[0]);
      __syncthreads();
      int A = Tm.nq[0];
      for (int i = 1; i < D; ++i) {
        nb_rest /= Tm.nb[i];
        T* nxt = (cur == A0) ? A1 : A0;
        contract<T>(cur, Vt, nxt, Vt, s_div.fq[i], Tm.nb[i], Tm.nq[i], nb_rest, s_div.fv, mb + Tm.m_d0b[i], T(1), false);
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
        T* P0 = X0 + e * stride;
        T* Acc = X1 + e * stride;
        if (p.jgrid) {  // psi * sqRhoOVERJac (V psi is done)
          items_jac_pre<T>(p, Tm, P0, Vt, NQ);
          __syncthreads();
        }
        int A = 1, Bq = NQ;
        for (int j = 0; j < D; ++j) {  // Y[j] = d1_j . psi_G
          Bq /= Tm.nq[j];
          contract<T>(P0, Vt, Y + j * stride, Vt, s_div.fq[j], Tm.nq[j], Tm.nq[j], Bq, s_div.fv, mb + Tm.m_d1[j], T(1), false);
          A *= Tm.nq[j];
        }
        __syncthreads();
        // Y[i] <- sum_j G_ij(q) Y[j]
        if (D <= 4) items_pointwise_G<T, 4, GFLY>(p, Tm, Y, stride, Vt, NQ);
        else if (D <= 6) items_pointwise_G<T, 6, GFLY>(p, Tm, Y, stride, Vt, NQ);
        else if (D <= 8) items_pointwise_G<T, 8, GFLY>(p, Tm, Y, stride, Vt, NQ);
        else pointwise_G_wide<T, GFLY>(p, Tm, Y, stride, Y + (D - 1) * stride, Vt, NQ, 0,
                                       p.jgrid ? p.jgrid + 2 * Tm.off_nq : nullptr);
        __syncthreads();
        A = 1; Bq = NQ;
        // Acc += -1/2 d1_i . Y[i]; same-fibre updates per mode.  With a Jacobian the
        // divergence is summed in P0 (psi is no longer needed) and then divided by
        // Jac sqRhoOVERJac point by point
        T* Kd = p.jgrid ? P0 : Acc;
        for (int i = 0; i < D; ++i) {
          Bq /= Tm.nq[i];
          contract<T>(Y + i * stride, Vt, Kd, Vt, s_div.fq[i], Tm.nq[i], Tm.nq[i], Bq, s_div.fv, mb + Tm.m_d1[i],
                      p.jgrid ? T(1) : T(-0.5), p.jgrid ? i > 0 : true);
          __syncthreads();
          A *= Tm.nq[i];
        }
        if (p.jgrid) {
          items_jac_post<T>(p, Tm, P0, Acc, Vt, NQ);
          __syncthreads();
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
          const T f = (T)(-0.5 * __ldg(p.G0 + Tm.g0off + Tm.perm[i] + Tm.Dp * Tm.perm[i]));
          if (f != T(0))
            contract<T>(P0, Vt, Acc, Vt, s_div.fq[i], Tm.nq[i], Tm.nq[i], Bq, s_div.fv, mb + Tm.m_d2[i], f, true);
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
              const T f = (T)(-__ldg(p.G0 + Tm.g0off + Tm.perm[i] + Tm.Dp * Tm.perm[j]));
              if (f != T(0)) {
                contract<T>(P0, Vt, Y, Vt, s_div.fq[i], Tm.nq[i], Tm.nq[i], Bi, s_div.fv, mb + Tm.m_d1[i], T(1), false);
                __syncthreads();
                contract<T>(Y, Vt, Acc, Vt, s_div.fq[j], Tm.nq[j], Tm.nq[j], Bj, s_div.fv, mb + Tm.m_d1[j], f, true);
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
          contract<T>(cur, Vt, dst, p.ldh, s_div.fb[i], Tm.nq[i], Tm.nb[i], Bq, s_div.fv, mb + Tm.m_bgw[i], T(1), false);
        } else {
          T* nxt = (cur == A0) ? A1 : A0;
          contract<T>(cur, Vt, nxt, Vt, s_div.fb[i], Tm.nq[i], Tm.nb[i], Bq, s_div.fv, mb + Tm.m_bgw[i], T(1), false);
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
  const int s32 = (int)ss;  // 32-bit index arithmetic (a slab tensor has < 2^31 elements)
  for (int a = threadIdx.x; a < s32; a += blockDim.x) {
    T s = T(0);
    for (int k0 = 0; k0 < nL; k0 += 8) {
      T t[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) t[j] = (k0 + j < nL) ? Tg[a + s32 * (k0 + j)] : T(0);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (k0 + j < nL) s = fma(X[ldx * (k0 + j)], t[j], s);
    }
    P[a] = s;
  }
}

// One pass over the partially transformed tensor for the type-10 slab: psi (row X of the
// grid<-basis matrix) and its derivative along the streamed position (row X1 of d1.d0b) on
// the slab, and Acc = (vw V + mw mu) psi
template <typename T>
__device__ __forceinline__ void slab_extract_fused(const T* __restrict__ Tg, int64_t ss, int nL,
                                                   const T* __restrict__ X, const T* __restrict__ X1, int ldx,
                                                   T* __restrict__ P, T* __restrict__ P1, T* __restrict__ Acc,
                                                   const T* __restrict__ Vq, const T* __restrict__ Mq, T vw, T mw,
                                                   const FastDiv& dvt) {
  const int s32 = (int)ss;
  for (int a = threadIdx.x; a < s32; a += blockDim.x) {
    T s = T(0), s1 = T(0);
    for (int k0 = 0; k0 < nL; k0 += 8) {
      T t[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) t[j] = (k0 + j < nL) ? Tg[a + s32 * (k0 + j)] : T(0);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (k0 + j < nL) {
          s = fma(X[ldx * (k0 + j)], t[j], s);
          s1 = fma(X1[ldx * (k0 + j)], t[j], s1);
        }
    }
    P[a] = s;
    P1[a] = s1;
    const int pt = (int)dvt.div((uint32_t)a);
    T v = __ldg(Vq + pt);
    if (Mq) v = fma(mw, __ldg(Mq + pt), vw * v);
    Acc[a] = v * s;
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
  const int s32 = (int)ss;
  for (int a = threadIdx.x; a < s32; a += blockDim.x) {
    const T u = A1[a];
    const T z = A2 ? A2[a] : T(0);
#pragma unroll
    for (int k = 0; k < MAXL; ++k)
      if (k < nL) W[a + s32 * k] = fma(e[k], z, fma(o[k], u, W[a + s32 * k]));
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
template <typename T, int DM, bool GFLY>
__device__ __forceinline__ void slab_pointwise_G(const ItemParams<T>& p, const TermDesc& Tm, T* Y, T* P, int64_t ss,
                                                 int Vt, int q, int NQs, int nG) {
  const int D = Tm.D, L = D - 1;
  // registers hold the point's G for the vector loop when it is small (D <= 6 in FP64,
  // D <= 8 in FP32)
  constexpr bool kCache = DM <= (sizeof(T) == 4 ? 8 : 6);
  constexpr int kG = kCache ? DM * (DM + 1) / 2 : 1;
  // a thread owns a point and a residue class of the tile's vectors: with fewer points in
  // the slab than threads, several threads share a point (each loads its G)
  const int nch = max(1, min(Vt, (int)blockDim.x / max(NQs, 1)));
  for (int task = threadIdx.x; task < NQs * nch; task += blockDim.x) {
    const int pt = task / nch, ch = task - pt * nch;
    T G[kG];
    const T* Gp = p.ggrid ? p.ggrid + (Tm.off_nq + (int64_t)q * NQs + pt) * nG : nullptr;
    T xq[DM];
    if constexpr (GFLY) {
      point_coords<T, DM>(p, Tm, pt, L, xq);
#pragma unroll
      for (int k = 0; k < DM; ++k)
        if (k == L) xq[k] = p.mats[Tm.m_x[k] + q];
    }
    // packed slot of (i, j), i <= j < D, in the table's order
    auto slot = [D](int i, int j) { return i * D - i * (i - 1) / 2 + (j - i); };
    auto gload = [&](int i, int j) -> T {
      if (i >= D || j >= D) return T(0);
      if constexpr (GFLY) return g_model<T, DM>(p, Tm, xq, i, j);
      return Gp ? __ldg(Gp + slot(i, j)) : __ldg(p.G0t + Tm.g0off + Tm.perm[i] + Tm.Dp * Tm.perm[j]);
    };
    if constexpr (kCache) {
      if (!GFLY && Gp && D == DM) {
        load_g_row<T, kG>(Gp, G);
      } else {
#pragma unroll
        for (int i = 0; i < DM; ++i)
#pragma unroll
          for (int j = i; j < DM; ++j) G[i * DM - i * (i - 1) / 2 + (j - i)] = gload(i, j);
      }
    }
    // vectors in an order rotated by the point (bank-conflict free, as in items_pointwise_G)
    const int cnt = (Vt - ch + nch - 1) / nch;
    int jv = cnt > 0 ? pt % cnt : 0;
    for (int iv = 0; iv < cnt; ++iv) {
      const int v = ch + nch * jv;
      jv = (jv + 1 == cnt) ? 0 : jv + 1;
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

// Type-10 kinetic part of one grid slab of the streamed position, from psi (P) and its
// derivative along the streamed position (P1 = Y[L]):  Y[j] = d1_j psi (j < L),
// Phi = G(Q) y in place, Acc += -1/2 sum_{i<L} d1_i Phi_i  (Phi_L stays in P1 for the
// grid->basis side of the streamed position).  Starts after a barrier, ends with one.
template <typename T, bool GFLY>
__device__ __forceinline__ void slab_keo10(const ItemParams<T>& p, const TermDesc& Tm, const ItemDivs& s_div,
                                           const T* mb, T* P, T* Y, T* P1, T* Acc, int64_t ss, int Vt, int q,
                                           int NQs, int nG, tc::TcState* ts) {
  const int D = Tm.D, L = D - 1;
  int A = 1, Bq = NQs;
  for (int j = 0; j < L; ++j) {  // Y[j] = d1_j psi
    Bq /= Tm.nq[j];
    contract_x<T>(ts, P, Vt, Y + j * ss, Vt, s_div.fq[j], Tm.nq[j], Tm.nq[j], Bq, s_div.fv, mb + Tm.m_d1[j], T(1), false);
    A *= Tm.nq[j];
  }
  __syncthreads();
  // Phi_i = sum_j G_ij(Q) y_j, in place (Y[i], i <= L)
  if (D <= 4) slab_pointwise_G<T, 4, GFLY>(p, Tm, Y, P1, ss, Vt, q, NQs, nG);
  else if (D <= 6) slab_pointwise_G<T, 6, GFLY>(p, Tm, Y, P1, ss, Vt, q, NQs, nG);
  else if (D <= 8) slab_pointwise_G<T, 8, GFLY>(p, Tm, Y, P1, ss, Vt, q, NQs, nG);
  else pointwise_G_wide<T, GFLY>(p, Tm, Y, ss, P1, Vt, NQs, (int64_t)q * NQs, nullptr);
  __syncthreads();
  A = 1;
  Bq = NQs;
  for (int i = 0; i < L; ++i) {  // Acc += -1/2 d1_i Phi_i
    Bq /= Tm.nq[i];
    contract_x<T>(ts, Y + i * ss, Vt, Acc, Vt, s_div.fq[i], Tm.nq[i], Tm.nq[i], Bq, s_div.fv, mb + Tm.m_d1[i], T(-0.5), true);
    __syncthreads();
    A *= Tm.nq[i];
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
// TC (FP32 only): the mode contractions with K*M >= p.tc_min_km on the tensor cores; a
// separate instantiation, so that the CUDA-core kernel carries no call into them.
template <typename T, bool GFLY, bool TC>
__global__ void __launch_bounds__(slab_threads<T>(), slab_ctas<T>()) hpsi_slab_kernel(ItemParams<T> p) {
  static_assert(!TC || sizeof(T) == 4, "tensor-core contractions are FP32");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ TermDesc s_term;
  __shared__ StageBlocks s_blocks;
  __shared__ ItemDivs s_div;
  // the tensor-core contractions' shared block and TMEM accumulator for the CTA's life
  tc::TcState tcs;
  tc::TcState* ts = nullptr;
  if constexpr (TC) {
    tc::tc_setup(tcs, reinterpret_cast<tc::TcSmem*>(smem_raw + p.tc_off), p.err);
    tcs.min_km = p.tc_min_km;
    ts = &tcs;
  }
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
    const int D = s_term.D, L = D - 1;
    {
      const int64_t ss0 = (int64_t)(s_term.NQ / s_term.nq[L]) * w.vt, tsz0 = ss0 * s_term.nb[L];
      // type 10: the first derivatives, and d_L psi in FP32 (fused extraction)
      const int64_t ny = p.keo_type == 10 ? L + (sizeof(T) == 4 ? 1 : 0) : 1;
      const int64_t need = max(2 * tsz0, tsz0 + (2 + ny) * ss0), mp = (s_term.msz + 3) & ~3;
      // modes: 1 Tg global, 2 Tg in shared memory, 3 W in global, 4 W and the staged term
      // grid (two tensors of NQ vectors) in global
      const int64_t gst = w.smem == 4 ? 2 * ss0 * s_term.nq[L] : 0;
      const bool bad = w.smem >= 3 ? (mp + (2 + ny) * ss0 > p.smem_elems || 3 * tsz0 + gst > p.slab_per_cta)
                                   : (mp + need + (w.smem == 2 ? tsz0 : 0) > p.smem_elems ||
                                      (w.smem != 2 && tsz0 > p.slab_per_cta));
      if (bad) {
        if (threadIdx.x == 0) atomicExch(p.err, 1);
        continue;
      }
    }
    T* const mb = reinterpret_cast<T*>(smem_raw);
    fill_item_divs(s_div, s_term, w.vt);  // visible after the barriers of stage_matrices
    stage_matrices<T>(s_term, D, p.mats, mb, s_blocks);
    const TermDesc& Tm = s_term;
    const int Vt = w.vt;
    const int gL = Tm.nq[L], nL = Tm.nb[L];
    const int NQs = Tm.NQ / gL;
    const int64_t ss = (int64_t)NQs * Vt;  // one slab array
    const int64_t tsz = ss * nL;           // T and W
    T* sm = reinterpret_cast<T*>(smem_raw) + ((Tm.msz + 3) & ~3);
    // The partially transformed tensor Tg: after the phase buffers in shared memory
    // (smem == 2) or in the CTA's global buffer.  smem == 3 (terms whose W does not fit):
    // W and the ping-pong tensors of phases A and C also in the global buffer
    // [Tg | W (= A ping) | A and C pong], only the slab arrays in shared memory.  smem == 4
    // (FP32 type 10): as 3, followed by the staged term grid [Psi | DPsi].
    const bool wg = w.smem >= 3;
    T* const gbuf = p.slab + (int64_t)blockIdx.x * p.slab_per_cta;
    T* Tg = w.smem == 2 ? sm + max(2 * tsz, tsz + (2 + (p.keo_type == 10 ? L + (sizeof(T) == 4 ? 1 : 0) : 1)) * ss)
                        : gbuf;
    T* const wbuf = wg ? gbuf + tsz : sm;            // W, and the first ping-pong tensor
    T* const pong = wg ? gbuf + 2 * tsz : sm + tsz;  // second ping-pong tensor of phases A and C
    T* const slabs = wg ? sm : sm + tsz;             // Acc, P, Y
    const FastDiv& dvt = s_div.fv;

    // ---- A: gather + B->G over positions 0..L-1
    if (L == 0) {
      for (int64_t i = threadIdx.x; i < (int64_t)nL * Vt; i += blockDim.x) {
        const int v = (int)(i % Vt), k = (int)(i / Vt);
        const int pk = __ldg(p.map + Tm.off_nb + k);
        Tg[i] = pk >= 0 ? (T)__ldg(p.x + (int64_t)pk * p.ldx + w.v0 + v) : T(0);
      }
    } else {
      T* b0 = wbuf;
      T* b1 = pong;
      int nb_rest = Tm.NB / Tm.nb[0];
      T* cur = (L == 1) ? Tg : b0;
      gather_contract<T>(p.x + w.v0, p.ldx, p.map + Tm.off_nb, 0, cur, Tm.nb[0], Tm.nq[0], nb_rest, s_div.fv,
                         mb + Tm.m_d0b[0]);
      __syncthreads();
      int A = Tm.nq[0];
      for (int i = 1; i < L; ++i) {
        nb_rest /= Tm.nb[i];
        T* nxt = (i == L - 1) ? Tg : (cur == b0 ? b1 : b0);
        contract_x<T>(ts, cur, Vt, nxt, Vt, s_div.fq[i], Tm.nb[i], Tm.nq[i], nb_rest, s_div.fv, mb + Tm.m_d0b[i], T(1), false);
        __syncthreads();
        cur = nxt;
        A *= Tm.nq[i];
      }
    }
    __syncthreads();

    // ---- B: stream the grid slabs of position L
    T* W = wbuf;
    T* Acc = slabs;
    T* P = Acc + ss;
    T* Y = P + ss;
    const int ldx0 = (gL + 3) & ~3, ldo = (nL + 3) & ~3;
    const T* X0 = mb + Tm.m_d0b[L];
    const T* OUT = mb + Tm.m_bgw[L];
    const int nG = g_table_stride(Tm.Dp);  // G-table row of a point
    const bool staged = sizeof(T) == 4 && w.smem == 4 && p.keo_on && p.keo_type == 10;
    if (staged) {
      // grid-staged (FP32 type 10, buffers in global memory): the streamed position's
      // grid<-basis transform of psi and of d_L psi for all slabs at once (Psi, DPsi: the
      // term grid), each slab's kinetic and potential part in shared memory, written back
      // over its Psi and DPsi slab (Acc, Phi_L), then one basis<-grid contraction into W
      T* const Psi = gbuf + 3 * tsz;
      T* const DPsi = Psi + (int64_t)gL * ss;
      contract_x<T>(ts, Tg, Vt, Psi, Vt, s_div.fq[L], nL, gL, 1, s_div.fv, X0, T(1), false);
      contract_x<T>(ts, Tg, Vt, DPsi, Vt, s_div.fq[L], nL, gL, 1, s_div.fv, mb + Tm.m_x1L, T(1), false);
      const T mw = p.mu_dev ? (T)__ldg(p.mu_dev) : p.mw;
      const T vw = p.mugrid ? p.vw : T(1);
      const int s32 = (int)ss;
      T* P1 = Y + (int64_t)L * ss;
      for (int q = 0; q < gL; ++q) {
        __syncthreads();
        const T* Vq = p.vgrid + Tm.off_nq + (int64_t)q * NQs;
        const T* Mq = p.mugrid ? p.mugrid + Tm.off_nq + (int64_t)q * NQs : nullptr;
        T* ps = Psi + (int64_t)q * ss;
        T* ds = DPsi + (int64_t)q * ss;
        for (int a = threadIdx.x; a < s32; a += blockDim.x) {
          const T x = ps[a];
          const int pt = (int)dvt.div((uint32_t)a);
          T v = __ldg(Vq + pt);
          if (Mq) v = fma(mw, __ldg(Mq + pt), vw * v);
          P[a] = x;
          P1[a] = ds[a];
          Acc[a] = v * x;
        }
        __syncthreads();
        slab_keo10<T, GFLY>(p, Tm, s_div, mb, P, Y, P1, Acc, ss, Vt, q, NQs, nG, ts);
        for (int a = threadIdx.x; a < s32; a += blockDim.x) {
          ps[a] = Acc[a];
          ds[a] = P1[a];
        }
      }
      __syncthreads();
      contract_x<T>(ts, Psi, Vt, W, Vt, s_div.fq[L], gL, nL, 1, s_div.fv, OUT, T(1), false);
      __syncthreads();
      contract_x<T>(ts, DPsi, Vt, W, Vt, s_div.fq[L], gL, nL, 1, s_div.fv, mb + Tm.m_e1L, T(-0.5), true);
    } else {
      for (int64_t i = threadIdx.x; i < tsz; i += blockDim.x) W[i] = T(0);
    }
    for (int q = 0; q < (staged ? 0 : gL); ++q) {
      __syncthreads();
      if (sizeof(T) == 4 && p.keo_on && p.keo_type == 10) {
        // FP32: psi, d_L psi (kept in Y[L], later Phi_L) and Acc = V psi in one pass (FP64
        // keeps the two passes below, with fewer live registers)
        T* P1 = Y + (int64_t)L * ss;
        const T* Mq = p.mugrid ? p.mugrid + Tm.off_nq + (int64_t)q * NQs : nullptr;
        const T mw = p.mu_dev ? (T)__ldg(p.mu_dev) : p.mw;
        slab_extract_fused<T>(Tg, ss, nL, X0 + q, mb + Tm.m_x1L + q, ldx0, P, P1, Acc,
                              p.vgrid + Tm.off_nq + (int64_t)q * NQs, Mq, p.mugrid ? p.vw : T(1), mw, dvt);
        __syncthreads();
        slab_keo10<T, GFLY>(p, Tm, s_div, mb, P, Y, P1, Acc, ss, Vt, q, NQs, nG, ts);
        slab_accumulate<T>(W, ss, nL, OUT + (int64_t)ldo * q, Acc, T(1), mb + Tm.m_e1L + (int64_t)ldo * q, P1,
                           T(-0.5));
        continue;
      }
      slab_extract<T>(Tg, ss, nL, X0 + q, ldx0, P);
      __syncthreads();
      const T* Vq = p.vgrid + Tm.off_nq + (int64_t)q * NQs;
      if (p.mugrid) {
        const T* Mq = p.mugrid + Tm.off_nq + (int64_t)q * NQs;
        const T mw = p.mu_dev ? (T)__ldg(p.mu_dev) : p.mw;
        for (int64_t a = threadIdx.x; a < ss; a += blockDim.x) {
          const int pt = (int)dvt.div((uint32_t)a);
          Acc[a] = fma(mw, __ldg(Mq + pt), p.vw * __ldg(Vq + pt)) * P[a];
        }
      } else {
        for (int64_t a = threadIdx.x; a < ss; a += blockDim.x) Acc[a] = __ldg(Vq + dvt.div((uint32_t)a)) * P[a];
      }
      if (!p.keo_on) {
        __syncthreads();
        slab_accumulate<T>(W, ss, nL, OUT + (int64_t)ldo * q, Acc, T(1), nullptr, nullptr, T(0));
      } else if (p.keo_type == 10) {
        int A = 1, Bq = NQs;
        for (int j = 0; j < L; ++j) {  // Y[j] = d1_j P
          Bq /= Tm.nq[j];
          contract_x<T>(ts, P, Vt, Y + j * ss, Vt, s_div.fq[j], Tm.nq[j], Tm.nq[j], Bq, s_div.fv, mb + Tm.m_d1[j], T(1), false);
          A *= Tm.nq[j];
        }
        __syncthreads();
        slab_extract<T>(Tg, ss, nL, mb + Tm.m_x1L + q, ldx0, P);  // P <- d_L psi on the slab
        __syncthreads();
        // Phi_i = sum_j G_ij(Q) y_j, in place (Y[i] for i < L, P for i = L)
        if (D <= 4) slab_pointwise_G<T, 4, GFLY>(p, Tm, Y, P, ss, Vt, q, NQs, nG);
        else if (D <= 6) slab_pointwise_G<T, 6, GFLY>(p, Tm, Y, P, ss, Vt, q, NQs, nG);
        else if (D <= 8) slab_pointwise_G<T, 8, GFLY>(p, Tm, Y, P, ss, Vt, q, NQs, nG);
        else pointwise_G_wide<T, GFLY>(p, Tm, Y, ss, P, Vt, NQs, (int64_t)q * NQs, nullptr);
        __syncthreads();
        A = 1;
        Bq = NQs;
        for (int i = 0; i < L; ++i) {  // Acc += -1/2 d1_i Phi_i
          Bq /= Tm.nq[i];
          contract_x<T>(ts, Y + i * ss, Vt, Acc, Vt, s_div.fq[i], Tm.nq[i], Tm.nq[i], Bq, s_div.fv, mb + Tm.m_d1[i], T(-0.5), true);
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
          const T f = (T)(-0.5 * __ldg(p.G0 + Tm.g0off + Tm.perm[i] + Tm.Dp * Tm.perm[i]));
          if (f != T(0))
            contract_x<T>(ts, P, Vt, Acc, Vt, s_div.fq[i], Tm.nq[i], Tm.nq[i], Bq, s_div.fv, mb + Tm.m_d2[i], f, true);
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
              const T f = (T)(-__ldg(p.G0 + Tm.g0off + Tm.perm[i] + Tm.Dp * Tm.perm[j]));
              if (f != T(0)) {
                contract_x<T>(ts, P, Vt, Y, Vt, s_div.fq[i], Tm.nq[i], Tm.nq[i], Bi, s_div.fv, mb + Tm.m_d1[i], T(1), false);
                __syncthreads();
                contract_x<T>(ts, Y, Vt, Acc, Vt, s_div.fq[j], Tm.nq[j], Tm.nq[j], Bj, s_div.fv, mb + Tm.m_d1[j], f, true);
                __syncthreads();
              }
              Aj *= Tm.nq[j];
            }
            Ai *= Tm.nq[i];
          }
        }
        const T fLL = (T)(-0.5 * __ldg(p.G0 + Tm.g0off + Tm.perm[L] + Tm.Dp * Tm.perm[L]));
        slab_accumulate<T>(W, ss, nL, OUT + (int64_t)ldo * q, Acc, T(1), mb + Tm.m_e2L + (int64_t)ldo * q, P,
                           fLL);
        if (p.has_offdiag) {  // F2_iL d1_i d_L: d_L through (bgw.d1)_L on the way back
          int Ai = 1;
          for (int i = 0; i < L; ++i) {
            const int Bi = NQs / (Ai * Tm.nq[i]);
            const T f = (T)(-__ldg(p.G0 + Tm.g0off + Tm.perm[i] + Tm.Dp * Tm.perm[L]));
            if (f != T(0)) {
              __syncthreads();
              contract_x<T>(ts, P, Vt, Y, Vt, s_div.fq[i], Tm.nq[i], Tm.nq[i], Bi, s_div.fv, mb + Tm.m_d1[i], T(1), false);
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
      T* b1 = pong;
      T* cur = b0;
      int A = 1, Bq = NQs;
      for (int i = 0; i < L; ++i) {
        Bq /= Tm.nq[i];
        const int Bt = Bq * nL;
        if (i == L - 1) {
          contract_x<T>(ts, cur, Vt, dst, p.ldh, s_div.fb[i], Tm.nq[i], Tm.nb[i], Bt, s_div.fv, mb + Tm.m_bgw[i], T(1), false);
        } else {
          T* nxt = (cur == b0) ? b1 : b0;
          contract_x<T>(ts, cur, Vt, nxt, Vt, s_div.fb[i], Tm.nq[i], Tm.nb[i], Bt, s_div.fv, mb + Tm.m_bgw[i], T(1), false);
          cur = nxt;
        }
        __syncthreads();
        A *= Tm.nb[i];
      }
    }
  }
  if constexpr (TC) tc::tc_teardown(tcs);
}


// launchers, instantiated in evr_kern_*.cu
template <typename T, bool GFLY>
cudaError_t launch_items_kernel(int grid, size_t smem, cudaStream_t s, const ItemParams<T>& p,
                                int threads = kThreads);
// slab kernel: TC = true only for float (the tensor-core instantiation, its own units)
template <typename T, bool GFLY, bool TC>
cudaError_t launch_slab_kernel(int grid, size_t smem, cudaStream_t s, const ItemParams<T>& p);
template <typename T, bool GFLY>
cudaError_t set_items_kernel_smem(int bytes);
template <typename T, bool GFLY, bool TC>
cudaError_t set_slab_kernel_smem(int bytes);
// static shared memory of the kernels (the dynamic budget is what the SM has left)
template <typename T, bool GFLY, bool TC>
cudaError_t slab_kernel_static_smem(int* bytes);
template <typename T, bool GFLY>
cudaError_t items_kernel_static_smem(int* bytes);
// resident CTAs per SM of the general kernel at a dynamic shared-memory size
template <typename T, bool GFLY>
cudaError_t occupancy_items_kernel(int* per_sm, int smem_bytes);
template <typename T, bool GFLY>
cudaError_t set_term_kernel_smem(int items_bytes, int slab_bytes) {
  cudaError_t e = set_items_kernel_smem<T, GFLY>(items_bytes);
  if (e == cudaSuccess) e = set_slab_kernel_smem<T, GFLY, false>(slab_bytes);
  if constexpr (sizeof(T) == 4) {
    if (e == cudaSuccess) e = set_slab_kernel_smem<T, GFLY, true>(slab_bytes);
  }
  return e;
}

}  // namespace kern
}  // namespace evr
