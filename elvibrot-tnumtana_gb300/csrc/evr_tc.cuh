// evr_tc.cuh -- mode contractions on the 5th-generation tensor cores (tcgen05), FP32 data
// with three TF32 products (split operands, FP32 accumulation in tensor memory).
//
// A mode contraction of the term pipeline,
//     out(a, m, b, v) = alpha * sum_k mat[m + ldm*k] * in(a, k, b, v)   (+ out when acc)
// (BDP_TO_GDP_OF_SmolyakRep / GDP_TO_BDP_OF_SmolyakRep / DerivOp_TO_RDP_OF_SmolaykRep,
// Source_ElVibRot/sub_Basis/sub_Basis_SG4/sub_module_basis_BtoG_GtoB_SG4.f90:2385-2581,
// 2690-2795) is a product of a (fibres x K) matrix by the (K x M) transposed 1-D matrix,
// fibres f = v + Vt*(a + A*b).  Here 128 fibres are the M side of one MMA (a row per
// TMEM lane), the 1-D matrix is the N side (M padded to 16 or 32 columns) and the
// contraction runs in chunks of 8 (K padded to 8, 16 or 24):
//   * the CTA stages the fibre tile into shared memory in the canonical K-major layout
//     without swizzle (8-row x 16-byte core matrices; LBO = 128 B between core matrices
//     along K, SBO = 32*Kp B between 8-row groups), split x = hi + lo with hi the nearest
//     TF32 value and lo the nearest TF32 value of x - hi, both written by the staging threads;
//   * one thread issues hi*Bhi + lo*Bhi + hi*Blo (3*Kp/8 MMAs, kind::tf32, M=128) into a
//     TMEM accumulator and commits them to an mbarrier;
//   * every warp reads its lane quarter of the accumulator (tcgen05.ld 32x32b) and writes
//     its fibres' outputs (coalesced: consecutive lanes are consecutive fibres).
// The dropped lo*lo term and the rounding of lo leave a relative error near 2^-23 per
// product, FP32 level.  Waits on the mbarrier are bounded: on expiry the CTA gives the
// pending MMAs one more bounded wait, records an error code, leaves the contraction and
// runs its later contractions on the CUDA cores; it frees its accumulator at its end.
#pragma once
#include <cstdint>

namespace evr {
namespace tc {

constexpr int kRows = 128;     // fibres per MMA tile
constexpr int kMaxKp = 24;     // padded contraction length (multiple of 8)
constexpr int kMaxNp = 32;     // padded output length (multiple of 16)
constexpr int kTmemCols = 32;  // one accumulator of kMaxNp FP32 columns
constexpr unsigned kWaitLimit = 1u << 22;  // try_wait rounds before a wait is declared lost

// Shared-memory block of the tensor-core contractions (16-byte aligned operand tiles).
struct alignas(16) TcSmem {
  float a_hi[kRows * kMaxKp];
  float a_lo[kRows * kMaxKp];
  float b_hi[kMaxNp * kMaxKp];
  float b_lo[kMaxNp * kMaxKp];
  unsigned long long mbar;
  uint32_t tmem;     // TMEM address of the accumulator
  int failed;        // a bounded wait ran out
};

// Per-thread state of the contractions of one CTA (all threads run every contraction, so
// every thread tracks the same mbarrier phase).
struct TcState {
  TcSmem* sm;
  uint32_t phase;
  int* err;          // global error flag (value 2: a tensor-core wait ran out)
  int min_km;        // contractions with K*M below this stay on the CUDA cores (caller's choice)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// canonical K-major, no swizzle: element (r, k) of a tile with Kp columns
__device__ __forceinline__ int kmajor_index(int r, int k, int Kp) {
  return ((r >> 3) * (Kp >> 2) + (k >> 2)) * 32 + (r & 7) * 4 + (k & 3);
}

// shared-memory matrix descriptor: start address, LBO (K direction), SBO (8-row groups),
// descriptor version 1 (bits 46-47), no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// instruction descriptor of kind::tf32: D FP32, A and B TF32, both K-major, N and M
__device__ __forceinline__ uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// x rounded to the nearest TF32 value (10-bit mantissa), low 13 bits cleared
__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t u;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
  return __uint_as_float(u & 0xFFFFE000u);
}
// x = hi + lo with hi, lo TF32 values: |x - hi - lo| <= 2^-24 |x| (each rounded to nearest),
// so that the MMA reads both exactly, whatever it does with low mantissa bits
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
  hi = tf32_rna(x);
  lo = tf32_rna(x - hi);
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar_addr) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_addr)
               : "memory");
}

// bounded wait for the mbarrier phase with parity `parity`; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint32_t mbar_addr, uint32_t parity) {
  for (unsigned i = 0; i < kWaitLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar_addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 8 consecutive FP32 columns of the warp's lane quarter
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n\t"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

// CTA prologue: mbarrier and TMEM accumulator (warp 0 allocates).  Ends with a barrier.
__device__ __forceinline__ void tc_setup(TcState& st, TcSmem* sm, int* err) {
  st.sm = sm;
  st.phase = 0;
  st.err = err;
  st.min_km = 0;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&sm->mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sm->failed = 0;
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm->tmem)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
}

// CTA epilogue: frees the accumulator (warp 0).  Call after a barrier that every thread
// reaches once its last contraction is done.
__device__ __forceinline__ void tc_teardown(TcState& st) {
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(st.sm->tmem), "r"(kTmemCols)
                 : "memory");
  }
}

// out(a, m, b, v) = alpha * sum_k mat[m + ldm*k] * in(a, k, b, v) (+ out if acc); element
// (a, k, b, v) at ((a + A*(k + K*b))*ld + v).  A CTA-wide call (all threads, blockDim a
// multiple of 128), K <= kMaxKp, M <= kMaxNp.  FastDiv: the divisor type of the caller.
// Software pipeline with one barrier per 128-fibre tile: the loads of tile i+1 are issued
// into registers right after the MMAs of tile i, so they are in flight while the MMAs run
// and while tile i's accumulator is read back; then they are split into the (free) operand
// tile and the barrier hands it to the MMA-issuing thread.
template <typename Div>
__device__ __noinline__ void contract_tc(TcState& st, const float* __restrict__ in, int64_t ldi, float* __restrict__ out,
                            int64_t ldo, const Div& da, int K, int M, int B, const Div& dvt,
                            const float* __restrict__ mat, float alpha, bool acc) {
  TcSmem* sm = st.sm;
  const int A = (int)da.d, Vt = (int)dvt.d;
  const int Kp = (K + 7) & ~7;
  const int Np = M <= 16 ? 16 : 32;
  const int ldm = (M + 3) & ~3;
  const int nthr = blockDim.x;
  const int nfib = A * B * Vt;
  const int64_t istr = (int64_t)A * ldi, ostr = (int64_t)A * ldo;
  const uint32_t mbar = smem_u32(&sm->mbar);

  // the 1-D matrix as the N x Kp operand: B[n][k] = mat[n + ldm*k], split
  for (int i = threadIdx.x; i < Np * Kp; i += nthr) {
    const int n = i / Kp, k = i - n * Kp;
    const float x = (n < M && k < K) ? mat[n + ldm * k] : 0.0f;
    float h, l;
    tf32_split(x, h, l);
    const int o = kmajor_index(n, k, Kp);
    sm->b_hi[o] = h;
    sm->b_lo[o] = l;
  }
  const uint32_t idesc = idesc_tf32(kRows, Np);
  const uint32_t sbo_a = 32u * Kp, sbo_b = 32u * Kp;
  const uint32_t a_hi = smem_u32(sm->a_hi), a_lo = smem_u32(sm->a_lo);
  const uint32_t b_hi = smem_u32(sm->b_hi), b_lo = smem_u32(sm->b_lo);
  const int kgroups = Kp >> 2;
  const int ntask = kRows * kgroups;  // staging tasks of a tile: (fibre row, group of 4 k)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int quarter = warp & 3, chunk = warp >> 2, nchunk = nthr >> 7;

  // a thread's staging tasks of one tile: threadIdx.x + t*nthr (at most kTasks with >= 128 threads)
  constexpr int kTasks = kMaxKp / 4;
  float x[kTasks][4];
  auto load_tile = [&](int f0) {
#pragma unroll
    for (int t = 0; t < kTasks; ++t) {
      x[t][0] = x[t][1] = x[t][2] = x[t][3] = 0.f;
      const int i = threadIdx.x + t * nthr;
      const int f = f0 + (i & (kRows - 1)), c = i >> 7;
      if (i < ntask && f < nfib) {
        const int t1 = (int)dvt.div((uint32_t)f);
        const int v = f - t1 * Vt;
        const int b = (int)da.div((uint32_t)t1);
        const int a = t1 - b * A;
        const float* ip = in + (int64_t)(a + (int64_t)A * K * b) * ldi + v;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (4 * c + j < K) x[t][j] = ip[(4 * c + j) * istr];
      }
    }
  };
  auto store_tile = [&]() {
#pragma unroll
    for (int t = 0; t < kTasks; ++t) {
      const int i = threadIdx.x + t * nthr;
      if (i < ntask) {
        const int r = i & (kRows - 1), c = i >> 7;
        float4 h, l;
        tf32_split(x[t][0], h.x, l.x);
        tf32_split(x[t][1], h.y, l.y);
        tf32_split(x[t][2], h.z, l.z);
        tf32_split(x[t][3], h.w, l.w);
        const int o = ((r >> 3) * kgroups + c) * 32 + (r & 7) * 4;
        *reinterpret_cast<float4*>(sm->a_hi + o) = h;
        *reinterpret_cast<float4*>(sm->a_lo + o) = l;
      }
    }
  };

  bool ok = true;
  load_tile(0);
  for (int f0 = 0; f0 < nfib; f0 += kRows) {
    // the operand tile is free: the previous tile's MMAs have completed (waited below)
    store_tile();
    fence_async_smem();
    fence_before_sync();
    // one barrier per tile; it also carries the outcome of the previous tile's wait (a lost
    // wait on any thread ends the contraction for all)
    const bool lost = __syncthreads_or(!ok) != 0;
    fence_after_sync();
    if (lost) break;
    // ---- one thread issues hi*Bhi + lo*Bhi + hi*Blo over the K chunks
    if (threadIdx.x == 0) {
      uint32_t accum = 0;
      for (int kc = 0; kc < Kp; kc += 8) {
        const uint32_t off = (uint32_t)kc * 32u;  // two core matrices of 128 B per chunk of 8
        mma_tf32(sm->tmem, smem_desc(a_hi + off, 128, sbo_a), smem_desc(b_hi + off, 128, sbo_b), idesc, accum);
        accum = 1;
        mma_tf32(sm->tmem, smem_desc(a_lo + off, 128, sbo_a), smem_desc(b_hi + off, 128, sbo_b), idesc, 1);
        mma_tf32(sm->tmem, smem_desc(a_hi + off, 128, sbo_a), smem_desc(b_lo + off, 128, sbo_b), idesc, 1);
      }
      mma_commit(mbar);
    }
    // ---- the next tile's loads go out while the MMAs run
    if (f0 + kRows < nfib) load_tile(f0 + kRows);
    ok = mbar_wait(mbar, st.phase);
    st.phase ^= 1u;
    fence_after_sync();
    // ---- epilogue: warp (quarter, chunk) reads lanes 32*quarter.., columns 8*chunk..
    if (ok) {
      for (int cc = chunk; cc * 8 < Np; cc += nchunk) {
        float vals[8];
        tmem_ld8(sm->tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(8 * cc), vals);
        const int f = f0 + 32 * quarter + lane;
        if (f < nfib) {
          const int t1 = (int)dvt.div((uint32_t)f);
          const int v = f - t1 * Vt;
          const int b = (int)da.div((uint32_t)t1);
          const int a = t1 - b * A;
          float* op = out + (int64_t)(a + (int64_t)A * M * b) * ldo + v;
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int m = 8 * cc + j;
            if (m < M) {
              float val = alpha * vals[j];
              if (acc) val += op[m * ostr];
              op[m * ostr] = val;
            }
          }
        }
      }
    }
    // the accumulator reads are complete (wait::ld) before the next barrier releases the
    // next tile's MMAs
    fence_before_sync();
  }
  // the last tile's outcome; the caller's next contraction may overwrite the operands
  const bool lost = __syncthreads_or(!ok) != 0;
  fence_after_sync();
  if (lost) {
    // give the MMAs whose commit was not seen one more bounded wait (the phase before the
    // flip), so that the accumulator is normally idle when the CTA frees it at its end;
    // later contractions of the CTA run on the CUDA cores
    (void)mbar_wait(mbar, st.phase ^ 1u);
    if (threadIdx.x == 0) {
      sm->failed = 1;
      atomicExch(st.err, 2);
    }
  }
}

}  // namespace tc
}  // namespace evr
