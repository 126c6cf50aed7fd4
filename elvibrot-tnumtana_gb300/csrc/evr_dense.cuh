// evr_dense.cuh -- the dense FP64 algebra of the block Davidson on the device, hand-written
// and deterministic: projections (Gram matrices) and linear combinations of vector blocks
// (Overlap_psi1_psi2 / sub_LCpsi_TO_psi, Source_ElVibRot/sub_WP/sub_module_psi_Op.f90:146-466,
// as the Davidson uses them in sub_MakeH_Davidson and the Ritz/residual steps,
// sub_propagation/sub_module_Davidson.f90:1028-1288), and the eigen-decomposition of the
// projected matrix (the reference's dsyev through diagonalization type 3, :345) by a
// parallel cyclic Jacobi iteration.
//
// Vector blocks are interleaved: row r of an N x ld block holds component r of every
// vector (X[r*ld + i]).  Sums over the N rows run in fixed chunks whose partial results are
// added in chunk order, so every product is reproducible run to run.
#pragma once
#include <cooperative_groups.h>

#include <cstdint>

namespace evr {
namespace dense {

constexpr int kTile = 64;        // Gram output tile (both sides)
constexpr int kStage = 32;       // rows staged in shared memory per step
constexpr int kMaxEig = 512;     // largest projected matrix of the Jacobi kernel

// partial Gram of one chunk of rows: part[chunk] (na x nb, column-major) =
// sum_{r in chunk} A[r, i] B[r, j] over the 64 x 64 output tile of blockIdx.y; a thread owns
// a 4 x 4 block of the tile
static __global__ void __launch_bounds__(256) gram_part_kernel(const double* __restrict__ A, int lda,
                                                        const double* __restrict__ B, int ldb, int na, int nb,
                                                        int64_t N, int64_t rows_per_chunk, double* __restrict__ part) {
  __shared__ double sA[kStage][kTile + 2];
  __shared__ double sB[kStage][kTile + 2];
  const int tilesI = (na + kTile - 1) / kTile;
  const int i0 = (blockIdx.y % tilesI) * kTile, j0 = (blockIdx.y / tilesI) * kTile;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  const int64_t rb = blockIdx.x * rows_per_chunk;
  const int64_t re = rb + rows_per_chunk < N ? rb + rows_per_chunk : N;
  for (int64_t r0 = rb; r0 < re; r0 += kStage) {
    const int nr = (int)(re - r0 < kStage ? re - r0 : kStage);
    __syncthreads();
    for (int e = threadIdx.x; e < kStage * kTile; e += blockDim.x) {
      const int r = e / kTile, i = e % kTile;
      sA[r][i] = (r < nr && i0 + i < na) ? A[(r0 + r) * lda + i0 + i] : 0.0;
      sB[r][i] = (r < nr && j0 + i < nb) ? B[(r0 + r) * ldb + j0 + i] : 0.0;
    }
    __syncthreads();
    for (int r = 0; r < nr; ++r) {
      double x[4], y[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        x[a] = sA[r][4 * tx + a];
        y[a] = sB[r][4 * ty + a];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fma(x[a], y[b], acc[a][b]);
    }
  }
  double* out = part + (int64_t)blockIdx.x * na * nb;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int i = i0 + 4 * tx + a, j = j0 + 4 * ty + b;
      if (i < na && j < nb) out[i + (int64_t)na * j] = acc[a][b];
    }
}

// C (ld ldc) = sum over the chunks of the partial Grams, in chunk order (+ beta C)
static __global__ void gram_reduce_kernel(const double* __restrict__ part, int nchunk, int na, int nb,
                                   double* __restrict__ C, int ldc, double beta) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < na * nb; e += gridDim.x * blockDim.x) {
    const int i = e % na, j = e / na;
    double s = 0.0;
    for (int c = 0; c < nchunk; ++c) s += part[(int64_t)c * na * nb + e];
    double* d = C + i + (int64_t)ldc * j;
    *d = beta == 0.0 ? s : s + beta * *d;
  }
}

// Y[r, j] = alpha sum_{i < n} X[r, i] Mat[i + ldm j] + beta Y[r, j]  (j < k): 64 rows x 32
// columns per CTA, the contraction in steps of 32 through shared memory; a thread forms
// 2 rows x 4 columns
static __global__ void __launch_bounds__(256) combine_kernel(const double* __restrict__ X, int ldx, int n,
                                                      const double* __restrict__ Mat, int ldm, int k,
                                                      double* __restrict__ Y, int ldy, double alpha, double beta,
                                                      int64_t N) {
  __shared__ double sX[64][33];
  __shared__ double sM[32][33];
  const int64_t row0 = (int64_t)blockIdx.x * 64;
  const int j0 = blockIdx.y * 32;
  const int tr = threadIdx.x / 8, tc = threadIdx.x % 8;
  double acc[2][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int i0 = 0; i0 < n; i0 += 32) {
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * 32; e += blockDim.x) {
      const int r = e / 32, i = e % 32;
      sX[r][i] = (row0 + r < N && i0 + i < n) ? X[(row0 + r) * ldx + i0 + i] : 0.0;
    }
    for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
      const int i = e % 32, j = e / 32;
      sM[i][j] = (i0 + i < n && j0 + j < k) ? Mat[(i0 + i) + (int64_t)ldm * (j0 + j)] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int i = 0; i < 32; ++i) {
      const double x0 = sX[2 * tr][i], x1 = sX[2 * tr + 1][i];
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const double m = sM[i][4 * tc + b];
        acc[0][b] = fma(x0, m, acc[0][b]);
        acc[1][b] = fma(x1, m, acc[1][b]);
      }
    }
  }
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const int64_t r = row0 + 2 * tr + a;
    if (r >= N) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = j0 + 4 * tc + b;
      if (j < k) {
        double* y = Y + r * ldy + j;
        *y = beta == 0.0 ? alpha * acc[a][b] : alpha * acc[a][b] + beta * *y;
      }
    }
  }
}

// per-chunk sums of squares of the k columns of an interleaved block: part[chunk*k + c];
// a warp holds 32 consecutive columns, the 8 warps of a CTA take interleaved rows and are
// summed in warp order
static __global__ void colnorm_part_kernel(const double* __restrict__ X, int ldx, int k, int64_t N, int64_t rows_per_chunk,
                                    double* __restrict__ part) {
  __shared__ double red[8][33];
  const int c = blockIdx.y * 32 + threadIdx.x;
  const int64_t rb = blockIdx.x * rows_per_chunk;
  const int64_t re = rb + rows_per_chunk < N ? rb + rows_per_chunk : N;
  double s = 0.0;
  if (c < k)
    for (int64_t r = rb + threadIdx.y; r < re; r += 8) {
      const double v = X[r * ldx + c];
      s = fma(v, v, s);
    }
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && c < k) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < 8; ++w) t += red[w][threadIdx.x];
    part[(int64_t)blockIdx.x * k + c] = t;
  }
}

// Hs(n0 + j, i) = Hs(i, n0 + j) for i < n0, j < n1 - n0: the new columns of the projected
// matrix mirrored into its new rows
static __global__ void mirror_kernel(double* __restrict__ Hs, int ld, int n0, int n1) {
  const int nn = n1 - n0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n0 * nn; e += gridDim.x * blockDim.x) {
    const int i = e % n0, j = e / n0;
    Hs[(n0 + j) + (int64_t)ld * i] = Hs[i + (int64_t)ld * (n0 + j)];
  }
}

// Eigen-decomposition of the symmetric part of an n x n matrix (n <= kMaxEig) by cyclic
// Jacobi with the round-robin pair ordering, spread over a cooperative grid: each round
// rotates np/2 disjoint pairs (angles from the matrix before the round); every CTA computes
// all pairs' angles from the same values, so all CTAs take the same decisions without
// communicating, and the rows, then the columns (of A and of the eigenvector matrix) are
// updated by the whole grid between grid barriers.  A pair is rotated unless
// |a_pq| <= tol sqrt(|a_pp a_qq|); the iteration stops after a sweep without rotation or
// after max_sweeps.  Work arrays wa, wv: np x np each; word: np ints.  Output: eigenvalues
// ascending in W, eigenvectors as the columns of V (ld ldv).  The working matrices are read
// and written with L2-coherent accesses (__ldcg / __stcg).
static __global__ void __launch_bounds__(256) jacobi_coop_kernel(const double* __restrict__ A, int lda, int n,
                                                          double* __restrict__ W, double* __restrict__ V, int ldv,
                                                          double* __restrict__ wa, double* __restrict__ wv,
                                                          int* __restrict__ word, int max_sweeps, double tol) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  __shared__ double c_[kMaxEig / 2], s_[kMaxEig / 2];
  __shared__ int p_[kMaxEig / 2], q_[kMaxEig / 2];
  __shared__ int s_rot;
  const int np = (n + 1) & ~1, npair = np / 2;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nthr = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = tid; e < (int64_t)np * np; e += nthr) {
    const int i = (int)(e % np), j = (int)(e / np);
    __stcg(wa + e, (i < n && j < n) ? 0.5 * (A[i + (int64_t)lda * j] + A[j + (int64_t)lda * i]) : 0.0);
    __stcg(wv + e, i == j ? 1.0 : 0.0);
  }
  grid.sync();
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    bool rotated = false;
    for (int r = 0; r < np - 1; ++r) {
      if (threadIdx.x == 0) s_rot = 0;
      __syncthreads();
      for (int k = threadIdx.x; k < npair; k += blockDim.x) {
        const int pa = k == 0 ? 0 : ((k - 1 + r) % (np - 1)) + 1;
        const int qa = ((np - 1 - k - 1 + r) % (np - 1)) + 1;
        const int p = pa < qa ? pa : qa, q = pa < qa ? qa : pa;
        const double app = __ldcg(wa + p + (int64_t)np * p), aqq = __ldcg(wa + q + (int64_t)np * q);
        const double apq = __ldcg(wa + p + (int64_t)np * q);
        double c = 1.0, s = 0.0;
        if (fabs(apq) > 1e-300 && fabs(apq) > tol * sqrt(fabs(app * aqq))) {
          s_rot = 1;
          const double tau = (aqq - app) / (2.0 * apq);
          const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
          c = 1.0 / sqrt(1.0 + t * t);
          s = t * c;
        }
        c_[k] = c; s_[k] = s; p_[k] = p; q_[k] = q;
      }
      __syncthreads();
      rotated |= s_rot != 0;
      // rows p, q: a_pj <- c a_pj - s a_qj, a_qj <- s a_pj + c a_qj
      for (int64_t e = tid; e < (int64_t)npair * np; e += nthr) {
        const int k = (int)(e / np), j = (int)(e % np);
        const double c = c_[k], s = s_[k];
        if (s == 0.0) continue;
        double* xp = wa + p_[k] + (int64_t)np * j;
        double* xq = wa + q_[k] + (int64_t)np * j;
        const double x = __ldcg(xp), y = __ldcg(xq);
        __stcg(xp, c * x - s * y);
        __stcg(xq, s * x + c * y);
      }
      grid.sync();
      // columns p, q of A and of the eigenvectors
      for (int64_t e = tid; e < (int64_t)npair * np; e += nthr) {
        const int k = (int)(e / np), i = (int)(e % np);
        const double c = c_[k], s = s_[k];
        if (s == 0.0) continue;
        double* xp = wa + i + (int64_t)np * p_[k];
        double* xq = wa + i + (int64_t)np * q_[k];
        const double x = __ldcg(xp), y = __ldcg(xq);
        __stcg(xp, c * x - s * y);
        __stcg(xq, s * x + c * y);
        double* vp = wv + i + (int64_t)np * p_[k];
        double* vq = wv + i + (int64_t)np * q_[k];
        const double vx = __ldcg(vp), vy = __ldcg(vq);
        __stcg(vp, c * vx - s * vy);
        __stcg(vq, s * vx + c * vy);
      }
      grid.sync();
    }
    if (!rotated) break;
  }
  // ascending order of the n eigenvalues (a padding index, if any, is np - 1 = n and stays
  // decoupled)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) word[i] = i;
    for (int i = 1; i < n; ++i) {
      const int t = word[i];
      const double x = __ldcg(wa + t + (int64_t)np * t);
      int j = i - 1;
      while (j >= 0 && __ldcg(wa + word[j] + (int64_t)np * word[j]) > x) {
        word[j + 1] = word[j];
        --j;
      }
      word[j + 1] = t;
    }
  }
  grid.sync();
  for (int64_t e = tid; e < (int64_t)n * n; e += nthr) {
    const int i = (int)(e % n), j = (int)(e / n);
    const int oj = __ldcg(word + j);
    V[i + (int64_t)ldv * j] = __ldcg(wv + i + (int64_t)np * oj);
    if (i == 0) W[j] = __ldcg(wa + oj + (int64_t)np * oj);
  }
}

}  // namespace dense
}  // namespace evr
