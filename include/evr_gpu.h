/*
 * evr_gpu.h -- C ABI of the GB300 (sm_103a) H.psi library for ElVibRot-TnumTana.
 *
 * The library replaces the reference's OpPsi hot path and the loops that drive it.
 * Every entry point returns an int status (EVR_OK = 0) and never stops the process;
 * the message of the last failure is available from evr_last_error().
 * No entry point takes C++ or torch types: plain pointers, sizes and flags only, so
 * a Fortran ISO_C_BINDING interface, ctypes or cgo can bind it directly.
 *
 * Vector layouts
 *   "basis column-major" (EVR_LAYOUT_COLMAJOR): nvec columns, each a packed basis
 *       vector of length N = Np*nb0 (the reference's RvecB, electronic index slowest:
 *       element (ib0, iB) at ib0*Np + iB), column stride ld >= N.  This is what the
 *       Fortran host passes (TabPsi(i)%RvecB).
 *   "interleaved" (EVR_LAYOUT_INTERLEAVED): element (k, v) at k*ld + v with ld >= nvec;
 *       the library's native device layout (vectors fastest).
 */
#ifndef EVR_GPU_H
#define EVR_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define EVR_OK          0
#define EVR_EINVAL      22   /* bad argument, shape or table entry            */
#define EVR_ENOMEM      12   /* device or host allocation failed              */
#define EVR_ETIMEDOUT  110   /* a bounded device wait expired                  */
#define EVR_EDEVICE    1001  /* CUDA runtime / library error                   */
#define EVR_ENOCONV    1002  /* iterative solver did not converge              */

/* basis kinds */
#define EVR_BASIS_SG4  0     /* Smolyak SparseGrid_type=4                       */
#define EVR_BASIS_DP   1     /* direct product                                  */

/* precisions of the basis<->grid contractions */
#define EVR_PREC_FP64  0     /* plain form: everything in FP64                  */
#define EVR_PREC_FP32  1     /* contractions and grid terms in FP32             */

/* vector layouts */
#define EVR_LAYOUT_COLMAJOR    0
#define EVR_LAYOUT_INTERLEAVED 1

typedef struct evr_ctx evr_ctx;

/*
 * Problem description: the basis tables the reference builds in
 *   construct_primitive_basis (Source_ElVibRot/sub_Basis/sub_module_basis.f90:391-782),
 *   RecSparseGrid_ForDP_type4 (sub_Basis/sub_quadra_SparseBasis.f90:924-1435) and
 *   Set_tables_FOR_SmolyakRepBasis_TO_tabPackedBasis
 *   (sub_Basis/sub_Basis_SG4/sub_module_basis_BtoG_GtoB_SG4.f90:625-949),
 * and the operator of sub_TabOpPsi_OF_ONEDP_FOR_SGtype4
 *   (Source_ElVibRot/sub_Operator/sub_OpPsi_SG4.f90:1354-1668).
 * The library builds all tables itself from these few numbers.
 */
/* A primitive basis of one (mode, level) given as tables on its grid, as the reference holds
 * them after construct_primitive_basis and sub_scale_basis
 * (Source_ElVibRot/sub_Basis/sub_module_basis.f90:391-782, 1540-1638): any primitive
 * basis and any grid (for instance non-HO bases, or the Nested=1 Hermite grids of
 * grid_HermiteNested1, :734-822).  x, w: nq grid points and weights (wrho); d0b, d1b, d2b:
 * the basis functions and their first and second derivatives on the grid, nq x nb,
 * column-major.  The library forms d0b^T w and the grid derivatives d1b pinv(d0b),
 * d2b pinv(d0b) (sub_dnGB_TO_dnGG, :2195-2460) itself. */
typedef struct evr_basis1d {
  int nq, nb;
  const double *x, *w;
  const double *d0b, *d1b, *d2b;
} evr_basis1d;

typedef struct evr_problem_desc {
  int kind;              /* EVR_BASIS_SG4 or EVR_BASIS_DP                          */
  int D;                 /* number of modes, 1..24                                  */
  int nb0;               /* electronic states (nb_elec), >= 1                       */
  int LG, LB;            /* SG4: L_SparseGrid, L_SparseBasis (LB <= LG)             */
  const int *Aq, *Bq;    /* SG4: nq(l) = Aq[i] + Bq[i]*l   (L_TO_nq_A/B)            */
  const int *Ab, *Bb;    /* SG4: nb(l) = Ab[i] + Bb[i]*l   (L_TO_nb_A/B)            */
  const int *nq_dp;      /* DP: grid points per mode                                */
  const int *nb_dp;      /* DP: basis functions per mode                            */
  const double *scaleQ;  /* per mode (sub_scale_basis), NULL = 1                    */
  const double *Q0;      /* per mode, NULL = 0                                      */
  /* potential: V_{ab}(Q) += coef[m] * prod_{k<4, idx>=0} Q[idx[4m+k]] for (a,b) = elec[2m..] */
  int n_mono;
  const double *mono_coef;
  const int *mono_idx;   /* n_mono*4, -1 = unused                                   */
  const int *mono_elec;  /* n_mono*2 or NULL (all on (0,0))                          */
  /* KEO: keo_type 10: -1/2 sum_ij d_i G_ij(Q) d_j, G = G0 + sum_k g[i+D*(j+D*k)] Q_k;
   *      keo_type 1 : sum_ij F2_ij d_i d_j with F2 = -G0/2 constant (second derivative
   *                   matrices on the diagonal), diagonal in the electronic index. */
  int keo_type;
  const double *G0;      /* D*D column-major, NULL = identity                       */
  const double *g;       /* D*D*D, NULL = 0                                          */
  /* optional host tables of the primitive bases: SG4 D*(LG+1) entries, (mode i, level L)
   * at bases[i*(LG+1) + L], sizes equal to the level rules Aq/Bq/Ab/Bb; DP D entries with
   * sizes nq_dp, nb_dp.  NULL: harmonic-oscillator bases on Gauss-Hermite grids scaled by
   * scaleQ and Q0, which are then unused. */
  const evr_basis1d *bases;
} evr_problem_desc;

/* sizes reported by evr_sizes(): */
typedef struct evr_sizes_t {
  int64_t Np;            /* packed basis size per electronic state                  */
  int64_t N;             /* Np*nb0, length of one vector                             */
  int64_t n_terms;       /* Smolyak terms (1 for DP)                                 */
  int64_t sum_nb;        /* sum over terms of prod nb_i                              */
  int64_t sum_nq;        /* sum over terms of prod nq_i (grid points)                */
  int64_t max_nq_term;   /* largest term grid                                        */
  double  flop_per_hpsi; /* algorithmic FLOP of one H.psi on one real vector         */
} evr_sizes_t;

/* Replaces the reference's set-up of para_Op/BasisnD for the OpPsi path
 * (sub_module_basis.f90:391, sub_quadra_SparseBasis.f90:924, BtoG_GtoB_SG4.f90:625,
 * grid fill sub_OpPsi_SG4.f90:2642-2767).  Builds every table on the host and
 * uploads them; the potential is evaluated on the device grid. */
/* device < 0 creates a host-only context: tables are built and can be read back
 * (evr_get_tables, evr_get_basis, evr_sizes); the device entry points return EVR_EDEVICE. */
int evr_create(evr_ctx **ctx, const evr_problem_desc *desc, int device);
int evr_destroy(evr_ctx *ctx);
const char *evr_last_error(const evr_ctx *ctx);
int evr_sizes(const evr_ctx *ctx, evr_sizes_t *out);

/* Read back the tables (host arrays sized from evr_sizes; any pointer may be NULL):
 * term_l[n_terms*D] Smolyak levels (first index fastest order of the reference),
 * weight[n_terms], map[sum_nb] 0-based packed index or -1, packed[Np*D] 1-based n. */
int evr_get_tables(const evr_ctx *ctx, int *term_l, double *weight, int *map, int *packed);
/* 1-D tables of (mode, level): nb, nq, x, w, d0b (nq x nb), d1b, d2b, bgw (nb x nq),
 * d1gg, d2gg (nq x nq), column-major.  Buffers of at least nq*nq doubles. */
int evr_get_basis(const evr_ctx *ctx, int mode, int level, int *nb_nq, double *x, double *w, double *d0b,
                  double *d1b, double *d2b, double *bgw, double *d1gg, double *d2gg);
/* Potential on the grid, sum_nq*nb0*nb0 values (term-major, point fastest, then (a,b)). */
int evr_get_vgrid(const evr_ctx *ctx, double *v);
/* Potential given as grid values, for a host whose potential is not a polynomial: the
 * values its calcN_op plugin put in the grid cache (Source_PrimOperator/sub_PrimOp.f90:
 * 283-655; SG4 fill Source_ElVibRot/sub_Operator/sub_OpPsi_SG4.f90:2754-2767, read per
 * term through tabR2gridbis_TO_tabR1_AT_iG :2655-2666).  Replaces the V the context evaluated from its
 * monomials for every later H.psi, Davidson, Chebyshev and control call (FP64 and FP32
 * tables).  layout EVR_VGRID_TERMS: the layout of evr_get_vgrid; EVR_VGRID_REF: the
 * reference's OpGrid(iterm)%Grid(sum_nq, nb0, nb0), element (iq, a, b) at
 * iq + sum_nq*(a + nb0*b), with iq the point of the whole Smolyak grid (terms in the
 * reference's order, first mode fastest inside a term) and a the output state.  The two
 * layouts agree for nb0 = 1.  Non-finite values are rejected with EVR_EINVAL (the message
 * names the first).  Synchronous (waits for the device first); a set-up call, not for use
 * inside stream capture; not for batched contexts. */
#define EVR_VGRID_TERMS 0
#define EVR_VGRID_REF   1
int evr_set_vgrid(evr_ctx *ctx, const double *v, int layout);
/* The kinetic metric G(Q) as grid values, for a type-10 context: what Tnum's get_d0GG gives
 * at each grid point (Source_ElVibRot/sub_Operator/sub_OpPsi_SG4.f90:2717-2728, where the
 * reference recomputes it on every H.psi), in place of G0 + sum_k g_ijk Q_k.  G: sum_nq
 * symmetric D x D matrices, point iq (the reference's whole-grid order, as EVR_VGRID_REF)
 * at G + iq*D*D, column-major.  Values must be finite, and each matrix symmetric: entries with
 * |G_ij - G_ji| > 1e-12 max(1, |G_ij|) are rejected with EVR_EINVAL, and the table stores
 * 0.5 (G_ij + G_ji).  The operator stays -1/2 sum_ij d_i G_ij(Q) d_j (Jacobian and rho
 * constant).  A context created with a constant G gets its per-point table here (captured
 * launch sequences of that context are dropped and recaptured).  Synchronous; a set-up
 * call; not for batches. */
int evr_set_ggrid(evr_ctx *ctx, const double *G);
/* The Jacobian and rho of a type-10 operator as grid values, the other two quantities
 * Tnum's get_d0GG gives per point (Source_ElVibRot/sub_Operator/sub_OpPsi_SG4.f90:2717-2728).
 * With them the kinetic part becomes, as in sub_TabOpPsi_OF_ONEDP_FOR_SGtype4 (:1579-1620),
 *   -1/2 [sum_i d_i (Jac sum_j G_ji d_j (s psi))] / (Jac s),   s = sqrt(rho/Jac).
 * jac, rho: sum_nq positive values in the reference's whole-grid point order (as
 * EVR_VGRID_REF); both null removes the table (Jac = rho = 1).  A context with a Jacobian
 * table runs every term in the general term kernel.  Synchronous; a set-up call; not for
 * batches. */
int evr_set_jacobian(evr_ctx *ctx, const double *jac, const double *rho);

/* H.psi on a block of vectors.
 * Replaces sub_TabOpPsi (Source_ElVibRot/sub_Operator/sub_OpPsi.f90:701-795) on SG4,
 * i.e. sub_TabOpPsi_FOR_SGtype4 (sub_OpPsi_SG4.f90:678-979), and on direct-product
 * bases sub_OpPsi_WITH_MemGrid_BGG_Hamil10 (sub_OpPsi.f90:1528-1794).
 * evr_hpsi_host: psi/hpsi are HOST arrays; copies in and out are inside the call.
 * evr_hpsi_device: psi/hpsi are DEVICE pointers; stream-ordered on `stream`
 *   (a cudaStream_t, NULL = the context's stream); no host synchronisation. */
int evr_hpsi_host(evr_ctx *ctx, const double *psi, int64_t ld_psi, double *hpsi, int64_t ld_hpsi, int nvec,
                  int layout, int prec);
int evr_hpsi_device(evr_ctx *ctx, const double *psi, int64_t ld_psi, double *hpsi, int64_t ld_hpsi, int nvec,
                    int layout, int prec, void *stream);

/* Operator applied by evr_hpsi_*: EVR_OP_H (default) is the reference's OpPsi;
 * EVR_OP_HT its transpose; EVR_OP_HSYM (H + H^T)/2.  The grid-derivative matrices
 * d1b.pinv(d0b) of sub_dnGB_TO_dnGG make H non-symmetric whenever nq > nb. */
#define EVR_OP_H    0
#define EVR_OP_HT   1
#define EVR_OP_HSYM 2
int evr_set_operator(evr_ctx *ctx, int form);

/* Kernel path of evr_hpsi_*: 1 (default) runs a problem of a single term (a direct
 * product basis) on the grid-wide stage kernels, and otherwise the small terms (below the
 * size threshold of evr_autotune) in the general kernel, every other term whose slab
 * pipeline fits one CTA's shared memory in the slab-streaming kernel and the rest in the
 * general kernel; 2 runs every term whose slab pipeline fits in the slab-streaming kernel,
 * small ones included, and the rest in the general kernel, without the stage kernels; 0
 * runs every term in the general kernel.  All compute the same operator. */
int evr_set_kernel_path(evr_ctx *ctx, int path);

/* Tensor cores for the FP32 path (no counterpart in the reference): on != 0 runs the mode
 * contractions of the slab-streaming kernel in FP32 H.psi on tcgen05 tensor cores (three
 * TF32 products of split operands, FP32 accumulation in tensor memory), those with K*M
 * below min_km on the CUDA cores; on = 0 (the default) runs them all on the CUDA cores.
 * The same operator either way, to FP32 accuracy.  FP64 H.psi is unaffected.
 * evr_autotune with EVR_PREC_FP32 also times this choice and keeps the faster. */
int evr_set_tensor_cores(evr_ctx *ctx, int on, int min_km);

/* H.psi that allocates nothing (no counterpart in the reference).
 * For callers that cannot let the library allocate device memory on the H.psi path --
 * a host that owns every device buffer through its own memory pool, or code that must
 * not enter the CUDA allocator at that point -- this variant of evr_hpsi_device takes its
 * scratch (item counter, term-basis output, per-CTA work buffers) from one file-scope
 * device array of 32 MiB that every GPU loading the library holds until the process
 * exits.  psi/hpsi: DEVICE pointers, interleaved layout (ld >= nvec), FP64, operator H
 * (evr_set_operator and evr_set_field do not apply; batched contexts are rejected).
 * Problems whose scratch exceeds 32 MiB are rejected with EVR_EINVAL (message gives the
 * size needed).  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.  All calls
 * share the one array: calls that overlap on the GPU (other streams, other threads)
 * race and must be serialised by the caller.  The call returns once the H.psi has
 * completed on the stream: it reads back the kernel's buffer-check flag (a plain copy into
 * a host variable) and returns EVR_EDEVICE if a work item was skipped. */
int evr_hpsi_noalloc(evr_ctx *ctx, const double *psi, int64_t ld_psi, double *hpsi, int64_t ld_hpsi, int nvec,
                     void *stream);

/* Self-test of the tensor-core mode contraction that the FP32 H.psi path uses (no
 * counterpart in the reference): one CTA of `threads` threads (128, 256 or 512) computes
 *   out(a, m, b, v) = alpha * sum_k mat[m + ldm*k] * in(a, k, b, v)  (+ out when acc != 0)
 * with element (a, k, b, v) of in at ((a + A*(k + K*b))*Vt + v), of out likewise with M,
 * ldm = 4*ceil(M/4), K <= 24, M <= 32, on tcgen05 tensor cores (three TF32 products of split
 * operands, FP32 accumulation in tensor memory).  Host arrays; out is read and written.
 * Returns EVR_ETIMEDOUT when a bounded wait of the kernel ran out. */
int evr_tc_selftest(int device, int A, int K, int M, int B, int Vt, const float *in, float *out, const float *mat,
                    float alpha, int acc, int threads);

/* Autotuner (no counterpart in the reference; its Tune_SG4threads_HPsi, vib.f90:1598-1705,
 * tunes OpenMP thread counts): times the term kernels on an nvec-vector block for each
 * cap of the vector tile of a work item (2..32, slab kernel then general kernel) and for
 * the size (grid points x vector tile, default 2048) below which a term runs in the general
 * kernel (as eight 64-thread CTAs per SM when its buffers fit one), and keeps the fastest
 * for later calls; with EVR_PREC_FP32 also whether the slab kernel's contractions run on the tensor
 * cores and from which size K*M (evr_set_tensor_cores).  caps[4] (optional): slab cap,
 * general cap, size threshold, tensor-core threshold (-1: CUDA cores); best_ms: the time. */
int evr_autotune(evr_ctx *ctx, int nvec, int prec, int *caps, double *best_ms);

/* Launch statistics of the last evr_hpsi_* call (kernels launched, work items). */
int evr_last_launch_count(const evr_ctx *ctx, int64_t *kernels, int64_t *items);
/* Device time (ms) of the term-pipeline kernel and of the weighted reduction of the last
 * H.psi call, from CUDA events recorded on the launching stream (waits for them). */
int evr_last_kernel_ms(evr_ctx *ctx, float *items_ms, float *reduce_ms);

/*
 * Block Davidson for the lowest levels.
 * Replaces sub_propagation_Davidson (Source_ElVibRot/sub_propagation/sub_module_Davidson.f90:54-748):
 * H.psi of the new vectors, Rayleigh-Ritz on the subspace (FP64 on the GPU), residuals
 * g_j = sum_i (H psi_i - E_j psi_i) V_ij (MakeResidual_Davidson :1214-1288), new vectors
 * from the residuals, two classical Gram-Schmidt passes (:1513-1529), restarts.
 * prec selects the H.psi precision; with EVR_PREC_FP32 the iteration runs on FP32
 * contractions and finishes with FP64 H.psi refinement so the returned levels are
 * converged with the FP64 operator.
 * guess: optional HOST array (N x n_guess column-major); NULL = unit vectors on the
 *   lowest diagonal elements of H.
 * eig: out, n_levels eigenvalues (au).  vec: optional HOST out (N x n_levels col-major).
 * info: optional out [iterations, H.psi count (FP64), H.psi count (FP32), converged]. */
typedef struct evr_davidson_opts {
  int n_levels;          /* levels wanted (nb_WP)                                   */
  int block;             /* start / block size                                      */
  int max_dim;           /* subspace size that triggers a restart (max_WP)          */
  int max_it;            /* max_it                                                  */
  double conv_resi;      /* residual norm tolerance (au)                            */
  double conv_ene;       /* eigenvalue change tolerance (au)                         */
  int prec;              /* EVR_PREC_FP64 or EVR_PREC_FP32                           */
  int n_guess;
  int sym;               /* operator: 0 = H, 1 = (H + H^T)/2, -1 = (H + H^T)/2 when H is
                            not symmetric by construction (some nq > nb)               */
} evr_davidson_opts;
int evr_davidson(evr_ctx *ctx, const evr_davidson_opts *opts, const double *guess, double *eig, double *vec,
                 int64_t *info);

/*
 * Chebyshev propagation of complex wave packets.
 * Replaces march_cheby (Source_ElVibRot/sub_propagation/sub_module_propa_march.f90:4142-4434):
 * psi(t+dt) = exp(-i E0 dt) sum_k c_k T_k(Hs) psi(t), c_0 = J_0(r), c_k = 2 J_k(r)
 * (cof :5734-5757), r = dE*dt/2, Hs = (H - E0)/(dE/2), E0 = (Emin+Emax)/2; the series
 * stops when |c_k|*||w_k|| < poly_tol.  psi0: HOST complex array (N x npsi interleaved
 * re/im pairs per element, column-major per packet).  autocorr (HOST, optional):
 * (nsteps+1) x npsi complex <psi0|psi(t_n)>.  psi_out (HOST, optional): final packets.
 * info: [max order used, total H.psi count, status]. */
int evr_cheby_propagate(evr_ctx *ctx, const double *psi0, int npsi, double dt, int nsteps, double emin,
                        double emax, double poly_tol, int prec, double *autocorr, double *psi_out,
                        int64_t *info);

/*
 * Short-iterative-Lanczos propagation of complex wave packets.
 * Replaces march_SIL (Source_ElVibRot/sub_propagation/sub_module_propa_march.f90:2899-3100)
 * with UPsi_spec (:3101-3160): per step and packet, q_1 = psi/|psi|, E0 = <q_1|H q_1>, a
 * Lanczos space of H - E0 grown until the last component of u = exp(-i T_k dt) e_1 falls
 * below poly_tol (or k = npoly), psi(t+dt) = |psi| exp(-i E0 dt) sum_k u_k q_k.  The
 * operator is the context's form (evr_set_operator): Lanczos assumes a symmetric H, so for
 * a type-10 operator with some nq > nb use EVR_OP_HSYM.  Arguments and outputs as
 * evr_cheby_propagate (no spectral bounds needed); npsi <= 32, npoly <= 256.
 * info: [largest Krylov dimension used, total H.psi count, status]. */
int evr_sil_propagate(evr_ctx *ctx, const double *psi0, int npsi, double dt, int nsteps, int npoly,
                      double poly_tol, int prec, double *autocorr, double *psi_out, int64_t *info);

/*
 * Gaussian filter diagonalisation: the levels of H in an energy window.
 * Replaces sub_GaussianFilterDiagonalization
 * (Source_ElVibRot/sub_propagation/sub_module_Filter.f90:70-520): n_filters Gaussian
 * filters exp(-((x - E_l)/sigma)^2), sigma = width/Esc/n_filters, centred at
 * lambda_min + l*width/(n_filters-1) with lambda_min = max(hmin, e0 - width/2), are
 * expanded in Chebyshev polynomials of Hs = (H - E0)/Esc (hmin/hmax widened by 1 % of their
 * range; the coefficients by the reference's Gauss-Chebyshev rule and kernel damping
 * factor, :300-345 and :2538-2579; the series length grown by 10 % until the central
 * filter's tail is below 1e-8 or it exceeds max_order, :199-283) and applied to each start
 * vector by the Chebyshev recursion (one H.psi per order for all start vectors,
 * sub_chebychev_recursion :2221-2298).  The filtered vectors are orthonormalised as
 * sub_Lowdin and sub_Schmidt do, those with an overlap eigenvalue above 1e-9 kept, and H is
 * diagonalised in their span (symmetrised, as sub_hermitic_H), with the residual norm of
 * every Ritz pair (:405-470).  The reference stops after this diagonalisation; the call
 * returns its results.  The operator is the context's form (evr_set_operator).
 * q0: optional HOST start vectors (N x nstart column-major; NULL = seeded random).
 * eig, resid: out, up to n_filters*nstart values (eigenvalues ascending, residual norms).
 * vec: optional HOST out (N x n_out column-major Ritz vectors).  n_out: kept vectors.
 * window: optional out [lambda_min, lambda_max, non_hermitic].
 * info: optional out [series length, H.psi count, kept vectors, levels in the window,
 *   levels in the window with a residual below max(conv_resi, non_hermitic)]. */
typedef struct evr_filter_opts {
  double hmin, hmax;     /* spectral bounds of H (au); hmin is also the window's floor   */
  double e0;             /* window centre (au; the reference's E0_filter + Hmin)          */
  double width;          /* window width (au; W_filter)                                  */
  int n_filters;         /* L_filter >= 2                                               */
  int max_order;         /* M_filter: cap of the series length (>= 4)                     */
  int nstart;            /* start vectors, n_filters filtered vectors each (1 = the reference) */
  int prec;              /* EVR_PREC_FP64 or EVR_PREC_FP32 contractions in the H.psi      */
  double conv_resi;      /* residual norm below which a level counts as converged (au)    */
  unsigned long long seed; /* random start vectors when q0 is NULL                        */
} evr_filter_opts;
int evr_filter_diag(evr_ctx *ctx, const evr_filter_opts *opts, const double *q0, double *eig, double *resid,
                    double *vec, int *n_out, double *window, int64_t *info);

/*
 * Restarted Lanczos for the lowest levels (the reference's ARPACK path).
 * Replaces sub_propagation_Arpack_Sym (Source_ElVibRot/sub_propagation/sub_module_Arpack.f90:
 * 680-1139), which calls ARPACK's dsaupd/dseupd (implicitly restarted Lanczos with exact
 * shifts, which = 'SM', ncv = 2*nev + 10, tol = 0) with one OpPsi per request.  Here a
 * thick-restart Lanczos on the GPU (the same Krylov spaces as exact-shift implicit
 * restarts): Lanczos steps with full re-orthogonalisation up to ncv vectors, Ritz pairs of
 * the projected matrix, convergence when the Ritz bound |beta y_m| <= tol max(eps^(2/3),
 * |E|) for all nev levels (ARPACK's test), else a restart that keeps the lowest Ritz vectors
 * and the last Lanczos vector.  The lowest (smallest algebraic) levels are computed, which
 * is what 'SM' selects on the positive spectra of vibrational Hamiltonians.  FP64 H.psi;
 * the operator is H or (H + H^T)/2 as sym selects (Lanczos needs a symmetric operator).
 * v0: optional HOST start vector (N); NULL = seeded random.  eig: out, nev eigenvalues.
 * vec: optional HOST out (N x nev column-major).  rel_resid: optional out, |H x - E x|/|E|
 * per level, computed with one more H.psi of the Ritz vectors (as the reference's d(j,2)).
 * info: optional out [restarts, H.psi count, converged levels, ncv].  Returns EVR_ENOCONV
 * (outputs filled) when max_restarts passes leave levels unconverged. */
typedef struct evr_lanczos_opts {
  int nev;               /* levels wanted (nb_diago)                                       */
  int ncv;               /* basis size; 0 = 2*nev + 10 as the reference (at most N, 512)   */
  int max_restarts;      /* maxitr (the reference: min(max_diago, max_it))                 */
  double tol;            /* relative Ritz bound; 0 = machine epsilon (the reference's tol=0) */
  int sym;               /* 0 = H, 1 = (H + H^T)/2, -1 = (H + H^T)/2 when some nq > nb     */
  unsigned long long seed; /* random start vector when v0 is NULL                          */
} evr_lanczos_opts;
int evr_lanczos(evr_ctx *ctx, const evr_lanczos_opts *opts, const double *v0, double *eig, double *vec,
                double *rel_resid, int64_t *info);

/* FMA issue-rate micro-benchmark of the device (independent FMA chains, no memory
 * traffic): the peak of the CUDA-core pipe the contractions run on, in TFLOP/s.
 * Utility for roofline reporting; no counterpart in the reference. */
int evr_fma_peak(int device, int prec, double *tflops);

/*
 * Field coupling H(t) = H0 - E(t) mu (one polarisation).
 * evr_set_dipole: the dipole operator mu(Q), given like the potential (n_mono monomials
 * coef * Q_i Q_j Q_k Q_l, idx[4m..4m+3] 0-based modes or -1, on the electronic block
 * (elec[2m], elec[2m+1])), evaluated on every grid like V.  Replaces the dipole
 * operators para_Dip(3) of sub_Opt_control (Source_ElVibRot/sub_propagation/sub_control.f90:290).
 * evr_set_field: the grid operator of later evr_hpsi_*, evr_davidson and
 * evr_cheby_propagate calls becomes vw*V + mw*mu, with the kinetic part when keo != 0
 * (H0 - E mu: vw = 1, mw = -E, keo = 1; mu alone: vw = 0, mw = 1, keo = 0;
 * (1, 0, 1) restores H0).  fcn_field's dWP = -i (H - E(t) Dip) WP
 * (sub_module_propa_march.f90:1494-1503) with a static field.
 */
int evr_set_dipole(evr_ctx *ctx, int n_mono, const double *coef, const int *idx, const int *elec);
/* The dipole as grid values instead of monomials: the grid of the scalar operator the
 * reference's plugin fills for the dipole (calcN_op, Source_PrimOperator/sub_PrimOp.f90:
 * 283-655), in either layout of evr_set_vgrid.  Replaces what evr_set_dipole evaluated, and
 * the bound max_q sum_b |mu_ab(q)| that widens the control propagator's spectral range.
 * Synchronous; a set-up call. */
int evr_set_dipole_grid(evr_ctx *ctx, const double *mu, int layout);
int evr_set_field(evr_ctx *ctx, double vw, double mw, int keo);

/*
 * Optimal control: objective J = |<target|psi(T)>|^2 (calc_fidelity,
 * sub_control.f90:1007-1050) under H(t) = H0 - E_n mu on step n (piecewise-constant field,
 * field[n] for t in [n dt, (n+1) dt)); each step is the Chebyshev expansion of
 * exp(-i (H0 - E_n mu) dt) on [emin - max|E| max|mu|, emax + max|E| max|mu|].
 * evr_oc_forward propagates psi0 (HOST, N complex as re/im pairs), returns
 * out3 = {J, Re c, Im c}, c = <target|psi(T)>, psi(T) in psiT (HOST, optional), and keeps
 * the state every `checkpoint` steps on the device (0: ceil(sqrt(nsteps))).
 * info: [Chebyshev order, H.psi columns applied, checkpoints kept].
 * evr_oc_backward returns dJ/dE_n (grad, nsteps values) for the field and states of the
 * last evr_oc_forward: the exact gradient of the discrete propagator, from the target
 * propagated backwards through the adjoint of every step's Chebyshev recurrence (the
 * transposed H, so also for the non-symmetric type-10 operator), the states recomputed
 * segment by segment from the checkpoints.  ref (HOST, nsteps+1 values, optional): the
 * continuous-time field gradient of build_field (sub_control.f90:955-975),
 * -2 Im(<psi(t_n)|chi(t_n)><chi(t_n)|mu|psi(t_n)>) at t_n = n dt, where the reference's
 * field update is E_new = ref / (2 alpha).  info: [H.psi columns applied, checkpoints,
 * steps per segment].  The reference has no discrete adjoint and no checkpointing.
 */
typedef struct {
  int nsteps;          /* steps of the control interval                              */
  double dt;           /* time step (au)                                             */
  double emin, emax;   /* spectral bounds of H0 (au)                                 */
  double poly_tol;     /* Chebyshev truncation, e.g. 1e-14                           */
  int checkpoint;      /* steps between stored states, 0 = ceil(sqrt(nsteps))        */
  int prec;            /* EVR_PREC_FP64 (EVR_PREC_FP32: FP32 contractions)           */
} evr_oc_opts;
int evr_oc_forward(evr_ctx *ctx, const evr_oc_opts *opts, const double *field, const double *psi0,
                   const double *target, double *out3, double *psiT, int64_t *info);
int evr_oc_backward(evr_ctx *ctx, double *grad, double *ref, int64_t *info);

/*
 * Batches of independent problems (no counterpart in the reference, which runs one
 * problem per process).  evr_create_batch stacks n_sys problems (any D and levels, the same
 * nb0 and KEO type) into one context: a vector of the context holds every problem's
 * packed functions, problem s in rows offsets[s] .. offsets[s+1]-1 (evr_batch_offsets,
 * n_sys + 1 values), and evr_hpsi_* apply the block-diagonal H -- every problem, every
 * column -- in one launch of the term kernels.  evr_batch_davidson: the lowest n_levels of
 * every problem (eig: n_sys x n_levels, problem-major), one state per problem (nb0 = 1),
 * subspace at most 64; info as evr_davidson (H.psi counts are per problem summed).  With
 * prec = EVR_PREC_FP32 an FP32 phase runs first and the FP64 iteration continues from its
 * Ritz vectors, so the levels are those of the FP64 operator.
 */
int evr_create_batch(evr_ctx **ctx, const evr_problem_desc *descs, int n_sys, int device);
int evr_batch_offsets(const evr_ctx *ctx, int64_t *offsets);
int evr_batch_davidson(evr_ctx *ctx, const evr_davidson_opts *opts, double *eig, int64_t *info);

/*
 * Wave-packet files in the reference's save formats (host only; any context but a batch,
 * host-only contexts included).  A basis function is written as its tuple
 * n_1..n_D i_h i_e (1-based; i_h = 1, i_e = electronic state), as Rec_ndim_index gives it.
 *   EVR_WP_FORMATTED_V0   "nb_psi nb_tot", then per packet every entry "n.. i_h i_e a [b]"
 *                         and " end wp k" -- sub_save_psi with FilePsiVersion = 0, the
 *                         reference's default (Source_ElVibRot/sub_WP/sub_module_psi_io.f90:
 *                         365-424, Write_Psi_nDBasis version 0 :1607-1700)
 *   EVR_WP_FORMATTED_V1   &headerFile namelist, the nb_tot tuples, then each packet as one
 *                         list-directed record (complex as (re,im)) (:1441-1604, :1736-1760)
 *   EVR_WP_UNFORMATTED_V1 Fortran sequential unformatted records with 4-byte markers:
 *                         'X', nb_psi, nb_tot, 1, 'X', one int32 record of D+2 per
 *                         function, one record of nb_tot values per packet (:1483-1489)
 *   EVR_WP_SPARSE         "nb_psi", then per packet the entries of modulus >= epsi and
 *                         " end wp k" (ecri_psiBasisRepnotall_nD :783-917)
 * psi: N x npsi column-major host array (N = Np*nb0, ld >= N); cplx = 1: Fortran COMPLEX(8)
 * layout, (re, im) of element k of packet j at psi[2*(k + ld*j)].
 */
#define EVR_WP_FORMATTED_V0   0
#define EVR_WP_FORMATTED_V1   1
#define EVR_WP_UNFORMATTED_V1 2
#define EVR_WP_SPARSE         3
int evr_psi_write(evr_ctx *ctx, const char *path, int format, const double *psi, int64_t ld, int npsi, int cplx,
                  double epsi);
/* Replaces sub_read_psi0's file branch (sub_module_psi_io.f90:55-263 with
 * Read_header_saveFile_psi :1294-1439, Read_list_nDindBasis1_TO_nDindBasis2 :1143-1292,
 * Read_psi_nDBasis :920-1141, lect_psiBasisRepnotall_nD :563-780).  The form is detected:
 * unformatted version 1, or formatted with a headerFile namelist (version 1), an
 * "nb_psi nb_tot" line (version 0, entries read by position after the first packet's
 * tuples), an "nb_psi" line (sparse packets), or no header (sparse packets as in an input
 * file after its namelists).  Each file function goes to the function of this basis with
 * the same tuple; functions this basis does not hold are dropped and counted in
 * *n_dropped (entries over the packets read), functions absent from the file stay zero.
 * Reads min(packets in the file, npsi_max) packets (*npsi_read).  Unlike sub_read_psi0
 * it does not renormalise the packets.  A malformed file returns EVR_EINVAL with the
 * line or record at fault, where the reference STOPs. */
int evr_psi_read(evr_ctx *ctx, const char *path, double *psi, int64_t ld, int npsi_max, int cplx, int *npsi_read,
                 int64_t *n_dropped);
/* Propagation restart file: SaveWP_restart / ReadWP_restart
 * (Source_ElVibRot/sub_propagation/sub_module_propagation.f90:376-488): a "T nb_WP size"
 * record, then each packet's complex coefficients as one list-directed record.  psi: complex
 * packets in the Fortran COMPLEX(8) layout (ld >= N).  evr_restart_read: a file without
 * that first record means no restart (*found = 0, *t = 0, psi untouched); nb_WP != npsi or
 * size != N returns EVR_EINVAL, where the reference STOPs. */
int evr_restart_write(evr_ctx *ctx, const char *path, double t, const double *psi, int64_t ld, int npsi);
int evr_restart_read(evr_ctx *ctx, const char *path, double *t, double *psi, int64_t ld, int npsi, int *found);
/* Autocorrelation file lines "AutoCor T Re Im |C|" (Write_AutoCorr / Read_AutoCorr, :548-578);
 * cdot: n complex values (re, im).  append != 0 adds to an existing file.  The reader keeps
 * the lines that read as such (at most n_max) and skips the others. */
int evr_autocorr_write(const char *path, const double *t, const double *cdot, int n, int append);
int evr_autocorr_read(const char *path, double *t, double *cdot, int n_max, int *n);

#ifdef __cplusplus
}
#endif
#endif /* EVR_GPU_H */
