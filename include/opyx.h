/*
 * opyx.h -- C ABI of libopyx, the GB300 (sm_103a) kernels behind
 * opymize_gb300's PDHG path.
 *
 * Every entry point replaces one kernel (or kernel family) that the reference
 * compiles at run time through PyCUDA (opymize/tools/gpu.py:39-80,
 * `prepare_kernels` -> `{name: kernelfun(*gpudata)}`), and is what a binding
 * of that path would call instead.  Conventions:
 *
 *   - all array arguments are DEVICE pointers owned by the caller; the library
 *     never allocates memory (scratch comes from caller-sized workspaces);
 *   - `dtype` is OPYX_F32 or OPYX_F64 and applies to every iterate array of
 *     the call; constant operator data (weights, matrices) is double;
 *   - `add` = 0 writes the result, `add` = 1 accumulates into the target,
 *     as `Operator.__call__(x, y, add=...)` (opymize/__init__.py:64-84);
 *   - `stream` is a cudaStream_t (NULL = legacy default stream); calls are
 *     asynchronous and capturable in a CUDA graph unless stated otherwise;
 *   - every function returns an int status (OPYX_OK = 0); nothing throws
 *     across the ABI.
 */
#ifndef OPYX_H
#define OPYX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  OPYX_OK = 0,
  OPYX_ERR_ARG = 1,           /* bad shape, size, pointer or enum value      */
  OPYX_ERR_LAUNCH = 2,        /* CUDA launch / runtime error                  */
  OPYX_ERR_UNSUPPORTED = 3,   /* valid request this build does not implement */
  OPYX_ERR_WORKSPACE = 4,     /* workspace too small or misaligned           */
  OPYX_ERR_NOT_CONVERGED = 5, /* an iterative device routine hit its bound   */
  OPYX_ERR_SCRATCH_LIMIT = 6  /* problem exceeds the static scratch of
                                 opyx_rof_iterate_noalloc                     */
};

enum { OPYX_F32 = 0, OPYX_F64 = 1 };

/* Library version (major*10000 + minor*100 + patch). */
int opyx_version(void);
/* Static description of a status code. */
const char* opyx_status_string(int status);
/* Number of SMs of the current device (grid sizing). */
int opyx_sm_count(void);

/* ------------------------------------------------------------ utilities */
/* y[i] = value  (gpuarray.fill, used before every reference LinOp call:
 * opymize/linear/diff.py:143, :182). */
int opyx_fill(int dtype, void* y, int64_t n, double value, void* stream);
/* y = a*x + b*y  (gpuarray `y[:] = x`, `y += x`, ScaleOp; scale.py:44-67). */
int opyx_axpby(int dtype, int64_t n, double a, const void* x, double b, void* y,
               void* stream);
/* y = |x| elementwise (numpy `np.abs`, power iteration of normest:
 * opymize/linear/__init__.py:11-46). */
int opyx_abs(int dtype, int64_t n, const void* x, void* y, void* stream);
/* y = x converted between OPYX_F64 and OPYX_F32 (uploads of FP64 host data
 * for FP32 iterates are converted on the device). */
int opyx_cast(int src_dtype, int dst_dtype, int64_t n, const void* x, void* y, void* stream);
/* x_i <- 1/x_i where x_i > eps, unchanged elsewhere: the diagonal
 * preconditioners from rowwise norms (opymize/solvers/pdhg.py:197-198). */
int opyx_recip_positive(int dtype, int64_t n, void* x, double eps, void* stream);
/* y[(o*N + i)*inner + r] (+)= pat[o*inner + r]: broadcasts a small per-row
 * pattern (rowwise norms of per-pixel operators) over N pixels. */
int opyx_broadcast_mid(int dtype, const double* pat, int64_t outer, int64_t N,
                       int64_t inner, void* y, int add, void* stream);
/* out[0] = sum_i x_i^2, out[1] = max_i |x_i| in FP64 (device double[2]);
 * `ws` >= opyx_reduce_workspace_size() bytes. */
size_t opyx_reduce_workspace_size(void);
int opyx_norms(int dtype, int64_t n, const void* x, double* out, void* ws,
               void* stream);

/* out[0] = sum_i x_i y_i in FP64 (deterministic; ws as opyx_norms): the
 * inner products of the semismooth Newton solver's CG and line search
 * (np.einsum('i,i->', ...), opymize/solvers/semismooth_newton.py:106-116). */
int opyx_dot(int dtype, int64_t n, const void* x, const void* y, double* out, void* ws,
             void* stream);

/* ---------------------------------------------- finite differences (diff) */
#define OPYX_MAX_DIMS 6
typedef struct {
  int32_t ndim;                 /* D, 1..OPYX_MAX_DIMS                      */
  int32_t nchannels;            /* C >= 1                                   */
  int64_t dims[OPYX_MAX_DIMS];  /* image shape, row-major, last contiguous  */
  double h[OPYX_MAX_DIMS];      /* grid step per axis (imageh)              */
} opyx_grid;

enum { OPYX_SCHEME_FORWARD = 0, OPYX_SCHEME_CENTERED = 1 };

/* y[i,t,k] (+)= D x : GradientOp (opymize/linear/diff.py:67-144), kernel
 * `gradient` (opymize/linear/diff.cu:37-75).  x is (N, C), y is (N, D, C);
 * `weights` is a device double[C] or NULL (all ones). */
int opyx_gradient(const opyx_grid* g, int scheme, const double* weights, int dtype,
                  const void* x, void* y, int add, void* stream);
/* x (+)= D^T y : DivergenceOp (diff.py:146-183), kernel `divergence`
 * (diff.cu:77-127). */
int opyx_divergence(const opyx_grid* g, int scheme, const double* weights, int dtype,
                    const void* y, void* x, int add, void* stream);
/* Rowwise l^p norms of the gradient (transpose = 0, y of size N*D*C) or of
 * the divergence (transpose = 1, y of size N*C):  y_i (+)= (sum_j |A_ij|^p)^(1/p),
 * as LinOp.rowwise_lp on the reference's sparse matrix (opymize/__init__.py:122-142). */
int opyx_gradient_rowlp(const opyx_grid* g, int scheme, const double* weights,
                        int transpose, double p, int dtype, void* y, int add,
                        void* stream);

enum { OPYX_BC_NEUMANN = 0, OPYX_BC_CURVATURE = 1, OPYX_BC_SECOND_ORDER = 2 };
/* y (+)= Laplacian x with boundary `bc` (or its adjoint):  LaplacianOp
 * (diff.py:185-249), kernel `laplacian` (diff.cu:131-243). */
int opyx_laplacian(const opyx_grid* g, int bc, int adjoint, int dtype,
                   const void* x, void* y, int add, void* stream);
int opyx_laplacian_rowlp(const opyx_grid* g, int bc, int adjoint, double p,
                         int dtype, void* y, int add, void* stream);

/* -------------------------------------------- per-pixel products (einsum) */
/* y_ji (+)= sum_k A_jk x_ki, x (K,N), y (J,N); trans: A stored (K,J).
 * MatrixMult (opymize/linear/einsum.py:17-56), kernel `matrixmult`
 * (einsum.cu:3-28).  A is a device double array. */
int opyx_matrixmult(int dtype, int64_t N, int J, int K, const double* A, int trans,
                    const void* x, void* y, int add, void* stream);
/* y_ij (+)= sum_k x_ik A_kj, x (N,K), y (N,J); trans: A stored (J,K).
 * MatrixMultR (einsum.py:58-97), kernel `matrixmultr` (einsum.cu:32-57). */
int opyx_matrixmultr(int dtype, int64_t N, int K, int J, const double* A, int trans,
                     const void* x, void* y, int add, void* stream);
/* y_jlk (+)= sum_m x_jlm A_jmk, x (J,L,M), y (J,L,K); trans: A stored (J,K,M).
 * MatrixMultRBatched (einsum.py:175-214), kernel `matrixmultrbatched`
 * (einsum.cu:61-87). */
int opyx_matrixmultr_batched(int dtype, int J, int64_t L, int M, int K,
                             const double* A, int trans, const void* x, void* y,
                             int add, void* stream);
/* y_mik (+)= sum_jl x_jil A_jlmk, x (J,N,L), y (M,N,K); trans: A stored
 * (M,K,J,L).  TangledMatrixMultR (einsum.py:130-173), kernel
 * `tangledmatrixmultr` (einsum.cu:91-122). */
int opyx_tangled_matrixmultr(int dtype, int J, int64_t N, int L, int M, int K,
                             const double* A, int trans, const void* x, void* y,
                             int add, void* stream);
/* y_ik (+)= x_ik A_k.  DiagMatrixMultR (einsum.py:104-128). */
int opyx_diag_matrixmultr(int dtype, int64_t N, int K, const double* A,
                          const void* x, void* y, int add, void* stream);

/* ------------------------------------------------- label gather / scatter */
/* y[j,i,m] (+)= -sum_l B[j,m,l] x[i,P[j,l]], x (N,K), y (J,N,M); B device
 * double (J,M,L), P device int64 (J,L).  IndexedMult
 * (opymize/linear/indexed.py:63-94), kernel `indexedmult` (indexed.cu:28-48). */
int opyx_indexedmult(int dtype, int J, int64_t N, int M, int L, int K,
                     const double* B, const int64_t* P, const void* x, void* y,
                     int add, void* stream);
/* y[i,P[j,l]] (+)= -sum_m B[j,m,l] x[j,i,m]: IndexedMultAdj
 * (indexed.py:34-61), kernel `indexedmultadj` (indexed.cu:2-26). */
int opyx_indexedmult_adj(int dtype, int J, int64_t N, int M, int L, int K,
                         const double* B, const int64_t* P, const void* x, void* y,
                         int add, void* stream);

/* ------------------------------------------------ piecewise-linear epigraphs */
/* Instance (j, i) of x (nregions, nfuns, ndim+1) is constrained by
 * <v[l], y[:ndim]> - y[ndim] <= b[i, l] for l = J[j, k] (k < nsubpoints) with
 * I[i, l] != 0: the epigraph of the conjugate of the convex piece j of the
 * piecewise-linear function i (opymize/operators/proj.py:388-480).  v and b
 * are in the iterate dtype; the EpigraphSupp value additionally needs the
 * affine pieces of every instance (eq_off, eqns) and the region checks, both
 * FP64 (functionals/epigraph.py:56-112). */
typedef struct {
  int32_t ndim;               /* 1..3                                       */
  int32_t nsubpoints;
  int64_t nfuns, nregions, npoints;
  const uint8_t* I;           /* (nfuns, npoints)                           */
  const int64_t* J;           /* (nregions, nsubpoints), values < npoints   */
  const void* v;              /* (npoints, ndim)                            */
  const void* b;              /* (nfuns, npoints)                           */
  const int64_t* eq_off;      /* (nregions*nfuns + 1) row offsets, or NULL  */
  const double* eqns;         /* (eq_off[last], ndim+1), or NULL            */
  const double* checks;       /* (nregions, ndim+1, ndim+1), or NULL        */
  const void* bt;             /* (npoints, nfuns) copy of b, or NULL: ndim 1
                                 projections read it coalesced              */
  const uint8_t* It;          /* (npoints, nfuns) copy of I, or NULL        */
} opyx_epigraph;

/* y = EpigraphProj(x) (proj.py:388-480; reference kernel `epigraphproj` with
 * `solve_qp`, proj.cu:660-831): per-instance active-set QP; for ndim 1 with
 * at most 16 points per region the exact projection onto the piecewise-
 * linear epigraph's pieces in one pass instead.  y may equal x.
 * Instances whose QP did not finish within maxiter steps (the reference uses
 * ndim*nsubpoints, tolerance 1e-9) are counted into *nonconv (device
 * unsigned, may be NULL); the reference prints a warning instead. */
int opyx_epigraph_proj(const opyx_epigraph* e, int dtype, const void* x, void* y,
                       int maxiter, double tol, unsigned* nonconv, void* stream);
/* out (device double[2]) = {val, infeas} of EpigraphInd (which = 0,
 * epigraph.py:40-46) or EpigraphSupp (which = 1, epigraph.py:101-112) at x,
 * reduced in FP64; ws as for opyx_fct_eval.  EpigraphSupp takes the max over
 * the given faces (eq_off, eqns); with eq_off = NULL (ndim 1 only) it
 * evaluates the convex envelope of each instance's points directly, which
 * equals the faces' max when the faces are the points' lower convex hull. */
int opyx_epigraph_eval(const opyx_epigraph* e, int dtype, int which, const void* x,
                       double* out, void* ws, void* stream);

/* ---------------------------------------------- fused sublabel-lifted model */
/* One fused pass of the PDHG iteration (opymize/solvers/pdhg.py:124-187) of
 * the sublabel-lifted scalar model that opymize_gb300/tools/lifting.py
 * assembles from the reference's operators:
 *   x = (u [N, L], gamma [N], mu [L-1, N, 2]),
 *   y = (q [N, L], e [N], p [N, 2], s [N], z [L-1, N, 2]),
 *   A x = (u + IndexedMultAdj(mu) [P[j] = (j, j+1), coefficients B],
 *          <t, u> - gamma, forward gradient of gamma (h = 1), <1, u>, mu),
 *   prox_tauG = (max(u, 0), gamma, mu),
 *   prox_sigmaF* = (q, e, projection of p onto |p_i| <= lbd, s - sigma,
 *                   EpigraphInd projection of every z[j, i] (ndim 1)).
 * which = 0 (pass A): xkp1 = prox(xk - tau A^T yk), xbar = (1+theta) xkp1 -
 * theta xk; which = 1 (pass B): ykp1 = prox(yk + sigma A xbar); which = 2:
 * the envelopes' live lines of every interval instance into `hull` (once per
 * solve: they depend on the data term only).  It replaces
 * the generic path's chain of BlockOp / IndexedMultAdj / MatrixMultR /
 * ScaleOp / GradientOp and prox launches for this model (about 22 per
 * iteration).  Steps: tau and sigma of u, mu, q, e, s, z per label /
 * interval / component (the same for every pixel, as the preconditioner
 * of this A gives), gamma's tau and p's sigma per pixel (tau_g (N), sig_p
 * (N, 2) device arrays) or, if NULL, the scalars tau_g0, sig_p0.  The
 * epigraph data: v (npoints) points, bt (npoints, N) values at the points,
 * It (npoints, N) point masks or NULL (all set), J (L-1, nsub) the points
 * of each interval (nsub <= 16).  L: 2 to 32. */
typedef struct {
  int32_t dtype, L, nsub, pad;
  int64_t H, W;
  const void* xk;
  void* xkp1;
  void* xbar;
  const void* yk;
  void* ykp1;
  double t[32];
  double B[31 * 2 * 2];          /* B[j][m][k] */
  double tau_u[32], tau_mu[31 * 2];
  double sig_q[32], sig_z[31 * 2];
  double sig_e, sig_s;
  const void* tau_g;
  const void* sig_p;
  double tau_g0, sig_p0;
  double lbd, theta;
  const void* v;
  const void* bt;
  const uint8_t* It;
  const int64_t* J;
  int32_t sorted;                /* perm gives each interval's points by increasing, */
  uint8_t perm[31 * 16];         /* distinct slope (the projection skips its sort)   */
  double vsorted[31 * 16];       /* those slopes, in that order (host copy)          */
  uint8_t* hull;                 /* (L-1, N) device bytes, or NULL: bit k set if the
                                    k-th point (increasing slope) carries a piece of
                                    the instance's envelope; which = 2 fills it (needs
                                    sorted), pass B then projects over those lines  */
} opyx_sublabel;
int opyx_sublabel_pass(const opyx_sublabel* d, int which, void* stream);

/* ------------------------------------------- piecewise convexification (host) */
/* The lower convex hull of every function's graph over every region, the
 * input data of EpigraphInd / EpigraphSupp (I = base, If = faces):
 * piecewise_convexify (opymize/quickhull/__init__.pyx:8-140, hull code
 * convexhull.cpp:118-216).  HOST code: every pointer is host memory and no
 * device work is done.  points (npoints, ndim) doubles, vals (nfuns, npoints)
 * doubles, regions (nregions, nsub) indices into the points, the first ndim+1
 * of each region its simplex's vertices.  Outputs: base (nfuns, npoints) 0/1;
 * faces (nfuns, nregions, max_faces, ndim+1) positions in the region's row of
 * `regions` (-1 past the count), nfaces (nfuns, nregions).  ndim 1, 2 or 3;
 * max_faces >= opyx_convexify_max_faces(ndim, nsub), else
 * OPYX_ERR_WORKSPACE; nthreads <= 0 uses every host thread. */
int opyx_convexify_max_faces(int ndim, int nsub);
int opyx_convexify(int ndim, int64_t npoints, const double* points, int64_t nfuns,
                   const double* vals, int64_t nregions, int nsub, const int64_t* regions,
                   uint8_t* base, int32_t* faces, int32_t* nfaces, int max_faces, int nthreads);

/* ------------------------------------------------------------- step sizes */
/* A step size is a per-element device vector (`vec`, of the iterate dtype,
 * preconditioned steps), else a device double written by the solver
 * (`dev`, adaptive steps), else the constant `value`. */
typedef struct {
  const void* vec;
  const double* dev;
  double value;
} opyx_step;

/* ----------------------------------------------------------- prox maps */
/* y (+)= a*(x + b*shift) with each of a, b, shift a device vector of the
 * iterate dtype or (NULL) the scalar given.  ShiftScaleOp
 * (opymize/operators/affine.py:85-146). */
int opyx_shiftscale(int dtype, int64_t n, const void* a_vec, double a,
                    const void* b_vec, double b, const void* shift_vec, double shift,
                    const void* x, void* y, int add, void* stream);
/* y = a*(x - tau*c), a and c a device vector or (NULL) the scalar given, tau
 * an opyx_step: the prox of tau*AffineFct / MaskedAffineFct
 * (opymize/functionals/affine.py:38-42, :86-90, which set ShiftScaleOp's b to
 * -tau) for scalar, per-element and device-held adaptive steps alike. */
int opyx_affine_prox(int dtype, int64_t n, const void* a_vec, double a, const void* c_vec,
                     double c, opyx_step tau, const void* x, void* y, void* stream);
/* SSD prox: y = (x + t*f)/(1 + t) with t = tau*vol_k on masked pixels, y = x
 * elsewhere; x, y, f (N,C); vol device double[C] (NULL = ones); mask device
 * uint8[N] (NULL = all).  SSD.prox -> ShiftScaleOp (functionals/quad.py:45-55). */
int opyx_ssd_prox(int dtype, int64_t N, int C, const void* f, const double* vol,
                  const uint8_t* mask, opyx_step tau, const void* x, void* y,
                  void* stream);
/* y (+)= max(0,x) / min(0,x): PosProj / NegProj (operators/proj.py:19-85). */
int opyx_posproj(int dtype, int64_t n, const void* x, void* y, int add, void* stream);
int opyx_negproj(int dtype, int64_t n, const void* x, void* y, int add, void* stream);
/* y (+)= mask[i] ? c[i,:] : x[i,:] for (N,M) data: ConstrainOp
 * (operators/affine.py:46-83). */
int opyx_constrain(int dtype, int64_t N, int M, const uint8_t* mask, const void* c,
                   const void* x, void* y, int add, void* stream);

enum { OPYX_NORM_FROBENIUS = 0, OPYX_NORM_SPECTRAL = 1 };
/* In-place projection of each x_i (an M1 x M2 matrix) onto the ball of
 * radius lbd in the Frobenius norm or (2 x M / M x 2 only) the spectral norm.
 * L1NormsProj (operators/proj.py:170-226), kernel `l1normsproj`
 * (operators/proj.cu:2-108). */
int opyx_l1normsproj(int dtype, int64_t N, int M1, int M2, double lbd, int matrixnorm,
                     void* x, void* stream);
/* In-place prox of sigma*F* for F = lbd*sum_i huber_alpha(|x_i|_F):
 * x_i <- proj_{|.|_F<=lbd}(x_i / (1 + sigma*alpha/lbd)), groups of m values. */
/* Frobenius-ball projection of N groups of M values in place, recording the
 * map's Jacobian at x: xn (N*M) = x/|x| and s (N) = lbd/|x| outside the ball,
 * 0 and 1 inside (L1NormsProj(jacobian=True) + L12ProjJacobian.update,
 * opymize/operators/proj.py:206-252). */
int opyx_l1normsproj_jac(int dtype, int64_t N, int M, double lbd, void* x, void* xn, void* s,
                         void* stream);
/* y (+)= s_i (x_i - <xn_i, x_i> xn_i): L12ProjJacobian applied
 * (opymize/operators/proj.py:254-276); symmetric. */
int opyx_l12proj_jacobian(int dtype, int64_t N, int M, const void* xn, const void* s, const void* x,
                          void* y, int add, void* stream);
int opyx_huber_conj_prox(int dtype, int64_t N, int m, double lbd, double alpha,
                         opyx_step sigma, void* x, void* stream);
/* In-place projection of (x1, x2) in R^M x R onto the epigraph of
 * 0.5*alph*|x1 - s1|^2 + s2 (shift s device (N, M+1) of the iterate dtype or
 * NULL), truncated at |x1 - s1| <= lbd when lbd is finite.  The cubic
 * root-finding runs in FP64 for both dtypes.  QuadEpiProj
 * (operators/proj.py:278-374), kernel `quadepiproj` (operators/proj.cu:110-220). */
int opyx_quadepiproj(int dtype, int64_t N, int M, double alph, const void* shift,
                     double lbd, void* x, void* stream);

/* --------------------------------------------------- generic PDHG steps */
/* zkp1 = zk + direction*step*zgrad: `take_step` (opymize/solvers/pdhg.py:62-65). */
int opyx_take_step(int dtype, int64_t n, void* zkp1, const void* zk, int direction,
                   opyx_step step, const void* zgrad, void* stream);
/* ykp1 = yk + sigma*((1+theta)*ygkp1 - theta*ygk): `overrelax` followed by
 * `take_step` (pdhg.py:66-69, :145-151) in one pass. */
int opyx_dual_step(int dtype, int64_t n, void* ykp1, const void* yk, opyx_step sigma,
                   double theta, const void* ygkp1, const void* ygk, void* stream);
/* out[0] += sum((zk - zkp1)/a - b*zgk + c1*zgkp1)^2,
 * out[1] += sum((zk - zkp1)/a - b*zgk + c2*zgkp1)^2 in FP64: two `residual`
 * reductions (pdhg.py:74-78) sharing their reads.  `out` is device double[2]
 * (accumulated), `ws` a reduction workspace. */
int opyx_residual_pair(int dtype, int64_t n, opyx_step a, const void* zk,
                       const void* zkp1, double b, const void* zgk, double c1,
                       double c2, const void* zgkp1, double* out, void* ws,
                       void* stream);

/* Device state of the adaptive step rule (pdhg.py:156-183), all double. */
typedef struct {
  double tau, sigma, alpha;       /* current steps and damping              */
  double eta, Delta, theta;       /* constants (0.95, 1.5, 1.0)             */
  double eps[4];                  /* eps_abs_p, eps_rel_p, eps_abs_d, eps_rel_d */
  double sums[4];                 /* |r_p|^2, |g_p|^2, |r_d|^2, |g_d|^2 (accumulated) */
  double resp, resd, epsp, epsd;  /* outputs of the last update             */
  double xsize, ysize;            /* primal and dual sizes                  */
} opyx_adaptive_state;

/* Apply the adaptive rule to `st` (device pointer) from its `sums`, then
 * zero the sums.  Single-thread kernel; no host synchronisation. */
int opyx_adaptive_update(opyx_adaptive_state* st, void* stream);

/* ------------------------------------------------ functional evaluation */
/* Value and infeasibility of a functional at x, reduced in FP64 on the
 * device (the reference evaluates them in numpy on the host for the gap,
 * opymize/solvers/pdhg.py:23-44, :292-301).  x holds `ngroups` groups of
 * m1*m2 values; out is a device double[2] = {val, infeas}; ws is a reduction
 * workspace (opyx_reduce_workspace_size bytes, zero-filled before first use). */
enum {
  OPYX_FCT_SSD = 0,          /* functionals/quad.py:7-43; v0 = f, vol, mask, scalar0 = shift */
  OPYX_FCT_L1NORMS,          /* l1norms.py:34-63; lbd, matrixnorm SPECTRAL = nuclear   */
  OPYX_FCT_L1NORMS_CONJ,     /* l1norms.py:65-88; lbd, matrixnorm                     */
  OPYX_FCT_HUBER,            /* lbd*sum huber_alpha(|x_i|)                            */
  OPYX_FCT_HUBER_CONJ,       /* alpha/(2 lbd) sum |x_i|^2 + indicator(|x_i| <= lbd)     */
  OPYX_FCT_QUADEPI_IND,      /* epigraph.py:169-197; a, v0 = b (N,M), v1 = c (N)        */
  OPYX_FCT_QUADEPI_SUPP,     /* epigraph.py:135-166; a, v0 = b, v1 = c                 */
  OPYX_FCT_HUBER_PERSP,      /* epigraph.py:203-236; lbd, alpha                         */
  OPYX_FCT_TRUNCQUAD_IND,    /* epigraph.py:238-270; lbd, alpha                         */
  OPYX_FCT_POSITIVITY,       /* indicators.py:74-93                                    */
  OPYX_FCT_NEGATIVITY,       /* indicators.py:95-98                                    */
  OPYX_FCT_AFFINE,           /* functionals/affine.py:9-44; scalar0 = b, v0 or scalar1 = c */
  OPYX_FCT_INDICATOR,        /* indicators.py:8-29; v0 or scalar1 = c1, scalar0 = c2   */
  OPYX_FCT_CONSTRAIN,        /* indicators.py:31-58; mask, v0 = c                       */
  OPYX_FCT_MASKED_AFFINE     /* functionals/affine.py:59-90; mask, v0 = c               */
};

typedef struct {
  int32_t kind;
  int32_t matrixnorm;
  int64_t ngroups;
  int32_t m1, m2;
  double lbd, alpha, a;
  double scalar0, scalar1;
  const void* v0;            /* iterate dtype, or NULL */
  const void* v1;            /* iterate dtype, or NULL */
  const double* vol;         /* device double[m1*m2] or NULL */
  const uint8_t* mask;       /* device uint8[ngroups] or NULL */
} opyx_fct;

int opyx_fct_eval(const opyx_fct* f, int dtype, const void* x, double* out, void* ws,
                  void* stream);

/* ------------------------------------------------ fused ROF-type PDHG path */
/* min_x G(x) + F(Ax) with G = SSD(f, vol, mask, shift), F = lbd*L1Norms
 * (Frobenius) or its Huber smoothing, A = forward-difference GradientOp:
 * PDHG.solve(use_gpu=True) for this (G, F, A) (opymize/solvers/pdhg.py:229-315,
 * functionals/quad.py, functionals/l1norms.py, linear/diff.py) with each
 * iteration fused into two passes (three for adaptive steps). */
#define OPYX_ROF_MAX_C 4
enum { OPYX_STEPS_CONST = 0, OPYX_STEPS_ADAPTIVE = 1, OPYX_STEPS_PRECOND = 2 };

typedef struct {
  int32_t dtype;                    /* OPYX_F32 / OPYX_F64                   */
  int32_t ndim;                     /* D, 1..3                               */
  int32_t nchannels;                /* C, 1..OPYX_ROF_MAX_C                  */
  int32_t steps;                    /* OPYX_STEPS_*                          */
  int64_t dims[3];                  /* image shape (dims[0..D-1])            */
  double h[3];                      /* grid steps (GradientOp imageh)        */
  double weights[OPYX_ROF_MAX_C];   /* GradientOp channel weights            */
  double vol[OPYX_ROF_MAX_C];       /* SSD volume element per channel        */
  double ssd_shift;                 /* SSD constant                          */
  double lbd;                       /* regularisation weight (> 0)           */
  double huber_alpha;               /* 0: L1Norms; > 0: Huber parameter      */
  double tau, sigma;                /* initial steps (constant / adaptive)   */
  double theta;                     /* overrelaxation (the reference uses 1) */
  double alpha0, eta, Delta;        /* adaptive rule (0.5, 0.95, 1.5)        */
  double eps[4];                    /* adaptive tolerances (pdhg.py:275-280) */
  double term_relgap;               /* device-side stop test of opyx_rof_gap:  */
  double term_infeas;               /*   term_mode 1: |relgap| < term_relgap and
                                         max(infeasp, infeasd) < term_infeas;
                                       term_mode 2: resp < epsp, resd < epsd
                                         (adaptive steps)                   */
  int32_t term_mode;                /* 0: no device-side stop               */
  int32_t rows_per_thread;          /* tile height of the vectorised FP32
                                       kernels; 0 = automatic               */
  int32_t flags;                    /* bit 0: never use the vectorised FP32
                                       kernels; bit 1: never use the
                                       row-streaming FP32 kernels (both for
                                       cross-checks)                        */
  int32_t reserved;
} opyx_rof_problem;

typedef struct {
  void* x;              /* (N, C) primal iterate, updated in place           */
  void* xbar;           /* (N, C) extrapolated primal                        */
  void* y;              /* (N, D, C) dual iterate, updated in place          */
  const void* f;        /* (N, C) data                                       */
  const uint8_t* mask;  /* (N) SSD mask or NULL                              */
  void* xgrad;          /* (N, C) adaptive steps only: A^T y (else NULL)     */
  void* gp;             /* (N, C) adaptive steps only: residual part         */
  void* ws;             /* workspace of opyx_rof_workspace_size() bytes,
                           256-byte aligned, zero-filled once before its
                           first use                                         */
  void* y2;             /* (N, D, C) or NULL.  Given, 2-D FP32 problems with
                           constant or preconditioned steps run each
                           iteration as ONE sweep over HBM (xbar kept on
                           chip), ping-ponging x <-> xbar and y <-> y2; after
                           opyx_rof_iterate returns, x and y hold the state
                           as without it (an odd count ends with one
                           two-pass iteration)                               */
} opyx_rof_buffers;

/* Values of the last opyx_rof_gap (pdhg.py:23-44) and of the step state.
 * `checks` counts the gap evaluations since opyx_rof_init; `done` becomes 1
 * at the first one that passes the stop test of the problem's term_mode,
 * after which every opyx_rof_* kernel returns at once (so the host may queue
 * iterations ahead of its checks).  `fault` becomes 1 (and `done` with it)
 * if a kernel gave up a bounded wait for its own asynchronous copies; the
 * iterates are then not valid. */
typedef struct {
  double objp, objd, infeasp, infeasd, gap, relgap;
  double tau, sigma, alpha, resp, resd, epsp, epsd;
  double checks, done, fault;
} opyx_rof_info;

size_t opyx_rof_workspace_size(void);
/* Byte offset of the opyx_rof_info record inside the workspace. */
size_t opyx_rof_info_offset(void);
/* Validate and set up: device step state from `p`; for adaptive steps also
 * xgrad = A^T y of the initial y.  x, y hold the starting point. */
int opyx_rof_init(const opyx_rof_problem* p, const opyx_rof_buffers* b, void* stream);
/* Run `iters` PDHG iterations (pdhg.py:124-187). */
/* 1 if opyx_rof_iterate runs single sweeps for this problem and buffers
 * (FP32, constant or preconditioned steps, y2 given; 2-D, or 3-D with one
 * channel, rows of 128, 256 or 512 pixels and no mask), else 0. */
int opyx_rof_uses_sweep(const opyx_rof_problem* p, const opyx_rof_buffers* b);
int opyx_rof_iterate(const opyx_rof_problem* p, const opyx_rof_buffers* b, int iters,
                     void* stream);
/* One pass of an iteration (0 = primal pass A, 1 = dual pass B, 2 = the
 * adaptive residual pass R, 3 = one single-sweep iteration (x, y) -> (xbar,
 * y2), which needs y2), for per-kernel timing and profiling. */
int opyx_rof_pass(const opyx_rof_problem* p, const opyx_rof_buffers* b, int which,
                  void* stream);
/* Batched solves (the reference solves one problem per PDHG object; a batch
 * serves workloads of many independent images, e.g. a data set): 2-D FP32
 * problems with constant or preconditioned steps, all with the same channel
 * count, their buffers as for the single sweep (x, xbar, y, y2, f; ws unused).
 * One launch per iteration covers every active instance.
 *
 * records: device array of ninst * opyx_rof_batch_record_bytes() bytes
 *   (256-aligned): instance i's step state at records + i*512 and its
 *   opyx_rof_info at records + i*512 + 256 (stop test per instance's
 *   term_mode, `done`, `fault` as for single solves).
 * opyx_rof_batch_describe fills, ON THE HOST, a descriptor of
 *   opyx_rof_batch_desc_bytes(ninst, nitems) bytes: per instance its
 *   coefficients and pointers, and work items (rows_per_item rows x a
 *   column tile: the instance's rows cut into equal tiles of at most 128,
 *   256 or 512 pixels, in the width class that leaves the fewest lanes
 *   idle) for the instances with active[i] != 0 (all if active is NULL);
 *   the caller copies it to device memory and passes both copies below (the
 *   host copy for the launch shapes, the device copy to the kernels).
 *   *nitems receives the work item count; with host_desc NULL and
 *   host_bytes 0 (or any buffer too small) the call returns
 *   OPYX_ERR_WORKSPACE after setting it, so a first call sizes the buffer.
 *   An item's tile spans [q_beg, q_end) of its rows; the sweep stores
 *   nothing past q_end.
 * opyx_rof_batch_init writes every instance's step state and clears its info.
 * opyx_rof_batch_iterate runs `iters` (even) iterations of the active items.
 * opyx_rof_batch_gap evaluates the gap of every instance with items, using
 *   `partials` (device, nitems * 5 doubles). */
size_t opyx_rof_batch_record_bytes(void);
size_t opyx_rof_batch_desc_bytes(int ninst, int nitems);
int opyx_rof_batch_describe(const opyx_rof_problem* probs, const opyx_rof_buffers* bufs,
                            int ninst, void* records, const uint8_t* active, int rows_per_item,
                            void* host_desc, size_t host_bytes, int* nitems);
int opyx_rof_batch_init(const void* host_desc, const void* dev_desc, void* stream);
int opyx_rof_batch_iterate(const void* host_desc, const void* dev_desc, int iters, void* stream);
/* The iterations of one tile-width class (0: 128, 1: 256, 2: 512 pixels):
 * classes hold disjoint instances, so a caller may run them on separate
 * streams and join before the gap. */
int opyx_rof_batch_iterate_class(const void* host_desc, const void* dev_desc, int cls, int iters,
                                 void* stream);
int opyx_rof_batch_gap(const void* host_desc, const void* dev_desc, double* partials,
                       void* stream);

/* Persistent batched solve of one-channel instances with constant or
 * preconditioned steps (all alike): ONE cooperative launch runs `maxiter`
 * (even) iterations of every instance of the descriptor, checks the gap of
 * the active ones every `gran` (even) iterations and retires each instance
 * at its own stop test (the reference's per-solve loop, pdhg.py:287-305,
 * for every instance of the batch; each reference solve is one PDHG
 * object).  Work items are strips of 128 pixels by runs of rows_per_item
 * rows (the descriptor's), taken by warps from a counter every iteration;
 * a grid barrier separates the iterations.  Iterates equal those of the
 * single-image solve bit for bit.  ws: device memory of
 * opyx_rof_batch_persist_ws_bytes(host_desc) bytes, 256-byte aligned; it
 * starts with the control record opyx_rof_persist_ctl (cleared by the call;
 * after the launch `error` != 0 means a barrier timed out -- every wait is
 * bounded -- `nact`/`nwork` are the instances / sweep items still active and
 * `iters` the iterations at the last check).  When few instances remain the
 * sweep items get fewer rows (rows_per_item halved down to 2) so that every
 * warp keeps several; the gap uses strips of rows_per_item rows.  Call opyx_rof_batch_init
 * first.  The info records hold each instance's objectives, check count
 * and stop flag as for opyx_rof_batch_gap. */
typedef struct {
  uint64_t arrive;
  uint32_t grab[4];
  int32_t error, nact, nwork, iters;
  int32_t rows, nwork_gap;    /* rows of the current sweep items; gap strips */
} opyx_rof_persist_ctl;
size_t opyx_rof_batch_persist_ws_bytes(const void* host_desc);
int opyx_rof_batch_persist(const void* host_desc, const void* dev_desc, void* ws, int gran,
                           int maxiter, void* stream);

/* Allocation-free variant of opyx_rof_init + opyx_rof_iterate (+ opyx_rof_gap).
 * It has no counterpart in the reference: it serves callers that cannot
 * allocate device memory (code running inside another framework's memory
 * pool, or hosts that only receive device pointers for f, x and y).  The
 * scratch -- step/info/reduction workspace, xbar and, for adaptive steps,
 * A^T y and the residual part -- is a file-scope __device__ array of
 * OPYX_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * the process exits.  Limit: the workspace (about 161 KiB) plus one
 * (const / precond) or three (adaptive) N*C iterate arrays must fit, e.g.
 * N*C <= 8,347,456 FP32 values for precond steps; larger problems return
 * OPYX_ERR_SCRATCH_LIMIT before any launch.  Each call starts a fresh
 * segment from the x, y it is given (step state from `p`), runs `iters`
 * iterations and, if `gap_out` (device double[6]) is not NULL, writes
 * objp, objd, infeasp, infeasd, gap, relgap there.  It always runs the
 * two-pass iteration (pass A, pass B per iteration): the single sweep needs a
 * second y buffer, which this entry point does not hold, so FP32 const and
 * precond problems run at the two passes' speed rather than the sweep's.
 * Dims whose product overflows (N * D * C above 2^40) also return
 * OPYX_ERR_SCRATCH_LIMIT.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress); make
 * that first call before any stream capture.  All calls share the one
 * array: calls that overlap on the GPU (other streams, other threads) race. */
#define OPYX_NOALLOC_SCRATCH_BYTES (32u << 20)
int opyx_rof_iterate_noalloc(const opyx_rof_problem* p, void* x, void* y, const void* f,
                             const uint8_t* mask, int iters, double* gap_out, void* stream);
/* Primal-dual gap of the current iterate into the workspace's info record
 * (FP64 device reductions; pdhg.py:23-44, :287-305). */
int opyx_rof_gap(const opyx_rof_problem* p, const opyx_rof_buffers* b, void* stream);
/* opyx_rof_gap followed by opyx_rof_iterate(iters): the check at the end of
 * one granularity chunk (pdhg.py:285-305) queued with the iterations of the
 * next.  With single sweeps (iters >= 2) the first sweep computes the gap of
 * the state it reads from the rows it loads anyway -- no pass over HBM of its
 * own -- and writes its iteration into the second buffers, so when the stop
 * test passes, x and y keep the checked state and the later launches return
 * at once, as after the two calls.  The info record then equals the two
 * calls' up to the order of the FP64 sums. */
int opyx_rof_gap_iterate(const opyx_rof_problem* p, const opyx_rof_buffers* b, int iters,
                         void* stream);


/* ---- Learned warm start: U-Net kernels (BF16 tensor cores, FP32 accumulation) ----
 * Activations are NHWC bf16 with `stride` channels per pixel; a layer reads
 * or writes the channel slice [offset, offset + channels).  3x3 convolutions
 * are implicit GEMMs on the tcgen05 tensor cores (TMEM accumulators, TMA
 * operand copies): 128-pixel tiles of one or more whole rows, so
 * min(width, 128) must divide 128 and the width, and 128 / min(width, 128)
 * the height.  Weights are bf16 [9][out_channels][in_channels] (tap = 3 *
 * (dy + 1) + (dx + 1)).  No counterpart in the reference (its solvers start
 * from zero or from `continue_at`, opymize/solvers/pdhg.py:229-255). */
enum { OPYX_CONV_GELU = 0, OPYX_CONV_F32 = 1, OPYX_CONV_BF16 = 2 };

typedef struct {
  int32_t batch, height, width;
  int32_t in_channels, in_stride, in_offset;    /* in_channels a multiple of 32 */
  int32_t out_channels, out_stride, out_offset; /* out_channels 32, 64, 128 or 256 */
  int32_t epilogue;   /* GELU: y = gelu(acc + bias) bf16 and z = acc + bias (bf16, dense,
                         if z != NULL); F32: y (+)= acc + bias as fp32; BF16: y = acc + bias */
  int32_t accumulate; /* F32 epilogue: add into y */
  const void* x;      /* bf16 activations */
  const void* w;      /* bf16 weights */
  const float* bias;  /* [out_channels] or NULL */
  void* y;
  void* z;
} opyx_conv3x3_desc;

int opyx_conv3x3(const opyx_conv3x3_desc* d, void* stream);
/* dw[tap][co][ci] (+)= sum_p x[p + offset(tap), ci] * dy[p, co] (fp32), dy
 * dense bf16 [batch, height, width, out_channels] (32, 64 or 128). */
size_t opyx_conv3x3_wgrad_workspace(const opyx_conv3x3_desc* d);
int opyx_conv3x3_wgrad(const opyx_conv3x3_desc* d, const void* dy, float* dw, int accumulate,
                       void* ws, size_t ws_bytes, void* stream);
/* Sticky flag set by a network kernel that gave up a bounded wait. */
int opyx_net_fault(unsigned* out);
/* dz = da * gelu'(z) (bf16, dense), dbias (+)= column sums of dz. */
size_t opyx_gelu_bwd_workspace(int64_t npix, int C);
int opyx_gelu_bwd(int64_t npix, int C, const float* da, int da_stride, int da_off, const void* z,
                  void* dz, float* dbias, int accumulate, void* ws, size_t ws_bytes, void* stream);
int opyx_pool2(int B, int H, int W, int C, const void* x, int xs, int xo, void* y, void* stream);
int opyx_pool2_bwd(int B, int H, int W, int C, const float* dy, float* dx, int dxs, int dxo,
                   int accumulate, void* stream);
int opyx_up2(int B, int h, int w, int C, const void* x, void* y, int ys, int yo, void* stream);
int opyx_up2_bwd(int B, int h, int w, int C, const float* dy, int dys, int dyo, float* dx,
                 void* stream);
/* Input channels: f, lambda * lam_scale (per image), zeros up to 32 (bf16). */
int opyx_pack_input(int B, int64_t hw, const float* f, const float* lam, double lam_scale, void* x,
                    void* stream);
/* Input of the restart mode: f, lambda * lam_scale, xb - f, yb / lambda
 * (2 channels), zeros up to 32 (xb, yb: the current PDHG iterate). */
int opyx_pack_input_state(int B, int64_t hw, const float* f, const float* lam, double lam_scale,
                          const float* xb, const float* yb, void* x, void* stream);
/* 1x1 head to K = 3 outputs (fp32) and its backward. */
int opyx_head(int64_t npix, int K, const void* a, const float* w, const float* b, float* out,
              void* stream);
size_t opyx_head_bwd_workspace(int64_t npix, int K);
int opyx_head_bwd(int64_t npix, int K, const void* a, const float* w, const float* dout, float* da,
                  float* dw, float* db, void* ws, size_t ws_bytes, void* stream);
/* Weighted mean squared error: grad = 2 wk (pred - tgt) / n, per-block loss partials (fp64). */
int opyx_mse(int64_t n, int K, const float* pred, const float* tgt, const float* wk, float* grad,
             double* partials, int nparts, void* stream);
/* Warm-start loss on head outputs out = (x - f, y / lambda) against targets:
 * (1/n) sum w_x (o0 - t0)^2 + w_div (lambda div(o12 - t12))^2 + w_u |o12 - t12|^2
 * + w_pool (4096/n) sum over 8x8 blocks of (block mean of o0 - t0)^2 + (block
 * mean of lambda div(o12 - t12))^2, with div adjoint to the forward gradient;
 * writes d loss / d out (grad) and per-block loss partials; scratch holds
 * B*H*W + B*H*W/32 floats (H, W multiples of 8 when w_pool != 0). */
int opyx_warm_loss(int B, int H, int W, const float* out, const float* tgt, const float* lam,
                   double w_x, double w_div, double w_u, double w_pool, float* grad, float* scratch,
                   double* partials, int nparts, void* stream);
/* Proposal from head outputs: x0 = f + o0, y0 = lambda * o12 / max(1, |o12|). */
int opyx_warm_unpack(int B, int64_t hw, const float* f, const float* lam, const float* out, float* x0,
                     float* y0, void* stream);
/* Correction of an iterate (xb, yb): x0 = xb + o0, y0 = lambda * o12' / max(1, |o12'|)
 * with o12' = yb / lambda + o12. */
int opyx_warm_unpack_rel(int B, int64_t hw, const float* xb, const float* yb, const float* lam,
                         const float* out, float* x0, float* y0, void* stream);
/* Adam step on fp32 weights; wb / wt (optional): bf16 copy, and the
 * tap-flipped [9][in][out] copy for input-gradient convolutions. */
int opyx_adam(int64_t n, float* w, const float* g, float* m, float* v, double lr, double b1, double b2,
              double eps, int step, void* wb, void* wt, int cin, int cout, void* stream);
int opyx_conv_weights(int cin, int cout, const float* w, void* wb, void* wt, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* OPYX_H */
