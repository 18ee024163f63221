/*
 * shenfun_gb300 C ABI: GB300 (sm_103a) kernels for the tensor-product
 * spectral-Galerkin forward / banded-solve / backward path of shenfun.
 *
 * Conventions
 *  - Every pointer argument named in/out/u/b/d0/... is a DEVICE pointer to
 *    C-contiguous FP64 (or interleaved complex FP64) data.  The caller owns all
 *    memory.  Plan and problem creation allocate their tables once; the
 *    sgpu_*_workspace_size queries return the scratch an execution needs, and
 *    the *_ws / _noalloc entry points allocate nothing.  Entry points that
 *    need scratch without taking it from the caller say so (stream-ordered
 *    cudaMallocAsync on the call's stream).
 *  - An N-D array is handed over as a 3-D view (outer, n, inner) around the
 *    axis being transformed or solved: element (o, k, i) lives at
 *    o*n*inner + k*inner + i.  This covers every axis of a C-contiguous array
 *    (outer = product of the dims before the axis, inner = after it), which is
 *    how the reference's `axis` argument is mapped.
 *  - Scale arrays (alpha, beta) have one entry per system, laid out as
 *    (outer, inner) - the reference's broadcast shape with the solve axis
 *    collapsed to 1.
 *  - Every entry point returns an int status (0 = ok); none throws.  Kernels
 *    are enqueued on `stream` (0 = legacy default stream) and are asynchronous.
 *
 * Each declaration cites the reference (shenfun 4.3.0) interface it replaces;
 * paths are inside the reference project.
 */
#ifndef SHENFUN_GB300_H
#define SHENFUN_GB300_H

#include <stdint.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SGPU_OK 0
#define SGPU_ERR_ARG 1          /* bad shape / pointer / enum            */
#define SGPU_ERR_UNSUPPORTED 2  /* valid request this library does not do */
#define SGPU_ERR_CUDA 3         /* a CUDA runtime call failed            */
#define SGPU_ERR_NOMEM 4        /* plan tables could not be allocated    */
#define SGPU_ERR_NONFINITE 5    /* non-finite value detected in input    */
#define SGPU_ERR_ZERO_PIVOT 6   /* zero pivot in a factorisation         */
#define SGPU_ERR_TIMEOUT 7      /* a bounded device wait ran out         */
#define SGPU_ERR_SCRATCH_LIMIT 8 /* problem too large for the built-in scratch */

/* data kinds */
#define SGPU_REAL 0     /* float64                     */
#define SGPU_COMPLEX 1  /* complex128 (re, im interleaved) */

/* 1D bases of the Chebyshev / Legendre families */
#define SGPU_BASIS_ORTHO 0  /* T_k (Chebyshev) / L_k (Legendre)        */
#define SGPU_BASIS_SD 1     /* ShenDirichlet  phi_k = P_k - P_{k+2}    */
#define SGPU_BASIS_SB 2     /* ShenBiharmonic (chebyshev/bases.py:1249) */
#define SGPU_BASIS_SN 3     /* ShenNeumann phi_k = T_k - (k/(k+2))^2 T_{k+2}
                               (chebyshev/bases.py:863-937), Chebyshev only */
/* flag OR'ed into SGPU_BASIS_SD / SGPU_BASIS_SN: non-homogeneous boundary
 * values.  A SGPU_XF_CHEB_BACKWARD plan then adds the boundary functions of
 * the last two coefficients (the boundary dofs) of every line, SD
 * (T0 -/+ T1)/2 and SN T1/2 -/+ T2/8 (BoundaryValues._add_to_orthogonal,
 * tensorproductspace.py:2072-2089); the other kinds ignore the flag (the
 * forward lift is sgpu_bc_apply). */
#define SGPU_BASIS_BC 0x10

/* transform kinds */
#define SGPU_XF_R2C 1        /* rfft along axis, n -> n/2+1 (FFTW r2c)             */
#define SGPU_XF_C2R 2        /* irfft along axis, n/2+1 -> n, unnormalised (c2r)   */
#define SGPU_XF_C2C_FWD 3    /* fft along axis (FFTW_FORWARD)                      */
#define SGPU_XF_C2C_BWD 4    /* ifft along axis, unnormalised (FFTW_BACKWARD)      */
#define SGPU_XF_DCT2 5       /* FFTW REDFT10                                       */
#define SGPU_XF_DCT3 6       /* FFTW REDFT01                                       */
#define SGPU_XF_CHEB_SCALAR 7   /* Chebyshev GC scalar product of a basis      */
#define SGPU_XF_CHEB_FORWARD 8  /* scalar product + inverse mass (forward)     */
#define SGPU_XF_CHEB_BACKWARD 9 /* to_ortho + GC backward                      */

/* arithmetic form */
#define SGPU_PLAIN_F64 0   /* all FP64                                        */
#define SGPU_FP32_REFINED 2 /* banded solves only: FP32 factor cache and sweeps,
                              FP64-level residual, iterative refinement */
#define SGPU_MIXED_DF 1    /* the mixed form, FP64 in and out: double-float (FP32
                              pair, ~48-bit) arithmetic on the FP32 pipes for
                              the Fourier line transforms and for Chebyshev
                              lines outside 16..1024; BF16 digit slices on the
                              tensor cores for the Chebyshev composite
                              transforms of 16..1024 points (8 digits, ~1e-15
                              normwise) and the Legendre contractions (7
                              digits, ~1e-13; N <= 8192 in K chunks of 1024) */

const char* sgpu_status_string(int status);
int sgpu_version(void);
/* 1 if the library was built with device code for sm_103a and a device is visible */
int sgpu_device_ok(void);

/* ---- transform plans ----------------------------------------------------
 * Replace the per-axis serial plan objects created in the bases' plan()
 * (mpi4py_fft.fftw.dctn/rfftn/irfftn/fftn/ifftn; chebyshev/bases.py:407-469,
 * fourier/bases.py:218-279) together with the scaling and Shen-stencil work
 * the reference does around them:
 *   SGPU_XF_R2C / C2C_FWD   = FourierBase._evaluate_scalar_product (fourier/bases.py:157-162) when scale = 1/n
 *   SGPU_XF_C2R / C2C_BWD   = R2C/C2C._evaluate_expansion_all (fourier/bases.py:380-407, 526-533)
 *   SGPU_XF_CHEB_SCALAR     = Orthogonal._evaluate_scalar_product (chebyshev/bases.py:340-347)
 *                             + CompositeBase._evaluate_scalar_product (spectralbase.py:1462-1474)
 *   SGPU_XF_CHEB_FORWARD    = SpectralBase.forward (spectralbase.py:235-263), homogeneous BCs
 *   SGPU_XF_CHEB_BACKWARD   = CompositeBase._evaluate_expansion_all (spectralbase.py:1450-1460)
 *                             + Orthogonal._evaluate_expansion_all (chebyshev/bases.py:315-329)
 * `scale` multiplies the result of the raw kinds (1 = FFTW's unnormalised
 * output); the Chebyshev kinds ignore it (their scaling is the reference's).
 */
typedef struct sgpu_plan sgpu_plan;
int sgpu_plan_create(sgpu_plan** plan, int kind, int n, int basis, int form);
int sgpu_plan_destroy(sgpu_plan* plan);
/* in: (outer, n_in, inner), out: (outer, n_out, inner).  data_kind applies to
 * the Chebyshev/DCT kinds (real or complex lines); Fourier kinds fix it. */
int sgpu_plan_execute(const sgpu_plan* plan, const void* in, void* out, int64_t outer,
                      int64_t inner, int data_kind, double scale, cudaStream_t stream);
/* In the mixed form the Chebyshev kinds with 16 <= n <= 1024 run as a
 * split-BF16 contraction on the tensor cores, which needs device scratch:
 * sgpu_plan_workspace_size gives its size (0 for every other plan) and
 * sgpu_plan_execute_ws takes it from the caller (256-byte aligned);
 * sgpu_plan_execute takes it from cudaMallocAsync on `stream` for the call. */
int sgpu_plan_workspace_size(const sgpu_plan* plan, int64_t outer, int64_t inner, int data_kind,
                             size_t* bytes);
int sgpu_plan_execute_ws(const sgpu_plan* plan, const void* in, void* out, int64_t outer,
                         int64_t inner, int data_kind, double scale, void* work, size_t work_bytes,
                         cudaStream_t stream);
/* The same for a stack of independent arrays of pair_lines lines each
 * (outer x inner = their total): real lines are transformed two at a time as
 * one complex line, and here the pairs never cross a block of pair_lines
 * lines, so every array of the stack gets the bits it gets alone
 * (pair_lines = 0: one block, as sgpu_plan_execute_ws). */
int sgpu_plan_execute_blocks(const sgpu_plan* plan, const void* in, void* out, int64_t outer, int64_t inner,
                             int data_kind, double scale, void* work, size_t work_bytes, int64_t pair_lines,
                             cudaStream_t stream);
/* Mixed-form Chebyshev plans with 16 <= n whose operator uses at most 339
 * input entries (n <= 339; backward transforms n <= 341) run contiguous lines
 * (inner = 1) through a fused kernel that splits the lines into digits on
 * the fly; its scratch is 4 bytes per line (the line scales).  For n > 130
 * it does not run
 * in place: sgpu_plan_execute_ws returns SGPU_ERR_ARG for in == out there,
 * and sgpu_plan_execute goes through a stream-ordered temporary output. */
/* Kernel variant of a plan.  Fused-contraction plans: 1 = 64-line tiles with
 * one TMEM accumulator set, 2 = 32-line tiles with two (the next tile's MMAs
 * overlap this tile's epilogue).  Length-256 Fourier plans (R2C, C2R, C2C):
 * 1 = the strided-pass kernel for axes with inner >= 16 (pass 1 and pass 2
 * of a 16 x 16 register FFT reading and writing global memory directly, one
 * shared-memory transpose) in its default arithmetic and occupancy (FP64,
 * or the mixed form in 64-bit fixed point, at 2 CTAs per SM; fixed-point
 * R2C / C2R transform each real line as a half-length complex FFT), 2 = the
 * generic line programs, 3 / 4 = the
 * strided-pass kernel at 2 / 3 CTAs per SM in FP64 (plain form) or
 * double-float (mixed form), 5 / 6 = the mixed form in 64-bit fixed point
 * at 2 / 3 CTAs per SM (SGPU_ERR_UNSUPPORTED for the plain form; complex
 * arrays that are not 16-byte aligned run the generic programs), 7 = C2C
 * plans only: variant 5 with each CTA's input tile (its 16 lines x 256
 * points) staged in shared memory by one tensor copy (cp.async.bulk.tensor)
 * where the lines of a CTA lie in one outer block, else variant 5; the same
 * bits as 5.  0 = the
 * library's default (1).  SGPU_ERR_UNSUPPORTED for other plans; get returns
 * 0 for them.  No counterpart in the reference (a tuning knob of this
 * library's kernels). */
int sgpu_plan_set_variant(sgpu_plan* plan, int variant);
int sgpu_plan_get_variant(const sgpu_plan* plan, int* variant);

/* ---- padded (3/2-rule dealiased) Fourier transforms ---------------------
 * FourierBase._padding_backward / _truncation_forward (fourier/bases.py:409-435
 * R2C, :570-598 C2C) on complex (outer, n, inner) arrays: pad N spectral
 * coefficients (N/2+1 for R2C) to M (M/2+1), or truncate M back to N, with the
 * reference's handling of an even N's Nyquist coefficient.  kind is
 * SGPU_XF_R2C/C2R or SGPU_XF_C2C_FWD/BWD; in and out must not alias.  A padded
 * backward transform is pad + the length-M plan; a padded forward one is the
 * length-M plan with scale 1/M + truncate. */
int sgpu_fourier_pad(const void* in, void* out, int64_t outer, int N, int M, int64_t inner, int kind,
                     cudaStream_t stream);
int sgpu_fourier_truncate(const void* in, void* out, int64_t outer, int N, int M, int64_t inner, int kind,
                          cudaStream_t stream);

/* ---- the other banded solvers of the dispatch list: DiagMA (offsets 0),
 * TwoDMA (0, 2), ThreeDMA (0, 2, 4), FDMA (-2, 0, 2, 4), HeptaDMA
 * (-4 .. 8) (la.py:291-800; la.pyx DiagMA/TwoDMA/ThreeDMA/FDMA/HeptaDMA
 * _LU / _Solve) --------------------------------------------------------------
 * data: ndiag rows of n in the reference's column-aligned (scipy DIA)
 * layout, row r holding M[i][i + offsets[r]] at column i + offsets[r];
 * offsets (host array) ascending, containing 0 and every even value between
 * the first and the last, or every value (consecutive: TDMA_O's -1, 0, 1).  LU in place without pivoting; the solve
 * runs along the middle axis of u (outer, n, inner), in place. */
int sgpu_banded_LU(double* data, int ndiag, const int* offsets, int64_t n, cudaStream_t stream);
int sgpu_banded_Solve(void* u, const double* data, int ndiag, const int* offsets, int64_t outer,
                      int64_t n, int64_t inner, int data_kind, cudaStream_t stream);

/* ---- banded solvers (optimization/cython/la.pyx) ------------------------
 * TDMA: offsets (-2, 0, 2); data is (3, n): data[0,:-2] = ld, data[1] = d,
 * data[2,2:] = ud (la.py:331-393).  PDMA: offsets (-4..4) in (5, n) rows
 * a, b, d, e, f with the same offset convention (la.py:450-543).
 */
/* la.pyx:243 TDMA_LU(data) - in place */
int sgpu_TDMA_LU(double* data, int64_t n, cudaStream_t stream);
/* la.pyx:77 TDMA_Solve(u, data, axis) + TDMA_inner_solve_ptr (la.pyx:516-532) */
int sgpu_TDMA_Solve(void* u, const double* data, int64_t outer, int64_t n, int64_t inner,
                    int data_kind, cudaStream_t stream);
/* la.pyx:213 PDMA_LU(data) - in place */
int sgpu_PDMA_LU(double* data, int64_t n, cudaStream_t stream);
/* la.pyx:61 PDMA_Solve(u, data, axis) + PDMA_inner_solve_ptr (la.pyx:496-514) */
int sgpu_PDMA_Solve(void* u, const double* data, int64_t outer, int64_t n, int64_t inner,
                    int data_kind, cudaStream_t stream);

/* ---- Chebyshev Dirichlet / Neumann Helmholtz (chebyshev/la.py:131-351) ----
 * (alfa A + beta B) u = b with A = ASDSD, B = BSDSD of a ShenDirichlet space
 * (neumann = 0) or A = ASNSN, B = BSNSN of a ShenNeumann space (neumann = 1)
 * of N modes, one system per (outer, inner) index.  Factor arrays d0, d1, d2,
 * L have the reference's layout (outer, N, inner).  The Neumann branch
 * follows la.pyx:735-751 and 907-912: columns j >= 1 scaled by 1/j^2, a pure
 * stiffness system (|beta| < 1e-8) solved with u_0 = 0.
 */
/* la.pyx:708 LU_Helmholtz(A, B, As, Bs, neumann, d0, d1, d2, L, axis) */
int sgpu_LU_Helmholtz(int64_t N, const double* alfa, const double* beta, int neumann,
                      double* d0, double* d1, double* d2, double* L, int64_t outer,
                      int64_t inner, cudaStream_t stream);
/* la.pyx:845 Solve_Helmholtz(b, u, neumann, d0, d1, d2, L, axis) */
int sgpu_Solve_Helmholtz(const void* b, void* u, int neumann, const double* d0,
                         const double* d1, const double* d2, const double* L,
                         int64_t outer, int64_t N, int64_t inner, int data_kind,
                         cudaStream_t stream);
/* Matvec.pyx:697 Helmholtz_matvec(v, b, alfa, beta, A, B, axis): b = (alfa A + beta B) v */
int sgpu_Helmholtz_matvec(const void* v, void* b, const double* alfa, const double* beta,
                          int64_t outer, int64_t N, int64_t inner, int data_kind,
                          cudaStream_t stream);
/* Matvec.pyx:769 Helmholtz_Neumann_matvec(v, b, alfa, beta, A, B, axis):
 * b = (alfa ASNSN + beta BSNSN) v on the N-2 dofs, the two tail entries zero */
int sgpu_Helmholtz_Neumann_matvec(const void* v, void* b, const double* alfa,
                                  const double* beta, int64_t outer, int64_t N, int64_t inner,
                                  int data_kind, cudaStream_t stream);

/* ---- non-homogeneous boundary values (tensorproductspace.py:1909-2128) ----
 * For every line of u (outer, N, inner) along a Chebyshev SD / SN axis, with
 * boundary values g0, g1 = g[o][0|1][i] (g has u's element type):
 *   u[k] -= (alfa_s CA[k][0] + beta_s CB[k][0]) g0 + (... [1]) g1, k < N-2,
 * CA, CB row-major (N-2) x 2 (either may be NULL; alfa / beta NULL mean 1),
 * s = o * inner + i; then, if set_dofs, u[N-2] = g0, u[N-1] = g1.
 * The forward lift (BoundaryValues._add_mass_rhs followed by the mass solve)
 * is CA = B^-1 B_bc; the Helmholtz right-hand side (the boundary matrices of
 * chebyshev.la.Helmholtz.__call__) is CA = A_bc, CB = B_bc with the solver's
 * scales. */
int sgpu_bc_apply(void* u, const double* CA, const double* alfa, const double* CB,
                  const double* beta, const void* g, int64_t outer, int64_t N, int64_t inner,
                  int set_dofs, int data_kind, cudaStream_t stream);

/* ---- Chebyshev Poisson solvers along one axis ------------------------------
 * la.pyx:614 Poisson_Solve_ADD(A, b, u, axis) / chebyshev/la.py:11 ADDSolver:
 * scale * ASDSD u = b on the N-2 dofs of a ShenDirichlet axis (N modes);
 * the two boundary dofs of u are set to 0.  b may alias u. */
int sgpu_Poisson_Solve_ADD(const void* b, void* u, double scale, int64_t outer, int64_t N,
                           int64_t inner, int data_kind, cudaStream_t stream);
/* chebyshev/la.py:74 ANNSolver.__call__(b, u, axis, constraints=((0, u0),)):
 * scale * ASNSN u = b on a ShenNeumann axis; u_0 = u0 (the constraint),
 * boundary dofs 0.  b may alias u. */
int sgpu_Poisson_Solve_ANN(const void* b, void* u, double scale, double u0, int64_t outer,
                           int64_t N, int64_t inner, int data_kind, cudaStream_t stream);

/* ---- Helmholtz factorisation cache (no reference counterpart as a separate
 * call: it is LU_Helmholtz's result (la.pyx:717-763) stored for the GPU) ---
 * fac holds 4 * (N-2) * outer * inner entries of 8 bytes laid out
 * [q][k][system] for q = (multiplier L, 1/d0, d1, d2): consecutive systems are
 * contiguous.  form SGPU_PLAIN_F64 stores FP64, SGPU_MIXED_DF double-float
 * pairs.  The LU is computed in FP64 in the reference's order either way. */
int sgpu_helmholtz_factor(int64_t N, const double* alfa, const double* beta, int neumann,
                          int64_t outer, int64_t inner, int form, void* fac, cudaStream_t stream);
/* form SGPU_FP32_REFINED (Dirichlet only) stores the cache as FP32: 4 bytes
 * per entry, the LU computed in FP64 and rounded once. */
/* Solve_Helmholtz (la.pyx:845-947) from the cache: b, u in the (outer, N,
 * inner) layout; one thread per (system, parity); b may alias u.  neumann
 * must match the factorisation. */
int sgpu_helmholtz_solve_cached(const void* b, void* u, const void* fac, int neumann,
                                int64_t outer, int64_t N, int64_t inner, int data_kind, int form,
                                cudaStream_t stream);

/* FP32 solve with iterative refinement (the mixed-precision form of the
 * banded solves: FP32 sweeps, FP64 residual; no reference counterpart as a
 * call: it returns the same
 * solution as Solve_Helmholtz, la.pyx:845-947, to FP64 accuracy).  One
 * thread per (system, parity) chain: u = A32^-1 b; repeat r = b - A u,
 * d = A32^-1 r, u += d until max|d| <= tol max|u| or max_it corrections.
 * fac32 from sgpu_helmholtz_factor(form = SGPU_FP32_REFINED); A = alfa ASDSD
 * + beta BSDSD with the factorisation's scales; r is scratch of b's size;
 * b, u, r distinct.  residual_form SGPU_PLAIN_F64 computes the residual in
 * FP64, SGPU_MIXED_DF in double-float on the FP32 pipes.  iters (device, 2
 * outer inner ints, may be NULL) receives each chain's correction count,
 * chain 2 s + parity.  The two tail entries of u are not written. */
int sgpu_helmholtz_solve_refined(const void* b, void* u, void* r, const void* fac32, const double* alfa,
                                 const double* beta, int64_t outer, int64_t N, int64_t inner, int data_kind,
                                 double tol, int max_it, int residual_form, int* iters, cudaStream_t stream);

/* ---- per-wavenumber systems: banded + rank-2 upper semiseparable ----------
 * M_s = sum_t coef[t][s] M_t, offsets -4..4 (even) plus, for term gen_term,
 * M[k][j] = p_k q_j + r_k t_j for j >= k+2.  Replaces la.SolverGeneric1ND's
 * per-wavenumber LU (la.py:1183-1434, SolverGeneric1ND_solve_data la.pyx:371)
 * and chebyshev.la.Biharmonic's LU_Biharmonic / Biharmonic_Solve
 * (chebyshev/la.py:354-558, la.pyx:975-1492).
 *   bands [nterms][5][n] (device): row k of offsets -4, -2, 0, 2, 4
 *   gens  [4][n] (device): p, q, r, t;   coef [nterms][nsys] (device)
 *   fac   7 * ((n+1)/2) * 2 * nsys doubles (device, caller-allocated)
 * The solve reads b and writes u in the (outer, Nb, inner) layout; the first
 * n entries along the axis are the unknowns, the rest are left untouched. */
int sgpu_band_sep_factor(int n, int nterms, int gen_term, const double* bands,
                         const double* gens, const double* coef, int64_t nsys, double* fac,
                         cudaStream_t stream);
int sgpu_band_sep_solve(const void* b, void* u, const double* fac, const double* gens, int n,
                        int64_t outer, int64_t Nb, int64_t inner, int data_kind,
                        cudaStream_t stream);
/* The same systems with an FP32 factor cache (half the bytes; LU in FP64,
 * rounded once) and FP32 sweeps refined by an FP64 residual (the matvec
 * below), as sgpu_helmholtz_solve_refined: fac 7 * ((n+1)/2) * 2 * nsys
 * floats; b, u, r distinct, r scratch of b's size; iters as there. */
int sgpu_band_sep_factor32(int n, int nterms, int gen_term, const double* bands, const double* gens,
                           const double* coef, int64_t nsys, float* fac, cudaStream_t stream);
int sgpu_band_sep_solve_refined(const void* b, void* u, void* r, const float* fac32, int n, int nterms,
                                int gen_term, const double* bands, const double* gens, const double* coef,
                                int64_t outer, int64_t Nb, int64_t inner, int data_kind, double tol, int max_it,
                                int* iters, cudaStream_t stream);
/* Matvec.pyx:908 Biharmonic_matvec (and the product of every other system
 * above): c = (sum_t coef[t][s] M_t) v per system, with the same description
 * as sgpu_band_sep_factor; v, c in the (outer, Nb, inner) layout, entries
 * k >= n zeroed; v must not alias c. */
int sgpu_band_sep_matvec(const void* v, void* c, int n, int nterms, int gen_term,
                         const double* bands, const double* gens, const double* coef,
                         int64_t outer, int64_t Nb, int64_t inner, int data_kind,
                         cudaStream_t stream);

/* ---- Helmholtz problem: the whole hot-path step in one call ----------------
 * (-lap + c) u = f on 2D R2C(N0) x D(N1) or 3D C2C(N0) x R2C(N1) x D(N2), D a
 * ShenDirichlet space (Chebyshev GC or Legendre LG) along the last axis.  One
 * solve = inner(v, f) -> H(f_hat, u_hat) -> u_hat.backward(), the sequence of
 * chebyshev/la.py:288-317 with tensorproductspace.py:45-259 around it.
 * create factorises every per-wavenumber system (device allocations happen
 * here); solve allocates nothing and uses the caller's scratch (workspace
 * size from sgpu_helmholtz_workspace_size, 256-byte aligned).  f and u are
 * physical-space FP64 arrays (C-contiguous); u may not alias the scratch. */
#define SGPU_FAMILY_CHEBYSHEV 1
#define SGPU_FAMILY_LEGENDRE 2
typedef struct sgpu_helmholtz_problem sgpu_helmholtz_problem;
int sgpu_helmholtz_create(sgpu_helmholtz_problem** problem, int ndim, const int64_t* N,
                          int family, double c, int form);
/* Stream-ordered creation for serving: the per-axis plans come from a
 * process-wide cache (shared by problems with the same axis lengths), device
 * memory comes from cudaMallocAsync on `stream` and the factorisation is left
 * queued on `stream` (no device synchronisation).  Destroying such a problem
 * frees its memory with cudaFreeAsync on the same stream. */
int sgpu_helmholtz_create_on(sgpu_helmholtz_problem** problem, int ndim, const int64_t* N,
                             int family, double c, int form, cudaStream_t stream);
/* destroy every cached plan (no problem created by _create_on may be in use) */
int sgpu_plan_cache_clear(void);
int sgpu_helmholtz_destroy(sgpu_helmholtz_problem* problem);
int sgpu_helmholtz_shape(const sgpu_helmholtz_problem* problem, int64_t* phys, int64_t* spec);
int sgpu_helmholtz_workspace_size(const sgpu_helmholtz_problem* problem, size_t* bytes);
int sgpu_helmholtz_solve(const sgpu_helmholtz_problem* problem, const double* f, double* u,
                         void* work, size_t work_bytes, cudaStream_t stream);
/* Batched step for serving: K problems of one shape, family and form
 * (different shifts c) solved together, their right-hand sides f and
 * solutions u stacked as K physical arrays.  Every transform pass runs once
 * over the stacked lines with `problem`'s plans, and one solve launch covers
 * every member's systems, member k with the factor cache facs[k] (a device
 * array of K pointers, each from sgpu_helmholtz_factor_ptr of a problem of
 * that shape).  Scratch from sgpu_helmholtz_batch_workspace_size; allocates
 * nothing, so a caller can capture it in a CUDA graph and replay it with new
 * right-hand sides and a new factor table.  Results equal K single solves
 * bit for bit.  No counterpart in the reference. */
int sgpu_helmholtz_batch_workspace_size(const sgpu_helmholtz_problem* problem, int K, size_t* bytes);
int sgpu_helmholtz_factor_ptr(const sgpu_helmholtz_problem* problem, const void** fac);
/* The transform plans of a problem's step, in order: Dirichlet-axis scalar
 * product, R2C forward, C2C forward, C2C backward, C2R backward,
 * Dirichlet-axis backward (null where the grid has no such pass or the family
 * is Legendre), and each pass's (outer, inner) in lines[2 i], lines[2 i + 1];
 * for tuning their kernel variants (sgpu_plan_set_variant). */
int sgpu_helmholtz_plan_handles(const sgpu_helmholtz_problem* problem, sgpu_plan** plans, int64_t* lines);
int sgpu_helmholtz_solve_batch(const sgpu_helmholtz_problem* problem, int K, const void* const* facs,
                               const double* f, double* u, void* work, size_t work_bytes, cudaStream_t stream);
/* the batched solves under it: systems of member k at b + k nsys N (nsys =
 * outer x inner per member) with factor cache facs[k] (device array) */
int sgpu_helmholtz_solve_cached_batch(const void* b, void* u, const void* const* facs, int K, int neumann,
                                      int64_t outer, int64_t N, int64_t inner, int data_kind, int form,
                                      cudaStream_t stream);
int sgpu_band_sep_solve_batch(const void* b, void* u, const double* const* facs, const double* gens, int K,
                              int n, int64_t outer, int64_t Nb, int64_t inner, int data_kind, cudaStream_t stream);
/* Same step without any scratch argument, for callers that cannot provide or
 * allocate device memory (a host program whose device memory belongs to
 * another allocator, an FFI caller that only has its input and output arrays,
 * a loop that must not allocate).  No counterpart in the reference.  It uses a
 * 64 MiB scratch array built into the library (held on every GPU that loads
 * the library until exit); larger problems return SGPU_ERR_SCRATCH_LIMIT.  The
 * first call on a device looks up the array's address (make it before any
 * stream capture); all calls share the array, so calls that overlap on the
 * GPU race and must be serialised.  Allocates nothing. */
int sgpu_helmholtz_solve_noalloc(const sgpu_helmholtz_problem* problem, const double* f,
                                 double* u, cudaStream_t stream);

/* ---- Legendre spaces (Gauss-Legendre quadrature) --------------------------
 * Replace legendre.Orthogonal / ShenDirichlet / ShenBiharmonic's transforms
 * (legendre/bases.py:76-572): the 'recursive' kind (transforms.pyx:175-325)
 * and the 'vandermonde' kind (spectralbase.py:472-483, 539-549) are one dense
 * contraction per direction with the Shen stencil folded into the matrix.
 */
/* fastgl_wrap.pyx:31 leggauss(N): nodes ascending, weights; host pointers */
int sgpu_leggauss(int N, double* x, double* w);
typedef struct sgpu_legendre_plan sgpu_legendre_plan;
/* form SGPU_PLAIN_F64: FP64 contraction.  form SGPU_MIXED_DF: the matrices
 * are split into BF16 digit slices and contracted on the tensor cores with
 * FP32 accumulation (about 48 bits; N <= 1024, else SGPU_ERR_UNSUPPORTED). */
int sgpu_legendre_plan_create(sgpu_legendre_plan** plan, int N, int basis, int form);
int sgpu_legendre_plan_destroy(sgpu_legendre_plan* plan);
/* copy the plan's nodes and weights to host arrays of N entries */
int sgpu_legendre_nodes(const sgpu_legendre_plan* plan, double* x, double* w);
/* direction 0: scalar product (SpectralBase.scalar_product, spectralbase.py:200-233)
 *           1: forward (+ mass solve, spectralbase.py:235-263)
 *           2: backward (spectralbase.py:265-313)
 * in and out are (outer, N, inner) arrays and must not alias. */
int sgpu_legendre_execute(const sgpu_legendre_plan* plan, int direction, const void* in,
                          void* out, int64_t outer, int64_t inner, int data_kind,
                          cudaStream_t stream);
/* device scratch an execution of (outer, N, inner) lines needs (0 for the
 * plain form); the _ws entry takes it from the caller (256-byte aligned) and
 * allocates nothing.  sgpu_legendre_execute without it takes the mixed form's
 * scratch from cudaMallocAsync on `stream` for the call. */
int sgpu_legendre_workspace_size(const sgpu_legendre_plan* plan, int64_t outer, int64_t inner,
                                 int data_kind, size_t* bytes);
int sgpu_legendre_execute_ws(const sgpu_legendre_plan* plan, int direction, const void* in,
                             void* out, int64_t outer, int64_t inner, int data_kind, void* work,
                             size_t work_bytes, cudaStream_t stream);
/* number of bounded device-side waits of the tensor-core kernels that gave up
 * since load (0 unless a pipeline stalled; such a launch's output is invalid) */
int sgpu_wait_timeouts(unsigned int* count);
/* Synchronise `stream` and report whether any tensor-core launch since the
 * previous call gave up a bounded wait: SGPU_ERR_TIMEOUT (its outputs are
 * invalid), SGPU_OK, or SGPU_ERR_CUDA when the synchronisation itself
 * failed.  The kernels never trap: a pipeline that stalls past its limit
 * records the event, drains the work it issued and returns.  No counterpart
 * in the reference (its kernels are synchronous CPU code). */
int sgpu_last_error(cudaStream_t stream);
/* Limit of each pipeline wait of the fused tensor-core contraction, in
 * nanoseconds (0: the default, one second).  For tests that make a wait run
 * out; process-wide. */
int sgpu_set_wait_limit_ns(unsigned long long ns);

/* ---- reference-signature entry points (optimization/cython) ---------------
 * The kernels shenfun's optimization modules export by name, on the
 * reference's own argument arrays (device copies, same shapes and layouts),
 * so that a shenfun optimization mode can forward to them unchanged.  An
 * N-D array with the solve axis `axis` is (outer, N, inner) with outer and
 * inner the products of the dimensions before and after it.
 *
 * Chebyshev biharmonic (chebyshev/la.py:354-558): the factor arrays u0, u1,
 * u2, l0, l1, ak, bk have the reference's shape (2, outer, M, inner) (M per
 * parity; the space has N - 4 = 2M dofs); alfa, beta hold one value per
 * system (outer x inner, the scale arrays broadcast to the systems); the 11
 * diagonals are the reference's sii, siu, siuu (SBB 0, +2, +4), ail, aii,
 * aiu (ABB -2, 0, +2), bill, bil, bii, biu, biuu (BBB -4 .. +4) of lengths
 * 2M, 2M-2, 2M-4, ...  M >= 5.  The reference's row elimination is O(M^2)
 * per system; the LU here keeps each row's full upper part as two
 * coefficients (O(M)), the same factors to rounding. */
/* la.pyx:975 LU_Biharmonic(a0, alfa, beta, sii, siu, siuu, ail, aii, aiu, bill,
 * bil, bii, biu, biuu, u0, u1, u2, l0, l1, axis) */
int sgpu_LU_Biharmonic(double a0, const double* alfa, const double* beta, const double* sii,
                       const double* siu, const double* siuu, const double* ail, const double* aii,
                       const double* aiu, const double* bill, const double* bil, const double* bii,
                       const double* biu, const double* biuu, double* u0, double* u1, double* u2,
                       double* l0, double* l1, int64_t outer, int64_t M, int64_t inner, cudaStream_t stream);
/* la.pyx:1195 Biharmonic_factor_pr(ak, bk, l0, l1, axis): rows 0 .. M-3 */
int sgpu_Biharmonic_factor_pr(double* ak, double* bk, const double* l0, const double* l1, int64_t outer,
                              int64_t M, int64_t inner, cudaStream_t stream);
/* la.pyx:1235 Biharmonic_Solve(b, u, u0, u1, u2, l0, l1, ak, bk, a0, axis):
 * b, u (outer, N, inner) with 2M <= N; entries 2M .. N-1 of u are left as
 * they are; u may alias b */
int sgpu_Biharmonic_Solve(const void* b, void* u, const double* u0, const double* u1, const double* u2,
                          const double* l0, const double* l1, const double* ak, const double* bk, double a0,
                          int64_t outer, int64_t N, int64_t inner, int64_t M, int data_kind,
                          cudaStream_t stream);
/* Matvec.pyx:908 Biharmonic_matvec(v, b, a0, alfa, beta, sii, ..., biuu, axis):
 * b[0 .. M-1] = (a0 SBB + alfa ABB + beta BBB) v with M = len(sii) = N - 4 >= 10;
 * v and b must not alias */
int sgpu_Biharmonic_matvec(const void* v, void* b, double a0, const double* alfa, const double* beta,
                           const double* sii, const double* siu, const double* siuu, const double* ail,
                           const double* aii, const double* aiu, const double* bill, const double* bil,
                           const double* bii, const double* biu, const double* biuu, int64_t outer, int64_t N,
                           int64_t inner, int64_t M, int data_kind, cudaStream_t stream);

/* the *_inner_solve kernels SolverGeneric1ND_solve_data dispatches to by name
 * (la.pyx:307-325, 466-613), each reading the reference's LU'd data layout */
#define SGPU_SOL_DIAGMA 0
#define SGPU_SOL_TWODMA 1
#define SGPU_SOL_THREEDMA 2 /* reads its +4 band from the +2 row, 4 columns on (la.pyx:569-584) */
#define SGPU_SOL_TDMA 3
#define SGPU_SOL_TDMA_O 4
#define SGPU_SOL_PDMA 5
#define SGPU_SOL_FDMA 6
#define SGPU_SOL_HEPTADMA 7
/* la.pyx:371 SolverGeneric1ND_solve_data(u, data, sol, naxes, is_zero_index):
 * u (outer, N, inner) along the solve axis naxes, in place; data holds one
 * (rows, cols) LU'd matrix per system, systems in (outer, inner) order (the
 * reference's data[i, j]); the first cols entries of each line are solved;
 * is_zero_index skips system 0 (solved separately by the caller). */
int sgpu_SolverGeneric1ND_solve_data(void* u, const double* data, int sol, int is_zero_index, int64_t outer,
                                     int64_t N, int64_t inner, int64_t rows, int64_t cols, int data_kind,
                                     cudaStream_t stream);
/* la.pyx DiagMA_Solve / TwoDMA_Solve / ThreeDMA_Solve / TDMA_O_Solve /
 * FDMA_Solve / HeptaDMA_Solve(u, data, axis): one (rows, cols) LU'd matrix
 * for every line */
int sgpu_DMA_Solve(int sol, void* u, const double* data, int64_t rows, int64_t cols, int64_t outer, int64_t N,
                   int64_t inner, int data_kind, cudaStream_t stream);

/* Recursive Legendre transforms (transforms.pyx:175-216, called at
 * spectralbase.py:485-491, 551-558): x the points, w the weights, a the DIA
 * data (a_rows = 2 or 3 rows of a_cols >= N + 2) of the basis' recursion
 * matrix.  The recurrence builds the point-by-degree matrix once (one thread
 * per point, the reference's operation order), then an FP64 GEMM applies it
 * to every line; the matrix (N x Nx doubles) lives in `work` when given
 * (work_bytes >= 8 N Nx), else in cudaMallocAsync memory on `stream`.
 * input and output must not alias. */
/* scalar_product(input, output, x, w, axis, a): output[i] = sum_j P_i(x_j) w_j input[j],
 * input and output of N entries along the axis */
int sgpu_scalar_product(const void* input, void* output, const double* x, const double* w, const double* a,
                        int a_rows, int64_t a_cols, int64_t outer, int64_t N, int64_t inner, int data_kind,
                        void* work, size_t work_bytes, cudaStream_t stream);
/* evaluate_expansion_all(input, output, x, axis, a): output[j] = sum_i P_i(x_j) input[i],
 * N coefficients in, Nx points out */
int sgpu_evaluate_expansion_all(const void* input, void* output, const double* x, const double* a, int a_rows,
                                int64_t a_cols, int64_t outer, int64_t N, int64_t Nx, int64_t inner, int data_kind,
                                void* work, size_t work_bytes, cudaStream_t stream);

/* A dense matrix along an axis: out(l, k) [+]= s_l sum_j in(l, j) M[j][k] for
 * every line l = (o, i) of in (outer, Nin, inner) and out (outer, Nout,
 * inner); M is Nin x Nout (row-major, device); line_scale (optional) holds one
 * factor per line in (outer, inner) order, complex (re, im pairs) for complex
 * data; accumulate adds to out.  FP64 tiled GEMM.  Serves the generic
 * SparseMatrix solve (la.py:823-840) and projections of expressions
 * (forms/project.py:124-199), whose operators are dense along the axis. */
int sgpu_line_gemm(const void* in, void* out, const double* M, int64_t Nin, int64_t Nout, int64_t outer,
                   int64_t inner, int data_kind, const double* line_scale, int accumulate, cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* SHENFUN_GB300_H */
