/*
 * clowns_gpu.h -- C ABI of the GB300 pressure-Poisson solve for 2CLOWNS-3D.
 *
 * The library (libclowns_gpu.so, sm_103a) replaces the reference's pressure
 * correction path: the static matrix coefficients (init_matrix), the row
 * numbering and right-hand side (cal_err_of_continuity), the per-step matrix
 * assembly (cal_matrix_element), the left-preconditioned BiCGSTAB solve
 * (PCGPME) and the pressure / velocity correction.  Every entry point takes
 * plain pointers and sizes in the reference's own array layouts:
 *
 *   dims[6]   = is, js, ks, ie, je, ke  (computational cells i = is..ie-1 ...)
 *   mn        : mn(is-2:ie+2, ks-2:ke+2, js-2:je+2), int32, i fastest
 *   mno       : mno(1:ie, 1:ke, 1:je), int32, i fastest
 *   x, dx     : x(0:2, 1:mx2), component fastest
 *   in/jn/kn  : in(1:inne2) etc., passed as a pointer to element 0 (unused)
 *   nf, nfb   : nff(0:inne2+1)%f and %b as two plain int32 arrays
 *   f, fb     : f(0:inne2+1), fb(0:inne2+1)
 *   a, un     : a(0:2, 0:inne2+1), component fastest
 *   sp        : sp(0:inne2+1, 0:2), cell index fastest
 *   alu_c     : ALU_C(1:inne, 1:nl) column-major (leading dimension inne); ll_c alike
 *   alu, llu  : alu(1:na, 1:nl) column-major (leading dimension na = mm2)
 *   nl        : 6 in 3D, 4 in the 2DV mode of a grid one cell wide in x or y
 *               (clowns_grid_nl); columns 2q-1, 2q are the minus and plus faces
 *               of the q-th axis that is not one cell wide, in the order x, y, z
 *   b, de, xe : 1-based row arrays passed as a pointer to their element 1
 *               (xe(0) is not touched by the solver)
 *   fln, sfn  : fln(1:ifln) passed as a pointer to element 1
 *
 * Functions whose name ends in _dev take DEVICE pointers and a cudaStream_t
 * (as void*; NULL = legacy default stream) and allocate nothing: scratch space
 * is a caller-provided device workspace whose size a *_workspace_bytes query
 * returns.  Functions without the suffix take HOST pointers, manage device
 * memory inside the library and return when the results are back on the host.
 *
 * Return codes: 0 on success, a negative CLOWNS_ERR_* value on failure (the
 * message is available from clowns_last_error()).  Solver outcomes use the
 * reference's IER convention (0 converged or stagnated, 3000 iteration cap) plus
 * the CLOWNS_IER_* codes below, all non-zero and distinct from 3000 so that the
 * reference's caller maps them to icon = 911 and stops
 * (1sub-momentum.F90:568-587).
 */
#ifndef CLOWNS_GPU_H
#define CLOWNS_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define CLOWNS_OK 0
#define CLOWNS_ERR_CUDA (-1)      /* a CUDA runtime call failed                 */
#define CLOWNS_ERR_ARG (-2)       /* invalid argument (sizes, NULL, alignment)  */
#define CLOWNS_ERR_WORKSPACE (-3) /* workspace smaller than required            */
#define CLOWNS_ERR_NOCONV (-4)    /* a device fixed point did not settle        */
#define CLOWNS_ERR_LIMIT (-5)     /* size beyond a stated maximum               */

/* IER values beyond the reference's 0 / 3000 */
#define CLOWNS_IER_MAXITER 3000   /* iteration cap (pcgpme_para.F90:250-251)     */
#define CLOWNS_IER_NONFINITE 9101 /* RQ, SS or RN became NaN/Inf                 */
#define CLOWNS_IER_DEVICE 9102    /* CUDA failure inside the solve               */
#define CLOWNS_IER_ARG 9104       /* invalid arguments to the drop-in            */

/* Stop reasons reported by the solvers */
#define CLOWNS_STOP_TOL 0         /* ERR <= EPS(1)            (pcgpme_para.F90:232) */
#define CLOWNS_STOP_STAGNATION 1  /* |ERR-ERRP| <= 1e-6 ERR   (pcgpme_para.F90:228) */
#define CLOWNS_STOP_AMU_ZERO 2    /* AMU == 0                 (pcgpme_para.F90:234) */
#define CLOWNS_STOP_C1_ZERO 3     /* C1 == 0                  (pcgpme_para.F90:240) */
#define CLOWNS_STOP_MAXITER 4     /* loop exhausted           (pcgpme_para.F90:250) */
#define CLOWNS_STOP_NONFINITE 5   /* non-finite scalar (new, no reference counterpart) */

typedef struct clowns_solve_info {
    double eps;     /* final ERR = sqrt(RN/BN), the value PCGPME returns in EPS(1) */
    double bn;      /* BN = ||PM W b||^2                                           */
    int iter;       /* the value PCGPME returns in ITER                            */
    int ier;        /* 0, 3000 or CLOWNS_IER_*                                     */
    int reason;     /* CLOWNS_STOP_*                                               */
    int outer;      /* refinement sweeps (mixed precision), else 0                 */
} clowns_solve_info;

const char* clowns_last_error(void);
int clowns_version(void);

/* ========================================================================== */
/* PCGPME -- left-preconditioned BiCGSTAB, plain FP64                          */
/* ========================================================================== */

/* Drop-in for SUBROUTINE PCGPME(AL,NL,NA,LL,D,N,N2,B,X,EPS,PARM,ITER,IER)
 * (src2LOWNS/pcgpme_para.F90:1-354), called by cal_poisson_equation at
 * src2LOWNS/1sub-momentum.F90:564.  Same by-reference arguments, host arrays:
 *   AL(NA,NL), LL(NA,NL) column-major (LL 1-based, 0 = no neighbour), D(N),
 *   B(N), X(N+N2) (initial guess in, solution out), EPS(2) (tolerance in,
 *   final ERR out), PARM, ITER (cap in, iterations used out), IER out.
 * Differences from the reference, by design: AL, LL, D and B are left unmodified
 * (the reference scales/sorts them in place and leaves the final residual in B;
 * its only caller rebuilds all four before the next call, 1sub-momentum.F90:48
 * and 267-360), and a NaN/Inf in RQ, SS or RN ends the solve with
 * IER = CLOWNS_IER_NONFINITE instead of running on to the iteration cap. */
void pcgpme_gpu(double* al, const int* nl, const int* na, int* ll, double* d, const int* n,
                const int* n2, double* b, double* x, double* eps, const double* parm,
                int* iter, int* ier);

/* Link-level alias with the name ifort gives the Fortran subroutine, so that an
 * executable linked against this library instead of pcgpme_para.o calls the GPU
 * solve with no source change. */
void pcgpme_(double* al, const int* nl, const int* na, int* ll, double* d, const int* n,
             const int* n2, double* b, double* x, double* eps, const double* parm,
             int* iter, int* ier);

/* Device-resident variant of the same solve (replaces pcgpme_para.F90:1-354
 * when the matrix already lives in HBM, as inside the ik loop of
 * 1sub-momentum.F90:42-60).  al/ll: (na, nl) column-major device arrays,
 * d/b: length n, x: length >= n (initial guess in, solution out).  The scaled
 * and sorted copy of the matrix and all Krylov vectors live in `work`. */
size_t clowns_pcgpme_workspace_bytes(int n, int nl);
int clowns_pcgpme_dev(const double* al, int nl, int na, const int* ll, const double* d, int n,
                      const double* b, double* x, double eps, double parm, int iter,
                      void* work, size_t work_bytes, void* stream, clowns_solve_info* info);

/* ========================================================================== */
/* Mixed precision and batched ensembles (no reference counterpart: new       */
/* capabilities of the same PCGPME method)                                    */
/* ========================================================================== */

/* Precision selectors */
#define CLOWNS_PREC_FP64 0   /* plain FP64, the reference's arithmetic and stop tests  */
#define CLOWNS_PREC_MIXED 1  /* FP32 coefficients/Krylov vectors + FP64 refinement     */

/* Mixed-precision solve of the same system as clowns_pcgpme_dev.  The row scaling
 * and per-row sort are computed in FP64 exactly as the reference does; the scaled,
 * sorted coefficients and the Krylov vectors of an inner BiCGSTAB are stored in
 * FP32.  An FP64 outer loop forms r = W (b - A x) from the caller's original FP64
 * matrix, measures ERR = ||PM r|| / ||PM W b|| (the reference's EPS definition)
 * in FP64, solves PM W A d = PM r / ||PM r|| in FP32 to the relative residual
 * max(inner_tol, eps / (2 ERR)) (inner_tol <= 0: 3e-2) -- no further than the
 * outer tolerance still needs -- and accumulates x += ||PM r|| d in FP64, until
 * ERR <= eps.  info->iter counts
 * inner iterations, info->outer the refinement sweeps; IER = 3000 after
 * max_outer sweeps (<= 0: 30).  inner_max <= 0: 2000. */
size_t clowns_pcgpme_mixed_workspace_bytes(int n, int nl);
int clowns_pcgpme_mixed_dev(const double* al, int nl, int na, const int* ll, const double* d, int n,
                            const double* b, double* x, double eps, double parm, double inner_tol,
                            int inner_max, int max_outer, void* work, size_t work_bytes,
                            void* stream, clowns_solve_info* info);

/* One independent system of an ensemble (device pointers, layouts as for
 * clowns_pcgpme_dev).  x: initial guess in, solution out. */
typedef struct clowns_member {
    const double* al;
    const int* ll;
    const double* d;
    const double* b;
    double* x;
    int na, n, nl, pad;
} clowns_member;

/* Batched ensemble: m independent systems of different sizes solved together in
 * one CUDA-graph launch per solve (FP64) or per refinement sweep (mixed).  Rows of
 * all members share one tile-aligned row space; every kernel serves all members
 * and skips members whose stop test fired (per-member convergence masks);
 * dot products reduce per member.  members: HOST array of m descriptors;
 * infos: HOST array of m results.  Each member gets exactly the single-system
 * semantics of its precision. */
size_t clowns_pcgpme_batched_workspace_bytes(int m, const int* n, int precision);
int clowns_pcgpme_batched_dev(int m, const clowns_member* members, int precision, double eps,
                              double parm, int iter, double inner_tol, int inner_max, int max_outer,
                              void* work, size_t work_bytes, void* stream, clowns_solve_info* infos);

/* Execution the autotuner chose for the iteration loop of a row space (m
 * systems of sizes n[], precision as above).  mode: CLOWNS_LOOP_PERSISTENT
 * (one cooperative kernel, phases separated by grid barriers),
 * CLOWNS_LOOP_GRAPH (a CUDA graph of per-phase kernels chained by programmatic
 * dependent launch) or CLOWNS_LOOP_WAVE (one cooperative kernel running
 * (stage, tile) items in wavefront order; single systems only).  block:
 * threads per block; grid: blocks of the cooperative kernels (0 for the graph);
 * regs: their register budget per thread (0 for the graph); fused (graph): bit 0
 * set when LDUSUB's sweeps 1-2 and 3-4 run as fused pairs, bit 1 set when the
 * dot-product kernels run 64 threads per 512-row tile (8 rows per thread), bit 2
 * set when a single system runs the balanced kernels (each kernel one wave of
 * 256-thread blocks over even row ranges, one reduction per block), bit 3 set
 * when those take 8 rows per thread per step (else 4), bit 4 set when an FP32
 * single system's AXSUB has its streams staged in shared memory by bulk copies.
 * CLOWNS_ERR_ARG until a solve of that size has run. */
#define CLOWNS_LOOP_PERSISTENT 0
#define CLOWNS_LOOP_GRAPH 1
#define CLOWNS_LOOP_WAVE 3
int clowns_tuned_shape(int m, const int* n, int precision, int* mode, int* block, int* grid, int* regs,
                       int* fused);

/* Test hook of failure detection (no counterpart in the reference): the next
 * plain FP64 solve whose iteration loop runs as one cooperative kernel
 * (CLOWNS_LOOP_PERSISTENT or CLOWNS_LOOP_WAVE, e.g. forced by
 * CLOWNS_LOOP_MODE=persistent|wave) gives every device-wide wait `polls` polls
 * instead of 2^24 and makes its block `absent_block` leave the kernel without
 * arriving anywhere.  The other blocks' waits then run out: they raise the
 * abort flag and return, nothing hangs or faults, and the solve reports
 * CLOWNS_ERR_NOCONV (through pcgpme_gpu: IER = CLOWNS_IER_DEVICE).  Applies to
 * one solve, then disarms; later solves on the same context run normally. */
int clowns_test_arm_wait_timeout(long polls, int absent_block);

/* Kernels the calling thread's last solve (plain or mixed, single or batched)
 * launched: host launches plus the kernel nodes its loop graphs executed
 * (per iteration 16 with single LDUSUB sweeps, 12 with fused sweep pairs, the
 * loop guard included), not counting the autotuner's one-time trial runs.
 * Engine bookkeeping with no counterpart in the reference. */
long clowns_last_kernel_launches(void);

/* Measured FP64 fused multiply-add rate of the current device (lane operations
 * per second, independent chains with no memory traffic): the ceiling of the
 * FP64 solve's arithmetic, reported beside the copy bandwidth: the best of five
 * timed launches of 5.1 G FMAs after two warm-ups, about 70 ms on `stream`.  Diagnostic with no counterpart in the reference. */
int clowns_fp64_fma_rate(double* fma_per_s, void* stream);

/* PCGPME_WILL, the 2DH dispersion solve (replaces src2LOWNS/pcgpme_2DH.f90:1-374,
 * called at 1sub-2DH-momentum.f90:325 as PCGPME_WILL(L%AL,4,L%indisp,L%LL,
 * L%DIAG,L%indisp,64,PSI,eps0,PARM,ITER)).  The same preconditioned BiCGSTAB
 * as PCGPME on an NL = 4 (or 6) matrix with BETA = C1 / (AMU RQ) (line 255),
 * x0 = 0 and EPS used as given; AL, LL and D are not modified.  On return B
 * holds what the reference leaves there (265-279): the solution with
 * |x| <= 1e-14 set to 0 and x(i) replaced by a neighbour's value when they
 * differ by at most 1e-14 (lower rows already processed, in row order), and,
 * for a row whose neighbour loop ends before writing B (its first LL is 0, or
 * its neighbours are itself or equal to it), the last recursive residual.
 * The reference has no error argument: these return 0 or a CLOWNS_ERR_* code
 * (ignored by a Fortran CALL) and leave B unchanged on error.  iter >= 1.
 * pcgpme_will_ is the name ifort gives the subroutine (link-level drop-in). */
int pcgpme_will_gpu(const double* al, const int* nl, const int* na, const int* ll, const double* d,
                    const int* n, const int* n2, double* b, const double* eps, const double* parm,
                    const int* iter);
int pcgpme_will_(const double* al, const int* nl, const int* na, const int* ll, const double* d,
                 const int* n, const int* n2, double* b, const double* eps, const double* parm,
                 const int* iter);
/* Device-resident PCGPME_WILL: device arrays, b in/out, a workspace of
 * clowns_pcgpme_will_workspace_bytes(n, nl) bytes; info (may be NULL) as for
 * clowns_pcgpme_dev (ier 3000 when ITER was reached, which the reference does
 * not report). */
size_t clowns_pcgpme_will_workspace_bytes(int n, int nl);
int clowns_pcgpme_will_dev(const double* al, int nl, int na, const int* ll, const double* d, int n,
                           double* b, double eps, double parm, int iter, void* work, size_t work_bytes,
                           void* stream, clowns_solve_info* info);
/* Test hook: the post-processing of pcgpme_2DH.f90:268-279 alone, on a
 * solution x and residual r (device arrays of n), ll as the caller's LL:
 * writes b and, if x_out is not NULL, the processed x. */
size_t clowns_will_postprocess_workspace_bytes(int n);
int clowns_will_postprocess_dev(const double* x, const double* r, const int* ll, int nl, int na, int n,
                                double* b, double* x_out, void* work, size_t work_bytes, void* stream);

/* Test hooks of the solve's building blocks (device pointers; workspace sized by
 * clowns_pcgpme_workspace_bytes(n, nl)).  clowns_pcgpme_setup_dev performs only
 * the row scaling and per-row sort of pcgpme_para.F90:77-112 and copies the
 * scaled, sorted matrix out: al_s/ll_s (na_out, nl) column-major, 0-based ll_s
 * with every empty slot pointing at row n (a zero pad row); d_s, b_s length n. */
int clowns_pcgpme_setup_dev(const double* al, int nl, int na, const int* ll, const double* d,
                            int n, const double* b, double parm, double* al_s, int* ll_s,
                            double* d_s, double* b_s, int na_out, void* work,
                            size_t work_bytes, void* stream);
/* y = PM * (W A) * x: the scaled/sorted operator of the setup above applied with
 * AXSUB then LDUSUB (pcgpme_para.F90:263-352).  x, y: device, length n. */
int clowns_apply_pm_a_dev(const double* al, int nl, int na, const int* ll, const double* d, int n,
                          double parm, const double* x, double* y, void* work, size_t work_bytes,
                          void* stream);

/* ========================================================================== */
/* Classification, static coefficients, rows, right-hand side, assembly       */
/* ========================================================================== */

/* set_nflag (src2LOWNS/nfd2015.F90:7-306, NORMAL+OBJECT build), called every
 * step from cal_vof (1sub-vof.F90:37).  Updates nf/nfb/f in place, writes the
 * fluid list fln(1:ifln) and surface list sfn(1:isfn) (pointers to element 1).
 * The reference's pruning and orientation loops run as OpenMP loops that read
 * flags other iterations write; this entry reproduces their serial order
 * (descending list position).  The isfn2 tail list (nfd2015.F90:285-304),
 * which only feeds subsystems outside the pressure solve, is not produced. */
size_t clowns_set_nflag_workspace_bytes(const int* dims, int inne2);
int clowns_set_nflag_dev(const int* dims, int inne, int inne2, int mx2, const int* mn,
                         const int* in_, const int* jn, const int* kn, int* nf, int* nfb,
                         double* f, const double* fb, const double* a, const double* dx,
                         const int* objno, int* fln, int* ifln, int* sfn, int* isfn,
                         int* passes, void* work, size_t work_bytes, void* stream);

/* Matrix columns of a grid (dims as above), the value init_matrix gives the
 * module variable nl (src2LOWNS/1sub-matrix.F90:15-21): 6 in 3D, 4 in the 2DV
 * mode the reference enters when the grid is one cell wide in x or in y
 * (main_2CLOWNS.F90:43-44).  0 for invalid bounds or a grid one cell wide in
 * both, which has no matrix form in the reference (its init_matrix sets two of
 * four columns); init_matrix, assembly, the face gradient and the session
 * refuse such grids with CLOWNS_ERR_ARG.  Host function, no device work. */
int clowns_grid_nl(const int* dims);

/* init_matrix (src2LOWNS/1sub-matrix.F90:3-66): ALU_C, LL_C, DE_C (nl columns,
 * nl = clowns_grid_nl(dims)) for cells 1..inne and mp = minval(dx, dx>0)**2
 * over every axis in 3D, over the two axes of the x-z or y-z plane in 2DV
 * (written to device *mp).  Rows of cells that are solid or have zero porosity
 * are zero-filled (the reference leaves them unset; they are never read). */
int clowns_init_matrix_dev(const int* dims, int inne, int mx2, const int* mn, const int* in_,
                           const int* jn, const int* kn, const int* nf, const int* nfb,
                           const double* a, const double* fb, const double* dx, double* mp,
                           double* alu_c, int* ll_c, double* de_c, void* stream);

/* cal_err_of_continuity at ik == 0 (src2LOWNS/1sub-momentum.F90:235-360): zero
 * b/xe/de(1:mm2) and mno, number the rows in fluid-list order (mno,
 * mno2mn(1:mnoe)), and build b(1:mnoe) = mp*DR1/dt for fluid rows.  mp is a
 * device pointer.  mnoe and dmax = max |DR1| are returned on the host.  Like the
 * reference, fewer than 10 rows leaves b at zero; mm2 must exceed mnoe by 64
 * (the reference re-allocates at 302-310; here the caller sizes mm2). */
size_t clowns_rows_rhs_workspace_bytes(int ifln);
int clowns_rows_rhs_dev(const int* dims, int inne2, int mx2, const int* mn, const int* in_,
                        const int* jn, const int* kn, const int* nf, const int* nfb,
                        const double* f, const double* fb, const double* a, const double* un,
                        const double* dx, const double* mp, double dt, int ifln, const int* fln,
                        int mm2, int* mno, int* mno2mn, double* b, double* xe, double* de,
                        int* mnoe, double* dmax, void* work, size_t work_bytes, void* stream);

/* cal_matrix_element (src2LOWNS/1sub-momentum.F90:465-551), NORMAL build:
 * alu/llu(1:mm2, 1:nl) column-major and de(1:mm2) for every row; in 2DV a
 * surface row's normal axis is found past the collapsed one (lines 517-520).  *err_cell
 * (device int) receives a cell index if a row cell carries a flag other than 1
 * or 2 (the reference stops there, line 491-492), else 0. */
int clowns_assemble_dev(const int* dims, int inne, int inne2, int mx2, const int* in_,
                        const int* jn, const int* kn, const int* nf, const int* nfb,
                        const double* x, const double* dx, const double* sp, int ifln,
                        const int* fln, const int* mno, const double* alu_c, const int* ll_c,
                        const double* de_c, int mm2, double* alu, int* llu, double* de,
                        int* err_cell, void* stream);

/* Pressure update p(mno2mn(r)) -= xe(r) and estimate_velocity2
 * (src2LOWNS/1sub-momentum.F90:52-58, 590-651).  xe0 addresses xe(0), which
 * the reference reads for neighbours that are not rows. */
int clowns_correct_dev(const int* dims, int inne, int mx2, const int* mn, const int* in_,
                       const int* jn, const int* kn, const int* nf, const int* nfb,
                       const double* a, const double* dx, double dt, int mnoe,
                       const int* mno2mn, const int* mno, const double* xe0, double* p,
                       double* un, void* stream);

/* ========================================================================== */
/* Discrete adjoint (no reference counterpart)                                */
/* ========================================================================== */

/* Explicit transpose of an assembled ELL matrix: row i of (alt, llt, det) holds
 * column i of A; the coefficient of row j toward its neighbour i in direction d
 * lands in row i at the opposite direction slot (minus <-> plus face of the same
 * axis).  n rows, leading dimension na, nl columns (6 or 4), 1-based llu (0 =
 * none).  *bad (device int) is set if an index lies outside 1..n.  The adjoint solve then runs clowns_pcgpme_dev (or
 * the mixed / batched variants) on (alt, llt, det): the reference's PCGPME
 * method applied to A^T, with its own row scaling and sort. */
int clowns_transpose_dev(int n, int na, int nl, const double* alu, const int* llu, const double* de,
                         double* alt, int* llt, double* det, int* bad, void* stream);

/* Face-coefficient gradient dJ/da(l, owner) = -lambda^T (dA/da) x for the face
 * area fractions a(0:2, 0:inne2+1) that enter A through ALU_C
 * (1sub-matrix.F90:49-61): x solves A x = b, lambda solves A^T lambda = dJ/dx.
 * Faces of surface rows (whose coefficients do not depend on a) and faces
 * cancelled by the Neumann fix (1sub-momentum.F90:502-509) get zero.  grad has
 * the layout of a and is overwritten.  The right-hand side is an independent
 * input; its gradient is lambda itself. */
int clowns_face_grad_dev(const int* dims, int inne, int inne2, int ifln, const int* fln,
                         const int* in_, const int* jn, const int* kn, const int* nf,
                         const int* mno, const double* alu_c, const int* ll_c, const double* a,
                         const double* x, const double* lambda, double* grad, void* stream);

/* ========================================================================== */
/* Allocation-free FP64 solve (no counterpart in the reference)               */
/* ========================================================================== */

/* Largest system the allocation-free solve accepts. */
#define CLOWNS_STATIC_MAX_ROWS 32768

/* The FP64 solve of clowns_pcgpme_dev for callers that cannot allocate device
 * memory -- a host model whose device memory belongs to another runtime or to
 * a fixed budget, which therefore can neither cudaMalloc a workspace nor hand
 * one over.  Inputs and outputs are the caller's device arrays as for
 * clowns_pcgpme_dev; all scratch space lives in one static device array of
 * about 5 MB that every GPU loading the library holds until the process exits.
 * The call allocates nothing (no cudaMalloc/cudaFree, no allocating library
 * routine) and returns CLOWNS_ERR_LIMIT for n > CLOWNS_STATIC_MAX_ROWS.  The
 * first call on a device looks up the array's device address (once per device,
 * with that device current).  Every call shares the array and re-initialises what it reads, so calls that
 * overlap on the GPU (other streams or host threads) race on it. */
int clowns_pcgpme_static_dev(const double* al, int nl, int na, const int* ll, const double* d,
                             int n, const double* b, double* x, double eps, double parm, int iter,
                             void* stream, clowns_solve_info* info);

/* ========================================================================== */
/* Device-resident pressure-correction loop of one domain                     */
/* ========================================================================== */

/* The ik loop of cal_momentum (src2LOWNS/1sub-momentum.F90:41-60) with the
 * domain's module arrays kept in HBM: cal_err_of_continuity, check_dmax,
 * cal_matrix_element, cal_poisson_equation, p -= xe and estimate_velocity2, with
 * one host read-back of dmax per ik.  Host arrays in the reference layouts; the
 * session owns its device memory. */
typedef struct clowns_session clowns_session;

/* Static grid: dims, mn, in/jn/kn, x, dx, objno (uploaded once). */
int clowns_session_create(clowns_session** s, const int* dims, int inne, int inne2, int mx2,
                          const int* mn, const int* in_, const int* jn, const int* kn,
                          const double* x, const double* dx, const int* objno);
/* Fields of the current step: nff%f, nff%b, f, fb, a, un, sp, p. */
int clowns_session_set_fields(clowns_session* s, const int* nf, const int* nfb, const double* f,
                              const double* fb, const double* a, const double* un,
                              const double* sp, const double* p);
/* set_nflag (every step) and, on the first call, init_matrix; sizes the
 * matrix rows to ifln + 5000 as the reference does. */
int clowns_session_classify(clowns_session* s, int* ifln, int* isfn);
/* The ik loop until dmax < d0 or ik > 1000 or a solver failure.  Returns ik and
 * dmax at exit, the last solve's iteration count and ERR, and icon as the
 * reference's caller sets it (0, 12, 96, 911 or 1030). */
int clowns_session_pressure_loop(clowns_session* s, double dt, double d0, double eps0,
                                 int precision, int* ik, double* dmax, int* iter, double* err,
                                 int* icon);
/* Read back nff%f, nff%b, f, p, un (any may be NULL) and mnoe. */
int clowns_session_get_fields(clowns_session* s, int* nf, int* nfb, double* f, double* p,
                              double* un, int* mnoe);
int clowns_session_destroy(clowns_session* s);

#ifdef __cplusplus
}
#endif
#endif /* CLOWNS_GPU_H */
