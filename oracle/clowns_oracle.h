/*
 * clowns_oracle.h -- CPU restatement of the 2CLOWNS-3D pressure-Poisson path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path: the
 * tests, the smoke check and the CPU-baseline leg of the benchmark call it; the
 * product library never links or calls it.
 *
 * Parity status: pinned to the reference's own source, executed.  The
 * reference is Fortran 90 built only with ifort (src2LOWNS/Makefile:1,5), no
 * Fortran compiler exists where this was written, and the reference ships no
 * tests, golden vectors or input cases.  Its routines are run instead through
 * a translator of the Fortran subset they use (tests/golden/fortran_exec.py,
 * whose semantics tests/test_fortran_exec.py fixes), and this restatement
 * reproduces their outputs bit for bit (tests/test_oracle_reference_runs.py):
 * set_nflag, init_matrix, numbering and right-hand side, cal_matrix_element,
 * PCGPME, the ik loop with the correction, and PCGPME_WILL.  The pin is to the
 * source's written evaluation order; the ifort build (-O3 -xHost) may fuse or
 * reorder floating-point operations, which nothing here can reproduce.
 * Hand-derived known answers and a scipy direct solve check it as well.
 *
 * Array conventions (identical to the reference's module arrays):
 *   dims[6]      = is, js, ks, ie, je, ke
 *   mn           : mn(is-2:ie+2, ks-2:ke+2, js-2:je+2), i fastest
 *   mno          : mno(1:ie, 1:ke, 1:je), i fastest
 *   x, dx        : (0:2, 1:mx2), component fastest
 *   in/jn/kn     : 1-based cell index nn (element 0 unused)
 *   nf, nfb      : nff(0:inne2+1)%f and %b as two plain int arrays
 *   f, fb        : (0:inne2+1)
 *   a, un        : (0:2, 0:inne2+1), component fastest
 *   sp           : sp(0:inne2+1, 0:2), cell index fastest
 *   alu_c, ll_c  : ALU_C(1:inne, 1:6), column-major, leading dimension inne
 *   alu, llu     : alu(1:mm2, 1:6), column-major, leading dimension mm2
 *   fln, sfn     : 1-based lists (element 0 unused)
 * Every pointer addresses the element with the lowest index.
 */
#ifndef CLOWNS_ORACLE_H
#define CLOWNS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* set_nflag (nfd2015.F90:7-306), NORMAL+OBJECT build, serial semantics.
 * Returns the number of classification passes (label-4 restarts + 1). */
int ora_set_nflag(const int* dims, int inne, int mx2, const int* mn, const int* in_,
                  const int* jn, const int* kn, int* nf, int* nfb, double* f,
                  const double* fb, const double* a, const double* dx,
                  const int* objno, int* fln, int* ifln, int* sfn, int* isfn);

/* init_matrix (1sub-matrix.F90:3-66), 3D (nl = 6).  Writes mp. */
/* Matrix columns of a grid: 6 (3D), 4 (2DV: one cell wide in x or y,
 * main_2CLOWNS.F90:43-44, 1sub-matrix.F90:15-21) or 0 (one cell wide in both). */
int ora_grid_nl(const int* dims);

void ora_init_matrix(const int* dims, int inne, int mx2, const int* mn, const int* in_,
                     const int* jn, const int* kn, const int* nf, const int* nfb,
                     const double* a, const double* fb, const double* dx,
                     double* mp, double* alu_c, int* ll_c, double* de_c);

/* cal_err_of_continuity at ik==0 (1sub-momentum.F90:265-360): row numbering and
 * right-hand side.  Returns mnoe (or -1 if mm2 is too small). */
int ora_rows_rhs(const int* dims, int inne2, int mx2, const int* mn, const int* in_,
                 const int* jn, const int* kn, const int* nf, const int* nfb,
                 const double* f, const double* fb, const double* a, const double* un,
                 const double* dx, double mp, double dt, int ifln, const int* fln,
                 int mm2, int* mno, int* mno2mn, double* b, double* xe, double* de,
                 double* dmax);

/* cal_matrix_element (1sub-momentum.F90:465-551), NORMAL build.
 * Returns 0, or the offending cell index if a row carries an unexpected flag. */
int ora_assemble(const int* dims, int inne, int inne2, int mx2, const int* in_,
                 const int* jn, const int* kn, const int* nf, const int* nfb,
                 const double* x, const double* dx, const double* sp, int ifln,
                 const int* fln, const int* mno, const double* alu_c, const int* ll_c,
                 const double* de_c, int mm2, double* alu, int* llu, double* de);

/* PCGPME (pcgpme_para.F90:1-354).  Same by-reference arguments; AL, LL, D and B
 * are modified in place exactly as the reference does.  nthreads <= 1 runs the
 * loops serially (deterministic sums); otherwise OpenMP with the reference's
 * static schedule.  stop_reason (may be NULL): 0 tolerance, 1 stagnation,
 * 2 AMU==0, 3 C1==0, 4 iteration cap. */
void ora_pcgpme(double* al, const int* nl, const int* na, int* ll, double* d,
                const int* n, const int* n2, double* b, double* x, double* eps,
                const double* parm, int* iter, int* ier, int nthreads, int* stop_reason);

/* PCGPME_WILL (src2LOWNS/pcgpme_2DH.f90:1-374): AL, LL, D are left unchanged,
 * B (length n) is the right-hand side on entry and the post-processed solution
 * on return.  iters_out / reason_out (may be NULL) as for ora_pcgpme. */
void ora_pcgpme_will(const double* al, int nl, int na, const int* ll, const double* d, int n, int n2,
                     double* b, double eps, double parm, int iter, int nthreads, int* iters_out,
                     int* reason_out);
/* The post-processing alone (pcgpme_2DH.f90:268-279), in place on x and b. */
void ora_will_postprocess(double* x, double* b, const int* ll, int nl, long na, int n);

/* One operator application Q = PM * A * P using a matrix already scaled and
 * sorted by ora_pcgpme_setup (test helper). */
void ora_pcgpme_setup(double* al, int nl, int na, int* ll, double* d, int n,
                      double* b, double parm);
void ora_axsub(const double* al, int nl, int na, const int* ll, const double* d, int n,
               int n2, const double* x, double* y);
void ora_ldusub(const double* al, int nl, int na, const int* ll, int n, int n2,
                double* p_inout);

/* Pressure update and velocity correction (1sub-momentum.F90:52-59, 590-651). */
void ora_correct(const int* dims, int inne, int mx2, const int* mn, const int* in_,
                 const int* jn, const int* kn, const int* nf, const int* nfb,
                 const double* a, const double* dx, double dt, int mnoe,
                 const int* mno2mn, const int* mno, const double* xe, double* p,
                 double* un);

/* Transposed operator of an assembled (unscaled) ELL matrix: row i of the result
 * holds column i of A in the same direction slots.  No reference counterpart. */
void ora_transpose(int n, int na, int nl, const double* alu, const int* llu, const double* de,
                   double* alt, int* llt, double* det);

/* y = A x on the assembled (unscaled) ELL matrix, 1-based llu, 0 = absent. */
void ora_spmv(int n, int na, int nl, const double* alu, const int* llu, const double* de,
              const double* x, double* y);

#ifdef __cplusplus
}
#endif
#endif
