/*
 * clowns_oracle.c -- CPU restatement of the 2CLOWNS-3D pressure-Poisson path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path.  Only the tests, the
 * smoke check and the CPU-baseline leg of the benchmark load this library.
 *
 * Parity status: pinned to the reference's own source, run through a Fortran
 * translator (no Fortran compiler exists here); see the header file.  Each
 * function cites the reference lines it restates.  The
 * arithmetic keeps the reference's evaluation order; the build uses
 * -ffp-contract=off so no multiply-add is fused on any host, which keeps the
 * matrix coefficients (and hence the per-row sort) bit-reproducible.
 *
 * Reference constants (src2LOWNS/0mod-variables.F90:32-44, 68-69):
 *   TINY = 1e-15, VSMALL = 1e-12, SMALL = 1e-9, iob = -1, ifu = 1.
 */
#include "clowns_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ZERO 0.0
#define HALF 0.5
#define ONE 1.0
#define TWO 2.0
#define TINY 1.0e-15
#define VSMALL 1.0e-12
#define SMALL 1.0e-9
#define IOB (-1)
#define IFU 1

typedef struct {
    int is, js, ks, ie, je, ke;
    long ni, nk, nj;
} grid_t;

static grid_t mkgrid(const int* dims) {
    grid_t g;
    g.is = dims[0]; g.js = dims[1]; g.ks = dims[2];
    g.ie = dims[3]; g.je = dims[4]; g.ke = dims[5];
    g.ni = g.ie - g.is + 5;
    g.nk = g.ke - g.ks + 5;
    g.nj = g.je - g.js + 5;
    return g;
}

/* mn(i,k,j) with lower bounds (is-2, ks-2, js-2), i fastest. */
static inline long mn_off(const grid_t* g, int i, int k, int j) {
    return (long)(i - (g->is - 2)) + g->ni * ((long)(k - (g->ks - 2)) + g->nk * (long)(j - (g->js - 2)));
}
#define MN(i, k, j) mn[mn_off(&g, (i), (k), (j))]
/* neighbour of (i,j,k) at signed step s along axis l (lf = identity, main_2CLOWNS.F90:33) */
#define NBR(i, j, k, l, s) MN((i) + (s) * ((l) == 0), (k) + (s) * ((l) == 2), (j) + (s) * ((l) == 1))
#define XC(l, i) x[3L * ((i) - 1) + (l)]
#define DXC(l, i) dx[3L * ((i) - 1) + (l)]
#define AF(l, nn) a[3L * (nn) + (l)]
#define UNF(l, nn) un[3L * (nn) + (l)]

static inline int iabs_(int v) { return v < 0 ? -v : v; }
static inline double dmax_(double a, double b) { return a > b ? a : b; }
static inline double dmin_(double a, double b) { return a < b ? a : b; }

/* ------------------------------------------------------------------------- */
/* fxx1 (nfd2015.F90:308-332): weighted wet volume on the far side of a candidate
 * surface orientation. */
static double fxx1(const grid_t* gp, const int* mn, const double* dx, const double* f,
                   const double* fb, int ix, int ll, int i, int j, int k) {
    grid_t g = *gp;
    int lg[3] = {i, j, k};
    double r = ZERO;
    for (int l = 0; l <= 2; l++) {
        if (l == ll) continue;
        if (g.is == g.ie - 1 && l == 0) continue;
        if (g.js == g.je - 1 && l == 1) continue;
        for (int ii = -1; ii <= 1; ii++) {
            int ci = lg[0] + ix * (ll == 0) + ii * (l == 0);
            int ck = lg[2] + ix * (ll == 2) + ii * (l == 2);
            int cj = lg[1] + ix * (ll == 1) + ii * (l == 1);
            int nnc = MN(ci, ck, cj);
            r = r + DXC(l, lg[l] + ii) * f[nnc] * fb[nnc];
        }
        for (int lll = 0; lll <= 2; lll++) {
            if (lll == l || ll == lll) continue;
            r = r * DXC(lll, lg[lll]);
        }
    }
    r = r * DXC(ll, lg[ll] + ix);
    return r;
}

/* set_nflag (nfd2015.F90:7-306), compiled with -DNORMAL -DOBJECT (Makefile:5).
 * The reference runs the pruning and orientation loops as OpenMP loops that
 * write flags other iterations read; this restatement fixes their serial order
 * (descending list position), which is also what the GPU classification
 * reproduces.  The isfn2 bookkeeping (nfd2015.F90:285-304) feeds only
 * subsystems outside the pressure solve and is not restated. */
int ora_set_nflag(const int* dims, int inne, int mx2, const int* mn, const int* in_,
                  const int* jn, const int* kn, int* nf, int* nfb, double* f,
                  const double* fb, const double* a, const double* dx,
                  const int* objno, int* fln, int* ifln_out, int* sfn, int* isfn_out) {
    (void)mx2;
    grid_t g = mkgrid(dims);
    int imax = 0, kmax = 0;
    /* nfd2015.F90:35-59: fluid / air by VOF */
    for (int nn = 1; nn <= inne; nn++) {
        if (nf[nn] == -1) continue;
        int i = in_[nn], j = jn[nn], k = kn[nn];
        if (f[nn] <= VSMALL ||
            (f[nn] * fb[nn] < 1.0e-3 && nf[MN(i, k - 1, j)] == -1 && f[MN(i, k + 1, j)] == ZERO)) {
            int c = MN(i, k, j);
            nf[c] = 0;
            nfb[c] = 0;
            f[nn] = dmax_(ZERO, f[nn]);
        } else {
            nf[nn] = 1;
            nfb[nn] = 0;
            if (i > imax) imax = i;
            if (k > kmax) kmax = k;
        }
    }
    imax = (g.ie - 1 < imax + 1) ? g.ie - 1 : imax + 1;
    kmax = (g.ke - 1 < kmax + 1) ? g.ke - 1 : kmax + 1;

    int passes = 0;
    int ifln = 0, isfn = 0;
label4:
    passes++;
    if (passes > 100000) return -passes;
    ifln = 0;
    isfn = 0;
    /* nfd2015.F90:69-102: fluid list in k, j, i order; surface = wet cell with an
     * open face to an air cell */
    for (int k = g.ks; k <= kmax; k++)
        for (int j = g.js; j <= g.je - 1; j++)
            for (int i = g.is; i <= imax; i++) {
                int nn = MN(i, k, j);
                if (nf[nn] == -1) continue;
                if (nf[nn] >= 1) {
                    fln[++ifln] = nn;
                    int surf = 0;
                    for (int l = 0; l <= 2 && !surf; l++) {
                        int p = NBR(i, j, k, l, +1);
                        if (nf[p] == 0 && AF(l, p) > ZERO) { surf = 1; break; }
                        int m = NBR(i, j, k, l, -1);
                        if (nf[m] == 0 && AF(l, nn) > ZERO) { surf = 1; break; }
                    }
                    if (surf) {
                        nf[nn] = 2;
                        sfn[++isfn] = nn;
                        nfb[nn] = -3;
                    } else {
                        nf[nn] = 1;
                    }
                }
            }
    /* nfd2015.F90:107-131: drop surface cells touching no fluid cell */
    int n2 = 0;
    for (int nnf = isfn; nnf >= 1; nnf--) {
        int nn = sfn[nnf];
        int i = in_[nn], j = jn[nn], k = kn[nn];
        if (nf[MN(i, k - 1, j)] == -1) continue;
        int keep = 0;
        for (int l = 0; l <= 2; l++) {
            if (nf[NBR(i, j, k, l, +1)] == 1) { keep = 1; break; }
            if (nf[NBR(i, j, k, l, -1)] == 1) { keep = 1; break; }
        }
        if (!keep) {
            n2 = 1;
            nf[nn] = 0;
            nfb[nn] = 0;
        }
    }
    if (n2 == 1) goto label4;
    /* nfd2015.F90:133-158: keep only cells between fluid and air along some axis */
    for (int nnf = isfn; nnf >= 1; nnf--) {
        int nn = sfn[nnf];
        int i = in_[nn], j = jn[nn], k = kn[nn];
        if (nf[MN(i, k - 1, j)] == -1 && nf[MN(i, k + 1, j)] == 0) continue;
        int keep = 0;
        for (int l = 0; l <= 2; l++) {
            int p = NBR(i, j, k, l, +1), m = NBR(i, j, k, l, -1);
            if (nf[p] == 1 && nf[m] == 0) { keep = 1; break; }
            if (nf[m] == 1 && nf[p] == 0) { keep = 1; break; }
        }
        if (!keep) {
            n2 = 1;
            nf[nn] = 0;
            nfb[nn] = 0;
        }
    }
    if (n2 == 1) goto label4;
    /* nfd2015.F90:163-246: surface orientation nfb = +-(axis+1) */
    int igai = 0;
    for (int nnf = isfn; nnf >= 1; nnf--) {
        int nn = sfn[nnf];
        int i = in_[nn], j = jn[nn], k = kn[nn];
        nfb[nn] = 0;
        int ix[3] = {0, 0, 0};
        for (int l = 0; l <= 2; l++) {
            int m = NBR(i, j, k, l, -1), p = NBR(i, j, k, l, +1);
            if (nf[m] == 1 && nf[p] == 0 && AF(l, p) > ZERO) {
                ix[l] = -1;
            } else if (nf[m] == 0 && nf[p] == 1 && AF(l, nn) > ZERO) {
                ix[l] = 1;
            }
        }
        if (iabs_(ix[0]) + iabs_(ix[1]) + iabs_(ix[2]) == 0) {
            if (nf[MN(i, k - 1, j)] == -1 && nf[MN(i, k + 1, j)] == 0) {
                if (objno[nn] != 0 || fb[nn] != ZERO) {
                    ix[2] = -1;
                } else {
                    for (int l = 0; l <= 1; l++) {
                        int m = NBR(i, j, k, l, -1), p = NBR(i, j, k, l, +1);
                        if (nf[m] > 0 && nf[p] == 0 && AF(l, p) > ZERO) {
                            ix[l] = -1;
                        } else if (nf[m] == 0 && nf[p] > 0 && AF(l, nn) > ZERO) {
                            ix[l] = 1;
                        }
                    }
                    if (iabs_(ix[0]) + iabs_(ix[1]) == 0) ix[2] = -1;
                }
            }
        }
        int s = iabs_(ix[0]) + iabs_(ix[1]) + iabs_(ix[2]);
        if (s == 1) {
            int dir = 1, best = iabs_(ix[0]);
            for (int l = 1; l <= 2; l++)
                if (iabs_(ix[l]) > best) { best = iabs_(ix[l]); dir = l + 1; }
            nfb[nn] = dir * ix[dir - 1];
        } else if (s == 0) {
            igai++;
            nf[nn] = 0;
        } else {
            double fxx[3];
            for (int l = 0; l <= 2; l++)
                fxx[l] = (ix[l] == 0) ? ZERO : fxx1(&g, mn, dx, f, fb, ix[l], l, i, j, k);
            int dir = 1;
            double best = fxx[0];
            for (int l = 1; l <= 2; l++)
                if (fxx[l] > best) { best = fxx[l]; dir = l + 1; }
            nfb[nn] = dir * ix[dir - 1];
        }
    }
    if (igai != 0) goto label4;
    *ifln_out = ifln;
    *isfn_out = isfn;
    return passes;
}

/* ------------------------------------------------------------------------- */
/* cal_alu_f (1sub-matrix.F90:82-87) and cal_alu (75-80) */
static inline double cal_alu_f(double dx, double dxm, double ax, double fb) {
    return TWO / dx / (dx + dxm) * ax / fb;
}
static inline double cal_alu(double fnn, double dx, double dxm) {
    return (fnn - HALF) * dx / (fnn * dx + dxm * HALF) * (-ONE);
}

/* init_matrix (1sub-matrix.F90:3-66), dim3d branch (nl = 6). */
/* Matrix columns (1sub-matrix.F90:15-21): 6 in 3D, 4 in the 2DV mode the
 * reference enters for a grid one cell wide in x or y (main_2CLOWNS.F90:43-44);
 * 0 for a grid one cell wide in both, whose column numbering the reference
 * leaves undefined (only two of four columns are set). */
int ora_grid_nl(const int* dims) {
    grid_t g = mkgrid(dims);
    int cx = g.is == g.ie - 1, cy = g.js == g.je - 1;
    return (cx && cy) ? 0 : (cx || cy) ? 4 : 6;
}

void ora_init_matrix(const int* dims, int inne, int mx2, const int* mn, const int* in_,
                     const int* jn, const int* kn, const int* nf, const int* nfb,
                     const double* a, const double* fb, const double* dx,
                     double* mp_out, double* alu_c, int* ll_c, double* de_c) {
    grid_t g = mkgrid(dims);
    int nl = ora_grid_nl(dims);
    /* mp = minval(dx, dx > 0)**2 over every axis (line 17); 2DV: over x and z
     * when one cell wide in y, over y and z when one cell wide in x (20-21) */
    int use[3] = {1, 1, 1};
    if (nl == 4) {
        if (g.js == g.je - 1) { use[0] = 1; use[1] = 0; use[2] = 1; }
        if (g.is == g.ie - 1) { use[0] = 0; use[1] = 1; use[2] = 1; }
    }
    double m = 0.0;
    int have = 0;
    for (long t = 0; t < 3L * mx2; t++) {
        if (!use[t % 3]) continue;
        if (dx[t] > ZERO && (!have || dx[t] < m)) { m = dx[t]; have = 1; }
    }
    double mp = m * m;
    *mp_out = mp;
    long ld = inne;
    memset(alu_c, 0, sizeof(double) * (size_t)nl * (size_t)ld);
    memset(ll_c, 0, sizeof(int) * (size_t)nl * (size_t)ld);
    memset(de_c, 0, sizeof(double) * (size_t)ld);
    for (int nnn = 1; nnn <= inne; nnn++) {
        if (nf[nnn] == IOB || fb[nnn] == ZERO) continue;
        int i = in_[nnn], j = jn[nnn], k = kn[nnn];
        int lg[3] = {i, j, k};
        int ll = 0;
        double de = ZERO;
        for (int l = 0; l <= 2; l++) {
            if (g.is == g.ie - 1 && l == 0) continue;     /* nl = 4 (lines 34-35) */
            if (g.js == g.je - 1 && l == 1) continue;
            ll++;
            for (int ii = -1; ii <= 1; ii += 2) {
                int np = NBR(i, j, k, l, ii);
                int iip = ii > 0 ? ii : 0;
                int npp = NBR(i, j, k, l, iip);
                int col = 2 * ll + (ii < 0 ? ii : 0);   /* 1-based */
                long off = (long)(col - 1) * ld + (nnn - 1);
                if ((nf[np] == IOB && nfb[np] != 4) || AF(l, npp) == ZERO || fb[np] == ZERO) {
                    ll_c[off] = 0;
                    alu_c[off] = ZERO;
                } else {
                    ll_c[off] = np;
                    alu_c[off] = -(mp * cal_alu_f(DXC(l, lg[l]), DXC(l, lg[l] + ii), AF(l, npp), fb[nnn]));
                    de = de - alu_c[off];
                }
            }
        }
        de_c[nnn - 1] = de;
    }
}

/* ------------------------------------------------------------------------- */
/* renzoku_fv (lib/src/math_func.F90:51-54) through renzoku_n (1sub-main.F90:579-602) */
static inline double renzoku_fv(double axp, double axm, double ayp, double aym, double azp,
                                double azm, double up, double um, double vp, double vm,
                                double wp, double wm, double dx, double dy, double dz,
                                double fb) {
    return ((up * axp - um * axm) / dx + (vp * ayp - vm * aym) / dy + (wp * azp - wm * azm) / dz) / fb;
}

int ora_rows_rhs(const int* dims, int inne2, int mx2, const int* mn, const int* in_,
                 const int* jn, const int* kn, const int* nf, const int* nfb,
                 const double* f, const double* fb, const double* a, const double* un,
                 const double* dx, double mp, double dt, int ifln, const int* fln,
                 int mm2, int* mno, int* mno2mn, double* b, double* xe, double* de,
                 double* dmax_out) {
    (void)inne2; (void)mx2;
    grid_t g = mkgrid(dims);
    /* 1sub-momentum.F90:266-271 */
    for (int r = 1; r <= mm2; r++) { b[r] = ZERO; xe[r] = ZERO; de[r] = ZERO; }
    /* 273-294: rows in fluid-list order */
    long nmno = (long)g.ie * g.ke * g.je;
    memset(mno, 0, sizeof(int) * (size_t)nmno);
    int nn = 0;
    for (int nnf = 1; nnf <= ifln; nnf++) {
        int nnn = fln[nnf];
        int i = in_[nnn], j = jn[nnn], k = kn[nnn];
        double fbc = fb[nnn];
        if (nf[nnn] == 0 || nf[nnn] == IOB || fbc == ZERO) continue;
        if (nf[nnn] == 2) {
            int l = iabs_(nfb[nnn]) - 1;
            int s = nfb[nnn] >= 0 ? 1 : -1;
            /* an orientation of 0 makes the reference index lf(-1,:), which is
             * undefined; such a cell is kept as a row here */
            if (l >= 0 && l <= 2 && nf[NBR(i, j, k, l, s)] == IOB) continue;
        }
        nn++;
        if (nn > mm2) return -1;
        mno[(long)(i - 1) + (long)g.ie * ((long)(k - 1) + (long)g.ke * (j - 1))] = nn;
        mno2mn[nn] = nnn;
    }
    int mnoe = nn;
    *dmax_out = ZERO;
    if (nn < 10) return mnoe;          /* 297-300 */
    if (mnoe + 64 > mm2) return -1;    /* the reference re-allocates here (302-310) */
    /* 313-360: right-hand side of the fluid rows */
    double dmax = ZERO;
    for (int nnf = 1; nnf <= mnoe; nnf++) {
        int c = mno2mn[nnf];
        if (nf[c] != 1) continue;
        int i = in_[c], j = jn[c], k = kn[c];
        double ff = dmax_(-0.001, dmin_(ONE - f[c], 0.001));
        double rz;
        if (fb[c] != ZERO) {
            int ip = MN(i + 1, k, j), jp = MN(i, k, j + 1), kp = MN(i, k + 1, j);
            rz = renzoku_fv(AF(0, ip), AF(0, c), AF(1, jp), AF(1, c), AF(2, kp), AF(2, c),
                            UNF(0, ip), UNF(0, c), UNF(1, jp), UNF(1, c), UNF(2, kp), UNF(2, c),
                            DXC(0, i), DXC(1, j), DXC(2, k), fb[c]);
        } else {
            rz = -10000.0;
        }
        double dr1 = rz + ff / dt;
        double q = dr1 / dt;
        if (fabs(q) <= TINY && fabs(q) != ZERO) {
            /* left at zero */
        } else {
            b[nnf] = mp * dr1 / dt;
        }
        if (fabs(dr1) > dmax) dmax = fabs(dr1);
    }
    *dmax_out = dmax;
    return mnoe;
}

/* ------------------------------------------------------------------------- */
/* cal_matrix_element (1sub-momentum.F90:465-551), NORMAL build, dim3d */
int ora_assemble(const int* dims, int inne, int inne2, int mx2, const int* in_,
                 const int* jn, const int* kn, const int* nf, const int* nfb,
                 const double* x, const double* dx, const double* sp, int ifln,
                 const int* fln, const int* mno, const double* alu_c, const int* ll_c,
                 const double* de_c, int mm2, double* alu, int* llu, double* de) {
    (void)mx2;
    grid_t g = mkgrid(dims);
    const int nl = ora_grid_nl(dims);
    const double rate = -1.0e-20;
    long ldc = inne, ld = mm2;
    long spld = (long)inne2 + 2;
#define MNO(i, k, j) mno[(long)((i) - 1) + (long)g.ie * ((long)((k) - 1) + (long)g.ke * ((j) - 1))]
    for (int nnf = 1; nnf <= ifln; nnf++) {
        int nnn = fln[nnf];
        int i = in_[nnn], j = jn[nnn], k = kn[nnn];
        int nn = MNO(i, k, j);
        if (nn == 0) continue;
        if (nf[nnn] == IFU) {
            de[nn] = de_c[nnn - 1];
        } else if (nf[nnn] == 2) {
            de[nn] = ONE;
        } else {
            return nnn;
        }
        for (int ll = 1; ll <= nl; ll++) {
            long oc = (long)(ll - 1) * ldc + (nnn - 1);
            long o = (long)(ll - 1) * ld + (nn - 1);
            int lc = ll_c[oc];
            if (lc == 0) {
                llu[o] = 0;
                alu[o] = ZERO;
            } else {
                int np = MNO(in_[lc], kn[lc], jn[lc]);
                if (nf[lc] == 0 || np == 0) {
                    llu[o] = 0;
                    alu[o] = ZERO;
                    if (nf[nnn] == IFU && nf[lc] != 2) de[nn] = de[nn] + alu_c[oc];
                } else {
                    llu[o] = np;
                    if (nf[nnn] == IFU) {
                        alu[o] = alu_c[oc];
                    } else {
                        int l = (ll + ll % 2) / 2 - 1;
                        if (g.is == g.ie - 1) l = l + 1;            /* 2DV (lines 519-520) */
                        if (g.js == g.je - 1 && ll > 2) l = l + 1;
                        if (iabs_(nfb[nnn]) - 1 == l) {
                            int ii = (l == 0) ? i : (l == 1) ? j : k;
                            int md = ll % 2;
                            double fss = (double)(1 - 2 * md) * (XC(l, ii - md + 1) - sp[nnn + spld * l]) / DXC(l, ii);
                            alu[o] = cal_alu(fss, DXC(l, ii), DXC(l, ii - 2 * md + 1));
                        } else {
                            alu[o] = rate;
                        }
                    }
                }
            }
        }
    }
#undef MNO
    return 0;
}

/* ------------------------------------------------------------------------- */
/* PCGPME (pcgpme_para.F90:1-354).  1-based reference indices map to [I-1]. */
#define ALX(I, K) al[(long)((K) - 1) * NA + ((I) - 1)]
#define LLX(I, K) ll[(long)((K) - 1) * NA + ((I) - 1)]

/* AXSUB (pcgpme_para.F90:323-352): Y = D*X + sum_k AL(:,k) X(LL(:,k)) */
static void axsub_(const double* al, int NL, long NA, const int* ll, const double* D, int N,
                   const double* X, double* Y, int nt) {
    (void)nt;
    if (NL == 6) {
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt > 1 ? nt : 1)
        for (int I = 1; I <= N; I++) {
            Y[I - 1] = X[I - 1] * D[I - 1] + ALX(I, 1) * X[LLX(I, 1) - 1] + ALX(I, 2) * X[LLX(I, 2) - 1]
                     + ALX(I, 3) * X[LLX(I, 3) - 1] + ALX(I, 4) * X[LLX(I, 4) - 1]
                     + ALX(I, 5) * X[LLX(I, 5) - 1] + ALX(I, 6) * X[LLX(I, 6) - 1];
        }
    } else if (NL == 4) {
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt > 1 ? nt : 1)
        for (int I = 1; I <= N; I++) {
            Y[I - 1] = X[I - 1] * D[I - 1] + ALX(I, 1) * X[LLX(I, 1) - 1] + ALX(I, 2) * X[LLX(I, 2) - 1]
                     + ALX(I, 3) * X[LLX(I, 3) - 1] + ALX(I, 4) * X[LLX(I, 4) - 1];
        }
    }
}

/* LDUSUB (pcgpme_para.F90:263-320): Q = PM*P as five gather sweeps, each reading
 * only the previous sweep's full vector.  Every call site passes P and Q as the
 * same array; the private temporary W is zeroed on each call as in the source. */
static void ldusub_(const double* al, int NL, long NA, const int* ll, int N, int N2,
                    double* PQ, double* W, int nt) {
    (void)nt;
    double* P = PQ;
    double* Q = PQ;
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt > 1 ? nt : 1)
    for (int I = 1; I <= N + N2; I++) W[I - 1] = ZERO;
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt > 1 ? nt : 1)
    for (int I = 1; I <= N; I++) W[I - 1] = P[I - 1] - ALX(I, 1) * P[LLX(I, 1) - 1];
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt > 1 ? nt : 1)
    for (int I = 1; I <= N; I++) Q[I - 1] = W[I - 1] - ALX(I, 2) * W[LLX(I, 2) - 1];
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt > 1 ? nt : 1)
    for (int I = 1; I <= N; I++) W[I - 1] = Q[I - 1] - ALX(I, 3) * Q[LLX(I, 3) - 1];
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt > 1 ? nt : 1)
    for (int I = 1; I <= N; I++) Q[I - 1] = W[I - 1] - ALX(I, 4) * W[LLX(I, 4) - 1];
    if (NL > 4) {
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt > 1 ? nt : 1)
        for (int I = 1; I <= N; I++)
            W[I - 1] = Q[I - 1] - ALX(I, 5) * Q[LLX(I, 5) - 1] - ALX(I, 6) * Q[LLX(I, 6) - 1];
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt > 1 ? nt : 1)
        for (int I = 1; I <= N; I++) Q[I - 1] = W[I - 1];
    }
}

/* Setup of pcgpme_para.F90:77-112: pad empty columns, row scaling, per-row sort. */
static void setup_(double* al, int NL, long NA, int* ll, double* D, int N, double* B,
                   double P1, double P2, double* W, int nt) {
    (void)nt;
    int N1 = N + 1;
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt > 1 ? nt : 1)
    for (int I = 1; I <= N; I++) {
        double w = W[I - 1];
        for (int K = 1; K <= NL; K++) {
            if (LLX(I, K) == 0) LLX(I, K) = N1 + I % 64;
            w = w + fabs(ALX(I, K));
        }
        double TEMP = D[I - 1];
        w = P2 / (dmax_(w, TEMP) + TEMP * P1);
        W[I - 1] = w;
        for (int K = 1; K <= NL; K++) ALX(I, K) = ALX(I, K) * w;
        D[I - 1] = D[I - 1] * w;
        B[I - 1] = B[I - 1] * w;
    }
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt > 1 ? nt : 1)
    for (int I = 1; I <= N; I++) {
        for (int K = 1; K <= NL - 1; K++)
            for (int KK = K + 1; KK <= NL; KK++)
                if (fabs(ALX(I, K)) < fabs(ALX(I, KK))) {
                    double TEMP = ALX(I, K);
                    int ITEMP = LLX(I, K);
                    ALX(I, K) = ALX(I, KK);
                    LLX(I, K) = LLX(I, KK);
                    ALX(I, KK) = TEMP;
                    LLX(I, KK) = ITEMP;
                }
    }
}

void ora_pcgpme(double* al, const int* nl_, const int* na_, int* ll, double* D,
                const int* n_, const int* n2_, double* B, double* X, double* EPS,
                const double* parm_, int* ITER, int* IER, int nthreads, int* stop_reason) {
    int NL = *nl_, N = *n_, N2 = *n2_;
    long NA = *na_;
    int nt = nthreads > 1 ? nthreads : 1;
    double PARM = *parm_;
    double BN, C1, ALP, AMU, RN, RQ, BETA, ERR = ZERO, SS, ERRP, P1, P2;
    int K, reason = 4;

    if (EPS[0] <= TINY) EPS[0] = SMALL;                              /* 51 */
    if (*ITER <= 0) *ITER = (int)(10 * (sqrt((double)N) + 1));       /* 52 */
    *IER = 0;
    ERRP = ZERO;
    P1 = PARM;
    if (PARM < ONE) P1 = TWO * TWO;
    P2 = P1 + ONE;
    long L = (long)N + N2;
    double* WK = (double*)calloc((size_t)L * 5, sizeof(double));      /* 59-68 */
    double* W = (double*)calloc((size_t)L, sizeof(double));
    double* WL = (double*)calloc((size_t)L, sizeof(double));         /* LDUSUB's private W */
    int* LLTEMP = (int*)malloc(sizeof(int) * (size_t)NA * NL);       /* 71-75: dead copy */
    memcpy(LLTEMP, ll, sizeof(int) * (size_t)NA * NL);
    double* WK1 = WK;
    double* WK2 = WK + L;
    double* WK3 = WK + 2 * L;
    double* WK4 = WK + 3 * L;
    double* WK5 = WK + 4 * L;

    setup_(al, NL, NA, ll, D, N, B, P1, P2, W, nt);                  /* 77-112 */
    for (int I = 0; I < N; I++) WK1[I] = B[I];                       /* 115-119 */
    ldusub_(al, NL, NA, ll, N, N2, WK1, WL, nt);                     /* 123 */
    axsub_(al, NL, NA, ll, D, N, X, WK3, nt);                        /* 126 */
    ldusub_(al, NL, NA, ll, N, N2, WK3, WL, nt);                     /* 127 */
    BN = ZERO;
    C1 = ZERO;
#pragma omp parallel for schedule(static) reduction(+ : BN, C1) if (nt > 1) num_threads(nt)
    for (int I = 0; I < N; I++) {                                    /* 133-143 */
        double TEMP = WK1[I];
        BN = BN + TEMP * TEMP;
        TEMP = TEMP - WK3[I];
        B[I] = TEMP;
        C1 = C1 + TEMP * TEMP;
        WK1[I] = TEMP;
        WK2[I] = TEMP;
    }
    for (K = 1; K <= *ITER; K++) {                                   /* 148 */
        axsub_(al, NL, NA, ll, D, N, WK1, WK3, nt);
        ldusub_(al, NL, NA, ll, N, N2, WK3, WL, nt);
        RQ = ZERO;
#pragma omp parallel for schedule(static) reduction(+ : RQ) if (nt > 1) num_threads(nt)
        for (int I = 0; I < N; I++) RQ = RQ + WK2[I] * WK3[I];
        ALP = C1 / RQ;
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt)
        for (int I = 0; I < N; I++) WK4[I] = B[I] - ALP * WK3[I];
        axsub_(al, NL, NA, ll, D, N, WK4, WK5, nt);
        ldusub_(al, NL, NA, ll, N, N2, WK5, WL, nt);
        AMU = ZERO;
        SS = ZERO;
#pragma omp parallel for schedule(static) reduction(+ : AMU, SS) if (nt > 1) num_threads(nt)
        for (int I = 0; I < N; I++) {
            double TEMP = WK5[I];
            AMU = AMU + WK4[I] * TEMP;
            SS = SS + TEMP * TEMP;
        }
        AMU = AMU / SS;
        C1 = ZERO;
        RN = ZERO;
#pragma omp parallel for schedule(static) reduction(+ : RN, C1) if (nt > 1) num_threads(nt)
        for (int I = 0; I < N; I++) {
            double TEMP = WK4[I];
            X[I] = X[I] + ALP * WK1[I] + AMU * TEMP;
            TEMP = TEMP - AMU * WK5[I];
            B[I] = TEMP;
            RN = RN + TEMP * TEMP;
            C1 = C1 + TEMP * WK2[I];
        }
        ERR = sqrt(RN / BN);                                         /* 215 */
        if (K >= 10 && fabs(ERR - ERRP) <= ERR * 1.0e-6) { reason = 1; goto done; }  /* 228 */
        if (ERR <= EPS[0]) { reason = 0; goto done; }                /* 232 */
        ERRP = ERR;
        if (AMU == ZERO) { reason = 2; goto done; }                  /* 234 */
        if (C1 == ZERO) { reason = 3; goto done; }                   /* 240 */
        BETA = C1 / AMU / RQ;
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt)
        for (int I = 0; I < N; I++) WK1[I] = B[I] + BETA * (WK1[I] - AMU * WK3[I]);
    }
    *IER = 3000;                                                     /* 251 */
    reason = 4;
done:
    *ITER = K;                                                       /* 254 */
    EPS[0] = ERR;
    if (stop_reason) *stop_reason = reason;
    free(WK);
    free(W);
    free(WL);
    free(LLTEMP);
}

/* ------------------------------------------------------------------------- */
/* PCGPME_WILL (src2LOWNS/pcgpme_2DH.f90:1-374), the 2DH dispersion solve: the
 * same scaling, sort, LDUSUB and AXSUB as PCGPME on copies of AL, LL and D
 * (57-120), x0 = 0 (59-66), no EPS substitution, BETA = C1 / (AMU RQ) (255),
 * and the solution post-processed into B (265-279). */

/* Post-processing of pcgpme_2DH.f90:268-279, serial in row order: |x| <= 1e-14
 * becomes 0; a neighbour (original LL, 0 ends the list, a self-reference is
 * skipped) whose value differs by at most 1e-14 replaces x(i); B(i) = x(i) is
 * written inside the neighbour loop only, so a row whose loop never reaches
 * that statement keeps B(i), the last residual. */
void ora_will_postprocess(double* X, double* B, const int* ll, int nl, long na, int n) {
    const double L_Limit = 1.0e-14;
    for (int i = 1; i <= n; i++) {
        if (fabs(X[i - 1]) <= L_Limit) X[i - 1] = ZERO;
        for (int k = 1; k <= nl; k++) {
            const int j = ll[(long)(k - 1) * na + (i - 1)];
            if (j == i) continue;
            if (j == 0) break;
            if (X[i - 1] == X[j - 1]) continue;
            if (fabs(X[i - 1] - X[j - 1]) <= L_Limit) X[i - 1] = X[j - 1];
            B[i - 1] = X[i - 1];
        }
    }
}

void ora_pcgpme_will(const double* al_in, int NL, int na, const int* ll_in, const double* d_in, int N, int N2,
                     double* B, double EPS, double PARM, int ITER, int nthreads, int* iters_out, int* reason_out) {
    long NA = na;
    int nt = nthreads > 1 ? nthreads : 1;
    double BN, C1, ALP, AMU, RN, RQ, BETA, ERR = ZERO, SS, ERRP = ZERO, P1, P2;
    int K, reason = 4;
    P1 = PARM;                                                       /* 51-53 */
    if (PARM < ONE) P1 = TWO * TWO;
    P2 = P1 + ONE;
    long L = (long)N + N2;
    double* al = (double*)malloc(sizeof(double) * (size_t)NA * NL);  /* ALTEMP, LLTEMP, DTEMP */
    int* ll = (int*)malloc(sizeof(int) * (size_t)NA * NL);
    double* D = (double*)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
    memcpy(al, al_in, sizeof(double) * (size_t)NA * NL);
    memcpy(ll, ll_in, sizeof(int) * (size_t)NA * NL);
    memcpy(D, d_in, sizeof(double) * (size_t)N);
    double* X = (double*)calloc((size_t)L, sizeof(double));
    double* WK = (double*)calloc((size_t)L * 5, sizeof(double));
    double* W = (double*)calloc((size_t)L, sizeof(double));
    double* WL = (double*)calloc((size_t)L, sizeof(double));
    double* WK1 = WK;
    double* WK2 = WK + L;
    double* WK3 = WK + 2 * L;
    double* WK4 = WK + 3 * L;
    double* WK5 = WK + 4 * L;

    setup_(al, NL, NA, ll, D, N, B, P1, P2, W, nt);                  /* 81-120 */
    for (int I = 0; I < N; I++) WK1[I] = B[I];                       /* 122-126 */
    ldusub_(al, NL, NA, ll, N, N2, WK1, WL, nt);                     /* 130 */
    axsub_(al, NL, NA, ll, D, N, X, WK3, nt);                        /* 133 */
    ldusub_(al, NL, NA, ll, N, N2, WK3, WL, nt);                     /* 134 */
    BN = ZERO;
    C1 = ZERO;
#pragma omp parallel for schedule(static) reduction(+ : BN, C1) if (nt > 1) num_threads(nt)
    for (int I = 0; I < N; I++) {                                    /* 139-150 */
        double TEMP = WK1[I];
        BN = BN + TEMP * TEMP;
        TEMP = TEMP - WK3[I];
        B[I] = TEMP;
        C1 = C1 + TEMP * TEMP;
        WK1[I] = TEMP;
        WK2[I] = TEMP;
    }
    for (K = 1; K <= ITER; K++) {                                    /* 155 */
        axsub_(al, NL, NA, ll, D, N, WK1, WK3, nt);
        ldusub_(al, NL, NA, ll, N, N2, WK3, WL, nt);
        RQ = ZERO;
#pragma omp parallel for schedule(static) reduction(+ : RQ) if (nt > 1) num_threads(nt)
        for (int I = 0; I < N; I++) RQ = RQ + WK2[I] * WK3[I];
        ALP = C1 / RQ;
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt)
        for (int I = 0; I < N; I++) WK4[I] = B[I] - ALP * WK3[I];
        axsub_(al, NL, NA, ll, D, N, WK4, WK5, nt);
        ldusub_(al, NL, NA, ll, N, N2, WK5, WL, nt);
        AMU = ZERO;
        SS = ZERO;
#pragma omp parallel for schedule(static) reduction(+ : AMU, SS) if (nt > 1) num_threads(nt)
        for (int I = 0; I < N; I++) {
            double TEMP = WK5[I];
            AMU = AMU + WK4[I] * TEMP;
            SS = SS + TEMP * TEMP;
        }
        AMU = AMU / SS;
        C1 = ZERO;
        RN = ZERO;
#pragma omp parallel for schedule(static) reduction(+ : RN, C1) if (nt > 1) num_threads(nt)
        for (int I = 0; I < N; I++) {
            double TEMP = WK4[I];
            X[I] = X[I] + ALP * WK1[I] + AMU * TEMP;
            TEMP = TEMP - AMU * WK5[I];
            B[I] = TEMP;
            RN = RN + TEMP * TEMP;
            C1 = C1 + TEMP * WK2[I];
        }
        ERR = sqrt(RN / BN);                                         /* 222 */
        if (K >= 10 && fabs(ERR - ERRP) <= ERR * 1.0e-6) { reason = 1; goto done; }  /* 246 */
        if (ERR <= EPS) { reason = 0; goto done; }                   /* 250 */
        ERRP = ERR;
        if (AMU == ZERO) { reason = 2; goto done; }                  /* 252 */
        if (C1 == ZERO) { reason = 3; goto done; }                   /* 254 */
        BETA = C1 / (AMU * RQ);                                      /* 255 */
#pragma omp parallel for schedule(static) if (nt > 1) num_threads(nt)
        for (int I = 0; I < N; I++) WK1[I] = B[I] + BETA * (WK1[I] - AMU * WK3[I]);
    }
    reason = 4;                                                      /* 263: IER = 3000, not returned */
done:
    if (iters_out) *iters_out = K;
    if (reason_out) *reason_out = reason;
    ora_will_postprocess(X, B, ll_in, NL, NA, N);                    /* 265-279 */
    free(al);
    free(ll);
    free(D);
    free(X);
    free(WK);
    free(W);
    free(WL);
}

void ora_pcgpme_setup(double* al, int nl, int na, int* ll, double* d, int n, double* b,
                      double parm) {
    double P1 = parm < ONE ? TWO * TWO : parm, P2 = P1 + ONE;
    double* W = (double*)calloc((size_t)n, sizeof(double));
    setup_(al, nl, na, ll, d, n, b, P1, P2, W, 1);
    free(W);
}

void ora_axsub(const double* al, int nl, int na, const int* ll, const double* d, int n,
               int n2, const double* x, double* y) {
    (void)n2;
    axsub_(al, nl, na, ll, d, n, x, y, 1);
}

void ora_ldusub(const double* al, int nl, int na, const int* ll, int n, int n2,
                double* p_inout) {
    double* W = (double*)calloc((size_t)n + n2, sizeof(double));
    ldusub_(al, nl, na, ll, n, n2, p_inout, W, 1);
    free(W);
}

/* ------------------------------------------------------------------------- */
/* Pressure update (1sub-momentum.F90:52-58) and estimate_velocity2 (590-651),
 * with momentum_d (lib/src/math_func.F90:251-254).  xe addresses xe(0). */
void ora_correct(const int* dims, int inne, int mx2, const int* mn, const int* in_,
                 const int* jn, const int* kn, const int* nf, const int* nfb,
                 const double* a, const double* dx, double dt, int mnoe,
                 const int* mno2mn, const int* mno, const double* xe, double* p,
                 double* un) {
    (void)mx2;
    grid_t g = mkgrid(dims);
#define MNO(i, k, j) mno[(long)((i) - 1) + (long)g.ie * ((long)((k) - 1) + (long)g.ke * ((j) - 1))]
    for (int r = 1; r <= mnoe; r++) p[mno2mn[r]] = p[mno2mn[r]] - xe[r];
    for (int nn = 1; nn <= inne; nn++) {
        if (nf[nn] == 0) continue;
        if (nf[nn] == IOB && nfb[nn] != 4) continue;
        int i = in_[nn], j = jn[nn], k = kn[nn];
        int ic[3] = {i, j, k};
        int nnn = MNO(i, k, j);
        double xec = -xe[nnn];
        int nno[3] = {MNO(i - 1, k, j), MNO(i, k, j - 1), MNO(i, k - 1, j)};
        int nnm[3] = {MN(i - 1, k, j), MN(i, k, j - 1), MN(i, k - 1, j)};
        int nfm[3] = {nf[nnm[0]], nf[nnm[1]], nf[nnm[2]]};
        int nfbm[3] = {nfb[nnm[0]], nfb[nnm[1]], nfb[nnm[2]]};
        if (nf[nn] == IOB && nfb[nn] == 4) {
            for (int l = 0; l <= 2; l++) {
                if (nfm[l] >= 1) {
                    double dxc = (DXC(l, ic[l]) + DXC(l, ic[l] - 1)) * HALF;
                    UNF(l, nn) = UNF(l, nn) + dt * (-xe[nno[l]] - (-xe[nnn])) / dxc;
                }
            }
        } else {
            for (int l = 0; l <= 2; l++) {
                if (AF(l, nn) != ZERO) {
                    double dxc = (DXC(l, ic[l]) + DXC(l, ic[l] - 1)) * HALF;
                    if (nfm[l] >= 1) {
                        UNF(l, nn) = UNF(l, nn) + dt * (-xe[nno[l]] - xec) / dxc;
                        if (fabs(UNF(l, nn)) < TINY) UNF(l, nn) = ZERO;
                    } else if (nfm[l] == -1 && nfbm[l] == 4) {
                        UNF(l, nn) = UNF(l, nn) + dt * (-xe[nno[l]] - xec) / dxc;
                    }
                }
            }
        }
    }
#undef MNO
}

/* ------------------------------------------------------------------------- */
/* Transposed ELL (adjoint support; no reference counterpart).  alu/llu are the
 * assembled arrays (1-based llu, leading dimension na); column d of row j names
 * the neighbour in direction d, so A(j,i) lands in row i at the opposite slot. */
void ora_transpose(int n, int na, int nl, const double* alu, const int* llu, const double* de,
                   double* alt, int* llt, double* det) {
    for (int d = 0; d < nl; d++)
        for (int r = 0; r < na; r++) { alt[(long)d * na + r] = ZERO; llt[(long)d * na + r] = 0; }
    for (int r = 0; r < n; r++) det[r] = de[r];
    for (int j = 1; j <= n; j++)
        for (int d = 1; d <= nl; d++) {
            int i = llu[(long)(d - 1) * na + (j - 1)];
            if (i == 0) continue;
            int od = (d % 2) ? d + 1 : d - 1;
            alt[(long)(od - 1) * na + (i - 1)] = alu[(long)(d - 1) * na + (j - 1)];
            llt[(long)(od - 1) * na + (i - 1)] = j;
        }
}

void ora_spmv(int n, int na, int nl, const double* alu, const int* llu, const double* de,
              const double* x, double* y) {
    for (int i = 1; i <= n; i++) {
        double s = de[i - 1] * x[i - 1];
        for (int d = 1; d <= nl; d++) {
            int c = llu[(long)(d - 1) * na + (i - 1)];
            if (c) s += alu[(long)(d - 1) * na + (i - 1)] * x[c - 1];
        }
        y[i - 1] = s;
    }
}
