// session.cu -- the pressure-correction ik loop of one 3D domain on the device.
//
// The reference runs, for every time step (src2LOWNS/1sub-momentum.F90:41-60):
//   ik = 0; do
//     cal_err_of_continuity  (rows at ik == 0, RHS, dmax)        235-360
//     check_dmax             (stop on dmax < d0, icon, ik > 1000) 419-463
//     cal_matrix_element                                          465-551
//     cal_poisson_equation   (PCGPME, ier -> icon)                553-588
//     p(mno2mn) -= xe ; estimate_velocity2                        52-59, 590-651
//   end do
// A session keeps the domain's module arrays in HBM and runs that loop with one
// host read-back of dmax per ik (the loop's only control input).
#include <cstring>
#include <mutex>

#include "engine.cuh"
#include "engine_api.h"
#include "grid_index.cuh"
#include "trace.h"

extern "C" {
size_t clowns_set_nflag_workspace_bytes(const int* dims, int inne2);
int clowns_set_nflag_dev(const int* dims, int inne, int inne2, int mx2, const int* mn, const int* in_,
                         const int* jn, const int* kn, int* nf, int* nfb, double* f, const double* fb,
                         const double* a, const double* dx, const int* objno, int* fln, int* ifln_out,
                         int* sfn, int* isfn_out, int* passes_out, void* work, size_t work_bytes, void* stream);
int clowns_init_matrix_dev(const int* dims, int inne, int mx2, const int* mn, const int* in_, const int* jn,
                           const int* kn, const int* nf, const int* nfb, const double* a, const double* fb,
                           const double* dx, double* mp, double* alu_c, int* ll_c, double* de_c, void* stream);
size_t clowns_rows_rhs_workspace_bytes(int ifln);
int clowns_rows_rhs_dev(const int* dims, int inne2, int mx2, const int* mn, const int* in_, const int* jn,
                        const int* kn, const int* nf, const int* nfb, const double* f, const double* fb,
                        const double* a, const double* un, const double* dx, const double* mp, double dt,
                        int ifln, const int* fln, int mm2, int* mno, int* mno2mn, double* b, double* xe,
                        double* de, int* mnoe_out, double* dmax_out, void* work, size_t work_bytes, void* stream);
int clowns_assemble_dev(const int* dims, int inne, int inne2, int mx2, const int* in_, const int* jn,
                        const int* kn, const int* nf, const int* nfb, const double* x, const double* dx,
                        const double* sp, int ifln, const int* fln, const int* mno, const double* alu_c,
                        const int* ll_c, const double* de_c, int mm2, double* alu, int* llu, double* de,
                        int* err_cell, void* stream);
int clowns_correct_dev(const int* dims, int inne, int mx2, const int* mn, const int* in_, const int* jn,
                       const int* kn, const int* nf, const int* nfb, const double* a, const double* dx, double dt,
                       int mnoe, const int* mno2mn, const int* mno, const double* xe0, double* p, double* un,
                       void* stream);
}

using namespace clowns;

struct clowns_session {
    int dims[6];
    int inne, inne2, mx2;
    cudaStream_t stream;
    // static grid
    int *mn, *in_, *jn, *kn, *objno;
    double *x, *dx;
    size_t n_mn;
    // per-step fields
    int *nf, *nfb;
    double *f, *fb, *a, *un, *sp, *p;
    // classification
    int *fln, *sfn;
    int ifln, isfn;
    // static coefficients (init_matrix, once)
    double *mp, *alu_c, *de_c;
    int* ll_c;
    int have_static;
    // matrix rows (sized on first use: mm2 = ifln + 5000, 1sub-momentum.F90:254)
    int mm2, mnoe;
    int *mno, *mno2mn, *llu, *err_cell;
    double *b, *xe, *de, *alu;
    // workspaces
    void *ws_nflag, *ws_rows, *ws_solve;
    size_t ws_nflag_bytes, ws_rows_bytes, ws_solve_bytes;
};

#define SESSION_TRY(expr)                                   \
    do {                                                    \
        int _rc = (expr);                                   \
        if (_rc) return _rc;                                \
    } while (0)

static int dev_alloc(void** p, size_t bytes) {
    CLOWNS_CUDA_TRY(cudaMalloc(p, bytes ? bytes : 16));
    return CLOWNS_OK;
}

static int upload(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    return CLOWNS_OK;
}

static int download(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    return CLOWNS_OK;
}

extern "C" int clowns_session_create(clowns_session** out, const int* dims, int inne, int inne2, int mx2,
                                     const int* mn, const int* in_, const int* jn, const int* kn,
                                     const double* x, const double* dx, const int* objno) {
    if (!out || !grid_dims_ok(dims) || !grid_has_matrix(dims) || inne < 1 || inne2 < inne || mx2 < 1 || !mn || !in_ ||
        !jn || !kn || !x || !dx || !objno) {
        set_last_error_msg("session_create: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    clowns_session* S = new clowns_session;
    memset(S, 0, sizeof(*S));
    memcpy(S->dims, dims, sizeof(S->dims));
    S->inne = inne;
    S->inne2 = inne2;
    S->mx2 = mx2;
    *out = S;
    GridIdx g = GridIdx::make(dims);
    S->n_mn = (size_t)g.ni * g.nk * g.nj;
    const size_t nc = (size_t)inne2 + 2;
    CLOWNS_CUDA_TRY(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
    cudaStream_t s = S->stream;
    SESSION_TRY(dev_alloc((void**)&S->mn, sizeof(int) * S->n_mn));
    SESSION_TRY(dev_alloc((void**)&S->in_, sizeof(int) * nc));
    SESSION_TRY(dev_alloc((void**)&S->jn, sizeof(int) * nc));
    SESSION_TRY(dev_alloc((void**)&S->kn, sizeof(int) * nc));
    SESSION_TRY(dev_alloc((void**)&S->objno, sizeof(int) * nc));
    SESSION_TRY(dev_alloc((void**)&S->x, sizeof(double) * 3 * mx2));
    SESSION_TRY(dev_alloc((void**)&S->dx, sizeof(double) * 3 * mx2));
    SESSION_TRY(dev_alloc((void**)&S->nf, sizeof(int) * nc));
    SESSION_TRY(dev_alloc((void**)&S->nfb, sizeof(int) * nc));
    SESSION_TRY(dev_alloc((void**)&S->f, sizeof(double) * nc));
    SESSION_TRY(dev_alloc((void**)&S->fb, sizeof(double) * nc));
    SESSION_TRY(dev_alloc((void**)&S->a, sizeof(double) * 3 * nc));
    SESSION_TRY(dev_alloc((void**)&S->un, sizeof(double) * 3 * nc));
    SESSION_TRY(dev_alloc((void**)&S->sp, sizeof(double) * 3 * nc));
    SESSION_TRY(dev_alloc((void**)&S->p, sizeof(double) * nc));
    SESSION_TRY(dev_alloc((void**)&S->fln, sizeof(int) * (nc + 1)));
    SESSION_TRY(dev_alloc((void**)&S->sfn, sizeof(int) * (nc + 1)));
    SESSION_TRY(dev_alloc((void**)&S->mp, sizeof(double)));
    SESSION_TRY(dev_alloc((void**)&S->alu_c, sizeof(double) * 6 * (size_t)inne));
    SESSION_TRY(dev_alloc((void**)&S->ll_c, sizeof(int) * 6 * (size_t)inne));
    SESSION_TRY(dev_alloc((void**)&S->de_c, sizeof(double) * (size_t)inne));
    SESSION_TRY(dev_alloc((void**)&S->err_cell, sizeof(int)));
    S->ws_nflag_bytes = clowns_set_nflag_workspace_bytes(dims, inne2);
    SESSION_TRY(dev_alloc(&S->ws_nflag, S->ws_nflag_bytes));
    SESSION_TRY(upload(S->mn, mn, sizeof(int) * S->n_mn, s));
    SESSION_TRY(upload(S->in_, in_, sizeof(int) * nc, s));
    SESSION_TRY(upload(S->jn, jn, sizeof(int) * nc, s));
    SESSION_TRY(upload(S->kn, kn, sizeof(int) * nc, s));
    SESSION_TRY(upload(S->objno, objno, sizeof(int) * nc, s));
    SESSION_TRY(upload(S->x, x, sizeof(double) * 3 * mx2, s));
    SESSION_TRY(upload(S->dx, dx, sizeof(double) * 3 * mx2, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    return CLOWNS_OK;
}

extern "C" int clowns_session_set_fields(clowns_session* S, const int* nf, const int* nfb, const double* f,
                                         const double* fb, const double* a, const double* un, const double* sp,
                                         const double* p) {
    if (!S || !nf || !nfb || !f || !fb || !a || !un || !sp || !p) {
        set_last_error_msg("session_set_fields: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    const size_t nc = (size_t)S->inne2 + 2;
    cudaStream_t s = S->stream;
    SESSION_TRY(upload(S->nf, nf, sizeof(int) * nc, s));
    SESSION_TRY(upload(S->nfb, nfb, sizeof(int) * nc, s));
    SESSION_TRY(upload(S->f, f, sizeof(double) * nc, s));
    SESSION_TRY(upload(S->fb, fb, sizeof(double) * nc, s));
    SESSION_TRY(upload(S->a, a, sizeof(double) * 3 * nc, s));
    SESSION_TRY(upload(S->un, un, sizeof(double) * 3 * nc, s));
    SESSION_TRY(upload(S->sp, sp, sizeof(double) * 3 * nc, s));
    SESSION_TRY(upload(S->p, p, sizeof(double) * nc, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    return CLOWNS_OK;
}

// set_nflag on the session's fields (called every step by cal_vof, 1sub-vof.F90:37)
extern "C" int clowns_session_classify(clowns_session* S, int* ifln, int* isfn) {
    clowns::TraceRange trace_range_("clowns_session_classify");
    if (!S) return CLOWNS_ERR_ARG;
    int passes = 0;
    SESSION_TRY(clowns_set_nflag_dev(S->dims, S->inne, S->inne2, S->mx2, S->mn, S->in_, S->jn, S->kn, S->nf,
                                     S->nfb, S->f, S->fb, S->a, S->dx, S->objno, S->fln, &S->ifln, S->sfn,
                                     &S->isfn, &passes, S->ws_nflag, S->ws_nflag_bytes, S->stream));
    if (ifln) *ifln = S->ifln;
    if (isfn) *isfn = S->isfn;
    if (!S->have_static) {
        // init_matrix runs once, at initial_setting (main_2CLOWNS.F90:54)
        SESSION_TRY(clowns_init_matrix_dev(S->dims, S->inne, S->mx2, S->mn, S->in_, S->jn, S->kn, S->nf, S->nfb,
                                           S->a, S->fb, S->dx, S->mp, S->alu_c, S->ll_c, S->de_c, S->stream));
        S->have_static = 1;
    }
    // (re)size the matrix rows: m_alloc = ifln + 5000 (1sub-momentum.F90:253-263)
    const int need = S->ifln + 5000;
    if (S->mm2 < S->ifln + 60) {
        cudaFree(S->mno); cudaFree(S->mno2mn); cudaFree(S->llu); cudaFree(S->b); cudaFree(S->xe);
        cudaFree(S->de); cudaFree(S->alu); cudaFree(S->ws_rows); cudaFree(S->ws_solve);
        S->mm2 = need;
        GridIdx g = GridIdx::make(S->dims);
        SESSION_TRY(dev_alloc((void**)&S->mno, sizeof(int) * (size_t)g.ie * g.ke * g.je));
        SESSION_TRY(dev_alloc((void**)&S->mno2mn, sizeof(int) * (size_t)need));
        SESSION_TRY(dev_alloc((void**)&S->llu, sizeof(int) * 6 * (size_t)need));
        SESSION_TRY(dev_alloc((void**)&S->alu, sizeof(double) * 6 * (size_t)need));
        SESSION_TRY(dev_alloc((void**)&S->b, sizeof(double) * (size_t)need));
        SESSION_TRY(dev_alloc((void**)&S->xe, sizeof(double) * ((size_t)need + 1)));
        SESSION_TRY(dev_alloc((void**)&S->de, sizeof(double) * (size_t)need));
        S->ws_rows_bytes = clowns_rows_rhs_workspace_bytes(S->ifln);
        SESSION_TRY(dev_alloc(&S->ws_rows, S->ws_rows_bytes));
        S->ws_solve_bytes = 0;
        S->ws_solve = nullptr;
        CLOWNS_CUDA_TRY(cudaMemsetAsync(S->xe, 0, sizeof(double), S->stream));   // xe(0)
    } else if (clowns_rows_rhs_workspace_bytes(S->ifln) > S->ws_rows_bytes) {
        cudaFree(S->ws_rows);
        S->ws_rows_bytes = clowns_rows_rhs_workspace_bytes(S->ifln);
        SESSION_TRY(dev_alloc(&S->ws_rows, S->ws_rows_bytes));
    }
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(S->stream));
    return CLOWNS_OK;
}

// The ik loop.  precision: CLOWNS_PREC_FP64 (PCGPME) or CLOWNS_PREC_MIXED.
// Outputs: ik and dmax at exit, the last solve's iterations and ERR, and icon as
// the reference's caller would set it (0, or 12/96/911/1030 for failures).
extern "C" int clowns_session_pressure_loop(clowns_session* S, double dt, double d0, double eps0, int precision,
                                            int* ik_out, double* dmax_out, int* iter_out, double* err_out,
                                            int* icon_out) {
    clowns::TraceRange trace_range_("clowns_session_pressure_loop");
    if (!S || S->mm2 == 0 || dt <= 0) {
        set_last_error_msg("session_pressure_loop: classify the fields first");
        return CLOWNS_ERR_ARG;
    }
    cudaStream_t s = S->stream;
    int ik = 0, icon = 0, last_iter = 0;
    double dmax = 0.0, last_err = 0.0;
    for (;;) {
        int mnoe = 0;
        // cal_err_of_continuity: the numbering is recomputed each ik from the same
        // fluid list, which leaves it unchanged (the reference numbers at ik == 0)
        SESSION_TRY(clowns_rows_rhs_dev(S->dims, S->inne2, S->mx2, S->mn, S->in_, S->jn, S->kn, S->nf, S->nfb,
                                        S->f, S->fb, S->a, S->un, S->dx, S->mp, dt, S->ifln, S->fln, S->mm2,
                                        S->mno, S->mno2mn, S->b, S->xe + 1, S->de, &mnoe, &dmax, S->ws_rows,
                                        S->ws_rows_bytes, s));
        S->mnoe = mnoe;
        // check_dmax (1sub-momentum.F90:419-463)
        if (icon != 0) { icon = 1030; break; }
        if (dmax < d0) break;
        ik += 1;
        if (ik > 1000) break;
        // cal_matrix_element
        SESSION_TRY(clowns_assemble_dev(S->dims, S->inne, S->inne2, S->mx2, S->in_, S->jn, S->kn, S->nf, S->nfb,
                                        S->x, S->dx, S->sp, S->ifln, S->fln, S->mno, S->alu_c, S->ll_c, S->de_c,
                                        S->mm2, S->alu, S->llu, S->de, S->err_cell, s));
        int bad = 0;
        SESSION_TRY(download(&bad, S->err_cell, sizeof(int), s));
        CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
        if (bad) {
            set_last_error_msg("cal_matrix_element: unexpected flag on a row cell");
            return CLOWNS_ERR_ARG;
        }
        // cal_poisson_equation: iter = 10000, eps1 = (eps0, 0), parm = 5
        const int mixed = precision == CLOWNS_PREC_MIXED;
        const size_t need = engine_workspace_bytes(1, &mnoe, mixed);
        if (need > S->ws_solve_bytes) {
            cudaFree(S->ws_solve);
            S->ws_solve_bytes = need + need / 8;
            SESSION_TRY(dev_alloc(&S->ws_solve, S->ws_solve_bytes));
        }
        MemberIn in;
        in.al = S->alu; in.ll = S->llu; in.d = S->de; in.b = S->b; in.x = S->xe + 1;
        in.na = S->mm2; in.n = mnoe; in.nl = GridIdx::make(S->dims).nl(); in.pad = 0;
        clowns_solve_info info;
        memset(&info, 0, sizeof(info));
        if (mixed)
            SESSION_TRY(engine_solve_mixed(1, &in, eps0, 5.0, 0.0, 0, 0, S->ws_solve, S->ws_solve_bytes, s, &info));
        else
            SESSION_TRY(engine_solve_plain(1, &in, eps0, 5.0, 10000, S->ws_solve, S->ws_solve_bytes, s, &info));
        last_iter = info.iter;
        last_err = info.eps;
        // ier -> icon (1sub-momentum.F90:568-587)
        if (info.ier == 3000) {
        } else if (info.ier == 2100 || info.ier == 2200 || info.ier == 2300) {
            icon = 96;
        } else if (info.ier == 12) {
            icon = 12;
        } else if (info.ier != 0) {
            icon = 911;
        }
        // p -= xe ; estimate_velocity2
        SESSION_TRY(clowns_correct_dev(S->dims, S->inne, S->mx2, S->mn, S->in_, S->jn, S->kn, S->nf, S->nfb, S->a,
                                       S->dx, dt, mnoe, S->mno2mn, S->mno, S->xe, S->p, S->un, s));
    }
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    if (ik_out) *ik_out = ik;
    if (dmax_out) *dmax_out = dmax;
    if (iter_out) *iter_out = last_iter;
    if (err_out) *err_out = last_err;
    if (icon_out) *icon_out = icon;
    return CLOWNS_OK;
}

extern "C" int clowns_session_get_fields(clowns_session* S, int* nf, int* nfb, double* f, double* p, double* un,
                                         int* mnoe) {
    if (!S) return CLOWNS_ERR_ARG;
    const size_t nc = (size_t)S->inne2 + 2;
    cudaStream_t s = S->stream;
    if (nf) SESSION_TRY(download(nf, S->nf, sizeof(int) * nc, s));
    if (nfb) SESSION_TRY(download(nfb, S->nfb, sizeof(int) * nc, s));
    if (f) SESSION_TRY(download(f, S->f, sizeof(double) * nc, s));
    if (p) SESSION_TRY(download(p, S->p, sizeof(double) * nc, s));
    if (un) SESSION_TRY(download(un, S->un, sizeof(double) * 3 * nc, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    if (mnoe) *mnoe = S->mnoe;
    return CLOWNS_OK;
}

extern "C" int clowns_session_destroy(clowns_session* S) {
    if (!S) return CLOWNS_OK;
    cudaStreamSynchronize(S->stream);
    void* bufs[] = {S->mn, S->in_, S->jn, S->kn, S->objno, S->x, S->dx, S->nf, S->nfb, S->f, S->fb, S->a,
                    S->un, S->sp, S->p, S->fln, S->sfn, S->mp, S->alu_c, S->ll_c, S->de_c, S->mno,
                    S->mno2mn, S->llu, S->err_cell, S->b, S->xe, S->de, S->alu, S->ws_nflag, S->ws_rows,
                    S->ws_solve};
    for (void* b : bufs)
        if (b) cudaFree(b);
    cudaStreamDestroy(S->stream);
    delete S;
    return CLOWNS_OK;
}
