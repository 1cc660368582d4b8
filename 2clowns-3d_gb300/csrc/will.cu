// will.cu -- PCGPME_WILL, the 2DH dispersion solve (src2LOWNS/pcgpme_2DH.f90:1-374).
//
// The iteration is PCGPME's (same scaling, per-row sort, LDUSUB and AXSUB on an
// NL = 4 matrix) with BETA = C1 / (AMU RQ), x0 = 0 and EPS taken as given; it
// runs on the engine as a one-member solve in mode 2.  What differs is the
// output: the reference returns the solution in B after a serial pass
// (268-279) that clamps |x| <= 1e-14 to 0 and replaces x(i) by a neighbour's
// value when they differ by at most 1e-14, comparing with the already
// processed x of lower rows and the unprocessed x of higher ones, and that
// writes B(i) = x(i) only inside its neighbour loop -- a row whose loop ends
// before that statement (no neighbour before the first LL = 0, or only equal
// or self neighbours) keeps B(i), the last recursive residual.
//
// On the GPU that serial pass is a fixed point: row i's result depends only on
// the results of lower rows, so repeating a parallel pass that reads the
// previous pass's values for lower rows and the raw solution for higher rows
// reaches the serial result after (longest chain of replacements + 1) passes;
// the loop stops at the first pass that changes nothing.
#include <cmath>
#include <cstring>
#include <mutex>

#include "engine.cuh"
#include "engine_api.h"
#include "trace.h"

namespace clowns {

constexpr double kWillLimit = 1.0e-14;      // L_Limit, pcgpme_2DH.f90:48
constexpr int kWillMaxPasses = 4096;

// One pass of the post-processing.  yold: the previous pass's processed x
// (any values on the first pass); ynew, b: this pass's results.
__global__ void k_will_pass(const double* __restrict__ x, const double* __restrict__ yold, double* __restrict__ ynew,
                            const double* __restrict__ r, const int* __restrict__ ll, long na, int nl, int n,
                            double* __restrict__ b, int* changed) {
    for (int ii = blockIdx.x * blockDim.x + threadIdx.x; ii < n; ii += gridDim.x * blockDim.x) {
        const int i = ii + 1;
        double xi = x[ii];
        if (fabs(xi) <= kWillLimit) xi = 0.0;
        double bo = r[ii];
        for (int k = 0; k < nl; k++) {
            const int j = ll[(long)k * na + ii];
            if (j == i) continue;
            if (j <= 0 || j > n) break;            // 0 ends the list (indices were validated by the solve)
            const double xj = j < i ? yold[j - 1] : x[j - 1];
            if (xi == xj) continue;
            if (fabs(xi - xj) <= kWillLimit) xi = xj;
            bo = xi;
        }
        ynew[ii] = xi;
        b[ii] = bo;
        if (__double_as_longlong(xi) != __double_as_longlong(yold[ii])) *changed = 1;
    }
}

static size_t will_post_bytes(int n) { return 2 * align_up(sizeof(double) * (size_t)n, 256) + 256; }

// Post-processing into b (and the processed x into x_out, may be null) with
// two scratch vectors and a flag in `work`.
static int will_postprocess(const double* x, const double* r, const int* ll, int nl, int na, int n, double* b,
                            double* x_out, void* work, cudaStream_t s) {
    char* w = (char*)work;
    double* ya = (double*)w;
    double* yb = (double*)(w + align_up(sizeof(double) * (size_t)n, 256));
    int* flag = (int*)(w + 2 * align_up(sizeof(double) * (size_t)n, 256));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(ya, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    const int block = 256;
    const int grid = std::min((n + block - 1) / block, kNumSMs * 16);
    for (int pass = 0; pass < kWillMaxPasses; pass++) {
        int changed = 0;
        CLOWNS_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), s));
        k_will_pass<<<grid, block, 0, s>>>(x, ya, yb, r, ll, na, nl, n, b, flag);
        CLOWNS_CUDA_TRY(cudaGetLastError());
        CLOWNS_CUDA_TRY(cudaMemcpyAsync(&changed, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
        std::swap(ya, yb);                        // ya: this pass's processed x
        if (!changed) {
            if (x_out) CLOWNS_CUDA_TRY(cudaMemcpyAsync(x_out, ya, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
            return CLOWNS_OK;
        }
    }
    set_last_error_msg("pcgpme_will: post-processing did not settle (chain of replacements too long)");
    return CLOWNS_ERR_NOCONV;
}

struct WillLayout {
    size_t o_x, o_post, o_eng, eng_bytes, total;
};

static WillLayout will_layout(int n) {
    WillLayout L;
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return at; };
    L.o_x = take(sizeof(double) * (size_t)n);
    L.o_post = take(will_post_bytes(n));
    L.eng_bytes = engine_workspace_bytes(1, &n, 0);
    L.o_eng = take(L.eng_bytes);
    L.total = o;
    return L;
}

}  // namespace clowns

using namespace clowns;

extern "C" size_t clowns_pcgpme_will_workspace_bytes(int n, int nl) {
    if (n < 1 || nl != 4 && nl != 6) return 0;
    return will_layout(n).total;
}

extern "C" int clowns_pcgpme_will_dev(const double* al, int nl, int na, const int* ll, const double* d, int n,
                                      double* b, double eps, double parm, int iter, void* work, size_t work_bytes,
                                      void* stream, clowns_solve_info* info) {
    clowns::TraceRange trace_range_("clowns_pcgpme_will_dev");
    if (!al || !ll || !d || !b || !work || n < 1 || na < n || (nl != 4 && nl != 6)) {
        set_last_error_msg("pcgpme_will: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    const WillLayout L = will_layout(n);
    if (work_bytes < L.total) {
        set_last_error_msg("pcgpme_will: workspace too small");
        return CLOWNS_ERR_WORKSPACE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    char* w = (char*)work;
    double* x = (double*)(w + L.o_x);
    CLOWNS_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, s));        // x0 = 0 (pcgpme_2DH.f90:59-66)
    MemberIn in;
    in.al = al; in.ll = ll; in.d = d; in.b = b; in.x = x;
    in.na = na; in.n = n; in.nl = nl; in.pad = 0;
    clowns_solve_info local;
    clowns_solve_info* inf = info ? info : &local;
    int rc = engine_solve_plain(1, &in, eps, parm, iter, w + L.o_eng, L.eng_bytes, s, inf, 2);
    if (rc) return rc;
    if (inf->ier == CLOWNS_IER_ARG) {
        set_last_error_msg("pcgpme_will: a column index is outside 0..n");
        return CLOWNS_ERR_ARG;
    }
    const double* r = engine_residual_ptr(w + L.o_eng, n);
    return will_postprocess(x, r, ll, nl, na, n, b, nullptr, w + L.o_post, s);
}

extern "C" size_t clowns_will_postprocess_workspace_bytes(int n) { return n < 1 ? 0 : will_post_bytes(n); }

extern "C" int clowns_will_postprocess_dev(const double* x, const double* r, const int* ll, int nl, int na, int n,
                                           double* b, double* x_out, void* work, size_t work_bytes, void* stream) {
    clowns::TraceRange trace_range_("clowns_will_postprocess_dev");
    if (!x || !r || !ll || !b || !work || n < 1 || na < n || nl < 1) {
        set_last_error_msg("will_postprocess: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    if (work_bytes < will_post_bytes(n)) {
        set_last_error_msg("will_postprocess: workspace too small");
        return CLOWNS_ERR_WORKSPACE;
    }
    return will_postprocess(x, r, ll, nl, na, n, b, x_out, work, (cudaStream_t)stream);
}
