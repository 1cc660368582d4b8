// capi.cu -- error reporting and the host-array drop-in for PCGPME.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "engine.cuh"
#include "engine_api.h"
#include "trace.h"

namespace clowns {

static thread_local char g_err[512] = "";

void set_last_error(cudaError_t e, const char* what, const char* file, int line) {
    snprintf(g_err, sizeof(g_err), "%s: %s (%s:%d)", cudaGetErrorString(e), what, file, line);
}
void set_last_error_msg(const char* msg) { snprintf(g_err, sizeof(g_err), "%s", msg); }

// Device buffers backing the host-array drop-in: grow-only, one set per process,
// reused by every call so that repeated solves of one size replay one cached
// CUDA graph.
struct HostPath {
    std::mutex mu;
    char* dev = nullptr;
    size_t cap = 0;
    cudaStream_t stream = nullptr;
};
static HostPath g_host;

static int host_reserve(size_t bytes) {
    if (!g_host.stream) CLOWNS_CUDA_TRY(cudaStreamCreateWithFlags(&g_host.stream, cudaStreamNonBlocking));
    if (bytes <= g_host.cap) return CLOWNS_OK;
    if (g_host.dev) {
        CLOWNS_CUDA_TRY(cudaStreamSynchronize(g_host.stream));
        release_all_graphs();
        cudaFree(g_host.dev);
        g_host.dev = nullptr;
        g_host.cap = 0;
    }
    size_t want = bytes + bytes / 8;
    CLOWNS_CUDA_TRY(cudaMalloc((void**)&g_host.dev, want));
    g_host.cap = want;
    return CLOWNS_OK;
}

// Host-array solve: packs AL/LL rows 1..N (leading dimension NA) into device
// buffers, solves, and copies X(1:N) back.
static int pcgpme_host(const double* al, int nl, int na, const int* ll, const double* d, int n,
                       const double* b, double* x, double* eps, double parm, int* iter,
                       clowns_solve_info* info) {
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return at; };
    size_t o_al = take(sizeof(double) * (size_t)nl * n);
    size_t o_ll = take(sizeof(int) * (size_t)nl * n);
    size_t o_d = take(sizeof(double) * n);
    size_t o_b = take(sizeof(double) * n);
    size_t o_x = take(sizeof(double) * n);
    size_t wbytes = engine_workspace_bytes(1, &n, 0);
    size_t o_w = take(wbytes);
    int rc = host_reserve(o);
    if (rc) return rc;
    char* base = g_host.dev;
    cudaStream_t s = g_host.stream;
    double* d_al = (double*)(base + o_al);
    int* d_ll = (int*)(base + o_ll);
    double* d_d = (double*)(base + o_d);
    double* d_b = (double*)(base + o_b);
    double* d_x = (double*)(base + o_x);
    CLOWNS_CUDA_TRY(cudaMemcpy2DAsync(d_al, sizeof(double) * n, al, sizeof(double) * (size_t)na,
                                      sizeof(double) * n, nl, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpy2DAsync(d_ll, sizeof(int) * n, ll, sizeof(int) * (size_t)na,
                                      sizeof(int) * n, nl, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(d_d, d, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(d_b, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(d_x, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    MemberIn in;
    in.al = d_al; in.ll = d_ll; in.d = d_d; in.b = d_b; in.x = d_x;
    in.na = n; in.n = n; in.nl = nl; in.pad = 0;
    rc = engine_solve_plain(1, &in, eps[0], parm, *iter, base + o_w, wbytes, s, info);
    if (rc) return rc;
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(x, d_x, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    return CLOWNS_OK;
}

}  // namespace clowns

using namespace clowns;

extern "C" size_t clowns_pcgpme_will_workspace_bytes(int n, int nl);
extern "C" int clowns_pcgpme_will_dev(const double* al, int nl, int na, const int* ll, const double* d, int n,
                                      double* b, double eps, double parm, int iter, void* work, size_t work_bytes,
                                      void* stream, clowns_solve_info* info);

namespace clowns {

// Host-array PCGPME_WILL: packs AL/LL rows 1..N, solves, copies B(1:N) back.
static int pcgpme_will_host(const double* al, int nl, int na, const int* ll, const double* d, int n, double* b,
                            double eps, double parm, int iter) {
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return at; };
    size_t o_al = take(sizeof(double) * (size_t)nl * n);
    size_t o_ll = take(sizeof(int) * (size_t)nl * n);
    size_t o_d = take(sizeof(double) * n);
    size_t o_b = take(sizeof(double) * n);
    size_t wbytes = clowns_pcgpme_will_workspace_bytes(n, nl);
    size_t o_w = take(wbytes);
    int rc = host_reserve(o);
    if (rc) return rc;
    char* base = g_host.dev;
    cudaStream_t s = g_host.stream;
    double* d_al = (double*)(base + o_al);
    int* d_ll = (int*)(base + o_ll);
    double* d_d = (double*)(base + o_d);
    double* d_b = (double*)(base + o_b);
    CLOWNS_CUDA_TRY(cudaMemcpy2DAsync(d_al, sizeof(double) * n, al, sizeof(double) * (size_t)na,
                                      sizeof(double) * n, nl, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpy2DAsync(d_ll, sizeof(int) * n, ll, sizeof(int) * (size_t)na,
                                      sizeof(int) * n, nl, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(d_d, d, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(d_b, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    rc = clowns_pcgpme_will_dev(d_al, nl, n, d_ll, d_d, n, d_b, eps, parm, iter, base + o_w, wbytes, s, nullptr);
    if (rc) return rc;
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b, d_b, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    return CLOWNS_OK;
}

}  // namespace clowns

extern "C" const char* clowns_last_error(void) { return g_err; }
extern "C" int clowns_version(void) { return 10000; }

extern "C" void pcgpme_gpu(double* al, const int* nl, const int* na, int* ll, double* d,
                           const int* n, const int* n2, double* b, double* x, double* eps,
                           const double* parm, int* iter, int* ier) {
    clowns::TraceRange trace_range_("pcgpme_gpu");
    if (!al || !nl || !na || !ll || !d || !n || !n2 || !b || !x || !eps || !parm || !iter || !ier) {
        if (ier) *ier = CLOWNS_IER_ARG;
        set_last_error_msg("pcgpme_gpu: NULL argument");
        return;
    }
    const int NL = *nl, NA = *na, N = *n;
    if (N < 1 || NA < N || (NL != 6 && NL != 4) || *n2 < 0) {
        *ier = CLOWNS_IER_ARG;
        set_last_error_msg("pcgpme_gpu: invalid sizes");
        return;
    }
    std::lock_guard<std::mutex> lk(g_host.mu);
    clowns_solve_info info;
    memset(&info, 0, sizeof(info));
    int rc = pcgpme_host(al, NL, NA, ll, d, N, b, x, eps, *parm, iter, &info);
    if (rc) {
        *ier = CLOWNS_IER_DEVICE;
        return;
    }
    eps[0] = info.eps;
    *iter = info.iter;
    *ier = info.ier;
}

extern "C" void pcgpme_(double* al, const int* nl, const int* na, int* ll, double* d, const int* n,
                        const int* n2, double* b, double* x, double* eps, const double* parm,
                        int* iter, int* ier) {
    pcgpme_gpu(al, nl, na, ll, d, n, n2, b, x, eps, parm, iter, ier);
}

// PCGPME_WILL(AL,NL,NA,LL,D,N,N2,B,EPS,PARM,ITER) with host arrays: B in: right-
// hand side, out: the post-processed solution.  The reference has no error
// argument; a failed call leaves B unchanged and returns a CLOWNS_ERR_* code
// (ignored by a Fortran CALL), with the reason in clowns_last_error().
extern "C" int pcgpme_will_gpu(const double* al, const int* nl, const int* na, const int* ll, const double* d,
                               const int* n, const int* n2, double* b, const double* eps, const double* parm,
                               const int* iter) {
    clowns::TraceRange trace_range_("pcgpme_will_gpu");
    if (!al || !nl || !na || !ll || !d || !n || !n2 || !b || !eps || !parm || !iter) {
        set_last_error_msg("pcgpme_will_gpu: NULL argument");
        return CLOWNS_ERR_ARG;
    }
    const int NL = *nl, NA = *na, N = *n;
    if (N < 1 || NA < N || (NL != 4 && NL != 6) || *n2 < 0 || *iter < 1) {
        set_last_error_msg("pcgpme_will_gpu: invalid sizes");
        return CLOWNS_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(g_host.mu);
    return pcgpme_will_host(al, NL, NA, ll, d, N, b, *eps, *parm, *iter);
}

extern "C" int pcgpme_will_(const double* al, const int* nl, const int* na, const int* ll, const double* d,
                            const int* n, const int* n2, double* b, const double* eps, const double* parm,
                            const int* iter) {
    return pcgpme_will_gpu(al, nl, na, ll, d, n, n2, b, eps, parm, iter);
}
