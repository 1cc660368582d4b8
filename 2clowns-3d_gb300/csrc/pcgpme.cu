// pcgpme.cu -- C ABI of the pressure solves (plain FP64, mixed precision and
// batched ensembles) on top of the batched BiCGSTAB engine (engine.cu).
#include <cstring>
#include <vector>

#include "engine.cuh"
#include "engine_api.h"
#include "trace.h"

using namespace clowns;

static_assert(sizeof(clowns_member) == sizeof(MemberIn), "clowns_member must mirror MemberIn");

static MemberIn member(const double* al, int nl, int na, const int* ll, const double* d, int n,
                       const double* b, double* x) {
    MemberIn in;
    in.al = al;
    in.ll = ll;
    in.d = d;
    in.b = b;
    in.x = x;
    in.na = na;
    in.n = n;
    in.nl = nl;
    in.pad = 0;
    return in;
}

extern "C" size_t clowns_pcgpme_workspace_bytes(int n, int nl) {
    (void)nl;
    if (n < 1) return 0;
    return engine_workspace_bytes(1, &n, 0);
}

extern "C" int clowns_pcgpme_dev(const double* al, int nl, int na, const int* ll, const double* d, int n,
                                 const double* b, double* x, double eps, double parm, int iter, void* work,
                                 size_t work_bytes, void* stream, clowns_solve_info* info) {
    clowns::TraceRange trace_range_("clowns_pcgpme_dev");
    MemberIn in = member(al, nl, na, ll, d, n, b, x);
    return engine_solve_plain(1, &in, eps, parm, iter, work, work_bytes, (cudaStream_t)stream, info);
}

extern "C" size_t clowns_pcgpme_mixed_workspace_bytes(int n, int nl) {
    (void)nl;
    if (n < 1) return 0;
    return engine_workspace_bytes(1, &n, 1);
}

extern "C" int clowns_pcgpme_mixed_dev(const double* al, int nl, int na, const int* ll, const double* d, int n,
                                       const double* b, double* x, double eps, double parm, double inner_tol,
                                       int inner_max, int max_outer, void* work, size_t work_bytes, void* stream,
                                       clowns_solve_info* info) {
    clowns::TraceRange trace_range_("clowns_pcgpme_mixed_dev");
    MemberIn in = member(al, nl, na, ll, d, n, b, x);
    return engine_solve_mixed(1, &in, eps, parm, inner_tol, inner_max, max_outer, work, work_bytes,
                              (cudaStream_t)stream, info);
}

extern "C" size_t clowns_pcgpme_batched_workspace_bytes(int m, const int* n, int precision) {
    if (m < 1 || !n) return 0;
    return engine_workspace_bytes(m, n, precision == CLOWNS_PREC_MIXED);
}

extern "C" int clowns_pcgpme_batched_dev(int m, const clowns_member* members, int precision, double eps,
                                         double parm, int iter, double inner_tol, int inner_max, int max_outer,
                                         void* work, size_t work_bytes, void* stream, clowns_solve_info* infos) {
    clowns::TraceRange trace_range_("clowns_pcgpme_batched_dev");
    if (m < 1 || !members || (precision != CLOWNS_PREC_FP64 && precision != CLOWNS_PREC_MIXED)) {
        set_last_error_msg("pcgpme_batched: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    const MemberIn* ins = reinterpret_cast<const MemberIn*>(members);
    if (precision == CLOWNS_PREC_FP64)
        return engine_solve_plain(m, ins, eps, parm, iter, work, work_bytes, (cudaStream_t)stream, infos);
    return engine_solve_mixed(m, ins, eps, parm, inner_tol, inner_max, max_outer, work, work_bytes,
                              (cudaStream_t)stream, infos);
}

extern "C" int clowns_pcgpme_setup_dev(const double* al, int nl, int na, const int* ll, const double* d, int n,
                                       const double* b, double parm, double* al_s, int* ll_s, double* d_s,
                                       double* b_s, int na_out, void* work, size_t work_bytes, void* stream) {
    clowns::TraceRange trace_range_("clowns_pcgpme_setup_dev");
    if (!al_s || !ll_s || !d_s || !b_s || na_out < n) {
        set_last_error_msg("setup: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    // the initial guess is not read by the export; point it at b
    MemberIn in = member(al, nl, na, ll, d, n, b, const_cast<double*>(b));
    return engine_setup_export(in, parm, al_s, ll_s, d_s, b_s, na_out, work, work_bytes, (cudaStream_t)stream);
}

extern "C" int clowns_apply_pm_a_dev(const double* al, int nl, int na, const int* ll, const double* d, int n,
                                     double parm, const double* x, double* y, void* work, size_t work_bytes,
                                     void* stream) {
    clowns::TraceRange trace_range_("clowns_apply_pm_a_dev");
    if (!x || !y) {
        set_last_error_msg("apply: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    MemberIn in = member(al, nl, na, ll, d, n, x, const_cast<double*>(x));
    return engine_apply_pm_a(in, parm, x, y, work, work_bytes, (cudaStream_t)stream);
}

extern "C" int clowns_tuned_shape(int m, const int* n, int precision, int* mode, int* block, int* grid, int* regs,
                                  int* fused) {
    if (m < 1 || !n || !mode || !block || !grid || !regs || !fused) {
        set_last_error_msg("tuned_shape: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    const int mixed = precision == CLOWNS_PREC_MIXED;
    int minb = 0;
    int rc = engine_tuned_shape(engine_row_space(m, n, mixed), mixed, m == 1, mode, block, grid, &minb, fused);
    if (rc) {
        set_last_error_msg("tuned_shape: no solve of this size has run yet");
        return rc;
    }
    *regs = minb > 0 ? (65536 / (minb * *block)) & ~7 : 0;   // register budget of a co-resident kernel
    return CLOWNS_OK;
}

extern "C" long clowns_last_kernel_launches(void) { return engine_last_launches(); }

// FP64 pipe probe: eight independent fused multiply-add chains per thread, no
// memory traffic in the loop, 8 blocks of 256 threads per SM.  The measured
// rate bounds the FP64 solve's arithmetic the way the copy bandwidth bounds its
// streams.  The chains' sum is kept alive by a conditional store through a
// pointer argument (measured: 599 G FMA/s; the same loop ending in a store to
// a file-scope variable ran at 505).
static __device__ double g_fma_sink;
static __global__ void __launch_bounds__(256) k_fma_rate(double* sink, int iters, double a, double b) {
    double v[8];
#pragma unroll
    for (int j = 0; j < 8; j++) v[j] = threadIdx.x * 1e-9 + j;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) v[j] = __fma_rn(v[j], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; j++) s += v[j];
    if (s == 12345.678) *sink = s;      // never true; keeps the chains
}

extern "C" int clowns_fp64_fma_rate(double* fma_per_s, void* stream) {
    if (!fma_per_s) {
        set_last_error_msg("fp64_fma_rate: fma_per_s is null");
        return CLOWNS_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    CLOWNS_CUDA_TRY(cudaGetDevice(&dev));
    CLOWNS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // 5.1 G FMAs per launch (about 9 ms); two warm-up launches, then the best
    // of five timed ones
    const int blocks = 8 * sms, threads = 256, iters = 2048, warm = 2, reps = 5;
    double* sink = nullptr;
    CLOWNS_CUDA_TRY(cudaGetSymbolAddress((void**)&sink, g_fma_sink));
    cudaEvent_t ev[2 * reps];
    int made = 0;
    cudaError_t err = cudaSuccess;
    while (made < 2 * reps && (err = cudaEventCreate(&ev[made])) == cudaSuccess) made++;
    if (err == cudaSuccess) {
        for (int r = 0; r < warm; r++) k_fma_rate<<<blocks, threads, 0, s>>>(sink, iters, 0.999999, 1e-7);
        for (int r = 0; r < reps; r++) {
            cudaEventRecord(ev[2 * r], s);
            k_fma_rate<<<blocks, threads, 0, s>>>(sink, iters, 0.999999, 1e-7);
            cudaEventRecord(ev[2 * r + 1], s);
        }
        err = cudaEventSynchronize(ev[2 * reps - 1]);
    }
    float best = 0.f;
    for (int r = 0; r < reps && err == cudaSuccess; r++) {
        float ms = 0.f;
        err = cudaEventElapsedTime(&ms, ev[2 * r], ev[2 * r + 1]);
        if (r == 0 || ms < best) best = ms;
    }
    for (int k = 0; k < made; k++) cudaEventDestroy(ev[k]);
    CLOWNS_CUDA_TRY(err);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    *fma_per_s = (double)blocks * threads * iters * 8.0 / (best * 1e-3);
    return CLOWNS_OK;
}

extern "C" int clowns_test_arm_wait_timeout(long polls, int absent_block) {
    if (polls < 1 || absent_block < 0) {
        set_last_error_msg("test_arm_wait_timeout: polls >= 1 and absent_block >= 0 required");
        return CLOWNS_ERR_ARG;
    }
    engine_arm_wait_fault(polls, absent_block);
    return CLOWNS_OK;
}
