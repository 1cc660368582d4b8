// pcgpme.cu -- GB300 FP64 restatement of PCGPME (src2LOWNS/pcgpme_para.F90:1-354).
//
// The reference's left-preconditioned BiCGSTAB runs here as a chain of
// bandwidth-bound kernels:
//   * k_setup       : row scaling W = P2/(max(sum|AL|,D)+P1*D), in-place scaling of
//                     AL, D, B and the per-row exchange sort of (AL, LL) by |AL|
//                     (pcgpme_para.F90:77-112), written to a private SoA copy;
//   * k_axsub       : Y = D X + sum_k AL_k X[LL_k]   (AXSUB, 323-352);
//   * k_sweep / k_sweep56 : the five gather sweeps of LDUSUB (263-320);
//   * fused reductions: (r0,q) in the last sweep of q = PM A p, (e,v),(v,v) in the
//                     last sweep of v = PM A e, (r,r),(r0,r) in the x/r update;
//                     the last block of each reduction finalises the scalars on
//                     the device (ALP, AMU, ERR, BETA and the stop tests of
//                     228-240), so no scalar ever travels to the host mid-solve.
// The iteration body is captured once into a CUDA graph whose WHILE conditional
// node repeats it until the device-side stop test clears the condition: one
// graph launch per solve.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "solver_internal.cuh"

namespace clowns {

// ---------------------------------------------------------------------------
// Workspace layout
WsLayout ws_layout(int n, int nl) {
    (void)nl;
    WsLayout L;
    L.NV = (long)align_up((size_t)n + 1, 64);
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return at; };
    L.al = take(sizeof(double) * 6 * L.NV);
    L.ll = take(sizeof(int) * 6 * L.NV);
    L.d = take(sizeof(double) * L.NV);
    for (int v = 0; v < kNumVec; v++) L.vec[v] = take(sizeof(double) * L.NV);
    L.partials = take(sizeof(double) * 4 * kMaxBlocks);
    L.scal = take(sizeof(SolverScalars));
    L.total = o;
    return L;
}

Ws ws_bind(void* work, int n, int nl) {
    WsLayout L = ws_layout(n, nl);
    char* base = (char*)work;
    Ws w;
    w.NV = L.NV;
    w.n = n;
    w.al = (double*)(base + L.al);
    w.ll = (int*)(base + L.ll);
    w.d = (double*)(base + L.d);
    double* v[kNumVec];
    for (int i = 0; i < kNumVec; i++) v[i] = (double*)(base + L.vec[i]);
    w.r = v[0]; w.p = v[1]; w.r0 = v[2]; w.q = v[3]; w.e = v[4]; w.v = v[5]; w.t = v[6]; w.x = v[7];
    w.partials = (double*)(base + L.partials);
    w.S = (SolverScalars*)(base + L.scal);
    return w;
}

int stream_grid(long n) {
    long b = (n + kBlock - 1) / kBlock;
    if (b < 1) b = 1;
    if (b > kMaxBlocks) b = kMaxBlocks;
    return (int)b;
}

// ---------------------------------------------------------------------------
// Kernels

__global__ void k_init_scalars(SolverScalars* S, double eps, int iter) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        SolverScalars z;
        memset(&z, 0, sizeof(z));
        z.EPS = eps;
        z.ITER = iter;
        *S = z;
    }
}

// Scaling + sort (pcgpme_para.F90:77-112).  Every multiply/add is explicitly
// rounded (no fused multiply-add) so W, the scaled coefficients and hence the
// sort decisions are bit-identical to a plain IEEE evaluation of the source.
template <int NL>
__global__ void __launch_bounds__(kBlock) k_setup(const double* __restrict__ al,
                                                 const int* __restrict__ ll,
                                                 const double* __restrict__ d,
                                                 const double* __restrict__ b,
                                                 const double* __restrict__ xin, long na,
                                                 double P1, double P2, Ws w) {
    const long NV = w.NV;
    const int n = w.n;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < NV; i += (long)gridDim.x * blockDim.x) {
        if (i >= n) {
#pragma unroll
            for (int k = 0; k < 6; k++) { w.al[k * NV + i] = 0.0; w.ll[k * NV + i] = n; }
            w.d[i] = 0.0;
            w.r[i] = 0.0; w.p[i] = 0.0; w.r0[i] = 0.0; w.q[i] = 0.0;
            w.e[i] = 0.0; w.v[i] = 0.0; w.t[i] = 0.0; w.x[i] = 0.0;
            continue;
        }
        double a[6];
        int c[6];
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 6; k++) {
            if (k < NL) {
                a[k] = al[k * na + i];
                int cc = ll[k * na + i];
                c[k] = (cc == 0) ? n : cc - 1;
                s = __dadd_rn(s, fabs(a[k]));
            } else {
                a[k] = 0.0;
                c[k] = n;
            }
        }
        const double temp = d[i];
        const double wv = __ddiv_rn(P2, __dadd_rn(fmax(s, temp), __dmul_rn(temp, P1)));
#pragma unroll
        for (int k = 0; k < NL; k++) a[k] = __dmul_rn(a[k], wv);
        const double dd = __dmul_rn(temp, wv);
        const double bb = __dmul_rn(b[i], wv);
#pragma unroll
        for (int K = 0; K < NL - 1; K++) {
#pragma unroll
            for (int KK = K + 1; KK < NL; KK++) {
                if (fabs(a[K]) < fabs(a[KK])) {
                    double ta = a[K]; a[K] = a[KK]; a[KK] = ta;
                    int tc = c[K]; c[K] = c[KK]; c[KK] = tc;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 6; k++) { w.al[k * NV + i] = a[k]; w.ll[k * NV + i] = c[k]; }
        w.d[i] = dd;
        w.r[i] = bb;
        w.p[i] = bb;
        w.x[i] = xin[i];
    }
}

// Y = D X + sum AL_k X[LL_k]  (AXSUB, pcgpme_para.F90:323-352)
__global__ void __launch_bounds__(kBlock) k_axsub(Ws w, const double* __restrict__ in,
                                                 double* __restrict__ out, int check_done) {
    if (check_done && w.S->done) return;
    const long NV = w.NV;
    const int n = w.n;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double s = in[i] * ld_stream(w.d + i);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const double a = ld_stream(w.al + k * NV + i);
            const int c = ld_stream(w.ll + k * NV + i);
            s += a * in[c];
        }
        out[i] = s;
    }
}

// One single-neighbour sweep of LDUSUB: out = in - AL_k in[LL_k]
__global__ void __launch_bounds__(kBlock) k_sweep(Ws w, int k, const double* __restrict__ in,
                                                 double* __restrict__ out, int check_done) {
    if (check_done && w.S->done) return;
    const long NV = w.NV;
    const int n = w.n;
    const double* __restrict__ a = w.al + k * NV;
    const int* __restrict__ c = w.ll + k * NV;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        out[i] = in[i] - ld_stream(a + i) * in[ld_stream(c + i)];
    }
}

// Last sweep (J=5,6 of LDUSUB) with an optional fused reduction:
//   MODE 0: plain;  MODE 1: RQ = (r0, out);  MODE 2: AMU = (e, out), SS = (out, out)
template <int MODE>
__global__ void __launch_bounds__(kBlock) k_sweep56(Ws w, const double* __restrict__ in,
                                                   double* __restrict__ out, int check_done) {
    if (check_done && w.S->done) return;
    __shared__ double red[64];
    __shared__ bool am_last;
    const long NV = w.NV;
    const int n = w.n;
    const double* __restrict__ a5 = w.al + 4 * NV;
    const double* __restrict__ a6 = w.al + 5 * NV;
    const int* __restrict__ c5 = w.ll + 4 * NV;
    const int* __restrict__ c6 = w.ll + 5 * NV;
    double acc[2] = {0.0, 0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double y = in[i] - ld_stream(a5 + i) * in[ld_stream(c5 + i)] - ld_stream(a6 + i) * in[ld_stream(c6 + i)];
        out[i] = y;
        if (MODE == 1) acc[0] += w.r0[i] * y;
        if (MODE == 2) { acc[0] += w.e[i] * y; acc[1] += y * y; }
    }
    if (MODE == 0) return;
    block_sum<2>(acc, red);
    if (threadIdx.x == 0) {
        w.partials[blockIdx.x * 2 + 0] = acc[0];
        w.partials[blockIdx.x * 2 + 1] = acc[1];
        __threadfence();
        unsigned t = atomicAdd(&w.S->ticket[MODE], 1u);
        am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!am_last || threadIdx.x >= 32) return;
    __threadfence();
    double tot[2];
    warp_sum_partials<2>(w.partials, gridDim.x, tot);
    if (threadIdx.x == 0) {
        SolverScalars* S = w.S;
        S->ticket[MODE] = 0;
        if (MODE == 1) {
            const double RQ = tot[0];
            S->RQ = RQ;
            S->ALP = S->C1 / RQ;                                     // 167
            if (!isfinite(RQ) || !isfinite(S->ALP)) {
                S->done = 1; S->reason = CLOWNS_STOP_NONFINITE; S->ier = CLOWNS_IER_NONFINITE;
                S->K += 1;
            }
        } else {
            double AMU = tot[0];
            const double SS = tot[1];
            S->SS = SS;
            AMU = AMU / SS;                                          // 197
            S->AMU = AMU;
            if (!isfinite(SS) || !isfinite(AMU)) {
                S->done = 1; S->reason = CLOWNS_STOP_NONFINITE; S->ier = CLOWNS_IER_NONFINITE;
                S->K += 1;
            }
        }
    }
}

// E = R - ALP Q  (pcgpme_para.F90:171-175)
__global__ void __launch_bounds__(kBlock) k_eupdate(Ws w) {
    if (w.S->done) return;
    const double ALP = w.S->ALP;
    const int n = w.n;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        w.e[i] = w.r[i] - ALP * w.q[i];
}

// X += ALP P + AMU E ; R = E - AMU V ; RN = (R,R) ; C1 = (R0,R)  (199-213),
// then the stop tests and BETA (215-241) in the last block.
__global__ void __launch_bounds__(kBlock) k_xrupdate(Ws w) {
    if (w.S->done) return;
    __shared__ double red[64];
    __shared__ bool am_last;
    const double ALP = w.S->ALP, AMU = w.S->AMU;
    const int n = w.n;
    double acc[2] = {0.0, 0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double temp = w.e[i];
        w.x[i] = w.x[i] + ALP * w.p[i] + AMU * temp;
        temp = temp - AMU * w.v[i];
        w.r[i] = temp;
        acc[0] += temp * temp;
        acc[1] += temp * w.r0[i];
    }
    block_sum<2>(acc, red);
    if (threadIdx.x == 0) {
        w.partials[blockIdx.x * 2 + 0] = acc[0];
        w.partials[blockIdx.x * 2 + 1] = acc[1];
        __threadfence();
        unsigned t = atomicAdd(&w.S->ticket[3], 1u);
        am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!am_last || threadIdx.x >= 32) return;
    __threadfence();
    double tot[2];
    warp_sum_partials<2>(w.partials, gridDim.x, tot);
    if (threadIdx.x == 0) {
        SolverScalars* S = w.S;
        S->ticket[3] = 0;
        const double RN = tot[0], C1 = tot[1];
        S->RN = RN;
        S->C1 = C1;
        S->K += 1;
        const int K = S->K;
        const double ERR = sqrt(RN / S->BN);                         // 215
        S->ERR = ERR;
        int stop = -1;
        if (!isfinite(RN) || !isfinite(C1)) {
            stop = CLOWNS_STOP_NONFINITE;
            S->ier = CLOWNS_IER_NONFINITE;
        } else if (K >= 10 && fabs(ERR - S->ERRP) <= ERR * 1.0e-6) {  // 228
            stop = CLOWNS_STOP_STAGNATION;
        } else if (ERR <= S->EPS) {                                  // 232
            stop = CLOWNS_STOP_TOL;
        } else {
            S->ERRP = ERR;                                           // 233
            if (S->AMU == 0.0) {
                stop = CLOWNS_STOP_AMU_ZERO;                         // 234
            } else if (C1 == 0.0) {
                stop = CLOWNS_STOP_C1_ZERO;                          // 240
            } else {
                S->BETA = C1 / S->AMU / S->RQ;                       // 241
                if (K >= S->ITER) {                                  // loop exhausted, 250-251
                    stop = CLOWNS_STOP_MAXITER;
                    S->ier = CLOWNS_IER_MAXITER;
                    S->K = S->ITER + 1;
                }
            }
        }
        if (stop >= 0) {
            S->done = 1;
            S->reason = stop;
        }
    }
}

// Last node of the loop body: the only writer of the WHILE condition.  It stops
// the loop once a stop test fired, and -- as a backstop that no correct run
// reaches -- after ITER+2 body executions.
__global__ void k_guard(SolverScalars* S, cudaGraphConditionalHandle h) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    S->body_count += 1;
    if (!S->done && S->body_count > S->ITER + 1) {
        S->done = 1;
        S->reason = CLOWNS_STOP_MAXITER;
        S->ier = CLOWNS_IER_MAXITER;
    }
    cudaGraphSetConditional(h, S->done ? 0u : 1u);
}

// P = R + BETA (P - AMU Q)  (pcgpme_para.F90:242-246)
__global__ void __launch_bounds__(kBlock) k_pupdate(Ws w) {
    if (w.S->done) return;
    const double BETA = w.S->BETA, AMU = w.S->AMU;
    const int n = w.n;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        w.p[i] = w.r[i] + BETA * (w.p[i] - AMU * w.q[i]);
}

// BN = (b^,b^); R = b^ - PM A x0; C1 = (R,R); P = R0 = R  (pcgpme_para.F90:129-145)
__global__ void __launch_bounds__(kBlock) k_initres(Ws w) {
    __shared__ double red[64];
    __shared__ bool am_last;
    const int n = w.n;
    double acc[2] = {0.0, 0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double temp = w.p[i];
        acc[0] += temp * temp;
        temp = temp - w.q[i];
        w.r[i] = temp;
        acc[1] += temp * temp;
        w.p[i] = temp;
        w.r0[i] = temp;
    }
    block_sum<2>(acc, red);
    if (threadIdx.x == 0) {
        w.partials[blockIdx.x * 2 + 0] = acc[0];
        w.partials[blockIdx.x * 2 + 1] = acc[1];
        __threadfence();
        unsigned t = atomicAdd(&w.S->ticket[0], 1u);
        am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!am_last || threadIdx.x >= 32) return;
    __threadfence();
    double tot[2];
    warp_sum_partials<2>(w.partials, gridDim.x, tot);
    if (threadIdx.x == 0) {
        w.S->ticket[0] = 0;
        w.S->BN = tot[0];
        w.S->C1 = tot[1];
    }
}

__global__ void k_fill_int(int* p, long count, int value) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (long)gridDim.x * blockDim.x)
        p[i] = value;
}

__global__ void k_copy_out(const double* __restrict__ src, double* __restrict__ dst, int n) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

__global__ void k_export_setup(Ws w, double* al_s, int* ll_s, double* d_s, double* b_s, int nl,
                               long na_out) {
    const int n = w.n;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        for (int k = 0; k < nl; k++) {
            al_s[k * na_out + i] = w.al[k * w.NV + i];
            ll_s[k * na_out + i] = w.ll[k * w.NV + i];
        }
        d_s[i] = w.d[i];
        b_s[i] = w.r[i];
    }
}

// ---------------------------------------------------------------------------
// Host orchestration

// PM A in -> out, using tmp (apply: AXSUB then the five LDUSUB sweeps)
static void launch_apply(const Ws& w, const double* in, double* out, double* tmp, int mode,
                         int check_done, cudaStream_t s) {
    const int g = stream_grid(w.n);
    k_axsub<<<g, kBlock, 0, s>>>(w, in, tmp, check_done);
    k_sweep<<<g, kBlock, 0, s>>>(w, 0, tmp, out, check_done);
    k_sweep<<<g, kBlock, 0, s>>>(w, 1, out, tmp, check_done);
    k_sweep<<<g, kBlock, 0, s>>>(w, 2, tmp, out, check_done);
    k_sweep<<<g, kBlock, 0, s>>>(w, 3, out, tmp, check_done);
    if (mode == 0) k_sweep56<0><<<g, kBlock, 0, s>>>(w, tmp, out, check_done);
    if (mode == 1) k_sweep56<1><<<g, kBlock, 0, s>>>(w, tmp, out, check_done);
    if (mode == 2) k_sweep56<2><<<g, kBlock, 0, s>>>(w, tmp, out, check_done);
}

// LDUSUB alone on vec (in place), scratch a and b
static void launch_ldusub(const Ws& w, double* vec, double* a, double* b, cudaStream_t s) {
    const int g = stream_grid(w.n);
    k_sweep<<<g, kBlock, 0, s>>>(w, 0, vec, a, 0);
    k_sweep<<<g, kBlock, 0, s>>>(w, 1, a, b, 0);
    k_sweep<<<g, kBlock, 0, s>>>(w, 2, b, a, 0);
    k_sweep<<<g, kBlock, 0, s>>>(w, 3, a, b, 0);
    k_sweep56<0><<<g, kBlock, 0, s>>>(w, b, vec, 0);
}

static void launch_iteration(const Ws& w, cudaStream_t s) {
    const int g = stream_grid(w.n);
    launch_apply(w, w.p, w.q, w.t, 1, 1, s);           // q = PM A p ; RQ ; ALP
    k_eupdate<<<g, kBlock, 0, s>>>(w);                 // e = r - ALP q
    launch_apply(w, w.e, w.v, w.t, 2, 1, s);           // v = PM A e ; AMU
    k_xrupdate<<<g, kBlock, 0, s>>>(w);                // x, r, RN, C1, stop tests
    k_pupdate<<<g, kBlock, 0, s>>>(w);                 // p
}

void launch_setup(const Ws& w, const double* al, int nl, long na, const int* ll, const double* d,
                  const double* b, const double* x, double P1, double P2, cudaStream_t s) {
    const int g = stream_grid(w.NV);
    if (nl == 6)
        k_setup<6><<<g, kBlock, 0, s>>>(al, ll, d, b, x, na, P1, P2, w);
    else
        k_setup<4><<<g, kBlock, 0, s>>>(al, ll, d, b, x, na, P1, P2, w);
}

void launch_init(const Ws& w, cudaStream_t s) {
    const int g = stream_grid(w.n);
    launch_ldusub(w, w.p, w.t, w.q, s);                     // b^ = PM W b
    launch_apply(w, w.x, w.q, w.t, 0, 0, s);                // q = PM A x0
    k_initres<<<g, kBlock, 0, s>>>(w);
}

// Graph cache: one instantiated graph per (workspace, inputs, sizes)
struct GraphKey {
    const void *al, *ll, *d, *b, *x, *work;
    int nl, na, n;
    double P1;
    bool operator==(const GraphKey& o) const {
        return al == o.al && ll == o.ll && d == o.d && b == o.b && x == o.x && work == o.work &&
               nl == o.nl && na == o.na && n == o.n && P1 == o.P1;
    }
};
struct GraphEntry {
    GraphKey key;
    cudaGraphExec_t exec;
};
static std::mutex g_graph_mu;
static std::vector<GraphEntry> g_graphs;
static cudaStream_t g_capture_stream = nullptr;
static cudaStream_t g_body_stream = nullptr;

static int build_solve_graph(const GraphKey& key, const Ws& w, double P1, double P2,
                             double eps, int iter, cudaGraphExec_t* out) {
    (void)eps; (void)iter;
    if (!g_capture_stream) CLOWNS_CUDA_TRY(cudaStreamCreateWithFlags(&g_capture_stream, cudaStreamNonBlocking));
    if (!g_body_stream) CLOWNS_CUDA_TRY(cudaStreamCreateWithFlags(&g_body_stream, cudaStreamNonBlocking));
    cudaStream_t s = g_capture_stream;
    cudaGraph_t graph = nullptr;
    CLOWNS_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    // Scalars are (re)initialised by a parameter node updated per launch.
    launch_setup(w, (const double*)key.al, key.nl, key.na, (const int*)key.ll, (const double*)key.d,
                 (const double*)key.b, (const double*)key.x, P1, P2, s);
    launch_init(w, s);
    cudaStreamCaptureStatus st;
    cudaGraph_t cap_graph;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    CLOWNS_CUDA_TRY(cudaStreamGetCaptureInfo(s, &st, nullptr, &cap_graph, &deps, nullptr, &ndeps));
    cudaGraphConditionalHandle handle;
    CLOWNS_CUDA_TRY(cudaGraphConditionalHandleCreate(&handle, cap_graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode;
    CLOWNS_CUDA_TRY(cudaGraphAddNode(&cnode, cap_graph, deps, nullptr, ndeps, &cp));
    CLOWNS_CUDA_TRY(cudaStreamUpdateCaptureDependencies(s, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    // Populate the loop body on a second capture into the body graph.
    cudaStream_t s2 = g_body_stream;
    CLOWNS_CUDA_TRY(cudaStreamBeginCaptureToGraph(s2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    launch_iteration(w, s2);
    k_guard<<<1, 32, 0, s2>>>(w.S, handle);
    cudaGraph_t body_out;
    CLOWNS_CUDA_TRY(cudaStreamEndCapture(s2, &body_out));
    k_copy_out<<<stream_grid(w.n), kBlock, 0, s>>>(w.x, (double*)key.x, w.n);
    CLOWNS_CUDA_TRY(cudaStreamEndCapture(s, &graph));
    cudaGraphExec_t exec;
    CLOWNS_CUDA_TRY(cudaGraphInstantiate(&exec, graph, 0));
    cudaGraphDestroy(graph);
    *out = exec;
    return CLOWNS_OK;
}

static int get_solve_graph(const GraphKey& key, const Ws& w, double P1, double P2, double eps,
                           int iter, cudaGraphExec_t* out) {
    std::lock_guard<std::mutex> lk(g_graph_mu);
    for (auto& e : g_graphs)
        if (e.key == key) { *out = e.exec; return CLOWNS_OK; }
    cudaGraphExec_t ex;
    int rc = build_solve_graph(key, w, P1, P2, eps, iter, &ex);
    if (rc) return rc;
    if (g_graphs.size() >= 16) {
        cudaGraphExecDestroy(g_graphs.front().exec);
        g_graphs.erase(g_graphs.begin());
    }
    g_graphs.push_back({key, ex});
    *out = ex;
    return CLOWNS_OK;
}

void release_graphs_for(const void* work) {
    std::lock_guard<std::mutex> lk(g_graph_mu);
    for (size_t i = 0; i < g_graphs.size();) {
        if (g_graphs[i].key.work == work) {
            cudaGraphExecDestroy(g_graphs[i].exec);
            g_graphs.erase(g_graphs.begin() + i);
        } else {
            i++;
        }
    }
}

void release_all_graphs() {
    std::lock_guard<std::mutex> lk(g_graph_mu);
    for (auto& e : g_graphs) cudaGraphExecDestroy(e.exec);
    g_graphs.clear();
}

// Resolve PCGPME's defaults (pcgpme_para.F90:51-58)
void resolve_params(int n, double eps, double parm, int iter, double* eps_o, int* iter_o,
                    double* P1, double* P2) {
    if (eps <= kTiny) eps = kSmall;
    if (iter <= 0) iter = (int)(10 * (std::sqrt((double)n) + 1));
    double p1 = parm;
    if (parm < 1.0) p1 = 4.0;
    *eps_o = eps;
    *iter_o = iter;
    *P1 = p1;
    *P2 = p1 + 1.0;
}

int read_info(const Ws& w, cudaStream_t s, clowns_solve_info* info) {
    SolverScalars h;
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(&h, w.S, sizeof(h), cudaMemcpyDeviceToHost, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    if (info) {
        info->eps = h.ERR;
        info->bn = h.BN;
        info->iter = h.K;
        info->ier = h.ier;
        info->reason = h.reason;
        info->outer = 0;
    }
    return CLOWNS_OK;
}

int pcgpme_dev_impl(const double* al, int nl, int na, const int* ll, const double* d, int n,
                    const double* b, double* x, double eps, double parm, int iter, void* work,
                    size_t work_bytes, cudaStream_t s, clowns_solve_info* info) {
    if (!al || !ll || !d || !b || !x || !work || n < 1 || na < n || (nl != 6 && nl != 4)) {
        set_last_error_msg("pcgpme: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    if (work_bytes < ws_layout(n, nl).total) {
        set_last_error_msg("pcgpme: workspace too small");
        return CLOWNS_ERR_WORKSPACE;
    }
    Ws w = ws_bind(work, n, nl);
    double eps_r, P1, P2;
    int iter_r;
    resolve_params(n, eps, parm, iter, &eps_r, &iter_r, &P1, &P2);
    GraphKey key{al, ll, d, b, x, work, nl, na, n, P1};
    cudaGraphExec_t exec;
    int rc = get_solve_graph(key, w, P1, P2, eps_r, iter_r, &exec);
    if (rc) return rc;
    k_init_scalars<<<1, 1, 0, s>>>(w.S, eps_r, iter_r);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    CLOWNS_CUDA_TRY(cudaGraphLaunch(exec, s));
    return read_info(w, s, info);
}

}  // namespace clowns

using namespace clowns;

extern "C" size_t clowns_pcgpme_workspace_bytes(int n, int nl) {
    if (n < 1) return 0;
    return ws_layout(n, nl).total;
}

extern "C" int clowns_pcgpme_dev(const double* al, int nl, int na, const int* ll, const double* d,
                                 int n, const double* b, double* x, double eps, double parm, int iter,
                                 void* work, size_t work_bytes, void* stream,
                                 clowns_solve_info* info) {
    return pcgpme_dev_impl(al, nl, na, ll, d, n, b, x, eps, parm, iter, work, work_bytes,
                           (cudaStream_t)stream, info);
}

extern "C" int clowns_pcgpme_setup_dev(const double* al, int nl, int na, const int* ll,
                                       const double* d, int n, const double* b, double parm,
                                       double* al_s, int* ll_s, double* d_s, double* b_s,
                                       int na_out, void* work, size_t work_bytes, void* stream) {
    if (!al || !ll || !d || !b || !work || n < 1 || na < n || na_out < n || (nl != 6 && nl != 4)) {
        set_last_error_msg("setup: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    if (work_bytes < ws_layout(n, nl).total) {
        set_last_error_msg("setup: workspace too small");
        return CLOWNS_ERR_WORKSPACE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    Ws w = ws_bind(work, n, nl);
    double e, P1, P2;
    int it;
    resolve_params(n, 0.0, parm, 0, &e, &it, &P1, &P2);
    // x0 = b (any finite vector; the hook exports only matrix data)
    launch_setup(w, al, nl, na, ll, d, b, b, P1, P2, s);
    k_export_setup<<<stream_grid(n), kBlock, 0, s>>>(w, al_s, ll_s, d_s, b_s, nl, na_out);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    return CLOWNS_OK;
}

extern "C" int clowns_apply_pm_a_dev(const double* al_s, const int* ll_s, const double* d_s, int nl,
                                     int na_s, int n, const double* x, double* y, void* work,
                                     size_t work_bytes, void* stream) {
    if (!al_s || !ll_s || !d_s || !x || !y || !work || n < 1 || na_s < n || (nl != 6 && nl != 4)) {
        set_last_error_msg("apply: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    if (work_bytes < ws_layout(n, nl).total) {
        set_last_error_msg("apply: workspace too small");
        return CLOWNS_ERR_WORKSPACE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    Ws w = ws_bind(work, n, nl);
    // Copy the exported matrix into the workspace layout.
    for (int k = 0; k < 6; k++) {
        if (k < nl) {
            CLOWNS_CUDA_TRY(cudaMemcpyAsync(w.al + k * w.NV, al_s + (size_t)k * na_s, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
            CLOWNS_CUDA_TRY(cudaMemcpyAsync(w.ll + k * w.NV, ll_s + (size_t)k * na_s, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
        } else {
            CLOWNS_CUDA_TRY(cudaMemsetAsync(w.al + k * w.NV, 0, sizeof(double) * n, s));
            k_fill_int<<<stream_grid(n), kBlock, 0, s>>>(w.ll + k * w.NV, n, n);
        }
    }
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(w.d, d_s, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemsetAsync(w.d + n, 0, sizeof(double) * (w.NV - n), s));
    CLOWNS_CUDA_TRY(cudaMemsetAsync(w.x, 0, sizeof(double) * w.NV, s));
    CLOWNS_CUDA_TRY(cudaMemsetAsync(w.t, 0, sizeof(double) * w.NV, s));
    CLOWNS_CUDA_TRY(cudaMemsetAsync(w.q, 0, sizeof(double) * w.NV, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(w.x, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    launch_apply(w, w.x, w.q, w.t, 0, 0, s);
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(y, w.q, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    CLOWNS_CUDA_TRY(cudaGetLastError());
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    return CLOWNS_OK;
}
