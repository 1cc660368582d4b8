// solver_internal.cuh -- workspace layout and scalar block of the FP64 solve.
#pragma once

#include "common.cuh"

namespace clowns {

constexpr int kBlock = 256;
constexpr int kMaxBlocks = kNumSMs * 8;   // grid-stride streaming kernels
constexpr int kNumVec = 8;

// Device-side scalars of one PCGPME solve (names follow pcgpme_para.F90:47).
struct SolverScalars {
    double BN, C1, ALP, AMU, RN, RQ, BETA, ERR, ERRP, SS, EPS, pad0;
    int K;            // iteration counter (the reference's loop variable)
    int ITER;         // iteration cap
    int done;         // 1 once a stop test fired
    int reason;       // CLOWNS_STOP_*
    int ier;          // IER
    int body_count;   // loop-body executions (backstop against a runaway loop)
    unsigned ticket[6];
};

struct WsLayout {
    long NV;
    size_t al, ll, d, vec[kNumVec], partials, scal, total;
};

// Views into the workspace.  Vectors have NV >= n+1 entries; entry n is a zero
// row that every empty stencil slot points at.
struct Ws {
    long NV;
    int n;
    double* al;   // 6 columns, scaled and sorted (SoA, stride NV)
    int* ll;      // 6 columns, 0-based
    double* d;
    double *r, *p, *r0, *q, *e, *v, *t, *x;
    double* partials;
    SolverScalars* S;
};

WsLayout ws_layout(int n, int nl);
Ws ws_bind(void* work, int n, int nl);
int stream_grid(long n);
void resolve_params(int n, double eps, double parm, int iter, double* eps_o, int* iter_o,
                    double* P1, double* P2);
int pcgpme_dev_impl(const double* al, int nl, int na, const int* ll, const double* d, int n,
                    const double* b, double* x, double eps, double parm, int iter, void* work,
                    size_t work_bytes, cudaStream_t s, clowns_solve_info* info);
void release_graphs_for(const void* work);
void release_all_graphs();

}  // namespace clowns
