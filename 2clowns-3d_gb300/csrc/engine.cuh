// engine.cuh -- batched left-preconditioned BiCGSTAB engine (PCGPME's method,
// src2LOWNS/pcgpme_para.F90:1-354) over a concatenation of independent systems.
//
// One solve of the reference is a batch of one member.  Members occupy disjoint,
// tile-aligned row ranges of one row space; every kernel walks tiles of kTile
// rows, looks up the tile's member, skips members whose solve has stopped, and
// reduces dot products per member: the last tile of a member to finish sums
// that member's tile partials in tile order (deterministic) and finalises its
// scalars on the device.  Coefficients and Krylov vectors are stored as T
// (double for the plain path, float for the inner solve of the mixed path);
// all dot products and scalars are double.
#pragma once

#include "common.cuh"

namespace clowns {

constexpr int kTile = 2048;          // rows per tile (multiple of kEngBlock)
constexpr int kEngBlock = 256;
constexpr int kEngMaxGrid = kNumSMs * 8;

// Per-member scalars; names follow pcgpme_para.F90:47.
struct MemberScalars {
    double BN, C1, ALP, AMU, RN, RQ, BETA, ERR, ERRP, SS, EPS, SIGMA;
    double BN64;    // ||PM W b||^2 in FP64 (mixed path)
    double ERR64;   // outer (FP64) ERR of the mixed path
    double EPS64;   // outer tolerance
    double pad64;
    int odone;      // mixed path: outer tolerance reached
    int outer;      // refinement sweeps performed
    int OITER;      // refinement sweep cap
    int pad_i;
    int K;          // iteration counter of the current (inner) solve
    int ITER;       // iteration cap
    int done;       // stop test fired (or member excluded)
    int reason;     // CLOWNS_STOP_*
    int ier;
    int mode;       // 0: reference stop tests; 1: inner solve of the refinement loop
    int bad_index;  // an input column index was outside 0..n
    int total_iter; // iterations summed over refinement sweeps
};

// Original (unscaled, unsorted) FP64 system of one member, as the caller holds it.
struct MemberIn {
    const double* al;   // (na, nl) column-major
    const int* ll;      // (na, nl), 1-based, 0 = none
    const double* d;    // (n)
    const double* b;    // (n)
    double* x;          // (n) in: initial guess, out: solution
    int na, n, nl, pad;
};

template <typename T>
struct Eng {
    long NV;                  // rows of the concatenated space (multiple of kTile)
    int M, nblk;              // members, kTile-blocks of the row space
    T* al;                    // 6 columns, stride NV, scaled + sorted
    int* ll;                  // 6 columns, global 0-based indices
    T* d;
    T *r, *p, *r0, *q, *e, *v, *t, *xi;   // Krylov vectors (xi: inner solution)
    double* W;                // row scaling (mixed path), NV
    double* x64;              // FP64 solution (mixed path)
    double* r64;              // FP64 work vectors (mixed path)
    double* s64;
    double* t64;
    const int* blk_member;    // member of each block (-1: none)
    const int* blk_rows;      // real rows in each block (0: pad only)
    const int* mem_off;       // first row of each member
    const int* mem_n;         // rows of each member
    const int* mem_nblk;      // blocks with real rows per member
    const int* mem_blk0;      // first block of each member
    const MemberIn* in;       // per-member inputs (device copy of the table)
    MemberScalars* S;
    double* partials;         // 2 per block
    unsigned* ticket;         // one per member
    int* ctrl;                // [0] loop-body count, [1] max ITER over members
};

// ---------------------------------------------------------------------------
// Tile walk helpers

template <typename T>
__device__ __forceinline__ bool tile_active(const Eng<T>& E, int blk, int& m, long& row0, int& rows) {
    m = E.blk_member[blk];
    if (m < 0) return false;
    rows = E.blk_rows[blk];
    if (rows == 0) return false;
    if (E.S[m].done) return false;
    row0 = (long)blk * kTile;
    return true;
}

// Reduce (v0, v1) over the block, record the block's partial and, if this is the
// last block of member m, return true in the whole block with tot[] holding the
// member totals (summed over the member's blocks in block order).
template <typename T>
__device__ __forceinline__ bool member_reduce(const Eng<T>& E, int blk, int m, double v0, double v1,
                                              double* red, double (&tot)[2]) {
    __shared__ int s_last;
    double acc[2] = {v0, v1};
    block_sum<2>(acc, red);
    if (threadIdx.x == 0) {
        E.partials[2L * blk + 0] = acc[0];
        E.partials[2L * blk + 1] = acc[1];
        __threadfence();
        unsigned t = atomicAdd(&E.ticket[m], 1u);
        s_last = (t == (unsigned)E.mem_nblk[m] - 1u);
    }
    __syncthreads();
    const bool last = s_last;
    __syncthreads();
    if (!last) return false;
    __threadfence();
    if (threadIdx.x < 32) {
        const int b0 = E.mem_blk0[m];
        const int nb = E.mem_nblk[m];
        double s0 = 0.0, s1 = 0.0;
        // blocks of a member are contiguous; pad-only blocks contribute zero records
        for (int b = threadIdx.x; b < nb; b += 32) {
            s0 += __ldcg(E.partials + 2L * (b0 + b) + 0);
            s1 += __ldcg(E.partials + 2L * (b0 + b) + 1);
        }
        tot[0] = warp_sum(s0);
        tot[1] = warp_sum(s1);
    }
    return true;
}

__device__ __forceinline__ void stop_member(MemberScalars* S, int reason, int ier) {
    S->done = 1;
    S->reason = reason;
    if (ier) S->ier = ier;
}

// ---------------------------------------------------------------------------
// Setup: scaling W = P2/(max(sum|AL|,D)+P1 D), scaled copies and the per-row
// exchange sort (pcgpme_para.F90:77-112).  Explicitly rounded arithmetic so the
// sort decisions equal an IEEE evaluation of the source.  For rows beyond a
// member's n (its pad rows) all vectors are zeroed and slots point at the
// member's zero row.  init_x: copy the member's initial guess into xi / x64.
template <typename T, int NL>
__global__ void __launch_bounds__(kEngBlock) k_eng_setup(Eng<T> E, double P1, double P2, int mixed) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < E.NV; i += (long)gridDim.x * blockDim.x) {
        const int blk = (int)(i / kTile);
        const int m = E.blk_member[blk];
        const long NV = E.NV;
        if (m < 0) continue;
        const long off = E.mem_off[m];
        const int n = E.mem_n[m];
        const long li = i - off;
        const MemberIn in = E.in[m];
        const long pad = off + n;
        if (li >= n) {
#pragma unroll
            for (int k = 0; k < 6; k++) { E.al[k * NV + i] = T(0); E.ll[k * NV + i] = (int)pad; }
            E.d[i] = T(0);
            E.r[i] = T(0); E.p[i] = T(0); E.r0[i] = T(0); E.q[i] = T(0);
            E.e[i] = T(0); E.v[i] = T(0); E.t[i] = T(0); E.xi[i] = T(0);
            if (mixed) { E.W[i] = 0.0; E.x64[i] = 0.0; E.r64[i] = 0.0; E.s64[i] = 0.0; E.t64[i] = 0.0; }
            continue;
        }
        double a[6];
        int c[6];
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 6; k++) {
            if (k < NL) {
                a[k] = in.al[k * (long)in.na + li];
                int cc = in.ll[k * (long)in.na + li];
                if (cc < 0 || cc > n) {
                    atomicOr(&E.S[m].bad_index, 1);
                    cc = 0;
                }
                c[k] = (cc == 0) ? (int)pad : (int)(off + cc - 1);
                s = __dadd_rn(s, fabs(a[k]));
            } else {
                a[k] = 0.0;
                c[k] = (int)pad;
            }
        }
        const double temp = in.d[li];
        const double wv = __ddiv_rn(P2, __dadd_rn(fmax(s, temp), __dmul_rn(temp, P1)));
#pragma unroll
        for (int k = 0; k < NL; k++) a[k] = __dmul_rn(a[k], wv);
        const double dd = __dmul_rn(temp, wv);
        const double bb = __dmul_rn(in.b[li], wv);
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
        for (int k = 0; k < 6; k++) { E.al[k * NV + i] = T(a[k]); E.ll[k * NV + i] = c[k]; }
        E.d[i] = T(dd);
        const double x0 = in.x[li];
        if (mixed) {
            E.W[i] = wv;
            E.x64[i] = x0;
            E.r64[i] = bb;       // W b, the refinement right-hand side
            E.xi[i] = T(0);
        } else {
            E.r[i] = T(bb);
            E.p[i] = T(bb);
            E.xi[i] = T(x0);
        }
    }
}

static __global__ void k_eng_init_scalars(MemberScalars* S, int M, double eps, int iter, int mode, int* ctrl) {
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
        MemberScalars z;
        memset(&z, 0, sizeof(z));
        z.EPS = eps;
        z.ITER = iter;
        z.mode = mode;
        S[m] = z;
    }
    if (threadIdx.x == 0) { ctrl[0] = 0; ctrl[1] = iter; }
}

// ---------------------------------------------------------------------------
// Operator pieces.  MEMBER-AWARE: every kernel skips tiles of stopped members.

// out = D in + sum_k AL_k in[LL_k]   (AXSUB, pcgpme_para.F90:323-352)
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_axsub(Eng<T> E, const T* __restrict__ in,
                                                        T* __restrict__ out) {
    const long NV = E.NV;
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_active(E, blk, m, row0, rows)) continue;
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const long i = row0 + r;
            T s = in[i] * ld_stream(E.d + i);
#pragma unroll
            for (int k = 0; k < 6; k++) {
                const T a = ld_stream(E.al + k * NV + i);
                const int c = ld_stream(E.ll + k * NV + i);
                s += a * in[c];
            }
            out[i] = s;
        }
    }
}

// One single-neighbour sweep of LDUSUB: out = in - AL_k in[LL_k]  (263-304)
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_sweep(Eng<T> E, int k, const T* __restrict__ in,
                                                        T* __restrict__ out) {
    const long NV = E.NV;
    const T* __restrict__ a = E.al + k * NV;
    const int* __restrict__ c = E.ll + k * NV;
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_active(E, blk, m, row0, rows)) continue;
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const long i = row0 + r;
            out[i] = in[i] - ld_stream(a + i) * in[ld_stream(c + i)];
        }
    }
}

// Last sweep (J=5,6, 306-318) with an optional fused per-member reduction:
//   MODE 0 none; 1: RQ = (r0,out) -> ALP = C1/RQ; 2: AMU = (e,out)/(out,out)
template <typename T, int MODE>
__global__ void __launch_bounds__(kEngBlock) k_eng_sweep56(Eng<T> E, const T* __restrict__ in,
                                                          T* __restrict__ out) {
    __shared__ double red[64];
    const long NV = E.NV;
    const T* __restrict__ a5 = E.al + 4 * NV;
    const T* __restrict__ a6 = E.al + 5 * NV;
    const int* __restrict__ c5 = E.ll + 4 * NV;
    const int* __restrict__ c6 = E.ll + 5 * NV;
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_active(E, blk, m, row0, rows)) continue;
        T acc0 = T(0), acc1 = T(0);
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const long i = row0 + r;
            const T y = in[i] - ld_stream(a5 + i) * in[ld_stream(c5 + i)] - ld_stream(a6 + i) * in[ld_stream(c6 + i)];
            out[i] = y;
            if (MODE == 1) acc0 += E.r0[i] * y;
            if (MODE == 2) { acc0 += E.e[i] * y; acc1 += y * y; }
        }
        if (MODE == 0) continue;
        double tot[2];
        if (!member_reduce(E, blk, m, (double)acc0, (double)acc1, red, tot)) continue;
        if (threadIdx.x == 0) {
            MemberScalars* S = E.S + m;
            E.ticket[m] = 0;
            if (MODE == 1) {
                S->RQ = tot[0];
                S->ALP = S->C1 / tot[0];                               // 167
                if (!isfinite(tot[0]) || !isfinite(S->ALP)) {
                    S->K += 1;
                    stop_member(S, CLOWNS_STOP_NONFINITE, S->mode == 0 ? CLOWNS_IER_NONFINITE : 0);
                }
            } else {
                S->SS = tot[1];
                S->AMU = tot[0] / tot[1];                              // 197
                if (!isfinite(tot[1]) || !isfinite(S->AMU)) {
                    S->K += 1;
                    stop_member(S, CLOWNS_STOP_NONFINITE, S->mode == 0 ? CLOWNS_IER_NONFINITE : 0);
                }
            }
        }
        __syncthreads();
    }
}

// E = R - ALP Q  (171-175)
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_eupdate(Eng<T> E) {
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_active(E, blk, m, row0, rows)) continue;
        const T ALP = T(E.S[m].ALP);
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const long i = row0 + r;
            E.e[i] = E.r[i] - ALP * E.q[i];
        }
    }
}

// X += ALP P + AMU E ; R = E - AMU V ; RN = (R,R) ; C1 = (R0,R)  (199-213),
// then ERR and the stop tests (215-241).
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_xrupdate(Eng<T> E) {
    __shared__ double red[64];
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_active(E, blk, m, row0, rows)) continue;
        const T ALP = T(E.S[m].ALP), AMU = T(E.S[m].AMU);
        T acc0 = T(0), acc1 = T(0);
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const long i = row0 + r;
            const T temp = E.e[i];
            E.xi[i] = E.xi[i] + ALP * E.p[i] + AMU * temp;
            const T rn = temp - AMU * E.v[i];
            E.r[i] = rn;
            acc0 += rn * rn;
            acc1 += rn * E.r0[i];
        }
        double tot[2];
        if (!member_reduce(E, blk, m, (double)acc0, (double)acc1, red, tot)) continue;
        if (threadIdx.x == 0) {
            MemberScalars* S = E.S + m;
            E.ticket[m] = 0;
            const double RN = tot[0], C1 = tot[1];
            S->RN = RN;
            S->C1 = C1;
            S->K += 1;
            S->total_iter += 1;
            const int K = S->K;
            const double ERR = sqrt(RN / S->BN);                        // 215
            S->ERR = ERR;
            if (!isfinite(RN) || !isfinite(C1)) {
                stop_member(S, CLOWNS_STOP_NONFINITE, S->mode == 0 ? CLOWNS_IER_NONFINITE : 0);
            } else if (K >= 10 && fabs(ERR - S->ERRP) <= ERR * 1.0e-6) {  // 228
                stop_member(S, CLOWNS_STOP_STAGNATION, 0);
            } else if (ERR <= S->EPS) {                                  // 232
                stop_member(S, CLOWNS_STOP_TOL, 0);
            } else {
                S->ERRP = ERR;
                if (S->AMU == 0.0) {                                     // 234
                    stop_member(S, CLOWNS_STOP_AMU_ZERO, 0);
                } else if (C1 == 0.0) {                                  // 240
                    stop_member(S, CLOWNS_STOP_C1_ZERO, 0);
                } else {
                    S->BETA = C1 / S->AMU / S->RQ;                       // 241
                    if (K >= S->ITER) {                                  // 250-254
                        if (S->mode == 0) {
                            stop_member(S, CLOWNS_STOP_MAXITER, CLOWNS_IER_MAXITER);
                            S->K = S->ITER + 1;
                        } else {
                            stop_member(S, CLOWNS_STOP_MAXITER, 0);
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
}

// P = R + BETA (P - AMU Q)  (242-246)
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_pupdate(Eng<T> E) {
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_active(E, blk, m, row0, rows)) continue;
        const T BETA = T(E.S[m].BETA), AMU = T(E.S[m].AMU);
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const long i = row0 + r;
            E.p[i] = E.r[i] + BETA * (E.p[i] - AMU * E.q[i]);
        }
    }
}

// BN = (b^,b^); R = b^ - q; C1 = (R,R); P = R0 = R  (129-145).  p holds b^ = PM W b
// and q holds PM A x0 on entry.
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_initres(Eng<T> E) {
    __shared__ double red[64];
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_active(E, blk, m, row0, rows)) continue;
        T acc0 = T(0), acc1 = T(0);
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const long i = row0 + r;
            T temp = E.p[i];
            acc0 += temp * temp;
            temp = temp - E.q[i];
            E.r[i] = temp;
            acc1 += temp * temp;
            E.p[i] = temp;
            E.r0[i] = temp;
        }
        double tot[2];
        if (!member_reduce(E, blk, m, (double)acc0, (double)acc1, red, tot)) continue;
        if (threadIdx.x == 0) {
            E.ticket[m] = 0;
            E.S[m].BN = tot[0];
            E.S[m].C1 = tot[1];
        }
        __syncthreads();
    }
}

// Loop guard: the only writer of the WHILE condition.  Continue while any
// member is still iterating; as a backstop no correct run reaches, stop after
// max ITER + 2 body executions.
static __global__ void k_eng_guard(MemberScalars* S, int M, int* ctrl, cudaGraphConditionalHandle h) {
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int m = threadIdx.x; m < M; m += blockDim.x)
        if (!S[m].done) atomicOr(&any, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        ctrl[0] += 1;
        int go = any;
        if (go && ctrl[0] > ctrl[1] + 1) {
            go = 0;
            for (int m = 0; m < M; m++)
                if (!S[m].done) stop_member(S + m, CLOWNS_STOP_MAXITER, S[m].mode == 0 ? CLOWNS_IER_MAXITER : 0);
        }
        cudaGraphSetConditional(h, go ? 1u : 0u);
    }
}

// Copy each member's solution back to the caller's x (plain path).
template <typename T>
__global__ void k_eng_copy_out(Eng<T> E) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < E.NV; i += (long)gridDim.x * blockDim.x) {
        const int m = E.blk_member[i / kTile];
        if (m < 0) continue;
        const long li = i - E.mem_off[m];
        if (li < E.mem_n[m]) E.in[m].x[li] = (double)E.xi[i];
    }
}

}  // namespace clowns
