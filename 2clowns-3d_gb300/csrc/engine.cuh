// engine.cuh -- batched left-preconditioned BiCGSTAB engine (PCGPME's method,
// src2LOWNS/pcgpme_para.F90:1-354) over a concatenation of independent systems.
//
// One solve of the reference is a batch of one member.  Members occupy disjoint,
// tile-aligned row ranges of one row space; every kernel serves all members and
// skips members whose solve has stopped.  Coefficients and Krylov vectors are
// stored as T (double for the plain path, float for the inner solve of the
// mixed path); all scalars are double.
//
// Dot products follow ONE summation tree, whichever kernel computes them (tile
// or balanced kernels, 4 or 8 rows per thread, 64 or 128 threads per tile, the
// persistent or the wavefront loop, a single system or a member of an
// ensemble), so that a solve's iteration count and pressure do not depend on
// the launch shape the autotuner picks:
//   - chunk c of a member is its rows [128 c, 128 c + 128); lane l of the chunk
//     folds the rows 128 c + 32 u + l, u = 0..3, in that order, with fused
//     multiply-adds into a value of T's precision (rows past the member's end
//     are not folded);
//   - the chunk total is the xor butterfly of the 32 lane values (offsets 16,
//     8, 4, 2, 1), converted to double;
//   - group g is the chunks [64 g, 64 g + 64): lane l adds the totals of chunks
//     l and l + 32 that exist, then the butterfly;
//   - the member total: lane l sums the group totals l, l + 32, ... in order,
//     then the butterfly.
// Each add of a butterfly is commutative, so every lane ends with the same
// bits, and a warp that reduces several chunks at once (a transposed butterfly,
// warp_tsum) forms the same tree for each.  Whoever accounts the last chunk of a
// group (a ticket per group) sums the group; whoever sums a member's last group
// sums the member and finalises its scalars on the device.
#pragma once

#include "common.cuh"

namespace clowns {

constexpr int kTile = 512;           // rows per tile (member ranges are tile-aligned)
constexpr int kEngBlock = 256;
constexpr int kRowsPerThread = 4;   // rows a thread handles per step (explicit ILP)
constexpr int kStepBlock = kTile / kRowsPerThread;   // threads covering one tile in one step
constexpr int kEngMaxGrid = kNumSMs * 8;
constexpr int kChunk = 128;         // rows of a reduction chunk: 32 lanes x 4 rows
constexpr int kChunkRows = kChunk / 32;
constexpr int kTileChunks = kTile / kChunk;
constexpr int kGroupChunks = 64;    // chunks per reduction group
constexpr int kWaveChunk = 16;     // tiles per completion counter of the wavefront loop
constexpr int kWaveStages = 7;     // stages of each of the wavefront loop's two apply segments
constexpr int kWaveBufs = 5;       // intermediate vectors of one operator application

// Polls a device-wide wait makes before it gives up (seconds; no correct run
// comes near it: a phase lasts microseconds to milliseconds).
constexpr long kBarSpinLimit = 1L << 24;

// Control block of the wavefront loop (single system).  D: the largest
// distance, in tiles, between a row and a real (non-zero-row) neighbour it
// gathers from, set by the setup kernel.  alp/amu/beta: finalisations of the
// three per-iteration reductions published in the current launch.  Followed
// in the workspace by 12 x nchunk completion counters.
struct WaveCtl {
    int D;
    int pad0;
    unsigned alp, amu, beta;
    int pad[27];
};

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
    int mode;       // 0: PCGPME; 1: inner solve of the refinement loop; 2: PCGPME_WILL (2DH)
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

// Block of a balanced launch: member m, index j among the member's gm blocks,
// the member's first block b0.
struct BalBlock {
    int m, j, gm, b0;
};
constexpr int kBalTabMax = kNumSMs * 16;   // entries of one block table (one wave at most)

template <typename T>
struct Eng {
    long NV;                  // rows of the concatenated space (multiple of kTile)
    int M, nblk;              // members, kTile-blocks of the row space
    int n1;                   // rows of the system when M == 1
    T* al;                    // 6 columns, stride NV, scaled + sorted
    int* ll;                  // 6 columns, global 0-based indices
    T* d;
    T *r, *p, *r0, *q, *e, *v, *t, *xi;   // Krylov vectors (xi: inner solution)
    double* W;                // row scaling (mixed path), NV
    double* x64;              // FP64 solution (mixed path)
    double* r64;              // FP64 work vectors (mixed path)
    double* s64;
    double* t64;
    const int* blk_member;    // member of each tile (-1: none)
    const int* blk_rows;      // real rows in each tile (0: pad only)
    const int* mem_off;       // first row of each member (a multiple of kTile)
    const int* mem_n;         // rows of each member
    const int* mem_nblk;      // tiles with real rows per member
    const int* mem_blk0;      // first tile of each member
    const int* mem_grp0;      // first reduction group of each member
    const int* mem_ngrp;      // reduction groups of each member
    unsigned* gticket;        // chunks accounted, one per group
    double* gpartials;        // 2 per group
    T* w[kWaveBufs];          // wavefront loop: intermediates of one application (single system)
    WaveCtl* wave;            // wavefront loop control (nullptr: not available)
    const MemberIn* in;       // per-member inputs (device copy of the table)
    MemberScalars* S;
    double* partials;         // 2 per chunk of the row space (chunk totals)
    unsigned* ticket;         // groups summed, one per member
    int* ctrl;                // [0] loop-body count, [1] max ITER over members, [2] bodies of earlier sweeps
    const BalBlock* baltab;   // ensembles: 16 block tables of the balanced kernels (nullptr: none)
    const int* balg;          // ensembles: the blocks of each table's launch (16)
    int nl;                   // columns the members' matrices fill: 6 (3D) or 4 (2DV, and the 2DH
                              // systems of PCGPME_WILL); the rest are empty
    int pf;                   // balanced kernels: rows per block and stream asked of L2 before the
                              // wait on the previous kernel (0: none)
    int* abort;               // set by a kernel whose bounded wait ran out (the grid barrier's flag)
    int keep;                 // balanced kernels: the first `keep` matrix columns are loaded with an L2
                              // evict_last policy (0: all streamed)
};

// ---------------------------------------------------------------------------
// Loads of data other blocks wrote.  Vectors are read with plain loads: every
// phase that reads a vector is separated from the phase that wrote it by a
// kernel boundary or by grid_sync, whose gpu-scope fence orders the block's
// later loads after the other blocks' stores (the L1 is not a source of stale
// lines across it).  Scalars and reduction partials, which can be written by
// other blocks within the same phase, are read through L2 (ld.global.cg).

template <typename V>
__device__ __forceinline__ V ldg2(const V* p) { return *p; }

// Per-row arithmetic with explicit single roundings, so that every kernel that
// evaluates a formula (tile, balanced, fused or not) rounds it identically.
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// c - a b with one rounding
template <typename V>
__device__ __forceinline__ V fnma(V a, V b, V c) { return fma_rn(-a, b, c); }
__device__ __forceinline__ double sld(const double* p) { return __ldcg(p); }
__device__ __forceinline__ int sld(const int* p) { return __ldcg(p); }

// ---------------------------------------------------------------------------
// The canonical reduction

// Transposed xor butterfly of V values per lane (V a power of two <= 32): value
// q of every lane is summed over the warp with the butterfly tree 16, 8, 4, 2, 1,
// and each lane returns one of the V totals, number `idx` (from the lane's bits
// 4, 3, ... : the same total sits in 32 / V lanes).  V = 1 is the plain
// butterfly; V = 2 the pair sum (lanes 0-15: value 0, lanes 16-31: value 1).
template <typename A, int V>
__device__ __forceinline__ A warp_tsum(A (&v)[V], int& idx) {
    const int lane = threadIdx.x & 31;
    idx = 0;
    int off = 16;
#pragma unroll
    for (int h = V / 2; h >= 1; h /= 2) {          // h values remain after this level
        const bool hi = (lane & off) != 0;
#pragma unroll
        for (int j = 0; j < h; j++) {
            const A keep = hi ? v[h + j] : v[j];
            const A send = hi ? v[j] : v[h + j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
        idx = 2 * idx + (hi ? 1 : 0);
        off >>= 1;
    }
    A s = v[0];
#pragma unroll
    for (; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    return s;
}

// Record a chunk total (global chunk index gc, value k of NV) -- by one lane.
// Plain store: account_chunks orders every thread's stores before the block's
// tickets (a block barrier, then acquire-release ticket increments).
template <typename T>
__device__ __forceinline__ void put_chunk(const Eng<T>& E, long gc, int k, double v) {
    E.partials[2 * gc + k] = v;
}

// Reduce one chunk's lane values (NV = 1 or 2 per lane) and record its totals.
// Every lane of the warp calls it.
template <typename T, typename A, int NV>
__device__ __forceinline__ void chunk_total(const Eng<T>& E, long gc, A (&v)[NV]) {
    int idx;
    const A s = warp_tsum<A, NV>(v, idx);
    if ((threadIdx.x & (32 / NV - 1)) == 0) put_chunk(E, gc, idx, (double)s);
}

// Ticket increment with acquire-release semantics at GPU scope: it releases
// the writes that precede it in the issuing thread's order -- the writes of the
// other threads of the block included, when a block or warp barrier separates
// them from it -- and acquires the writes released by earlier increments, for
// the issuing thread and for whatever a barrier orders after it.
__device__ __forceinline__ unsigned ticket_add(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// Called by EVERY thread of the block once the block's writers recorded the
// totals of member m's chunks [c0, c1) (member-relative; empty allowed).
// Accounts the chunks to their groups; the block that completes a group sums it
// in one warp, and the warp that completes the member's last group sums the
// member.  Returns true in all lanes of that warp, with the member
// totals in tot[] (every lane); false elsewhere.
template <typename T>
__device__ __noinline__ bool account_chunks(const Eng<T>& E, int m, int c0, int c1, double (&tot)[2]) {
    constexpr int kList = 256;
    __shared__ int s_list[kList];
    __shared__ int s_n;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int n = E.mem_n[m];
    const int nc = (n + kChunk - 1) / kChunk;
    const long gc0 = E.mem_off[m] / kChunk;
    const int G0 = E.mem_grp0[m], ng = E.mem_ngrp[m];
    bool fin = false;
    const int g_lo = c1 > c0 ? c0 / kGroupChunks : 0;
    const int g_hi = c1 > c0 ? (c1 - 1) / kGroupChunks : -1;
    __syncthreads();                              // the block's chunk totals precede its tickets
    for (int gb = g_lo; gb <= g_hi || gb == g_lo; gb += kList) {
        if (threadIdx.x == 0) s_n = 0;
        __syncthreads();
        for (int g = gb + threadIdx.x; g <= g_hi && g < gb + kList; g += blockDim.x) {
            const int cnt = min(c1, (g + 1) * kGroupChunks) - max(c0, g * kGroupChunks);
            const int need = min(kGroupChunks, nc - g * kGroupChunks);
            const unsigned old = ticket_add(&E.gticket[G0 + g], (unsigned)cnt);
            if (old + (unsigned)cnt == (unsigned)need) s_list[atomicAdd(&s_n, 1)] = g;
        }
        __syncthreads();
        const int nd = s_n;
        for (int q = wid; q < nd; q += nw) {
            const int g = s_list[q];                // acquired by the ticket that completed it
            const long p0 = 2 * (gc0 + (long)g * kGroupChunks);
            const int cg = min(kGroupChunks, nc - g * kGroupChunks);
            double a = 0.0, b = 0.0;
            if (lane < cg) {
                a = __ldcg(E.partials + p0 + 2 * lane);
                b = __ldcg(E.partials + p0 + 2 * lane + 1);
            }
            if (lane + 32 < cg) {
                a += __ldcg(E.partials + p0 + 2 * (lane + 32));
                b += __ldcg(E.partials + p0 + 2 * (lane + 32) + 1);
            }
            double s = warp_pair_sum(a, b);
            if (lane == 0) E.gpartials[2L * (G0 + g) + 0] = s;
            if (lane == 16) E.gpartials[2L * (G0 + g) + 1] = s;
            __syncwarp();                           // both totals precede lane 0's ticket
            unsigned last = 0;
            if (lane == 0) {
                E.gticket[G0 + g] = 0;
                last = ticket_add(&E.ticket[m], 1u) == (unsigned)ng - 1u;
            }
            __syncwarp();                           // lane 0's acquire precedes the warp's loads
            if (__shfl_sync(0xffffffffu, last, 0)) {
                a = b = 0.0;
                for (int j = lane; j < ng; j += 32) {
                    a += __ldcg(E.gpartials + 2L * (G0 + j) + 0);
                    b += __ldcg(E.gpartials + 2L * (G0 + j) + 1);
                }
                s = warp_pair_sum(a, b);
                tot[0] = __shfl_sync(0xffffffffu, s, 0);
                tot[1] = __shfl_sync(0xffffffffu, s, 16);
                fin = true;
            }
        }
        if (g_hi < gb + kList) break;
        __syncthreads();                          // s_list is reused by the next round
    }
    return fin;
}

// ---------------------------------------------------------------------------
// Tile walk helpers

// Member, first row and real rows of tile blk; false for tiles without real
// rows.  Single system: `done` (the stop flag) is loaded but not waited for --
// callers issue their data loads first and test it before any store or
// reduction, so its latency overlaps theirs (it is set only once, at the end),
// and no table loads are needed.  Ensembles: tiles of a stopped member return
// at once (false), before any data load -- members stop at different
// iterations, and their tiles must not keep streaming the matrix.
template <typename T>
__device__ __forceinline__ bool tile_active(const Eng<T>& E, int blk, int& m, long& row0, int& rows, int& done) {
    row0 = (long)blk * kTile;
    if (E.M == 1) {
        m = 0;
        rows = (int)max(0L, min((long)kTile, (long)E.n1 - row0));
    } else {
        m = E.blk_member[blk];
        if (m < 0) return false;
        rows = E.blk_rows[blk];
    }
    if (rows == 0) return false;
    done = sld(&E.S[m].done);
    return E.M == 1 || !done;
}

// Member-relative chunk range of a tile's real rows.
template <typename T>
__device__ __forceinline__ void tile_chunks(const Eng<T>& E, int m, long row0, int rows, int& c0, int& c1) {
    const long off = E.M == 1 ? 0L : (long)E.mem_off[m];
    c0 = (int)((row0 - off) / kChunk);
    c1 = c0 + (rows + kChunk - 1) / kChunk;
}

__device__ __forceinline__ void stop_member(MemberScalars* S, int reason, int ier) {
    S->done = 1;
    S->reason = reason;
    if (ier) S->ier = ier;
}

// The member's scalars copied into the block's shared memory at a kernel's
// start (44 words, one per thread), for the finalisation at its end.
__device__ __forceinline__ void copy_scalars(MemberScalars& dst, const MemberScalars* S) {
    constexpr int W = (int)(sizeof(MemberScalars) / 4);
    if (threadIdx.x < W) ((int*)&dst)[threadIdx.x] = __ldcg((const int*)S + threadIdx.x);
}

// Old scalar values for a finalisation: read through L2 from the member's
// scalars (PRE = false) or from a copy the block took when the kernel started
// (PRE = true; nothing writes them while the kernel runs).
template <bool PRE>
__device__ __forceinline__ double rd(const double* p) { return PRE ? *p : sld(p); }
template <bool PRE>
__device__ __forceinline__ int rd(const int* p) { return PRE ? *p : sld(p); }

// Finalisation of the reductions, by one thread once a member's totals are
// known.  MODE 1: RQ -> ALP = C1 / RQ (pcgpme_para.F90:167); MODE 2: AMU =
// (e,v) / (v,v) (197).
template <int MODE, bool PRE = false>
__device__ __forceinline__ void finish_sweep56(MemberScalars* S, const double (&tot)[2],
                                               const MemberScalars* src = nullptr) {
    if (!PRE) src = S;
    if (MODE == 1) {
        const double C1 = rd<PRE>(&src->C1);
        S->RQ = tot[0];
        const double ALP = C1 / tot[0];                         // 167
        S->ALP = ALP;
        if (!isfinite(tot[0]) || !isfinite(ALP)) {
            S->K = rd<PRE>(&src->K) + 1;
            stop_member(S, CLOWNS_STOP_NONFINITE, rd<PRE>(&src->mode) != 1 ? CLOWNS_IER_NONFINITE : 0);
        }
    } else {
        S->SS = tot[1];
        const double AMU = tot[0] / tot[1];                     // 197
        S->AMU = AMU;
        if (!isfinite(tot[1]) || !isfinite(AMU)) {
            S->K = rd<PRE>(&src->K) + 1;
            stop_member(S, CLOWNS_STOP_NONFINITE, rd<PRE>(&src->mode) != 1 ? CLOWNS_IER_NONFINITE : 0);
        }
    }
}

// RN, C1 -> ERR, the stop tests and BETA (pcgpme_para.F90:215-254).
template <bool PRE = false>
__device__ __forceinline__ void finish_xrupdate(MemberScalars* S, const double (&tot)[2],
                                                const MemberScalars* src = nullptr) {
    if (!PRE) src = S;
    const double RN = tot[0], C1 = tot[1];
    const double AMUs = rd<PRE>(&src->AMU), RQ = rd<PRE>(&src->RQ), BN = rd<PRE>(&src->BN);
    const double ERRP = rd<PRE>(&src->ERRP), EPS = rd<PRE>(&src->EPS);
    const int mode = rd<PRE>(&src->mode), ITER = rd<PRE>(&src->ITER);
    S->RN = RN;
    S->C1 = C1;
    const int K = rd<PRE>(&src->K) + 1;
    S->K = K;
    S->total_iter = rd<PRE>(&src->total_iter) + 1;
    const double ERR = sqrt(RN / BN);                            // 215
    S->ERR = ERR;
    if (!isfinite(RN) || !isfinite(C1)) {
        stop_member(S, CLOWNS_STOP_NONFINITE, mode != 1 ? CLOWNS_IER_NONFINITE : 0);
    } else if (K >= 10 && fabs(ERR - ERRP) <= ERR * 1.0e-6) {    // 228
        stop_member(S, CLOWNS_STOP_STAGNATION, 0);
    } else if (ERR <= EPS) {                                     // 232
        stop_member(S, CLOWNS_STOP_TOL, 0);
    } else {
        S->ERRP = ERR;
        if (AMUs == 0.0) {                                       // 234
            stop_member(S, CLOWNS_STOP_AMU_ZERO, 0);
        } else if (C1 == 0.0) {                                  // 240
            stop_member(S, CLOWNS_STOP_C1_ZERO, 0);
        } else {
            // 241 (pcgpme_para.F90); PCGPME_WILL forms C1 / (AMU RQ), pcgpme_2DH.f90:255
            S->BETA = mode == 2 ? C1 / (AMUs * RQ) : C1 / AMUs / RQ;
            if (K >= ITER) {                                     // 250-254
                if (mode != 1) {
                    stop_member(S, CLOWNS_STOP_MAXITER, CLOWNS_IER_MAXITER);
                    S->K = ITER + 1;
                } else {
                    stop_member(S, CLOWNS_STOP_MAXITER, 0);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Setup: scaling W = P2/(max(sum|AL|,D)+P1 D), scaled copies and the per-row
// exchange sort (pcgpme_para.F90:77-112).  Explicitly rounded arithmetic so the
// sort decisions equal an IEEE evaluation of the source.  For rows beyond a
// member's n (its pad rows) all vectors are zeroed and slots point at the
// member's zero row.  NL: the batch's widest matrix; a member with fewer
// columns (a 2DV member, 4, beside 3D ones) reads only its own, and its other
// slots are empty -- zero coefficients never move ahead of others in the
// exchange sort (strict <), so its first columns sort exactly as a sort of its
// own columns would.  init_x: copy the member's initial guess into xi / x64.
template <typename T, int NL>
__global__ void __launch_bounds__(kEngBlock) k_eng_setup(Eng<T> E, double P1, double P2, int mixed) {
    int reach = 0;    // gather distance in tiles (wavefront loop), real neighbours only
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
            if (E.wave)
#pragma unroll
                for (int k = 0; k < kWaveBufs; k++) E.w[k][i] = T(0);
            continue;
        }
        double a[6];
        int c[6];
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 6; k++) {
            if (k < NL && k < in.nl) {
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
        for (int k = 0; k < 6; k++) {
            E.al[k * NV + i] = T(a[k]);
            E.ll[k * NV + i] = c[k];
            if (c[k] < pad) reach = max(reach, abs((int)(c[k] / kTile) - blk));
        }
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
    if (E.wave) {
        __shared__ int s_reach;
        if (threadIdx.x == 0) s_reach = 0;
        __syncthreads();
        if (reach) atomicMax(&s_reach, reach);
        __syncthreads();
        if (threadIdx.x == 0 && s_reach) atomicMax(&E.wave->D, s_reach);
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
    if (threadIdx.x == 0) { ctrl[0] = 0; ctrl[1] = iter; ctrl[2] = 0; }
}

// ---------------------------------------------------------------------------
// Operator pieces as phase functions: a phase walks the tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... so the same code runs as a
// standalone kernel (one block per tile) and inside the persistent kernel
// (a co-resident grid, phases separated by grid barriers).  MEMBER-AWARE:
// tiles of stopped members are skipped.

// out = D in + sum_k AL_k in[LL_k]   (AXSUB, pcgpme_para.F90:323-352)
template <typename T>
__device__ __forceinline__ void tl_axsub(const Eng<T>& E, int blk, const T* __restrict__ in, T* __restrict__ out) {
    constexpr int R = kRowsPerThread;
    const long NV = E.NV;
    {
        int m, rows;
        long row0;
        int done;
        if (!tile_active(E, blk, m, row0, rows, done)) return;
        for (int base = threadIdx.x; base < rows; base += blockDim.x * R) {
            T s[R];
            bool ok[R];
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int r = base + u * blockDim.x;
                ok[u] = r < rows;
                const long i = row0 + (ok[u] ? r : 0);
                s[u] = ldg2(in + i) * ld_stream(E.d + i);
            }
#pragma unroll
            for (int k = 0; k < 6; k++) {
                T a[R];
                int c[R];
#pragma unroll
                for (int u = 0; u < R; u++) {
                    const long i = row0 + (ok[u] ? base + u * blockDim.x : 0);
                    a[u] = ld_stream(E.al + k * NV + i);
                    c[u] = ld_stream(E.ll + k * NV + i);
                }
#pragma unroll
                for (int u = 0; u < R; u++) s[u] = fma_rn(a[u], ldg2(in + c[u]), s[u]);
            }
#pragma unroll
            for (int u = 0; u < R; u++)
                if (ok[u] && !done) out[row0 + base + u * blockDim.x] = s[u];
        }
    }
}

template <typename T>
__device__ __forceinline__ void ph_axsub(const Eng<T>& E, const T* __restrict__ in, T* __restrict__ out) {
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) tl_axsub(E, blk, in, out);
}

// One single-neighbour sweep of LDUSUB: out = in - AL_k in[LL_k]  (263-304)
template <typename T>
__device__ __forceinline__ void tl_sweep(const Eng<T>& E, int blk, int k, const T* __restrict__ in,
                                         T* __restrict__ out) {
    constexpr int R = kRowsPerThread;
    const long NV = E.NV;
    const T* __restrict__ a = E.al + k * NV;
    const int* __restrict__ c = E.ll + k * NV;
    {
        int m, rows;
        long row0;
        int done;
        if (!tile_active(E, blk, m, row0, rows, done)) return;
        for (int base = threadIdx.x; base < rows; base += blockDim.x * R) {
            T av[R], xv[R], gv[R];
            int cv[R];
            bool ok[R];
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int r = base + u * blockDim.x;
                ok[u] = r < rows;
                const long i = row0 + (ok[u] ? r : 0);
                av[u] = ld_stream(a + i);
                cv[u] = ld_stream(c + i);
                xv[u] = ldg2(in + i);
            }
#pragma unroll
            for (int u = 0; u < R; u++) gv[u] = ldg2(in + cv[u]);
#pragma unroll
            for (int u = 0; u < R; u++)
                if (ok[u] && !done) out[row0 + base + u * blockDim.x] = fnma(av[u], gv[u], xv[u]);
        }
    }
}

template <typename T>
__device__ __forceinline__ void ph_sweep(const Eng<T>& E, int k, const T* __restrict__ in, T* __restrict__ out) {
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) tl_sweep(E, blk, k, in, out);
}

// Two consecutive single-neighbour sweeps k, k+1 in one pass:
//   o = in - AL_k in[LL_k] ;  out = o - AL_k+1 o[LL_k+1]
// The value of o at the gathered row j = LL_k+1(i) is recomputed from in, AL_k
// and LL_k at j with the same fused multiply-add, so the result equals two
// separate sweeps bit for bit while the intermediate vector never goes to
// memory and one kernel boundary goes away.  The zero row (j = pad) has
// AL = 0, LL = pad and in = 0, so its o is 0 as it must be.
template <typename T>
__device__ __forceinline__ void tl_sweep2(const Eng<T>& E, int blk, int k, const T* __restrict__ in,
                                          T* __restrict__ out) {
    constexpr int R = kRowsPerThread;
    const long NV = E.NV;
    const T* __restrict__ a0 = E.al + k * NV;
    const int* __restrict__ c0 = E.ll + k * NV;
    const T* __restrict__ a1 = a0 + NV;
    const int* __restrict__ c1 = c0 + NV;
    {
        int m, rows;
        long row0;
        int done;
        if (!tile_active(E, blk, m, row0, rows, done)) return;
        for (int base = threadIdx.x; base < rows; base += blockDim.x * R) {
            T x[R], aa[R], ab[R], xj[R], aj[R];
            int ca[R], cb[R], cj[R];
            bool ok[R];
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int r = base + u * blockDim.x;
                ok[u] = r < rows;
                const long i = row0 + (ok[u] ? r : 0);
                x[u] = ldg2(in + i);
                aa[u] = ld_stream(a0 + i);
                ca[u] = ld_stream(c0 + i);
                ab[u] = ld_stream(a1 + i);
                cb[u] = ld_stream(c1 + i);
            }
#pragma unroll
            for (int u = 0; u < R; u++) {
                xj[u] = ldg2(in + cb[u]);
                aj[u] = ldg2(a0 + cb[u]);
                cj[u] = ldg2(c0 + cb[u]);
            }
            T oi[R], oj[R];
#pragma unroll
            for (int u = 0; u < R; u++) {
                oi[u] = fnma(aa[u], ldg2(in + ca[u]), x[u]);
                oj[u] = fnma(aj[u], ldg2(in + cj[u]), xj[u]);
            }
#pragma unroll
            for (int u = 0; u < R; u++)
                if (ok[u] && !done) out[row0 + base + u * blockDim.x] = fnma(ab[u], oj[u], oi[u]);
        }
    }
}

template <typename T>
__device__ __forceinline__ void ph_sweep2(const Eng<T>& E, int k, const T* __restrict__ in, T* __restrict__ out) {
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) tl_sweep2(E, blk, k, in, out);
}

// Rows of one chunk as lanes see them: warp-wide lane l takes rows
// 32 u + l (u = 0..kChunkRows-1) of the chunk starting at tile row cr.

// Last sweep (J=5,6, 306-318) with an optional fused per-member reduction:
//   MODE 0 none; 1: RQ = (r0,out) -> ALP = C1/RQ; 2: AMU = (e,out)/(out,out)
// Warp w of the block takes the tile's chunks w, w + nw, ...  Returns true in
// the one thread that finalised the member's scalars.
template <typename T, int MODE>
__device__ __forceinline__ bool tl_sweep56(const Eng<T>& E, int blk, const T* __restrict__ in, T* __restrict__ out) {
    const long NV = E.NV;
    const T* __restrict__ a5 = E.al + 4 * NV;
    const T* __restrict__ a6 = E.al + 5 * NV;
    const int* __restrict__ c5 = E.ll + 4 * NV;
    const int* __restrict__ c6 = E.ll + 5 * NV;
    int m, rows;
    long row0;
    int done;
    if (!tile_active(E, blk, m, row0, rows, done)) return false;
    constexpr int U = kChunkRows;
    constexpr int NVAL = MODE == 2 ? 2 : 1;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q = wid; q < kTileChunks; q += nw) {
        const int cr = q * kChunk;
        if (cr >= rows) break;
        T a5v[U], a6v[U], xv[U], g5[U], g6[U];
        int c5v[U], c6v[U];
        bool ok[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = cr + 32 * u + lane;
            ok[u] = r < rows;
            const long i = row0 + (ok[u] ? r : cr);
            a5v[u] = ld_stream(a5 + i);
            a6v[u] = ld_stream(a6 + i);
            c5v[u] = ld_stream(c5 + i);
            c6v[u] = ld_stream(c6 + i);
            xv[u] = ldg2(in + i);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            g5[u] = ldg2(in + c5v[u]);
            g6[u] = ldg2(in + c6v[u]);
        }
        T acc[NVAL];
#pragma unroll
        for (int k = 0; k < NVAL; k++) acc[k] = T(0);
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (!ok[u] || done) continue;
            const long i = row0 + cr + 32 * u + lane;
            const T y = fnma(a6v[u], g6[u], fnma(a5v[u], g5[u], xv[u]));
            out[i] = y;
            if (MODE == 1) acc[0] = fma_rn(ldg2(E.r0 + i), y, acc[0]);
            if (MODE == 2) {
                acc[0] = fma_rn(ldg2(E.e + i), y, acc[0]);
                acc[NVAL - 1] = fma_rn(y, y, acc[NVAL - 1]);
            }
        }
        if (MODE != 0 && !done) chunk_total(E, (row0 + cr) / kChunk, acc);
    }
    if (MODE == 0 || done) return false;
    int c0, c1;
    tile_chunks(E, m, row0, rows, c0, c1);
    double tot[2];
    if (!account_chunks(E, m, c0, c1, tot) || lane != 0) return false;
    E.ticket[m] = 0;
    finish_sweep56<MODE>(E.S + m, tot);
    __threadfence();
    return true;
}

template <typename T, int MODE>
__device__ __forceinline__ void ph_sweep56(const Eng<T>& E, const T* __restrict__ in, T* __restrict__ out) {
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) tl_sweep56<T, MODE>(E, blk, in, out);
}

// E = R - ALP Q  (171-175)
template <typename T>
__device__ __forceinline__ void tl_eupdate(const Eng<T>& E, int blk) {
    {
        int m, rows;
        long row0;
        int done;
        if (!tile_active(E, blk, m, row0, rows, done)) return;
        const T ALP = T(sld(&E.S[m].ALP));
        constexpr int R = kRowsPerThread;
        for (int base = threadIdx.x; base < rows; base += blockDim.x * R) {
            T rv[R], qv[R];
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int r = base + u * blockDim.x;
                const long i = row0 + (r < rows ? r : 0);
                rv[u] = ldg2(E.r + i);
                qv[u] = ldg2(E.q + i);
            }
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int r = base + u * blockDim.x;
                if (r < rows && !done) E.e[row0 + r] = fnma(ALP, qv[u], rv[u]);
            }
        }
    }
}

template <typename T>
__device__ __forceinline__ void ph_eupdate(const Eng<T>& E) {
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) tl_eupdate(E, blk);
}

// X += ALP P + AMU E ; R = E - AMU V ; RN = (R,R) ; C1 = (R0,R)  (199-213),
// then ERR and the stop tests (215-241).  Warp w takes the tile's chunks w,
// w + nw, ...  Returns true in the one thread that finalised the member's
// scalars.
template <typename T>
__device__ __forceinline__ bool tl_xrupdate(const Eng<T>& E, int blk) {
    int m, rows;
    long row0;
    int done;
    if (!tile_active(E, blk, m, row0, rows, done)) return false;
    const T ALP = T(sld(&E.S[m].ALP)), AMU = T(sld(&E.S[m].AMU));
    constexpr int U = kChunkRows;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q = wid; q < kTileChunks; q += nw) {
        const int cr = q * kChunk;
        if (cr >= rows) break;
        T ev[U], xv[U], pv[U], vv[U], r0v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = cr + 32 * u + lane;
            const long i = row0 + (r < rows ? r : cr);
            ev[u] = ldg2(E.e + i);
            xv[u] = ldg2(E.xi + i);
            pv[u] = ldg2(E.p + i);
            vv[u] = ldg2(E.v + i);
            r0v[u] = ldg2(E.r0 + i);
        }
        T acc[2] = {T(0), T(0)};
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int r = cr + 32 * u + lane;
            if (r >= rows || done) continue;
            const long i = row0 + r;
            E.xi[i] = fma_rn(AMU, ev[u], fma_rn(ALP, pv[u], xv[u]));
            const T rn = fnma(AMU, vv[u], ev[u]);
            E.r[i] = rn;
            acc[0] = fma_rn(rn, rn, acc[0]);
            acc[1] = fma_rn(rn, r0v[u], acc[1]);
        }
        if (!done) chunk_total(E, (row0 + cr) / kChunk, acc);
    }
    if (done) return false;
    int c0, c1;
    tile_chunks(E, m, row0, rows, c0, c1);
    double tot[2];
    if (!account_chunks(E, m, c0, c1, tot) || lane != 0) return false;
    E.ticket[m] = 0;
    finish_xrupdate(E.S + m, tot);
    __threadfence();
    return true;
}

template <typename T>
__device__ __forceinline__ void ph_xrupdate(const Eng<T>& E) {
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) tl_xrupdate(E, blk);
}

// P = R + BETA (P - AMU Q)  (242-246)
template <typename T>
__device__ __forceinline__ void tl_pupdate(const Eng<T>& E, int blk) {
    {
        int m, rows;
        long row0;
        int done;
        if (!tile_active(E, blk, m, row0, rows, done)) return;
        const T BETA = T(sld(&E.S[m].BETA)), AMU = T(sld(&E.S[m].AMU));
        constexpr int R = kRowsPerThread;
        for (int base = threadIdx.x; base < rows; base += blockDim.x * R) {
            T rv[R], pv[R], qv[R];
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int r = base + u * blockDim.x;
                const long i = row0 + (r < rows ? r : 0);
                rv[u] = ldg2(E.r + i);
                pv[u] = ldg2(E.p + i);
                qv[u] = ldg2(E.q + i);
            }
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int r = base + u * blockDim.x;
                if (r < rows && !done) E.p[row0 + r] = fma_rn(BETA, fnma(AMU, qv[u], pv[u]), rv[u]);
            }
        }
    }
}

template <typename T>
__device__ __forceinline__ void ph_pupdate(const Eng<T>& E) {
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) tl_pupdate(E, blk);
}

// BN = (b^,b^); R = b^ - q; C1 = (R,R); P = R0 = R  (129-145).  p holds b^ = PM W b
// and q holds PM A x0 on entry.  Warp w takes the tile's chunks w, w + nw, ...
template <typename T>
__device__ __forceinline__ void ph_initres(const Eng<T>& E) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        int done;
        if (!tile_active(E, blk, m, row0, rows, done) || done) continue;
        for (int q = wid; q < kTileChunks; q += nw) {
            const int cr = q * kChunk;
            if (cr >= rows) break;
            T acc[2] = {T(0), T(0)};
#pragma unroll
            for (int u = 0; u < kChunkRows; u++) {
                const int r = cr + 32 * u + lane;
                if (r >= rows) continue;
                const long i = row0 + r;
                T temp = ldg2(E.p + i);
                acc[0] = fma_rn(temp, temp, acc[0]);
                temp = temp - ldg2(E.q + i);
                E.r[i] = temp;
                acc[1] = fma_rn(temp, temp, acc[1]);
                E.p[i] = temp;
                E.r0[i] = temp;
            }
            chunk_total(E, (row0 + cr) / kChunk, acc);
        }
        int c0, c1;
        tile_chunks(E, m, row0, rows, c0, c1);
        double tot[2];
        if (!account_chunks(E, m, c0, c1, tot) || lane != 0) continue;
        E.ticket[m] = 0;
        E.S[m].BN = tot[0];
        E.S[m].C1 = tot[1];
        __threadfence();
    }
}

// Standalone kernels (one block per tile): the same phases.  Each kernel opens
// with pdl_enter(): under programmatic dependent launch (graph mode) it lets the
// next kernel's blocks be scheduled as this grid's blocks retire, then waits
// for the previous grid to complete; without PDL both calls are no-ops.
__device__ __forceinline__ void pdl_trigger() {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 900)
    cudaTriggerProgrammaticLaunchCompletion();
#endif
}
__device__ __forceinline__ void pdl_wait() {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 900)
    cudaGridDependencySynchronize();
#endif
}
__device__ __forceinline__ void pdl_enter() {
    pdl_trigger();
    pdl_wait();
}

template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_axsub(Eng<T> E, const T* __restrict__ in, T* __restrict__ out) {
    pdl_enter();
    ph_axsub(E, in, out);
}
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_sweep(Eng<T> E, int k, const T* __restrict__ in,
                                                        T* __restrict__ out) {
    pdl_enter();
    ph_sweep(E, k, in, out);
}
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_sweep2(Eng<T> E, int k, const T* __restrict__ in,
                                                         T* __restrict__ out) {
    pdl_enter();
    ph_sweep2(E, k, in, out);
}
// Register budget of the dot-product kernels: the FP32 instances are held to
// 48 registers (10 blocks of 128 threads per SM, no spills; 2-3 % faster inner
// iterations measured), the FP64 instances keep their 61-64 (a cap spills and
// was 4-13 % slower).
template <typename T>
constexpr int kReduceMinBlocks = sizeof(T) == 4 ? 5 : 0;   // blocks of kEngBlock threads (0: no bound)

template <typename T, int MODE>
__global__ void __launch_bounds__(kEngBlock, kReduceMinBlocks<T>) k_eng_sweep56(Eng<T> E, const T* __restrict__ in, T* __restrict__ out) {
    pdl_enter();
    ph_sweep56<T, MODE>(E, in, out);
}
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_eupdate(Eng<T> E) {
    pdl_enter();
    ph_eupdate(E);
}
template <typename T>
__global__ void __launch_bounds__(kEngBlock, kReduceMinBlocks<T>) k_eng_xrupdate(Eng<T> E) {
    pdl_enter();
    ph_xrupdate(E);
}
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_pupdate(Eng<T> E) {
    pdl_enter();
    ph_pupdate(E);
}
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_eng_initres(Eng<T> E) {
    pdl_enter();
    ph_initres(E);
}

// ---------------------------------------------------------------------------
// Balanced kernels.  The iteration's kernels can instead run as exactly one
// wave each: G = (resident blocks per SM) x SMs blocks, block b owning the
// chunks [nc b / G, nc (b+1) / G) of its member (nc = its 128-row chunks).  An
// ensemble splits the G blocks over its members still iterating in proportion
// to their rows, at least one block each, by a table (BalBlock per block) that
// bal_rebuild writes on the device; blocks of a stopped member return before
// loading anything.  Every block then does the same work and all retire
// together, and the per-block costs -- launch, the stop-flag and scalar loads,
// the reduction tail -- are paid G times per kernel instead of once per
// 512-row tile (5517 times at 2.8 M rows).  The per-row arithmetic is the tile
// kernels'.  Every kernel gives warp w of the block the block's chunks w, w + 8,
// ... (R / 4 adjacent chunks per step; the element-wise kernels rotate w by the
// block index), so a warp past the block's range leaves the loop instead of
// computing on dummy rows.  The dot-product kernels fold each chunk as the
// canonical reduction prescribes and form the chunk totals in shared memory (4
// rows per thread, kTreeSmem) or four chunks at a time with one transposed
// butterfly (8 rows per thread).
//
// For a single system only the kernels whose results outlive a stop test read
// the stop flag: sweep56 (its reduction and finalisation) and xrupdate (x, r
// and the stop tests); after a stop the other kernels of the body write scratch vectors (t,
// q, e, v, p) the finished solve no longer reads, and the loop guard ends the
// graph at the end of the body.  (A flag load in every kernel cost 2-4 us per
// kernel at 2.8 M rows, as did reading the scalars once per block behind a
// barrier; each thread loads them, and the load overlaps its data loads.)
// FP64 kernels at 4 rows per thread are held to 85 registers (3 blocks per SM).

// This block's member, the member's first row and rows, and its chunk range.
// tab == nullptr: a single system, every block belongs to member 0.  Returns
// false for a block of an ensemble member that has stopped.
template <typename T>
__device__ __forceinline__ bool bal_block(const Eng<T>& E, const BalBlock* __restrict__ tab, BalBlock& bb,
                                          long& off, int& n, int& c0, int& c1) {
    if (!tab) {
        bb.m = 0;
        bb.j = blockIdx.x;
        bb.gm = gridDim.x;
        bb.b0 = 0;
        off = 0;
        n = E.n1;
    } else {
        bb = tab[blockIdx.x];
        off = E.mem_off[bb.m];
        n = E.mem_n[bb.m];
    }
    const long nc = (n + kChunk - 1) / kChunk;
    c0 = (int)(nc * bb.j / bb.gm);
    c1 = (int)(nc * (bb.j + 1) / bb.gm);
    return !tab || !sld(&E.S[bb.m].done);
}

// Row range of the same block.
template <typename T>
__device__ __forceinline__ bool bal_rows(const Eng<T>& E, const BalBlock* __restrict__ tab, BalBlock& bb, long& lo,
                                         long& hi) {
    long off;
    int n, c0, c1;
    const bool go = bal_block(E, tab, bb, off, n, c0, c1);
    lo = off + (long)c0 * kChunk;
    hi = off + min((long)n, (long)c1 * kChunk);
    return go;
}

// L2 prologue of the balanced kernels.  Under programmatic dependent launch a
// kernel's blocks take the SM slots the previous kernel's blocks leave, while
// that kernel's last block still runs its reduction tail (6-8 us in which HBM
// has nothing to do).  Before waiting on the previous kernel, a block asks L2
// for the first E.pf rows of its range of each stream it reads (the matrix and
// the vectors the previous kernel does not write), so that those bytes arrive
// during the tail.  A prefetch returns nothing to the thread: the values the
// kernel computes with are loaded after the wait, whatever the prefetch found.
// Single systems only: an ensemble block's rows come from a table that the loop
// rewrites on the device.
__device__ __forceinline__ void l2_prefetch_lines(const void* p0, const void* p1) {
    const unsigned long long b = (unsigned long long)p1;
    for (unsigned long long q = ((unsigned long long)p0 & ~127ull) + 128ull * threadIdx.x; q < b;
         q += 128ull * blockDim.x)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(q));
}
template <typename T>
__device__ __forceinline__ bool pf_range(const Eng<T>& E, const BalBlock* tab, long& lo, long& hi) {
    if (E.pf <= 0 || tab) return false;
    BalBlock bb;
    bal_rows(E, tab, bb, lo, hi);
    hi = min(hi, lo + (long)E.pf);
    return lo < hi;
}
template <typename U>
__device__ __forceinline__ void pf_rows(const U* s, long lo, long hi) {
    l2_prefetch_lines(s + lo, s + hi);
}

template <typename T, int R>
constexpr int kBalMinBlocks = R == 4 ? (sizeof(T) == 8 ? 3 : 4) : 1;

// Chunks per transposed butterfly in the register path of the balanced
// dot-product kernels (8 rows per thread; at 4 rows per thread they form the
// chunk totals in shared memory, kTreeSmem): four, 2.25 additions per chunk and
// value pair instead of five.
template <typename T, int R, int NVAL>
constexpr int kBalBatch = 4;

// Loads of the matrix columns.  Each application of PM A reads every column
// twice (AXSUB and its LDUSUB sweep) and an iteration does two applications;
// the first E.keep columns are loaded with an L2 evict_last policy, which keeps
// them resident across iterations, the others with evict_first (both evict-first
// in L1): one load instruction either way (ld.global.L2::cache_hint with a
// policy from createpolicy), the column picking the policy register.  E.keep
// comes from a byte budget that leaves most of L2 to the Krylov vectors.
struct ColPolicy {
    unsigned long long keep, stream;
    __device__ __forceinline__ ColPolicy() {
        asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(keep));
        asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(stream));
    }
    __device__ __forceinline__ unsigned long long col(int k, int kept) const { return k < kept ? keep : stream; }
};
__device__ __forceinline__ double ld_col(const double* a, unsigned long long pol) {
    double v;
    asm("ld.global.L1::evict_first.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ float ld_col(const float* a, unsigned long long pol) {
    float v;
    asm("ld.global.L1::evict_first.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ int ld_col(const int* a, unsigned long long pol) {
    int v;
    asm("ld.global.L1::evict_first.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
    return v;
}

// Keeps the compiler from hoisting the next step's loads above this step's
// stores: each step keeps its own window of R rows in flight, as the kernels'
// register budgets assume.
__device__ __forceinline__ void step_fence() { asm volatile("" ::: "memory"); }

// Chunk mapping of the element-wise balanced kernels (as the dot-product ones):
// warp w of a block takes the block's chunks c0 + CPS w', c0 + CPS (w' + 8), ...
// (CPS = R / 4 chunks per step, w' = w rotated by the block index, so that the
// block's last, incomplete round of chunks does not always fall on the same SM
// sub-partitions) and lane l row 32 u + l of each chunk.  A warp whose chunk
// lies past the block's range leaves the loop: only the member's last chunk
// has lanes without a row (ok = false), which compute on row `off` and store
// nothing.
__device__ __forceinline__ int bal_warp() {
    const int nw = blockDim.x >> 5;
    return (int)(((threadIdx.x >> 5) + blockIdx.x) % nw);
}
template <int R>
__device__ __forceinline__ void chunk_step(long off, int n, int cb, int c1, long (&i)[R], bool (&ok)[R]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int u = 0; u < R; u++) {
        const int cc = cb + u / kChunkRows;
        const long r = (long)cc * kChunk + 32 * (u % kChunkRows) + lane;
        ok[u] = cc < c1 && r < n;
        i[u] = off + (ok[u] ? r : 0);
    }
}

// NL: the columns the matrix fills (6, or 4 for a 2DH system, whose two empty
// columns hold zero coefficients at the zero row and are not read).
template <typename T, int R, int NL>
__global__ void __launch_bounds__(kEngBlock, kBalMinBlocks<T, R>) k_bal_axsub(Eng<T> E, const BalBlock* __restrict__ tab, const T* __restrict__ in, T* __restrict__ out) {
    pdl_trigger();
    const long NV = E.NV;
    long plo, phi;
    if (pf_range(E, tab, plo, phi)) {
        pf_rows(E.d, plo, phi);
#pragma unroll
        for (int k = 0; k < NL; k++) {
            pf_rows(E.al + k * NV, plo, phi);
            pf_rows(E.ll + k * NV, plo, phi);
        }
    }
    pdl_wait();
    BalBlock bb;
    long off;
    int n, c0, c1;
    if (!bal_block(E, tab, bb, off, n, c0, c1)) return;
    const ColPolicy cp;
    constexpr int CPS = R / kChunkRows;
    const int nw = blockDim.x >> 5;
    for (int cb = c0 + bal_warp() * CPS; cb < c1; cb += nw * CPS) {
        long i[R];
        bool ok[R];
        chunk_step<R>(off, n, cb, c1, i, ok);
        T s[R];
#pragma unroll
        for (int u = 0; u < R; u++) s[u] = ldg2(in + i[u]) * ld_stream(E.d + i[u]);
#pragma unroll
        for (int k = 0; k < NL; k++) {
            T a[R];
            int c[R];
            const unsigned long long pol = cp.col(k, E.keep);
#pragma unroll
            for (int u = 0; u < R; u++) {
                a[u] = ld_col(E.al + k * NV + i[u], pol);
                c[u] = ld_col(E.ll + k * NV + i[u], pol);
            }
#pragma unroll
            for (int u = 0; u < R; u++) s[u] = fma_rn(a[u], ldg2(in + c[u]), s[u]);
        }
#pragma unroll
        for (int u = 0; u < R; u++)
            if (ok[u]) out[i[u]] = s[u];
    }
}

template <typename T, int R>
__global__ void __launch_bounds__(kEngBlock, kBalMinBlocks<T, R>) k_bal_sweep(Eng<T> E, const BalBlock* __restrict__ tab, int k, const T* __restrict__ in,
                                                        T* __restrict__ out) {
    pdl_trigger();
    const long NV = E.NV;
    const T* __restrict__ a = E.al + k * NV;
    const int* __restrict__ c = E.ll + k * NV;
    long lo, hi;
    if (pf_range(E, tab, lo, hi)) {
        pf_rows(a, lo, hi);
        pf_rows(c, lo, hi);
    }
    pdl_wait();
    BalBlock bb;
    long off;
    int n, c0, c1;
    if (!bal_block(E, tab, bb, off, n, c0, c1)) return;
    const unsigned long long pol = ColPolicy().col(k, E.keep);
    constexpr int CPS = R / kChunkRows;
    const int nw = blockDim.x >> 5;
    for (int cb = c0 + bal_warp() * CPS; cb < c1; cb += nw * CPS) {
        long i[R];
        bool ok[R];
        chunk_step<R>(off, n, cb, c1, i, ok);
        T av[R], xv[R], gv[R];
        int cv[R];
#pragma unroll
        for (int u = 0; u < R; u++) {
            av[u] = ld_col(a + i[u], pol);
            cv[u] = ld_col(c + i[u], pol);
            xv[u] = ldg2(in + i[u]);
        }
#pragma unroll
        for (int u = 0; u < R; u++) gv[u] = ldg2(in + cv[u]);
#pragma unroll
        for (int u = 0; u < R; u++)
            if (ok[u]) out[i[u]] = fnma(av[u], gv[u], xv[u]);
    }
}

// ---------------------------------------------------------------------------
// AXSUB with its streams staged in shared memory by the bulk-copy engine (FP32
// inner solve of the mixed path, single systems).  Warp w of a block takes the
// block's chunks c0 + w, c0 + w + 8, ...; for each it needs D, AL(:, 1..NL) and
// LL(:, 1..NL) of 128 rows (13 rows of 512 B for NL = 6), which one lane asks
// of `cp.async.bulk` into the warp's two-stage ring while the warp gathers and
// computes the previous chunk, completion counted on one mbarrier per stage.
// The matrix does not change during the loop, so the first stages are asked
// for before the wait on the previous kernel.  The arithmetic is
// k_bal_axsub's, in the same order.  Every wait is bounded: a warp whose copy
// has not landed (in every lane) after kStgSpinLimit polls raises E.abort (the
// host reports the solve as failed) and, before its block exits, waits (bounded
// again) for the copies it has in flight.
constexpr int kStgStages = 2;
constexpr long kStgSpinLimit = 1L << 22;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned phase) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}
// global -> shared bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

template <int NL>
constexpr int kStgStageBytes = kChunk * ((1 + NL) * 4 + NL * 4);   // FP32 D, AL, int LL
template <int NL>
constexpr size_t kStgSmem = (size_t)(kEngBlock / 32) * kStgStages * kStgStageBytes<NL>;

template <int NL>
__global__ void __launch_bounds__(kEngBlock, 1) k_bal_axsub_stg(Eng<float> E, const float* __restrict__ in,
                                                               float* __restrict__ out) {
    extern __shared__ __align__(128) unsigned char stg_smem[];
    __shared__ __align__(8) unsigned long long full[kEngBlock / 32][kStgStages];
    constexpr int NW = kEngBlock / 32, SB = kStgStageBytes<NL>;
    pdl_trigger();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int q = 0; q < NW; q++)
            for (int b = 0; b < kStgStages; b++) mbar_init(&full[q][b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    BalBlock bb;
    long off;
    int n, c0, c1;
    bal_block(E, (const BalBlock*)nullptr, bb, off, n, c0, c1);
    const long NV = E.NV;
    unsigned char* ring = stg_smem + (size_t)w * kStgStages * SB;
    auto issue = [&](int k) {           // one lane: chunk k of this warp into stage k % kStgStages
        const int b = k % kStgStages;
        const long r0 = off + (long)(c0 + w + NW * k) * kChunk;
        unsigned char* st = ring + (size_t)b * SB;
        mbar_expect_tx(&full[w][b], SB);
        bulk_g2s(st, E.d + r0, kChunk * 4, &full[w][b]);
#pragma unroll
        for (int c = 0; c < NL; c++) {
            bulk_g2s(st + kChunk * 4 * (1 + c), E.al + c * NV + r0, kChunk * 4, &full[w][b]);
            bulk_g2s(st + kChunk * 4 * (1 + NL + c), E.ll + c * NV + r0, kChunk * 4, &full[w][b]);
        }
    };
    const int nk = c1 - c0 > w ? (c1 - c0 - w + NW - 1) / NW : 0;     // chunks of this warp
    if (lane == 0)
        for (int k = 0; k < kStgStages && k < nk; k++) issue(k);
    __syncwarp();
    pdl_wait();                           // `in` is the previous kernel's output
    int issued = min(nk, kStgStages), waited = 0;
    for (int k = 0; k < nk; k++) {
        const int b = k % kStgStages;
        bool landed = false;
        for (long spins = 0; spins < kStgSpinLimit && !landed; spins++)
            landed = mbar_try_wait(&full[w][b], (k / kStgStages) & 1);
        if (!__all_sync(0xffffffffu, landed)) {
            if (lane == 0) atomicExch(E.abort, 1);
            break;
        }
        waited = k + 1;
        const int cb = c0 + w + NW * k;
        const unsigned char* st = ring + (size_t)b * SB;
        const float* sd = (const float*)st;
        const float* sa = sd + kChunk;
        const int* sc = (const int*)(st + kChunk * 4 * (1 + NL));
        float s[kChunkRows];
        float g[NL][kChunkRows];
#pragma unroll
        for (int u = 0; u < kChunkRows; u++) {
            const long r = (long)cb * kChunk + 32 * u + lane;
            s[u] = in[off + (r < n ? r : 0)];
#pragma unroll
            for (int c = 0; c < NL; c++) g[c][u] = in[sc[c * kChunk + 32 * u + lane]];
        }
#pragma unroll
        for (int u = 0; u < kChunkRows; u++) {
            const int rr = 32 * u + lane;
            s[u] = s[u] * sd[rr];
#pragma unroll
            for (int c = 0; c < NL; c++) s[u] = fma_rn(sa[c * kChunk + rr], g[c][u], s[u]);
        }
        __syncwarp();                     // every lane has read stage b
        if (lane == 0 && k + kStgStages < nk) {
            issue(k + kStgStages);
            issued = k + kStgStages + 1;
        }
#pragma unroll
        for (int u = 0; u < kChunkRows; u++) {
            const long r = (long)cb * kChunk + 32 * u + lane;
            if (r < n) out[off + r] = s[u];
        }
    }
    // after a wait ran out: the copies still in flight land before the block's
    // shared memory is released
    issued = __shfl_sync(0xffffffffu, issued, 0);
    for (int k = waited; k < issued; k++) {
        long spins = 0;
        while (!mbar_try_wait(&full[w][k % kStgStages], (k / kStgStages) & 1) && ++spins < kStgSpinLimit) {
        }
    }
}

// the fused pair of sweeps k, k+1 (as tl_sweep2)
template <typename T, int R>
__global__ void __launch_bounds__(kEngBlock, kBalMinBlocks<T, R>) k_bal_sweep2(Eng<T> E, const BalBlock* __restrict__ tab, int k, const T* __restrict__ in,
                                                         T* __restrict__ out) {
    pdl_trigger();
    const long NV = E.NV;
    const T* __restrict__ a0 = E.al + k * NV;
    const int* __restrict__ c0 = E.ll + k * NV;
    const T* __restrict__ a1 = a0 + NV;
    const int* __restrict__ c1 = c0 + NV;
    long lo, hi;
    if (pf_range(E, tab, lo, hi)) {
        pf_rows(a0, lo, hi);
        pf_rows(c0, lo, hi);
        pf_rows(a1, lo, hi);
        pf_rows(c1, lo, hi);
    }
    pdl_wait();
    BalBlock bb;
    long off;
    int n, k0, k1;
    if (!bal_block(E, tab, bb, off, n, k0, k1)) return;
    const ColPolicy cp;
    const unsigned long long pol0 = cp.col(k, E.keep), pol1 = cp.col(k + 1, E.keep);
    constexpr int CPS = R / kChunkRows;
    const int nw = blockDim.x >> 5;
    for (int kb = k0 + bal_warp() * CPS; kb < k1; kb += nw * CPS) {
        long i[R];
        bool ok[R];
        chunk_step<R>(off, n, kb, k1, i, ok);
        T x[R], aa[R], ab[R], xj[R], aj[R];
        int ca[R], cb[R], cj[R];
#pragma unroll
        for (int u = 0; u < R; u++) {
            x[u] = ldg2(in + i[u]);
            aa[u] = ld_col(a0 + i[u], pol0);
            ca[u] = ld_col(c0 + i[u], pol0);
            ab[u] = ld_col(a1 + i[u], pol1);
            cb[u] = ld_col(c1 + i[u], pol1);
        }
#pragma unroll
        for (int u = 0; u < R; u++) {
            xj[u] = ldg2(in + cb[u]);
            aj[u] = ldg2(a0 + cb[u]);
            cj[u] = ldg2(c0 + cb[u]);
        }
        T oi[R], oj[R];
#pragma unroll
        for (int u = 0; u < R; u++) {
            oi[u] = fnma(aa[u], ldg2(in + ca[u]), x[u]);
            oj[u] = fnma(aj[u], ldg2(in + cj[u]), xj[u]);
        }
#pragma unroll
        for (int u = 0; u < R; u++)
            if (ok[u]) out[i[u]] = fnma(ab[u], oj[u], oi[u]);
    }
}

// Sum the batch's lane values (kBalBatch chunks x NVAL values) with one
// transposed butterfly and record the chunk totals.  Slot q of the batch is the
// chunk c0 + (8 (s0 + q / CPS) + w) CPS + q % CPS of the block's member.
template <typename T, int NVAL, int CPS, int B>
__device__ __forceinline__ void bal_flush(const Eng<T>& E, T (&v)[B * NVAL], long gc_member, int c0,
                                          int c1, int s0, int w, int nwarps) {
    constexpr int V = B * NVAL;
    int idx;
    const T s = warp_tsum<T, V>(v, idx);
    const int q = idx / NVAL, k = idx % NVAL;
    const int cc = c0 + (nwarps * (s0 + q / CPS) + w) * CPS + q % CPS;
    if ((threadIdx.x & (32 / V - 1)) == 0 && cc < c1) put_chunk(E, gc_member + cc, k, (double)s);
}

// Chunk totals through shared memory.  A butterfly over one or two values
// costs every lane five additions per value (on GB300's slow FP64 pipe, the
// bound of the FP64 dot-product kernels) and holds the batch of values in
// registers.  The dot-product kernels at 4 rows per thread (one chunk per warp
// and step) instead store each chunk's 32 lane values and, every kTreeSteps
// steps, let one thread per (chunk, value) add them up in T along the
// butterfly's own tree -- lanes differing in bit 4 first, in bit 0 last -- so
// the total has the same bits at about one addition per lane value.
template <typename T, int R>
constexpr bool kTreeSmem = R == 4;
constexpr int kTreeSteps = 8;
constexpr int kTreeRow = 33;    // padded row of 32 lane values (no bank conflicts)

template <typename A, int BIT, int PAT>
__device__ __forceinline__ A lane_tree(const A* r) {
    if constexpr (BIT == 4) {
        return r[PAT] + r[PAT | 16];
    } else {
        return lane_tree<A, BIT + 1, PAT>(r) + lane_tree<A, BIT + 1, PAT | (1 << BIT)>(r);
    }
}

// Chunk totals of one round: slot (st, w, q) holds the lane values of value q
// of the chunk warp w took at step s0 + st.  Reducing threads rotate with the
// block index over the SM sub-partitions.
template <typename T, int NVAL>
__device__ __forceinline__ void tree_flush(const Eng<T>& E, const T* tbuf, long gcm, int c0, int c1, int s0,
                                           int nsteps, int nwarps) {
    const int t = (int)((threadIdx.x + 32u * (blockIdx.x % (unsigned)nwarps)) % blockDim.x);
    if (t >= kTreeSteps * nwarps * NVAL) return;
    const int slot = t / NVAL, q = t % NVAL;
    const int st = slot / nwarps, ww = slot % nwarps;
    const int cb = c0 + nwarps * (s0 + st) + ww;
    if (s0 + st >= nsteps || cb >= c1) return;
    put_chunk(E, gcm + cb, q, (double)lane_tree<T, 0, 0>(tbuf + t * kTreeRow));
}

// sweeps 5, 6 with the RQ (MODE 1) or AMU (MODE 2) reduction (as tl_sweep56);
// NL = 4: a copy with the reduction
template <typename T, int MODE, int R, int NL>
__global__ void __launch_bounds__(kEngBlock, kBalMinBlocks<T, R>) k_bal_sweep56(Eng<T> E, const BalBlock* __restrict__ tab, const T* __restrict__ in, T* __restrict__ out) {
    pdl_trigger();
    const long NV = E.NV;
    const T* __restrict__ a5 = E.al + 4 * NV;
    const T* __restrict__ a6 = E.al + 5 * NV;
    const int* __restrict__ c5 = E.ll + 4 * NV;
    const int* __restrict__ c6 = E.ll + 5 * NV;
    {
        long plo, phi;
        if (pf_range(E, tab, plo, phi)) {
            if (NL == 6) {
                pf_rows(a5, plo, phi);
                pf_rows(c5, plo, phi);
                pf_rows(a6, plo, phi);
                pf_rows(c6, plo, phi);
            }
            if (MODE == 1) pf_rows(E.r0, plo, phi);
            if (MODE == 2) pf_rows(E.e, plo, phi);
        }
    }
    pdl_wait();
    BalBlock bb;
    long off;
    int n, c0, c1;
    if (!bal_block(E, tab, bb, off, n, c0, c1)) return;
    const int done = sld(&E.S[bb.m].done);
    __shared__ MemberScalars s_pre;
    if (MODE != 0) copy_scalars(s_pre, E.S + bb.m);
    constexpr int CPS = R / kChunkRows;              // chunks per warp and step
    constexpr int NVAL = MODE == 2 ? 2 : 1;
    constexpr int B = kBalBatch<T, R, NVAL>;
    constexpr int SPB = B / CPS;                     // steps per batch
    constexpr bool six = NL == 6;                    // NL = 4: sweeps 5 and 6 are empty, out = in
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const long gcm = off / kChunk;
    if constexpr (kTreeSmem<T, R> && MODE != 0) {
        __shared__ T tbuf[kTreeSteps * (kEngBlock / 32) * NVAL * kTreeRow];
        if (done) return;
        const int nsteps = (c1 - c0 + nwarps - 1) / nwarps;
        for (int s0 = 0; s0 < nsteps; s0 += kTreeSteps) {
#pragma unroll 1
            for (int st = 0; st < kTreeSteps; st++) {
                const int cb = c0 + nwarps * (s0 + st) + w;
                if (s0 + st >= nsteps || cb >= c1) break;          // the same for the whole warp
                T a5v[R], a6v[R], xv[R], wv[R], g5[R], g6[R];
                int c5v[R], c6v[R];
                bool ok[R];
                long i[R];
#pragma unroll
                for (int u = 0; u < R; u++) {
                    const long r = (long)cb * kChunk + 32 * u + lane;
                    ok[u] = r < n;
                    i[u] = off + (ok[u] ? r : 0);
                    if (six) {
                        a5v[u] = ld_stream(a5 + i[u]);
                        a6v[u] = ld_stream(a6 + i[u]);
                        c5v[u] = ld_stream(c5 + i[u]);
                        c6v[u] = ld_stream(c6 + i[u]);
                    }
                    xv[u] = ldg2(in + i[u]);
                    wv[u] = ldg2((MODE == 1 ? E.r0 : E.e) + i[u]);
                }
                if (six) {
#pragma unroll
                    for (int u = 0; u < R; u++) {
                        g5[u] = ldg2(in + c5v[u]);
                        g6[u] = ldg2(in + c6v[u]);
                    }
                }
                T v[NVAL];
#pragma unroll
                for (int q = 0; q < NVAL; q++) v[q] = T(0);
#pragma unroll
                for (int u = 0; u < R; u++) {
                    if (!ok[u]) continue;
                    const T y = six ? fnma(a6v[u], g6[u], fnma(a5v[u], g5[u], xv[u])) : xv[u];
                    out[i[u]] = y;
                    v[0] = fma_rn(wv[u], y, v[0]);
                    if (MODE == 2) v[NVAL - 1] = fma_rn(y, y, v[NVAL - 1]);
                }
#pragma unroll
                for (int q = 0; q < NVAL; q++) tbuf[((st * nwarps + w) * NVAL + q) * kTreeRow + lane] = v[q];
                step_fence();
            }
            __syncthreads();
            tree_flush<T, NVAL>(E, tbuf, gcm, c0, c1, s0, nsteps, nwarps);
            __syncthreads();
        }
    } else
    for (int s0 = 0; c0 + (nwarps * s0 + w) * CPS < c1; s0 += SPB) {
        T v[B * NVAL];
#pragma unroll
        for (int q = 0; q < B * NVAL; q++) v[q] = T(0);
#pragma unroll
        for (int st = 0; st < SPB; st++) {
            const int cb = c0 + (nwarps * (s0 + st) + w) * CPS;
            T a5v[R], a6v[R], xv[R], wv[R], g5[R], g6[R];
            int c5v[R], c6v[R];
            bool ok[R];
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int cc = cb + u / kChunkRows;
                const long r = (long)cc * kChunk + 32 * (u % kChunkRows) + lane;
                ok[u] = cc < c1 && r < n;
                const long i = off + (ok[u] ? r : 0);
                if (six) {
                    a5v[u] = ld_stream(a5 + i);
                    a6v[u] = ld_stream(a6 + i);
                    c5v[u] = ld_stream(c5 + i);
                    c6v[u] = ld_stream(c6 + i);
                }
                xv[u] = ldg2(in + i);
                if (MODE != 0) wv[u] = ldg2((MODE == 1 ? E.r0 : E.e) + i);   // with the streams, not after the stores
            }
            if (six) {
#pragma unroll
                for (int u = 0; u < R; u++) {
                    g5[u] = ldg2(in + c5v[u]);
                    g6[u] = ldg2(in + c6v[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < R; u++) {
                if (!ok[u] || done) continue;
                const long i = off + (long)(cb + u / kChunkRows) * kChunk + 32 * (u % kChunkRows) + lane;
                const T y = six ? fnma(a6v[u], g6[u], fnma(a5v[u], g5[u], xv[u])) : xv[u];
                out[i] = y;
                const int q = (st * CPS + u / kChunkRows) * NVAL;
                if (MODE != 0) v[q] = fma_rn(wv[u], y, v[q]);
                if (MODE == 2) v[q + NVAL - 1] = fma_rn(y, y, v[q + NVAL - 1]);
            }
            step_fence();
        }
        if (MODE != 0 && !done) bal_flush<T, NVAL, CPS, B>(E, v, gcm, c0, c1, s0, w, nwarps);
    }
    if (MODE == 0 || done) return;
    double tot[2];
    if (!account_chunks(E, bb.m, c0, c1, tot) || lane != 0) return;
    E.ticket[bb.m] = 0;
    finish_sweep56<MODE, true>(E.S + bb.m, tot, &s_pre);   // kernel completion publishes it
}

template <typename T, int R>
__global__ void __launch_bounds__(kEngBlock, kBalMinBlocks<T, R>) k_bal_eupdate(Eng<T> E, const BalBlock* __restrict__ tab) {
    pdl_trigger();
    long lo, hi;
    if (pf_range(E, tab, lo, hi)) pf_rows(E.r, lo, hi);
    pdl_wait();
    BalBlock bb;
    long off;
    int n, c0, c1;
    if (!bal_block(E, tab, bb, off, n, c0, c1)) return;
    const T ALP = T(sld(&E.S[bb.m].ALP));
    constexpr int CPS = R / kChunkRows;
    const int nw = blockDim.x >> 5;
    for (int cb = c0 + bal_warp() * CPS; cb < c1; cb += nw * CPS) {
        long i[R];
        bool ok[R];
        chunk_step<R>(off, n, cb, c1, i, ok);
        T rv[R], qv[R];
#pragma unroll
        for (int u = 0; u < R; u++) {
            rv[u] = ldg2(E.r + i[u]);
            qv[u] = ldg2(E.q + i[u]);
        }
#pragma unroll
        for (int u = 0; u < R; u++)
            if (ok[u]) E.e[i[u]] = fnma(ALP, qv[u], rv[u]);
    }
}

template <typename T, int R>
__global__ void __launch_bounds__(kEngBlock, kBalMinBlocks<T, R>) k_bal_xrupdate(Eng<T> E, const BalBlock* __restrict__ tab) {
    pdl_trigger();
    {
        long plo, phi;
        if (pf_range(E, tab, plo, phi)) {
            pf_rows(E.e, plo, phi);
            pf_rows(E.xi, plo, phi);
            pf_rows(E.p, plo, phi);
            pf_rows(E.v, plo, phi);
            pf_rows(E.r0, plo, phi);
        }
    }
    pdl_wait();
    BalBlock bb;
    long off;
    int n, c0, c1;
    if (!bal_block(E, tab, bb, off, n, c0, c1)) return;
    const int done = sld(&E.S[bb.m].done);
    const T ALP = T(sld(&E.S[bb.m].ALP)), AMU = T(sld(&E.S[bb.m].AMU));
    __shared__ MemberScalars s_pre;
    copy_scalars(s_pre, E.S + bb.m);
    constexpr int CPS = R / kChunkRows;
    constexpr int B = kBalBatch<T, R, 2>;
    constexpr int SPB = B / CPS;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const long gcm = off / kChunk;
    if constexpr (kTreeSmem<T, R>) {
        __shared__ T tbuf[kTreeSteps * (kEngBlock / 32) * 2 * kTreeRow];
        if (done) return;
        const int nsteps = (c1 - c0 + nwarps - 1) / nwarps;
        for (int s0 = 0; s0 < nsteps; s0 += kTreeSteps) {
#pragma unroll 1
            for (int st = 0; st < kTreeSteps; st++) {
                const int cb = c0 + nwarps * (s0 + st) + w;
                if (s0 + st >= nsteps || cb >= c1) break;          // the same for the whole warp
                T ev[R], xv[R], pv[R], vv[R], r0v[R];
                bool ok[R];
                long i[R];
#pragma unroll
                for (int u = 0; u < R; u++) {
                    const long r = (long)cb * kChunk + 32 * u + lane;
                    ok[u] = r < n;
                    i[u] = off + (ok[u] ? r : 0);
                    ev[u] = ldg2(E.e + i[u]);
                    xv[u] = ldg2(E.xi + i[u]);
                    pv[u] = ldg2(E.p + i[u]);
                    vv[u] = ldg2(E.v + i[u]);
                    r0v[u] = ldg2(E.r0 + i[u]);
                }
                T v0 = T(0), v1 = T(0);
#pragma unroll
                for (int u = 0; u < R; u++) {
                    if (!ok[u]) continue;
                    E.xi[i[u]] = fma_rn(AMU, ev[u], fma_rn(ALP, pv[u], xv[u]));
                    const T rn = fnma(AMU, vv[u], ev[u]);
                    E.r[i[u]] = rn;
                    v0 = fma_rn(rn, rn, v0);
                    v1 = fma_rn(rn, r0v[u], v1);
                }
                tbuf[((st * nwarps + w) * 2 + 0) * kTreeRow + lane] = v0;
                tbuf[((st * nwarps + w) * 2 + 1) * kTreeRow + lane] = v1;
                step_fence();
            }
            __syncthreads();
            tree_flush<T, 2>(E, tbuf, gcm, c0, c1, s0, nsteps, nwarps);
            __syncthreads();
        }
    } else
    for (int s0 = 0; c0 + (nwarps * s0 + w) * CPS < c1; s0 += SPB) {
        T v[B * 2];
#pragma unroll
        for (int q = 0; q < B * 2; q++) v[q] = T(0);
#pragma unroll
        for (int st = 0; st < SPB; st++) {
            const int cb = c0 + (nwarps * (s0 + st) + w) * CPS;
            T ev[R], xv[R], pv[R], vv[R], r0v[R];
            bool ok[R];
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int cc = cb + u / kChunkRows;
                const long r = (long)cc * kChunk + 32 * (u % kChunkRows) + lane;
                ok[u] = cc < c1 && r < n;
                const long i = off + (ok[u] ? r : 0);
                ev[u] = ldg2(E.e + i);
                xv[u] = ldg2(E.xi + i);
                pv[u] = ldg2(E.p + i);
                vv[u] = ldg2(E.v + i);
                r0v[u] = ldg2(E.r0 + i);
            }
#pragma unroll
            for (int u = 0; u < R; u++) {
                if (!ok[u] || done) continue;
                const long i = off + (long)(cb + u / kChunkRows) * kChunk + 32 * (u % kChunkRows) + lane;
                E.xi[i] = fma_rn(AMU, ev[u], fma_rn(ALP, pv[u], xv[u]));
                const T rn = fnma(AMU, vv[u], ev[u]);
                E.r[i] = rn;
                const int q = (st * CPS + u / kChunkRows) * 2;
                v[q] = fma_rn(rn, rn, v[q]);
                v[q + 1] = fma_rn(rn, r0v[u], v[q + 1]);
            }
            step_fence();
        }
        if (!done) bal_flush<T, 2, CPS, B>(E, v, gcm, c0, c1, s0, w, nwarps);
    }
    if (done) return;
    double tot[2];
    if (!account_chunks(E, bb.m, c0, c1, tot) || lane != 0) return;
    E.ticket[bb.m] = 0;
    finish_xrupdate<true>(E.S + bb.m, tot, &s_pre);          // kernel completion publishes it
}

template <typename T, int R>
__global__ void __launch_bounds__(kEngBlock, kBalMinBlocks<T, R>) k_bal_pupdate(Eng<T> E, const BalBlock* __restrict__ tab) {
    pdl_trigger();
    long lo, hi;
    if (pf_range(E, tab, lo, hi)) {
        pf_rows(E.r, lo, hi);
        pf_rows(E.p, lo, hi);
        pf_rows(E.q, lo, hi);
    }
    pdl_wait();
    BalBlock bb;
    long off;
    int n, c0, c1;
    if (!bal_block(E, tab, bb, off, n, c0, c1)) return;
    const T BETA = T(sld(&E.S[bb.m].BETA)), AMU = T(sld(&E.S[bb.m].AMU));
    constexpr int CPS = R / kChunkRows;
    const int nw = blockDim.x >> 5;
    for (int cb = c0 + bal_warp() * CPS; cb < c1; cb += nw * CPS) {
        long i[R];
        bool ok[R];
        chunk_step<R>(off, n, cb, c1, i, ok);
        T rv[R], pv[R], qv[R];
#pragma unroll
        for (int u = 0; u < R; u++) {
            rv[u] = ldg2(E.r + i[u]);
            pv[u] = ldg2(E.p + i[u]);
            qv[u] = ldg2(E.q + i[u]);
        }
#pragma unroll
        for (int u = 0; u < R; u++)
            if (ok[u]) E.p[i[u]] = fma_rn(BETA, fnma(AMU, qv[u], pv[u]), rv[u]);
    }
}

// Graph mode: the last node of the WHILE body and the only writer of the loop
// condition.  Continue while any member iterates; as a backstop no correct
// run reaches, stop after max ITER + 2 bodies.
// Ensembles with the balanced kernels: rebuild the 16 block tables over the
// members still iterating -- member m (active) takes blocks [C_m, C_m+1) of a
// launch of G blocks, C_m = A_m + floor((G - NA) R_m / RT), A_m and R_m the
// active members and their rows before m, NA and RT their totals -- so that
// blocks go to members that still work.  Skipped while NA equals the count of
// the last rebuild (*last_na), unless force.  One block; NA <= M <= G holds
// for every table (the host uploads G only then).
constexpr int kBalScanThreads = 256;
__device__ __forceinline__ void bal_rebuild(const MemberScalars* S, int M, const int* mem_n, BalBlock* tab,
                                            const int* balg, int* last_na, bool force) {
    __shared__ int s_cnt[kBalScanThreads + 1];
    __shared__ long long s_rows[kBalScanThreads + 1];
    const int t = threadIdx.x, nt = blockDim.x;
    const int per = (M + nt - 1) / nt, m0 = min(M, t * per), m1 = min(M, m0 + per);
    int c = 0;
    long long r = 0;
    for (int m = m0; m < m1; m++)
        if (!sld(&S[m].done)) { c++; r += mem_n[m]; }
    s_cnt[t + 1] = c;
    s_rows[t + 1] = r;
    __syncthreads();
    if (t == 0) {                         // exclusive prefix over the threads' chunks (nt <= 256)
        s_cnt[0] = 0;
        s_rows[0] = 0;
        for (int q = 1; q <= nt; q++) {
            s_cnt[q] += s_cnt[q - 1];
            s_rows[q] += s_rows[q - 1];
        }
    }
    __syncthreads();
    const int NA = s_cnt[nt];
    const long long RT = s_rows[nt];
    if (NA == 0 || (!force && NA == *last_na)) return;
    __syncthreads();
    if (t == 0) *last_na = NA;
    for (int k = 0; k < 16; k++) {
        const int G = balg[k];
        BalBlock* tk = tab + (size_t)k * kBalTabMax;
        int a = s_cnt[t];
        long long rb = s_rows[t];
        for (int m = m0; m < m1; m++) {
            if (sld(&S[m].done)) continue;
            const int c0 = a + (int)((long long)(G - NA) * rb / RT);
            rb += mem_n[m];
            const int c1 = a + 1 + (int)((long long)(G - NA) * rb / RT);
            for (int b = c0; b < c1; b++) tk[b] = BalBlock{m, b - c0, c1 - c0, c0};
            a++;
        }
    }
}

// Standalone rebuild before a loop starts (every member active again).
static __global__ void k_bal_rebuild(const MemberScalars* S, int M, const int* mem_n, BalBlock* tab,
                                     const int* balg, int* last_na) {
    bal_rebuild(S, M, mem_n, tab, balg, last_na, true);
}

static __global__ void k_eng_guard(MemberScalars* S, int M, int* ctrl, cudaGraphConditionalHandle h,
                                   const int* mem_n, BalBlock* baltab, const int* balg) {
    pdl_enter();
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int m = threadIdx.x; m < M; m += blockDim.x)
        if (!sld(&S[m].done)) atomicOr(&any, 1);
    __syncthreads();
    if (baltab) bal_rebuild(S, M, mem_n, baltab, balg, ctrl + 4, false);
    __syncthreads();
    if (threadIdx.x == 0) {
        ctrl[0] += 1;
        int go = any;
        if (go && ctrl[0] > ctrl[1] + 1) {
            go = 0;
            for (int m = 0; m < M; m++)
                if (!S[m].done) stop_member(S + m, CLOWNS_STOP_MAXITER, S[m].mode != 1 ? CLOWNS_IER_MAXITER : 0);
        }
        cudaGraphSetConditional(h, go ? 1u : 0u);
    }
}

// ---------------------------------------------------------------------------
// Persistent iteration loop.
//
// One cooperative launch runs the whole BiCGSTAB loop of every member: the 16
// phases of an iteration are separated by grid barriers instead of kernel
// boundaries.  Every barrier wait is bounded: a block that waits longer than
// `limit` polls raises the abort flag, and every block leaves the kernel at its
// next barrier; the host then reports the failure.  The limit is a kernel
// argument (kBarSpinLimit in every solve; a test gives a short one).

struct GridBar {
    unsigned count;
    unsigned gen;
    int abort;
    int pad[29];
};

__device__ __forceinline__ bool grid_sync(GridBar* gb, long limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* genp = &gb->gen;
        volatile int* abortp = &gb->abort;
        const unsigned g0 = *genp;
        __threadfence();
        const unsigned arrived = atomicAdd(&gb->count, 1u);
        if (arrived == gridDim.x - 1) {
            gb->count = 0;                 // nobody arrives again before gen moves
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            long spins = 0;
            while (*genp == g0) {
                if (*abortp) break;
                if (++spins > limit) {
                    atomicExch(&gb->abort, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = (*abortp == 0);
    }
    __syncthreads();
    return s_ok != 0;
}

template <typename T>
__device__ __forceinline__ bool ph_apply(const Eng<T>& E, GridBar* gb, long lim, const T* in, T* out, T* tmp,
                                         int mode) {
    ph_axsub(E, in, tmp);
    if (!grid_sync(gb, lim)) return false;
    ph_sweep2(E, 0, tmp, out);
    if (!grid_sync(gb, lim)) return false;
    ph_sweep2(E, 2, out, tmp);
    if (!grid_sync(gb, lim)) return false;
    if (mode == 0) ph_sweep56<T, 0>(E, tmp, out);
    if (mode == 1) ph_sweep56<T, 1>(E, tmp, out);
    if (mode == 2) ph_sweep56<T, 2>(E, tmp, out);
    return grid_sync(gb, lim);
}

// init != 0: also run the start of PCGPME (b^ = PM W b, q = PM A x0, residuals).
// lim: polls per barrier wait; absent >= 0: that block leaves at once without
// arriving anywhere (a test of the bounded waits: the others give up).
template <typename T, int MINB>
__global__ void __launch_bounds__(kEngBlock, MINB) k_eng_loop(Eng<T> E, GridBar* gb, int init, long lim, int absent) {
    if ((int)blockIdx.x == absent) return;
    if (init) {
        // b^ = PM W b in place on p (sweeps p->t->q->t->q->p)
        ph_sweep2(E, 0, E.p, E.t);
        if (!grid_sync(gb, lim)) return;
        ph_sweep2(E, 2, E.t, E.q);
        if (!grid_sync(gb, lim)) return;
        ph_sweep56<T, 0>(E, E.q, E.p);
        if (!grid_sync(gb, lim)) return;
        if (!ph_apply(E, gb, lim, E.xi, E.q, E.t, 0)) return;      // q = PM A x0
        ph_initres(E);
        if (!grid_sync(gb, lim)) return;
    }
    const int cap = sld(E.ctrl + 1) + 2;
    for (int body = 0;; body++) {
        // every block reads the same flags: their last writers finished before
        // the barrier that ended the previous iteration
        int any = 0;
        for (int m = 0; m < E.M; m++) any |= !sld(&E.S[m].done);
        if (!any) break;
        if (body >= cap) {                       // backstop: ITER bounds every member
            if (blockIdx.x == 0 && threadIdx.x == 0)
                for (int m = 0; m < E.M; m++)
                    if (!sld(&E.S[m].done))
                        stop_member(E.S + m, CLOWNS_STOP_MAXITER, sld(&E.S[m].mode) == 0 ? CLOWNS_IER_MAXITER : 0);
            break;
        }
        if (!ph_apply(E, gb, lim, E.p, E.q, E.t, 1)) return;       // q = PM A p ; ALP
        ph_eupdate(E);                                             // e = r - ALP q
        if (!grid_sync(gb, lim)) return;
        if (!ph_apply(E, gb, lim, E.e, E.v, E.t, 2)) return;       // v = PM A e ; AMU
        ph_xrupdate(E);                                            // x, r ; stop tests
        if (!grid_sync(gb, lim)) return;
        ph_pupdate(E);                                             // p
        if (!grid_sync(gb, lim)) return;
    }
}

// ---------------------------------------------------------------------------
// Wavefront loop (single system).
//
// One cooperative launch runs the iteration loop as a stream of (stage, tile)
// items instead of kernel-wide phases.  An iteration has three segments, each
// ended by one of BiCGSTAB's per-iteration reductions:
//   A: p = r + BETA (p - AMU q) | q = PM A p (axsub, 4 sweeps, sweep56) | RQ -> ALP
//   B: e = r - ALP q            | v = PM A e                            | AMU, SS
//   C: x, r ; RN, C1 ; stop tests -> BETA
// Within A and B a stage of tile t needs the previous stage only on tiles
// [t-D, t+D] (D: gather reach), so stage s of tile t is ordered at key
// t + s L with a lag L > D + kWaveChunk: every item comes after the items it
// waits for, and the FP64-heavy axsub of one tile runs beside the memory-bound
// sweeps of others.  Items are dealt round-robin to the co-resident blocks,
// which take them in order; each waits on per-chunk completion counters
// (monotone across iterations) and publishes its own.  The reductions are the
// canonical ones; their finalising thread publishes an epoch that the next
// segment waits for.  Every wait is bounded (`limit` polls): a block that gives
// up raises the abort flag, every other block leaves at its next wait, and the
// host reports the error.

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_s32(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Warp 0 waits until the counters of chunks c0..c1 reach (it + 1) x (tiles of
// the chunk); the whole block then proceeds.  False: abort raised.
__device__ __forceinline__ bool wave_wait_counts(const unsigned* cnt, int c0, int c1, int it, int nblk,
                                                 GridBar* gb, long limit) {
    __shared__ int s_ok;
    if (threadIdx.x < 32) {
        bool ok = true;
        for (int c = c0 + (int)threadIdx.x; c <= c1 && ok; c += 32) {
            const unsigned need = (unsigned)(it + 1) * (unsigned)min(kWaveChunk, nblk - c * kWaveChunk);
            long spins = 0;
            while (ld_relaxed_u32(cnt + c) < need) {
                if (ld_relaxed_s32(&gb->abort)) { ok = false; break; }
                if (++spins > limit) { atomicExch(&gb->abort, 1); ok = false; break; }
                __nanosleep(32);
            }
        }
        ok = __all_sync(0xffffffffu, ok);
        __threadfence();
        if (threadIdx.x == 0) s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Thread 0 waits until *ep >= need.  False: abort raised.
__device__ __forceinline__ bool wave_wait_epoch(const unsigned* ep, unsigned need, GridBar* gb, long limit) {
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        bool ok = true;
        long spins = 0;
        while (ld_relaxed_u32(ep) < need) {
            if (ld_relaxed_s32(&gb->abort)) { ok = false; break; }
            if (++spins > limit) { atomicExch(&gb->abort, 1); ok = false; break; }
            __nanosleep(64);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Stage s (0..6) of segment seg (0: A, 1: B) on tiles t0 .. t0+K-1 (K divides
// kWaveChunk) in iteration it.
template <typename T>
__device__ __forceinline__ bool wave_item(const Eng<T>& E, GridBar* gb, long lim, unsigned* cnt, int nchunk,
                                          int seg, int s, int t0, int K, int it, int D) {
    const int nblk = E.nblk;
    const int t1 = min(nblk, t0 + K);
    if (s >= 1) {
        const int lo = max(0, t0 - D), hi = min(nblk - 1, t1 - 1 + D);
        if (!wave_wait_counts(cnt + (long)(seg * 6 + s - 1) * nchunk, lo / kWaveChunk, hi / kWaveChunk, it, nblk,
                              gb, lim))
            return false;
    }
    for (int t = t0; t < t1; t++) {
        if (s == 6) {
            const bool fin = seg == 0 ? tl_sweep56<T, 1>(E, t, E.w[4], E.q)    // q = PM A p ; RQ ; ALP
                                      : tl_sweep56<T, 2>(E, t, E.w[4], E.v);   // v = PM A e ; AMU
            if (fin) {
                __threadfence();
                atomicAdd(seg == 0 ? &E.wave->alp : &E.wave->amu, 1u);
            }
        } else if (s == 0) {
            if (seg == 1) tl_eupdate(E, t);              // e = r - ALP q
            else if (it > 0) tl_pupdate(E, t);           // p (the start set p = r0 before iteration 0)
        } else if (s == 1) {
            tl_axsub(E, t, seg == 0 ? (const T*)E.p : (const T*)E.e, E.w[0]);
        } else {
            tl_sweep(E, t, s - 2, (const T*)E.w[s - 2], E.w[s - 1]);
        }
    }
    if (s < 6) {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(cnt + (long)(seg * 6 + s) * nchunk + t0 / kWaveChunk, (unsigned)(t1 - t0));
        }
    }
    return true;
}

// K: tiles per item (divides kWaveChunk); slack: rounds of G items between an
// item and the items it waits for, beyond the gather reach.  lim and absent as
// for k_eng_loop.
template <typename T, int MINB>
__global__ void __launch_bounds__(kStepBlock, MINB) k_eng_wave(Eng<T> E, GridBar* gb, int K, int slack, long lim,
                                                               int absent) {
    if ((int)blockIdx.x == absent) return;
    WaveCtl* W = E.wave;
    unsigned* cnt = (unsigned*)(W + 1);
    const int G = gridDim.x;
    const int nblk = E.nblk;
    const int nchunk = (nblk + kWaveChunk - 1) / kWaveChunk;
    const int D = min(__ldcg(&W->D), nblk);
    const int nsup = (nblk + K - 1) / K;            // items per stage
    // lag between stages, in items: beyond the reach (in items, chunk-rounded) by slack rounds
    const long L = (long)(D + kWaveChunk + K) / K + 1 + (long)slack * ((G + kWaveStages - 1) / kWaveStages);
    const long nitems = ((long)nsup + (kWaveStages - 1) * L) * kWaveStages;
    const int cap = sld(E.ctrl + 1) + 2;
    MemberScalars* S = E.S;
    for (int it = 0;; it++) {
        if (it > 0 && !wave_wait_epoch(&W->beta, (unsigned)it, gb, lim)) return;
        if (sld(&S->done)) return;
        if (it >= cap) {                        // backstop: ITER stops the member first
            if (blockIdx.x == 0 && threadIdx.x == 0)
                stop_member(S, CLOWNS_STOP_MAXITER, sld(&S->mode) != 1 ? CLOWNS_IER_MAXITER : 0);
            return;
        }
        for (int seg = 0; seg < 2; seg++) {
            for (long q = blockIdx.x; q < nitems; q += G) {
                const int s = (int)(q % kWaveStages);
                const long u = q / kWaveStages - (long)s * L;
                if (u < 0 || u >= nsup) continue;
                if (!wave_item(E, gb, lim, cnt, nchunk, seg, s, (int)u * K, K, it, D)) return;
            }
            if (!wave_wait_epoch(seg == 0 ? &W->alp : &W->amu, (unsigned)(it + 1), gb, lim)) return;
            if (sld(&S->done)) return;
        }
        for (int t = blockIdx.x; t < nblk; t += G) {
            if (tl_xrupdate(E, t)) {
                __threadfence();
                atomicAdd(&W->beta, 1u);
            }
        }
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
