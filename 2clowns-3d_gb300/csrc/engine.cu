// engine.cu -- host orchestration of the batched BiCGSTAB engine: workspace
// layout, member tables, launch-shape autotuning, CUDA-graph capture of the
// solve (a WHILE conditional node repeats the iteration body until the device
// stop tests clear it), the plain FP64 path and the mixed-precision path
// (FP32 storage, FP64 iterative refinement).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <climits>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "engine.cuh"
#include "engine_api.h"
#include "trace.h"

namespace clowns {

// ---------------------------------------------------------------------------
// Mixed-path kernels (FP64 vectors, coefficients of type T)

template <typename T>
__device__ __forceinline__ bool tile_outer(const Eng<T>& E, int blk, int& m, long& row0, int& rows) {
    m = E.blk_member[blk];
    if (m < 0) return false;
    rows = E.blk_rows[blk];
    if (rows == 0) return false;
    if (E.S[m].odone) return false;
    row0 = (long)blk * kTile;
    return true;
}

// r64 = W (b - A x64) with the caller's original FP64 matrix (refinement residual)
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_mx_residual(Eng<T> E) {
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_outer(E, blk, m, row0, rows)) continue;
        const MemberIn in = E.in[m];
        const long off = E.mem_off[m];
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const long i = row0 + r;
            const long li = i - off;
            double s = in.d[li] * E.x64[i];
            for (int k = 0; k < in.nl; k++) {
                const int c = in.ll[k * (long)in.na + li];
                if (c > 0 && c <= in.n) s = fma_rn(in.al[k * (long)in.na + li], E.x64[off + c - 1], s);
            }
            E.r64[i] = E.W[i] * (in.b[li] - s);
        }
    }
}

// One LDUSUB sweep on FP64 vectors with the stored (type T) coefficients
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_mx_sweep(Eng<T> E, int k, const double* __restrict__ in,
                                                       double* __restrict__ out) {
    const long NV = E.NV;
    const T* __restrict__ a = E.al + k * NV;
    const int* __restrict__ c = E.ll + k * NV;
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_outer(E, blk, m, row0, rows)) continue;
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const long i = row0 + r;
            out[i] = fnma((double)a[i], in[c[i]], in[i]);
        }
    }
}

// Last sweep on FP64 vectors with the squared norm of the result per member
// (the canonical reduction: warp w takes the tile's chunks w, w + nw, ...).
//   PHASE 0: BN64 = ||PM W b||^2
//   PHASE 1: ERR64 = sqrt(||PM r||^2 / BN64); stop the member at the outer
//            tolerance or sweep cap, else arm its inner solve (mode 1) with
//            the relative reduction the outer tolerance still needs, halved
//            for margin, but no tighter than inner_tol: the last sweep then
//            stops near EPS64 instead of overshooting by up to inner_tol.
template <typename T, int PHASE>
__global__ void __launch_bounds__(kEngBlock) k_mx_sweep56(Eng<T> E, const double* __restrict__ in,
                                                         double* __restrict__ out, double inner_tol,
                                                         int inner_max) {
    const long NV = E.NV;
    const T* __restrict__ a5 = E.al + 4 * NV;
    const T* __restrict__ a6 = E.al + 5 * NV;
    const int* __restrict__ c5 = E.ll + 4 * NV;
    const int* __restrict__ c6 = E.ll + 5 * NV;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_outer(E, blk, m, row0, rows)) continue;
        for (int q = wid; q < kTileChunks; q += nw) {
            const int cr = q * kChunk;
            if (cr >= rows) break;
            double acc[1] = {0.0};
#pragma unroll
            for (int u = 0; u < kChunkRows; u++) {
                const int r = cr + 32 * u + lane;
                if (r >= rows) continue;
                const long i = row0 + r;
                const double y = fnma((double)a6[i], in[c6[i]], fnma((double)a5[i], in[c5[i]], in[i]));
                out[i] = y;
                acc[0] = fma_rn(y, y, acc[0]);
            }
            chunk_total(E, (row0 + cr) / kChunk, acc);
        }
        int c0, c1;
        tile_chunks(E, m, row0, rows, c0, c1);
        double tot[2];
        if (!account_chunks(E, m, c0, c1, tot) || lane != 0) continue;
        MemberScalars* S = E.S + m;
        E.ticket[m] = 0;
        if (PHASE == 0) {
            S->BN64 = tot[0];
        } else {
            const double err = sqrt(tot[0] / S->BN64);
            S->ERR64 = err;
            if (!isfinite(err)) {
                S->odone = 1;
                stop_member(S, CLOWNS_STOP_NONFINITE, CLOWNS_IER_NONFINITE);
            } else if (err <= S->EPS64) {
                S->odone = 1;
                stop_member(S, CLOWNS_STOP_TOL, 0);
            } else if (S->outer >= S->OITER) {
                S->odone = 1;
                stop_member(S, CLOWNS_STOP_MAXITER, CLOWNS_IER_MAXITER);
            } else {
                S->outer += 1;
                S->SIGMA = sqrt(tot[0]);
                S->K = 0;
                S->ERRP = 0.0;
                S->done = 0;
                S->mode = 1;
                S->EPS = fmax(inner_tol, 0.5 * S->EPS64 / err);
                S->ITER = inner_max;
            }
        }
        __threadfence();
    }
}

// Inner right-hand side: r = p = r0 = T(PM r64 / sigma), xi = 0; BN = C1 = ||r||^2
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_mx_normalize(Eng<T> E) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_outer(E, blk, m, row0, rows)) continue;
        const double inv = 1.0 / E.S[m].SIGMA;
        for (int q = wid; q < kTileChunks; q += nw) {
            const int cr = q * kChunk;
            if (cr >= rows) break;
            double acc[1] = {0.0};
#pragma unroll
            for (int u = 0; u < kChunkRows; u++) {
                const int r = cr + 32 * u + lane;
                if (r >= rows) continue;
                const long i = row0 + r;
                const T v = T(E.r64[i] * inv);
                E.r[i] = v;
                E.p[i] = v;
                E.r0[i] = v;
                E.xi[i] = T(0);
                acc[0] = fma_rn((double)v, (double)v, acc[0]);
            }
            chunk_total(E, (row0 + cr) / kChunk, acc);
        }
        int c0, c1;
        tile_chunks(E, m, row0, rows, c0, c1);
        double tot[2];
        if (!account_chunks(E, m, c0, c1, tot) || lane != 0) continue;
        E.ticket[m] = 0;
        E.S[m].BN = tot[0];
        E.S[m].C1 = tot[0];
        __threadfence();
    }
}

// x64 += sigma * xi (FP64 pressure accumulation)
template <typename T>
__global__ void __launch_bounds__(kEngBlock) k_mx_update(Eng<T> E) {
    for (int blk = blockIdx.x; blk < E.nblk; blk += gridDim.x) {
        int m, rows;
        long row0;
        if (!tile_outer(E, blk, m, row0, rows)) continue;
        const double sg = E.S[m].SIGMA;
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const long i = row0 + r;
            E.x64[i] += sg * (double)E.xi[i];
        }
    }
}

// ctrl[2] accumulates the loop bodies of earlier sweeps.
__global__ void k_mx_reset_ctrl(int* ctrl, int inner_max) {
    if (threadIdx.x == 0 && blockIdx.x == 0) { ctrl[2] += ctrl[0]; ctrl[0] = 0; ctrl[1] = inner_max; }
}

template <typename T>
__global__ void k_mx_copy_out(Eng<T> E) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < E.NV; i += (long)gridDim.x * blockDim.x) {
        const int m = E.blk_member[i / kTile];
        if (m < 0) continue;
        const long li = i - E.mem_off[m];
        if (li < E.mem_n[m]) E.in[m].x[li] = E.x64[i];
    }
}

__global__ void k_mixed_init_scalars(MemberScalars* S, int M, double eps, int oiter, int* ctrl) {
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
        MemberScalars z;
        memset(&z, 0, sizeof(z));
        z.EPS64 = eps;
        z.OITER = oiter;
        z.mode = 1;
        S[m] = z;
    }
    if (threadIdx.x == 0) { ctrl[0] = 0; ctrl[1] = 0; ctrl[2] = 0; }
}

// Export of the scaled/sorted matrix (test hook), member 0 only.
template <typename T>
__global__ void k_eng_export(Eng<T> E, double* al_s, int* ll_s, double* d_s, double* b_s, int nl, long na_out) {
    const int n = E.mem_n[0];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        for (int k = 0; k < nl; k++) {
            al_s[k * na_out + i] = (double)E.al[k * E.NV + i];
            ll_s[k * na_out + i] = E.ll[k * E.NV + i];
        }
        d_s[i] = (double)E.d[i];
        b_s[i] = (double)E.r[i];
    }
}

// ---------------------------------------------------------------------------
// Layout

// Reduction groups of a member of n rows: kGroupChunks consecutive 128-row chunks each.
static inline int member_groups(int n) {
    const int nc = (n + kChunk - 1) / kChunk;
    return (nc + kGroupChunks - 1) / kGroupChunks;
}

struct EngLayout {
    long NV = 0;
    int M = 0, nblk = 0, ngrp = 0, mixed = 0, tsize = 8, wave = 0, nchunk = 0, n1 = 0;
    size_t o_blk_member, o_blk_rows, o_mem_off, o_mem_n, o_mem_nblk, o_mem_blk0, o_ticket, o_ctrl;
    size_t o_mem_grp0, o_mem_ngrp, o_gticket, o_gpartials;
    size_t o_in, o_S, o_partials, o_bar, o_al, o_ll, o_d, o_vec[8], o_W, o_x64, o_r64, o_s64, o_t64;
    size_t o_wave, o_wbuf[kWaveBufs];
    size_t o_baltab = 0;   // ensembles: block tables of the balanced kernels
    size_t o_balg = 0;     // ensembles: blocks of each table's launch
    size_t total = 0;
};

// wave: -1 = the wavefront loop's buffers for single systems (M == 1), 0 = none.
static EngLayout eng_layout(int M, const int* n, int mixed, int wave = -1) {
    EngLayout L;
    L.M = M;
    L.mixed = mixed;
    L.wave = wave < 0 ? (M == 1) : wave;
    L.n1 = M == 1 ? n[0] : 0;
    L.tsize = mixed ? 4 : 8;
    long NV = 0;
    int ngrp = 0;
    for (int m = 0; m < M; m++) {
        NV += (long)align_up((size_t)n[m] + 1, kTile);
        ngrp += member_groups(n[m]);
    }
    L.NV = NV;
    L.nblk = (int)(NV / kTile);
    L.ngrp = ngrp;
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + (bytes ? bytes : 1), 256); return at; };
    L.o_blk_member = take(sizeof(int) * L.nblk);
    L.o_blk_rows = take(sizeof(int) * L.nblk);
    L.o_mem_off = take(sizeof(int) * M);
    L.o_mem_n = take(sizeof(int) * M);
    L.o_mem_nblk = take(sizeof(int) * M);
    L.o_mem_blk0 = take(sizeof(int) * M);
    L.o_ticket = take(sizeof(unsigned) * M);
    L.o_mem_grp0 = take(sizeof(int) * M);
    L.o_mem_ngrp = take(sizeof(int) * M);
    L.o_gticket = take(sizeof(unsigned) * ngrp);
    L.o_gpartials = take(sizeof(double) * 2 * ngrp);
    L.o_ctrl = take(sizeof(int) * 8);
    L.o_in = take(sizeof(MemberIn) * M);
    L.o_S = take(sizeof(MemberScalars) * M);
    L.o_partials = take(sizeof(double) * 2 * (NV / kChunk));
    L.o_bar = take(sizeof(GridBar));
    L.o_al = take((size_t)L.tsize * 6 * NV);
    L.o_ll = take(sizeof(int) * 6 * NV);
    L.o_d = take((size_t)L.tsize * NV);
    for (int v = 0; v < 8; v++) L.o_vec[v] = take((size_t)L.tsize * NV);
    if (mixed) {
        L.o_W = take(sizeof(double) * NV);
        L.o_x64 = take(sizeof(double) * NV);
        L.o_r64 = take(sizeof(double) * NV);
        L.o_s64 = take(sizeof(double) * NV);
        L.o_t64 = take(sizeof(double) * NV);
    } else {
        L.o_W = L.o_x64 = L.o_r64 = L.o_s64 = L.o_t64 = 0;
    }
    L.nchunk = (L.nblk + kWaveChunk - 1) / kWaveChunk;
    if (L.wave) {
        L.o_wave = take(sizeof(WaveCtl) + sizeof(unsigned) * 12 * (size_t)L.nchunk);
        for (int k = 0; k < kWaveBufs; k++) L.o_wbuf[k] = take((size_t)L.tsize * NV);
    } else {
        L.o_wave = 0;
        for (int k = 0; k < kWaveBufs; k++) L.o_wbuf[k] = 0;
    }
    if (M > 1) {
        L.o_baltab = take(sizeof(BalBlock) * 16 * (size_t)kBalTabMax);
        L.o_balg = take(sizeof(int) * 16);
    }
    L.total = o;
    return L;
}

// Matrix columns the balanced kernels keep in L2 (the first ones of the sorted
// order): as many as fit a budget of CLOWNS_L2_KEEP_MB (default kL2KeepMB) at
// (word + index) bytes per row.
constexpr int kL2KeepMB = 40;
static int l2_keep_cols(long NV, int tsize) {
    static const long mb = [] {
        const char* v = getenv("CLOWNS_L2_KEEP_MB");
        return v ? std::max(0L, atol(v)) : (long)kL2KeepMB;
    }();
    const long col = NV * (tsize + 4L);
    return (int)std::min(6L, mb * 1000000L / std::max(1L, col));
}

// Rows per block and stream of the balanced kernels' L2 prologue (0: none);
// CLOWNS_L2_PREFETCH overrides the default.  Measured at 2.8 M rows (FP64 /
// mixed ms per solve): 0 -> 117.2 / 72.4, 512 -> 116.1 / 71.5, 1024 -> 117.3 /
// 71.9, 2048 and more -> 120.2 / 72.7-75.4 (prefetched lines evicted before use).
constexpr int kL2PrefetchRows = 512;
static int l2_prefetch_rows() {
    static const int rows = [] {
        const char* v = getenv("CLOWNS_L2_PREFETCH");
        return v ? std::max(0, atoi(v)) : kL2PrefetchRows;
    }();
    return rows;
}

template <typename T>
static Eng<T> eng_bind(void* work, const EngLayout& L) {
    char* b = (char*)work;
    Eng<T> E;
    E.NV = L.NV;
    E.M = L.M;
    E.nblk = L.nblk;
    E.n1 = L.n1;
    E.blk_member = (const int*)(b + L.o_blk_member);
    E.blk_rows = (const int*)(b + L.o_blk_rows);
    E.mem_off = (const int*)(b + L.o_mem_off);
    E.mem_n = (const int*)(b + L.o_mem_n);
    E.mem_nblk = (const int*)(b + L.o_mem_nblk);
    E.mem_blk0 = (const int*)(b + L.o_mem_blk0);
    E.ticket = (unsigned*)(b + L.o_ticket);
    E.mem_grp0 = (const int*)(b + L.o_mem_grp0);
    E.mem_ngrp = (const int*)(b + L.o_mem_ngrp);
    E.gticket = (unsigned*)(b + L.o_gticket);
    E.gpartials = (double*)(b + L.o_gpartials);
    E.ctrl = (int*)(b + L.o_ctrl);
    E.in = (const MemberIn*)(b + L.o_in);
    E.S = (MemberScalars*)(b + L.o_S);
    E.partials = (double*)(b + L.o_partials);
    E.al = (T*)(b + L.o_al);
    E.ll = (int*)(b + L.o_ll);
    E.d = (T*)(b + L.o_d);
    T* v[8];
    for (int i = 0; i < 8; i++) v[i] = (T*)(b + L.o_vec[i]);
    E.r = v[0]; E.p = v[1]; E.r0 = v[2]; E.q = v[3]; E.e = v[4]; E.v = v[5]; E.t = v[6]; E.xi = v[7];
    if (L.mixed) {
        E.W = (double*)(b + L.o_W);
        E.x64 = (double*)(b + L.o_x64);
        E.r64 = (double*)(b + L.o_r64);
        E.s64 = (double*)(b + L.o_s64);
        E.t64 = (double*)(b + L.o_t64);
    } else {
        E.W = E.x64 = E.r64 = E.s64 = E.t64 = nullptr;
    }
    E.wave = L.wave ? (WaveCtl*)(b + L.o_wave) : nullptr;
    for (int k = 0; k < kWaveBufs; k++) E.w[k] = L.wave ? (T*)(b + L.o_wbuf[k]) : nullptr;
    E.baltab = nullptr;       // set once the launch sizes are uploaded (upload_bal_tables)
    E.nl = 6;                 // set by the solve from its members' NL
    E.abort = &((GridBar*)(b + L.o_bar))->abort;
    E.keep = l2_keep_cols(L.NV, L.tsize);
    E.pf = l2_prefetch_rows();
    E.balg = L.o_balg ? (const int*)(b + L.o_balg) : nullptr;
    return E;
}

// Reduction groups: member m's groups are mem_grp0[m] .. mem_grp0[m] +
// mem_ngrp[m] - 1 (kGroupChunks chunks of 128 rows each).
static void fill_groups(int M, const int* n, int* mem_grp0, int* mem_ngrp) {
    int g = 0;
    for (int m = 0; m < M; m++) {
        mem_grp0[m] = g;
        mem_ngrp[m] = member_groups(n[m]);
        g += mem_ngrp[m];
    }
}

// Upload the member tables (static for a given layout) and the input table.
static int eng_upload_tables(void* work, const EngLayout& L, const int* n, const MemberIn* ins,
                             cudaStream_t s) {
    const int M = L.M;
    std::vector<int> blk_member(L.nblk, -1), blk_rows(L.nblk, 0), off(M), nn(M), nblk(M), blk0(M);
    long o = 0;
    for (int m = 0; m < M; m++) {
        off[m] = (int)o;
        nn[m] = n[m];
        blk0[m] = (int)(o / kTile);
        nblk[m] = (n[m] + kTile - 1) / kTile;
        const long R = (long)align_up((size_t)n[m] + 1, kTile);
        for (long b = o / kTile; b < (o + R) / kTile; b++) {
            blk_member[b] = m;
            long rows = n[m] - (b * kTile - o);
            blk_rows[b] = (int)std::max(0L, std::min((long)kTile, rows));
        }
        o += R;
    }
    std::vector<int> mem_grp0(M), mem_ngrp(M);
    fill_groups(M, n, mem_grp0.data(), mem_ngrp.data());
    std::vector<unsigned> zeros(std::max(M, L.ngrp), 0u);
    char* b = (char*)work;
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_blk_member, blk_member.data(), sizeof(int) * L.nblk, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_blk_rows, blk_rows.data(), sizeof(int) * L.nblk, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_off, off.data(), sizeof(int) * M, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_n, nn.data(), sizeof(int) * M, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_nblk, nblk.data(), sizeof(int) * M, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_blk0, blk0.data(), sizeof(int) * M, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_ticket, zeros.data(), sizeof(unsigned) * M, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_grp0, mem_grp0.data(), sizeof(int) * M, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_ngrp, mem_ngrp.data(), sizeof(int) * M, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_gticket, zeros.data(), sizeof(unsigned) * L.ngrp, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_in, ins, sizeof(MemberIn) * M, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    return CLOWNS_OK;
}

// ---------------------------------------------------------------------------
// Launch shapes (autotuned per row-space size and precision)

struct Shape {
    int block = kStepBlock;
    int grid = 0;   // 0: one block per tile
    int fuse = 1;   // LDUSUB sweeps 1-2 and 3-4 as fused pairs (else four single sweeps)
    int rblock = kStepBlock;   // threads per tile of the dot-product kernels (64: 8 rows per thread)
    int bal = 0;    // single systems: balanced one-wave kernels with bal rows per thread per step (4 or 8)
    int stg = 0;    // FP32 single systems, balanced at 4 rows: AXSUB with its streams staged by bulk copies
};


static int grid_of(const Shape& sh, int nblk) { return sh.grid > 0 ? std::min(sh.grid, nblk) : nblk; }

template <typename T>
static void launch_apply(const Eng<T>& E, const Shape& sh, const T* in, T* out, T* tmp, int mode,
                         cudaStream_t s) {
    const int g = grid_of(sh, E.nblk), b = sh.block;
    k_eng_axsub<T><<<g, b, 0, s>>>(E, in, tmp);
    k_eng_sweep2<T><<<g, b, 0, s>>>(E, 0, tmp, out);
    k_eng_sweep2<T><<<g, b, 0, s>>>(E, 2, out, tmp);
    if (mode == 0) k_eng_sweep56<T, 0><<<g, b, 0, s>>>(E, tmp, out);
    if (mode == 1) k_eng_sweep56<T, 1><<<g, b, 0, s>>>(E, tmp, out);
    if (mode == 2) k_eng_sweep56<T, 2><<<g, b, 0, s>>>(E, tmp, out);
}

template <typename T>
static void launch_ldusub_inplace(const Eng<T>& E, const Shape& sh, T* vec, T* a, T* bb, cudaStream_t s) {
    const int g = grid_of(sh, E.nblk), b = sh.block;
    k_eng_sweep2<T><<<g, b, 0, s>>>(E, 0, vec, a);
    k_eng_sweep2<T><<<g, b, 0, s>>>(E, 2, a, bb);
    k_eng_sweep56<T, 0><<<g, b, 0, s>>>(E, bb, vec);
}

template <typename T>
static void launch_iteration(const Eng<T>& E, const Shape& sh, cudaStream_t s) {
    const int g = grid_of(sh, E.nblk), b = sh.block;
    launch_apply(E, sh, E.p, E.q, E.t, 1, s);     // q = PM A p ; RQ ; ALP
    k_eng_eupdate<T><<<g, b, 0, s>>>(E);          // e = r - ALP q
    launch_apply(E, sh, E.e, E.v, E.t, 2, s);     // v = PM A e ; AMU
    k_eng_xrupdate<T><<<g, b, 0, s>>>(E);         // x, r ; RN, C1 ; stop tests
    k_eng_pupdate<T><<<g, b, 0, s>>>(E);          // p
}

// PM r64 in place (FP64 vectors), last sweep with the member norm phase
template <typename T, int PHASE>
static void launch_ldusub64(const Eng<T>& E, const Shape& sh, double inner_tol, int inner_max, cudaStream_t s) {
    const int g = grid_of(sh, E.nblk), b = sh.block;
    k_mx_sweep<T><<<g, b, 0, s>>>(E, 0, E.r64, E.s64);
    k_mx_sweep<T><<<g, b, 0, s>>>(E, 1, E.s64, E.t64);
    k_mx_sweep<T><<<g, b, 0, s>>>(E, 2, E.t64, E.s64);
    k_mx_sweep<T><<<g, b, 0, s>>>(E, 3, E.s64, E.t64);
    k_mx_sweep56<T, PHASE><<<g, b, 0, s>>>(E, E.t64, E.r64, inner_tol, inner_max);
}

// ---------------------------------------------------------------------------
// The iteration loop, executed one of three ways (the autotuner times them on
// the actual row space and keeps the fastest):
//   graph:      a CUDA graph whose WHILE node repeats the iteration's kernels,
//               chained by programmatic dependent launch (dynamic scheduling,
//               full occupancy, launch latency overlapped with the previous
//               kernel's tail), with fused or single LDUSUB sweep pairs;
//   persistent: one cooperative launch of k_eng_loop; phases separated by grid
//               barriers (no launch gaps, static tile assignment);
//   wavefront:  one cooperative launch of k_eng_wave (single systems); (stage,
//               tile) items ordered by gather reach, per-chunk completion
//               counters instead of phase-wide barriers.

struct LoopShape {
    int block = kStepBlock;
    int grid = 0;
    int minb = 8;     // register budget of the loop kernel: 8 -> 32, 4 -> 64 registers
    int graph = 0;    // 1: CUDA graph; 2: host-launched kernels; 3: wavefront kernel
    int wk = 1;       // wavefront: tiles per item
    int wslack = 3;   // wavefront: slack rounds
    int fuse = 1;     // graph / host launches: fused sweep pairs
    int rblock = kStepBlock;   // graph / host launches: block of the dot-product kernels
    int bal = 0;      // graph / host launches, single systems: balanced kernels, rows per thread (4, 8)
    int stg = 0;      // with bal = 4, FP32 single systems: the staged AXSUB (k_bal_axsub_stg)
};

// CLOWNS_LOOP_MODE=graph|persistent|launch|wave forces one execution of the loop
// (with graph and launch, CLOWNS_SWEEP_FUSE=0 selects the four single sweeps and,
// for single systems, CLOWNS_BALANCED_ROWS=4|8 the balanced one-wave kernels)
// ("launch": the iteration's kernels launched from the host, eight iterations
// between polls of the stop flags -- the same kernels, visible one by one to a
// profiler); unset or "auto": the autotuner decides.
static int forced_loop_mode() {
    const char* v = getenv("CLOWNS_LOOP_MODE");
    if (!v || !*v || !strcmp(v, "auto")) return -1;
    if (!strcmp(v, "persistent")) return 0;
    if (!strcmp(v, "graph")) return 1;
    if (!strcmp(v, "launch")) return 2;
    if (!strcmp(v, "wave")) return 3;
    return -1;
}

template <typename T>
static const void* loop_fn(int minb) {
    return minb == 4 ? (const void*)k_eng_loop<T, 4> : (const void*)k_eng_loop<T, 8>;
}

template <typename T>
static const void* wave_fn(int minb) {
    return minb == 12 ? (const void*)k_eng_wave<T, 12> : (const void*)k_eng_wave<T, 8>;
}

static std::mutex g_loop_mu;
// (row space, precision, wave loop available, forced execution or -1): a forced
// execution is tuned among its own shapes and never served an automatic pick.
static std::map<std::tuple<long, int, int, int>, LoopShape> g_loop_shapes;

template <typename T>
static int loop_max_grid(int block, int minb, int* out, bool wave = false) {
    int per_sm = 0, dev = 0, sms = 0;
    CLOWNS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wave ? wave_fn<T>(minb) : loop_fn<T>(minb),
                                                                  block, 0));
    CLOWNS_CUDA_TRY(cudaGetDevice(&dev));
    CLOWNS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    *out = per_sm * sms;
    return CLOWNS_OK;
}

// Kernel launch with optional programmatic serialization (captured as a
// programmatic edge inside a graph).
template <typename... KArgs, typename... Args>
static void klaunch_smem(bool pdl, void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t s,
                         Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    if (pdl) {
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
    }
    cudaLaunchKernelEx(&cfg, kern, args...);
}
template <typename... KArgs, typename... Args>
static void klaunch(bool pdl, void (*kern)(KArgs...), int grid, int block, cudaStream_t s, Args... args) {
    klaunch_smem(pdl, kern, grid, block, 0, s, args...);
}

template <typename T>
static void g_apply(bool pdl, const Eng<T>& E, const Shape& sh, const T* in, T* out, T* tmp, int mode,
                    cudaStream_t s) {
    const int g = grid_of(sh, E.nblk), b = sh.block;
    klaunch(pdl, k_eng_axsub<T>, g, b, s, E, in, tmp);
    if (sh.fuse) {
        klaunch(pdl, k_eng_sweep2<T>, g, b, s, E, 0, (const T*)tmp, out);
        klaunch(pdl, k_eng_sweep2<T>, g, b, s, E, 2, (const T*)out, tmp);
    } else {
        klaunch(pdl, k_eng_sweep<T>, g, b, s, E, 0, (const T*)tmp, out);
        klaunch(pdl, k_eng_sweep<T>, g, b, s, E, 1, (const T*)out, tmp);
        klaunch(pdl, k_eng_sweep<T>, g, b, s, E, 2, (const T*)tmp, out);
        klaunch(pdl, k_eng_sweep<T>, g, b, s, E, 3, (const T*)out, tmp);
    }
    if (mode == 0) klaunch(pdl, k_eng_sweep56<T, 0>, g, b, s, E, (const T*)tmp, out);
    if (mode == 1) klaunch(pdl, k_eng_sweep56<T, 1>, g, sh.rblock, s, E, (const T*)tmp, out);
    if (mode == 2) klaunch(pdl, k_eng_sweep56<T, 2>, g, sh.rblock, s, E, (const T*)tmp, out);
}

// One wave of a balanced kernel: its resident blocks per SM x SMs, at most one
// block per tile (the reduction partials hold two values per tile).
template <typename K>
static int bal_grid(K kern, int nblk) {
    int per_sm = 0, dev = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kEngBlock, 0) != cudaSuccess ||
        cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 1;
        sms = kNumSMs;
    }
    return std::max(1, std::min(std::max(1, per_sm) * sms, nblk));
}

struct BalGrids {
    int ax, sw, s2, r1, r2, eu, xr, pu;
};

// One wave of the staged AXSUB (its dynamic shared memory raised once, before
// any capture; 0 if the device refuses it, and the tuner then leaves it out).
template <int NL>
static int stg_grid() {
    static const int g = [] {
        if (cudaFuncSetAttribute(k_bal_axsub_stg<NL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kStgSmem<NL>) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        int per_sm = 0, dev = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bal_axsub_stg<NL>, kEngBlock, kStgSmem<NL>) !=
                cudaSuccess ||
            cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || per_sm < 1) {
            cudaGetLastError();
            return 0;
        }
        return per_sm * sms;
    }();
    return g;
}

// The balanced kernels' one-wave grids (queried once; before any capture)
template <typename T, int R>
static const BalGrids& bal_grids() {
    static const BalGrids g = {bal_grid(k_bal_axsub<T, R, 6>, INT_MAX), bal_grid(k_bal_sweep<T, R>, INT_MAX),
                               bal_grid(k_bal_sweep2<T, R>, INT_MAX), bal_grid(k_bal_sweep56<T, 1, R, 6>, INT_MAX),
                               bal_grid(k_bal_sweep56<T, 2, R, 6>, INT_MAX), bal_grid(k_bal_eupdate<T, R>, INT_MAX),
                               bal_grid(k_bal_xrupdate<T, R>, INT_MAX), bal_grid(k_bal_pupdate<T, R>, INT_MAX)};
    return g;
}

template <typename T>
static void prepare_bal(int bal, int stg) {
    if (bal == 8) bal_grids<T, 8>();
    else if (bal) bal_grids<T, 4>();
    if (stg) {
        stg_grid<6>();
        stg_grid<4>();
    }
}

// Kernel kinds of the balanced iteration, in the order of BalGrids and of the
// ensembles' block tables (table of rows-per-thread R and kind k at index
// (R == 8 ? 8 : 0) + k).
enum BalKind { kBalAx, kBalSw, kBalS2, kBalR1, kBalR2, kBalEu, kBalXr, kBalPu, kBalKinds };

static int bal_grid_of(const BalGrids& g, int kind) {
    const int v[kBalKinds] = {g.ax, g.sw, g.s2, g.r1, g.r2, g.eu, g.xr, g.pu};
    return v[kind];
}

// Ensembles: the blocks of each balanced launch (both rows-per-thread settings,
// every kernel kind), which the block tables are built for on the device
// (bal_rebuild: before each loop, and by the loop guard whenever members
// stop).  *ok is false (nothing uploaded) when a launch has fewer blocks than
// members: the ensemble then keeps the tile kernels.
template <typename T>
static int upload_bal_tables(void* work, const EngLayout& L, cudaStream_t s, bool* ok) {
    *ok = false;
    const int M = L.M;
    if (M <= 1 || !L.o_baltab) return CLOWNS_OK;
    int g16[16];
    for (int ri = 0; ri < 2; ri++) {
        const BalGrids& g = ri ? bal_grids<T, 8>() : bal_grids<T, 4>();
        for (int k = 0; k < kBalKinds; k++) {
            const int G = std::min(bal_grid_of(g, k), L.nblk);
            if (G < M || G > kBalTabMax) return CLOWNS_OK;
            g16[ri * 8 + k] = G;
        }
    }
    CLOWNS_CUDA_TRY(cudaMemcpyAsync((char*)work + L.o_balg, g16, sizeof(g16), cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    *ok = true;
    return CLOWNS_OK;
}

template <typename T, int R, int NL>
static void g_iteration_bal(bool pdl, const Eng<T>& E, const Shape& sh, cudaStream_t s) {
    const int B = kEngBlock, n = E.nblk;
    const BalGrids& G = bal_grids<T, R>();
    auto grid = [&](int k) { return std::min(bal_grid_of(G, k), n); };
    auto tab = [&](int k) -> const BalBlock* {
        return E.M == 1 ? nullptr : E.baltab + (size_t)((R == 8 ? 8 : 0) + k) * kBalTabMax;
    };
    auto apply = [&](const T* in, T* out, int mode) {
        if constexpr (std::is_same<T, float>::value && R == 4) {
            if (sh.stg && E.M == 1 && stg_grid<NL>() > 0)
                klaunch_smem(pdl, k_bal_axsub_stg<NL>, std::min(stg_grid<NL>(), n), B, kStgSmem<NL>, s, E, in, E.t);
            else
                klaunch(pdl, k_bal_axsub<T, R, NL>, grid(kBalAx), B, s, E, tab(kBalAx), in, E.t);
        } else {
            klaunch(pdl, k_bal_axsub<T, R, NL>, grid(kBalAx), B, s, E, tab(kBalAx), in, E.t);
        }
        if (sh.fuse) {
            klaunch(pdl, k_bal_sweep2<T, R>, grid(kBalS2), B, s, E, tab(kBalS2), 0, (const T*)E.t, out);
            klaunch(pdl, k_bal_sweep2<T, R>, grid(kBalS2), B, s, E, tab(kBalS2), 2, (const T*)out, E.t);
        } else {
            klaunch(pdl, k_bal_sweep<T, R>, grid(kBalSw), B, s, E, tab(kBalSw), 0, (const T*)E.t, out);
            klaunch(pdl, k_bal_sweep<T, R>, grid(kBalSw), B, s, E, tab(kBalSw), 1, (const T*)out, E.t);
            klaunch(pdl, k_bal_sweep<T, R>, grid(kBalSw), B, s, E, tab(kBalSw), 2, (const T*)E.t, out);
            klaunch(pdl, k_bal_sweep<T, R>, grid(kBalSw), B, s, E, tab(kBalSw), 3, (const T*)out, E.t);
        }
        if (mode == 1) klaunch(pdl, k_bal_sweep56<T, 1, R, NL>, grid(kBalR1), B, s, E, tab(kBalR1), (const T*)E.t, out);
        else klaunch(pdl, k_bal_sweep56<T, 2, R, NL>, grid(kBalR2), B, s, E, tab(kBalR2), (const T*)E.t, out);
    };
    apply((const T*)E.p, E.q, 1);                                                    // q = PM A p ; RQ ; ALP
    klaunch(pdl, k_bal_eupdate<T, R>, grid(kBalEu), B, s, E, tab(kBalEu));          // e = r - ALP q
    apply((const T*)E.e, E.v, 2);                                                    // v = PM A e ; AMU
    klaunch(pdl, k_bal_xrupdate<T, R>, grid(kBalXr), B, s, E, tab(kBalXr));         // x, r ; RN, C1 ; stop tests
    klaunch(pdl, k_bal_pupdate<T, R>, grid(kBalPu), B, s, E, tab(kBalPu));          // p
}

// Balanced kernels serve single systems, and ensembles whose tables are uploaded.
template <typename T>
static bool bal_usable(const Eng<T>& E) { return E.M == 1 || E.baltab != nullptr; }

// The staged AXSUB serves FP32 single systems on the balanced kernels at 4 rows
// per thread (its grid is its own, so ensembles' block tables do not fit it).
template <typename T>
static bool stg_usable(const Eng<T>& E, int bal) {
    if constexpr (std::is_same<T, float>::value)
        return E.M == 1 && bal == 4 && (E.nl == 4 ? stg_grid<4>() : stg_grid<6>()) > 0;
    else
        return false;
}

template <typename T>
static void g_iteration(bool pdl, const Eng<T>& E, const Shape& sh, cudaStream_t s) {
    if (sh.bal && bal_usable(E)) {
        if (E.nl == 4) {
            if (sh.bal == 8) g_iteration_bal<T, 8, 4>(pdl, E, sh, s);
            else g_iteration_bal<T, 4, 4>(pdl, E, sh, s);
        } else {
            if (sh.bal == 8) g_iteration_bal<T, 8, 6>(pdl, E, sh, s);
            else g_iteration_bal<T, 4, 6>(pdl, E, sh, s);
        }
        return;
    }
    const int g = grid_of(sh, E.nblk), b = sh.block;
    g_apply(pdl, E, sh, (const T*)E.p, E.q, E.t, 1, s);
    klaunch(pdl, k_eng_eupdate<T>, g, b, s, E);
    g_apply(pdl, E, sh, (const T*)E.e, E.v, E.t, 2, s);
    klaunch(pdl, k_eng_xrupdate<T>, g, sh.rblock, s, E);
    klaunch(pdl, k_eng_pupdate<T>, g, b, s, E);
}

// Graph cache: one instantiated loop graph per engine state and kernel shape.
// The captured kernels take the Eng struct by value -- its row counts, member
// tables and workspace pointers -- so the key holds all of its fields: two
// systems of the same row space but different sizes (or ensembles with
// different members) must not share a graph.
struct GraphKey {
    std::string eng;
    int prec, fuse, rblock, bal, stg;
    bool operator<(const GraphKey& o) const {
        return std::tie(eng, prec, fuse, rblock, bal, stg) < std::tie(o.eng, o.prec, o.fuse, o.rblock, o.bal, o.stg);
    }
};

// Every field of E, field by field (no padding bytes).
template <typename T>
static std::string eng_key(const Eng<T>& E) {
    std::string k;
    auto put = [&](const auto& v) { k.append((const char*)&v, sizeof(v)); };
    put(E.NV); put(E.M); put(E.nblk); put(E.n1); put(E.nl); put(E.pf); put(E.abort); put(E.keep);
    put(E.al); put(E.ll); put(E.d); put(E.r); put(E.p); put(E.r0); put(E.q); put(E.e); put(E.v); put(E.t);
    put(E.xi); put(E.W); put(E.x64); put(E.r64); put(E.s64); put(E.t64);
    put(E.blk_member); put(E.blk_rows); put(E.mem_off); put(E.mem_n); put(E.mem_nblk); put(E.mem_blk0);
    put(E.mem_grp0); put(E.mem_ngrp); put(E.gticket); put(E.gpartials);
    for (int i = 0; i < kWaveBufs; i++) put(E.w[i]);
    put(E.wave); put(E.in); put(E.S); put(E.partials); put(E.ticket); put(E.ctrl); put(E.baltab); put(E.balg);
    return k;
}
static std::mutex g_graph_mu;
static std::map<GraphKey, cudaGraphExec_t> g_graphs;
static cudaStream_t g_cap = nullptr;

void release_all_graphs() {
    std::lock_guard<std::mutex> lk(g_graph_mu);
    for (auto& kv : g_graphs) cudaGraphExecDestroy(kv.second);
    g_graphs.clear();
}

// WHILE { iteration ; guard } captured into a fresh graph
template <typename T>
static int build_loop_graph(const Eng<T>& E, bool pdl, int fuse, int rblock, int bal, int stg, cudaGraphExec_t* out) {
    if (!g_cap) CLOWNS_CUDA_TRY(cudaStreamCreateWithFlags(&g_cap, cudaStreamNonBlocking));
    cudaGraph_t graph;
    CLOWNS_CUDA_TRY(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle h;
    CLOWNS_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode;
    CLOWNS_CUDA_TRY(cudaGraphAddNode(&cnode, graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    prepare_bal<T>(bal, stg);
    CLOWNS_CUDA_TRY(cudaStreamBeginCaptureToGraph(g_cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    Shape sh;
    sh.fuse = fuse;
    sh.rblock = rblock;
    sh.bal = bal;
    sh.stg = stg;
    g_iteration(pdl, E, sh, g_cap);
    BalBlock* tabs = bal && E.M > 1 && E.baltab ? (BalBlock*)E.baltab : nullptr;
    klaunch(pdl, k_eng_guard, 1, 256, g_cap, E.S, E.M, E.ctrl, h, (const int*)E.mem_n, tabs, E.balg);
    cudaGraph_t captured;
    cudaError_t ec = cudaStreamEndCapture(g_cap, &captured);
    if (ec != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(graph);
        set_last_error(ec, "capture of the iteration graph", __FILE__, __LINE__);
        return CLOWNS_ERR_CUDA;
    }
    cudaGraphExec_t ex;
    cudaError_t ei = cudaGraphInstantiate(&ex, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        cudaGetLastError();
        set_last_error(ei, "instantiation of the iteration graph", __FILE__, __LINE__);
        return CLOWNS_ERR_CUDA;
    }
    *out = ex;
    return CLOWNS_OK;
}

template <typename T>
static int loop_graph(const Eng<T>& E, const void* work, int prec, int fuse, int rblock, int bal, int stg,
                      cudaGraphExec_t* out) {
    std::lock_guard<std::mutex> lk(g_graph_mu);
    (void)work;
    GraphKey key{eng_key(E), prec, fuse, rblock, bal, stg};
    auto it = g_graphs.find(key);
    if (it != g_graphs.end()) { *out = it->second; return CLOWNS_OK; }
    cudaGraphExec_t ex;
    int rc = build_loop_graph(E, true, fuse, rblock, bal, stg, &ex);         // programmatic edges
    if (rc) rc = build_loop_graph(E, false, fuse, rblock, bal, stg, &ex);    // plain edges if refused
    if (rc) return rc;
    if (g_graphs.size() >= 64) {
        cudaGraphExecDestroy(g_graphs.begin()->second);
        g_graphs.erase(g_graphs.begin());
    }
    g_graphs[key] = ex;
    *out = ex;
    return CLOWNS_OK;
}

// Kernels the calling thread's last solve launched (host launches plus the
// kernel nodes executed inside loop graphs).
static thread_local long t_launches = 0;
// Kernels of one iteration: two operator applications (4 with fused sweep
// pairs, else 6) + 3 vector updates; a graph body adds the loop guard.
static int iter_kernels(int fuse) { return fuse ? 11 : 15; }

// Kernel launches of one run_loop call, given the loop bodies it executed.
static long loop_launches(const LoopShape& sh, long bodies) {
    if (sh.graph == 1) return bodies * (iter_kernels(sh.fuse) + 1);
    if (sh.graph == 2) return bodies * iter_kernels(sh.fuse);
    return 1;
}

// Test hook of the bounded device waits (clowns_test_arm_wait_timeout): the
// next solve whose loop runs as one cooperative kernel gives every wait
// `limit` polls and makes block `absent` leave without arriving.  One use.
struct WaitFault {
    long limit = kBarSpinLimit;
    int absent = -1;
    bool armed = false;
};
static std::mutex g_fault_mu;
static WaitFault g_fault;

void engine_arm_wait_fault(long limit, int absent) {
    std::lock_guard<std::mutex> lk(g_fault_mu);
    g_fault.limit = limit;
    g_fault.absent = absent;
    g_fault.armed = true;
}

// Wait parameters of a cooperative launch: the armed fault (once) when `take`.
static void wait_params(bool take, long* limit, int* absent) {
    *limit = kBarSpinLimit;
    *absent = -1;
    if (!take) return;
    std::lock_guard<std::mutex> lk(g_fault_mu);
    if (!g_fault.armed) return;
    *limit = g_fault.limit;
    *absent = g_fault.absent;
    g_fault = WaitFault();
}

// take_fault: this run is a solve's (not a tuning trial's), so an armed wait
// fault applies to it.
template <typename T>
static int run_loop(Eng<T> E, const void* work, GridBar* gb, int prec, const LoopShape& sh, cudaStream_t s,
                    bool take_fault = false) {
    TraceRange trace_range_("iteration loop");
    if (sh.bal && E.M > 1 && E.baltab && (sh.graph == 1 || sh.graph == 2)) {
        // ensembles on the balanced kernels: block tables over the members that iterate
        k_bal_rebuild<<<1, kBalScanThreads, 0, s>>>(E.S, E.M, E.mem_n, (BalBlock*)E.baltab, E.balg, E.ctrl + 4);
        CLOWNS_CUDA_TRY(cudaGetLastError());
        t_launches += 1;
    }
    if (sh.graph == 2) {
        CLOWNS_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBar), s));
        Shape ksh;
        ksh.fuse = sh.fuse;
        ksh.rblock = sh.rblock;
        ksh.bal = sh.bal;
        ksh.stg = sh.stg;
        prepare_bal<T>(sh.bal, sh.stg);
        int cap = 0;
        CLOWNS_CUDA_TRY(cudaMemcpyAsync(&cap, E.ctrl + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
        CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
        std::vector<MemberScalars> h(E.M);
        for (long body = 0; body <= (long)cap + 16; body += 8) {
            for (int k = 0; k < 8; k++) g_iteration(false, E, ksh, s);
            CLOWNS_CUDA_TRY(cudaGetLastError());
            CLOWNS_CUDA_TRY(cudaMemcpyAsync(h.data(), E.S, sizeof(MemberScalars) * E.M, cudaMemcpyDeviceToHost, s));
            CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
            bool any = false;
            for (int m = 0; m < E.M; m++) any = any || !h[m].done;
            if (!any) {
                t_launches += loop_launches(sh, body + 8);
                return CLOWNS_OK;
            }
        }
        set_last_error_msg("pcgpme: stop flags not raised after ITER iterations");
        return CLOWNS_ERR_NOCONV;
    }
    if (sh.graph == 3) {
        if (!E.wave || E.M != 1) {
            set_last_error_msg("pcgpme: the wavefront loop serves single systems only");
            return CLOWNS_ERR_ARG;
        }
        const int nchunk = (E.nblk + kWaveChunk - 1) / kWaveChunk;
        CLOWNS_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBar), s));
        CLOWNS_CUDA_TRY(cudaMemsetAsync(&E.wave->alp, 0, 3 * sizeof(unsigned), s));
        CLOWNS_CUDA_TRY(cudaMemsetAsync(E.wave + 1, 0, sizeof(unsigned) * 12 * (size_t)nchunk, s));
        int K = sh.wk, slack = sh.wslack;
        long lim;
        int absent;
        wait_params(take_fault, &lim, &absent);
        void* args[] = {(void*)&E, (void*)&gb, (void*)&K, (void*)&slack, (void*)&lim, (void*)&absent};
        CLOWNS_CUDA_TRY(cudaLaunchCooperativeKernel(wave_fn<T>(sh.minb), dim3(sh.grid), dim3(kStepBlock), args, 0, s));
        t_launches += 1;
        return CLOWNS_OK;
    }
    if (sh.graph) {
        cudaGraphExec_t ex;
        int rc = loop_graph(E, work, prec, sh.fuse, sh.rblock, sh.bal, sh.stg, &ex);
        if (rc) return rc;
        CLOWNS_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBar), s));
        CLOWNS_CUDA_TRY(cudaGraphLaunch(ex, s));
        return CLOWNS_OK;     // bodies are counted from ctrl[0] + ctrl[2] after the solve
    }
    int grid = std::max(1, std::min(sh.grid, E.nblk));
    CLOWNS_CUDA_TRY(cudaMemsetAsync(gb, 0, sizeof(GridBar), s));
    int init = 0;
    long lim;
    int absent;
    wait_params(take_fault, &lim, &absent);
    void* args[] = {(void*)&E, (void*)&gb, (void*)&init, (void*)&lim, (void*)&absent};
    CLOWNS_CUDA_TRY(cudaLaunchCooperativeKernel(loop_fn<T>(sh.minb), dim3(grid), dim3(sh.block), args, 0, s));
    t_launches += 1;
    return CLOWNS_OK;
}

static int check_abort(GridBar* gb, cudaStream_t s) {
    int abort = 0;
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(&abort, &gb->abort, sizeof(int), cudaMemcpyDeviceToHost, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    if (abort) {
        set_last_error_msg("pcgpme: a bounded device wait (grid barrier or staged copy) timed out; the solve was abandoned");
        return CLOWNS_ERR_NOCONV;
    }
    return CLOWNS_OK;
}

// Autotuner: time kTuneIters iterations of the loop for each candidate -- the
// wavefront kernel, the persistent kernel, the graph of tile kernels with fused
// or single sweep pairs, and the graph of balanced kernels -- on the actual row
// space, in four rounds over all candidates (the first warms up and builds the
// graphs); cache, per (row-space size, precision), the first candidate whose
// best-of-three time is within 1 % of the fastest.
// `prime` re-creates the state the loop starts from.
constexpr int kTuneIters = 24;
template <typename T, typename Prime>
static int tune_loop(Eng<T> E, const void* work, GridBar* gb, long key_nv, int key_prec, Prime prime,
                     cudaStream_t s, LoopShape* out) {
    TraceRange trace_range_("loop autotuner");
    const int forced = forced_loop_mode();
    const bool wave_ok = E.wave != nullptr && E.M == 1;
    if (forced == 1 || forced == 2) {
        LoopShape sh;
        sh.graph = forced;
        const char* fz = getenv("CLOWNS_SWEEP_FUSE");     // forced executions: fused pairs unless "0"
        sh.fuse = !(fz && !strcmp(fz, "0"));
        const char* rz = getenv("CLOWNS_REDUCE_BLOCK");   // forced executions: 128 unless "64"
        sh.rblock = (rz && !strcmp(rz, "64")) ? 64 : kStepBlock;
        const char* bz = getenv("CLOWNS_BALANCED_ROWS");  // forced executions: tile kernels unless 4 or 8
        sh.bal = !bal_usable(E) || !bz ? 0 : !strcmp(bz, "8") ? 8 : !strcmp(bz, "4") ? 4 : 0;
        const char* sz = getenv("CLOWNS_AXSUB_STAGED");   // forced: the staged FP32 AXSUB if "1"
        sh.stg = stg_usable(E, sh.bal) && sz && !strcmp(sz, "1");
        *out = sh;
        return CLOWNS_OK;
    }
    const auto key = std::make_tuple(key_nv, key_prec, (int)wave_ok, forced);
    // CLOWNS_WAVE_PARAMS="K,slack,minb,frac" pins the wavefront candidate (tuning sweeps; read on every call)
    const char* wp = getenv("CLOWNS_WAVE_PARAMS");
    int pk = 0, ps = 0, pm = 0, pf = 0;
    const bool pinned = wp && sscanf(wp, "%d,%d,%d,%d", &pk, &ps, &pm, &pf) == 4 && (pk == 1 || pk == 2 ||
                        pk == 4 || pk == 8 || pk == 16) && ps >= 0 && (pm == 8 || pm == 12) && pf >= 1 && pf <= 4;
    if (!pinned) {
        std::lock_guard<std::mutex> lk(g_loop_mu);
        auto it = g_loop_shapes.find(key);
        if (it != g_loop_shapes.end()) { *out = it->second; return CLOWNS_OK; }
    }
    std::vector<LoopShape> cands;
    // Automatic tuning keeps one shape each of the wavefront and persistent
    // kernels (their other shapes never came close on 0.1-8.5 M-row systems);
    // CLOWNS_LOOP_MODE=wave|persistent times all of them.
    const bool all_shapes = forced >= 0;
    if (wave_ok && (forced < 0 || forced == 3)) {
        for (int minb : {12, 8}) {
            if (pinned && minb != pm) continue;
            if (!pinned && !all_shapes && minb != 12) continue;
            int gmax = 0;
            int rc = loop_max_grid<T>(kStepBlock, minb, &gmax, true);
            if (rc) return rc;
            for (int frac : {4, 3}) {
                if (pinned && frac != pf) continue;
                if (!pinned && !all_shapes && frac != 4) continue;
                for (int wk : {2, 1}) {
                    if (!pinned && !all_shapes && wk != 2) continue;
                    if (pinned && wk != pk) continue;
                    LoopShape sh;
                    sh.graph = 3;
                    sh.minb = minb;
                    sh.grid = std::max(1, gmax * (pinned ? pf : frac) / 4);
                    sh.wk = pinned ? pk : wk;
                    sh.wslack = pinned ? ps : 3;
                    cands.push_back(sh);
                }
            }
            if (pinned && cands.empty()) {
                LoopShape sh;
                sh.graph = 3;
                sh.minb = pm;
                sh.grid = std::max(1, gmax * pf / 4);
                sh.wk = pk;
                sh.wslack = ps;
                cands.push_back(sh);
            }
        }
    }
    if (forced < 0 || forced == 0) for (int minb : {8, 4}) {
        if (!all_shapes && minb != 8) continue;
        int gmax = 0;
        int rc = loop_max_grid<T>(kStepBlock, minb, &gmax);
        if (rc) return rc;
        for (int frac : {4, 3, 2}) {
            if (!all_shapes && frac != 4) continue;
            LoopShape sh;
            sh.block = kStepBlock;
            sh.minb = minb;
            sh.grid = std::max(1, gmax * frac / 4);
            cands.push_back(sh);
        }
    }
    if (forced < 0 || (forced == 3 && !wave_ok)) {     // forced wave: ensembles keep the graph
        // FP64 dot-product kernels may run 64 threads per tile (8 rows per
        // thread before the warp sums: half the FP64 additions per row); the
        // FP32 ones have FP32 warp sums and keep 128
        for (int fuse : {1, 0})
            for (int rb : {kStepBlock, 64}) {
                if (rb != kStepBlock && sizeof(T) != 8) continue;
                LoopShape gsh;
                gsh.graph = 1;
                gsh.fuse = fuse;
                gsh.rblock = rb;
                cands.push_back(gsh);
            }
        // the balanced one-wave kernels, 4 or 8 rows per thread per step
        if (bal_usable(E))
            for (int fuse : {1, 0})
                for (int rows : {4, 8}) {
                    LoopShape gsh;
                    gsh.graph = 1;
                    gsh.fuse = fuse;
                    gsh.bal = rows;
                    cands.push_back(gsh);
                }
        // FP32 single systems: the same with the staged AXSUB
        if (stg_usable(E, 4))
            for (int fuse : {1, 0}) {
                LoopShape gsh;
                gsh.graph = 1;
                gsh.fuse = fuse;
                gsh.bal = 4;
                gsh.stg = 1;
                cands.push_back(gsh);
            }
    }
    if (cands.empty()) {
        set_last_error_msg("pcgpme: the forced loop execution does not serve this system");
        return CLOWNS_ERR_ARG;
    }
    cudaEvent_t e0, e1;
    CLOWNS_CUDA_TRY(cudaEventCreate(&e0));
    CLOWNS_CUDA_TRY(cudaEventCreate(&e1));
    std::vector<float> best_of(cands.size(), 1e30f);
    std::vector<char> failed(cands.size(), 0);
    for (int round = 0; round < 4; round++) {
        for (size_t c = 0; c < cands.size(); c++) {
            if (failed[c]) continue;
            prime(s);
            CLOWNS_CUDA_TRY(cudaEventRecord(e0, s));
            if (run_loop(E, work, gb, key_prec, cands[c], s)) {
                cudaGetLastError();
                failed[c] = 1;
                continue;
            }
            CLOWNS_CUDA_TRY(cudaEventRecord(e1, s));
            CLOWNS_CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0.f;
            CLOWNS_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
            int rc2 = check_abort(gb, s);
            if (rc2) return rc2;
            if (round > 0) best_of[c] = std::min(best_of[c], ms);
        }
    }
    // The first candidate (in the fixed order above) within 1 % of the fastest:
    // candidates closer than the timing noise would otherwise swap from run to
    // run, and with them the summation order and the iteration count.
    float best_ms = 1e30f;
    for (size_t c = 0; c < cands.size(); c++)
        if (!failed[c]) best_ms = std::min(best_ms, best_of[c]);
    LoopShape best = cands[0];
    for (size_t c = 0; c < cands.size(); c++)
        if (!failed[c] && best_of[c] <= best_ms * 1.01f) { best = cands[c]; break; }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lk(g_loop_mu);
    g_loop_shapes[key] = best;
    *out = best;
    return CLOWNS_OK;
}

// mode: 0 persistent, 1 CUDA graph, 3 wavefront; fuse (graph): bit 0 fused sweep
// pairs, bit 1 dot-product kernels at 64 threads per tile, bit 2 balanced
// one-wave kernels (bit 3: 8 rows per thread per step, else 4), bit 4 the
// staged FP32 AXSUB
int engine_tuned_shape(long nv, int prec, int single, int* mode, int* block, int* grid, int* minb, int* fuse) {
    std::lock_guard<std::mutex> lk(g_loop_mu);
    auto it = g_loop_shapes.find(std::make_tuple(nv, prec, single, forced_loop_mode()));
    if (it == g_loop_shapes.end()) return CLOWNS_ERR_ARG;
    const LoopShape& sh = it->second;
    *mode = sh.graph;
    *block = sh.block;
    *grid = sh.graph == 1 ? 0 : sh.grid;
    *minb = sh.graph == 1 ? 0 : sh.minb;
    *fuse = sh.graph == 1 ? (sh.fuse | (sh.rblock != kStepBlock ? 2 : 0) | (sh.bal ? 4 : 0) | (sh.bal == 8 ? 8 : 0) |
                             (sh.stg ? 16 : 0))
                          : 0;
    return CLOWNS_OK;
}

long engine_row_space(int M, const int* n, int mixed) { return eng_layout(M, n, mixed).NV; }

long engine_last_launches() { return t_launches; }

double* engine_residual_ptr(void* work, int n) {
    return (double*)((char*)work + eng_layout(1, &n, 0).o_vec[0]);
}

// ---------------------------------------------------------------------------
// Solves

static void params(int n, double eps, double parm, int iter, double* eps_o, int* iter_o, double* P1, double* P2) {
    if (eps <= kTiny) eps = kSmall;                                 // pcgpme_para.F90:51
    if (iter <= 0) iter = (int)(10 * (std::sqrt((double)n) + 1));   // 52
    const double p1 = parm < 1.0 ? 4.0 : parm;                      // 56-58
    *eps_o = eps;
    *iter_o = iter;
    *P1 = p1;
    *P2 = p1 + 1.0;
}

// Per-member results; also adds the kernel nodes executed by loop graphs
// (16 per body, ctrl[0] + ctrl[2] bodies) to the launch count.
static int read_infos(void* work, const EngLayout& L, cudaStream_t s, clowns_solve_info* info, int mixed,
                      const LoopShape& sh) {
    std::vector<MemberScalars> h(L.M);
    int ctrl[8];
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(h.data(), (char*)work + L.o_S, sizeof(MemberScalars) * L.M,
                                    cudaMemcpyDeviceToHost, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(ctrl, (char*)work + L.o_ctrl, sizeof(ctrl), cudaMemcpyDeviceToHost, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    if (sh.graph == 1) t_launches += loop_launches(sh, (long)ctrl[0] + ctrl[2]);
    if (!info) return CLOWNS_OK;
    for (int m = 0; m < L.M; m++) {
        clowns_solve_info& o = info[m];
        o.eps = mixed ? h[m].ERR64 : h[m].ERR;
        o.bn = mixed ? h[m].BN64 : h[m].BN;
        o.iter = mixed ? h[m].total_iter : h[m].K;
        o.ier = h[m].bad_index ? CLOWNS_IER_ARG : h[m].ier;
        o.reason = h[m].reason;
        o.outer = mixed ? h[m].outer : 0;
    }
    return CLOWNS_OK;
}

size_t engine_workspace_bytes(int M, const int* n, int mixed) {
    if (M < 1) return 0;
    for (int m = 0; m < M; m++)
        if (n[m] < 1) return 0;
    return eng_layout(M, n, mixed).total;
}

static int check_members(int M, const MemberIn* ins, std::vector<int>& n, int* nl_out) {
    n.resize(M);
    int nl = -1;
    for (int m = 0; m < M; m++) {
        const MemberIn& in = ins[m];
        if (!in.al || !in.ll || !in.d || !in.b || !in.x || in.n < 1 || in.na < in.n || (in.nl != 6 && in.nl != 4)) {
            set_last_error_msg("pcgpme: invalid member arguments");
            return CLOWNS_ERR_ARG;
        }
        nl = std::max(nl, in.nl);          // 2DV (4) and 3D (6) members may share a batch
        n[m] = in.n;
    }
    long tot = 0;
    for (int m = 0; m < M; m++) tot += (long)align_up((size_t)n[m] + 1, kTile);
    if (tot >= (1L << 31) - kTile) {
        set_last_error_msg("pcgpme: total rows exceed the 32-bit index range");
        return CLOWNS_ERR_LIMIT;
    }
    *nl_out = nl;
    return CLOWNS_OK;
}

// Plain FP64 (reference method and stop tests) over M members: setup kernel,
// one persistent launch for PCGPME's start and its whole iteration loop, copy-out.
int engine_solve_plain(int M, const MemberIn* ins, double eps, double parm, int iter, void* work,
                       size_t work_bytes, cudaStream_t s, clowns_solve_info* info, int variant) {
    std::vector<int> n;
    int nl = 6;
    int rc = check_members(M, ins, n, &nl);
    if (rc) return rc;
    EngLayout L = eng_layout(M, n.data(), 0);
    if (!work || work_bytes < L.total) {
        set_last_error_msg("pcgpme: workspace too small");
        return CLOWNS_ERR_WORKSPACE;
    }
    int maxn = *std::max_element(n.begin(), n.end());
    double eps_r, P1, P2;
    int iter_r;
    params(maxn, eps, parm, iter, &eps_r, &iter_r, &P1, &P2);
    const int mode = variant == 2 ? 2 : 0;
    if (variant == 2) {              // PCGPME_WILL: no EPS substitution, no ITER default
        if (iter < 1) {
            set_last_error_msg("pcgpme_will: iter must be at least 1");
            return CLOWNS_ERR_ARG;
        }
        eps_r = eps;
        iter_r = iter;
    }
    rc = eng_upload_tables(work, L, n.data(), ins, s);
    if (rc) return rc;
    Eng<double> E = eng_bind<double>(work, L);
    E.nl = nl;
    bool bal_ok = false;
    rc = upload_bal_tables<double>(work, L, s, &bal_ok);
    if (rc) return rc;
    if (bal_ok) E.baltab = (const BalBlock*)((const char*)work + L.o_baltab);
    GridBar* gb = (GridBar*)((char*)work + L.o_bar);
    const int gs = std::min(L.nblk * 2, kEngMaxGrid * 4);
    auto prime = [&](cudaStream_t cs, double e, int it) {
        if (E.wave) cudaMemsetAsync(&E.wave->D, 0, sizeof(int), cs);
        k_eng_init_scalars<<<1, 256, 0, cs>>>(E.S, M, e, it, mode, E.ctrl);
        if (nl == 6) k_eng_setup<double, 6><<<gs, kEngBlock, 0, cs>>>(E, P1, P2, 0);
        else k_eng_setup<double, 4><<<gs, kEngBlock, 0, cs>>>(E, P1, P2, 0);
    };
    // PCGPME's start (b^ = PM W b, q = PM A x0, residuals) as plain launches
    const Shape ksh;
    auto start = [&](cudaStream_t cs) {
        launch_ldusub_inplace(E, ksh, E.p, E.t, E.q, cs);
        launch_apply(E, ksh, E.xi, E.q, E.t, 0, cs);
        k_eng_initres<double><<<grid_of(ksh, E.nblk), ksh.block, 0, cs>>>(E);
    };
    LoopShape sh;
    // tuning runs: kTuneIters iterations from the real start (not counted as the solve's launches)
    rc = tune_loop(E, work, gb, L.NV, 0, [&](cudaStream_t cs) { prime(cs, 1e-300, kTuneIters); start(cs); }, s, &sh);
    if (rc) return rc;
    t_launches = 0;
    prime(s, eps_r, iter_r);
    start(s);
    t_launches += 2 + 8;
    CLOWNS_CUDA_TRY(cudaGetLastError());
    rc = run_loop(E, work, gb, 0, sh, s, true);
    if (rc) return rc;
    k_eng_copy_out<double><<<gs, kEngBlock, 0, s>>>(E);
    t_launches += 1;
    CLOWNS_CUDA_TRY(cudaGetLastError());
    rc = check_abort(gb, s);
    if (rc) return rc;
    return read_infos(work, L, s, info, 0, sh);
}

// Default relative reduction per inner solve.  Short FP32 inner solves
// restarted from a fresh FP64 residual lose less to FP32 rounding than long
// ones: on 0.4-8.5 M-row beaches the optimum is flat between 1.6e-2 and 5e-2
// (six to eight sweeps to 1e-10), and 3e-2 took the least time with the
// balanced kernels (1e-4: a third more inner iterations).
constexpr double kInnerTol = 3e-2;

// Mixed precision: FP32 coefficients and Krylov vectors in the inner BiCGSTAB,
// FP64 refinement residual r = W (b - A x), FP64 norms and FP64 x accumulation.
int engine_solve_mixed(int M, const MemberIn* ins, double eps, double parm, double inner_tol,
                       int inner_max, int max_outer, void* work, size_t work_bytes, cudaStream_t s,
                       clowns_solve_info* info) {
    std::vector<int> n;
    int nl = 6;
    int rc = check_members(M, ins, n, &nl);
    if (rc) return rc;
    EngLayout L = eng_layout(M, n.data(), 1);
    if (!work || work_bytes < L.total) {
        set_last_error_msg("pcgpme_mixed: workspace too small");
        return CLOWNS_ERR_WORKSPACE;
    }
    int maxn = *std::max_element(n.begin(), n.end());
    double eps_r, P1, P2;
    int iter_r;
    params(maxn, eps, parm, 0, &eps_r, &iter_r, &P1, &P2);
    if (inner_tol <= 0) inner_tol = kInnerTol;
    if (inner_max <= 0) inner_max = 2000;
    if (max_outer <= 0) max_outer = 30;
    rc = eng_upload_tables(work, L, n.data(), ins, s);
    if (rc) return rc;
    Eng<float> E = eng_bind<float>(work, L);
    E.nl = nl;
    bool bal_ok = false;
    rc = upload_bal_tables<float>(work, L, s, &bal_ok);
    if (rc) return rc;
    if (bal_ok) E.baltab = (const BalBlock*)((const char*)work + L.o_baltab);
    GridBar* gb = (GridBar*)((char*)work + L.o_bar);
    const int gs = std::min(L.nblk * 2, kEngMaxGrid * 4);
    const Shape ksh;                               // standalone FP64 refinement kernels
    const int kg = grid_of(ksh, E.nblk);
    auto setup = [&](cudaStream_t cs) {
        if (E.wave) cudaMemsetAsync(&E.wave->D, 0, sizeof(int), cs);
        k_mixed_init_scalars<<<1, 256, 0, cs>>>(E.S, M, eps_r, max_outer, E.ctrl);
        if (nl == 6) k_eng_setup<float, 6><<<gs, kEngBlock, 0, cs>>>(E, P1, P2, 1);
        else k_eng_setup<float, 4><<<gs, kEngBlock, 0, cs>>>(E, P1, P2, 1);
        launch_ldusub64<float, 0>(E, ksh, inner_tol, inner_max, cs);   // BN64 = ||PM W b||^2
    };
    // one refinement sweep up to the inner loop: residual, PM r, ERR test, inner RHS
    auto sweep_head = [&](cudaStream_t cs, double itol, int imax) {
        k_mx_reset_ctrl<<<1, 32, 0, cs>>>(E.ctrl, imax);
        k_mx_residual<float><<<kg, ksh.block, 0, cs>>>(E);
        launch_ldusub64<float, 1>(E, ksh, itol, imax, cs);
        k_mx_normalize<float><<<kg, ksh.block, 0, cs>>>(E);
    };
    LoopShape sh;
    rc = tune_loop(E, work, gb, L.NV, 1, [&](cudaStream_t cs) { setup(cs); sweep_head(cs, 1e-30, kTuneIters); },
                   s, &sh);
    if (rc) return rc;
    t_launches = 0;
    setup(s);
    t_launches += 7;
    CLOWNS_CUDA_TRY(cudaGetLastError());
    std::vector<MemberScalars> h(M);
    for (int sweep = 0; sweep <= max_outer + 1; sweep++) {
        TraceRange trace_sweep_("refinement sweep");
        sweep_head(s, inner_tol, inner_max);
        t_launches += 8;
        CLOWNS_CUDA_TRY(cudaMemcpyAsync(h.data(), E.S, sizeof(MemberScalars) * M, cudaMemcpyDeviceToHost, s));
        CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
        bool all = true;
        for (int m = 0; m < M; m++) all = all && h[m].odone;
        if (all) break;
        rc = run_loop(E, work, gb, 1, sh, s);
        if (rc) return rc;
        k_mx_update<float><<<kg, ksh.block, 0, s>>>(E);
        t_launches += 1;
        CLOWNS_CUDA_TRY(cudaGetLastError());
        rc = check_abort(gb, s);
        if (rc) return rc;
    }
    k_mx_copy_out<float><<<gs, kEngBlock, 0, s>>>(E);
    t_launches += 1;
    CLOWNS_CUDA_TRY(cudaGetLastError());
    return read_infos(work, L, s, info, 1, sh);
}

// Test hooks -------------------------------------------------------------------

int engine_setup_export(const MemberIn& in, double parm, double* al_s, int* ll_s, double* d_s, double* b_s,
                        int na_out, void* work, size_t work_bytes, cudaStream_t s) {
    std::vector<int> n;
    int nl;
    int rc = check_members(1, &in, n, &nl);
    if (rc) return rc;
    EngLayout L = eng_layout(1, n.data(), 0);
    if (!work || work_bytes < L.total) {
        set_last_error_msg("setup: workspace too small");
        return CLOWNS_ERR_WORKSPACE;
    }
    double e, P1, P2;
    int it;
    params(in.n, 0.0, parm, 0, &e, &it, &P1, &P2);
    rc = eng_upload_tables(work, L, n.data(), &in, s);
    if (rc) return rc;
    Eng<double> E = eng_bind<double>(work, L);
    k_eng_init_scalars<<<1, 32, 0, s>>>(E.S, 1, 1e-10, 1, 0, E.ctrl);
    if (nl == 6) k_eng_setup<double, 6><<<std::min(L.nblk * 4, 4096), kEngBlock, 0, s>>>(E, P1, P2, 0);
    else k_eng_setup<double, 4><<<std::min(L.nblk * 4, 4096), kEngBlock, 0, s>>>(E, P1, P2, 0);
    k_eng_export<double><<<std::min(L.nblk * 4, 4096), kEngBlock, 0, s>>>(E, al_s, ll_s, d_s, b_s, nl, na_out);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    return CLOWNS_OK;
}

__global__ void k_hook_load_x(Eng<double> E, const double* x, int n) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) E.xi[i] = x[i];
}
__global__ void k_hook_store_y(Eng<double> E, double* y, int n) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) y[i] = E.q[i];
}

int engine_apply_pm_a(const MemberIn& in, double parm, const double* x, double* y, void* work, size_t work_bytes,
                      cudaStream_t s) {
    std::vector<int> n;
    int nl;
    int rc = check_members(1, &in, n, &nl);
    if (rc) return rc;
    EngLayout L = eng_layout(1, n.data(), 0);
    if (!work || work_bytes < L.total) {
        set_last_error_msg("apply: workspace too small");
        return CLOWNS_ERR_WORKSPACE;
    }
    double e, P1, P2;
    int it;
    params(in.n, 0.0, parm, 0, &e, &it, &P1, &P2);
    rc = eng_upload_tables(work, L, n.data(), &in, s);
    if (rc) return rc;
    Eng<double> E = eng_bind<double>(work, L);
    k_eng_init_scalars<<<1, 32, 0, s>>>(E.S, 1, 1e-10, 1, 0, E.ctrl);
    const int gs = std::min(L.nblk * 4, 4096);
    if (nl == 6) k_eng_setup<double, 6><<<gs, kEngBlock, 0, s>>>(E, P1, P2, 0);
    else k_eng_setup<double, 4><<<gs, kEngBlock, 0, s>>>(E, P1, P2, 0);
    k_hook_load_x<<<gs, kEngBlock, 0, s>>>(E, x, in.n);
    Shape sh;
    launch_apply(E, sh, E.xi, E.q, E.t, 0, s);
    k_hook_store_y<<<gs, kEngBlock, 0, s>>>(E, y, in.n);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    return CLOWNS_OK;
}

}  // namespace clowns

// ---------------------------------------------------------------------------
// Allocation-free FP64 solve.
//
// For callers that cannot allocate device memory: a Fortran time loop whose
// device memory is owned by another runtime or a fixed memory budget, or a
// library that must not grow the process's allocations while a solve runs.
// The scratch space of the solve lives in one file-scope device array of fixed
// size, loaded with the library; the entry point itself calls no allocator and
// builds no CUDA graph -- it launches the same kernels as clowns_pcgpme_dev and
// polls the device stop flag every eight iterations.  The array is shared by
// every call on a device: calls that overlap on the GPU (different streams or
// host threads) race on it.  Every call re-initialises all scratch it reads.

namespace clowns {

constexpr int kStaticMaxRows = CLOWNS_STATIC_MAX_ROWS;
constexpr long kStaticNV = ((long)(kStaticMaxRows + 1) + kTile - 1) / kTile * kTile;
constexpr int kStaticMaxBlk = (int)(kStaticNV / kTile);
// matrix (6 T + 6 int + 1 T) + 8 Krylov vectors, plus tables and alignment slack
constexpr size_t kStaticBytes = (size_t)kStaticNV * (6 * 8 + 6 * 4 + 8 + 8 * 8) + 64 * 1024;
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];
static void* g_static_addr[kStaticMaxDevices];
static std::mutex g_static_mu;

// Device address of the scratch array for the current device, resolved once
// per device on the first call (the host-side name is only a stand-in).
static int static_scratch(void** out) {
    int dev = 0;
    CLOWNS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kStaticMaxDevices) {
        set_last_error_msg("pcgpme_static: device ordinal beyond the supported 64");
        return CLOWNS_ERR_LIMIT;
    }
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) {
            set_last_error(e, "cudaGetSymbolAddress(g_static_scratch)", __FILE__, __LINE__);
            return CLOWNS_ERR_CUDA;
        }
        g_static_addr[dev] = p;
    }
    *out = g_static_addr[dev];
    return CLOWNS_OK;
}

// Member tables of a single system from stack arrays (no allocation).
static int static_upload_tables(void* work, const EngLayout& L, int n, const MemberIn& in, cudaStream_t s) {
    int blk_member[kStaticMaxBlk], blk_rows[kStaticMaxBlk];
    for (int b = 0; b < L.nblk; b++) {
        blk_member[b] = 0;
        long rows = (long)n - (long)b * kTile;
        blk_rows[b] = (int)std::max(0L, std::min((long)kTile, rows));
    }
    const int off = 0, nblk = (n + kTile - 1) / kTile, blk0 = 0;
    constexpr int kStaticMaxGrp = (kStaticMaxBlk * kTileChunks + kGroupChunks - 1) / kGroupChunks;
    int mem_grp0 = 0, mem_ngrp = 0;
    const unsigned zeros[kStaticMaxGrp] = {};
    fill_groups(1, &n, &mem_grp0, &mem_ngrp);
    const unsigned zero = 0u;
    char* b = (char*)work;
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_blk_member, blk_member, sizeof(int) * L.nblk, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_blk_rows, blk_rows, sizeof(int) * L.nblk, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_off, &off, sizeof(int), cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_n, &n, sizeof(int), cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_nblk, &nblk, sizeof(int), cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_blk0, &blk0, sizeof(int), cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_ticket, &zero, sizeof(unsigned), cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_grp0, &mem_grp0, sizeof(int), cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_mem_ngrp, &mem_ngrp, sizeof(int), cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_gticket, zeros, sizeof(unsigned) * L.ngrp, cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(b + L.o_in, &in, sizeof(MemberIn), cudaMemcpyHostToDevice, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));   // stack sources must outlive the copies
    return CLOWNS_OK;
}

}  // namespace clowns

extern "C" int clowns_pcgpme_static_dev(const double* al, int nl, int na, const int* ll, const double* d, int n,
                                        const double* b, double* x, double eps, double parm, int iter, void* stream,
                                        clowns_solve_info* info) {
    clowns::TraceRange trace_range_("clowns_pcgpme_static_dev");
    using namespace clowns;
    if (n > kStaticMaxRows) {
        set_last_error_msg("pcgpme_static: n exceeds CLOWNS_STATIC_MAX_ROWS (32768 rows)");
        return CLOWNS_ERR_LIMIT;
    }
    if (!al || !ll || !d || !b || !x || n < 1 || na < n || (nl != 6 && nl != 4)) {
        set_last_error_msg("pcgpme_static: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    void* work = nullptr;
    int rc = static_scratch(&work);
    if (rc) return rc;
    EngLayout L = eng_layout(1, &n, 0, 0);
    if (L.total > kStaticBytes || L.nblk > kStaticMaxBlk) {
        set_last_error_msg("pcgpme_static: layout exceeds the static scratch");
        return CLOWNS_ERR_LIMIT;
    }
    MemberIn in;
    in.al = al; in.ll = ll; in.d = d; in.b = b; in.x = x;
    in.na = na; in.n = n; in.nl = nl; in.pad = 0;
    double eps_r, P1, P2;
    int iter_r;
    params(n, eps, parm, iter, &eps_r, &iter_r, &P1, &P2);
    std::lock_guard<std::mutex> lk(g_static_mu);
    rc = static_upload_tables(work, L, n, in, s);
    if (rc) return rc;
    Eng<double> E = eng_bind<double>(work, L);
    const Shape sh;                                 // one 256-thread block per tile
    const int g = grid_of(sh, E.nblk);
    k_eng_init_scalars<<<1, 256, 0, s>>>(E.S, 1, eps_r, iter_r, 0, E.ctrl);
    if (nl == 6) k_eng_setup<double, 6><<<4 * L.nblk, kEngBlock, 0, s>>>(E, P1, P2, 0);
    else k_eng_setup<double, 4><<<4 * L.nblk, kEngBlock, 0, s>>>(E, P1, P2, 0);
    launch_ldusub_inplace(E, sh, E.p, E.t, E.q, s);       // b^ = PM W b
    launch_apply(E, sh, E.xi, E.q, E.t, 0, s);             // q = PM A x0
    k_eng_initres<double><<<g, sh.block, 0, s>>>(E);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    // Iterations: kernels of a stopped member return at once, so batches of
    // eight between polls are exact; the stop tests cap the count at ITER.
    int done = 0;
    for (long launched = 0; !done; launched += 8) {
        for (int k = 0; k < 8; k++) launch_iteration(E, sh, s);
        CLOWNS_CUDA_TRY(cudaGetLastError());
        CLOWNS_CUDA_TRY(cudaMemcpyAsync(&done, &E.S->done, sizeof(int), cudaMemcpyDeviceToHost, s));
        CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
        if (!done && launched > (long)iter_r + 16) {
            set_last_error_msg("pcgpme_static: stop flag not raised after ITER iterations");
            return CLOWNS_ERR_NOCONV;
        }
    }
    k_eng_copy_out<double><<<4 * L.nblk, kEngBlock, 0, s>>>(E);
    MemberScalars h;
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(&h, E.S, sizeof(MemberScalars), cudaMemcpyDeviceToHost, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    if (info) {
        info->eps = h.ERR;
        info->bn = h.BN;
        info->iter = h.K;
        info->ier = h.bad_index ? CLOWNS_IER_ARG : h.ier;
        info->reason = h.reason;
        info->outer = 0;
    }
    return CLOWNS_OK;
}
