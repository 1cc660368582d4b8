// nflag.cu -- cell classification set_nflag (src2LOWNS/nfd2015.F90:7-306) on the
// GPU, NORMAL + OBJECT build.
//
// The reference is a sequence of passes over the cells, restarted whenever a
// pass removes a surface cell (goto 4 / goto 3).  Three of its loops write flags
// that later iterations of the same loop read (the second pruning loop and the
// orientation loop, nfd2015.F90:133-158 and 163-244, walked in descending list
// order).  Their serial semantics are reproduced exactly here: the decision for
// list position p depends only on decisions at positions > p, so a Jacobi
// iteration over all positions reaches the serial answer after at most
// (longest dependency chain + 1) sweeps and is detected as a fixed point.
#include <cstring>

#include "common.cuh"
#include "grid_index.cuh"
#include "trace.h"

namespace clowns {

constexpr int kNfBlock = 256;

static inline int nf_grid(long n) {
    long b = (n + kNfBlock - 1) / kNfBlock;
    if (b < 1) b = 1;
    if (b > 152L * 16) b = 152L * 16;
    return (int)b;
}

struct NfArgs {
    GridIdx g;
    int inne;
    const int* mn;
    const int* in_;
    const int* jn;
    const int* kn;
    int* nf;
    int* nfb;
    const double* fb;
    const double* a;
    const double* dx;
    const int* objno;
};

// ---- nfd2015.F90:35-59 --------------------------------------------------
__global__ void k_vof_flags(NfArgs A, const double* __restrict__ f, int* __restrict__ dec, int* imax_k) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < A.inne; t += (long)gridDim.x * blockDim.x) {
        const int nn = (int)t + 1;
        if (A.nf[nn] == -1) { dec[nn] = -1; continue; }
        const int i = A.in_[nn], j = A.jn[nn], k = A.kn[nn];
        const double fv = f[nn];
        const bool air = fv <= 1.0e-12 ||
                         (fv * A.fb[nn] < 1.0e-3 && A.nf[A.mn[A.g.mn_off(i, k - 1, j)]] == -1 &&
                          f[A.mn[A.g.mn_off(i, k + 1, j)]] == 0.0);
        dec[nn] = air ? 0 : 1;
        if (!air) {
            atomicMax(imax_k + 0, i);
            atomicMax(imax_k + 1, k);
        }
    }
}

__global__ void k_vof_apply(NfArgs A, double* __restrict__ f, const int* __restrict__ dec) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < A.inne; t += (long)gridDim.x * blockDim.x) {
        const int nn = (int)t + 1;
        const int d = dec[nn];
        if (d < 0) continue;
        A.nf[nn] = d;
        A.nfb[nn] = 0;
        if (d == 0) f[nn] = fmax(0.0, f[nn]);
    }
}

// ---- nfd2015.F90:66-102: wet cells and surface detection over the k,j,i box --
struct Box {
    int ks, kmax, js, je1, is, imax;
    long nbi, nbj, nbk, total;
    __device__ __forceinline__ void ijk(long t, int& i, int& j, int& k) const {
        i = is + (int)(t % nbi);
        long r = t / nbi;
        j = js + (int)(r % nbj);
        k = ks + (int)(r / nbj);
    }
};

__global__ void k_surface_flags(NfArgs A, Box B, int* __restrict__ wet, int* __restrict__ surf) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < B.total; t += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        B.ijk(t, i, j, k);
        const int nn = A.mn[A.g.mn_off(i, k, j)];
        const int fl = A.nf[nn];
        int w = 0, s = 0;
        if (fl >= 1) {
            w = 1;
            for (int l = 0; l < 3 && !s; l++) {
                const int p = A.mn[A.g.nbr(i, j, k, l, +1)];
                if (A.nf[p] == 0 && A.a[3L * p + l] > 0.0) s = 1;
                if (!s) {
                    const int m = A.mn[A.g.nbr(i, j, k, l, -1)];
                    if (A.nf[m] == 0 && A.a[3L * nn + l] > 0.0) s = 1;
                }
            }
        }
        wet[t] = w;
        surf[t] = s;
    }
}

__global__ void k_surface_scatter(NfArgs A, Box B, const int* __restrict__ wet, const int* __restrict__ surf,
                                  const int* __restrict__ wpos, const int* __restrict__ spos_box,
                                  int* __restrict__ fln, int* __restrict__ sfn, int* __restrict__ spos_cell) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < B.total; t += (long)gridDim.x * blockDim.x) {
        if (!wet[t]) continue;
        int i, j, k;
        B.ijk(t, i, j, k);
        const int nn = A.mn[A.g.mn_off(i, k, j)];
        fln[wpos[t]] = nn;
        if (surf[t]) {
            const int p = spos_box[t];
            sfn[p] = nn;
            spos_cell[nn] = p;
            A.nf[nn] = 2;
            A.nfb[nn] = -3;
        } else {
            A.nf[nn] = 1;
            spos_cell[nn] = -1;
        }
    }
}

// ---- nfd2015.F90:107-131: first pruning (order-independent) -------------------
__global__ void k_prune1(NfArgs A, int isfn, const int* __restrict__ sfn, int* __restrict__ rem, int* count) {
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < isfn; p += (long)gridDim.x * blockDim.x) {
        const int nn = sfn[p];
        const int i = A.in_[nn], j = A.jn[nn], k = A.kn[nn];
        int r = 0;
        if (A.nf[A.mn[A.g.mn_off(i, k - 1, j)]] != -1) {
            int keep = 0;
            for (int l = 0; l < 3 && !keep; l++) {
                if (A.nf[A.mn[A.g.nbr(i, j, k, l, +1)]] == 1) keep = 1;
                else if (A.nf[A.mn[A.g.nbr(i, j, k, l, -1)]] == 1) keep = 1;
            }
            r = !keep;
        }
        rem[p] = r;
        if (r) atomicAdd(count, 1);
    }
}

__global__ void k_remove(NfArgs A, int isfn, const int* __restrict__ sfn, const int* __restrict__ rem) {
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < isfn; p += (long)gridDim.x * blockDim.x) {
        if (rem[p]) {
            const int nn = sfn[p];
            A.nf[nn] = 0;
            A.nfb[nn] = 0;
        }
    }
}

// Flag of cell q as seen by list position p in a loop walked from the end of
// the list: cells later in the list (already visited) show their removal.
__device__ __forceinline__ int nf_seen(const NfArgs& A, int q, long p, const int* __restrict__ spos_cell,
                                       const int* __restrict__ state) {
    const int fl = A.nf[q];
    if (fl == 2) {
        const int pq = spos_cell[q];
        if (pq > p && state[pq]) return 0;
    }
    return fl;
}

// ---- nfd2015.F90:133-158: second pruning, serial semantics ---------------------
__global__ void k_prune2_sweep(NfArgs A, int isfn, const int* __restrict__ sfn, const int* __restrict__ spos_cell,
                               const int* __restrict__ st_in, int* __restrict__ st_out, int* changed) {
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < isfn; p += (long)gridDim.x * blockDim.x) {
        const int nn = sfn[p];
        const int i = A.in_[nn], j = A.jn[nn], k = A.kn[nn];
        int r = 0;
        const int below = nf_seen(A, A.mn[A.g.mn_off(i, k - 1, j)], p, spos_cell, st_in);
        const int above = nf_seen(A, A.mn[A.g.mn_off(i, k + 1, j)], p, spos_cell, st_in);
        if (!(below == -1 && above == 0)) {
            int keep = 0;
            for (int l = 0; l < 3 && !keep; l++) {
                const int pv = nf_seen(A, A.mn[A.g.nbr(i, j, k, l, +1)], p, spos_cell, st_in);
                const int mv = nf_seen(A, A.mn[A.g.nbr(i, j, k, l, -1)], p, spos_cell, st_in);
                if ((pv == 1 && mv == 0) || (mv == 1 && pv == 0)) keep = 1;
            }
            r = !keep;
        }
        st_out[p] = r;
        if (r != st_in[p]) atomicAdd(changed, 1);
    }
}

// fxx1 (nfd2015.F90:308-332)
__device__ double fxx1_dev(const NfArgs& A, const double* __restrict__ f, int ix, int ll, int i, int j, int k) {
    const GridIdx& g = A.g;
    const int lg[3] = {i, j, k};
    double r = 0.0;
    for (int l = 0; l <= 2; l++) {
        if (l == ll) continue;
        if (g.is == g.ie - 1 && l == 0) continue;
        if (g.js == g.je - 1 && l == 1) continue;
        for (int ii = -1; ii <= 1; ii++) {
            const int ci = lg[0] + ix * (ll == 0) + ii * (l == 0);
            const int ck = lg[2] + ix * (ll == 2) + ii * (l == 2);
            const int cj = lg[1] + ix * (ll == 1) + ii * (l == 1);
            const int nnc = A.mn[g.mn_off(ci, ck, cj)];
            r = __dadd_rn(r, __dmul_rn(__dmul_rn(A.dx[g.dxo(l, lg[l] + ii)], f[nnc]), A.fb[nnc]));
        }
        for (int lll = 0; lll <= 2; lll++) {
            if (lll == l || ll == lll) continue;
            r = __dmul_rn(r, A.dx[g.dxo(lll, lg[lll])]);
        }
    }
    return __dmul_rn(r, A.dx[g.dxo(ll, lg[ll] + ix)]);
}

// ---- nfd2015.F90:163-244: orientation, serial semantics ------------------------
__global__ void k_orient_sweep(NfArgs A, const double* __restrict__ f, int isfn, const int* __restrict__ sfn,
                               const int* __restrict__ spos_cell, const int* __restrict__ st_in,
                               int* __restrict__ st_out, int* __restrict__ bout, int* changed) {
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < isfn; p += (long)gridDim.x * blockDim.x) {
        const int nn = sfn[p];
        const int i = A.in_[nn], j = A.jn[nn], k = A.kn[nn];
        int ix[3] = {0, 0, 0};
        for (int l = 0; l < 3; l++) {
            const int m = A.mn[A.g.nbr(i, j, k, l, -1)], pc = A.mn[A.g.nbr(i, j, k, l, +1)];
            const int mv = nf_seen(A, m, p, spos_cell, st_in), pv = nf_seen(A, pc, p, spos_cell, st_in);
            if (mv == 1 && pv == 0 && A.a[3L * pc + l] > 0.0) ix[l] = -1;
            else if (mv == 0 && pv == 1 && A.a[3L * nn + l] > 0.0) ix[l] = 1;
        }
        if (abs(ix[0]) + abs(ix[1]) + abs(ix[2]) == 0) {
            const int below = nf_seen(A, A.mn[A.g.mn_off(i, k - 1, j)], p, spos_cell, st_in);
            const int above = nf_seen(A, A.mn[A.g.mn_off(i, k + 1, j)], p, spos_cell, st_in);
            if (below == -1 && above == 0) {
                if (A.objno[nn] != 0 || A.fb[nn] != 0.0) {
                    ix[2] = -1;
                } else {
                    for (int l = 0; l <= 1; l++) {
                        const int m = A.mn[A.g.nbr(i, j, k, l, -1)], pc = A.mn[A.g.nbr(i, j, k, l, +1)];
                        const int mv = nf_seen(A, m, p, spos_cell, st_in), pv = nf_seen(A, pc, p, spos_cell, st_in);
                        if (mv > 0 && pv == 0 && A.a[3L * pc + l] > 0.0) ix[l] = -1;
                        else if (mv == 0 && pv > 0 && A.a[3L * nn + l] > 0.0) ix[l] = 1;
                    }
                    if (abs(ix[0]) + abs(ix[1]) == 0) ix[2] = -1;
                }
            }
        }
        const int s = abs(ix[0]) + abs(ix[1]) + abs(ix[2]);
        int g = 0, b = 0;
        if (s == 1) {
            int dir = 1, best = abs(ix[0]);
            for (int l = 1; l <= 2; l++)
                if (abs(ix[l]) > best) { best = abs(ix[l]); dir = l + 1; }
            b = dir * ix[dir - 1];
        } else if (s == 0) {
            g = 1;
        } else {
            double fx[3];
            for (int l = 0; l < 3; l++) fx[l] = ix[l] == 0 ? 0.0 : fxx1_dev(A, f, ix[l], l, i, j, k);
            int dir = 1;
            double best = fx[0];
            for (int l = 1; l <= 2; l++)
                if (fx[l] > best) { best = fx[l]; dir = l + 1; }
            b = dir * ix[dir - 1];
        }
        st_out[p] = g;
        bout[p] = b;
        if (g != st_in[p]) atomicAdd(changed, 1);
    }
}

__global__ void k_orient_apply(NfArgs A, int isfn, const int* __restrict__ sfn, const int* __restrict__ st,
                               const int* __restrict__ b, int* count) {
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < isfn; p += (long)gridDim.x * blockDim.x) {
        const int nn = sfn[p];
        A.nfb[nn] = b[p];
        if (st[p]) {
            A.nf[nn] = 0;
            atomicAdd(count, 1);
        }
    }
}

__global__ void k_count_nonzero(const int* __restrict__ v, long n, int* count) {
    int c = 0;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) c += v[t] != 0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

__global__ void k_fill(int* p, long n, int v) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) p[t] = v;
}

// Workspace: box-sized flag and position arrays, the per-cell list position,
// the Jacobi state buffers and scan scratch.
struct NfWs {
    int *wet, *surf, *wpos, *spos_box, *spos_cell, *st0, *st1, *bout, *ctr;
    void* scan_tmp;
};

static size_t nf_layout(const int* dims, int inne2, NfWs* w, char* base) {
    GridIdx g = GridIdx::make(dims);
    long box = (long)(g.ie - g.is) * (g.je - g.js) * (g.ke - g.ks);
    if (box < 1) box = 1;
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = align_up(o + bytes, 256); return at; };
    size_t o_wet = take(sizeof(int) * (box + 1));
    size_t o_surf = take(sizeof(int) * (box + 1));
    size_t o_wpos = take(sizeof(int) * (box + 1));
    size_t o_spos = take(sizeof(int) * (box + 1));
    size_t o_cell = take(sizeof(int) * ((size_t)inne2 + 2));
    size_t o_st0 = take(sizeof(int) * (box + 1));
    size_t o_st1 = take(sizeof(int) * (box + 1));
    size_t o_b = take(sizeof(int) * (box + 1));
    size_t o_ctr = take(sizeof(int) * 16);
    size_t o_scan = take(scan_workspace_bytes(box + 1));
    if (w && base) {
        w->wet = (int*)(base + o_wet);
        w->surf = (int*)(base + o_surf);
        w->wpos = (int*)(base + o_wpos);
        w->spos_box = (int*)(base + o_spos);
        w->spos_cell = (int*)(base + o_cell);
        w->st0 = (int*)(base + o_st0);
        w->st1 = (int*)(base + o_st1);
        w->bout = (int*)(base + o_b);
        w->ctr = (int*)(base + o_ctr);
        w->scan_tmp = base + o_scan;
    }
    return o;
}

static int read_int(const int* dptr, cudaStream_t s, int* out) {
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(out, dptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    return CLOWNS_OK;
}

}  // namespace clowns

using namespace clowns;

extern "C" size_t clowns_set_nflag_workspace_bytes(const int* dims, int inne2) {
    if (!dims) return 0;
    return nf_layout(dims, inne2, nullptr, nullptr);
}

extern "C" int clowns_set_nflag_dev(const int* dims, int inne, int inne2, int mx2, const int* mn, const int* in_,
                                    const int* jn, const int* kn, int* nf, int* nfb, double* f, const double* fb,
                                    const double* a, const double* dx, const int* objno, int* fln, int* ifln_out,
                                    int* sfn, int* isfn_out, int* passes_out, void* work, size_t work_bytes,
                                    void* stream) {
    clowns::TraceRange trace_range_("clowns_set_nflag_dev");
    (void)mx2;
    if (!grid_dims_ok(dims) || inne < 1 || !mn || !in_ || !jn || !kn || !nf || !nfb || !f || !fb || !a || !dx || !objno ||
        !fln || !ifln_out || !sfn || !isfn_out || !work) {
        set_last_error_msg("set_nflag: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    if (work_bytes < nf_layout(dims, inne2, nullptr, nullptr)) {
        set_last_error_msg("set_nflag: workspace too small");
        return CLOWNS_ERR_WORKSPACE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    NfWs W;
    nf_layout(dims, inne2, &W, (char*)work);
    NfArgs A;
    A.g = GridIdx::make(dims);
    A.inne = inne;
    A.mn = mn; A.in_ = in_; A.jn = jn; A.kn = kn; A.nf = nf; A.nfb = nfb;
    A.fb = fb; A.a = a; A.dx = dx; A.objno = objno;

    // VOF pass; W.wet doubles as the per-cell decision array here (size >= inne2+2
    // is not guaranteed, so use spos_cell which is).
    CLOWNS_CUDA_TRY(cudaMemsetAsync(W.ctr, 0, sizeof(int) * 16, s));
    k_vof_flags<<<nf_grid(inne), kNfBlock, 0, s>>>(A, f, W.spos_cell, W.ctr);
    k_vof_apply<<<nf_grid(inne), kNfBlock, 0, s>>>(A, f, W.spos_cell);
    int ik[2];
    CLOWNS_CUDA_TRY(cudaMemcpyAsync(ik, W.ctr, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    const GridIdx& g = A.g;
    int imax = ik[0] + 1 < g.ie - 1 ? ik[0] + 1 : g.ie - 1;
    int kmax = ik[1] + 1 < g.ke - 1 ? ik[1] + 1 : g.ke - 1;
    Box B;
    B.ks = g.ks; B.kmax = kmax; B.js = g.js; B.je1 = g.je - 1; B.is = g.is; B.imax = imax;
    B.nbi = imax >= g.is ? imax - g.is + 1 : 0;
    B.nbj = g.je - g.js;
    B.nbk = kmax >= g.ks ? kmax - g.ks + 1 : 0;
    B.total = B.nbi * B.nbj * B.nbk;

    int passes = 0, ifln = 0, isfn = 0;
    const int kMaxPasses = 100000;
    for (;;) {
        if (++passes > kMaxPasses) {
            set_last_error_msg("set_nflag: classification did not settle");
            return CLOWNS_ERR_NOCONV;
        }
        ifln = 0;
        isfn = 0;
        if (B.total > 0) {
            const int gb = nf_grid(B.total);
            k_surface_flags<<<gb, kNfBlock, 0, s>>>(A, B, W.wet, W.surf);
            int rc = exclusive_scan_dev(W.wet, W.wpos, B.total, W.ctr + 2, W.scan_tmp, s);
            if (rc) return rc;
            rc = exclusive_scan_dev(W.surf, W.spos_box, B.total, W.ctr + 3, W.scan_tmp, s);
            if (rc) return rc;
            k_surface_scatter<<<gb, kNfBlock, 0, s>>>(A, B, W.wet, W.surf, W.wpos, W.spos_box, fln, sfn,
                                                      W.spos_cell);
            int cnt[2];
            CLOWNS_CUDA_TRY(cudaMemcpyAsync(cnt, W.ctr + 2, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
            CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
            ifln = cnt[0];
            isfn = cnt[1];
        }
        if (isfn == 0) break;
        const int gs = nf_grid(isfn);
        // first pruning
        CLOWNS_CUDA_TRY(cudaMemsetAsync(W.ctr + 4, 0, sizeof(int), s));
        k_prune1<<<gs, kNfBlock, 0, s>>>(A, isfn, sfn, W.st0, W.ctr + 4);
        int removed = 0;
        int rc = read_int(W.ctr + 4, s, &removed);
        if (rc) return rc;
        if (removed) {
            k_remove<<<gs, kNfBlock, 0, s>>>(A, isfn, sfn, W.st0);
            continue;
        }
        // second pruning: Jacobi to the serial fixed point
        k_fill<<<gs, kNfBlock, 0, s>>>(W.st0, isfn, 0);
        int* cur = W.st0;
        int* nxt = W.st1;
        bool settled = false;
        for (int sweep = 0; sweep <= isfn + 1; sweep++) {
            CLOWNS_CUDA_TRY(cudaMemsetAsync(W.ctr + 5, 0, sizeof(int), s));
            k_prune2_sweep<<<gs, kNfBlock, 0, s>>>(A, isfn, sfn, W.spos_cell, cur, nxt, W.ctr + 5);
            int changed = 0;
            rc = read_int(W.ctr + 5, s, &changed);
            if (rc) return rc;
            int* tmp = cur; cur = nxt; nxt = tmp;
            if (!changed) { settled = true; break; }
        }
        if (!settled) {
            set_last_error_msg("set_nflag: second pruning did not settle");
            return CLOWNS_ERR_NOCONV;
        }
        // apply the removals of the settled state
        CLOWNS_CUDA_TRY(cudaMemsetAsync(W.ctr + 6, 0, sizeof(int), s));
        k_count_nonzero<<<gs, kNfBlock, 0, s>>>(cur, isfn, W.ctr + 6);
        k_remove<<<gs, kNfBlock, 0, s>>>(A, isfn, sfn, cur);
        int removed2 = 0;
        rc = read_int(W.ctr + 6, s, &removed2);
        if (rc) return rc;
        if (removed2) continue;
        // orientation: Jacobi to the serial fixed point
        k_fill<<<gs, kNfBlock, 0, s>>>(W.st0, isfn, 0);
        cur = W.st0;
        nxt = W.st1;
        settled = false;
        for (int sweep = 0; sweep <= isfn + 1; sweep++) {
            CLOWNS_CUDA_TRY(cudaMemsetAsync(W.ctr + 5, 0, sizeof(int), s));
            k_orient_sweep<<<gs, kNfBlock, 0, s>>>(A, f, isfn, sfn, W.spos_cell, cur, nxt, W.bout, W.ctr + 5);
            int changed = 0;
            rc = read_int(W.ctr + 5, s, &changed);
            if (rc) return rc;
            int* tmp = cur; cur = nxt; nxt = tmp;
            if (!changed) { settled = true; break; }
        }
        if (!settled) {
            set_last_error_msg("set_nflag: orientation did not settle");
            return CLOWNS_ERR_NOCONV;
        }
        CLOWNS_CUDA_TRY(cudaMemsetAsync(W.ctr + 9, 0, sizeof(int), s));
        k_orient_apply<<<gs, kNfBlock, 0, s>>>(A, isfn, sfn, cur, W.bout, W.ctr + 9);
        int igai = 0;
        rc = read_int(W.ctr + 9, s, &igai);
        if (rc) return rc;
        if (igai) continue;
        break;
    }
    CLOWNS_CUDA_TRY(cudaGetLastError());
    CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
    *ifln_out = ifln;
    *isfn_out = isfn;
    if (passes_out) *passes_out = passes;
    return CLOWNS_OK;
}
