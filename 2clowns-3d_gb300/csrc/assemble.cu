// assemble.cu -- static coefficients, row numbering, right-hand side, per-step
// matrix assembly and the pressure / velocity correction on the GPU.
//
// This translation unit is compiled with --fmad=false: every coefficient is
// produced with separately rounded multiplies and adds, in the reference's
// evaluation order, so the assembled matrix is bit-identical to an IEEE
// evaluation of the Fortran source (the per-row sort inside the solve compares
// these values, and ties must break the same way).
#include <cstring>

#include "common.cuh"
#include "grid_index.cuh"
#include "trace.h"

namespace clowns {

constexpr int kAsmBlock = 256;

static inline int grid_for(long n) {
    long b = (n + kAsmBlock - 1) / kAsmBlock;
    if (b < 1) b = 1;
    if (b > 152L * 16) b = 152L * 16;
    return (int)b;
}

// ---------------------------------------------------------------------------
// mp = minval(dx, dx > 0)**2 over the axes in `axes` (bit l: axis l): every
// axis in 3D (1sub-matrix.F90:17), the two of the x-z or y-z plane in 2DV (20-21)
__global__ void k_min_dx(const double* __restrict__ dx, int count, int axes, double* mp) {
    __shared__ double s[256];
    double m = 1.0e300;
    for (int t = threadIdx.x; t < count; t += blockDim.x) {
        if (!((axes >> (t % 3)) & 1)) continue;
        double v = dx[t];
        if (v > 0.0 && v < m) m = v;
    }
    s[threadIdx.x] = m;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o && s[threadIdx.x + o] < s[threadIdx.x]) s[threadIdx.x] = s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *mp = s[0] * s[0];
}

// cal_alu_f (1sub-matrix.F90:82-87)
__device__ __forceinline__ double cal_alu_f(double dx, double dxm, double ax, double fb) {
    return 2.0 / dx / (dx + dxm) * ax / fb;
}
// cal_alu (1sub-matrix.F90:75-80)
__device__ __forceinline__ double cal_alu(double fnn, double dx, double dxm) {
    return (fnn - 0.5) * dx / (fnn * dx + dxm * 0.5) * (-1.0);
}

// init_matrix (1sub-matrix.F90:25-65), one thread per cell nnn = 1..inne;
// columns 2q, 2q+1 hold the minus and plus faces of axis col_axis(q)
__global__ void __launch_bounds__(kAsmBlock) k_init_matrix(GridIdx g, int inne, const int* __restrict__ mn,
                                                          const int* __restrict__ in_, const int* __restrict__ jn,
                                                          const int* __restrict__ kn, const int* __restrict__ nf,
                                                          const int* __restrict__ nfb, const double* __restrict__ a,
                                                          const double* __restrict__ fb, const double* __restrict__ dx,
                                                          const double* __restrict__ mp_p, double* __restrict__ alu_c,
                                                          int* __restrict__ ll_c, double* __restrict__ de_c) {
    const double mp = *mp_p;
    const long ld = inne;
    const int nl = g.nl();
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < inne; t += (long)gridDim.x * blockDim.x) {
        const int nnn = (int)t + 1;
        if (nf[nnn] == -1 || fb[nnn] == 0.0) {
            for (int c = 0; c < nl; c++) { alu_c[c * ld + t] = 0.0; ll_c[c * ld + t] = 0; }
            de_c[t] = 0.0;
            continue;
        }
        const int i = in_[nnn], j = jn[nnn], k = kn[nnn];
        const int lg[3] = {i, j, k};
        double de = 0.0;
        for (int q = 0; q < nl / 2; q++) {
            const int l = g.col_axis(q);
#pragma unroll
            for (int side = 0; side < 2; side++) {
                const int ii = side ? 1 : -1;
                const int np = mn[g.nbr(i, j, k, l, ii)];
                const int npp = side ? np : mn[g.mn_off(i, k, j)];
                const int col = 2 * q + side;      // 0-based; 3D: x-, x+, y-, y+, z-, z+
                if ((nf[np] == -1 && nfb[np] != 4) || a[3L * npp + l] == 0.0 || fb[np] == 0.0) {
                    ll_c[col * ld + t] = 0;
                    alu_c[col * ld + t] = 0.0;
                } else {
                    const double v = -(mp * cal_alu_f(dx[g.dxo(l, lg[l])], dx[g.dxo(l, lg[l] + ii)], a[3L * npp + l], fb[nnn]));
                    ll_c[col * ld + t] = np;
                    alu_c[col * ld + t] = v;
                    de = de - v;
                }
            }
        }
        de_c[t] = de;
    }
}

// ---------------------------------------------------------------------------
// Row numbering (1sub-momentum.F90:273-296): a fluid-list entry becomes a row
// unless it is air, solid, has zero porosity, or is a surface cell whose
// normal-side neighbour is solid.  Rows keep fluid-list order (an exclusive scan).
__global__ void __launch_bounds__(kAsmBlock) k_row_flags(GridIdx g, int ifln, const int* __restrict__ fln,
                                                        const int* __restrict__ mn, const int* __restrict__ in_,
                                                        const int* __restrict__ jn, const int* __restrict__ kn,
                                                        const int* __restrict__ nf, const int* __restrict__ nfb,
                                                        const double* __restrict__ fb, int* __restrict__ keep) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < ifln; t += (long)gridDim.x * blockDim.x) {
        const int nnn = fln[t];
        int kp = 1;
        if (nf[nnn] == 0 || nf[nnn] == -1 || fb[nnn] == 0.0) {
            kp = 0;
        } else if (nf[nnn] == 2) {
            const int b = nfb[nnn];
            const int l = (b < 0 ? -b : b) - 1;
            const int s = b >= 0 ? 1 : -1;
            // an orientation of 0 has no defined neighbour in the reference; kept
            if (l >= 0 && l <= 2 && nf[mn[g.nbr(in_[nnn], jn[nnn], kn[nnn], l, s)]] == -1) kp = 0;
        }
        keep[t] = kp;
    }
}

__global__ void __launch_bounds__(kAsmBlock) k_row_scatter(GridIdx g, int ifln, const int* __restrict__ fln,
                                                          const int* __restrict__ in_, const int* __restrict__ jn,
                                                          const int* __restrict__ kn, const int* __restrict__ keep,
                                                          const int* __restrict__ pos, int* __restrict__ mno,
                                                          int* __restrict__ mno2mn) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < ifln; t += (long)gridDim.x * blockDim.x) {
        if (!keep[t]) continue;
        const int nnn = fln[t];
        const int row = pos[t] + 1;                     // 1-based row number
        mno[g.mno_off(in_[nnn], kn[nnn], jn[nnn])] = row;
        mno2mn[row - 1] = nnn;                          // mno2mn(row)
    }
}

// renzoku_fv (lib/src/math_func.F90:51-54)
__device__ __forceinline__ double renzoku_fv(double axp, double axm, double ayp, double aym, double azp,
                                             double azm, double up, double um, double vp, double vm,
                                             double wp, double wm, double dx, double dy, double dz,
                                             double fb) {
    return ((up * axp - um * axm) / dx + (vp * ayp - vm * aym) / dy + (wp * azp - wm * azm) / dz) / fb;
}

// RHS of the fluid rows (1sub-momentum.F90:313-360) and dmax = max |DR1|
__global__ void __launch_bounds__(kAsmBlock) k_rhs(GridIdx g, int mnoe, const int* __restrict__ mno2mn,
                                                  const int* __restrict__ mn, const int* __restrict__ in_,
                                                  const int* __restrict__ jn, const int* __restrict__ kn,
                                                  const int* __restrict__ nf, const double* __restrict__ f,
                                                  const double* __restrict__ fb, const double* __restrict__ a,
                                                  const double* __restrict__ un, const double* __restrict__ dx,
                                                  const double* __restrict__ mp_p, double dt,
                                                  double* __restrict__ b, unsigned long long* dmax_bits) {
    const double mp = *mp_p;
    double local = 0.0;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < mnoe; t += (long)gridDim.x * blockDim.x) {
        const int c = mno2mn[t];
        if (nf[c] != 1) continue;
        const int i = in_[c], j = jn[c], k = kn[c];
        const double ff = fmax(-0.001, fmin(1.0 - f[c], 0.001));
        double rz;
        if (fb[c] != 0.0) {
            const int ip = mn[g.mn_off(i + 1, k, j)], jp = mn[g.mn_off(i, k, j + 1)], kp = mn[g.mn_off(i, k + 1, j)];
            rz = renzoku_fv(a[3L * ip + 0], a[3L * c + 0], a[3L * jp + 1], a[3L * c + 1], a[3L * kp + 2], a[3L * c + 2],
                            un[3L * ip + 0], un[3L * c + 0], un[3L * jp + 1], un[3L * c + 1], un[3L * kp + 2],
                            un[3L * c + 2], dx[g.dxo(0, i)], dx[g.dxo(1, j)], dx[g.dxo(2, k)], fb[c]);
        } else {
            rz = -10000.0;
        }
        const double dr1 = rz + ff / dt;
        const double q = dr1 / dt;
        if (!(fabs(q) <= 1.0e-15 && fabs(q) != 0.0)) b[t] = mp * dr1 / dt;
        const double ad = fabs(dr1);
        if (ad > local) local = ad;
    }
    // |DR1| >= 0: the IEEE bit pattern orders like the value
    for (int o = 16; o > 0; o >>= 1) local = fmax(local, __shfl_xor_sync(0xffffffffu, local, o));
    if ((threadIdx.x & 31) == 0 && local > 0.0) atomicMax(dmax_bits, (unsigned long long)__double_as_longlong(local));
}

// ---------------------------------------------------------------------------
// cal_matrix_element (1sub-momentum.F90:465-551), NORMAL build, one thread per
// fluid-list entry.
__global__ void __launch_bounds__(kAsmBlock) k_assemble(GridIdx g, int ifln, long inne, long na, long spld,
                                                       const int* __restrict__ fln, const int* __restrict__ in_,
                                                       const int* __restrict__ jn, const int* __restrict__ kn,
                                                       const int* __restrict__ nf, const int* __restrict__ nfb,
                                                       const double* __restrict__ x, const double* __restrict__ dx,
                                                       const double* __restrict__ sp, const int* __restrict__ mno,
                                                       const double* __restrict__ alu_c, const int* __restrict__ ll_c,
                                                       const double* __restrict__ de_c, double* __restrict__ alu,
                                                       int* __restrict__ llu, double* __restrict__ de, int* err) {
    const double rate = -1.0e-20;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < ifln; t += (long)gridDim.x * blockDim.x) {
        const int nnn = fln[t];
        const int i = in_[nnn], j = jn[nnn], k = kn[nnn];
        const int nn = mno[g.mno_off(i, k, j)];
        if (nn == 0) continue;
        const long r = nn - 1;
        const int fl = nf[nnn];
        double dd;
        if (fl == 1) {
            dd = de_c[nnn - 1];
        } else if (fl == 2) {
            dd = 1.0;
        } else {
            atomicCAS(err, 0, nnn);
            continue;
        }
        const int bl = nfb[nnn];
        const int axis = (bl < 0 ? -bl : bl) - 1;
        const int nl = g.nl();
        for (int ll = 1; ll <= nl; ll++) {
            const long oc = (long)(ll - 1) * inne + (nnn - 1);
            const long o = (long)(ll - 1) * na + r;
            const int lc = ll_c[oc];
            if (lc == 0) {
                llu[o] = 0;
                alu[o] = 0.0;
                continue;
            }
            const int np = mno[g.mno_off(in_[lc], kn[lc], jn[lc])];
            const int fn = nf[lc];
            if (fn == 0 || np == 0) {
                llu[o] = 0;
                alu[o] = 0.0;
                if (fl == 1 && fn != 2) dd = dd + alu_c[oc];
                continue;
            }
            llu[o] = np;
            if (fl == 1) {
                alu[o] = alu_c[oc];
            } else {
                const int l = g.col_axis((ll - 1) / 2);    // 2DV: past the collapsed axis (517-520)
                if (axis == l) {
                    const int ii = (l == 0) ? i : (l == 1) ? j : k;
                    const int md = ll % 2;
                    const double fss = (double)(1 - 2 * md) * (x[g.dxo(l, ii - md + 1)] - sp[nnn + spld * l]) / dx[g.dxo(l, ii)];
                    alu[o] = cal_alu(fss, dx[g.dxo(l, ii)], dx[g.dxo(l, ii - 2 * md + 1)]);
                } else {
                    alu[o] = rate;
                }
            }
        }
        de[r] = dd;
    }
}

// ---------------------------------------------------------------------------
// p(mno2mn(r)) -= xe(r)  (1sub-momentum.F90:53-58)
__global__ void k_pressure_update(int mnoe, const int* __restrict__ mno2mn, const double* __restrict__ xe0,
                                  double* __restrict__ p) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < mnoe; t += (long)gridDim.x * blockDim.x) {
        const int c = mno2mn[t];
        p[c] = p[c] - xe0[t + 1];
    }
}

// estimate_velocity2 (1sub-momentum.F90:590-651) with momentum_d
// (lib/src/math_func.F90:251-254); xe0 addresses xe(0).
__global__ void __launch_bounds__(kAsmBlock) k_velocity(GridIdx g, int inne, const int* __restrict__ mn,
                                                       const int* __restrict__ in_, const int* __restrict__ jn,
                                                       const int* __restrict__ kn, const int* __restrict__ nf,
                                                       const int* __restrict__ nfb, const double* __restrict__ a,
                                                       const double* __restrict__ dx, double dt,
                                                       const int* __restrict__ mno, const double* __restrict__ xe0,
                                                       double* __restrict__ un) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < inne; t += (long)gridDim.x * blockDim.x) {
        const int nn = (int)t + 1;
        const int fl = nf[nn];
        if (fl == 0) continue;
        if (fl == -1 && nfb[nn] != 4) continue;
        const int i = in_[nn], j = jn[nn], k = kn[nn];
        const int ic[3] = {i, j, k};
        const int nnn = mno[g.mno_off(i, k, j)];
        const double xec = -xe0[nnn];
        const int nno[3] = {mno[g.mno_off(i - 1, k, j)], mno[g.mno_off(i, k, j - 1)], mno[g.mno_off(i, k - 1, j)]};
        const int nnm[3] = {mn[g.mn_off(i - 1, k, j)], mn[g.mn_off(i, k, j - 1)], mn[g.mn_off(i, k - 1, j)]};
        if (fl == -1 && nfb[nn] == 4) {
            for (int l = 0; l < 3; l++) {
                if (nf[nnm[l]] >= 1) {
                    const double dxc = (dx[g.dxo(l, ic[l])] + dx[g.dxo(l, ic[l] - 1)]) * 0.5;
                    un[3L * nn + l] = un[3L * nn + l] + dt * (-xe0[nno[l]] - (-xe0[nnn])) / dxc;
                }
            }
        } else {
            for (int l = 0; l < 3; l++) {
                if (a[3L * nn + l] != 0.0) {
                    const double dxc = (dx[g.dxo(l, ic[l])] + dx[g.dxo(l, ic[l] - 1)]) * 0.5;
                    const int nfm = nf[nnm[l]];
                    if (nfm >= 1) {
                        double u = un[3L * nn + l] + dt * (-xe0[nno[l]] - xec) / dxc;
                        if (fabs(u) < 1.0e-15) u = 0.0;
                        un[3L * nn + l] = u;
                    } else if (nfm == -1 && nfb[nnm[l]] == 4) {
                        un[3L * nn + l] = un[3L * nn + l] + dt * (-xe0[nno[l]] - xec) / dxc;
                    }
                }
            }
        }
    }
}

}  // namespace clowns

using namespace clowns;

// ---------------------------------------------------------------------------
// C ABI

extern "C" int clowns_grid_nl(const int* dims) {
    if (!grid_dims_ok(dims) || !grid_has_matrix(dims)) return 0;
    return GridIdx::make(dims).nl();
}

extern "C" int clowns_init_matrix_dev(const int* dims, int inne, int mx2, const int* mn, const int* in_,
                                      const int* jn, const int* kn, const int* nf, const int* nfb,
                                      const double* a, const double* fb, const double* dx, double* mp,
                                      double* alu_c, int* ll_c, double* de_c, void* stream) {
    clowns::TraceRange trace_range_("clowns_init_matrix_dev");
    if (!grid_dims_ok(dims) || inne < 1 || mx2 < 1 || !mn || !in_ || !jn || !kn || !nf || !nfb || !a || !fb || !dx || !mp ||
        !alu_c || !ll_c || !de_c) {
        set_last_error_msg("init_matrix: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    if (!grid_has_matrix(dims)) {
        set_last_error_msg("init_matrix: a grid one cell wide in both x and y has no matrix form");
        return CLOWNS_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    GridIdx g = GridIdx::make(dims);
    // 2DV: x and z when one cell wide in y, y and z when one cell wide in x
    const int axes = g.ie == g.is + 1 ? 6 : g.je == g.js + 1 ? 5 : 7;
    k_min_dx<<<1, 256, 0, s>>>(dx, 3 * mx2, axes, mp);
    k_init_matrix<<<grid_for(inne), kAsmBlock, 0, s>>>(g, inne, mn, in_, jn, kn, nf, nfb, a, fb, dx, mp, alu_c,
                                                       ll_c, de_c);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    return CLOWNS_OK;
}

extern "C" size_t clowns_rows_rhs_workspace_bytes(int ifln) {
    return scan_workspace_bytes(ifln) + align_up(sizeof(int) * (size_t)(ifln + 1), 256) * 2 + 256;
}

extern "C" int clowns_rows_rhs_dev(const int* dims, int inne2, int mx2, const int* mn, const int* in_,
                                   const int* jn, const int* kn, const int* nf, const int* nfb, const double* f,
                                   const double* fb, const double* a, const double* un, const double* dx,
                                   const double* mp, double dt, int ifln, const int* fln, int mm2, int* mno,
                                   int* mno2mn, double* b, double* xe, double* de, int* mnoe_out,
                                   double* dmax_out, void* work, size_t work_bytes, void* stream) {
    clowns::TraceRange trace_range_("clowns_rows_rhs_dev");
    (void)inne2; (void)mx2;
    if (!grid_dims_ok(dims) || !mn || !in_ || !jn || !kn || !nf || !nfb || !f || !fb || !a || !un || !dx || !mp || !fln ||
        !mno || !mno2mn || !b || !xe || !de || !mnoe_out || ifln < 0 || mm2 < 1 || !work) {
        set_last_error_msg("rows_rhs: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    if (work_bytes < clowns_rows_rhs_workspace_bytes(ifln)) {
        set_last_error_msg("rows_rhs: workspace too small");
        return CLOWNS_ERR_WORKSPACE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    GridIdx g = GridIdx::make(dims);
    char* wb = (char*)work;
    int* keep = (int*)wb;
    wb += align_up(sizeof(int) * (size_t)(ifln + 1), 256);
    int* pos = (int*)wb;
    wb += align_up(sizeof(int) * (size_t)(ifln + 1), 256);
    unsigned long long* dmax_bits = (unsigned long long*)wb;
    wb += 256;
    void* scan_tmp = wb;
    // 1sub-momentum.F90:267-271 and 276
    CLOWNS_CUDA_TRY(cudaMemsetAsync(b, 0, sizeof(double) * mm2, s));
    CLOWNS_CUDA_TRY(cudaMemsetAsync(xe, 0, sizeof(double) * mm2, s));
    CLOWNS_CUDA_TRY(cudaMemsetAsync(de, 0, sizeof(double) * mm2, s));
    CLOWNS_CUDA_TRY(cudaMemsetAsync(mno, 0, sizeof(int) * (size_t)g.ie * g.ke * g.je, s));
    CLOWNS_CUDA_TRY(cudaMemsetAsync(dmax_bits, 0, sizeof(unsigned long long), s));
    int mnoe = 0;
    if (ifln > 0) {
        k_row_flags<<<grid_for(ifln), kAsmBlock, 0, s>>>(g, ifln, fln, mn, in_, jn, kn, nf, nfb, fb, keep);
        int rc = exclusive_scan_dev(keep, pos, ifln, pos + ifln, scan_tmp, s);
        if (rc) return rc;
        CLOWNS_CUDA_TRY(cudaMemcpyAsync(&mnoe, pos + ifln, sizeof(int), cudaMemcpyDeviceToHost, s));
        CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
        if (mnoe > mm2) {
            set_last_error_msg("rows_rhs: mm2 smaller than the number of rows");
            return CLOWNS_ERR_ARG;
        }
        k_row_scatter<<<grid_for(ifln), kAsmBlock, 0, s>>>(g, ifln, fln, in_, jn, kn, keep, pos, mno, mno2mn);
    }
    *mnoe_out = mnoe;
    if (dmax_out) *dmax_out = 0.0;
    if (mnoe < 10) {                                // 1sub-momentum.F90:297-300
        CLOWNS_CUDA_TRY(cudaGetLastError());
        CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
        return CLOWNS_OK;
    }
    if (mnoe + 64 > mm2) {                          // the reference re-allocates (302-310)
        set_last_error_msg("rows_rhs: mm2 must exceed the number of rows by at least 64");
        return CLOWNS_ERR_ARG;
    }
    k_rhs<<<grid_for(mnoe), kAsmBlock, 0, s>>>(g, mnoe, mno2mn, mn, in_, jn, kn, nf, f, fb, a, un, dx, mp, dt, b,
                                              dmax_bits);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    if (dmax_out) {
        unsigned long long bits = 0;
        CLOWNS_CUDA_TRY(cudaMemcpyAsync(&bits, dmax_bits, sizeof(bits), cudaMemcpyDeviceToHost, s));
        CLOWNS_CUDA_TRY(cudaStreamSynchronize(s));
        double v;
        memcpy(&v, &bits, sizeof(v));
        *dmax_out = v;
    }
    return CLOWNS_OK;
}

extern "C" int clowns_assemble_dev(const int* dims, int inne, int inne2, int mx2, const int* in_, const int* jn,
                                   const int* kn, const int* nf, const int* nfb, const double* x, const double* dx,
                                   const double* sp, int ifln, const int* fln, const int* mno, const double* alu_c,
                                   const int* ll_c, const double* de_c, int mm2, double* alu, int* llu, double* de,
                                   int* err_cell, void* stream) {
    clowns::TraceRange trace_range_("clowns_assemble_dev");
    (void)mx2;
    if (!grid_dims_ok(dims) || inne < 1 || !in_ || !jn || !kn || !nf || !nfb || !x || !dx || !sp || !fln || !mno || !alu_c ||
        !ll_c || !de_c || mm2 < 1 || !alu || !llu || !de || !err_cell) {
        set_last_error_msg("assemble: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    if (!grid_has_matrix(dims)) {
        set_last_error_msg("assemble: a grid one cell wide in both x and y has no matrix form");
        return CLOWNS_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    GridIdx g = GridIdx::make(dims);
    CLOWNS_CUDA_TRY(cudaMemsetAsync(err_cell, 0, sizeof(int), s));
    if (ifln > 0)
        k_assemble<<<grid_for(ifln), kAsmBlock, 0, s>>>(g, ifln, inne, mm2, (long)inne2 + 2, fln, in_, jn, kn, nf,
                                                        nfb, x, dx, sp, mno, alu_c, ll_c, de_c, alu, llu, de,
                                                        err_cell);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    return CLOWNS_OK;
}

extern "C" int clowns_correct_dev(const int* dims, int inne, int mx2, const int* mn, const int* in_, const int* jn,
                                  const int* kn, const int* nf, const int* nfb, const double* a, const double* dx,
                                  double dt, int mnoe, const int* mno2mn, const int* mno, const double* xe0,
                                  double* p, double* un, void* stream) {
    clowns::TraceRange trace_range_("clowns_correct_dev");
    (void)mx2;
    if (!grid_dims_ok(dims) || inne < 1 || !mn || !in_ || !jn || !kn || !nf || !nfb || !a || !dx || mnoe < 0 || !mno2mn ||
        !mno || !xe0 || !p || !un) {
        set_last_error_msg("correct: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    GridIdx g = GridIdx::make(dims);
    if (mnoe > 0) k_pressure_update<<<grid_for(mnoe), kAsmBlock, 0, s>>>(mnoe, mno2mn, xe0, p);
    k_velocity<<<grid_for(inne), kAsmBlock, 0, s>>>(g, inne, mn, in_, jn, kn, nf, nfb, a, dx, dt, mno, xe0, un);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    return CLOWNS_OK;
}
