// adjoint.cu -- discrete adjoint of the pressure solve (no reference counterpart).
//
// For J = sum_g w_g x_g with A x = b (A assembled by cal_matrix_element,
// 1sub-momentum.F90:465-551), the adjoint A^T lambda = w gives dJ/db = lambda
// and, for a face area fraction a_f that enters A through the static
// coefficients ALU_C = -mp * 2/(dx (dx+dxm)) * a_f / fb (1sub-matrix.F90:49-61),
// dJ/da_f = -lambda^T (dA/da_f) x.  A is not symmetric (rows are divided by their
// own porosity and spacing; surface rows carry extrapolation coefficients), so
// A^T is formed explicitly: row j's coefficient toward its neighbour i in
// direction d becomes row i's coefficient toward j in the opposite direction.
#include "common.cuh"
#include "grid_index.cuh"
#include "trace.h"

namespace clowns {

__global__ void k_transpose_zero(long n, long na, int nl, double* alt, int* llt) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nl * na; t += (long)gridDim.x * blockDim.x) {
        alt[t] = 0.0;
        llt[t] = 0;
    }
}

__global__ void k_transpose(long n, long na, int nl, const double* __restrict__ alu, const int* __restrict__ llu,
                            const double* __restrict__ de, double* __restrict__ alt, int* __restrict__ llt,
                            double* __restrict__ det, int* bad) {
    for (long j = (long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long)gridDim.x * blockDim.x) {
        det[j] = de[j];
        for (int d = 0; d < nl; d++) {
            const int i = llu[d * na + j];          // 1-based row, 0 = none
            if (i == 0) continue;
            if (i < 0 || i > n) { atomicOr(bad, 1); continue; }
            const int od = d ^ 1;                   // minus <-> plus face of the same axis
            alt[od * na + (i - 1)] = alu[d * na + j];
            llt[od * na + (i - 1)] = (int)j + 1;
        }
    }
}

// dJ/da(l, owner) accumulated over the (at most two) rows that own a face.
// g is laid out like a(0:2, 0:inne2+1); lambda, x are row vectors (0-based).
__global__ void k_face_grad(GridIdx g, int ifln, long inne, const int* __restrict__ fln,
                            const int* __restrict__ in_, const int* __restrict__ jn, const int* __restrict__ kn,
                            const int* __restrict__ nf, const int* __restrict__ mno,
                            const double* __restrict__ alu_c, const int* __restrict__ ll_c,
                            const double* __restrict__ a, const double* __restrict__ x,
                            const double* __restrict__ lam, double* __restrict__ grad) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < ifln; t += (long)gridDim.x * blockDim.x) {
        const int c = fln[t];
        if (nf[c] != 1) continue;                   // surface rows do not depend on a
        const int r = mno[g.mno_off(in_[c], kn[c], jn[c])];
        if (r == 0) continue;
        const double lr = lam[r - 1], xr = x[r - 1];
        const int nl = g.nl();
        for (int ll = 0; ll < nl; ll++) {
            const long oc = (long)ll * inne + (c - 1);
            const int lc = ll_c[oc];
            if (lc == 0) continue;
            const int l = g.col_axis(ll >> 1), side = ll & 1;
            const int owner = side ? lc : c;
            const double af = a[3L * owner + l];
            if (af == 0.0) continue;
            const double dcoef = alu_c[oc] / af;    // d ALU_C / d a_f
            const int np = mno[g.mno_off(in_[lc], kn[lc], jn[lc])];
            double contrib;
            if (nf[lc] == 0 || np == 0) {
                // dropped neighbour: Neumann rows cancel the face (no dependence);
                // a surface cell that is not a row keeps it in the diagonal only
                if (nf[lc] != 2) continue;
                contrib = lr * dcoef * xr;
            } else {
                contrib = -lr * dcoef * (x[np - 1] - xr);
            }
            atomicAdd(grad + 3L * owner + l, contrib);
        }
    }
}

}  // namespace clowns

using namespace clowns;

extern "C" int clowns_transpose_dev(int n, int na, int nl, const double* alu, const int* llu, const double* de,
                                    double* alt, int* llt, double* det, int* bad, void* stream) {
    clowns::TraceRange trace_range_("clowns_transpose_dev");
    if (n < 1 || na < n || (nl != 6 && nl != 4) || !alu || !llu || !de || !alt || !llt || !det || !bad) {
        set_last_error_msg("transpose: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int gb = (int)std::min<long>(((long)nl * na + 255) / 256, 152L * 16);
    CLOWNS_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), s));
    k_transpose_zero<<<gb, 256, 0, s>>>(n, na, nl, alt, llt);
    k_transpose<<<(int)std::min<long>((n + 255) / 256, 152L * 16), 256, 0, s>>>(n, na, nl, alu, llu, de, alt, llt,
                                                                               det, bad);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    return CLOWNS_OK;
}

extern "C" int clowns_face_grad_dev(const int* dims, int inne, int inne2, int ifln, const int* fln,
                                    const int* in_, const int* jn, const int* kn, const int* nf, const int* mno,
                                    const double* alu_c, const int* ll_c, const double* a, const double* x,
                                    const double* lambda, double* grad, void* stream) {
    clowns::TraceRange trace_range_("clowns_face_grad_dev");
    if (!grid_dims_ok(dims) || !grid_has_matrix(dims) || inne < 1 || ifln < 0 || !fln || !in_ || !jn || !kn || !nf ||
        !mno || !alu_c || !ll_c || !a || !x || !lambda || !grad) {
        set_last_error_msg("face_grad: invalid arguments");
        return CLOWNS_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    GridIdx g = GridIdx::make(dims);
    CLOWNS_CUDA_TRY(cudaMemsetAsync(grad, 0, sizeof(double) * 3 * ((size_t)inne2 + 2), s));
    if (ifln > 0)
        k_face_grad<<<(int)std::min<long>((ifln + 255) / 256, 152L * 16), 256, 0, s>>>(
            g, ifln, inne, fln, in_, jn, kn, nf, mno, alu_c, ll_c, a, x, lambda, grad);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    return CLOWNS_OK;
}
