// grid_index.cuh -- index arithmetic for the reference's dense arrays, plus a
// device-wide exclusive scan used to number rows and list cells.
#pragma once

#include "common.cuh"

namespace clowns {

// Bounds of the reference's index space (dims = is, js, ks, ie, je, ke).
struct GridIdx {
    int is, js, ks, ie, je, ke;
    long ni, nk, nj;   // extents of mn(is-2:ie+2, ks-2:ke+2, js-2:je+2)

    static GridIdx make(const int* dims) {
        GridIdx g;
        g.is = dims[0]; g.js = dims[1]; g.ks = dims[2];
        g.ie = dims[3]; g.je = dims[4]; g.ke = dims[5];
        g.ni = g.ie - g.is + 5;
        g.nk = g.ke - g.ks + 5;
        g.nj = g.je - g.js + 5;
        return g;
    }
    // offset of mn(i,k,j)
    __host__ __device__ __forceinline__ long mn_off(int i, int k, int j) const {
        return (long)(i - (is - 2)) + ni * ((long)(k - (ks - 2)) + nk * (long)(j - (js - 2)));
    }
    // neighbour of (i,j,k) at signed step s along axis l (lf = identity, main_2CLOWNS.F90:33)
    __host__ __device__ __forceinline__ long nbr(int i, int j, int k, int l, int s) const {
        return mn_off(i + s * (l == 0), k + s * (l == 2), j + s * (l == 1));
    }
    // offset of mno(i,k,j), mno(1:ie, 1:ke, 1:je)
    __host__ __device__ __forceinline__ long mno_off(int i, int k, int j) const {
        return (long)(i - 1) + (long)ie * ((long)(k - 1) + (long)ke * (long)(j - 1));
    }
    // offset of x(l,i) / dx(l,i), (0:2, 1:mx2)
    __host__ __device__ __forceinline__ long dxo(int l, int i) const { return 3L * (i - 1) + l; }
    // Matrix columns: 6 in 3D; 4 in the 2DV mode the reference enters for a grid
    // one cell wide in x or in y (main_2CLOWNS.F90:43-44, 1sub-matrix.F90:15-21).
    __host__ __device__ __forceinline__ int nl() const { return (ie == is + 1 || je == js + 1) ? 4 : 6; }
    // Physical axis of matrix columns 2q, 2q+1 (0-based; minus side first): the
    // axes that are not one cell wide, in the order x, y, z (1sub-matrix.F90:33-36;
    // the shift of 1sub-momentum.F90:517-520).
    __host__ __device__ __forceinline__ int col_axis(int q) const {
        if (ie == is + 1) return q + 1;
        if (je == js + 1) return q == 0 ? 0 : 2;
        return q;
    }
};

// A grid one cell wide in both x and y has no matrix form in the reference
// (init_matrix sets two of its four columns, and the surface-row axis shift of
// cal_matrix_element reaches 3): the entry points that build or read matrix
// columns refuse it.
inline bool grid_has_matrix(const int* d) { return d && !(d[3] == d[0] + 1 && d[4] == d[1] + 1); }

// The reference stores x(l, ls-2 .. le+1) in x(0:2, 1:mx2) (data_io.F90:114,
// 0mod-arrays.F90:205) and numbers cells from ls-1, whose minus neighbours at
// ls-2 are addressed in mn and mno: so ls >= 3 on every axis, and each axis
// holds at least one cell.
inline bool grid_dims_ok(const int* d) {
    return d && d[0] >= 3 && d[1] >= 3 && d[2] >= 3 && d[3] > d[0] && d[4] > d[1] && d[5] > d[2];
}

// Exclusive scan of n int32 flags/counts: out[t] = sum_{u<t} in[u], *total = sum.
size_t scan_workspace_bytes(long n);
int exclusive_scan_dev(const int* in, int* out, long n, int* total, void* tmp, cudaStream_t s);

}  // namespace clowns
