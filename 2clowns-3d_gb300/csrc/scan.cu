// scan.cu -- device-wide exclusive scan of int32 values (three passes:
// per-tile sums, a single-block scan of the tile sums, per-tile scan + offset).
#include "grid_index.cuh"

namespace clowns {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ int block_exclusive_scan(int v, int* smem /* >= 32 */, int* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = lane < nw ? smem[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        smem[lane] = w;   // inclusive prefix of warp totals
    }
    __syncthreads();
    const int warp_off = wid > 0 ? smem[wid - 1] : 0;
    const int tot = smem[nw - 1];
    __syncthreads();
    *total = tot;
    return warp_off + x - v;
}

__global__ void k_tile_sums(const int* __restrict__ in, long n, int* __restrict__ sums) {
    __shared__ int sm[32];
    const long base = (long)blockIdx.x * kScanTile;
    int s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; q++) {
        long t = base + (long)threadIdx.x * kScanItems + q;
        if (t < n) s += in[t];
    }
    int tot;
    block_exclusive_scan(s, sm, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums(int* __restrict__ sums, int nt, int* __restrict__ total) {
    __shared__ int sm[32];
    const int per = (nt + blockDim.x - 1) / blockDim.x;
    const int lo = threadIdx.x * per;
    int s = 0;
    for (int q = 0; q < per; q++)
        if (lo + q < nt) s += sums[lo + q];
    int tot;
    int off = block_exclusive_scan(s, sm, &tot);
    for (int q = 0; q < per; q++) {
        if (lo + q < nt) {
            int v = sums[lo + q];
            sums[lo + q] = off;
            off += v;
        }
    }
    if (threadIdx.x == 0) *total = tot;
}

__global__ void k_tile_apply(const int* __restrict__ in, long n, const int* __restrict__ sums,
                             int* __restrict__ out) {
    __shared__ int sm[32];
    const long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; q++) {
        v[q] = (base + q < n) ? in[base + q] : 0;
        s += v[q];
    }
    int tot;
    int off = block_exclusive_scan(s, sm, &tot) + sums[blockIdx.x];
#pragma unroll
    for (int q = 0; q < kScanItems; q++) {
        if (base + q < n) out[base + q] = off;
        off += v[q];
    }
}

size_t scan_workspace_bytes(long n) {
    long nt = (n + kScanTile - 1) / kScanTile;
    return align_up(sizeof(int) * (size_t)(nt + 1), 256);
}

int exclusive_scan_dev(const int* in, int* out, long n, int* total, void* tmp, cudaStream_t s) {
    if (n <= 0) {
        CLOWNS_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(int), s));
        return CLOWNS_OK;
    }
    int nt = (int)((n + kScanTile - 1) / kScanTile);
    int* sums = (int*)tmp;
    k_tile_sums<<<nt, kScanThreads, 0, s>>>(in, n, sums);
    k_scan_sums<<<1, 1024, 0, s>>>(sums, nt, total);
    k_tile_apply<<<nt, kScanThreads, 0, s>>>(in, n, sums, out);
    CLOWNS_CUDA_TRY(cudaGetLastError());
    return CLOWNS_OK;
}

}  // namespace clowns
