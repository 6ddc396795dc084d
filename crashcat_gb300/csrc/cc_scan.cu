// Device-wide exclusive scan and stable LSD radix sort (64-bit keys, int
// values) used by the broadphase and island construction.  Both are written
// for this project: tiles of 4096 elements per CTA, three launches per scan
// and per radix pass.
#include "cc_internal.cuh"

namespace cc {

// SM count of the current device, read once per device (a benign race: every writer stores the
// same value); 152 when the attribute cannot be read
int device_sm_count() {
    constexpr int MAX_DEVICES = 64;
    static int cached[MAX_DEVICES] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return 152;
    int v = cached[dev];
    if (v > 0) return v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
    cached[dev] = v;
    return v;
}

constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

__device__ __forceinline__ int warp_incl_scan(int v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// exclusive block scan of one value per thread; returns exclusive prefix, writes block total
__device__ int block_excl_scan(int v, int *total) {
    __shared__ int warp_sums[32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = warp_incl_scan(v);
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int nw = (blockDim.x + 31) >> 5;
        int s = lane < nw ? warp_sums[lane] : 0;
        int si = warp_incl_scan(s);
        if (lane < nw) warp_sums[lane] = si - s;
        if (lane == nw - 1 && total) *total = si;
    }
    __syncthreads();
    int r = warp_sums[wid] + inc - v;
    __syncthreads();
    return r;
}

__global__ void k_scan_reduce(const int *in, int n, int *block_sums) {
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int i = base + k;
        if (i < n) s += in[i];
    }
    __shared__ int tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

__global__ void k_scan_blocks(int *block_sums, int nb, int *total) {
    // single CTA scans up to SCAN_TILE block sums
    int base = threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = (base + k < nb) ? block_sums[base + k] : 0;
        s += v[k];
    }
    __shared__ int tot;
    int off = block_excl_scan(s, &tot);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < nb) block_sums[base + k] = off;
        off += v[k];
    }
    if (threadIdx.x == 0 && total) *total = tot;
}

__global__ void k_scan_apply(const int *in, int *out, int n, const int *block_offsets) {
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        s += v[k];
    }
    int off = block_excl_scan(s, nullptr) + block_offsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n) out[base + k] = off;
        off += v[k];
    }
}

size_t scan_tmp_ints(int n) {
    size_t nb = (size_t)(n + SCAN_TILE - 1) / SCAN_TILE + 1;
    // radix histograms: 256 digits x blocks of 4096 keys
    size_t rb = (size_t)(n + 4095) / 4096 + 1;
    size_t need = rb * 256 + 64;
    return (nb > need ? nb : need) + 64;
}

// out[i] = sum in[0..i-1]; *total = sum of all (device pointer, may be null)
void exclusive_scan_int(const int *in, int *out, int n, int *total, int *tmp, cudaStream_t s) {
    if (n <= 0) return;
    int nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_reduce<<<nb, SCAN_BLOCK, 0, s>>>(in, n, tmp);
    k_scan_blocks<<<1, SCAN_BLOCK, 0, s>>>(tmp, nb, total);
    k_scan_apply<<<nb, SCAN_BLOCK, 0, s>>>(in, out, n, tmp);
}

// ---------------------------------------------------------------------------
// radix sort
// ---------------------------------------------------------------------------
constexpr int RS_BLOCK = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_BLOCK * RS_ITEMS;  // 4096 keys per CTA

__global__ void k_radix_hist(const unsigned long long *keys, int n, int shift, int *hist, int nblocks) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int base = blockIdx.x * RS_TILE;
    for (int k = 0; k < RS_ITEMS; k++) {
        int i = base + k * RS_BLOCK + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255], 1);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// stable scatter: chunks of 256 keys processed in order; within a chunk the
// rank among equal digits follows thread order (warp match + popc, then warps
// in order).
__global__ void k_radix_scatter(const unsigned long long *keys, const int *vals, unsigned long long *okeys,
                                int *ovals, int n, int shift, const int *hist_off, int nblocks) {
    __shared__ int running[256];
    __shared__ int wcount[RS_BLOCK / 32][256];
    int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    running[tid] = hist_off[tid * nblocks + blockIdx.x];
    int base = blockIdx.x * RS_TILE;
    for (int k = 0; k < RS_ITEMS; k++) {
#pragma unroll
        for (int w = 0; w < RS_BLOCK / 32; w++) wcount[w][tid] = 0;
        __syncthreads();
        int i = base + k * RS_BLOCK + tid;
        bool valid = i < n;
        unsigned long long key = valid ? keys[i] : 0ull;
        int d = valid ? (int)((key >> shift) & 255) : 256 + lane;  // invalid lanes never match valid ones
        unsigned peers = __match_any_sync(0xffffffffu, d);
        unsigned lt = (1u << lane) - 1u;
        int rank = __popc(peers & lt);
        int leader = __ffs(peers) - 1;
        if (valid && lane == leader) wcount[wid][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            int off = running[d];
            for (int w = 0; w < wid; w++) off += wcount[w][d];
            off += rank;
            okeys[off] = key;
            ovals[off] = vals[i];
        }
        __syncthreads();
        int add = 0;
#pragma unroll
        for (int w = 0; w < RS_BLOCK / 32; w++) add += wcount[w][tid];
        running[tid] += add;
        __syncthreads();
    }
}

// Sorts (keys, vals) by the low `bits` bits of the keys; result ends in keys/vals.
// ints of scratch radix_sort_pairs_u64 needs for n keys
size_t radix_tmp_ints(int n) {
    size_t nblocks = (size_t)(n + RS_TILE - 1) / RS_TILE;
    return nblocks * 256 + 32 + scan_tmp_ints((int)(nblocks * 256));
}

void radix_sort_pairs_u64(unsigned long long *keys, unsigned long long *keys_alt, int *vals, int *vals_alt, int n,
                          int bits, int *tmp, cudaStream_t s, const int *) {
    if (n <= 1) return;
    int nblocks = (n + RS_TILE - 1) / RS_TILE;
    int passes = (bits + 7) / 8;
    if (passes & 1) passes++;  // even number of passes leaves the result in the primary buffers
    int *hist = tmp;
    int *scan_tmp = tmp + (size_t)nblocks * 256 + 32;
    unsigned long long *ki = keys, *ko = keys_alt;
    int *vi = vals, *vo = vals_alt;
    for (int p = 0; p < passes; p++) {
        int shift = p * 8;
        k_radix_hist<<<nblocks, RS_BLOCK, 0, s>>>(ki, n, shift, hist, nblocks);
        exclusive_scan_int(hist, hist, nblocks * 256, nullptr, scan_tmp, s);
        k_radix_scatter<<<nblocks, RS_BLOCK, 0, s>>>(ki, vi, ko, vo, n, shift, hist, nblocks);
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
}

}  // namespace cc
