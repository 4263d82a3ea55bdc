// fl_bin.cu — counting-sort particle binning.
//
// Replaces the reference's mark.wgsl (histogram), sort_scan_block/spine/add.wgsl
// (exclusive scan) and sort_scatter.wgsl (cursor scatter).  The reference's GPU
// scatter claims slots with an atomic cursor, so its order inside a bucket is
// unspecified; this path produces the STABLE permutation of the reference's CPU
// mirror (app/crates/fluid-lab/src/lib.rs:1188-1211): the cursor scatter is
// followed by an in-bucket sort of particle indices.
//
//   k_bin_count    key per particle + warp-aggregated histogram (mark.wgsl:33-44)
//   k_scan_*       exclusive prefix sum of the histogram (lib.rs:1176-1184)
//   k_bin_scatter  warp-aggregated cursor claim, writes perm (sort_scatter.wgsl:47-53)
//   k_bin_fix*     sort each bucket's particle indices -> stable order
//   k_bin_gather   copy particles into bin order, flag stray particles
#include "fl_device.cuh"

namespace fl {

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__global__ void __launch_bounds__(256) k_bin_count(DevBufs b) {
    const DevParams P = *b.prm;
    const uint32_t n = P.n;
    const uint32_t lane = lane_id();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < n; i0 += stride) {
        const uint32_t p = i0 + lane;
        const bool valid = p < n;
        uint32_t key = 0xffffffffu;
        if (valid) {
            float4 pos = b.part_in[2 * (size_t)p];
            uint32_t kc[3];
            key = cell_key(P, pos, kc);
            b.keys[p] = key;
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        const uint32_t leader = __ffs(peers) - 1;
        if (valid && lane == leader) atomicAdd(&b.counts[key], (uint32_t)__popc(peers));
    }
}

// Block-wide exclusive scan of one value per thread (SCAN_THREADS threads).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (blockDim.x >> 5) ? s_warp[lane] : 0u;
        uint32_t ws = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, ws, o);
            if (lane >= (uint32_t)o) ws += y;
        }
        if (lane < (blockDim.x >> 5)) s_warp[lane] = ws - w;  // exclusive warp offsets
        if (lane == 31) *total = ws;
    }
    __syncthreads();
    return s_warp[warp] + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t* __restrict__ counts, uint32_t C,
                                                             uint32_t* __restrict__ spine) {
    __shared__ uint32_t s_warp[32];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++)
        if (base + i < C) sum += counts[base + i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if (lane_id() == 0) s_warp[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t w = s_warp[threadIdx.x];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
        if (threadIdx.x == 0) spine[blockIdx.x] = w;
    }
}

// One block scans the spine of per-tile totals in place (exclusive).
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_spine(uint32_t* __restrict__ spine, uint32_t nb) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_total;
    uint32_t carry = 0;
    for (uint32_t c0 = 0; c0 < nb; c0 += SCAN_THREADS) {
        const uint32_t idx = c0 + threadIdx.x;
        const uint32_t v = idx < nb ? spine[idx] : 0u;
        const uint32_t ex = block_exclusive_scan(v, s_warp, &s_total);
        if (idx < nb) spine[idx] = ex + carry;
        __syncthreads();
        carry += s_total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(const uint32_t* __restrict__ counts, uint32_t C,
                                                           const uint32_t* __restrict__ spine,
                                                           uint32_t* __restrict__ offsets,
                                                           uint32_t* __restrict__ cursor) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_total;
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        v[i] = base + i < C ? counts[base + i] : 0u;
        sum += v[i];
    }
    uint32_t run = block_exclusive_scan(sum, s_warp, &s_total) + spine[blockIdx.x];
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        if (base + i < C) {
            offsets[base + i] = run;
            cursor[base + i] = run;
        }
        run += v[i];
    }
}

__global__ void __launch_bounds__(256) k_bin_scatter(DevBufs b) {
    const uint32_t n = b.prm->n;
    const uint32_t lane = lane_id();
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (uint32_t i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < n; i0 += stride) {
        const uint32_t p = i0 + lane;
        const bool valid = p < n;
        const uint32_t key = valid ? b.keys[p] : 0xffffffffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        const uint32_t leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (valid && lane == leader) base = atomicAdd(&b.cursor[key], (uint32_t)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (valid) b.perm[base + __popc(peers & lt_mask)] = p;
    }
}

// In-bucket sort of small buckets in registers: Batcher's odd-even merge
// sort networks for 8 and 16 keys (19 and 63 comparators; each puts the
// smaller key at the lower index), checked for every 0/1 input (the 0-1
// principle).  Padding keys are 0xffffffff, above every particle index.
#define BIN_CX(i, j)                                  \
    {                                                 \
        const uint32_t lo_ = min(a[i], a[j]);         \
        const uint32_t hi_ = max(a[i], a[j]);         \
        a[i] = lo_;                                   \
        a[j] = hi_;                                   \
    }
__device__ __forceinline__ void sort8(uint32_t (&a)[16]) {
        BIN_CX(0, 1) BIN_CX(2, 3) BIN_CX(0, 2) BIN_CX(1, 3) BIN_CX(1, 2) BIN_CX(4, 5) BIN_CX(6, 7) BIN_CX(4, 6)
        BIN_CX(5, 7) BIN_CX(5, 6) BIN_CX(0, 4) BIN_CX(2, 6) BIN_CX(2, 4) BIN_CX(1, 5) BIN_CX(3, 7) BIN_CX(3, 5)
        BIN_CX(1, 2) BIN_CX(3, 4) BIN_CX(5, 6)
}
__device__ __forceinline__ void sort16(uint32_t (&a)[16]) {
        BIN_CX(0, 1) BIN_CX(2, 3) BIN_CX(0, 2) BIN_CX(1, 3) BIN_CX(1, 2) BIN_CX(4, 5) BIN_CX(6, 7) BIN_CX(4, 6)
        BIN_CX(5, 7) BIN_CX(5, 6) BIN_CX(0, 4) BIN_CX(2, 6) BIN_CX(2, 4) BIN_CX(1, 5) BIN_CX(3, 7) BIN_CX(3, 5)
        BIN_CX(1, 2) BIN_CX(3, 4) BIN_CX(5, 6) BIN_CX(8, 9) BIN_CX(10, 11) BIN_CX(8, 10) BIN_CX(9, 11) BIN_CX(9, 10)
        BIN_CX(12, 13) BIN_CX(14, 15) BIN_CX(12, 14) BIN_CX(13, 15) BIN_CX(13, 14) BIN_CX(8, 12) BIN_CX(10, 14) BIN_CX(10, 12)
        BIN_CX(9, 13) BIN_CX(11, 15) BIN_CX(11, 13) BIN_CX(9, 10) BIN_CX(11, 12) BIN_CX(13, 14) BIN_CX(0, 8) BIN_CX(4, 12)
        BIN_CX(4, 8) BIN_CX(2, 10) BIN_CX(6, 14) BIN_CX(6, 10) BIN_CX(2, 4) BIN_CX(6, 8) BIN_CX(10, 12) BIN_CX(1, 9)
        BIN_CX(5, 13) BIN_CX(5, 9) BIN_CX(3, 11) BIN_CX(7, 15) BIN_CX(7, 11) BIN_CX(3, 5) BIN_CX(7, 9) BIN_CX(11, 13)
        BIN_CX(1, 2) BIN_CX(3, 4) BIN_CX(5, 6) BIN_CX(7, 8) BIN_CX(9, 10) BIN_CX(11, 12) BIN_CX(13, 14)
}
#undef BIN_CX

// Sort small buckets (the networks above up to 16 keys, an insertion sort up
// to 32); queue large ones for k_bin_fix_big.
__global__ void __launch_bounds__(256) k_bin_fix(DevBufs b, uint32_t C) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const uint32_t n = b.counts[c];
    if (n < 2) return;
    const uint32_t off = b.offsets[c];
    if (n > 32) {
        const uint32_t slot = atomicAdd(&b.st->big_buckets, 1u);
        b.big_list[slot] = c;
        return;
    }
    if (n <= 16) {
        uint32_t k[16];
#pragma unroll
        for (uint32_t i = 0; i < 16; i++) k[i] = i < n ? b.perm[off + i] : 0xffffffffu;
        if (n <= 8) sort8(k);
        else sort16(k);
#pragma unroll
        for (uint32_t i = 0; i < 16; i++)
            if (i < n) b.perm[off + i] = k[i];
        return;
    }
    uint32_t a[32];
    for (uint32_t i = 0; i < n; i++) a[i] = b.perm[off + i];
    for (uint32_t i = 1; i < n; i++) {
        const uint32_t x = a[i];
        uint32_t j = i;
        while (j > 0 && a[j - 1] > x) {
            a[j] = a[j - 1];
            j--;
        }
        a[j] = x;
    }
    for (uint32_t i = 0; i < n; i++) b.perm[off + i] = a[i];
}

// One block per large bucket: bitonic sort in shared memory up to
// BIG_BUCKET_SMEM entries, else a rank pass through global memory (a bucket that
// large is > 500x the rest density; correct, quadratic in the bucket size).
__global__ void __launch_bounds__(1024) k_bin_fix_big(DevBufs b) {
    __shared__ uint32_t s[BIG_BUCKET_SMEM];
    const uint32_t nbig = b.st->big_buckets;
    for (uint32_t bi = blockIdx.x; bi < nbig; bi += gridDim.x) {
        const uint32_t c = b.big_list[bi];
        const uint32_t n = b.counts[c];
        const uint32_t off = b.offsets[c];
        if (n <= BIG_BUCKET_SMEM) {
            uint32_t size = 1;
            while (size < n) size <<= 1;
            for (uint32_t i = threadIdx.x; i < size; i += blockDim.x) s[i] = i < n ? b.perm[off + i] : 0xffffffffu;
            __syncthreads();
            for (uint32_t k = 2; k <= size; k <<= 1) {
                for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                    for (uint32_t i = threadIdx.x; i < size; i += blockDim.x) {
                        const uint32_t ixj = i ^ j;
                        if (ixj > i) {
                            const bool up = (i & k) == 0;
                            const uint32_t x = s[i], y = s[ixj];
                            if ((x > y) == up) {
                                s[i] = y;
                                s[ixj] = x;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) b.perm[off + i] = s[i];
            __syncthreads();
        } else {
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                const uint32_t v = b.perm[off + i];
                uint32_t rank = 0;
                for (uint32_t j = 0; j < n; j++) rank += b.perm[off + j] < v ? 1u : 0u;
                b.scratch_u32[off + rank] = v;
            }
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) b.perm[off + i] = b.scratch_u32[off + i];
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(256) k_bin_gather(DevBufs b) {
    const DevParams P = *b.prm;
    const uint32_t n = P.n;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < n; d += stride) {
        const uint32_t src = b.perm[d];
        float4 pos = b.part_in[2 * (size_t)src];
        const float4 vel = b.part_in[2 * (size_t)src + 1];
        uint32_t kc[3];
        cell_key(P, pos, kc);
        const bool stray = is_stray(P, pos, kc);
        pos.w = stray ? 1.0f : 0.0f;
        b.part_sorted[2 * (size_t)d] = pos;
        b.part_sorted[2 * (size_t)d + 1] = vel;
        if (b.ids_in) b.ids_sorted[d] = b.ids_in[src];
        if (stray) {
            const uint32_t slot = atomicAdd(&b.st->strays, 1u);
            b.stray_list[slot] = d;
        }
    }
}

cudaError_t launch_bin(const DevBufs& b, const LaunchCfg& L, uint32_t C, uint32_t cap, cudaStream_t s) {
    (void)cap;
    const uint32_t nb = (C + SCAN_TILE - 1) / SCAN_TILE;
    k_bin_count<<<L.particle_blocks, 256, 0, s>>>(b);
    k_scan_reduce<<<nb, SCAN_THREADS, 0, s>>>(b.counts, C, b.spine);
    k_scan_spine<<<1, SCAN_THREADS, 0, s>>>(b.spine, nb);
    k_scan_down<<<nb, SCAN_THREADS, 0, s>>>(b.counts, C, b.spine, b.offsets, b.cursor);
    k_bin_scatter<<<L.particle_blocks, 256, 0, s>>>(b);
    k_bin_fix<<<(C + 255) / 256, 256, 0, s>>>(b, C);
    k_bin_fix_big<<<L.num_sms, 1024, 0, s>>>(b);
    k_bin_gather<<<L.particle_blocks, 256, 0, s>>>(b);
    return cudaGetLastError();
}

}  // namespace fl
