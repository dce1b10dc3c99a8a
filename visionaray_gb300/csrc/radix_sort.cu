// Stable LSD radix sort of (key, value) pairs, 8-bit digits, one pass per digit.
//
// Replaces the CUB DeviceMergeSort::StableSortKeys call of visionaray's GPU LBVH
// (detail/bvh/lbvh.h:737-755), which also cudaMalloc/cudaFree'd its temporary storage
// on every build.  Only the order is observable: keys ascending, equal keys in input
// order (std::stable_sort semantics).  Per pass:
//   1. count_digits: per 4096-key tile, a shared-memory digit histogram written
//      digit-major (counts[d * tiles + tile]) so that one exclusive scan of the whole
//      table yields every (digit, tile) output offset in stable order.
//   2. three-phase exclusive scan of the table (tile sums, scan of sums, rescan).
//   3. scatter: each warp ranks its 512 keys in input order with __match_any_sync, the
//      tile is reordered by digit in shared memory, and every digit's run is written
//      out contiguously (coalesced) at its scanned offset.
// An odd number of passes ends in the alternate buffers: the result is copied back
// unless the caller asks where the sorted values are (sorted_values).

#include "api_internal.h"

namespace gbrt {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;                     // keys per thread
constexpr int kTile = kThreads * kItems;       // 4096 keys per tile
constexpr int kWarpKeys = 32 * kItems;         // 512 keys per warp
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kScanBlock = 1024;               // threads of the scan kernels
constexpr int kScanItems = 4;                  // entries per scan thread
constexpr int kScanChunk = kScanBlock * kScanItems;

__global__ void __launch_bounds__(kThreads) count_digits(const uint32_t* __restrict__ keys, uint32_t n,
                                                         int shift, uint32_t* __restrict__ counts,
                                                         uint32_t tiles)
{
    __shared__ uint32_t hist[kRadix];
    for (int d = threadIdx.x; d < kRadix; d += kThreads) hist[d] = 0;
    __syncthreads();
    const uint64_t base = uint64_t(blockIdx.x) * kTile;
    if (base + kTile <= n)
    {
        // a full tile: four 128-bit loads per thread, all issued before the first use
        // (tiles start at multiples of 4096 keys of a 256-byte aligned array)
        const uint4* k4 = reinterpret_cast<const uint4*>(keys + base);
        uint4 v[kItems / 4];
#pragma unroll
        for (int j = 0; j < kItems / 4; ++j) v[j] = __ldg(&k4[j * kThreads + threadIdx.x]);
#pragma unroll
        for (int j = 0; j < kItems / 4; ++j)
        {
            atomicAdd(&hist[(v[j].x >> shift) & (kRadix - 1)], 1u);
            atomicAdd(&hist[(v[j].y >> shift) & (kRadix - 1)], 1u);
            atomicAdd(&hist[(v[j].z >> shift) & (kRadix - 1)], 1u);
            atomicAdd(&hist[(v[j].w >> shift) & (kRadix - 1)], 1u);
        }
    }
    else
    {
#pragma unroll 4
        for (int k = 0; k < kItems; ++k)
        {
            uint64_t i = base + uint64_t(k) * kThreads + threadIdx.x;
            if (i < n)
            {
                uint32_t d = (__ldg(&keys[i]) >> shift) & (kRadix - 1);
                atomicAdd(&hist[d], 1u);
            }
        }
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += kThreads)
        counts[uint64_t(d) * tiles + blockIdx.x] = hist[d];
}

__device__ __forceinline__ uint32_t block_exclusive_scan_1024(uint32_t v, uint32_t* warp_sums,
                                                              uint32_t& total)
{
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        uint32_t s = warp_sums[lane];
        uint32_t t = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, t, o);
            if (lane >= o) t += y;
        }
        warp_sums[lane] = t - s;   // exclusive prefix of warp sums
        if (lane == 31) warp_sums[32] = t;
    }
    __syncthreads();
    uint32_t r = x - v + warp_sums[warp];
    total = warp_sums[32];
    __syncthreads();
    return r;
}

// Phase 1: sum of each kScanChunk-entry chunk.
__global__ void __launch_bounds__(kScanBlock) scan_chunk_sums(const uint32_t* __restrict__ in, uint64_t len,
                                                              uint32_t* __restrict__ sums)
{
    __shared__ uint32_t ws[33];
    uint64_t base = uint64_t(blockIdx.x) * kScanChunk + uint64_t(threadIdx.x) * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < len) s += in[base + k];
    uint32_t total;
    block_exclusive_scan_1024(s, ws, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Phase 2: exclusive scan of the chunk sums by one block (loops for long tables).
__global__ void __launch_bounds__(kScanBlock) scan_sums(uint32_t* __restrict__ sums, uint32_t count)
{
    __shared__ uint32_t ws[33];
    uint32_t carry = 0;
    for (uint32_t b = 0; b < count; b += kScanBlock)
    {
        uint32_t i = b + threadIdx.x;
        uint32_t v = i < count ? sums[i] : 0u;
        uint32_t total;
        uint32_t ex = block_exclusive_scan_1024(v, ws, total);
        if (i < count) sums[i] = ex + carry;
        carry += total;
    }
}

// Phase 3: exclusive scan within each chunk plus the chunk's offset, in place.
__global__ void __launch_bounds__(kScanBlock) scan_apply(uint32_t* __restrict__ data, uint64_t len,
                                                         const uint32_t* __restrict__ sums)
{
    __shared__ uint32_t ws[33];
    uint64_t base = uint64_t(blockIdx.x) * kScanChunk + uint64_t(threadIdx.x) * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
    {
        v[k] = base + k < len ? data[base + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t ex = block_exclusive_scan_1024(s, ws, total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
    {
        if (base + k < len) data[base + k] = ex;
        ex += v[k];
    }
}

// Resident blocks of the scatter kernel the register allocation must allow: 5 x 256
// threads at <= 48 registers (no spills; 5 x 43 KB of shared memory also fit).  The ranking keeps one packed word per item (rank within
// the warp's 512 keys in the low half, digit in the high half); keys and values are
// read again, from L1, when the tile is reordered.  Holding keys, values and ranks in
// registers through the block prefix took 111 registers (2 blocks per SM).
constexpr int kScatterMinBlocks = 5;

__global__ void __launch_bounds__(kThreads, kScatterMinBlocks) scatter_digits(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t n, int shift,
    const uint32_t* __restrict__ offsets, uint32_t tiles)
{
    __shared__ uint32_t warp_hist[kWarps][kRadix];
    __shared__ uint32_t digit_start[kRadix];   // exclusive start of each digit in the tile
    __shared__ uint32_t digit_out[kRadix];     // global output offset of each digit's run
    __shared__ uint32_t ws[33];
    __shared__ uint32_t skeys[kTile];
    __shared__ uint32_t svals[kTile];

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const uint64_t tile_base = uint64_t(blockIdx.x) * kTile;
    const uint64_t warp_base = tile_base + uint64_t(warp) * kWarpKeys;
    const uint32_t lanemask_lt = (1u << lane) - 1u;

    for (int d = lane; d < kRadix; d += 32) warp_hist[warp][d] = 0;
    __syncwarp();

    uint32_t packed[kItems];   // rank within the warp's keys | digit << 16
#pragma unroll
    for (int k = 0; k < kItems; ++k)
    {
        uint64_t i = warp_base + uint64_t(k) * 32 + lane;
        bool valid = i < n;
        // invalid items get a digit outside [0, kRadix) so they never match a real one
        uint32_t d = valid ? (__ldg(&keys_in[i]) >> shift) & (kRadix - 1) : uint32_t(kRadix);
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        uint32_t before = valid ? warp_hist[warp][d] : 0u;
        __syncwarp();
        if (valid && (peers & lanemask_lt) == 0) warp_hist[warp][d] = before + __popc(peers);
        __syncwarp();
        packed[k] = (before + __popc(peers & lanemask_lt)) | (d << 16);
    }
    __syncthreads();

    // Per digit: exclusive prefix over warps (stable: warp 0 first), then the tile's
    // exclusive prefix over digits.
    uint32_t digit_total = 0;
    {
        int d = threadIdx.x;   // kThreads == kRadix
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w)
        {
            uint32_t c = warp_hist[w][d];
            warp_hist[w][d] = run;
            run += c;
        }
        digit_total = run;
    }
    uint32_t tile_total;
    // kThreads == 256: reuse the 1024-thread scan helper shape with 8 warps
    {
        uint32_t x = digit_total;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0)
        {
            uint32_t s = lane < kWarps ? ws[lane] : 0u;
            uint32_t t = s;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                uint32_t y = __shfl_up_sync(0xFFFFFFFFu, t, o);
                if (lane >= o) t += y;
            }
            if (lane < kWarps) ws[lane] = t - s;
            if (lane == kWarps - 1) ws[32] = t;
        }
        __syncthreads();
        digit_start[threadIdx.x] = x - digit_total + ws[warp];
        tile_total = ws[32];
        digit_out[threadIdx.x] = offsets[uint64_t(threadIdx.x) * tiles + blockIdx.x];
    }
    __syncthreads();

#pragma unroll
    for (int k = 0; k < kItems; ++k)
    {
        uint64_t i = warp_base + uint64_t(k) * 32 + lane;
        if (i < n)
        {
            uint32_t d = packed[k] >> 16;
            uint32_t pos = digit_start[d] + warp_hist[warp][d] + (packed[k] & 0xFFFFu);
            skeys[pos] = __ldg(&keys_in[i]);
            svals[pos] = __ldg(&vals_in[i]);
        }
    }
    __syncthreads();

    for (uint32_t p = threadIdx.x; p < tile_total; p += kThreads)
    {
        uint32_t k = skeys[p];
        uint32_t d = (k >> shift) & (kRadix - 1);
        uint32_t dst = digit_out[d] + (p - digit_start[d]);
        keys_out[dst] = k;
        vals_out[dst] = svals[p];
    }
}

inline uint32_t num_tiles(uint32_t n) { return (n + kTile - 1) / kTile; }

} // namespace

size_t radix_sort_scratch_bytes(uint32_t n)
{
    uint64_t len = uint64_t(kRadix) * num_tiles(n);
    uint64_t chunks = (len + kScanChunk - 1) / kScanChunk;
    return size_t((len + chunks + 64) * sizeof(uint32_t));
}

gbrt_status radix_sort_pairs(gbrt_context* ctx, uint32_t* keys, uint32_t* values, uint32_t* keys_alt,
                             uint32_t* values_alt, uint32_t n, int key_bits, void* scratch, cudaStream_t stream,
                             uint32_t** sorted_values)
{
    if (n == 0) return GBRT_OK;
    const uint32_t tiles = num_tiles(n);
    const uint64_t len = uint64_t(kRadix) * tiles;
    const uint32_t chunks = uint32_t((len + kScanChunk - 1) / kScanChunk);
    uint32_t* counts = static_cast<uint32_t*>(scratch);
    uint32_t* sums = counts + len;

    uint32_t* kin = keys;
    uint32_t* vin = values;
    uint32_t* kout = keys_alt;
    uint32_t* vout = values_alt;
    int passes = (key_bits + kRadixBits - 1) / kRadixBits;
    for (int p = 0; p < passes; ++p)
    {
        int shift = p * kRadixBits;
        count_digits<<<tiles, kThreads, 0, stream>>>(kin, n, shift, counts, tiles);
        GBRT_LAUNCH_CHECK(ctx, "count_digits");
        scan_chunk_sums<<<chunks, kScanBlock, 0, stream>>>(counts, len, sums);
        GBRT_LAUNCH_CHECK(ctx, "scan_chunk_sums");
        scan_sums<<<1, kScanBlock, 0, stream>>>(sums, chunks);
        GBRT_LAUNCH_CHECK(ctx, "scan_sums");
        scan_apply<<<chunks, kScanBlock, 0, stream>>>(counts, len, sums);
        GBRT_LAUNCH_CHECK(ctx, "scan_apply");
        scatter_digits<<<tiles, kThreads, 0, stream>>>(kin, vin, kout, vout, n, shift, counts, tiles);
        GBRT_LAUNCH_CHECK(ctx, "scatter_digits");
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    if (sorted_values)
    {
        *sorted_values = vin;   // the caller takes the values where the last pass left them
        return GBRT_OK;
    }
    if (kin != keys)
    {
        GBRT_CUDA(ctx, cudaMemcpyAsync(keys, kin, size_t(n) * 4, cudaMemcpyDeviceToDevice, stream));
        GBRT_CUDA(ctx, cudaMemcpyAsync(values, vin, size_t(n) * 4, cudaMemcpyDeviceToDevice, stream));
    }
    return GBRT_OK;
}

} // namespace gbrt
