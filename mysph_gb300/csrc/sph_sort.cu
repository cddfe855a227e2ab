// sph_sort.cu — stable LSD radix sort of (cell key, particle index) pairs and
// an exclusive scan, the two primitives of the cell hash.
//
// The reference builds its background grid serially with per-cell index
// lists appended in particle order (src/NNPS/asymmetricSearch.f90:49-158).
// Here the same ordering — by cell, ties by ascending particle index — comes
// from a stable radix sort: 8-bit digits, as many passes as the key needs,
// each pass = per-tile digit histogram (upsweep), one exclusive scan over
// (digit, tile) counts, and a stable scatter (downsweep) whose in-tile ranks
// come from warp match/ballot instead of per-thread counters.
#include <cstdint>
#include <mutex>
#include <cuda_runtime.h>

#include "../../include/sph_gpu.h"
#include "sph_internal.h"

namespace sph {
namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_BINS = 256;

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---- scan -------------------------------------------------------------------
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total.
__device__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t wtot;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    uint32_t inc = warp_incl_scan(v, lane);
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nwarps ? wsum[lane] : 0;
        uint32_t wi = warp_incl_scan(w, lane);
        if (lane < nwarps) wsum[lane] = wi - w;
        if (lane == nwarps - 1) wtot = wi;
    }
    __syncthreads();
    uint32_t out = inc - v + wsum[warp];
    *total = wtot;
    __syncthreads();
    return out;
}

__global__ void scan_reduce_kernel(const uint32_t* __restrict__ in, int64_t n, uint32_t* __restrict__ partials) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < n) s += in[base + k];
    uint32_t tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) partials[blockIdx.x] = tot;
}

// single block: exclusive scan of the per-tile partials (count <= SCAN_TILE)
__global__ void scan_partials_kernel(uint32_t* partials, int64_t count) {
    uint32_t v[SCAN_ITEMS];
    int64_t base = (int64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = base + k < count ? partials[base + k] : 0;
        s += v[k];
    }
    uint32_t tot;
    uint32_t run = block_excl_scan(s, &tot);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < count) partials[base + k] = run;
        run += v[k];
    }
}

// single block, n <= SCAN_THREADS * SCAN1_ITEMS: the whole exclusive scan in
// one launch (small systems' cell starts, small sort histograms).  In place
// is allowed: each thread reads its values before the block synchronises.
constexpr int SCAN1_ITEMS = 16;
__global__ void __launch_bounds__(SCAN_THREADS) scan_single_kernel(const uint32_t* in, uint32_t* out, int64_t n) {
    const int64_t base = (int64_t)threadIdx.x * SCAN1_ITEMS;
    uint32_t v[SCAN1_ITEMS];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN1_ITEMS; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    uint32_t tot;
    uint32_t run = block_excl_scan(s, &tot);
#pragma unroll
    for (int k = 0; k < SCAN1_ITEMS; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

__global__ void scan_down_kernel(const uint32_t* in, uint32_t* out, int64_t n,
                                 const uint32_t* __restrict__ partials) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    uint32_t tot;
    uint32_t run = block_excl_scan(s, &tot) + partials[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

// ---- radix sort ------------------------------------------------------------
__global__ void __launch_bounds__(RS_THREADS)
rs_upsweep(const uint32_t* __restrict__ keys, int64_t n, int shift, uint32_t mask,
           uint32_t* __restrict__ hist) {
    __shared__ uint32_t cnt[RS_BINS];
    for (int b = threadIdx.x; b < RS_BINS; b += RS_THREADS) cnt[b] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int k = 0; k < RS_ITEMS; ++k) {
        int64_t idx = base + (int64_t)k * RS_THREADS + threadIdx.x;
        bool valid = idx < n;
        uint32_t dig = valid ? (keys[idx] >> shift) & mask : 0x100u + lane;
        unsigned peers = __match_any_sync(0xffffffffu, dig);
        if (valid && lane == __ffs(peers) - 1) atomicAdd(&cnt[dig], (uint32_t)__popc(peers));
    }
    __syncthreads();
    for (int b = threadIdx.x; b < RS_BINS; b += RS_THREADS) hist[(int64_t)b * gridDim.x + blockIdx.x] = cnt[b];
}

__global__ void __launch_bounds__(RS_THREADS)
rs_downsweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
             uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int64_t n, int shift,
             uint32_t mask, const uint32_t* __restrict__ hist) {
    __shared__ uint32_t base[RS_BINS];
    __shared__ uint32_t run[RS_BINS];
    __shared__ uint32_t wcnt[RS_WARPS][RS_BINS];
    __shared__ uint32_t woff[RS_WARPS][RS_BINS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b = threadIdx.x; b < RS_BINS; b += RS_THREADS) {
        base[b] = hist[(int64_t)b * gridDim.x + blockIdx.x];
        run[b] = 0;
        for (int w = 0; w < RS_WARPS; ++w) wcnt[w][b] = 0;
    }
    __syncthreads();
    const int64_t tile = (int64_t)blockIdx.x * RS_TILE;
    const unsigned lt = lanemask_lt();
    for (int r = 0; r < RS_ITEMS; ++r) {
        int64_t idx = tile + (int64_t)r * RS_THREADS + threadIdx.x;
        bool valid = idx < n;
        uint32_t key = valid ? keys_in[idx] : 0u;
        uint32_t val = valid ? vals_in[idx] : 0u;
        uint32_t dig = valid ? (key >> shift) & mask : 0x100u + lane;
        unsigned peers = __match_any_sync(0xffffffffu, dig);
        uint32_t rank = __popc(peers & lt);
        if (valid && lane == __ffs(peers) - 1) wcnt[warp][dig] = __popc(peers);
        __syncthreads();
        for (int b = threadIdx.x; b < RS_BINS; b += RS_THREADS) {
            uint32_t s = run[b];
#pragma unroll
            for (int w = 0; w < RS_WARPS; ++w) {
                uint32_t t = wcnt[w][b];
                wcnt[w][b] = 0;
                woff[w][b] = s;
                s += t;
            }
            run[b] = s;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = base[dig] + woff[warp][dig] + rank;
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
    }
}

// ---- small sorts: every digit pass in one block ---------------------------
// For n <= SS_MAX (small systems) the passes of the same stable LSD sort run
// in one block of SS_THREADS: per pass a shared histogram, its exclusive
// scan, then rounds of SS_THREADS consecutive items scattered in order (rank
// among equal digits from warp match, then per-warp offsets in warp order),
// so the order is the multi-block sort's.  Passes hand over through global
// memory, ordered by __syncthreads within the block (plain loads, no
// read-only cache).
constexpr int SS_THREADS = 512;
constexpr int SS_WARPS = SS_THREADS / 32;
constexpr int64_t SS_MAX = 16384;

__global__ void __launch_bounds__(SS_THREADS)
rs_small_kernel(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                uint32_t* keys_alt, uint32_t* vals_alt, int n, int key_bits) {
    __shared__ uint32_t cnt[RS_BINS];
    __shared__ uint32_t run[RS_BINS];
    __shared__ uint32_t wcnt[SS_WARPS][RS_BINS];
    __shared__ uint32_t woff[SS_WARPS][RS_BINS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = lanemask_lt();
    const int passes = (key_bits + 7) / 8;
    const uint32_t* ki = keys_in;
    const uint32_t* vi = vals_in;
    for (int ps = 0; ps < passes; ++ps) {
        const bool to_out = ((passes - ps) % 2) == 1;   // the last pass lands in *_out
        uint32_t* ko = to_out ? keys_out : keys_alt;
        uint32_t* vo = to_out ? vals_out : vals_alt;
        const int shift = ps * 8;
        const int bits = key_bits - shift < 8 ? key_bits - shift : 8;
        const uint32_t mask = (1u << bits) - 1u;
        for (int b = threadIdx.x; b < RS_BINS; b += SS_THREADS) cnt[b] = 0;
        for (int k = threadIdx.x; k < SS_WARPS * RS_BINS; k += SS_THREADS) wcnt[k / RS_BINS][k % RS_BINS] = 0;
        __syncthreads();
        for (int idx = threadIdx.x; idx < n; idx += SS_THREADS) atomicAdd(&cnt[(ki[idx] >> shift) & mask], 1u);
        __syncthreads();
        if (warp == 0) {   // exclusive scan of the 256 bins, 8 per lane
            uint32_t v[RS_BINS / 32];
            uint32_t sum = 0;
#pragma unroll
            for (int k = 0; k < RS_BINS / 32; ++k) {
                v[k] = cnt[lane * (RS_BINS / 32) + k];
                sum += v[k];
            }
            uint32_t ex = warp_incl_scan(sum, lane) - sum;
#pragma unroll
            for (int k = 0; k < RS_BINS / 32; ++k) {
                run[lane * (RS_BINS / 32) + k] = ex;
                ex += v[k];
            }
        }
        __syncthreads();
        for (int base = 0; base < n; base += SS_THREADS) {
            const int idx = base + (int)threadIdx.x;
            const bool valid = idx < n;
            const uint32_t key = valid ? ki[idx] : 0u;
            const uint32_t val = valid ? vi[idx] : 0u;
            const uint32_t dig = valid ? (key >> shift) & mask : 0x100u + lane;
            const unsigned peers = __match_any_sync(0xffffffffu, dig);
            const uint32_t rank = __popc(peers & lt);
            if (valid && lane == __ffs(peers) - 1) wcnt[warp][dig] = __popc(peers);
            __syncthreads();
            for (int b = threadIdx.x; b < RS_BINS; b += SS_THREADS) {
                uint32_t sum = run[b];
                for (int w = 0; w < SS_WARPS; ++w) {
                    const uint32_t t = wcnt[w][b];
                    wcnt[w][b] = 0;
                    woff[w][b] = sum;
                    sum += t;
                }
                run[b] = sum;
            }
            __syncthreads();
            if (valid) {
                const uint32_t pos = woff[warp][dig] + rank;
                ko[pos] = key;
                vo[pos] = val;
            }
        }
        __syncthreads();
        ki = ko;
        vi = vo;
    }
}

constexpr int64_t align256(int64_t b) { return (b + 255) & ~(int64_t)255; }

// uint32 words of scan partials for n values: one per tile of SCAN_TILE
// values, and, when there are more tiles than one block scans, the partials
// of the scan over those (any n below 2^31 needs at most three levels).
constexpr int64_t scan_partials_c(int64_t n) {
    return (n + SCAN_TILE - 1) / SCAN_TILE <= SCAN_TILE
               ? (n + SCAN_TILE - 1) / SCAN_TILE + 1
               : (n + SCAN_TILE - 1) / SCAN_TILE + scan_partials_c((n + SCAN_TILE - 1) / SCAN_TILE);
}

// Bytes of sort scratch for n pairs: [keys_alt][vals_alt][hist][scan partials].
constexpr int64_t scratch_bytes_c(int64_t n) {
    return align256(n * 4) * 2 + align256(RS_BINS * ((n + RS_TILE - 1) / RS_TILE) * 4) +
           align256(scan_partials_c(RS_BINS * ((n + RS_TILE - 1) / RS_TILE)) * 4);
}

// Fixed scratch of the allocation-free sort.  Its name is a host-side
// stand-in in host code; the device address comes from cudaGetSymbolAddress.
constexpr int64_t kNoAllocBytes = scratch_bytes_c(SPH_NOALLOC_MAX_PAIRS);
static_assert(kNoAllocBytes == 8651008, "the documented size of the allocation-free sort's scratch");
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device, with that
// device current.  Outside a stream capture it is looked up on every call
// (a host-side lookup, no allocation), so an address made stale by a device
// reset (cudaDeviceReset) is replaced; a call whose stream is being captured
// uses the address of the device's last call outside capture, and fails with
// cudaErrorStreamCaptureUnsupported if there was none.
cudaError_t noalloc_scratch(cudaStream_t stream, void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) {
        (void)cudaGetLastError();
        cap = cudaStreamCaptureStatusActive;   // unknown: do not call into the runtime again
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = p;
    }
    if (!g_noalloc_ptr[dev]) return cudaErrorStreamCaptureUnsupported;
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

}  // namespace

int64_t scan_partials(int64_t n) { return scan_partials_c(n); }

// Three launches per level: tile sums, an exclusive scan of the tile sums
// (one block when they fit a block's tile, else the same scan one level
// up, on the partials after this level's), and the tile scans with their
// offsets.  The scan of level-2 partials runs in place: each thread reads its
// values before the block synchronises and writes them after.
void exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* partials,
                        cudaStream_t s, int64_t* launches) {
    if (n <= 0) return;
    if (n <= (int64_t)SCAN_THREADS * SCAN1_ITEMS) {
        scan_single_kernel<<<1, SCAN_THREADS, 0, s>>>(in, out, n);
        if (launches) *launches += 1;
        return;
    }
    int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    scan_reduce_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, partials);
    if (nb <= SCAN_TILE) {
        scan_partials_kernel<<<1, SCAN_THREADS, 0, s>>>(partials, nb);
        if (launches) *launches += 1;
    } else {
        exclusive_scan_u32(partials, partials, nb, partials + nb, s, launches);
    }
    scan_down_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n, partials);
    if (launches) *launches += 2;
}

// scratch: [keys_alt n][vals_alt n][hist 256*tiles][scan partials]
int64_t sort_scratch_bytes(int64_t n, int key_bits) {
    (void)key_bits;
    return scratch_bytes_c(n);
}

cudaError_t sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                       uint32_t* vals_out, int64_t n, int key_bits, void* scratch,
                       cudaStream_t s, int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    if (key_bits < 1) key_bits = 1;
    if (key_bits > 32) key_bits = 32;
    const int64_t tiles = (n + RS_TILE - 1) / RS_TILE;
    char* p = (char*)scratch;
    uint32_t* keys_alt = (uint32_t*)p; p += align256(n * 4);
    uint32_t* vals_alt = (uint32_t*)p; p += align256(n * 4);
    uint32_t* hist = (uint32_t*)p; p += align256(RS_BINS * tiles * 4);
    uint32_t* part = (uint32_t*)p;
    if (n <= SS_MAX) {
        rs_small_kernel<<<1, SS_THREADS, 0, s>>>(keys_in, vals_in, keys_out, vals_out, keys_alt, vals_alt, (int)n,
                                                key_bits);
        if (launches) *launches += 1;
        return cudaGetLastError();
    }
    const int passes = (key_bits + 7) / 8;
    const uint32_t* ki = keys_in;
    const uint32_t* vi = vals_in;
    for (int ps = 0; ps < passes; ++ps) {
        // the last pass must land in *_out: odd pass counts start there
        bool to_out = ((passes - ps) % 2) == 1;
        uint32_t* ko = to_out ? keys_out : keys_alt;
        uint32_t* vo = to_out ? vals_out : vals_alt;
        int shift = ps * 8;
        int bits = key_bits - shift < 8 ? key_bits - shift : 8;
        uint32_t mask = (bits >= 32) ? 0xffffffffu : ((1u << bits) - 1u);
        rs_upsweep<<<(unsigned)tiles, RS_THREADS, 0, s>>>(ki, n, shift, mask, hist);
        exclusive_scan_u32(hist, hist, RS_BINS * tiles, part, s, launches);
        rs_downsweep<<<(unsigned)tiles, RS_THREADS, 0, s>>>(ki, vi, ko, vo, n, shift, mask, hist);
        if (launches) *launches += 2;
        ki = ko;
        vi = vo;
    }
    return cudaGetLastError();
}

}  // namespace sph

extern "C" int64_t sph_sort_scratch_bytes(int64_t n, int32_t key_bits) {
    if (n < 0) return -1;
    return sph::sort_scratch_bytes(n, key_bits);
}

extern "C" int sph_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                              uint32_t* vals_out, int64_t n, int32_t key_bits, void* scratch,
                              int64_t scratch_bytes, void* stream) {
    if (n < 0 || (n > 0 && (!keys_in || !vals_in || !keys_out || !vals_out || !scratch)))
        return SPH_E_INVALID;
    if (n >= ((int64_t)1 << 31)) return SPH_E_INVALID;
    if (scratch_bytes < sph::sort_scratch_bytes(n, key_bits)) return SPH_E_INVALID;
    cudaError_t e = sph::sort_pairs(keys_in, vals_in, keys_out, vals_out, n, key_bits, scratch,
                                    (cudaStream_t)stream, nullptr);
    return e == cudaSuccess ? SPH_OK : SPH_E_CUDA;
}

// Allocation-free sort: the same passes as sph_sort_pairs on the library's
// fixed device scratch.  Nothing in the scratch has to start at zero: every
// pass writes its histogram and scan partials in full before reading them,
// and the alternate key/value buffers are written before they are read.
extern "C" int sph_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                                      uint32_t* vals_out, int64_t n, int32_t key_bits, void* stream) {
    if (n < 0 || (n > 0 && (!keys_in || !vals_in || !keys_out || !vals_out))) return SPH_E_INVALID;
    if (n > SPH_NOALLOC_MAX_PAIRS) return SPH_E_TOO_LARGE;
    void* scratch = nullptr;
    cudaError_t e = sph::noalloc_scratch((cudaStream_t)stream, &scratch);
    if (e != cudaSuccess) return SPH_E_CUDA;
    e = sph::sort_pairs(keys_in, vals_in, keys_out, vals_out, n, key_bits, scratch, (cudaStream_t)stream, nullptr);
    return e == cudaSuccess ? SPH_OK : SPH_E_CUDA;
}
