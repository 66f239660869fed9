// k_noalloc.cu -- free-space analysis of caller-owned rows that allocates no
// device memory.
//
// Some callers cannot call cudaMalloc: a host framework that owns every byte
// of device memory through its own pool, or a deployment that reserves its
// memory once at start-up and forbids allocation afterwards.  They still need
// the fixed/lost/free analysis of their population.  clotho_free_space_noalloc
// runs it on rows the caller passes (device pointers in, device pointers out)
// and keeps its working state -- the per-column AND and OR accumulators -- in
// the file-scope array below, which every GPU that loads this library holds
// until the process exits.
//
// Limits and rules of use:
//  * rows of at most kNoAllocMaxWords 64-bit words (A <= 1,048,576 alleles);
//    larger widths are rejected with CLOTHO_E_CAPACITY;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current); make that first call
//    before any stream capture (inside a capture it returns CLOTHO_E_STATE).
//    Later calls on a stream that is not capturing look it up again, so a
//    context made after cudaDeviceReset is followed;
//  * every call shares the one array and resets the accumulators it uses at
//    its start, so calls that overlap on the GPU (different streams, or
//    concurrent host threads without ordering) race: order them on one stream.
#include "engine.cuh"
#include "../../include/clotho_gpu.h"

#include <mutex>

namespace clotho {

constexpr uint32_t kNoAllocMaxWords = 16384;

// [0, max) AND accumulators, [max, 2*max) OR accumulators
static __device__ __align__(256) unsigned long long g_fs_scratch[2 * kNoAllocMaxWords];

namespace {

__global__ void k_na_reset(unsigned long long* acc, uint32_t W) {
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < W; w += gridDim.x * blockDim.x) {
        acc[w] = ~0ull;
        acc[kNoAllocMaxWords + w] = 0ull;
    }
}

// AND/OR over rows (free_space_task_population_space_row_interlaced.hpp:51-72)
__global__ void __launch_bounds__(256) k_na_reduce(const uint64_t* __restrict__ rows, uint32_t S, uint32_t stride,
                                                   uint32_t W, unsigned long long* acc) {
    const uint32_t groups = gridDim.y;
    const uint32_t per = (S + groups - 1) / groups;
    const uint32_t r0 = blockIdx.y * per, r1 = min(S, r0 + per);
    if (r0 >= r1) return;
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < W; w += gridDim.x * blockDim.x) {
        uint64_t f = ~0ull, v = 0ull;
        for (uint32_t r = r0; r < r1; ++r) {
            const uint64_t x = __ldg(rows + (size_t)r * stride + w);
            f &= x;
            v |= x;
        }
        atomicAnd(&acc[w], (unsigned long long)f);
        atomicOr(&acc[kNoAllocMaxWords + w], (unsigned long long)v);
    }
}

__device__ inline uint32_t na_block_scan(uint32_t v, uint32_t* s_warp, uint32_t& total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= (uint32_t)o) t += y;
        }
        s_warp[lane] = t;
    }
    __syncthreads();
    total = s_warp[31];
    const uint32_t excl = x - v + (warp ? s_warp[warp - 1] : 0u);
    __syncthreads();
    return excl;
}

// Tail padding and ordered compaction: fixed indices ascending, then lost
// indices ascending (free_space_mt_population_space_row_interlaced.hpp:52-81,
// free_space_details.hpp:299-357).  One CTA of 1024 threads.
__global__ void __launch_bounds__(1024) k_na_compact(const unsigned long long* acc, uint32_t W, uint32_t A,
                                                     uint32_t S, uint32_t* __restrict__ free_list,
                                                     uint32_t* __restrict__ counts) {
    __shared__ uint32_t s_warp[32];
    auto word = [&](uint32_t w, uint64_t& F, uint64_t& L) {
        if (w >= W) { F = 0; L = 0; return; }
        if (S == 0) { F = 0; L = ~0ull; return; }
        const uint32_t b = w * 64u;
        const uint64_t valid = (b + 64u <= A) ? ~0ull : (b >= A ? 0ull : ((1ull << (A - b)) - 1ull));
        F = acc[w] & valid;
        L = ~(acc[kNoAllocMaxWords + w] | ~valid);
    };
    uint32_t cf = 0, cl = 0;
    for (uint32_t w = threadIdx.x; w < W; w += 1024u) {
        uint64_t F, L;
        word(w, F, L);
        cf += __popcll(F);
        cl += __popcll(L);
    }
    uint32_t totF, totL;
    na_block_scan(cf, s_warp, totF);
    na_block_scan(cl, s_warp, totL);
    uint32_t base_f = 0, base_l = totF;
    for (uint32_t c = 0; c < W; c += 1024u) {
        const uint32_t w = c + threadIdx.x;
        uint64_t F, L;
        word(w, F, L);
        uint32_t tf, tl;
        const uint32_t of = na_block_scan(__popcll(F), s_warp, tf);
        const uint32_t ol = na_block_scan(__popcll(L), s_warp, tl);
        if (w < W) {
            uint32_t i = base_f + of;
            for (uint64_t b = F; b; b &= b - 1ull) free_list[i++] = w * 64u + (uint32_t)(__ffsll((long long)b) - 1);
            i = base_l + ol;
            for (uint64_t b = L; b; b &= b - 1ull) free_list[i++] = w * 64u + (uint32_t)(__ffsll((long long)b) - 1);
        }
        base_f += tf;
        base_l += tl;
    }
    if (threadIdx.x == 0) {
        counts[0] = totF;
        counts[1] = totL;
        counts[2] = totF + totL;
    }
}

// Device address of g_fs_scratch, per device.  It is looked up on the first
// call on a device and again on every call whose stream is not capturing, so
// a context made anew after cudaDeviceReset (which loads the module at a new
// address) is followed; a capturing stream uses the address found last.
constexpr int kMaxDevices = 64;
std::mutex g_na_mutex;
void* g_na_addr[kMaxDevices] = {};

int scratch_address(cudaStream_t stream, void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return CLOTHO_E_CUDA;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusActive;  // the legacy stream under another stream's global capture
    }
    std::lock_guard<std::mutex> g(g_na_mutex);
    if (!g_na_addr[dev] || cap == cudaStreamCaptureStatusNone) {
        if (cap != cudaStreamCaptureStatusNone) return CLOTHO_E_STATE;  // first call inside a capture
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_fs_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return CLOTHO_E_CUDA;
        }
        g_na_addr[dev] = p;
    }
    *out = g_na_addr[dev];
    return 0;
}

}  // namespace
}  // namespace clotho

extern "C" int clotho_free_space_noalloc(const uint64_t* rows, uint32_t S, uint32_t row_stride_words, uint32_t A,
                                         uint32_t* free_list, uint32_t* counts, void* stream) {
    using namespace clotho;
    if (!free_list || !counts) return CLOTHO_E_ARG;
    const uint32_t W = ref_width(A);
    if (W > kNoAllocMaxWords) return CLOTHO_E_CAPACITY;
    if (S > 0 && W > 0 && (!rows || row_stride_words < W)) return CLOTHO_E_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaGetLastError();  // an error left by earlier, unrelated work is not this call's
    if (A == 0) {  // nothing to analyse (free_space_mt_population_space_row_interlaced.hpp:46)
        if (cudaMemsetAsync(counts, 0, 3 * sizeof(uint32_t), st) != cudaSuccess) {
            cudaGetLastError();
            return CLOTHO_E_CUDA;
        }
        return 0;
    }
    void* addr = nullptr;
    int rc = scratch_address(st, &addr);
    if (rc) return rc;
    unsigned long long* acc = static_cast<unsigned long long*>(addr);
    k_na_reset<<<(W + 255) / 256, 256, 0, st>>>(acc, W);
    if (S > 0) {
        const uint32_t gx = (W + 255) / 256;
        uint32_t gy = 1024u / gx;
        if (gy > S) gy = S;
        if (gy < 1u) gy = 1u;
        k_na_reduce<<<dim3(gx, gy), 256, 0, st>>>(rows, S, row_stride_words, W, acc);
    }
    k_na_compact<<<1, 1024, 0, st>>>(acc, W, A, S, free_list, counts);
    if (cudaGetLastError() != cudaSuccess) return CLOTHO_E_CUDA;
    return 0;
}
