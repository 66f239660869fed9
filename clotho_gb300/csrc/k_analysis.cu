// k_analysis.cu -- pairwise differences between sampled sequences.
//
// The reference's statistic (association_matrix_pairwise_difference.hpp:75-120
// on the CPU, cuda/analysis/pairwise_difference_kernel.hpp:56-339 on its GPU
// path): for every pair i < j of a sample of rows, the number of allele slots
// where the two sequences differ, popcount(row_i XOR row_j); summarised by
// count, total, min, max, mean and variance (and, from the distances, the
// median).
//
// One CTA takes a 64 x 64 tile of the pair matrix (tiles on or above the
// diagonal only); the two row groups are staged 16 words at a time in shared
// memory and every thread accumulates a 4 x 4 block of pair distances.
#include "engine.cuh"

namespace clotho {

namespace {
constexpr uint32_t kTile = 64;    // rows per tile side
constexpr uint32_t kStageW = 16;  // words per stage
constexpr uint32_t kPad = kStageW + 1;
}  // namespace

__global__ void __launch_bounds__(256) k_pairwise(const PopDev* __restrict__ pops, uint32_t p,
                                                  const uint32_t* __restrict__ sample, uint32_t n,
                                                  uint32_t* __restrict__ dist, PairwiseOut* __restrict__ out) {
    __shared__ uint64_t sA[kTile][kPad];
    __shared__ uint64_t sB[kTile][kPad];
    __shared__ unsigned long long s_sum[8], s_sq[8], s_cnt[8];
    __shared__ unsigned int s_min[8], s_max[8];
    const PopDev& P = pops[p];
    const DevStatus* st = P.st;
    const uint32_t W = st->W;
    const uint64_t* rows = P.rows[st->cur];
    // tile (ti, tj), ti <= tj, from the linear block index
    const uint32_t T = (n + kTile - 1) / kTile;
    uint32_t b = blockIdx.x, ti = 0;
    while (b >= T - ti) {
        b -= T - ti;
        ++ti;
    }
    const uint32_t tj = ti + b;
    const uint32_t tx = threadIdx.x & 15u, ty = threadIdx.x >> 4;
    uint32_t acc[4][4] = {};
    for (uint32_t w0 = 0; w0 < W; w0 += kStageW) {
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < kTile * kStageW; e += blockDim.x) {
            const uint32_t r = e / kStageW, c = e % kStageW, w = w0 + c;
            const uint32_t ia = ti * kTile + r, ib = tj * kTile + r;
            sA[r][c] = (ia < n && w < W) ? rows[(size_t)sample[ia] * P.Wcap + w] : 0ull;
            sB[r][c] = (ib < n && w < W) ? rows[(size_t)sample[ib] * P.Wcap + w] : 0ull;
        }
        __syncthreads();
#pragma unroll 4
        for (uint32_t c = 0; c < kStageW; ++c) {
            uint64_t a[4], bb[4];
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k) {
                a[k] = sA[ty * 4u + k][c];
                bb[k] = sB[tx * 4u + k][c];
            }
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k)
#pragma unroll
                for (uint32_t l = 0; l < 4; ++l) acc[k][l] += (uint32_t)__popcll(a[k] ^ bb[l]);
        }
    }
    unsigned long long sum = 0, sq = 0, cnt = 0;
    unsigned int mn = 0xffffffffu, mx = 0;
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
#pragma unroll
        for (uint32_t l = 0; l < 4; ++l) {
            const uint32_t i = ti * kTile + ty * 4u + k, j = tj * kTile + tx * 4u + l;
            if (i < j && j < n) {
                const uint32_t d = acc[k][l];
                if (dist) {
                    const uint64_t at = (uint64_t)i * n - (uint64_t)i * (i + 1) / 2 + (j - i - 1);
                    dist[at] = d;
                }
                sum += d;
                sq += (unsigned long long)d * d;
                cnt += 1;
                mn = min(mn, d);
                mx = max(mx, d);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        sq += __shfl_xor_sync(0xffffffffu, sq, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_sum[warp] = sum;
        s_sq[warp] = sq;
        s_cnt[warp] = cnt;
        s_min[warp] = mn;
        s_max[warp] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (uint32_t i = 1; i < blockDim.x / 32u; ++i) {
            sum += s_sum[i];
            sq += s_sq[i];
            cnt += s_cnt[i];
            mn = min(mn, s_min[i]);
            mx = max(mx, s_max[i]);
        }
        if (cnt) {
            atomicAdd(&out->count, cnt);
            atomicAdd(&out->total, sum);
            atomicAdd(&out->sumsq, sq);
            atomicMin(&out->min, mn);
            atomicMax(&out->max, mx);
        }
    }
}

// Blocks: one per tile on or above the diagonal of the pair matrix.
void launch_pairwise(const LaunchCfg& L, const PopDev* pops, uint32_t p, const uint32_t* sample, uint32_t n,
                     uint32_t* dist, PairwiseOut* out) {
    const uint32_t T = (n + kTile - 1) / kTile;
    const uint32_t blocks = T * (T + 1) / 2;
    if (blocks)
        k_pairwise<<<blocks, 256, 0, L.stream>>>(pops, p, sample, n, dist, out);
}

}  // namespace clotho
