// k_generation.cu -- the fused generation pass: one warp builds one offspring
// row in a single sweep over the parent rows.
//
// Per row (gamete g of mate pair g/2, parent individual pairs[g]):
//   crossover  batch_crossover_taskwe<...population_space_row>::run_crossover_task
//              (crossover/batch_crossover_taskwe_population_space_row.hpp:157-217)
//              and block_crossover::crossover (crossover/block_crossover.hpp:46-63):
//              only heterozygous bits are classified; a bit takes the bottom
//              strand iff an odd number of breakpoints is <= its position
//              (region_classifier upper_bound, classifiers/region_classifier.hpp:62-77).
//              Fixed columns of the parent are masked on load, which is the
//              in-register form of remove_fixed_allele
//              (population_space_row_block.hpp:127-147, engine_batched_task.hpp:315-319).
//   mutation   XOR of the row's new alleles (population_space_row_block.hpp:111-125),
//              applied in registers before the store.
//   phenotype  per-genome FP32 sums of effects over set bits
//              (batch_phenotype_task_population_space_row.hpp:127-153).
//   free space AND/OR of the finished words into shared-memory accumulators,
//              folded into accF/accV, which are the next generation's
//              FreeSpaceAnalyzerMT input
//              (free_space_task_population_space_row_interlaced.hpp:51-72).
//
// Rows are 64-word chunks, 2 words (one 128-bit load) per lane.  The kernel is
// persistent: CTAs take 64-row items from a device counter.
#include "engine.cuh"

namespace clotho {

namespace {

constexpr uint32_t kWarps = kGenThreads / 32;

__device__ __forceinline__ uint32_t count_le_reg(uint64_t key, const uint64_t (&ev)[kMaxEvReg], uint32_t E) {
    uint32_t c = 0;
#pragma unroll
    for (uint32_t k = 0; k < kMaxEvReg; ++k) c += (k < E && ev[k] <= key) ? 1u : 0u;
    return c;
}

__device__ __forceinline__ uint32_t count_le_far(uint64_t key, const uint64_t* ev, uint32_t E) {
    uint32_t c = 0;
    for (uint32_t k = 0; k < E; ++k) c += (ev[k] <= key) ? 1u : 0u;
    return c;
}

// block_crossover::crossover on one word; base = slot index of bit 0.
__device__ __forceinline__ uint64_t xover_word(uint64_t t, uint64_t b, uint32_t base,
                                               const uint64_t* __restrict__ poskey,
                                               const uint64_t (&ev)[kMaxEvReg], uint32_t E,
                                               const uint64_t* ev_far) {
    uint64_t h = t ^ b, m = 0;
    if (E <= kMaxEvReg) {
        while (h) {
            const uint32_t j = (uint32_t)(__ffsll((long long)h) - 1);
            h &= h - 1ull;
            const uint64_t key = __ldg(poskey + base + j);
            m |= (uint64_t)(count_le_reg(key, ev, E) & 1u) << j;
        }
    } else {
        while (h) {
            const uint32_t j = (uint32_t)(__ffsll((long long)h) - 1);
            h &= h - 1ull;
            const uint64_t key = __ldg(poskey + base + j);
            m |= (uint64_t)(count_le_far(key, ev_far, E) & 1u) << j;
        }
    }
    return (t & ~m) | (b & m);
}

__device__ __forceinline__ void add_effects(uint64_t x, uint32_t base, const float* __restrict__ eff,
                                            uint32_t T, float (&acc)[kMaxTraits]) {
    if (T == 1) {
        while (x) {
            const uint32_t j = (uint32_t)(__ffsll((long long)x) - 1);
            x &= x - 1ull;
            acc[0] += __ldg(eff + base + j);
        }
    } else if (T == 4) {
        while (x) {
            const uint32_t j = (uint32_t)(__ffsll((long long)x) - 1);
            x &= x - 1ull;
            const float4 e = __ldg(reinterpret_cast<const float4*>(eff) + base + j);
            acc[0] += e.x; acc[1] += e.y; acc[2] += e.z; acc[3] += e.w;
        }
    } else {
        while (x) {
            const uint32_t j = (uint32_t)(__ffsll((long long)x) - 1);
            x &= x - 1ull;
            const float* e = eff + (size_t)(base + j) * T;
            for (uint32_t t = 0; t < T; ++t) acc[t] += __ldg(e + t);
        }
    }
}

}  // namespace

__global__ void __launch_bounds__(kGenThreads, 2)
k_generation(const PopDev* __restrict__ pops, uint32_t npops, WorkCtl* __restrict__ ctl, uint32_t fuse,
             int profile) {
    extern __shared__ uint64_t s_acc[];  // [2 * maxW]: AND then OR accumulators
    __shared__ uint64_t s_ev[kWarps][kMaxEvDevice];
    __shared__ uint32_t s_item;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const bool do_mut = (fuse & kFuseMut) != 0, do_ph = (fuse & kFusePheno) != 0, do_fs = (fuse & kFuseFs) != 0;
    int cur_pop = -1;
    uint32_t cur_W = 0, maxW_smem = 0;
    uint64_t* sF = s_acc;
    uint64_t* sV = nullptr;
    uint64_t rows_done = 0, words_done = 0;

    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(&ctl->gen_counter, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        __syncthreads();
        if (item >= ctl->gen_items) break;
        uint32_t p = 0;
        {
            uint32_t lo = 0, hi = npops;  // last p with item_base[p] <= item
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (ctl->item_base[mid] <= item) lo = mid; else hi = mid;
            }
            p = lo;
        }
        const PopDev& P = pops[p];
        const DevStatus st = *P.st;
        if ((int)p != cur_pop) {
            if (cur_pop >= 0 && do_fs) {
                const PopDev& Q = pops[cur_pop];
                for (uint32_t w = threadIdx.x; w < cur_W; w += blockDim.x) {
                    atomicAnd((unsigned long long*)&Q.accF[w], (unsigned long long)sF[w]);
                    atomicOr((unsigned long long*)&Q.accV[w], (unsigned long long)sV[w]);
                }
                __syncthreads();
            }
            cur_pop = (int)p;
            cur_W = st.W;
            maxW_smem = cur_W;
            sV = s_acc + maxW_smem;
            if (do_fs) {
                for (uint32_t w = threadIdx.x; w < cur_W; w += blockDim.x) { sF[w] = ~0ull; sV[w] = 0ull; }
            }
            __syncthreads();
        }

        const uint32_t S = 2u * st.N;
        const uint32_t Wc = st.W, Wp = st.pW;
        const uint64_t* prow = P.rows[st.cur ^ 1u];
        uint64_t* crow = P.rows[st.cur];
        const uint64_t* poskey = reinterpret_cast<const uint64_t*>(P.pos);
        const bool q1 = (P.flags & 1u) != 0;
        const bool philox = P.mode == kModePhilox;
        const uint32_t row0 = (item - ctl->item_base[p]) * kRowsPerItem + warp * (kRowsPerItem / kWarps);

        for (uint32_t rr = 0; rr < kRowsPerItem / kWarps; ++rr) {
            const uint32_t g = row0 + rr;
            if (g >= S) break;
            // ---- parent strands and events of gamete g
            uint32_t pind = P.pairs[g];
            if (pind >= st.pN) {
                if (lane == 0) atomicOr(&P.st->err, kErrParent);
                pind = 0;
            }
            const uint64_t* r0 = prow + (size_t)(2u * pind) * P.Wcap;
            const uint64_t* r1 = r0 + P.Wcap;
            const uint32_t h = g & 1u;
            bool swap;
            uint32_t E;
            uint64_t ev[kMaxEvReg];
            const uint64_t* ev_far = nullptr;
            if (philox) {
                const U4 x = philox4x32(g, 0u, st.gen, kStreamGamete, P.seed);
                E = poisson_inv(u01(x.x, x.y), P.rho, P.exp_neg_rho);
                swap = u01(x.z, x.w) < P.bias;
                if (q1 && h) E = 0;
                if (E > kMaxEvDevice) {
                    if (lane == 0) atomicOr(&P.st->err, kErrEvents);
                    E = kMaxEvDevice;
                }
                // lane l draws events 2l, 2l+1 (and 64+2l, 65+2l)
                double d[4];
                {
                    const U4 a = philox4x32(g, 1u + lane, st.gen, kStreamGamete, P.seed);
                    d[0] = u01(a.x, a.y); d[1] = u01(a.z, a.w);
                    if (E > 64u) {
                        const U4 b = philox4x32(g, 33u + lane, st.gen, kStreamGamete, P.seed);
                        d[2] = u01(b.x, b.y); d[3] = u01(b.z, b.w);
                    } else {
                        d[2] = d[3] = 0.0;
                    }
                }
#pragma unroll
                for (uint32_t k = 0; k < kMaxEvReg; ++k) {
                    const double v = __shfl_sync(0xffffffffu, (k & 1u) ? d[1] : d[0], k >> 1);
                    ev[k] = dkey(v);
                }
                if (E > kMaxEvReg) {
                    for (uint32_t m = 0; m < 2; ++m)
                        for (uint32_t q = 0; q < 2; ++q) {
                            const uint32_t j = 64u * m + 2u * lane + q;
                            if (j < E) s_ev[warp][j] = dkey(d[2u * m + q]);
                        }
                    __syncwarp();
                    ev_far = s_ev[warp];
                }
            } else {
                swap = P.swap[g] != 0;
                const uint32_t e0 = P.ev_off[g], e1 = P.ev_off[g + 1u];
                E = (q1 && h) ? 0u : e1 - e0;
                const uint64_t* src = reinterpret_cast<const uint64_t*>(P.ev_pos) + e0;
                const uint64_t mine = (lane < E) ? __ldg(src + lane) : ~0ull;
#pragma unroll
                for (uint32_t k = 0; k < kMaxEvReg; ++k) ev[k] = __shfl_sync(0xffffffffu, mine, k);
                ev_far = src;
            }
            const uint64_t* top = swap ? r1 : r0;
            const uint64_t* bot = swap ? r0 : r1;
            uint64_t* out = crow + (size_t)g * P.Wcap;

            // ---- new mutations of this row (slot indices), lanes hold up to 32
            uint32_t mo = 0, mc = 0, my_slot = 0xffffffffu;
            if (do_mut) {
                mo = P.row_off[g];
                mc = P.row_off[g + 1u] - mo;
                if (lane < mc) {
                    const uint32_t i = mo + lane;
                    const uint32_t mi = philox ? i : P.row_mut[i];
                    my_slot = (mi < st.M) ? P.mut_slot[mi] : 0xffffffffu;
                }
            }

            float acc[kMaxTraits] = {0.f, 0.f, 0.f, 0.f};
            for (uint32_t w0 = 0; w0 < Wc; w0 += 64u) {
                const uint32_t w = w0 + 2u * lane;
                // XOR masks of this lane's two words from the row's new alleles;
                // the shuffles run with the whole warp converged.
                uint64_t mx0 = 0, mx1 = 0;
                if (do_mut && mc) {
                    const uint32_t lim = mc < 32u ? mc : 32u;
                    for (uint32_t j = 0; j < lim; ++j) {
                        const uint32_t s = __shfl_sync(0xffffffffu, my_slot, j);
                        if (s == 0xffffffffu) continue;
                        const uint32_t sw = s >> 6;
                        if (sw == w) mx0 ^= 1ull << (s & 63u);
                        else if (sw == w + 1u) mx1 ^= 1ull << (s & 63u);
                    }
                    for (uint32_t j = 32; j < mc; ++j) {  // rows with more than 32 new alleles
                        const uint32_t mi = philox ? mo + j : P.row_mut[mo + j];
                        if (mi >= st.M) continue;
                        const uint32_t s = P.mut_slot[mi];
                        if (s == 0xffffffffu) continue;
                        const uint32_t sw = s >> 6;
                        if (sw == w) mx0 ^= 1ull << (s & 63u);
                        else if (sw == w + 1u) mx1 ^= 1ull << (s & 63u);
                    }
                }
                if (w < Wc) {
                    uint64_t t0 = 0, t1 = 0, b0 = 0, b1 = 0;
                    if (w < Wp) {
                        const ulonglong2 fm = *reinterpret_cast<const ulonglong2*>(P.fixmask + w);
                        const ulonglong2 tt = __ldg(reinterpret_cast<const ulonglong2*>(top + w));
                        t0 = tt.x & ~fm.x; t1 = tt.y & ~fm.y;
                        if (E) {
                            const ulonglong2 bb = __ldg(reinterpret_cast<const ulonglong2*>(bot + w));
                            b0 = bb.x & ~fm.x; b1 = bb.y & ~fm.y;
                        }
                    }
                    uint64_t x0 = t0, x1 = t1;
                    if (E) {
                        x0 = xover_word(t0, b0, w * 64u, poskey, ev, E, ev_far);
                        x1 = xover_word(t1, b1, (w + 1u) * 64u, poskey, ev, E, ev_far);
                    }
                    x0 ^= mx0;
                    x1 ^= mx1;
                    *reinterpret_cast<ulonglong2*>(out + w) = make_ulonglong2(x0, x1);
                    if (do_ph) {
                        add_effects(x0, w * 64u, P.eff, P.T, acc);
                        add_effects(x1, (w + 1u) * 64u, P.eff, P.T, acc);
                    }
                    if (do_fs) {
                        atomicAnd((unsigned long long*)&sF[w], (unsigned long long)x0);
                        atomicAnd((unsigned long long*)&sF[w + 1u], (unsigned long long)x1);
                        atomicOr((unsigned long long*)&sV[w], (unsigned long long)x0);
                        atomicOr((unsigned long long*)&sV[w + 1u], (unsigned long long)x1);
                    }
                }
            }
            if (do_ph) {
#pragma unroll
                for (uint32_t t = 0; t < kMaxTraits; ++t) {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) acc[t] += __shfl_xor_sync(0xffffffffu, acc[t], o);
                }
                if (lane == 0) reinterpret_cast<float4*>(P.zg)[g] = make_float4(acc[0], acc[1], acc[2], acc[3]);
            }
            if (profile && lane == 0) { rows_done += 1; words_done += Wc; }
        }
    }
    if (cur_pop >= 0 && do_fs) {
        __syncthreads();
        const PopDev& Q = pops[cur_pop];
        for (uint32_t w = threadIdx.x; w < cur_W; w += blockDim.x) {
            atomicAnd((unsigned long long*)&Q.accF[w], (unsigned long long)sF[w]);
            atomicOr((unsigned long long*)&Q.accV[w], (unsigned long long)sV[w]);
        }
    }
    if (profile && lane == 0 && rows_done) {
        atomicAdd((unsigned long long*)&ctl->rows_done, (unsigned long long)rows_done);
        atomicAdd((unsigned long long*)&ctl->words_done, (unsigned long long)words_done);
    }
}

void launch_generation(const LaunchCfg& L, const PopDev* pops, uint32_t npops, WorkCtl* ctl, uint32_t maxW,
                       uint32_t fuse, int profile) {
    const size_t smem = 2ull * maxW * sizeof(uint64_t);
    static size_t configured = 0;
    if (smem > 48u * 1024u && smem > configured) {
        cudaFuncSetAttribute(k_generation, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = smem;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_generation, kGenThreads, smem);
    if (per_sm < 1) per_sm = 1;
    k_generation<<<L.num_sms * per_sm, kGenThreads, smem, L.stream>>>(pops, npops, ctl, fuse, profile);
}

// ---------------------------------------------------------------------------
// Standalone phenotype (staged API): BatchPhenotypeMT<...row>::updateHaploidGenomeWeights
// (batch_phenotype_mt_population_space_row.hpp:111-132), one warp per genome.
__global__ void __launch_bounds__(256) k_phenotype(const PopDev* __restrict__ pops, uint32_t npops) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t p = 0; p < npops; ++p) {
        const PopDev& P = pops[p];
        const DevStatus st = *P.st;
        const uint32_t S = 2u * st.N, W = st.W;
        const uint64_t* rows = P.rows[st.cur];
        for (uint32_t g = gw; g < S; g += nw) {
            float acc[kMaxTraits] = {0.f, 0.f, 0.f, 0.f};
            const uint64_t* r = rows + (size_t)g * P.Wcap;
            for (uint32_t w = 2u * lane; w < W; w += 64u) {
                const ulonglong2 x = *reinterpret_cast<const ulonglong2*>(r + w);
                add_effects(x.x, w * 64u, P.eff, P.T, acc);
                add_effects(x.y, (w + 1u) * 64u, P.eff, P.T, acc);
            }
#pragma unroll
            for (uint32_t t = 0; t < kMaxTraits; ++t) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc[t] += __shfl_xor_sync(0xffffffffu, acc[t], o);
            }
            if (lane == 0) reinterpret_cast<float4*>(P.zg)[g] = make_float4(acc[0], acc[1], acc[2], acc[3]);
        }
    }
}
void launch_phenotype(const LaunchCfg& L, const PopDev* pops, uint32_t npops) {
    k_phenotype<<<L.num_sms * 8, 256, 0, L.stream>>>(pops, npops);
}

}  // namespace clotho
