// k_step.cu -- the small per-generation kernels around the generation pass:
// step begin/end, mutation bookkeeping (slot resolution, per-row CSR), device
// draws (Philox), fitness-proportional parent sampling (FP64 prefix sum),
// per-individual phenotype + fitness, seeding and column statistics.
//
// All kernels walk every population of the batch; sizes are read from the
// device status words so a step needs no host synchronisation and can be
// captured in a CUDA graph.
#include "engine.cuh"

namespace clotho {

int init_recip_step() { return fill_recip_table(); }

namespace {
constexpr uint32_t kScanChunk = 4096;  // elements per scan chunk (1024 threads x 4)

__device__ inline uint32_t warp_incl_u32(uint32_t x) {
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    return x;
}
__device__ inline double warp_incl_f64(double x) {
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        double y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    return x;
}
}  // namespace

// ---------------------------------------------------------------------------
// Step begin: the child becomes the parent (engine_batched_task.hpp:164), the
// offspring count comes from the tape header / growth rule, and the item
// prefix of the generation kernel is rebuilt.
__global__ void k_begin(const PopDev* __restrict__ pops, uint32_t npops, const uint32_t* __restrict__ hdr,
                        WorkCtl* ctl) {
    const uint32_t p = threadIdx.x;
    __shared__ uint32_t s_items[kMaxPops];
    if (p < npops) {
        const PopDev& P = pops[p];
        DevStatus* st = P.st;
        uint32_t N = hdr[2 * p], M = hdr[2 * p + 1];
        if (N > P.Ncap) { st->err |= kErrAlleles; N = P.Ncap; }
        if (M > P.Mcap) { st->err |= kErrMut; M = P.Mcap; }
        st->pN = st->N;
        st->pA = st->A;
        st->pW = st->W;
        st->N = N;
        st->M = M;
        st->ev_used = 0;
        st->cur ^= 1u;
        const uint32_t rpi = ctl->rows_per_item ? ctl->rows_per_item : kRowsPerItem;
        s_items[p] = (2u * N + rpi - 1u) / rpi;
    }
    __syncthreads();
    if (p == 0) {
        uint32_t acc = 0;
        for (uint32_t q = 0; q < npops; ++q) {
            ctl->item_base[q] = acc;
            acc += s_items[q];
        }
        ctl->item_base[npops] = acc;
        ctl->gen_items = acc;
        ctl->gen_counter = 0;
        ctl->gen_counter_iv = 0;
        ctl->gen_counter_cm = 0;
    }
}

void launch_begin(const LaunchCfg& L, const PopDev* pops, uint32_t npops, const uint32_t* hdr, WorkCtl* ctl) {
    k_begin<<<1, kMaxPops, 0, L.stream>>>(pops, npops, hdr, ctl);
}

__global__ void k_end(const PopDev* __restrict__ pops, uint32_t npops) {
    const uint32_t p = threadIdx.x;
    if (p < npops) {
        DevStatus* st = pops[p].st;
        st->last_M = st->M;
        st->gen += 1u;  // ++m_generation (engine_batched_task.hpp:222)
    }
}
void launch_end(const LaunchCfg& L, const PopDev* pops, uint32_t npops) {
    k_end<<<1, kMaxPops, 0, L.stream>>>(pops, npops);
}

// ---------------------------------------------------------------------------
// Exclusive u32 scan of row_cnt[0..S] into row_off[0..S], chunked, per
// population.  Also zeroes row_cnt and row_cur for the next step.  When
// set_M is set, row_off[S] (the total) becomes the step's mutation count.
struct ScanSel {
    uint32_t* cnt;
    uint32_t* off;
    uint32_t* cur;
    uint32_t L;      // elements (counts) to scan; off gets L entries
    uint32_t ncur;   // cursors to zero
    uint32_t* part;  // chunk partials (the ordering scan has its own: it runs beside the other two)
};
// which == 0: per-row mutation counts; 1: position buckets; 2: rows per ordering key.  The ordering keys
// are parent individuals (below pN, which exceeds 2N when the population shrinks more than twofold) or, in
// the measurement orders, below 2N or N + pN: the scan covers max(2N, N + pN) keys, at most 2 * Ncap.
__device__ inline ScanSel scan_sel(const PopDev& P, int which) {
    if (which == 0) return ScanSel{P.row_cnt, P.row_off, P.row_cur, 2u * P.st->N + 1u, 2u * P.st->N, P.scan_upart};
    if (which == 2) {
        const uint32_t keys = max(2u * P.st->N, P.st->N + P.st->pN);
        return ScanSel{P.ord_cnt, P.ord_off, P.ord_cur, keys + 1u, keys, P.scan_opart};
    }
    return ScanSel{P.bcnt, P.boff, P.bcur, P.NB + 1u, P.NB, P.scan_upart};
}

__global__ void __launch_bounds__(1024) k_uscan_a(const PopDev* __restrict__ pops, uint32_t npops, int which) {
    __shared__ uint32_t s_w[32];
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        const ScanSel Z = scan_sel(P, which);
        if (!Z.cnt) continue;  // the ordering keys exist only with the suffix-table classifier
        const uint32_t L = Z.L;
        const uint32_t nch = (L + kScanChunk - 1) / kScanChunk;
        for (uint32_t c = blockIdx.x; c < nch; c += gridDim.x) {
            const uint32_t b = c * kScanChunk + threadIdx.x * 4u;
            uint32_t s = 0;
            for (uint32_t k = 0; k < 4; ++k) s += (b + k < L) ? Z.cnt[b + k] : 0u;
            s = warp_incl_u32(s);
            if ((threadIdx.x & 31u) == 31u) s_w[threadIdx.x >> 5] = s;
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t t = 0;
                for (int i = 0; i < 32; ++i) t += s_w[i];
                Z.part[c] = t;
            }
            __syncthreads();
        }
    }
}

__global__ void k_uscan_b(const PopDev* __restrict__ pops, uint32_t npops, int which) {
    const uint32_t p = blockIdx.x;
    if (p >= npops || threadIdx.x != 0) return;
    const PopDev& P = pops[p];
    const ScanSel Z = scan_sel(P, which);
    if (!Z.cnt) return;
    const uint32_t L = Z.L;
    const uint32_t nch = (L + kScanChunk - 1) / kScanChunk;
    uint32_t acc = 0;
    for (uint32_t c = 0; c < nch; ++c) {
        uint32_t t = Z.part[c];
        Z.part[c] = acc;
        acc += t;
    }
}

__global__ void __launch_bounds__(1024) k_uscan_c(const PopDev* __restrict__ pops, uint32_t npops, int which,
                                                  int set_M) {
    __shared__ uint32_t s_w[32];
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        const ScanSel Z = scan_sel(P, which);
        if (!Z.cnt) continue;
        const uint32_t S = Z.ncur, L = Z.L;
        const uint32_t nch = (L + kScanChunk - 1) / kScanChunk;
        for (uint32_t c = blockIdx.x; c < nch; c += gridDim.x) {
            const uint32_t b = c * kScanChunk + threadIdx.x * 4u;
            uint32_t v[4], s = 0;
            for (uint32_t k = 0; k < 4; ++k) {
                v[k] = (b + k < L) ? Z.cnt[b + k] : 0u;
                s += v[k];
            }
            const uint32_t incl = warp_incl_u32(s);
            if ((threadIdx.x & 31u) == 31u) s_w[threadIdx.x >> 5] = incl;
            __syncthreads();
            uint32_t woff = 0;
            for (uint32_t i = 0; i < (threadIdx.x >> 5); ++i) woff += s_w[i];
            uint32_t run = Z.part[c] + woff + incl - s;
            for (uint32_t k = 0; k < 4; ++k) {
                if (b + k < L) {
                    Z.off[b + k] = run;
                    Z.cnt[b + k] = 0u;
                    if (b + k < S) Z.cur[b + k] = 0u;
                    if (set_M && b + k == S) {
                        DevStatus* st = P.st;
                        if (run > P.Mcap) { st->err |= kErrMut; run = P.Mcap; }
                        st->M = run;
                    }
                }
                run += v[k];
            }
            __syncthreads();
        }
    }
}

static void launch_uscan(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxLen, int which,
                         int set_M) {
    const uint32_t nch = (maxLen + 1 + kScanChunk - 1) / kScanChunk;
    const dim3 g = pop_grid(npops, nch, L.num_sms, 2);
    k_uscan_a<<<g, 1024, 0, L.stream>>>(pops, npops, which);
    k_uscan_b<<<npops, 32, 0, L.stream>>>(pops, npops, which);
    k_uscan_c<<<g, 1024, 0, L.stream>>>(pops, npops, which, set_M);
}

void launch_uscan_buckets(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxNB) {
    launch_uscan(L, pops, npops, maxNB, 1, 0);
}
void launch_uscan_order(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxS) {
    launch_uscan(L, pops, npops, maxS, 2, 0);
}

// ---------------------------------------------------------------------------
// Tape mutations grouped by target row (device counting sort, then each row's
// list in ascending mutation index: the list order is the order in which the
// new alleles' FP32 effects enter the row's carried phenotype, so it must not
// depend on the order of the scatter's atomics).
__global__ void k_csr_count(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        DevStatus* st = P.st;
        const uint32_t M = st->M, S = 2u * st->N;
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
            const uint32_t s = P.mut_seq[i];
            if (s >= S) { atomicOr(&st->err, kErrSeq); continue; }
            atomicAdd(&P.row_cnt[s], 1u);
        }
    }
}
__global__ void k_csr_scatter(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        const uint32_t M = P.st->M, S = 2u * P.st->N;
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
            const uint32_t s = P.mut_seq[i];
            if (s >= S) continue;
            const uint32_t k = atomicAdd(&P.row_cur[s], 1u);
            P.row_mut[P.row_off[s] + k] = i;
        }
    }
}
// Ascending order of a[0..n): insertion sort for short lists, heapsort beyond
// (a tape may send many mutations to one row).
__device__ void sort_ascending(uint32_t* a, uint32_t n) {
    if (n <= 16u) {
        for (uint32_t i = 1; i < n; ++i) {
            const uint32_t x = a[i];
            uint32_t j = i;
            for (; j > 0 && a[j - 1] > x; --j) a[j] = a[j - 1];
            a[j] = x;
        }
        return;
    }
    auto sift = [a](uint32_t r, uint32_t end) {
        const uint32_t x = a[r];
        for (uint32_t c = 2u * r + 1u; c < end; c = 2u * r + 1u) {
            if (c + 1u < end && a[c + 1u] > a[c]) ++c;
            if (a[c] <= x) break;
            a[r] = a[c];
            r = c;
        }
        a[r] = x;
    };
    for (uint32_t r = n / 2u; r-- > 0;) sift(r, n);
    for (uint32_t end = n - 1u; end > 0; --end) {
        const uint32_t x = a[0];
        a[0] = a[end];
        a[end] = x;
        sift(0, end);
    }
}
// One thread per list position; the thread at a row's first position sorts the
// row's list.  Ownership is decided by position, which never moves, and every
// entry of a row's segment names that row, so no other thread acts on it.
__global__ void k_csr_order(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        const uint32_t S = 2u * P.st->N, listed = P.row_off[S];
        for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < listed; t += gridDim.x * blockDim.x) {
            const uint32_t s = P.mut_seq[P.row_mut[t]];
            const uint32_t off = P.row_off[s], n = P.row_off[s + 1u] - off;
            if (t == off && n >= 2u) sort_ascending(P.row_mut + off, n);
        }
    }
}
void launch_mut_csr_tape(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxS) {
    const dim3 g = pop_grid(npops, L.num_sms * 2u, L.num_sms, 2);
    k_csr_count<<<g, 256, 0, L.stream>>>(pops, npops);
    launch_uscan(L, pops, npops, maxS, 0, 0);
    k_csr_scatter<<<g, 256, 0, L.stream>>>(pops, npops);
    k_csr_order<<<g, 256, 0, L.stream>>>(pops, npops);
}

// Device-drawn mutation counts: Poisson(mu) per offspring row.  The sum over
// rows is Poisson(2N mu) and, given the total, the rows are uniform -- the
// same law as M ~ Poisson(mu * 2N) with uniform target rows
// (mutation_allocator.hpp:41-47, batch_mutation_task_population_space_row.hpp:77).
__global__ void k_philox_rowcnt(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        if (P.mode != kModePhilox) continue;
        const DevStatus* st = P.st;
        const uint32_t S = 2u * st->N, gen = st->gen;
        for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < S; r += gridDim.x * blockDim.x) {
            const U4 x = philox4x32(r, 0u, gen, kStreamMutCount, P.seed);
            P.row_cnt[r] = poisson_inv(u01(x.x, x.y), P.mu, P.exp_neg_mu);
        }
    }
}
void launch_mut_counts_philox(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxS) {
    k_philox_rowcnt<<<pop_grid(npops, blocks_for(maxS, 256), L.num_sms, 4), 256, 0, L.stream>>>(pops, npops);
    launch_uscan(L, pops, npops, maxS, 0, 1);
}

// ---------------------------------------------------------------------------
// Mutation i takes free_indices[i]; beyond the free list new slots are
// appended at the parent allele count (batch_mutation_mt.hpp:69-80).  Writes
// the allele table (AlleleGenerator, allele_generator_vector.hpp:76-83) and
// the trait table (TraitSpaceGenerator2, trait_space_generator.hpp:118-129).
__global__ void k_mut_resolve(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        DevStatus* st = P.st;
        const uint32_t M = st->M, fr = st->free_cnt, pA = st->pA, gen = st->gen, T = P.T;
        const uint32_t Alim = st->A;
        int nz_delta = 0;
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
            const uint32_t slot = (i < fr) ? P.free_list[i] : pA + (i - fr);
            if (slot >= Alim) { atomicOr(&st->err, kErrAlleles); P.mut_slot[i] = 0xffffffffu; continue; }
            P.mut_slot[i] = slot;
            double pos;
            float e[kMaxTraits];
            if (P.mode == kModePhilox) {
                const U4 x = philox4x32(i, 0u, gen, kStreamMutAllele, P.seed);
                pos = u01(x.x, x.y);
                for (uint32_t t = 0; t < T; ++t) {
                    const U4 a = philox4x32(i, 1u + t, gen, kStreamMutAllele, P.seed);
                    float w = 0.0f;
                    if (!(u01(a.x, a.y) < P.p_neutral)) {
                        // Box-Muller on two fresh uniforms, first in (0,1]
                        const double u1 = 1.0 - u01(a.z, a.w);
                        const U4 b = philox4x32(i, 1u + kMaxTraits + t, gen, kStreamMutAllele, P.seed);
                        const double u2 = u01(b.x, b.y);
                        const double n = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
                        w = (float)(P.eff_mean + P.eff_sigma * n);
                    }
                    e[t] = w;
                }
            } else {
                pos = P.mut_pos[i];
                for (uint32_t t = 0; t < T; ++t) e[t] = P.mut_eff[(size_t)i * T + t];
            }
            P.pos[slot] = pos;
            P.age[slot] = gen;
            for (uint32_t t = 0; t < T; ++t) {
                const float old = P.eff[(size_t)slot * 4u + t];
                nz_delta += (e[t] != 0.0f) - (old != 0.0f);
                P.eff[(size_t)slot * 4u + t] = e[t];
            }
        }
        if (nz_delta) atomicAdd(&st->nz_eff, nz_delta);
    }
}
void launch_mut_resolve(const LaunchCfg& L, const PopDev* pops, uint32_t npops) {
    k_mut_resolve<<<pop_grid(npops, L.num_sms * 2u, L.num_sms, 2), 256, 0, L.stream>>>(pops, npops);
}

// Standalone mutation scatter (staged API): child->mutate(seq, slot) is a
// single-bit XOR (population_space_row_block.hpp:111-125).
__global__ void k_mut_scatter(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        const DevStatus* st = P.st;
        const uint32_t M = st->M, S = 2u * st->N;
        uint64_t* rows = P.rows[st->cur];
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
            const uint32_t slot = P.mut_slot[i], s = P.mut_seq[i];
            if (slot == 0xffffffffu || s >= S) continue;
            atomicXor((unsigned long long*)&rows[(size_t)s * P.Wcap + (slot >> 6)], 1ull << (slot & 63u));
        }
    }
}
void launch_mut_scatter(const LaunchCfg& L, const PopDev* pops, uint32_t npops) {
    k_mut_scatter<<<pop_grid(npops, L.num_sms * 2u, L.num_sms, 2), 256, 0, L.stream>>>(pops, npops);
}

// ---------------------------------------------------------------------------
// Parent sampling on the device (SelectionGenerator::update,
// general_fitness_selection_generator.hpp:45-69): uniform when every fitness
// is equal, else the FP64 inclusive prefix sum and an upper_bound per draw.
__global__ void k_select_philox(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        const DevStatus* st = P.st;
        const uint32_t N = st->N, Np = st->pN, gen = st->gen;
        const bool uni = st->fit_const != 0u || !(st->fit_total > 0.0);
        const double total = st->fit_total;
        for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
            const U4 x = philox4x32(k, 0u, gen, kStreamSelect, P.seed);
            const double u[2] = {u01(x.x, x.y), u01(x.z, x.w)};
            for (int h = 0; h < 2; ++h) {
                uint32_t id;
                if (Np == 0) id = 0;
                else if (uni) {
                    id = (uint32_t)(u[h] * (double)Np);
                    if (id >= Np) id = Np - 1u;
                } else {
                    const double target = u[h] * total;
                    uint32_t lo = 0, hi = Np;  // first i with cdf[i] > target (both >= +0: integer compares)
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (lt_nonneg(target, P.cdf[mid])) hi = mid; else lo = mid + 1u;
                    }
                    id = lo >= Np ? Np - 1u : lo;
                }
                P.pairs[2u * k + h] = id;
            }
        }
    }
}
void launch_select_philox(const LaunchCfg& L, const PopDev* pops, uint32_t npops) {
    k_select_philox<<<pop_grid(npops, L.num_sms * 2u, L.num_sms, L.ind_per_sm), 256, 0, L.stream>>>(pops, npops);
}

// ---------------------------------------------------------------------------
// Individual phenotype = genome 0 + genome 1 (individual_reducer_task_population_space_row.hpp:51-79),
// or the constant 1.0 when every trait weight is zero (engine_batched_task.hpp:207-211);
// then the fitness metric (GeneralFitness::operator(), general_fitness.hpp:101-119).
__global__ void k_individuals(const PopDev* __restrict__ pops, uint32_t npops) {
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        DevStatus* st = P.st;
        const uint32_t N = st->N, T = P.T;
        const bool neutral = st->nz_eff == 0;
        if (blockIdx.x == 0 && threadIdx.x == 0) st->all_neutral = neutral ? 1u : 0u;
        const double sig = sqrt(4.0 * (double)N * P.mu);  // normal/quadratic generators
        const double* zg = P.zg[st->cur];
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
            double z[4];
            for (uint32_t t = 0; t < 4; ++t) {
                if (t >= T) z[t] = 0.0;
                else if (neutral) z[t] = 1.0;
                else z[t] = zg[(size_t)(2u * i) * 4u + t] + zg[(size_t)(2u * i + 1u) * 4u + t];
                P.zi[(size_t)i * 4u + t] = z[t];
            }
            double f = 1.0;
            const double z0 = z[0];
            switch (P.fitness) {
                case 1: {  // gaussian (normal_fitness_metric.cpp:25-31)
                    const double coeff = (1.0 / sig) * 0.398942280401432677939946059934;
                    f = coeff * exp(-(z0 * z0) / (2.0 * sig * sig));
                } break;
                case 2: {  // quadratic (quadratic_fitness_metric.cpp:23-28)
                    const double s = P.fit_param * sig;
                    double r = z0 / s;
                    r *= r;
                    f = (r >= 1.0) ? 0.0 : 1.0 - r;
                } break;
                case 3: {  // gaussian_vs
                    const double ss = z[0] * z[0] + z[1] * z[1] + z[2] * z[2] + z[3] * z[3];
                    f = exp(-ss / (2.0 * P.fit_param));
                } break;
                default: f = 1.0;
            }
            P.fit[i] = f;
        }
    }
}
void launch_individuals(const LaunchCfg& L, const PopDev* pops, uint32_t npops) {
    k_individuals<<<pop_grid(npops, L.num_sms * 2u, L.num_sms, L.ind_per_sm), 256, 0, L.stream>>>(pops, npops);
}

// ---------------------------------------------------------------------------
// Deterministic FP64 inclusive prefix sum of fitness (three phases with a
// fixed association order), plus the total and the all-equal check.
__global__ void __launch_bounds__(1024) k_fscan_a(const PopDev* __restrict__ pops, uint32_t npops) {
    __shared__ double s_w[32];
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        DevStatus* st = P.st;
        const uint32_t N = st->N;
        const uint32_t nch = (N + kScanChunk - 1) / kScanChunk;
        if (blockIdx.x == 0 && threadIdx.x == 0) st->fit_const = 1u;
        for (uint32_t c = blockIdx.x; c < nch; c += gridDim.x) {
            const uint32_t b = c * kScanChunk + threadIdx.x * 4u;
            double s = 0.0;
            for (uint32_t k = 0; k < 4; ++k) s += (b + k < N) ? P.fit[b + k] : 0.0;
            s = warp_incl_f64(s);
            if ((threadIdx.x & 31u) == 31u) s_w[threadIdx.x >> 5] = s;
            __syncthreads();
            if (threadIdx.x == 0) {
                double t = 0.0;
                for (int i = 0; i < 32; ++i) t += s_w[i];
                P.scan_part[c] = t;
            }
            __syncthreads();
        }
    }
}
__global__ void k_fscan_b(const PopDev* __restrict__ pops, uint32_t npops) {
    const uint32_t p = blockIdx.x;
    if (p >= npops || threadIdx.x != 0) return;
    const PopDev& P = pops[p];
    DevStatus* st = P.st;
    const uint32_t N = st->N;
    const uint32_t nch = (N + kScanChunk - 1) / kScanChunk;
    double acc = 0.0;
    for (uint32_t c = 0; c < nch; ++c) {
        const double t = P.scan_part[c];
        P.scan_part[c] = acc;
        acc += t;
    }
    st->fit_total = acc;
    if (!(acc > 0.0) && N > 0) st->err |= kErrFitness;
}
__global__ void __launch_bounds__(1024) k_fscan_c(const PopDev* __restrict__ pops, uint32_t npops) {
    __shared__ double s_w[32];
    for (uint32_t p = blockIdx.z; p < npops; p += gridDim.z) {
        const PopDev& P = pops[p];
        DevStatus* st = P.st;
        const uint32_t N = st->N;
        const uint32_t nch = (N + kScanChunk - 1) / kScanChunk;
        const double f0 = N ? P.fit[0] : 0.0;
        for (uint32_t c = blockIdx.x; c < nch; c += gridDim.x) {
            const uint32_t b = c * kScanChunk + threadIdx.x * 4u;
            double v[4], s = 0.0;
            bool same = true;
            for (uint32_t k = 0; k < 4; ++k) {
                v[k] = (b + k < N) ? P.fit[b + k] : 0.0;
                if (b + k < N && v[k] != f0) same = false;
                s += v[k];
            }
            const double incl = warp_incl_f64(s);
            if ((threadIdx.x & 31u) == 31u) s_w[threadIdx.x >> 5] = incl;
            if (!__all_sync(0xffffffffu, same) && (threadIdx.x & 31u) == 0u) atomicAnd(&st->fit_const, 0u);
            __syncthreads();
            double woff = 0.0;
            for (uint32_t i = 0; i < (threadIdx.x >> 5); ++i) woff += s_w[i];
            // exclusive prefix inside the warp = inclusive value of the previous lane
            const double prev = __shfl_up_sync(0xffffffffu, incl, 1);
            const double excl_w = (threadIdx.x & 31u) ? prev : 0.0;
            double r = P.scan_part[c] + (woff + excl_w);
            for (uint32_t k = 0; k < 4; ++k) {
                r += v[k];
                if (b + k < N) P.cdf[b + k] = r;
            }
            __syncthreads();
        }
    }
}
void launch_cdf(const LaunchCfg& L, const PopDev* pops, uint32_t npops, uint32_t maxN) {
    const uint32_t nch = (maxN + kScanChunk - 1) / kScanChunk;
    const dim3 g = pop_grid(npops, nch, L.num_sms, 2);
    k_fscan_a<<<g, 1024, 0, L.stream>>>(pops, npops);
    k_fscan_b<<<npops, 32, 0, L.stream>>>(pops, npops);
    k_fscan_c<<<g, 1024, 0, L.stream>>>(pops, npops);
}

// ---------------------------------------------------------------------------
// Pre-seeded rows: bit (row, slot) iff seed_hash(seed,row,slot) < thr[slot].
__global__ void k_seed_rows(const PopDev* __restrict__ pops, uint32_t p, const uint32_t* __restrict__ thr,
                            uint64_t seed, uint32_t A) {
    const PopDev& P = pops[p];
    const DevStatus* st = P.st;
    const uint32_t S = 2u * st->N, W = st->W;
    uint64_t* rows = P.rows[st->cur];
    const size_t total = (size_t)S * W;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t r = (uint32_t)(i / W), w = (uint32_t)(i % W);
        uint64_t x = 0;
        for (uint32_t j = 0; j < 64; ++j) {
            const uint32_t a = w * 64u + j;
            if (a < A && seed_hash(seed, r, a) < thr[a]) x |= 1ull << j;
        }
        rows[(size_t)r * P.Wcap + w] = x;
    }
}
void launch_seed_rows(const LaunchCfg& L, const PopDev* pops, uint32_t p, const uint32_t* thr, uint64_t seed,
                      uint32_t A) {
    k_seed_rows<<<L.num_sms * 8, 256, 0, L.stream>>>(pops, p, thr, seed, A);
}

// ---------------------------------------------------------------------------
// Column counts of the current child (count_alleles,
// cuda/analysis/allele_frequency_kernels.hpp:20-73; column margins of
// population_space_row_frequency_evaluator.hpp:37-62).
__global__ void k_col_counts(const PopDev* __restrict__ pops, uint32_t p, uint32_t* __restrict__ counts, uint32_t A) {
    const PopDev& P = pops[p];
    const DevStatus* st = P.st;
    const uint32_t S = 2u * st->N, W = st->W;
    const uint64_t* rows = P.rows[st->cur];
    // block (x: word, y: row group); thread = one bit of the word
    const uint32_t w = blockIdx.x;
    if (w >= W) return;
    const uint32_t groups = gridDim.y, per = (S + groups - 1) / groups;
    const uint32_t r0 = blockIdx.y * per, r1 = min(S, r0 + per);
    const uint32_t j = threadIdx.x;  // 64 threads
    uint32_t c = 0;
    for (uint32_t r = r0; r < r1; ++r) c += (uint32_t)((rows[(size_t)r * P.Wcap + w] >> j) & 1ull);
    const uint32_t a = w * 64u + j;
    if (a < A && c) atomicAdd(&counts[a], c);
}
void launch_stats(const LaunchCfg& L, const PopDev* pops, uint32_t p, uint32_t* counts, uint32_t W) {
    dim3 grid(max(1u, W), 64);
    k_col_counts<<<grid, 64, 0, L.stream>>>(pops, p, counts, W * 64u);
}

// Row margins: alleles carried by each sequence (the row margin of
// population_space_row_frequency_evaluator.hpp:37-62), one warp per row.
__global__ void __launch_bounds__(256) k_row_counts(const PopDev* __restrict__ pops, uint32_t p,
                                                    uint32_t* __restrict__ counts) {
    const PopDev& P = pops[p];
    const DevStatus* st = P.st;
    const uint32_t S = 2u * st->N, W = st->W;
    const uint64_t* rows = P.rows[st->cur];
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < S; r += (gridDim.x * blockDim.x) >> 5) {
        uint32_t c = 0;
        for (uint32_t w = lane; w < W; w += 32u) c += (uint32_t)__popcll(rows[(size_t)r * P.Wcap + w]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) counts[r] = c;
    }
}
void launch_row_counts(const LaunchCfg& L, const PopDev* pops, uint32_t p, uint32_t* counts, uint32_t S) {
    k_row_counts<<<max(1u, min(blocks_for(S, 8), (uint32_t)L.num_sms * 8u)), 256, 0, L.stream>>>(pops, p, counts);
}

}  // namespace clotho
