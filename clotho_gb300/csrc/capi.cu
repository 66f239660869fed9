// capi.cu -- host side of the C-ABI (include/clotho_gpu.h).
//
// A context owns a set of resident populations (one for the plain engine) and
// two CUDA streams: a compute stream for every kernel and a copy stream for
// tape uploads.  Tape buffers are double-buffered so the host->device copy of
// generation g+1 overlaps the kernels of generation g.
#include "engine.cuh"
#include "../../include/clotho_gpu.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace clotho;

namespace {

struct PopHost {
    clotho_desc desc{};
    bool counting = false;    // asked for fused column counts (clotho_pop_count_columns)
    PopDev dev[3]{};          // tape set 0, tape set 1, device-drawn (Philox)
    void* arena = nullptr;          // every device table of the population, one pool block
    size_t bytes = 0;
    bool acc_valid = false;   // accF/accV hold AND/OR of the current child rows
    bool ready = false;       // init/seed done
    uint32_t hostN = 0;       // host view of N after the last completed call
};

struct Geometry {
    uint32_t Ncap, Scap, Wcap, Aslots, Mcap, EVcap, FXcap, T, NB;
    bool table;  // the population has a suffix table (its crossover classifier)
};

// Suffix tables above kSufMaxSlots slots (masks chunk by chunk) pay for themselves at low recombination: on
// GB300 at 2,352-word rows and rho = 1 the chunk-mask kernel took 2.65 against the interval classifier's
// 3.20 ms, while at 472-word rows it took 0.44 / 0.59 / 0.82 ms a generation against 0.45 / 0.51 / 0.60 ms at
// rho = 0.5 / 2 / 5 (each row's breakpoints cost a table load per chunk).
constexpr double kChunkMaxRho = 1.0;

Geometry geometry(const clotho_desc& d) {
    Geometry g{};
    g.Ncap = d.max_individuals ? d.max_individuals : 1;
    g.Scap = 2 * g.Ncap;
    uint32_t w = ref_width(d.max_alleles ? d.max_alleles : 1);
    g.Wcap = (w + kWordAlign - 1) / kWordAlign * kWordAlign;
    g.Aslots = g.Wcap * 64u;
    g.Mcap = d.max_mutations ? d.max_mutations : 1;
    g.EVcap = d.max_events ? d.max_events : 1;
    g.FXcap = d.max_fixed ? d.max_fixed : 1;
    g.T = d.traits;
    g.NB = 1024;
    while (g.NB < g.Aslots) g.NB <<= 1;
    g.table = g.Aslots <= kSufMaxSlots || (g.Aslots <= kTableMaxSlots && d.rho <= kChunkMaxRho);
    return g;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Byte sizes of every device array of one population, in allocation order.
std::vector<size_t> sizes_of(const Geometry& g) {
    const size_t S = g.Scap, N = g.Ncap, W = g.Wcap, A = g.Aslots, T = g.T;
    return {
        S * W * 8, S * W * 8,            // rows[0], rows[1]
        W * 8, W * 8, W * 8,             // fixmask, accF, accV
        A * 4, A * 8, A * 4, A * 16,     // free_list, pos, age, eff (traits padded to 4)
        g.FXcap * 8ull, g.FXcap * 4ull, g.FXcap * T * 4ull,
        S * 32, S * 32, N * 32, N * 8, N * 8,    // zg[0], zg[1], zi, fit, cdf
        (N / 1024 + 8) * 8, ((S > g.NB ? S : g.NB) / 1024 + 8) * 4ull, ((S > g.NB ? S : g.NB) / 1024 + 8) * 4ull,
        (S + 1) * 4 * 2ull,              // row_cnt, row_off
        S * 4, g.Mcap * 4ull, g.Mcap * 4ull,  // row_cur, row_mut, mut_slot
        (g.NB + 1ull) * 4 * 2, g.NB * 4ull, A * 8, A * 4, A * 4,  // bcnt+boff, bcur, bpos, bslot, rank
        g.table ? A * 4 : 0,                            // inv
        g.table ? (A / 64 + 1) * W * 8 : 0,             // suf
        g.table ? S * 16 : 0,                           // plan_row
        g.table ? (S + 1) * 4 * 2 : 0,                  // ord_cnt + ord_off
        g.table ? S * 4 : 0,                            // ord_cur
        g.table ? S * 4 : 0,                            // ord_pos
        g.table ? g.EVcap * 4ull : 0,                   // plan_go
        g.table ? g.EVcap * 4ull : 0,                   // plan_cr
        g.table ? S * 8 : 0,                            // plan_mut
        g.table ? S * 32 : 0,                           // plan_z
        A * 4,                                                    // colcnt
        sizeof(DevStatus),
        // two tape sets: pairs, swap, ev_off, ev_pos, mut_seq, mut_pos, mut_eff
        S * 4, S, (S + 1) * 4, g.EVcap * 8ull, g.Mcap * 4ull, g.Mcap * 8ull, g.Mcap * T * 4ull,
        S * 4, S, (S + 1) * 4, g.EVcap * 8ull, g.Mcap * 4ull, g.Mcap * 8ull, g.Mcap * T * 4ull,
    };
}

}  // namespace

struct clotho_ctx {
    int device = 0;
    int num_sms = 152;
    cudaStream_t stream = nullptr, copy_stream = nullptr;
    cudaStream_t own_stream = nullptr;  // the context's own compute stream (stream may be the caller's)
    // a step's parent selection and row ordering run on side_stream beside the allele-space work (mutation
    // counts, free space, new alleles, ranks, suffix tables), forked after the step's header and joined
    // before the row plans; a captured step keeps the two branches as parallel graph branches
    cudaStream_t side_stream = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    // populations' device tables come from the context's own stream-ordered pool, which keeps freed
    // blocks for the next population (a serving loop adds and removes populations every few steps)
    cudaMemPool_t pool = nullptr;
    std::vector<PopHost*> pops;
    PopDev* d_pops[3] = {nullptr, nullptr, nullptr};  // per set: npops contiguous PopDev
    WorkCtl* d_ctl = nullptr;
    uint32_t* d_hdr[3] = {nullptr, nullptr, nullptr}; // per set: [2*npops]
    // step headers (N, M per population) are staged in a ring of pinned slots:
    // a slot is reused only after the copy that read it has completed
    uint32_t* h_ring = nullptr;                         // [kHdrRing][2 * kMaxPops]
    // asynchronous status read-back: a pinned ring of status copies, each behind an event
    DevStatus* h_stat = nullptr;                        // [kStatRing]
    cudaEvent_t stat_ev[8]{};
    uint32_t stat_next = 0;                             // tickets issued so far
    cudaEvent_t ring_ev[64]{};
    bool ring_used[64]{};
    uint32_t ring_next = 0;
    uint32_t set = 0;                                    // next tape set
    uint32_t pairs_set = 0;                              // the set whose pairs the last generation used
    cudaEvent_t copy_done[2]{}, kern_done[2]{};
    std::string err;
    bool profiling = false;
    bool phase_clocks = false;      // profiling with the phase-clock build of k_generation
    std::vector<cudaEvent_t> prof_ev;  // pairs around each k_generation launch
    size_t prof_used = 0;
    double prof_ms = 0.0;
    uint32_t prof_launches = 0;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    uint64_t launches = 0;
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_launches = 0;  // kernels per replay of graph
    std::vector<uint32_t> graph_key;
    bool in_step = false;
    uint32_t maxW = 0, maxS = 0, maxN = 0, maxNB = 0, maxA = 0;
    // per generation-kernel build: suffix-table masks in bitmaps (bm, at most kSufMaxSlots slots) or chunk by
    // chunk (cm, the other populations with a table), interval classifier (iv, no table); suf = bm + cm
    uint32_t n_suf = 0, n_iv = 0, maxW_suf = 0, maxW_iv = 0, maxA_suf = 0, maxA_iv = 0;
    uint32_t n_bm = 0, n_cm = 0, maxW_bm = 0, maxW_cm = 0, maxA_bm = 0, maxA_cm = 0;
    cudaError_t launch_err = cudaSuccess;  // a launch set-up failure, reported by the next check_launch
    uint32_t ind_per_sm = 16;               // tuning (clotho_set_tuning)
    bool narrow_ok = true;
    uint32_t tuning_epoch = 0;              // part of every graph's key: a new tuning re-captures
    uint32_t counting = 0;                  // populations that asked for fused column counts
};

namespace {

constexpr uint32_t kHdrRing = 64;
constexpr uint32_t kStatRing = 8;   // outstanding asynchronous status reads (clotho_info_request)
static_assert(sizeof(((clotho_ctx*)nullptr)->ring_ev) / sizeof(cudaEvent_t) == kHdrRing, "header ring size");
static_assert(sizeof(((clotho_ctx*)nullptr)->stat_ev) / sizeof(cudaEvent_t) == kStatRing, "status ring size");

int fail(clotho_ctx* c, int code, const std::string& m) {
    if (c) c->err = m;
    return code;
}

#define CK(call)                                                                    \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess)                                                      \
            return fail(ctx, CLOTHO_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

LaunchCfg cfg(clotho_ctx* ctx) {
    LaunchCfg L{ctx->stream, ctx->num_sms};
    L.ind_per_sm = ctx->ind_per_sm;
    L.narrow_ok = ctx->narrow_ok;
    return L;
}

// A pinned slot for one step header; nullptr if pinned memory is unavailable.
uint32_t* hdr_stage(clotho_ctx* ctx, uint32_t* slot) {
    if (!ctx->h_ring) {
        if (cudaMallocHost(&ctx->h_ring, sizeof(uint32_t) * 2 * kMaxPops * kHdrRing) != cudaSuccess) {
            cudaGetLastError();
            ctx->h_ring = nullptr;
            return nullptr;
        }
        for (uint32_t k = 0; k < kHdrRing; ++k) cudaEventCreateWithFlags(&ctx->ring_ev[k], cudaEventDisableTiming);
    }
    const uint32_t k = ctx->ring_next;
    ctx->ring_next = (k + 1) % kHdrRing;
    if (ctx->ring_used[k]) cudaEventSynchronize(ctx->ring_ev[k]);
    *slot = k;
    return ctx->h_ring + (size_t)k * 2 * kMaxPops;
}

// Copy n headers from slot into dst on stream s and mark the slot busy until then.
int hdr_copy(clotho_ctx* ctx, uint32_t slot, uint32_t* dst, uint32_t n, cudaStream_t s) {
    CK(cudaMemcpyAsync(dst, ctx->h_ring + (size_t)slot * 2 * kMaxPops, 8ull * n, cudaMemcpyHostToDevice, s));
    CK(cudaEventRecord(ctx->ring_ev[slot], s));
    ctx->ring_used[slot] = true;
    return 0;
}

// Scratch device memory for a call, from the context's stream-ordered pool (freed with cudaFreeAsync on
// the context's stream): no device-wide synchronisation, unlike cudaMalloc / cudaFree.
template <class T>
cudaError_t pool_alloc(clotho_ctx* ctx, T** p, size_t bytes) {
    return cudaMallocFromPoolAsync(reinterpret_cast<void**>(p), bytes, ctx->pool, ctx->stream);
}

int check_launch(clotho_ctx* ctx, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (ctx->launch_err != cudaSuccess) {
        e = ctx->launch_err;
        ctx->launch_err = cudaSuccess;
    }
    if (e != cudaSuccess) return fail(ctx, CLOTHO_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return 0;
}

// The caller has synchronized the context's streams: nothing reads the tables any more.
void free_pop(clotho_ctx* ctx, PopHost* p) {
    if (p->arena) cudaFreeAsync(p->arena, ctx->own_stream);
    p->arena = nullptr;
    delete p;
}

int alloc_pop(clotho_ctx* ctx, const clotho_desc& d, PopHost** out) {
    if (d.traits < 1 || d.traits > kMaxTraits) return fail(ctx, CLOTHO_E_ARG, "traits must be 1..4");
    if (d.max_individuals == 0 || d.max_alleles == 0) return fail(ctx, CLOTHO_E_ARG, "zero capacity");
    const Geometry g = geometry(d);
    PopHost* p = new PopHost();
    p->desc = d;
    std::vector<size_t> sz = sizes_of(g);
    std::vector<void*> ptr(sz.size(), nullptr);
    // one block for all tables, each at a 256-byte aligned offset (optional tables of size 0 stay null)
    size_t total = 0;
    for (size_t x : sz) total += align256(x);
    cudaError_t e = cudaMallocFromPoolAsync(&p->arena, total, ctx->pool, ctx->own_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->own_stream);  // ready before other streams use it
    if (e != cudaSuccess) {
        cudaGetLastError();
        p->arena = nullptr;
        delete p;
        return fail(ctx, CLOTHO_E_NOMEM, "device allocation refused (" + std::to_string(total) + " bytes)");
    }
    p->bytes = total;
    for (size_t i = 0, off = 0; i < sz.size(); off += align256(sz[i]), ++i)
        if (sz[i]) ptr[i] = static_cast<char*>(p->arena) + off;
    // zero the tables and the status: everything after the two row sets, in one call
    const size_t rows_bytes = align256(sz[0]) + align256(sz[1]);
    if (total > rows_bytes) cudaMemsetAsync(static_cast<char*>(p->arena) + rows_bytes, 0, total - rows_bytes, ctx->stream);
    PopDev b{};
    size_t k = 0;
    b.rows[0] = (uint64_t*)ptr[k++]; b.rows[1] = (uint64_t*)ptr[k++];
    b.fixmask = (uint64_t*)ptr[k++]; b.accF = (uint64_t*)ptr[k++]; b.accV = (uint64_t*)ptr[k++];
    b.free_list = (uint32_t*)ptr[k++]; b.pos = (double*)ptr[k++]; b.age = (uint32_t*)ptr[k++]; b.eff = (float*)ptr[k++];
    b.fx_pos = (double*)ptr[k++]; b.fx_age = (uint32_t*)ptr[k++]; b.fx_eff = (float*)ptr[k++];
    b.zg[0] = (double*)ptr[k++]; b.zg[1] = (double*)ptr[k++];
    b.zi = (double*)ptr[k++]; b.fit = (double*)ptr[k++]; b.cdf = (double*)ptr[k++];
    b.scan_part = (double*)ptr[k++]; b.scan_upart = (uint32_t*)ptr[k++]; b.scan_opart = (uint32_t*)ptr[k++];
    b.row_cnt = (uint32_t*)ptr[k++];
    b.row_off = b.row_cnt + (g.Scap + 1);
    b.row_cur = (uint32_t*)ptr[k++]; b.row_mut = (uint32_t*)ptr[k++]; b.mut_slot = (uint32_t*)ptr[k++];
    b.bcnt = (uint32_t*)ptr[k++];
    b.boff = b.bcnt + (g.NB + 1);
    b.bcur = (uint32_t*)ptr[k++]; b.bpos = (double*)ptr[k++]; b.bslot = (uint32_t*)ptr[k++];
    b.rank = (uint32_t*)ptr[k++]; b.inv = (uint32_t*)ptr[k++]; b.suf = (uint64_t*)ptr[k++];
    b.plan_row = (uint4*)ptr[k++];
    b.ord_cnt = (uint32_t*)ptr[k++];
    b.ord_off = b.ord_cnt ? b.ord_cnt + (g.Scap + 1) : nullptr;
    b.ord_cur = (uint32_t*)ptr[k++]; b.ord_pos = (uint32_t*)ptr[k++];
    b.plan_go = (uint32_t*)ptr[k++]; b.plan_cr = (uint32_t*)ptr[k++];
    b.plan_mut = (uint2*)ptr[k++]; b.plan_z = (double*)ptr[k++];
    b.colcnt = (uint32_t*)ptr[k++];
    b.st = (DevStatus*)ptr[k++];
    b.Scap = g.Scap; b.Ncap = g.Ncap; b.Wcap = g.Wcap; b.Acap = g.Aslots; b.Mcap = g.Mcap;
    b.EVcap = g.EVcap; b.FXcap = g.FXcap; b.T = g.T; b.NB = g.NB;
    b.mu = d.mu; b.rho = d.rho; b.bias = d.bias; b.p_neutral = d.p_neutral;
    b.eff_mean = d.eff_mean; b.eff_sigma = d.eff_sigma; b.fit_param = d.fit_param;
    b.exp_neg_rho = std::exp(-d.rho);
    b.exp_neg_mu = std::exp(-d.mu);
    b.seed = d.seed; b.fitness = d.fitness; b.flags = d.flags;
    for (int s = 0; s < 2; ++s) {
        PopDev t = b;
        t.mode = kModeTape;
        t.pairs = (uint32_t*)ptr[k++]; t.swap = (uint8_t*)ptr[k++]; t.ev_off = (uint32_t*)ptr[k++];
        t.ev_pos = (double*)ptr[k++]; t.mut_seq = (uint32_t*)ptr[k++]; t.mut_pos = (double*)ptr[k++];
        t.mut_eff = (float*)ptr[k++];
        p->dev[s] = t;
    }
    p->dev[2] = p->dev[0];
    p->dev[2].mode = kModePhilox;
    *out = p;
    return 0;
}

// Rebuild the device PopDev arrays after the population set changed: entries
// [from, n) are copied (an add changes the last one, a remove shifts the rest).
int sync_pop_arrays(clotho_ctx* ctx, uint32_t from = 0) {
    const uint32_t n = (uint32_t)ctx->pops.size();
    if (n > kMaxPops) return fail(ctx, CLOTHO_E_CAPACITY, "more than 256 populations");
    for (int s = 0; s < 3; ++s) {
        // sized for kMaxPops once, so adding or removing a population allocates nothing here
        if (!ctx->d_pops[s]) CK(cudaMalloc(&ctx->d_pops[s], sizeof(PopDev) * kMaxPops));
        if (!ctx->d_hdr[s]) CK(cudaMalloc(&ctx->d_hdr[s], sizeof(uint32_t) * 2 * kMaxPops));
        if (from >= n) continue;
        std::vector<PopDev> h(n - from);
        for (uint32_t i = from; i < n; ++i) h[i - from] = ctx->pops[i]->dev[s];
        CK(cudaMemcpyAsync(ctx->d_pops[s] + from, h.data(), sizeof(PopDev) * (n - from), cudaMemcpyHostToDevice,
                           ctx->stream));
    }
    ctx->maxW = ctx->maxS = ctx->maxN = ctx->maxNB = ctx->maxA = 0;
    ctx->n_suf = ctx->n_iv = ctx->maxW_suf = ctx->maxW_iv = ctx->maxA_suf = ctx->maxA_iv = 0;
    ctx->n_bm = ctx->n_cm = ctx->maxW_bm = ctx->maxW_cm = ctx->maxA_bm = ctx->maxA_cm = 0;
    for (PopHost* p : ctx->pops) {
        const PopDev& D = p->dev[0];
        ctx->maxW = std::max(ctx->maxW, D.Wcap);
        ctx->maxS = std::max(ctx->maxS, D.Scap);
        ctx->maxN = std::max(ctx->maxN, D.Ncap);
        ctx->maxNB = std::max(ctx->maxNB, D.NB);
        ctx->maxA = std::max(ctx->maxA, D.Acap);
        if (D.suf != nullptr) {
            ctx->n_suf += 1;
            ctx->maxW_suf = std::max(ctx->maxW_suf, D.Wcap);
            ctx->maxA_suf = std::max(ctx->maxA_suf, D.Acap);
            if (D.Acap <= kSufMaxSlots) {
                ctx->n_bm += 1;
                ctx->maxW_bm = std::max(ctx->maxW_bm, D.Wcap);
                ctx->maxA_bm = std::max(ctx->maxA_bm, D.Acap);
            } else {
                ctx->n_cm += 1;
                ctx->maxW_cm = std::max(ctx->maxW_cm, D.Wcap);
                ctx->maxA_cm = std::max(ctx->maxA_cm, D.Acap);
            }
        } else {
            ctx->n_iv += 1;
            ctx->maxW_iv = std::max(ctx->maxW_iv, D.Wcap);
            ctx->maxA_iv = std::max(ctx->maxA_iv, D.Acap);
        }
    }
    if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; }
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

DevStatus read_status(clotho_ctx* ctx, PopHost* p, int* rc) {
    DevStatus s{};
    cudaError_t e = cudaMemcpyAsync(&s, p->dev[0].st, sizeof(DevStatus), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    *rc = (e == cudaSuccess) ? 0 : fail(ctx, CLOTHO_E_CUDA, std::string("status read: ") + cudaGetErrorString(e));
    return s;
}

// ---- profiling around the generation kernel
void prof_begin(clotho_ctx* ctx) {
    if (!ctx->profiling) return;
    if (ctx->prof_used + 2 > ctx->prof_ev.size()) {
        for (int i = 0; i < 64; ++i) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) {  // out of events: stop timing, keep running
                cudaGetLastError();
                ctx->profiling = false;
                return;
            }
            ctx->prof_ev.push_back(e);
        }
    }
    cudaEventRecord(ctx->prof_ev[ctx->prof_used], ctx->stream);
}
void prof_end(clotho_ctx* ctx) {
    if (!ctx->profiling) return;
    cudaEventRecord(ctx->prof_ev[ctx->prof_used + 1], ctx->stream);
    ctx->prof_used += 2;
    ctx->prof_launches += 1;
}
int prof_collect(clotho_ctx* ctx) {
    if (ctx->prof_used == 0) return 0;
    CK(cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i + 1 < ctx->prof_used; i += 2) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ctx->prof_ev[i], ctx->prof_ev[i + 1]));
        ctx->prof_ms += ms;
    }
    ctx->prof_used = 0;
    return 0;
}

// The fused step's generation kernel counts columns (its counting build) when a population asked and the
// counters fit in shared memory; k_fs_finalize of the same step zeroes those counts and marks them valid.
bool count_on(clotho_ctx* ctx, uint32_t fuse) {
    return ctx->counting > 0 && ctx->n_bm > 0 && (fuse & kFuseFs) && !(ctx->profiling && ctx->phase_clocks) &&
           generation_counts_fit(ctx->maxW_bm, ctx->maxA_bm);
}

// The generation kernel over every population: one launch when all populations use the same build; in a
// batch that mixes them, one launch per build (bitmap, chunk-mask, interval), each over its own populations,
// so every population runs the build it runs alone.
// ordered: the rows' processing order is already enqueued (the fused step's side branch).
void launch_gen(clotho_ctx* ctx, const PopDev* pops, uint32_t npops, uint32_t fuse, bool ordered = false) {
    if (ctx->n_suf > 0) {  // per-row crossover plans of the suffix-table classifier (other populations skip it)
        if (!ordered) {
            launch_order(cfg(ctx), pops, npops, ctx->maxS);
            ctx->launches += 5;  // order count, 3-kernel scan, order scatter
        }
        launch_row_plan(cfg(ctx), pops, npops, ctx->maxS);
        ctx->launches += 1;
    }
    const int prof = ctx->profiling ? (ctx->phase_clocks ? 2 : 1) : 0;
    const uint32_t kinds = (ctx->n_bm > 0) + (ctx->n_cm > 0) + (ctx->n_iv > 0);
    const bool mixed = kinds > 1;
    const bool cnt = count_on(ctx, fuse);
    const uint32_t pn[3] = {ctx->n_bm, ctx->n_cm, ctx->n_iv};
    const uint32_t pW[3] = {ctx->maxW_bm, ctx->maxW_cm, ctx->maxW_iv};
    const uint32_t pA[3] = {ctx->maxA_bm, ctx->maxA_cm, ctx->maxA_iv};
    const GenBuild builds[3] = {kBuildBitmap, kBuildChunk, kBuildInterval};
    for (int pass = 0; pass < 3; ++pass) {
        if (pn[pass] == 0) continue;
        const uint32_t W = mixed ? pW[pass] : ctx->maxW;
        const uint32_t A = mixed ? pA[pass] : ctx->maxA;
        prof_begin(ctx);
        const cudaError_t e =
            launch_generation(cfg(ctx), pops, npops, ctx->d_ctl, W, A, fuse, prof, builds[pass], cnt, mixed);
        if (e != cudaSuccess && ctx->launch_err == cudaSuccess) ctx->launch_err = e;
        prof_end(ctx);
        ctx->launches += 1;
    }
}

template <class T>
int h2d(clotho_ctx* ctx, T* dst, const T* src, size_t n, cudaStream_t s) {
    if (n == 0) return 0;
    if (!src) return fail(ctx, CLOTHO_E_ARG, "null host array");
    CK(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, s));
    return 0;
}

// Upload one generation's tape into tape set s of population p (copy stream).
int upload_tape(clotho_ctx* ctx, PopHost* p, uint32_t s, const clotho_gen_tape* t) {
    const PopDev& D = p->dev[s];
    const uint32_t N = t->N, M = t->M, T = D.T;
    if (N > D.Ncap) return fail(ctx, CLOTHO_E_CAPACITY, "tape N exceeds max_individuals");
    if (M > D.Mcap) return fail(ctx, CLOTHO_E_CAPACITY, "tape M exceeds max_mutations");
    if (!t->ev_off) return fail(ctx, CLOTHO_E_ARG, "tape ev_off is null");
    const uint32_t ev_total = t->ev_off[2ull * N];
    if (ev_total > D.EVcap) return fail(ctx, CLOTHO_E_CAPACITY, "tape events exceed max_events");
    for (uint64_t g = 0; g < 2ull * N; ++g)
        if (t->ev_off[g] > t->ev_off[g + 1]) return fail(ctx, CLOTHO_E_ARG, "tape ev_off not monotone");
    cudaStream_t cs = ctx->copy_stream;
    int rc;
    if ((rc = h2d(ctx, D.pairs, t->pairs, 2ull * N, cs))) return rc;
    if ((rc = h2d(ctx, D.swap, t->swap, 2ull * N, cs))) return rc;
    if ((rc = h2d(ctx, D.ev_off, t->ev_off, 2ull * N + 1, cs))) return rc;
    if ((rc = h2d(ctx, D.ev_pos, t->ev_pos, (size_t)ev_total, cs))) return rc;
    if ((rc = h2d(ctx, D.mut_seq, t->mut_seq, (size_t)M, cs))) return rc;
    if ((rc = h2d(ctx, D.mut_pos, t->mut_pos, (size_t)M, cs))) return rc;
    if ((rc = h2d(ctx, D.mut_eff, t->mut_eff, (size_t)M * T, cs))) return rc;
    return 0;
}

int require_ready(clotho_ctx* ctx) {
    if (!ctx) return CLOTHO_E_ARG;
    for (PopHost* p : ctx->pops)
        if (!p->ready) return fail(ctx, CLOTHO_E_STATE, "population not initialised (clotho_init / clotho_seed_population)");
    return 0;
}

// Make accF/accV of every population hold the AND/OR of its parent rows
// (called right after k_begin when the previous step did not fuse them).
void ensure_parent_acc(clotho_ctx* ctx, const PopDev* pops, uint32_t npops) {
    bool need = false;
    for (PopHost* p : ctx->pops) need |= !p->acc_valid;
    if (need) {
        launch_fs_reduce(cfg(ctx), pops, npops, ctx->maxW, 1u);
        ctx->launches += 1;
    }
}

// The fused step shared by tape and device-drawn modes, for every population.
void enqueue_fused_step(clotho_ctx* ctx, uint32_t set, bool philox) {
    const uint32_t n = (uint32_t)ctx->pops.size();
    const PopDev* pops = ctx->d_pops[set];
    LaunchCfg L = cfg(ctx);
    ctx->pairs_set = set == 1u ? 1u : 0u;  // the device-drawn set (2) shares set 0's buffers
    launch_begin(L, pops, n, ctx->d_hdr[set], ctx->d_ctl);
    ensure_parent_acc(ctx, pops, n);
    // side branch: parents (from the parent generation's fitness) and the rows' processing order (from the
    // parents) read only the step header and the pairs, and write only the pairs, the ordering arrays and
    // their own scan partials, none of which the main branch touches before the join
    auto note = [ctx](cudaError_t e) {
        if (e != cudaSuccess && ctx->launch_err == cudaSuccess) ctx->launch_err = e;
    };
    LaunchCfg Ls = L;
    Ls.stream = ctx->side_stream;
    note(cudaEventRecord(ctx->fork_ev, L.stream));
    note(cudaStreamWaitEvent(ctx->side_stream, ctx->fork_ev, 0));
    if (philox) launch_select_philox(Ls, pops, n);
    if (ctx->n_suf > 0) {
        launch_order(Ls, pops, n, ctx->maxS);
        ctx->launches += 5;  // order count, 3-kernel scan, order scatter
    }
    note(cudaEventRecord(ctx->join_ev, ctx->side_stream));
    // main branch: the child's allele space
    if (philox) launch_mut_counts_philox(L, pops, n, ctx->maxS);
    launch_fs_finalize(L, pops, n, count_on(ctx, kFuseMut | kFusePheno | kFuseFs));
    if (!philox) launch_mut_csr_tape(L, pops, n, ctx->maxS);
    launch_mut_resolve(L, pops, n);
    launch_ranks(L, pops, n, ctx->maxNB, ctx->maxW_suf, ctx->n_suf > 0);
    note(cudaStreamWaitEvent(L.stream, ctx->join_ev, 0));
    launch_gen(ctx, pops, n, kFuseMut | kFusePheno | kFuseFs, true);
    launch_individuals(L, pops, n);
    launch_cdf(L, pops, n, ctx->maxN);
    launch_end(L, pops, n);
    // begin, mutation counts or CSR (4 or 6), finalize, resolve, ranks (6, + suffix table), selection (device
    // draws), individuals, 3-kernel prefix sum, end; launch_gen and ensure_parent_acc count their own
    ctx->launches += 19u + (philox ? 0u : 1u) + (ctx->n_suf > 0 ? 1u : 0u);
    for (PopHost* p : ctx->pops) p->acc_valid = true;
}

// Captures one fused device-drawn step as the context's graph, keyed by the sizes it serves (a graph
// with the same key is reused).  Whatever fails between the start of the capture and the graph's
// instantiation, the capture is ended and the partial graph discarded, so the stream stays usable.
int capture_step_graph(clotho_ctx* ctx, std::vector<uint32_t> key) {
    key.push_back(ctx->tuning_epoch);
    if (ctx->graph && ctx->graph_key == key) return 0;
    if (ctx->graph) {
        cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
    }
    ctx->graph_key.clear();
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const uint64_t l0 = ctx->launches;
    enqueue_fused_step(ctx, 2, true);
    ctx->graph_launches = ctx->launches - l0;
    ctx->launches = l0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && ctx->launch_err != cudaSuccess) e = ctx->launch_err;
    ctx->launch_err = cudaSuccess;
    cudaGraph_t gr = nullptr;
    const cudaError_t e_end = cudaStreamEndCapture(ctx->stream, &gr);  // ends the capture in every case
    if (e == cudaSuccess) e = e_end;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->graph, gr, 0);
    if (gr) cudaGraphDestroy(gr);
    if (e != cudaSuccess) {
        ctx->graph = nullptr;
        cudaGetLastError();
        return fail(ctx, CLOTHO_E_CUDA, std::string("graph capture of a generation: ") + cudaGetErrorString(e));
    }
    ctx->graph_key = key;
    return 0;
}

}  // namespace

// ===========================================================================
extern "C" {

size_t clotho_footprint_for(const clotho_desc* d) {
    if (!d) return 0;
    size_t t = 0;
    for (size_t s : sizes_of(geometry(*d))) t += align256(s);
    return t;
}

int clotho_create(const clotho_desc* desc, clotho_ctx** out) {
    if (!desc || !out) return CLOTHO_E_ARG;
    *out = nullptr;
    clotho_ctx* ctx = new clotho_ctx();
    cudaError_t e = cudaGetDevice(&ctx->device);
    if (e != cudaSuccess) {
        delete ctx;
        return CLOTHO_E_CUDA;
    }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (init_recip_step() || init_recip_gen()) {  // constant tables of this device
        cudaGetLastError();
        delete ctx;
        return CLOTHO_E_CUDA;
    }
    if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->side_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->join_ev, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        clotho_destroy(ctx);  // releases whichever stream was made
        return CLOTHO_E_CUDA;
    }
    ctx->stream = ctx->own_stream;
    {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = ctx->device;
        if (cudaMemPoolCreate(&ctx->pool, &props) != cudaSuccess) {
            cudaGetLastError();
            ctx->pool = nullptr;
            clotho_destroy(ctx);
            return CLOTHO_E_CUDA;
        }
        // freed blocks stay in the pool until the context ends; if the attribute is refused, the pool
        // returns memory at each synchronization instead, which is slower, not wrong
        uint64_t keep = ~0ull;
        if (cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess)
            cudaGetLastError();
    }
    {
        bool ok = true;
        for (int i = 0; i < 2; ++i) {
            ok = ok && cudaEventCreateWithFlags(&ctx->copy_done[i], cudaEventDisableTiming) == cudaSuccess;
            ok = ok && cudaEventCreateWithFlags(&ctx->kern_done[i], cudaEventDisableTiming) == cudaSuccess;
            ok = ok && cudaEventRecord(ctx->kern_done[i], ctx->stream) == cudaSuccess;
        }
        ok = ok && cudaEventCreate(&ctx->t0) == cudaSuccess && cudaEventCreate(&ctx->t1) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            clotho_destroy(ctx);
            return CLOTHO_E_CUDA;
        }
    }
    if (cudaMalloc(&ctx->d_ctl, sizeof(WorkCtl)) != cudaSuccess) {
        cudaGetLastError();
        clotho_destroy(ctx);
        return CLOTHO_E_NOMEM;
    }
    {
        const uint32_t rpi = kRowsPerItem;
        if (cudaMemsetAsync(ctx->d_ctl, 0, sizeof(WorkCtl), ctx->stream) != cudaSuccess ||
            cudaMemcpyAsync(&ctx->d_ctl->rows_per_item, &rpi, 4, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
            cudaGetLastError();
            clotho_destroy(ctx);
            return CLOTHO_E_CUDA;
        }
    }
    PopHost* p = nullptr;
    int rc = alloc_pop(ctx, *desc, &p);
    if (rc) {
        std::string m = ctx->err;
        clotho_destroy(ctx);
        fprintf(stderr, "clotho_create: %s\n", m.c_str());
        return rc;
    }
    ctx->pops.push_back(p);
    rc = sync_pop_arrays(ctx);
    if (rc) {
        clotho_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return 0;
}

int clotho_destroy(clotho_ctx* ctx) {
    if (!ctx) return CLOTHO_E_ARG;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    if (ctx->side_stream) cudaStreamSynchronize(ctx->side_stream);
    for (PopHost* p : ctx->pops) free_pop(ctx, p);
    ctx->pops.clear();
    if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);  // its blocks are back: free_pop returned them
    for (int s = 0; s < 3; ++s) {
        if (ctx->d_pops[s]) cudaFree(ctx->d_pops[s]);
        if (ctx->d_hdr[s]) cudaFree(ctx->d_hdr[s]);
    }
    if (ctx->h_ring) cudaFreeHost(ctx->h_ring);
    if (ctx->h_stat) cudaFreeHost(ctx->h_stat);
    for (uint32_t k = 0; k < kStatRing; ++k)
        if (ctx->stat_ev[k]) cudaEventDestroy(ctx->stat_ev[k]);
    for (uint32_t k = 0; k < kHdrRing; ++k)
        if (ctx->ring_ev[k]) cudaEventDestroy(ctx->ring_ev[k]);
    if (ctx->d_ctl) cudaFree(ctx->d_ctl);
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    for (cudaEvent_t e : ctx->prof_ev) cudaEventDestroy(e);
    for (int i = 0; i < 2; ++i) {
        if (ctx->copy_done[i]) cudaEventDestroy(ctx->copy_done[i]);
        if (ctx->kern_done[i]) cudaEventDestroy(ctx->kern_done[i]);
    }
    if (ctx->t0) cudaEventDestroy(ctx->t0);
    if (ctx->t1) cudaEventDestroy(ctx->t1);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->side_stream) cudaStreamDestroy(ctx->side_stream);
    if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
    if (ctx->join_ev) cudaEventDestroy(ctx->join_ev);
    delete ctx;
    return 0;
}

const char* clotho_last_error(const clotho_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

size_t clotho_footprint(const clotho_ctx* ctx) {
    size_t t = 0;
    if (ctx)
        for (PopHost* p : ctx->pops) t += p->bytes;
    return t;
}

int clotho_sync(clotho_ctx* ctx) {
    if (!ctx) return CLOTHO_E_ARG;
    CK(cudaStreamSynchronize(ctx->copy_stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int clotho_set_stream(clotho_ctx* ctx, void* stream) {
    if (!ctx) return CLOTHO_E_ARG;
    if (ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "set the stream between generations");
    // work already queued on the old stream finishes before the new one is used
    CK(cudaStreamSynchronize(ctx->copy_stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    return 0;
}

uint64_t clotho_launch_count(const clotho_ctx* ctx) { return ctx ? ctx->launches : 0; }

static int init_pop(clotho_ctx* ctx, uint32_t idx, uint32_t N0) {
    if (!ctx || idx >= ctx->pops.size()) return fail(ctx, CLOTHO_E_ARG, "no such population");
    PopHost* p = ctx->pops[idx];
    const PopDev& D = p->dev[0];
    if (N0 > D.Ncap) return fail(ctx, CLOTHO_E_CAPACITY, "N0 exceeds max_individuals");
    CK(cudaStreamSynchronize(ctx->stream));
    DevStatus s{};
    s.gen = 1;
    s.cur = 0;
    s.N = N0;
    s.count_cols = p->counting ? 1u : 0u;
    s.fit_const = 1;
    s.fit_total = (double)N0;
    s.all_neutral = 1;
    CK(cudaMemcpyAsync(D.st, &s, sizeof(s), cudaMemcpyHostToDevice, ctx->stream));
    std::vector<double> ones(N0, 1.0);
    if (N0) CK(cudaMemcpyAsync(D.fit, ones.data(), N0 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(D.pos, 0, (size_t)D.Acap * 8, ctx->stream));
    CK(cudaMemsetAsync(D.eff, 0, (size_t)D.Acap * 16, ctx->stream));
    CK(cudaMemsetAsync(D.age, 0, (size_t)D.Acap * 4, ctx->stream));
    CK(cudaMemsetAsync(D.accF, 0xff, (size_t)D.Wcap * 8, ctx->stream));
    CK(cudaMemsetAsync(D.accV, 0, (size_t)D.Wcap * 8, ctx->stream));
    CK(cudaMemsetAsync(D.row_cnt, 0, ((size_t)D.Scap + 1) * 4, ctx->stream));
    CK(cudaMemsetAsync(D.row_cur, 0, (size_t)D.Scap * 4, ctx->stream));
    CK(cudaMemsetAsync(D.bcnt, 0, ((size_t)D.NB + 1) * 4, ctx->stream));
    CK(cudaMemsetAsync(D.bcur, 0, (size_t)D.NB * 4, ctx->stream));
    CK(cudaMemsetAsync(D.zg[0], 0, (size_t)D.Scap * 32, ctx->stream));
    CK(cudaMemsetAsync(D.zg[1], 0, (size_t)D.Scap * 32, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    p->acc_valid = true;  // A == 0: the first analysis is skipped (free_space_mt...:46)
    p->ready = true;
    p->hostN = N0;
    return 0;
}

int clotho_init(clotho_ctx* ctx, uint32_t N0) { return init_pop(ctx, 0, N0); }

// Shared set-up of an explicit or seeded start: status, allele tables, then
// (after the caller fills the rows) reduction, phenotype and fitness.
static int start_population(clotho_ctx* ctx, uint32_t N, uint32_t A, const double* pos, const float* eff) {
    PopHost* p = ctx->pops[0];
    const PopDev& D = p->dev[0];
    if (A > D.Acap || ref_width(A) > D.Wcap) return fail(ctx, CLOTHO_E_CAPACITY, "A exceeds max_alleles");
    int rc = clotho_init(ctx, N);
    if (rc) return rc;
    const uint32_t T = D.T;
    int32_t nz = 0;
    for (size_t i = 0; i < (size_t)A * T; ++i) nz += (eff[i] != 0.0f);
    DevStatus s{};
    s.gen = 1;
    s.cur = 0;
    s.N = N;
    s.A = A;
    s.count_cols = p->counting ? 1u : 0u;
    s.W = ref_width(A);
    s.nz_eff = nz;
    s.fit_const = 1;
    s.fit_total = (double)N;
    CK(cudaMemcpyAsync(D.st, &s, sizeof(s), cudaMemcpyHostToDevice, ctx->stream));
    if (A) {
        CK(cudaMemcpyAsync(D.pos, pos, (size_t)A * 8, cudaMemcpyHostToDevice, ctx->stream));
        std::vector<float> pad((size_t)A * 4, 0.0f);
        for (size_t i = 0; i < A; ++i)
            for (uint32_t t = 0; t < T; ++t) pad[i * 4 + t] = eff[i * T + t];
        CK(cudaMemcpyAsync(D.eff, pad.data(), (size_t)A * 16, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return 0;
}

static int finish_start(clotho_ctx* ctx) {
    PopHost* p = ctx->pops[0];
    LaunchCfg L = cfg(ctx);
    launch_fs_reduce(L, ctx->d_pops[0], 1, ctx->maxW, 0u);
    launch_phenotype(L, ctx->d_pops[0], 1);
    launch_individuals(L, ctx->d_pops[0], 1);
    launch_cdf(L, ctx->d_pops[0], 1, ctx->maxN);
    ctx->launches += 6;
    int rc = check_launch(ctx, "start");
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    p->acc_valid = true;
    return 0;
}

int clotho_load_population(clotho_ctx* ctx, uint32_t N, uint32_t A, const uint64_t* rows, const double* pos,
                           const float* eff) {
    if (!ctx || (A && (!pos || !eff || !rows))) return CLOTHO_E_ARG;
    int rc = start_population(ctx, N, A, pos, eff);
    if (rc) return rc;
    const PopDev& D = ctx->pops[0]->dev[0];
    const size_t W = ref_width(A), S = 2ull * N;
    if (S * W) {
        // keep only slots < A (the reference never sets bits past its allele count)
        std::vector<uint64_t> tmp(rows, rows + S * W);
        for (size_t r = 0; r < S; ++r)
            for (size_t w = 0; w < W; ++w) {
                const size_t b = w * 64;
                uint64_t valid = (b + 64 <= A) ? ~0ull : (b >= A ? 0ull : ((1ull << (A - b)) - 1ull));
                tmp[r * W + w] &= valid;
            }
        CK(cudaMemcpy2DAsync(D.rows[0], (size_t)D.Wcap * 8, tmp.data(), W * 8, W * 8, S, cudaMemcpyHostToDevice,
                             ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return finish_start(ctx);
}

int clotho_seed_population(clotho_ctx* ctx, uint32_t N, uint32_t A, const double* pos, const float* eff,
                           const uint32_t* thr, uint64_t seed) {
    if (!ctx || (A && (!pos || !eff || !thr))) return CLOTHO_E_ARG;
    {
        int rc0 = start_population(ctx, N, A, pos, eff);
        if (rc0) return rc0;
        uint32_t* d_thr = nullptr;
        CK(pool_alloc(ctx, &d_thr, std::max<size_t>(4, (size_t)A * 4)));
        if (A) CK(cudaMemcpyAsync(d_thr, thr, (size_t)A * 4, cudaMemcpyHostToDevice, ctx->stream));
        launch_seed_rows(cfg(ctx), ctx->d_pops[0], 0, d_thr, seed, A);
        ctx->launches += 1;
        CK(cudaFreeAsync(d_thr, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        return finish_start(ctx);
    }
}

int clotho_generation_tape(clotho_ctx* ctx, const clotho_gen_tape* tape) {
    int rc = require_ready(ctx);
    if (rc) return rc;
    if (!tape || ctx->pops.size() != 1) return fail(ctx, CLOTHO_E_ARG, "bad tape");
    if (ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "a staged generation is in progress");
    const uint32_t s = ctx->set;
    // the tape set s was last read by the kernels of two steps ago
    CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->kern_done[s], 0));
    if ((rc = upload_tape(ctx, ctx->pops[0], s, tape))) return rc;
    uint32_t slot;
    uint32_t* h = hdr_stage(ctx, &slot);
    if (!h) return fail(ctx, CLOTHO_E_NOMEM, "pinned host memory refused");
    h[0] = tape->N;
    h[1] = tape->M;
    if ((rc = hdr_copy(ctx, slot, ctx->d_hdr[s], 1, ctx->copy_stream))) return rc;
    CK(cudaEventRecord(ctx->copy_done[s], ctx->copy_stream));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->copy_done[s], 0));
    enqueue_fused_step(ctx, s, false);
    if ((rc = check_launch(ctx, "generation_tape"))) return rc;
    CK(cudaEventRecord(ctx->kern_done[s], ctx->stream));
    // the caller's host arrays are free once the copies are done
    CK(cudaEventSynchronize(ctx->copy_done[s]));
    ctx->set ^= 1u;
    ctx->pops[0]->hostN = tape->N;
    return 0;
}

int clotho_generation_philox(clotho_ctx* ctx, uint32_t N) {
    int rc = require_ready(ctx);
    if (rc) return rc;
    if (ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "a staged generation is in progress");
    for (size_t i = 0; i < ctx->pops.size(); ++i)
        if (N > ctx->pops[i]->dev[2].Ncap) return fail(ctx, CLOTHO_E_CAPACITY, "N exceeds max_individuals");
    uint32_t slot;
    uint32_t* h = hdr_stage(ctx, &slot);
    if (!h) return fail(ctx, CLOTHO_E_NOMEM, "pinned host memory refused");
    for (size_t i = 0; i < ctx->pops.size(); ++i) {
        h[2 * i] = N;
        h[2 * i + 1] = 0;
    }
    if ((rc = hdr_copy(ctx, slot, ctx->d_hdr[2], (uint32_t)ctx->pops.size(), ctx->stream))) return rc;
    enqueue_fused_step(ctx, 2, true);
    if ((rc = check_launch(ctx, "generation_philox"))) return rc;
    for (PopHost* p : ctx->pops) p->hostN = N;
    return 0;
}

int clotho_run_philox(clotho_ctx* ctx, uint32_t N, uint32_t G) {
    int rc = require_ready(ctx);
    if (rc) return rc;
    if (ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "a staged generation is in progress");
    if (G == 0) return 0;
    // the first generation runs eagerly (it may need the parent reduction)
    if ((rc = clotho_generation_philox(ctx, N))) return rc;
    if (G == 1) return 0;
    if (ctx->profiling) {  // per-launch events are taken from eager launches
        for (uint32_t g = 1; g < G; ++g)
            if ((rc = clotho_generation_philox(ctx, N))) return rc;
        return 0;
    }
    const std::vector<uint32_t> key(ctx->pops.size(), N);
    if ((rc = capture_step_graph(ctx, key))) return rc;
    for (uint32_t g = 1; g < G; ++g) {
        CK(cudaGraphLaunch(ctx->graph, ctx->stream));
        ctx->launches += ctx->graph_launches;
    }
    return 0;
}

// ---- staged entry points -------------------------------------------------
int clotho_begin_generation(clotho_ctx* ctx, uint32_t N, uint32_t M) {
    int rc = require_ready(ctx);
    if (rc) return rc;
    if (ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "generation already begun");
    PopHost* p = ctx->pops[0];
    if (N > p->dev[0].Ncap) return fail(ctx, CLOTHO_E_CAPACITY, "N exceeds max_individuals");
    if (M > p->dev[0].Mcap) return fail(ctx, CLOTHO_E_CAPACITY, "M exceeds max_mutations");
    CK(cudaStreamSynchronize(ctx->copy_stream));
    uint32_t slot;
    uint32_t* h = hdr_stage(ctx, &slot);
    if (!h) return fail(ctx, CLOTHO_E_NOMEM, "pinned host memory refused");
    h[0] = N;
    h[1] = M;
    if ((rc = hdr_copy(ctx, slot, ctx->d_hdr[0], 1, ctx->stream))) return rc;
    launch_begin(cfg(ctx), ctx->d_pops[0], 1, ctx->d_hdr[0], ctx->d_ctl);
    ctx->launches += 1;
    ctx->in_step = true;
    p->hostN = N;
    return check_launch(ctx, "begin");
}

int clotho_free_space(clotho_ctx* ctx, uint32_t* counts) {
    if (!ctx || !ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "clotho_begin_generation first");
    PopHost* p = ctx->pops[0];
    if (!p->acc_valid) {
        launch_fs_reduce(cfg(ctx), ctx->d_pops[0], 1, ctx->maxW, 1u);
        ctx->launches += 1;
    }
    launch_fs_finalize(cfg(ctx), ctx->d_pops[0], 1);
    ctx->launches += 1;
    p->acc_valid = false;  // reset for the child; the staged crossover does not refill it
    int rc = check_launch(ctx, "free_space");
    if (rc) return rc;
    if (counts) {
        DevStatus s = read_status(ctx, p, &rc);
        if (rc) return rc;
        counts[0] = s.fixed_cnt;
        counts[1] = s.lost_cnt;
        counts[2] = s.free_cnt;
    }
    return 0;
}

int clotho_set_pairs(clotho_ctx* ctx, const uint32_t* pairs) {
    if (!ctx || !ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "clotho_begin_generation first");
    PopHost* p = ctx->pops[0];
    int rc = h2d(ctx, p->dev[0].pairs, pairs, 2ull * p->hostN, ctx->stream);
    ctx->pairs_set = 0;
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int clotho_select(clotho_ctx* ctx, uint32_t* pairs_out) {
    if (!ctx || !ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "clotho_begin_generation first");
    PopHost* p = ctx->pops[0];
    // device draws write the pairs of the Philox set, which shares buffers with set 0
    launch_select_philox(cfg(ctx), ctx->d_pops[2], 1);
    ctx->launches += 1;
    ctx->pairs_set = 0;
    int rc = check_launch(ctx, "select");
    if (rc) return rc;
    if (pairs_out) {
        CK(cudaMemcpyAsync(pairs_out, p->dev[2].pairs, 2ull * p->hostN * 4, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return 0;
}

int clotho_crossover(clotho_ctx* ctx, const uint8_t* swap, const uint32_t* ev_off, const double* ev_pos) {
    if (!ctx || !ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "clotho_begin_generation first");
    PopHost* p = ctx->pops[0];
    const PopDev& D = p->dev[0];
    const uint32_t N = p->hostN;
    if (!ev_off) return fail(ctx, CLOTHO_E_ARG, "ev_off is null");
    const uint32_t ev_total = ev_off[2ull * N];
    if (ev_total > D.EVcap) return fail(ctx, CLOTHO_E_CAPACITY, "events exceed max_events");
    int rc;
    if ((rc = h2d(ctx, D.swap, swap, 2ull * N, ctx->stream))) return rc;
    if ((rc = h2d(ctx, D.ev_off, ev_off, 2ull * N + 1, ctx->stream))) return rc;
    if ((rc = h2d(ctx, D.ev_pos, ev_pos, (size_t)ev_total, ctx->stream))) return rc;
    // item prefix is already set by begin; ranks over the current positions
    launch_ranks(cfg(ctx), ctx->d_pops[0], 1, ctx->maxNB, ctx->maxW, ctx->n_suf > 0);
    ctx->launches += 6u + (ctx->n_suf > 0 ? 1u : 0u);
    launch_gen(ctx, ctx->d_pops[0], 1, 0u);
    if ((rc = check_launch(ctx, "crossover"))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int clotho_mutate(clotho_ctx* ctx, const uint32_t* mut_seq, const double* mut_pos, const float* mut_eff) {
    if (!ctx || !ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "clotho_begin_generation first");
    PopHost* p = ctx->pops[0];
    const PopDev& D = p->dev[0];
    int rc;
    DevStatus s = read_status(ctx, p, &rc);
    if (rc) return rc;
    const uint32_t M = s.M;
    if ((rc = h2d(ctx, D.mut_seq, mut_seq, (size_t)M, ctx->stream))) return rc;
    if ((rc = h2d(ctx, D.mut_pos, mut_pos, (size_t)M, ctx->stream))) return rc;
    if ((rc = h2d(ctx, D.mut_eff, mut_eff, (size_t)M * D.T, ctx->stream))) return rc;
    launch_mut_resolve(cfg(ctx), ctx->d_pops[0], 1);
    launch_mut_scatter(cfg(ctx), ctx->d_pops[0], 1);
    ctx->launches += 2;
    if ((rc = check_launch(ctx, "mutate"))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int clotho_phenotype(clotho_ctx* ctx) {
    if (!ctx) return CLOTHO_E_ARG;
    launch_phenotype(cfg(ctx), ctx->d_pops[0], 1);
    ctx->launches += 1;
    return check_launch(ctx, "phenotype");
}

int clotho_fitness(clotho_ctx* ctx) {
    if (!ctx) return CLOTHO_E_ARG;
    launch_individuals(cfg(ctx), ctx->d_pops[0], 1);
    launch_cdf(cfg(ctx), ctx->d_pops[0], 1, ctx->maxN);
    ctx->launches += 4;
    return check_launch(ctx, "fitness");
}

int clotho_end_generation(clotho_ctx* ctx) {
    if (!ctx || !ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "no generation in progress");
    launch_end(cfg(ctx), ctx->d_pops[0], 1);
    ctx->launches += 1;
    ctx->in_step = false;
    int rc = check_launch(ctx, "end");
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

// ---- read-back -------------------------------------------------------------
static int info_of(clotho_ctx* ctx, uint32_t idx, clotho_info* out) {
    if (!ctx || !out || idx >= ctx->pops.size()) return fail(ctx, CLOTHO_E_ARG, "no such population");
    CK(cudaStreamSynchronize(ctx->copy_stream));
    int rc;
    DevStatus s = read_status(ctx, ctx->pops[idx], &rc);
    if (rc) return rc;
    out->generation = s.gen;
    out->N = s.N;
    out->A = s.A;
    out->W = s.W;
    out->fixed_count = s.fixed_cnt;
    out->lost_count = s.lost_cnt;
    out->free_count = s.free_cnt;
    out->variable_count = (s.pA > s.free_cnt ? s.pA - s.free_cnt : 0);
    out->fixed_total = s.fixed_total;
    out->last_M = s.last_M;
    out->all_neutral = s.all_neutral;
    out->device_error = s.err;
    out->mean_fitness = s.N ? s.fit_total / (double)s.N : 0.0;
    return 0;
}

int clotho_get_info(clotho_ctx* ctx, clotho_info* out) { return info_of(ctx, 0, out); }

static void info_from_status(const DevStatus& s, clotho_info* out) {
    out->generation = s.gen;
    out->N = s.N;
    out->A = s.A;
    out->W = s.W;
    out->fixed_count = s.fixed_cnt;
    out->lost_count = s.lost_cnt;
    out->free_count = s.free_cnt;
    out->variable_count = (s.pA > s.free_cnt ? s.pA - s.free_cnt : 0);
    out->fixed_total = s.fixed_total;
    out->last_M = s.last_M;
    out->all_neutral = s.all_neutral;
    out->device_error = s.err;
    out->mean_fitness = s.N ? s.fit_total / (double)s.N : 0.0;
}


// The status copy is ordered behind everything issued so far on the context's stream; the host
// thread goes on issuing work and collects the copy with clotho_info_wait.
static int info_request(clotho_ctx* ctx, uint32_t idx, uint32_t* ticket) {
    if (!ctx || !ticket || idx >= ctx->pops.size()) return fail(ctx, CLOTHO_E_ARG, "no such population");
    if (!ctx->h_stat) {
        if (cudaMallocHost(&ctx->h_stat, sizeof(DevStatus) * kStatRing) != cudaSuccess) {
            cudaGetLastError();
            ctx->h_stat = nullptr;
            return fail(ctx, CLOTHO_E_NOMEM, "pinned host memory refused");
        }
        for (uint32_t k = 0; k < kStatRing; ++k) CK(cudaEventCreateWithFlags(&ctx->stat_ev[k], cudaEventDisableTiming));
    }
    const uint32_t t = ctx->stat_next;
    const uint32_t k = t % kStatRing;
    if (t >= kStatRing) CK(cudaEventSynchronize(ctx->stat_ev[k]));  // the slot's previous copy has landed
    CK(cudaMemcpyAsync(&ctx->h_stat[k], ctx->pops[idx]->dev[0].st, sizeof(DevStatus), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaEventRecord(ctx->stat_ev[k], ctx->stream));
    ctx->stat_next = t + 1;
    *ticket = t;
    return 0;
}

static int info_wait(clotho_ctx* ctx, uint32_t ticket, clotho_info* out) {
    if (!ctx || !out) return CLOTHO_E_ARG;
    if (ticket >= ctx->stat_next || ctx->stat_next - ticket > kStatRing)
        return fail(ctx, CLOTHO_E_ARG, "unknown or overwritten info ticket");
    const uint32_t k = ticket % kStatRing;
    CK(cudaEventSynchronize(ctx->stat_ev[k]));
    info_from_status(ctx->h_stat[k], out);
    return 0;
}

int clotho_info_request(clotho_ctx* ctx, uint32_t* ticket) { return info_request(ctx, 0, ticket); }
int clotho_pop_info_request(clotho_ctx* ctx, uint32_t index, uint32_t* ticket) {
    return info_request(ctx, index, ticket);
}
int clotho_info_wait(clotho_ctx* ctx, uint32_t ticket, clotho_info* out) { return info_wait(ctx, ticket, out); }

static int rows_of(clotho_ctx* ctx, uint32_t idx, uint64_t* dst, size_t dst_words) {
    if (!ctx || idx >= ctx->pops.size()) return fail(ctx, CLOTHO_E_ARG, "no such population");
    int rc;
    PopHost* p = ctx->pops[idx];
    DevStatus s = read_status(ctx, p, &rc);
    if (rc) return rc;
    const size_t S = 2ull * s.N, W = s.W;
    if (S * W == 0) return 0;
    if (!dst || dst_words < S * W) return fail(ctx, CLOTHO_E_ARG, "destination too small");
    CK(cudaMemcpy2DAsync(dst, W * 8, p->dev[0].rows[s.cur], (size_t)p->dev[0].Wcap * 8, W * 8, S,
                         cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int clotho_get_rows(clotho_ctx* ctx, uint64_t* dst, size_t dst_words) { return rows_of(ctx, 0, dst, dst_words); }

int clotho_get_alleles(clotho_ctx* ctx, double* pos, uint32_t* age, float* eff) {
    if (!ctx) return CLOTHO_E_ARG;
    int rc;
    PopHost* p = ctx->pops[0];
    DevStatus s = read_status(ctx, p, &rc);
    if (rc) return rc;
    const PopDev& D = p->dev[0];
    if (pos && s.A) CK(cudaMemcpyAsync(pos, D.pos, (size_t)s.A * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (age && s.A) CK(cudaMemcpyAsync(age, D.age, (size_t)s.A * 4, cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<float> pad((size_t)s.A * 4);
    if (eff && s.A) CK(cudaMemcpyAsync(pad.data(), D.eff, (size_t)s.A * 16, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (eff)
        for (size_t i = 0; i < s.A; ++i)
            for (uint32_t t = 0; t < D.T; ++t) eff[i * D.T + t] = pad[i * 4 + t];
    return 0;
}

int clotho_get_fixed(clotho_ctx* ctx, double* pos, uint32_t* age, float* eff) {
    if (!ctx) return CLOTHO_E_ARG;
    int rc;
    PopHost* p = ctx->pops[0];
    DevStatus s = read_status(ctx, p, &rc);
    if (rc) return rc;
    const PopDev& D = p->dev[0];
    const size_t F = s.fixed_total;
    if (pos && F) CK(cudaMemcpyAsync(pos, D.fx_pos, F * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (age && F) CK(cudaMemcpyAsync(age, D.fx_age, F * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (eff && F) CK(cudaMemcpyAsync(eff, D.fx_eff, F * D.T * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int clotho_get_free(clotho_ctx* ctx, uint32_t* dst) {
    if (!ctx) return CLOTHO_E_ARG;
    int rc;
    PopHost* p = ctx->pops[0];
    DevStatus s = read_status(ctx, p, &rc);
    if (rc) return rc;
    if (s.free_cnt && !dst) return fail(ctx, CLOTHO_E_ARG, "null destination");
    if (s.free_cnt)
        CK(cudaMemcpyAsync(dst, p->dev[0].free_list, (size_t)s.free_cnt * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

static int get_double4(clotho_ctx* ctx, const double* src, size_t n, double* dst) {
    const uint32_t T = ctx->pops[0]->dev[0].T;
    std::vector<double> tmp(n * 4);
    if (n) CK(cudaMemcpyAsync(tmp.data(), src, n * 32, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i < n; ++i)
        for (uint32_t t = 0; t < T; ++t) dst[i * T + t] = tmp[i * 4 + t];
    return 0;
}

int clotho_get_genome_traits(clotho_ctx* ctx, double* dst) {
    if (!ctx) return CLOTHO_E_ARG;
    int rc;
    DevStatus s = read_status(ctx, ctx->pops[0], &rc);
    if (rc) return rc;
    return get_double4(ctx, ctx->pops[0]->dev[0].zg[s.cur], 2ull * s.N, dst);
}

int clotho_get_phenotypes(clotho_ctx* ctx, double* dst) {
    if (!ctx) return CLOTHO_E_ARG;
    int rc;
    DevStatus s = read_status(ctx, ctx->pops[0], &rc);
    if (rc) return rc;
    return get_double4(ctx, ctx->pops[0]->dev[0].zi, s.N, dst);
}

int clotho_get_fitness(clotho_ctx* ctx, double* dst) {
    if (!ctx) return CLOTHO_E_ARG;
    int rc;
    DevStatus s = read_status(ctx, ctx->pops[0], &rc);
    if (rc) return rc;
    if (s.N) CK(cudaMemcpyAsync(dst, ctx->pops[0]->dev[0].fit, (size_t)s.N * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int clotho_get_pairs(clotho_ctx* ctx, uint32_t* dst) {
    if (!ctx) return CLOTHO_E_ARG;
    int rc;
    DevStatus s = read_status(ctx, ctx->pops[0], &rc);
    if (rc) return rc;
    // tape steps alternate between sets 0 and 1; device draws and the staged calls use set 0's buffer
    const PopDev& D = ctx->pops[0]->dev[ctx->pairs_set];
    if (s.N) CK(cudaMemcpyAsync(dst, D.pairs, 2ull * s.N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

static int stats_of(clotho_ctx* ctx, uint32_t idx, clotho_stats* out, uint32_t* sfs, uint32_t sfs_len) {
    if (!ctx || !out || idx >= ctx->pops.size()) return fail(ctx, CLOTHO_E_ARG, "no such population");
    int rc;
    PopHost* p = ctx->pops[idx];
    DevStatus s = read_status(ctx, p, &rc);
    if (rc) return rc;
    const PopDev& D = p->dev[0];
    const uint32_t A = s.A, S = 2 * s.N;
    std::vector<uint32_t> counts(std::max<size_t>(1, (size_t)s.W * 64), 0);
    if (s.cols_valid) {
        // the last fused step counted the columns of these rows: no pass over the rows
        if (A) CK(cudaMemcpyAsync(counts.data(), D.colcnt, (size_t)A * 4, cudaMemcpyDeviceToHost, ctx->stream));
    } else {
        // scratch column counts from the context's pool: stream-ordered, no device-wide synchronisation
        uint32_t* d_counts = nullptr;
        CK(pool_alloc(ctx, &d_counts, counts.size() * 4));
        CK(cudaMemsetAsync(d_counts, 0, counts.size() * 4, ctx->stream));
        if (S && s.W) launch_stats(cfg(ctx), ctx->d_pops[0], idx, d_counts, s.W);
        CK(cudaMemcpyAsync(counts.data(), d_counts, counts.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaFreeAsync(d_counts, ctx->stream));
        ctx->launches += 1;
    }
    std::vector<double> zi((size_t)s.N * 4);
    if (s.N) CK(cudaMemcpyAsync(zi.data(), D.zi, (size_t)s.N * 32, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    *out = clotho_stats{};
    if (sfs)
        for (uint32_t k = 0; k < sfs_len; ++k) sfs[k] = 0;
    double het = 0.0;
    for (uint32_t a = 0; a < A; ++a) {
        const uint32_t c = counts[a];
        if (c > 0 && c < S) out->segregating += 1;
        if (S && c == S) out->fixed_now += 1;
        if (S) {
            const double f = (double)c / (double)S;
            het += 2.0 * f * (1.0 - f);
        }
        if (sfs && sfs_len) sfs[c < sfs_len ? c : sfs_len - 1] += 1;
    }
    out->heterozygosity = het;
    out->mean_fitness = s.N ? s.fit_total / (double)s.N : 0.0;
    for (uint32_t t = 0; t < 4; ++t) {
        double m = 0.0;
        for (uint32_t i = 0; i < s.N; ++i) m += zi[(size_t)i * 4 + t];
        out->mean_phenotype[t] = s.N ? m / s.N : 0.0;
    }
    return 0;
}

int clotho_stats_compute(clotho_ctx* ctx, clotho_stats* out, uint32_t* sfs, uint32_t sfs_len) {
    return stats_of(ctx, 0, out, sfs, sfs_len);
}

static int margins_of(clotho_ctx* ctx, uint32_t idx, uint32_t* col, uint32_t* row) {
    if (!ctx || idx >= ctx->pops.size()) return fail(ctx, CLOTHO_E_ARG, "no such population");
    int rc;
    PopHost* p = ctx->pops[idx];
    const DevStatus s = read_status(ctx, p, &rc);
    if (rc) return rc;
    const uint32_t S = 2 * s.N;
    const size_t ncol = std::max<size_t>(1, (size_t)s.W * 64), nrow = std::max<uint32_t>(1, S);
    uint32_t* d = nullptr;
    CK(pool_alloc(ctx, &d, (ncol + nrow) * 4));
    CK(cudaMemsetAsync(d, 0, (ncol + nrow) * 4, ctx->stream));
    if (col && S && s.W) launch_stats(cfg(ctx), ctx->d_pops[0], idx, d, s.W);
    if (row && S) launch_row_counts(cfg(ctx), ctx->d_pops[0], idx, d + ncol, S);
    if (col && s.A) CK(cudaMemcpyAsync(col, d, (size_t)s.A * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (row && S) CK(cudaMemcpyAsync(row, d + ncol, (size_t)S * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaFreeAsync(d, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->launches += (col ? 1 : 0) + (row ? 1 : 0);
    return check_launch(ctx, "margins");
}

int clotho_margins(clotho_ctx* ctx, uint32_t* col, uint32_t* row) { return margins_of(ctx, 0, col, row); }
int clotho_pop_margins(clotho_ctx* ctx, uint32_t index, uint32_t* col, uint32_t* row) {
    return margins_of(ctx, index, col, row);
}

static int pairwise_of(clotho_ctx* ctx, uint32_t idx, const uint32_t* sample, uint32_t n, uint32_t* dist,
                       clotho_pairwise* out) {
    if (!ctx || !out || idx >= ctx->pops.size()) return fail(ctx, CLOTHO_E_ARG, "no such population");
    if (n > 65536u) return fail(ctx, CLOTHO_E_CAPACITY, "pairwise difference: sample of more than 65,536 rows");
    if (dist && n > 16384u) return fail(ctx, CLOTHO_E_CAPACITY, "pairwise distances: sample of more than 16,384 rows");
    int rc;
    PopHost* p = ctx->pops[idx];
    const DevStatus s = read_status(ctx, p, &rc);
    if (rc) return rc;
    const uint32_t S = 2 * s.N;
    std::vector<uint32_t> smp(n);
    for (uint32_t i = 0; i < n; ++i) {
        smp[i] = sample ? sample[i] : i;
        if (smp[i] >= S) return fail(ctx, CLOTHO_E_ARG, "pairwise difference: sample row out of range");
    }
    *out = clotho_pairwise{};
    const uint64_t pairs = n > 1 ? (uint64_t)n * (n - 1) / 2 : 0;
    if (!pairs) return 0;
    uint32_t* d_smp = nullptr;
    uint32_t* d_dist = nullptr;
    PairwiseOut* d_out = nullptr;
    CK(pool_alloc(ctx, &d_smp, (size_t)n * 4));
    CK(pool_alloc(ctx, &d_out, sizeof(PairwiseOut)));
    if (dist) CK(pool_alloc(ctx, &d_dist, pairs * 4));
    PairwiseOut h{};
    h.min = 0xffffffffu;
    CK(cudaMemcpyAsync(d_smp, smp.data(), (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(d_out, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
    launch_pairwise(cfg(ctx), ctx->d_pops[0], idx, d_smp, n, d_dist, d_out);
    rc = check_launch(ctx, "pairwise difference");
    CK(cudaMemcpyAsync(&h, d_out, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    if (dist) CK(cudaMemcpyAsync(dist, d_dist, pairs * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaFreeAsync(d_smp, ctx->stream));
    CK(cudaFreeAsync(d_out, ctx->stream));
    if (d_dist) CK(cudaFreeAsync(d_dist, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->launches += 1;
    if (rc) return rc;
    out->count = h.count;
    out->total = h.total;
    out->min = h.count ? h.min : 0;
    out->max = h.max;
    out->mean = h.count ? (double)h.total / (double)h.count : 0.0;
    out->variance = h.count ? (double)h.sumsq / (double)h.count - out->mean * out->mean : 0.0;
    if (out->variance < 0.0) out->variance = 0.0;
    return 0;
}

int clotho_pairwise_difference(clotho_ctx* ctx, const uint32_t* sample, uint32_t n, uint32_t* dist,
                               clotho_pairwise* out) {
    return pairwise_of(ctx, 0, sample, n, dist, out);
}
int clotho_pop_pairwise_difference(clotho_ctx* ctx, uint32_t index, const uint32_t* sample, uint32_t n,
                                   uint32_t* dist, clotho_pairwise* out) {
    return pairwise_of(ctx, index, sample, n, dist, out);
}

// ---- checkpoint / resume ---------------------------------------------------
namespace {
constexpr char kSnapMagic[8] = {'C', 'L', 'O', 'T', 'H', 'O', 'S', '1'};

struct SnapHeader {
    char magic[8];
    uint32_t version, header_bytes;
    clotho_desc desc;
    DevStatus st;
    uint64_t total_bytes;
};

struct SnapLayout {
    size_t rows, pos, age, eff, fx_pos, fx_age, fx_eff, free_list, zg, zi, fit, cdf, total;
};

// Byte offsets of the sections after the header, each 8-byte aligned.
SnapLayout snap_layout(const DevStatus& st, uint32_t T) {
    SnapLayout L{};
    const size_t S = 2ull * st.N, N = st.N, A = st.A, F = st.fixed_total;
    size_t o = sizeof(SnapHeader);
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += (bytes + 7) & ~(size_t)7;
        return at;
    };
    L.rows = take(S * st.W * 8);
    L.pos = take(A * 8);
    L.age = take(A * 4);
    L.eff = take(A * 16);
    L.fx_pos = take(F * 8);
    L.fx_age = take(F * 4);
    L.fx_eff = take(F * T * 4);
    L.free_list = take((size_t)st.free_cnt * 4);
    L.zg = take(S * 32);
    L.zi = take(N * 32);
    L.fit = take(N * 8);
    L.cdf = take(N * 8);
    L.total = o;
    return L;
}

bool same_parameters(const clotho_desc& a, const clotho_desc& b) {
    return a.traits == b.traits && a.fitness == b.fitness && a.flags == b.flags && a.fit_param == b.fit_param &&
           a.mu == b.mu && a.rho == b.rho && a.bias == b.bias && a.p_neutral == b.p_neutral &&
           a.eff_mean == b.eff_mean && a.eff_sigma == b.eff_sigma && a.seed == b.seed;
}
}  // namespace

size_t clotho_snapshot_size(clotho_ctx* ctx) {
    if (!ctx || ctx->pops.size() != 1 || ctx->in_step || !ctx->pops[0]->ready) return 0;
    int rc;
    const DevStatus st = read_status(ctx, ctx->pops[0], &rc);
    return rc ? 0 : snap_layout(st, ctx->pops[0]->dev[0].T).total;
}

int clotho_snapshot(clotho_ctx* ctx, void* dst, size_t len) {
    if (!ctx || !dst) return CLOTHO_E_ARG;
    if (ctx->pops.size() != 1) return fail(ctx, CLOTHO_E_ARG, "snapshot takes a single-population context");
    if (ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "snapshot between generations only");
    PopHost* p = ctx->pops[0];
    if (!p->ready) return fail(ctx, CLOTHO_E_STATE, "population not initialised");
    int rc;
    const DevStatus st = read_status(ctx, p, &rc);
    if (rc) return rc;
    const PopDev& D = p->dev[0];
    const SnapLayout L = snap_layout(st, D.T);
    if (len < L.total) return fail(ctx, CLOTHO_E_CAPACITY, "snapshot buffer too small");
    char* b = static_cast<char*>(dst);
    SnapHeader h{};
    std::memcpy(h.magic, kSnapMagic, 8);
    h.version = 2;
    h.header_bytes = sizeof(SnapHeader);
    h.desc = p->desc;
    h.st = st;
    h.total_bytes = L.total;
    std::memcpy(b, &h, sizeof(h));
    const size_t S = 2ull * st.N, F = st.fixed_total;
    cudaStream_t s = ctx->stream;
    if (S * st.W)
        CK(cudaMemcpy2DAsync(b + L.rows, (size_t)st.W * 8, D.rows[st.cur], (size_t)D.Wcap * 8, (size_t)st.W * 8, S,
                             cudaMemcpyDeviceToHost, s));
    if (st.A) {
        CK(cudaMemcpyAsync(b + L.pos, D.pos, (size_t)st.A * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(b + L.age, D.age, (size_t)st.A * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(b + L.eff, D.eff, (size_t)st.A * 16, cudaMemcpyDeviceToHost, s));
    }
    if (F) {
        CK(cudaMemcpyAsync(b + L.fx_pos, D.fx_pos, F * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(b + L.fx_age, D.fx_age, F * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(b + L.fx_eff, D.fx_eff, F * D.T * 4, cudaMemcpyDeviceToHost, s));
    }
    if (st.free_cnt)
        CK(cudaMemcpyAsync(b + L.free_list, D.free_list, (size_t)st.free_cnt * 4, cudaMemcpyDeviceToHost, s));
    if (S) CK(cudaMemcpyAsync(b + L.zg, D.zg[st.cur], S * 32, cudaMemcpyDeviceToHost, s));
    if (st.N) {
        CK(cudaMemcpyAsync(b + L.zi, D.zi, (size_t)st.N * 32, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(b + L.fit, D.fit, (size_t)st.N * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(b + L.cdf, D.cdf, (size_t)st.N * 8, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    return 0;
}

int clotho_restore(clotho_ctx* ctx, const void* src, size_t len) {
    if (!ctx || !src) return CLOTHO_E_ARG;
    if (ctx->pops.size() != 1) return fail(ctx, CLOTHO_E_ARG, "restore takes a single-population context");
    if (ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "restore between generations only");
    if (len < sizeof(SnapHeader)) return fail(ctx, CLOTHO_E_ARG, "not a snapshot (too short)");
    SnapHeader h;
    std::memcpy(&h, src, sizeof(h));
    if (std::memcmp(h.magic, kSnapMagic, 8) != 0 || h.version != 2 || h.header_bytes != sizeof(SnapHeader))
        return fail(ctx, CLOTHO_E_ARG, "not a snapshot of this library version");
    PopHost* p = ctx->pops[0];
    const PopDev& D = p->dev[0];
    DevStatus st = h.st;
    if (st.cur > 1u || st.W != ref_width(st.A)) return fail(ctx, CLOTHO_E_ARG, "snapshot status is inconsistent");
    const SnapLayout L = snap_layout(st, D.T);
    if (h.total_bytes != L.total || len < L.total) return fail(ctx, CLOTHO_E_ARG, "snapshot truncated");
    if (!same_parameters(h.desc, p->desc))
        return fail(ctx, CLOTHO_E_ARG, "snapshot parameters differ from the context's");
    if (st.N > D.Ncap || st.A > D.Acap || st.W > D.Wcap || st.fixed_total > D.FXcap || st.free_cnt > D.Acap)
        return fail(ctx, CLOTHO_E_CAPACITY, "snapshot does not fit the context's capacities");
    const char* b = static_cast<const char*>(src);
    const size_t S = 2ull * st.N, F = st.fixed_total;
    // Everything below reaches device kernels as an index or a count: check it here, on the host, so a
    // damaged or hand-edited snapshot is refused instead of sending a kernel out of bounds.
    {
        if ((uint64_t)st.fixed_cnt + st.lost_cnt != st.free_cnt)
            return fail(ctx, CLOTHO_E_ARG, "snapshot free-list counts are inconsistent");
        std::vector<uint32_t> fl(st.free_cnt);
        if (st.free_cnt) std::memcpy(fl.data(), b + L.free_list, fl.size() * 4);
        for (uint32_t v : fl)
            if (v >= st.W * 64u) return fail(ctx, CLOTHO_E_ARG, "snapshot free list holds a slot beyond the rows");
        std::vector<double> pos(st.A);
        if (st.A) std::memcpy(pos.data(), b + L.pos, pos.size() * 8);
        for (double x : pos)
            if (!(x >= 0.0) || !std::isfinite(x)) return fail(ctx, CLOTHO_E_ARG, "snapshot allele position invalid");
        std::vector<float> eff((size_t)st.A * 4);
        if (st.A) std::memcpy(eff.data(), b + L.eff, eff.size() * 4);
        int64_t nz = 0;
        for (size_t a = 0; a < st.A; ++a)
            for (uint32_t t = 0; t < 4; ++t) {
                if (t >= D.T && eff[a * 4 + t] != 0.0f)
                    return fail(ctx, CLOTHO_E_ARG, "snapshot effects of unused traits are not zero");
                nz += eff[a * 4 + t] != 0.0f;
            }
        if (nz != st.nz_eff) return fail(ctx, CLOTHO_E_ARG, "snapshot effect count is inconsistent");
        // no row carries a slot at or beyond A (the reference never sets one; the classifiers index by slot)
        const uint32_t tail = st.A % 64u, last = st.A / 64u;
        if (st.W && (tail || last < st.W))
            for (size_t r = 0; r < S; ++r) {
                const uint64_t* row = reinterpret_cast<const uint64_t*>(b + L.rows) + r * st.W;
                uint64_t beyond = 0;
                std::memcpy(&beyond, row + last, last < st.W ? 8 : 0);
                if (tail) beyond &= ~((1ull << tail) - 1ull);
                for (uint32_t w = last + 1; w < st.W; ++w) {
                    uint64_t x;
                    std::memcpy(&x, row + w, 8);
                    beyond |= x;
                }
                if (beyond) return fail(ctx, CLOTHO_E_ARG, "snapshot rows carry slots beyond the allele count");
            }
    }
    int rc = init_pop(ctx, 0, st.N);  // zeroed tables and counters
    if (rc) return rc;
    st.count_cols = ctx->pops[0]->counting ? 1u : 0u;  // the context's own choice, not the snapshot's
    st.cols_valid = 0u;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(D.st, &st, sizeof(DevStatus), cudaMemcpyHostToDevice, s));
    if (S * st.W)
        CK(cudaMemcpy2DAsync(D.rows[st.cur], (size_t)D.Wcap * 8, b + L.rows, (size_t)st.W * 8, (size_t)st.W * 8, S,
                             cudaMemcpyHostToDevice, s));
    if (st.A) {
        CK(cudaMemcpyAsync(D.pos, b + L.pos, (size_t)st.A * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.age, b + L.age, (size_t)st.A * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.eff, b + L.eff, (size_t)st.A * 16, cudaMemcpyHostToDevice, s));
    }
    if (F) {
        CK(cudaMemcpyAsync(D.fx_pos, b + L.fx_pos, F * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.fx_age, b + L.fx_age, F * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.fx_eff, b + L.fx_eff, F * D.T * 4, cudaMemcpyHostToDevice, s));
    }
    if (st.free_cnt)
        CK(cudaMemcpyAsync(D.free_list, b + L.free_list, (size_t)st.free_cnt * 4, cudaMemcpyHostToDevice, s));
    if (S) CK(cudaMemcpyAsync(D.zg[st.cur], b + L.zg, S * 32, cudaMemcpyHostToDevice, s));
    if (st.N) {
        CK(cudaMemcpyAsync(D.zi, b + L.zi, (size_t)st.N * 32, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.fit, b + L.fit, (size_t)st.N * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.cdf, b + L.cdf, (size_t)st.N * 8, cudaMemcpyHostToDevice, s));
    }
    CK(cudaStreamSynchronize(s));
    p->acc_valid = false;  // the next step reduces the restored rows again
    p->hostN = st.N;
    if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; }
    return 0;
}

// ---- timing --------------------------------------------------------------
int clotho_profile(clotho_ctx* ctx, int enable) {
    if (!ctx) return CLOTHO_E_ARG;
    int rc = prof_collect(ctx);
    if (rc) return rc;
    ctx->profiling = enable != 0;
    ctx->phase_clocks = enable == 2;
    ctx->prof_ms = 0.0;
    ctx->prof_launches = 0;
    if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; }
    CK(cudaMemsetAsync(&ctx->d_ctl->rows_done, 0, 16 + sizeof(ctx->d_ctl->phase), ctx->stream));
    return 0;
}

int clotho_phase_clocks(clotho_ctx* ctx, uint64_t* out, uint32_t n) {
    static_assert(kPhCount == CLOTHO_PHASE_COUNT, "phase list of the header and the kernel differ");
    if (!ctx || (!out && n) || n > CLOTHO_PHASE_COUNT) return CLOTHO_E_ARG;
    uint64_t ph[kPhCount];
    CK(cudaMemcpyAsync(ph, ctx->d_ctl->phase, sizeof(ph), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (uint32_t i = 0; i < n; ++i) out[i] = ph[i];
    return 0;
}

int clotho_kernel_time(clotho_ctx* ctx, double* total_ms, uint32_t* launches, uint64_t* rows, uint64_t* words) {
    if (!ctx) return CLOTHO_E_ARG;
    int rc = prof_collect(ctx);
    if (rc) return rc;
    uint64_t rw[2] = {0, 0};
    CK(cudaMemcpyAsync(rw, &ctx->d_ctl->rows_done, 16, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (total_ms) *total_ms = ctx->prof_ms;
    if (launches) *launches = ctx->prof_launches;
    if (rows) *rows = rw[0];
    if (words) *words = rw[1];
    return 0;
}

int clotho_host_alloc(size_t bytes, void** out) {
    if (!out) return CLOTHO_E_ARG;
    *out = nullptr;
    if (cudaMallocHost(out, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        return CLOTHO_E_NOMEM;
    }
    return 0;
}

int clotho_host_free(void* p) {
    if (p && cudaFreeHost(p) != cudaSuccess) return CLOTHO_E_CUDA;
    return 0;
}

int clotho_timer_begin(clotho_ctx* ctx) {
    if (!ctx) return CLOTHO_E_ARG;
    CK(cudaEventRecord(ctx->t0, ctx->stream));
    return 0;
}

int clotho_timer_end(clotho_ctx* ctx, double* ms) {
    if (!ctx) return CLOTHO_E_ARG;
    CK(cudaEventRecord(ctx->t1, ctx->stream));
    CK(cudaEventSynchronize(ctx->t1));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, ctx->t0, ctx->t1));
    if (ms) *ms = f;
    return 0;
}

// ---- batched and served populations --------------------------------------
int clotho_batch_create(const clotho_desc* descs, uint32_t n, clotho_ctx** out) {
    if (!out || (n && !descs) || n > kMaxPops) return CLOTHO_E_ARG;
    *out = nullptr;
    clotho_ctx* ctx = nullptr;
    if (n == 0) {
        // an empty context for a serving loop: create with a tiny population, then drop it
        clotho_desc d{};
        d.max_individuals = 1;
        d.max_alleles = 64;
        d.traits = 1;
        int rc = clotho_create(&d, &ctx);
        if (rc) return rc;
        free_pop(ctx, ctx->pops[0]);
        ctx->pops.clear();
        rc = sync_pop_arrays(ctx);
        if (rc) { clotho_destroy(ctx); return rc; }
        *out = ctx;
        return 0;
    }
    int rc = clotho_create(&descs[0], &ctx);
    if (rc) return rc;
    for (uint32_t i = 1; i < n; ++i) {
        PopHost* p = nullptr;
        rc = alloc_pop(ctx, descs[i], &p);
        if (rc) { clotho_destroy(ctx); return rc; }
        ctx->pops.push_back(p);
    }
    rc = sync_pop_arrays(ctx);
    if (rc) { clotho_destroy(ctx); return rc; }
    *out = ctx;
    return 0;
}

uint32_t clotho_pop_count(const clotho_ctx* ctx) { return ctx ? (uint32_t)ctx->pops.size() : 0u; }

int clotho_pop_add(clotho_ctx* ctx, const clotho_desc* desc, uint32_t* index) {
    if (!ctx || !desc) return CLOTHO_E_ARG;
    if (ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "a staged generation is in progress");
    if (ctx->pops.size() >= kMaxPops) return fail(ctx, CLOTHO_E_CAPACITY, "256 populations resident");
    CK(cudaStreamSynchronize(ctx->stream));
    PopHost* p = nullptr;
    int rc = alloc_pop(ctx, *desc, &p);
    if (rc) return rc;
    ctx->pops.push_back(p);
    rc = sync_pop_arrays(ctx, (uint32_t)ctx->pops.size() - 1);
    if (rc) return rc;
    if (index) *index = (uint32_t)ctx->pops.size() - 1;
    return 0;
}

int clotho_pop_remove(clotho_ctx* ctx, uint32_t index) {
    if (!ctx || index >= ctx->pops.size()) return fail(ctx, CLOTHO_E_ARG, "no such population");
    CK(cudaStreamSynchronize(ctx->copy_stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->pops[index]->counting) {
        ctx->counting -= 1;
        ctx->tuning_epoch += 1;  // the step's kernels change when the last counting population leaves
    }
    free_pop(ctx, ctx->pops[index]);
    ctx->pops.erase(ctx->pops.begin() + index);
    return sync_pop_arrays(ctx, index);
}

int clotho_pop_count_columns(clotho_ctx* ctx, uint32_t index, int enable) {
    if (!ctx || index >= ctx->pops.size()) return fail(ctx, CLOTHO_E_ARG, "no such population");
    PopHost* p = ctx->pops[index];
    const bool on = enable != 0;
    if (p->counting == on) return 0;
    const uint32_t v = on ? 1u : 0u;
    CK(cudaMemcpyAsync(&p->dev[0].st->count_cols, &v, 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    p->counting = on;
    ctx->counting += on ? 1u : (uint32_t)-1;
    ctx->tuning_epoch += 1;  // a captured step re-captures with (or without) the counting build
    return 0;
}

int clotho_pop_init(clotho_ctx* ctx, uint32_t index, uint32_t N0) { return init_pop(ctx, index, N0); }

int clotho_pop_info(clotho_ctx* ctx, uint32_t index, clotho_info* out) { return info_of(ctx, index, out); }

int clotho_pop_rows(clotho_ctx* ctx, uint32_t index, uint64_t* dst, size_t dst_words) {
    return rows_of(ctx, index, dst, dst_words);
}

int clotho_pop_stats(clotho_ctx* ctx, uint32_t index, clotho_stats* out, uint32_t* sfs, uint32_t sfs_len) {
    return stats_of(ctx, index, out, sfs, sfs_len);
}

int clotho_batch_generation_philox(clotho_ctx* ctx, const uint32_t* N) {
    int rc = require_ready(ctx);
    if (rc) return rc;
    if (!N) return fail(ctx, CLOTHO_E_ARG, "null N");
    if (ctx->pops.empty()) return 0;
    if (ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "a staged generation is in progress");
    for (size_t i = 0; i < ctx->pops.size(); ++i)
        if (N[i] > ctx->pops[i]->dev[2].Ncap) return fail(ctx, CLOTHO_E_CAPACITY, "N exceeds max_individuals");
    uint32_t slot;
    uint32_t* h = hdr_stage(ctx, &slot);
    if (!h) return fail(ctx, CLOTHO_E_NOMEM, "pinned host memory refused");
    for (size_t i = 0; i < ctx->pops.size(); ++i) {
        h[2 * i] = N[i];
        h[2 * i + 1] = 0;
    }
    if ((rc = hdr_copy(ctx, slot, ctx->d_hdr[2], (uint32_t)ctx->pops.size(), ctx->stream))) return rc;
    enqueue_fused_step(ctx, 2, true);
    if ((rc = check_launch(ctx, "batch_generation_philox"))) return rc;
    for (size_t i = 0; i < ctx->pops.size(); ++i) ctx->pops[i]->hostN = N[i];
    return 0;
}

int clotho_batch_run_philox(clotho_ctx* ctx, const uint32_t* N, uint32_t G) {
    int rc = require_ready(ctx);
    if (rc) return rc;
    if (G == 0 || ctx->pops.empty()) return 0;
    if ((rc = clotho_batch_generation_philox(ctx, N))) return rc;
    if (G == 1) return 0;
    if (ctx->profiling) {
        for (uint32_t g = 1; g < G; ++g)
            if ((rc = clotho_batch_generation_philox(ctx, N))) return rc;
        return 0;
    }
    const std::vector<uint32_t> key(N, N + ctx->pops.size());
    if ((rc = capture_step_graph(ctx, key))) return rc;
    for (uint32_t g = 1; g < G; ++g) {
        CK(cudaGraphLaunch(ctx->graph, ctx->stream));
        ctx->launches += ctx->graph_launches;
    }
    return 0;
}

int clotho_run_philox_schedule(clotho_ctx* ctx, const uint32_t* N, uint32_t G) {
    int rc = require_ready(ctx);
    if (rc) return rc;
    if (!N) return fail(ctx, CLOTHO_E_ARG, "null schedule");
    if (ctx->in_step) return fail(ctx, CLOTHO_E_STATE, "a staged generation is in progress");
    const uint32_t n = (uint32_t)ctx->pops.size();
    if (G == 0 || n == 0) return 0;
    std::vector<uint32_t> hdr(2ull * n * G, 0u);
    for (uint32_t g = 0; g < G; ++g)
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t v = N[(size_t)g * n + i];
            if (v > ctx->pops[i]->dev[2].Ncap)
                return fail(ctx, CLOTHO_E_CAPACITY, "schedule N exceeds max_individuals");
            hdr[2ull * ((size_t)g * n + i)] = v;
        }
    if (ctx->profiling) {  // per-launch events are taken from eager launches
        for (uint32_t g = 0; g < G; ++g)
            if ((rc = clotho_batch_generation_philox(ctx, N + (size_t)g * n))) return rc;
        return 0;
    }
    uint32_t* d_sched = nullptr;
    CK(pool_alloc(ctx, &d_sched, hdr.size() * 4));
    // every exit after the allocation goes through the one free below
    auto body = [&]() -> int {
        CK(cudaMemcpyAsync(d_sched, hdr.data(), hdr.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
        // the first generation runs eagerly (it may need the parent reduction)
        CK(cudaMemcpyAsync(ctx->d_hdr[2], d_sched, 8ull * n, cudaMemcpyDeviceToDevice, ctx->stream));
        enqueue_fused_step(ctx, 2, true);
        int r = check_launch(ctx, "run_philox_schedule");
        if (r || G == 1) return r;
        // every size of a step is read from the device status word, so one graph
        // serves all generations; only the step header changes between replays
        if ((r = capture_step_graph(ctx, std::vector<uint32_t>{0xffffffffu, n}))) return r;
        for (uint32_t g = 1; g < G; ++g) {
            CK(cudaMemcpyAsync(ctx->d_hdr[2], d_sched + 2ull * n * g, 8ull * n, cudaMemcpyDeviceToDevice,
                               ctx->stream));
            CK(cudaGraphLaunch(ctx->graph, ctx->stream));
            ctx->launches += ctx->graph_launches;
        }
        return 0;
    };
    rc = body();
    const cudaError_t e_free = cudaFreeAsync(d_sched, ctx->stream);
    const cudaError_t e_sync = cudaStreamSynchronize(ctx->stream);
    if (rc) return rc;
    CK(e_free);
    CK(e_sync);
    for (uint32_t i = 0; i < n; ++i) ctx->pops[i]->hostN = N[(size_t)(G - 1) * n + i];
    return 0;
}

int clotho_set_copy_wait_limit(clotho_ctx* ctx, uint32_t rounds) {
    if (!ctx) return CLOTHO_E_ARG;
    if (rounds > (1u << 30)) return fail(ctx, CLOTHO_E_ARG, "wait limit above 2^30 rounds");
    CK(cudaMemcpyAsync(&ctx->d_ctl->wait_limit, &rounds, sizeof(rounds), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return 0;
}

int clotho_set_tuning(clotho_ctx* ctx, const clotho_tuning* t) {
    if (!ctx || !t) return CLOTHO_E_ARG;
    if (t->rows_per_item > 65536 || t->row_blocks_per_sm > 64 || t->narrow_build > 1)
        return fail(ctx, CLOTHO_E_ARG, "tuning value out of range");
    if (t->rows_per_item) {
        int rc = clotho_set_rows_per_item(ctx, t->rows_per_item);
        if (rc) return rc;
    }
    ctx->ind_per_sm = t->row_blocks_per_sm ? t->row_blocks_per_sm : 16u;
    ctx->narrow_ok = t->narrow_build != 0u;
    ctx->tuning_epoch += 1;  // graphs captured under the old launch shapes are not replayed
    return 0;
}

int clotho_get_tuning(clotho_ctx* ctx, clotho_tuning* t) {
    if (!ctx || !t) return CLOTHO_E_ARG;
    uint32_t rpi = 0;
    CK(cudaMemcpyAsync(&rpi, &ctx->d_ctl->rows_per_item, 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    t->rows_per_item = rpi;
    t->narrow_build = ctx->narrow_ok ? 1u : 0u;
    t->row_blocks_per_sm = ctx->ind_per_sm;
    return 0;
}

int clotho_set_rows_per_item(clotho_ctx* ctx, uint32_t rows) {
    if (!ctx || rows == 0 || rows > 65536) return CLOTHO_E_ARG;
    CK(cudaMemcpyAsync(&ctx->d_ctl->rows_per_item, &rows, 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; }
    return 0;
}

int clotho_mem_info(size_t* free_bytes, size_t* total_bytes) {
    size_t f = 0, t = 0;
    if (cudaMemGetInfo(&f, &t) != cudaSuccess) {
        cudaGetLastError();
        return CLOTHO_E_CUDA;
    }
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return 0;
}

}  // extern "C"
