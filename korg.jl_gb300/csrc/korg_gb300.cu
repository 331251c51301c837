// korg_gb300.cu -- C ABI, context, scratch arena and launch orchestration of the GB300
// synthesis hot path.  Kernels live in lines.cuh, hydrogen.cuh and rt.cuh.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "../../include/korg_gb300.h"
#include "adjoint.cuh"
#include "continuum.cuh"
#include "hydrogen.cuh"
#include "hydrogen_adj.cuh"
#include "lines.cuh"
#include "postprocess.cuh"
#include "physics.cuh"
#include "rt.cuh"
#include "statmech.cuh"

using namespace korg;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
};

constexpr int NEV = 13;  // 0-7: forward stages and probes; 8-12: reverse-mode stages

// Tile shape of the line tile kernel: wavelengths per CTA and lines per shared-memory batch
// (0: the default for the precision).
struct TileCfg {
    int tw, stage, split;  // split: one layer group per CTA
};
struct TuneRecord {
    int L, mixed, tw, stage, split;
    float ms;
};

}  // namespace

struct korg_ctx {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;  // used by the host-pointer calls and for graph capture
    std::string err;
    // scratch arena: grown on demand, never shrunk, freed by korg_destroy
    DevBuf lines_scratch, counters, tune_alpha;
    DevBuf hrec, hQ, hQ32, hulb, huub;
    DevBuf stage_dev, aref, alpha, flux, cntm, math;
    DevBuf vjp_g, vjp_dpar, vjp_small, vjp_hder, vjp_hdq;  // reverse mode
    DevBuf mx_layers;                            // molecular cross-section layer inputs
    void* stage_host = nullptr;
    size_t stage_host_cap = 0;
    int* dev_err_host = nullptr;  // mapped host word: set by kernels whose bounded waits ran out
    int* dev_err_dev = nullptr;
    // batched synthesis: chunk alpha, per-spectrum line scratch, tile arguments + reference
    // wavelengths + queue counters (device), their host staging (pinned, batch-only)
    DevBuf b_alpha, b_lines, b_meta;
    void* b_host = nullptr;
    size_t b_host_cap = 0;
    cudaEvent_t b_host_ev = nullptr;  // after the last copy out of b_host
    int64_t batch_budget = int64_t(32) << 30;
    // the last batch: its key, whether it ran in one chunk (then every spectrum's alpha, line
    // prologue and alpha_ref stay in b_alpha / b_lines / b_meta until the next batch), and where
    // the per-spectrum pieces lie -- for a batched reverse mode that reuses the forward's opacity
    std::vector<unsigned char> b_last_key;
    bool b_last_resident = false;
    std::vector<size_t> b_last_line_off;
    size_t b_last_o_aref = 0, b_last_o_refwl = 0;
    // CUDA graph of the last batch: replayed while the same batch is submitted again
    bool use_graph = false, capturing = false;
    cudaGraphExec_t gexec = nullptr;
    std::vector<unsigned char> gkey, pending_key;
    // autotuned tile shapes per (layers, precision)
    bool autotune = false;
    std::map<std::pair<int, int>, TileCfg> tuned;
    std::vector<TuneRecord> tune_log;
    // continuum-absorption tables (one device buffer)
    bool have_cntm = false;
    CntmTables cntm_tab{};
    void* cntm_buf = nullptr;
    // chemical-equilibrium tables (one device buffer)
    bool have_chem = false;
    ChemTables chem_tab{};
    void* chem_buf = nullptr;
    double chem_lnT0 = 0, chem_lnT1 = 0;  // knot range of the atomic partition functions
    // Stehle tables
    bool have_stark = false;
    StarkDev stark{};
    int n_max = 0;
    std::vector<void*> stark_allocs;
    // the hydrogen prep records and tables now in hrec / hQ: -1 none, 0 FP64, 1 mixed (FP64 and FP32)
    int hyd_prep = -1;
    // statistics
    bool timing = false;
    cudaEvent_t ev[NEV] = {};
    korg_stats stats{};
    bool stats_pending = false;
    bool vjp_timed = false;
};

namespace {

int set_err(korg_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->err = buf;
    return code;
}

#define KCUDA(call)                                                                       \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return set_err(ctx, KORG_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                           __FILE__, __LINE__);                                           \
    } while (0)

#define KCHECK(expr)                  \
    do {                              \
        int r_ = (expr);              \
        if (r_ != KORG_OK) return r_; \
    } while (0)

// precision must be KORG_FP64 or KORG_MIXED; anything else is a caller error, not the FP64 form
#define KPREC(prec)                                                                          \
    do {                                                                                     \
        if ((prec) != KORG_FP64 && (prec) != KORG_MIXED)                                     \
            return set_err(ctx, KORG_EINVAL, "precision must be KORG_FP64 (0) or KORG_MIXED (1), got %d", \
                           int(prec));                                                       \
    } while (0)

void drop_graph(korg_ctx* ctx) {
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
    ctx->gkey.clear();
    ctx->pending_key.clear();
}

int ensure(korg_ctx* ctx, DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return KORG_OK;
    if (ctx->capturing) return set_err(ctx, KORG_EINVAL, "scratch would grow during graph capture");
    if (b.p) {
        drop_graph(ctx);  // a captured graph holds the old address
        KCUDA(cudaStreamSynchronize(ctx->stream));
        KCUDA(cudaDeviceSynchronize());
        cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
    }
    size_t want = bytes + bytes / 4;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return set_err(ctx, KORG_ENOMEM, "cudaMalloc(%zu): %s", want, cudaGetErrorString(e));
    }
    b.cap = want;
    return KORG_OK;
}

// zero the evaluation counters at the start of a public call that runs line kernels
int reset_counters(korg_ctx* ctx, cudaStream_t s) {
    KCHECK(ensure(ctx, ctx->counters, 4 * sizeof(unsigned long long)));
    KCUDA(cudaMemsetAsync(ctx->counters.p, 0, 4 * sizeof(unsigned long long), s));
    ctx->stats_pending = true;
    return KORG_OK;
}

void record(korg_ctx* ctx, int i, cudaStream_t s) {
    if (ctx->timing && !ctx->capturing) cudaEventRecord(ctx->ev[i], s);
}

// Layers per thread (K) and layer groups per CTA (G = ceil(L/K) <= 8); layers are padded to
// G*K.  56-layer (MARCS) atmospheres split exactly into 4 x 14.
// Tables of the table-driven FP64 exp / log (physics.cuh), in extended precision on the host.
void fill_math_tables(MathTables& t) {
    for (int j = 0; j < MATH_TABLE_N; j++) {
        t.exp2j[j] = double(exp2l((long double)j / (long double)MATH_TABLE_N));
        const long double c = 1.0L + ((long double)j + 0.5L) / (long double)MATH_TABLE_N;
        const double ic = double(1.0L / c);
        t.inv_c[j] = ic;
        t.log_c[j] = double(-logl((long double)ic));
    }
}

int layer_groups(int L, int* kmax) {
    if (L % 14 == 0 && L / 14 <= 8) { *kmax = 14; return L / 14; }
    int G = (L + 15) / 16;
    if (G <= 8) { *kmax = 16; return G; }
    G = (L + 31) / 32;
    if (G <= 8) { *kmax = 32; return G; }
    return -1;
}

LinesDev lines_dev(const korg_lines* l) {
    return LinesDev{l->n, l->wl, l->log_gf, l->E_lower, l->gamma_rad, l->gamma_stark, l->vdW1, l->vdW2,
                    l->mass, l->is_mol, l->species};
}
LayersDev layers_dev(const korg_layers* y) {
    return LayersDev{y->L, y->S, y->T, y->ne, y->n_eff_vdW, y->xi, y->n_div_U};
}

// ------------------------------------------------------------------ line opacity
constexpr int TILE_TW = 128;  // default wavelengths per CTA of the line tile kernel

// Pieces of the per-spectrum scratch of the line prologue and candidate lists.
struct LineScratch {
    LayerConst* lc = nullptr;
    void* params = nullptr;
    float* xfar = nullptr;
    uint32_t* amask = nullptr;
    int32_t *lb = nullptr, *ub = nullptr, *ci = nullptr, *tier_idx = nullptr, *tier_ci = nullptr, *tier_meta = nullptr;
    float4* params_w = nullptr;  // mixed: wing cubics, after the packed constants
    float* xcub = nullptr;       // mixed: cubic boundaries [n][G], after xfar
};

size_t a256(size_t x) { return (x + 255) & ~size_t(255); }
int part_blocks(int64_t n) { return int((n + PART_CHUNK - 1) / PART_CHUNK); }

// Bytes of one LineScratch for n lines (every piece 256-byte aligned); with base != null, the
// pieces are carved out of base.
size_t line_scratch(unsigned char* base, int64_t n, int L, int Lp, int G, bool mixed, LineScratch* out) {
    const size_t nn = size_t(std::max<int64_t>(n, 1));
    const size_t sz[10] = {sizeof(LayerConst) * L, (mixed ? 2 * sizeof(float4) : sizeof(P64)) * nn * Lp,
                           sizeof(float) * nn * G * (mixed ? 2 : 1), sizeof(uint32_t) * nn, 4 * nn, 4 * nn, 4 * nn,
                           4 * nn, 4 * nn,
                           sizeof(int32_t) * (NTIER * size_t(part_blocks(n)) + NTIER + 2)};
    size_t off[10], tot = 0;
    for (int i = 0; i < 10; i++) { off[i] = tot; tot += a256(sz[i]); }
    if (base && out) {
        out->lc = reinterpret_cast<LayerConst*>(base + off[0]);
        out->params = base + off[1];
        out->params_w = mixed ? reinterpret_cast<float4*>(base + off[1]) + nn * Lp : nullptr;
        out->xfar = reinterpret_cast<float*>(base + off[2]);
        out->xcub = mixed ? out->xfar + nn * G : nullptr;
        out->amask = reinterpret_cast<uint32_t*>(base + off[3]);
        out->lb = reinterpret_cast<int32_t*>(base + off[4]);
        out->ub = reinterpret_cast<int32_t*>(base + off[5]);
        out->ci = reinterpret_cast<int32_t*>(base + off[6]);
        out->tier_idx = reinterpret_cast<int32_t*>(base + off[7]);
        out->tier_ci = reinterpret_cast<int32_t*>(base + off[8]);
        out->tier_meta = reinterpret_cast<int32_t*>(base + off[9]);
    }
    return tot;
}

// Tile-kernel arguments that follow from the scratch and the inputs (launch geometry aside).
TileArgs make_tile_args(const LineScratch& sc, double* alpha, const double* wls, int64_t nwl, const LinesDev& ln,
                        int L, int Lp, int G) {
    TileArgs ta{};
    ta.alpha = alpha;
    ta.wls = wls;
    ta.nwl = nwl;
    ta.L = L;
    ta.Lp = Lp;
    ta.G = G;
    ta.xfar = sc.xfar;
    ta.amask = sc.amask;
    ta.n = ln.n;
    ta.wl = ln.wl;
    ta.params = sc.params;
    ta.params_w = sc.params_w;
    ta.xcub = sc.xcub;
    ta.lb = sc.lb;
    ta.ub = sc.ub;
    ta.tier_idx = sc.tier_idx;
    ta.tier_ci = sc.tier_ci;
    ta.tier_start = sc.tier_meta;                 // [start: NTIER+1][unsorted][block counts]
    ta.unsorted = sc.tier_meta + NTIER + 1;
    return ta;
}

// Per-line prologue (constants, windows, classes) and the width-tier candidate lists.
int prep_lines(korg_ctx* ctx, const LineScratch& sc, const double* wls, int64_t nwl, const LinesDev& ln,
               const LayersDev& lay, const CntmDev& cn, double cutoff, bool mixed, int kmax, int G,
               cudaStream_t s) {
    const int L = lay.L, Lp = G * kmax;
    auto* ctr = static_cast<unsigned long long*>(ctx->counters.p);
    layer_const_kernel<<<(L + 127) / 128, 128, 0, s>>>(lay, sc.lc);
    PrepOut po{sc.params, sc.lb, sc.ub, sc.ci, sc.xfar, sc.amask, Lp, kmax, G, ctr, ctr + 1, sc.params_w, sc.xcub};
    const size_t prep_smem = size_t(256 / 32) * Lp * (sizeof(float) + sizeof(int));
    const unsigned pblocks = unsigned((ln.n * 32 + 255) / 256);
    auto* math = static_cast<MathTables*>(ctx->math.p);
    if (mixed)
        line_prep_mixed_kernel<<<prep_mixed_blocks(ln.n), 32 * PREP_WARPS, prep_mixed_smem(Lp), s>>>(
            ln, lay, sc.lc, cn, wls, nwl, cutoff, po, math);
    else
        line_prep64_kernel<<<pblocks, 256, prep_smem, s>>>(ln, lay, sc.lc, cn, wls, nwl, cutoff, po, math);
    KCUDA(cudaGetLastError());
    const int nblk = part_blocks(ln.n);
    TierLists tl{sc.tier_idx, sc.tier_ci, sc.tier_meta, sc.tier_meta + NTIER + 1};
    int32_t* bcnt = sc.tier_meta + NTIER + 2;
    KCUDA(cudaMemsetAsync(tl.unsorted, 0, sizeof(int32_t), s));
    tier_count_kernel<<<nblk, PART_THREADS, 0, s>>>(sc.lb, sc.ub, sc.ci, ln.n, bcnt, tl.unsorted);
    tier_scatter_kernel<<<nblk, PART_THREADS, 0, s>>>(sc.lb, sc.ub, sc.ci, ln.n, bcnt, nblk, tl);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

// Launch shape of the tile kernel: TW wavelengths x G layer groups per CTA, `stage` lines per
// shared-memory batch.
struct TileGeom {
    int tw, threads, stage, region, split, G;
    size_t smem;
};

// One wavelength per thread; the mixed form always takes one layer group per CTA, the FP64 form
// one or all layer groups.
bool tile_geom(bool mixed, int Lp, int G, TileCfg c, TileGeom* g) {
    const size_t psz = mixed ? sizeof(float4) : sizeof(P64);
    const int B = c.stage > 0 ? c.stage : (mixed ? 2 * STAGE_LINES : STAGE_LINES / 2);
    if (mixed && !c.split) return false;
    const int Gc = c.split ? 1 : G;  // layer groups per CTA
    const int SL = c.split ? Lp / G : Lp;
    const int maxt = mixed ? 256 : 512;
    if (c.tw < 32 || c.tw % 32 != 0 || c.tw * Gc > maxt || B < 1) return false;
    size_t region = size_t(B) * SL * psz;
    region = std::max(region, (size_t(c.tw) * (SL + 1) * sizeof(double) + 1) / 2);
    region = (region + 15) & ~size_t(15);
    g->tw = c.tw;
    g->threads = c.tw * Gc;
    g->stage = B;
    g->region = int(region);
    g->split = c.split ? 1 : 0;
    g->G = G;
    g->smem = 2 * region + size_t(g->threads) * (mixed ? sizeof(LineStage32) : sizeof(LineStage));
    return g->smem <= 227 * 1024;
}

// Default tile shape: 128 wavelengths x one layer group (mixed: 64-line batches, FP64: 16).
TileCfg default_tile(bool) { return TileCfg{TILE_TW, 0, 1}; }

template <bool MIXED, int KMAX, int MAXT, int MINB>
int launch_tile(korg_ctx* ctx, TileArgs ta, const TileGeom& g, const TileQueue* q, cudaStream_t s) {
    ta.stage = g.stage;
    ta.region = g.region;
    ta.split = g.split;
    if (q) {
        auto kern = line_tile_queue_kernel<MIXED, KMAX, MAXT, MINB>;
        KCUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(g.smem)));
        int per_sm = 0;
        KCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, g.threads, g.smem));
        const int64_t grid = std::min<int64_t>(q->nitems, int64_t(ctx->sms) * std::max(per_sm, 1));
        if (grid > 0) kern<<<unsigned(grid), g.threads, g.smem, s>>>(*q);
    } else {
        auto kern = line_tile_kernel<MIXED, KMAX, MAXT, MINB>;
        KCUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(g.smem)));
        const int64_t tiles = (ta.nwl + g.tw - 1) / g.tw;
        kern<<<dim3(unsigned(tiles), g.split ? unsigned(g.G) : 1u), g.threads, g.smem, s>>>(ta);
    }
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

template <bool MIXED>
int dispatch_tile(korg_ctx* ctx, const TileArgs& ta, int kmax, const TileGeom& g, const TileQueue* q,
                  cudaStream_t s) {
    if constexpr (MIXED) {  // at most 256 threads (one layer group per CTA)
        if (kmax == 14) return launch_tile<true, 14, 256, 3>(ctx, ta, g, q, s);
        if (kmax == 16) return launch_tile<true, 16, 256, 2>(ctx, ta, g, q, s);
        return launch_tile<true, 32, 256, 2>(ctx, ta, g, q, s);
    } else {
        if (kmax == 14 && g.threads <= 256) return launch_tile<false, 14, 256, 2>(ctx, ta, g, q, s);
        if (kmax == 14) return launch_tile<false, 14, 512, 1>(ctx, ta, g, q, s);
        if (kmax == 16) return launch_tile<false, 16, 512, 1>(ctx, ta, g, q, s);
        return launch_tile<false, 32, 512, 1>(ctx, ta, g, q, s);
    }
}

int run_tiles(korg_ctx* ctx, const TileArgs& ta, int kmax, const TileGeom& g, const TileQueue* q, bool mixed,
              cudaStream_t s) {
    return mixed ? dispatch_tile<true>(ctx, ta, kmax, g, q, s) : dispatch_tile<false>(ctx, ta, kmax, g, q, s);
}

// The tile shape for (L, precision): the autotuned one when there is one, else the default.
TileCfg tile_cfg(const korg_ctx* ctx, int L, bool mixed) {
    auto it = ctx->tuned.find(std::make_pair(L, int(mixed)));
    return it != ctx->tuned.end() ? it->second : default_tile(mixed);
}

// Autotuner: times every candidate shape (FP64: TW in {32, 64, 128} x stage in {8, 16} x split
// or not; mixed: TW in {64, 128, 256} x stage in {32, 64}, split) on the real candidate lists of
// one spectrum, writing into a scratch alpha, and keeps the fastest for (L, precision).  Runs
// once per (L, precision) per context, outside any stream capture.
int autotune_tiles(korg_ctx* ctx, const TileArgs& ta0, int kmax, bool mixed, cudaStream_t s) {
    const int L = ta0.L, Lp = ta0.Lp, G = ta0.G;
    const auto key = std::make_pair(L, int(mixed));
    if (ctx->tuned.count(key)) return KORG_OK;
    KCHECK(ensure(ctx, ctx->tune_alpha, sizeof(double) * size_t(L) * ta0.nwl));
    KCUDA(cudaMemsetAsync(ctx->tune_alpha.p, 0, sizeof(double) * size_t(L) * ta0.nwl, s));
    TileArgs ta = ta0;
    ta.alpha = static_cast<double*>(ctx->tune_alpha.p);
    const int B0 = mixed ? 2 * STAGE_LINES : STAGE_LINES / 2;
    TileCfg best = default_tile(mixed);
    float best_ms = 1e30f;
    for (int split : {0, 1})
    for (int tw : {64, 32, 128, 256, 512})
        for (int B : {B0, B0 / 2}) {
            if (mixed ? (tw < 64 || !split) : tw > 128) continue;
            TileGeom g;
            if (!tile_geom(mixed, Lp, G, TileCfg{tw, B, split}, &g)) continue;
            float t = 1e30f;
            for (int rep = 0; rep < 3; rep++) {
                KCUDA(cudaEventRecord(ctx->ev[6], s));
                KCHECK(run_tiles(ctx, ta, kmax, g, nullptr, mixed, s));
                KCUDA(cudaEventRecord(ctx->ev[7], s));
                KCUDA(cudaEventSynchronize(ctx->ev[7]));
                float ms = 0;
                KCUDA(cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]));
                if (rep > 0) t = std::min(t, ms);
            }
            ctx->tune_log.push_back({L, int(mixed), tw, B, split, t});
            if (t < best_ms) { best_ms = t; best = TileCfg{tw, B, split}; }
        }
    ctx->tuned[key] = best;
    return KORG_OK;
}

// Candidate lists big enough to be worth tuning on (a few thousand tiles).
bool worth_tuning(int64_t nwl, int64_t nlines) { return nwl >= 100000 && nlines >= 10000; }

int run_line_absorption(korg_ctx* ctx, double* alpha, const double* wls, int64_t nwl, const LinesDev& ln,
                        const LayersDev& lay, const CntmDev& cn, double cutoff, bool mixed,
                        cudaStream_t s) {
    if (ln.n == 0) return KORG_OK;  // src/line_absorption.jl:35-37
    const int L = lay.L;
    int kmax = 0;
    const int G = layer_groups(L, &kmax);
    if (G < 0) return set_err(ctx, KORG_EINVAL, "at most 256 layers are supported (got %d)", L);
    if (ln.n > INT32_MAX || nwl > INT32_MAX - 1) return set_err(ctx, KORG_EINVAL, "sizes exceed int32 indexing");
    const int Lp = G * kmax;
    KCHECK(ensure(ctx, ctx->lines_scratch, line_scratch(nullptr, ln.n, L, Lp, G, mixed, nullptr)));
    LineScratch sc;
    line_scratch(static_cast<unsigned char*>(ctx->lines_scratch.p), ln.n, L, Lp, G, mixed, &sc);
    KCHECK(prep_lines(ctx, sc, wls, nwl, ln, lay, cn, cutoff, mixed, kmax, G, s));
    record(ctx, 2, s);
    const TileArgs ta = make_tile_args(sc, alpha, wls, nwl, ln, L, Lp, G);
    if (ctx->autotune && !ctx->capturing && worth_tuning(nwl, ln.n)) KCHECK(autotune_tiles(ctx, ta, kmax, mixed, s));
    TileGeom g;
    if (!tile_geom(mixed, Lp, G, tile_cfg(ctx, L, mixed), &g)) return set_err(ctx, KORG_EINVAL, "bad tile shape");
    ctx->stats_pending = true;
    return run_tiles(ctx, ta, kmax, g, nullptr, mixed, s);
}

// ------------------------------------------------------------------ hydrogen lines
// The per-(transition, layer) records and profile tables of the hydrogen lines (the prep kernels).
int run_hydrogen_prep(korg_ctx* ctx, const double* wls, int64_t nwl, const HLayers& hl, double window, int use_MHD,
                      bool mixed, cudaStream_t s, HOut* out) {
    if (!ctx->have_stark) return set_err(ctx, KORG_ENOTABLES, "korg_set_stark_tables() has not been called");
    const int L = hl.L;
    const int ntrans = ctx->stark.ntrans;
    const int nbr = std::max(0, ctx->n_max - 4);
    const int ntot = ntrans + nbr;
    KCHECK(ensure(ctx, ctx->hrec, sizeof(HRec) * size_t(ntot) * L));
    KCHECK(ensure(ctx, ctx->hQ, sizeof(double) * (size_t(ntrans) * L * HND_MAX + size_t(nbr) * L * BR_NP)));
    KCHECK(ensure(ctx, ctx->hQ32, sizeof(float) * size_t(ntrans) * L * HND_MAX));
    KCHECK(ensure(ctx, ctx->hulb, sizeof(int32_t) * ntot));
    KCHECK(ensure(ctx, ctx->huub, sizeof(int32_t) * ntot));
    KCUDA(cudaMemsetAsync(ctx->hulb.p, 0x7f, sizeof(int32_t) * ntot, s));
    KCUDA(cudaMemsetAsync(ctx->huub.p, 0xff, sizeof(int32_t) * ntot, s));
    HOut ho{static_cast<HRec*>(ctx->hrec.p), static_cast<double*>(ctx->hQ.p), static_cast<float*>(ctx->hQ32.p),
            static_cast<int32_t*>(ctx->hulb.p), static_cast<int32_t*>(ctx->huub.p)};
    const int n = ntrans * L;
    if (mixed)
        hline_prep_kernel<true><<<(n + 127) / 128, 128, 0, s>>>(ctx->stark, hl, wls, nwl, window, use_MHD, ho, ho.Q);
    else
        hline_prep_kernel<false><<<(n + 127) / 128, 128, 0, s>>>(ctx->stark, hl, wls, nwl, window, use_MHD, ho, ho.Q);
    KCUDA(cudaGetLastError());
    double* brQ = ho.Q + size_t(ntrans) * L * HND_MAX;
    if (nbr > 0) {
        if (mixed)
            brackett_prep_kernel<true><<<dim3(nbr, L), 256, 0, s>>>(hl, ntrans, ctx->n_max, wls, nwl, use_MHD, ho, brQ);
        else
            brackett_prep_kernel<false><<<dim3(nbr, L), 256, 0, s>>>(hl, ntrans, ctx->n_max, wls, nwl, use_MHD, ho, brQ);
        KCUDA(cudaGetLastError());
    }
    ctx->hyd_prep = mixed ? 1 : 0;
    *out = ho;
    return KORG_OK;
}

int run_hydrogen(korg_ctx* ctx, double* alpha, const double* wls, int64_t nwl, const HLayers& hl, double window,
                 int use_MHD, bool mixed, cudaStream_t s) {
    const int L = hl.L;
    // the hydrogen tile kernel interleaves layers: thread group g owns layers g, g+G, ...
    int kmax = 16, G = (L + 15) / 16;
    if (G > 8) { kmax = 32; G = (L + 31) / 32; }
    if (G > 8) return set_err(ctx, KORG_EINVAL, "at most 256 layers are supported (got %d)", L);
    HOut ho;
    KCHECK(run_hydrogen_prep(ctx, wls, nwl, hl, window, use_MHD, mixed, s, &ho));
    const int ntrans = ctx->stark.ntrans;
    const int ntot = ntrans + std::max(0, ctx->n_max - 4);
    HTileArgs ha{};
    ha.alpha = alpha;
    ha.wls = wls;
    ha.nwl = nwl;
    ha.L = L;
    ha.G = G;
    ha.ntrans = ntrans;
    ha.ntot = ntot;
    ha.rec = ho.rec;
    ha.Q = ho.Q;
    ha.Q32 = ho.Q32;
    ha.ulb = ho.ulb;
    ha.uub = ho.uub;
    ha.d_off = ctx->stark.d_off;
    ha.logdnu = ctx->stark.logdnu;
    ha.logdnu32 = ctx->stark.logdnu32;
    const int TW = G <= 4 ? 128 : 64;
    const unsigned tiles = unsigned((nwl + TW - 1) / TW);
    const int threads = TW * G;
    if (mixed) {
        if (kmax == 16) hline_tile_kernel<true, 16><<<tiles, threads, 0, s>>>(ha);
        else hline_tile_kernel<true, 32><<<tiles, threads, 0, s>>>(ha);
    } else {
        if (kmax == 16) hline_tile_kernel<false, 16><<<tiles, threads, 0, s>>>(ha);
        else hline_tile_kernel<false, 32><<<tiles, threads, 0, s>>>(ha);
    }
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

// ------------------------------------------------------------------ transfer
int run_rt(korg_ctx* ctx, const double* alpha, const double* S, const double* T, const double* wls, int64_t nwl,
           int L, const double* tau_ref, const double* alpha_ref, CntmDev cn, double* flux, double* cntm,
           double unit, cudaStream_t s) {
    RtArgs ra{alpha, S, T, wls, nwl, L, tau_ref, alpha_ref, static_cast<MathTables*>(ctx->math.p), cn, flux, cntm, unit};
    const unsigned blocks = unsigned((nwl + 127) / 128);
    rt_kernel<<<blocks, 128, sizeof(double) * 3 * L, s>>>(ra);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

// ------------------------------------------------------------------ synthesize (device pointers)
int run_synthesize(korg_ctx* ctx, const korg_synth_inputs* in, const LinesDev& ln, const LinesDev& ln5,
                   const double* wls, int64_t nwl, bool mixed, double* flux, double* cntm, double* alpha,
                   double* aref, const double* ref_wl_dev, cudaStream_t s) {
    const LayersDev lay = layers_dev(&in->layers);
    const int L = lay.L;
    const CntmDev cn{in->cntm.nk, in->cntm.knots, in->cntm.vals};
    record(ctx, 0, s);
    // src/synthesize.jl:249-252 alpha from the continuum interpolants
    alpha_init_kernel<<<unsigned((nwl + 63) / 64), 256, 0, s>>>(alpha, wls, nwl, L, cn);
    KCUDA(cudaGetLastError());
    // :265-283 reference-wavelength line opacity on a copy of the continuum alpha_ref, in FP64 in
    // both precisions (one wavelength): the anchored optical depths, and so the continuum flux,
    // carry no FP32 rounding
    KCUDA(cudaMemcpyAsync(aref, in->alpha_ref_cntm, sizeof(double) * L, cudaMemcpyDeviceToDevice, s));
    const CntmDev cref{1, nullptr, in->alpha_ref_cntm};
    record(ctx, 1, s);
    KCHECK(run_line_absorption(ctx, aref, ref_wl_dev, 1, ln5, lay, cref, in->cutoff_threshold, false, s));
    // :293-303 hydrogen lines
    record(ctx, 3, s);
    if (in->hydrogen_lines) {
        const HLayers hl{L, lay.T, lay.ne, in->nH_I, in->nHe_I, in->UH_I, lay.xi};
        KCHECK(run_hydrogen(ctx, alpha, wls, nwl, hl, in->hydrogen_window, in->use_MHD, mixed, s));
    }
    // :305-306 metal and molecular lines
    record(ctx, 4, s);
    KCHECK(run_line_absorption(ctx, alpha, wls, nwl, ln, lay, cn, in->cutoff_threshold, mixed, s));
    // :287-291 and :310-318 both transfers in one pass over the columns
    record(ctx, 5, s);
    KCHECK(run_rt(ctx, alpha, nullptr, lay.T, wls, nwl, L, in->tau_ref, aref, cn, flux, cntm, 1e-8, s));
    record(ctx, 6, s);
    return KORG_OK;
}

// ------------------------------------------------------------------ batched synthesis
// Many spectra on one wavelength grid, each with its own atmosphere and (pruned) line list:
// the per-spectrum prologues run first, then ONE persistent tile launch per chunk works
// through the (spectrum, tile) queue, then the transfers.  Spectra are grouped into chunks
// whose alpha and line scratch fit the context's batch budget.
struct BatchPlan {
    int L, Lp, G, kmax;
    bool mixed;
    TileGeom geom;
    std::vector<int> chunk_first;        // first spectrum of each chunk, plus nspec at the end
    std::vector<size_t> line_off;        // offset of each spectrum's line scratch in b_lines
    size_t alpha_bytes, lines_bytes, meta_bytes, host_bytes;
    size_t o_targs, o_refwl, o_aref, o_ctr, o_zero;  // pieces of b_meta (b_host holds the first two)
};

int plan_batch(korg_ctx* ctx, int nspec, const korg_batch_item* it, int64_t nwl, bool mixed, BatchPlan* p) {
    const int L = it[0].in.layers.L;
    for (int i = 0; i < nspec; i++) {
        const korg_batch_item& b = it[i];
        if (b.in.layers.L != L) return set_err(ctx, KORG_EINVAL, "all spectra of a batch need the same layer count");
        if (!b.flux || !b.cntm || b.in.cntm.nk < 2 || !b.in.tau_ref || !b.in.alpha_ref_cntm || b.lines.n < 0 ||
            b.lines5.n < 0 || b.lines.n > INT32_MAX)
            return set_err(ctx, KORG_EINVAL, "bad batch item %d", i);
        if (b.in.hydrogen_lines && !ctx->have_stark)
            return set_err(ctx, KORG_ENOTABLES, "korg_set_stark_tables() has not been called");
    }
    p->L = L;
    p->mixed = mixed;
    p->G = layer_groups(L, &p->kmax);
    if (p->G < 0) return set_err(ctx, KORG_EINVAL, "at most 256 layers are supported (got %d)", L);
    p->Lp = p->G * p->kmax;
    if (!tile_geom(mixed, p->Lp, p->G, tile_cfg(ctx, L, mixed), &p->geom))
        return set_err(ctx, KORG_EINVAL, "bad tile shape");
    const size_t per_alpha = a256(sizeof(double) * size_t(L) * nwl);
    p->chunk_first.assign(1, 0);
    p->line_off.assign(nspec, 0);
    size_t cur_a = 0, cur_l = 0;
    p->alpha_bytes = p->lines_bytes = 0;
    for (int i = 0; i < nspec; i++) {
        const size_t lb = line_scratch(nullptr, it[i].lines.n, L, p->Lp, p->G, mixed, nullptr);
        if (i > p->chunk_first.back() && int64_t(cur_a + cur_l + per_alpha + lb) > ctx->batch_budget) {
            p->chunk_first.push_back(i);
            cur_a = cur_l = 0;
        }
        p->line_off[i] = cur_l;
        cur_a += per_alpha;
        cur_l += lb;
        p->alpha_bytes = std::max(p->alpha_bytes, cur_a);
        p->lines_bytes = std::max(p->lines_bytes, cur_l);
    }
    p->chunk_first.push_back(nspec);
    const int nchunk = int(p->chunk_first.size()) - 1;
    p->o_targs = 0;
    p->o_refwl = a256(sizeof(TileArgs) * nspec);
    p->host_bytes = p->o_refwl + a256(sizeof(double) * nspec);
    p->o_aref = p->host_bytes;
    p->o_ctr = p->o_aref + a256(sizeof(double) * size_t(L) * nspec);
    p->o_zero = p->o_ctr + a256(sizeof(unsigned long long) * nchunk);
    p->meta_bytes = p->o_zero + a256(sizeof(int32_t) * (NTIER + 2));
    return KORG_OK;
}

// Enqueues the whole batch on stream s (also what a graph capture records).
int enqueue_batch(korg_ctx* ctx, const BatchPlan& p, int nspec, const korg_batch_item* it, const double* wls,
                  int64_t nwl, cudaStream_t s) {
    const int L = p.L;
    const bool mixed = p.mixed;
    unsigned char* meta = static_cast<unsigned char*>(ctx->b_meta.p);
    auto* d_targs = reinterpret_cast<TileArgs*>(meta + p.o_targs);
    auto* d_refwl = reinterpret_cast<double*>(meta + p.o_refwl);
    auto* d_aref = reinterpret_cast<double*>(meta + p.o_aref);
    auto* d_ctr = reinterpret_cast<unsigned long long*>(meta + p.o_ctr);
    const int nchunk = int(p.chunk_first.size()) - 1;
    record(ctx, 0, s);
    KCHECK(reset_counters(ctx, s));
    // tile arguments and reference wavelengths, prepared on the host (pinned, batch-only buffer)
    KCUDA(cudaMemcpyAsync(meta, ctx->b_host, p.host_bytes, cudaMemcpyHostToDevice, s));
    // queue counters, and the empty tier table of spectra without lines
    KCUDA(cudaMemsetAsync(d_ctr, 0, p.meta_bytes - p.o_ctr, s));
    const int64_t ntiles = (nwl + p.geom.tw - 1) / p.geom.tw;
    for (int c = 0; c < nchunk; c++) {
        const int s0 = p.chunk_first[c], s1 = p.chunk_first[c + 1];
        for (int i = s0; i < s1; i++) {
            const korg_synth_inputs& in = it[i].in;
            const LayersDev lay = layers_dev(&in.layers);
            const CntmDev cn{in.cntm.nk, in.cntm.knots, in.cntm.vals};
            double* alpha = static_cast<double*>(ctx->b_alpha.p) + size_t(i - s0) * a256(8 * size_t(L) * nwl) / 8;
            double* aref = d_aref + size_t(i) * L;
            // src/synthesize.jl:249-252, 265-283, 293-303 as in the single-spectrum path
            alpha_init_kernel<<<unsigned((nwl + 63) / 64), 256, 0, s>>>(alpha, wls, nwl, L, cn);
            KCUDA(cudaGetLastError());
            KCUDA(cudaMemcpyAsync(aref, in.alpha_ref_cntm, sizeof(double) * L, cudaMemcpyDeviceToDevice, s));
            const CntmDev cref{1, nullptr, in.alpha_ref_cntm};
            KCHECK(run_line_absorption(ctx, aref, d_refwl + i, 1, lines_dev(&it[i].lines5), lay, cref,
                                       in.cutoff_threshold, false, s));
            if (in.hydrogen_lines) {
                const HLayers hl{L, lay.T, lay.ne, in.nH_I, in.nHe_I, in.UH_I, lay.xi};
                KCHECK(run_hydrogen(ctx, alpha, wls, nwl, hl, in.hydrogen_window, in.use_MHD, mixed, s));
            }
            if (it[i].lines.n > 0) {
                LineScratch sc;
                line_scratch(static_cast<unsigned char*>(ctx->b_lines.p) + p.line_off[i], it[i].lines.n, L, p.Lp,
                             p.G, mixed, &sc);
                KCHECK(prep_lines(ctx, sc, wls, nwl, lines_dev(&it[i].lines), lay, cn, in.cutoff_threshold, mixed,
                                  p.kmax, p.G, s));
            }
        }
        record(ctx, 2, s);
        const int groups = p.geom.split ? p.G : 1;
        const TileQueue q{d_targs + s0, s1 - s0, groups, int64_t(s1 - s0) * ntiles * groups, d_ctr + c};
        KCHECK(run_tiles(ctx, TileArgs{}, p.kmax, p.geom, &q, mixed, s));
        record(ctx, 5, s);
        for (int i = s0; i < s1; i++) {
            const korg_synth_inputs& in = it[i].in;
            const CntmDev cn{in.cntm.nk, in.cntm.knots, in.cntm.vals};
            double* alpha = static_cast<double*>(ctx->b_alpha.p) + size_t(i - s0) * a256(8 * size_t(L) * nwl) / 8;
            KCHECK(run_rt(ctx, alpha, nullptr, in.layers.T, wls, nwl, L, in.tau_ref, d_aref + size_t(i) * L, cn,
                          it[i].flux, it[i].cntm, 1e-8, s));
        }
    }
    record(ctx, 6, s);
    ctx->stats_pending = true;
    return KORG_OK;
}

// Device address of spectrum i's alpha in the chunk buffer.
double* batch_alpha(korg_ctx* ctx, const BatchPlan& p, int i, int64_t nwl) {
    int c = 0;
    while (p.chunk_first[c + 1] <= i) c++;
    return static_cast<double*>(ctx->b_alpha.p) + size_t(i - p.chunk_first[c]) * (a256(8 * size_t(p.L) * nwl) / 8);
}

// Host copies of the tile arguments (one per spectrum) and of the reference wavelengths.
void fill_batch_host(korg_ctx* ctx, const BatchPlan& p, int nspec, const korg_batch_item* it, const double* wls,
                     int64_t nwl) {
    unsigned char* h = static_cast<unsigned char*>(ctx->b_host);
    auto* targs = reinterpret_cast<TileArgs*>(h + p.o_targs);
    auto* refwl = reinterpret_cast<double*>(h + p.o_refwl);
    unsigned char* meta = static_cast<unsigned char*>(ctx->b_meta.p);
    auto* zero = reinterpret_cast<int32_t*>(meta + p.o_zero);
    for (int i = 0; i < nspec; i++) {
        LineScratch sc;
        line_scratch(static_cast<unsigned char*>(ctx->b_lines.p) + p.line_off[i], it[i].lines.n, p.L, p.Lp, p.G,
                     p.mixed, &sc);
        if (it[i].lines.n == 0) {
            sc.tier_meta = zero;  // all tier runs empty
        }
        TileArgs ta = make_tile_args(sc, batch_alpha(ctx, p, i, nwl), wls, nwl, lines_dev(&it[i].lines), p.L, p.Lp, p.G);
        ta.stage = p.geom.stage;
        ta.region = p.geom.region;
        ta.split = p.geom.split;
        targs[i] = ta;
        refwl[i] = it[i].in.ref_wl;
    }
}

// Identity of a batch submission: everything the enqueued work depends on.
std::vector<unsigned char> batch_key(korg_ctx* ctx, int nspec, const korg_batch_item* it, const double* wls,
                                     int64_t nwl, int precision) {
    std::vector<unsigned char> k;
    auto put = [&](const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        k.insert(k.end(), c, c + n);
    };
    const int L = it[0].in.layers.L;
    const TileCfg cfg = tile_cfg(ctx, L, precision == KORG_MIXED);
    put(&nspec, sizeof nspec);
    put(it, sizeof(korg_batch_item) * size_t(nspec));
    put(&wls, sizeof wls);
    put(&nwl, sizeof nwl);
    put(&precision, sizeof precision);
    put(&ctx->batch_budget, sizeof ctx->batch_budget);
    put(&cfg, sizeof cfg);
    return k;
}

// ------------------------------------------------------------------ reverse mode (VJP)
__global__ void to_float_kernel(const double* x, int64_t n, float* y) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) y[i] = float(x[i]);
}

// Opacity of a spectrum of the last batch forward, still in the batch buffers.
struct VjpOpacity {
    double* alpha;
    double* aref;
    unsigned char* lines;  // the spectrum's line scratch (prologue constants, windows, tiers)
};

int run_vjp(korg_ctx* ctx, const korg_synth_inputs* in, const LinesDev& ln, const LinesDev& ln5, const double* wls,
            int64_t nwl, bool mixed, const double* dflux, const double* dcntm, const korg_synth_grads& gr, int flags,
            const double* ref_wl_dev, cudaStream_t s, const VjpOpacity* op = nullptr) {
    const LayersDev lay = layers_dev(&in->layers);
    const int L = lay.L, S = lay.S;
    if (L > RTA_LMAX) return set_err(ctx, KORG_EINVAL, "the adjoint supports at most %d layers", RTA_LMAX);
    int kmax = 0;
    const int G = layer_groups(L, &kmax);
    if (G < 0) return set_err(ctx, KORG_EINVAL, "at most 256 layers are supported (got %d)", L);
    const int Lp = G * kmax;
    const CntmDev cn{in->cntm.nk, in->cntm.knots, in->cntm.vals};
    const size_t nLw = size_t(L) * nwl;
    const int64_t nmax = std::max<int64_t>(std::max<int64_t>(ln.n, ln5.n), 1);
    KCHECK(ensure(ctx, ctx->alpha, sizeof(double) * nLw));
    KCHECK(ensure(ctx, ctx->aref, sizeof(double) * (L + 1)));
    KCHECK(ensure(ctx, ctx->vjp_g, (mixed ? sizeof(float) : sizeof(double)) * nLw));
    KCHECK(ensure(ctx, ctx->vjp_dpar, sizeof(double) * 3 * size_t(nmax) * Lp));
    // small pieces: daref [L], a scratch dT [L], counter
    const size_t o_dar = 0, o_dT = a256(8 * L), o_ctr = o_dT + a256(8 * L), o_g32 = o_ctr + 256;
    // line-adjoint items ((chunk, tier) pairs) and the wavelengths as FP32 pairs
    const int np_max = int((nwl + ADJ_CHUNK - 1) / ADJ_CHUNK) * NTIER;
    const size_t o_ilo = o_g32 + a256(4 * L), o_ipre = o_ilo + a256(4 * size_t(np_max)),
                 o_wl2 = o_ipre + a256(8 * size_t(np_max + 1)), small = o_wl2 + a256(8 * size_t(nwl));
    KCHECK(ensure(ctx, ctx->vjp_small, small));
    unsigned char* sm = static_cast<unsigned char*>(ctx->vjp_small.p);
    double* daref = reinterpret_cast<double*>(sm + o_dar);
    double* dT = gr.T ? gr.T : reinterpret_cast<double*>(sm + o_dT);
    auto* ctr = reinterpret_cast<unsigned long long*>(sm + o_ctr);
    // outputs start at zero (every kernel below accumulates)
    auto zero = [&](double* p, size_t n) -> int {
        if (p) KCUDA(cudaMemsetAsync(p, 0, 8 * n, s));
        return KORG_OK;
    };
    KCHECK(zero(dT, L));
    KCHECK(zero(gr.ne, L));
    KCHECK(zero(gr.n_eff_vdW, L));
    KCHECK(zero(gr.xi, L));
    KCHECK(zero(gr.n_div_U, size_t(S) * L));
    KCHECK(zero(gr.nH_I, L));
    KCHECK(zero(gr.nHe_I, L));
    KCHECK(zero(gr.UH_I, L));
    KCHECK(zero(gr.log_gf, size_t(ln.n)));
    KCHECK(zero(gr.cntm_vals, size_t(L) * in->cntm.nk));
    KCHECK(zero(daref, L));
    KCHECK(reset_counters(ctx, s));

    // 1. opacity, recomputed (src/synthesize.jl:249-306 as in the forward), unless the caller
    //    states that the previous call on this context was korg_synthesize[_dev] of the same
    //    inputs, whose alpha, alpha_ref and metal-line prologue are still in the scratch
    record(ctx, 8, s);
    double* alpha = op ? op->alpha : static_cast<double*>(ctx->alpha.p);
    double* aref = op ? op->aref : static_cast<double*>(ctx->aref.p);
    const CntmDev cref{1, nullptr, in->alpha_ref_cntm};
    const HLayers hl{L, lay.T, lay.ne, in->nH_I, in->nHe_I, in->UH_I, lay.xi};
    if (!(flags & KORG_VJP_REUSE_FORWARD) && !op) {
        alpha_init_kernel<<<unsigned((nwl + 63) / 64), 256, 0, s>>>(alpha, wls, nwl, L, cn);
        KCUDA(cudaGetLastError());
        KCUDA(cudaMemcpyAsync(aref, in->alpha_ref_cntm, sizeof(double) * L, cudaMemcpyDeviceToDevice, s));
        KCHECK(run_line_absorption(ctx, aref, ref_wl_dev, 1, ln5, lay, cref, in->cutoff_threshold, false, s));
        if (in->hydrogen_lines)
            KCHECK(run_hydrogen(ctx, alpha, wls, nwl, hl, in->hydrogen_window, in->use_MHD, mixed, s));
        KCHECK(run_line_absorption(ctx, alpha, wls, nwl, ln, lay, cn, in->cutoff_threshold, mixed, s));
    }
    // the metal-line prologue: the batch's for this spectrum, else the context's line scratch (read
    // after step 1, which may have grown it)
    unsigned char* line_base = op ? op->lines : static_cast<unsigned char*>(ctx->lines_scratch.p);
    record(ctx, 9, s);

    // 2. transfer adjoint: opacity cotangent G, dL/dT through the source function, dL/dalpha_ref
    RtAdjArgs ra{alpha, lay.T, wls, nwl, L, in->tau_ref, aref, static_cast<MathTables*>(ctx->math.p), cn, dflux,
                 dcntm, 1e-8, ctx->vjp_g.p, int32_t(mixed), dT, daref, gr.cntm_vals};
    {
        const size_t smem = size_t(RTA_WARPS) * RTA_ARRAYS * (L + 1) * sizeof(double);
        KCUDA(cudaFuncSetAttribute(rt_adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        const int64_t blocks = std::min<int64_t>((nwl + RTA_WARPS - 1) / RTA_WARPS, int64_t(ctx->sms) * 8);
        rt_adjoint_kernel<<<unsigned(blocks), 32 * RTA_WARPS, smem, s>>>(ra);
        KCUDA(cudaGetLastError());
    }
    record(ctx, 10, s);

    // 3. hydrogen lines: alpha_H[l, :] depends only on layer l's inputs.  The forward prep's
    //    records and tables, their derivatives (hline_adj_prep_kernel, brackett_adj_prep_kernel:
    //    dual numbers in T, n_e, xi, n(H I), n(He I)), then one pass over the opacity cotangent
    //    that forms d alpha_H / d input per (wavelength, layer) and contracts it
    //    (hline_adj_kernel); U(H I) from alpha_H itself (alpha_H is proportional to 1 / U(H I)).
    if (in->hydrogen_lines && (flags & KORG_VJP_HYDROGEN)) {
        const int ntrans = ctx->stark.ntrans, nbr = std::max(0, ctx->n_max - 4), ntot = ntrans + nbr;
        if (ntot > HADJ_MAXT)
            return set_err(ctx, KORG_EINVAL, "the hydrogen reverse mode supports %d transitions (got %d)", HADJ_MAXT,
                           ntot);
        // the forward's records and tables when the caller reuses its opacity (unless a batch
        // forward, which overwrote them spectrum by spectrum, ran), else the prep again
        HOut ho{static_cast<HRec*>(ctx->hrec.p), static_cast<double*>(ctx->hQ.p), static_cast<float*>(ctx->hQ32.p),
                static_cast<int32_t*>(ctx->hulb.p), static_cast<int32_t*>(ctx->huub.p)};
        const bool have_prep = (flags & KORG_VJP_REUSE_FORWARD) && !op && ctx->hyd_prep >= int(mixed);
        if (!have_prep) KCHECK(run_hydrogen_prep(ctx, wls, nwl, hl, in->hydrogen_window, in->use_MHD, mixed, s, &ho));
        const size_t n_dq = size_t(ntrans) * L * 2 * HND_MAX + size_t(nbr) * L * 3 * BR_NP;
        // mixed: the Stehle table derivatives, then the Brackett profiles with theirs, in FP32
        const size_t n_dq32 = mixed ? size_t(ntrans) * L * 2 * HND_MAX + size_t(nbr) * L * 4 * BR_NP : 0;
        const size_t o_der32 = a256(sizeof(HDer) * size_t(ntot) * L);
        KCHECK(ensure(ctx, ctx->vjp_hder, o_der32 + (mixed ? sizeof(HDer32) * size_t(ntot) * L : 0)));
        KCHECK(ensure(ctx, ctx->vjp_hdq, sizeof(double) * n_dq + sizeof(float) * n_dq32));
        HDer* hder = static_cast<HDer*>(ctx->vjp_hder.p);
        HDer32* hder32 = mixed ? reinterpret_cast<HDer32*>(static_cast<unsigned char*>(ctx->vjp_hder.p) + o_der32)
                               : nullptr;
        double* hdq = static_cast<double*>(ctx->vjp_hdq.p);
        float* hdq32 = mixed ? reinterpret_cast<float*>(hdq + n_dq) : nullptr;
        hline_adj_prep_kernel<<<(ntrans * L + 127) / 128, 128, 0, s>>>(ctx->stark, hl, in->use_MHD, ho.rec, hder, hdq,
                                                                      hder32, hdq32);
        KCUDA(cudaGetLastError());
        if (nbr > 0) {
            brackett_adj_prep_kernel<<<dim3(nbr, L), 256, 0, s>>>(
                hl, ntrans, wls, nwl, in->use_MHD, ho.rec, hder, hdq + size_t(ntrans) * L * 2 * HND_MAX, hder32,
                mixed ? hdq32 + size_t(ntrans) * L * 2 * HND_MAX : nullptr);
            KCUDA(cudaGetLastError());
        }
        HAdjArgs ha{};
        ha.G = ctx->vjp_g.p;
        ha.g32 = int32_t(mixed);
        ha.wls = wls;
        ha.nwl = nwl;
        ha.L = L;
        ha.ntrans = ntrans;
        ha.ntot = ntot;
        ha.rec = ho.rec;
        ha.der = hder;
        ha.der32 = hder32;
        ha.Q = ho.Q;
        ha.Q32 = ho.Q32;
        ha.dQ = hdq;
        ha.dQ32 = hdq32;
        ha.bq32 = mixed ? hdq32 + size_t(ntrans) * L * 2 * HND_MAX : nullptr;
        ha.ulb = ho.ulb;
        ha.uub = ho.uub;
        ha.d_off = ctx->stark.d_off;
        ha.logdnu = ctx->stark.logdnu;
        ha.logdnu32 = ctx->stark.logdnu32;
        ha.UH = in->UH_I;
        double* outs[6] = {dT, gr.ne, gr.xi, gr.nH_I, gr.nHe_I, gr.UH_I};
        for (int k = 0; k < 6; k++) ha.out[k] = outs[k];
        const int64_t tiles = (nwl + 31) / 32;
        const int64_t blocks = std::min<int64_t>((tiles + HADJ_WARPS - 1) / HADJ_WARPS, int64_t(ctx->sms) * 4);
        if (mixed) hline_adj_kernel<true><<<unsigned(blocks), 32 * HADJ_WARPS, 0, s>>>(ha);
        else hline_adj_kernel<false><<<unsigned(blocks), 32 * HADJ_WARPS, 0, s>>>(ha);
        KCUDA(cudaGetLastError());
    }
    record(ctx, 11, s);

    // 4. metal and molecular lines: window sums per (line, layer), then the prologue chain rule
    const LineAdjOut lo{dT, gr.ne, gr.n_eff_vdW, gr.xi, gr.n_div_U, gr.log_gf};
    auto line_adjoint = [&](const LinesDev& lns, unsigned char* scratch, const void* Gp, int g32_in, const double* w,
                            int64_t nw, const LineAdjOut& out) -> int {
        if (lns.n == 0) return KORG_OK;
        if (mixed && !g32_in) {  // the mixed kernel stages float G: convert (a few values)
            float* g32buf = reinterpret_cast<float*>(sm + o_g32);
            to_float_kernel<<<unsigned((nw * L + 255) / 256), 256, 0, s>>>(static_cast<const double*>(Gp), nw * L,
                                                                         g32buf);
            KCUDA(cudaGetLastError());
            Gp = g32buf;
            g32_in = 1;
        }
        LineScratch sc;
        line_scratch(scratch, lns.n, L, Lp, G, mixed, &sc);
        double* dpar = static_cast<double*>(ctx->vjp_dpar.p);
        KCUDA(cudaMemsetAsync(dpar, 0, sizeof(double) * 3 * size_t(lns.n) * Lp, s));
        KCUDA(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), s));
        const AdjShape sh = adj_shape(L, Gp, mixed);
        auto* ilo = reinterpret_cast<int32_t*>(sm + o_ilo);
        auto* ipre = reinterpret_cast<int64_t*>(sm + o_ipre);
        auto* wl2 = reinterpret_cast<float2*>(sm + o_wl2);
        const int npairs = int((nw + ADJ_CHUNK - 1) / ADJ_CHUNK) * NTIER;
        adj_items_kernel<<<1, 1024, 0, s>>>(sc.tier_idx, sc.tier_ci, sc.tier_meta, sc.lb, sc.ub, nw, ilo, ipre);
        KCUDA(cudaGetLastError());
        if (mixed) {
            wl_pairs_kernel<<<unsigned((nw + 255) / 256), 256, 0, s>>>(w, nw, wl2);
            KCUDA(cudaGetLastError());
        }
        LineAdjArgs la{Gp, g32_in, w, wl2, nw, L, Lp, lns.wl, sc.params, sc.lb, sc.ub, sc.tier_idx, ilo, ipre, npairs,
                       dpar, ctr, sh.Ls, sh.bulk, ctx->dev_err_dev, sh.sub};
        const int threads = sh.threads;
        if ((g32_in != 0) != mixed) return set_err(ctx, KORG_EINVAL, "opacity cotangent precision mismatch");
        const size_t smem = adj_smem(sh, mixed);
        int per_sm = 0;
        if (mixed) {
            KCUDA(cudaFuncSetAttribute(line_adj_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
            KCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, line_adj_kernel<true>, threads, smem));
            line_adj_kernel<true><<<ctx->sms * std::max(per_sm, 1), threads, smem, s>>>(la);
        } else {
            KCUDA(cudaFuncSetAttribute(line_adj_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
            KCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, line_adj_kernel<false>, threads, smem));
            line_adj_kernel<false><<<ctx->sms * std::max(per_sm, 1), threads, smem, s>>>(la);
        }
        KCUDA(cudaGetLastError());
        const size_t psmem = sizeof(double) * size_t(4 + S) * L;
        KCUDA(cudaFuncSetAttribute(line_adj_prologue_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(psmem)));
        line_adj_prologue_kernel<<<unsigned((lns.n * 32 + 255) / 256), 256, psmem, s>>>(
            lns, lay, sc.lc, dpar, Lp, out, static_cast<MathTables*>(ctx->math.p));
        KCUDA(cudaGetLastError());
        return KORG_OK;
    };
    // the metal-line prologue of step 1 is still in the line scratch
    KCHECK(line_adjoint(ln, line_base, ctx->vjp_g.p, int(mixed), wls, nwl, lo));
    // 5. reference-wavelength lines: alpha_ref = continuum + lines at ref_wl, cotangent daref
    if (ln5.n > 0) {
        LineScratch sc;
        KCHECK(ensure(ctx, ctx->lines_scratch, line_scratch(nullptr, ln5.n, L, Lp, G, mixed, nullptr)));
        line_scratch(static_cast<unsigned char*>(ctx->lines_scratch.p), ln5.n, L, Lp, G, mixed, &sc);
        KCHECK(prep_lines(ctx, sc, ref_wl_dev, 1, ln5, lay, cref, in->cutoff_threshold, mixed, kmax, G, s));
        const LineAdjOut lo5{dT, gr.ne, gr.n_eff_vdW, gr.xi, gr.n_div_U, nullptr};
        KCHECK(line_adjoint(ln5, static_cast<unsigned char*>(ctx->lines_scratch.p), daref, 0, ref_wl_dev, 1, lo5));
    }
    if (gr.alpha_ref_cntm)
        KCUDA(cudaMemcpyAsync(gr.alpha_ref_cntm, daref, sizeof(double) * L, cudaMemcpyDeviceToDevice, s));
    record(ctx, 12, s);
    ctx->vjp_timed = ctx->timing;
    ctx->stats_pending = true;
    return KORG_OK;
}


// ------------------------------------------------------------------ molecular cross-sections
// Trilinear interpolation of a precomputed molecular cross-section table into alpha
// (interpolate_molecular_cross_sections!, src/molecular_cross_sections.jl:101-117): Gridded
// Linear in (vmic, log10 T, wavelength), zero outside the table (extrapolate(..., 0.0)).
struct MolXsArgs {
    double* alpha;             // [nwl][L] (+=)
    const double* wls;         // [nwl]
    int64_t nwl;
    int32_t L;
    const double *T, *vmic, *n;  // [L]: temperature, microturbulence (km/s), number density
    const double* table;       // [nv][ntw][nT]
    const double* twls;        // [ntw] table wavelengths
    int64_t ntw;
    const double* vmic_vals;   // [nv]
    int32_t nv;
    const double* logT_vals;   // [nT]
    int32_t nT;
};

// knot interval and weight of x on increasing knots; false outside [k0, k_{n-1}]
__device__ __forceinline__ bool grid_pos(const double* k, int64_t n, double x, int64_t* i, double* t) {
    if (!(x >= k[0] && x <= k[n - 1])) return false;
    if (n == 1) { *i = 0; *t = 0.0; return true; }
    int64_t lo = search_last(k, n, x);
    lo = lo < 0 ? 0 : (lo > n - 2 ? n - 2 : lo);
    *i = lo;
    *t = (x - k[lo]) / (k[lo + 1] - k[lo]);
    return true;
}

__global__ void __launch_bounds__(256) molxs_interp_kernel(MolXsArgs a) {
    __shared__ int64_t s_iw[64];
    __shared__ double s_tw[64];
    __shared__ int s_okw[64];
    extern __shared__ double s_lay[];  // per layer: iv, tv, iT, tT, n, ok
    const int L = a.L;
    for (int l = threadIdx.x; l < L; l += blockDim.x) {
        int64_t iv = 0, iT = 0;
        double tv = 0, tT = 0;
        const bool ok = grid_pos(a.vmic_vals, a.nv, a.vmic[l], &iv, &tv) &&
                        grid_pos(a.logT_vals, a.nT, log10(a.T[l]), &iT, &tT);
        double* p = s_lay + 6 * l;
        p[0] = double(iv); p[1] = tv; p[2] = double(iT); p[3] = tT; p[4] = a.n[l]; p[5] = ok ? 1.0 : 0.0;
    }
    const int64_t j0 = int64_t(blockIdx.x) * 64;
    const int64_t jn = min(int64_t(64), a.nwl - j0);
    if (threadIdx.x < jn) {
        int64_t iw = 0;
        double tw = 0;
        s_okw[threadIdx.x] = grid_pos(a.twls, a.ntw, a.wls[j0 + threadIdx.x], &iw, &tw);
        s_iw[threadIdx.x] = iw;
        s_tw[threadIdx.x] = tw;
    }
    __syncthreads();
    for (int64_t e = threadIdx.x; e < jn * L; e += blockDim.x) {
        const int jj = int(e / L), l = int(e % L);
        const double* p = s_lay + 6 * l;
        if (!s_okw[jj] || p[5] == 0.0) continue;
        const int64_t iv = int64_t(p[0]), iT = int64_t(p[2]), iw = s_iw[jj];
        const double tv = p[1], tT = p[3], tw = s_tw[jj];
        const int64_t dv = (a.nv > 1) ? a.ntw * a.nT : 0, dw = (a.ntw > 1) ? a.nT : 0, dT = (a.nT > 1) ? 1 : 0;
        const double* c = a.table + (iv * a.ntw + iw) * a.nT + iT;
        const double c000 = c[0], c001 = c[dT], c010 = c[dw], c011 = c[dw + dT];
        const double c100 = c[dv], c101 = c[dv + dT], c110 = c[dv + dw], c111 = c[dv + dw + dT];
        const double c00 = c000 * (1 - tT) + c001 * tT, c01 = c010 * (1 - tT) + c011 * tT;
        const double c10 = c100 * (1 - tT) + c101 * tT, c11 = c110 * (1 - tT) + c111 * tT;
        const double c0 = c00 * (1 - tw) + c01 * tw, c1 = c10 * (1 - tw) + c11 * tw;
        a.alpha[(j0 + jj) * L + l] += (c0 * (1 - tv) + c1 * tv) * p[4];
    }
}

// per-temperature inputs of the cross-section precompute: n_e = 0, n_eff_vdW = NaN,
// n/U = (1/cutoff_alpha) / U(T), continuum 1
__global__ void molxs_layers_kernel(const double* inv_U, int nT, double cutoff_alpha, double* d) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nT) return;
    d[t] = 0.0;
    d[nT + t] = __longlong_as_double(0x7ff8000000000000LL);
    d[2 * nT + t] = inv_U[t] / cutoff_alpha;
    d[3 * nT + t] = 1.0;
}

// x[i] = *v * scale (a device scalar broadcast)
__global__ void fill_kernel(double* x, int n, const double* v, double scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = *v * scale;
}

__global__ void scale_kernel(double* x, int64_t n, double s) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        x[i] *= s;
}

// ------------------------------------------------------------------ host staging
struct Stager {
    std::vector<std::pair<const void*, size_t>> items;
    std::vector<size_t> offs;
    size_t total = 0;
    size_t add(const void* p, size_t bytes) {
        size_t o = (total + 255) & ~size_t(255);
        items.push_back({p, bytes});
        offs.push_back(o);
        total = o + bytes;
        return o;
    }
};

// Host-side copies between the caller's buffers and the pinned staging buffer of the
// host-pointer calls, split over threads in pieces of at most 1 MiB: one core copies at a
// fraction of the socket's memory bandwidth (30 MB of line list take 1.3 ms on one Grace core).
struct HostPiece {
    void* dst;
    const void* src;
    size_t bytes;
};
void par_copy(const std::vector<HostPiece>& in) {
    constexpr size_t PIECE = size_t(1) << 20;
    std::vector<HostPiece> v;
    size_t total = 0;
    for (const HostPiece& p : in)
        for (size_t o = 0; o < p.bytes; o += PIECE) {
            v.push_back({static_cast<char*>(p.dst) + o, static_cast<const char*>(p.src) + o, std::min(PIECE, p.bytes - o)});
            total += v.back().bytes;
        }
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nt = std::min<size_t>(std::min<size_t>(hw, 16), total / (2 * PIECE));
    auto work = [&v](size_t k0, size_t step) {
        for (size_t k = k0; k < v.size(); k += step) memcpy(v[k].dst, v[k].src, v[k].bytes);
    };
    if (nt <= 1) {
        work(0, 1);
        return;
    }
    std::vector<std::thread> ts;
    for (size_t t = 1; t < nt; t++) ts.emplace_back(work, t, nt);
    work(0, nt);
    for (auto& t : ts) t.join();
}

int upload(korg_ctx* ctx, Stager& st, char** dev_base) {
    KCHECK(ensure(ctx, ctx->stage_dev, st.total));
    if (ctx->stage_host_cap < st.total) {
        if (ctx->stage_host) cudaFreeHost(ctx->stage_host);
        ctx->stage_host = nullptr;
        size_t want = st.total + st.total / 4;
        KCUDA(cudaHostAlloc(&ctx->stage_host, want, cudaHostAllocDefault));
        ctx->stage_host_cap = want;
    }
    char* h = static_cast<char*>(ctx->stage_host);
    std::vector<HostPiece> pieces;
    for (size_t i = 0; i < st.items.size(); i++)
        if (st.items[i].first && st.items[i].second) pieces.push_back({h + st.offs[i], st.items[i].first, st.items[i].second});
    par_copy(pieces);
    KCUDA(cudaMemcpyAsync(ctx->stage_dev.p, h, st.total, cudaMemcpyHostToDevice, ctx->stream));
    *dev_base = static_cast<char*>(ctx->stage_dev.p);
    return KORG_OK;
}

struct LinesStage {
    size_t o[10];
};
LinesStage stage_lines(Stager& st, const korg_lines* l) {
    LinesStage s;
    const size_t n = size_t(l->n);
    s.o[0] = st.add(l->wl, 8 * n);
    s.o[1] = st.add(l->log_gf, 8 * n);
    s.o[2] = st.add(l->E_lower, 8 * n);
    s.o[3] = st.add(l->gamma_rad, 8 * n);
    s.o[4] = st.add(l->gamma_stark, 8 * n);
    s.o[5] = st.add(l->vdW1, 8 * n);
    s.o[6] = st.add(l->vdW2, 8 * n);
    s.o[7] = st.add(l->mass, 8 * n);
    s.o[8] = st.add(l->is_mol, 4 * n);
    s.o[9] = st.add(l->species, 4 * n);
    return s;
}
LinesDev lines_from_stage(const LinesStage& s, char* b, int64_t n) {
    return LinesDev{n, (double*)(b + s.o[0]), (double*)(b + s.o[1]), (double*)(b + s.o[2]), (double*)(b + s.o[3]),
                    (double*)(b + s.o[4]), (double*)(b + s.o[5]), (double*)(b + s.o[6]), (double*)(b + s.o[7]),
                    (int32_t*)(b + s.o[8]), (int32_t*)(b + s.o[9])};
}

int check_lines(korg_ctx* ctx, const korg_lines* l, int S) {
    if (!l || l->n < 0) return set_err(ctx, KORG_EINVAL, "null line list");
    if (l->n == 0) return KORG_OK;
    if (!l->wl || !l->log_gf || !l->E_lower || !l->gamma_rad || !l->gamma_stark || !l->vdW1 || !l->vdW2 ||
        !l->mass || !l->is_mol || !l->species)
        return set_err(ctx, KORG_EINVAL, "null array in line list");
    for (int64_t i = 0; i < l->n; i++)
        if (l->species[i] < 0 || l->species[i] >= S)
            return set_err(ctx, KORG_EINVAL, "line %lld: species row %d outside n_div_U (S=%d)", (long long)i,
                           l->species[i], S);
    return KORG_OK;
}

int check_wls(korg_ctx* ctx, const double* wls, int64_t nwl) {
    if (!wls || nwl < 1) return set_err(ctx, KORG_EINVAL, "empty wavelength grid");
    for (int64_t j = 1; j < nwl; j++)
        if (!(wls[j] >= wls[j - 1])) return set_err(ctx, KORG_EINVAL, "wavelengths must be sorted");
    return KORG_OK;
}

int check_layers(korg_ctx* ctx, const korg_layers* y) {
    if (!y || y->L < 1 || y->S < 0 || !y->T || !y->ne || !y->n_eff_vdW || !y->xi || (y->S > 0 && !y->n_div_U))
        return set_err(ctx, KORG_EINVAL, "bad layer inputs");
    return KORG_OK;
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

KORG_API int korg_create(korg_ctx** out, int device) {
    if (!out) return KORG_EINVAL;
    *out = nullptr;
    korg_ctx* ctx = new korg_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    for (int i = 0; e == cudaSuccess && i < NEV; i++) e = cudaEventCreate(&ctx->ev[i]);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->b_host_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&ctx->dev_err_host), sizeof(int), cudaHostAllocMapped);
    if (e == cudaSuccess) {
        *ctx->dev_err_host = 0;
        e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->dev_err_dev), ctx->dev_err_host, 0);
    }
    if (e == cudaSuccess) {
        MathTables t;
        fill_math_tables(t);
        e = cudaMalloc(&ctx->math.p, sizeof(MathTables));
        if (e == cudaSuccess) {
            ctx->math.cap = sizeof(MathTables);
            e = cudaMemcpy(ctx->math.p, &t, sizeof t, cudaMemcpyHostToDevice);
        }
    }
    if (e != cudaSuccess) {
        korg_destroy(ctx);
        return KORG_ECUDA;
    }
    *out = ctx;
    return KORG_OK;
}

KORG_API void korg_destroy(korg_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    drop_graph(ctx);
    DevBuf* bufs[] = {&ctx->lines_scratch, &ctx->counters, &ctx->tune_alpha, &ctx->hrec, &ctx->hQ, &ctx->hQ32,
                      &ctx->hulb, &ctx->huub, &ctx->stage_dev, &ctx->aref, &ctx->alpha, &ctx->flux, &ctx->cntm,
                      &ctx->math, &ctx->b_alpha, &ctx->b_lines, &ctx->b_meta, &ctx->vjp_g, &ctx->vjp_dpar,
                      &ctx->vjp_small, &ctx->vjp_hder, &ctx->vjp_hdq, &ctx->mx_layers};
    for (DevBuf* b : bufs)
        if (b->p) cudaFree(b->p);
    for (void* p : ctx->stark_allocs) cudaFree(p);
    if (ctx->cntm_buf) cudaFree(ctx->cntm_buf);
    if (ctx->chem_buf) cudaFree(ctx->chem_buf);
    if (ctx->stage_host) cudaFreeHost(ctx->stage_host);
    if (ctx->b_host) cudaFreeHost(ctx->b_host);
    if (ctx->dev_err_host) cudaFreeHost(ctx->dev_err_host);
    for (int i = 0; i < NEV; i++)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    if (ctx->b_host_ev) cudaEventDestroy(ctx->b_host_ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

KORG_API const char* korg_last_error(const korg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

KORG_API int korg_set_timing(korg_ctx* ctx, int enabled) {
    if (!ctx) return KORG_EINVAL;
    ctx->timing = enabled != 0;
    return KORG_OK;
}

KORG_API int korg_get_stats(korg_ctx* ctx, korg_stats* out) {
    if (!ctx || !out) return KORG_EINVAL;
    KCUDA(cudaSetDevice(ctx->device));
    if (ctx->stats_pending && ctx->counters.p) {
        KCUDA(cudaDeviceSynchronize());
        unsigned long long c[2];
        KCUDA(cudaMemcpy(c, ctx->counters.p, sizeof c, cudaMemcpyDeviceToHost));
        ctx->stats.line_evals = int64_t(c[0]);
        ctx->stats.lines_in_window = int64_t(c[1]);
    }
    if (ctx->timing) {
        KCUDA(cudaDeviceSynchronize());
        float ms;
        auto el = [&](int a, int b) {
            return cudaEventElapsedTime(&ms, ctx->ev[a], ctx->ev[b]) == cudaSuccess ? ms : -1.f;
        };
        ctx->stats.ms_ref_lines = el(1, 3);
        ctx->stats.ms_hydrogen = el(3, 4);
        ctx->stats.ms_line_prep = el(4, 2);
        ctx->stats.ms_line_tile = el(2, 5);
        ctx->stats.ms_rt = el(5, 6);
        ctx->stats.ms_total = el(0, 6);
        if (ctx->vjp_timed) {
            ctx->stats.ms_vjp_alpha = el(8, 9);
            ctx->stats.ms_vjp_rt = el(9, 10);
            ctx->stats.ms_vjp_hydrogen = el(10, 11);
            ctx->stats.ms_vjp_lines = el(11, 12);
        }
        cudaGetLastError();
    }
    *out = ctx->stats;
    return KORG_OK;
}

KORG_API int korg_set_stark_tables(korg_ctx* ctx, const korg_stark_tables* t) {
    if (!ctx || !t || t->ntrans < 1) return KORG_EINVAL;
    KCUDA(cudaSetDevice(ctx->device));
    drop_graph(ctx);  // a captured batch holds the old table addresses
    KCUDA(cudaDeviceSynchronize());
    for (void* p : ctx->stark_allocs) cudaFree(p);
    ctx->stark_allocs.clear();
    ctx->have_stark = false;
    ctx->hyd_prep = -1;  // records made with the previous tables are not reused
    const int n = t->ntrans;
    int64_t sz_t = 0, sz_ne = 0, sz_d = 0, sz_p = 0, sz_l = 0;
    int n_max = 0, nd_max = 0;
    for (int i = 0; i < n; i++) {
        sz_t = std::max(sz_t, t->t_off[i] + t->nT[i]);
        sz_ne = std::max(sz_ne, t->ne_off[i] + t->nNe[i]);
        sz_d = std::max(sz_d, t->d_off[i] + t->nD[i]);
        sz_p = std::max(sz_p, t->p_off[i] + int64_t(t->nT[i]) * t->nNe[i] * t->nD[i]);
        sz_l = std::max(sz_l, t->l_off[i] + int64_t(t->nT[i]) * t->nNe[i]);
        n_max = std::max(n_max, t->upper[i]);
        nd_max = std::max(nd_max, t->nD[i]);
        if (t->nT[i] < 2 || t->nNe[i] < 2 || t->nD[i] < 3)
            return set_err(ctx, KORG_EINVAL, "Stark table %d is too small", i);
    }
    if (nd_max > HND_MAX) return set_err(ctx, KORG_EINVAL, "Stark tables with more than %d knots", HND_MAX);
    auto up = [&](const void* src, size_t bytes, void** dst) -> int {
        KCUDA(cudaMalloc(dst, bytes));
        ctx->stark_allocs.push_back(*dst);
        KCUDA(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
        return KORG_OK;
    };
    StarkDev d{};
    d.ntrans = n;
    void* p;
    KCHECK(up(t->lower, 4 * n, &p)); d.lower = (int32_t*)p;
    KCHECK(up(t->upper, 4 * n, &p)); d.upper = (int32_t*)p;
    KCHECK(up(t->nT, 4 * n, &p)); d.nT = (int32_t*)p;
    KCHECK(up(t->nNe, 4 * n, &p)); d.nNe = (int32_t*)p;
    KCHECK(up(t->nD, 4 * n, &p)); d.nD = (int32_t*)p;
    KCHECK(up(t->t_off, 8 * n, &p)); d.t_off = (int64_t*)p;
    KCHECK(up(t->ne_off, 8 * n, &p)); d.ne_off = (int64_t*)p;
    KCHECK(up(t->d_off, 8 * n, &p)); d.d_off = (int64_t*)p;
    KCHECK(up(t->p_off, 8 * n, &p)); d.p_off = (int64_t*)p;
    KCHECK(up(t->l_off, 8 * n, &p)); d.l_off = (int64_t*)p;
    KCHECK(up(t->log_gf, 8 * n, &p)); d.log_gf = (double*)p;
    KCHECK(up(t->temps, 8 * sz_t, &p)); d.temps = (double*)p;
    KCHECK(up(t->nes, 8 * sz_ne, &p)); d.nes = (double*)p;
    KCHECK(up(t->logdnu, 8 * sz_d, &p)); d.logdnu = (double*)p;
    KCHECK(up(t->logP, 8 * sz_p, &p)); d.logP = (double*)p;
    KCHECK(up(t->lambda0, 8 * sz_l, &p)); d.lambda0 = (double*)p;
    std::vector<float> k32(sz_d);
    for (int64_t i = 0; i < sz_d; i++) k32[i] = float(std::max(t->logdnu[i], -3.0e38));
    KCHECK(up(k32.data(), 4 * sz_d, &p)); d.logdnu32 = (float*)p;
    ctx->stark = d;
    ctx->n_max = n_max;
    ctx->have_stark = true;
    return KORG_OK;
}

// ------------------------------------------------------------------ continuum absorption
KORG_API int korg_set_continuum_tables(korg_ctx* ctx, const korg_continuum_tables* t) {
    if (!ctx) return KORG_EINVAL;
    if (!t || t->h_n < 2 || t->hm_n < 2 || t->hff_nl < 2 || t->hff_nt < 2 || t->heff_nl < 2 || t->heff_nt < 2 ||
        t->h2_nT < 2 || t->h2_nbf < 2 || t->h2_nff < 2 || t->g_nu < 2 || t->g_ng < 2 || t->p_ns < 2)
        return set_err(ctx, KORG_EINVAL, "bad continuum tables");
    for (int k = 0; k < CNT_PEACH; k++)
        if (t->p_nT[k] < 2 || !t->p_T[k] || !t->p_D[k]) return set_err(ctx, KORG_EINVAL, "bad Peach table %d", k);
    KCUDA(cudaSetDevice(ctx->device));
    struct Piece { const double* src; size_t n; const double** dst; };
    CntmTables d{};
    d.h_n = t->h_n; d.hm_n = t->hm_n; d.hff_nl = t->hff_nl; d.hff_nt = t->hff_nt; d.heff_nl = t->heff_nl;
    d.heff_nt = t->heff_nt; d.h2_nT = t->h2_nT; d.h2_nbf = t->h2_nbf; d.h2_nff = t->h2_nff; d.g_nu = t->g_nu;
    d.g_ng = t->g_ng; d.p_ns = t->p_ns;
    std::vector<Piece> pcs = {
        {t->h_E, size_t(6) * t->h_n, &d.h_E}, {t->h_sigma, size_t(6) * t->h_n, &d.h_sigma},
        {t->hm_nu, size_t(t->hm_n), &d.hm_nu}, {t->hm_sigma, size_t(t->hm_n), &d.hm_sigma},
        {t->hff_lambda, size_t(t->hff_nl), &d.hff_lambda}, {t->hff_theta, size_t(t->hff_nt), &d.hff_theta},
        {t->hff_K, size_t(t->hff_nl) * t->hff_nt, &d.hff_K},
        {t->heff_lambda, size_t(t->heff_nl), &d.heff_lambda}, {t->heff_theta, size_t(t->heff_nt), &d.heff_theta},
        {t->heff_K, size_t(t->heff_nl) * t->heff_nt, &d.heff_K},
        {t->h2_T, size_t(t->h2_nT), &d.h2_T}, {t->h2_K, size_t(t->h2_nT), &d.h2_K},
        {t->h2_bf_lambda, size_t(t->h2_nbf), &d.h2_bf_lambda},
        {t->h2_bf_sigma, size_t(t->h2_nbf) * t->h2_nT, &d.h2_bf_sigma},
        {t->h2_ff_lambda, size_t(t->h2_nff), &d.h2_ff_lambda},
        {t->h2_ff_sigma, size_t(t->h2_nff) * t->h2_nT, &d.h2_ff_sigma},
        {t->g_log_u, size_t(t->g_nu), &d.g_log_u}, {t->g_log_g2, size_t(t->g_ng), &d.g_log_g2},
        {t->g_ff, size_t(t->g_nu) * t->g_ng, &d.g_ff}, {t->p_sigma, size_t(t->p_ns), &d.p_sigma}};
    for (int k = 0; k < CNT_PEACH; k++) {
        d.p_nT[k] = t->p_nT[k];
        pcs.push_back({t->p_T[k], size_t(t->p_nT[k]), &d.p_T[k]});
        pcs.push_back({t->p_D[k], size_t(t->p_nT[k]) * t->p_ns, &d.p_D[k]});
    }
    size_t total = 0;
    for (const Piece& q : pcs) {
        if (!q.src) return set_err(ctx, KORG_EINVAL, "null continuum table");
        total += a256(8 * q.n);
    }
    std::vector<unsigned char> host(total);
    size_t off = 0;
    for (const Piece& q : pcs) {
        memcpy(host.data() + off, q.src, 8 * q.n);
        off += a256(8 * q.n);
    }
    void* buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, total);
    if (e != cudaSuccess) return set_err(ctx, KORG_ENOMEM, "cudaMalloc(%zu): %s", total, cudaGetErrorString(e));
    e = cudaMemcpy(buf, host.data(), total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(buf);
        return set_err(ctx, KORG_ECUDA, "continuum tables: %s", cudaGetErrorString(e));
    }
    off = 0;
    for (const Piece& q : pcs) {
        *q.dst = reinterpret_cast<const double*>(static_cast<unsigned char*>(buf) + off);
        off += a256(8 * q.n);
    }
    if (ctx->cntm_buf) {
        KCUDA(cudaDeviceSynchronize());
        cudaFree(ctx->cntm_buf);
    }
    ctx->cntm_buf = buf;
    ctx->cntm_tab = d;
    ctx->have_cntm = true;
    return KORG_OK;
}

namespace {
CntmLayers cntm_layers(const korg_continuum_layers* y) {
    CntmLayers c{y->L, y->T, y->ne, y->nH_I, y->nH_II, y->nHe_I, y->nH2, y->nH_minus, y->invU_H_I, y->invU_He_I,
                 y->n_Z1, y->n_Z2, {}};
    for (int k = 0; k < CNT_PEACH; k++) c.n_peach[k] = y->n_peach[k];
    return c;
}
bool cntm_layers_ok(const korg_continuum_layers* y) {
    if (!y || y->L < 1) return false;
    const double* p[] = {y->T, y->ne, y->nH_I, y->nH_II, y->nHe_I, y->nH2, y->nH_minus, y->invU_H_I, y->invU_He_I,
                         y->n_Z1, y->n_Z2, y->n_peach[0], y->n_peach[1], y->n_peach[2], y->n_peach[3]};
    for (const double* q : p)
        if (!q) return false;
    return true;
}
}  // namespace

KORG_API int korg_continuum_absorption_dev(korg_ctx* ctx, const double* wls, int64_t nwl,
                                           const korg_continuum_layers* layers, double* vals, void* stream) {
    if (!ctx) return KORG_EINVAL;
    if (!wls || nwl < 1 || !vals || !cntm_layers_ok(layers)) return set_err(ctx, KORG_EINVAL, "bad arguments");
    if (!ctx->have_cntm) return set_err(ctx, KORG_ENOTABLES, "korg_set_continuum_tables() has not been called");
    KCUDA(cudaSetDevice(ctx->device));
    const int64_t n = nwl * layers->L;
    continuum_kernel<<<unsigned((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        ctx->cntm_tab, cntm_layers(layers), wls, nwl, vals);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

KORG_API int korg_continuum_absorption(korg_ctx* ctx, const double* wls, int64_t nwl,
                                       const korg_continuum_layers* layers, double* vals) {
    if (!ctx) return KORG_EINVAL;
    KCHECK(check_wls(ctx, wls, nwl));
    if (!vals || !cntm_layers_ok(layers)) return set_err(ctx, KORG_EINVAL, "bad arguments");
    if (!ctx->have_cntm) return set_err(ctx, KORG_ENOTABLES, "korg_set_continuum_tables() has not been called");
    KCUDA(cudaSetDevice(ctx->device));
    const int L = layers->L;
    Stager st;
    const size_t o_w = st.add(wls, 8 * size_t(nwl));
    const double* arrs[] = {layers->T, layers->ne, layers->nH_I, layers->nH_II, layers->nHe_I, layers->nH2,
                            layers->nH_minus, layers->invU_H_I, layers->invU_He_I, layers->n_Z1, layers->n_Z2,
                            layers->n_peach[0], layers->n_peach[1], layers->n_peach[2], layers->n_peach[3]};
    size_t o_a[15];
    for (int k = 0; k < 15; k++) o_a[k] = st.add(arrs[k], 8 * size_t(L));
    const size_t o_v = st.add(nullptr, 8 * size_t(L) * nwl);
    char* b = nullptr;
    KCHECK(upload(ctx, st, &b));
    korg_continuum_layers d{};
    d.L = L;
    const double** dst[] = {&d.T, &d.ne, &d.nH_I, &d.nH_II, &d.nHe_I, &d.nH2, &d.nH_minus, &d.invU_H_I,
                            &d.invU_He_I, &d.n_Z1, &d.n_Z2, &d.n_peach[0], &d.n_peach[1], &d.n_peach[2],
                            &d.n_peach[3]};
    for (int k = 0; k < 15; k++) *dst[k] = (const double*)(b + o_a[k]);
    KCHECK(korg_continuum_absorption_dev(ctx, (const double*)(b + o_w), nwl, &d, (double*)(b + o_v), ctx->stream));
    KCUDA(cudaMemcpyAsync(vals, b + o_v, 8 * size_t(L) * nwl, cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaStreamSynchronize(ctx->stream));
    return KORG_OK;
}

KORG_API int korg_line_absorption_dev(korg_ctx* ctx, double* alpha, const double* wls, int64_t nwl,
                                      const korg_lines* lines, const korg_layers* layers, const korg_cntm* cntm,
                                      double cutoff, int precision, void* stream) {
    if (!ctx || !alpha || !wls || nwl < 1 || !lines || !layers || !cntm || cntm->nk < 1)
        return ctx ? set_err(ctx, KORG_EINVAL, "bad arguments") : KORG_EINVAL;
    KPREC(precision);
    KCUDA(cudaSetDevice(ctx->device));
    KCHECK(reset_counters(ctx, static_cast<cudaStream_t>(stream)));
    return run_line_absorption(ctx, alpha, wls, nwl, lines_dev(lines), layers_dev(layers),
                               CntmDev{cntm->nk, cntm->knots, cntm->vals}, cutoff, precision == KORG_MIXED,
                               static_cast<cudaStream_t>(stream));
}

// ------------------------------------------------------------------ chemical equilibrium
KORG_API int korg_set_equilibrium_tables(korg_ctx* ctx, const korg_equilibrium_tables* t) {
    if (!ctx) return KORG_EINVAL;
    if (!t || t->n_knots < 2 || !t->lnT || !t->U_u || !t->U_z || !t->chi || t->n_mol < 0 ||
        t->n_mol > KORG_CHEM_MAX_MOL || (t->n_mol > 0 && (!t->atoms || !t->charge || !t->kind || !t->off ||
                                                           !t->spl_t || !t->spl_u || !t->spl_z)))
        return set_err(ctx, KORG_EINVAL, "bad equilibrium tables");
    for (int k = 1; k < t->n_knots; k++)
        if (!(t->lnT[k] > t->lnT[k - 1])) return set_err(ctx, KORG_EINVAL, "partition-function knots not increasing");
    const int M = t->n_mol;
    // derived per-molecule data: atom count, distinct atoms with counts, element incidence lists
    std::vector<int32_t> nat(M);
    std::vector<std::vector<std::pair<int32_t, int32_t>>> inc(CE_NZ);
    std::map<std::pair<int32_t, int32_t>, std::vector<std::pair<int32_t, int32_t>>> pairs;  // (Z, W) -> (m, cnt_Z cnt_W)
    bool polyatomic = false;
    for (int m = 0; m < M; m++) {
        const int32_t* at = t->atoms + size_t(m) * CE_MAXATOMS;
        int n = 0;
        while (n < CE_MAXATOMS && at[n]) n++;
        for (int j = n; j < CE_MAXATOMS; j++)
            if (at[j]) return set_err(ctx, KORG_EINVAL, "molecule %d: atoms not 0-padded", m);
        if (n < 2) return set_err(ctx, KORG_EINVAL, "molecule %d has %d atoms", m, n);
        for (int j = 0; j < n; j++)
            if (at[j] < 1 || at[j] > CE_NZ || (j && at[j] < at[j - 1]))
                return set_err(ctx, KORG_EINVAL, "molecule %d: atomic numbers not ascending in 1..92", m);
        if (t->charge[m] != 0 && !(t->charge[m] == 1 && n == 2))
            return set_err(ctx, KORG_EINVAL, "molecule %d: only neutral or singly ionized diatomics", m);
        if (t->kind[m] != 0 && t->kind[m] != 1) return set_err(ctx, KORG_EINVAL, "molecule %d: kind", m);
        polyatomic |= t->kind[m] == 1;
        if (t->off[m + 1] - t->off[m] < 2 || t->off[m] < 0)
            return set_err(ctx, KORG_EINVAL, "molecule %d: spline needs two knots", m);
        nat[m] = n;
        std::vector<std::pair<int32_t, int32_t>> dist;  // distinct atoms and their counts
        for (int j = 0; j < n; j++) {
            if (j && at[j] == at[j - 1]) dist.back().second++;
            else dist.push_back({at[j], 1});
        }
        for (const auto& a : dist) {
            inc[a.first - 1].push_back({m, a.second});
            for (const auto& b : dist)
                if (b.first != a.first) pairs[{a.first - 1, b.first - 1}].push_back({m, a.second * b.second});
        }
    }
    if (polyatomic && (!t->D00 || !t->lmr)) return set_err(ctx, KORG_EINVAL, "polyatomic molecules need D00 and lmr");
    std::vector<int32_t> inc_ptr(CE_NZ + 1, 0), inc_mol, inc_cnt;
    for (int Z = 0; Z < CE_NZ; Z++) {
        for (const auto& e : inc[Z]) {
            inc_mol.push_back(e.first);
            inc_cnt.push_back(e.second);
        }
        inc_ptr[Z + 1] = int32_t(inc_mol.size());
    }
    // work items of the element sums: runs of <= CE_CHUNK consecutive incidences of one element
    std::vector<int32_t> item_elem, item_begin, elem_item_ptr(CE_NZ + 1, 0);
    for (int Z = 0; Z < CE_NZ; Z++) {
        for (int k = inc_ptr[Z]; k < inc_ptr[Z + 1]; k += CE_CHUNK) {
            item_elem.push_back(Z);
            item_begin.push_back(k);
        }
        elem_item_ptr[Z + 1] = int32_t(item_elem.size());
    }
    item_begin.push_back(inc_ptr[CE_NZ]);
    if (item_elem.size() > size_t(CE_MAXITEM))
        return set_err(ctx, KORG_EINVAL, "molecule set too large: %zu work items (max %d)", item_elem.size(), CE_MAXITEM);
    if (inc_mol.size() > size_t(CE_MAXINC) || pairs.size() > size_t(CE_MAXPAIR))
        return set_err(ctx, KORG_EINVAL, "molecule set too large: %zu incidences (max %d), %zu element pairs (max %d)",
                       inc_mol.size(), CE_MAXINC, pairs.size(), CE_MAXPAIR);
    std::vector<int32_t> pair_row, pair_col, pair_ptr(1, 0), pair_mol, pair_coef;
    for (const auto& pr : pairs) {
        pair_row.push_back(pr.first.first);
        pair_col.push_back(pr.first.second);
        for (const auto& e : pr.second) {
            pair_mol.push_back(e.first);
            pair_coef.push_back(e.second);
        }
        pair_ptr.push_back(int32_t(pair_mol.size()));
    }
    if (pair_mol.size() > size_t(CE_MAXPENT))
        return set_err(ctx, KORG_EINVAL, "molecule set too large: %zu pair entries (max %d)", pair_mol.size(), CE_MAXPENT);
    const int64_t nspl = M ? t->off[M] : 0;
    std::vector<double> zeros(std::max<int64_t>(M, 1), 0.0);
    std::vector<int32_t> izeros(1, 0);
    KCUDA(cudaSetDevice(ctx->device));
    struct Piece { const void* src; size_t bytes; const void** dst; };
    ChemTables d{};
    d.nk = t->n_knots;
    d.n_mol = M;
    d.n_pairs = int32_t(pair_row.size());
    d.n_items = int32_t(item_elem.size());
    const size_t nk = size_t(t->n_knots);
    auto ip = [&](const std::vector<int32_t>& v) { return v.empty() ? (const void*)izeros.data() : (const void*)v.data(); };
    std::vector<Piece> pcs = {
        {t->lnT, 8 * nk, (const void**)&d.lnT}, {t->U_u, 8 * nk * 3 * CE_NZ, (const void**)&d.U_u},
        {t->U_z, 8 * nk * 3 * CE_NZ, (const void**)&d.U_z}, {t->chi, 8 * 3 * size_t(CE_NZ), (const void**)&d.chi},
        {M ? (const void*)t->atoms : izeros.data(), 4 * std::max<size_t>(size_t(M) * CE_MAXATOMS, 1), (const void**)&d.atoms},
        {M ? (const void*)t->charge : izeros.data(), 4 * std::max<size_t>(M, 1), (const void**)&d.charge},
        {M ? (const void*)t->kind : izeros.data(), 4 * std::max<size_t>(M, 1), (const void**)&d.kind},
        {M ? (const void*)t->off : zeros.data(), 8 * size_t(M + 1 > 1 ? M + 1 : 1), (const void**)&d.off},
        {M ? (const void*)t->spl_t : zeros.data(), 8 * std::max<size_t>(nspl, 1), (const void**)&d.t},
        {M ? (const void*)t->spl_u : zeros.data(), 8 * std::max<size_t>(nspl, 1), (const void**)&d.u},
        {M ? (const void*)t->spl_z : zeros.data(), 8 * std::max<size_t>(nspl, 1), (const void**)&d.z},
        {polyatomic ? (const void*)t->D00 : zeros.data(), 8 * (polyatomic ? size_t(M) : 1), (const void**)&d.D00},
        {polyatomic ? (const void*)t->lmr : zeros.data(), 8 * (polyatomic ? size_t(M) : 1), (const void**)&d.lmr},
        {ip(nat), 4 * std::max<size_t>(M, 1), (const void**)&d.nat},
        {inc_ptr.data(), 4 * inc_ptr.size(), (const void**)&d.inc_ptr},
        {ip(inc_mol), 4 * std::max<size_t>(inc_mol.size(), 1), (const void**)&d.inc_mol},
        {ip(inc_cnt), 4 * std::max<size_t>(inc_cnt.size(), 1), (const void**)&d.inc_cnt},
        {ip(item_elem), 4 * std::max<size_t>(item_elem.size(), 1), (const void**)&d.item_elem},
        {item_begin.data(), 4 * item_begin.size(), (const void**)&d.item_begin},
        {elem_item_ptr.data(), 4 * elem_item_ptr.size(), (const void**)&d.elem_item_ptr},
        {ip(pair_row), 4 * std::max<size_t>(pair_row.size(), 1), (const void**)&d.pair_row},
        {ip(pair_col), 4 * std::max<size_t>(pair_col.size(), 1), (const void**)&d.pair_col},
        {pair_ptr.data(), 4 * pair_ptr.size(), (const void**)&d.pair_ptr},
        {ip(pair_mol), 4 * std::max<size_t>(pair_mol.size(), 1), (const void**)&d.pair_mol},
        {ip(pair_coef), 4 * std::max<size_t>(pair_coef.size(), 1), (const void**)&d.pair_coef}};
    size_t total = 0;
    for (const Piece& q : pcs) {
        if (!q.src) return set_err(ctx, KORG_EINVAL, "null equilibrium table");
        total += a256(q.bytes);
    }
    std::vector<unsigned char> host(total);
    size_t off = 0;
    for (const Piece& q : pcs) {
        memcpy(host.data() + off, q.src, q.bytes);
        off += a256(q.bytes);
    }
    void* buf = nullptr;
    cudaError_t e = cudaMalloc(&buf, total);
    if (e != cudaSuccess) return set_err(ctx, KORG_ENOMEM, "cudaMalloc(%zu): %s", total, cudaGetErrorString(e));
    e = cudaMemcpy(buf, host.data(), total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(buf);
        return set_err(ctx, KORG_ECUDA, "equilibrium tables: %s", cudaGetErrorString(e));
    }
    off = 0;
    for (const Piece& q : pcs) {
        *q.dst = static_cast<unsigned char*>(buf) + off;
        off += a256(q.bytes);
    }
    if (ctx->chem_buf) {
        KCUDA(cudaDeviceSynchronize());
        cudaFree(ctx->chem_buf);
    }
    ctx->chem_buf = buf;
    ctx->chem_tab = d;
    ctx->chem_lnT0 = t->lnT[0];
    ctx->chem_lnT1 = t->lnT[t->n_knots - 1];
    ctx->have_chem = true;
    return KORG_OK;
}

KORG_API int korg_chemical_equilibrium_dev(korg_ctx* ctx, const korg_chem_layers* y, int32_t n_atm, double* dens,
                                           int32_t* status, double* info, void* stream) {
    if (!ctx) return KORG_EINVAL;
    if (!y || y->L < 1 || !y->T || !y->n_tot || !y->ne_model || !y->abundances || n_atm < 1 || !dens || !status)
        return set_err(ctx, KORG_EINVAL, "bad arguments");
    if (!ctx->have_chem) return set_err(ctx, KORG_ENOTABLES, "korg_set_equilibrium_tables() has not been called");
    KCUDA(cudaSetDevice(ctx->device));
    const int smem = int(sizeof(CeShared));
    KCUDA(cudaFuncSetAttribute(chem_eq_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const ChemLayersDev ly{y->L, y->T, y->n_tot, y->ne_model, y->abundances, y->atm};
    chem_eq_kernel<<<unsigned(y->L), CE_THREADS, smem, static_cast<cudaStream_t>(stream)>>>(ctx->chem_tab, ly, dens,
                                                                                            status, info);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

KORG_API int korg_chemical_equilibrium(korg_ctx* ctx, const korg_chem_layers* y, int32_t n_atm, double* dens,
                                       int32_t* status, double* info) {
    if (!ctx) return KORG_EINVAL;
    if (!y || y->L < 1 || !y->T || !y->n_tot || !y->ne_model || !y->abundances || n_atm < 1 || !dens || !status)
        return set_err(ctx, KORG_EINVAL, "bad arguments");
    if (!ctx->have_chem) return set_err(ctx, KORG_ENOTABLES, "korg_set_equilibrium_tables() has not been called");
    const int L = y->L;
    for (int l = 0; l < L; l++) {
        const double T = y->T[l], nt = y->n_tot[l], ne = y->ne_model[l];
        if (!(std::isfinite(T) && T > 0 && std::log(T) >= ctx->chem_lnT0 && std::log(T) <= ctx->chem_lnT1))
            return set_err(ctx, KORG_EINVAL, "layer %d: T = %g outside the partition functions' range", l, T);
        if (!(std::isfinite(nt) && std::isfinite(ne) && ne > 0 && nt > ne))
            return set_err(ctx, KORG_EINVAL, "layer %d: need 0 < n_e < n_tot (n_e = %g, n_tot = %g)", l, ne, nt);
        if (y->atm && (y->atm[l] < 0 || y->atm[l] >= n_atm))
            return set_err(ctx, KORG_EINVAL, "layer %d: atmosphere index %d", l, y->atm[l]);
    }
    for (int64_t k = 0; k < int64_t(n_atm) * CE_NZ; k++)
        if (!(std::isfinite(y->abundances[k]) && y->abundances[k] > 0))
            return set_err(ctx, KORG_EINVAL, "abundance %lld is not positive", (long long)k);
    KCUDA(cudaSetDevice(ctx->device));
    const size_t nspec = size_t(KORG_CHEM_MOL0 + ctx->chem_tab.n_mol);
    Stager st;
    const size_t o_T = st.add(y->T, 8 * size_t(L)), o_n = st.add(y->n_tot, 8 * size_t(L));
    const size_t o_e = st.add(y->ne_model, 8 * size_t(L));
    const size_t o_a = st.add(y->abundances, 8 * size_t(n_atm) * CE_NZ);
    const size_t o_m = y->atm ? st.add(y->atm, 4 * size_t(L)) : 0;
    const size_t o_d = st.add(nullptr, 8 * size_t(L) * nspec);
    const size_t o_s = st.add(nullptr, 4 * size_t(L));
    const size_t o_i = st.add(nullptr, 8 * size_t(L) * CE_NINFO);
    char* b = nullptr;
    KCHECK(upload(ctx, st, &b));
    const korg_chem_layers d{L, (const double*)(b + o_T), (const double*)(b + o_n), (const double*)(b + o_e),
                             (const double*)(b + o_a), y->atm ? (const int32_t*)(b + o_m) : nullptr};
    KCHECK(korg_chemical_equilibrium_dev(ctx, &d, n_atm, (double*)(b + o_d), (int32_t*)(b + o_s), (double*)(b + o_i),
                                         ctx->stream));
    KCUDA(cudaMemcpyAsync(dens, b + o_d, 8 * size_t(L) * nspec, cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaMemcpyAsync(status, b + o_s, 4 * size_t(L), cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<double> inf(size_t(L) * CE_NINFO);  // iterations, solves, log xi, inf-norm, FP64 steps
    KCUDA(cudaMemcpyAsync(inf.data(), b + o_i, 8 * inf.size(), cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaStreamSynchronize(ctx->stream));
    if (info) memcpy(info, inf.data(), 8 * inf.size());
    int nbad = 0, first = -1;
    for (int l = 0; l < L; l++)
        if (status[l] != KORG_CHEM_OK) {
            nbad++;
            if (first < 0) first = l;
        }
    if (nbad)
        return set_err(ctx, KORG_ECHEM, "chemical equilibrium failed in %d layer(s); first: layer %d, status %d "
                       "(log xi %g, inf-norm %g)", nbad, first, status[first], inf[size_t(first) * CE_NINFO + 2],
                       inf[size_t(first) * CE_NINFO + 3]);
    return KORG_OK;
}

KORG_API int korg_chemical_equilibrium_vjp_dev(korg_ctx* ctx, const korg_chem_layers* y, int32_t n_atm,
                                               const double* dens, const double* gbar, double* dT, double* dn_tot,
                                               double* dab, int32_t* status, void* stream) {
    if (!ctx) return KORG_EINVAL;
    if (!y || y->L < 1 || !y->T || !y->n_tot || !y->ne_model || !y->abundances || n_atm < 1 || !dens || !gbar ||
        !dT || !dn_tot || !dab || !status)
        return set_err(ctx, KORG_EINVAL, "bad arguments");
    if (!ctx->have_chem) return set_err(ctx, KORG_ENOTABLES, "korg_set_equilibrium_tables() has not been called");
    KCUDA(cudaSetDevice(ctx->device));
    const int smem = int(sizeof(CeShared));
    KCUDA(cudaFuncSetAttribute(chem_vjp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const ChemLayersDev ly{y->L, y->T, y->n_tot, y->ne_model, y->abundances, y->atm};
    chem_vjp_kernel<<<unsigned(y->L), CE_THREADS, smem, static_cast<cudaStream_t>(stream)>>>(ctx->chem_tab, ly, dens,
                                                                                             gbar, dT, dn_tot, dab,
                                                                                             status);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

KORG_API int korg_chemical_equilibrium_vjp(korg_ctx* ctx, const korg_chem_layers* y, int32_t n_atm,
                                           const double* dens, const double* gbar, double* dT, double* dn_tot,
                                           double* dab) {
    if (!ctx) return KORG_EINVAL;
    if (!y || y->L < 1 || !y->T || !y->n_tot || !y->ne_model || !y->abundances || n_atm < 1 || !dens || !gbar ||
        !dT || !dn_tot || !dab)
        return set_err(ctx, KORG_EINVAL, "bad arguments");
    if (!ctx->have_chem) return set_err(ctx, KORG_ENOTABLES, "korg_set_equilibrium_tables() has not been called");
    const int L = y->L;
    for (int l = 0; l < L; l++) {
        const double T = y->T[l];
        if (!(std::isfinite(T) && T > 0 && std::log(T) >= ctx->chem_lnT0 && std::log(T) <= ctx->chem_lnT1))
            return set_err(ctx, KORG_EINVAL, "layer %d: T = %g outside the partition functions' range", l, T);
        if (y->atm && (y->atm[l] < 0 || y->atm[l] >= n_atm))
            return set_err(ctx, KORG_EINVAL, "layer %d: atmosphere index %d", l, y->atm[l]);
    }
    KCUDA(cudaSetDevice(ctx->device));
    const size_t nspec = size_t(KORG_CHEM_MOL0 + ctx->chem_tab.n_mol);
    Stager st;
    const size_t o_T = st.add(y->T, 8 * size_t(L)), o_n = st.add(y->n_tot, 8 * size_t(L));
    const size_t o_e = st.add(y->ne_model, 8 * size_t(L));
    const size_t o_a = st.add(y->abundances, 8 * size_t(n_atm) * CE_NZ);
    const size_t o_m = y->atm ? st.add(y->atm, 4 * size_t(L)) : 0;
    const size_t o_d = st.add(dens, 8 * size_t(L) * nspec), o_g = st.add(gbar, 8 * size_t(L) * nspec);
    const size_t o_dT = st.add(nullptr, 8 * size_t(L)), o_dn = st.add(nullptr, 8 * size_t(L));
    const size_t o_da = st.add(nullptr, 8 * size_t(L) * CE_NZ), o_s = st.add(nullptr, 4 * size_t(L));
    char* b = nullptr;
    KCHECK(upload(ctx, st, &b));
    const korg_chem_layers d{L, (const double*)(b + o_T), (const double*)(b + o_n), (const double*)(b + o_e),
                             (const double*)(b + o_a), y->atm ? (const int32_t*)(b + o_m) : nullptr};
    KCHECK(korg_chemical_equilibrium_vjp_dev(ctx, &d, n_atm, (const double*)(b + o_d), (const double*)(b + o_g),
                                             (double*)(b + o_dT), (double*)(b + o_dn), (double*)(b + o_da),
                                             (int32_t*)(b + o_s), ctx->stream));
    std::vector<int32_t> status(L);
    KCUDA(cudaMemcpyAsync(dT, b + o_dT, 8 * size_t(L), cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaMemcpyAsync(dn_tot, b + o_dn, 8 * size_t(L), cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaMemcpyAsync(dab, b + o_da, 8 * size_t(L) * CE_NZ, cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaMemcpyAsync(status.data(), b + o_s, 4 * size_t(L), cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaStreamSynchronize(ctx->stream));
    for (int l = 0; l < L; l++)
        if (status[l] != KORG_CHEM_OK)
            return set_err(ctx, KORG_ECHEM, "chemical-equilibrium reverse mode: singular or non-finite system in layer %d",
                           l);
    return KORG_OK;
}

KORG_API int korg_line_absorption(korg_ctx* ctx, double* alpha, const double* wls, int64_t nwl,
                                  const korg_lines* lines, const korg_layers* layers, const korg_cntm* cntm,
                                  double cutoff, int precision, int64_t* n_evals) {
    if (!ctx) return KORG_EINVAL;
    KPREC(precision);
    if (!alpha || !cntm || cntm->nk < 1 || !cntm->vals || (cntm->nk > 1 && !cntm->knots))
        return set_err(ctx, KORG_EINVAL, "bad alpha / continuum arguments");
    KCHECK(check_wls(ctx, wls, nwl));
    KCHECK(check_layers(ctx, layers));
    KCHECK(check_lines(ctx, lines, layers->S));
    if (n_evals) *n_evals = 0;
    if (lines->n == 0) return KORG_OK;  // src/line_absorption.jl:35-37
    KCUDA(cudaSetDevice(ctx->device));
    const int L = layers->L;
    Stager st;
    const size_t o_alpha = st.add(alpha, sizeof(double) * L * size_t(nwl));
    const size_t o_wls = st.add(wls, sizeof(double) * nwl);
    LinesStage ls = stage_lines(st, lines);
    const size_t o_T = st.add(layers->T, 8 * L), o_ne = st.add(layers->ne, 8 * L);
    const size_t o_nv = st.add(layers->n_eff_vdW, 8 * L), o_xi = st.add(layers->xi, 8 * L);
    const size_t o_nu = st.add(layers->n_div_U, 8 * size_t(L) * layers->S);
    const size_t o_ck = cntm->nk > 1 ? st.add(cntm->knots, 8 * cntm->nk) : 0;
    const size_t o_cv = st.add(cntm->vals, 8 * size_t(L) * cntm->nk);
    char* b = nullptr;
    KCHECK(upload(ctx, st, &b));
    KCHECK(reset_counters(ctx, ctx->stream));
    LayersDev lay{L, layers->S, (double*)(b + o_T), (double*)(b + o_ne), (double*)(b + o_nv), (double*)(b + o_xi),
                  (double*)(b + o_nu)};
    CntmDev cn{cntm->nk, cntm->nk > 1 ? (double*)(b + o_ck) : nullptr, (double*)(b + o_cv)};
    double* d_alpha = (double*)(b + o_alpha);
    KCHECK(run_line_absorption(ctx, d_alpha, (double*)(b + o_wls), nwl, lines_from_stage(ls, b, lines->n), lay, cn,
                               cutoff, precision == KORG_MIXED, ctx->stream));
    KCUDA(cudaMemcpyAsync(alpha, d_alpha, sizeof(double) * L * size_t(nwl), cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaStreamSynchronize(ctx->stream));
    if (n_evals) {
        korg_stats s;
        KCHECK(korg_get_stats(ctx, &s));
        *n_evals = s.line_evals;
    }
    return KORG_OK;
}

KORG_API int korg_hydrogen_lines_dev(korg_ctx* ctx, double* alpha, const double* wls, int64_t nwl, int32_t L,
                                     const double* T, const double* ne, const double* nH_I, const double* nHe_I,
                                     const double* UH_I, const double* xi, double window, int use_MHD,
                                     int precision, void* stream) {
    if (!ctx || !alpha || !wls || nwl < 1 || L < 1 || !T || !ne || !nH_I || !nHe_I || !UH_I || !xi)
        return ctx ? set_err(ctx, KORG_EINVAL, "bad arguments") : KORG_EINVAL;
    KPREC(precision);
    KCUDA(cudaSetDevice(ctx->device));
    const HLayers hl{L, T, ne, nH_I, nHe_I, UH_I, xi};
    return run_hydrogen(ctx, alpha, wls, nwl, hl, window, use_MHD, precision == KORG_MIXED,
                        static_cast<cudaStream_t>(stream));
}

KORG_API int korg_hydrogen_line_absorption(korg_ctx* ctx, double* alphas, const double* wls, int64_t nwl,
                                           double T, double ne, double nH_I, double nHe_I, double UH_I, double xi,
                                           double window, int use_MHD, int precision) {
    if (!ctx) return KORG_EINVAL;
    KPREC(precision);
    if (!alphas) return set_err(ctx, KORG_EINVAL, "null alphas");
    KCHECK(check_wls(ctx, wls, nwl));
    KCUDA(cudaSetDevice(ctx->device));
    const double scal[6] = {T, ne, nH_I, nHe_I, UH_I, xi};
    Stager st;
    const size_t o_a = st.add(alphas, 8 * size_t(nwl));
    const size_t o_w = st.add(wls, 8 * size_t(nwl));
    const size_t o_s = st.add(scal, sizeof scal);
    char* b = nullptr;
    KCHECK(upload(ctx, st, &b));
    const double* s = (double*)(b + o_s);
    const HLayers hl{1, s, s + 1, s + 2, s + 3, s + 4, s + 5};
    KCHECK(run_hydrogen(ctx, (double*)(b + o_a), (double*)(b + o_w), nwl, hl, window, use_MHD,
                        precision == KORG_MIXED, ctx->stream));
    KCUDA(cudaMemcpyAsync(alphas, b + o_a, 8 * size_t(nwl), cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaStreamSynchronize(ctx->stream));
    return KORG_OK;
}

KORG_API int korg_radiative_transfer_dev(korg_ctx* ctx, const double* alpha, const double* S, int32_t L,
                                         int64_t nwl, const double* tau_ref, const double* alpha_ref, double* flux,
                                         void* stream) {
    if (!ctx || !alpha || !S || L < 1 || nwl < 1 || !tau_ref || !alpha_ref || !flux)
        return ctx ? set_err(ctx, KORG_EINVAL, "bad arguments") : KORG_EINVAL;
    KCUDA(cudaSetDevice(ctx->device));
    return run_rt(ctx, alpha, S, nullptr, nullptr, nwl, L, tau_ref, alpha_ref, CntmDev{0, nullptr, nullptr}, flux,
                  nullptr, 1.0, static_cast<cudaStream_t>(stream));
}

KORG_API int korg_radiative_transfer(korg_ctx* ctx, const double* alpha, const double* S, int32_t L, int64_t nwl,
                                     const double* tau_ref, const double* alpha_ref, double* flux) {
    if (!ctx) return KORG_EINVAL;
    if (!alpha || !S || L < 1 || nwl < 1 || !tau_ref || !alpha_ref || !flux)
        return set_err(ctx, KORG_EINVAL, "bad arguments");
    KCUDA(cudaSetDevice(ctx->device));
    Stager st;
    const size_t n = size_t(L) * nwl;
    const size_t o_a = st.add(alpha, 8 * n), o_s = st.add(S, 8 * n);
    const size_t o_t = st.add(tau_ref, 8 * L), o_r = st.add(alpha_ref, 8 * L);
    const size_t o_f = st.add(nullptr, 8 * size_t(nwl));
    char* b = nullptr;
    KCHECK(upload(ctx, st, &b));
    KCHECK(run_rt(ctx, (double*)(b + o_a), (double*)(b + o_s), nullptr, nullptr, nwl, L, (double*)(b + o_t),
                  (double*)(b + o_r), CntmDev{0, nullptr, nullptr}, (double*)(b + o_f), nullptr, 1.0, ctx->stream));
    KCUDA(cudaMemcpyAsync(flux, b + o_f, 8 * size_t(nwl), cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaStreamSynchronize(ctx->stream));
    return KORG_OK;
}

KORG_API int korg_radiative_transfer_general(korg_ctx* ctx, const double* alpha, const double* S, int32_t L,
                                             int64_t nwl, const double* spatial, int spherical,
                                             const double* tau_ref, const double* alpha_ref, const double* mu,
                                             const double* mu_weights, int32_t n_mu, int include_inward_rays,
                                             int tau_scheme, int I_scheme, double* flux, double* I_surface) {
    if (!ctx) return KORG_EINVAL;
    if (!alpha || !S || L < 1 || nwl < 1 || !spatial || !tau_ref || !alpha_ref || !mu || !mu_weights || n_mu < 1 ||
        !flux)
        return set_err(ctx, KORG_EINVAL, "bad arguments");
    if (tau_scheme < 0 || tau_scheme > 1)
        return set_err(ctx, KORG_EINVAL, "tau_scheme must be one of \"anchored\" or \"bezier\"");
    if (I_scheme < 0 || I_scheme > 3)
        return set_err(ctx, KORG_EINVAL, "I_scheme must be one of \"linear\", \"bezier\", or \"linear_flux_only\"");
    if (I_scheme == 3 && (spherical || tau_scheme != 0))
        return set_err(ctx, KORG_EINVAL, "the exponential-integral flux needs a planar atmosphere and anchored tau");
    if (L > RTG_LMAX) return set_err(ctx, KORG_EINVAL, "at most %d layers", RTG_LMAX);
    // rays (RadiativeTransfer.jl:218-242): path length s and ds/dz per surface mu
    std::vector<int32_t> nlay(n_mu);
    std::vector<double> s(size_t(n_mu) * L), dsdz(size_t(n_mu) * L);
    for (int u = 0; u < n_mu; u++) {
        if (spherical) {
            const double b = spatial[0] * std::sqrt(1 - mu[u] * mu[u]);
            int low;
            if (b < spatial[L - 1]) {
                low = L;
            } else {
                int am = 0;
                for (int k = 1; k < L; k++)
                    if (std::fabs(spatial[k] - b) < std::fabs(spatial[am] - b)) am = k;
                if (spatial[am] < b) am -= 1;
                low = am + 1;
            }
            nlay[u] = low;
            for (int k = 0; k < low; k++) {
                s[size_t(u) * L + k] = std::sqrt(spatial[k] * spatial[k] - b * b);
                dsdz[size_t(u) * L + k] = spatial[k] / s[size_t(u) * L + k];
            }
        } else {
            nlay[u] = L;
            for (int k = 0; k < L; k++) {
                s[size_t(u) * L + k] = spatial[k] / mu[u];
                dsdz[size_t(u) * L + k] = 1.0 / mu[u];
            }
        }
    }
    // inward rays: all, or those that do not reach the bottom (:94-98)
    std::vector<int> in_idx;
    for (int u = 0; u < n_mu; u++)
        if (include_inward_rays || nlay[u] < L) in_idx.push_back(u);
    const int n_in = int(in_idx.size()), nrays = n_in + n_mu;
    if (nrays > RTG_RMAX) return set_err(ctx, KORG_EINVAL, "at most %d rays (inward + outward)", RTG_RMAX);
    std::vector<int32_t> rn(nrays);
    std::vector<double> rfac(size_t(nrays) * L, 0.0), rlt(size_t(nrays) * L, 0.0), rpath(size_t(nrays) * L, 0.0);
    for (int r = 0; r < nrays; r++) {
        const bool inward = r < n_in;
        const int u = inward ? in_idx[r] : r - n_in;
        const int n = nlay[u];
        rn[r] = n;
        for (int k = 0; k < n; k++) {
            const int lk = inward ? n - 1 - k : k;
            rpath[size_t(r) * L + k] = inward ? -s[size_t(u) * L + lk] : s[size_t(u) * L + lk];
            rfac[size_t(r) * L + k] = tau_ref[lk] / alpha_ref[lk] * dsdz[size_t(u) * L + lk];
            rlt[size_t(r) * L + k] = inward ? -std::log(tau_ref[lk]) : std::log(tau_ref[lk]);
        }
    }
    std::vector<double> wmu(n_mu);
    for (int u = 0; u < n_mu; u++) wmu[u] = mu_weights[u] * mu[u];
    KCUDA(cudaSetDevice(ctx->device));
    Stager st;
    const size_t n = size_t(L) * nwl;
    const size_t o_a = st.add(alpha, 8 * n), o_s = st.add(S, 8 * n);
    const size_t o_rn = st.add(rn.data(), 4 * rn.size()), o_rf = st.add(rfac.data(), 8 * rfac.size());
    const size_t o_rl = st.add(rlt.data(), 8 * rlt.size()), o_rp = st.add(rpath.data(), 8 * rpath.size());
    const size_t o_w = st.add(wmu.data(), 8 * wmu.size());
    const size_t o_f = st.add(nullptr, 8 * size_t(nwl));
    const size_t o_i = I_surface ? st.add(nullptr, 8 * size_t(nwl) * n_mu) : 0;
    char* b = nullptr;
    KCHECK(upload(ctx, st, &b));
    RtGenArgs ra{(double*)(b + o_a), (double*)(b + o_s), L, nwl, nrays, n_in, n_mu, (int32_t*)(b + o_rn),
                 (double*)(b + o_rf), (double*)(b + o_rl), (double*)(b + o_rp), (double*)(b + o_w), tau_scheme,
                 I_scheme, static_cast<MathTables*>(ctx->math.p), (double*)(b + o_f),
                 I_surface ? (double*)(b + o_i) : nullptr};
    rt_general_kernel<<<unsigned((nwl + 127) / 128), 128, 0, ctx->stream>>>(ra);
    KCUDA(cudaGetLastError());
    KCUDA(cudaMemcpyAsync(flux, b + o_f, 8 * size_t(nwl), cudaMemcpyDeviceToHost, ctx->stream));
    if (I_surface)
        KCUDA(cudaMemcpyAsync(I_surface, b + o_i, 8 * size_t(nwl) * n_mu, cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaStreamSynchronize(ctx->stream));
    return KORG_OK;
}

KORG_API int korg_synthesize_dev(korg_ctx* ctx, const korg_synth_inputs* in, const korg_lines* lines,
                                 const korg_lines* lines5, const double* wls, int64_t nwl, int precision,
                                 double* flux, double* cntm, double* alpha_out, void* stream) {
    if (!ctx || !in || !lines || !lines5 || !wls || nwl < 1 || !flux || !cntm)
        return ctx ? set_err(ctx, KORG_EINVAL, "bad arguments") : KORG_EINVAL;
    KPREC(precision);
    if (in->cntm.nk < 2 || in->layers.L < 1)
        return set_err(ctx, KORG_EINVAL, "synthesize needs a continuum grid of at least 2 knots");
    KCUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int L = in->layers.L;
    double* alpha = alpha_out;
    if (!alpha) {
        KCHECK(ensure(ctx, ctx->alpha, sizeof(double) * size_t(L) * nwl));
        alpha = static_cast<double*>(ctx->alpha.p);
    }
    KCHECK(ensure(ctx, ctx->aref, sizeof(double) * (L + 1)));
    double* aref = static_cast<double*>(ctx->aref.p);
    KCUDA(cudaMemcpyAsync(aref + L, &in->ref_wl, sizeof(double), cudaMemcpyHostToDevice, s));
    KCHECK(reset_counters(ctx, s));
    return run_synthesize(ctx, in, lines_dev(lines), lines_dev(lines5), wls, nwl, precision == KORG_MIXED, flux,
                          cntm, alpha, aref, aref + L, s);
}

KORG_API int korg_synthesize(korg_ctx* ctx, const korg_synth_inputs* in, const korg_lines* lines,
                             const korg_lines* lines5, const double* wls, int64_t nwl, int precision, double* flux,
                             double* cntm, double* alpha_out, double* alpha_ref_out) {
    if (!ctx) return KORG_EINVAL;
    KPREC(precision);
    if (!in || !flux || !cntm) return set_err(ctx, KORG_EINVAL, "bad arguments");
    KCHECK(check_wls(ctx, wls, nwl));
    KCHECK(check_layers(ctx, &in->layers));
    KCHECK(check_lines(ctx, lines, in->layers.S));
    KCHECK(check_lines(ctx, lines5, in->layers.S));
    if (in->cntm.nk < 2 || !in->cntm.knots || !in->cntm.vals || !in->tau_ref || !in->alpha_ref_cntm)
        return set_err(ctx, KORG_EINVAL, "bad continuum / reference inputs");
    if (in->hydrogen_lines && (!in->nH_I || !in->nHe_I || !in->UH_I))
        return set_err(ctx, KORG_EINVAL, "hydrogen lines need nH_I, nHe_I and UH_I");
    KCUDA(cudaSetDevice(ctx->device));
    const int L = in->layers.L;
    const int S = in->layers.S;
    Stager st;
    const size_t o_w = st.add(wls, 8 * size_t(nwl));
    LinesStage ls = stage_lines(st, lines), ls5 = stage_lines(st, lines5);
    const korg_layers& y = in->layers;
    const size_t o_T = st.add(y.T, 8 * L), o_ne = st.add(y.ne, 8 * L), o_nv = st.add(y.n_eff_vdW, 8 * L),
                 o_xi = st.add(y.xi, 8 * L), o_nu = st.add(y.n_div_U, 8 * size_t(L) * S);
    const size_t o_tr = st.add(in->tau_ref, 8 * L), o_ar = st.add(in->alpha_ref_cntm, 8 * L);
    const size_t o_h1 = in->hydrogen_lines ? st.add(in->nH_I, 8 * L) : 0;
    const size_t o_h2 = in->hydrogen_lines ? st.add(in->nHe_I, 8 * L) : 0;
    const size_t o_h3 = in->hydrogen_lines ? st.add(in->UH_I, 8 * L) : 0;
    const size_t o_ck = st.add(in->cntm.knots, 8 * in->cntm.nk);
    const size_t o_cv = st.add(in->cntm.vals, 8 * size_t(L) * in->cntm.nk);
    const size_t o_fl = st.add(nullptr, 8 * size_t(nwl));
    const size_t o_cn = st.add(nullptr, 8 * size_t(nwl));
    char* b = nullptr;
    KCHECK(upload(ctx, st, &b));
    korg_synth_inputs d = *in;
    d.layers = korg_layers{L, S, (double*)(b + o_T), (double*)(b + o_ne), (double*)(b + o_nv), (double*)(b + o_xi),
                           (double*)(b + o_nu)};
    d.tau_ref = (double*)(b + o_tr);
    d.alpha_ref_cntm = (double*)(b + o_ar);
    d.nH_I = in->hydrogen_lines ? (double*)(b + o_h1) : nullptr;
    d.nHe_I = in->hydrogen_lines ? (double*)(b + o_h2) : nullptr;
    d.UH_I = in->hydrogen_lines ? (double*)(b + o_h3) : nullptr;
    d.cntm = korg_cntm{in->cntm.nk, (double*)(b + o_ck), (double*)(b + o_cv)};
    KCHECK(ensure(ctx, ctx->alpha, sizeof(double) * size_t(L) * nwl));
    KCHECK(ensure(ctx, ctx->aref, sizeof(double) * (L + 1)));
    double* aref = static_cast<double*>(ctx->aref.p);
    KCUDA(cudaMemcpyAsync(aref + L, &in->ref_wl, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    double* d_alpha = static_cast<double*>(ctx->alpha.p);
    KCHECK(reset_counters(ctx, ctx->stream));
    KCHECK(run_synthesize(ctx, &d, lines_from_stage(ls, b, lines->n), lines_from_stage(ls5, b, lines5->n),
                          (double*)(b + o_w), nwl, precision == KORG_MIXED, (double*)(b + o_fl), (double*)(b + o_cn),
                          d_alpha, aref, aref + L, ctx->stream));
    // flux and continuum come back through the pinned staging buffer (same offsets as on the
    // device; the upload from it precedes them on the stream)
    char* hb = static_cast<char*>(ctx->stage_host);
    KCUDA(cudaMemcpyAsync(hb + o_fl, b + o_fl, o_cn - o_fl + 8 * size_t(nwl), cudaMemcpyDeviceToHost, ctx->stream));
    if (alpha_out)
        KCUDA(cudaMemcpyAsync(alpha_out, d_alpha, 8 * size_t(L) * nwl, cudaMemcpyDeviceToHost, ctx->stream));
    if (alpha_ref_out) KCUDA(cudaMemcpyAsync(alpha_ref_out, aref, 8 * size_t(L), cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaStreamSynchronize(ctx->stream));
    par_copy({{flux, hb + o_fl, 8 * size_t(nwl)}, {cntm, hb + o_cn, 8 * size_t(nwl)}});
    return KORG_OK;
}


// A kernel whose bounded wait for staged data ran out sets the mapped error word; read and clear
// it (the caller has synchronised).
int take_device_error(korg_ctx* ctx) {
    if (ctx->dev_err_host && *reinterpret_cast<volatile int*>(ctx->dev_err_host)) {
        *reinterpret_cast<volatile int*>(ctx->dev_err_host) = 0;
        return set_err(ctx, KORG_ETIMEOUT, "a device-side wait for staged data ran past its limit; results are invalid");
    }
    return KORG_OK;
}

KORG_API int korg_device_status(korg_ctx* ctx) {
    if (!ctx) return KORG_EINVAL;
    KCUDA(cudaSetDevice(ctx->device));
    KCUDA(cudaDeviceSynchronize());
    return take_device_error(ctx);
}

KORG_API int korg_selftest_wait_timeout(korg_ctx* ctx, int polls) {
    if (!ctx || polls < 1) return KORG_EINVAL;
    KCUDA(cudaSetDevice(ctx->device));
    wait_timeout_selftest_kernel<<<1, 64, 0, ctx->stream>>>(ctx->dev_err_dev, polls);
    KCUDA(cudaGetLastError());
    return korg_device_status(ctx);
}

KORG_API int korg_synthesize_vjp_dev(korg_ctx* ctx, const korg_synth_inputs* in, const korg_lines* lines,
                                     const korg_lines* lines5, const double* wls, int64_t nwl, int precision,
                                     const double* dflux, const double* dcntm, const korg_synth_grads* grads,
                                     int flags, void* stream) {
    if (!ctx) return KORG_EINVAL;
    KPREC(precision);
    if (!in || !lines || !lines5 || !wls || nwl < 1 || !grads || (!dflux && !dcntm))
        return set_err(ctx, KORG_EINVAL, "bad arguments");
    if (in->cntm.nk < 2 || in->layers.L < 1)
        return set_err(ctx, KORG_EINVAL, "synthesize needs a continuum grid of at least 2 knots");
    if (in->hydrogen_lines && !ctx->have_stark)
        return set_err(ctx, KORG_ENOTABLES, "korg_set_stark_tables() has not been called");
    KCUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int L = in->layers.L;
    KCHECK(ensure(ctx, ctx->aref, sizeof(double) * (L + 1)));
    double* aref = static_cast<double*>(ctx->aref.p);
    KCUDA(cudaMemcpyAsync(aref + L, &in->ref_wl, sizeof(double), cudaMemcpyHostToDevice, s));
    return run_vjp(ctx, in, lines_dev(lines), lines_dev(lines5), wls, nwl, precision == KORG_MIXED, dflux, dcntm,
                   *grads, flags, aref + L, s);
}

KORG_API int korg_synthesize_vjp(korg_ctx* ctx, const korg_synth_inputs* in, const korg_lines* lines,
                                 const korg_lines* lines5, const double* wls, int64_t nwl, int precision,
                                 const double* dflux, const double* dcntm, const korg_synth_grads* grads, int flags) {
    if (!ctx) return KORG_EINVAL;
    KPREC(precision);
    if (!in || !grads || (!dflux && !dcntm)) return set_err(ctx, KORG_EINVAL, "bad arguments");
    KCHECK(check_wls(ctx, wls, nwl));
    KCHECK(check_layers(ctx, &in->layers));
    KCHECK(check_lines(ctx, lines, in->layers.S));
    KCHECK(check_lines(ctx, lines5, in->layers.S));
    if (in->cntm.nk < 2 || !in->cntm.knots || !in->cntm.vals || !in->tau_ref || !in->alpha_ref_cntm)
        return set_err(ctx, KORG_EINVAL, "bad continuum / reference inputs");
    if (in->hydrogen_lines && (!in->nH_I || !in->nHe_I || !in->UH_I))
        return set_err(ctx, KORG_EINVAL, "hydrogen lines need nH_I, nHe_I and UH_I");
    KCUDA(cudaSetDevice(ctx->device));
    const int L = in->layers.L, S = in->layers.S;
    const int64_t nk = in->cntm.nk;
    Stager st;
    const size_t o_w = st.add(wls, 8 * size_t(nwl));
    LinesStage ls = stage_lines(st, lines), ls5 = stage_lines(st, lines5);
    const korg_layers& y = in->layers;
    const size_t o_T = st.add(y.T, 8 * L), o_ne = st.add(y.ne, 8 * L), o_nv = st.add(y.n_eff_vdW, 8 * L),
                 o_xi = st.add(y.xi, 8 * L), o_nu = st.add(y.n_div_U, 8 * size_t(L) * S);
    const size_t o_tr = st.add(in->tau_ref, 8 * L), o_ar = st.add(in->alpha_ref_cntm, 8 * L);
    const size_t o_h1 = in->hydrogen_lines ? st.add(in->nH_I, 8 * L) : 0;
    const size_t o_h2 = in->hydrogen_lines ? st.add(in->nHe_I, 8 * L) : 0;
    const size_t o_h3 = in->hydrogen_lines ? st.add(in->UH_I, 8 * L) : 0;
    const size_t o_ck = st.add(in->cntm.knots, 8 * nk);
    const size_t o_cv = st.add(in->cntm.vals, 8 * size_t(L) * nk);
    const size_t o_df = dflux ? st.add(dflux, 8 * size_t(nwl)) : 0;
    const size_t o_dc = dcntm ? st.add(dcntm, 8 * size_t(nwl)) : 0;
    // device outputs: one slot per gradient the caller asked for
    const size_t sizes[11] = {size_t(L), size_t(L), size_t(L), size_t(L), size_t(S) * L, size_t(L), size_t(L),
                              size_t(L), size_t(lines->n), size_t(L) * nk, size_t(L)};
    double* const host_out[11] = {grads->T, grads->ne, grads->n_eff_vdW, grads->xi, grads->n_div_U, grads->nH_I,
                                  grads->nHe_I, grads->UH_I, grads->log_gf, grads->cntm_vals, grads->alpha_ref_cntm};
    size_t o_out[11];
    for (int k = 0; k < 11; k++) o_out[k] = host_out[k] ? st.add(nullptr, 8 * std::max<size_t>(sizes[k], 1)) : 0;
    char* b = nullptr;
    KCHECK(upload(ctx, st, &b));
    korg_synth_inputs d = *in;
    d.layers = korg_layers{L, S, (double*)(b + o_T), (double*)(b + o_ne), (double*)(b + o_nv), (double*)(b + o_xi),
                           (double*)(b + o_nu)};
    d.tau_ref = (double*)(b + o_tr);
    d.alpha_ref_cntm = (double*)(b + o_ar);
    d.nH_I = in->hydrogen_lines ? (double*)(b + o_h1) : nullptr;
    d.nHe_I = in->hydrogen_lines ? (double*)(b + o_h2) : nullptr;
    d.UH_I = in->hydrogen_lines ? (double*)(b + o_h3) : nullptr;
    d.cntm = korg_cntm{nk, (double*)(b + o_ck), (double*)(b + o_cv)};
    double* dev_out[11];
    for (int k = 0; k < 11; k++) dev_out[k] = host_out[k] ? (double*)(b + o_out[k]) : nullptr;
    const korg_synth_grads dg{dev_out[0], dev_out[1], dev_out[2], dev_out[3], dev_out[4], dev_out[5],
                              dev_out[6], dev_out[7], dev_out[8], dev_out[9], dev_out[10]};
    KCHECK(ensure(ctx, ctx->aref, sizeof(double) * (L + 1)));
    double* aref = static_cast<double*>(ctx->aref.p);
    KCUDA(cudaMemcpyAsync(aref + L, &in->ref_wl, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    KCHECK(run_vjp(ctx, &d, lines_from_stage(ls, b, lines->n), lines_from_stage(ls5, b, lines5->n),
                   (double*)(b + o_w), nwl, precision == KORG_MIXED, dflux ? (double*)(b + o_df) : nullptr,
                   dcntm ? (double*)(b + o_dc) : nullptr, dg, flags, aref + L, ctx->stream));
    for (int k = 0; k < 11; k++)
        if (host_out[k] && sizes[k])
            KCUDA(cudaMemcpyAsync(host_out[k], dev_out[k], 8 * sizes[k], cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaStreamSynchronize(ctx->stream));
    return take_device_error(ctx);
}

// ------------------------------------------------------------------ post-processing
// Gaussian LSF and rotational broadening (src/utils.jl:45-240); kernels in postprocess.cuh.
namespace {
int lsf_args(korg_ctx* ctx, const double* wls, int64_t nwl, const double* owl, int64_t nout, const double* R,
             int64_t nR, double window, LsfArgs* a) {
    if (!wls || nwl < 1 || !owl || nout < 1 || !R || (nR != 1 && nR != nout) || !(window > 0))
        return set_err(ctx, KORG_EINVAL, "bad LSF arguments");
    *a = LsfArgs{wls, nwl, owl, nout, R, nR == nout && nout > 1 ? 1 : 0, window, 2 * std::sqrt(2 * std::log(2.0))};
    return KORG_OK;
}
int rot_args(korg_ctx* ctx, const double* wls, int64_t nwl, const korg_wl_range* ranges, int32_t nranges,
             double vsini, double eps, RotArgs* a) {
    if (!wls || nwl < 1 || !ranges || nranges < 1 || nranges > ROT_MAX_RANGES || !(vsini >= 0))
        return set_err(ctx, KORG_EINVAL, "bad rotation arguments (at most %d wavelength ranges)", ROT_MAX_RANGES);
    *a = RotArgs{};
    a->wls = wls;
    a->nwl = nwl;
    a->nranges = nranges;
    int64_t first = 0;
    for (int k = 0; k < nranges; k++) {
        if (ranges[k].n < 1) return set_err(ctx, KORG_EINVAL, "empty wavelength range");
        a->r[k] = RotRange{first, ranges[k].n, ranges[k].step};
        first += ranges[k].n;
    }
    if (first != nwl) return set_err(ctx, KORG_EINVAL, "the ranges do not cover the %lld wavelengths", (long long)nwl);
    a->v_over_c = vsini * 1e5 / C_CGS;  // km/s -> cm/s (:198)
    a->c1 = 2 * (1 - eps);              // :205-209
    a->c2 = PI * eps / 2;
    a->c3 = PI * (1 - eps / 3);
    return KORG_OK;
}
__global__ void add_kernel(double* dst, const double* src, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) dst[i] += src[i];
}
unsigned warp_blocks(int64_t n) { return unsigned((n * 32 + 255) / 256); }
}  // namespace

KORG_API int korg_apply_lsf_dev(korg_ctx* ctx, const double* wls, int64_t nwl, const double* out_wls, int64_t nout,
                                const double* R, int64_t nR, double window_size, const double* flux, int32_t nspec,
                                double* out, void* stream) {
    if (!ctx) return KORG_EINVAL;
    LsfArgs a;
    KCHECK(lsf_args(ctx, wls, nwl, out_wls, nout, R, nR, window_size, &a));
    if (!flux || !out || nspec < 1) return set_err(ctx, KORG_EINVAL, "bad LSF arguments");
    KCUDA(cudaSetDevice(ctx->device));
    lsf_apply_kernel<<<warp_blocks(nout), 256, 0, static_cast<cudaStream_t>(stream)>>>(a, flux, nspec, out);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

KORG_API int korg_apply_lsf_vjp_dev(korg_ctx* ctx, const double* wls, int64_t nwl, const double* out_wls,
                                    int64_t nout, const double* R, int64_t nR, double window_size, const double* dout,
                                    int32_t nspec, double* dflux, void* stream) {
    if (!ctx) return KORG_EINVAL;
    LsfArgs a;
    KCHECK(lsf_args(ctx, wls, nwl, out_wls, nout, R, nR, window_size, &a));
    if (!dout || !dflux || nspec < 1) return set_err(ctx, KORG_EINVAL, "bad LSF arguments");
    KCUDA(cudaSetDevice(ctx->device));
    lsf_vjp_kernel<<<dim3(warp_blocks(nout), unsigned((nspec + LSF_SPEC - 1) / LSF_SPEC)), 256, 0,
                     static_cast<cudaStream_t>(stream)>>>(a, dout, nspec, dflux);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

KORG_API int korg_lsf_windows_dev(korg_ctx* ctx, const double* wls, int64_t nwl, const double* out_wls, int64_t nout,
                                  const double* R, int64_t nR, double window_size, int64_t* lb, int64_t* ub,
                                  void* stream) {
    if (!ctx) return KORG_EINVAL;
    LsfArgs a;
    KCHECK(lsf_args(ctx, wls, nwl, out_wls, nout, R, nR, window_size, &a));
    if (!lb || !ub) return set_err(ctx, KORG_EINVAL, "bad LSF arguments");
    KCUDA(cudaSetDevice(ctx->device));
    lsf_windows_kernel<<<unsigned((nout + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(a, lb, ub);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

KORG_API int korg_lsf_matrix_values_dev(korg_ctx* ctx, const double* wls, int64_t nwl, const double* out_wls,
                                        int64_t nout, const double* R, int64_t nR, double window_size,
                                        const int64_t* row_ptr, double* vals, void* stream) {
    if (!ctx) return KORG_EINVAL;
    LsfArgs a;
    KCHECK(lsf_args(ctx, wls, nwl, out_wls, nout, R, nR, window_size, &a));
    if (!row_ptr || !vals) return set_err(ctx, KORG_EINVAL, "bad LSF arguments");
    KCUDA(cudaSetDevice(ctx->device));
    lsf_values_kernel<<<warp_blocks(nout), 256, 0, static_cast<cudaStream_t>(stream)>>>(a, row_ptr, vals);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

KORG_API int korg_apply_rotation_dev(korg_ctx* ctx, const double* wls, int64_t nwl, const korg_wl_range* ranges,
                                     int32_t nranges, double vsini, double eps, const double* flux, int32_t nspec,
                                     double* out, void* stream) {
    if (!ctx) return KORG_EINVAL;
    RotArgs a;
    KCHECK(rot_args(ctx, wls, nwl, ranges, nranges, vsini, eps, &a));
    if (!flux || !out || nspec < 1) return set_err(ctx, KORG_EINVAL, "bad rotation arguments");
    KCUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (vsini == 0) {  // :196-198
        KCUDA(cudaMemcpyAsync(out, flux, sizeof(double) * size_t(nwl) * nspec, cudaMemcpyDeviceToDevice, s));
        return KORG_OK;
    }
    rotation_fwd_kernel<<<unsigned((nwl + ROT_TP - 1) / ROT_TP), ROT_TP, 0, s>>>(a, flux, nspec, out);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

KORG_API int korg_apply_rotation_vjp_dev(korg_ctx* ctx, const double* wls, int64_t nwl, const korg_wl_range* ranges,
                                         int32_t nranges, double vsini, double eps, const double* dout, int32_t nspec,
                                         double* dflux, void* stream) {
    if (!ctx) return KORG_EINVAL;
    RotArgs a;
    KCHECK(rot_args(ctx, wls, nwl, ranges, nranges, vsini, eps, &a));
    if (!dout || !dflux || nspec < 1) return set_err(ctx, KORG_EINVAL, "bad rotation arguments");
    KCUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (vsini == 0) {
        const int64_t n = nwl * nspec;
        add_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(dflux, dout, n);
    } else {
        rotation_vjp_kernel<<<dim3(unsigned((nwl + 127) / 128), unsigned((nspec + ROT_SPEC - 1) / ROT_SPEC)), 128, 0,
                              s>>>(a, dout, nspec, dflux);
    }
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

KORG_API int korg_molecular_cross_section_dev(korg_ctx* ctx, const korg_lines* lines, const double* wls,
                                              int64_t nwl, const double* T, const double* inv_U, int32_t nT,
                                              const double* vmic_vals, int32_t nv, double cutoff_alpha,
                                              int precision, double* table, void* stream) {
    if (!ctx) return KORG_EINVAL;
    KPREC(precision);
    if (!lines || !wls || nwl < 1 || !T || !inv_U || nT < 1 || !vmic_vals || nv < 1 || !table || !(cutoff_alpha > 0))
        return set_err(ctx, KORG_EINVAL, "bad arguments");
    KCUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the temperatures are the "layers" (src/molecular_cross_sections.jl:63-81): n_e = 0, the
    // molecule's n / U = (1 / cutoff_alpha) / U(T), continuum 1 and cutoff threshold 1, so a line
    // is truncated where its absorption coefficient per molecule falls to cutoff_alpha; the vdW
    // perturber density is NaN (molecular lines have no vdW broadening)
    const size_t bytes = sizeof(double) * 6 * size_t(nT);
    KCHECK(ensure(ctx, ctx->mx_layers, bytes));
    double* d = static_cast<double*>(ctx->mx_layers.p);
    double* xi = d + 4 * nT;
    molxs_layers_kernel<<<(nT + 127) / 128, 128, 0, s>>>(inv_U, nT, cutoff_alpha, d);
    KCUDA(cudaGetLastError());
    KCHECK(reset_counters(ctx, s));
    const LayersDev lay{nT, 1, T, d, d + nT, xi, d + 2 * nT};
    const CntmDev cn{1, nullptr, d + 3 * nT};
    const size_t slice = size_t(nwl) * nT;
    KCUDA(cudaMemsetAsync(table, 0, sizeof(double) * slice * nv, s));
    for (int v = 0; v < nv; v++) {
        fill_kernel<<<(nT + 127) / 128, 128, 0, s>>>(xi, nT, vmic_vals + v, 1e5);  // km/s -> cm/s
        KCUDA(cudaGetLastError());
        KCHECK(run_line_absorption(ctx, table + v * slice, wls, nwl, lines_dev(lines), lay, cn, 1.0,
                                   precision == KORG_MIXED, s));
    }
    scale_kernel<<<ctx->sms * 4, 256, 0, s>>>(table, int64_t(slice) * nv, cutoff_alpha);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

KORG_API int korg_interpolate_molecular_cross_section_dev(korg_ctx* ctx, double* alpha, const double* wls,
                                                          int64_t nwl, int32_t L, const double* T,
                                                          const double* vmic, const double* n,
                                                          const double* table, const double* table_wls,
                                                          int64_t ntw, const double* vmic_vals, int32_t nv,
                                                          const double* log_temp_vals, int32_t nT, void* stream) {
    if (!ctx) return KORG_EINVAL;
    if (!alpha || !wls || nwl < 1 || L < 1 || !T || !vmic || !n || !table || !table_wls || ntw < 1 || !vmic_vals ||
        nv < 1 || !log_temp_vals || nT < 1)
        return set_err(ctx, KORG_EINVAL, "bad arguments");
    KCUDA(cudaSetDevice(ctx->device));
    const MolXsArgs ma{alpha, wls, nwl, L, T, vmic, n, table, table_wls, ntw, vmic_vals, nv, log_temp_vals, nT};
    const size_t smem = sizeof(double) * 6 * size_t(L);
    molxs_interp_kernel<<<unsigned((nwl + 63) / 64), 256, smem, static_cast<cudaStream_t>(stream)>>>(ma);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

KORG_API int korg_synthesize_batch_vjp_dev(korg_ctx* ctx, int32_t nspec, const korg_batch_item* items,
                                           const korg_batch_vjp_item* cot, const double* wls, int64_t nwl,
                                           int precision, int flags, void* stream) {
    if (!ctx) return KORG_EINVAL;
    KPREC(precision);
    if (nspec < 1 || !items || !cot || !wls || nwl < 1 || nwl > INT32_MAX - 1)
        return set_err(ctx, KORG_EINVAL, "bad batch arguments");
    const int L = items[0].in.layers.L;
    int64_t nmax = 1;
    for (int i = 0; i < nspec; i++) {
        const korg_batch_item& b = items[i];
        if (b.in.layers.L != L || b.in.cntm.nk < 2 || (!cot[i].dflux && !cot[i].dcntm))
            return set_err(ctx, KORG_EINVAL, "bad batch item %d", i);
        if (b.in.hydrogen_lines && !ctx->have_stark)
            return set_err(ctx, KORG_ENOTABLES, "korg_set_stark_tables() has not been called");
        nmax = std::max<int64_t>(nmax, std::max<int64_t>(b.lines.n, b.lines5.n));
    }
    KCUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool mixed = precision == KORG_MIXED;
    const bool reuse = flags & KORG_VJP_REUSE_FORWARD;
    if (reuse && (!ctx->b_last_resident || ctx->b_last_key != batch_key(ctx, nspec, items, wls, nwl, precision)))
        return set_err(ctx, KORG_EINVAL,
                       "KORG_VJP_REUSE_FORWARD needs the previous batch call to be korg_synthesize_batch_dev of the "
                       "same items, run in one chunk (raise max_scratch_bytes)");
    // scratch sized once for the largest spectrum, so no spectrum grows it (a growth synchronises)
    int kmax = 0;
    const int G = layer_groups(L, &kmax);
    if (G < 0) return set_err(ctx, KORG_EINVAL, "at most 256 layers are supported (got %d)", L);
    KCHECK(ensure(ctx, ctx->vjp_dpar, sizeof(double) * 3 * size_t(nmax) * size_t(G * kmax)));
    KCHECK(ensure(ctx, ctx->aref, sizeof(double) * (L + 1)));
    unsigned char* meta = static_cast<unsigned char*>(ctx->b_meta.p);
    for (int i = 0; i < nspec; i++) {
        const korg_batch_item& b = items[i];
        const double* ref_wl_dev;
        VjpOpacity op{};
        if (reuse) {
            op.alpha = static_cast<double*>(ctx->b_alpha.p) + size_t(i) * (a256(8 * size_t(L) * nwl) / 8);
            op.aref = reinterpret_cast<double*>(meta + ctx->b_last_o_aref) + size_t(i) * L;
            op.lines = static_cast<unsigned char*>(ctx->b_lines.p) + ctx->b_last_line_off[i];
            ref_wl_dev = reinterpret_cast<const double*>(meta + ctx->b_last_o_refwl) + i;
        } else {
            double* aref = static_cast<double*>(ctx->aref.p);
            KCUDA(cudaMemcpyAsync(aref + L, &b.in.ref_wl, sizeof(double), cudaMemcpyHostToDevice, s));
            ref_wl_dev = aref + L;
        }
        KCHECK(run_vjp(ctx, &b.in, lines_dev(&b.lines), lines_dev(&b.lines5), wls, nwl, mixed, cot[i].dflux,
                       cot[i].dcntm, cot[i].grads, flags & ~KORG_VJP_REUSE_FORWARD, ref_wl_dev, s,
                       reuse ? &op : nullptr));
    }
    return KORG_OK;
}

KORG_API int korg_set_batch_options(korg_ctx* ctx, int use_graph, int autotune, int64_t max_scratch_bytes) {
    if (!ctx) return KORG_EINVAL;
    if (max_scratch_bytes < 0) return set_err(ctx, KORG_EINVAL, "negative scratch budget");
    drop_graph(ctx);
    ctx->use_graph = use_graph != 0;
    ctx->autotune = autotune != 0;
    if (max_scratch_bytes > 0) ctx->batch_budget = max_scratch_bytes;
    return KORG_OK;
}

KORG_API int korg_get_tile_config(korg_ctx* ctx, int32_t L, int precision, int32_t* tw, int32_t* stage,
                                  int32_t* split, int32_t* tuned) {
    if (!ctx || !tw || !stage) return KORG_EINVAL;
    KPREC(precision);
    const bool mixed = precision == KORG_MIXED;
    const TileCfg c = tile_cfg(ctx, L, mixed);
    *tw = c.tw;
    *stage = c.stage > 0 ? c.stage : (mixed ? 2 * STAGE_LINES : STAGE_LINES / 2);
    if (split) *split = c.split;
    if (tuned) *tuned = ctx->tuned.count(std::make_pair(int(L), int(mixed))) ? 1 : 0;
    return KORG_OK;
}

KORG_API int korg_set_tile_config(korg_ctx* ctx, int32_t L, int precision, int32_t tw, int32_t stage,
                                  int32_t split) {
    if (!ctx) return KORG_EINVAL;
    KPREC(precision);
    const bool mixed = precision == KORG_MIXED;
    int kmax = 0;
    const int G = layer_groups(L, &kmax);
    TileGeom g;
    if (G < 0 || !tile_geom(mixed, G * kmax, G, TileCfg{tw, stage, split ? 1 : 0}, &g))
        return set_err(ctx, KORG_EINVAL, "tile shape (tw %d, stage %d, split %d) is not valid for %d layers", tw,
                       stage, split, L);
    drop_graph(ctx);
    ctx->tuned[std::make_pair(int(L), int(mixed))] = TileCfg{tw, stage, split ? 1 : 0};
    return KORG_OK;
}

KORG_API int korg_synthesize_batch_dev(korg_ctx* ctx, int32_t nspec, const korg_batch_item* items,
                                       const double* wls, int64_t nwl, int precision, void* stream) {
    if (!ctx) return KORG_EINVAL;
    KPREC(precision);
    if (nspec < 1 || !items || !wls || nwl < 1 || nwl > INT32_MAX - 1)
        return set_err(ctx, KORG_EINVAL, "bad batch arguments");
    KCUDA(cudaSetDevice(ctx->device));
    cudaStream_t us = static_cast<cudaStream_t>(stream);
    const bool mixed = precision == KORG_MIXED;
    std::vector<unsigned char> key = batch_key(ctx, nspec, items, wls, nwl, precision);
    if (ctx->use_graph && ctx->gexec && key == ctx->gkey) {  // same batch again: replay
        KCUDA(cudaGraphLaunch(ctx->gexec, us));
        KCUDA(cudaEventRecord(ctx->b_host_ev, us));
        ctx->stats_pending = true;
        return KORG_OK;  // the plan of the captured batch (b_last_*) still holds
    }
    ctx->b_last_key.clear();
    BatchPlan p;
    KCHECK(plan_batch(ctx, nspec, items, nwl, mixed, &p));
    if (ctx->autotune && !ctx->tuned.count(std::make_pair(p.L, int(mixed)))) {
        int first = -1;  // the spectrum with most lines stands for the batch
        for (int i = 0; i < nspec; i++)
            if (first < 0 || items[i].lines.n > items[first].lines.n) first = i;
        if (worth_tuning(nwl, items[first].lines.n)) {
            const korg_batch_item& b = items[first];
            const LinesDev ln = lines_dev(&b.lines);
            KCHECK(ensure(ctx, ctx->lines_scratch, line_scratch(nullptr, ln.n, p.L, p.Lp, p.G, mixed, nullptr)));
            LineScratch sc;
            line_scratch(static_cast<unsigned char*>(ctx->lines_scratch.p), ln.n, p.L, p.Lp, p.G, mixed, &sc);
            KCHECK(reset_counters(ctx, us));
            KCHECK(prep_lines(ctx, sc, wls, nwl, ln, layers_dev(&b.in.layers),
                              CntmDev{b.in.cntm.nk, b.in.cntm.knots, b.in.cntm.vals}, b.in.cutoff_threshold, mixed,
                              p.kmax, p.G, us));
            KCHECK(autotune_tiles(ctx, make_tile_args(sc, nullptr, wls, nwl, ln, p.L, p.Lp, p.G), p.kmax, mixed, us));
            KCHECK(plan_batch(ctx, nspec, items, nwl, mixed, &p));
            key = batch_key(ctx, nspec, items, wls, nwl, precision);
        }
    }
    KCHECK(ensure(ctx, ctx->b_alpha, p.alpha_bytes));
    KCHECK(ensure(ctx, ctx->b_lines, p.lines_bytes));
    KCHECK(ensure(ctx, ctx->b_meta, p.meta_bytes));
    // the previous batch's copy out of the host buffer (eager or replayed) must have run
    KCUDA(cudaEventSynchronize(ctx->b_host_ev));
    if (ctx->b_host_cap < p.host_bytes) {
        drop_graph(ctx);
        if (ctx->b_host) cudaFreeHost(ctx->b_host);
        ctx->b_host = nullptr;
        ctx->b_host_cap = 0;
        KCUDA(cudaHostAlloc(&ctx->b_host, p.host_bytes + p.host_bytes / 4, cudaHostAllocDefault));
        ctx->b_host_cap = p.host_bytes + p.host_bytes / 4;
    }
    fill_batch_host(ctx, p, nspec, items, wls, nwl);
    if (ctx->use_graph && !ctx->pending_key.empty() && key == ctx->pending_key) {
        // second submission of the same batch: capture it on the context's stream, then replay
        if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
        ctx->gexec = nullptr;
        ctx->gkey.clear();
        KCUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
        ctx->capturing = true;
        const int rc = enqueue_batch(ctx, p, nspec, items, wls, nwl, ctx->stream);
        ctx->capturing = false;
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
        if (rc != KORG_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return set_err(ctx, KORG_ECUDA, "graph capture: %s", cudaGetErrorString(e));
        const cudaError_t e2 = cudaGraphInstantiate(&ctx->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e2 != cudaSuccess) {
            ctx->gexec = nullptr;
            return set_err(ctx, KORG_ECUDA, "graph instantiation: %s", cudaGetErrorString(e2));
        }
        ctx->gkey = key;
        ctx->pending_key.clear();
        KCUDA(cudaGraphLaunch(ctx->gexec, us));
    } else {
        KCHECK(enqueue_batch(ctx, p, nspec, items, wls, nwl, us));
        if (ctx->use_graph) ctx->pending_key = key;
    }
    KCUDA(cudaEventRecord(ctx->b_host_ev, us));
    ctx->b_last_key = key;
    ctx->b_last_resident = p.chunk_first.size() == 2;
    ctx->b_last_line_off = p.line_off;
    ctx->b_last_o_aref = p.o_aref;
    ctx->b_last_o_refwl = p.o_refwl;
    return KORG_OK;
}

}  // extern "C"

// ====================================================================== math self-test
namespace {
__device__ __forceinline__ void atomic_max_pos(unsigned long long* a, double v) {
    atomicMax(a, (unsigned long long)__double_as_longlong(v));  // non-negative doubles order as integers
}
// fexp64 against exp over [-700, 700] (error in ulps of the CUDA result) and flog64 against
// log over [1e-300, 1e300] (error relative to max(1, |log x|)).
__global__ void math_selftest_kernel(const MathTables* tab, int64_t n, unsigned long long* out) {
    __shared__ MathTables t;
    load_math_tables(t, tab);
    __syncthreads();
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const double u = (double(i) + 0.5) / double(n);
        const double x = -700.0 + 1400.0 * u;
        const double a = fexp64(x, t), b = exp(x);
        const int eb = int((__double_as_longlong(b) >> 52) & 0x7ff);
        const double ulp = __longlong_as_double((long long)(eb > 52 ? eb - 52 : 1) << 52);
        atomic_max_pos(out, fabs(a - b) / ulp);
        const double y = exp10(-300.0 + 600.0 * u);
        const double ly = log(y);
        atomic_max_pos(out + 1, fabs(flog64(y, t) - ly) / fmax(1.0, fabs(ly)));
    }
}
}  // namespace

// Not a counterpart of any reference function: checks the table-driven FP64 exp / log used by
// the prologue and transfer kernels against the CUDA functions on n points.
extern "C" KORG_API int korg_math_selftest(korg_ctx* ctx, int64_t n, double* max_ulp_exp, double* max_abs_log) {
    if (!ctx || n < 1 || !max_ulp_exp || !max_abs_log) return KORG_EINVAL;
    KCUDA(cudaSetDevice(ctx->device));
    KCHECK(ensure(ctx, ctx->counters, 4 * sizeof(unsigned long long)));
    unsigned long long* c = static_cast<unsigned long long*>(ctx->counters.p);
    KCUDA(cudaMemsetAsync(c, 0, 2 * sizeof(unsigned long long), ctx->stream));
    math_selftest_kernel<<<608, 256, 0, ctx->stream>>>(static_cast<MathTables*>(ctx->math.p), n, c);
    KCUDA(cudaGetLastError());
    unsigned long long h[2];
    KCUDA(cudaMemcpyAsync(h, c, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaStreamSynchronize(ctx->stream));
    ctx->stats_pending = false;
    memcpy(max_ulp_exp, &h[0], 8);
    memcpy(max_abs_log, &h[1], 8);
    return KORG_OK;
}

// ====================================================================== pipe-throughput probe
namespace {
// Independent FMA chains (8 per thread) to measure the sustained FP32 / FP64 FMA rate that
// bounds the line-profile and transfer kernels; the result is the roofline denominator.
template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T* out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = T(threadIdx.x + k) * T(1e-3);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = x[k] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k];
    if (s == T(12345.678)) out[0] = s;  // keeps the chains live
}
}  // namespace

extern "C" KORG_API int korg_probe_flops(korg_ctx* ctx, int fp64, double* tflops) {
    if (!ctx || !tflops) return KORG_EINVAL;
    KCUDA(cudaSetDevice(ctx->device));
    int sms = 0;
    KCUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    KCHECK(ensure(ctx, ctx->counters, 4 * sizeof(unsigned long long)));
    const int blocks = sms * 8, threads = 256;
    const int iters = fp64 ? 256 : 16384;
    cudaStream_t s = ctx->stream;
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        KCUDA(cudaEventRecord(ctx->ev[6], s));
        if (fp64)
            fma_probe_kernel<double><<<blocks, threads, 0, s>>>((double*)ctx->counters.p, iters, 0.999999, 1e-7);
        else
            fma_probe_kernel<float><<<blocks, threads, 0, s>>>((float*)ctx->counters.p, iters, 0.999999f, 1e-7f);
        KCUDA(cudaGetLastError());
        KCUDA(cudaEventRecord(ctx->ev[7], s));
        KCUDA(cudaEventSynchronize(ctx->ev[7]));
        float ms = 0;
        KCUDA(cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]));
        if (rep > 0) best = std::min(best, ms);
    }
    const double flops = 2.0 * 8.0 * double(iters) * blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return KORG_OK;
}

// ====================================================================== allocation-free entry point
// Some callers cannot allocate device memory: code running inside a memory pool or arena that
// the caller owns, a process whose allocator is locked down after start-up, or a caller in the
// middle of stream capture.  korg_line_absorption_noalloc serves them: it runs the same
// line-opacity kernels as korg_line_absorption_dev but keeps all of its scratch (line constants,
// windows, candidate lists, counters, math tables) in one file-scope device array of fixed
// size, so it never calls cudaMalloc, cudaFree or any allocating library routine.
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(64) << 20;  // KORG_NOALLOC_SCRATCH_BYTES in the header
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mutex;
// Device address of the array per CUDA context, keyed by the driver's process-unique context
// id: a device reset (or another driver-API context on the same device) gets a new id, and so
// a fresh lookup and a fresh copy of the math tables, instead of a stale address.
std::map<unsigned long long, unsigned char*> g_noalloc_ptr;
PFN_cuCtxGetCurrent_v4000 g_cu_ctx_get_current = nullptr;
PFN_cuCtxGetId_v12000 g_cu_ctx_get_id = nullptr;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Id of the current context (made current by the runtime if no context is current yet).
int noalloc_context_id(unsigned long long* id) {
    if (!g_cu_ctx_get_current || !g_cu_ctx_get_id) {
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", reinterpret_cast<void**>(&g_cu_ctx_get_current),
                                             12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", reinterpret_cast<void**>(&g_cu_ctx_get_id), 12000,
                                             cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess) {
            g_cu_ctx_get_current = nullptr;
            return KORG_ECUDA;
        }
    }
    CUcontext c = nullptr;
    if (g_cu_ctx_get_current(&c) != CUDA_SUCCESS) return KORG_ECUDA;
    if (!c) {  // no context yet: the runtime makes the current device's primary context current
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) return KORG_ECUDA;
        if (g_cu_ctx_get_current(&c) != CUDA_SUCCESS || !c) return KORG_ECUDA;
    }
    return g_cu_ctx_get_id(c, id) == CUDA_SUCCESS ? KORG_OK : KORG_ECUDA;
}

// Device address of the scratch array in the current context; the first call in a context
// looks it up and writes the math tables into it (a synchronous copy, hence before any capture).
int noalloc_setup(unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    unsigned long long id = 0;
    const int rc = noalloc_context_id(&id);
    if (rc != KORG_OK) return rc;
    auto it = g_noalloc_ptr.find(id);
    if (it == g_noalloc_ptr.end()) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return KORG_ECUDA;
        MathTables t;
        fill_math_tables(t);
        if (cudaMemcpy(p, &t, sizeof t, cudaMemcpyHostToDevice) != cudaSuccess) return KORG_ECUDA;
        it = g_noalloc_ptr.emplace(id, static_cast<unsigned char*>(p)).first;
    }
    *out = it->second;
    return KORG_OK;
}

// The context's default tile shape and the same kernel instances as korg_line_absorption_dev,
// so results are bitwise equal.  (No context: the tile kernel is launched directly.)
int noalloc_tiles(const TileArgs& ta, int G, int kmax, bool mixed, cudaStream_t s) {
    TileGeom g;
    if (!tile_geom(mixed, ta.Lp, G, default_tile(mixed), &g)) return KORG_EINVAL;
    TileArgs t = ta;
    t.stage = g.stage;
    t.region = g.region;
    t.split = g.split;
    t.G = G;
    const dim3 grid(unsigned((ta.nwl + g.tw - 1) / g.tw), unsigned(G));
    auto go = [&](auto kern) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(g.smem)) != cudaSuccess)
            return KORG_ECUDA;
        kern<<<grid, g.threads, g.smem, s>>>(t);
        return cudaGetLastError() == cudaSuccess ? KORG_OK : KORG_ECUDA;
    };
    if (mixed) {
        if (kmax == 14) return go(line_tile_kernel<true, 14, 256, 3>);
        if (kmax == 16) return go(line_tile_kernel<true, 16, 256, 2>);
        return go(line_tile_kernel<true, 32, 256, 2>);
    }
    if (kmax == 14) return go(line_tile_kernel<false, 14, 256, 2>);  // TILE_TW threads, one group
    if (kmax == 16) return go(line_tile_kernel<false, 16, 512, 1>);
    return go(line_tile_kernel<false, 32, 512, 1>);
}

}  // namespace

extern "C" KORG_API int korg_line_absorption_noalloc(double* alpha, const double* wls, int64_t nwl,
                                                    const korg_lines* lines, const korg_layers* layers,
                                                    const korg_cntm* cntm, double cutoff, int precision,
                                                    void* stream) {
    if (!alpha || !wls || nwl < 1 || !lines || !layers || !cntm || cntm->nk < 1 || lines->n < 0) return KORG_EINVAL;
    if (precision != KORG_FP64 && precision != KORG_MIXED) return KORG_EINVAL;
    if (lines->n == 0) return KORG_OK;  // src/line_absorption.jl:35-37: alpha untouched
    const bool mixed = precision == KORG_MIXED;
    const int L = layers->L;
    int kmax = 0;
    const int G = layer_groups(L, &kmax);
    if (L < 1 || G < 0 || lines->n > INT32_MAX || nwl > INT32_MAX - 1) return KORG_EINVAL;
    const int64_t n = lines->n;
    const int Lp = G * kmax;
    const int nblk = int((n + PART_CHUNK - 1) / PART_CHUNK);
    // scratch layout (every piece 256-byte aligned)
    size_t off = 0;
    const size_t o_math = off; off += align256(sizeof(MathTables));
    const size_t o_ctr = off; off += align256(4 * sizeof(unsigned long long));
    const size_t o_lc = off; off += align256(sizeof(LayerConst) * L);
    const size_t o_par = off; off += align256((mixed ? 2 * sizeof(float4) : sizeof(P64)) * size_t(n) * Lp);
    const size_t o_xfar = off; off += align256(sizeof(float) * size_t(n) * G * (mixed ? 2 : 1));
    const size_t o_am = off; off += align256(sizeof(uint32_t) * size_t(n));
    const size_t o_lb = off; off += align256(sizeof(int32_t) * size_t(n));
    const size_t o_ub = off; off += align256(sizeof(int32_t) * size_t(n));
    const size_t o_ci = off; off += align256(sizeof(int32_t) * size_t(n));
    const size_t o_ti = off; off += align256(sizeof(int32_t) * size_t(n));
    const size_t o_tc = off; off += align256(sizeof(int32_t) * size_t(n));
    const size_t o_meta = off; off += align256(sizeof(int32_t) * (NTIER * size_t(nblk) + NTIER + 2));
    if (off > NOALLOC_SCRATCH_BYTES) return KORG_ETOOBIG;
    unsigned char* sp = nullptr;
    int rc = noalloc_setup(&sp);
    if (rc != KORG_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    auto* ctr = reinterpret_cast<unsigned long long*>(sp + o_ctr);
    int32_t* meta = reinterpret_cast<int32_t*>(sp + o_meta);  // [start: NTIER+1][unsorted][block counts]
    // the array keeps the previous call's contents: zero the counters and the sortedness flag
    if (cudaMemsetAsync(ctr, 0, 4 * sizeof(unsigned long long), s) != cudaSuccess) return KORG_ECUDA;
    if (cudaMemsetAsync(meta + NTIER + 1, 0, sizeof(int32_t), s) != cudaSuccess) return KORG_ECUDA;
    const LinesDev ln = lines_dev(lines);
    const LayersDev lay = layers_dev(layers);
    const CntmDev cn{cntm->nk, cntm->knots, cntm->vals};
    auto* lc = reinterpret_cast<LayerConst*>(sp + o_lc);
    auto* math = reinterpret_cast<MathTables*>(sp + o_math);
    layer_const_kernel<<<(L + 127) / 128, 128, 0, s>>>(lay, lc);
    PrepOut po{sp + o_par, reinterpret_cast<int32_t*>(sp + o_lb), reinterpret_cast<int32_t*>(sp + o_ub),
               reinterpret_cast<int32_t*>(sp + o_ci), reinterpret_cast<float*>(sp + o_xfar),
               reinterpret_cast<uint32_t*>(sp + o_am), Lp, kmax, G, ctr, ctr + 1,
               mixed ? reinterpret_cast<float4*>(sp + o_par) + size_t(n) * Lp : nullptr,
               mixed ? reinterpret_cast<float*>(sp + o_xfar) + size_t(n) * G : nullptr};
    const size_t prep_smem = size_t(256 / 32) * Lp * (sizeof(float) + sizeof(int));
    const unsigned pblocks = unsigned((n * 32 + 255) / 256);
    if (mixed)
        line_prep_mixed_kernel<<<prep_mixed_blocks(n), 32 * PREP_WARPS, prep_mixed_smem(Lp), s>>>(
            ln, lay, lc, cn, wls, nwl, cutoff, po, math);
    else
        line_prep64_kernel<<<pblocks, 256, prep_smem, s>>>(ln, lay, lc, cn, wls, nwl, cutoff, po, math);
    TierLists tl{reinterpret_cast<int32_t*>(sp + o_ti), reinterpret_cast<int32_t*>(sp + o_tc), meta, meta + NTIER + 1};
    int32_t* bcnt = meta + NTIER + 2;
    tier_count_kernel<<<nblk, PART_THREADS, 0, s>>>(po.lb, po.ub, po.ci, n, bcnt, tl.unsorted);
    tier_scatter_kernel<<<nblk, PART_THREADS, 0, s>>>(po.lb, po.ub, po.ci, n, bcnt, nblk, tl);
    if (cudaGetLastError() != cudaSuccess) return KORG_ECUDA;
    TileArgs ta{};
    ta.alpha = alpha;
    ta.wls = wls;
    ta.nwl = nwl;
    ta.L = L;
    ta.Lp = Lp;
    ta.xfar = po.xfar;
    ta.amask = po.amask;
    ta.n = n;
    ta.wl = ln.wl;
    ta.params = po.params;
    ta.params_w = po.params_w;
    ta.xcub = po.xcub;
    ta.lb = po.lb;
    ta.ub = po.ub;
    ta.tier_idx = tl.idx;
    ta.tier_ci = tl.ci;
    ta.tier_start = tl.start;
    ta.unsorted = tl.unsorted;
    return noalloc_tiles(ta, G, kmax, mixed, s);
}
