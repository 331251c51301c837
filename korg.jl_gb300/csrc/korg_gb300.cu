// korg_gb300.cu -- C ABI, context, scratch arena and launch orchestration of the GB300
// synthesis hot path.  Kernels live in lines.cuh, hydrogen.cuh and rt.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/korg_gb300.h"
#include "hydrogen.cuh"
#include "lines.cuh"
#include "physics.cuh"
#include "rt.cuh"

using namespace korg;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
};

constexpr int NEV = 8;

}  // namespace

struct korg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;  // used by the host-pointer calls
    std::string err;
    // scratch arena: grown on demand, never shrunk, freed by korg_destroy
    DevBuf lc, params, xfar, amask, lb, ub, ci, tier_idx, tier_ci, tier_meta, counters;
    DevBuf hrec, hQ, hQ32, hulb, huub;
    DevBuf stage_dev, aref, alpha, flux, cntm, math;
    void* stage_host = nullptr;
    size_t stage_host_cap = 0;
    // Stehle tables
    bool have_stark = false;
    StarkDev stark{};
    int n_max = 0;
    std::vector<void*> stark_allocs;
    // statistics
    bool timing = false;
    cudaEvent_t ev[NEV] = {};
    korg_stats stats{};
    bool stats_pending = false;
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

int ensure(korg_ctx* ctx, DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return KORG_OK;
    if (b.p) {
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
    if (ctx->timing) cudaEventRecord(ctx->ev[i], s);
}

// Layers per thread (K) and layer groups per CTA (G = ceil(L/K) <= 8); layers are padded to
// G*K.  56-layer (MARCS) atmospheres split exactly into 4 x 14.
// Tables of the table-driven FP64 exp / log (physics.cuh), in extended precision on the host.
void fill_math_tables(MathTables& t) {
    for (int j = 0; j < 64; j++) {
        t.exp2j[j] = double(exp2l((long double)j / 64.0L));
        const long double c = 1.0L + ((long double)j + 0.5L) / 64.0L;
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
constexpr int TILE_TW = 64;  // wavelengths per CTA of the line tile kernel

template <bool MIXED, int KMAX, int MAXT, int MINB>
int launch_tile(korg_ctx* ctx, TileArgs ta, int G, cudaStream_t s) {
    using P = typename ParamT<MIXED>::type;
    const int Lp = ta.Lp;
    const int B = MIXED ? STAGE_LINES : STAGE_LINES / 2;
    ta.stage = B;
    ta.G = G;
    const int TW = TILE_TW;
    const int threads = TW * G;
    size_t region = size_t(B) * Lp * sizeof(P);
    region = std::max(region, (size_t(TW) * (Lp + 1) * sizeof(double) + 1) / 2);
    region = (region + 15) & ~size_t(15);
    ta.region = int(region);
    const size_t smem = 2 * region + size_t(threads) * sizeof(LineStage);
    auto kern = line_tile_kernel<MIXED, KMAX, MAXT, MINB>;
    KCUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const int64_t tiles = (ta.nwl + TW - 1) / TW;
    kern<<<dim3(unsigned(tiles)), threads, smem, s>>>(ta);
    KCUDA(cudaGetLastError());
    return KORG_OK;
}

template <bool MIXED>
int dispatch_tile(korg_ctx* ctx, const TileArgs& ta, int G, int kmax, cudaStream_t s) {
    if (kmax == 14 && G <= 4) return launch_tile<MIXED, 14, 256, MIXED ? 3 : 2>(ctx, ta, G, s);
    if (kmax == 14) return launch_tile<MIXED, 14, 512, 1>(ctx, ta, G, s);
    if (kmax == 16) return launch_tile<MIXED, 16, 512, 1>(ctx, ta, G, s);
    return launch_tile<MIXED, 32, 512, 1>(ctx, ta, G, s);
}

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
    const size_t psz = mixed ? sizeof(float4) : sizeof(P64);
    KCHECK(ensure(ctx, ctx->lc, sizeof(LayerConst) * L));
    KCHECK(ensure(ctx, ctx->params, psz * size_t(ln.n) * Lp));
    KCHECK(ensure(ctx, ctx->xfar, sizeof(float) * size_t(ln.n) * G));
    KCHECK(ensure(ctx, ctx->amask, sizeof(uint32_t) * ln.n));
    KCHECK(ensure(ctx, ctx->lb, sizeof(int32_t) * ln.n));
    KCHECK(ensure(ctx, ctx->ub, sizeof(int32_t) * ln.n));
    KCHECK(ensure(ctx, ctx->ci, sizeof(int32_t) * ln.n));
    KCHECK(ensure(ctx, ctx->tier_idx, sizeof(int32_t) * ln.n));
    KCHECK(ensure(ctx, ctx->tier_ci, sizeof(int32_t) * ln.n));
    const int nblk = int((ln.n + PART_CHUNK - 1) / PART_CHUNK);
    KCHECK(ensure(ctx, ctx->tier_meta, sizeof(int32_t) * (NTIER * size_t(nblk) + NTIER + 2)));
    auto* ctr = static_cast<unsigned long long*>(ctx->counters.p);
    layer_const_kernel<<<(L + 127) / 128, 128, 0, s>>>(lay, static_cast<LayerConst*>(ctx->lc.p));
    PrepOut po{ctx->params.p, static_cast<int32_t*>(ctx->lb.p), static_cast<int32_t*>(ctx->ub.p),
               static_cast<int32_t*>(ctx->ci.p), static_cast<float*>(ctx->xfar.p), static_cast<uint32_t*>(ctx->amask.p), Lp, kmax, G, ctr, ctr + 1};
    const size_t prep_smem = size_t(256 / 32) * Lp * (sizeof(float) + sizeof(int));
    const int64_t pthreads = ln.n * 32;
    const unsigned pblocks = unsigned((pthreads + 255) / 256);
    if (mixed)
        line_prep_mixed_kernel<<<pblocks, 256, prep_smem, s>>>(ln, lay, static_cast<LayerConst*>(ctx->lc.p), cn, wls, nwl, cutoff, po,
                                                       static_cast<MathTables*>(ctx->math.p));
    else
        line_prep64_kernel<<<pblocks, 256, prep_smem, s>>>(ln, lay, static_cast<LayerConst*>(ctx->lc.p), cn, wls, nwl, cutoff, po,
                                                   static_cast<MathTables*>(ctx->math.p));
    KCUDA(cudaGetLastError());
    int32_t* meta = static_cast<int32_t*>(ctx->tier_meta.p);  // [start: NTIER+1][unsorted][block counts]
    TierLists tl{static_cast<int32_t*>(ctx->tier_idx.p), static_cast<int32_t*>(ctx->tier_ci.p), meta, meta + NTIER + 1};
    int32_t* bcnt = meta + NTIER + 2;
    KCUDA(cudaMemsetAsync(tl.unsorted, 0, sizeof(int32_t), s));
    tier_count_kernel<<<nblk, PART_THREADS, 0, s>>>(po.lb, po.ub, po.ci, ln.n, bcnt, tl.unsorted);
    tier_scatter_kernel<<<nblk, PART_THREADS, 0, s>>>(po.lb, po.ub, po.ci, ln.n, bcnt, nblk, tl);
    KCUDA(cudaGetLastError());
    record(ctx, 2, s);
    TileArgs ta{};
    ta.alpha = alpha;
    ta.wls = wls;
    ta.nwl = nwl;
    ta.L = L;
    ta.Lp = Lp;
    ta.xfar = po.xfar;
    ta.amask = po.amask;
    ta.n = ln.n;
    ta.wl = ln.wl;
    ta.params = ctx->params.p;
    ta.lb = po.lb;
    ta.ub = po.ub;
    ta.tier_idx = tl.idx;
    ta.tier_ci = tl.ci;
    ta.tier_start = tl.start;
    ta.unsorted = tl.unsorted;
    int rc;
    if (mixed)
        rc = dispatch_tile<true>(ctx, ta, G, kmax, s);
    else
        rc = dispatch_tile<false>(ctx, ta, G, kmax, s);
    ctx->stats_pending = true;
    return rc;
}

// ------------------------------------------------------------------ hydrogen lines
int run_hydrogen(korg_ctx* ctx, double* alpha, const double* wls, int64_t nwl, const HLayers& hl, double window,
                 int use_MHD, bool mixed, cudaStream_t s) {
    if (!ctx->have_stark) return set_err(ctx, KORG_ENOTABLES, "korg_set_stark_tables() has not been called");
    const int L = hl.L;
    // the hydrogen tile kernel interleaves layers: thread group g owns layers g, g+G, ...
    int kmax = 16, G = (L + 15) / 16;
    if (G > 8) { kmax = 32; G = (L + 31) / 32; }
    if (G > 8) return set_err(ctx, KORG_EINVAL, "at most 256 layers are supported (got %d)", L);
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
    // :265-283 reference-wavelength line opacity on a copy of the continuum alpha_ref
    KCUDA(cudaMemcpyAsync(aref, in->alpha_ref_cntm, sizeof(double) * L, cudaMemcpyDeviceToDevice, s));
    const CntmDev cref{1, nullptr, in->alpha_ref_cntm};
    record(ctx, 1, s);
    KCHECK(run_line_absorption(ctx, aref, ref_wl_dev, 1, ln5, lay, cref, in->cutoff_threshold, mixed, s));
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
    for (size_t i = 0; i < st.items.size(); i++)
        if (st.items[i].first && st.items[i].second) memcpy(h + st.offs[i], st.items[i].first, st.items[i].second);
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
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    for (int i = 0; e == cudaSuccess && i < NEV; i++) e = cudaEventCreate(&ctx->ev[i]);
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
    DevBuf* bufs[] = {&ctx->lc, &ctx->params, &ctx->xfar, &ctx->amask, &ctx->lb, &ctx->ub, &ctx->ci, &ctx->tier_idx, &ctx->tier_ci, &ctx->tier_meta, &ctx->counters,
                      &ctx->hrec, &ctx->hQ, &ctx->hQ32, &ctx->hulb, &ctx->huub, &ctx->stage_dev, &ctx->aref,
                      &ctx->alpha, &ctx->flux, &ctx->cntm, &ctx->math};
    for (DevBuf* b : bufs)
        if (b->p) cudaFree(b->p);
    for (void* p : ctx->stark_allocs) cudaFree(p);
    if (ctx->stage_host) cudaFreeHost(ctx->stage_host);
    for (int i = 0; i < NEV; i++)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
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
        cudaGetLastError();
    }
    *out = ctx->stats;
    return KORG_OK;
}

KORG_API int korg_set_stark_tables(korg_ctx* ctx, const korg_stark_tables* t) {
    if (!ctx || !t || t->ntrans < 1) return KORG_EINVAL;
    KCUDA(cudaSetDevice(ctx->device));
    for (void* p : ctx->stark_allocs) cudaFree(p);
    ctx->stark_allocs.clear();
    ctx->have_stark = false;
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

KORG_API int korg_line_absorption_dev(korg_ctx* ctx, double* alpha, const double* wls, int64_t nwl,
                                      const korg_lines* lines, const korg_layers* layers, const korg_cntm* cntm,
                                      double cutoff, int precision, void* stream) {
    if (!ctx || !alpha || !wls || nwl < 1 || !lines || !layers || !cntm || cntm->nk < 1)
        return ctx ? set_err(ctx, KORG_EINVAL, "bad arguments") : KORG_EINVAL;
    KCUDA(cudaSetDevice(ctx->device));
    KCHECK(reset_counters(ctx, static_cast<cudaStream_t>(stream)));
    return run_line_absorption(ctx, alpha, wls, nwl, lines_dev(lines), layers_dev(layers),
                               CntmDev{cntm->nk, cntm->knots, cntm->vals}, cutoff, precision == KORG_MIXED,
                               static_cast<cudaStream_t>(stream));
}

KORG_API int korg_line_absorption(korg_ctx* ctx, double* alpha, const double* wls, int64_t nwl,
                                  const korg_lines* lines, const korg_layers* layers, const korg_cntm* cntm,
                                  double cutoff, int precision, int64_t* n_evals) {
    if (!ctx) return KORG_EINVAL;
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
    KCUDA(cudaSetDevice(ctx->device));
    const HLayers hl{L, T, ne, nH_I, nHe_I, UH_I, xi};
    return run_hydrogen(ctx, alpha, wls, nwl, hl, window, use_MHD, precision == KORG_MIXED,
                        static_cast<cudaStream_t>(stream));
}

KORG_API int korg_hydrogen_line_absorption(korg_ctx* ctx, double* alphas, const double* wls, int64_t nwl,
                                           double T, double ne, double nH_I, double nHe_I, double UH_I, double xi,
                                           double window, int use_MHD, int precision) {
    if (!ctx) return KORG_EINVAL;
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

KORG_API int korg_synthesize_dev(korg_ctx* ctx, const korg_synth_inputs* in, const korg_lines* lines,
                                 const korg_lines* lines5, const double* wls, int64_t nwl, int precision,
                                 double* flux, double* cntm, double* alpha_out, void* stream) {
    if (!ctx || !in || !lines || !lines5 || !wls || nwl < 1 || !flux || !cntm)
        return ctx ? set_err(ctx, KORG_EINVAL, "bad arguments") : KORG_EINVAL;
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
    KCUDA(cudaMemcpyAsync(flux, b + o_fl, 8 * size_t(nwl), cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaMemcpyAsync(cntm, b + o_cn, 8 * size_t(nwl), cudaMemcpyDeviceToHost, ctx->stream));
    if (alpha_out)
        KCUDA(cudaMemcpyAsync(alpha_out, d_alpha, 8 * size_t(L) * nwl, cudaMemcpyDeviceToHost, ctx->stream));
    if (alpha_ref_out) KCUDA(cudaMemcpyAsync(alpha_ref_out, aref, 8 * size_t(L), cudaMemcpyDeviceToHost, ctx->stream));
    KCUDA(cudaStreamSynchronize(ctx->stream));
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

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
unsigned char* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};  // device address of the array, per device

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Device address of the scratch array for the current device; the first call on a device looks
// it up and writes the math tables into it (a synchronous copy, hence before any capture).
int noalloc_setup(int dev, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return KORG_EINVAL;
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return KORG_ECUDA;
        MathTables t;
        fill_math_tables(t);
        if (cudaMemcpy(p, &t, sizeof t, cudaMemcpyHostToDevice) != cudaSuccess) return KORG_ECUDA;
        g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return KORG_OK;
}

template <bool MIXED, int KMAX, int MAXT, int MINB>
int noalloc_launch_tile(TileArgs ta, int G, cudaStream_t s) {
    using P = typename ParamT<MIXED>::type;
    const int Lp = ta.Lp;
    const int B = MIXED ? STAGE_LINES : STAGE_LINES / 2;
    ta.stage = B;
    ta.G = G;
    const int TW = TILE_TW, threads = TW * G;
    size_t region = size_t(B) * Lp * sizeof(P);
    region = std::max(region, (size_t(TW) * (Lp + 1) * sizeof(double) + 1) / 2);
    region = (region + 15) & ~size_t(15);
    ta.region = int(region);
    const size_t smem = 2 * region + size_t(threads) * sizeof(LineStage);
    auto kern = line_tile_kernel<MIXED, KMAX, MAXT, MINB>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
        return KORG_ECUDA;
    kern<<<dim3(unsigned((ta.nwl + TW - 1) / TW)), threads, smem, s>>>(ta);
    return cudaGetLastError() == cudaSuccess ? KORG_OK : KORG_ECUDA;
}

template <bool MIXED>
int noalloc_dispatch_tile(const TileArgs& ta, int G, int kmax, cudaStream_t s) {
    if (kmax == 14 && G <= 4) return noalloc_launch_tile<MIXED, 14, 256, MIXED ? 3 : 2>(ta, G, s);
    if (kmax == 14) return noalloc_launch_tile<MIXED, 14, 512, 1>(ta, G, s);
    if (kmax == 16) return noalloc_launch_tile<MIXED, 16, 512, 1>(ta, G, s);
    return noalloc_launch_tile<MIXED, 32, 512, 1>(ta, G, s);
}

}  // namespace

extern "C" KORG_API int korg_line_absorption_noalloc(double* alpha, const double* wls, int64_t nwl,
                                                    const korg_lines* lines, const korg_layers* layers,
                                                    const korg_cntm* cntm, double cutoff, int precision,
                                                    void* stream) {
    if (!alpha || !wls || nwl < 1 || !lines || !layers || !cntm || cntm->nk < 1 || lines->n < 0) return KORG_EINVAL;
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
    const size_t o_par = off; off += align256((mixed ? sizeof(float4) : sizeof(P64)) * size_t(n) * Lp);
    const size_t o_xfar = off; off += align256(sizeof(float) * size_t(n) * G);
    const size_t o_am = off; off += align256(sizeof(uint32_t) * size_t(n));
    const size_t o_lb = off; off += align256(sizeof(int32_t) * size_t(n));
    const size_t o_ub = off; off += align256(sizeof(int32_t) * size_t(n));
    const size_t o_ci = off; off += align256(sizeof(int32_t) * size_t(n));
    const size_t o_ti = off; off += align256(sizeof(int32_t) * size_t(n));
    const size_t o_tc = off; off += align256(sizeof(int32_t) * size_t(n));
    const size_t o_meta = off; off += align256(sizeof(int32_t) * (NTIER * size_t(nblk) + NTIER + 2));
    if (off > NOALLOC_SCRATCH_BYTES) return KORG_ETOOBIG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return KORG_ECUDA;
    unsigned char* sp = nullptr;
    int rc = noalloc_setup(dev, &sp);
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
               reinterpret_cast<uint32_t*>(sp + o_am), Lp, kmax, G, ctr, ctr + 1};
    const size_t prep_smem = size_t(256 / 32) * Lp * (sizeof(float) + sizeof(int));
    const unsigned pblocks = unsigned((n * 32 + 255) / 256);
    if (mixed)
        line_prep_mixed_kernel<<<pblocks, 256, prep_smem, s>>>(ln, lay, lc, cn, wls, nwl, cutoff, po, math);
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
    ta.lb = po.lb;
    ta.ub = po.ub;
    ta.tier_idx = tl.idx;
    ta.tier_ci = tl.ci;
    ta.tier_start = tl.start;
    ta.unsorted = tl.unsorted;
    return mixed ? noalloc_dispatch_tile<true>(ta, G, kmax, s) : noalloc_dispatch_tile<false>(ta, G, kmax, s);
}
