// lines.cuh -- line opacity: per-(line, layer) prologue, width-tier candidate lists and the
// wavelength-tile accumulation kernels.  Restates line_absorption! (src/line_absorption.jl:33-129).
//
// Work decomposition
//   prep:  per-(line, layer) constants, the continuum-cutoff window (line_absorption.jl:86-119)
//          and, per group of K layers, the distances from the line centre beyond which every
//          layer of the group is in a closed-form wing branch of the Hjerting approximation and
//          (mixed) in its cubic regime, where the branch is a cubic in t' = cref / dl^2.
//   tiers: line indices partitioned by window half-width, each tier ordered by centre, so a
//          wavelength tile finds its candidate lines with two binary searches per tier.
//   tile:  one CTA per tile of wavelengths x one layer group (or, FP64, all groups).  Each thread
//          owns one (FP64) or two (mixed) wavelengths and the K consecutive layers of its group;
//          alpha accumulates in registers (FP64, or FP32 batch sums with Kahan compensation).
//          Lines are visited in list order (deterministic, no atomics on alpha); each chunk of
//          candidates is compacted with warp ballots, and the constants of each batch of lines
//          are copied to shared memory with cp.async, double buffered.
#pragma once
#include "physics.cuh"

namespace korg {

constexpr int STAGE_LINES = 32;  // lines staged in shared memory per batch
constexpr int MAX_GROUPS = 8;    // layer groups per CTA

// FP64 profile constants of one (line, layer): c = 2 sigma^2 (so 1/v^2 = c / x^2), w as in the
// mixed form, inv_s = 1/(sigma sqrt2), a = gamma inv_s, scale = amp inv_s / sqrt(pi)
struct alignas(16) P64 {
    double c, w, inv_s, a, scale, pad;
};

struct LinesDev {
    int64_t n;
    const double *wl, *log_gf, *E_lower, *gamma_rad, *gamma_stark, *vdW1, *vdW2, *mass;
    const int32_t *is_mol, *species;
};
struct LayersDev {
    int32_t L, S;
    const double *T, *ne, *n_eff_vdW, *xi, *n_div_U;
};
struct CntmDev {
    int64_t nk;
    const double *knots, *vals;
};

// Per-layer constants shared by all lines (line_absorption.jl:39 and the temperature scalings
// of :195 and :210), computed once per call.
struct LayerConst {
    double beta;    // 1/(k T)
    double stark6;  // (T/10^4)^(1/6)
    double vdw3;    // (T/10^4)^0.3
    // FP32 copies for the mixed-precision prologue: T, xi, n_e, n_eff_vdW, stark6, vdw3
    float T32, xi32, ne32, nv32, stark6_32, vdw3_32;
};

__global__ void layer_const_kernel(LayersDev lay, LayerConst* out) {
    int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= lay.L) return;
    double T = lay.T[l];
    LayerConst c;
    c.beta = 1 / (KBOLTZ_EV * T);
    c.stark6 = pow(T / 10000.0, 1.0 / 6.0);
    c.vdw3 = pow(T / 10000.0, 0.3);
    c.T32 = float(T);
    c.xi32 = float(lay.xi[l]);
    c.ne32 = float(lay.ne[l]);
    c.nv32 = float(lay.n_eff_vdW[l]);
    c.stark6_32 = float(c.stark6);
    c.vdw3_32 = float(c.vdw3);
    out[l] = c;
}

struct PrepOut {
    void* params;            // [n][Lp] P64 (FP64) or float4 (mixed); layers L..Lp-1 are zero padding
    int32_t* lb;             // [n]
    int32_t* ub;             // [n]
    int32_t* ci;             // [n] index of the first wavelength >= the line centre
    float* xfar;             // [n][G] |wl - wl0| beyond which every layer of group g is in a wing
                             //        branch: v >= 5 (a <= 0.2) or a + v >= 3.2 / a > 1.4 (a > 0.2)
    uint32_t* amask;         // [n] bit g: every layer of group g has a <= 0.2
    int32_t Lp, K, G;
    unsigned long long* evals;   // running totals: evaluations, lines in window
    unsigned long long* nlines;
    float4* params_w;        // [n][Lp] mixed, or null: wing cubic {A1, A2, A3, 0} in t' = cref / dl^2
                             //   (cref = 2 sigma^2 of layer 0), valid beyond the layer's cubic boundary
    float* xcub;             // [n][G] mixed, or null: |wl - wl0| beyond which every layer of group g
                             //   is given by its wing cubic to FP32 rounding
};

// Per-line quantities shared by every layer (line_absorption.jl:83,101,105,219).
struct LineConst {
    double wl, m, El, E_upper, strength, wl2c, abo_pre, v1, v2, gstark, grad;
    bool mol;
    int sp;
};

__device__ __forceinline__ LineConst line_const(const LinesDev& ln, int64_t i) {
    LineConst q;
    q.wl = ln.wl[i];
    q.m = ln.mass[i];
    q.El = ln.E_lower[i];
    q.mol = ln.is_mol[i] != 0;
    q.v1 = ln.vdW1[i];
    q.v2 = ln.vdW2[i];
    q.gstark = ln.gamma_stark[i];
    q.grad = ln.gamma_rad[i];
    q.sp = ln.species[i];
    q.E_upper = q.El + C_CGS * HPLANCK_EV / q.wl;
    q.strength = pow(10.0, ln.log_gf[i]) * sigma_line(q.wl);
    q.wl2c = (q.wl * q.wl) / (C_CGS * (4 * PI));
    q.abo_pre = (!q.mol && q.v2 != -1) ? 2 * pow(4 / PI, q.v2 / 2) * tgamma((4 - q.v2) / 2) * 1e6 * q.v1 : 0.0;
    return q;
}

// One (line, layer) in FP64 exactly as line_absorption.jl:86-112 computes it.
struct LineLayer64 {
    double sigma, gamma, amp, dw, lw;
};

__device__ __forceinline__ LineLayer64 line_layer64(const LineConst& q, const LayersDev& lay, const LayerConst& c,
                                                    const CntmDev& cn, const KnotPos& kp, double cutoff, int l,
                                                    const MathTables& mt) {
    LineLayer64 r;
    const double T = lay.T[l];
    r.sigma = doppler_width(q.wl, T, q.m, lay.xi[l]);  // :86
    double G = q.grad;                                 // :90-94
    if (!q.mol) {
        G = G + lay.ne[l] * (q.gstark * c.stark6);
        double vdw;
        if (q.v2 == -1) {
            vdw = q.v1 * c.vdw3;
        } else {
            const double invmu = 1 / (1.008 * AMU_CGS) + 1 / q.m;
            const double vbar = sqrt(8 * KBOLTZ_CGS * T / PI * invmu);
            vdw = q.abo_pre * pow(vbar / 1e6, 1 - q.v2);
        }
        G = G + lay.n_eff_vdW[l] * vdw;
    }
    r.gamma = G * q.wl2c;                                                       // :99
    const double levels = fexp64(-c.beta * q.El, mt) - fexp64(-c.beta * q.E_upper, mt);  // :101-102
    r.amp = q.strength * levels * lay.n_div_U[int64_t(q.sp) * lay.L + l];                // :105-106
    const double acntm = knot_eval(cn.vals + int64_t(l) * cn.nk, cn.nk, kp);    // :108
    const double rho = acntm * cutoff / r.amp;
    r.dw = (rho > 1 / (SQRT_2PI * r.sigma)) ? 0.0                              // :109-112 (:140-145)
                                            : r.sigma * sqrt(-2 * flog64(SQRT_2PI * r.sigma * rho, mt));
    r.lw = inverse_lorentz_density(rho, r.gamma);
    return r;
}

__device__ __forceinline__ void store_window(const PrepOut& out, int64_t i, double lwin, double dwin, double wl,
                                             const double* wls, int64_t nwl, int L) {
    const double window = sqrt(lwin * lwin + dwin * dwin);   // :113
    const int64_t lb = search_first(wls, nwl, wl - window);  // :114-115
    const int64_t ub = search_last(wls, nwl, wl + window);
    out.lb[i] = int32_t(lb);
    out.ub[i] = int32_t(ub);
    out.ci[i] = int32_t(search_first(wls, nwl, wl));
    if (lb <= ub) {
        atomicAdd(out.evals, (unsigned long long)((ub - lb + 1) * L));
        atomicAdd(out.nlines, 1ull);
    }
}

// Per-(line, group) wing boundaries from per-layer ones held in shared memory: lanes g < G
// reduce their group and write xfar / amask.
__device__ __forceinline__ void group_bounds(const PrepOut& out, int64_t i, const float* s_bnd, const int* s_cls,
                                             int lane) {
    unsigned bits = 0;
    float mx = 0.f;
    int allA = 1;
    if (lane < out.G) {
        for (int k = 0; k < out.K; k++) {
            mx = fmaxf(mx, s_bnd[lane * out.K + k]);
            allA &= s_cls[lane * out.K + k];
        }
        out.xfar[i * out.G + lane] = mx;
    }
    bits = __ballot_sync(0xffffffffu, lane < out.G && allA);
    if (lane == 0) out.amask[i] = bits;
}

// FP64 prologue: one warp per line, lanes over layers.
__global__ void __launch_bounds__(256) line_prep64_kernel(LinesDev ln, LayersDev lay, const LayerConst* lc, CntmDev cn,
                                                          const double* wls, int64_t nwl, double cutoff, PrepOut out,
                                                          const MathTables* math) {
    __shared__ MathTables s_math;
    extern __shared__ float s_dyn[];  // [warps][Lp] boundaries, then [warps][Lp] class flags
    load_math_tables(s_math, math);
    __syncthreads();
    const int64_t i = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    if (i >= ln.n) return;
    const int L = lay.L, Lp = out.Lp;
    float* s_bnd = s_dyn + wib * Lp;
    int* s_cls = reinterpret_cast<int*>(s_dyn + (blockDim.x >> 5) * Lp) + wib * Lp;
    const LineConst q = line_const(ln, i);
    const KnotPos kp = knot_pos(cn.knots, cn.nk, q.wl);
    double dwin = 0.0, lwin = 0.0;
    P64* dst = reinterpret_cast<P64*>(out.params) + i * Lp;
    for (int l = lane; l < Lp; l += 32) {
        if (l >= L) {
            dst[l] = P64{1.0, 0.0, 1.0, 0.0, 0.0, 0.0};
            s_bnd[l] = 0.f;
            s_cls[l] = 1;
            continue;
        }
        const LineLayer64 r = line_layer64(q, lay, lc[l], cn, kp, cutoff, l, s_math);
        dwin = fmax(dwin, r.dw);
        lwin = fmax(lwin, r.lw);
        const double inv_s = 1 / (r.sigma * SQRT_2);  // :246-248
        const double a = r.gamma * inv_s, scale = inv_s / SQRT_PI * r.amp;
        const double c = 1 / (inv_s * inv_s);
        const bool A = a <= 0.2;
        dst[l] = P64{c, A ? a / SQRT_PI * scale : 1 / (r.gamma * r.gamma), inv_s, a, scale, 0.0};
        // v >= 5 (a <= 0.2) or a + v >= 3.2 (0.2 < a <= 1.4) or any v (a > 1.4), v = x inv_s
        s_bnd[l] = float((A ? 5.0 : (a <= 1.4 ? 3.2 - a : 0.0)) / inv_s * 1.0001);
        s_cls[l] = A;
    }
    __syncwarp();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dwin = fmax(dwin, __shfl_xor_sync(0xffffffffu, dwin, o));
        lwin = fmax(lwin, __shfl_xor_sync(0xffffffffu, lwin, o));
    }
    group_bounds(out, i, s_bnd, s_cls, lane);
    if (lane == 0) store_window(out, i, lwin, dwin, q.wl, wls, nwl, L);
}

// FP32 forms of line_absorption.jl:140-161 (used to locate the widest layers)
__device__ __forceinline__ float inverse_gaussian32(float rho, float sigma) {
    if (rho > 1.f / (2.5066282746f * sigma)) return 0.f;
    return sigma * sqrtf(-2.f * __logf(2.5066282746f * sigma * rho));
}
__device__ __forceinline__ float inverse_lorentz32(float rho, float gamma) {
    if (rho > 1.f / (3.14159265f * gamma)) return 0.f;
    return sqrtf(fmaxf(gamma / (3.14159265f * rho) - gamma * gamma, 0.f));
}

__device__ __forceinline__ void argmax_reduce(float& v, int& idx) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
}

// Distance (in units of gamma) beyond which the far-Lorentz branch of voigt_hjerting
// (line_absorption.jl:305-308) equals its cubic series in w = 1/r^2 = gamma^2/dl^2 to FP32
// rounding.  With q = 1/(sqrt2 a) and u = 1/(1 + r^2) the branch is
//   H = sqrt(2/pi) q u (1 + (3 r^2 - 1 + (15 r^4 - 30 r^2 + 2) q^2 u^2) q^2 u^2)
//     = sqrt(2/pi) [q w + (3q^3 - q) w^2 + (q - 10q^3 + 15q^5) w^3 + (-q + 21q^3 - 105q^5) w^4 + ...]
// (u = w - w^2 + w^3 - ...), so the cubic's relative error is about C4 w^3 with
// C4 = |-1 + 21 q^2 - 105 q^4|; w^3 C4 <= 2^-26 gives r >= (2^26 C4)^(1/6).  C4 is clamped at 1
// so that the next term stays negligible near its root (a ~ 2).
__device__ __forceinline__ float far_lorentz_cubic_rmin(float a) {
    const float q2 = 0.5f / (a * a);
    const float C4 = fmaxf(fabsf(fmaf(fmaf(-105.f, q2, 21.f), q2, -1.f)), 1.f);
    return powf(67108864.f * C4, 1.f / 6.f);
}

// Mixed-precision prologue.  sigma, gamma and the profile constants are FP32; the line
// strength (Boltzmann factor, 10^loggf sigma_line, n/U) is FP64 (line_absorption.jl:101-106).
// The window is the FP64 window of the reference rule: FP32 locates the layers with the widest
// Gaussian and Lorentzian windows, and those two layers are re-evaluated in FP64.
// Packed constants: {c = 1/v-scale^2 = 2 sigma^2, a, w, scale} with scale = amp/(sigma sqrt(2 pi))
// and w = a/sqrt(pi)*scale (a <= 0.2, asymptotic wing) or 1/gamma^2 (a > 0.2, far Lorentz).
//
// Each warp handles 32 lines.  The per-line FP64 work (10^loggf, the continuum knot search,
// the exact window at two layers) runs with one lane per line; the per-(line, layer) work runs
// line by line with lanes over layers.  FP64 is 1/64 of the FP32 rate here, so keeping the
// per-line FP64 work lane-parallel is what bounds this kernel.
struct LinePrep32 {
    double El, Eu, strength;   // FP64 line-strength inputs
    float wlc, k_m, wl2c, grad, gstark, v1, abo_pre, vexp, invmu, t32;
    int32_t flags, sp, ki;     // flags: 1 molecule, 2 ABO broadening; ki: continuum knot interval
};
constexpr int PREP_WARPS = 8;

__global__ void __launch_bounds__(32 * PREP_WARPS) line_prep_mixed_kernel(LinesDev ln, LayersDev lay,
                                                                          const LayerConst* lc, CntmDev cn,
                                                                          const double* wls, int64_t nwl,
                                                                          double cutoff, PrepOut out,
                                                                          const MathTables* math) {
    __shared__ MathTables s_math;
    __shared__ LinePrep32 s_line[PREP_WARPS][32];
    extern __shared__ float s_dyn[];  // [warps][Lp] boundaries, [warps][Lp] class flags, [warps][Lp] cubic boundaries
    load_math_tables(s_math, math);
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t base = (int64_t(blockIdx.x) * PREP_WARPS + wib) * 32;
    if (base >= ln.n) return;
    const int nl = int(min(int64_t(32), ln.n - base));
    const int L = lay.L, Lp = out.Lp;
    float* s_bnd = s_dyn + wib * Lp;
    int* s_cls = reinterpret_cast<int*>(s_dyn + PREP_WARPS * Lp) + wib * Lp;
    float* s_cub = s_dyn + 2 * PREP_WARPS * Lp + wib * Lp;
    // phase A: one lane per line
    KnotPos kp_mine{0, 0.0};
    if (lane < nl) {
        const int64_t i = base + lane;
        const LineConst q = line_const(ln, i);
        kp_mine = knot_pos(cn.knots, cn.nk, q.wl);
        LinePrep32 p;
        p.El = q.El;
        p.Eu = q.E_upper;
        p.strength = q.strength;
        p.wlc = float(q.wl / C_CGS);
        p.k_m = float(KBOLTZ_CGS / q.m);
        p.wl2c = float(q.wl2c);
        p.grad = float(q.grad);
        p.gstark = float(q.gstark);
        p.v1 = float(q.v1);
        p.abo_pre = float(q.abo_pre);
        p.vexp = float(1 - q.v2);
        p.invmu = float(1 / (1.008 * AMU_CGS)) + 1.f / float(q.m);
        p.t32 = float(kp_mine.t);
        p.flags = (q.mol ? 1 : 0) | ((!q.mol && q.v2 != -1) ? 2 : 0);
        p.sp = q.sp;
        p.ki = int32_t(kp_mine.i);
        s_line[wib][lane] = p;
    }
    __syncwarp();
    // phase B: line by line, lanes over layers
    int my_dl = 0, my_ll = 0;
    for (int t = 0; t < nl; t++) {
        const int64_t i = base + t;
        const LinePrep32& q = s_line[wib][t];
        const bool mol = q.flags & 1, abo = q.flags & 2;
        float dmax = -1.f, lmax = -1.f;
        int dl = 0, ll = 0;
        float4* dst = reinterpret_cast<float4*>(out.params) + i * Lp;
        float4* dstw = out.params_w ? out.params_w + i * Lp : nullptr;
        float cref = 0.f;
        for (int l0 = 0; l0 < Lp; l0 += 32) {
            const int l = l0 + lane;
            float4 p = make_float4(1.f, 0.f, 0.f, 0.f);  // padding layers contribute nothing
            bool A = true;
            if (l < L) {
                const LayerConst c = lc[l];
                const float sigma = q.wlc * sqrtf(q.k_m * c.T32 + 0.5f * c.xi32 * c.xi32);
                float G = q.grad;
                if (!mol) {
                    float vdw;
                    if (!abo) {
                        vdw = q.v1 * c.vdw3_32;
                    } else {
                        const float vbar = sqrtf(float(8 * KBOLTZ_CGS / PI) * c.T32 * q.invmu);
                        vdw = q.abo_pre * powf(vbar * 1e-6f, q.vexp);
                    }
                    G = G + c.ne32 * (q.gstark * c.stark6_32) + c.nv32 * vdw;
                }
                const float gamma = G * q.wl2c;
                const double levels = fexp64(-c.beta * q.El, s_math) - fexp64(-c.beta * q.Eu, s_math);  // FP64
                const float amp = float(q.strength * levels * lay.n_div_U[int64_t(q.sp) * L + l]);
                const double* row = cn.vals + int64_t(l) * cn.nk;
                const float acntm = cn.nk == 1 ? float(row[0])
                                               : float(row[q.ki]) * (1.f - q.t32) + float(row[q.ki + 1]) * q.t32;
                const float rho = acntm * float(cutoff) / amp;
                const float dw = inverse_gaussian32(rho, sigma), lw = inverse_lorentz32(rho, gamma);
                if (dw > dmax) { dmax = dw; dl = l; }
                if (lw > lmax) { lmax = lw; ll = l; }
                const float s = 1.f / (sigma * 1.41421356f);
                const float a = gamma * s;
                const float scale = s * 0.56418958f * amp;  // 1/sqrt(pi)
                A = a <= 0.2f;
                p.x = 2.f * sigma * sigma;
                p.y = a;
                p.z = A ? a * 0.56418958f * scale : 1.f / (gamma * gamma);
                p.w = scale;
                // v >= 5 (a <= 0.2) or a + v >= 3.2 (0.2 < a <= 1.4) or any v (a > 1.4), v = x / sqrt(c)
                s_bnd[l] = (A ? 5.f : (a <= 1.4f ? 3.2f - a : 0.f)) * sqrtf(p.x) * 1.0001f;
                s_cls[l] = A;
                // the layer's cubic boundary: the asymptotic branch is exactly a cubic in 1/v^2; the
                // far-Lorentz branch is one beyond r_min gamma (far_lorentz_cubic_rmin)
                s_cub[l] = A ? s_bnd[l] : fmaxf(s_bnd[l], far_lorentz_cubic_rmin(a) * gamma * 1.0001f);
            } else if (l < Lp) {
                s_bnd[l] = 0.f;
                s_cls[l] = 1;
                s_cub[l] = 0.f;
            }
            if (l0 == 0) cref = __shfl_sync(0xffffffffu, p.x, 0);  // 2 sigma^2 of layer 0
            if (l < Lp) {
                dst[l] = p;
                if (dstw) {
                    // wing cubic in t' = cref / dl^2: A1 t' + A2 t'^2 + A3 t'^3.  Asymptotic branch:
                    // w u (1 + 1.5 u + 3.75 u^2) with u = 1/v^2 = (c / cref) t'.  Far-Lorentz branch:
                    // sqrt(2/pi) scale [q w + (3q^3 - q) w^2 + (q - 10q^3 + 15q^5) w^3] with
                    // w = gamma^2 / dl^2 = (gamma^2 / cref) t' (see far_lorentz_cubic_rmin).
                    float4 pw = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (l < L) {
                        if (A) {
                            const float rr = p.x / cref;
                            pw.x = p.z * rr;
                            pw.y = 1.5f * pw.x * rr;
                            pw.z = 2.5f * pw.y * rr;
                        } else {
                            const float q = 0.70710678118654752f / p.y, q2 = q * q;
                            const float kap = (1.f / p.z) / cref;  // gamma^2 / cref
                            const float k0 = 0.7978845608028654f * p.w;
                            pw.x = k0 * q * kap;
                            pw.y = k0 * q * fmaf(3.f, q2, -1.f) * kap * kap;
                            pw.z = k0 * q * fmaf(fmaf(15.f, q2, -10.f), q2, 1.f) * kap * kap * kap;
                        }
                    }
                    dstw[l] = pw;
                }
            }
        }
        __syncwarp();
        argmax_reduce(dmax, dl);
        argmax_reduce(lmax, ll);
        group_bounds(out, i, s_bnd, s_cls, lane);
        if (out.xcub && lane < out.G) {
            float mx = 0.f;
            for (int k = 0; k < out.K; k++) mx = fmaxf(mx, s_cub[lane * out.K + k]);
            out.xcub[i * out.G + lane] = mx;
        }
        __syncwarp();  // s_bnd / s_cls / s_cub are rewritten by the next line
        if (lane == t) { my_dl = dl; my_ll = ll; }
    }
    // phase C: the exact FP64 window of each line at its two widest layers, one lane per line
    if (lane < nl) {
        const int64_t i = base + lane;
        const LineConst q = line_const(ln, i);
        const LineLayer64 rd = line_layer64(q, lay, lc[my_dl], cn, kp_mine, cutoff, my_dl, s_math);
        const LineLayer64 rl = line_layer64(q, lay, lc[my_ll], cn, kp_mine, cutoff, my_ll, s_math);
        store_window(out, i, rl.lw, rd.dw, q.wl, wls, nwl, L);
    }
}

// Launch geometry of line_prep_mixed_kernel for n lines.
inline unsigned prep_mixed_blocks(int64_t n) { return unsigned((n + 32 * PREP_WARPS - 1) / (32 * PREP_WARPS)); }
inline size_t prep_mixed_smem(int Lp) { return size_t(PREP_WARPS) * Lp * (2 * sizeof(float) + sizeof(int)); }

// Candidate lists.  Lines are split by window half-width into tiers (at most 256, 4096, 65536
// wavelength points, and wider).  Within a tier the lines keep list order, so their centre
// indices are non-decreasing, and the lines that can overlap a tile [j0, j1] are the contiguous
// run with centre index in [j0 - W - 1, j1 + W + 1]: two binary searches per tier.  A single
// list with running max/min window bounds degenerates when a few lines have very wide windows
// (one synthetic line can span the whole grid); the tiers bound the over-scan per tier.
constexpr int NTIER = 4;
__device__ __constant__ int32_t c_tier_w[NTIER] = {256, 4096, 65536, 0x3fffffff};
constexpr int PART_THREADS = 256, PART_ITEMS = 8, PART_CHUNK = PART_THREADS * PART_ITEMS;

__device__ __forceinline__ int line_tier(int32_t lb, int32_t ub, int32_t ci) {
    if (lb > ub) return -1;  // empty window: never a candidate
    const int32_t h = max(ci - lb, ub - ci);
    int k = 0;
    while (k < NTIER - 1 && h > c_tier_w[k]) k++;
    return k;
}

struct TierLists {
    int32_t* idx;       // [n] line indices, tier by tier
    int32_t* ci;        // [n] their centre indices
    int32_t* start;     // [NTIER + 1] tier offsets into idx / ci
    int32_t* unsorted;  // set when centre indices decrease along the list (full scans then)
};

// per-block tier counts, and the sortedness check
__global__ void __launch_bounds__(PART_THREADS) tier_count_kernel(const int32_t* lb, const int32_t* ub,
                                                                  const int32_t* ci, int64_t n, int32_t* bcnt,
                                                                  int32_t* unsorted) {
    __shared__ int32_t s_cnt[NTIER];
    if (threadIdx.x < NTIER) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = int64_t(blockIdx.x) * PART_CHUNK;
    int c[NTIER] = {0, 0, 0, 0};
    bool bad = false;
    for (int k = threadIdx.x; k < PART_CHUNK; k += PART_THREADS) {
        const int64_t i = base + k;
        if (i >= n) break;
        const int t = line_tier(lb[i], ub[i], ci[i]);
        if (t >= 0) c[t]++;
        if (i > 0 && ci[i] < ci[i - 1]) bad = true;
    }
    for (int t = 0; t < NTIER; t++)
        if (c[t]) atomicAdd(&s_cnt[t], c[t]);
    if (bad) atomicOr(unsorted, 1);
    __syncthreads();
    if (threadIdx.x < NTIER) bcnt[blockIdx.x * NTIER + threadIdx.x] = s_cnt[threadIdx.x];
}

// stable scatter: position = tier base + lines of the tier in earlier blocks + rank in the block
__global__ void __launch_bounds__(PART_THREADS) tier_scatter_kernel(const int32_t* lb, const int32_t* ub,
                                                                    const int32_t* ci, int64_t n,
                                                                    const int32_t* bcnt, int nblocks, TierLists out) {
    __shared__ int32_t s_base[NTIER];
    __shared__ int32_t s_scan[NTIER][PART_THREADS];
    const int t0 = threadIdx.x;
    if (t0 < NTIER) {
        int32_t before = 0, total[NTIER] = {0, 0, 0, 0};
        for (int b = 0; b < nblocks; b++) {
            for (int k = 0; k < NTIER; k++) total[k] += bcnt[b * NTIER + k];
            if (b < int(blockIdx.x)) before += bcnt[b * NTIER + t0];
        }
        int32_t tb = 0;
        for (int k = 0; k < t0; k++) tb += total[k];
        s_base[t0] = tb + before;
        if (blockIdx.x == 0) {
            out.start[t0] = tb;
            if (t0 == NTIER - 1) out.start[NTIER] = tb + total[NTIER - 1];
        }
    }
    // each thread owns PART_ITEMS consecutive lines
    const int64_t i0 = int64_t(blockIdx.x) * PART_CHUNK + int64_t(t0) * PART_ITEMS;
    int tier[PART_ITEMS];
    int c[NTIER] = {0, 0, 0, 0};
    for (int k = 0; k < PART_ITEMS; k++) {
        const int64_t i = i0 + k;
        tier[k] = i < n ? line_tier(lb[i], ub[i], ci[i]) : -1;
        if (tier[k] >= 0) c[tier[k]]++;
    }
    for (int k = 0; k < NTIER; k++) s_scan[k][t0] = c[k];
    __syncthreads();
    for (int o = 1; o < PART_THREADS; o <<= 1) {  // inclusive scans of the per-thread counts
        int32_t v[NTIER];
        for (int k = 0; k < NTIER; k++) v[k] = t0 >= o ? s_scan[k][t0 - o] : 0;
        __syncthreads();
        for (int k = 0; k < NTIER; k++) s_scan[k][t0] += v[k];
        __syncthreads();
    }
    int32_t pos[NTIER];
    for (int k = 0; k < NTIER; k++) pos[k] = s_base[k] + s_scan[k][t0] - c[k];
    for (int k = 0; k < PART_ITEMS; k++) {
        if (tier[k] < 0) continue;
        const int32_t p = pos[tier[k]]++;
        out.idx[p] = int32_t(i0 + k);
        out.ci[p] = ci[i0 + k];
    }
}

struct TileArgs {
    double* alpha;        // [nwl][L]
    const double* wls;
    int64_t nwl;
    int32_t L, Lp, G, stage;  // layers, padded layers (G * K), layer groups, lines per batch
    int32_t split;            // 1: each CTA takes one layer group of the tile (blockIdx.y / queue)
    int32_t region;           // bytes of one shared buffer of line constants (x2, double buffered)
    int64_t n;
    const double* wl;     // line centres
    const void* params;
    const float* xfar;
    const uint32_t* amask;
    const int32_t *lb, *ub;
    const int32_t *tier_idx, *tier_ci, *tier_start, *unsorted;
    const float4* params_w;   // mixed, or null: wing cubics (see PrepOut)
    const float* xcub;        // mixed, or null: cubic boundaries (see PrepOut)
};

// first index in [lo, hi) with a[i] >= v (a non-decreasing)
__device__ __forceinline__ int64_t lower_bound_i32(const int32_t* a, int64_t lo, int64_t hi, int32_t v) {
    while (lo < hi) {
        int64_t mid = lo + ((hi - lo) >> 1);
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}
// first index in [lo, hi) with a[i] > v (a non-decreasing)
__device__ __forceinline__ int64_t upper_bound_i32(const int32_t* a, int64_t lo, int64_t hi, int32_t v) {
    while (lo < hi) {
        int64_t mid = lo + ((hi - lo) >> 1);
        if (a[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// A candidate line of the current chunk, as an FP64 tile sees it.
struct LineStage {
    double wl;        // centre
    int32_t lb, ub;   // window (grid indices)
    uint32_t cls;     // 2 bits per layer group: 2 = every layer in a closed-form wing branch, 0 = general
    int32_t li;       // line index
};

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// Far-Lorentz branch of voigt_hjerting (line_absorption.jl:305-308) with r^2 = x^2/gamma^2.
__device__ __forceinline__ float far_lorentz32(float4 p, float x2) {
    const float r2 = x2 * p.z;
    const float au = __fdividef(0.70710678118654752f, (r2 + 1.f) * p.y);
    const float au2 = au * au;
    return 0.7978845608028654f * au * (1.f + (3.f * r2 - 1.f + ((r2 - 2.f) * 15.f * r2 + 2.f) * au2) * au2) * p.w;
}
__device__ __forceinline__ double far_lorentz64(const P64& p, double x2) {
    const double r2 = x2 * p.w;
    const double au = 1 / SQRT_2 / ((r2 + 1) * p.a);
    const double au2 = au * au;
    return 0.7978845608028654 * au * (1 + (3 * r2 - 1 + ((r2 - 2) * 15 * r2 + 2) * au2) * au2) * p.scale;
}

// FP64 tile: TW = blockDim.x / G wavelengths x all layers (or, with gsplit >= 0, x the layers of
// group gsplit), computed by one CTA.  Thread (j, g) owns wavelength j and the K consecutive
// (padded) layers g*K .. g*K+K-1, accumulated in FP64 registers.  `smem` is the dynamic shared
// memory of the launch (two line-constant buffers, then the LineStage array).
template <int K>
__device__ __forceinline__ void line_tile_body64(const TileArgs& a, int64_t tile, int gsplit, unsigned char* smem) {
    const int L = a.L, Lp = a.Lp, G = a.G, B = a.stage;
    double* s_alpha = reinterpret_cast<double*>(smem);                          // [TW][SL+1], at the end
    LineStage* s_ln = reinterpret_cast<LineStage*>(smem + 2 * size_t(a.region));  // [blockDim]
    __shared__ int32_t s_warp[32];
    __shared__ int32_t s_count;

    // gsplit >= 0: this CTA computes layer group gsplit only (its own candidate list, constants
    // and barriers), so groups of cheap and expensive layers do not wait for each other
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int TW = gsplit >= 0 ? nthr : nthr / G;
    const int jl = tid % TW, g = gsplit >= 0 ? gsplit : tid / TW;
    const int SL = gsplit >= 0 ? K : Lp;       // layers of one staged line
    const int goff = gsplit >= 0 ? 0 : g * K;  // this thread's first layer within a staged line
    const int64_t j0 = tile * TW;
    const int64_t jg = j0 + jl;
    const int64_t jlast = min(j0 + TW, a.nwl) - 1;
    const bool live = jg < a.nwl;
    const double wl_j = live ? a.wls[jg] : 0.0;
    const double wl_ref = a.wls[j0], wl_last = a.wls[jlast];

    // candidate runs of the width tiers (threads 0..NTIER-1 search one tier each)
    __shared__ int64_t s_tier[NTIER][2];
    if (tid < NTIER) {
        const int64_t t0 = a.tier_start[tid], t1 = a.tier_start[tid + 1];
        if (*a.unsorted) {
            s_tier[tid][0] = t0;
            s_tier[tid][1] = t1;
        } else {
            const int32_t w = c_tier_w[tid] + 1;
            const int32_t lo = int32_t(max(int64_t(j0) - w, int64_t(INT32_MIN / 2)));
            const int32_t hi = int32_t(min(int64_t(jlast) + w, int64_t(INT32_MAX / 2)));
            s_tier[tid][0] = lower_bound_i32(a.tier_ci, t0, t1, lo);
            s_tier[tid][1] = upper_bound_i32(a.tier_ci, t0, t1, hi);
        }
    }
    __syncthreads();

    double acc[K];
#pragma unroll
    for (int k = 0; k < K; k++) acc[k] = 0.0;

    const int warp = tid >> 5, lane = tid & 31, nwarps = nthr >> 5;
    const int chunks16 = SL * int(sizeof(P64) / 16);  // 16-byte pieces of one line's staged constants
    const int cb0 = tid / chunks16, cr0 = tid - cb0 * chunks16;       // this thread's first staged piece
    const int cdb = nthr / chunks16, cdr = nthr - cdb * chunks16;     // and the step between its pieces
    const int64_t src0 = gsplit >= 0 ? int64_t(g) * K * int64_t(sizeof(P64) / 16) : 0;
    for (int tier = 0; tier < NTIER; tier++)
    for (int64_t base = s_tier[tier][0]; base < s_tier[tier][1]; base += nthr) {
        const int64_t pidx = base + tid;
        int64_t i = 0;
        bool take = false;
        int32_t lbi = 0, ubi = -1;
        if (pidx < s_tier[tier][1]) {
            i = a.tier_idx[pidx];
            lbi = a.lb[i];
            ubi = a.ub[i];
            take = lbi <= jlast && ubi >= j0;
        }
        const unsigned m = __ballot_sync(0xffffffffu, take);
        if (lane == 0) s_warp[warp] = __popc(m);
        __syncthreads();
        if (tid == 0) {
            int run = 0;
            for (int w = 0; w < nwarps; w++) { int c = s_warp[w]; s_warp[w] = run; run += c; }
            s_count = run;
        }
        __syncthreads();
        if (take) {  // the thread that found the line describes it for the whole CTA
            LineStage st;
            const double wl0 = a.wl[i];
            const double dist = wl0 < wl_ref ? wl_ref - wl0 : (wl0 > wl_last ? wl0 - wl_last : 0.0);
            uint32_t cls = 0;
            const int g_lo = gsplit >= 0 ? gsplit : 0, g_hi = gsplit >= 0 ? gsplit + 1 : G;
            for (int gg = g_lo; gg < g_hi; gg++)
                if (dist > double(a.xfar[i * G + gg])) cls |= 2u << (2 * gg);
            st.wl = wl0;
            st.lb = lbi;
            st.ub = ubi;
            st.cls = cls;
            st.li = int32_t(i);
            s_ln[s_warp[warp] + __popc(m & ((1u << lane) - 1))] = st;
        }
        const int cnt = s_count;
        __syncthreads();

        // batches of B lines: constants copied with cp.async into two alternating buffers
        const int nq = (cnt + B - 1) / B;
        auto issue = [&](int q) {
            if (q < nq) {
                const int b0 = q * B, nb = min(B, cnt - b0);
                unsigned char* buf = smem + size_t(q & 1) * a.region;
                // piece e = tid + k nthr of the batch is (line b, chunk r) = divmod(e, chunks16),
                // stepped without a division
                int b = cb0, r = cr0;
                for (int e = tid; e < nb * chunks16; e += nthr) {
                    const int64_t li = s_ln[b0 + b].li;
                    cp_async16(buf + (size_t(b) * chunks16 + r) * 16,
                               reinterpret_cast<const unsigned char*>(a.params) +
                                   (li * Lp * int64_t(sizeof(P64) / 16) + src0 + r) * 16);
                    b += cdb;
                    r += cdr;
                    if (r >= chunks16) {
                        r -= chunks16;
                        b++;
                    }
                }
            }
            cp_async_commit();
        };
        issue(0);
        for (int q = 0; q < nq; q++) {
            issue(q + 1);
            cp_async_wait_1();  // batch q has landed (this thread's copies) ...
            __syncthreads();    // ... and everybody else's
            const int b0 = q * B, nb = min(B, cnt - b0);
            const P64* s_par = reinterpret_cast<const P64*>(smem + size_t(q & 1) * a.region);
            if (live) {
                for (int b = 0; b < nb; b++) {
                    const LineStage& st = s_ln[b0 + b];
                    if (jg < st.lb || jg > st.ub) continue;
                    const double x = fabs(wl_j - st.wl);
                    const P64* pr = s_par + b * SL + goff;
                    if ((st.cls >> (2 * g)) & 3u) {
                        const double x2 = x * x, t = 1 / x2;
#pragma unroll
                        for (int k = 0; k < K; k++) {
                            if (pr[k].a <= 0.2) {
                                const double iv = t * pr[k].c;
                                acc[k] += (pr[k].w * iv) * (1 + iv * (1.5 + 3.75 * iv));
                            } else {
                                acc[k] += far_lorentz64(pr[k], x2);
                            }
                        }
                    } else {
#pragma unroll
                        for (int k = 0; k < K; k++) acc[k] += voigt64(pr[k].a, x * pr[k].inv_s) * pr[k].scale;
                    }
                }
            }
            __syncthreads();  // buffer (q & 1) is refilled by issue(q + 2)
        }
    }
    // alpha += accumulated lines, staged through shared memory for coalesced updates
    const int stride = SL + 1;
#pragma unroll
    for (int k = 0; k < K; k++) s_alpha[jl * stride + goff + k] = acc[k];
    __syncthreads();
    const int64_t nj = jlast - j0 + 1;
    double* dst = a.alpha + j0 * L;
    if (gsplit >= 0) {
        const int l0 = g * K, nk = min(K, L - l0);
        for (int64_t e = tid; e < nj * nk; e += nthr) {
            const int j = int(e / nk), k = int(e - int64_t(j) * nk);
            dst[int64_t(j) * L + l0 + k] += s_alpha[j * stride + k];
        }
    } else {
        for (int64_t e = tid; e < nj * L; e += nthr) {
            const int j = int(e / L), l = int(e - int64_t(j) * L);
            dst[e] = dst[e] + s_alpha[j * stride + l];
        }
    }
}

// A candidate line of the current chunk, as a mixed tile sees it (one layer group per CTA).
struct LineStage32 {
    float dhi, dlo;   // centre - first wavelength of the tile, as an FP32 pair
    int32_t lb, ub;   // window (grid indices)
    float cref;       // 2 sigma^2 of layer 0: the wing cubics' variable is t' = cref / dl^2
    float xfar;       // |dl| beyond which every layer of the group is in a closed-form wing branch
    uint32_t cubic;   // 1: every layer of the group is in its cubic regime over the whole tile
    int32_t li;       // line index
};
static_assert(sizeof(LineStage32) == 32, "LineStage32 is two 16-byte loads");

// Mixed-precision tile: TW = blockDim.x wavelengths x the K layers of group g.  Thread t owns
// wavelength j0 + t and all K layers.  Per staged line:
//   * lines whose layers are all in their cubic regime over the tile (most evaluations: far
//     wings) were staged as wing cubics: t' = cref / dl^2 per wavelength (zero outside the
//     window), then three FMAs per layer;
//   * other lines were staged as packed constants; each warp then checks whether its in-window
//     wavelengths are all beyond the wing boundary (one vote per line and warp) and evaluates
//     the closed-form wing branches, else the full profile.
// Accumulation: FP32 partial sums per batch of B lines, added to the accumulators with Kahan
// compensation.  Lines are visited in list order: results do not depend on the launch shape
// beyond the batch boundaries and the tile origins.  (Two wavelengths per thread, sharing each
// shared-memory load of a layer's constants, measured slower: the third accumulator set costs
// registers and occupancy than the saved loads gain.)
template <int K>
__device__ __forceinline__ void line_tile_body_mixed(const TileArgs& a, int64_t tile, int g, unsigned char* smem) {
    const int Lp = a.Lp, G = a.G, B = a.stage;
    double* s_alpha = reinterpret_cast<double*>(smem);                              // [TW][K+1], at the end
    LineStage32* s_ln = reinterpret_cast<LineStage32*>(smem + 2 * size_t(a.region));  // [blockDim]
    __shared__ int32_t s_warp[32];
    __shared__ int32_t s_count;
    __shared__ int64_t s_tier[NTIER][2];
    const int tid = threadIdx.x, nthr = blockDim.x, TW = nthr;
    const int warp = tid >> 5, lane = tid & 31, nwarps = nthr >> 5;
    const int64_t j0 = tile * TW;
    const int64_t jlast = min(j0 + TW, a.nwl) - 1;
    const double wl_ref = a.wls[j0], wl_last = a.wls[jlast];
    const float span32 = float(wl_last - wl_ref);
    // this thread's wavelength, and its offset from the tile's first one as an FP32 hi + lo pair
    // (formed in FP64), so |wl_j - wl0| is recovered in FP32 to about one rounding; a wavelength
    // past the grid end lies in no window
    const int32_t jm = int32_t(j0 + tid);
    const double dj = (j0 + tid < a.nwl ? a.wls[j0 + tid] : wl_ref) - wl_ref;
    const float xh = float(dj), xl = float(dj - double(xh));
    if (tid < NTIER) {  // candidate runs of the width tiers
        const int64_t t0 = a.tier_start[tid], t1 = a.tier_start[tid + 1];
        if (*a.unsorted) {
            s_tier[tid][0] = t0;
            s_tier[tid][1] = t1;
        } else {
            const int32_t w = c_tier_w[tid] + 1;
            const int32_t lo = int32_t(max(int64_t(j0) - w, int64_t(INT32_MIN / 2)));
            const int32_t hi = int32_t(min(int64_t(jlast) + w, int64_t(INT32_MAX / 2)));
            s_tier[tid][0] = lower_bound_i32(a.tier_ci, t0, t1, lo);
            s_tier[tid][1] = upper_bound_i32(a.tier_ci, t0, t1, hi);
        }
    }
    __syncthreads();

    float acc[K], comp[K];
#pragma unroll
    for (int k = 0; k < K; k++) { acc[k] = 0.f; comp[k] = 0.f; }

    const int64_t src0 = int64_t(g) * K;  // the group's first float4 within a line's Lp constants
    const int cb0 = tid / K, cr0 = tid - cb0 * K;      // this thread's first staged (line, layer)
    const int cdb = nthr / K, cdr = nthr - cdb * K;    // and the step between its pieces
    for (int tier = 0; tier < NTIER; tier++)
    for (int64_t base = s_tier[tier][0]; base < s_tier[tier][1]; base += nthr) {
        const int64_t pidx = base + tid;
        int64_t i = 0;
        bool take = false;
        int32_t lbi = 0, ubi = -1;
        if (pidx < s_tier[tier][1]) {
            i = a.tier_idx[pidx];
            lbi = a.lb[i];
            ubi = a.ub[i];
            take = lbi <= jlast && ubi >= j0;
        }
        const unsigned msk = __ballot_sync(0xffffffffu, take);
        if (lane == 0) s_warp[warp] = __popc(msk);
        __syncthreads();
        if (tid == 0) {
            int run = 0;
            for (int w = 0; w < nwarps; w++) { int c = s_warp[w]; s_warp[w] = run; run += c; }
            s_count = run;
        }
        __syncthreads();
        if (take) {  // the thread that found the line describes it for the whole CTA
            LineStage32 st;
            const double d = a.wl[i] - wl_ref;
            const float dh = float(d);
            // distance of the centre from the tile in FP32 (the boundaries carry a 1e-4
            // relative margin, far above the rounding)
            const float fdist = dh < 0.f ? -dh : (dh > span32 ? dh - span32 : 0.f);
            st.dhi = dh;
            st.dlo = float(d - double(dh));
            st.lb = lbi;
            st.ub = ubi;
            st.cref = reinterpret_cast<const float4*>(a.params)[i * Lp].x;  // 2 sigma^2, layer 0
            st.xfar = a.xfar[i * G + g];
            st.cubic = fdist > a.xcub[i * G + g] ? 1u : 0u;
            st.li = int32_t(i);
            s_ln[s_warp[warp] + __popc(msk & ((1u << lane) - 1))] = st;
        }
        const int cnt = s_count;
        __syncthreads();

        // batches of B lines: the group's constants copied with cp.async into two alternating
        // buffers (wing cubics for cubic-regime lines, packed constants otherwise)
        const int nq = (cnt + B - 1) / B;
        auto issue = [&](int q) {
            if (q < nq) {
                const int b0 = q * B, nb = min(B, cnt - b0);
                unsigned char* buf = smem + size_t(q & 1) * a.region;
                int b = cb0, r = cr0;  // piece e = tid + k nthr is (line b, layer r), stepped without a division
                for (int e = tid; e < nb * K; e += nthr) {
                    const LineStage32& sl = s_ln[b0 + b];
                    const float4* src = sl.cubic ? a.params_w : reinterpret_cast<const float4*>(a.params);
                    cp_async16(buf + (size_t(b) * K + r) * 16, src + (int64_t(sl.li) * Lp + src0 + r));
                    b += cdb;
                    r += cdr;
                    if (r >= K) {
                        r -= K;
                        b++;
                    }
                }
            }
            cp_async_commit();
        };
        issue(0);
        for (int q = 0; q < nq; q++) {
            issue(q + 1);
            cp_async_wait_1();  // batch q has landed (this thread's copies) ...
            __syncthreads();    // ... and everybody else's
            const int b0 = q * B, nb = min(B, cnt - b0);
            const float4* s_par = reinterpret_cast<const float4*>(smem + size_t(q & 1) * a.region);
            float part[K];
#pragma unroll
            for (int k = 0; k < K; k++) part[k] = 0.f;
            for (int b = 0; b < nb; b++) {
                const LineStage32 st = s_ln[b0 + b];
                const float4* pr = s_par + b * K;
                const bool in = jm >= st.lb && jm <= st.ub;
                const float x = fabsf((xh - st.dhi) + (xl - st.dlo));
                if (st.cubic) {
                    const float tp = in ? __fdividef(st.cref, x * x) : 0.f;
#pragma unroll
                    for (int k = 0; k < K; k++) {
                        const float4 p = pr[k];
                        part[k] = fmaf(tp, fmaf(tp, fmaf(tp, p.z, p.y), p.x), part[k]);
                    }
                } else if (__all_sync(0xffffffffu, !in || x > st.xfar)) {
                    // every in-window wavelength of the warp in a closed-form wing branch, chosen
                    // per layer (uniform across the warp)
                    if (in) {
                        const float x2 = x * x, t = __fdividef(1.f, x2);
#pragma unroll
                        for (int k = 0; k < K; k++) {
                            const float4 p = pr[k];
                            if (p.y <= 0.2f) {
                                const float iv = t * p.x;
                                part[k] = fmaf(p.z * iv, fmaf(fmaf(3.75f, iv, 1.5f), iv, 1.f), part[k]);
                            } else {
                                part[k] += far_lorentz32(p, x2);
                            }
                        }
                    }
                } else if (in) {
                    const float t = __fdividef(1.f, x * x);
#pragma unroll
                    for (int k = 0; k < K; k++) part[k] += profile32x(pr[k], x, t);
                }
            }
            // batch partial sums enter the accumulators with Kahan compensation
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float y = part[k] - comp[k];
                const float tt = acc[k] + y;
                comp[k] = (tt - acc[k]) - y;
                acc[k] = tt;
            }
            __syncthreads();  // buffer (q & 1) is refilled by issue(q + 2)
        }
    }
    // alpha += accumulated lines, staged through shared memory for coalesced updates
    const int stride = K + 1;
#pragma unroll
    for (int k = 0; k < K; k++) s_alpha[tid * stride + k] = double(acc[k]) - double(comp[k]);
    __syncthreads();
    const int64_t nj = jlast - j0 + 1;
    double* dst = a.alpha + j0 * a.L;
    const int l0 = g * K, nk = min(K, a.L - l0);
    for (int64_t e = tid; e < nj * nk; e += nthr) {
        const int j = int(e / nk), k = int(e - int64_t(j) * nk);
        dst[int64_t(j) * a.L + l0 + k] += s_alpha[j * stride + k];
    }
}

// One CTA per tile of one spectrum (per tile and layer group in the mixed form).
template <bool MIXED, int K, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) line_tile_kernel(TileArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    if constexpr (MIXED)
        line_tile_body_mixed<K>(a, blockIdx.x, int(blockIdx.y), smem);
    else
        line_tile_body64<K>(a, blockIdx.x, a.split ? int(blockIdx.y) : -1, smem);
}

// Work queue of (spectrum, tile) items for a batch of spectra on one wavelength grid.  Item k
// is tile k / nspec of spectrum k % nspec: the queue walks the grid once, visiting every
// spectrum's tile before moving on, so spectra with few and many lines are interleaved.
struct TileQueue {
    const TileArgs* spec;        // [nspec], device
    int32_t nspec;
    int32_t groups;              // layer groups per tile item (G when split, else 1)
    int64_t nitems;              // nspec * tiles * groups
    unsigned long long* next;    // item counter, zero before the launch
};

// Persistent form: a grid sized to the resident CTAs of the GPU takes items from the queue
// until it is empty.
template <bool MIXED, int K, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) line_tile_queue_kernel(TileQueue q) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ TileArgs s_a;
    __shared__ long long s_item;
    for (;;) {
        if (threadIdx.x == 0) {
            const long long it = (long long)atomicAdd(q.next, 1ull);
            s_item = it;
            if (it < q.nitems) s_a = q.spec[it % q.nspec];
        }
        __syncthreads();
        const long long it = s_item;
        if (it >= q.nitems) break;
        const long long r = it / q.nspec;
        if constexpr (MIXED)
            line_tile_body_mixed<K>(s_a, r / q.groups, int(r % q.groups), smem);
        else
            line_tile_body64<K>(s_a, r / q.groups, q.groups > 1 ? int(r % q.groups) : -1, smem);
        __syncthreads();  // s_a and s_item are rewritten for the next item
    }
}

}  // namespace korg
