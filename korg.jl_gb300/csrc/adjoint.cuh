// adjoint.cuh -- reverse-mode (vector-Jacobian) kernels of the synthesis hot path.
//
// Given cotangents dL/dF(lambda) and dL/dC(lambda) of the flux and continuum flux, they give
// dL/d(layer temperatures, n_e, n_eff_vdW, microturbulence, n/U per species, per-line log gf,
// continuum opacity knots, reference-wavelength continuum opacity):
//
//   rt_adjoint_kernel    one warp per wavelength column: tau by a warp-shuffle prefix scan,
//                        E2 / exp per layer in parallel, the segment partial derivatives of the
//                        exponential-integral formal solution, and the reverse (suffix) scan of
//                        the tau recursion.  Outputs dL/dalpha[l, j] (the opacity cotangent G),
//                        and per-layer sums through the Planck source function and alpha_ref.
//   line_adj_kernel      (line, window chunk) items, one thread per layer, a sequential walk
//                        over the chunk's wavelengths: sums of G * dphi/d(amplitude, sigma,
//                        gamma) with dH/da, dH/dv of every Hjerting branch from forward-mode
//                        dual numbers (the derivative of the approximation itself, as
//                        ForwardDiff differentiates line_absorption.jl:286-310).
//   line_adj_prologue    one warp per line, lanes over layers: the chain rule of
//                        line_absorption.jl:86-106 from (amplitude, sigma, gamma) to the layer
//                        inputs and log gf, in FP64.
//
// The windows [lb, ub] are integer functions of the inputs and carry no derivative, as in the
// reference under ForwardDiff.  alpha itself is recomputed by the forward kernels before the
// reverse pass; nothing of the forward synthesis is stored between the two.
#pragma once
#include "lines.cuh"
#include "physics.cuh"
#include "rt.cuh"

namespace korg {

// ---------------------------------------------------------------- dual numbers in (a, v)
template <class R>
struct Dual {
    R x, da, dv;
};
template <class R>
__device__ __forceinline__ Dual<R> operator+(Dual<R> p, Dual<R> q) { return {p.x + q.x, p.da + q.da, p.dv + q.dv}; }
template <class R>
__device__ __forceinline__ Dual<R> operator-(Dual<R> p, Dual<R> q) { return {p.x - q.x, p.da - q.da, p.dv - q.dv}; }
template <class R>
__device__ __forceinline__ Dual<R> operator*(Dual<R> p, Dual<R> q) {
    return {p.x * q.x, p.da * q.x + p.x * q.da, p.dv * q.x + p.x * q.dv};
}
__device__ __forceinline__ float recip(float x) { return __fdividef(1.f, x); }
__device__ __forceinline__ double recip(double x) { return 1.0 / x; }
template <class R>
__device__ __forceinline__ Dual<R> operator/(Dual<R> p, Dual<R> q) {
    const R inv = recip(q.x), r = p.x * inv;
    return {r, (p.da - r * q.da) * inv, (p.dv - r * q.dv) * inv};
}
template <class R>
__device__ __forceinline__ Dual<R> operator+(Dual<R> p, R c) { return {p.x + c, p.da, p.dv}; }
template <class R>
__device__ __forceinline__ Dual<R> operator+(R c, Dual<R> p) { return {p.x + c, p.da, p.dv}; }
template <class R>
__device__ __forceinline__ Dual<R> operator-(R c, Dual<R> p) { return {c - p.x, -p.da, -p.dv}; }
template <class R>
__device__ __forceinline__ Dual<R> operator-(Dual<R> p, R c) { return {p.x - c, p.da, p.dv}; }
template <class R>
__device__ __forceinline__ Dual<R> operator*(R c, Dual<R> p) { return {c * p.x, c * p.da, c * p.dv}; }
template <class R>
__device__ __forceinline__ Dual<R> operator*(Dual<R> p, R c) { return {c * p.x, c * p.da, c * p.dv}; }
template <class R>
__device__ __forceinline__ Dual<R> operator/(R c, Dual<R> q) {
    const R iq = recip(q.x), r = c * iq;
    return {r, -r * iq * q.da, -r * iq * q.dv};
}
__device__ __forceinline__ double dexp(double x) { return exp(x); }
__device__ __forceinline__ float dexp(float x) { return __expf(x); }
template <class R>
__device__ __forceinline__ Dual<R> dual_exp(Dual<R> p) {
    const R e = dexp(p.x);
    return {e, e * p.da, e * p.dv};
}

// harris_series (line_absorption.jl:251-265) on duals
template <class R>
__device__ __forceinline__ void harris_dual(Dual<R> v, Dual<R>& H0, Dual<R>& H1, Dual<R>& H2) {
    const Dual<R> v2 = v * v;
    H0 = dual_exp(R(0) - v2);
    if (v.x < R(1.3))
        H1 = R(-1.12470432) + (R(-0.15516677) + (R(3.288675912) + (R(-2.34357915) + R(0.42139162) * v) * v) * v) * v;
    else if (v.x < R(2.4))
        H1 = R(-4.48480194) + (R(9.39456063) + (R(-6.61487486) + (R(1.98919585) - R(0.22041650) * v) * v) * v) * v;
    else
        H1 = (R(0.554153432) + (R(0.278711796) + (R(-0.1883256872) + (R(0.042991293) - R(0.003278278) * v) * v) * v) * v) /
             (v2 - R(1.5));
    H2 = (R(1) - R(2) * v2) * H0;
}

// voigt_hjerting (line_absorption.jl:286-310) with its partial derivatives: returns
// {H, dH/da, dH/dv} of the branch the value (a, v) selects.
template <class R>
__device__ __forceinline__ Dual<R> voigt_dual(R a_, R v_) {
    const Dual<R> a{a_, R(1), R(0)}, v{v_, R(0), R(1)};
    const Dual<R> v2 = v * v;
    const R SQPI = R(1.7724538509055159);
    if (a_ <= R(0.2) && v_ >= R(5)) {
        const Dual<R> iv2 = R(1) / v2;
        return (a * (R(1) / SQPI) * iv2) * (R(1) + R(1.5) * iv2 + R(3.75) * (iv2 * iv2));
    }
    Dual<R> H0, H1, H2;
    if (a_ <= R(0.2)) {
        harris_dual(v, H0, H1, H2);
        return H0 + (H1 + H2 * a) * a;
    }
    if (a_ <= R(1.4) && a_ + v_ < R(3.2)) {
        harris_dual(v, H0, H1, H2);
        const R c2 = R(2) / SQPI, c23 = R(2) / (R(3) * SQPI);
        const Dual<R> M0 = H0;
        const Dual<R> M1 = H1 + c2 * M0;
        const Dual<R> M2 = H2 - M0 + c2 * M1;
        const Dual<R> M3 = c23 * (R(1) - H2) - (R(2) / R(3)) * v2 * M1 + c2 * M2;
        const Dual<R> M4 = (R(2) / R(3)) * v2 * v2 * M0 - c23 * M1 + c2 * M3;
        const Dual<R> psi = R(0.979895023) + (R(-0.962846325) + (R(0.532770573) - R(0.122727278) * a) * a) * a;
        return psi * (M0 + (M1 + (M2 + (M3 + M4 * a) * a) * a) * a);
    }
    const Dual<R> r2 = v2 / (a * a);
    const Dual<R> au = (R(1) / R(1.4142135623730951)) / ((r2 + R(1)) * a);
    const Dual<R> au2 = au * au;
    return R(0.7978845608028654) * au * (R(1) + (R(3) * r2 - R(1) + ((r2 - R(2)) * R(15) * r2 + R(2)) * au2) * au2);
}

// ---------------------------------------------------------------- transfer adjoint
struct RtAdjArgs {
    const double* alpha;      // [nwl][L] full opacity
    const double* T;          // [L]
    const double* wls;        // [nwl]
    int64_t nwl;
    int32_t L;
    const double* tau_ref;    // [L]
    const double* alpha_ref;  // [L]
    const MathTables* math;
    CntmDev cn;               // continuum interpolant (continuum-only pass and d/d knots)
    const double* dflux;      // [nwl] or null
    const double* dcntm;      // [nwl] or null
    double unit;              // flux = 2 pi I unit
    void* G;                  // out [nwl][L]: dL/dalpha (float when g32)
    int32_t g32;
    double* dT;               // out [L] (+=): through the source function
    double* daref;            // out [L] (+=): through alpha_ref
    double* dvals;            // out [L][nk] (+=) or null: continuum knots
};

constexpr int RTA_WARPS = 4;
constexpr int RTA_LMAX = 128;
constexpr int RTA_ARRAYS = 14;  // per-warp column arrays of the kernel's dynamic shared memory

// Per-warp scratch of one column (each array L + 1 doubles of dynamic shared memory).
struct RtaCol {
    double *S, *tau, *e2, *d2, *ex, *ib, *ta, *tb, *sa, *sb, *Sbar, *col, *g, *gc;
};

// Taylor coefficients of the piecewise E2 (RadiativeTransfer.jl:441-490) around x0 = 2..8
__device__ __constant__ double c_e2poly[7][6] = {
    {0.037534261820486914, -0.04890051070806112, 0.033833820809153176, -0.016916910404576574,
     0.007048712668573576, -0.0026785108140579598},
    {0.010641925085272673, -0.013048381094197039, 0.008297844727977323, -0.003687930990212144,
     0.0013061422257001345, -0.0003995258572729822},
    {0.0031982292493385146, -0.0037793524098489054, 0.0022894548610917728, -0.0009539395254549051,
     0.00031003034577284415, -8.466213288412284e-5},
    {0.000996469042708825, -0.0011482955912753257, 0.0006737946999085467, -0.00026951787996341863,
     8.310134632205409e-5, -2.1202073223788938e-5},
    {0.0003182574636904001, -0.0003600824521626587, 0.00020656268138886323, -8.032993165122457e-5,
     2.390771775334065e-5, -5.8334831318151185e-6},
    {0.00010350984428214624, -0.00011548173161033826, 6.513442611103688e-5, -2.4813114708966427e-5,
     7.200234178941151e-6, -1.7027366981408086e-6},
    {3.413764515111217e-5, -3.76656228439249e-5, 2.096641424390699e-5, -7.862405341465122e-6,
     2.2386015208338193e-6, -5.173353514609864e-7}};

// d/dx of that piecewise approximation of E2, branch by branch (the derivative ForwardDiff
// takes), given e2 = E2(x) and ex = exp(-x) of the same branch.
__device__ __forceinline__ double expint2_deriv(double x, double e2, double ex, const MathTables& t) {
    if (x < 1.1) {  // E2 = 1 + x (ln x + EM - 1) + x Q(x)
        const double EM = 0.57721566490153286060651209008240243104215933593992;
        const double c2 = 0.08333333333333333, c3 = -0.013888888888888888, c4 = 0.0020833333333333333;
        const double Q = (-0.5 + (c2 + (c3 + c4 * x) * x) * x) * x;
        const double dQ = -0.5 + (2 * c2 + (3 * c3 + 4 * c4 * x) * x) * x;
        return flog64(x, t) + EM + Q + x * dQ;
    }
    if (x < 9) {
        const int k = x < 2.5 ? 0 : (x < 3.5 ? 1 : (x < 4.5 ? 2 : (x < 5.5 ? 3 : (x < 6.5 ? 4 : (x < 7.5 ? 5 : 6)))));
        const double y = x - (2 + k);
        const double* a = c_e2poly[k];
        return a[1] + y * (2 * a[2] + y * (3 * a[3] + y * (4 * a[4] + y * 5 * a[5])));
    }
    // E2 = e^-x u R(u), u = 1/x
    const double u = 1 / x;
    const double R = 1 + (-2 + (6 + (-24 + 120 * u) * u) * u) * u;
    const double dR = -2 + (12 + (-72 + 480 * u) * u) * u;
    return -e2 - ex * u * u * (R + u * dR);
}

// One transfer pass over the column `al` (global or shared) with cotangent w of 2 pi I unit:
// writes dL/dalpha of the pass into gout[l], adds dL/dS into c.Sbar and dL/dalpha_ref into
// s_daref (shared, atomically).
__device__ __forceinline__ void rt_adj_pass(const RtaCol& c, const double* al, double w, const double* s_fac,
                                            const double* s_dlt, const double* s_aref, int L, const MathTables& mt,
                                            double* gout, double* s_daref, int lane) {
    // optical depth (RadiativeTransfer.jl:244-253): ib, trapezoid increments, warp scans
    for (int l = lane; l < L; l += 32) c.ib[l] = al[l] * s_fac[l];
    __syncwarp();
    double carry = 0.0;
    for (int base = 0; base < L; base += 32) {
        const int l = base + lane;
        double inc = (l >= 1 && l < L) ? 0.5 * (c.ib[l] + c.ib[l - 1]) * s_dlt[l] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (l < L) c.tau[l] = carry + inc;
        carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    __syncwarp();
    // the forward recursion stops after the first layer whose tau exceeds TAU_STOP
    int lc = L - 1;
    for (int base = 0; base < L; base += 32) {
        const int l = base + lane;
        const unsigned m = __ballot_sync(0xffffffffu, l >= 1 && l < L && c.tau[l] > TAU_STOP);
        if (m) { lc = min(lc, base + __ffs(m) - 1); break; }
    }
    for (int l = lane; l <= L; l += 32) {
        if (l < L) {
            const double t = c.tau[l];
            const double ex = l == 0 ? 1.0 : fexp64(-t, mt);
            const double e2 = l == 0 ? 1.0 : expint2_ex(t, ex, mt);
            c.ex[l] = ex;
            c.e2[l] = e2;
            c.d2[l] = l == 0 ? 0.0 : expint2_deriv(t, e2, ex, mt);  // tau_0 = 0 is not a variable
            c.tb[l] = 0.0;
            c.sb[l] = 0.0;
        }
        c.ta[l] = 0.0;
        c.sa[l] = 0.0;
    }
    __syncwarp();
    // segment l joins layers l-1 and l (RadiativeTransfer.jl:379-388); the partial derivatives
    // of C(tau_b) - C(tau_a), C(tau) = (tau E2 (3b + 2m tau) - e^-tau (3b + 2m (tau + 1))) / 6,
    // m = (S_b - S_a)/(tau_b - tau_a), b = S_a - m tau_a, differentiating the E2 approximation
    // itself (for the exact E2, dC/dtau would be (m tau + b) E2).
    auto dC = [&](double t, double e2, double d2, double ex, double m, double bb) {
        return (1.0 / 6.0) * ((e2 + t * d2) * (3 * bb + 2 * m * t) + 2 * m * t * e2 +
                              ex * (3 * bb + 2 * m * (t + 1)) - 2 * m * ex);
    };
    for (int l = 1 + lane; l <= lc; l += 32) {
        const double ta_ = c.tau[l - 1], tb_ = c.tau[l];
        const double Sa = c.S[l - 1], Sb = c.S[l];
        const double D = tb_ - ta_;
        const double m = (Sb - Sa) / D;
        const double bb = Sa - m * ta_;
        const double Pb = 0.5 * ((tb_ * c.e2[l] - c.ex[l]) - (ta_ * c.e2[l - 1] - c.ex[l - 1]));
        const double Pm = (1.0 / 3.0) * ((tb_ * tb_ * c.e2[l] - c.ex[l] * (tb_ + 1)) -
                                         (ta_ * ta_ * c.e2[l - 1] - c.ex[l - 1] * (ta_ + 1)));
        const double Q = Pm - ta_ * Pb;  // total derivative through m (b depends on m)
        const double Ctb = dC(tb_, c.e2[l], c.d2[l], c.ex[l], m, bb);
        const double Cta = l == 1 ? 0.0 : dC(ta_, c.e2[l - 1], c.d2[l - 1], c.ex[l - 1], m, bb);
        c.tb[l] = w * (Ctb - Q * m / D);
        c.ta[l - 1] = w * (-Cta - Pb * m + Q * m / D);
        c.sb[l] = w * (Q / D);
        c.sa[l - 1] = w * (Pb - Q / D);
    }
    __syncwarp();
    // tau_bar[l] = sum over k >= l of the direct cotangents (tau_k = tau_{k-1} + increment):
    // a reverse warp scan; tau[] is free now and receives tau_bar
    double carry2 = 0.0;
    for (int top = ((L - 1) / 32) * 32; top >= 0; top -= 32) {
        const int l = top + (31 - lane);  // lane 0 holds the deepest layer of the chunk
        double d = (l >= 1 && l < L) ? c.tb[l] + c.ta[l] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, d, o);
            if (lane >= o) d += y;
        }
        if (l < L) c.tau[l] = carry2 + d;
        carry2 += __shfl_sync(0xffffffffu, d, 31);
    }
    __syncwarp();
    for (int l = lane; l < L; l += 32) {
        // ib_l enters the increments of tau_l and tau_{l+1} (RadiativeTransfer.jl:250-251)
        double ibar = 0.0;
        if (l >= 1) ibar += 0.5 * s_dlt[l] * c.tau[l];
        if (l + 1 < L) ibar += 0.5 * s_dlt[l + 1] * c.tau[l + 1];
        gout[l] = ibar * s_fac[l];
        if (ibar != 0.0) atomicAdd(s_daref + l, -ibar * c.ib[l] / s_aref[l]);  // fac = tau_ref/alpha_ref
        c.Sbar[l] += c.sb[l] + c.sa[l];
    }
    __syncwarp();
}

__global__ void __launch_bounds__(32 * RTA_WARPS) rt_adjoint_kernel(RtAdjArgs a) {
    __shared__ MathTables s_math;
    __shared__ double s_fac[RTA_LMAX], s_dlt[RTA_LMAX], s_aref[RTA_LMAX], s_T[RTA_LMAX];
    __shared__ double s_dT[RTA_LMAX], s_dar[RTA_LMAX];
    extern __shared__ double s_cols[];  // [warps][RTA_ARRAYS][L + 1]
    load_math_tables(s_math, a.math);
    const int L = a.L;
    for (int l = threadIdx.x; l < L; l += blockDim.x) {
        s_fac[l] = a.tau_ref[l] / a.alpha_ref[l];
        s_dlt[l] = l == 0 ? 0.0 : log(a.tau_ref[l]) - log(a.tau_ref[l - 1]);
        s_aref[l] = a.alpha_ref[l];
        s_T[l] = a.T[l];
        s_dT[l] = 0.0;
        s_dar[l] = 0.0;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* base = s_cols + size_t(warp) * RTA_ARRAYS * (L + 1);
    RtaCol c;
    double** f[RTA_ARRAYS] = {&c.S, &c.tau, &c.e2, &c.d2, &c.ex, &c.ib, &c.ta, &c.tb, &c.sa, &c.sb, &c.Sbar, &c.col,
                              &c.g, &c.gc};
    for (int k = 0; k < RTA_ARRAYS; k++) *f[k] = base + k * (L + 1);
    const bool two = a.cn.nk > 0;
    const int64_t stride = int64_t(gridDim.x) * RTA_WARPS;
    for (int64_t j = int64_t(blockIdx.x) * RTA_WARPS + warp; j < a.nwl; j += stride) {
        const double wl = a.wls[j];
        const double wf = a.dflux ? a.dflux[j] * 2 * PI * a.unit : 0.0;
        const double wc = (two && a.dcntm) ? a.dcntm[j] * 2 * PI * a.unit : 0.0;
        const double pre = 2 * HPLANCK_CGS * (C_CGS * C_CGS) / (wl * wl * wl * wl * wl);
        const double hcw = HPLANCK_CGS * C_CGS / wl;
        for (int l = lane; l < L; l += 32) {
            c.S[l] = planck(pre, hcw, s_T[l]);
            c.Sbar[l] = 0.0;
        }
        __syncwarp();
        rt_adj_pass(c, a.alpha + j * L, wf, s_fac, s_dlt, s_aref, L, s_math, c.g, s_dar, lane);
        if (two) {
            // continuum-only column (src/synthesize.jl:287-291), as the forward interpolates it
            const KnotPos kp = knot_pos(a.cn.knots, a.cn.nk, wl);
            for (int l = lane; l < L; l += 32) c.col[l] = knot_eval(a.cn.vals + int64_t(l) * a.cn.nk, a.cn.nk, kp);
            __syncwarp();
            rt_adj_pass(c, c.col, wc, s_fac, s_dlt, s_aref, L, s_math, c.gc, s_dar, lane);
            // the knots feed both passes' opacity (alpha = continuum + hydrogen + lines)
            if (a.dvals) {
                for (int l = lane; l < L; l += 32) {
                    const double gsum = c.g[l] + c.gc[l];
                    if (gsum == 0.0) continue;
                    double* row = a.dvals + int64_t(l) * a.cn.nk;
                    if (a.cn.nk == 1) {
                        atomicAdd(row, gsum);
                    } else {
                        atomicAdd(row + kp.i, gsum * (1.0 - kp.t));
                        atomicAdd(row + kp.i + 1, gsum * kp.t);
                    }
                }
            }
        }
        // Planck source function (src/synthesize.jl:412-418): dB/dT = B x/T (1 + B/pre)
        for (int l = lane; l < L; l += 32) {
            const double B = c.S[l];
            const double x = hcw / KBOLTZ_CGS / s_T[l];
            const double d = c.Sbar[l] * B * (x / s_T[l]) * (1.0 + B / pre);
            if (d != 0.0) atomicAdd(s_dT + l, d);
            if (a.g32)
                static_cast<float*>(a.G)[j * L + l] = float(c.g[l]);
            else
                static_cast<double*>(a.G)[j * L + l] = c.g[l];
        }
        __syncwarp();
    }
    __syncthreads();
    for (int l = threadIdx.x; l < L; l += blockDim.x) {
        if (s_dT[l] != 0.0) atomicAdd(a.dT + l, s_dT[l]);
        if (s_dar[l] != 0.0) atomicAdd(a.daref + l, s_dar[l]);
    }
}

// ---------------------------------------------------------------- line adjoint
struct LineAdjArgs {
    const void* G;            // [nwl][L] opacity cotangent (float when g32)
    int32_t g32;
    const double* wls;
    int64_t nwl;
    int32_t L, Lp;
    const double* wl;         // line centres
    const void* params;       // forward constants [n][Lp]: float4 {2 sigma^2, a, w, scale} or P64
    const int32_t *lb, *ub;
    const int32_t *tier_idx, *tier_start;  // lines with non-empty windows, by width tier
    double* dpar;             // out [n][Lp][3] (+=): window sums of G H, G (a H_a + v H_v), G H_a
    unsigned long long* next; // item counter (zero before the launch)
};

constexpr int ADJ_CHUNK = 4096;  // wavelengths per item

// Items: tier 3 lines x ceil(nwl / CHUNK) chunks first, then tier 2 x 33, tier 1 x 3, tier 0 x 1
// (window half-widths of at most 65536, 4096 and 256 points bound the chunks per line).
__device__ __forceinline__ int64_t adj_chunks(int tier, int64_t nwl) {
    return tier == 3 ? (nwl + ADJ_CHUNK - 1) / ADJ_CHUNK : (tier == 2 ? 33 : (tier == 1 ? 3 : 1));
}

__device__ __forceinline__ float fast_div(float p, float q) { return __fdividef(p, q); }
__device__ __forceinline__ double fast_div(double p, double q) { return p / q; }

// Compensated running sums of N values (mixed: FP32 partials enter Kahan-compensated totals;
// FP64: plain sums).
template <bool MIXED, int N>
struct AdjSums {
    using R = typename std::conditional<MIXED, float, double>::type;
    R s[N], c[N];
    __device__ __forceinline__ AdjSums() {
#pragma unroll
        for (int k = 0; k < N; k++) { s[k] = R(0); c[k] = R(0); }
    }
    __device__ __forceinline__ void add(const R* p) {
#pragma unroll
        for (int k = 0; k < N; k++) {
            if (MIXED) {
                const R y = p[k] - c[k], t = s[k] + y;
                c[k] = (t - s[k]) - y;
                s[k] = t;
            } else {
                s[k] += p[k];
            }
        }
    }
    __device__ __forceinline__ double get(int k) const { return double(s[k]) - double(c[k]); }
};

__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gmem_src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem_dst, const void* gmem_src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gmem_src) : "memory");
}

// Far-Lorentz branch of voigt_hjerting (line_absorption.jl:305-308: a > 1.4, or a > 0.2 with
// a + v >= 3.2) with its derivatives in closed form: H, X = a H_a + v H_v and A = H_a.  With
// r^2 = v^2/a^2 (degree 0) and au = 1/(sqrt2 a (1 + r^2)) (degree -1), H = C au (1 + P b + Q b^2),
// b = au^2, P = 3r^2 - 1, Q = 15r^4 - 30r^2 + 2:  X = -C au (1 + 3P b + 5Q b^2), and
// A = C au/a [w (1 + P b + Q b^2) + b (-6r^2 + 2P w) + b^2 (-60 r^2 (r^2 - 1) + 4Q w)] with
// w = (r^2 - 1)/(r^2 + 1).
template <class R>
__device__ __forceinline__ void far_lorentz_d(R a, R v, R& H, R& X, R& A) {
    const R ia = recip(a);
    const R r2 = v * v * ia * ia;
    const R iz = recip(R(1) + r2);
    const R au = R(0.70710678118654752) * ia * iz;
    const R b = au * au;
    const R P = R(3) * r2 - R(1);
    const R Q = (r2 - R(2)) * R(15) * r2 + R(2);
    const R Cau = R(0.7978845608028654) * au;
    const R poly = R(1) + (P + Q * b) * b;
    const R w = (r2 - R(1)) * iz;
    H = Cau * poly;
    X = -Cau * (R(1) + (R(3) * P + R(5) * Q * b) * b);
    A = Cau * ia * (w * poly + (R(-6) * r2 + R(2) * P * w) * b + (R(-60) * r2 * (r2 - R(1)) + R(4) * Q * w) * b * b);
}

// H, a H_a + v H_v and H_a of every branch but the asymptotic wing: far Lorentz in closed form,
// the Harris branches through dual numbers.
template <class R>
__device__ __forceinline__ void central_derivs(R av, R v, R* out) {
    R H, X, A;
    if (av > R(0.2) && (av > R(1.4) || av + v >= R(3.2))) {
        far_lorentz_d<R>(av, v, H, X, A);
    } else {
        const Dual<R> d = voigt_dual<R>(av, v);
        H = d.x;
        A = d.da;
        X = av * d.da + v * d.dv;
    }
    out[0] = H;
    out[1] = X;
    out[2] = A;
}

constexpr int ADJ_SUB = 64;  // wavelengths of G staged in shared memory at a time

// One block per item (a line and a chunk of its window).  The item's G rows (ADJ_SUB wavelengths
// x L layers, contiguous in global memory) are copied to shared memory with cp.async, double
// buffered, with 1/|dl|^2 of every staged wavelength; thread (l = tid mod L, jr = tid / L)
// walks every NJ-th staged wavelength for layer l, so a warp reads consecutive G entries.
// In the asymptotic wing (a <= 0.2, v >= 5: most evaluations of a wide window)
// H = a/sqrt(pi) u (1 + 1.5u + 3.75u^2) with u = 1/v^2 = c t (c = 2 sigma^2, t = 1/|dl|^2), so
// the three window sums follow from the moments M_k = sum G u^k, k = 1..3 (three FMAs per
// evaluation):  sum G H = a/sqrt(pi) (M1 + 1.5 M2 + 3.75 M3),  sum G H_a = that / a,
// sum G (a H_a + v H_v) = sum G H - 2 a/sqrt(pi) (M1 + 3 M2 + 11.25 M3).  Nearer the centre
// central_derivs differentiates the far-Lorentz branch in closed form and the Harris branches
// with dual numbers.
template <bool MIXED>
__global__ void __launch_bounds__(512) line_adj_kernel(LineAdjArgs a) {
    using R = typename std::conditional<MIXED, float, double>::type;
    using GT = typename std::conditional<MIXED, float, double>::type;  // G element (g32 == MIXED)
    __shared__ long long s_item;
    __shared__ int64_t s_cnt[NTIER + 1];
    __shared__ R s_x[2][ADJ_SUB], s_t[2][ADJ_SUB];
    extern __shared__ __align__(16) unsigned char s_adj[];  // [2][ADJ_SUB][L] G, then [3][NJ][L] sums
    const int L = a.L, Lp = a.Lp;
    const int NJ = blockDim.x / L;
    const int l = threadIdx.x % L, jr = threadIdx.x / L;
    const bool active = jr < NJ;
    GT* s_g = reinterpret_cast<GT*>(s_adj);
    double* s_red = reinterpret_cast<double*>(s_adj + sizeof(GT) * 2 * ADJ_SUB * L);
    if (threadIdx.x == 0) {
        int64_t acc = 0;
        for (int t = NTIER - 1; t >= 0; t--) {
            s_cnt[NTIER - 1 - t] = acc;
            acc += int64_t(a.tier_start[t + 1] - a.tier_start[t]) * adj_chunks(t, a.nwl);
        }
        s_cnt[NTIER] = acc;
    }
    __syncthreads();
    const int64_t total = s_cnt[NTIER];
    const GT* G = static_cast<const GT*>(a.G);
    for (;;) {
        if (threadIdx.x == 0) s_item = (long long)atomicAdd(a.next, 1ull);
        __syncthreads();
        const int64_t it = s_item;
        __syncthreads();  // everyone has read s_item
        if (it >= total) break;
        int q = 0;
        while (it >= s_cnt[q + 1]) q++;
        const int tier = NTIER - 1 - q;
        const int64_t nch = adj_chunks(tier, a.nwl);
        const int64_t rel = it - s_cnt[q];
        const int64_t i = a.tier_idx[a.tier_start[tier] + rel / nch];
        const int64_t j0 = int64_t(a.lb[i]) + (rel % nch) * ADJ_CHUNK;
        const int64_t j1 = min(int64_t(a.ub[i]), j0 + ADJ_CHUNK - 1);
        if (j0 > j1) continue;  // uniform across the block
        const double wl0 = a.wl[i];
        const int64_t nj = j1 - j0 + 1;
        const int nsub = int((nj + ADJ_SUB - 1) / ADJ_SUB);
        // stage sub-chunk q of the item's wavelengths into buffer q & 1
        auto issue = [&](int sq) {
            if (sq < nsub) {
                const int64_t js = j0 + int64_t(sq) * ADJ_SUB;
                const int nw = int(min(int64_t(ADJ_SUB), j1 - js + 1));
                GT* dst = s_g + size_t(sq & 1) * ADJ_SUB * L;
                const GT* src = G + js * L;
                const int ne = nw * L;
                if ((L * int(sizeof(GT))) % 16 == 0) {  // every row start is 16-byte aligned
                    constexpr int V = 16 / int(sizeof(GT));
                    for (int e = threadIdx.x * V; e < ne; e += blockDim.x * V) cp_async16(dst + e, src + e);
                } else {
                    for (int e = threadIdx.x; e < ne; e += blockDim.x) {
                        if (MIXED) cp_async4(dst + e, src + e);
                        else cp_async8(dst + e, src + e);
                    }
                }
                if (threadIdx.x < nw) {
                    const double dx = fabs(a.wls[js + threadIdx.x] - wl0);
                    s_x[sq & 1][threadIdx.x] = R(dx);
                    s_t[sq & 1][threadIdx.x] = R(1.0 / (dx * dx));
                }
            }
            cp_async_commit();
        };
        AdjSums<MIXED, 3> cen;  // central evaluations: G H, G (a H_a + v H_v), G H_a
        AdjSums<MIXED, 3> mom;  // wing moments M1, M2, M3
        R s = R(1), av = R(0), c2 = R(1), xw = R(3.0e38);
        if (active) {
            if (MIXED) {
                const float4 p = reinterpret_cast<const float4*>(a.params)[i * Lp + l];
                s = R(rsqrtf(p.x));
                av = R(p.y);
            } else {
                const P64 p = reinterpret_cast<const P64*>(a.params)[i * Lp + l];
                s = R(p.inv_s);
                av = R(p.a);
            }
            c2 = R(1) / (s * s);                   // 2 sigma^2
            if (av <= R(0.2)) xw = R(5) / s;       // the wing starts at v = 5
        }
        issue(0);
        for (int sq = 0; sq < nsub; sq++) {
            issue(sq + 1);
            cp_async_wait_1();
            __syncthreads();
            const int nw = int(min(int64_t(ADJ_SUB), nj - int64_t(sq) * ADJ_SUB));
            const GT* gb = s_g + size_t(sq & 1) * ADJ_SUB * L;
            const R* xb = s_x[sq & 1];
            const R* tb = s_t[sq & 1];
            if (active) {
                R pc[3] = {0, 0, 0}, pm[3] = {0, 0, 0};
                for (int jj = jr; jj < nw; jj += NJ) {
                    const R g = R(gb[jj * L + l]);
                    const R x = xb[jj];
                    if (x >= xw) {
                        const R u = c2 * tb[jj];
                        const R gu = g * u, gu2 = gu * u;
                        pm[0] += gu;
                        pm[1] += gu2;
                        pm[2] += gu2 * u;
                    } else {
                        R d[3];
                        central_derivs<R>(av, x * s, d);
                        pc[0] += g * d[0];
                        pc[1] += g * d[1];
                        pc[2] += g * d[2];
                    }
                }
                cen.add(pc);
                mom.add(pm);
            }
            __syncthreads();  // buffer sq & 1 is refilled by issue(sq + 2)
        }
        // window sums of this thread: central + wing (from the moments)
        if (active) {
            const double k = 0.5641895835477563 * double(av);  // a / sqrt(pi)
            const double M1 = mom.get(0), M2 = mom.get(1), M3 = mom.get(2);
            const double wH = k * (M1 + 1.5 * M2 + 3.75 * M3);
            const double wA = 0.5641895835477563 * (M1 + 1.5 * M2 + 3.75 * M3);
            const double wX = wH - 2 * k * (M1 + 3 * M2 + 11.25 * M3);
            s_red[(0 * NJ + jr) * L + l] = cen.get(0) + wH;
            s_red[(1 * NJ + jr) * L + l] = cen.get(1) + wX;
            s_red[(2 * NJ + jr) * L + l] = cen.get(2) + wA;
        }
        __syncthreads();
        if (active && jr == 0) {
            double* dp = a.dpar + (i * Lp + l) * 3;
            for (int k = 0; k < 3; k++) {
                double t = 0.0;
                for (int r = 0; r < NJ; r++) t += s_red[(k * NJ + r) * L + l];
                atomicAdd(dp + k, t);
            }
        }
        __syncthreads();  // s_red is rewritten by the next item
    }
}

// Dynamic shared memory of line_adj_kernel: two staged G buffers and the partial sums.
inline size_t adj_smem(int L, int threads, bool mixed) {
    return (mixed ? sizeof(float) : sizeof(double)) * 2 * ADJ_SUB * size_t(L) + sizeof(double) * 3 * size_t(threads);
}

// Threads per block of line_adj_kernel for L layers: L * NJ, the smallest multiple of 32 that
// is at least 128 (at most 512).
inline int adj_threads(int L) {
    int nj = 1;
    while (nj * L < 512 && ((nj * L) % 32 != 0 || nj * L < 128)) nj++;
    if (nj * L > 512) nj = 512 / L;
    return nj * L;
}

// Chain rule of the per-(line, layer) prologue (line_absorption.jl:86-106), FP64, one warp per
// line.  dpar holds the window sums {sum G H, sum G (a H_a + v H_v), sum G H_a}; with
// phi = amp s / sqrt(pi) H(gamma s, |dl| s) and s = 1/(sigma sqrt 2):
//   dL/damp = s/sqrt(pi) sum G H,  dL/ds = amp/sqrt(pi) (sum G H + sum G (a H_a + v H_v)),
//   dL/dgamma = amp s^2/sqrt(pi) sum G H_a,  dL/dsigma = -s/sigma dL/ds.
struct LineAdjOut {
    double *dT, *dne, *dnv, *dxi, *dnU;  // [L], [L], [L], [L], [S][L] (+=); any may be null
    double* dloggf;                       // [n] (written) or null
};

__global__ void __launch_bounds__(256) line_adj_prologue_kernel(LinesDev ln, LayersDev lay, const LayerConst* lc,
                                                                const double* dpar, int32_t Lp, LineAdjOut out,
                                                                const MathTables* math) {
    __shared__ MathTables s_math;
    extern __shared__ double s_acc[];  // [4][L] per-layer sums of the block, then [S][L]
    load_math_tables(s_math, math);
    const int L = lay.L, S = lay.S;
    for (int e = threadIdx.x; e < (4 + S) * L; e += blockDim.x) s_acc[e] = 0.0;
    __syncthreads();
    const int64_t i = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    double glog = 0.0;
    if (i < ln.n) {
        const LineConst q = line_const(ln, i);
        for (int l = lane; l < L; l += 32) {
            const double* d = dpar + (i * Lp + l) * 3;
            if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0) continue;  // outside every window
            const double T = lay.T[l], xi = lay.xi[l];
            const LayerConst c = lc[l];
            // sigma (:86, line_absorption.jl:190)
            const double var = KBOLTZ_CGS * T / q.m + (xi * xi) / 2;
            const double sigma = q.wl * sqrt(var) / C_CGS;
            const double dsig_dT = sigma * (KBOLTZ_CGS / q.m) / (2 * var);
            const double dsig_dxi = sigma * xi / (2 * var);
            // gamma (:90-99)
            double dG_dT = 0.0, dG_dne = 0.0, dG_dnv = 0.0;
            if (!q.mol) {
                const double st = q.gstark * c.stark6;
                double vdw, ex;
                if (q.v2 == -1) {
                    vdw = q.v1 * c.vdw3;
                    ex = 0.3;
                } else {
                    const double invmu = 1 / (1.008 * AMU_CGS) + 1 / q.m;
                    const double vbar = sqrt(8 * KBOLTZ_CGS * T / PI * invmu);
                    vdw = q.abo_pre * pow(vbar / 1e6, 1 - q.v2);
                    ex = (1 - q.v2) / 2;
                }
                dG_dne = st;
                dG_dnv = vdw;
                dG_dT = lay.ne[l] * st / (6 * T) + lay.n_eff_vdW[l] * vdw * ex / T;
            }
            // amplitude (:101-106)
            const double e1 = fexp64(-c.beta * q.El, s_math), e2 = fexp64(-c.beta * q.E_upper, s_math);
            const double levels = e1 - e2;
            const double nU = lay.n_div_U[int64_t(q.sp) * L + l];
            const double amp = q.strength * levels * nU;
            const double dlev_dT = c.beta / T * (q.El * e1 - q.E_upper * e2);
            // cotangents of (amp, sigma, gamma)
            const double s = 1 / (sigma * SQRT_2);
            const double g_amp = s / SQRT_PI * d[0];
            const double g_s = amp / SQRT_PI * (d[0] + d[1]);
            const double g_gam = amp * s * s / SQRT_PI * d[2];
            const double g_sig = -s / sigma * g_s;
            atomicAdd(s_acc + 0 * L + l, g_amp * q.strength * nU * dlev_dT + g_sig * dsig_dT + g_gam * q.wl2c * dG_dT);
            atomicAdd(s_acc + 1 * L + l, g_gam * q.wl2c * dG_dne);
            atomicAdd(s_acc + 2 * L + l, g_gam * q.wl2c * dG_dnv);
            atomicAdd(s_acc + 3 * L + l, g_sig * dsig_dxi);
            atomicAdd(s_acc + (4 + q.sp) * L + l, g_amp * q.strength * levels);
            glog += g_amp * amp * 2.302585092994046;  // d amp / d log gf = amp ln 10
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) glog += __shfl_xor_sync(0xffffffffu, glog, o);
        if (lane == 0 && out.dloggf) out.dloggf[i] = glog;
    }
    __syncthreads();
    double* dst[4] = {out.dT, out.dne, out.dnv, out.dxi};
    for (int e = threadIdx.x; e < (4 + S) * L; e += blockDim.x) {
        const double v = s_acc[e];
        if (v == 0.0) continue;
        const int r = e / L, l = e - r * L;
        double* p = r < 4 ? dst[r] : out.dnU;
        if (p) atomicAdd(p + (r < 4 ? l : int64_t(r - 4) * L + l), v);
    }
}

// Hydrogen-line opacity is layer-local (each layer's row depends on that layer's T, n_e,
// n(H I), n(He I), U(H I), xi only), so its Jacobian is block diagonal: per layer and input,
// d alpha_H[l, :]/dp_l is a central difference of two FP64 evaluations with every layer
// perturbed at once, and the cotangent is its contraction with G.
__global__ void hydro_fd_contract_kernel(const void* G, int32_t g32, const double* ap, const double* am,
                                         const double* h, int64_t nwl, int32_t L, double* out) {
    __shared__ double s_acc[RTA_LMAX];
    for (int l = threadIdx.x; l < L; l += blockDim.x) s_acc[l] = 0.0;
    __syncthreads();
    const int64_t n = nwl * L;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x) {
        const double d = ap[e] - am[e];
        if (d == 0.0) continue;
        const int l = int(e % L);
        const double g = g32 ? double(static_cast<const float*>(G)[e]) : static_cast<const double*>(G)[e];
        atomicAdd(s_acc + l, g * d);
    }
    __syncthreads();
    for (int l = threadIdx.x; l < L; l += blockDim.x)
        if (s_acc[l] != 0.0) atomicAdd(out + l, s_acc[l] / (2 * h[l]));
}

}  // namespace korg
