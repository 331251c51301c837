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
    const double u = recip64(x);
    const double R = 1 + (-2 + (6 + (-24 + 120 * u) * u) * u) * u;
    const double dR = -2 + (12 + (-72 + 480 * u) * u) * u;
    return -e2 - ex * u * u * (R + u * dR);
}

// E2(x) as expint2_ex evaluates it, with d/dx of the same branch (expint2_deriv) from one
// logarithm: for x < 1.1 both need ln x.
__device__ __forceinline__ double expint2_and_deriv(double x, double ex, const MathTables& t, double& d2) {
    if (x < 1.1 && x != 0) {  // E2 = 1 + x (ln x + EM - 1) + x Q(x)
        const double EM = 0.57721566490153286060651209008240243104215933593992;
        const double c2 = 0.08333333333333333, c3 = -0.013888888888888888, c4 = 0.0020833333333333333;
        const double lg = flog64(x, t);
        const double Q = (-0.5 + (c2 + (c3 + c4 * x) * x) * x) * x;
        const double dQ = -0.5 + (2 * c2 + (3 * c3 + 4 * c4 * x) * x) * x;
        d2 = lg + EM + Q + x * dQ;
        return 1 + ((lg + EM - 1) + Q) * x;
    }
    const double e2 = expint2_ex(x, ex, t);
    d2 = expint2_deriv(x, e2, ex, t);
    return e2;
}

// One transfer pass over the column `al` (global or shared) with cotangent w of 2 pi I unit:
// writes dL/dalpha of the pass into gout[l], adds dL/dS into c.Sbar and dL/dalpha_ref into
// s_daref (shared, atomically).  s_iaref = 1 / alpha_ref.  No FP64 division: one Newton
// reciprocal of each segment's dtau (recip64) serves its three quotients.
__device__ __forceinline__ void rt_adj_pass(const RtaCol& c, const double* al, double w, const double* s_fac,
                                            const double* s_dlt, const double* s_iaref, int L, const MathTables& mt,
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
            double d2 = 0.0;  // tau_0 = 0 is not a variable
            const double e2 = l == 0 ? 1.0 : expint2_and_deriv(t, ex, mt, d2);
            c.ex[l] = ex;
            c.e2[l] = e2;
            c.d2[l] = d2;
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
        const double iD = recip64(D);
        const double m = (Sb - Sa) * iD;
        const double bb = Sa - m * ta_;
        const double Pb = 0.5 * ((tb_ * c.e2[l] - c.ex[l]) - (ta_ * c.e2[l - 1] - c.ex[l - 1]));
        const double Pm = (1.0 / 3.0) * ((tb_ * tb_ * c.e2[l] - c.ex[l] * (tb_ + 1)) -
                                         (ta_ * ta_ * c.e2[l - 1] - c.ex[l - 1] * (ta_ + 1)));
        const double Q = Pm - ta_ * Pb;  // total derivative through m (b depends on m)
        const double Ctb = dC(tb_, c.e2[l], c.d2[l], c.ex[l], m, bb);
        const double Cta = l == 1 ? 0.0 : dC(ta_, c.e2[l - 1], c.d2[l - 1], c.ex[l - 1], m, bb);
        const double QD = Q * iD, QmD = QD * m;
        c.tb[l] = w * (Ctb - QmD);
        c.ta[l - 1] = w * (-Cta - Pb * m + QmD);
        c.sb[l] = w * QD;
        c.sa[l - 1] = w * (Pb - QD);
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
        if (ibar != 0.0) atomicAdd(s_daref + l, -ibar * c.ib[l] * s_iaref[l]);  // fac = tau_ref/alpha_ref
        c.Sbar[l] += c.sb[l] + c.sa[l];
    }
    __syncwarp();
}

__global__ void __launch_bounds__(32 * RTA_WARPS) rt_adjoint_kernel(RtAdjArgs a) {
    __shared__ MathTables s_math;
    __shared__ double s_fac[RTA_LMAX], s_dlt[RTA_LMAX], s_iaref[RTA_LMAX], s_iT[RTA_LMAX], s_ikT[RTA_LMAX];
    __shared__ double s_dT[RTA_LMAX], s_dar[RTA_LMAX];
    extern __shared__ double s_cols[];  // [warps][RTA_ARRAYS][L + 1]
    load_math_tables(s_math, a.math);
    const int L = a.L;
    for (int l = threadIdx.x; l < L; l += blockDim.x) {
        s_fac[l] = a.tau_ref[l] / a.alpha_ref[l];
        s_dlt[l] = l == 0 ? 0.0 : log(a.tau_ref[l]) - log(a.tau_ref[l - 1]);
        s_iaref[l] = 1.0 / a.alpha_ref[l];
        s_iT[l] = 1.0 / a.T[l];
        s_ikT[l] = 1.0 / (KBOLTZ_CGS * a.T[l]);  // as the forward transfer forms it
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
        const double ipre = recip64(pre);
        for (int l = lane; l < L; l += 32) {
            c.S[l] = planck_t(pre, hcw, s_ikT[l], s_math);  // the forward transfer's source function
            c.Sbar[l] = 0.0;
        }
        __syncwarp();
        rt_adj_pass(c, a.alpha + j * L, wf, s_fac, s_dlt, s_iaref, L, s_math, c.g, s_dar, lane);
        if (two) {
            // continuum-only column (src/synthesize.jl:287-291), as the forward interpolates it
            const KnotPos kp = knot_pos(a.cn.knots, a.cn.nk, wl);
            for (int l = lane; l < L; l += 32) c.col[l] = knot_eval(a.cn.vals + int64_t(l) * a.cn.nk, a.cn.nk, kp);
            __syncwarp();
            rt_adj_pass(c, c.col, wc, s_fac, s_dlt, s_iaref, L, s_math, c.gc, s_dar, lane);
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
            const double x = hcw * s_ikT[l];
            const double d = c.Sbar[l] * B * (x * s_iT[l]) * (1.0 + B * ipre);
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
constexpr int ADJ_CHUNK = 16384;  // wavelengths per chunk; an item is (chunk, line)

struct LineAdjArgs {
    const void* G;            // [nwl][L] opacity cotangent (float when g32)
    int32_t g32;
    const double* wls;
    const float2* wl2;        // wavelengths as FP32 (hi, lo) pairs (mixed)
    int64_t nwl;
    int32_t L, Lp;
    const double* wl;         // line centres
    const void* params;       // forward constants [n][Lp]: float4 {2 sigma^2, a, w, scale} or P64
    const int32_t *lb, *ub;
    const int32_t* tier_idx;  // lines with non-empty windows, by width tier
    const int32_t* ilo;       // [npairs] first candidate of each (chunk, tier), in the tier lists
    const int64_t* ipre;      // [npairs + 1] items before each (chunk, tier)
    int32_t npairs;
    double* dpar;             // out [n][Lp][3] (+=): window sums of G H, G (a H_a + v H_v), G H_a
    unsigned long long* next; // item counter (zero before the launch)
    int32_t Ls;               // largest staged row stride (elements)
    int32_t bulk;             // rows of G start on 16-byte boundaries: one bulk copy per stage
    int* err;                 // set to 1 when a wait for staged data runs past its limit
    int32_t sub;              // wavelengths per stage
};

// The items of line_adj_kernel, chunk-major so that the blocks running at any time share one
// chunk of G in L2: pair p = k NTIER + t lists the lines of tier t whose centre index lies within
// the tier's widest half-width of chunk k (a contiguous run of the tier list, which keeps list
// order).  One block: the per-tier widest half-width, two binary searches per pair, an
// exclusive scan of the counts.  Unsorted lists take whole tiers.
__global__ void __launch_bounds__(1024) adj_items_kernel(const int32_t* tier_idx, const int32_t* tier_ci,
                                                         const int32_t* tmeta, const int32_t* lb, const int32_t* ub,
                                                         int64_t nwl, int32_t* ilo, int64_t* ipre) {
    __shared__ int s_hw[NTIER];
    __shared__ int64_t s_part[1024];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int nck = int((nwl + ADJ_CHUNK - 1) / ADJ_CHUNK), np = nck * NTIER;
    if (tid < NTIER) s_hw[tid] = 0;
    __syncthreads();
    const int n = tmeta[NTIER];
    for (int p = tid; p < n; p += nt) {
        int t = 0;
        while (t < NTIER - 1 && p >= tmeta[t + 1]) t++;
        const int i = tier_idx[p], c = tier_ci[p];
        atomicMax(&s_hw[t], max(c - lb[i], ub[i] - c));
    }
    __syncthreads();
    const bool unsorted = tmeta[NTIER + 1] != 0;
    const int seg = (np + nt - 1) / nt;
    const int p0 = min(tid * seg, np), p1 = min(p0 + seg, np);
    int64_t sum = 0;
    for (int p = p0; p < p1; p++) {
        const int t = p % NTIER;
        const int64_t k0 = int64_t(p / NTIER) * ADJ_CHUNK;
        int64_t lo = tmeta[t], hi = tmeta[t + 1];
        if (!unsorted && hi > lo) {
            const int64_t cmin = k0 - s_hw[t] - 1, cmax = k0 + ADJ_CHUNK + s_hw[t];
            const int32_t vmin = int32_t(cmin < INT32_MIN ? int64_t(INT32_MIN) : cmin);
            const int32_t vmax = int32_t(cmax > INT32_MAX ? int64_t(INT32_MAX) : cmax);
            const int64_t l0 = lower_bound_i32(tier_ci, lo, hi, vmin);
            hi = upper_bound_i32(tier_ci, l0, hi, vmax);
            lo = l0;
        }
        ilo[p] = int32_t(lo);
        ipre[p] = hi - lo;  // count, turned into the prefix below
        sum += hi - lo;
    }
    s_part[tid] = sum;
    __syncthreads();
    for (int o = 1; o < nt; o <<= 1) {
        const int64_t v = tid >= o ? s_part[tid - o] : 0;
        __syncthreads();
        s_part[tid] += v;
        __syncthreads();
    }
    int64_t run = s_part[tid] - sum;
    for (int p = p0; p < p1; p++) {
        const int64_t c = ipre[p];
        ipre[p] = run;
        run += c;
    }
    if (tid == nt - 1) ipre[np] = s_part[nt - 1];
}

// Wavelengths as FP32 (hi, lo) pairs: |wl - centre| = (hi - chi) + (lo - clo) in FP32 keeps the
// full offset accuracy without FP64 arithmetic.
__global__ void wl_pairs_kernel(const double* w, int64_t n, float2* out) {
    const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j < n) {
        const float hi = float(w[j]);
        out[j] = make_float2(hi, float(w[j] - double(hi)));
    }
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

// mbarrier + bulk-copy (TMA) helpers.  Every wait is bounded: mbar_wait gives up after 2^22
// polls (each try_wait suspends the thread for a while), and the caller reports the timeout.
__device__ __forceinline__ unsigned smem_u32(const void* p) { return static_cast<unsigned>(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// one contiguous global -> shared copy by the bulk-copy engine; completes bytes on bar
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_u32(bar)) : "memory");
}
// arrive on bar once this thread's earlier cp.async copies have landed (counted in the init count)
__device__ __forceinline__ void cp_async_mbar_arrive(uint64_t* bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int limit = 1 << 22) {
    for (int k = 0; k < limit; k++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// A bounded wait on an mbarrier that nothing arrives on: exercises the timeout path of the
// staged-data waits (the error word is set and the kernel returns) without a fault or hang.
__global__ void wait_timeout_selftest_kernel(int* err, int limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    const bool ok = mbar_wait(&bar, 0u, limit);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) *reinterpret_cast<volatile int*>(err) = 1;
}

// Far-Lorentz branch of voigt_hjerting (line_absorption.jl:305-308: a > 1.4, or a > 0.2 with
// a + v >= 3.2) with its derivatives in closed form: H, X = a H_a + v H_v and A = H_a.  With
// r^2 = v^2/a^2 (degree 0) and au = 1/(sqrt2 a (1 + r^2)) (degree -1), H = C au (1 + P b + Q b^2),
// b = au^2, P = 3r^2 - 1, Q = 15r^4 - 30r^2 + 2:  X = -C au (1 + 3P b + 5Q b^2), and
// A = C au/a [w (1 + P b + Q b^2) + b (-6r^2 + 2P w) + b^2 (-60 r^2 (r^2 - 1) + 4Q w)] with
// w = (r^2 - 1)/(r^2 + 1).
template <class R>
__device__ __forceinline__ void far_lorentz_r2(R r2, R ia, R& H, R& X, R& A) {
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
template <class R>
__device__ __forceinline__ void far_lorentz_d(R a, R v, R& H, R& X, R& A) {
    const R ia = recip(a);
    far_lorentz_r2<R>(v * v * ia * ia, ia, H, X, A);
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

constexpr int ADJ_SUB = 96;     // wavelengths of G staged in shared memory per stage
constexpr int ADJ_STAGES = 3;   // ring of staged blocks: one barrier per stage, two in flight
static_assert(ADJ_SUB % 32 == 0, "the stage table is written by whole warps");

// One staged wavelength: x = |dl|, t1 = cref / dl^2 and its square and cube (cref = 2 sigma^2 of
// the item's line in layer 0, which keeps t1^3 within FP32 range over any window).
template <class R>
struct __align__(4 * sizeof(R)) AdjW {
    R x, t1, t2, t3;
};

// One block per item (a line and one ADJ_CHUNK-wavelength chunk of the grid that its window
// meets); items run chunk-major, so the blocks at work share a chunk of G in L2.
//
// Pipeline.  The last warp of the block is the producer: for every stage (ADJ_SUB wavelengths
// of the item) it waits until the ring slot is empty, has the bulk-copy engine fetch the stage's
// G rows (ADJ_SUB x L values, one contiguous block of global memory) with one cp.async.bulk
// completing on the slot's "full" mbarrier, writes the stage's wavelength table AdjW from
// wavelengths it loaded one stage earlier, and arrives on "full".  The other warps consume: wait
// for "full", sum, and arrive on the slot's "empty" mbarrier.  No block-wide barrier separates
// stages, so warps drift apart by up to ADJ_STAGES stages.  When rows are not 16-byte multiples
// the producer copies elements with cp.async into rows padded to Ls (chosen so that the
// NJ-strided reads below hit distinct banks) and each lane arrives through
// cp.async.mbarrier.arrive.  Every wait is bounded; a wait that runs out sets the error word,
// and the block finishes the item without waiting further and stops.
//
// Work balance.  A layer with a <= 0.2 ("wing layer") spends most of a wide window in the
// asymptotic wing, three FMAs per evaluation; a layer with a > 0.2 has no asymptotic wing and
// evaluates the far-Lorentz (or Harris) branch at every wavelength, several times the work.  Per
// item the block lists the a > 0.2 layers first and gives each NJs consumer threads, then each
// wing layer NJf (powers of two, NJs >= NJf, chosen so that both kinds finish together);
// thread (layer, jr) walks every NJ-th staged wavelength, and the NJ partial sums of a layer
// meet by warp shuffles.
//
// In the asymptotic wing (a <= 0.2, v >= 5) H = a/sqrt(pi) u (1 + 1.5u + 3.75u^2) with
// u = 1/v^2 = rho t1 (rho = 2 sigma_l^2 / cref), so the three window sums follow from the
// moments M_k = rho^k sum G t1^k, k = 1..3:  sum G H = a/sqrt(pi) (M1 + 1.5 M2 + 3.75 M3),
// sum G H_a = that / a,  sum G (a H_a + v H_v) = sum G H - 2 a/sqrt(pi) (M1 + 3 M2 + 11.25 M3).
// A stage whose nearest wavelength is already in the layer's wing takes a branch-free loop, and
// so does a stage entirely in the far-Lorentz branch.  Elsewhere central_derivs differentiates
// the far-Lorentz branch in closed form and the Harris branches with dual numbers.
// Mixed form: |dl| beyond which a far-Lorentz layer (a > 0.2) is given by the cubic series of
// its branch to FP32 rounding (far_lorentz_cubic_rmin), as in the forward tiles: the wing
// moments then serve it too.  In u = 1/v^2 both wing forms are
//   H = (c1 u + c2 u^2 + c3 u^3) / sqrt(pi),
// asymptotic branch (a <= 0.2): c = (a, 1.5 a, 3.75 a); far-Lorentz series (w = 1/r^2 = a^2 u):
// c = (a, 1.5 a - a^3, 3.75 a - 5 a^3 + a^5).
__device__ __forceinline__ float adj_fl_cubic_x(float a, float s) {
    const float xfl = a <= 1.4f ? (3.2f - a) / s : 0.f;
    return fmaxf(xfl, far_lorentz_cubic_rmin(a) * a / s) * 1.0001f;
}

template <bool MIXED>
__global__ void __launch_bounds__(512, MIXED ? 2 : 1) line_adj_kernel(LineAdjArgs a) {
    using R = typename std::conditional<MIXED, float, double>::type;
    using GT = typename std::conditional<MIXED, float, double>::type;  // G element (g32 == MIXED)
    using WP = typename std::conditional<MIXED, float2, double>::type; // a wavelength as loaded
    using W = AdjW<R>;
    constexpr int MAXW = 16;                 // warps per block (512 threads)
    constexpr int PER = ADJ_SUB / 32;        // table entries per producer lane
    __shared__ long long s_item;
    __shared__ int64_t s_i, s_j0, s_j1;
    __shared__ float s_dmin;                 // mixed: |dl| from the line centre to the item's nearest wavelength
    __shared__ __align__(8) uint64_t s_full[ADJ_STAGES], s_empty[ADJ_STAGES];
    __shared__ W s_w[ADJ_STAGES][ADJ_SUB];
    __shared__ R s_xmin[ADJ_STAGES];
    __shared__ int s_wslow[MAXW];            // a > 0.2 layers per warp of layer indices
    __shared__ int s_ns, s_lnf, s_lns, s_Ls;
    __shared__ volatile int s_abort;
    extern __shared__ __align__(16) unsigned char s_adj[];  // [ADJ_STAGES][ADJ_SUB][<= Lsmax] G, then [L] order
    const int L = a.L, Lp = a.Lp;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int PW = nwarps - 1;               // the producer warp
    const int TC = PW * 32;                  // consumer threads
    GT* s_g = reinterpret_cast<GT*>(s_adj);
    const int SUB = a.sub;                   // wavelengths per stage (<= ADJ_SUB, a multiple of 32)
    int* s_order = reinterpret_cast<int*>(s_adj + sizeof(GT) * ADJ_STAGES * SUB * a.Ls);
    const int64_t total = a.ipre[a.npairs];
    const GT* G = static_cast<const GT*>(a.G);
    const bool bulk = a.bulk != 0;
    if (threadIdx.x == 0) {
        for (int b = 0; b < ADJ_STAGES; b++) {
            mbar_init(&s_full[b], bulk ? 2u : 33u);  // expect_tx + table arrive, or 32 copy lanes + table
            mbar_init(&s_empty[b], unsigned(PW));    // one arrive per consumer warp
        }
        mbar_fence_init();
        s_abort = 0;
    }
    __syncthreads();
    int64_t g0 = 0;      // stages this block has run before the current item (ring slot = stage mod ADJ_STAGES)
    int64_t issued = 0;  // producer warp: stages whose copies it has issued (all items so far)
    int pcur = 0;        // thread 0: the (chunk, tier) pair of the last item (items arrive in increasing order)
    // bounded wait; a wait that runs out marks the block aborted and reports it.  Returns false
    // once the block is aborted (the caller then stops waiting).
    auto wait = [&](uint64_t* bar, unsigned parity) -> bool {
        if (s_abort) return false;
        if (!mbar_wait(bar, parity)) {
            s_abort = 1;
            *reinterpret_cast<volatile int*>(a.err) = 1;
            return false;
        }
        return true;
    };
    for (;;) {
        if (threadIdx.x == 0) {  // the next item whose window meets its chunk
            for (;;) {
                const long long it = (long long)atomicAdd(a.next, 1ull);
                s_item = it;
                if (it >= total) break;
                while (a.ipre[pcur + 1] <= it) pcur++;
                const int64_t i = a.tier_idx[a.ilo[pcur] + (it - a.ipre[pcur])];
                const int64_t k0 = int64_t(pcur / NTIER) * ADJ_CHUNK;
                s_i = i;
                s_j0 = max(int64_t(a.lb[i]), k0);
                s_j1 = min(int64_t(a.ub[i]), k0 + ADJ_CHUNK - 1);
                if (s_j0 <= s_j1) {
                    const double c = a.wl[i], lo = a.wls[s_j0], hi = a.wls[s_j1];
                    s_dmin = float(c < lo ? lo - c : (c > hi ? c - hi : 0.0));
                    break;
                }
            }
        }
        __syncthreads();
        if (s_item >= total || s_abort) {
            // An aborted block may have bulk copies in flight into its ring (the producer stops
            // issuing once it sees the abort, but the consumers stopped waiting for the last
            // stages).  Before the block's shared memory is released, the producer waits, with
            // the same bound, for the full barriers of the last stages it issued; earlier stages
            // were waited for by the consumers before the abort.
            if (s_abort && warp == PW && lane == 0)
                for (int64_t gq = issued > ADJ_STAGES ? issued - ADJ_STAGES : 0; gq < issued; gq++)
                    mbar_wait(&s_full[gq % ADJ_STAGES], unsigned((gq / ADJ_STAGES) & 1));
            break;
        }
        const int64_t i = s_i, j0 = s_j0, j1 = s_j1;
        // classify the layers: a > 0.2 ("slow") or not, counted per warp of layer indices; in
        // the mixed form a far-Lorentz layer whose cubic regime covers the whole item costs what
        // a wing layer does and counts as one
        bool slow_l = false;
        unsigned ball = 0;
        if (warp * 32 < L) {
            if (threadIdx.x < L) {
                if (MIXED) {
                    const float4 p = reinterpret_cast<const float4*>(a.params)[i * Lp + threadIdx.x];
                    slow_l = p.y > 0.2f && adj_fl_cubic_x(p.y, rsqrtf(p.x)) > s_dmin;
                } else {
                    slow_l = reinterpret_cast<const P64*>(a.params)[i * Lp + threadIdx.x].a > 0.2;
                }
            }
            ball = __ballot_sync(0xffffffffu, slow_l);
            if (lane == 0) s_wslow[warp] = __popc(ball);
        }
        __syncthreads();  // the item read by all; s_wslow complete
        if (threadIdx.x < L) {
            int before = 0;
            for (int w = 0; w < warp; w++) before += s_wslow[w];
            const int sr = before + __popc(ball & ((1u << lane) - 1u));  // slow layers below this one
            int ns = 0;
            for (int w = 0; w * 32 < L; w++) ns += s_wslow[w];
            s_order[slow_l ? sr : ns + (int(threadIdx.x) - sr)] = int(threadIdx.x);
            if (threadIdx.x == 0) {
                // consumer-thread shares: slow layers NJs = 2^lns, wing layers NJf = 2^lnf,
                // minimising the larger of 1/NJf and 6/NJs (the evaluation cost ratio)
                const int nf = L - ns;
                int bf = 0, bs = 0;
                float best = 3.0e38f;
                for (int lf = 0; lf <= 3; lf++)
                    for (int ls = lf; ls <= 5; ls++) {
                        if (nf * (1 << lf) + ns * (1 << ls) > TC) continue;
                        const float c = fmaxf(nf ? 1.0f / float(1 << lf) : 0.f, ns ? 6.0f / float(1 << ls) : 0.f);
                        if (c < best) { best = c; bf = lf; bs = ls; }
                    }
                s_ns = ns;
                s_lnf = bf;
                s_lns = bs;
                // staged row stride: dense for bulk copies; else, for NJf >= 2, Ls = 32/NJf
                // (mod 64/NJf) spreads a wing warp's reads over 32 banks
                const int nj = 1 << bf;
                int Ls = (L + 3) & ~3;
                if (nj >= 2)
                    while (Ls % (64 / nj) != 32 / nj) Ls += 4;
                s_Ls = bulk ? L : Ls;
            }
        }
        __syncthreads();
        const int ns = s_ns, lnf = s_lnf, lns = s_lns, Ls = s_Ls;
        const int64_t nj = j1 - j0 + 1;
        const int nsub = int((nj + SUB - 1) / SUB);
        const double wl0 = a.wl[i];
        const double cref = MIXED ? double(reinterpret_cast<const float4*>(a.params)[i * Lp].x)
                                  : reinterpret_cast<const P64*>(a.params)[i * Lp].c;
        if (warp == PW) {
            // ---------------- producer: G rows by the bulk-copy engine, the wavelength table
            const float chi = float(wl0), clo = float(wl0 - double(chi));
            const R cref_r = R(cref);
            auto load_wl = [&](int sq, WP* v) {
#pragma unroll
                for (int k = 0; k < PER; k++) {
                    const int64_t j = min(j0 + int64_t(sq) * SUB + lane + 32 * k, j1);
                    if constexpr (MIXED) v[k] = a.wl2[j];
                    else v[k] = a.wls[j];
                }
            };
            WP pf[PER];
            load_wl(0, pf);
            for (int sq = 0; sq < nsub; sq++) {
                const int64_t gq = g0 + sq;
                const int b = int(gq % ADJ_STAGES);
                bool ok = true;
                if (gq >= ADJ_STAGES) ok = wait(&s_empty[b], unsigned((gq / ADJ_STAGES - 1) & 1));
                // warp-uniform: no copy is issued once any wait has failed or the block is aborted
                if (__any_sync(0xffffffffu, !ok || s_abort != 0)) break;
                issued = gq + 1;
                const int64_t js = j0 + int64_t(sq) * SUB;
                const int nw = int(min(int64_t(SUB), j1 - js + 1));
                GT* dst = s_g + size_t(b) * SUB * Ls;
                const GT* src = G + js * L;
                if (bulk) {
                    if (lane == 0) {
                        const unsigned bytes = unsigned(nw) * unsigned(L) * unsigned(sizeof(GT));
                        mbar_expect_tx(&s_full[b], bytes);
                        bulk_load(dst, src, bytes, &s_full[b]);
                    }
                } else {
                    for (int r = 0; r < nw; r++)
                        for (int c = lane; c < L; c += 32) {
                            if (MIXED) cp_async4(dst + r * Ls + c, src + int64_t(r) * L + c);
                            else cp_async8(dst + r * Ls + c, src + int64_t(r) * L + c);
                        }
                    cp_async_mbar_arrive(&s_full[b]);
                }
                WP cur[PER];
#pragma unroll
                for (int k = 0; k < PER; k++) cur[k] = pf[k];
                if (sq + 1 < nsub) load_wl(sq + 1, pf);  // lands while this stage's table is written
                R m = R(3.0e38);
#pragma unroll
                for (int k = 0; k < PER; k++) {
                    const int e = lane + 32 * k;
                    R x;
                    if constexpr (MIXED) x = fabsf((cur[k].x - chi) + (cur[k].y - clo));
                    else x = fabs(cur[k] - wl0);
                    const R t1 = fast_div(cref_r, x * x);
                    if (e < nw) {
                        s_w[b][e] = W{x, t1, t1 * t1, t1 * t1 * t1};
                        m = x < m ? x : m;
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const R q = __shfl_xor_sync(0xffffffffu, m, o);
                    m = q < m ? q : m;
                }
                if (lane == 0) s_xmin[b] = m;
                __syncwarp();
                if (lane == 0) mbar_arrive(&s_full[b]);
            }
        } else {
            // ---------------- consumers
            int l = -1, lnj = 0;
            {
                const int slot = int(threadIdx.x), cs = ns << lns;
                if (slot < cs) {
                    l = s_order[slot >> lns];
                    lnj = lns;
                } else if (slot - cs < ((L - ns) << lnf)) {
                    l = s_order[ns + ((slot - cs) >> lnf)];
                    lnj = lnf;
                }
            }
            const bool active = l >= 0;
            const int NJ = 1 << lnj, jr = int(threadIdx.x) & (NJ - 1);
            AdjSums<MIXED, 3> cen;  // central evaluations: G H, G (a H_a + v H_v), G H_a
            AdjSums<MIXED, 3> mom;  // wing sums S_k = sum G t1^k
            R s = R(1), av = R(0), xw = R(3.0e38);
            double rho = 1.0;
            if (active) {
                double c2;
                if (MIXED) {
                    const float4 p = reinterpret_cast<const float4*>(a.params)[i * Lp + l];
                    s = R(rsqrtf(p.x));
                    av = R(p.y);
                    c2 = double(p.x);
                } else {
                    const P64 p = reinterpret_cast<const P64*>(a.params)[i * Lp + l];
                    s = R(p.inv_s);
                    av = R(p.a);
                    c2 = p.c;
                }
                rho = c2 / cref;
                if (av <= R(0.2)) xw = R(5) / s;  // the wing starts at v = 5
                else if (MIXED) xw = R(adj_fl_cubic_x(float(av), float(s)));  // far-Lorentz cubic regime
            }
            const R ia = recip(av), k1 = s * ia;  // far Lorentz: r = v / a = x s / a
            for (int sq = 0; sq < nsub; sq++) {
                const int64_t gq = g0 + sq;
                const int b = int(gq % ADJ_STAGES);
                wait(&s_full[b], unsigned((gq / ADJ_STAGES) & 1));
                const int nw = int(min(int64_t(SUB), nj - int64_t(sq) * SUB));
                const GT* gb = s_g + size_t(b) * SUB * Ls + (active ? l : 0);
                const W* wb = s_w[b];
                if (active) {
                    const R xmin = s_xmin[b];
                    R pm[3] = {0, 0, 0};
                    if (xmin >= xw) {  // every staged wavelength in the layer's cubic regime
#pragma unroll 4
                        for (int jj = jr; jj < nw; jj += NJ) {
                            const R g = R(gb[jj * Ls]);
                            const W w = wb[jj];
                            pm[0] += g * w.t1;
                            pm[1] += g * w.t2;
                            pm[2] += g * w.t3;
                        }
                    } else if (av > R(0.2) && (av > R(1.4) || av + xmin * s >= R(3.2))) {
                        // every staged wavelength in the far-Lorentz branch
                        R pc[3] = {0, 0, 0};
#pragma unroll 2
                        for (int jj = jr; jj < nw; jj += NJ) {
                            const R g = R(gb[jj * Ls]);
                            const R r = wb[jj].x * k1;
                            R H, X, A;
                            far_lorentz_r2<R>(r * r, ia, H, X, A);
                            pc[0] += g * H;
                            pc[1] += g * X;
                            pc[2] += g * A;
                        }
                        cen.add(pc);
                    } else {
                        R pc[3] = {0, 0, 0};
                        for (int jj = jr; jj < nw; jj += NJ) {
                            const R g = R(gb[jj * Ls]);
                            const W w = wb[jj];
                            if (w.x >= xw) {
                                pm[0] += g * w.t1;
                                pm[1] += g * w.t2;
                                pm[2] += g * w.t3;
                            } else {
                                R d[3];
                                central_derivs<R>(av, w.x * s, d);
                                pc[0] += g * d[0];
                                pc[1] += g * d[1];
                                pc[2] += g * d[2];
                            }
                        }
                        cen.add(pc);
                    }
                    mom.add(pm);
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&s_empty[b]);
            }
            // window sums of this thread: central + wing (from the moments)
            double v3[3] = {0.0, 0.0, 0.0};
            if (active) {
                // moments M_k = sum G u^k = rho^k S_k; with H = (c1 u + c2 u^2 + c3 u^3)/sqrt(pi)
                // (adj_fl_cubic_x) and v d/dv u^k = -2k u^k:
                //   sum G H = sum_k c_k M_k / sqrt(pi),  sum G H_a = sum_k c_k' M_k / sqrt(pi),
                //   sum G (a H_a + v H_v) = sum_k (a c_k' - 2k c_k) M_k / sqrt(pi)
                const double A = double(av), A2 = A * A;
                const bool fl = MIXED && A > 0.2;
                const double c1 = A, c2 = fl ? A * (1.5 - A2) : 1.5 * A,
                             c3 = fl ? A * (3.75 + A2 * (A2 - 5.0)) : 3.75 * A;
                const double d1 = 1.0, d2 = fl ? 1.5 - 3.0 * A2 : 1.5, d3 = fl ? 3.75 + A2 * (5.0 * A2 - 15.0) : 3.75;
                const double M1 = rho * mom.get(0), M2 = rho * rho * mom.get(1), M3 = rho * rho * rho * mom.get(2);
                const double isp = 0.5641895835477563;  // 1/sqrt(pi)
                const double wH = isp * (c1 * M1 + c2 * M2 + c3 * M3);
                const double wA = isp * (d1 * M1 + d2 * M2 + d3 * M3);
                const double wX = isp * ((A * d1 - 2 * c1) * M1 + (A * d2 - 4 * c2) * M2 + (A * d3 - 6 * c3) * M3);
                v3[0] = cen.get(0) + wH;
                v3[1] = cen.get(1) + wX;
                v3[2] = cen.get(2) + wA;
            }
            // the NJ threads of a layer are aligned lanes of one warp
            for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    const double o = __shfl_xor_sync(0xffffffffu, v3[k], off);
                    if (off < NJ) v3[k] += o;
                }
            }
            if (active && jr == 0 && !s_abort) {
                double* dp = a.dpar + (i * Lp + l) * 3;
#pragma unroll
                for (int k = 0; k < 3; k++) atomicAdd(dp + k, v3[k]);
            }
        }
        g0 += nsub;
        __syncthreads();  // the item, s_order, s_ns and s_Ls are rewritten by the next item
    }
}

// Block shape of line_adj_kernel for L layers (1 <= L <= 480): consumer warps for about 5
// threads per layer (at least 4 warps, at most 15) and one producer warp; Ls is the largest
// staged row stride an item may pick (L itself when G rows are bulk-copied).
struct AdjShape {
    int Ls, threads, bulk, sub;
};
inline AdjShape adj_shape(int L, const void* G, bool mixed) {
    int t = ((5 * L + 31) / 32) * 32;
    t = t < 128 ? 128 : (t > 480 ? 480 : t);
    if (t < L) t = ((L + 31) / 32) * 32;
    const size_t esz = mixed ? 4 : 8;
    const bool bulk = (size_t(L) * esz) % 16 == 0 && (reinterpret_cast<uintptr_t>(G) & 15) == 0;
    const int Ls = bulk ? L : ((L + 3) & ~3) + 32;
    // stages of ADJ_SUB wavelengths, fewer (whole warps of table entries) when the ring would
    // not fit in a block's shared memory beside the static arrays (many layers in FP64)
    int sub = ADJ_SUB;
    while (sub > 32 && esz * ADJ_STAGES * size_t(sub) * Ls + sizeof(int) * size_t(Ls) > size_t(216) * 1024) sub -= 32;
    return {Ls, t + 32, int(bulk), sub};
}

// Dynamic shared memory of line_adj_kernel: the staged G ring, then the per-item layer order.
inline size_t adj_smem(const AdjShape& sh, bool mixed) {
    return (mixed ? sizeof(float) : sizeof(double)) * ADJ_STAGES * size_t(sh.sub) * size_t(sh.Ls) +
           sizeof(int) * size_t(sh.Ls);
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

}  // namespace korg
