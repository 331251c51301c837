// rt.cuh -- planar radiative transfer: anchored optical depth and exponential-integral flux.
// Restates RadiativeTransfer.jl:62-139 for the default planar path (tau_scheme "anchored",
// I_scheme "linear_flux_only" -> "linear_flux_only_expint", mu = [1], weights = [1]).
//
// One thread per wavelength column; the layer recursion (the tau prefix integral of :244-253
// and the segment sum of :379-388) is sequential per column and entirely FP64.  E2(tau) and
// exp(-tau) are evaluated once per layer and shared by the two segments meeting there.  When
// a continuum interpolant is given, the continuum-only transfer of synthesize
// (src/synthesize.jl:287-291) runs in the same loop, so the source function is evaluated once
// per (layer, wavelength) for both passes.
#pragma once
#include "physics.cuh"
#include "lines.cuh"

namespace korg {

struct RtArgs {
    const double* alpha;     // [nwl][L] full opacity
    const double* S;         // [nwl][L] source function, or null: Planck B(T_l, wl_j)
    const double* T;         // [L] (when S is null)
    const double* wls;       // [nwl] (when S is null or a continuum pass is requested)
    int64_t nwl;
    int32_t L;
    const double* tau_ref;   // [L]
    const double* alpha_ref; // [L]
    const MathTables* math;
    CntmDev cn;              // nk > 0: also run the continuum-only transfer into cntm
    double* flux;
    double* cntm;
    double unit;             // multiplies 2*pi*I (1e-8 in synthesize, src/synthesize.jl:315-318)
};

// src/synthesize.jl:412-418 with the column factors hoisted
__device__ __forceinline__ double planck(double pre, double hc_over_wl, double T) {
    return pre * 1 / expm1(hc_over_wl / KBOLTZ_CGS / T);
}

// Once tau at a layer exceeds TAU_STOP, every deeper segment of that column contributes less
// than S_max * exp(-TAU_STOP) (~1e-44 relative): the recursion stops there.
constexpr double TAU_STOP = 100.0;

// One pass of the column recursion; the continuum-only and full passes share the loop.
struct RtPass {
    double ib_prev, tau_prev, e2_prev, ex_prev, I;
    bool live;
    __device__ __forceinline__ void step(double alpha, double fac, double dlt, double S, double S_prev,
                                         const MathTables& mt) {
        const double ib = alpha * fac;
        const double tau = tau_prev + 0.5 * (ib + ib_prev) * dlt;  // RadiativeTransfer.jl:250-251
        const double m = (S - S_prev) / (tau - tau_prev);          // :382
        const double b = S_prev - m * tau_prev;                    // :383
        const double ex = fexp64(-tau, mt);
        const double e2 = expint2_ex(tau, ex, mt);
        I += (expint_core(tau, e2, ex, m, b) - expint_core(tau_prev, e2_prev, ex_prev, m, b));  // :384-385
        ib_prev = ib;
        tau_prev = tau;
        e2_prev = e2;
        ex_prev = ex;
        live = tau <= TAU_STOP;
    }
};

__global__ void __launch_bounds__(128) rt_kernel(RtArgs a) {
    extern __shared__ double s_rt[];
    __shared__ MathTables s_math;
    load_math_tables(s_math, a.math);
    const int L = a.L;
    double* s_fac = s_rt;          // tau_ref/alpha_ref * ds/dz (= 1)
    double* s_ltr = s_rt + L;      // log(tau_ref)
    double* s_T = s_rt + 2 * L;
    for (int l = threadIdx.x; l < L; l += blockDim.x) {
        s_fac[l] = a.tau_ref[l] / a.alpha_ref[l] * 1.0;  // RadiativeTransfer.jl:160
        s_ltr[l] = log(a.tau_ref[l]);                     // :114
        s_T[l] = a.T ? a.T[l] : 0.0;
    }
    __syncthreads();
    const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= a.nwl) return;
    const bool two = a.cn.nk > 0;
    double pre = 0, hcw = 0;
    KnotPos kp{0, 0.0};
    if (!a.S || two) {
        const double wl = a.wls[j];
        pre = 2 * HPLANCK_CGS * (C_CGS * C_CGS) / (wl * wl * wl * wl * wl);
        hcw = HPLANCK_CGS * C_CGS / wl;
        if (two) kp = knot_pos(a.cn.knots, a.cn.nk, wl);
    }
    const double* al = a.alpha + j * L;
    const double* Sc = a.S ? a.S + j * L : nullptr;

    // layer 0: tau = 0, E2(0) = 1, exp(0) = 1
    double S_prev = Sc ? Sc[0] : planck(pre, hcw, s_T[0]);
    RtPass full{al[0] * s_fac[0], 0.0, 1.0, 1.0, 0.0, true};
    RtPass cont{two ? knot_eval(a.cn.vals, a.cn.nk, kp) * s_fac[0] : 0.0, 0.0, 1.0, 1.0, 0.0, two};
    for (int l = 1; l < L && (full.live || cont.live); l++) {
        const double S = Sc ? Sc[l] : planck(pre, hcw, s_T[l]);
        const double dlt = s_ltr[l] - s_ltr[l - 1];
        if (full.live) full.step(al[l], s_fac[l], dlt, S, S_prev, s_math);
        if (cont.live)
            cont.step(knot_eval(a.cn.vals + int64_t(l) * a.cn.nk, a.cn.nk, kp), s_fac[l], dlt, S, S_prev, s_math);
        S_prev = S;
    }
    a.flux[j] = 2 * PI * (full.I * 1.0) * a.unit;  // :136
    if (two) a.cntm[j] = 2 * PI * (cont.I * 1.0) * a.unit;
}

// alpha[j][l] = continuum interpolant of layer l at wl_j (src/synthesize.jl:226-252)
__global__ void __launch_bounds__(256) alpha_init_kernel(double* alpha, const double* wls, int64_t nwl, int32_t L,
                                                         CntmDev cn) {
    __shared__ int64_t s_i[64];
    __shared__ double s_t[64];
    const int64_t j0 = int64_t(blockIdx.x) * 64;
    const int64_t jn = min(int64_t(64), nwl - j0);
    if (threadIdx.x < jn) {
        const KnotPos p = knot_pos(cn.knots, cn.nk, wls[j0 + threadIdx.x]);
        s_i[threadIdx.x] = p.i;
        s_t[threadIdx.x] = p.t;
    }
    __syncthreads();
    const int64_t n = jn * L;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        const int jj = int(e / L), l = int(e % L);
        const KnotPos p{s_i[jj], s_t[jj]};
        alpha[j0 * L + e] = knot_eval(cn.vals + int64_t(l) * cn.nk, cn.nk, p);
    }
}

}  // namespace korg
