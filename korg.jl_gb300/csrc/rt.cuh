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

// src/synthesize.jl:412-418 with the column factors hoisted and 1/(kT) per layer precomputed,
// exp(x) - 1 from the table-driven exp and the Newton reciprocal: for x = hc/(lambda k T) >= 0.07
// (lambda <= 2 um, T <= 1e5 K) the subtraction loses under two bits, so the result stays within a
// few ulps of pre / expm1(x), at about half the FP64 work per (layer, wavelength).
__device__ __forceinline__ double planck_t(double pre, double hc_over_wl, double inv_kT, const MathTables& mt) {
    const double x = hc_over_wl * inv_kT;
    return x < 0.05 ? pre / expm1(x) : pre * recip64(fexp64(x, mt) - 1.0);
}

// Once tau at a layer exceeds TAU_STOP, every deeper segment of that column contributes at most
// S_max E2(TAU_STOP) < S_max exp(-TAU_STOP) / TAU_STOP ~ 1e-19 S_max; S_max / F stays below
// ~1e3 for stellar atmospheres (Planck contrast between the top and the bottom), so the
// neglected part is below 1e-16 of the flux: the recursion stops there.
constexpr double TAU_STOP = 40.0;

// One pass of the column recursion; the continuum-only and full passes share the loop.  The
// segment [l-1, l] adds core(tau_l) - core(tau_{l-1}) with the slope m and intercept b of the
// linear source function in tau (RadiativeTransfer.jl:382-385); with core = b G / 2 + m H / 3
// (expint_core) and b = S_{l-1} - m tau_{l-1}:
//   I += S_{l-1} dG / 2 + m (dH / 3 - tau_{l-1} dG / 2),  m = (S_l - S_{l-1}) / dtau.
struct RtPass {
    double ib_prev, tau_prev, G_prev, H_prev, I;
    bool live;
    __device__ __forceinline__ void step(double alpha, double fac, double hdlt, double dS, double half_Sp,
                                         const MathTables& mt) {
        const double ib = alpha * fac;
        const double dtau = (ib + ib_prev) * hdlt;                 // RadiativeTransfer.jl:250-251
        const double tau = tau_prev + dtau;
        const double m = dS * recip64(dtau);                        // :382
        const double ex = fexp64(-tau, mt);
        const double e2 = expint2_ex(tau, ex, mt);
        const double G = fma(tau, e2, -ex), H = fma(tau, G, -ex);
        const double dG = G - G_prev, dH = H - H_prev;
        I = fma(half_Sp, dG, I);                                    // :383-385
        I = fma(m, fma(-0.5 * tau_prev, dG, dH * (1.0 / 3.0)), I);
        ib_prev = ib;
        tau_prev = tau;
        G_prev = G;
        H_prev = H;
        live = tau <= TAU_STOP;
    }
};

__global__ void __launch_bounds__(128) rt_kernel(RtArgs a) {
    extern __shared__ double s_rt[];
    __shared__ MathTables s_math;
    load_math_tables(s_math, a.math);
    const int L = a.L;
    double* s_fac = s_rt;           // tau_ref/alpha_ref * ds/dz (= 1)
    double* s_hdl = s_rt + L;       // (log tau_ref[l] - log tau_ref[l-1]) / 2
    double* s_ikT = s_rt + 2 * L;   // 1/(k T)
    for (int l = threadIdx.x; l < L; l += blockDim.x) {
        s_fac[l] = a.tau_ref[l] / a.alpha_ref[l] * 1.0;  // RadiativeTransfer.jl:160
        s_hdl[l] = l > 0 ? 0.5 * (log(a.tau_ref[l]) - log(a.tau_ref[l - 1])) : 0.0;  // :114, :250-251
        s_ikT[l] = a.T ? 1.0 / (KBOLTZ_CGS * a.T[l]) : 0.0;
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

    // layer 0: tau = 0, E2(0) = 1, exp(0) = 1, so G = -1 and H = -1
    double S_prev = Sc ? Sc[0] : planck_t(pre, hcw, s_ikT[0], s_math);
    RtPass full{al[0] * s_fac[0], 0.0, -1.0, -1.0, 0.0, true};
    RtPass cont{two ? knot_eval(a.cn.vals, a.cn.nk, kp) * s_fac[0] : 0.0, 0.0, -1.0, -1.0, 0.0, two};
    for (int l = 1; l < L && (full.live || cont.live); l++) {
        const double S = Sc ? Sc[l] : planck_t(pre, hcw, s_ikT[l], s_math);
        const double hdl = s_hdl[l], dS = S - S_prev, half_Sp = 0.5 * S_prev;
        if (full.live) full.step(al[l], s_fac[l], hdl, dS, half_Sp, s_math);
        if (cont.live)
            cont.step(knot_eval(a.cn.vals + int64_t(l) * a.cn.nk, a.cn.nk, kp), s_fac[l], hdl, dS, half_Sp, s_math);
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

// ---------------------------------------------------------------- secondary schemes
// RadiativeTransfer.jl:77-139 and :147-371 for any atmosphere geometry and scheme: rays along
// the surface mu grid (planar or spherical), inward rays seeding the outward ones at the bottom,
// tau by the anchored or the Bezier scheme, intensity by the linear, linear-flux-only or Bezier
// formal solution, or the exponential-integral flux.  One thread per wavelength walks every ray;
// the ray geometry (path, ds/dz, layers reached) is computed once on the host.
constexpr int RTG_LMAX = 128;  // layers per ray
constexpr int RTG_RMAX = 64;   // rays (inward + outward)

struct RtGenArgs {
    const double* alpha;     // [nwl][L]
    const double* S;         // [nwl][L]
    int32_t L;
    int64_t nwl;
    int32_t nrays, n_in, n_mu;
    const int32_t* ray_n;    // [nrays] layers on the ray
    const double* ray_fac;   // [nrays][L] tau_ref/alpha_ref * ds/dz, in ray order
    const double* ray_lt;    // [nrays][L] +-log tau_ref, in ray order
    const double* ray_path;  // [nrays][L] +-s, in ray order
    const double* wmu;       // [n_mu] mu weight * mu of the outward rays
    int32_t tau_scheme;      // 0 anchored, 1 bezier
    int32_t I_scheme;        // 0 linear, 1 linear_flux_only, 2 bezier, 3 linear_flux_only_expint
    const MathTables* math;
    double* flux;            // [nwl] 2 pi sum_mu w mu I_surface
    double* Isurf;           // [n_mu][nwl] surface intensity of the outward rays, or null
};

// fritsch_butland_C (RadiativeTransfer.jl:361-371) evaluated for one interval k of n points
__device__ __forceinline__ double fb_control(const double* x, const double* y, int n, int k) {
    if (n < 3) return 0.5 * (y[0] + y[1]);  // two points: the reference has no interior slope
    auto yp = [&](int q) {  // interior slope estimate at point q + 1
        const double h0 = x[q + 1] - x[q], h1 = x[q + 2] - x[q + 1];
        const double d0 = (y[q + 1] - y[q]) / h0, d1 = (y[q + 2] - y[q + 1]) / h1;
        const double al = 1.0 / 3.0 * (1 + h1 / (h1 + h0));
        return (d0 * d1) / (al * d1 + (1 - al) * d0);
    };
    const double A = k < n - 2 ? y[k + 1] + (x[k + 1] - x[k]) * yp(k) / 2
                               : y[n - 2] - (x[n - 1] - x[n - 2]) * yp(n - 3) / 2;
    const double B = k == 0 ? y[1] + (x[1] - x[0]) * yp(0) / 2 : y[k] - (x[k + 1] - x[k]) * yp(k - 1) / 2;
    return (A + B) / 2;
}

__global__ void __launch_bounds__(128) rt_general_kernel(RtGenArgs a) {
    const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= a.nwl) return;
    const int L = a.L;
    double tau[RTG_LMAX], col[RTG_LMAX], Sc[RTG_LMAX], I[RTG_LMAX];
    double seed[RTG_RMAX];  // per ray: bottom intensity (linear) or start value (flux only)
    for (int r = 0; r < a.nrays; r++) seed[r] = 0.0;
    double F = 0.0;
    for (int r = 0; r < a.nrays; r++) {
        const bool inward = r < a.n_in;
        const int n = a.ray_n[r];
        double Iout = 0.0;
        const double* fac = a.ray_fac + int64_t(r) * L;
        const double* lt = a.ray_lt + int64_t(r) * L;
        const double* path = a.ray_path + int64_t(r) * L;
        if (!(n == 1 && (a.I_scheme == 2 || a.tau_scheme == 1))) {  // :150-154
            for (int k = 0; k < n; k++) {
                const int lk = inward ? n - 1 - k : k;  // reversed path for inward rays (:118-121)
                col[k] = a.alpha[j * L + lk];
                Sc[k] = a.S[j * L + lk];
            }
            if (a.tau_scheme == 0) {  // :244-253
                double prev = col[0] * fac[0];
                tau[0] = 0.0;
                for (int k = 1; k < n; k++) {
                    const double ib = col[k] * fac[k];
                    tau[k] = tau[k - 1] + 0.5 * (ib + prev) * (lt[k] - lt[k - 1]);
                    prev = ib;
                }
            } else {  // :263-273
                double amin = col[0], amax = col[0];
                for (int k = 1; k < n; k++) { amin = fmin(amin, col[k]); amax = fmax(amax, col[k]); }
                tau[0] = 1e-5;
                for (int i = 1; i < n; i++) {
                    const double C = fmin(fmax(fb_control(path, col, n, i - 1), 0.5 * amin), 2 * amax);
                    tau[i] = tau[i - 1] + (path[i - 1] - path[i]) / 3 * (col[i] + col[i - 1] + C);
                }
            }
            if (a.I_scheme == 0) {  // :286-298
                I[n - 1] = seed[r];
                for (int k = n - 2; k >= 0; k--) {
                    const double d = tau[k + 1] - tau[k];
                    const double m = (Sc[k + 1] - Sc[k]) / d;
                    I[k] = (I[k + 1] - Sc[k] - m * (d + 1)) * exp(-d) + m + Sc[k];
                }
                Iout = I[0];
                if (inward && r + a.n_in < a.nrays) seed[r + a.n_in] = I[0];  // :196-198
            } else if (a.I_scheme == 2) {  // :333-350 (the bottom value is not used)
                I[n - 1] = 0.0;
                for (int k = n - 2; k >= 0; k--) {
                    const double d = tau[k + 1] - tau[k], e = exp(-d), d2 = d * d;
                    const double al = (2 + d2 - 2 * d - 2 * e) / d2;
                    const double be = (2 - (2 + 2 * d + d2) * e) / d2;
                    const double ga = (2 * d - 4 + (2 * d + 4) * e) / d2;
                    I[k] = I[k + 1] * e + al * Sc[k] + be * Sc[k + 1] + ga * fb_control(tau, Sc, n, k);
                }
                I[0] *= exp(-tau[0]);
                Iout = I[0];
                if (inward && r + a.n_in < a.nrays) seed[r + a.n_in] = I[0];
            } else {
                double add = 0.0;
                if (a.I_scheme == 1) {  // :307-324
                    double next = exp(-tau[0]);
                    for (int i = 0; i + 1 < n; i++) {
                        double dt = tau[i + 1] - tau[i];
                        dt += (dt == 0);
                        const double m = (Sc[i + 1] - Sc[i]) / dt;
                        const double cur = next;
                        next = exp(-tau[i + 1]);
                        add += (-next * (Sc[i + 1] + m) + cur * (Sc[i] + m));
                    }
                } else {  // :379-388
                    double e2p = 1.0, exp_ = 1.0;
                    for (int i = 0; i + 1 < n; i++) {
                        const double m = (Sc[i + 1] - Sc[i]) / (tau[i + 1] - tau[i]);
                        const double b = Sc[i] - m * tau[i];
                        const double ex = exp(-tau[i + 1]);
                        const double e2 = expint2_64(tau[i + 1]);
                        add += expint_core(tau[i + 1], e2, ex, m, b) - expint_core(tau[i], e2p, exp_, m, b);
                        e2p = e2;
                        exp_ = ex;
                    }
                }
                Iout = seed[r] + add;  // += onto a seeded value (:177-180)
                if (inward && r + a.n_in < a.nrays) seed[r + a.n_in] = Iout * exp(-tau[n - 1]);
            }
        }
        if (!inward) {
            const int u = r - a.n_in;
            F += Iout * a.wmu[u];
            if (a.Isurf) a.Isurf[int64_t(u) * a.nwl + j] = Iout;
        }
    }
    a.flux[j] = 2 * PI * F;
}

}  // namespace korg
