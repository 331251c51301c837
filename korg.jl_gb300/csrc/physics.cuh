// physics.cuh -- device-side line-profile, transfer and hydrogen-line mathematics.
//
// FP64 functions keep the evaluation order of Korg.jl's Julia source (cited per function);
// the FP32 forms are the mixed-precision counterparts used by KORG_MIXED.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace korg {

// src/constants.jl:3-19
constexpr double KBOLTZ_CGS = 1.380649e-16;
constexpr double HPLANCK_CGS = 6.62607015e-27;
constexpr double C_CGS = 2.99792458e10;
constexpr double ELECTRON_MASS_CGS = 9.1093897e-28;
constexpr double ELECTRON_CHARGE_CGS = 4.80320425e-10;
constexpr double AMU_CGS = 1.6605402e-24;
constexpr double BOHR_RADIUS_CGS = 5.29177210903e-9;
constexpr double EV_TO_CGS = 1.602e-12;
constexpr double KBOLTZ_EV = 8.617333262145e-5;
constexpr double HPLANCK_EV = 4.135667696e-15;
constexpr double RYDBERGH_EV = 13.598287264;
constexpr double PI = 3.141592653589793;
constexpr double SQRT_PI = 1.7724538509055159;   // sqrt(pi)
constexpr double SQRT_2 = 1.4142135623730951;
constexpr double SQRT_2PI = 2.5066282746310002;  // sqrt(2*pi)

// ---------------------------------------------------------------- table-driven FP64 exp / log
// Tang's table-driven method (P. T. P. Tang, ACM TOMS 15 (1989) 144 and 16 (1990) 378),
// implemented from the mathematics with 256-entry tables: exp(x) = 2^m 2^(j/256) e^r with
// |r| <= ln2/512 and a degree-4 Taylor polynomial (truncation r^5/120 < 4e-17 relative);
// log(x) = e ln2 + log(c_j) + log(1 + r), c_j = 1 + (j + 1/2)/256, r = m/c_j - 1
// (|r| <= 1/513) and a degree-5 series (truncation r^6/6 < 1e-17).  About a third of the FP64
// operations of the general-purpose functions, which matters on GB300 where the FP64 pipe is
// 1/64 of FP32; the range checks are integer compares on the bit patterns.
// Tables (computed on the host in extended precision at context creation):
//   exp2j[j] = 2^(j/256), inv_c[j] = 1/c_j rounded to double, log_c[j] = -log(inv_c[j]).
// Accuracy: exp within 1 ulp for |x| < 700 (outside that range the CUDA function is used);
// log within 2e-15 absolute (0.5 ulp for |log x| >~ 4) for normal x.
constexpr int MATH_TABLE_BITS = 8;
constexpr int MATH_TABLE_N = 1 << MATH_TABLE_BITS;
struct MathTables {
    double exp2j[MATH_TABLE_N];
    double inv_c[MATH_TABLE_N];
    double log_c[MATH_TABLE_N];
};

__device__ __forceinline__ double fexp64(double x, const MathTables& t) {
    if ((__double2hiint(x) & 0x7fffffff) >= 0x4085E000) return exp(x);  // |x| >= 700, inf, NaN
    const double INV_L = 369.3299304675746;            // 256 / ln 2
    const double L_HI = 0.0027076061742263846;         // ln2 / 256 to 33 bits (k * L_HI exact)
    const double L_LO = -1.6409824502660487e-13;       // ln2 / 256 - L_HI
    const double MAGIC = 6755399441055744.0;           // 1.5 * 2^52: round to integer
    double kd = fma(x, INV_L, MAGIC);
    const int k = __double2loint(kd);
    kd -= MAGIC;
    double r = fma(-kd, L_HI, x);
    r = fma(-kd, L_LO, r);
    double p = fma(r, 1.0 / 24.0, 1.0 / 6.0);
    p = fma(p, r, 0.5);
    p = fma(p, r, 1.0);
    p *= r;
    const double tj = t.exp2j[k & (MATH_TABLE_N - 1)];
    const double res = fma(tj, p, tj);
    return __longlong_as_double(__double_as_longlong(res) + ((long long)(k >> MATH_TABLE_BITS) << 52));
}

__device__ __forceinline__ double flog64(double x, const MathTables& t) {
    const long long b = __double_as_longlong(x);
    if (b < 0x0010000000000000LL || b >= 0x7FF0000000000000LL) return log(x);  // not normal and positive
    const int e = int((b >> 52) & 0x7ff) - 1023;
    const double m = __longlong_as_double((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
    const int j = int((b >> (52 - MATH_TABLE_BITS)) & (MATH_TABLE_N - 1));
    const double r = fma(m, t.inv_c[j], -1.0);
    double p = fma(0.2, r, -0.25);
    p = fma(p, r, 1.0 / 3.0);
    p = fma(p, r, -0.5);
    p = fma(p, r, 1.0);
    p *= r;
    const double LN2_HI = 0.6931471805599453, LN2_LO = 2.3190468138462996e-17;
    return fma(double(e), LN2_HI, t.log_c[j] + fma(double(e), LN2_LO, p));
}

// copy the tables into shared memory (call from every thread, then __syncthreads())
__device__ __forceinline__ void load_math_tables(MathTables& dst, const MathTables* src) {
    const double* s = reinterpret_cast<const double*>(src);
    double* d = reinterpret_cast<double*>(&dst);
    for (int i = threadIdx.x; i < 3 * MATH_TABLE_N; i += blockDim.x) d[i] = s[i];
}

// ---------------------------------------------------------------- FP64 Voigt-Hjerting
// src/line_absorption.jl:251-265
__device__ __forceinline__ void harris64(double v, double& H0, double& H1, double& H2) {
    double v2 = v * v;
    H0 = exp(-(v2));
    if (v < 1.3)
        H1 = -1.12470432 + (-0.15516677 + (3.288675912 + (-2.34357915 + 0.42139162 * v) * v) * v) * v;
    else if (v < 2.4)
        H1 = -4.48480194 + (9.39456063 + (-6.61487486 + (1.98919585 - 0.22041650 * v) * v) * v) * v;
    else
        H1 = ((0.554153432 + (0.278711796 + (-0.1883256872 + (0.042991293 - 0.003278278 * v) * v) * v) * v) /
              (v2 - 1.5));
    H2 = (1 - 2 * v2) * H0;
}

// src/line_absorption.jl:286-310
__device__ __forceinline__ double voigt64(double a, double v) {
    double v2 = v * v;
    if (a <= 0.2 && (v >= 5)) {
        double invv2 = (1 / v2);
        return (a / SQRT_PI * invv2) * (1 + 1.5 * invv2 + 3.75 * (invv2 * invv2));
    } else if (a <= 0.2) {
        double H0, H1, H2;
        harris64(v, H0, H1, H2);
        return H0 + (H1 + H2 * a) * a;
    } else if ((a <= 1.4) && (a + v < 3.2)) {
        double H0, H1, H2;
        harris64(v, H0, H1, H2);
        const double c2 = 2 / SQRT_PI, c23 = 2 / (3 * SQRT_PI);
        double M0 = H0;
        double M1 = H1 + c2 * M0;
        double M2 = H2 - M0 + c2 * M1;
        double M3 = c23 * (1 - H2) - (2.0 / 3.0) * v2 * M1 + c2 * M2;
        double M4 = 2.0 / 3.0 * v2 * v2 * M0 - c23 * M1 + c2 * M3;
        double psi = 0.979895023 + (-0.962846325 + (0.532770573 - 0.122727278 * a) * a) * a;
        return psi * (M0 + (M1 + (M2 + (M3 + M4 * a) * a) * a) * a);
    } else {
        double r2 = (v2) / (a * a);
        double a_invu = 1 / SQRT_2 / ((r2 + 1) * a);
        double a2_invu2 = a_invu * a_invu;
        return 0.7978845608028654 * a_invu *  // sqrt(2/pi)
               (1 + (3 * r2 - 1 + ((r2 - 2) * 15 * r2 + 2) * a2_invu2) * a2_invu2);
    }
}

// src/line_absorption.jl:245-249
__device__ __forceinline__ double line_profile64(double wl0, double sigma, double gamma, double amp, double wl) {
    double inv_s = 1 / (sigma * SQRT_2);
    double scaling = inv_s / SQRT_PI * amp;
    return voigt64(gamma * inv_s, fabs(wl - wl0) * inv_s) * scaling;
}

// ---------------------------------------------------------------- FP32 Voigt-Hjerting
// Mixed-precision H(a, v) * scale for the wavelength-tile kernels.  Per (line, layer):
// p = {c = 2 sigma^2 (so v^2 = x^2 / c), a, w, scale} with w = a/sqrt(pi)*scale when a <= 0.2
// and w = 1/gamma^2 otherwise.  Per (line, wavelength), shared by all layers: x = |wl - wl0|
// and t = 1/x^2.  In the asymptotic wing (a <= 0.2, v >= 5), which holds most evaluations of a
// wide window, 1/v^2 = t*c and the profile costs one multiply and a short polynomial.
__device__ __forceinline__ float harris_mod32(float a, float v, bool modified) {
    const float v2 = v * v;
    const float H0 = __expf(-v2);
    float H1;
    if (v < 1.3f)
        H1 = -1.12470432f + (-0.15516677f + (3.288675912f + (-2.34357915f + 0.42139162f * v) * v) * v) * v;
    else if (v < 2.4f)
        H1 = -4.48480194f + (9.39456063f + (-6.61487486f + (1.98919585f - 0.22041650f * v) * v) * v) * v;
    else
        H1 = __fdividef(0.554153432f + (0.278711796f + (-0.1883256872f + (0.042991293f - 0.003278278f * v) * v) * v) * v,
                        v2 - 1.5f);
    const float H2 = (1.f - 2.f * v2) * H0;
    if (!modified) return H0 + (H1 + H2 * a) * a;
    const float c2 = 1.1283791670955126f, c23 = 0.37612638903183754f;  // 2/sqrt(pi), 2/(3 sqrt(pi))
    const float M0 = H0;
    const float M1 = H1 + c2 * M0;
    const float M2 = H2 - M0 + c2 * M1;
    const float M3 = c23 * (1.f - H2) - 0.6666666666666666f * v2 * M1 + c2 * M2;
    const float M4 = 0.6666666666666666f * v2 * v2 * M0 - c23 * M1 + c2 * M3;
    const float psi = 0.979895023f + (-0.962846325f + (0.532770573f - 0.122727278f * a) * a) * a;
    return psi * (M0 + (M1 + (M2 + (M3 + M4 * a) * a) * a) * a);
}

__device__ __forceinline__ float profile32x(float4 p, float x, float t) {
    const float a = p.y;
    if (a <= 0.2f) {
        const float i = t * p.x;  // 1/v^2
        if (i <= 0.04f) return (p.z * i) * fmaf(fmaf(3.75f, i, 1.5f), i, 1.f);  // v >= 5
        return harris_mod32(a, x * rsqrtf(p.x), false) * p.w;
    }
    const float v = x * rsqrtf(p.x);
    if (a <= 1.4f && a + v < 3.2f) return harris_mod32(a, v, true) * p.w;
    const float r2 = (x * x) * p.z;  // v^2 / a^2 = x^2 / gamma^2
    const float au = __fdividef(0.70710678118654752f, (r2 + 1.f) * a);
    const float au2 = au * au;
    return 0.7978845608028654f * au * (1.f + (3.f * r2 - 1.f + ((r2 - 2.f) * 15.f * r2 + 2.f) * au2) * au2) * p.w;
}

// ---------------------------------------------------------------- line-parameter helpers
// src/line_absorption.jl:190
__device__ __forceinline__ double doppler_width(double wl0, double T, double m, double xi) {
    return wl0 * sqrt(KBOLTZ_CGS * T / m + (xi * xi) / 2) / C_CGS;
}
// src/line_absorption.jl:229-237
__device__ __forceinline__ double sigma_line(double wl) {
    const double e = ELECTRON_CHARGE_CGS, me = ELECTRON_MASS_CGS, c = C_CGS;
    return (PI * (e * e) / me / c) * ((wl * wl) / c);
}
// src/line_absorption.jl:140-145
__device__ __forceinline__ double inverse_gaussian_density(double rho, double sigma) {
    if (rho > 1 / (SQRT_2PI * sigma)) return 0.0;
    return sigma * sqrt(-2 * log(SQRT_2PI * sigma * rho));
}
// src/line_absorption.jl:156-161
__device__ __forceinline__ double inverse_lorentz_density(double rho, double gamma) {
    if (rho > 1 / (PI * gamma)) return 0.0;
    return sqrt(gamma / (PI * rho) - gamma * gamma);
}

// Gridded(Linear()) interpolation on increasing knots (Interpolations.jl, used for the
// continuum interpolants of src/synthesize.jl:228).  Explicitly rounded operations so every
// call site produces bit-identical values.
__device__ __forceinline__ int64_t search_last(const double* x, int64_t n, double v) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = lo + ((hi - lo) >> 1);
        if (x[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo - 1;
}
__device__ __forceinline__ int64_t search_first(const double* x, int64_t n, double v) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = lo + ((hi - lo) >> 1);
        if (x[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}
struct KnotPos { int64_t i; double t; };
__device__ __forceinline__ KnotPos knot_pos(const double* k, int64_t n, double x) {
    KnotPos p{0, 0.0};
    if (n == 1) return p;
    int64_t i = search_last(k, n, x);
    i = i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
    p.i = i;
    p.t = __ddiv_rn(__dsub_rn(x, k[i]), __dsub_rn(k[i + 1], k[i]));
    return p;
}
__device__ __forceinline__ double knot_eval(const double* v, int64_t n, KnotPos p) {
    if (n == 1) return v[0];
    return __dadd_rn(__dmul_rn(v[p.i], __dsub_rn(1.0, p.t)), __dmul_rn(v[p.i + 1], p.t));
}

// ---------------------------------------------------------------- transfer
// 1/d by Newton-Raphson iteration from an FP32 seed: r0 = 1/float(d) (relative error about
// 2^-21), then one cubically convergent step r1 = r0 + r0 (e + e^2) with e = 1 - d r0, whose
// truncation error e^3 ~ 2^-63 is below FP64 rounding: within about one ulp of 1/d, in three
// FP64 fused multiply-adds instead of a full FP64 division.  Outside the FP32 normal range of
// the seed the FP64 division is used.
__device__ __forceinline__ double recip64(double d) {
    const float f = __double2float_rn(d);
    if (!(fabsf(f) > 1e-30f && fabsf(f) < 1e30f)) return 1.0 / d;
    double r = double(__fdividef(1.f, f));
    const double e = fma(-d, r, 1.0);
    return fma(r, fma(e, e, e), r);
}

// RadiativeTransfer.jl:408-497
__device__ __forceinline__ double expint2_64(double x) {
    if (x == 0) return 1.0;
    if (x < 1.1) {
        const double EM = 0.57721566490153286060651209008240243104215933593992;
        return 1 + ((log(x) + EM - 1) +
                    (-0.5 + (0.08333333333333333 + (-0.013888888888888888 + 0.0020833333333333333 * x) * x) * x) * x) * x;
    }
    if (x < 2.5) {
        x -= 2;
        return 0.037534261820486914 + (-0.04890051070806112 + (0.033833820809153176 + (-0.016916910404576574 +
               (0.007048712668573576 - 0.0026785108140579598 * x) * x) * x) * x) * x;
    }
    if (x < 3.5) {
        x -= 3;
        return 0.010641925085272673 + (-0.013048381094197039 + (0.008297844727977323 + (-0.003687930990212144 +
               (0.0013061422257001345 - 0.0003995258572729822 * x) * x) * x) * x) * x;
    }
    if (x < 4.5) {
        x -= 4;
        return 0.0031982292493385146 + (-0.0037793524098489054 + (0.0022894548610917728 + (-0.0009539395254549051 +
               (0.00031003034577284415 - 8.466213288412284e-5 * x) * x) * x) * x) * x;
    }
    if (x < 5.5) {
        x -= 5;
        return 0.000996469042708825 + (-0.0011482955912753257 + (0.0006737946999085467 + (-0.00026951787996341863 +
               (8.310134632205409e-5 - 2.1202073223788938e-5 * x) * x) * x) * x) * x;
    }
    if (x < 6.5) {
        x -= 6;
        return 0.0003182574636904001 + (-0.0003600824521626587 + (0.00020656268138886323 + (-8.032993165122457e-5 +
               (2.390771775334065e-5 - 5.8334831318151185e-6 * x) * x) * x) * x) * x;
    }
    if (x < 7.5) {
        x -= 7;
        return 0.00010350984428214624 + (-0.00011548173161033826 + (6.513442611103688e-5 + (-2.4813114708966427e-5 +
               (7.200234178941151e-6 - 1.7027366981408086e-6 * x) * x) * x) * x) * x;
    }
    if (x < 9) {
        x -= 8;
        return 3.413764515111217e-5 + (-3.76656228439249e-5 + (2.096641424390699e-5 + (-7.862405341465122e-6 +
               (2.2386015208338193e-6 - 5.173353514609864e-7 * x) * x) * x) * x) * x;
    }
    const double invx = 1 / x;
    return exp(-x) * (1 + (-2 + (6 + (-24 + 120 * invx) * invx) * invx) * invx) * invx;
}

// E2 with exp(-x) supplied by the caller (the x >= 9 branch reuses it, RadiativeTransfer.jl:440-443)
// and the table-driven log for the small-argument series (:432-439)
__device__ __forceinline__ double expint2_ex(double x, double ex, const MathTables& t) {
    if (x >= 9) {
        const double invx = recip64(x);
        return ex * (1 + (-2 + (6 + (-24 + 120 * invx) * invx) * invx) * invx) * invx;
    }
    if (x < 1.1 && x != 0) {
        const double EM = 0.57721566490153286060651209008240243104215933593992;
        return 1 + ((flog64(x, t) + EM - 1) +
                    (-0.5 + (0.08333333333333333 + (-0.013888888888888888 + 0.0020833333333333333 * x) * x) * x) * x) * x;
    }
    return expint2_64(x);
}

// RadiativeTransfer.jl:398-400 with E2(tau) and exp(-tau) supplied by the caller (they are
// per-layer quantities shared by the two segments that meet at a layer).  Expanded,
//   core = [3b (tau E2 - e^-tau) + 2m (tau^2 E2 - e^-tau (tau + 1))] / 6 = b G / 2 + m H / 3
// with G = tau E2 - e^-tau and H = tau G - e^-tau, which depend on the layer only: the planar
// kernel carries G and H per layer instead of evaluating the core twice per segment.
__device__ __forceinline__ double expint_core(double tau, double e2, double ex, double m, double b) {
    return 1.0 / 6.0 * (tau * e2 * (3 * b + 2 * m * tau) - ex * (3 * b + 2 * m * (tau + 1)));
}

// ---------------------------------------------------------------- hydrogen helpers
// src/statmech.jl:463-497 (default branch)
__device__ __forceinline__ double hummer_mihalas_w(double n_eff, double nH, double nHe, double ne) {
    double n2 = n_eff * n_eff, n4 = n2 * n2;
    double r_level = sqrt(5.0 / 2.0 * n4 + 1.0 / 2.0 * n2) * BOHR_RADIUS_CGS;
    double a = r_level + 1.7320508075688772 * BOHR_RADIUS_CGS, b = r_level + 1.02 * BOHR_RADIUS_CGS;
    double neutral_term = nH * (a * a * a) + nHe * (b * b * b);
    double K = 1.0;
    if (n_eff > 3) {
        double r = n_eff / (n_eff + 1);
        K = 16.0 / 3.0 * (r * r) * ((n_eff + 7.0 / 6.0) / (n2 + n_eff + 1.0 / 2.0));
    }
    double chi = RYDBERGH_EV / n2 * EV_TO_CGS;
    double e = ELECTRON_CHARGE_CGS;
    double q = (e * e) / (chi * sqrt(K));
    double charged_term = 16 * (q * q * q) * ne;
    return exp(-(4 * PI) / 3 * (neutral_term + charged_term));
}

// src/line_absorption.jl:208-221, ABO branch only
__device__ __forceinline__ double scaled_vdW_abo(double sigma, double alpha, double m, double T) {
    const double v0 = 1e6;
    double invmu = 1 / (1.008 * AMU_CGS) + 1 / m;
    double vbar = sqrt(8 * KBOLTZ_CGS * T / PI * invmu);
    return 2 * pow(4 / PI, alpha / 2) * tgamma((4 - alpha) / 2) * v0 * sigma * pow(vbar / v0, 1 - alpha);
}

// src/line_absorption.jl:169-182
__device__ __forceinline__ double expint1_64(double x) {
    if (x < 0) return 0.0;
    if (x <= 0.01) return -log(x) - 0.577215 + x;
    if (x <= 1.0)
        return -log(x) - 0.57721566 +
               x * (0.99999193 + x * (-0.24991055 + x * (0.05519968 + x * (-0.00976004 + x * 0.00107857))));
    if (x <= 30.0) return (x * (x + 2.334733) + 0.25062) / (x * (x + 3.330657) + 1.681534) / x * exp(-x);
    return 0.0;
}

}  // namespace korg
