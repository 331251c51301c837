// hydrogen.cuh -- hydrogen-line opacity on the device.  Restates hydrogen_line_absorption!
// (src/hydrogen_line_absorption.jl:75-163) for all layers at once.
//
//   hline_prep:   one thread per (Stehle transition, layer): range check, interpolated line
//                 centre, amplitude, window, the ABO Voigt constants for H-alpha/beta/gamma and
//                 the profile table interpolated to (T, ne) along the log(delta nu / F0) knots
//                 (trilinear interpolation = this bilinear step followed by a 1-D one).
//   brackett_prep: one CTA per (upper level m, layer): the 201-point Brackett profile of
//                 bracket_line_interpolator (:211-251), two direct convolutions in shared memory.
//   hline_tile:   one CTA per wavelength tile x all layers, like the metal-line tile kernel;
//                 each thread owns one wavelength and a set of layers and accumulates in
//                 registers, then adds to alpha once.
#pragma once
#include <type_traits>

#include "physics.cuh"

namespace korg {

constexpr int HND_MAX = 72;   // >= the largest number of delta-nu knots in the Stehle tables
constexpr int BR_NP = 201;    // Brackett profile points (n_wavelength_points)

struct StarkDev {
    int32_t ntrans;
    const int32_t *lower, *upper, *nT, *nNe, *nD;
    const int64_t *t_off, *ne_off, *d_off, *p_off, *l_off;
    const double *log_gf, *temps, *nes, *logdnu, *logP, *lambda0;
    const float* logdnu32;  // float copy of the knots (mixed precision)
};

enum { HK_OFF = 0, HK_STARK = 1, HK_STARK_ABO = 2, HK_BRACKETT = 3 };

struct HRec {
    double nu0, amp, invF0, F0;
    double wl0, inv_s, a, scale;   // ABO Voigt (kind 2) or Brackett grid start/step (kind 3)
    float nu0_hi, nu0_lo;          // mixed precision: line centre frequency as an FP32 pair
    float invF0_f, amp_f;
    float4 abo32;                  // ABO constants packed for profile32x
    int32_t lb, ub, kind, nD;
};

struct HLayers {
    int32_t L;
    const double *T, *ne, *nH, *nHe, *UH, *xi;
};

struct HOut {
    HRec* rec;             // [ntot][L]
    double* Q;             // [ntrans][L][HND_MAX] Stehle tables at (T, ne); [nbr][L][BR_NP] Brackett
    float* Q32;
    int32_t* ulb;          // [ntot] union window over layers
    int32_t* uub;
};

__device__ __forceinline__ int knot_idx(const double* k, int n, double x) {
    int i = int(search_last(k, n, x));
    return i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
}

// src/hydrogen_line_absorption.jl:100-144, one (transition, layer) per thread
template <bool MIXED>
__global__ void hline_prep_kernel(StarkDev st, HLayers hl, const double* wls, int64_t nwl, double window,
                                  int use_MHD, HOut out, double* Qbase) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int L = hl.L;
    if (idx >= st.ntrans * L) return;
    const int t = idx / L, l = idx % L;
    HRec r = {};
    r.kind = HK_OFF;
    r.lb = 0;
    r.ub = -1;
    r.nD = st.nD[t];
    const double T = hl.T[l], ne = hl.ne[l];
    const int nT = st.nT[t], nNe = st.nNe[t], nD = st.nD[t];
    const double* kT = st.temps + st.t_off[t];
    const double* kN = st.nes + st.ne_off[t];
    do {
        if (!(kT[0] < T && T < kT[nT - 1] && kN[0] < ne && ne < kN[nNe - 1])) break;  // :101-103
        const int i = knot_idx(kT, nT, T), j = knot_idx(kN, nNe, ne);
        const double wt = (T - kT[i]) / (kT[i + 1] - kT[i]);
        const double wn = (ne - kN[j]) / (kN[j + 1] - kN[j]);
        const double* L0 = st.lambda0 + st.l_off[t];
        // :104 bilinear line centre, every operation rounded separately (no FMA contraction):
        // table centres sit on 0.01 A multiples, so centre +- window often lands exactly on a
        // grid point and the window edge is decided by the last bit
        const double ut = __dsub_rn(1.0, wt), un = __dsub_rn(1.0, wn);
        double wl0 = __dmul_rn(__dmul_rn(ut, un), L0[j * nT + i]);
        wl0 = __dadd_rn(wl0, __dmul_rn(__dmul_rn(wt, un), L0[j * nT + i + 1]));
        wl0 = __dadd_rn(wl0, __dmul_rn(__dmul_rn(ut, wn), L0[(j + 1) * nT + i]));
        wl0 = __dadd_rn(wl0, __dmul_rn(__dmul_rn(wt, wn), L0[(j + 1) * nT + i + 1]));
        const int lo = st.lower[t], up = st.upper[t];
        const double beta = 1 / (KBOLTZ_EV * T);
        const double w = use_MHD ? hummer_mihalas_w(double(up), hl.nH[l], hl.nHe[l], ne) : 1.0;
        const double Elo = RYDBERGH_EV * (1 - 1.0 / (lo * lo));
        const double Eup = RYDBERGH_EV * (1 - 1.0 / (up * up));
        const double levels = w * (exp(-beta * Elo) - exp(-beta * Eup)) / hl.UH[l];        // :110
        const double amp = pow(10.0, st.log_gf[t]) * hl.nH[l] * sigma_line(wl0) * levels;  // :111
        const int64_t lb = search_first(wls, nwl, wl0 - window), ub = search_last(wls, nwl, wl0 + window);
        if (lb >= ub) break;  // :115-117
        r.lb = int32_t(lb);
        r.ub = int32_t(ub);
        r.amp = amp;
        r.kind = HK_STARK;
        if (lo == 2 && (up == 3 || up == 4 || up == 5)) {  // :120-137 Barklem p-d ABO profile
            double sABO, aABO;
            if (up == 3) { wl0 = 6.56460998e-5; sABO = 1180.0; aABO = 0.677; }
            else if (up == 4) { wl0 = 4.8626810200000004e-5; sABO = 2320.0; aABO = 0.455; }
            else { wl0 = 4.34168232e-5; sABO = 4208.0; aABO = 0.380; }
            const double Hmass = 1.008 * AMU_CGS;
            const double G = scaled_vdW_abo(sABO * (BOHR_RADIUS_CGS * BOHR_RADIUS_CGS), aABO, Hmass, T) * hl.nH[l];
            const double gam = G * (wl0 * wl0) / (C_CGS * (4 * PI));
            const double sig = doppler_width(wl0, T, Hmass, hl.xi[l]);
            r.inv_s = 1 / (sig * SQRT_2);
            r.a = gam * r.inv_s;
            r.scale = r.inv_s / SQRT_PI * amp;
            r.kind = HK_STARK_ABO;
        }
        r.wl0 = wl0;
        r.nu0 = C_CGS / (wl0);  // :140 (the ABO centre replaces the interpolated one)
        r.F0 = 1.25e-9 * pow(ne, 2.0 / 3.0);
        r.invF0 = 1 / r.F0;
        r.nu0_hi = float(r.nu0);
        r.nu0_lo = float(r.nu0 - double(r.nu0_hi));
        r.invF0_f = float(r.invF0);
        r.amp_f = float(amp);
        if (r.kind == HK_STARK_ABO) {
            const double sig = 1 / (r.inv_s * SQRT_2), gam = r.a / r.inv_s;
            const float af = float(r.a);
            r.abo32 = make_float4(float(2 * sig * sig), af,
                                  af <= 0.2f ? float(r.a / SQRT_PI * r.scale) : float(1 / (gam * gam)), float(r.scale));
        }
        // profile table at (T, ne) along the delta-nu knots
        const double* P = st.logP + st.p_off[t];
        double* Q = Qbase + (int64_t(t) * L + l) * HND_MAX;
        for (int k = 0; k < nD; k++) {
            const double* pk = P + int64_t(k) * nNe * nT;
            const double q = ((1 - wt) * (1 - wn)) * pk[j * nT + i] + (wt * (1 - wn)) * pk[j * nT + i + 1] +
                             ((1 - wt) * wn) * pk[(j + 1) * nT + i] + (wt * wn) * pk[(j + 1) * nT + i + 1];
            Q[k] = q;
            if (MIXED) out.Q32[(int64_t(t) * L + l) * HND_MAX + k] = float(q);
        }
        atomicMin(out.ulb + t, r.lb);
        atomicMax(out.uub + t, r.ub);
    } while (0);
    out.rec[int64_t(t) * L + l] = r;
}

// src/hydrogen_line_absorption.jl:451-470
__constant__ double c_holt_prob7[15][5] = {
    {0.005, 0.128, 0.260, 0.389, 0.504},     {0.004, 0.109, 0.220, 0.318, 0.389},
    {-0.007, 0.079, 0.162, 0.222, 0.244},    {-0.018, 0.041, 0.089, 0.106, 0.080},
    {-0.026, -0.003, 0.003, -0.023, -0.086}, {-0.025, -0.048, -0.087, -0.148, -0.234},
    {-0.008, -0.085, -0.165, -0.251, -0.343}, {0.018, -0.111, -0.223, -0.321, -0.407},
    {0.032, -0.130, -0.255, -0.354, -0.431}, {0.014, -0.148, -0.269, -0.359, -0.427},
    {-0.005, -0.140, -0.243, -0.323, -0.386}, {0.005, -0.095, -0.178, -0.248, -0.307},
    {-0.002, -0.068, -0.129, -0.187, -0.241}, {-0.007, -0.049, -0.094, -0.139, -0.186},
    {-0.010, -0.036, -0.067, -0.103, -0.143}};
__constant__ double c_holt_c7[5] = {511.318, 1.532, 4.044, 19.266, 41.812};
__constant__ double c_holt_d7[5] = {-6.070, -4.528, -8.759, -14.984, -23.956};
__constant__ double c_holt_pp[5] = {0.0, 0.2, 0.4, 0.6, 0.8};
__constant__ double c_holt_beta[15] = {1.0, 1.259, 1.585, 1.995, 2.512, 3.162, 3.981, 5.012,
                                       6.310, 7.943, 10.0, 12.59, 15.85, 19.95, 25.12};

// src/hydrogen_line_absorption.jl:402-448
__device__ double holtsmark_profile(double beta, double P) {
    if (beta > 500) return (1.5 / sqrt(beta) + 27 / (beta * beta)) / (beta * beta);
    int IM = int(floor((5 * P) + 1));
    if (IM > 4) IM = 4;
    const int IP = IM + 1;
    const double WTPP = 5 * (P - c_holt_pp[IM - 1]);
    const double WTPM = 1 - WTPP;
    if (beta <= 25.12) {
        int first = 15;
        for (int k = 0; k < 15; k++)
            if (beta <= c_holt_beta[k]) { first = k + 1; break; }
        const int JP = first > 2 ? first : 2, JM = JP - 1;
        const double WTBP = (beta - c_holt_beta[JM - 1]) / (c_holt_beta[JP - 1] - c_holt_beta[JM - 1]);
        const double WTBM = 1 - WTBP;
        const double CBP = c_holt_prob7[JP - 1][IP - 1] * WTPP + c_holt_prob7[JP - 1][IM - 1] * WTPM;
        const double CBM = c_holt_prob7[JM - 1][IP - 1] * WTPP + c_holt_prob7[JM - 1][IM - 1] * WTPM;
        const double CORR = 1 + CBP * WTBP + CBM * WTBM;
        const double WT = fmax(fmin(0.5 * (10 - beta), 1.0), 0.0);
        const double PR1 = beta <= 10 ? 8 / (83 + (2 + 0.95 * (beta * beta)) * beta) : 0.0;
        const double PR2 = beta >= 8 ? (1.5 / sqrt(beta) + 27 / (beta * beta)) / (beta * beta) : 0.0;
        return (PR1 * WT + PR2 * (1 - WT)) * CORR;
    }
    const double CC = c_holt_c7[IP - 1] * WTPP + c_holt_c7[IM - 1] * WTPM;
    const double DD = c_holt_d7[IP - 1] * WTPP + c_holt_d7[IM - 1] * WTPM;
    const double CORR = 1 + DD / (CC + beta * sqrt(beta));
    return (1.5 / sqrt(beta) + 27 / (beta * beta)) / (beta * beta) * CORR;
}

// src/hydrogen_line_absorption.jl:371-393
__device__ __forceinline__ double greim_1960_Knm(int n, int m) {
    if ((m - n <= 3) && (n <= 4)) {
        const double tab4[3] = {0.5820000, 0.8660000, 1.0200000};  // column n = 4 (Brackett)
        return tab4[m - n - 1];
    }
    const double n4 = double(n) * n * n * n, m4 = double(m) * m * m * m;
    return 5.5e-5 * n4 * m4 / double(m * m - n * n) / (1 + 0.13 / (m - n));
}

// src/hydrogen_line_absorption.jl:174-184
__device__ __forceinline__ double brackett_oscillator_strength(int n, int m) {
    const double GINF = 0.2027 / pow(double(n), 0.71);
    const double GCA = 0.124 / n;
    const double FKN = 1.9603 * n;
    const double WTC = 0.45 - 2.4 / double(n * n * n) * (n - 1);
    const double r = double(m) / double((m - n) * (m + n));
    const double FK = FKN * (r * r * r);
    const double XMN12 = pow(double(m - n), 1.2);
    const double WT = (XMN12 - 1) / (XMN12 + WTC);
    return FK * (1 - WT * GINF - (0.222 + GCA / m) * (1 - WT));
}

// One CTA per (m, layer): the Brackett line m profile (:147-162, :211-251, :272-369).
template <bool MIXED>
__global__ void __launch_bounds__(256) brackett_prep_kernel(HLayers hl, int ntrans, int n_max, const double* wls,
                                                            int64_t nwl, int use_MHD, HOut out, double* Qbase) {
    __shared__ double s_grid[BR_NP], s_imp[BR_NP], s_qs[BR_NP], s_tmp[BR_NP];
    __shared__ int s_red;
    const int n = 4, m = 5 + blockIdx.x, l = blockIdx.y, L = hl.L, k = threadIdx.x;
    const int slot = ntrans + blockIdx.x;
    const double T = hl.T[l], ne = hl.ne[l];
    const double E = RYDBERGH_EV * (1.0 / (n * n) - 1.0 / (m * m));
    const double wl0 = HPLANCK_EV * C_CGS / E;
    const double F0 = 1.25e-9 * pow(ne, 2.0 / 3.0);
    const double Knm = greim_1960_Knm(n, m);
    const double stark_width = 1.6678E-18 * Knm * F0 * C_CGS;
    const double sdop = doppler_width(wl0, T, 1.008 * AMU_CGS, hl.xi[l]);
    const double window = 5 * fmax(sdop, stark_width);
    const double wlmin = wls[0], wlmax = wls[nwl - 1];
    const double wstart = fmax(wlmin, wl0 - window), wend = fmin(wl0 + window, wlmax);
    HRec r = {};
    r.kind = HK_OFF;
    r.lb = 0;
    r.ub = -1;
    r.nD = BR_NP;
    if (wstart > wlmax || wend < wlmin || wstart == wend) {  // :228-232, no-op interpolator
        if (k == 0) out.rec[int64_t(slot) * L + l] = r;
        return;
    }
    const double step = (wend - wstart) / (BR_NP - 1);
    const double nu0 = C_CGS / wl0;
    if (k < BR_NP) s_grid[k] = (k == BR_NP - 1) ? wend : wstart + k * step;
    if (k == 0) s_red = -1;
    __syncthreads();
    // brackett_line_stark_profiles (:272-369)
    const double ne_1_6 = pow(ne, 1.0 / 6.0);
    const double GCON1 = 0.2 + 0.09 * sqrt(T / 10000) / (1 + ne / 1.E13);
    const double GCON2 = 0.2 / (1 + ne / 1.E15);
    const double Y1WHT = (m - n <= 3) ? 1e14 : 1e13;
    const double WTY1 = 1 / (1 + ne / Y1WHT);
    const double Y1B = 2 / (1 + 0.012 / T * sqrt(ne / T));
    const double mm_nn = double(m * m - n * n);
    const double C1CON = Knm / wl0 * (mm_nn * mm_nn) / double(n * n * m * m) * 1e-8;
    const double Y1SCAL = 320 * (pow(T / 10000, 0.3) / ne_1_6) * WTY1 + Y1B * (1 - WTY1);
    const double C1 = F0 * 78940 / T * C1CON * Y1SCAL;
    const double kl = Knm / wl0;
    const double C2 = (F0 * F0) / (5.96E-23 * ne) * (kl * kl) * 1e-16;
    const double G1 = 6.77 * sqrt(C1);
    const double Pp = ne_1_6 * 0.08989 / sqrt(T);
    const double dbdl = 1e8 / (Knm * F0);
    if (k < BR_NP) {
        const double wl = s_grid[k];
        if (C_CGS / wl < nu0) atomicMax(&s_red, k);
        const double beta = fabs(wl - wl0) / F0 / Knm * 1e8;
        const double y1 = C1 * beta, y2 = C2 * (beta * beta);
        double width;
        if ((y2 <= 1e-4) && (y1 <= 1e-5)) {
            width = G1 * fmax(0.0, 0.2114 + log(sqrt(C2) / C1)) * (1 - GCON1 - GCON2);
        } else {
            const double t90 = 90 * y1;
            const double GAM = (G1 * (0.5 * exp(-fmin(80.0, y1)) + expint1_64(y1) - 0.5 * expint1_64(y2)) *
                                (1 - GCON1 / (1 + t90 * t90 * t90) - GCON2 / (1 + 2000 * y1)));
            width = GAM <= 1e-20 ? 0.0 : GAM;
        }
        s_imp[k] = width > 0 ? width / (PI * (width * width + beta * beta)) : 0.0;
        const double ps = (0.9 * y1) * (0.9 * y1);
        double qe = (ps + 0.03 * sqrt(y1)) / (ps + 1.0);
        s_qs[k] = holtsmark_profile(beta, Pp) * (1 + qe);
    }
    __syncthreads();
    if (k < BR_NP) {
        const double wl = s_grid[k];
        const double f = sqrt(wl / wl0);
        double a = s_imp[k] * f, b = s_qs[k] * f;
        if (k <= s_red) {
            const double bz = exp((HPLANCK_CGS * (C_CGS / wl - nu0)) / KBOLTZ_CGS / T);
            a = a * bz;
            b = b * bz;
        }
        s_imp[k] = a * dbdl;
        s_qs[k] = b * dbdl;
    }
    __syncthreads();
    const int start = (BR_NP + 1) / 2 - 1;
    if (sdop / stark_width > 0.25) {  // :240-244 Doppler convolution of the quasistatic part
        if (k < BR_NP) {
            const double d = s_grid[k] - wl0;
            s_tmp[k] = exp(-0.5 * (d * d) / (sdop * sdop)) / SQRT_2PI / sdop;
        }
        __syncthreads();
        double s = 0;
        if (k < BR_NP) {
            const int q = start + k;
            const int lo = q - (BR_NP - 1) > 0 ? q - (BR_NP - 1) : 0, hi = q < BR_NP - 1 ? q : BR_NP - 1;
            for (int i = lo; i <= hi; i++) s += s_qs[i] * s_tmp[q - i];
        }
        __syncthreads();
        if (k < BR_NP) s_qs[k] = s * step;
        __syncthreads();
    }
    double* Q = Qbase + (int64_t(blockIdx.x) * L + l) * BR_NP;
    if (k < BR_NP) {  // :247-249 impact (x) quasistatic
        const int q = start + k;
        const int lo = q - (BR_NP - 1) > 0 ? q - (BR_NP - 1) : 0, hi = q < BR_NP - 1 ? q : BR_NP - 1;
        double s = 0;
        for (int i = lo; i <= hi; i++) s += s_imp[i] * s_qs[q - i];
        Q[k] = s * step;
    }
    if (k == 0) {
        const double beta = 1 / (KBOLTZ_EV * T);
        const double E_low = RYDBERGH_EV * (1 - 1.0 / (n * n));
        const double w = use_MHD ? hummer_mihalas_w(double(m), hl.nH[l], hl.nHe[l], ne) : 1.0;
        const double levels = w * exp(-beta * E_low) * (1 - exp(-beta * E)) / hl.UH[l];
        const double gf = 2 * (n * n) * brackett_oscillator_strength(n, m);
        r.amp = gf * hl.nH[l] * sigma_line(wl0) * levels;
        const int64_t lb = search_first(wls, nwl, wl0 - window), ub = search_last(wls, nwl, wl0 + window);
        r.lb = int32_t(lb);
        r.ub = int32_t(ub);
        r.kind = lb <= ub ? HK_BRACKETT : HK_OFF;
        r.wl0 = wstart;  // grid start
        r.inv_s = step;  // grid step
        r.a = 1 / step;
        out.rec[int64_t(slot) * L + l] = r;
        if (lb <= ub) {
            atomicMin(out.ulb + slot, r.lb);
            atomicMax(out.uub + slot, r.ub);
        }
    }
}

struct HTileArgs {
    double* alpha;
    const double* wls;
    int64_t nwl;
    int32_t L, G, ntrans, ntot;
    const HRec* rec;
    const double* Q;       // Stehle tables then Brackett profiles
    const float* Q32;
    const int32_t *ulb, *uub;
    const int64_t* d_off;
    const double* logdnu;
    const float* logdnu32;
};

template <bool MIXED, int KMAX>
__global__ void __launch_bounds__(512, (MIXED && KMAX <= 16) ? 2 : 1) hline_tile_kernel(HTileArgs a) {
    const int tid = threadIdx.x;
    const int L = a.L, G = a.G;
    const int TW = blockDim.x / G;
    const int jl = tid % TW, g = tid / TW;
    const int64_t j0 = int64_t(blockIdx.x) * TW, jg = j0 + jl;
    const int64_t jlast = min(j0 + TW, a.nwl) - 1;
    const bool live = jg < a.nwl;
    const double wl = live ? a.wls[jg] : 1.0;
    const double nu = C_CGS / wl;                // :78
    const double dnudl = C_CGS / (wl * wl);      // :79
    const float nu_hi = float(nu), nu_lo = float(nu - double(nu_hi)), dnudl_f = float(dnudl);
    // FP64 accumulators (plain) or FP32 with Kahan compensation (mixed)
    using Acc = typename std::conditional<MIXED, float, double>::type;
    Acc acc[KMAX], comp[KMAX];
#pragma unroll
    for (int k = 0; k < KMAX; k++) { acc[k] = Acc(0); comp[k] = Acc(0); }
    const int64_t brQ = int64_t(a.ntrans) * L * HND_MAX;
    for (int t = 0; t < a.ntot; t++) {
        if (a.uub[t] < j0 || a.ulb[t] > jlast) continue;  // uniform across the CTA
        if (!live) continue;
        const double* kd = t < a.ntrans ? a.logdnu + a.d_off[t] : nullptr;
        const float* kd32 = t < a.ntrans ? a.logdnu32 + a.d_off[t] : nullptr;
        int hint = -1;  // knot interval of the previous layer of this transition (mixed)
#pragma unroll
        for (int k = 0; k < KMAX; k++) {
            const int l = g + G * k;
            if (l >= L) continue;
            const HRec& r = a.rec[int64_t(t) * L + l];
            if (r.kind == HK_OFF || jg < r.lb || jg > r.ub) continue;
            if (r.kind == HK_BRACKETT) {
                // linear_interpolation over the 201-point range grid (:249, :160); the position on
                // the grid by the reciprocal step (one rounding more than a division, no FP64 divide)
                const double u = (wl - r.wl0) * r.a;
                int i = int(floor(u));
                i = i < 0 ? 0 : (i > BR_NP - 2 ? BR_NP - 2 : i);
                const double d = u - i;
                const double* q = a.Q + brQ + (int64_t(t - a.ntrans) * L + l) * BR_NP;
                const double term = (q[i] * (1 - d) + q[i + 1] * d) * r.amp;
                if (MIXED) {
                    const float y = float(term) - float(comp[k]), tt = float(acc[k]) + y;
                    comp[k] = Acc((tt - float(acc[k])) - y);
                    acc[k] = Acc(tt);
                } else {
                    acc[k] += Acc(term);
                }
                continue;
            }
            const int nDt = r.nD;
            if (MIXED) {
                float v32 = 0.f;
                if (r.kind == HK_STARK_ABO) {  // :136
                    const float x = float(fabs(wl - r.wl0));
                    v32 = profile32x(r.abo32, x, __fdividef(1.f, x * x));
                }
                // :140-143, frequency offset from FP32 pairs (exact difference of the high parts)
                const float dnu = fabsf((nu_hi - r.nu0_hi) + (nu_lo - r.nu0_lo));
                const float x = __logf(dnu * r.invF0_f);
                const float* Q = a.Q32 + (int64_t(t) * L + l) * HND_MAX;
                float v;
                if (!(x > kd32[1])) {
                    v = Q[1];
                } else if (x >= kd32[nDt - 1]) {
                    v = Q[nDt - 1];
                } else {
                    // kd32[1] < x < kd32[nDt - 1]: the interval with kd32[lo] <= x < kd32[lo + 1].
                    // Neighbouring layers differ little in log(dnu / F0), so after the first
                    // layer the interval is found by walking from the previous one (both walks
                    // stop inside [1, nDt - 2] by the bounds on x); the result is the binary
                    // search's.
                    int lo;
                    if (hint < 0) {
                        lo = 1;
                        int hi = nDt - 1;
                        while (hi - lo > 1) {
                            const int mid = (lo + hi) >> 1;
                            if (kd32[mid] <= x) lo = mid; else hi = mid;
                        }
                    } else {
                        lo = min(max(hint, 1), nDt - 2);
                        while (kd32[lo] > x) lo--;
                        while (kd32[lo + 1] <= x) lo++;
                    }
                    hint = lo;
                    const float w = (x - kd32[lo]) / (kd32[lo + 1] - kd32[lo]);
                    v = (1.f - w) * Q[lo] + w * Q[lo + 1];
                }
                const float term = v32 + __expf(v) * dnudl_f * r.amp_f;
                const float y = term - float(comp[k]), tt = float(acc[k]) + y;
                comp[k] = Acc((tt - float(acc[k])) - y);
                acc[k] = Acc(tt);
            } else {
                if (r.kind == HK_STARK_ABO) acc[k] += Acc(voigt64(r.a, fabs(wl - r.wl0) * r.inv_s) * r.scale);  // :136
                double sd = fabs(nu - r.nu0) / r.F0;  // :141
                sd = sd + (sd == 0) * 2.2250738585072014e-308;  // _zero2epsilon
                const double x = log(sd);
                const double* Q = a.Q + (int64_t(t) * L + l) * HND_MAX;
                double v;
                if (!(x > kd[1])) {
                    v = Q[1];  // first interval: the weight of the -floatmax knot rounds to 0
                } else if (x >= kd[nDt - 1]) {
                    v = Q[nDt - 1];  // flat extrapolation
                } else {
                    int lo = 1, hi = nDt - 1;
                    while (hi - lo > 1) {
                        const int mid = (lo + hi) >> 1;
                        if (kd[mid] <= x) lo = mid; else hi = mid;
                    }
                    const double w = (x - kd[lo]) / (kd[lo + 1] - kd[lo]);
                    v = (1 - w) * Q[lo] + w * Q[lo + 1];
                }
                acc[k] += Acc(exp(v) * dnudl * r.amp);  // :142-143
            }
        }
    }
    if (live) {
#pragma unroll
        for (int k = 0; k < KMAX; k++) {
            const int l = g + G * k;
            if (l < L) {
                double* dst = a.alpha + jg * L + l;
                *dst = *dst + (MIXED ? double(acc[k]) - double(comp[k]) : double(acc[k]));
            }
        }
    }
}

}  // namespace korg
