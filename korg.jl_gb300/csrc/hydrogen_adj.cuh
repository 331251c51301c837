// hydrogen_adj.cuh -- reverse mode of the hydrogen-line opacity (hydrogen_line_absorption!,
// src/hydrogen_line_absorption.jl:75-163): the exact derivatives of the restated approximation
// with respect to each layer's T, n_e, xi, n(H I) and n(He I), and U(H I) (alpha_H is
// proportional to 1/U(H I)), contracted with the opacity cotangent G.  What ForwardDiff takes
// through the reference: the derivative of each branch the value selects, the windows held fixed.
//
//   hline_adj_prep:    one thread per (Stehle transition, layer): forward-mode dual numbers over
//                      the five per-layer inputs through the line centre, amplitude (with the MHD
//                      occupation probability), F0 and the ABO Voigt constants, and the exact
//                      derivatives of the (T, n_e)-interpolated profile table.
//   brackett_adj_prep: one CTA per (upper level m, layer): the Brackett profile of
//                      brackett_prep_kernel on dual numbers in (T, n_e, xi), grid and convolutions
//                      included.
//   hline_adj:         one warp per 32-wavelength tile (grid-stride), loops over layers and the
//                      transitions in reach of the tile; per (wavelength, layer) the opacity and
//                      its five derivatives from the forward's records and the derivative
//                      records, times G, reduced over the warp into shared per-layer sums.
#pragma once
#include "adjoint.cuh"
#include "hydrogen.cuh"

namespace korg {

constexpr int HP = 5;  // derivative directions: T, n_e, xi, n(H I), n(He I)
enum { HD_T = 0, HD_NE = 1, HD_XI = 2, HD_NH = 3, HD_NHE = 4 };
constexpr int HADJ_MAXT = 128;  // transitions (Stehle + Brackett) the tile kernel's masks hold
constexpr int HADJ_WARPS = 8;

// ---------------------------------------------------------------- dual numbers in N inputs
template <int N>
struct Dn {
    double v, d[N];
};
template <int N>
__device__ __forceinline__ Dn<N> dn_const(double v) {
    Dn<N> r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = 0.0;
    return r;
}
template <int N>
__device__ __forceinline__ Dn<N> dn_var(double v, int k) {
    Dn<N> r = dn_const<N>(v);
    if (k < N) r.d[k] = 1.0;
    return r;
}
// f(p) with f(p.v) = fv and f'(p.v) = fd
template <int N>
__device__ __forceinline__ Dn<N> dn_chain(const Dn<N>& p, double fv, double fd) {
    Dn<N> r;
    r.v = fv;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = fd * p.d[i];
    return r;
}
template <int N>
__device__ __forceinline__ Dn<N> operator+(const Dn<N>& p, const Dn<N>& q) {
    Dn<N> r;
    r.v = p.v + q.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = p.d[i] + q.d[i];
    return r;
}
template <int N>
__device__ __forceinline__ Dn<N> operator-(const Dn<N>& p, const Dn<N>& q) {
    Dn<N> r;
    r.v = p.v - q.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = p.d[i] - q.d[i];
    return r;
}
template <int N>
__device__ __forceinline__ Dn<N> operator*(const Dn<N>& p, const Dn<N>& q) {
    Dn<N> r;
    r.v = p.v * q.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = p.d[i] * q.v + p.v * q.d[i];
    return r;
}
template <int N>
__device__ __forceinline__ Dn<N> operator/(const Dn<N>& p, const Dn<N>& q) {
    const double inv = 1.0 / q.v, v = p.v * inv;
    Dn<N> r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = (p.d[i] - v * q.d[i]) * inv;
    return r;
}
template <int N>
__device__ __forceinline__ Dn<N> operator+(const Dn<N>& p, double c) { return dn_chain(p, p.v + c, 1.0); }
template <int N>
__device__ __forceinline__ Dn<N> operator+(double c, const Dn<N>& p) { return dn_chain(p, c + p.v, 1.0); }
template <int N>
__device__ __forceinline__ Dn<N> operator-(const Dn<N>& p, double c) { return dn_chain(p, p.v - c, 1.0); }
template <int N>
__device__ __forceinline__ Dn<N> operator-(double c, const Dn<N>& p) { return dn_chain(p, c - p.v, -1.0); }
template <int N>
__device__ __forceinline__ Dn<N> operator-(const Dn<N>& p) { return dn_chain(p, -p.v, -1.0); }
template <int N>
__device__ __forceinline__ Dn<N> operator*(const Dn<N>& p, double c) { return dn_chain(p, p.v * c, c); }
template <int N>
__device__ __forceinline__ Dn<N> operator*(double c, const Dn<N>& p) { return dn_chain(p, c * p.v, c); }
template <int N>
__device__ __forceinline__ Dn<N> operator/(const Dn<N>& p, double c) { return dn_chain(p, p.v / c, 1.0 / c); }
template <int N>
__device__ __forceinline__ Dn<N> operator/(double c, const Dn<N>& q) {
    const double v = c / q.v;
    return dn_chain(q, v, -v / q.v);
}
template <int N>
__device__ __forceinline__ Dn<N> dn_exp(const Dn<N>& p) {
    const double e = exp(p.v);
    return dn_chain(p, e, e);
}
template <int N>
__device__ __forceinline__ Dn<N> dn_log(const Dn<N>& p) { return dn_chain(p, log(p.v), 1.0 / p.v); }
// at 0 the derivative is taken as 0: the one argument that reaches sqrt(0) is the Brackett
// profile's y1 at the grid point that sits on the line centre, which stays there (its tangent is 0)
template <int N>
__device__ __forceinline__ Dn<N> dn_sqrt(const Dn<N>& p) {
    const double s = sqrt(p.v);
    return dn_chain(p, s, s > 0 ? 0.5 / s : 0.0);
}
template <int N>
__device__ __forceinline__ Dn<N> dn_pow(const Dn<N>& p, double c) {
    const double v = pow(p.v, c);
    return dn_chain(p, v, c * v / p.v);
}
template <int N>
__device__ __forceinline__ Dn<N> dn_fabs(const Dn<N>& p) { return p.v < 0 ? -p : p; }
// max / min select the branch the values pick (a tie takes the second argument, as Julia's max)
template <int N>
__device__ __forceinline__ Dn<N> dn_fmax(const Dn<N>& p, double c) { return p.v > c ? p : dn_const<N>(c); }
template <int N>
__device__ __forceinline__ Dn<N> dn_fmax(double c, const Dn<N>& p) { return c > p.v ? dn_const<N>(c) : p; }
template <int N>
__device__ __forceinline__ Dn<N> dn_fmax(const Dn<N>& p, const Dn<N>& q) { return p.v > q.v ? p : q; }
template <int N>
__device__ __forceinline__ Dn<N> dn_fmin(const Dn<N>& p, double c) { return p.v < c ? p : dn_const<N>(c); }

// ---------------------------------------------------------------- physics on dual numbers
// src/statmech.jl:463-497 (default branch), n(H I), n(He I), n_e dual
template <int N>
__device__ Dn<N> hummer_mihalas_w_dn(double n_eff, const Dn<N>& nH, const Dn<N>& nHe, const Dn<N>& ne) {
    const double n2 = n_eff * n_eff, n4 = n2 * n2;
    const double r_level = sqrt(5.0 / 2.0 * n4 + 1.0 / 2.0 * n2) * BOHR_RADIUS_CGS;
    const double a = r_level + 1.7320508075688772 * BOHR_RADIUS_CGS, b = r_level + 1.02 * BOHR_RADIUS_CGS;
    const Dn<N> neutral_term = nH * (a * a * a) + nHe * (b * b * b);
    double K = 1.0;
    if (n_eff > 3) {
        const double r = n_eff / (n_eff + 1);
        K = 16.0 / 3.0 * (r * r) * ((n_eff + 7.0 / 6.0) / (n2 + n_eff + 1.0 / 2.0));
    }
    const double chi = RYDBERGH_EV / n2 * EV_TO_CGS;
    const double e = ELECTRON_CHARGE_CGS;
    const double q = (e * e) / (chi * sqrt(K));
    const Dn<N> charged_term = ne * (16 * (q * q * q));
    return dn_exp((neutral_term + charged_term) * (-(4 * PI) / 3));
}

// src/line_absorption.jl:169-182, differentiated branch by branch
template <int N>
__device__ Dn<N> expint1_dn(const Dn<N>& x) {
    if (x.v < 0) return dn_const<N>(0.0);
    if (x.v <= 0.01) return -dn_log(x) - 0.577215 + x;
    if (x.v <= 1.0)
        return -dn_log(x) - 0.57721566 +
               x * (0.99999193 + x * (-0.24991055 + x * (0.05519968 + x * (-0.00976004 + x * 0.00107857))));
    if (x.v <= 30.0)
        return (x * (x + 2.334733) + 0.25062) / (x * (x + 3.330657) + 1.681534) / x * dn_exp(-x);
    return dn_const<N>(0.0);
}

// src/hydrogen_line_absorption.jl:402-448 (tables in hydrogen.cuh), on dual numbers
template <int N>
__device__ Dn<N> holtsmark_profile_dn(const Dn<N>& beta, const Dn<N>& P) {
    const Dn<N> b2 = beta * beta;
    auto far = [&]() { return (1.5 / dn_sqrt(beta) + 27.0 / b2) / b2; };
    if (beta.v > 500) return far();
    int IM = int(floor((5 * P.v) + 1));
    if (IM > 4) IM = 4;
    const int IP = IM + 1;
    const Dn<N> WTPP = (P - c_holt_pp[IM - 1]) * 5.0;
    const Dn<N> WTPM = 1.0 - WTPP;
    if (beta.v <= 25.12) {
        int first = 15;
        for (int k = 0; k < 15; k++)
            if (beta.v <= c_holt_beta[k]) { first = k + 1; break; }
        const int JP = first > 2 ? first : 2, JM = JP - 1;
        const Dn<N> WTBP = (beta - c_holt_beta[JM - 1]) / (c_holt_beta[JP - 1] - c_holt_beta[JM - 1]);
        const Dn<N> WTBM = 1.0 - WTBP;
        const Dn<N> CBP = WTPP * c_holt_prob7[JP - 1][IP - 1] + WTPM * c_holt_prob7[JP - 1][IM - 1];
        const Dn<N> CBM = WTPP * c_holt_prob7[JM - 1][IP - 1] + WTPM * c_holt_prob7[JM - 1][IM - 1];
        const Dn<N> CORR = 1.0 + CBP * WTBP + CBM * WTBM;
        const Dn<N> WT = dn_fmax(dn_fmin((10.0 - beta) * 0.5, 1.0), 0.0);
        const Dn<N> PR1 = beta.v <= 10 ? 8.0 / (83.0 + (2.0 + 0.95 * b2) * beta) : dn_const<N>(0.0);
        const Dn<N> PR2 = beta.v >= 8 ? far() : dn_const<N>(0.0);
        return (PR1 * WT + PR2 * (1.0 - WT)) * CORR;
    }
    const Dn<N> CC = WTPP * c_holt_c7[IP - 1] + WTPM * c_holt_c7[IM - 1];
    const Dn<N> DD = WTPP * c_holt_d7[IP - 1] + WTPM * c_holt_d7[IM - 1];
    const Dn<N> CORR = 1.0 + DD / (CC + beta * dn_sqrt(beta));
    return far() * CORR;
}

// Derivative records, per (transition, layer), d/d(T, n_e, xi, n(H I), n(He I)) of:
struct HDer {
    double amp[HP];    // the amplitude
    double c[HP];      // Stehle: the line centre frequency nu0; Brackett: the profile grid's start
    double f[HP];      // Stehle: log F0; Brackett: the profile grid's step
    double inv_s[HP];  // ABO Voigt: 1 / (sigma sqrt 2)
    double a[HP];      //           the damping parameter
    double scale[HP];  //           inv_s / sqrt(pi) * amp
};
// The same in FP32 for the mixed-precision tile kernel, with values: Stehle lines the ABO Voigt
// constants (a, inv_s, scale); Brackett lines the grid's 1 / step in a_v and the amplitude in scale_v.
struct HDer32 {
    float amp[HP], c[HP], f[HP], inv_s[HP], a[HP], scale[HP];
    float a_v, inv_s_v, scale_v, pad;
};

// src/hydrogen_line_absorption.jl:100-144 on dual numbers, one (transition, layer) per thread;
// rec and Q are the forward prep's (plain FP64) records.  dQ [ntrans][L][2][HND_MAX]: d/dT and
// d/dn_e of the profile table at (T, n_e).  der32 / dQ32 (mixed precision; may be null): FP32 copies.
__global__ void hline_adj_prep_kernel(StarkDev st, HLayers hl, int use_MHD, const HRec* __restrict__ rec,
                                      HDer* __restrict__ der, double* __restrict__ dQ, HDer32* __restrict__ der32,
                                      float* __restrict__ dQ32) {
    using D = Dn<HP>;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int L = hl.L;
    if (idx >= st.ntrans * L) return;
    const int t = idx / L, l = idx % L;
    const HRec r = rec[int64_t(t) * L + l];
    if (r.kind == HK_OFF) return;  // the adjoint tile kernel reads no record of an inactive line
    const D T = dn_var<HP>(hl.T[l], HD_T), ne = dn_var<HP>(hl.ne[l], HD_NE), xi = dn_var<HP>(hl.xi[l], HD_XI);
    const D nH = dn_var<HP>(hl.nH[l], HD_NH), nHe = dn_var<HP>(hl.nHe[l], HD_NHE);
    const int nT = st.nT[t], nNe = st.nNe[t], nD = st.nD[t];
    const double* kT = st.temps + st.t_off[t];
    const double* kN = st.nes + st.ne_off[t];
    const int i = knot_idx(kT, nT, T.v), j = knot_idx(kN, nNe, ne.v);
    const double hT = 1.0 / (kT[i + 1] - kT[i]), hN = 1.0 / (kN[j + 1] - kN[j]);
    const D wt = (T - kT[i]) * hT, wn = (ne - kN[j]) * hN;
    const double* L0 = st.lambda0 + st.l_off[t];
    const D ut = 1.0 - wt, un = 1.0 - wn;
    D wl0 = ut * un * L0[j * nT + i] + wt * un * L0[j * nT + i + 1] + ut * wn * L0[(j + 1) * nT + i] +
            wt * wn * L0[(j + 1) * nT + i + 1];
    const int lo = st.lower[t], up = st.upper[t];
    const D beta = 1.0 / (T * KBOLTZ_EV);
    const D w = use_MHD ? hummer_mihalas_w_dn<HP>(double(up), nH, nHe, ne) : dn_const<HP>(1.0);
    const double Elo = RYDBERGH_EV * (1 - 1.0 / (lo * lo));
    const double Eup = RYDBERGH_EV * (1 - 1.0 / (up * up));
    const D levels = w * (dn_exp(-beta * Elo) - dn_exp(-beta * Eup)) / hl.UH[l];
    // sigma_line(wl) is proportional to wl^2
    const D amp = nH * (pow(10.0, st.log_gf[t]) * sigma_line(1.0)) * (wl0 * wl0) * levels;
    HDer o;
#pragma unroll
    for (int p = 0; p < HP; p++) {
        o.amp[p] = amp.d[p];
        o.c[p] = 0.0;
        o.inv_s[p] = o.a[p] = o.scale[p] = 0.0;
    }
    if (r.kind == HK_STARK_ABO) {
        double sABO, aABO;
        if (up == 3) { sABO = 1180.0; aABO = 0.677; }
        else if (up == 4) { sABO = 2320.0; aABO = 0.455; }
        else { sABO = 4208.0; aABO = 0.380; }
        const double wla = r.wl0;  // the ABO centre (a constant)
        const double Hmass = 1.008 * AMU_CGS;
        // scaled_vdW_abo is proportional to T^((1 - alpha) / 2)
        const D Tr = T / T.v;
        const D G = dn_pow(Tr, (1 - aABO) / 2) * nH *
                    scaled_vdW_abo(sABO * (BOHR_RADIUS_CGS * BOHR_RADIUS_CGS), aABO, Hmass, T.v);
        const D gam = G * ((wla * wla) / (C_CGS * (4 * PI)));
        const D sig = dn_sqrt(T * (KBOLTZ_CGS / Hmass) + xi * xi * 0.5) * (wla / C_CGS);
        const D inv_s = 1.0 / (sig * SQRT_2);
        const D a = gam * inv_s;
        const D scale = inv_s * amp / SQRT_PI;
#pragma unroll
        for (int p = 0; p < HP; p++) {
            o.inv_s[p] = inv_s.d[p];
            o.a[p] = a.d[p];
            o.scale[p] = scale.d[p];
        }
    } else {
        const D nu0 = C_CGS / wl0;
#pragma unroll
        for (int p = 0; p < HP; p++) o.c[p] = nu0.d[p];
    }
    const D lnF0 = dn_log(dn_pow(ne, 2.0 / 3.0) * 1.25e-9);
#pragma unroll
    for (int p = 0; p < HP; p++) o.f[p] = lnF0.d[p];
    der[int64_t(t) * L + l] = o;
    if (der32) {
        HDer32 o32;
#pragma unroll
        for (int p = 0; p < HP; p++) {
            o32.amp[p] = float(o.amp[p]);
            o32.c[p] = float(o.c[p]);
            o32.f[p] = float(o.f[p]);
            o32.inv_s[p] = float(o.inv_s[p]);
            o32.a[p] = float(o.a[p]);
            o32.scale[p] = float(o.scale[p]);
        }
        o32.a_v = float(r.a);
        o32.inv_s_v = float(r.inv_s);
        o32.scale_v = float(r.scale);
        o32.pad = 0.f;
        der32[int64_t(t) * L + l] = o32;
    }
    const double* P = st.logP + st.p_off[t];
    double* dq = dQ + (int64_t(t) * L + l) * 2 * HND_MAX;
    float* dq32 = dQ32 ? dQ32 + (int64_t(t) * L + l) * 2 * HND_MAX : nullptr;
    const double wtv = wt.v, wnv = wn.v;
    for (int k = 0; k < nD; k++) {
        const double* pk = P + int64_t(k) * nNe * nT;
        const double q00 = pk[j * nT + i], q01 = pk[j * nT + i + 1], q10 = pk[(j + 1) * nT + i],
                     q11 = pk[(j + 1) * nT + i + 1];
        dq[k] = ((1 - wnv) * (q01 - q00) + wnv * (q11 - q10)) * hT;
        dq[HND_MAX + k] = ((1 - wtv) * (q10 - q00) + wtv * (q11 - q01)) * hN;
        if (dq32) {
            dq32[k] = float(dq[k]);
            dq32[HND_MAX + k] = float(dq[HND_MAX + k]);
        }
    }
}

// brackett_prep_kernel (src/hydrogen_line_absorption.jl:147-162, :211-251, :272-369) on dual
// numbers in (T, n_e, xi); dQ [nbr][L][3][BR_NP]: the profile's derivatives on its grid.  Mixed
// precision (der32, q32 not null): FP32 records and q32 [nbr][L][4][BR_NP], the profile and its
// three derivatives.
__global__ void __launch_bounds__(256) brackett_adj_prep_kernel(HLayers hl, int ntrans, const double* wls,
                                                                int64_t nwl, int use_MHD, const HRec* __restrict__ rec,
                                                                HDer* __restrict__ der, double* __restrict__ dQ,
                                                                HDer32* __restrict__ der32, float* __restrict__ q32) {
    using D = Dn<3>;
    __shared__ D s_grid[BR_NP], s_imp[BR_NP], s_qs[BR_NP], s_tmp[BR_NP];
    __shared__ int s_red;
    const int n = 4, m = 5 + blockIdx.x, l = blockIdx.y, L = hl.L, k = threadIdx.x;
    const int slot = ntrans + blockIdx.x;
    if (rec[int64_t(slot) * L + l].kind == HK_OFF) return;  // uniform across the CTA
    const D T = dn_var<3>(hl.T[l], HD_T), ne = dn_var<3>(hl.ne[l], HD_NE), xi = dn_var<3>(hl.xi[l], HD_XI);
    const double E = RYDBERGH_EV * (1.0 / (n * n) - 1.0 / (m * m));
    const double wl0 = HPLANCK_EV * C_CGS / E;
    const D F0 = dn_pow(ne, 2.0 / 3.0) * 1.25e-9;
    const double Knm = greim_1960_Knm(n, m);
    const D stark_width = F0 * (1.6678E-18 * Knm * C_CGS);
    const double Hmass = 1.008 * AMU_CGS;
    const D sdop = dn_sqrt(T * (KBOLTZ_CGS / Hmass) + xi * xi * 0.5) * (wl0 / C_CGS);
    const D window = dn_fmax(sdop, stark_width) * 5.0;
    const double wlmin = wls[0], wlmax = wls[nwl - 1];
    const D wstart = dn_fmax(wlmin, wl0 - window), wend = dn_fmin(wl0 + window, wlmax);
    const D step = (wend - wstart) / double(BR_NP - 1);
    const double nu0 = C_CGS / wl0;
    if (k < BR_NP) s_grid[k] = (k == BR_NP - 1) ? wend : wstart + step * double(k);
    if (k == 0) s_red = -1;
    __syncthreads();
    const D ne_1_6 = dn_pow(ne, 1.0 / 6.0);
    const D GCON1 = 0.2 + 0.09 * dn_sqrt(T / 10000.0) / (1.0 + ne / 1.E13);
    const D GCON2 = 0.2 / (1.0 + ne / 1.E15);
    const double Y1WHT = (m - n <= 3) ? 1e14 : 1e13;
    const D WTY1 = 1.0 / (1.0 + ne / Y1WHT);
    const D Y1B = 2.0 / (1.0 + 0.012 / T * dn_sqrt(ne / T));
    const double mm_nn = double(m * m - n * n);
    const double C1CON = Knm / wl0 * (mm_nn * mm_nn) / double(n * n * m * m) * 1e-8;
    const D Y1SCAL = 320.0 * (dn_pow(T / 10000.0, 0.3) / ne_1_6) * WTY1 + Y1B * (1.0 - WTY1);
    const D C1 = F0 * 78940.0 / T * C1CON * Y1SCAL;
    const double kl = Knm / wl0;
    const D C2 = (F0 * F0) / (ne * 5.96E-23) * ((kl * kl) * 1e-16);
    const D G1 = 6.77 * dn_sqrt(C1);
    const D Pp = ne_1_6 * 0.08989 / dn_sqrt(T);
    const D dbdl = 1e8 / (F0 * Knm);
    if (k < BR_NP) {
        const D wl = s_grid[k];
        if (C_CGS / wl.v < nu0) atomicMax(&s_red, k);
        const D beta = dn_fabs(wl - wl0) / F0 / Knm * 1e8;
        const D y1 = C1 * beta, y2 = C2 * (beta * beta);
        D width;
        if ((y2.v <= 1e-4) && (y1.v <= 1e-5)) {
            width = G1 * dn_fmax(0.0, 0.2114 + dn_log(dn_sqrt(C2) / C1)) * (1.0 - GCON1 - GCON2);
        } else {
            const D t90 = 90.0 * y1;
            const D GAM = (G1 * (0.5 * dn_exp(-dn_fmin(y1, 80.0)) + expint1_dn(y1) - 0.5 * expint1_dn(y2)) *
                           (1.0 - GCON1 / (1.0 + t90 * t90 * t90) - GCON2 / (1.0 + 2000.0 * y1)));
            width = GAM.v <= 1e-20 ? dn_const<3>(0.0) : GAM;
        }
        s_imp[k] = width.v > 0 ? width / (PI * (width * width + beta * beta)) : dn_const<3>(0.0);
        const D ps = (0.9 * y1) * (0.9 * y1);
        const D qe = (ps + 0.03 * dn_sqrt(y1)) / (ps + 1.0);
        s_qs[k] = holtsmark_profile_dn(beta, Pp) * (1.0 + qe);
    }
    __syncthreads();
    if (k < BR_NP) {
        const D wl = s_grid[k];
        const D f = dn_sqrt(wl / wl0);
        D a = s_imp[k] * f, b = s_qs[k] * f;
        if (k <= s_red) {
            const D bz = dn_exp((HPLANCK_CGS * (C_CGS / wl - nu0)) / KBOLTZ_CGS / T);
            a = a * bz;
            b = b * bz;
        }
        s_imp[k] = a * dbdl;
        s_qs[k] = b * dbdl;
    }
    __syncthreads();
    const int start = (BR_NP + 1) / 2 - 1;
    if (sdop.v / stark_width.v > 0.25) {  // the Doppler convolution of the quasistatic part
        if (k < BR_NP) {
            const D d = s_grid[k] - wl0;
            s_tmp[k] = dn_exp(-0.5 * (d * d) / (sdop * sdop)) / SQRT_2PI / sdop;
        }
        __syncthreads();
        D s = dn_const<3>(0.0);
        if (k < BR_NP) {
            const int q = start + k;
            const int lo = q - (BR_NP - 1) > 0 ? q - (BR_NP - 1) : 0, hi = q < BR_NP - 1 ? q : BR_NP - 1;
            for (int i = lo; i <= hi; i++) s = s + s_qs[i] * s_tmp[q - i];
        }
        __syncthreads();
        if (k < BR_NP) s_qs[k] = s * step;
        __syncthreads();
    }
    if (k < BR_NP) {  // impact (x) quasistatic
        const int q = start + k;
        const int lo = q - (BR_NP - 1) > 0 ? q - (BR_NP - 1) : 0, hi = q < BR_NP - 1 ? q : BR_NP - 1;
        D s = dn_const<3>(0.0);
        for (int i = lo; i <= hi; i++) s = s + s_imp[i] * s_qs[q - i];
        s = s * step;
        double* dq = dQ + (int64_t(blockIdx.x) * L + l) * 3 * BR_NP;
#pragma unroll
        for (int p = 0; p < 3; p++) dq[p * BR_NP + k] = s.d[p];
        if (q32) {
            float* q = q32 + (int64_t(blockIdx.x) * L + l) * 4 * BR_NP;
            q[k] = float(s.v);
#pragma unroll
            for (int p = 0; p < 3; p++) q[(p + 1) * BR_NP + k] = float(s.d[p]);
        }
    }
    if (k == 0) {
        using D5 = Dn<HP>;
        const D5 T5 = dn_var<HP>(hl.T[l], HD_T), ne5 = dn_var<HP>(hl.ne[l], HD_NE);
        const D5 nH5 = dn_var<HP>(hl.nH[l], HD_NH), nHe5 = dn_var<HP>(hl.nHe[l], HD_NHE);
        const D5 beta = 1.0 / (T5 * KBOLTZ_EV);
        const double E_low = RYDBERGH_EV * (1 - 1.0 / (n * n));
        const D5 w = use_MHD ? hummer_mihalas_w_dn<HP>(double(m), nH5, nHe5, ne5) : dn_const<HP>(1.0);
        const D5 levels = w * dn_exp(-beta * E_low) * (1.0 - dn_exp(-beta * E)) / hl.UH[l];
        const double gf = 2 * (n * n) * brackett_oscillator_strength(n, m);
        const D5 amp = nH5 * (gf * sigma_line(wl0)) * levels;
        HDer o;
#pragma unroll
        for (int p = 0; p < HP; p++) {
            o.amp[p] = amp.d[p];
            o.c[p] = p < 3 ? wstart.d[p] : 0.0;
            o.f[p] = p < 3 ? step.d[p] : 0.0;
            o.inv_s[p] = o.a[p] = o.scale[p] = 0.0;
        }
        der[int64_t(slot) * L + l] = o;
        if (der32) {
            HDer32 o32;
#pragma unroll
            for (int p = 0; p < HP; p++) {
                o32.amp[p] = float(o.amp[p]);
                o32.c[p] = float(o.c[p]);
                o32.f[p] = float(o.f[p]);
                o32.inv_s[p] = o32.a[p] = o32.scale[p] = 0.f;
            }
            o32.a_v = float(1.0 / step.v);
            o32.inv_s_v = 0.f;
            o32.scale_v = float(amp.v);
            o32.pad = 0.f;
            der32[int64_t(slot) * L + l] = o32;
        }
    }
}

__device__ __forceinline__ double hadj_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct HAdjArgs {
    const void* G;  // opacity cotangent [nwl][L], float (g32) or double
    int32_t g32;
    const double* wls;
    int64_t nwl;
    int32_t L, ntrans, ntot;
    const HRec* rec;
    const HDer* der;
    const HDer32* der32;  // mixed precision: the Stehle records in FP32
    const double* Q;      // the forward's tables: Stehle [ntrans][L][HND_MAX], then Brackett [nbr][L][BR_NP]
    const float* Q32;     // mixed precision: the Stehle tables in FP32
    const double* dQ;     // Stehle [ntrans][L][2][HND_MAX], then Brackett [nbr][L][3][BR_NP]
    const float* dQ32;    // mixed precision: the Stehle part in FP32
    const float* bq32;    // mixed precision: Brackett profiles and their derivatives [nbr][L][4][BR_NP]
    const int32_t *ulb, *uub;
    const int64_t* d_off;
    const double* logdnu;
    const float* logdnu32;
    const double* UH;
    double* out[6];  // dL/dT, dL/dn_e, dL/dxi, dL/dn(H I), dL/dn(He I), dL/dU(H I) (each may be null)
};

// The per-layer sums s[0..4] = sum_lines d alpha / d input, s[5] = alpha at one (wavelength,
// layer): hline_tile_kernel's branches with their derivatives.  MIXED: the Stehle and ABO
// profiles and their derivatives in FP32 as the mixed forward evaluates them (FP32 line-centre
// offset from FP32 pairs, __logf / __expf), per-lane FP32 sums over the lines; Brackett lines and
// the contraction with G in FP64 in both forms.
template <bool MIXED>
__global__ void __launch_bounds__(32 * HADJ_WARPS, 3) hline_adj_kernel(HAdjArgs a) {
    __shared__ double s_acc[HP + 1][RTA_LMAX];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int L = a.L;
    for (int i = tid; i < (HP + 1) * RTA_LMAX; i += blockDim.x) (&s_acc[0][0])[i] = 0.0;
    __syncthreads();
    const int64_t ntiles = (a.nwl + 31) / 32;
    const int64_t brQ = int64_t(a.ntrans) * L * HND_MAX, brdQ = int64_t(a.ntrans) * L * 2 * HND_MAX;
    for (int64_t tile = int64_t(blockIdx.x) * HADJ_WARPS + warp; tile < ntiles;
         tile += int64_t(gridDim.x) * HADJ_WARPS) {
        const int64_t j0 = tile * 32, jg = j0 + lane, jlast = min(j0 + 32, a.nwl) - 1;
        const bool live = jg < a.nwl;
        // the transitions whose window (union over layers) reaches the tile
        unsigned mask[HADJ_MAXT / 32];
#pragma unroll
        for (int c = 0; c < HADJ_MAXT / 32; c++) {
            const int t = c * 32 + lane;
            mask[c] = __ballot_sync(0xffffffffu, t < a.ntot && a.uub[t] >= j0 && a.ulb[t] <= jlast);
        }
        bool none = true;
#pragma unroll
        for (int c = 0; c < HADJ_MAXT / 32; c++) none &= mask[c] == 0;
        if (none) continue;
        const double wl = live ? a.wls[jg] : 1.0;
        const double nu = C_CGS / wl, dnudl = C_CGS / (wl * wl);
        const float nu_hi = float(nu), nu_lo = float(nu - double(nu_hi)), dnudl_f = float(dnudl);
        for (int l = 0; l < L; l++) {
            double s[HP + 1];
            float sf[HP + 1];
#pragma unroll
            for (int p = 0; p <= HP; p++) {
                s[p] = 0.0;
                sf[p] = 0.f;
            }
            bool hit = false;
#pragma unroll
            for (int c = 0; c < HADJ_MAXT / 32; c++) {
                unsigned mk = mask[c];
                while (mk) {
                    const int t = c * 32 + __ffs(mk) - 1;
                    mk &= mk - 1;
                    const HRec& r = a.rec[int64_t(t) * L + l];
                    if (r.kind == HK_OFF || !live || jg < r.lb || jg > r.ub) continue;
                    hit = true;
                    if (MIXED && r.kind == HK_BRACKETT) {
                        const HDer32& d32 = a.der32[int64_t(t) * L + l];
                        const float u = float(wl - r.wl0) * d32.a_v;
                        int i = int(floorf(u));
                        i = i < 0 ? 0 : (i > BR_NP - 2 ? BR_NP - 2 : i);
                        const float w = u - float(i);
                        const float* q = a.bq32 + (int64_t(t - a.ntrans) * L + l) * 4 * BR_NP;
                        const float qv = q[i] * (1.f - w) + q[i + 1] * w, slope = q[i + 1] - q[i];
                        sf[HP] += qv * d32.scale_v;
#pragma unroll
                        for (int p = 0; p < HP; p++) {
                            float dqv = 0.f;
                            if (p < 3) {
                                const float du = -d32.a_v * (d32.c[p] + u * d32.f[p]);
                                dqv = q[(p + 1) * BR_NP + i] * (1.f - w) + q[(p + 1) * BR_NP + i + 1] * w + slope * du;
                            }
                            sf[p] += dqv * d32.scale_v + qv * d32.amp[p];
                        }
                        continue;
                    }
                    const HDer& d = a.der[int64_t(t) * L + l];
                    if (r.kind == HK_BRACKETT) {
                        const double u = (wl - r.wl0) * r.a;
                        int i = int(floor(u));
                        i = i < 0 ? 0 : (i > BR_NP - 2 ? BR_NP - 2 : i);
                        const double w = u - i;
                        const double* q = a.Q + brQ + (int64_t(t - a.ntrans) * L + l) * BR_NP;
                        const double* dq = a.dQ + brdQ + (int64_t(t - a.ntrans) * L + l) * 3 * BR_NP;
                        const double qv = q[i] * (1 - w) + q[i + 1] * w, slope = q[i + 1] - q[i];
                        s[HP] += qv * r.amp;
#pragma unroll
                        for (int p = 0; p < HP; p++) {
                            double dqv = 0.0;
                            if (p < 3) {
                                const double du = -r.a * (d.c[p] + u * d.f[p]);
                                dqv = dq[p * BR_NP + i] * (1 - w) + dq[p * BR_NP + i + 1] * w + slope * du;
                            }
                            s[p] += dqv * r.amp + qv * d.amp[p];
                        }
                        continue;
                    }
                    if (MIXED) {
                        const HDer32& d32 = a.der32[int64_t(t) * L + l];
                        if (r.kind == HK_STARK_ABO) {
                            const float xa = float(fabs(wl - r.wl0));
                            const Dual<float> H = voigt_dual<float>(d32.a_v, xa * d32.inv_s_v);
                            sf[HP] += H.x * d32.scale_v;
#pragma unroll
                            for (int p = 0; p < HP; p++)
                                sf[p] += H.x * d32.scale[p] + d32.scale_v * (H.da * d32.a[p] + H.dv * xa * d32.inv_s[p]);
                        }
                        const float dnu = (nu_hi - r.nu0_hi) + (nu_lo - r.nu0_lo);  // signed
                        const float x = __logf(fabsf(dnu) * r.invF0_f);
                        const int nDt = r.nD;
                        const float* kd = a.logdnu32 + a.d_off[t];
                        const float* Q = a.Q32 + (int64_t(t) * L + l) * HND_MAX;
                        const float* dQT = a.dQ32 + (int64_t(t) * L + l) * 2 * HND_MAX;
                        float v, vT, vN, slope = 0.f;
                        if (!(x > kd[1])) {
                            v = Q[1];
                            vT = dQT[1];
                            vN = dQT[HND_MAX + 1];
                        } else if (x >= kd[nDt - 1]) {
                            v = Q[nDt - 1];
                            vT = dQT[nDt - 1];
                            vN = dQT[HND_MAX + nDt - 1];
                        } else {
                            int lo = 1, hi = nDt - 1;
                            while (hi - lo > 1) {
                                const int mid = (lo + hi) >> 1;
                                if (kd[mid] <= x) lo = mid; else hi = mid;
                            }
                            const float ih = __fdividef(1.f, kd[lo + 1] - kd[lo]);
                            const float w = (x - kd[lo]) * ih;
                            v = (1.f - w) * Q[lo] + w * Q[lo + 1];
                            vT = (1.f - w) * dQT[lo] + w * dQT[lo + 1];
                            vN = (1.f - w) * dQT[HND_MAX + lo] + w * dQT[HND_MAX + lo + 1];
                            slope = (Q[lo + 1] - Q[lo]) * ih;
                        }
                        const float e = __expf(v) * dnudl_f, al = e * r.amp_f;
                        sf[HP] += al;
                        const float inv = dnu != 0.f ? __fdividef(1.f, dnu) : 0.f;
#pragma unroll
                        for (int p = 0; p < HP; p++) {
                            const float dx = -d32.c[p] * inv - d32.f[p];
                            const float dv = slope * dx + (p == HD_T ? vT : (p == HD_NE ? vN : 0.f));
                            sf[p] += e * d32.amp[p] + al * dv;
                        }
                        continue;
                    }
                    if (r.kind == HK_STARK_ABO) {
                        const double xa = fabs(wl - r.wl0);
                        const Dual<double> H = voigt_dual(r.a, xa * r.inv_s);
                        s[HP] += H.x * r.scale;
#pragma unroll
                        for (int p = 0; p < HP; p++)
                            s[p] += H.x * d.scale[p] + r.scale * (H.da * d.a[p] + H.dv * xa * d.inv_s[p]);
                    }
                    const double dnu = nu - r.nu0;
                    double sd = fabs(dnu) / r.F0;
                    sd = sd + (sd == 0) * 2.2250738585072014e-308;
                    const double x = log(sd);
                    const int nDt = r.nD;
                    const double* kd = a.logdnu + a.d_off[t];
                    const double* Q = a.Q + (int64_t(t) * L + l) * HND_MAX;
                    const double* dQT = a.dQ + (int64_t(t) * L + l) * 2 * HND_MAX;
                    double v, vT, vN, slope = 0.0;
                    if (!(x > kd[1])) {
                        v = Q[1];
                        vT = dQT[1];
                        vN = dQT[HND_MAX + 1];
                    } else if (x >= kd[nDt - 1]) {
                        v = Q[nDt - 1];
                        vT = dQT[nDt - 1];
                        vN = dQT[HND_MAX + nDt - 1];
                    } else {
                        int lo = 1, hi = nDt - 1;
                        while (hi - lo > 1) {
                            const int mid = (lo + hi) >> 1;
                            if (kd[mid] <= x) lo = mid; else hi = mid;
                        }
                        const double ih = 1.0 / (kd[lo + 1] - kd[lo]);
                        const double w = (x - kd[lo]) * ih;
                        v = (1 - w) * Q[lo] + w * Q[lo + 1];
                        vT = (1 - w) * dQT[lo] + w * dQT[lo + 1];
                        vN = (1 - w) * dQT[HND_MAX + lo] + w * dQT[HND_MAX + lo + 1];
                        slope = (Q[lo + 1] - Q[lo]) * ih;
                    }
                    const double e = exp(v) * dnudl, al = e * r.amp;
                    s[HP] += al;
                    // x = log|nu - nu0| - log F0
                    const double inv = dnu != 0 ? 1.0 / dnu : 0.0;
#pragma unroll
                    for (int p = 0; p < HP; p++) {
                        const double dx = -d.c[p] * inv - d.f[p];
                        const double dv = slope * dx + (p == HD_T ? vT : (p == HD_NE ? vN : 0.0));
                        s[p] += e * d.amp[p] + al * dv;
                    }
                }
            }
            if (!__any_sync(0xffffffffu, hit)) continue;
            if (MIXED) {
#pragma unroll
                for (int p = 0; p <= HP; p++) s[p] += double(sf[p]);
            }
            const int64_t e = jg * L + l;
            const double g = !hit ? 0.0 : (a.g32 ? double(static_cast<const float*>(a.G)[e]) : static_cast<const double*>(a.G)[e]);
#pragma unroll
            for (int p = 0; p <= HP; p++) {
                const double v = hadj_warp_sum(s[p] * g);
                if (lane == 0 && v != 0.0) atomicAdd(&s_acc[p][l], v);
            }
        }
    }
    __syncthreads();
    for (int l = tid; l < L; l += blockDim.x) {
#pragma unroll
        for (int p = 0; p < HP; p++)
            if (a.out[p] && s_acc[p][l] != 0.0) atomicAdd(a.out[p] + l, s_acc[p][l]);
        if (a.out[HP] && s_acc[HP][l] != 0.0) atomicAdd(a.out[HP] + l, -s_acc[HP][l] / a.UH[l]);
    }
}

}  // namespace korg
