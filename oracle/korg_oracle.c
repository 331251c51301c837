/*
 * korg_oracle.c -- FP64 CPU restatement of Korg.jl's synthesis hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library and the timed CPU baseline.
 * The product never links or calls this file.  Expressions keep the reference's evaluation
 * order so that rounding follows it closely; compile with -ffp-contract=off (Julia does not
 * contract a*b+c into FMAs).  Citations are to Korg.jl v1.2.1 source files.
 */
#include "korg_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/constants.jl:3-19 */
#define KBOLTZ_CGS 1.380649e-16
#define HPLANCK_CGS 6.62607015e-27
#define C_CGS 2.99792458e10
#define ELECTRON_MASS_CGS 9.1093897e-28
#define ELECTRON_CHARGE_CGS 4.80320425e-10
#define AMU_CGS 1.6605402e-24
#define BOHR_RADIUS_CGS 5.29177210903e-9
#define EV_TO_CGS 1.602e-12
#define KBOLTZ_EV 8.617333262145e-5
#define HPLANCK_EV 4.135667696e-15
#define RYDBERGH_EV 13.598287264

static const double PI = 3.141592653589793;

/* ------------------------------------------------------------------ line profile pieces */

/* src/line_absorption.jl:251-265 */
static inline void harris_series(double v, double *H0, double *H1, double *H2) {
    double v2 = v * v;
    *H0 = exp(-(v2));
    if (v < 1.3)
        *H1 = -1.12470432 + (-0.15516677 + (3.288675912 + (-2.34357915 + 0.42139162 * v) * v) * v) * v;
    else if (v < 2.4)
        *H1 = -4.48480194 + (9.39456063 + (-6.61487486 + (1.98919585 - 0.22041650 * v) * v) * v) * v;
    else
        *H1 = ((0.554153432 +
                (0.278711796 + (-0.1883256872 + (0.042991293 - 0.003278278 * v) * v) * v) * v) /
               (v2 - 3.0 / 2.0));
    *H2 = (1 - 2 * v2) * *H0;
}

/* src/line_absorption.jl:286-310 (Hunger 1965 approximation) */
double ko_voigt_hjerting(double a, double v) {
    double v2 = v * v;
    if (a <= 0.2 && (v >= 5)) {
        double invv2 = (1 / v2);
        return (a / sqrt(PI) * invv2) * (1 + 1.5 * invv2 + 3.75 * (invv2 * invv2));
    } else if (a <= 0.2) {
        double H0, H1, H2;
        harris_series(v, &H0, &H1, &H2);
        return H0 + (H1 + H2 * a) * a;
    } else if ((a <= 1.4) && (a + v < 3.2)) {
        double H0, H1, H2;
        harris_series(v, &H0, &H1, &H2);
        double M0 = H0;
        double M1 = H1 + 2 / sqrt(PI) * M0;
        double M2 = H2 - M0 + 2 / sqrt(PI) * M1;
        double M3 = 2 / (3 * sqrt(PI)) * (1 - H2) - (2.0 / 3.0) * v2 * M1 + (2 / sqrt(PI)) * M2;
        double M4 = 2.0 / 3.0 * v2 * v2 * M0 - 2 / (3 * sqrt(PI)) * M1 + 2 / sqrt(PI) * M3;
        double psi = 0.979895023 + (-0.962846325 + (0.532770573 - 0.122727278 * a) * a) * a;
        return psi * (M0 + (M1 + (M2 + (M3 + M4 * a) * a) * a) * a);
    } else {
        double r2 = (v2) / (a * a);
        double a_invu = 1 / sqrt(2.0) / ((r2 + 1) * a);
        double a2_invu2 = a_invu * a_invu;
        return sqrt(2 / PI) * a_invu *
               (1 + (3 * r2 - 1 + ((r2 - 2) * 15 * r2 + 2) * a2_invu2) * a2_invu2);
    }
}

/* src/line_absorption.jl:245-249 */
double ko_line_profile(double wl0, double sigma, double gamma, double amp, double wl) {
    double inv_s = 1 / (sigma * sqrt(2.0));
    double scaling = inv_s / sqrt(PI) * amp;
    return ko_voigt_hjerting(gamma * inv_s, fabs(wl - wl0) * inv_s) * scaling;
}

/* src/line_absorption.jl:140-145 */
static inline double inverse_gaussian_density(double rho, double sigma) {
    if (rho > 1 / (sqrt(2 * PI) * sigma)) return 0.0;
    return sigma * sqrt(-2 * log(sqrt(2 * PI) * sigma * rho));
}

/* src/line_absorption.jl:156-161 */
static inline double inverse_lorentz_density(double rho, double gamma) {
    if (rho > 1 / (PI * gamma)) return 0.0;
    return sqrt(gamma / (PI * rho) - gamma * gamma);
}

/* src/line_absorption.jl:169-182 (Kurucz VCSE1F) */
double ko_exponential_integral_1(double x) {
    if (x < 0) return 0.0;
    if (x <= 0.01) return -log(x) - 0.577215 + x;
    if (x <= 1.0)
        return -log(x) - 0.57721566 +
               x * (0.99999193 + x * (-0.24991055 + x * (0.05519968 + x * (-0.00976004 + x * 0.00107857))));
    if (x <= 30.0)
        return (x * (x + 2.334733) + 0.25062) / (x * (x + 3.330657) + 1.681534) / x * exp(-x);
    return 0.0;
}

/* src/line_absorption.jl:190 */
static inline double doppler_width(double wl0, double T, double m, double xi) {
    return wl0 * sqrt(KBOLTZ_CGS * T / m + (xi * xi) / 2) / C_CGS;
}

/* src/line_absorption.jl:195 */
static inline double scaled_stark(double gstark, double T) {
    return gstark * pow(T / 10000.0, 1.0 / 6.0);
}

/* src/line_absorption.jl:208-221 (simple power law or ABO theory) */
static inline double scaled_vdW(double v1, double v2, double m, double T) {
    if (v2 == -1) return v1 * pow(T / 10000.0, 0.3);
    double v0 = 1e6, sigma = v1, alpha = v2;
    double invmu = 1 / (1.008 * AMU_CGS) + 1 / m;
    double vbar = sqrt(8 * KBOLTZ_CGS * T / PI * invmu);
    return 2 * pow(4 / PI, alpha / 2) * tgamma((4 - alpha) / 2) * v0 * sigma * pow(vbar / v0, 1 - alpha);
}

/* src/line_absorption.jl:229-237 */
static inline double sigma_line(double wl) {
    double e = ELECTRON_CHARGE_CGS, me = ELECTRON_MASS_CGS, c = C_CGS;
    return (PI * (e * e) / me / c) * ((wl * wl) / c);
}

/* src/synthesize.jl:412-418 */
double ko_blackbody(double T, double wl) {
    double h = HPLANCK_CGS, c = C_CGS, k = KBOLTZ_CGS;
    double wl5 = wl * wl * wl * wl * wl;
    return 2 * h * (c * c) / wl5 * 1 / expm1(h * c / wl / k / T);
}

/* ------------------------------------------------------------------ wavelength search */

/* index (0-based) of the first element >= v (src/wavelengths.jl:188-198) */
int64_t ko_searchsortedfirst(const double *x, int64_t n, double v) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (x[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* index (0-based) of the last element <= v, -1 if none (src/wavelengths.jl:200-210) */
int64_t ko_searchsortedlast(const double *x, int64_t n, double v) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (x[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo - 1;
}

/* Interpolations.jl Gridded(Linear()) on a knot vector: i = clamp(searchsortedlast, 1, n-1),
 * t = (x - k_i)/(k_{i+1} - k_i), value = v_i (1 - t) + v_{i+1} t.  Used for the continuum
 * interpolants of src/synthesize.jl:228. */
static inline double gridded_linear(const double *k, const double *v, int64_t n, double x) {
    if (n == 1) return v[0];
    int64_t i = ko_searchsortedlast(k, n, x);
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    double t = (x - k[i]) / (k[i + 1] - k[i]);
    return v[i] * (1 - t) + v[i + 1] * t;
}

/* ------------------------------------------------------------------ line_absorption! */

typedef struct {
    const ko_lines *lines;
    const double *wls;
    int64_t nwl;
    const ko_layers *lay;
    const ko_cntm *cntm;
    double cutoff;
    int64_t *lb_out, *ub_out;
} la_ctx;

/* The body of one task of src/line_absorption.jl:68-124: lines [i0, i1) into alpha_task. */
static int64_t la_chunk(const la_ctx *c, int64_t i0, int64_t i1, double *alpha_task) {
    const ko_lines *ln = c->lines;
    const ko_layers *lay = c->lay;
    int32_t L = lay->L;
    double *sigma = malloc(sizeof(double) * L), *gam = malloc(sizeof(double) * L);
    double *amp = malloc(sizeof(double) * L), *Gam = malloc(sizeof(double) * L);
    int64_t evals = 0;
    for (int64_t i = i0; i < i1; i++) {
        double wl = ln->wl[i], m = ln->mass[i];
        double doppler_window = 0, lorentz_window = 0;
        for (int l = 0; l < L; l++) {
            double T = lay->T[l];
            /* :86 */
            sigma[l] = doppler_width(wl, T, m, lay->xi[l]);
            /* :90-94 */
            Gam[l] = ln->gamma_rad[i];
            if (!ln->is_mol[i]) {
                Gam[l] = Gam[l] + lay->ne[l] * scaled_stark(ln->gamma_stark[i], T);
                Gam[l] = Gam[l] + lay->n_eff_vdW[l] * scaled_vdW(ln->vdW1[i], ln->vdW2[i], m, T);
            }
            /* :99 */
            gam[l] = Gam[l] * (wl * wl) / (C_CGS * (4 * PI));
            /* :101-102 */
            double beta = 1 / (KBOLTZ_EV * T);
            double E_upper = ln->E_lower[i] + C_CGS * HPLANCK_EV / wl;
            double levels = exp(-beta * ln->E_lower[i]) - exp(-beta * E_upper);
            /* :105-106 */
            amp[l] = pow(10.0, ln->log_gf[i]) * sigma_line(wl) * levels *
                     lay->n_div_U[(int64_t)ln->species[i] * L + l];
            /* :108-112 */
            double acntm = gridded_linear(c->cntm->knots, c->cntm->vals + (int64_t)l * c->cntm->nk,
                                          c->cntm->nk, wl);
            double rho = acntm * c->cutoff / amp[l];
            double dw = inverse_gaussian_density(rho, sigma[l]);
            double lw = inverse_lorentz_density(rho, gam[l]);
            if (l == 0 || dw > doppler_window) doppler_window = dw;
            if (l == 0 || lw > lorentz_window) lorentz_window = lw;
        }
        /* :113-119 */
        double window = sqrt(lorentz_window * lorentz_window + doppler_window * doppler_window);
        int64_t lb = ko_searchsortedfirst(c->wls, c->nwl, wl - window);
        int64_t ub = ko_searchsortedlast(c->wls, c->nwl, wl + window);
        if (c->lb_out) { c->lb_out[i] = lb; c->ub_out[i] = ub; }
        if (lb > ub) continue;
        /* :121 */
        for (int64_t j = lb; j <= ub; j++) {
            double *col = alpha_task + j * L;
            for (int l = 0; l < L; l++)
                col[l] = col[l] + ko_line_profile(wl, sigma[l], gam[l], amp[l], c->wls[j]);
        }
        evals += (ub - lb + 1) * (int64_t)L;
    }
    free(sigma); free(gam); free(amp); free(Gam);
    return evals;
}

int64_t ko_line_absorption(double *alpha, const ko_lines *lines, const double *wls, int64_t nwl,
                           const ko_layers *lay, const ko_cntm *cntm, double cutoff_threshold,
                           int nthreads, int64_t *lb_out, int64_t *ub_out) {
    /* :35-37: an empty list leaves alpha untouched */
    if (lines->n == 0) return 0;
    la_ctx c = {lines, wls, nwl, lay, cntm, cutoff_threshold, lb_out, ub_out};
    int64_t N = lines->n, L = lay->L, size = L * nwl;
    int n_chunks = nthreads < 1 ? 1 : nthreads;
    /* :62-64 */
    int64_t chunk = N / n_chunks + (N % n_chunks > 0);
    if (chunk < 1) chunk = 1;
    int64_t nparts = (N + chunk - 1) / chunk;
    double **tasks = malloc(sizeof(double *) * nparts);
    int64_t *evals = calloc(nparts, sizeof(int64_t));
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_chunks) if (n_chunks > 1)
    for (int64_t p = 0; p < nparts; p++) {
        tasks[p] = calloc(size, sizeof(double)); /* :69 */
        int64_t i1 = (p + 1) * chunk < N ? (p + 1) * chunk : N;
        evals[p] = la_chunk(&c, p * chunk, i1, tasks[p]);
    }
    /* :127  alpha .+= sum(fetch.(tasks)): a left fold over the task matrices, then one add */
    int64_t total = 0;
#pragma omp parallel for num_threads(n_chunks) if (n_chunks > 1)
    for (int64_t e = 0; e < size; e++) {
        double s = tasks[0][e];
        for (int64_t p = 1; p < nparts; p++) s = s + tasks[p][e];
        alpha[e] = alpha[e] + s;
    }
    for (int64_t p = 0; p < nparts; p++) { total += evals[p]; free(tasks[p]); }
    free(tasks); free(evals);
    return total;
}

/* ------------------------------------------------------------------ hydrogen lines */

/* src/statmech.jl:463-497, default (non-Hubeny) branch */
double ko_hummer_mihalas_w(double T, double n_eff, double nH, double nHe, double ne) {
    (void)T;
    double n2 = n_eff * n_eff, n4 = n2 * n2;
    double r_level = sqrt(5.0 / 2.0 * n4 + 1.0 / 2.0 * n2) * BOHR_RADIUS_CGS;
    double a = r_level + sqrt(3.0) * BOHR_RADIUS_CGS, b = r_level + 1.02 * BOHR_RADIUS_CGS;
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

/* src/hydrogen_line_absorption.jl:174-184 */
double ko_brackett_oscillator_strength(int n, int m) {
    double GINF = 0.2027 / pow((double)n, 0.71);
    double GCA = 0.124 / n;
    double FKN = 1.9603 * n;
    double WTC = 0.45 - 2.4 / (double)(n * n * n) * (n - 1);
    double r = (double)m / (double)((m - n) * (m + n));
    double FK = FKN * (r * r * r);
    double XMN12 = pow((double)(m - n), 1.2);
    double WT = (XMN12 - 1) / (XMN12 + WTC);
    return FK * (1 - WT * GINF - (0.222 + GCA / m) * (1 - WT));
}

/* src/hydrogen_line_absorption.jl:371-393 */
static double greim_1960_Knm(int n, int m) {
    static const double tab[3][4] = {{0.0001716, 0.0090190, 0.1001000, 0.5820000},
                                     {0.0005235, 0.0177200, 0.1710000, 0.8660000},
                                     {0.0008912, 0.0250700, 0.2230000, 1.0200000}};
    if ((m - n <= 3) && (n <= 4)) return tab[m - n - 1][n - 1];
    double n4 = (double)n * n * n * n, m4 = (double)m * m * m * m;
    return 5.5e-5 * n4 * m4 / (double)(m * m - n * n) / (1 + 0.13 / (m - n));
}

/* src/hydrogen_line_absorption.jl:451-470 */
static const double HOLT_PROB7[15][5] = {
    {0.005, 0.128, 0.260, 0.389, 0.504},     {0.004, 0.109, 0.220, 0.318, 0.389},
    {-0.007, 0.079, 0.162, 0.222, 0.244},    {-0.018, 0.041, 0.089, 0.106, 0.080},
    {-0.026, -0.003, 0.003, -0.023, -0.086}, {-0.025, -0.048, -0.087, -0.148, -0.234},
    {-0.008, -0.085, -0.165, -0.251, -0.343}, {0.018, -0.111, -0.223, -0.321, -0.407},
    {0.032, -0.130, -0.255, -0.354, -0.431}, {0.014, -0.148, -0.269, -0.359, -0.427},
    {-0.005, -0.140, -0.243, -0.323, -0.386}, {0.005, -0.095, -0.178, -0.248, -0.307},
    {-0.002, -0.068, -0.129, -0.187, -0.241}, {-0.007, -0.049, -0.094, -0.139, -0.186},
    {-0.010, -0.036, -0.067, -0.103, -0.143}};
static const double HOLT_C7[5] = {511.318, 1.532, 4.044, 19.266, 41.812};
static const double HOLT_D7[5] = {-6.070, -4.528, -8.759, -14.984, -23.956};
static const double HOLT_PP[5] = {0.0, 0.2, 0.4, 0.6, 0.8};
static const double HOLT_BETA[15] = {1.0,  1.259, 1.585, 1.995, 2.512, 3.162, 3.981, 5.012,
                                     6.310, 7.943, 10.0, 12.59, 15.85, 19.95, 25.12};

/* src/hydrogen_line_absorption.jl:402-448 (1-based indices of the reference kept as IM/IP) */
double ko_holtsmark_profile(double beta, double P) {
    if (beta > 500) return (1.5 / sqrt(beta) + 27 / (beta * beta)) / (beta * beta);
    int IM = (int)floor((5 * P) + 1);
    if (IM > 4) IM = 4;
    int IP = IM + 1;
    double WTPP = 5 * (P - HOLT_PP[IM - 1]);
    double WTPM = 1 - WTPP;
    if (beta <= 25.12) {
        int first = 15; /* findfirst(beta .<= knots), 1-based */
        for (int k = 0; k < 15; k++)
            if (beta <= HOLT_BETA[k]) { first = k + 1; break; }
        int JP = first > 2 ? first : 2;
        int JM = JP - 1;
        double WTBP = (beta - HOLT_BETA[JM - 1]) / (HOLT_BETA[JP - 1] - HOLT_BETA[JM - 1]);
        double WTBM = 1 - WTBP;
        double CBP = HOLT_PROB7[JP - 1][IP - 1] * WTPP + HOLT_PROB7[JP - 1][IM - 1] * WTPM;
        double CBM = HOLT_PROB7[JM - 1][IP - 1] * WTPP + HOLT_PROB7[JM - 1][IM - 1] * WTPM;
        double CORR = 1 + CBP * WTBP + CBM * WTBM;
        double WT = fmax(fmin(0.5 * (10 - beta), 1), 0);
        double PR1 = beta <= 10 ? 8 / (83 + (2 + 0.95 * (beta * beta)) * beta) : 0.0;
        double PR2 = beta >= 8 ? (1.5 / sqrt(beta) + 27 / (beta * beta)) / (beta * beta) : 0.0;
        return (PR1 * WT + PR2 * (1 - WT)) * CORR;
    }
    double CC = HOLT_C7[IP - 1] * WTPP + HOLT_C7[IM - 1] * WTPM;
    double DD = HOLT_D7[IP - 1] * WTPP + HOLT_D7[IM - 1] * WTPM;
    double CORR = 1 + DD / (CC + beta * sqrt(beta));
    return (1.5 / sqrt(beta) + 27 / (beta * beta)) / (beta * beta) * CORR;
}

/* src/hydrogen_line_absorption.jl:272-369, evaluated on the 201-point grid wls */
static void brackett_line_stark_profiles(int m, const double *wls, int np, double wl0, double T,
                                         double ne, double *impact, double *quasi) {
    const int n = 4;
    double nu0 = C_CGS / wl0;
    double ne_1_6 = pow(ne, 1.0 / 6.0);
    double F0 = 1.25e-9 * pow(ne, 2.0 / 3.0);
    double GCON1 = 0.2 + 0.09 * sqrt(T / 10000) / (1 + ne / 1.E13);
    double GCON2 = 0.2 / (1 + ne / 1.E15);
    double Knm = greim_1960_Knm(n, m);
    double Y1WHT = (m - n <= 3) ? 1e14 : 1e13;
    double WTY1 = 1 / (1 + ne / Y1WHT);
    double Y1B = 2 / (1 + 0.012 / T * sqrt(ne / T));
    double mm_nn = (double)(m * m - n * n);
    double C1CON = Knm / wl0 * (mm_nn * mm_nn) / (double)(n * n * m * m) * 1e-8;
    double Y1NUM = 320;
    double Y1SCAL = Y1NUM * (pow(T / 10000, 0.3) / ne_1_6) * WTY1 + Y1B * (1 - WTY1);
    double C1 = F0 * 78940 / T * C1CON * Y1SCAL;
    double kl = Knm / wl0;
    double C2 = (F0 * F0) / (5.96E-23 * ne) * (kl * kl) * 1e-16;
    double G1 = 6.77 * sqrt(C1);
    double P = ne_1_6 * 0.08989 / sqrt(T);
    double dbeta_dlambda = 1e8 / (Knm * F0);
    int last_red = -1; /* findlast(nus .< nu0) */
    for (int k = 0; k < np; k++)
        if (C_CGS / wls[k] < nu0) last_red = k;
    for (int k = 0; k < np; k++) {
        double beta = fabs(wls[k] - wl0) / F0 / Knm * 1e8;
        double y1 = C1 * beta, y2 = C2 * (beta * beta);
        double width;
        if ((y2 <= 1e-4) && (y1 <= 1e-5)) {
            width = G1 * fmax(0, 0.2114 + log(sqrt(C2) / C1)) * (1 - GCON1 - GCON2);
        } else {
            double t90 = 90 * y1;
            double GAM = (G1 * (0.5 * exp(-fmin(80, y1)) + ko_exponential_integral_1(y1) -
                                0.5 * ko_exponential_integral_1(y2)) *
                          (1 - GCON1 / (1 + t90 * t90 * t90) - GCON2 / (1 + 2000 * y1)));
            width = GAM <= 1e-20 ? 0.0 : GAM;
        }
        impact[k] = width > 0 ? width / (PI * (width * width + beta * beta)) : 0.0;
        double q_ion = ko_holtsmark_profile(beta, P);
        double ps = (0.9 * y1) * (0.9 * y1);
        double qe = (ps + 0.03 * sqrt(y1)) / (ps + 1.0);
        if (qe == 0) qe = 0;
        quasi[k] = q_ion * (1 + qe);
    }
    for (int k = 0; k < np; k++) {
        double f = sqrt(wls[k] / wl0);
        impact[k] = impact[k] * f;
        quasi[k] = quasi[k] * f;
        if (k <= last_red) {
            double b = exp((HPLANCK_CGS * (C_CGS / wls[k] - nu0)) / KBOLTZ_CGS / T);
            impact[k] = impact[k] * b;
            quasi[k] = quasi[k] * b;
        }
        impact[k] = impact[k] * dbeta_dlambda;
        quasi[k] = quasi[k] * dbeta_dlambda;
    }
}

/* full linear convolution (DSP.conv), out has 2n-1 entries; restated as the direct sum */
static void conv_full(const double *f, const double *g, int n, double *out) {
    for (int k = 0; k < 2 * n - 1; k++) {
        double s = 0;
        int lo = k - (n - 1) > 0 ? k - (n - 1) : 0, hi = k < n - 1 ? k : n - 1;
        for (int i = lo; i <= hi; i++) s += f[i] * g[k - i];
        out[k] = s;
    }
}

/* src/hydrogen_line_absorption.jl:211-251 */
double ko_brackett_profile(int m, double wl0, double T, double ne, double xi, double wlmin,
                           double wlmax, double *grid, double *vals) {
    const int n = 4, np = 201, start = (np + 1) / 2 - 1; /* 0-based start_ind */
    double F0 = 1.25e-9 * pow(ne, 2.0 / 3.0);
    double Knm = greim_1960_Knm(n, m);
    double stark_width = 1.6678E-18 * Knm * F0 * C_CGS;
    double sdop = doppler_width(wl0, T, 1.008 * AMU_CGS, xi);
    double window = 5 * fmax(sdop, stark_width);
    double wstart = fmax(wlmin, wl0 - window);
    double wend = fmin(wl0 + window, wlmax);
    if (wstart > wlmax || wend < wlmin || wstart == wend) return 0.0;
    double step = (wend - wstart) / (np - 1);
    for (int k = 0; k < np; k++) grid[k] = wstart + k * step;
    grid[np - 1] = wend;
    double impact[201], quasi[201], tmp[401];
    brackett_line_stark_profiles(m, grid, np, wl0, T, ne, impact, quasi);
    if (sdop / stark_width > 0.25) {
        double dop[201];
        for (int k = 0; k < np; k++) {
            double d = grid[k] - wl0;
            dop[k] = exp(-0.5 * (d * d) / (sdop * sdop)) / sqrt(2 * PI) / sdop;
        }
        conv_full(quasi, dop, np, tmp);
        for (int k = 0; k < np; k++) quasi[k] = tmp[start + k] * step;
    }
    conv_full(impact, quasi, np, tmp);
    for (int k = 0; k < np; k++) vals[k] = tmp[start + k] * step;
    return window;
}

/* Flat-extrapolated 3-D Gridded(Linear()) interpolation of a Stehle table at (T, ne, x) */
static inline int knot_index(const double *k, int n, double x) {
    int i = (int)ko_searchsortedlast(k, n, x);
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    return i;
}
static inline double knot_weight(const double *k, int i, double x) {
    return (x - k[i]) / (k[i + 1] - k[i]);
}
static inline double clampd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

static double stark_interp(const ko_stark *s, int t, double T, double ne, double x) {
    int nT = s->nT[t], nNe = s->nNe[t], nD = s->nD[t];
    const double *kT = s->temps + s->t_off[t], *kN = s->nes + s->ne_off[t];
    const double *kD = s->logdnu + s->d_off[t], *P = s->logP + s->p_off[t];
    T = clampd(T, kT[0], kT[nT - 1]);
    ne = clampd(ne, kN[0], kN[nNe - 1]);
    x = clampd(x, kD[0], kD[nD - 1]);
    int i = knot_index(kT, nT, T), j = knot_index(kN, nNe, ne), k = knot_index(kD, nD, x);
    double wt = knot_weight(kT, i, T), wn = knot_weight(kN, j, ne), wd = knot_weight(kD, k, x);
    double r = 0;
    for (int c = 0; c < 2; c++)
        for (int b = 0; b < 2; b++)
            for (int a = 0; a < 2; a++) {
                double w = (a ? wt : 1 - wt) * (b ? wn : 1 - wn) * (c ? wd : 1 - wd);
                r += w * P[((int64_t)(k + c) * nNe + (j + b)) * nT + (i + a)];
            }
    return r;
}

static double lambda0_interp(const ko_stark *s, int t, double T, double ne) {
    int nT = s->nT[t], nNe = s->nNe[t];
    const double *kT = s->temps + s->t_off[t], *kN = s->nes + s->ne_off[t];
    const double *L0 = s->lambda0 + s->l_off[t];
    int i = knot_index(kT, nT, T), j = knot_index(kN, nNe, ne);
    double wt = knot_weight(kT, i, T), wn = knot_weight(kN, j, ne);
    return (1 - wt) * (1 - wn) * L0[j * nT + i] + wt * (1 - wn) * L0[j * nT + i + 1] +
           (1 - wt) * wn * L0[(j + 1) * nT + i] + wt * wn * L0[(j + 1) * nT + i + 1];
}

/* src/hydrogen_line_absorption.jl:75-163 */
void ko_hydrogen_line_absorption(double *alphas, const double *wls, int64_t nwl, double T,
                                 double ne, double nH_I, double nHe_I, double UH_I, double xi,
                                 double window_size, int use_MHD, const ko_stark *stark) {
    double Hmass = 1.008 * AMU_CGS;
    int n_max = 0;
    for (int t = 0; t < stark->ntrans; t++)
        if (stark->upper[t] > n_max) n_max = stark->upper[t];
    double *ws = malloc(sizeof(double) * (n_max + 1));
    for (int n = 1; n <= n_max; n++)
        ws[n] = use_MHD ? ko_hummer_mihalas_w(T, n, nH_I, nHe_I, ne) : 1.0;
    double beta = 1 / (KBOLTZ_EV * T);
    double F0 = 1.25e-9 * pow(ne, 2.0 / 3.0);
    for (int t = 0; t < stark->ntrans; t++) {
        const double *kT = stark->temps + stark->t_off[t], *kN = stark->nes + stark->ne_off[t];
        /* :101-103 */
        if (!(kT[0] < T && T < kT[stark->nT[t] - 1] && kN[0] < ne && ne < kN[stark->nNe[t] - 1]))
            continue;
        double wl0 = lambda0_interp(stark, t, T, ne);
        int lo = stark->lower[t], up = stark->upper[t];
        double Elo = RYDBERGH_EV * (1 - 1.0 / (lo * lo));
        double Eup = RYDBERGH_EV * (1 - 1.0 / (up * up));
        double levels = ws[up] * (exp(-beta * Elo) - exp(-beta * Eup)) / UH_I;
        double amplitude = pow(10.0, stark->log_gf[t]) * nH_I * sigma_line(wl0) * levels;
        int64_t lb = ko_searchsortedfirst(wls, nwl, wl0 - window_size);
        int64_t ub = ko_searchsortedlast(wls, nwl, wl0 + window_size);
        if (lb >= ub) continue;
        /* :120-137: Balmer alpha/beta/gamma get the ABO self-broadening Voigt profile; the
         * fixed ABO line centre then also replaces wl0 for the Stark part (Julia scoping) */
        if (lo == 2 && (up == 3 || up == 4 || up == 5)) {
            double sABO, aABO;
            if (up == 3) { wl0 = 6.56460998e-5; sABO = 1180.0; aABO = 0.677; }
            else if (up == 4) { wl0 = 4.8626810200000004e-5; sABO = 2320.0; aABO = 0.455; }
            else { wl0 = 4.34168232e-5; sABO = 4208.0; aABO = 0.380; }
            double G = scaled_vdW(sABO * (BOHR_RADIUS_CGS * BOHR_RADIUS_CGS), aABO, Hmass, T) * nH_I;
            double gam = G * (wl0 * wl0) / (C_CGS * (4 * PI));
            double sig = doppler_width(wl0, T, Hmass, xi);
            for (int64_t j = lb; j <= ub; j++)
                alphas[j] = alphas[j] + ko_line_profile(wl0, sig, gam, amplitude, wls[j]);
        }
        /* :140-143 */
        double nu0 = C_CGS / (wl0);
        for (int64_t j = lb; j <= ub; j++) {
            double nu = C_CGS / wls[j];
            double sd = fabs(nu - nu0) / F0;
            sd = sd + (sd == 0) * DBL_MIN;
            double dIdnu = exp(stark_interp(stark, t, T, ne, log(sd)));
            double dnudl = C_CGS / (wls[j] * wls[j]);
            alphas[j] = alphas[j] + dIdnu * dnudl * amplitude;
        }
    }
    /* :147-162 Brackett series */
    const int n = 4;
    double E_low = RYDBERGH_EV * (1 - 1.0 / (n * n));
    double grid[201], vals[201];
    for (int m = 5; m <= n_max; m++) {
        double E = RYDBERGH_EV * (1.0 / (n * n) - 1.0 / (m * m));
        double wl0 = HPLANCK_EV * C_CGS / E;
        double levels = ws[m] * exp(-beta * E_low) * (1 - exp(-beta * E)) / UH_I;
        double gf = 2 * (n * n) * ko_brackett_oscillator_strength(n, m);
        double amplitude = gf * nH_I * sigma_line(wl0) * levels;
        double win = ko_brackett_profile(m, wl0, T, ne, xi, wls[0], wls[nwl - 1], grid, vals);
        int64_t lb = ko_searchsortedfirst(wls, nwl, wl0 - win);
        int64_t ub = ko_searchsortedlast(wls, nwl, wl0 + win);
        if (win == 0.0) continue; /* no-op interpolator */
        double step = (grid[200] - grid[0]) / 200;
        for (int64_t j = lb; j <= ub; j++) {
            /* linear_interpolation over the range grid (BSpline(Linear()) scaled) */
            double u = (wls[j] - grid[0]) / step;
            int k = (int)floor(u);
            if (k < 0) k = 0;
            if (k > 199) k = 199;
            double d = u - k;
            double v = vals[k] * (1 - d) + vals[k + 1] * d;
            alphas[j] = alphas[j] + v * amplitude;
        }
    }
    free(ws);
}

/* ------------------------------------------------------------------ radiative transfer */

/* RadiativeTransfer.jl:408-497 */
double ko_exponential_integral_2(double x) {
    if (x == 0) return 1.0;
    if (x < 1.1) {
        const double EM = 0.57721566490153286060651209008240243104215933593992;
        return 1 + ((log(x) + EM - 1) +
                    (-0.5 + (0.08333333333333333 + (-0.013888888888888888 +
                                                    0.0020833333333333333 * x) * x) * x) * x) * x;
    }
    if (x < 2.5) {
        x -= 2;
        return 0.037534261820486914 +
               (-0.04890051070806112 +
                (0.033833820809153176 +
                 (-0.016916910404576574 + (0.007048712668573576 - 0.0026785108140579598 * x) * x) * x) * x) * x;
    }
    if (x < 3.5) {
        x -= 3;
        return 0.010641925085272673 +
               (-0.013048381094197039 +
                (0.008297844727977323 +
                 (-0.003687930990212144 + (0.0013061422257001345 - 0.0003995258572729822 * x) * x) * x) * x) * x;
    }
    if (x < 4.5) {
        x -= 4;
        return 0.0031982292493385146 +
               (-0.0037793524098489054 +
                (0.0022894548610917728 +
                 (-0.0009539395254549051 + (0.00031003034577284415 - 8.466213288412284e-5 * x) * x) * x) * x) * x;
    }
    if (x < 5.5) {
        x -= 5;
        return 0.000996469042708825 +
               (-0.0011482955912753257 +
                (0.0006737946999085467 +
                 (-0.00026951787996341863 + (8.310134632205409e-5 - 2.1202073223788938e-5 * x) * x) * x) * x) * x;
    }
    if (x < 6.5) {
        x -= 6;
        return 0.0003182574636904001 +
               (-0.0003600824521626587 +
                (0.00020656268138886323 +
                 (-8.032993165122457e-5 + (2.390771775334065e-5 - 5.8334831318151185e-6 * x) * x) * x) * x) * x;
    }
    if (x < 7.5) {
        x -= 7;
        return 0.00010350984428214624 +
               (-0.00011548173161033826 +
                (6.513442611103688e-5 +
                 (-2.4813114708966427e-5 + (7.200234178941151e-6 - 1.7027366981408086e-6 * x) * x) * x) * x) * x;
    }
    if (x < 9) {
        x -= 8;
        return 3.413764515111217e-5 +
               (-3.76656228439249e-5 +
                (2.096641424390699e-5 +
                 (-7.862405341465122e-6 + (2.2386015208338193e-6 - 5.173353514609864e-7 * x) * x) * x) * x) * x;
    }
    double invx = 1 / x;
    return exp(-x) * (1 + (-2 + (6 + (-24 + 120 * invx) * invx) * invx) * invx) * invx;
}

/* RadiativeTransfer.jl:398-400 */
static inline double expint_core(double tau, double m, double b) {
    return 1.0 / 6.0 * (tau * ko_exponential_integral_2(tau) * (3 * b + 2 * m * tau) -
                        exp(-tau) * (3 * b + 2 * m * (tau + 1)));
}

/* RadiativeTransfer.jl:244-253 (anchored) followed by :379-388 (expint flux) on one column */
static double column_flux_expint(const double *a, const double *S, int L, const double *fac,
                                 const double *ltr, double *tau, double *ib) {
    for (int k = 0; k < L; k++) ib[k] = a[k] * fac[k];
    tau[0] = 0.0;
    for (int i = 1; i < L; i++)
        tau[i] = tau[i - 1] + 0.5 * (ib[i] + ib[i - 1]) * (ltr[i] - ltr[i - 1]);
    double I = 0;
    for (int i = 0; i < L - 1; i++) {
        double m = (S[i + 1] - S[i]) / (tau[i + 1] - tau[i]);
        double b = S[i] - m * tau[i];
        I += (expint_core(tau[i + 1], m, b) - expint_core(tau[i], m, b));
    }
    return I;
}

void ko_rt_flux_expint(const double *alpha, const double *S, int32_t L, int64_t nwl,
                       const double *tau_ref, const double *alpha_ref, double *flux, int nthreads) {
    double *fac = malloc(sizeof(double) * L), *ltr = malloc(sizeof(double) * L);
    for (int k = 0; k < L; k++) {
        fac[k] = tau_ref[k] / alpha_ref[k] * 1.0; /* :160, ds/dz = 1/mu = 1 */
        ltr[k] = log(tau_ref[k]);
    }
    int nt = nthreads < 1 ? 1 : nthreads;
#pragma omp parallel num_threads(nt) if (nt > 1)
    {
        double *tau = malloc(sizeof(double) * L), *ib = malloc(sizeof(double) * L);
#pragma omp for schedule(static)
        for (int64_t j = 0; j < nwl; j++) {
            double I = 0 + column_flux_expint(alpha + j * L, S + j * L, L, fac, ltr, tau, ib);
            flux[j] = 2 * PI * (I * (1.0 * 1.0)); /* :136 with mu = [1], w = [1] */
        }
        free(tau); free(ib);
    }
    free(fac); free(ltr);
}

/* ---- secondary schemes (RadiativeTransfer.jl:218-371) */

/* :244-253 on a layer-index ordering */
static void tau_anchored(const double *a, const int *li, int n, const double *fac,
                         const double *ltr, double *tau) {
    double prev_ib = 0;
    for (int k = 0; k < n; k++) {
        double ib = a[li[k]] * fac[k];
        if (k == 0) tau[0] = 0.0;
        else tau[k] = tau[k - 1] + 0.5 * (ib + prev_ib) * (ltr[k] - ltr[k - 1]);
        prev_ib = ib;
    }
}

/* :361-371 */
static void fritsch_butland_C(const double *x, const double *y, int n, double *C) {
    /* returns n-1 control points */
    double *h = malloc(sizeof(double) * n), *d = malloc(sizeof(double) * n);
    double *C0 = malloc(sizeof(double) * n), *C1 = malloc(sizeof(double) * n);
    for (int k = 0; k < n - 1; k++) { h[k] = x[k + 1] - x[k]; d[k] = (y[k + 1] - y[k]) / h[k]; }
    for (int k = 0; k < n - 2; k++) {
        double al = 1.0 / 3.0 * (1 + h[k + 1] / (h[k + 1] + h[k]));
        double yp = (d[k] * d[k + 1]) / (al * d[k + 1] + (1 - al) * d[k]);
        C0[k] = y[k + 1] + h[k] * yp / 2;
        C1[k] = y[k + 1] - h[k + 1] * yp / 2;
    }
    /* ([C0; C1[end]] .+ [C0[1]; C1]) ./ 2 */
    for (int k = 0; k < n - 1; k++) {
        double a = k < n - 2 ? C0[k] : C1[n - 3];
        double b = k == 0 ? C0[0] : C1[k - 1];
        C[k] = (a + b) / 2;
    }
    free(h); free(d); free(C0); free(C1);
}

/* :263-273 */
static void tau_bezier(double *tau, const double *s, const double *a, int n) {
    double *C = malloc(sizeof(double) * n);
    tau[0] = 1e-5;
    fritsch_butland_C(s, a, n, C);
    double amin = a[0], amax = a[0];
    for (int k = 1; k < n; k++) { amin = fmin(amin, a[k]); amax = fmax(amax, a[k]); }
    for (int k = 0; k < n - 1; k++) C[k] = clampd(C[k], 1.0 / 2.0 * amin, 2 * amax);
    for (int i = 1; i < n; i++) tau[i] = tau[i - 1] + (s[i - 1] - s[i]) / 3 * (a[i] + a[i - 1] + C[i - 1]);
    free(C);
}

/* :286-298; I has n entries, I[n-1] is the incoming boundary value */
static void I_linear(double *I, const double *tau, const double *S, int n) {
    if (n == 1) return;
    for (int k = n - 2; k >= 0; k--) {
        double d = tau[k + 1] - tau[k];
        double m = (S[k + 1] - S[k]) / d;
        I[k] = (I[k + 1] - S[k] - m * (d + 1)) * exp(-d) + m + S[k];
    }
}

/* :307-324 */
static double I_linear_flux_only(const double *tau, const double *S, int n) {
    if (n == 1) return 0.0;
    double I = 0.0, next = exp(-tau[0]);
    for (int i = 0; i < n - 1; i++) {
        double dt = tau[i + 1] - tau[i];
        dt += (dt == 0);
        double m = (S[i + 1] - S[i]) / dt;
        double cur = next;
        next = exp(-tau[i + 1]);
        I += (-next * (S[i + 1] + m) + cur * (S[i] + m));
    }
    return I;
}

/* :333-350 */
static void I_bezier(double *I, const double *tau, const double *S, int n) {
    I[n - 1] = 0;
    if (n <= 1) return;
    double *C = malloc(sizeof(double) * n);
    fritsch_butland_C(tau, S, n, C);
    for (int k = n - 2; k >= 0; k--) {
        double d = tau[k + 1] - tau[k], e = exp(-d), d2 = d * d;
        double al = (2 + d2 - 2 * d - 2 * e) / d2;
        double be = (2 - (2 + 2 * d + d2) * e) / d2;
        double ga = (2 * d - 4 + (2 * d + 4) * e) / d2;
        I[k] = I[k + 1] * e + al * S[k] + be * S[k + 1] + ga * C[k];
    }
    I[0] *= exp(-tau[0]);
    free(C);
}

/* :77-139 and :147-201 for one wavelength at a time; returns 0 or -1 on a bad scheme */
int ko_rt_general(const double *alpha, const double *S, int32_t L, int64_t nwl,
                  const double *spatial, int spherical, const double *tau_ref,
                  const double *alpha_ref, const double *mu, const double *mu_w, int n_mu,
                  int include_inward_rays, int tau_scheme, int I_scheme, double *flux) {
    if (tau_scheme < 0 || tau_scheme > 1 || I_scheme < 0 || I_scheme > 3) return -1;
    if (I_scheme == 3 && (spherical || tau_scheme != 0)) return -1;
    /* rays (:218-242): path length s and ds/dz for each surface mu */
    int *nlay = malloc(sizeof(int) * n_mu);
    double *s = malloc(sizeof(double) * n_mu * L), *dsdz = malloc(sizeof(double) * n_mu * L);
    for (int u = 0; u < n_mu; u++) {
        if (spherical) {
            double b = spatial[0] * sqrt(1 - mu[u] * mu[u]);
            int low;
            if (b < spatial[L - 1]) low = L;
            else {
                int am = 0;
                for (int k = 1; k < L; k++)
                    if (fabs(spatial[k] - b) < fabs(spatial[am] - b)) am = k;
                if (spatial[am] < b) am -= 1;
                low = am + 1;
            }
            nlay[u] = low;
            for (int k = 0; k < low; k++) {
                s[u * L + k] = sqrt(spatial[k] * spatial[k] - b * b);
                dsdz[u * L + k] = spatial[k] / s[u * L + k];
            }
        } else {
            nlay[u] = L;
            for (int k = 0; k < L; k++) { s[u * L + k] = spatial[k] / mu[u]; dsdz[u * L + k] = 1.0 / mu[u]; }
        }
    }
    /* inward rays: all, or those that do not reach the bottom (:94-98) */
    int n_in = 0;
    int *in_idx = malloc(sizeof(int) * n_mu);
    for (int u = 0; u < n_mu; u++)
        if (include_inward_rays || nlay[u] < L) in_idx[n_in++] = u;
    int nrays = n_in + n_mu;
    int flux_only = (I_scheme == 1 || I_scheme == 3);
    double *Isurf = calloc((size_t)nrays * nwl, sizeof(double));
    double *Ibot = calloc((size_t)nrays * nwl, sizeof(double)); /* I at the deepest layer */
    double *ltr = malloc(sizeof(double) * L);
    for (int k = 0; k < L; k++) ltr[k] = log(tau_ref[k]);
    double *tau = malloc(sizeof(double) * L), *pathv = malloc(sizeof(double) * L);
    double *fac = malloc(sizeof(double) * L), *lt = malloc(sizeof(double) * L);
    double *acol = malloc(sizeof(double) * L), *Scol = malloc(sizeof(double) * L);
    double *Ilay = malloc(sizeof(double) * L);
    int *li = malloc(sizeof(int) * L);
    for (int r = 0; r < nrays; r++) {
        int inward = r < n_in;
        int u = inward ? in_idx[r] : r - n_in;
        int n = nlay[u];
        for (int k = 0; k < n; k++) {
            int lk = inward ? n - 1 - k : k; /* reversed path for inward rays (:118-121) */
            li[k] = lk;
            pathv[k] = inward ? -s[u * L + lk] : s[u * L + lk];
            fac[k] = tau_ref[lk] / alpha_ref[lk] * dsdz[u * L + lk];
            lt[k] = inward ? -ltr[lk] : ltr[lk];
        }
        if (n == 1 && (I_scheme == 2 || tau_scheme == 1)) continue; /* :150-154 */
        for (int64_t j = 0; j < nwl; j++) {
            for (int k = 0; k < n; k++) { acol[k] = alpha[j * L + li[k]]; Scol[k] = S[j * L + li[k]]; }
            if (tau_scheme == 0) tau_anchored(alpha + j * L, li, n, fac, lt, tau);
            else tau_bezier(tau, pathv, acol, n);
            double *Iout = Isurf + (size_t)r * nwl + j;
            if (I_scheme == 0 || I_scheme == 2) {
                for (int k = 0; k < n; k++) Ilay[k] = 0;
                Ilay[n - 1] = Ibot[(size_t)r * nwl + j];
                if (I_scheme == 0) I_linear(Ilay, tau, Scol, n);
                else I_bezier(Ilay, tau, Scol, n);
                *Iout = Ilay[0];
                /* the inward ray's intensity where it reaches its deepest layer (k = 0 on the
                   reversed path) seeds outward ray r + n_in at the bottom (:196-198) */
                if (inward) Ibot[(size_t)(r + n_in) * nwl + j] = Ilay[0];
            } else {
                double add = I_scheme == 1 ? I_linear_flux_only(tau, Scol, n)
                                           : column_flux_expint(acol, Scol, n, fac, lt, tau, Ilay);
                *Iout += add;
                if (inward) Isurf[(size_t)(r + n_in) * nwl + j] = *Iout * exp(-tau[n - 1]);
            }
        }
    }
    /* :135-136 */
    for (int64_t j = 0; j < nwl; j++) {
        double F = 0;
        for (int u = 0; u < n_mu; u++) F += Isurf[(size_t)(n_in + u) * nwl + j] * (mu_w[u] * mu[u]);
        flux[j] = 2 * PI * F;
    }
    (void)flux_only;
    free(nlay); free(s); free(dsdz); free(in_idx); free(Isurf); free(Ibot); free(ltr); free(tau);
    free(pathv); free(fac); free(lt); free(acol); free(Scol); free(Ilay); free(li);
    return 0;
}

/* ------------------------------------------------------------------ synthesize */

/* src/synthesize.jl:249-318 on host-prepared layer inputs */
int64_t ko_synthesize(const ko_synth_in *in, const ko_lines *lines, const ko_lines *lines5,
                      const ko_stark *stark, const double *wls, int64_t nwl, double *alpha,
                      double *flux, double *cntm_flux, double *alpha_ref_out) {
    int32_t L = in->L;
    int nt = in->nthreads < 1 ? 1 : in->nthreads;
    /* :249-252 alpha rows from the continuum interpolants */
#pragma omp parallel for num_threads(nt) if (nt > 1)
    for (int64_t j = 0; j < nwl; j++)
        for (int l = 0; l < L; l++)
            alpha[j * L + l] = gridded_linear(in->cntm.knots, in->cntm.vals + (int64_t)l * in->cntm.nk,
                                              in->cntm.nk, wls[j]);
    /* :265-283 alpha_ref gets the reference-wavelength line opacity */
    double *aref = alpha_ref_out;
    for (int l = 0; l < L; l++) aref[l] = in->alpha_ref_cntm[l];
    ko_layers lay = {L, in->S, in->T, in->ne, in->n_eff_vdW, in->xi, in->n_div_U};
    ko_cntm cref = {1, NULL, in->alpha_ref_cntm};
    double refwl = in->ref_wl;
    int64_t evals = ko_line_absorption(aref, lines5, &refwl, 1, &lay, &cref, in->cutoff_threshold,
                                       nt, NULL, NULL);
    /* :285 source function */
    double *S = malloc(sizeof(double) * L * nwl);
#pragma omp parallel for num_threads(nt) if (nt > 1)
    for (int64_t j = 0; j < nwl; j++)
        for (int l = 0; l < L; l++) S[j * L + l] = ko_blackbody(in->T[l], wls[j]);
    /* :287-291 continuum-only transfer */
    ko_rt_flux_expint(alpha, S, L, nwl, in->tau_ref, aref, cntm_flux, nt);
    /* :293-303 hydrogen lines, one layer at a time */
    if (in->hydrogen_lines) {
        double *row = malloc(sizeof(double) * nwl);
        for (int l = 0; l < L; l++) {
            for (int64_t j = 0; j < nwl; j++) row[j] = alpha[j * L + l];
            ko_hydrogen_line_absorption(row, wls, nwl, in->T[l], in->ne[l], in->nH_I[l],
                                        in->nHe_I[l], in->UH_I[l], in->xi[l], in->hydrogen_window,
                                        in->use_MHD, stark);
            for (int64_t j = 0; j < nwl; j++) alpha[j * L + l] = row[j];
        }
        free(row);
    }
    /* :305-306 metal and molecular lines */
    evals += ko_line_absorption(alpha, lines, wls, nwl, &lay, &in->cntm, in->cutoff_threshold, nt,
                                NULL, NULL);
    /* :310-318 final transfer and unit conversion */
    ko_rt_flux_expint(alpha, S, L, nwl, in->tau_ref, aref, flux, nt);
    for (int64_t j = 0; j < nwl; j++) { flux[j] *= 1e-8; cntm_flux[j] *= 1e-8; }
    free(S);
    return evals;
}

/* ------------------------------------------------------------------ vector helpers (tests) */
void ko_line_profile_many(int64_t n, double wl0, double sigma, double gamma, double amp,
                          const double *wls, double *out) {
    for (int64_t i = 0; i < n; i++) out[i] = ko_line_profile(wl0, sigma, gamma, amp, wls[i]);
}
void ko_voigt_many(int64_t n, const double *a, const double *v, double *out) {
    for (int64_t i = 0; i < n; i++) out[i] = ko_voigt_hjerting(a[i], v[i]);
}
void ko_expint2_many(int64_t n, const double *x, double *out) {
    for (int64_t i = 0; i < n; i++) out[i] = ko_exponential_integral_2(x[i]);
}
