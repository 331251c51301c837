// continuum.cuh -- continuum absorption on the device: total_continuum_absorption
// (src/ContinuumAbsorption/ContinuumAbsorption.jl:39-74) for every layer and wavelength of the
// continuum grid that synthesize evaluates (src/synthesize.jl:211-237), in FP64.
//
// Terms (each restated from the cited reference function, tables converted unchanged):
//   H I bound-free with MHD level dissolution          absorption_H.jl:54-163
//   H- bound-free (McLaughlin 2017)                    absorption_H.jl:166-228
//   H- free-free (Bell & Berrington 1987)              absorption_H.jl:230-325
//   H2+ bound-free and free-free (Stancil 1994)        absorption_H.jl:327-380, Stancil1994.jl
//   He- free-free (John 1994)                          absorption_He.jl:31-95
//   positive-ion free-free (hydrogenic, van Hoof 2014 Gaunt factors, Peach 1970 departures)
//                                                      absorption_ff_positive_ion.jl, hydrogenic_bf_ff.jl
//   Thomson and Rayleigh scattering                    scattering.jl
// Metal bound-free absorption (absorption_metals_bf.jl) needs the bf_cross-sections.h5 blob,
// which is not part of the reference checkout: it is not included.
//
// One thread per (layer, wavelength); the work is tiny next to the line opacity (a few hundred
// thousand points per atmosphere), so the kernel favours plainness: binary searches on the
// (read-only, cached) tables.
#pragma once
#include "physics.cuh"

namespace korg {

constexpr int CNT_PEACH = 4;  // He II, C II, Si II, Mg II (the ions taking part; charge 1)

// Device copies of the tables (one buffer, carved by the host).
struct CntmTables {
    int32_t h_n;                      // points per H I level table (levels 1..6)
    const double *h_E, *h_sigma;      // [6][h_n] eV, megabarn
    int64_t hm_n;
    const double *hm_nu, *hm_sigma;   // H- bf: Hz, cm^2
    int32_t hff_nl, hff_nt;
    const double *hff_lambda, *hff_theta, *hff_K;    // [nl][nt], 1e-26 cm^4/dyn
    int32_t heff_nl, heff_nt;
    const double *heff_lambda, *heff_theta, *heff_K;
    int32_t h2_nT, h2_nbf, h2_nff;
    const double *h2_T, *h2_K, *h2_bf_lambda, *h2_bf_sigma, *h2_ff_lambda, *h2_ff_sigma;  // sigma [n][nT]
    int32_t g_nu, g_ng;
    const double *g_log_u, *g_log_g2, *g_ff;         // [nu][ng]
    int32_t p_nT[CNT_PEACH], p_ns;
    const double *p_T[CNT_PEACH], *p_sigma, *p_D[CNT_PEACH];  // D [nT][ns]
};

// Per-layer inputs (device pointers).
struct CntmLayers {
    int32_t L;
    const double *T, *ne, *nH_I, *nH_II, *nHe_I, *nH2, *nH_minus, *invU_H_I, *invU_He_I;
    const double *n_Z1, *n_Z2;
    const double *n_peach[CNT_PEACH];
};

namespace cnt {

constexpr double KB_CGS = 1.380649e-16, H_CGS = 6.62607015e-27, C = 2.99792458e10;
constexpr double KB_EV = 8.617333262145e-5, H_EV = 4.135667696e-15;
constexpr double RYH_EV = 13.598287264, RY_EV = 13.605693122994;
constexpr double CHI_H = 13.5984;         // ionization energy of H I (Barklem & Collet 2016)
constexpr double HMINUS_ION_EV = 0.754204;

// index i with x[i] <= v < x[i+1], clamped to [0, n-2]
__device__ __forceinline__ int64_t seg(const double* x, int64_t n, double v) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = lo + ((hi - lo) >> 1);
        if (x[mid] <= v) lo = mid + 1; else hi = mid;
    }
    lo -= 1;
    return lo < 0 ? 0 : (lo > n - 2 ? n - 2 : lo);
}
// linear interpolation, linear extrapolation beyond the ends (Interpolations.jl Line())
__device__ __forceinline__ double lerp(const double* x, const double* y, int64_t n, double v) {
    const int64_t i = seg(x, n, v);
    const double t = (v - x[i]) / (x[i + 1] - x[i]);
    return y[i] * (1 - t) + y[i + 1] * t;
}
// bilinear interpolation on a grid, Z[i][j] over (x[i], y[j])
__device__ __forceinline__ double bilerp(const double* x, int nx, const double* y, int ny, const double* Z, double u,
                                         double v) {
    const int64_t i = seg(x, nx, u), j = seg(y, ny, v);
    const double tx = (u - x[i]) / (x[i + 1] - x[i]), ty = (v - y[j]) / (y[j + 1] - y[j]);
    return Z[i * ny + j] * (1 - tx) * (1 - ty) + Z[(i + 1) * ny + j] * tx * (1 - ty) +
           Z[i * ny + j + 1] * (1 - tx) * ty + Z[(i + 1) * ny + j + 1] * tx * ty;
}
__device__ __forceinline__ bool in(double x, double lo, double hi) { return x >= lo && x <= hi; }

// src/statmech.jl:463-497 (default branch), with T unused; n_eff may be +inf (w = 0)
__device__ __forceinline__ double mhd_w(double n_eff, double nH, double nHe, double ne) {
    return hummer_mihalas_w(n_eff, nH, nHe, ne);
}

// absorption_H.jl:54-163
__device__ double H_I_bf(const CntmTables& t, double nu, double T, double nH_I, double nHe_I, double ne,
                         double invU_H) {
    double total = 0.0;
    for (int n = 1; n <= 6; n++) {
        const double* Es = t.h_E + (n - 1) * t.h_n;
        const double* sig = t.h_sigma + (n - 1) * t.h_n;
        const double w_lower = mhd_w(double(n), nH_I, nHe_I, ne);
        const double occ = w_lower * exp(-CHI_H * (1 - 1.0 / (n * n)) / (KB_EV * T));
        const double nu_break = CHI_H / (n * n * H_EV);
        double cs, frac;
        if (nu > nu_break) {
            frac = 1.0;
            cs = lerp(Es, sig, t.h_n, H_EV * nu);
        } else {
            if (n == 1) {
                frac = 0.0;
            } else {
                const double n_eff = 1 / sqrt(1.0 / (n * n) - H_EV * nu / CHI_H);
                frac = 1 - mhd_w(n_eff, nH_I, nHe_I, ne) / w_lower;
            }
            const double sigma_break = lerp(Es, sig, t.h_n, nu_break * H_EV);
            cs = pow(nu, -3.0) * (sigma_break / pow(nu_break, -3.0));
        }
        total += occ * cs * frac;
    }
    for (int n = 7; n <= 40; n++) {
        const double w_lower = mhd_w(double(n), nH_I, nHe_I, ne);
        if (w_lower < 1e-5) break;
        const double occ = 2.0 * n * n * w_lower * exp(-CHI_H * (1 - 1.0 / (n * n)) / (KB_EV * T));
        const double inv_n = 1.0 / n, inv_n2 = inv_n * inv_n;
        if (!(H_EV * nu < RYH_EV * inv_n2)) {
            const double inv_nu = 1.0 / nu;
            total += occ * (2.815e29 * (inv_n2 * inv_n2 * inv_n) * (inv_nu * inv_nu * inv_nu) * 1e18);
        }
    }
    return nH_I * invU_H * total * (1.0 - exp(-H_EV * nu / (KB_EV * T))) * 1e-18;
}

// absorption_H.jl:170-228
__device__ double Hminus_bf(const CntmTables& t, double nu, double T, double n_Hminus) {
    if (!(nu >= 0.0 && nu <= 2.417989242625068e19 && T > 0)) return 0.0;
    const double nu_ion = HMINUS_ION_EV / H_EV, nu_min = t.hm_nu[0];
    double cs;
    if (nu <= nu_ion) {
        cs = 0.0;
    } else if (nu < nu_min) {
        cs = t.hm_sigma[0] / pow(nu_min - nu_ion, 1.5) * pow(nu - nu_ion, 1.5);
    } else {
        const int64_t i = seg(t.hm_nu, t.hm_n, nu);
        const double s = (t.hm_sigma[i + 1] - t.hm_sigma[i]) / (t.hm_nu[i + 1] - t.hm_nu[i]);
        cs = s * (nu - t.hm_nu[i]) + t.hm_sigma[i];
    }
    return n_Hminus * cs * (1 - exp(-H_CGS * nu / (KB_CGS * T)));
}

// absorption_H.jl:261-325: 1823 A <= lambda <= 151890 A, 1400 K <= T <= 10080 K
__device__ double Hminus_ff(const CntmTables& t, double nu, double T, double nH_I_div_U, double ne) {
    if (!(in(nu, C / 151890e-8, C / 1823e-8) && in(T, 1400, 10080))) return 0.0;
    const double K = 1e-26 * bilerp(t.hff_lambda, t.hff_nl, t.hff_theta, t.hff_nt, t.hff_K, C * 1e8 / nu, 5040.0 / T);
    return K * (ne * KB_CGS * T) * (2 * nH_I_div_U);
}

// absorption_H.jl:327-380, Stancil1994.jl: 700 A <= lambda <= 200000 A, 3150 K <= T <= 25200 K
__device__ double H2plus(const CntmTables& t, double nu, double T, double nH_I, double nH_II) {
    if (!(in(nu, C / 2e-3, C / 7e-6) && in(T, 3150, 25200))) return 0.0;
    const double lam = C * 1e8 / nu;
    const double K = lerp(t.h2_T, t.h2_K, t.h2_nT, T);
    const double sbf = 1e-18 * bilerp(t.h2_bf_lambda, t.h2_nbf, t.h2_T, t.h2_nT, t.h2_bf_sigma, lam, T);
    const double sff = 1e-39 * bilerp(t.h2_ff_lambda, t.h2_nff, t.h2_T, t.h2_nT, t.h2_ff_sigma, lam, T);
    return (sbf / K + sff) * nH_I * nH_II * (1 - exp(-H_EV * nu / (KB_EV * T)));
}

// absorption_He.jl:31-95: 5063 A <= lambda <= 151878 A, 1400 K <= T <= 10080 K
__device__ double Heminus_ff(const CntmTables& t, double nu, double T, double nHe_I_div_U, double ne) {
    if (!(in(nu, C / 1.518780e-3, C / 5.063e-5) && in(T, 1400, 10080))) return 0.0;
    const double K = 1e-26 * bilerp(t.heff_lambda, t.heff_nl, t.heff_theta, t.heff_nt, t.heff_K, C * 1e8 / nu,
                                    5040.0 / T);
    return K * nHe_I_div_U * (ne * KB_CGS * T);
}

// hydrogenic_bf_ff.jl:116-176
__device__ double hydrogenic_ff(const CntmTables& t, double nu, double T, int Z, double ni, double ne) {
    const double inv_T = 1.0 / T, Z2 = double(Z * Z);
    const double hnu_kT = (H_EV / KB_EV) * nu * inv_T;
    const double g = bilerp(t.g_log_u, t.g_nu, t.g_log_g2, t.g_ng, t.g_ff, log10(hnu_kT),
                            log10((RY_EV / KB_EV) * Z2 * inv_T));
    const double F = 3.6919e8 * g * Z2 * sqrt(inv_T) / (nu * nu * nu);
    return ni * ne * F * (1 - exp(-hnu_kT));
}

// Peach1970.jl: bilinear in (T, sigma), zero outside the table
__device__ double peach(const CntmTables& t, int k, double T, double sigma) {
    const double* Ts = t.p_T[k];
    const int nT = t.p_nT[k];
    if (!(in(T, Ts[0], Ts[nT - 1]) && in(sigma, t.p_sigma[0], t.p_sigma[t.p_ns - 1]))) return 0.0;
    return bilerp(Ts, nT, t.p_sigma, t.p_ns, t.p_D[k], T, sigma);
}

// absorption_ff_positive_ion.jl:44-84: 100 K <= T <= 1e6 K, 1e-6 cm < lambda < 1e-2 cm
__device__ double positive_ion_ff(const CntmTables& t, const CntmLayers& y, int l, double nu, double T, double ne) {
    if (!(T >= 100.0 && T <= 1e6) || !(C / 1e-2 < nu && nu < C / 1e-6)) return 0.0;
    double a = 0.0;
    const double sig = nu * (H_EV / RY_EV);  // photon energy in Rydberg Z^2 (Z = 1)
    for (int k = 0; k < CNT_PEACH; k++)
        a += hydrogenic_ff(t, nu, T, 1, y.n_peach[k][l], ne) * (1 + peach(t, k, T, sig));
    a += hydrogenic_ff(t, nu, T, 1, y.n_Z1[l], ne);
    a += hydrogenic_ff(t, nu, T, 2, y.n_Z2[l], ne);
    return a;
}

// scattering.jl
__device__ double rayleigh(double nu, double nH_I, double nHe_I, double nH2) {
    const double E2 = (H_EV * nu / (2 * RY_EV)) * (H_EV * nu / (2 * RY_EV));
    const double E4 = E2 * E2, E6 = E2 * E4, E8 = E4 * E4;
    const double sH = 20.24 * E4 + 239.2 * E6 + 2256 * E8, sHe = 1.913 * E4 + 4.52 * E6 + 7.90 * E8;
    const double i2 = (nu / (1e8 * C)) * (nu / (1e8 * C));
    const double i4 = i2 * i2, i6 = i2 * i4, i8 = i4 * i4;
    return (nH_I * sH + nHe_I * sHe) * 6.65246e-25 + (8.14e-13 * i4 + 1.28e-6 * i6 + 1.61 * i8) * nH2;
}
__device__ __forceinline__ double electron_scattering(double ne) {
    const double r = ELECTRON_CHARGE_CGS * ELECTRON_CHARGE_CGS / (ELECTRON_MASS_CGS * C * C);
    return 8 * PI / 3 * (r * r) * ne;
}

}  // namespace cnt

// vals[l * nwl + j] = total continuum absorption of layer l at wavelength wls[j] (cm), the
// layout of the continuum interpolants (korg_cntm)
__global__ void __launch_bounds__(256) continuum_kernel(CntmTables t, CntmLayers y, const double* wls, int64_t nwl,
                                                        double* vals) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= nwl * y.L) return;
    const int l = int(e / nwl);
    const int64_t j = e - int64_t(l) * nwl;
    const double nu = cnt::C / wls[j];
    const double T = y.T[l], ne = y.ne[l], nH = y.nH_I[l], nHe = y.nHe_I[l];
    double a = cnt::H_I_bf(t, nu, T, nH, nHe, ne, y.invU_H_I[l]);
    a += cnt::Hminus_bf(t, nu, T, y.nH_minus[l]);
    a += cnt::Hminus_ff(t, nu, T, nH * y.invU_H_I[l], ne);
    a += cnt::H2plus(t, nu, T, nH, y.nH_II[l]);
    a += cnt::Heminus_ff(t, nu, T, nHe * y.invU_He_I[l], ne);
    a += cnt::positive_ion_ff(t, y, l, nu, T, ne);
    a += cnt::electron_scattering(ne);
    a += cnt::rayleigh(nu, nH, nHe, y.nH2[l]);
    vals[e] = a;
}

}  // namespace korg
