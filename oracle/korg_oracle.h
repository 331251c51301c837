/*
 * korg_oracle.h -- FP64 CPU restatement of Korg.jl's synthesis hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path is compared
 * against (tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg).  Nothing in the
 * product links or calls it.  Every function cites the Korg.jl source (path:line, Korg.jl
 * v1.2.1) whose behaviour it restates.
 *
 * Layouts follow Korg: alpha is layers x wavelengths, column-major (layer index fastest):
 * alpha[j * L + l].  Wavelengths are in cm.  Lines are sorted by wavelength.
 */
#ifndef KORG_ORACLE_H
#define KORG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Line list as structure of arrays (src/linelist.jl:5-14). */
typedef struct {
    int64_t n;
    const double *wl;          /* cm */
    const double *log_gf;
    const double *E_lower;     /* eV */
    const double *gamma_rad;   /* s^-1 */
    const double *gamma_stark; /* s^-1 per perturber at 10,000 K */
    const double *vdW1;        /* gamma_vdW (vdW2 == -1) or ABO sigma */
    const double *vdW2;        /* -1 or ABO alpha */
    const double *mass;        /* g, get_mass(species) */
    const int32_t *is_mol;     /* ismolecule(species) */
    const int32_t *species;    /* row index into n_div_U */
} ko_lines;

/* Per-layer inputs of line_absorption! (src/line_absorption.jl:33-60). */
typedef struct {
    int32_t L;
    int32_t S;                 /* number of species rows in n_div_U */
    const double *T;           /* K */
    const double *ne;          /* cm^-3 */
    const double *n_eff_vdW;   /* cm^-3 (line_absorption.jl:59) */
    const double *xi;          /* cm/s, per layer */
    const double *n_div_U;     /* [S][L]: n(species)/U(species, ln T) */
} ko_layers;

/* Continuum opacity callables alpha_cntm[l](lambda): a piecewise-linear interpolant over
 * knots (src/synthesize.jl:226-228).  nk == 1 means a constant per layer (synthesize.jl:266). */
typedef struct {
    int64_t nk;
    const double *knots;       /* cm, increasing */
    const double *vals;        /* [L][nk] */
} ko_cntm;

/* Stehle & Hutcheon tables (src/hydrogen_line_absorption.jl:6-37), all transitions packed.
 * Transition t owns temps[t_off[t] ..], nes[ne_off[t] ..], logdnu (log of delta_nu_over_F0
 * with the first knot = -DBL_MAX) [d_off[t] ..], logP [p_off[t] + ((iD * nNe + iNe) * nT + iT)]
 * (-Inf replaced by -700) and lambda0 (cm) [l_off[t] + iNe * nT + iT]. */
typedef struct {
    int32_t ntrans;
    const int32_t *lower, *upper, *nT, *nNe, *nD;
    const int64_t *t_off, *ne_off, *d_off, *p_off, *l_off;
    const double *log_gf;
    const double *temps, *nes, *logdnu, *logP, *lambda0;
} ko_stark;

/* scalar physics (src/line_absorption.jl, src/RadiativeTransfer/RadiativeTransfer.jl) */
double ko_voigt_hjerting(double a, double v);
double ko_line_profile(double wl0, double sigma, double gamma, double amp, double wl);
double ko_exponential_integral_1(double x);
double ko_exponential_integral_2(double x);
double ko_blackbody(double T, double wl);
double ko_hummer_mihalas_w(double T, double n_eff, double nH, double nHe, double ne);
double ko_holtsmark_profile(double beta, double P);
double ko_brackett_oscillator_strength(int n, int m);

/* index bounds on a sorted wavelength array, 0-based (src/wavelengths.jl:188-210) */
int64_t ko_searchsortedfirst(const double *x, int64_t n, double v);
int64_t ko_searchsortedlast(const double *x, int64_t n, double v);

/* line_absorption! (src/line_absorption.jl:33-129).  alpha[L x nwl] is accumulated in place.
 * nthreads <= 1 reproduces a single-task run; otherwise the line list is split into
 * nthreads*tasks_per_thread chunks exactly as the reference does and the per-chunk private
 * alphas are summed at the end.  lb/ub (optional, may be NULL) receive each line's 0-based
 * window, ub < lb for skipped lines.  Returns the number of line-layer-wavelength
 * evaluations. */
int64_t ko_line_absorption(double *alpha, const ko_lines *lines, const double *wls, int64_t nwl,
                           const ko_layers *lay, const ko_cntm *cntm, double cutoff_threshold,
                           int nthreads, int64_t *lb_out, int64_t *ub_out);

/* hydrogen_line_absorption! for one layer (src/hydrogen_line_absorption.jl:75-163).
 * alphas[nwl] is accumulated in place. */
void ko_hydrogen_line_absorption(double *alphas, const double *wls, int64_t nwl, double T,
                                 double ne, double nH_I, double nHe_I, double UH_I, double xi,
                                 double window_size, int use_MHD, const ko_stark *stark);

/* Brackett-line profile on its own 201-point grid (hydrogen_line_absorption.jl:211-251).
 * Writes grid (wl, cm) and values; returns the window (0 when the line is off the grid). */
double ko_brackett_profile(int m, double wl0, double T, double ne, double xi, double wlmin,
                           double wlmax, double *grid201, double *vals201);

/* Planar radiative transfer, anchored tau + "linear_flux_only_expint"
 * (RadiativeTransfer.jl:62-139, 244-253, 379-497).  alpha, S are L x nwl col-major.
 * flux[nwl] receives 2*pi*I(mu=1 scheme) (no 1e-8 unit factor). */
void ko_rt_flux_expint(const double *alpha, const double *S, int32_t L, int64_t nwl,
                       const double *tau_ref, const double *alpha_ref, double *flux, int nthreads);

/* Planar or spherical RT with the secondary schemes (RadiativeTransfer.jl:77-139, 147-371):
 * tau_scheme 0 = anchored, 1 = bezier; I_scheme 0 = linear, 1 = linear_flux_only,
 * 2 = bezier, 3 = linear_flux_only_expint (only for planar+anchored).  mu/weights give the
 * surface mu grid (n_mu points).  spatial: z (planar) or radii (spherical).  flux[nwl]. */
int ko_rt_general(const double *alpha, const double *S, int32_t L, int64_t nwl,
                  const double *spatial, int spherical, const double *tau_ref,
                  const double *alpha_ref, const double *mu, const double *mu_w, int n_mu,
                  int include_inward_rays, int tau_scheme, int I_scheme, double *flux);

/* synthesize steps 5-12 (src/synthesize.jl:249-318) on host-prepared inputs.
 * alpha_out (L x nwl) receives the final alpha; flux/cntm (nwl) are in erg/s/cm^4/A. */
typedef struct {
    int32_t L;
    const double *T, *ne, *tau_ref, *xi, *n_eff_vdW, *n_div_U; int32_t S;
    const double *nH_I, *nHe_I, *UH_I;   /* per layer, for hydrogen lines */
    const double *alpha_ref_cntm;        /* per layer, continuum at the reference wavelength */
    double ref_wl;                       /* cm */
    ko_cntm cntm;                        /* continuum interpolants */
    int hydrogen_lines, use_MHD;
    double hydrogen_window;              /* cm */
    double cutoff_threshold;
    int nthreads;
} ko_synth_in;

int64_t ko_synthesize(const ko_synth_in *in, const ko_lines *lines, const ko_lines *lines5,
                      const ko_stark *stark, const double *wls, int64_t nwl, double *alpha_out,
                      double *flux, double *cntm_flux, double *alpha_ref_out);

/* vectorised helpers for the tests */
void ko_line_profile_many(int64_t n, double wl0, double sigma, double gamma, double amp,
                          const double *wls, double *out);
void ko_voigt_many(int64_t n, const double *a, const double *v, double *out);
void ko_expint2_many(int64_t n, const double *x, double *out);

#ifdef __cplusplus
}
#endif
#endif
