/*
 * korg_gb300.h -- C ABI of the GB300 (sm_103a) spectral-synthesis hot path.
 *
 * The entry points replace, one for one, the Julia functions of Korg.jl (v1.2.1) on the
 * synthesis hot path.  Each declaration names the reference function it stands in for.  The
 * ABI uses plain pointers and sizes only; every call returns a korg_status and never aborts.
 *
 * Layout conventions (identical to Korg):
 *   - wavelengths in cm, increasing;
 *   - alpha is a layers x wavelengths matrix stored column-major (layer index fastest):
 *     alpha[j * L + l] for wavelength j and layer l;
 *   - the line list is sorted by wavelength and given as a structure of arrays.
 *
 * Two families of calls:
 *   - host-pointer calls (korg_line_absorption, korg_synthesize, ...) take ordinary host
 *     arrays, copy them to the device, run, copy results back and return when done.  These
 *     are what a Julia `ccall` or Python `ctypes` binding uses as a drop-in for the reference.
 *   - `_dev` calls take device pointers (including the arrays inside the structs) and a
 *     CUDA stream, enqueue the work and return without synchronising.
 *
 * Precision: KORG_FP64 evaluates everything in FP64 (the plain form).  KORG_MIXED evaluates
 * line profiles in FP32 with Kahan-compensated accumulation, and keeps FP64 for the
 * wavelength offsets from line centres (rounded to FP32 afterwards), the per-layer line
 * strengths (Boltzmann factors, n/U), the reference-wavelength line opacity (one wavelength,
 * which anchors the optical depths), the optical-depth integration and the formal solution.
 */
#ifndef KORG_GB300_H
#define KORG_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KORG_API __attribute__((visibility("default")))

typedef enum {
    KORG_OK = 0,
    KORG_EINVAL = 1,   /* bad argument (sizes, null pointers, unsorted input, bad scheme) */
    KORG_ECUDA = 2,    /* a CUDA runtime call failed; korg_last_error() has the message */
    KORG_ENOMEM = 3,   /* device allocation failed */
    KORG_ENOTABLES = 4, /* hydrogen lines requested before korg_set_stark_tables() */
    KORG_ETOOBIG = 5,   /* the problem needs more scratch than KORG_NOALLOC_SCRATCH_BYTES */
    KORG_ETIMEOUT = 6,  /* a device-side wait for staged data ran past its limit (results invalid) */
    KORG_ECHEM = 7      /* chemical equilibrium failed in at least one layer (see its status) */
} korg_status;

/* Every call taking a `precision` returns KORG_EINVAL for any other value. */
enum { KORG_FP64 = 0, KORG_MIXED = 1 };

/* Line list (Korg.Line, src/linelist.jl:5-14), sorted by wl. */
typedef struct {
    int64_t n;
    const double *wl;          /* cm */
    const double *log_gf;
    const double *E_lower;     /* eV */
    const double *gamma_rad;   /* s^-1 */
    const double *gamma_stark; /* s^-1, per perturber at 10,000 K */
    const double *vdW1;        /* gamma_vdW at 10,000 K (vdW2 == -1) or ABO sigma (cm^2) */
    const double *vdW2;        /* -1 or ABO alpha */
    const double *mass;        /* g, get_mass(species) */
    const int32_t *is_mol;     /* ismolecule(species): no Stark / vdW broadening */
    const int32_t *species;    /* row of n_div_U for this line's species */
} korg_lines;

/* Per-layer inputs of line_absorption! (src/line_absorption.jl:33-60).  n_div_U[s * L + l] is
 * n(species s)/U(species s, ln T_l), the host precompute of line_absorption.jl:42-44;
 * n_eff_vdW is the perturber density of line_absorption.jl:59; xi is in cm/s. */
typedef struct {
    int32_t L;
    int32_t S;
    const double *T, *ne, *n_eff_vdW, *xi;
    const double *n_div_U;
} korg_layers;

/* Continuum-opacity callables alpha_cntm[l](wl) (src/synthesize.jl:226-228): piecewise linear
 * over nk knots (cm), vals[l * nk + k].  nk == 1 means a constant per layer (the form used
 * for the reference-wavelength opacity, src/synthesize.jl:266). */
typedef struct {
    int64_t nk;
    const double *knots;
    const double *vals;
} korg_cntm;

/* Stehle & Hutcheon hydrogen tables (src/hydrogen_line_absorption.jl:6-37), packed.  For
 * transition t: temps[t_off[t] + iT], nes[ne_off[t] + iNe], logdnu[d_off[t] + iD] (log of
 * delta_nu_over_F0, first knot -DBL_MAX), logP[p_off[t] + (iD * nNe + iNe) * nT + iT] (log
 * profile, -Inf clipped to -700), lambda0[l_off[t] + iNe * nT + iT] (cm). */
typedef struct {
    int32_t ntrans;
    const int32_t *lower, *upper, *nT, *nNe, *nD;
    const int64_t *t_off, *ne_off, *d_off, *p_off, *l_off;
    const double *log_gf;
    const double *temps, *nes, *logdnu, *logP, *lambda0;
} korg_stark_tables;

/* Everything synthesize() computes on the host before the hot path (src/synthesize.jl:211-262),
 * for one atmosphere. */
typedef struct {
    korg_layers layers;
    const double *tau_ref;        /* tau at the reference wavelength, per layer */
    const double *alpha_ref_cntm; /* continuum alpha at the reference wavelength, per layer */
    const double *nH_I, *nHe_I, *UH_I; /* per layer, for hydrogen lines */
    double ref_wl;                /* cm */
    korg_cntm cntm;
    int32_t hydrogen_lines, use_MHD;
    double hydrogen_window;       /* cm */
    double cutoff_threshold;
} korg_synth_inputs;

typedef struct {
    int64_t line_evals;        /* line-layer-wavelength Voigt evaluations of the last call */
    int64_t lines_in_window;   /* lines with a non-empty window */
    /* device time (ms) of the stages of the last korg_synthesize*, when timing is enabled:
     * reference-wavelength lines, hydrogen lines, metal-line prologue (per-line constants,
     * windows, scans), metal-line tile kernel, both transfers, whole call */
    float ms_ref_lines, ms_hydrogen, ms_line_prep, ms_line_tile, ms_rt, ms_total;
    /* the last korg_synthesize_vjp*: opacity recomputation, transfer adjoint, hydrogen-line
     * derivatives, line adjoint (metal and reference-wavelength lines) */
    float ms_vjp_alpha, ms_vjp_rt, ms_vjp_hydrogen, ms_vjp_lines;
} korg_stats;

typedef struct korg_ctx korg_ctx;

/* Context: device, stream-ordered scratch arena, uploaded hydrogen tables.  One per host
 * thread. */
KORG_API int korg_create(korg_ctx **ctx, int device);
KORG_API void korg_destroy(korg_ctx *ctx);
KORG_API const char *korg_last_error(const korg_ctx *ctx);
KORG_API int korg_get_stats(korg_ctx *ctx, korg_stats *out);
/* Timing of the stages with CUDA events (adds event records; off by default). */
KORG_API int korg_set_timing(korg_ctx *ctx, int enabled);

/* Uploads the Stehle & Hutcheon tables once (src/hydrogen_line_absorption.jl:38-39). */
KORG_API int korg_set_stark_tables(korg_ctx *ctx, const korg_stark_tables *host_tables);

/* Continuum absorption, total_continuum_absorption(nus, T, ne, number_densities, partition_funcs)
 * (src/ContinuumAbsorption/ContinuumAbsorption.jl:39-74) as synthesize evaluates it per layer on
 * the continuum grid (src/synthesize.jl:211-237): H I bound-free (with MHD level dissolution),
 * H- bound-free and free-free, H2+ bound-free and free-free, He- free-free, free-free of every
 * positive ion (hydrogenic with van Hoof Gaunt factors, Peach departure coefficients for He II,
 * C II, Si II and Mg II), Thomson and Rayleigh scattering.  Metal bound-free absorption
 * (absorption_metals_bf.jl) is not included: its cross-section tables are not distributed with
 * the reference.  FP64.
 *
 * korg_set_continuum_tables uploads the reference's tables once (sizes, host arrays, row-major):
 * H I bf cross-sections of levels 1..6 on energy grids [6][h_n] (eV, megabarn); H- bf [hm_n]
 * (Hz, cm^2); H- ff and He- ff K [nl][nt] in 1e-26 cm^4/dyn over wavelength (A) and theta =
 * 5040/T; H2+ K(T) [nT] and cross-sections [n][nT] (bf 1e-18 cm^2, ff 1e-39 cm^5) over
 * wavelength (A); free-free Gaunt factors [nu][ng] over log10 u and log10 gamma^2; Peach
 * departure coefficients D [nT][ns] over T and sigma, for He II, C II, Si II, Mg II in order. */
typedef struct {
    int32_t h_n;
    const double *h_E, *h_sigma;
    int64_t hm_n;
    const double *hm_nu, *hm_sigma;
    int32_t hff_nl, hff_nt;
    const double *hff_lambda, *hff_theta, *hff_K;
    int32_t heff_nl, heff_nt;
    const double *heff_lambda, *heff_theta, *heff_K;
    int32_t h2_nT, h2_nbf, h2_nff;
    const double *h2_T, *h2_K, *h2_bf_lambda, *h2_bf_sigma, *h2_ff_lambda, *h2_ff_sigma;
    int32_t g_nu, g_ng;
    const double *g_log_u, *g_log_g2, *g_ff;
    int32_t p_nT[4], p_ns;
    const double *p_T[4], *p_sigma, *p_D[4];
} korg_continuum_tables;
/* Per-layer inputs [L] (the host's chemical equilibrium): n(H I), n(H II), n(He I), n(H2),
 * n(H-), 1/U(H I, T) and 1/U(He I, T), n_Z1 / n_Z2 = summed densities of the other singly /
 * doubly charged species (H II included), n_peach = n(He II), n(C II), n(Si II), n(Mg II). */
typedef struct {
    int32_t L;
    const double *T, *ne, *nH_I, *nH_II, *nHe_I, *nH2, *nH_minus, *invU_H_I, *invU_He_I, *n_Z1, *n_Z2;
    const double *n_peach[4];
} korg_continuum_layers;
KORG_API int korg_set_continuum_tables(korg_ctx *ctx, const korg_continuum_tables *host_tables);
/* vals[l * nwl + j] = continuum absorption (cm^-1) of layer l at wls[j] (cm), the layout of
 * korg_cntm.vals.  _dev: device pointers (wls, layer arrays, vals), stream-ordered. */
KORG_API int korg_continuum_absorption(korg_ctx *ctx, const double *wls, int64_t nwl,
                                       const korg_continuum_layers *layers, double *vals);
KORG_API int korg_continuum_absorption_dev(korg_ctx *ctx, const double *wls, int64_t nwl,
                                           const korg_continuum_layers *layers, double *vals,
                                           void *stream);

/* Chemical equilibrium, chemical_equilibrium(T, n_tot, ne, absolute_abundances,
 * ionization_energies, partition_fns, log_equilibrium_constants) (src/statmech.jl:148-206),
 * solved for every layer of one or many atmospheres at once (synthesize calls it per layer,
 * src/synthesize.jl:210-219).  The unknowns are log10 of the 92 neutral-atom densities and of
 * n_e; the solver is the reference's (src/statmech.jl:215-305, src/newton.jl): Newton steps
 * clipped to 1 dex, tolerance 1e-8 on the scaled residuals, and a continuation on the molecule
 * and H- scale log xi when the plain solve fails.  FP64 throughout.
 *
 * korg_set_equilibrium_tables uploads the data once.  Every spline is Korg's natural cubic
 * spline over ln T (src/CubicSplines.jl) given by knots t, values u and second derivatives z:
 *   atomic partition functions on shared knots lnT[n_knots], U_u / U_z [92*3][n_knots] with
 *     species (Z, q) at row 3(Z-1)+q (the H III row is never read); T must lie in the knot range;
 *   chi [92*3]: ionization energies (eV) chi1, chi2, chi3 of each element;
 *   molecules m < n_mol (at most KORG_CHEM_MAX_MOL): atoms [n_mol][6] ascending atomic numbers,
 *     0-padded; charge 0 or 1 (a charged molecule is a diatomic whose first atom is the ion);
 *     kind 0: log10 K (partial-pressure form) is the spline at spl[off[m] .. off[m+1]);
 *     kind 1: a polyatomic, log10 K from its atomization energy D00 (eV), the log10 ratio lmr of
 *     its atoms' masses product to its mass, and its partition function, the spline at
 *     spl[off[m] .. off[m+1]) (src/read_statmech_quantities.jl:66-89).
 * Molecule splines extrapolate flat; the atomic ones do not. */
#define KORG_CHEM_MAX_MOL 384
typedef struct {
    int32_t n_knots;
    const double *lnT, *U_u, *U_z, *chi;
    int32_t n_mol;
    const int32_t *atoms, *charge, *kind;
    const int64_t *off;
    const double *spl_t, *spl_u, *spl_z, *D00, *lmr;
} korg_equilibrium_tables;
/* Layers: T (K), n_tot and the model atmosphere's n_e (cm^-3, the starting guess) per layer;
 * abundances [n_atm][92] = N_X / N_total of each atmosphere (positive, normalised by the
 * caller as src/synthesize.jl:208-209 does); atm [L] the atmosphere of each layer (NULL: all 0). */
typedef struct {
    int32_t L;
    const double *T, *n_tot, *ne_model, *abundances;
    const int32_t *atm;
} korg_chem_layers;
/* densities [L][KORG_CHEM_MOL0 + n_mol]: n_e, n(Z, q) for q = 0, 1, 2 (H III is 0), n(H-), then
 * each molecule in table order.  status [L]: KORG_CHEM_OK, or why the layer failed; info
 * [L][5] (may be NULL): Newton iterations, solves, the log xi reached (or where the
 * continuation stopped), the last residual inf-norm, and the Newton steps whose linear solve
 * fell back from FP32 factors with FP64 refinement to FP64 elimination.  The host entry point returns KORG_ECHEM
 * when any layer failed (densities of the other layers are valid); _dev takes device pointers
 * and is stream-ordered (read status after the stream). */
#define KORG_CHEM_NE 0
#define KORG_CHEM_ATOM(Z, q) (1 + 3 * ((Z) - 1) + (q))
#define KORG_CHEM_HMINUS 277
#define KORG_CHEM_MOL0 278
enum {
    KORG_CHEM_OK = 0,
    KORG_CHEM_ANCHOR = 1,     /* no anchor log xi in (-5, -20, -50) converged */
    KORG_CHEM_ANNEAL = 2,     /* the continuation step fell below 1/16 without converging */
    KORG_CHEM_NONFINITE = 3,  /* the solution contains non-finite values */
    KORG_CHEM_BUDGET = 4      /* more than KORG_CHEM_MAX_ITER Newton iterations in total */
};
#define KORG_CHEM_MAX_ITER 20000
KORG_API int korg_set_equilibrium_tables(korg_ctx *ctx, const korg_equilibrium_tables *host_tables);
KORG_API int korg_chemical_equilibrium(korg_ctx *ctx, const korg_chem_layers *layers, int32_t n_atm,
                                       double *densities, int32_t *status, double *info);
KORG_API int korg_chemical_equilibrium_dev(korg_ctx *ctx, const korg_chem_layers *layers,
                                           int32_t n_atm, double *densities, int32_t *status,
                                           double *info, void *stream);
/* Reverse mode of chemical_equilibrium at the solution `densities` returned for `layers` (what
 * the reference's ForwardDiff method computes, src/statmech.jl:307-355, by the implicit-function
 * rule): given gbar [L][KORG_CHEM_MOL0 + n_mol], the cotangents of every density in the same
 * layout, returns per layer dL/dT (dT [L]), dL/dn_tot (dn_tot [L]) and dL/d(abundance of each
 * element) (dab [L][92], the abundances as passed, i.e. normalised; sum over an atmosphere's
 * layers for its gradient).  The model n_e does not enter the solution.  KORG_ECHEM if a layer's
 * system is singular; _dev: device pointers, status [L] on the device, stream-ordered. */
KORG_API int korg_chemical_equilibrium_vjp(korg_ctx *ctx, const korg_chem_layers *layers, int32_t n_atm,
                                           const double *densities, const double *gbar, double *dT,
                                           double *dn_tot, double *dab);
KORG_API int korg_chemical_equilibrium_vjp_dev(korg_ctx *ctx, const korg_chem_layers *layers,
                                               int32_t n_atm, const double *densities,
                                               const double *gbar, double *dT, double *dn_tot,
                                               double *dab, int32_t *status, void *stream);

/* line_absorption!(alpha, linelist, wls, temps, ne, n_densities, partition_fns, xi, alpha_cntm;
 * cutoff_threshold) -- src/line_absorption.jl:33-129.  alpha (host, L x nwl) is accumulated in
 * place; an empty line list leaves it untouched (line_absorption.jl:35-37).  n_evals may be
 * NULL. */
KORG_API int korg_line_absorption(korg_ctx *ctx, double *alpha, const double *wls, int64_t nwl,
                                  const korg_lines *lines, const korg_layers *layers,
                                  const korg_cntm *cntm, double cutoff_threshold, int precision,
                                  int64_t *n_evals);
KORG_API int korg_line_absorption_dev(korg_ctx *ctx, double *alpha, const double *wls, int64_t nwl,
                                      const korg_lines *lines, const korg_layers *layers,
                                      const korg_cntm *cntm, double cutoff_threshold,
                                      int precision, void *stream);

/* hydrogen_line_absorption!(alphas, wls, T, ne, nH_I, nHe_I, UH_I, xi, window_size; use_MHD)
 * -- src/hydrogen_line_absorption.jl:75-163, one layer; alphas (host, nwl) accumulated. */
KORG_API int korg_hydrogen_line_absorption(korg_ctx *ctx, double *alphas, const double *wls,
                                           int64_t nwl, double T, double ne, double nH_I,
                                           double nHe_I, double UH_I, double xi,
                                           double window_size, int use_MHD, int precision);
/* All layers at once, as synthesize calls it per layer (src/synthesize.jl:293-303);
 * alpha is the device L x nwl matrix, per-layer arrays are device pointers. */
KORG_API int korg_hydrogen_lines_dev(korg_ctx *ctx, double *alpha, const double *wls, int64_t nwl,
                                     int32_t L, const double *T, const double *ne,
                                     const double *nH_I, const double *nHe_I, const double *UH_I,
                                     const double *xi, double window_size, int use_MHD,
                                     int precision, void *stream);

/* RadiativeTransfer.radiative_transfer(atm::PlanarAtmosphere, alpha, S, mu_points; alpha_ref,
 * tau_scheme="anchored", I_scheme="linear_flux_only") -- RadiativeTransfer.jl:62-139, the
 * default planar path (anchored tau, exponential-integral flux).  flux[nwl] = F (erg/s/cm^5,
 * without synthesize's 1e-8). */
KORG_API int korg_radiative_transfer(korg_ctx *ctx, const double *alpha, const double *S,
                                     int32_t L, int64_t nwl, const double *tau_ref,
                                     const double *alpha_ref, double *flux);
KORG_API int korg_radiative_transfer_dev(korg_ctx *ctx, const double *alpha, const double *S,
                                         int32_t L, int64_t nwl, const double *tau_ref,
                                         const double *alpha_ref, double *flux, void *stream);

/* RadiativeTransfer.radiative_transfer(alpha, S, spatial_coord, mu_points, spherical;
 * include_inward_rays, alpha_ref, tau_ref, I_scheme, tau_scheme) -- RadiativeTransfer.jl:77-139
 * with any scheme: spatial = heights (planar) or radii (spherical), the surface mu grid and its
 * weights (generate_mu_grid, :13-30, is the caller's), tau_scheme 0 = "anchored", 1 = "bezier";
 * I_scheme 0 = "linear", 1 = "linear_flux_only", 2 = "bezier", 3 = the exponential-integral
 * flux (planar, anchored).  flux[nwl] = 2 pi sum_mu w mu I(mu, surface); I_surface
 * (n_mu x nwl, may be NULL) gets the outward surface intensities.  The ShellAtmosphere
 * photosphere correction (:73) is the caller's.  Host pointers. */
KORG_API int korg_radiative_transfer_general(korg_ctx *ctx, const double *alpha, const double *S,
                                             int32_t L, int64_t nwl, const double *spatial,
                                             int spherical, const double *tau_ref,
                                             const double *alpha_ref, const double *mu,
                                             const double *mu_weights, int32_t n_mu,
                                             int include_inward_rays, int tau_scheme,
                                             int I_scheme, double *flux, double *I_surface);

/* synthesize(atm, linelist, A_X, wavelengths) steps after chemical equilibrium and continuum
 * (src/synthesize.jl:249-318): alpha_ref lines at the reference wavelength, source function,
 * continuum-only transfer, hydrogen lines, metal/molecular lines, final transfer.  lines5 is
 * the reference-wavelength line list (synthesize.jl:197-200).  flux and cntm (nwl, host) in
 * erg/s/cm^4/A; alpha_out (L x nwl) and alpha_ref_out (L) may be NULL. */
KORG_API int korg_synthesize(korg_ctx *ctx, const korg_synth_inputs *in, const korg_lines *lines,
                             const korg_lines *lines5, const double *wls, int64_t nwl,
                             int precision, double *flux, double *cntm, double *alpha_out,
                             double *alpha_ref_out);
KORG_API int korg_synthesize_dev(korg_ctx *ctx, const korg_synth_inputs *in,
                                 const korg_lines *lines, const korg_lines *lines5,
                                 const double *wls, int64_t nwl, int precision, double *flux,
                                 double *cntm, double *alpha_out, void *stream);

/* Reverse mode of korg_synthesize (the vector-Jacobian product of the hot path), for
 * gradient-based fitting (src/Fit/fit_via_synthesis.jl:304-390, where the reference uses
 * ForwardDiff through synthesize).  Given cotangents dflux and dcntm (nwl each; either may be
 * NULL) of synthesize's flux and continuum flux, fills the gradients the caller asks for
 * (NULL pointers are skipped; the others are overwritten):
 *   T, ne, n_eff_vdW, xi, nH_I, nHe_I, UH_I      [L]   layer inputs of korg_synth_inputs
 *   n_div_U                                      [S*L] n(species)/U(species, T) rows
 *   log_gf                                       [lines->n] per line of `lines`
 *   cntm_vals                                    [L*nk] continuum interpolant knots
 *   alpha_ref_cntm                               [L]   continuum opacity at the reference wl
 * The inputs are independent variables here: the chain rule through the host's chemical
 * equilibrium, partition functions and continuum (T -> n, U, alpha_cntm) is the caller's.
 * alpha is recomputed (not stored by the forward call); the line windows carry no derivative,
 * as under ForwardDiff.  With KORG_VJP_HYDROGEN the hydrogen-line opacity contributes too,
 * with the exact derivatives of its approximation (layer diagonal; forward-mode dual numbers
 * through the line records, the Stehle table interpolation, the ABO Voigt profiles and the
 * Brackett profiles); without it, hydrogen lines are held fixed. */
typedef struct {
    double *T, *ne, *n_eff_vdW, *xi;
    double *n_div_U;
    double *nH_I, *nHe_I, *UH_I;
    double *log_gf;
    double *cntm_vals;
    double *alpha_ref_cntm;
} korg_synth_grads;
/* KORG_VJP_REUSE_FORWARD: the previous call on this context was korg_synthesize[_dev] with the
 * same inputs; its alpha (kept in the context when alpha_out was NULL), alpha_ref, line prologue
 * and hydrogen-line records are reused instead of recomputed. */
enum { KORG_VJP_HYDROGEN = 1, KORG_VJP_REUSE_FORWARD = 2 };
KORG_API int korg_synthesize_vjp(korg_ctx *ctx, const korg_synth_inputs *in, const korg_lines *lines,
                                 const korg_lines *lines5, const double *wls, int64_t nwl,
                                 int precision, const double *dflux, const double *dcntm,
                                 const korg_synth_grads *grads, int flags);
KORG_API int korg_synthesize_vjp_dev(korg_ctx *ctx, const korg_synth_inputs *in,
                                     const korg_lines *lines, const korg_lines *lines5,
                                     const double *wls, int64_t nwl, int precision,
                                     const double *dflux, const double *dcntm,
                                     const korg_synth_grads *grads, int flags, void *stream);

/* Waits for all work on the context's device and reports KORG_ETIMEOUT (once) if a kernel of
 * an earlier asynchronous (_dev) call gave up a bounded wait for staged data; korg_synthesize_vjp
 * makes this check itself.  No counterpart in the reference (Julia has no device waits). */
KORG_API int korg_device_status(korg_ctx *ctx);
/* Self-test of that path, no counterpart in the reference: one block waits (at most `polls`
 * polls) on an mbarrier that nothing arrives on, the way the line adjoint waits for staged data,
 * sets the error word and returns; the call returns korg_device_status, i.e. KORG_ETIMEOUT, and
 * leaves the context usable. */
KORG_API int korg_selftest_wait_timeout(korg_ctx *ctx, int polls);

/* Spectral post-processing (src/utils.jl), device pointers, FP64, stream-ordered.
 *
 * korg_apply_lsf_dev: apply_LSF / compute_LSF_matrix(...) * flux (src/utils.jl:45-58, 94-155).
 * Each output wavelength out_wls[i] (cm) gets the Gaussian of FWHM out_wls[i] / R cut at
 * window_size sigma and renormalised over the window, applied to flux [nspec][nwl] on the sorted
 * grid wls [nwl] (cm): out [nspec][nout].  R has one value (nR = 1) or one per output
 * (nR = nout; the reference's R(lambda) function evaluated by the caller at out_wls in A).
 * apply_LSF is the case out_wls = wls.
 * korg_apply_lsf_vjp_dev: reverse mode, dflux [nspec][nwl] += L^T dout [nspec][nout].
 * korg_lsf_windows_dev / korg_lsf_matrix_values_dev: compute_LSF_matrix in CSR form -- the
 * window [lb[i], ub[i]] (0-based, inclusive) of every output, then, with row_ptr the exclusive
 * scan of ub - lb + 1, the normalised weights vals[row_ptr[i] + j - lb[i]]. */
KORG_API int korg_apply_lsf_dev(korg_ctx *ctx, const double *wls, int64_t nwl, const double *out_wls,
                                int64_t nout, const double *R, int64_t nR, double window_size,
                                const double *flux, int32_t nspec, double *out, void *stream);
KORG_API int korg_apply_lsf_vjp_dev(korg_ctx *ctx, const double *wls, int64_t nwl, const double *out_wls,
                                    int64_t nout, const double *R, int64_t nR, double window_size,
                                    const double *dout, int32_t nspec, double *dflux, void *stream);
KORG_API int korg_lsf_windows_dev(korg_ctx *ctx, const double *wls, int64_t nwl, const double *out_wls,
                                  int64_t nout, const double *R, int64_t nR, double window_size,
                                  int64_t *lb, int64_t *ub, void *stream);
KORG_API int korg_lsf_matrix_values_dev(korg_ctx *ctx, const double *wls, int64_t nwl,
                                        const double *out_wls, int64_t nout, const double *R, int64_t nR,
                                        double window_size, const int64_t *row_ptr, double *vals,
                                        void *stream);
/* korg_apply_rotation_dev: apply_rotation(flux, wls, vsini, eps) (src/utils.jl:168-240) --
 * rotational broadening with linear limb darkening, each uniform wavelength range separately.
 * wls [nwl] (cm) are the grid values; ranges (a host array of at most 64) give each range's
 * length and step (cm), in order, covering the grid; vsini in km/s.  flux, out [nspec][nwl].
 * korg_apply_rotation_vjp_dev: reverse mode, dflux += R^T dout. */
typedef struct {
    int64_t n;      /* points of the range */
    double start;   /* first wavelength (cm) */
    double step;    /* step (cm) */
} korg_wl_range;
KORG_API int korg_apply_rotation_dev(korg_ctx *ctx, const double *wls, int64_t nwl,
                                     const korg_wl_range *ranges, int32_t nranges, double vsini,
                                     double eps, const double *flux, int32_t nspec, double *out,
                                     void *stream);
KORG_API int korg_apply_rotation_vjp_dev(korg_ctx *ctx, const double *wls, int64_t nwl,
                                         const korg_wl_range *ranges, int32_t nranges, double vsini,
                                         double eps, const double *dout, int32_t nspec, double *dflux,
                                         void *stream);

/* MolecularCrossSection(linelist, wl_params; cutoff_alpha, vmic_vals, log_temp_vals) --
 * src/molecular_cross_sections.jl:51-88: the absorption cross-section per molecule of one
 * species' lines on a (vmic, T, wavelength) grid, with the line-opacity kernels.  Device
 * pointers: lines (species row 0 for every line), wls[nwl], T[nT] = 10^log_temp_vals,
 * inv_U[nT] = 1/U(T) of the species, vmic_vals[nv] in km/s; table[(v * nwl + j) * nT + t]. */
KORG_API int korg_molecular_cross_section_dev(korg_ctx *ctx, const korg_lines *lines, const double *wls,
                                              int64_t nwl, const double *T, const double *inv_U,
                                              int32_t nT, const double *vmic_vals, int32_t nv,
                                              double cutoff_alpha, int precision, double *table,
                                              void *stream);
/* interpolate_molecular_cross_sections! (src/molecular_cross_sections.jl:101-117) for one table:
 * alpha[j * L + l] += table(vmic[l], log10 T[l], wls[j]) * n[l], trilinear on the table's grid,
 * zero outside it.  Device pointers. */
KORG_API int korg_interpolate_molecular_cross_section_dev(korg_ctx *ctx, double *alpha, const double *wls,
                                                          int64_t nwl, int32_t L, const double *T,
                                                          const double *vmic, const double *n,
                                                          const double *table, const double *table_wls,
                                                          int64_t ntw, const double *vmic_vals, int32_t nv,
                                                          const double *log_temp_vals, int32_t nT,
                                                          void *stream);

/* Batched synthesis: many spectra on one wavelength grid, as the Fit module's repeated-synthesis
 * loop (src/Fit/fit_via_synthesis.jl:304-390) and grid building call synthesize.  Each item is
 * one synthesize call of korg_synthesize_dev (device pointers inside; flux and cntm are device
 * arrays of nwl); all items need the same layer count.  The per-spectrum prologues run first,
 * then one persistent launch of the line tile kernel works through a queue of
 * (spectrum, wavelength-tile) items, then the transfers; spectra are processed in chunks whose
 * scratch fits the budget of korg_set_batch_options.  Results equal korg_synthesize_dev's
 * for the same tile shape.  korg_stats for a batch: line_evals and lines_in_window are
 * totals, ms_total covers the batch, ms_line_tile and ms_rt the last chunk. */
typedef struct {
    korg_synth_inputs in;
    korg_lines lines;   /* this spectrum's (pruned) line list */
    korg_lines lines5;  /* reference-wavelength line list */
    double *flux, *cntm;
} korg_batch_item;
KORG_API int korg_synthesize_batch_dev(korg_ctx *ctx, int32_t nspec, const korg_batch_item *items,
                                       const double *wls, int64_t nwl, int precision, void *stream);
/* Reverse mode of a batch: korg_synthesize_vjp_dev for every spectrum of a batch, as the Fit
 * module's gradient over many atmospheres or abundance sets needs (src/Fit/fit_via_synthesis.jl:
 * 345-355 takes that Jacobian with ForwardDiff through synthesize).  cot[i] holds spectrum i's
 * cotangents (device arrays of nwl; either may be NULL) and its gradient outputs (device
 * pointers, as in korg_synthesize_vjp).  With KORG_VJP_REUSE_FORWARD the previous batch call on
 * the context was korg_synthesize_batch_dev of the same items and ran in one chunk (the default
 * budget holds 256 spectra of 56 x 400,001): every spectrum's opacity, alpha_ref and line
 * prologue are taken from it instead of recomputed, else KORG_EINVAL.  KORG_VJP_HYDROGEN as in
 * korg_synthesize_vjp.  Gradients equal korg_synthesize_vjp_dev's for each spectrum (up to the
 * order of the FP64 atomic additions of the line adjoint). */
typedef struct {
    const double *dflux, *dcntm;
    korg_synth_grads grads;
} korg_batch_vjp_item;
KORG_API int korg_synthesize_batch_vjp_dev(korg_ctx *ctx, int32_t nspec, const korg_batch_item *items,
                                           const korg_batch_vjp_item *cot, const double *wls, int64_t nwl,
                                           int precision, int flags, void *stream);
/* Batch options (no counterpart in the reference).  use_graph: a batch submitted twice in a row
 * with identical items (same pointers and sizes; the contents may change) is captured into a
 * CUDA graph on the second submission and replayed from then on.  autotune: the first large
 * line-opacity launch for a (layer count, precision) times every candidate tile shape on its
 * real inputs and keeps the fastest for the context.  max_scratch_bytes: chunk budget for the
 * batch's alpha and line scratch (0 keeps the current value, 32 GiB by default). */
KORG_API int korg_set_batch_options(korg_ctx *ctx, int use_graph, int autotune,
                                    int64_t max_scratch_bytes);
/* The tile shape the context uses for (L, precision): wavelengths per CTA, lines per shared
 * memory batch, whether each CTA takes a single layer group (split), and whether it came from
 * the autotuner (split and tuned may be NULL).  korg_set_tile_config fixes the shape instead
 * (counts as tuned); KORG_MIXED shapes always take one layer group per CTA (split = 0 is
 * KORG_EINVAL).  No counterpart in the reference. */
KORG_API int korg_get_tile_config(korg_ctx *ctx, int32_t L, int precision, int32_t *tw,
                                  int32_t *stage, int32_t *split, int32_t *tuned);
KORG_API int korg_set_tile_config(korg_ctx *ctx, int32_t L, int precision, int32_t tw,
                                  int32_t stage, int32_t split);

/* Not a counterpart of any reference function: measures the device's sustained FP32
 * (fp64 == 0) or FP64 FMA throughput in TFLOP/s with independent FMA chains, the roofline
 * denominator for the profile (FP32) and transfer (FP64) kernels. */
KORG_API int korg_probe_flops(korg_ctx *ctx, int fp64, double *tflops);

/* Not a counterpart of any reference function: compares the table-driven FP64 exp and log
 * used by the prologue and transfer kernels with the CUDA exp and log on n points; returns the
 * largest exp error in ulps and the largest log error relative to max(1, |log x|). */
KORG_API int korg_math_selftest(korg_ctx *ctx, int64_t n, double *max_ulp_exp, double *max_abs_log);

/* No counterpart in the reference: line_absorption! for callers that cannot allocate device
 * memory -- code running inside a memory pool or arena it does not own, a process whose
 * allocator is locked after start-up, or a caller in the middle of stream capture.  Same
 * arguments and results as korg_line_absorption_dev (device pointers, alpha accumulated in
 * place on `stream`), but no context and no cudaMalloc / cudaFree / allocating library call:
 * all scratch lives in one file-scope device array of KORG_NOALLOC_SCRATCH_BYTES (64 MiB) that
 * every GPU loading the library holds until exit.  That is enough for about 35,000 lines of a
 * 56-layer atmosphere in KORG_MIXED (constants take layers x 32 bytes per line, 48 in
 * KORG_FP64); larger problems return KORG_ETOOBIG without launching anything.
 * The first call in each CUDA context -- the first call on a device, and the first one again
 * after cudaDeviceReset or in another driver-API context -- looks up the array's address and
 * writes lookup tables into it with a synchronous copy: make that first call before any stream
 * capture.  Every call shares
 * the one array (its counters are cleared at the start of each call, the rest is overwritten),
 * so calls whose work overlaps on the GPU -- different streams, or threads without ordering --
 * race; serialise them on one stream. */
#define KORG_NOALLOC_SCRATCH_BYTES (64u << 20)
KORG_API int korg_line_absorption_noalloc(double *alpha, const double *wls, int64_t nwl,
                                          const korg_lines *lines, const korg_layers *layers,
                                          const korg_cntm *cntm, double cutoff_threshold,
                                          int precision, void *stream);

#ifdef __cplusplus
}
#endif
#endif
