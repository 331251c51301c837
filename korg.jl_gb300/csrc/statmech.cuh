// statmech.cuh -- chemical equilibrium on the device: chemical_equilibrium (src/statmech.jl:148-206)
// for every layer of one or many atmospheres, one thread block per layer, FP64.
//
// Unknowns x = (log10 n(X I) for the 92 elements, log10 n_e).  The residuals
// (setup_chemical_equilibrium_residuals, src/statmech.jl:360-439) are nuclei conservation of each
// element, scaled by abundance x n_tot, and charge balance, scaled by n_tot.  The solver is the
// reference's: Newton steps clipped to 1 dex (clipped_newton, src/newton.jl:2-35), and when the
// plain solve fails, a continuation on log xi, the log10 scale of every molecule and H- density
// (_solve_chemical_equilibrium, src/statmech.jl:215-305).
//
// The reference differentiates the residuals with ForwardDiff; here the Jacobian is assembled
// analytically.  With n_mol = 10^(sum of its constituents' x - log nK + log xi) every density is
// an exponential of a linear form in x, so
//   d F_Z / d x_W = ln10 [ sum_mol cnt_Z(mol) cnt_W(mol) n_mol + delta_ZW (n_I + n_II + n_III)_Z
//                          - ab_Z d n_nuclei / d x_W ] / (ab_Z n_tot)
// and similarly for the n_e column and the charge row.  The molecule sums run over a per-element
// incidence list (element -> molecules containing it, with multiplicity) in a fixed order, so a
// layer's result does not depend on thread timing.
//
// Layout: the augmented system [J | F] sits column-major in shared memory (column c at
// A[c * CE_LD + r]).  Gaussian elimination with partial pivoting (largest |entry| in the pivot
// column, lowest row on ties, as LAPACK's getrf) keeps rows in place and a logical-to-physical
// row permutation; the trailing update is spread over all threads; back substitution runs in one
// warp.  The work per Newton step is ~93^3/3 FP64 FMAs; GB300's FP64 pipe makes that the cost
// that bounds the kernel.
//
// Every loop is bounded: at most KORG_CHEM_MAX_ITER Newton iterations per layer in total (the
// reference's own loops are finite but its worst case is ~5e5 iterations); a layer that runs out
// reports KORG_CHEM_BUDGET.
#pragma once
#include <cstdint>

namespace korg {

constexpr int CE_NZ = 92;        // elements H..U
constexpr int CE_N = 93;         // unknowns
constexpr int CE_NCOL = 94;      // columns of the augmented matrix (J and the residuals)
constexpr int CE_LD = 96;        // column stride (rows padded)
constexpr int CE_MAXMOL = 384;
constexpr int CE_THREADS = 128;
constexpr int CE_MAXATOMS = 6;
constexpr int CE_MAX_ITER = 20000;
constexpr int CE_NINFO = 4;

// Device tables (one buffer carved by the host).  The incidence lists are derived on the host.
struct ChemTables {
    int32_t nk;                          // knots of the atomic partition functions
    const double *lnT, *U_u, *U_z;       // [nk], [276][nk] x2
    const double *chi;                   // [92][3]
    int32_t n_mol;
    const int32_t *atoms, *charge, *kind;  // [n_mol][6], [n_mol], [n_mol]
    const int64_t *off;                  // [n_mol + 1]
    const double *t, *u, *z;             // concatenated molecule splines
    const double *D00, *lmr;             // polyatomics
    const int32_t *nat;                  // atoms per molecule, with multiplicity
    const int32_t *ndist, *dist_Z, *dist_cnt;  // distinct atoms [n_mol], [n_mol][6] x2
    const int32_t *inc_ptr, *inc_mol, *inc_cnt;  // element Z-1 -> (molecule, count) at [inc_ptr[Z-1], inc_ptr[Z])
};

struct ChemLayersDev {
    int32_t L;
    const double *T, *n_tot, *ne_model, *ab;  // ab: [n_atm][92]
    const int32_t* atm;                       // [L] or null
};

namespace ce {

constexpr double KB_CGS = 1.380649e-16, H_CGS = 6.62607015e-27, ME_CGS = 9.1093897e-28;
constexpr double KB_EV = 8.617333262145e-5;
constexpr double LN10 = 2.302585092994046;
constexpr double TWO_PI = 6.283185307179586;
constexpr double HMINUS_EA_EV = 0.754204;  // electron affinity of H (McLaughlin+ 2017)

// Korg's natural cubic spline (src/CubicSplines.jl:65-83): knots t, values u, second
// derivatives z; flat outside the knots (only reached for the molecule splines).
__device__ inline double spline(const double* t, const double* u, const double* z, int n, double x) {
    if (!(t[0] <= x && x <= t[n - 1])) return x < t[0] ? u[0] : u[n - 1];
    int lo = 0, hi = n;  // last i with t[i] <= x (searchsortedlast)
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (t[mid] <= x) lo = mid; else hi = mid;
    }
    const int i = lo < n - 2 ? lo : n - 2;
    const double h = t[i + 1] - t[i];
    const double a = t[i + 1] - x, b = x - t[i];
    const double I = z[i] * (a * a * a) / (6 * h) + z[i + 1] * (b * b * b) / (6 * h);
    const double C = (u[i + 1] / h - z[i + 1] * h / 6) * b;
    const double D = (u[i] / h - z[i] * h / 6) * a;
    return I + C + D;
}

__device__ inline double translational_U(double m, double T) {  // src/statmech.jl:47-51
    return pow(TWO_PI * m * KB_CGS * T / (H_CGS * H_CGS), 1.5);
}

// warp arg-max of (value, index): larger value wins, the lower index on ties; index < 0 = none
__device__ inline void warp_argmax(double& v, int& i) {
    for (int o = 16; o; o >>= 1) {
        const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        if (i2 >= 0 && (i < 0 || v2 > v || (v2 == v && i2 < i))) {
            v = v2;
            i = i2;
        }
    }
}

__device__ inline double warp_sum(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace ce

struct CeShared {
    double A[CE_NCOL * CE_LD];
    double x[CE_N], xs[CE_N], x0[CE_N], y[CE_N], rinv[CE_N], sol[CE_N];
    double lwII[CE_NZ], lwIII[CE_NZ], rat1[CE_NZ], rat2[CE_NZ], e1[CE_NZ], e2[CE_NZ];
    double ab[CE_NZ], inv_scale[CE_NZ];
    double nI[CE_NZ], nII[CE_NZ], nIII[CE_NZ];
    double fm[CE_NZ], Sq[CE_NZ], dN[CE_N], F[CE_N];
    double lognK[CE_MAXMOL], nmol[CE_MAXMOL];
    double candv[4];
    double red[4];
    double ne, nHm, nn_mol, qn, dNe_mol, ion1, ion2, pinv, lognK_Hm, transU, lnT;
    int candi[4];
    int perm[CE_N];
    int prow, flag;
};

// One Newton solve at log xi from s.x (clipped_newton, src/newton.jl:2-35).  Every thread calls
// it; control flow is uniform.  Returns whether |F|_inf < tol was reached; budget counts the
// iterations left for the layer (exhausted: *out_of_budget is set).
__device__ bool ce_newton(const ChemTables& tb, CeShared& s, double nt, double logxi, int max_iter, int& budget,
                          bool& out_of_budget, double& last_inf) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int M = tb.n_mol;
    last_inf = INFINITY;
    for (int it = 0; it < max_iter; ++it) {
        if (budget <= 0) {
            out_of_budget = true;
            return false;
        }
        --budget;
        // densities of every species at x (src/statmech.jl:385-430)
        const double xe = s.x[CE_NZ];
        for (int m = tid; m < M; m += CE_THREADS) {
            const int* at = tb.atoms + m * CE_MAXATOMS;
            double lg = -s.lognK[m] + logxi;
            if (tb.charge[m] == 0) {
                for (int j = 0; j < CE_MAXATOMS && at[j]; ++j) lg += s.x[at[j] - 1];
            } else {
                const int Z1 = at[0] - 1, Z2 = at[1] - 1;
                lg += ((s.x[Z1] + s.lwII[Z1]) - xe) + s.x[Z2];
            }
            s.nmol[m] = exp10(lg);
        }
        for (int Z = tid; Z < CE_NZ; Z += CE_THREADS) {
            const double xz = s.x[Z];
            s.nI[Z] = exp10(xz);
            s.nII[Z] = exp10((xz + s.lwII[Z]) - xe);
            s.nIII[Z] = exp10((xz + s.lwIII[Z]) - 2 * xe);
        }
        if (tid == 0) {
            s.ne = exp10(xe);
            s.nHm = exp10(((s.lognK_Hm + s.x[0]) + xe) + logxi);
        }
        __syncthreads();
        // per-element molecule sums (fixed order) and the block-wide sums (warp 3)
        if (tid < CE_NZ) {
            double fm = 0, dn = 0, sq = 0;
            for (int k = tb.inc_ptr[tid]; k < tb.inc_ptr[tid + 1]; ++k) {
                const int m = tb.inc_mol[k];
                const double cn = double(tb.inc_cnt[k]) * s.nmol[m];
                fm += cn;
                dn += double(tb.nat[m] - 1) * cn;
                if (tb.charge[m]) sq += cn;
            }
            s.fm[tid] = fm;
            s.dN[tid] = ce::LN10 * dn;
            s.Sq[tid] = sq;
        } else if (warp == 3) {
            double nn = 0, qn = 0, dq = 0, i1 = 0, i2 = 0;
            for (int m = lane; m < M; m += 32) {
                const double n = s.nmol[m];
                nn += double(tb.nat[m] - 1) * n;
                if (tb.charge[m]) {
                    qn += n;
                    dq += double(tb.nat[m] - 1) * n;
                }
            }
            for (int Z = lane; Z < CE_NZ; Z += 32) {
                i1 += s.nII[Z] + 2 * s.nIII[Z];
                i2 += s.nII[Z] + 4 * s.nIII[Z];
            }
            nn = ce::warp_sum(nn);
            qn = ce::warp_sum(qn);
            dq = ce::warp_sum(dq);
            i1 = ce::warp_sum(i1);
            i2 = ce::warp_sum(i2);
            if (lane == 0) {
                s.nn_mol = nn;
                s.qn = qn;
                s.dNe_mol = dq;
                s.ion1 = i1;
                s.ion2 = i2;
            }
        }
        __syncthreads();
        // scaled residuals and their inf-norm (src/statmech.jl:418-438, newton.jl:8-14)
        double fabs_max = 0;
        bool bad = false;
        if (tid < CE_N) {
            double F;
            if (tid < CE_NZ) {
                const double n_nuclei = (nt - s.ne) + s.nn_mol;
                double f = s.fm[tid];
                if (tid == 0) f += s.nHm;
                f += ((s.nI[tid] + s.nII[tid]) + s.nIII[tid]) - s.ab[tid] * n_nuclei;
                F = f / (s.ab[tid] * nt);
            } else {
                F = (((s.qn - s.nHm) + s.ion1) - s.ne) / nt;
            }
            s.F[tid] = F;
            bad = !isfinite(F);
            fabs_max = fabs(F);
        }
        for (int o = 16; o; o >>= 1) fabs_max = fmax(fabs_max, __shfl_xor_sync(0xffffffffu, fabs_max, o));
        if (lane == 0) s.red[warp] = fabs_max;
        if (__syncthreads_or(bad)) return false;
        const double inf = fmax(fmax(s.red[0], s.red[1]), fmax(s.red[2], s.red[3]));
        last_inf = inf;
        if (inf < 1e-8) return true;
        // Jacobian, dense part: n_nuclei coupling, the atoms' own densities, the n_e column, the
        // charge row; residuals in column CE_N
        const double ln10 = ce::LN10;
        const double dNe = -ln10 * s.ne - ln10 * s.dNe_mol;
        const double inv_nt = 1.0 / nt;
        bool badJ = false;
        for (int idx = tid; idx < CE_N * CE_NCOL; idx += CE_THREADS) {
            const int r = idx % CE_N, c = idx / CE_N;
            double v;
            if (c == CE_N) {
                v = s.F[r];
            } else if (r < CE_NZ) {
                v = -s.ab[r] * (c < CE_NZ ? s.dN[c] : dNe);
                if (c == r) v += ln10 * ((s.nI[r] + s.nII[r]) + s.nIII[r]);
                if (c == CE_NZ) v += -ln10 * s.Sq[r] - ln10 * (s.nII[r] + 2 * s.nIII[r]);
                if (r == 0 && (c == 0 || c == CE_NZ)) v += ln10 * s.nHm;
                v *= s.inv_scale[r];
            } else if (c < CE_NZ) {
                v = ln10 * s.Sq[c] + ln10 * (s.nII[c] + 2 * s.nIII[c]);
                if (c == 0) v -= ln10 * s.nHm;
                v *= inv_nt;
            } else {
                v = (((-ln10 * s.qn) - ln10 * s.nHm) - ln10 * s.ion2 - ln10 * s.ne) * inv_nt;
            }
            s.A[c * CE_LD + r] = v;
        }
        __syncthreads();
        // Jacobian, molecule coupling: row Z gains ln10 cnt_Z cnt_W n_mol / (ab_Z n_tot) at W
        if (tid < CE_NZ) {
            const double sc = ln10 * s.inv_scale[tid];
            for (int k = tb.inc_ptr[tid]; k < tb.inc_ptr[tid + 1]; ++k) {
                const int m = tb.inc_mol[k];
                const double w = sc * double(tb.inc_cnt[k]) * s.nmol[m];
                for (int d = 0; d < tb.ndist[m]; ++d) {
                    const int W = tb.dist_Z[m * CE_MAXATOMS + d] - 1;
                    s.A[W * CE_LD + tid] += w * double(tb.dist_cnt[m * CE_MAXATOMS + d]);
                }
            }
            for (int c = 0; c < CE_N; ++c) badJ |= !isfinite(s.A[c * CE_LD + tid]);
        } else if (tid == CE_NZ) {
            for (int c = 0; c < CE_N; ++c) badJ |= !isfinite(s.A[c * CE_LD + tid]);
        }
        if (tid < CE_N) s.perm[tid] = tid;
        if (__syncthreads_or(badJ)) return false;
        // LU with partial pivoting of the augmented system (J \ F, as LAPACK getrf + getrs)
        {
            double v = -1;
            int i = -1;
            if (tid < CE_N) {
                v = fabs(s.A[tid]);
                i = tid;
            }
            ce::warp_argmax(v, i);
            if (lane == 0) {
                s.candv[warp] = v;
                s.candi[warp] = i;
            }
        }
        __syncthreads();
        bool singular = false;
        for (int k = 0; k < CE_N; ++k) {
            if (tid == 0) {
                double bv = -1;
                int bi = -1;
                for (int w = 0; w < 4; ++w) {
                    const int i2 = s.candi[w];
                    const double v2 = s.candv[w];
                    if (i2 >= 0 && (bi < 0 || v2 > bv || (v2 == bv && i2 < bi))) {
                        bv = v2;
                        bi = i2;
                    }
                }
                int fl = 0;
                if (bi < 0 || !(bv > 0)) {
                    fl = 1;
                } else {
                    const int pr = s.perm[bi];
                    s.perm[bi] = s.perm[k];
                    s.perm[k] = pr;
                    s.prow = pr;
                    s.pinv = 1.0 / s.A[k * CE_LD + pr];
                }
                s.flag = fl;
            }
            __syncthreads();
            if (s.flag) {
                singular = true;
                break;
            }
            if (k == CE_N - 1) break;
            const int prow = s.prow;
            const double pinv = s.pinv;
            for (int i = k + 1 + tid; i < CE_N; i += CE_THREADS) s.A[k * CE_LD + s.perm[i]] *= pinv;
            __syncthreads();
            const int nrow = CE_N - 1 - k, ncol = CE_NCOL - 1 - k;
            double cv = -1;
            int ci = -1;
            for (int idx = tid; idx < nrow * ncol; idx += CE_THREADS) {
                const int ii = idx % nrow, cc = idx / nrow;
                const int i = k + 1 + ii, c = k + 1 + cc;
                const int r = s.perm[i];
                const double v = fma(-s.A[k * CE_LD + r], s.A[c * CE_LD + prow], s.A[c * CE_LD + r]);
                s.A[c * CE_LD + r] = v;
                if (cc == 0) {
                    cv = fabs(v);
                    ci = i;
                }
            }
            ce::warp_argmax(cv, ci);
            if (lane == 0) {
                s.candv[warp] = cv;
                s.candi[warp] = ci;
            }
            __syncthreads();
        }
        if (singular) return false;
        // back substitution in one warp: x_j = y_j / U_jj, y_i -= U_ij x_j
        if (warp == 0) {
            for (int i = lane; i < CE_N; i += 32) {
                const int r = s.perm[i];
                s.y[i] = s.A[CE_N * CE_LD + r];
                s.rinv[i] = 1.0 / s.A[i * CE_LD + r];
            }
            __syncwarp();
            for (int j = CE_N - 1; j >= 0; --j) {
                const double xj = s.y[j] * s.rinv[j];
                if (lane == 0) s.sol[j] = xj;
                for (int i = lane; i < j; i += 32) s.y[i] = fma(-s.A[j * CE_LD + s.perm[i]], xj, s.y[i]);
                __syncwarp();
            }
        }
        __syncthreads();
        // step = -(J \ F), clipped so that no unknown moves more than 1 dex
        double smax = 0;
        bool badS = false;
        if (tid < CE_N) {
            const double st = -s.sol[tid];
            badS = !isfinite(st);
            smax = fabs(st);
        }
        for (int o = 16; o; o >>= 1) smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, o));
        if (lane == 0) s.red[warp] = smax;
        if (__syncthreads_or(badS)) return false;
        const double sm = fmax(fmax(s.red[0], s.red[1]), fmax(s.red[2], s.red[3]));
        const double alpha = sm > 1.0 ? 1.0 / sm : 1.0;
        if (tid < CE_N) s.x[tid] = s.x[tid] + alpha * (-s.sol[tid]);
        __syncthreads();
    }
    return false;
}

__global__ void __launch_bounds__(CE_THREADS) chem_eq_kernel(ChemTables tb, ChemLayersDev ly, double* __restrict__ dens,
                                                             int32_t* __restrict__ status, double* __restrict__ info) {
    extern __shared__ __align__(16) unsigned char ce_smem[];
    CeShared& s = *reinterpret_cast<CeShared*>(ce_smem);
    const int l = blockIdx.x;
    if (l >= ly.L) return;
    const int tid = threadIdx.x;
    const int M = tb.n_mol;
    const int nspec = 278 + M;
    const double T = ly.T[l], nt = ly.n_tot[l], ne_g = ly.ne_model[l];
    const int a = ly.atm ? ly.atm[l] : 0;
    const double lnT = log(T);
    const double transU = ce::translational_U(ce::ME_CGS, T);
    // per-layer constants: Saha factors (saha_ion_weights with n_e = 1, src/statmech.jl:19-35,
    // 362-372), the starting guess (atoms only, n_e from the model atmosphere, :151-155, 235-237),
    // molecular log nK (get_log_nK, :60-62; polyatomics read_statmech_quantities.jl:66-89)
    for (int Z = tid; Z < CE_NZ; Z += CE_THREADS) {
        const double* U = tb.U_u + size_t(3 * Z) * tb.nk;
        const double* Uz = tb.U_z + size_t(3 * Z) * tb.nk;
        const double UI = ce::spline(tb.lnT, U, Uz, tb.nk, lnT);
        const double UII = ce::spline(tb.lnT, U + tb.nk, Uz + tb.nk, tb.nk, lnT);
        const double chiI = tb.chi[3 * Z], chiII = tb.chi[3 * Z + 1];
        const double e1 = exp(-chiI / (ce::KB_EV * T));
        const double r1 = UII / UI;
        const double wII1 = 2.0 * r1 * transU * e1;
        const double wIIg = 2.0 / ne_g * r1 * transU * e1;
        double r2 = 0, e2 = 0, wIII1 = 0, wIIIg = 0;
        if (Z > 0) {
            const double UIII = ce::spline(tb.lnT, U + 2 * tb.nk, Uz + 2 * tb.nk, tb.nk, lnT);
            r2 = UIII / UII;
            e2 = exp(-chiII / (ce::KB_EV * T));
            wIII1 = wII1 * 2.0 * r2 * transU * e2;
            wIIIg = wIIg * 2.0 / ne_g * r2 * transU * e2;
        }
        s.rat1[Z] = r1;
        s.rat2[Z] = r2;
        s.e1[Z] = e1;
        s.e2[Z] = e2;
        s.lwII[Z] = log10(wII1);
        s.lwIII[Z] = Z > 0 ? log10(wIII1) : -INFINITY;
        const double abZ = ly.ab[size_t(a) * CE_NZ + Z];
        s.ab[Z] = abZ;
        s.inv_scale[Z] = 1.0 / (abZ * nt);
        s.x0[Z] = log10((nt - ne_g) * abZ * (1 / (1 + wIIg + wIIIg)));
    }
    for (int m = tid; m < M; m += CE_THREADS) {
        const int64_t o = tb.off[m];
        const int n = int(tb.off[m + 1] - o);
        const int na = tb.nat[m];
        double logK;
        if (tb.kind[m] == 0) {
            logK = ce::spline(tb.t + o, tb.u + o, tb.z + o, n, lnT);
        } else {
            const double Tp = exp(lnT);
            double prodU = 1.0;
            for (int j = 0; j < CE_MAXATOMS && tb.atoms[m * CE_MAXATOMS + j]; ++j) {
                const int Z = tb.atoms[m * CE_MAXATOMS + j] - 1;
                prodU *= ce::spline(tb.lnT, tb.U_u + size_t(3 * Z) * tb.nk, tb.U_z + size_t(3 * Z) * tb.nk, tb.nk, lnT);
            }
            const double log_Us = log10(prodU / ce::spline(tb.t + o, tb.u + o, tb.z + o, n, lnT));
            const double ltU = 1.5 * log10(ce::TWO_PI * ce::KB_CGS * Tp / (ce::H_CGS * ce::H_CGS));
            const double lnK = double(na - 1) * ltU + 1.5 * tb.lmr[m] + log_Us - tb.D00[m] / (ce::KB_EV * Tp * log(10.0));
            logK = lnK + double(na - 1) * log10(ce::KB_CGS * Tp);
        }
        s.lognK[m] = logK - double(na - 1) * log10(ce::KB_CGS * T);
    }
    if (tid == 0) {
        s.x0[CE_NZ] = log10(ne_g);
        s.lognK_Hm = log10(exp(ce::HMINUS_EA_EV / (ce::KB_EV * T)) / (4 * transU));
        s.transU = transU;
        s.lnT = lnT;
    }
    __syncthreads();
    // the solve (src/statmech.jl:240-305)
    int budget = CE_MAX_ITER;
    bool oob = false;
    double last_inf = INFINITY;
    int solves = 0, st = KORG_CHEM_OK;
    double logxi = 0.0;
    if (tid < CE_N) s.x[tid] = s.x0[tid];
    __syncthreads();
    ++solves;
    bool conv = ce_newton(tb, s, nt, 0.0, 50, budget, oob, last_inf);
    if (!conv && !oob) {
        const double anchors[3] = {-5.0, -20.0, -50.0};
        bool anchored = false;
        for (int q = 0; q < 3 && !anchored && !oob; ++q) {
            if (tid < CE_N) s.x[tid] = s.x0[tid];
            __syncthreads();
            ++solves;
            anchored = ce_newton(tb, s, nt, anchors[q], 100, budget, oob, last_inf);
            if (anchored) logxi = anchors[q];
        }
        if (!anchored) {
            st = oob ? KORG_CHEM_BUDGET : KORG_CHEM_ANCHOR;
        } else {
            const double dinit = 2.0;
            double dlx = dinit;
            if (tid < CE_N) s.xs[tid] = s.x[tid];
            __syncthreads();
            while (logxi < -1e-12) {
                double step = fmin(dlx, 0 - logxi);
                if (tid < CE_N) s.x[tid] = s.xs[tid];
                __syncthreads();
                ++solves;
                bool c2 = ce_newton(tb, s, nt, logxi + step, 100, budget, oob, last_inf);
                if (!c2) {
                    step /= 2;
                    while (!c2 && step >= 0.0625 && !oob) {
                        if (tid < CE_N) s.x[tid] = s.xs[tid];
                        __syncthreads();
                        ++solves;
                        c2 = ce_newton(tb, s, nt, logxi + step, 100, budget, oob, last_inf);
                        if (!c2) step /= 2;
                    }
                    if (!c2) {
                        st = oob ? KORG_CHEM_BUDGET : KORG_CHEM_ANNEAL;
                        logxi += 2 * step;
                        break;
                    }
                    dlx = step;
                } else {
                    dlx = fmin(dinit, 2 * step);
                }
                if (tid < CE_N) s.xs[tid] = s.x[tid];
                __syncthreads();
                logxi += step;
            }
        }
    } else if (oob) {
        st = KORG_CHEM_BUDGET;
    }
    if (st == KORG_CHEM_OK) {
        bool bad = false;
        if (tid < CE_N) bad = !isfinite(s.x[tid]);
        if (__syncthreads_or(bad)) st = KORG_CHEM_NONFINITE;
    }
    // number densities from the solution (src/statmech.jl:160-205)
    double* out = dens + size_t(l) * nspec;
    const double ne = exp10(s.x[CE_NZ]);
    for (int Z = tid; Z < CE_NZ; Z += CE_THREADS) {
        const double nI = exp10(s.x[Z]);
        const double wII = 2.0 / ne * s.rat1[Z] * s.transU * s.e1[Z];
        const double wIII = Z > 0 ? wII * 2.0 / ne * s.rat2[Z] * s.transU * s.e2[Z] : 0.0;
        out[1 + 3 * Z] = nI;
        out[2 + 3 * Z] = wII * nI;
        out[3 + 3 * Z] = wIII * nI;
        s.nI[Z] = nI;
        s.nII[Z] = wII * nI;
    }
    __syncthreads();
    if (tid == 0) {
        out[0] = ne;
        out[277] = exp(ce::HMINUS_EA_EV / (ce::KB_EV * T)) / (4 * s.transU) * s.nI[0] * ne;
    }
    for (int m = tid; m < M; m += CE_THREADS) {
        const int* at = tb.atoms + m * CE_MAXATOMS;
        double sum;
        if (tb.charge[m] == 0) {
            sum = 0;
            for (int j = 0; j < CE_MAXATOMS && at[j]; ++j) sum += log10(s.nI[at[j] - 1]);
        } else {
            sum = log10(s.nII[at[0] - 1]) + log10(s.nI[at[1] - 1]);
        }
        out[278 + m] = exp10(sum - s.lognK[m]);
    }
    if (tid == 0) {
        status[l] = st;
        if (info) {
            info[CE_NINFO * l + 0] = double(CE_MAX_ITER - budget);
            info[CE_NINFO * l + 1] = double(solves);
            info[CE_NINFO * l + 2] = logxi;
            info[CE_NINFO * l + 3] = last_inf;
        }
    }
}

}  // namespace korg
