// statmech.cuh -- chemical equilibrium on the device: chemical_equilibrium (src/statmech.jl:148-206)
// for every layer of one or many atmospheres, one thread block per layer.
//
// Unknowns x = (log10 n(X I) for the 92 elements, log10 n_e).  The residuals
// (setup_chemical_equilibrium_residuals, src/statmech.jl:360-439) are nuclei conservation of each
// element, scaled by abundance x n_tot, and charge balance, scaled by n_tot.  The solver is the
// reference's: Newton steps clipped to 1 dex (clipped_newton, src/newton.jl:2-35), and when the
// plain solve fails, a continuation on log xi, the log10 scale of every molecule and H- density
// (_solve_chemical_equilibrium, src/statmech.jl:215-305).
//
// Jacobian.  The reference differentiates the residuals with ForwardDiff; here the Jacobian is
// assembled analytically.  With n_mol = 10^(sum of its constituents' x - log nK + log xi) every
// density is an exponential of a linear form in x, so
//   d F_Z / d x_W = ln10 [ sum_mol cnt_Z(mol) cnt_W(mol) n_mol + delta_ZW (n_I + n_II + n_III)_Z
//                          - ab_Z d n_nuclei / d x_W ] / (ab_Z n_tot)
// and similarly for the n_e column and the charge row.  The molecule sums run over fixed lists
// (element -> molecules containing it; (row, column) pair -> molecules containing both), one
// thread per list, so a layer's result does not depend on thread timing.
//
// Newton step J s = F.  The system is assembled in FP64 (column-major in shared memory) and
// equilibrated with exact powers of two (rows, then columns, scaled to a largest entry in [1, 2)):
// the condition number of the equilibrated Jacobian at stellar solutions is ~10^2, against up to
// 10^12 unscaled.  The equilibrated matrix is factorised in FP32 (GB300 runs FP32 FMAs at 64x the
// FP64 rate) with partial pivoting, and the FP64 solution is recovered by iterative refinement
// as LAPACK's dsgesv does it: residuals F - J s in FP64, corrections from the FP32 factors, until
// the equilibrated residual is at the level of a backward-stable FP64 solve.  The refined step
// is then as accurate as an FP64 elimination (equal to it up to the conditioning of the system).
// When the refinement stops contracting (an ill-conditioned start of a continuation) or the FP32
// factorisation meets a zero pivot, the same elimination runs in FP64 on the FP64 matrix, as
// LAPACK's getrf + getrs would.
//
// Elimination: partial pivoting (largest |entry| of the pivot column, lowest row on ties) with
// rows left in place and a double-buffered logical-to-physical row permutation; one barrier per
// column (warps over columns, lanes over rows; multipliers written back one column late); warp
// 0, which updates the next pivot column, also picks the next pivot.  Triangular solves run in
// one warp with the vector in registers.
//
// Every loop is bounded: at most KORG_CHEM_MAX_ITER Newton iterations per layer in total (the
// reference's own loops are finite but its worst case is ~5e5 iterations); a layer that runs out
// reports KORG_CHEM_BUDGET.
#pragma once
#include <cstdint>

namespace korg {

constexpr int CE_NZ = 92;        // elements H..U
constexpr int CE_N = 93;         // unknowns
constexpr int CE_NCOL = 94;      // columns of the FP64 system (J and the residuals)
constexpr int CE_LD = 96;        // column stride (rows padded)
constexpr int CE_MAXMOL = 384;
constexpr int CE_THREADS = 256;
constexpr int CE_WARPS = CE_THREADS / 32;
constexpr int CE_MAXATOMS = 6;
constexpr int CE_MAX_ITER = 20000;
constexpr int CE_NINFO = 5;
constexpr int CE_REFINE_MAX = 8;
constexpr int CE_MAXINC = 1024;    // element -> molecule incidences
constexpr int CE_MAXPAIR = 1024;   // (Z, W), Z != W, pairs sharing a molecule
constexpr int CE_MAXPENT = 1024;   // molecule entries of the pair lists
constexpr int CE_CHUNK = 8;        // incidences per work item of the element sums
constexpr int CE_MAXITEM = 224;    // work items (threads of warps 0-6)

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
    const int32_t *inc_ptr, *inc_mol, *inc_cnt;  // element Z-1 -> (molecule, count) at [inc_ptr[Z-1], inc_ptr[Z])
    int32_t n_items;                     // element sums split in items of <= CE_CHUNK incidences
    const int32_t *item_elem, *item_begin, *elem_item_ptr;  // item i covers [item_begin[i], item_begin[i + 1])
    int32_t n_pairs;                     // (Z, W), Z != W, with a molecule containing both
    const int32_t *pair_row, *pair_col, *pair_ptr, *pair_mol, *pair_coef;  // coef = cnt_Z * cnt_W
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

// d/dx of the same spline (zero outside the knots, where it is flat)
__device__ inline double spline_deriv(const double* t, const double* u, const double* z, int n, double x) {
    if (!(t[0] <= x && x <= t[n - 1])) return 0.0;
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (t[mid] <= x) lo = mid; else hi = mid;
    }
    const int i = lo < n - 2 ? lo : n - 2;
    const double h = t[i + 1] - t[i];
    const double a = t[i + 1] - x, b = x - t[i];
    return -z[i] * (a * a) / (2 * h) + z[i + 1] * (b * b) / (2 * h) + (u[i + 1] / h - z[i + 1] * h / 6) -
           (u[i] / h - z[i] * h / 6);
}

__device__ inline double translational_U(double m, double T) {  // src/statmech.jl:47-51
    return pow(TWO_PI * m * KB_CGS * T / (H_CGS * H_CGS), 1.5);
}

// warp arg-max of (value, index): larger value wins, the lower index on ties; index < 0 = none
template <typename T>
__device__ inline void warp_argmax(T& v, int& i) {
    for (int o = 16; o; o >>= 1) {
        const T v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        if (i2 >= 0 && (i < 0 || v2 > v || (v2 == v && i2 < i))) {
            v = v2;
            i = i2;
        }
    }
}

// the same, carrying the signed value of the winning entry
template <typename T>
__device__ inline void warp_argmax_signed(T& v, T& sv, int& i) {
    for (int o = 16; o; o >>= 1) {
        const T v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const T s2 = __shfl_xor_sync(0xffffffffu, sv, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        if (i2 >= 0 && (i < 0 || v2 > v || (v2 == v && i2 < i))) {
            v = v2;
            sv = s2;
            i = i2;
        }
    }
}

__device__ inline double warp_sum(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ inline long long warp_max_ll(long long v) {
    for (int o = 16; o; o >>= 1) v = max(v, (long long)__shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// |v| as its IEEE bit pattern: for finite doubles the order of the patterns is the order of |v|
__device__ inline long long abits(double v) { return __double_as_longlong(v) & 0x7fffffffffffffffLL; }

// v * 2^-e rounded to FP32 with integer operations (v finite; results below FP32's normal range
// flush to zero, above it saturate to the largest float)
__device__ inline float scaled_to_float(double v, int e) {
    const long long b = __double_as_longlong(v);
    const long long a = b & 0x7fffffffffffffffLL;
    if (a == 0) return 0.0f;
    const int ex = int(a >> 52) - 1023 - e;  // unbiased exponent of the scaled value
    if (ex < -126) return 0.0f;
    const unsigned sign = unsigned((unsigned long long)b >> 32) & 0x80000000u;
    if (ex > 127) return __uint_as_float(sign | 0x7f7fffffu);
    const unsigned long long mant = (unsigned long long)(a & 0xfffffffffffffULL);
    unsigned fb = (unsigned(ex + 127) << 23) + unsigned((mant + (1ULL << 28)) >> 29);  // carry rounds up the exponent
    return __uint_as_float(sign | fb);
}

}  // namespace ce

struct CeShared {
    double A[CE_NCOL * CE_LD];  // FP64 [J | F], column-major
    float B[CE_N * CE_LD];      // FP32 equilibrated J, then its LU factors
    double x[CE_N], xs[CE_N], x0[CE_N], sol[CE_N], res[CE_N];
    double lwII[CE_NZ], lwIII[CE_NZ], rat1[CE_NZ], rat2[CE_NZ], e1[CE_NZ], e2[CE_NZ];
    double ab[CE_NZ], inv_scale[CE_NZ];
    double nI[CE_NZ], nII[CE_NZ], nIII[CE_NZ];
    double fm[CE_NZ], Sq[CE_NZ], dd[CE_NZ], dNn[CE_N];
    double part[CE_MAXITEM][4];  // per-item partial sums: cnt n, cnt (nat-1) n, cnt q n, cnt^2 n
    double lognK[CE_MAXMOL], nmol[CE_MAXMOL];
    double dlognK[CE_MAXMOL], wmol[CE_MAXMOL], dlwII[CE_NZ], dlwIII[CE_NZ];  // reverse mode
    double uinv64[CE_N];
    float uinv32[CE_N], vec32[CE_N];
    double red[CE_WARPS], red2[CE_WARPS];
    long long redl[4][CE_WARPS];
    double ne, nHm, nn_mol, qn, dNe_mol, ion1, ion2, lognK_Hm, transU, lnT, dlognK_Hm;
    double vsum[3];
    double piv64[2];
    float piv32[2];
    int perm[2][CE_LD];
    // the molecule tables, copied from global memory once per layer
    unsigned char m_atoms[CE_MAXMOL * CE_MAXATOMS], m_charge[CE_MAXMOL], m_nat[CE_MAXMOL];
    double inc_cntd[CE_MAXINC], natm1[CE_MAXMOL], chg[CE_MAXMOL], pair_coefd[CE_MAXPENT];
    short inc_ptr[CE_NZ + 1], inc_mol[CE_MAXINC];
    short item_begin[CE_MAXITEM + 1], elem_item_ptr[CE_NZ + 1];
    unsigned char pair_row[CE_MAXPAIR], pair_col[CE_MAXPAIR];
    short pair_ptr[CE_MAXPAIR + 1], pair_mol[CE_MAXPENT];
    int rexp[CE_N], cexp[CE_N];
    int pivi[2];
};

// block-wide max of a non-negative value (every thread gets it); two barriers
__device__ inline double ce_block_max(CeShared& s, double v) {
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) s.red[threadIdx.x >> 5] = v;
    __syncthreads();
    double m = s.red[0];
    for (int w = 1; w < CE_WARPS; ++w) m = fmax(m, s.red[w]);
    __syncthreads();
    return m;
}

// LU factorisation with partial pivoting of the n x n column-major matrix M (stride CE_LD, rows
// left in place): multipliers below the diagonal, U on and above it in logical row order; the
// final logical-to-physical permutation in s.perm[(CE_N - 1) & 1]; uinv = reciprocals of U's
// diagonal.  Returns false on a zero (or non-finite) pivot.  T = float or double.
//
// One barrier per column: every warp derives the multipliers of its rows from the pivot column
// (read-only during the step) and updates its columns of the trailing matrix; warp 0, whose first
// column is the next pivot column, also picks the next pivot, and writes this step's multipliers
// into the pivot column during the next step, when nothing reads it any more.
template <typename T>
__device__ bool ce_lu(CeShared& s, T* M, T* uinv) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // pivot slots, double-buffered by step parity (read at a step's start, the next one written
    // by warp 0 during the step)
    T* piv = reinterpret_cast<T*>(sizeof(T) == 4 ? (void*)s.piv32 : (void*)s.piv64);
    if (tid < CE_N) s.perm[0][tid] = tid;
    if (warp == 0) {  // first pivot: column 0
        T v = T(-1), sv = 0;
        int bi = -1;
        for (int i = lane; i < CE_N; i += 32)
            if (bi < 0 || fabs(M[i]) > v) {
                v = fabs(M[i]);
                sv = M[i];
                bi = i;
            }
        ce::warp_argmax_signed(v, sv, bi);
        if (lane == 0) {
            s.pivi[0] = bi;
            piv[0] = sv;
        }
    }
    __syncthreads();
    bool ok = true;
    int pr0 = -1, pr1 = -1, pr2 = -1;  // rows and multipliers of the previous step (warp 0 writes them)
    T pl0 = 0, pl1 = 0, pl2 = 0;
    for (int k = 0; k < CE_N; ++k) {
        const int* PR = s.perm[k & 1];
        int* PW = s.perm[(k + 1) & 1];
        const int p = s.pivi[k & 1];
        const T pv = piv[k & 1];
        if (p < 0 || !(fabs(pv) > T(0)) || !isfinite(pv)) {
            ok = false;
            break;
        }
        const int pr = PR[p];
        const T pinv = T(1) / pv;
        if (tid == 0) uinv[k] = pinv;
        if (warp == 0 && k > 0) {  // the previous step's multipliers into its pivot column
            T* colp = M + (k - 1) * CE_LD;
            if (pr0 >= 0) colp[pr0] = pl0;
            if (pr1 >= 0) colp[pr1] = pl1;
            if (pr2 >= 0) colp[pr2] = pl2;
        }
        if (k == CE_N - 1) break;
        if (tid < CE_N) {  // permutation of the next step: logical rows k and p exchange
            const int i = tid;
            PW[i] = i == k ? pr : (i == p ? PR[k] : PR[i]);
        }
        // this lane's rows (logical k+1+lane, +32, +64) and their multipliers
        const int i0 = k + 1 + lane, i1 = i0 + 32, i2 = i0 + 64;
        const T* colk = M + k * CE_LD;
        int r0 = -1, r1 = -1, r2 = -1;
        T l0 = 0, l1 = 0, l2 = 0;
        if (i0 < CE_N) { r0 = i0 == p ? PR[k] : PR[i0]; l0 = colk[r0] * pinv; }
        if (i1 < CE_N) { r1 = i1 == p ? PR[k] : PR[i1]; l1 = colk[r1] * pinv; }
        if (i2 < CE_N) { r2 = i2 == p ? PR[k] : PR[i2]; l2 = colk[r2] * pinv; }
        // trailing update, two columns at a time (loads first, then stores, for overlap)
        int c = k + 1 + warp;
        if (c == k + 1) {  // warp 0: the next pivot column first
            T* col = M + c * CE_LD;
            const T u = col[pr];
            T a0 = 0, a1 = 0, a2 = 0;
            if (r0 >= 0) a0 = fma(-l0, u, col[r0]);
            if (r1 >= 0) a1 = fma(-l1, u, col[r1]);
            if (r2 >= 0) a2 = fma(-l2, u, col[r2]);
            if (r0 >= 0) col[r0] = a0;
            if (r1 >= 0) col[r1] = a1;
            if (r2 >= 0) col[r2] = a2;
            T v = T(-1), sv = 0;
            int bi = -1;
            if (r0 >= 0) { v = fabs(a0); sv = a0; bi = i0; }
            if (r1 >= 0 && fabs(a1) > v) { v = fabs(a1); sv = a1; bi = i1; }
            if (r2 >= 0 && fabs(a2) > v) { v = fabs(a2); sv = a2; bi = i2; }
            ce::warp_argmax_signed(v, sv, bi);
            if (lane == 0) {
                s.pivi[(k + 1) & 1] = bi;
                piv[(k + 1) & 1] = sv;
            }
            c += CE_WARPS;
        }
        for (; c + CE_WARPS < CE_N; c += 2 * CE_WARPS) {
            T* ca = M + c * CE_LD;
            T* cb = ca + CE_WARPS * CE_LD;
            const T ua = ca[pr], ub = cb[pr];
            T a0 = 0, a1 = 0, a2 = 0, b0 = 0, b1 = 0, b2 = 0;
            if (r0 >= 0) { a0 = ca[r0]; b0 = cb[r0]; }
            if (r1 >= 0) { a1 = ca[r1]; b1 = cb[r1]; }
            if (r2 >= 0) { a2 = ca[r2]; b2 = cb[r2]; }
            if (r0 >= 0) { ca[r0] = fma(-l0, ua, a0); cb[r0] = fma(-l0, ub, b0); }
            if (r1 >= 0) { ca[r1] = fma(-l1, ua, a1); cb[r1] = fma(-l1, ub, b1); }
            if (r2 >= 0) { ca[r2] = fma(-l2, ua, a2); cb[r2] = fma(-l2, ub, b2); }
        }
        if (c < CE_N) {
            T* col = M + c * CE_LD;
            const T u = col[pr];
            T a0 = 0, a1 = 0, a2 = 0;
            if (r0 >= 0) a0 = col[r0];
            if (r1 >= 0) a1 = col[r1];
            if (r2 >= 0) a2 = col[r2];
            if (r0 >= 0) col[r0] = fma(-l0, u, a0);
            if (r1 >= 0) col[r1] = fma(-l1, u, a1);
            if (r2 >= 0) col[r2] = fma(-l2, u, a2);
        }
        pr0 = r0; pr1 = r1; pr2 = r2;
        pl0 = l0; pl1 = l1; pl2 = l2;
        __syncthreads();
    }
    __syncthreads();
    return ok;
}

// Solve L U x = P b in one warp (warp 0): b in physical row order, x in column order; M, the
// permutation P (logical -> physical row) and uinv from the factorisation.  Other warps return
// at once.
template <typename T>
__device__ void ce_trisolve(const int* P, const T* M, const T* uinv, const T* b, T* x) {
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid >= 32) return;
    const int i0 = lane, i1 = lane + 32, i2 = lane + 64;
    const bool v2 = i2 < CE_N;
    const int r0 = P[i0], r1 = P[i1], r2 = v2 ? P[i2] : 0;
    T y0 = b[r0], y1 = b[r1], y2 = v2 ? b[r2] : T(0);
    for (int j = 0; j < CE_N - 1; ++j) {  // forward: unit lower L
        const T yj = __shfl_sync(0xffffffffu, j < 32 ? y0 : (j < 64 ? y1 : y2), j & 31);
        const T* col = M + j * CE_LD;
        if (i0 > j) y0 = fma(-col[r0], yj, y0);
        if (i1 > j) y1 = fma(-col[r1], yj, y1);
        if (v2 && i2 > j) y2 = fma(-col[r2], yj, y2);
    }
    for (int j = CE_N - 1; j >= 0; --j) {  // backward: U
        const T yj = __shfl_sync(0xffffffffu, j < 32 ? y0 : (j < 64 ? y1 : y2), j & 31);
        const T xj = yj * uinv[j];
        if (lane == (j & 31)) {
            if (j < 32) y0 = xj; else if (j < 64) y1 = xj; else y2 = xj;
        }
        const T* col = M + j * CE_LD;
        if (i0 < j) y0 = fma(-col[r0], xj, y0);
        if (i1 < j) y1 = fma(-col[r1], xj, y1);
        if (v2 && i2 < j) y2 = fma(-col[r2], xj, y2);
    }
    x[i0] = y0;
    x[i1] = y1;
    if (v2) x[i2] = y2;
}

// The Newton step: s.sol = J^-1 F from the FP64 system in s.A.  Mixed-precision refinement on
// the equilibrated FP32 copy first, the FP64 elimination when that does not converge.  Returns
// false when J is singular or the step is not finite; *refined tells which path gave the step.
__device__ bool ce_solve(CeShared& s, bool& refined) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // equilibration: row exponents, then column exponents of the row-scaled matrix
    bool bad = false;
    if (tid < CE_N) {
        long long m = 0;
        for (int c = 0; c < CE_N; ++c) {
            const long long a = ce::abits(s.A[c * CE_LD + tid]);
            bad |= a >= 0x7ff0000000000000LL;
            m = max(m, a);
        }
        s.rexp[tid] = m ? int(m >> 52) - 1023 : 0;
    }
    if (__syncthreads_or(bad)) return false;
    if (tid < CE_N) {
        long long m = 0;
        const double* col = s.A + tid * CE_LD;
        for (int r = 0; r < CE_N; ++r) {
            const long long a = ce::abits(col[r]);
            if (a) m = max(m, a - ((long long)s.rexp[r] << 52));
        }
        s.cexp[tid] = m > 0 ? int(m >> 52) - 1023 : 0;
    }
    __syncthreads();
    for (int idx = tid; idx < CE_N * CE_N; idx += CE_THREADS) {
        const int c = idx / CE_N, r = idx - c * CE_N;
        s.B[c * CE_LD + r] = ce::scaled_to_float(s.A[c * CE_LD + r], s.rexp[r] + s.cexp[c]);
    }
    if (tid < CE_N) {
        s.sol[tid] = 0.0;
        s.res[tid] = s.A[CE_N * CE_LD + tid];
    }
    __syncthreads();
    // infinity norm of the equilibrated matrix (for the stopping rule)
    const double anorm = ce_block_max(s, [&] {
        float a = 0;
        if (tid < CE_N)
            for (int c = 0; c < CE_N; ++c) a += fabsf(s.B[c * CE_LD + tid]);
        return double(a);
    }());
    refined = ce_lu<float>(s, s.B, s.uinv32);
    if (refined) {
        // iterative refinement (as LAPACK's dsgesv): stop when the equilibrated residual is at
        // the level of an FP64 backward-stable solve, |R r| <= |C^-1 s| |J^| eps sqrt(n)
        const double cte = anorm * 0x1p-53 * sqrt(double(CE_N));
        double prev = INFINITY;
        bool conv = false;
        for (int it = 0; it < CE_REFINE_MAX; ++it) {
            // right-hand side: row-scaled residual, normalised by a power of two
            long long m = 0;
            if (tid < CE_N) {
                const long long a = ce::abits(s.res[tid]);
                if (a) m = a - ((long long)s.rexp[tid] << 52);
            }
            m = ce::warp_max_ll(m);
            if (lane == 0) s.redl[0][warp] = m;
            __syncthreads();
            long long g = s.redl[0][0];
            for (int w = 1; w < CE_WARPS; ++w) g = max(g, s.redl[0][w]);
            if (g <= 0) {  // zero residual: the step is exact
                conv = true;
                break;
            }
            const int G = int(g >> 52) - 1023;
            if (tid < CE_N) s.vec32[tid] = ce::scaled_to_float(s.res[tid], s.rexp[tid] + G);
            __syncthreads();
            ce_trisolve<float>(s.perm[(CE_N - 1) & 1], s.B, s.uinv32, s.vec32, s.vec32);
            __syncthreads();
            bool fin = true;
            long long dl = 0;
            if (tid < CE_N) {
                const double d = ldexp(double(s.vec32[tid]), G - s.cexp[tid]);
                fin = isfinite(d);
                s.sol[tid] += d;
                if (d != 0) dl = ce::abits(d) + ((long long)s.cexp[tid] << 52);
            }
            if (__syncthreads_or(!fin)) {
                refined = false;
                break;
            }
            // residual F - J s in FP64, its equilibrated norm and that of the step
            long long rl = 0, xl = 0;
            if (tid < CE_N) {
                double r = s.A[CE_N * CE_LD + tid];
                for (int c = 0; c < CE_N; ++c) r = fma(-s.A[c * CE_LD + tid], s.sol[c], r);
                s.res[tid] = r;
                const long long a = ce::abits(r);
                if (a) rl = max(0LL, a - ((long long)s.rexp[tid] << 52));
                if (s.sol[tid] != 0) xl = ce::abits(s.sol[tid]) + ((long long)s.cexp[tid] << 52);
            }
            dl = ce::warp_max_ll(dl);
            rl = ce::warp_max_ll(rl);
            xl = ce::warp_max_ll(xl);
            if (lane == 0) {
                s.redl[1][warp] = dl;
                s.redl[2][warp] = rl;
                s.redl[3][warp] = xl;
            }
            __syncthreads();
            long long D = 0, R = 0, X = 0;
            for (int w = 0; w < CE_WARPS; ++w) {
                D = max(D, s.redl[1][w]);
                R = max(R, s.redl[2][w]);
                X = max(X, s.redl[3][w]);
            }
            const double dmax = __longlong_as_double(D), rn = __longlong_as_double(R), xn = __longlong_as_double(X);
            if (rn <= xn * cte) {
                conv = true;
                break;
            }
            if (it > 0 && !(dmax <= 0.5 * prev)) break;  // not contracting: FP64 elimination
            prev = dmax;
        }
        __syncthreads();
        refined = refined && conv;
    }
    if (!refined) {
        // FP64 elimination in place (J is rebuilt by the next iteration); F from column CE_N
        if (tid < CE_N) s.res[tid] = s.A[CE_N * CE_LD + tid];
        __syncthreads();
        if (!ce_lu<double>(s, s.A, s.uinv64)) return false;
        ce_trisolve<double>(s.perm[(CE_N - 1) & 1], s.A, s.uinv64, s.res, s.sol);
        __syncthreads();
    }
    bool badS = false;
    if (tid < CE_N) badS = !isfinite(s.sol[tid]);
    return !__syncthreads_or(badS);
}

// Densities of every species, the scaled residuals F (column CE_N of s.A) and their inf-norm at
// s.x for log xi; then, unless |F|_inf < 1e-8 (or always_jacobian), the Jacobian in s.A.
// Returns 1 when converged, 0 with the system assembled, -1 when F is not finite.  Every thread
// calls it; control flow is uniform.
__device__ int ce_assemble(const ChemTables& tb, CeShared& s, double nt, double logxi, bool always_jacobian,
                           double& inf_out) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int M = tb.n_mol;
    const double ln10 = ce::LN10;
    const double inv_nt = 1.0 / nt;
    // densities of every species at x (src/statmech.jl:385-430)
    const double xe = s.x[CE_NZ];
    for (int m = tid; m < M; m += CE_THREADS) {
        const unsigned char* at = s.m_atoms + m * CE_MAXATOMS;
        double lg = -s.lognK[m] + logxi;
        if (s.m_charge[m] == 0) {
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
    // element sums in work items of <= CE_CHUNK incidences (warps 0-6), the block-wide sums
    // over molecules and ions (warp 7)
    if (tid < tb.n_items) {
        double fm = 0, dn = 0, sq = 0, dd = 0;
        for (int k = s.item_begin[tid]; k < s.item_begin[tid + 1]; ++k) {
            const int m = s.inc_mol[k];
            const double cn = s.inc_cntd[k] * s.nmol[m];
            fm += cn;
            dn = fma(s.natm1[m], cn, dn);
            sq = fma(s.chg[m], cn, sq);
            dd = fma(s.inc_cntd[k], cn, dd);
        }
        s.part[tid][0] = fm;
        s.part[tid][1] = dn;
        s.part[tid][2] = sq;
        s.part[tid][3] = dd;
    } else if (warp == CE_WARPS - 1) {
        double nn = 0, qn = 0, dq = 0, i1 = 0, i2 = 0;
        for (int m = lane; m < M; m += 32) {
            const double n = s.nmol[m];
            nn = fma(s.natm1[m], n, nn);
            qn = fma(s.chg[m], n, qn);
            dq = fma(s.chg[m] * s.natm1[m], n, dq);
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
            s.dNn[CE_NZ] = -(-ln10 * s.ne - ln10 * dq) * inv_nt;
        }
    }
    __syncthreads();
    // each element's sums from its items (fixed order); scaled residuals (src/statmech.jl:418-438)
    // into column CE_N; inf-norm (newton.jl:8-14)
    double fa = 0;
    bool bad = false;
    if (tid < CE_N) {
        double F;
        if (tid < CE_NZ) {
            double fm = 0, dn = 0, sq = 0, dd = 0;
            for (int i = s.elem_item_ptr[tid]; i < s.elem_item_ptr[tid + 1]; ++i) {
                fm += s.part[i][0];
                dn += s.part[i][1];
                sq += s.part[i][2];
                dd += s.part[i][3];
            }
            s.dNn[tid] = -(ln10 * dn) * inv_nt;
            s.Sq[tid] = sq;
            s.dd[tid] = dd;
            const double n_nuclei = (nt - s.ne) + s.nn_mol;
            double f = fm;
            if (tid == 0) f += s.nHm;
            f += ((s.nI[tid] + s.nII[tid]) + s.nIII[tid]) - s.ab[tid] * n_nuclei;
            F = f / (s.ab[tid] * nt);
        } else {
            F = (((s.qn - s.nHm) + s.ion1) - s.ne) / nt;
        }
        s.A[CE_N * CE_LD + tid] = F;
        bad = !isfinite(F);
        fa = fabs(F);
    }
    if (__syncthreads_or(bad)) return -1;
    inf_out = ce_block_max(s, fa);
    if (inf_out < 1e-8 && !always_jacobian) return 1;
    // Jacobian, dense part: the n_nuclei coupling (-d n_nuclei/dx_c / n_tot in every atom
    // row), the atoms' own densities, the n_e column, the charge row
    for (int idx = tid; idx < CE_NZ * CE_NZ; idx += CE_THREADS) {  // atom rows, atom columns
        const int c = idx / CE_NZ, r = idx - c * CE_NZ;
        if (c != r) s.A[c * CE_LD + r] = s.dNn[c];
    }
    for (int q = tid; q < 3 * CE_NZ + 1; q += CE_THREADS) {  // diagonal, n_e column, charge row
        const int r = q % CE_NZ, part = q / CE_NZ;
        if (part == 0) {
            double w = ln10 * (((s.nI[r] + s.nII[r]) + s.nIII[r]) + s.dd[r]);
            if (r == 0) w += ln10 * s.nHm;
            s.A[r * CE_LD + r] = s.dNn[r] + w * s.inv_scale[r];
        } else if (part == 1) {
            double w = -ln10 * s.Sq[r] - ln10 * (s.nII[r] + 2 * s.nIII[r]);
            if (r == 0) w += ln10 * s.nHm;
            s.A[CE_NZ * CE_LD + r] = s.dNn[CE_NZ] + w * s.inv_scale[r];
        } else if (part == 2) {
            double v = ln10 * s.Sq[r] + ln10 * (s.nII[r] + 2 * s.nIII[r]);
            if (r == 0) v -= ln10 * s.nHm;
            s.A[r * CE_LD + CE_NZ] = v * inv_nt;
        } else {
            s.A[CE_NZ * CE_LD + CE_NZ] = (((-ln10 * s.qn) - ln10 * s.nHm) - ln10 * s.ion2 - ln10 * s.ne) * inv_nt;
        }
    }
    __syncthreads();
    // Jacobian, molecule coupling off the diagonal (the diagonal's came with the element sums):
    // entry (Z, W) gains ln10 sum cnt_Z cnt_W n_mol / (ab_Z n_tot)
    for (int p = tid; p < tb.n_pairs; p += CE_THREADS) {
        const int Z = s.pair_row[p], W = s.pair_col[p];
        double sum = 0;
        for (int k = s.pair_ptr[p]; k < s.pair_ptr[p + 1]; ++k) sum = fma(s.pair_coefd[k], s.nmol[s.pair_mol[k]], sum);
        s.A[W * CE_LD + Z] += ln10 * sum * s.inv_scale[Z];
    }
    __syncthreads();
    return 0;
}

// Per-layer set-up shared by the solve and its reverse mode: the molecule tables in shared
// memory, Saha factors (saha_ion_weights with n_e = 1, src/statmech.jl:19-35, 362-372), the
// starting guess (atoms only, n_e from the model atmosphere, :151-155, 235-237), molecular log nK
// (get_log_nK, :60-62; polyatomics read_statmech_quantities.jl:66-89); with derivs, also the
// derivatives of log10 wII, log10 wIII, log10 nK (molecules and H-) with respect to T.
__device__ void ce_prologue(const ChemTables& tb, const ChemLayersDev& ly, int l, CeShared& s, bool derivs) {
    const int tid = threadIdx.x;
    const int M = tb.n_mol;
    const double T = ly.T[l], nt = ly.n_tot[l], ne_g = ly.ne_model[l];
    const int a = ly.atm ? ly.atm[l] : 0;
    const double lnT = log(T);
    const double transU = ce::translational_U(ce::ME_CGS, T);
    const double iTl = 1.0 / (T * ce::LN10);  // d log10(f) / dT = (d ln f / d ln T) / (T ln10)
    for (int i = tid; i < M * CE_MAXATOMS; i += CE_THREADS) s.m_atoms[i] = (unsigned char)tb.atoms[i];
    for (int m = tid; m < M; m += CE_THREADS) {
        s.m_charge[m] = (unsigned char)tb.charge[m];
        s.m_nat[m] = (unsigned char)tb.nat[m];
        s.natm1[m] = double(tb.nat[m] - 1);
        s.chg[m] = double(tb.charge[m]);
    }
    for (int i = tid; i <= CE_NZ; i += CE_THREADS) {
        s.inc_ptr[i] = (short)tb.inc_ptr[i];
        s.elem_item_ptr[i] = (short)tb.elem_item_ptr[i];
    }
    for (int i = tid; i < tb.inc_ptr[CE_NZ]; i += CE_THREADS) {
        s.inc_mol[i] = (short)tb.inc_mol[i];
        s.inc_cntd[i] = double(tb.inc_cnt[i]);
    }
    for (int i = tid; i <= tb.n_items; i += CE_THREADS) s.item_begin[i] = (short)tb.item_begin[i];
    for (int p = tid; p <= tb.n_pairs; p += CE_THREADS) {
        s.pair_ptr[p] = (short)tb.pair_ptr[p];
        if (p < tb.n_pairs) {
            s.pair_row[p] = (unsigned char)tb.pair_row[p];
            s.pair_col[p] = (unsigned char)tb.pair_col[p];
        }
    }
    for (int k = tid; k < tb.pair_ptr[tb.n_pairs]; k += CE_THREADS) {
        s.pair_mol[k] = (short)tb.pair_mol[k];
        s.pair_coefd[k] = double(tb.pair_coef[k]);
    }
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
        if (derivs) {  // d ln(U) / d ln T from the splines; d/dT of T^1.5 exp(-chi/kT)
            const double dI = ce::spline_deriv(tb.lnT, U, Uz, tb.nk, lnT) / UI;
            const double dII = ce::spline_deriv(tb.lnT, U + tb.nk, Uz + tb.nk, tb.nk, lnT) / UII;
            const double dw2 = (dII - dI + 1.5 + chiI / (ce::KB_EV * T)) * iTl;
            s.dlwII[Z] = dw2;
            if (Z > 0) {
                const double UIII = ce::spline(tb.lnT, U + 2 * tb.nk, Uz + 2 * tb.nk, tb.nk, lnT);
                const double dIII = ce::spline_deriv(tb.lnT, U + 2 * tb.nk, Uz + 2 * tb.nk, tb.nk, lnT) / UIII;
                s.dlwIII[Z] = dw2 + (dIII - dII + 1.5 + chiII / (ce::KB_EV * T)) * iTl;
            } else {
                s.dlwIII[Z] = 0.0;
            }
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
        double logK, dlog = 0;  // dlog: d log10 nK / dT
        if (tb.kind[m] == 0) {
            logK = ce::spline(tb.t + o, tb.u + o, tb.z + o, n, lnT);
            if (derivs) dlog = ce::spline_deriv(tb.t + o, tb.u + o, tb.z + o, n, lnT) / T - double(na - 1) * iTl;
        } else {
            const double Tp = exp(lnT);
            double prodU = 1.0, dlnU = 0;
            for (int j = 0; j < CE_MAXATOMS && tb.atoms[m * CE_MAXATOMS + j]; ++j) {
                const int Z = tb.atoms[m * CE_MAXATOMS + j] - 1;
                const double* Ua = tb.U_u + size_t(3 * Z) * tb.nk;
                const double* Uza = tb.U_z + size_t(3 * Z) * tb.nk;
                const double Uv = ce::spline(tb.lnT, Ua, Uza, tb.nk, lnT);
                prodU *= Uv;
                if (derivs) dlnU += ce::spline_deriv(tb.lnT, Ua, Uza, tb.nk, lnT) / Uv;
            }
            const double Umol = ce::spline(tb.t + o, tb.u + o, tb.z + o, n, lnT);
            const double log_Us = log10(prodU / Umol);
            if (derivs) {
                dlnU -= ce::spline_deriv(tb.t + o, tb.u + o, tb.z + o, n, lnT) / Umol;
                dlog = (double(na - 1) * 1.5 + dlnU + tb.D00[m] / (ce::KB_EV * T)) * iTl;
            }
            const double ltU = 1.5 * log10(ce::TWO_PI * ce::KB_CGS * Tp / (ce::H_CGS * ce::H_CGS));
            const double lnK = double(na - 1) * ltU + 1.5 * tb.lmr[m] + log_Us - tb.D00[m] / (ce::KB_EV * Tp * log(10.0));
            logK = lnK + double(na - 1) * log10(ce::KB_CGS * Tp);
        }
        s.lognK[m] = logK - double(na - 1) * log10(ce::KB_CGS * T);
        if (derivs) s.dlognK[m] = dlog;
    }
    if (tid == 0) {
        s.x0[CE_NZ] = log10(ne_g);
        s.lognK_Hm = log10(exp(ce::HMINUS_EA_EV / (ce::KB_EV * T)) / (4 * transU));
        s.dlognK_Hm = (-ce::HMINUS_EA_EV / (ce::KB_EV * T) - 1.5) * iTl;
        s.transU = transU;
        s.lnT = lnT;
    }
    __syncthreads();
}

// One Newton solve at log xi from s.x (clipped_newton, src/newton.jl:2-35).  Every thread calls
// it; control flow is uniform.  Returns whether |F|_inf < tol was reached; budget counts the
// iterations left for the layer (exhausted: out_of_budget is set); fallbacks counts the steps
// that needed the FP64 elimination.
__device__ bool ce_newton(const ChemTables& tb, CeShared& s, double nt, double logxi, int max_iter, int& budget,
                          bool& out_of_budget, double& last_inf, int& fallbacks) {
    const int tid = threadIdx.x;
    last_inf = INFINITY;
    for (int it = 0; it < max_iter; ++it) {
        if (budget <= 0) {
            out_of_budget = true;
            return false;
        }
        --budget;
        double inf = last_inf;
        const int st = ce_assemble(tb, s, nt, logxi, false, inf);
        if (st < 0) return false;
        last_inf = inf;
        if (st > 0) return true;
        bool refined = false;
        if (!ce_solve(s, refined)) return false;
        if (!refined) ++fallbacks;
        // step = -(J \ F), clipped so that no unknown moves more than 1 dex
        const double sm = ce_block_max(s, tid < CE_N ? fabs(s.sol[tid]) : 0.0);
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
    ce_prologue(tb, ly, l, s, false);
    const double T = ly.T[l], nt = ly.n_tot[l];
    // the solve (src/statmech.jl:240-305)
    int budget = CE_MAX_ITER;
    bool oob = false;
    double last_inf = INFINITY;
    int solves = 0, st = KORG_CHEM_OK, fallbacks = 0;
    double logxi = 0.0;
    if (tid < CE_N) s.x[tid] = s.x0[tid];
    __syncthreads();
    ++solves;
    bool conv = ce_newton(tb, s, nt, 0.0, 50, budget, oob, last_inf, fallbacks);
    if (!conv && !oob) {
        const double anchors[3] = {-5.0, -20.0, -50.0};
        bool anchored = false;
        for (int q = 0; q < 3 && !anchored && !oob; ++q) {
            if (tid < CE_N) s.x[tid] = s.x0[tid];
            __syncthreads();
            ++solves;
            anchored = ce_newton(tb, s, nt, anchors[q], 100, budget, oob, last_inf, fallbacks);
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
                bool c2 = ce_newton(tb, s, nt, logxi + step, 100, budget, oob, last_inf, fallbacks);
                if (!c2) {
                    step /= 2;
                    while (!c2 && step >= 0.0625 && !oob) {
                        if (tid < CE_N) s.x[tid] = s.xs[tid];
                        __syncthreads();
                        ++solves;
                        c2 = ce_newton(tb, s, nt, logxi + step, 100, budget, oob, last_inf, fallbacks);
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
            info[CE_NINFO * l + 4] = double(fallbacks);
        }
    }
}

// block-wide sum of one value per thread, in a fixed order (every thread gets it); two barriers
__device__ inline double ce_block_sum(CeShared& s, double v) {
    v = ce::warp_sum(v);
    if ((threadIdx.x & 31) == 0) s.red[threadIdx.x >> 5] = v;
    __syncthreads();
    double m = 0;
    for (int w = 0; w < CE_WARPS; ++w) m += s.red[w];
    __syncthreads();
    return m;
}

// s.part[i][slot] = sum over work item i's incidences of cnt * s.wmol[m] (threads < n_items)
__device__ inline void ce_item_sums(const ChemTables& tb, CeShared& s, int slot) {
    const int tid = threadIdx.x;
    if (tid < tb.n_items) {
        double acc = 0;
        for (int k = s.item_begin[tid]; k < s.item_begin[tid + 1]; ++k) acc = fma(s.inc_cntd[k], s.wmol[s.inc_mol[k]], acc);
        s.part[tid][slot] = acc;
    }
}

__device__ inline double ce_elem_total(const CeShared& s, int Z, int slot) {
    double acc = 0;
    for (int i = s.elem_item_ptr[Z]; i < s.elem_item_ptr[Z + 1]; ++i) acc += s.part[i][slot];
    return acc;
}

// Reverse mode of chemical_equilibrium at a solution, the implicit-function rule of the
// reference's ForwardDiff method (src/statmech.jl:307-355): with J dx/dp = -dF/dp at F = 0, the
// cotangents g of every output density (the layout of korg_chemical_equilibrium's densities)
// give, per layer, dL/dp = g (dn/dp)|x - lambda (dF/dp) with J^T lambda = (dn/dx)^T g, for p =
// T, n_tot and the (normalised) abundances.  J is the Newton step's system, solved the same way
// (equilibrated FP32 factors, FP64 refinement), transposed.
__global__ void __launch_bounds__(CE_THREADS) chem_vjp_kernel(ChemTables tb, ChemLayersDev ly, const double* __restrict__ dens,
                                                              const double* __restrict__ gbar, double* __restrict__ dT,
                                                              double* __restrict__ dnt, double* __restrict__ dab,
                                                              int32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char ce_smem[];
    CeShared& s = *reinterpret_cast<CeShared*>(ce_smem);
    const int l = blockIdx.x;
    if (l >= ly.L) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int M = tb.n_mol;
    const int nspec = 278 + M;
    const double ln10 = ce::LN10;
    ce_prologue(tb, ly, l, s, true);
    const double nt = ly.n_tot[l];
    const double* d = dens + size_t(l) * nspec;
    const double* g = gbar + size_t(l) * nspec;
    if (tid < CE_NZ) s.x[tid] = log10(d[1 + 3 * tid]);
    if (tid == CE_NZ) s.x[CE_NZ] = log10(d[0]);
    __syncthreads();
    double inf = 0;
    bool ok = ce_assemble(tb, s, nt, 0.0, true, inf) >= 0;  // densities, F and J at the solution
    // xbar = (dn/dx)^T g; molecule weights g_m n_m
    for (int m = tid; m < M; m += CE_THREADS) s.wmol[m] = g[278 + m] * s.nmol[m];
    if (tid < CE_N) s.x0[tid] = s.A[CE_N * CE_LD + tid];  // keep F (column CE_N becomes xbar)
    __syncthreads();
    ce_item_sums(tb, s, 0);
    if (warp == CE_WARPS - 1) {
        double wq = 0, gi = 0;
        for (int m = lane; m < M; m += 32) wq = fma(s.chg[m], s.wmol[m], wq);
        for (int Z = lane; Z < CE_NZ; Z += 32) gi += g[2 + 3 * Z] * s.nII[Z] + 2 * g[3 + 3 * Z] * s.nIII[Z];
        wq = ce::warp_sum(wq);
        gi = ce::warp_sum(gi);
        if (lane == 0) {
            s.vsum[0] = wq;
            s.vsum[1] = gi;
        }
    }
    __syncthreads();
    if (tid < CE_NZ) {
        double xb = g[1 + 3 * tid] * s.nI[tid] + g[2 + 3 * tid] * s.nII[tid] + g[3 + 3 * tid] * s.nIII[tid] +
                    ce_elem_total(s, tid, 0);
        if (tid == 0) xb += g[277] * s.nHm;
        s.A[CE_N * CE_LD + tid] = ln10 * xb;
    } else if (tid == CE_NZ) {
        s.A[CE_N * CE_LD + CE_NZ] = ln10 * (g[0] * s.ne - s.vsum[1] + g[277] * s.nHm - s.vsum[0]);
    }
    // J^T in place
    for (int idx = tid; idx < CE_N * CE_N; idx += CE_THREADS) {
        const int c = idx / CE_N, r = idx - c * CE_N;
        if (r < c) {
            const double t = s.A[c * CE_LD + r];
            s.A[c * CE_LD + r] = s.A[r * CE_LD + c];
            s.A[r * CE_LD + c] = t;
        }
    }
    __syncthreads();
    bool refined = false;
    ok = ce_solve(s, refined) && ok;  // s.sol = lambda
    // temperature sensitivities of the densities at fixed x: d n / d T = n * ln10 * d log10 n / dT
    for (int m = tid; m < M; m += CE_THREADS) {
        double dl = -s.dlognK[m];
        if (s.m_charge[m]) dl += s.dlwII[s.m_atoms[m * CE_MAXATOMS] - 1];
        s.wmol[m] = s.nmol[m] * ln10 * dl;
    }
    __syncthreads();
    ce_item_sums(tb, s, 1);
    if (warp == CE_WARPS - 1) {
        double sn = 0, sq = 0, si = 0;
        for (int m = lane; m < M; m += 32) {
            sn = fma(s.natm1[m], s.wmol[m], sn);
            sq = fma(s.chg[m], s.wmol[m], sq);
        }
        for (int Z = lane; Z < CE_NZ; Z += 32)
            si += ln10 * (s.nII[Z] * s.dlwII[Z] + 2 * s.nIII[Z] * s.dlwIII[Z]);
        sn = ce::warp_sum(sn);
        sq = ce::warp_sum(sq);
        si = ce::warp_sum(si);
        if (lane == 0) {
            s.vsum[0] = sn;
            s.vsum[1] = sq;
            s.vsum[2] = si;
        }
    }
    __syncthreads();
    // per-thread contributions to dL/dT and dL/dn_tot; dL/dab per element
    double cT = 0, cN = 0;
    const double dHm = s.nHm * ln10 * s.dlognK_Hm;
    if (tid < CE_NZ) {
        const double dII = s.nII[tid] * ln10 * s.dlwII[tid], dIII = s.nIII[tid] * ln10 * s.dlwIII[tid];
        double num = ce_elem_total(s, tid, 1) + dII + dIII - s.ab[tid] * s.vsum[0];
        if (tid == 0) num += dHm;
        const double lam = s.sol[tid], F = s.x0[tid];
        cT = g[2 + 3 * tid] * dII + g[3 + 3 * tid] * dIII - lam * num * s.inv_scale[tid];
        cN = lam * (1 + F) / nt;
        const double n_nuclei = (nt - s.ne) + s.nn_mol;
        dab[size_t(l) * CE_NZ + tid] = lam * (n_nuclei / nt + F) / s.ab[tid];
    } else if (tid == CE_NZ) {
        const double lam = s.sol[CE_NZ], F = s.x0[CE_NZ];
        cT = g[277] * dHm - lam * ((s.vsum[1] - dHm) + s.vsum[2]) / nt;
        cN = lam * F / nt;
    }
    for (int m = tid; m < M; m += CE_THREADS) cT = fma(g[278 + m], s.wmol[m], cT);
    const double sT = ce_block_sum(s, cT);
    const double sN = ce_block_sum(s, cN);
    if (tid == 0) {
        dT[l] = sT;
        dnt[l] = sN;
        status[l] = ok ? KORG_CHEM_OK : KORG_CHEM_NONFINITE;
    }
}

}  // namespace korg
