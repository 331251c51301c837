// postprocess.cuh -- spectral post-processing on the device: the Gaussian line-spread function
// (apply_LSF / compute_LSF_matrix, src/utils.jl:45-58, 94-106, 132-155) and rotational
// broadening (apply_rotation, src/utils.jl:168-240), each with its reverse mode (both maps are
// linear in the flux, so the reverse mode is the transposed map).
//
//   lsf kernels:       one warp per output wavelength: the window by two binary searches, the
//                      Gaussian weights by lanes, their sum by shuffles; the forward applies
//                      each chunk of weights to every spectrum, the reverse mode scatters them
//                      for a block of up to LSF_SPEC spectra.
//   rotation kernels:  one thread per output wavelength: a walk over the window carrying the
//                      previous kernel integral; the forward keeps each chunk's weights in
//                      shared memory and applies them to every spectrum, the reverse mode
//                      scatters them for a block of up to ROT_SPEC spectra.
//
// Everything is FP64, as in the reference (post-processing of the FP64 flux).
#pragma once
#include "physics.cuh"

namespace korg {

constexpr int LSF_SPEC = 8;   // spectra per warp pass
constexpr int ROT_SPEC = 8;   // spectra per thread pass
constexpr int ROT_MAX_RANGES = 64;

struct LsfArgs {
    const double* wls;    // synthesis grid (cm), sorted
    int64_t nwl;
    const double* owl;    // output wavelengths (cm)
    int64_t nout;
    const double* R;      // resolving power: R[0] for all outputs, or R[i] per output
    int32_t R_per_point;
    double window;        // window half-width in units of sigma
    double fwhm_to_sigma; // 2 sqrt(2 ln 2), as the reference computes it
};

// _lsf_bounds_and_kernel (src/utils.jl:45-58): sigma = wl0 / R / (2 sqrt(2 ln 2)); window
// [searchsortedfirst(wl0 - w sigma), searchsortedlast(wl0 + w sigma)].
__device__ __forceinline__ void lsf_window(const LsfArgs& a, int64_t i, int64_t& lb, int64_t& ub, double& wl0,
                                           double& sigma) {
    wl0 = a.owl[i];
    sigma = wl0 / a.R[a.R_per_point ? i : 0] / a.fwhm_to_sigma;
    lb = search_first(a.wls, a.nwl, wl0 - a.window * sigma);
    ub = search_last(a.wls, a.nwl, wl0 + a.window * sigma);
}

// normal_pdf (src/utils.jl:5)
__device__ __forceinline__ double lsf_phi(double d, double sigma) {
    return exp(-0.5 * (d * d) / (sigma * sigma)) / 2.5066282746310002 / sigma;
}

// window weight sum of output i, every lane gets it
__device__ __forceinline__ double lsf_norm(const LsfArgs& a, int64_t lb, int64_t ub, double wl0, double sigma,
                                           int lane) {
    double s = 0.0;
    for (int64_t j = lb + lane; j <= ub; j += 32) s += lsf_phi(a.wls[j] - wl0, sigma);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// out[s][i] = sum_j flux[s][j] phi_j / sum phi  (apply_LSF :94-106, compute_LSF_matrix * flux).
// The window is taken in chunks of 32 LSF_CW points; each lane keeps its LSF_CW normalised
// weights of the chunk in registers and applies them to every spectrum, so the Gaussian is
// evaluated twice per window point (sum, then weights) whatever the number of spectra.
constexpr int LSF_CW = 8;
__global__ void __launch_bounds__(256) lsf_apply_kernel(LsfArgs a, const double* flux, int32_t nspec, double* out) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (i >= a.nout) return;  // uniform across the warp
    int64_t lb, ub;
    double wl0, sigma;
    lsf_window(a, i, lb, ub, wl0, sigma);
    const double norm = lsf_norm(a, lb, ub, wl0, sigma, lane);
    if (ub < lb) {  // empty window: an empty sum
        for (int s = lane; s < nspec; s += 32) out[int64_t(s) * a.nout + i] = 0.0;
        return;
    }
    for (int64_t c0 = lb; c0 <= ub; c0 += 32 * LSF_CW) {
        double w[LSF_CW];
#pragma unroll
        for (int k = 0; k < LSF_CW; k++) {
            const int64_t j = c0 + lane + 32 * k;
            w[k] = j <= ub ? lsf_phi(a.wls[j] - wl0, sigma) / norm : 0.0;
        }
        for (int s = 0; s < nspec; s++) {
            const double* f = flux + int64_t(s) * a.nwl;
            double v = 0.0;
#pragma unroll
            for (int k = 0; k < LSF_CW; k++) {
                const int64_t j = c0 + lane + 32 * k;
                if (j <= ub) v += f[j] * w[k];
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) {
                double* dst = out + int64_t(s) * a.nout + i;
                *dst = c0 == lb ? v : *dst + v;
            }
        }
    }
}

// reverse mode: dflux[s][j] += sum_i dout[s][i] phi_ij / sum_j phi_ij
__global__ void __launch_bounds__(256) lsf_vjp_kernel(LsfArgs a, const double* dout, int32_t nspec, double* dflux) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int s0 = blockIdx.y * LSF_SPEC;
    if (i >= a.nout) return;
    int64_t lb, ub;
    double wl0, sigma;
    lsf_window(a, i, lb, ub, wl0, sigma);
    const double norm = lsf_norm(a, lb, ub, wl0, sigma, lane);
    const int ns = min(LSF_SPEC, nspec - s0);
    double g[LSF_SPEC];
#pragma unroll
    for (int k = 0; k < LSF_SPEC; k++) g[k] = k < ns ? dout[int64_t(s0 + k) * a.nout + i] : 0.0;
    for (int64_t j = lb + lane; j <= ub; j += 32) {
        const double w = lsf_phi(a.wls[j] - wl0, sigma) / norm;
#pragma unroll
        for (int k = 0; k < LSF_SPEC; k++)
            if (k < ns && g[k] != 0.0) atomicAdd(dflux + int64_t(s0 + k) * a.nwl + j, g[k] * w);
    }
}

// window bounds per output (0-based, inclusive; ub < lb for an empty window)
__global__ void lsf_windows_kernel(LsfArgs a, int64_t* lb_out, int64_t* ub_out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.nout) return;
    int64_t lb, ub;
    double wl0, sigma;
    lsf_window(a, i, lb, ub, wl0, sigma);
    lb_out[i] = lb;
    ub_out[i] = ub;
}

// normalised weights of output i at vals[row_ptr[i] + (j - lb)] (compute_LSF_matrix, :150-153)
__global__ void __launch_bounds__(256) lsf_values_kernel(LsfArgs a, const int64_t* row_ptr, double* vals) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (i >= a.nout) return;
    int64_t lb, ub;
    double wl0, sigma;
    lsf_window(a, i, lb, ub, wl0, sigma);
    const double norm = lsf_norm(a, lb, ub, wl0, sigma, lane);
    double* v = vals + row_ptr[i];
    for (int64_t j = lb + lane; j <= ub; j += 32) v[j - lb] = lsf_phi(a.wls[j] - wl0, sigma) / norm;
}

struct RotRange {
    int64_t first, n;  // grid indices of the range
    double step;       // step(wls) of the range (cm)
};
struct RotArgs {
    const double* wls;  // grid (cm)
    int64_t nwl;
    int32_t nranges;
    RotRange r[ROT_MAX_RANGES];
    double v_over_c;    // vsini (cm/s) / c
    double c1, c2, c3;  // 2(1 - eps), pi eps / 2, pi (1 - eps / 3)
};

// _rotation_kernel_integral_kernel (src/utils.jl:233-240)
__device__ __forceinline__ double rot_kernel_integral(const RotArgs& a, double c3dl, double d, double dl) {
    if (fabs(d) == dl) return d > 0 ? 0.5 : -0.5;
    return (0.5 * a.c1 * d * sqrt(1 - (d * d) / (dl * dl)) + 0.5 * a.c1 * dl * asin(d / dl) +
            a.c2 * (d - (d * d * d) / (3 * (dl * dl)))) / c3dl;
}

// the range holding grid index i
__device__ __forceinline__ const RotRange& rot_range(const RotArgs& a, int64_t i) {
    int k = 0;
    while (k + 1 < a.nranges && i >= a.r[k + 1].first) k++;
    return a.r[k];
}

// Reverse mode of the rotation of output i (_apply_rotation_core, :204-228: detunings
// [-dl, (lb - i + 1/2 .. ub - i - 1/2) step, dl], kernel integrals K_0 .. K_m+1, new
// F_i = sum K_{k+1} F_{lb+k} - sum K_k F_{lb+k}): dout_i (K_{k+1} - K_k) is scattered to
// dF_{lb+k}, for spectra s0 .. s0 + ns - 1.
__global__ void __launch_bounds__(128) rotation_vjp_kernel(RotArgs a, const double* dout, int32_t nspec,
                                                           double* dflux) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int s0 = blockIdx.y * ROT_SPEC;
    if (i >= a.nwl) return;
    const int ns = min(ROT_SPEC, nspec - s0);
    const RotRange& rg = rot_range(a, i);
    const double* w = a.wls + rg.first;
    const int64_t ii = i - rg.first;
    const double dl = a.wls[i] * a.v_over_c;
    const int64_t lb = search_first(w, rg.n, a.wls[i] - dl), ub = search_last(w, rg.n, a.wls[i] + dl);
    const double c3dl = a.c3 * dl;
    double g[ROT_SPEC];
#pragma unroll
    for (int k = 0; k < ROT_SPEC; k++) g[k] = k < ns ? dout[int64_t(s0 + k) * a.nwl + i] : 0.0;
    double Kp = rot_kernel_integral(a, c3dl, -dl, dl);
    for (int64_t m = lb; m <= ub; m++) {
        const double d = m < ub ? (double(m - ii) + 0.5) * rg.step : dl;
        const double Kn = rot_kernel_integral(a, c3dl, d, dl);
        const int64_t j = rg.first + m;
#pragma unroll
        for (int k = 0; k < ROT_SPEC; k++)
            if (k < ns) atomicAdd(dflux + int64_t(s0 + k) * a.nwl + j, g[k] * (Kn - Kp));
        Kp = Kn;
    }
}

// Forward rotation, all spectra at once: each thread owns one output wavelength and walks its
// window in chunks of ROT_CH points, keeping the chunk's weights K_{k+1} - K_k (one asin/sqrt
// pair per window point, whatever the number of spectra) in its own column of shared memory,
// then applies them to every spectrum, accumulating across chunks in the output.
constexpr int ROT_TP = 64;  // threads (output wavelengths) per block
constexpr int ROT_CH = 64;  // window points per chunk
__global__ void __launch_bounds__(ROT_TP) rotation_fwd_kernel(RotArgs a, const double* in, int32_t nspec,
                                                              double* out) {
    __shared__ double s_w[ROT_CH][ROT_TP];  // column t: this thread's weights
    const int t = threadIdx.x;
    const int64_t i = int64_t(blockIdx.x) * ROT_TP + t;
    if (i >= a.nwl) return;  // no block-wide synchronisation below
    const RotRange& rg = rot_range(a, i);
    const double* w = a.wls + rg.first;
    const int64_t ii = i - rg.first;
    const double dl = a.wls[i] * a.v_over_c;
    const int64_t lb = search_first(w, rg.n, a.wls[i] - dl), ub = search_last(w, rg.n, a.wls[i] + dl);
    const int64_t nwin = ub - lb + 1;
    const double c3dl = a.c3 * dl;
    double Kp = rot_kernel_integral(a, c3dl, -dl, dl);
    for (int64_t c0 = 0; c0 < nwin; c0 += ROT_CH) {
        const int nq = int(min(int64_t(ROT_CH), nwin - c0));
        for (int q = 0; q < nq; q++) {
            const int64_t m = lb + c0 + q;
            const double d = m < ub ? (double(m - ii) + 0.5) * rg.step : dl;
            const double Kn = rot_kernel_integral(a, c3dl, d, dl);
            s_w[q][t] = Kn - Kp;
            Kp = Kn;
        }
        const double* f0 = in + rg.first + lb + c0;
        for (int s = 0; s < nspec; s++) {
            const double* f = f0 + int64_t(s) * a.nwl;
            double acc = 0.0;
            for (int q = 0; q < nq; q++) acc += s_w[q][t] * f[q];
            double* o = out + int64_t(s) * a.nwl + i;
            *o = c0 == 0 ? acc : *o + acc;
        }
    }
    if (nwin <= 0) {  // empty window (cannot happen for a grid point, which is inside its own window)
        for (int s = 0; s < nspec; s++) out[int64_t(s) * a.nwl + i] = 0.0;
    }
}

}  // namespace korg
