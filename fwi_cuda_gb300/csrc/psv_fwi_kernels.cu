// psv_fwi_kernels.cu -- model-side kernels (compiled with -fmad=false so the
// FP64 arithmetic rounds like the reference's host code).
#include <math.h>

#include "psv_fwi.cuh"
#include "psv_kernels.cuh"

namespace psv {

static constexpr int RED_BLOCKS = kRedBlocks;
static constexpr int RED_THREADS = 256;

// ---------------------------------------------------------------------------
// mat_av2 (src/cpu/n_kernel_lib_PSV.cpp:853-898) and the dt-scaled
// coefficients the time-step kernels read.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_coeffs(const CoeffParams<T> c)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= c.nx || iz >= c.nz) return;
    const int nx = c.nx;
    const long long k = (long long)iz * nx + ix;
    const long long q = (long long)iz * c.pitch + ix;
    const double lam = c.lam[k], mu = c.mu[k];
    double muzx = 0.0, rzp = 0.0, rxp = 0.0;
    if (c.mu_zx) {
        muzx = c.mu_zx[k];
        rzp = c.rho_zp[k];
        rxp = c.rho_xp[k];
    } else if (iz < c.nz - 1 && ix < nx - 1) {
        const double m00 = mu, m01 = c.mu[k + 1], m10 = c.mu[k + nx], m11 = c.mu[k + nx + 1];
        muzx = 4.0 / ((1.0 / m00) + (1.0 / m01) + (1.0 / m10) + (1.0 / m11));
        if ((m00 == 0.0) || (m01 == 0.0) || (m10 == 0.0) || (m11 == 0.0)) muzx = 0.0;
        const double r00 = c.rho[k], r10 = c.rho[k + nx], r01 = c.rho[k + 1];
        rzp = 1.0 / (0.5 * (r00 + r10));
        rxp = 1.0 / (0.5 * (r00 + r01));
        if ((r00 < 1e-4) && (r10 < 1e-4)) rzp = 0.0;
        if ((r00 < 1e-4) && (r01 < 1e-4)) rzp = 0.0;  // the reference tests rho_xp's cells but zeroes rho_zp (:894-897)
    }
    const double dt = c.dt;
    c.c_lam[q] = (T)(dt * lam);
    c.c_l2m[q] = (T)(dt * (lam + 2.0 * mu));
    c.c_muzx[q] = (T)(dt * muzx);
    c.c_rz[q] = (T)(dt * rzp);
    c.c_rx[q] = (T)(dt * rxp);
    c.g1[q] = (T)(c.kimg * 0.25 / ((lam + mu) * (lam + mu)) * c.gscale);
    c.g2[q] = (T)(c.kimg / (mu * mu) * c.gscale);
    const double fs = 4.0 * dt * (lam * mu + mu * mu) / (lam + 2.0 * mu);
    if (c.st && iz == c.st) c.fs_top[ix] = (T)fs;
    if (c.sb && iz == c.sb) c.fs_bot[ix] = (T)fs;
    if (c.sl && ix == c.sl) c.fs_left[iz] = (T)fs;
    if (c.sr && ix == c.sr) c.fs_right[iz] = (T)fs;
}

template <typename T>
cudaError_t launch_coeffs(const CoeffParams<T> &c, cudaStream_t st)
{
    dim3 b(32, 8), g((c.nx + 31) / 32, (c.nz + 7) / 8);
    k_coeffs<T><<<g, b, 0, st>>>(c);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Deterministic block reductions.
// ---------------------------------------------------------------------------
// Butterfly sum of a warp's 32 values by register shuffles (every lane ends
// with the same, order-fixed result).
__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block: each warp by shuffles, then the warp sums by the
// first warp; the same order on every run.  sh needs RED_THREADS / 32 + 1
// doubles; every thread gets the result.
__device__ __forceinline__ double block_sum(double v, double *sh)
{
    static_assert(RED_THREADS % 32 == 0 && RED_THREADS <= 1024, "whole warps");
    constexpr int NW = RED_THREADS / 32;
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    v = warp_sum(v);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        double u = lane < NW ? sh[lane] : 0.0;
        u = warp_sum(u);
        if (lane == 0) sh[NW] = u;
    }
    __syncthreads();
    const double r = sh[NW];
    __syncthreads();  // sh is reused by the caller's next sum
    return r;
}

// Sums of lam, mu, rho over [0, nz-1) x [0, nx-1) (mat_av2's scalar averages, :899-909).
__global__ void __launch_bounds__(RED_THREADS) k_model_partial(const double *lam, const double *mu,
                                                               const double *rho, int nz, int nx,
                                                               double *partial)
{
    __shared__ double sh[RED_THREADS];
    const long long n = (long long)(nz - 1) * (nx - 1);
    double a = 0.0, b = 0.0, c = 0.0;
    for (long long k = (long long)blockIdx.x * RED_THREADS + threadIdx.x; k < n;
         k += (long long)RED_BLOCKS * RED_THREADS) {
        const long long iz = k / (nx - 1), ix = k % (nx - 1);
        const long long j = iz * nx + ix;
        a += lam[j];
        b += mu[j];
        c += rho[j];
    }
    a = block_sum(a, sh);
    b = block_sum(b, sh);
    c = block_sum(c, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = a;
        partial[RED_BLOCKS + blockIdx.x] = b;
        partial[2 * RED_BLOCKS + blockIdx.x] = c;
    }
}

// out[blockIdx.x] = scale * sum(partial[blockIdx.x * RED_BLOCKS ...]).
__global__ void __launch_bounds__(RED_THREADS) k_final_sum(const double *partial, double *out,
                                                           double scale)
{
    __shared__ double sh[RED_THREADS];
    const double v = partial[(long long)blockIdx.x * RED_BLOCKS + threadIdx.x];
    const double s = block_sum(v, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = s * scale;
}

cudaError_t launch_model_sums(const double *lam, const double *mu, const double *rho, int nz,
                              int nx, double *partial, double *out3, cudaStream_t st)
{
    k_model_partial<<<RED_BLOCKS, RED_THREADS, 0, st>>>(lam, mu, rho, nz, nx, partial);
    k_final_sum<<<3, RED_THREADS, 0, st>>>(partial, out3, 1.0);
    return cudaGetLastError();
}

// adjsrc2 (src/cpu/n_kernel_lib_PSV.cpp:579-626): r = mod - true, L2 = sum dt/2 (rz^2 + rx^2).
__global__ void __launch_bounds__(RED_THREADS) k_adjsrc_partial(const double *mz,
                                                                const double *mx,
                                                                const double *tz,
                                                                const double *tx, double *rz_out,
                                                                double *rx_out, long long n,
                                                                double dt, double *partial)
{
    __shared__ double sh[RED_THREADS];
    const long long off = (long long)blockIdx.y * n;
    double acc = 0.0;
    for (long long k = (long long)blockIdx.x * RED_THREADS + threadIdx.x; k < n;
         k += (long long)RED_BLOCKS * RED_THREADS) {
        const double rz = mz[off + k] - tz[off + k];
        const double rx = mx[off + k] - tx[off + k];
        if (rz_out) {
            rz_out[off + k] = rz;
            rx_out[off + k] = rx;
        }
        acc += 0.5 * dt * (rz * rz) + 0.5 * dt * (rx * rx);
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[(long long)blockIdx.y * RED_BLOCKS + blockIdx.x] = acc;
}

cudaError_t launch_adjsrc(const double *mod_z, const double *mod_x, const double *true_z,
                          const double *true_x, double *res_z, double *res_x,
                          long long n_per_shot, int nshot, double dt, double *partial,
                          double *out, cudaStream_t st)
{
    if (nshot <= 0) return cudaSuccess;
    dim3 g(RED_BLOCKS, nshot);
    k_adjsrc_partial<<<g, RED_THREADS, 0, st>>>(mod_z, mod_x, true_z, true_x, res_z, res_x,
                                                n_per_shot, dt, partial);
    k_final_sum<<<nshot, RED_THREADS, 0, st>>>(partial, out, 1.0);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// energy_weights2 (src/cpu/n_kernel_lib_PSV.cpp:696-757): per shot, the
// maximum over [z1, z2) x [x1, x2) of sqrt(We We_adj).  Non-negative doubles
// order like their bit patterns, so an atomicMax on the bits is exact and
// order-independent.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_energy_max(const T *fld, long long plane, long long shot_stride, int pitch,
                             int z1, int z2, int x1, int x2, double *wmax)
{
    const int ix = x1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = z1 + blockIdx.y * blockDim.y + threadIdx.y;
    double v = 0.0;
    if (ix < x2 && iz < z2) {
        const T *f = fld + (long long)blockIdx.z * shot_stride;
        const long long i = (long long)iz * pitch + ix;
        v = sqrt((double)f[F_WE * plane + i] * (double)f[F_WEA * plane + i]);
    }
    // warp max, then one atomic per warp
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0.0)
        atomicMax((unsigned long long *)&wmax[blockIdx.z], (unsigned long long)__double_as_longlong(v));
}

template <typename T>
cudaError_t launch_energy_max(const T *fld, long long plane, long long shot_stride, int pitch,
                              int z1, int z2, int x1, int x2, int nbatch, double *wmax,
                              cudaStream_t st)
{
    if (z2 <= z1 || x2 <= x1) return cudaSuccess;
    dim3 b(32, 8), g((x2 - x1 + 31) / 32, (z2 - z1 + 7) / 8, nbatch);
    k_energy_max<T><<<g, b, 0, st>>>(fld, plane, shot_stride, pitch, z1, z2, x1, x2, wmax);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// interpol_grad2 (src/cpu/n_kernel_lib_PSV.cpp:628-693) as a gather.  The
// reference interpolates into a scratch array that holds the adjoint energy
// We_adj; cells its loops never write keep that value, and so do they here.
// ---------------------------------------------------------------------------
template <typename T>
struct InterpView {
    const T *gs;  // one parameter's snapped gradient [snz][snx_pitch]
    const T *wa;  // We_adj plane [nz][pitch]
    int pitch, snx_pitch, z1, z2, x1, x2, sdz, sdx;
    double gs_un, wa_un;  // unscale of gs and of wa values

    int nz, nx;
    __device__ double stage_a(int iz, int ix) const
    {
        // The reference's loops can reach one interval past the window and,
        // at the grid edge, past its row; those cells read as 0 here.
        if (iz >= nz || ix >= nx) return 0.0;
        const int dz = iz - z1, dx = ix - x1;
        if (dz >= 0 && iz <= z2 && dx >= 0 && ix <= x2 && dz % sdz == 0 && dx % sdx == 0)
            return (double)gs[(long long)(dz / sdz) * snx_pitch + dx / sdx] * gs_un;
        return (double)wa[(long long)iz * pitch + ix] * wa_un;
    }
    __device__ double stage_b(int iz, int ix) const
    {
        const int dz = iz - z1, dx = ix - x1;
        if (sdx > 1 && dz >= 0 && iz < z2 && dz % sdz == 0 && dx > 0 && dx % sdx) {
            const int c0 = x1 + (dx / sdx) * sdx;
            if (c0 < x2) {
                const double a0 = stage_a(iz, c0), a1 = stage_a(iz, c0 + sdx);
                const double t = (a1 - a0) / sdx;
                return a0 + t * (dx % sdx);
            }
        }
        return stage_a(iz, ix);
    }
    __device__ double value(int iz, int ix) const
    {
        const int dz = iz - z1;
        if (sdz > 1 && ix >= x1 && ix < x2 && dz > 0 && dz % sdz) {
            const int r0 = z1 + (dz / sdz) * sdz;
            if (r0 < z2) {
                const double b0 = stage_b(r0, ix), b1 = stage_b(r0 + sdz, ix);
                const double t = (b1 - b0) / sdz;
                return b0 + t * (dz % sdz);
            }
        }
        return stage_b(iz, ix);
    }
};

// scale_grad_E2 (:760-783) for every shot of a batch, in shot order:
// grad += g / (We * C * C) with We = sqrt(We We_adj) + 0.005 max.
template <typename T>
__global__ void k_scale(const ScaleParams<T> s)
{
    const int ix = s.x1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = s.z1 + blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= s.x2 || iz >= s.z2) return;
    const long long i = (long long)iz * s.pitch + ix;
    const long long k = (long long)iz * s.nx + ix;
    double g0 = s.grad[0][k], g1 = s.grad[1][k], g2 = s.grad[2][k];
    for (int b = 0; b < s.nbatch; b++) {
        const T *f = s.fld + (long long)b * s.shot_stride;
        const double sf = s.fscale[s.s0 + b], sa = s.ascale[s.s0 + b];
        const double un = 1.0 / (sf * sa);
        const double we = (sqrt((double)f[F_WE * s.plane + i] * (double)f[F_WEA * s.plane + i]) +
                           0.005 * s.wmax[b]) * un;
        const double wa_un = 1.0 / (sa * sa);
        const T *gb = s.gshot + (long long)b * s.gshot_shot_stride;
        InterpView<T> v{gb, f + F_WEA * s.plane, s.pitch, s.snx_pitch, s.z1, s.z2,
                        s.x1, s.x2, s.sdz, s.sdx, s.gun[0] * un, wa_un, s.nz, s.nx};
        const double t0 = v.value(iz, ix);
        v.gs = gb + s.snap_plane;
        v.gs_un = s.gun[1] * un;
        const double t1 = v.value(iz, ix);
        v.gs = gb + 2 * s.snap_plane;
        v.gs_un = s.gun[2] * un;
        const double t2 = v.value(iz, ix);
        if (s.C[0] > 0) g0 += t0 / (we * s.C[0] * s.C[0]);
        if (s.C[1] > 0) g1 += t1 / (we * s.C[1] * s.C[1]);
        if (s.C[2] > 0) g2 += t2 / (we * s.C[2] * s.C[2]);
    }
    s.grad[0][k] = g0;
    s.grad[1][k] = g1;
    s.grad[2][k] = g2;
}

template <typename T>
cudaError_t launch_scale(const ScaleParams<T> &s, cudaStream_t st)
{
    if (s.z2 <= s.z1 || s.x2 <= s.x1 || s.nbatch <= 0) return cudaSuccess;
    dim3 b(32, 8), g((s.x2 - s.x1 + 31) / 32, (s.z2 - s.z1 + 7) / 8);
    k_scale<T><<<g, b, 0, st>>>(s);
    return cudaGetLastError();
}

// Per-shot max |r| of the residual traces, then the adjoint amplitude scale.
__global__ void k_shot_maxabs(const double *rz, const double *rx, long long n,
                              unsigned long long *bits)
{
    const long long off = (long long)blockIdx.y * n;
    double m = 0.0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        m = fmax(m, fmax(fabs(rz[off + k]), fabs(rx[off + k])));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0)
        atomicMax(&bits[blockIdx.y], (unsigned long long)__double_as_longlong(m));
}

__global__ void k_adj_scale(const unsigned long long *bits, int nshot, double inj, double *ascale)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nshot) return;
    const double r = __longlong_as_double((long long)bits[s]) * inj;
    ascale[s] = (r > 0.0 && isfinite(r)) ? exp2(-rint(log2(r))) : 1.0;
}

cudaError_t launch_adjoint_scale(const double *res_z, const double *res_x, long long n_per_shot,
                                 int nshot, double inj, unsigned long long *rmax_bits,
                                 double *ascale, cudaStream_t st)
{
    if (nshot <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(rmax_bits, 0, nshot * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    if (n_per_shot > 0) k_shot_maxabs<<<dim3(64, nshot), 256, 0, st>>>(res_z, res_x, n_per_shot, rmax_bits);
    k_adj_scale<<<(nshot + 127) / 128, 128, 0, st>>>(rmax_bits, nshot, inj, ascale);
    return cudaGetLastError();
}

// taper2 (src/cpu/n_kernel_lib_PSV.cpp:942-1010): the horizontal then the
// vertical Tukey factor, precomputed on the host (1 where no branch applies).
__global__ void k_taper(double *A, int nz, int nx, const double *tx, const double *tz)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = blockIdx.y * blockDim.y + threadIdx.y;
    if (ix >= nx || iz >= nz) return;
    const long long k = (long long)iz * nx + ix;
    double a = A[k];
    a *= tx[ix];
    a *= tz[iz];
    A[k] = a;
}

cudaError_t launch_taper(double *A, int nz, int nx, const double *tx, const double *tz,
                         cudaStream_t st)
{
    dim3 b(32, 8), g((nx + 31) / 32, (nz + 7) / 8);
    k_taper<<<g, b, 0, st>>>(A, nz, nx, tx, tz);
    return cudaGetLastError();
}

// update_mat2 (src/cpu/n_kernel_lib_PSV.cpp:785-832).
__global__ void k_maxabs(const double *grad, const double *old, int n, unsigned long long *bits2)
{
    double g = 0.0, m = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        g = fmax(g, fabs(grad[k]));
        m = fmax(m, fabs(old[k]));
    }
    for (int o = 16; o > 0; o >>= 1) {
        g = fmax(g, __shfl_xor_sync(0xffffffffu, g, o));
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&bits2[0], (unsigned long long)__double_as_longlong(g));
        atomicMax(&bits2[1], (unsigned long long)__double_as_longlong(m));
    }
}

__global__ void k_update(double *mat, const double *old, const double *grad, int n,
                         double mat_max, double mat_min, double step,
                         const unsigned long long *bits2)
{
    const double grad_max = __longlong_as_double((long long)bits2[0]);
    double mat_array_max = __longlong_as_double((long long)bits2[1]);
    if (mat_array_max < mat_max) mat_array_max = mat_max;
    const double step_factor = mat_array_max / grad_max;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        double v = old[k] + step * step_factor * grad[k];
        if (v > mat_max) v = mat_max;
        if (v < mat_min) v = mat_min;
        mat[k] = v;
    }
}

cudaError_t launch_update_mat(double *mat, const double *old, const double *grad, int n,
                              double mat_max, double mat_min, double step,
                              unsigned long long *maxbits2, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(maxbits2, 0, 2 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    const int blocks = 4 * 152;
    k_maxabs<<<blocks, 256, 0, st>>>(grad, old, n, maxbits2);
    k_update<<<blocks, 256, 0, st>>>(mat, old, grad, n, mat_max, mat_min, step, maxbits2);
    return cudaGetLastError();
}

// Zero `count` elements at offset `off` of each of nbatch shot blocks.
template <typename T>
__global__ void k_zero_planes(T *base, long long shot_stride, long long off, long long count)
{
    T *p = base + (long long)blockIdx.y * shot_stride + off;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < count;
         k += (long long)gridDim.x * blockDim.x)
        p[k] = T(0);
}

template <typename T>
cudaError_t launch_zero_planes(T *base, long long shot_stride, long long off, long long count,
                               int nbatch, cudaStream_t st)
{
    if (count <= 0 || nbatch <= 0 || !base) return cudaSuccess;
    long long blocks = (count + 1023) / 1024;
    if (blocks > 4 * 152) blocks = 4 * 152;
    k_zero_planes<T><<<dim3((unsigned)blocks, nbatch), 256, 0, st>>>(base, shot_stride, off, count);
    return cudaGetLastError();
}

// out[b][c][r] = in[b][r][c] for rows x cols matrices (trace layout changes
// between the reference's [rec][nt] and the engine's step-major [nt][rec]).
__global__ void k_transpose(const double *in, double *out, int rows, int cols)
{
    __shared__ double tile[32][33];
    const long long off = (long long)blockIdx.z * rows * cols;
    int c = blockIdx.x * 32 + threadIdx.x;
    int r = blockIdx.y * 32 + threadIdx.y;
    for (int j = 0; j < 32; j += 8)
        if (c < cols && r + j < rows) tile[threadIdx.y + j][threadIdx.x] = in[off + (long long)(r + j) * cols + c];
    __syncthreads();
    c = blockIdx.y * 32 + threadIdx.x;
    r = blockIdx.x * 32 + threadIdx.y;
    for (int j = 0; j < 32; j += 8)
        if (c < rows && r + j < cols) out[off + (long long)(r + j) * rows + c] = tile[threadIdx.x][threadIdx.y + j];
}

cudaError_t launch_transpose(const double *in, double *out, int rows, int cols, int nbatch,
                             cudaStream_t st)
{
    if (rows <= 0 || cols <= 0 || nbatch <= 0) return cudaSuccess;
    dim3 b(32, 8), g((cols + 31) / 32, (rows + 31) / 32, nbatch);
    k_transpose<<<g, b, 0, st>>>(in, out, rows, cols);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Optional preconditioners: Gaussian smoothing and the Fletcher-Reeves
// direction (gauss_filter_kernel / apply_gauss_filter,
// src/cpu/n_kernel_lib_PSV.cpp:1012-1084; PCG_PSV, src/cpu/n_PCG_PSV.cpp:13-44).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_gauss_filter(const T *src, T *dst, long long plane, int pitch, int nz, int nx,
                               const double *filt, int hfs)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x, iz = blockIdx.y * blockDim.y + threadIdx.y;
    if (iz < hfs || iz >= nz - hfs - 1 || ix < hfs || ix >= nx - hfs - 1) return;
    const T *s = src + (long long)blockIdx.z * plane;
    const int n = 2 * hfs + 1;
    double conv = 0.0;  // the reference's int accumulator truncates; see the header
    for (int jj = 0; jj < n; jj++) {
        const T *row = s + (long long)(iz + jj - hfs) * pitch + ix - hfs;
        for (int ii = 0; ii < n; ii++) conv += (double)row[ii] * filt[jj * n + ii];
    }
    dst[(long long)blockIdx.z * plane + (long long)iz * pitch + ix] = (T)conv;
}

template <typename T>
cudaError_t launch_gauss_filter(const T *src, T *dst, long long plane, int pitch, int nz, int nx,
                                int nplanes, const double *filt, int hfs, cudaStream_t st)
{
    if (nplanes <= 0 || nz <= 0 || nx <= 0) return cudaSuccess;
    const dim3 b(32, 8), g((nx + 31) / 32, (nz + 7) / 8, nplanes);
    k_gauss_filter<T><<<g, b, 0, st>>>(src, dst, plane, pitch, nz, nx, filt, hfs);
    return cudaGetLastError();
}

// Block partial sums of g^2 and old^2 (fixed grid: the same order every run).
__global__ void k_pcg_sums(const double *g, const double *old, long long n, double *part)
{
    __shared__ double sa[256], sb[256];
    double a = 0.0, b = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        a += g[i] * g[i];
        b += old[i] * old[i];
    }
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            sa[threadIdx.x] += sa[threadIdx.x + h];
            sb[threadIdx.x] += sb[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[blockIdx.x] = sa[0];
        part[gridDim.x + blockIdx.x] = sb[0];
    }
}

__global__ void k_pcg_apply(double *dir, double *old, double *g, long long n, const double *part)
{
    __shared__ double beta;
    if (threadIdx.x == 0) {  // every block sums the partials in the same order
        double bi = 0.0, bj = 0.0;
        for (int k = 0; k < (int)gridDim.x; k++) {
            bi += part[k];
            bj += part[gridDim.x + k];
        }
        double b = bj > 0.0 ? bi / bj : 0.0;  // the reference divides by zero on its first call
        beta = b > 0 ? b : 0.0;
    }
    __syncthreads();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double gi = g[i];
        old[i] = -gi;
        const double d = -gi + beta * dir[i];
        dir[i] = d;
        g[i] = d;
    }
}

cudaError_t launch_pcg(double *dir, double *old, double *g, long long n, double *part,
                       cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_pcg_sums<<<PCG_BLOCKS, 256, 0, st>>>(g, old, n, part);
    k_pcg_apply<<<PCG_BLOCKS, 256, 0, st>>>(dir, old, g, n, part);
    return cudaGetLastError();
}

template cudaError_t launch_gauss_filter<float>(const float *, float *, long long, int, int, int,
                                                int, const double *, int, cudaStream_t);
template cudaError_t launch_gauss_filter<double>(const double *, double *, long long, int, int,
                                                 int, int, const double *, int, cudaStream_t);
template cudaError_t launch_zero_planes<float>(float *, long long, long long, long long, int,
                                               cudaStream_t);
template cudaError_t launch_zero_planes<double>(double *, long long, long long, long long, int,
                                                cudaStream_t);
template cudaError_t launch_coeffs<float>(const CoeffParams<float> &, cudaStream_t);
template cudaError_t launch_coeffs<double>(const CoeffParams<double> &, cudaStream_t);
template cudaError_t launch_energy_max<float>(const float *, long long, long long, int, int, int,
                                              int, int, int, double *, cudaStream_t);
template cudaError_t launch_energy_max<double>(const double *, long long, long long, int, int,
                                               int, int, int, int, double *, cudaStream_t);
template cudaError_t launch_scale<float>(const ScaleParams<float> &, cudaStream_t);
template cudaError_t launch_scale<double>(const ScaleParams<double> &, cudaStream_t);

}  // namespace psv
