// Smooth particle-mesh Ewald: the reciprocal-space half of the Ewald sum whose
// real-space half is the cluster-pair kernel.
//
// Restates, for one rectangular box on one GPU and pme_order 4, the reference's PME path:
//  - grid sizes (calcFftGrid, src/gromacs/fft/calcgrid.cpp:63-160, with
//    minimalPmeGridSize, src/gromacs/ewald/pme.cpp:488-500);
//  - fractional coordinates and gridline indices (calc_interpolation_idx,
//    src/gromacs/ewald/pme_spread.cpp:65-140 with make_gridindex_to_localindex,
//    pme_grid.cpp:779-830 on one rank: t = n (x / L + 2), index = (int)t mod n);
//  - the B-spline weights and derivatives (CALC_SPLINE(4), pme_spread.cpp:220-266);
//  - spreading q theta_x theta_y theta_z onto the points index + 0..3, periodic
//    (spread_coefficients_bsplines_thread + wrap_periodic_pmegrid);
//  - the spline moduli (make_bspline_moduli / make_dft_mod,
//    src/gromacs/ewald/calculate_spline_moduli.cpp:52-122);
//  - the reciprocal solve with energy and virial (solve_pme_yzx,
//    src/gromacs/ewald/pme_solve.cpp:332-587);
//  - the force gather (gather_f_bsplines / do_fspline,
//    src/gromacs/ewald/pme_gather.cpp:78-360).
// The 3-D real<->complex transforms are hand-written (nbx_fft.cu: one warp per line, Stockham
// stages; unnormalised both ways, like the reference's).  Spreading accumulates with float atomics (16-byte vector reductions
// when nz is a multiple of 4); the energy and the virial terms are summed per warp in
// float and across the grid in FP64.
//
// Layouts in device memory: real grid [nx][ny][nz] (z fastest); half-complex grid
// [nx][ny][nz/2+1] of float2 (the usual real-to-complex layout), so the complex index
// (kx, ky, kz) is the reference's (x, y, z) complex-grid cell with z halved.
#include "../../include/nbnxm_gb300.h"
#include "nbx_internal.cuh"

#include "nbx_fft.cuh"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <type_traits>
#include <vector>

namespace
{

constexpr int kOrder = 4;  // pme_order (grid points per dimension and atom)

struct PmeDims
{
    int   n[3];
    float rec[3];  // recipbox diagonal: 1 / box edge (invertBoxMatrix, math/invertmatrix.cpp:62-64)
};

// CALC_SPLINE(4) for the fraction dr: weights th[0..3] and derivatives dth[0..3]
__device__ __forceinline__ void bspline4(float dr, float th[4], float dth[4])
{
    float d0 = 1.0f - dr, d1 = dr, d2;
    d2 = __fmul_rn(__fmul_rn(0.5f, dr), d1);
    d1 = __fmul_rn(0.5f, __fadd_rn(__fmul_rn(dr + 1.0f, d0), __fmul_rn(2.0f - dr, d1)));
    d0 = __fmul_rn(__fmul_rn(0.5f, 1.0f - dr), d0);
    dth[0] = -d0;
    dth[1] = d0 - d1;
    dth[2] = d1 - d2;
    dth[3] = d2;
    const float div = 1.0f / 3.0f;
    th[3]           = __fmul_rn(__fmul_rn(div, dr), d2);
    th[2]           = __fmul_rn(div, __fadd_rn(__fmul_rn(dr + 1.0f, d1), __fmul_rn(3.0f - dr, d2)));
    th[1]           = __fmul_rn(div, __fadd_rn(__fmul_rn(dr + 2.0f, d0), __fmul_rn(2.0f - dr, d1)));
    th[0]           = __fmul_rn(__fmul_rn(div, 1.0f - dr), d0);
}

// gridline index ((int)t mod n) and fraction of one coordinate, t = n (x / L + 2)
__device__ __forceinline__ int interp_index(float x, float rec, int n, float* frac)
{
    const float t  = __fmul_rn((float)n, __fadd_rn(__fmul_rn(x, rec), 2.0f));  // c_pmeMaxUnitcellShift = 2
    const int   ti = (int)floorf(t);  // the reference's truncation for t >= 0
    *frac          = t - (float)ti;
    const int i    = ti % n;
    return i < 0 ? i + n : i;
}

struct AtomSplines
{
    int   i0[3];
    float th[3][kOrder];
    float dth[3][kOrder];
};

__device__ __forceinline__ void atom_splines(const PmeDims& d, const float* __restrict__ x, int a, AtomSplines& s)
{
    for (int k = 0; k < 3; k++)
    {
        float fr;
        s.i0[k] = interp_index(x[3 * a + k], d.rec[k], d.n[k], &fr);
        bspline4(fr, s.th[k], s.dth[k]);
    }
}

__device__ __forceinline__ int wrap_once(int i, int n)
{
    return i >= n ? i - n : i;
}

// Spline data in the reference's test layout: idx [N][3], theta/dtheta [3][N][4].
__global__ void k_pme_splines(PmeDims d, int natoms, const float* __restrict__ x, int* idx, float* theta,
                              float* dtheta)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natoms)
    {
        return;
    }
    AtomSplines s;
    atom_splines(d, x, a, s);
    for (int k = 0; k < 3; k++)
    {
        idx[3 * a + k] = s.i0[k];
        for (int o = 0; o < kOrder; o++)
        {
            theta[((size_t)k * natoms + a) * kOrder + o]  = s.th[k][o];
            dtheta[((size_t)k * natoms + a) * kOrder + o] = s.dth[k][o];
        }
    }
}

__device__ __forceinline__ void red_add_v4(float* addr, float a, float b, float c, float d)
{
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d));
}

// The four z points gz0..gz0+3 of one (x, y) grid row as 16-byte vector reductions:
// with nz a multiple of 4 (and a 16-byte aligned grid) they fall in the aligned blocks
// [gz0 & ~3, +4) and the next one (periodic), which receive the weights shifted by gz0 & 3.
__device__ __forceinline__ void spread_row_v4(float* row, int gz0, int nz, const float w[4])
{
    const int a  = gz0 & 3;
    float*    pa = row + (gz0 - a);
    float*    pb = row + (gz0 - a + 4 == nz ? 0 : gz0 - a + 4);
    switch (a)
    {
        case 0: red_add_v4(pa, w[0], w[1], w[2], w[3]); break;
        case 1:
            red_add_v4(pa, 0.0f, w[0], w[1], w[2]);
            red_add_v4(pb, w[3], 0.0f, 0.0f, 0.0f);
            break;
        case 2:
            red_add_v4(pa, 0.0f, 0.0f, w[0], w[1]);
            red_add_v4(pb, w[2], w[3], 0.0f, 0.0f);
            break;
        default:
            red_add_v4(pa, 0.0f, 0.0f, 0.0f, w[0]);
            red_add_v4(pb, w[1], w[2], w[3], 0.0f);
            break;
    }
}

// Four threads per atom (one x point each); each adds its 4 x 4 (y, z) weights.
template<bool kVec>
__global__ void k_pme_spread(PmeDims d, int natoms, const float* __restrict__ x, const float* __restrict__ q,
                             float* grid)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int a = t >> 2, ix = t & 3;
    if (a >= natoms)
    {
        return;
    }
    const float qa = q[a];
    if (qa == 0.0f)
    {
        return;
    }
    AtomSplines s;
    atom_splines(d, x, a, s);
    const int   gx = wrap_once(s.i0[0] + ix, d.n[0]);
    const float vx = qa * s.th[0][ix];
    int         gz[kOrder];
    for (int iz = 0; iz < kOrder; iz++)
    {
        gz[iz] = wrap_once(s.i0[2] + iz, d.n[2]);
    }
    for (int iy = 0; iy < kOrder; iy++)
    {
        const int   gy  = wrap_once(s.i0[1] + iy, d.n[1]);
        const float vxy = vx * s.th[1][iy];
        float*      row = grid + ((size_t)gx * d.n[1] + gy) * d.n[2];
        float       w[kOrder];
        for (int iz = 0; iz < kOrder; iz++)
        {
            w[iz] = vxy * s.th[2][iz];
        }
        if (kVec)
        {
            spread_row_v4(row, s.i0[2], d.n[2], w);
        }
        else
        {
            for (int iz = 0; iz < kOrder; iz++)
            {
                atomicAdd(&row[gz[iz]], w[iz]);
            }
        }
    }
}

constexpr int kSolveThreads   = 256;
constexpr int kSolveMaxBlocks = 4096;  // one point per thread up to 1M points, grid-stride above
// With energies, 4 blocks per SM (grid-stride): each block adds once to the completion
// counter, and thousands of same-address atomics would serialise in L2.
constexpr int kSolveEnergyBlocksPerSm = 4;

// The solve's energy / virial sums: per warp in float, per block in FP64 into partials[block][8];
// the last block to finish (completion counter) adds the partials in FP64 and writes
// energy = 0.5 sum, virial = 0.25 sum.
__device__ void solve_finish(const float acc[7], double* partials, unsigned int* done, double* energy_out,
                             double* virial_out)
{
    __shared__ double red[7][kSolveThreads / 32];
    __shared__ bool   last;
    const int         lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 7; k++)
    {
        float v = acc[k];
        for (int o = 16; o > 0; o >>= 1)
        {
            v += __shfl_xor_sync(0xffffffffu, v, o);
        }
        if (lane == 0)
        {
            red[k][warp] = (double)v;
        }
    }
    __syncthreads();
    if (threadIdx.x < 7)
    {
        double v = 0.0;
        for (int w = 0; w < kSolveThreads / 32; w++)
        {
            v += red[threadIdx.x][w];
        }
        partials[blockIdx.x * 8 + threadIdx.x] = v;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last)
    {
        return;
    }
    // the last block: FP64 sum of every block's partials
    __threadfence();
    double sum[7] = { 0, 0, 0, 0, 0, 0, 0 };
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
    {
        for (int k = 0; k < 7; k++)
        {
            sum[k] += __ldcg(&partials[b * 8 + k]);
        }
    }
    __syncthreads();
    for (int k = 0; k < 7; k++)
    {
        double v = sum[k];
        for (int o = 16; o > 0; o >>= 1)
        {
            v += __shfl_xor_sync(0xffffffffu, v, o);
        }
        if (lane == 0)
        {
            red[k][warp] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double tot[7];
        for (int k = 0; k < 7; k++)
        {
            tot[k] = 0.0;
            for (int w = 0; w < kSolveThreads / 32; w++)
            {
                tot[k] += red[k][w];
            }
        }
        if (energy_out)
        {
            energy_out[0] = 0.5 * tot[0];
        }
        if (virial_out)
        {
            virial_out[0]                 = 0.25 * tot[1];
            virial_out[1] = virial_out[3] = 0.25 * tot[2];
            virial_out[2] = virial_out[6] = 0.25 * tot[3];
            virial_out[4]                 = 0.25 * tot[4];
            virial_out[5] = virial_out[7] = 0.25 * tot[5];
            virial_out[8]                 = 0.25 * tot[6];
        }
        *done = 0u;  // ready for the next solve on this stream
    }
}

// One point (kx, ky, kz) != 0 of solve_pme_yzx (pme_solve.cpp:332-587): scales c by eterm and, with
// energies, adds its energy and virial terms to acc.
__device__ __forceinline__ void solve_point(const PmeDims& d, const float* __restrict__ bsp, float elfac, float factor,
                                            float pivol, int kx, int ky, int kz, bool energy, float2& c, float acc[7])
{
    const int   mx    = kx < (d.n[0] + 1) / 2 ? kx : kx - d.n[0];
    const int   my    = ky < (d.n[1] + 1) / 2 ? ky : ky - d.n[1];
    const float mhx   = (float)mx * d.rec[0];
    const float mhy   = (float)my * d.rec[1];
    const float mhz   = (float)kz * d.rec[2];
    const float m2    = mhx * mhx + mhy * mhy + mhz * mhz;
    const float by    = pivol * bsp[d.n[0] + ky];
    const float den   = m2 * bsp[d.n[0] + d.n[1] + kz] * by * bsp[kx];
    const float eterm = elfac / den * expf(-factor * m2);
    if (energy)
    {
        const float corner  = (kz == 0 || kz == (d.n[2] + 1) / 2) ? 0.5f : 1.0f;
        const float struct2 = 2.0f * (c.x * c.x + c.y * c.y);
        const float ets2    = corner * eterm * struct2;
        const float ets2vf  = ets2 * ((factor * m2 + 1.0f) * 2.0f / m2);
        acc[0] += ets2;
        acc[1] += ets2vf * mhx * mhx - ets2;
        acc[2] += ets2vf * mhx * mhy;
        acc[3] += ets2vf * mhx * mhz;
        acc[4] += ets2vf * mhy * mhy - ets2;
        acc[5] += ets2vf * mhy * mhz;
        acc[6] += ets2vf * mhz * mhz - ets2;
    }
    c.x *= eterm;
    c.y *= eterm;
}

// The x transform of the forward FFT, the solve and the x transform of the backward FFT in one
// pass over the half-complex grid (the x lines are the last forward and the first backward
// transform): block (ky, z-tile) loads the tile [nx][T] of x lines, warp c transforms column c,
// solves its points (kx, ky, kz = tile * T + c) and transforms it back; energy and virial sums as
// k_pme_solve's.
template<bool kEnergy, int kN>
__global__ void __launch_bounds__(kSolveThreads, 6) k_pme_fft_x_solve(nbx::FftAxis ax, PmeDims d, float2* cgrid,
                                                                   const float* __restrict__ bsp, float elfac,
                                                                   float factor, float pivol, int ntiles, double* partials,
                                                                   unsigned int* done, double* energy_out,
                                                                   double* virial_out)
{
    constexpr int T    = nbx::kFftTile;
    extern __shared__ float2 xsm[];
    const int     n    = kN > 0 ? kN : ax.n;  // nx
    const int     nzc  = d.n[2] / 2 + 1;
    float2*       W    = xsm;
    float2*       tile = xsm + n;                  // [n][T + 1]
    float2*       scr  = tile + (size_t)n * (T + 1);  // [T][n]
    const int     ky   = blockIdx.x / ntiles;
    const int     t    = blockIdx.x - ky * ntiles;
    const int     warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t  base = (size_t)ky * nzc + (size_t)t * T;
    const size_t  es   = (size_t)d.n[1] * nzc;
    const int     cols = min(T, nzc - t * T);
    for (int k = threadIdx.x; k < n; k += blockDim.x)
    {
        W[k] = ax.roots[k];
    }
    for (int idx = threadIdx.x; idx < n * T; idx += blockDim.x)
    {
        const int i = idx / T, c = idx - i * T;
        tile[i * (T + 1) + c] = c < cols ? cgrid[base + (size_t)i * es + c] : make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    float acc[7] = { 0, 0, 0, 0, 0, 0, 0 };
    if (warp < cols)
    {
        float2*   col = tile + warp;
        float2*   s   = scr + (size_t)warp * n;
        const int kz  = t * T + warp;
        // forward along x, then the solve on the column wherever the transform left it
        const bool in_s = nbx::fft_line_any<kN, false>(col, T + 1, s, 1, W, ax, lane);
        float2*    v    = in_s ? s : col;
        const int  vs   = in_s ? 1 : T + 1;
        for (int kx = lane; kx < n; kx += 32)
        {
            if (kx != 0 || ky != 0 || kz != 0)
            {
                float2 c = v[kx * vs];
                solve_point(d, bsp, elfac, factor, pivol, kx, ky, kz, kEnergy, c, acc);
                v[kx * vs] = c;
            }
        }
        __syncwarp();
        // backward along x
        float2*    other = in_s ? col : s;
        const int  os    = in_s ? T + 1 : 1;
        const bool moved = nbx::fft_line_any<kN, true>(v, vs, other, os, W, ax, lane);
        // the result is in `other` when moved; bring it to the tile column
        if (moved != in_s)
        {
            // result in s
            for (int i = lane; i < n; i += 32)
            {
                col[i * (T + 1)] = s[i];
            }
        }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * T; idx += blockDim.x)
    {
        const int i = idx / T, c = idx - i * T;
        if (c < cols)
        {
            cgrid[base + (size_t)i * es + c] = tile[i * (T + 1) + c];
        }
    }
    if (kEnergy)
    {
        solve_finish(acc, partials, done, energy_out, virial_out);
    }
}

// solve_pme_yzx over the half-complex grid: scales each element by eterm and sums the
// energy and virial terms (energy = 0.5 sum, virial = 0.25 sum).  Per-point terms and
// per-thread / per-warp sums are float (the reference sums them in `real`); each block
// writes its 7 sums in FP64 to partials[block][8] and the last block to finish sums the
// partials in FP64 (no same-address atomics on the sums).
__global__ void __launch_bounds__(kSolveThreads) k_pme_solve(PmeDims d, float2* cgrid, const float* __restrict__ bsp,
                                                             float elfac, float factor, float pivol, double* partials,
                                                             unsigned int* done, double* energy_out,
                                                             double* virial_out)
{
    const bool energy = energy_out || virial_out;
    const int  nzc    = d.n[2] / 2 + 1;
    const int  total  = d.n[0] * d.n[1] * nzc;
    float      acc[7] = { 0, 0, 0, 0, 0, 0, 0 };
    // (kx, ky, kz) of t, advanced by the grid stride with carries instead of divisions
    const int t0     = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    int       kz = t0 % nzc, ky = (t0 / nzc) % d.n[1], kx = t0 / (nzc * d.n[1]);
    const int sz = stride % nzc, sy = (stride / nzc) % d.n[1], sx = stride / (nzc * d.n[1]);
    for (int t = t0; t < total; t += stride)
    {
        if (kx != 0 || ky != 0 || kz != 0)
        {
            float2 c = cgrid[t];
            solve_point(d, bsp, elfac, factor, pivol, kx, ky, kz, energy, c, acc);
            cgrid[t] = c;
        }
        kz += sz;
        int carry = 0;
        if (kz >= nzc)
        {
            kz -= nzc;
            carry = 1;
        }
        ky += sy + carry;
        carry = 0;
        if (ky >= d.n[1])
        {
            ky -= d.n[1];
            carry = 1;
        }
        kx += sx + carry;
    }
    if (energy)
    {
        solve_finish(acc, partials, done, energy_out, virial_out);
    }
}

// solve_pme_lj_yzx, geometric combination rule (one grid; pme_solve.cpp:588-915): the
// dispersion influence function eterm = -((1 - 2 b) e^-b + 2 b sqrt(pi) sqrt(b) erfc(sqrt(b))) / D,
// b = pi^2 m^2 / beta_lj^2, D = B_x B_y B_z 3 V / (pi^1.5 beta_lj^3); the k = 0 element is
// scaled too.  Energy and virial sums as in k_pme_solve.
__global__ void __launch_bounds__(kSolveThreads) k_pme_solve_lj(PmeDims d, float2* cgrid,
                                                                const float* __restrict__ bsp, float factor,
                                                                float by_pref, double* partials, unsigned int* done,
                                                                double* energy_out, double* virial_out)
{
    const bool energy = energy_out || virial_out;
    const int  nzc    = d.n[2] / 2 + 1;
    const int  total  = d.n[0] * d.n[1] * nzc;
    float      acc[7] = { 0, 0, 0, 0, 0, 0, 0 };
    const int  t0     = blockIdx.x * blockDim.x + threadIdx.x;
    const int  stride = gridDim.x * blockDim.x;
    int        kz = t0 % nzc, ky = (t0 / nzc) % d.n[1], kx = t0 / (nzc * d.n[1]);
    const int  sz = stride % nzc, sy = (stride / nzc) % d.n[1], sx = stride / (nzc * d.n[1]);
    for (int t = t0; t < total; t += stride)
    {
        const int   mx    = kx < (d.n[0] + 1) / 2 ? kx : kx - d.n[0];
        const int   my    = ky < (d.n[1] + 1) / 2 ? ky : ky - d.n[1];
        const float mhx   = (float)mx * d.rec[0];
        const float mhy   = (float)my * d.rec[1];
        const float mhz   = (float)kz * d.rec[2];
        const float m2    = mhx * mhx + mhy * mhy + mhz * mhz;
        const float den   = bsp[d.n[0] + d.n[1] + kz] * (by_pref * bsp[d.n[0] + ky]) * bsp[kx];
        const float b     = factor * m2;
        const float e1    = expf(-b);
        const float mk    = sqrtf(b);
        const float e2    = 1.7724538509055159f * mk * erfcf(mk);
        const float eterm = -((1.0f - 2.0f * b) * e1 + 2.0f * b * e2) / den;
        float2      c     = cgrid[t];
        if (energy)
        {
            const float vterm   = 3.0f * (-e1 + e2) / den;
            const float corner  = (kz == 0 || kz == (d.n[2] + 1) / 2) ? 0.5f : 1.0f;
            const float struct2 = 2.0f * (c.x * c.x + c.y * c.y);
            const float ets2    = corner * eterm * struct2;
            const float ets2vf  = corner * 2.0f * factor * vterm * struct2;
            acc[0] += ets2;
            acc[1] += ets2vf * mhx * mhx - ets2;
            acc[2] += ets2vf * mhx * mhy;
            acc[3] += ets2vf * mhx * mhz;
            acc[4] += ets2vf * mhy * mhy - ets2;
            acc[5] += ets2vf * mhy * mhz;
            acc[6] += ets2vf * mhz * mhz - ets2;
        }
        c.x *= eterm;
        c.y *= eterm;
        cgrid[t] = c;
        kz += sz;
        int carry = 0;
        if (kz >= nzc)
        {
            kz -= nzc;
            carry = 1;
        }
        ky += sy + carry;
        carry = 0;
        if (ky >= d.n[1])
        {
            ky -= d.n[1];
            carry = 1;
        }
        kx += sx + carry;
    }
    if (energy)
    {
        solve_finish(acc, partials, done, energy_out, virial_out);
    }
}

// Forces from the potential grid (do_fspline + gather_f_bsplines), added to f.
__global__ void k_pme_gather(PmeDims d, int natoms, const float* __restrict__ x, const float* __restrict__ q,
                             const float* __restrict__ grid, float* f)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= natoms)
    {
        return;
    }
    const float qa = q[a];
    if (qa == 0.0f)
    {
        return;
    }
    AtomSplines s;
    atom_splines(d, x, a, s);
    int gz[kOrder];
    for (int iz = 0; iz < kOrder; iz++)
    {
        gz[iz] = wrap_once(s.i0[2] + iz, d.n[2]);
    }
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    for (int ix = 0; ix < kOrder; ix++)
    {
        const int gx = wrap_once(s.i0[0] + ix, d.n[0]);
        for (int iy = 0; iy < kOrder; iy++)
        {
            const int    gy  = wrap_once(s.i0[1] + iy, d.n[1]);
            const float* row = grid + ((size_t)gx * d.n[1] + gy) * d.n[2];
            float        sz = 0.0f, sdz = 0.0f;
            for (int iz = 0; iz < kOrder; iz++)
            {
                const float g = __ldg(&row[gz[iz]]);
                sz            = fmaf(s.th[2][iz], g, sz);
                sdz           = fmaf(s.dth[2][iz], g, sdz);
            }
            fx = fmaf(s.dth[0][ix] * s.th[1][iy], sz, fx);
            fy = fmaf(s.th[0][ix] * s.dth[1][iy], sz, fy);
            fz = fmaf(s.th[0][ix] * s.th[1][iy], sdz, fz);
        }
    }
    f[3 * a + 0] -= qa * (fx * (float)d.n[0] * d.rec[0]);
    f[3 * a + 1] -= qa * (fy * (float)d.n[1] * d.rec[1]);
    f[3 * a + 2] -= qa * (fz * (float)d.n[2] * d.rec[2]);
}

// calcFftGrid for one dimension: the smallest listed size with spacing <= the target
int fft_grid_size(float length, float spacing)
{
    static const int init[] = { 6, 8, 10, 12, 14, 16, 20, 24, 25, 28, 32, 36, 40, 42, 44 };
    static const int base[] = { 45, 48, 50, 52, 54, 56, 60, 64, 70, 72, 75, 80, 81, 84 };
    const int        ninit  = (int)(sizeof(init) / sizeof(init[0]));
    const int        nbase  = (int)(sizeof(base) / sizeof(base[0]));
    const int        nmin   = std::max((int)((double)(length / spacing) + 0.999), 2 * (kOrder - 1));
    int              i      = ninit - 1;
    if (init[i] >= nmin)
    {
        while (i > 0 && init[i - 1] >= nmin)
        {
            i--;
        }
        return init[i];
    }
    int fac2 = 1;
    i        = nbase - 1;
    while (fac2 * base[i] < nmin)
    {
        fac2 *= 2;
    }
    int n = 0;
    do
    {
        const int attempt = fac2 * base[i];
        if (((attempt % 4 == 0 && attempt != 140) || attempt == 90) && attempt >= nmin)
        {
            n = attempt;
        }
        i--;
    } while (i > 0);
    return n;
}

// make_bspline_moduli + make_dft_mod for pme_order 4 (spline order 3)
void bspline_moduli(int n, float* mod)
{
    const int splineOrder  = kOrder - 1;
    double    data[kOrder] = { 1.0, 0.0, 0.0, 0.0 };
    for (int k = 2; k <= splineOrder; k++)
    {
        const double div = 1.0 / k;
        for (int m = k - 1; m > 0; m--)
        {
            data[m] = div * ((k - m) * data[m - 1] + (m + 1) * data[m]);
        }
        data[0] = div * data[0];
    }
    for (int i = 0; i < n; i++)
    {
        double sc = 0.0, ss = 0.0;
        for (int j = 0; j < splineOrder; j++)
        {
            const double arg = (2.0 * 3.14159265358979323846 * i * (j + 1)) / n;
            sc += data[j] * std::cos(arg);
            ss += data[j] * std::sin(arg);
        }
        mod[i] = (float)(sc * sc + ss * ss);
    }
    if (splineOrder % 2 == 0 && n % 2 == 0)
    {
        mod[n / 2] = (mod[n / 2 - 1] + mod[n / 2 + 1]) * 0.5f;
    }
}

thread_local std::string g_pme_error;

} // namespace

struct nbx_pme
{
    int          device     = 0;
    cudaStream_t stream     = nullptr;
    bool         own_stream = false;
    PmeDims      d{};
    float        box[3]    = { 0, 0, 0 };
    float        beta      = 0.0f;
    float        epsilon_r = 1.0f;
    int          lj        = 0;  // 1: the Lennard-Jones (dispersion) grid, coefficients sqrt(C6)
    float*       grid      = nullptr;  // real grid [nx][ny][nz]
    float2*      cgrid     = nullptr;  // half-complex grid [nx][ny][nz/2+1]
    float*       bsp       = nullptr;  // spline moduli x | y | z
    double*      sums      = nullptr;  // solve partials [kSolveMaxBlocks][8]: energy + 6 virial terms
    unsigned*    done      = nullptr;  // blocks of the running solve that have written their partials
    int          num_sms   = 1;
    nbx::FftPlan3 fft{};  // the hand-written 3D real <-> half-complex transform (nbx_fft.cu)
    bool          plan = false;
    bool          fused_smem_ok = false;  // the fused x pass + solve has its shared memory
    std::string  err;
};

namespace
{

int pme_error(nbx_pme* p, int code, const std::string& msg)
{
    (p ? p->err : g_pme_error) = msg;
    return code;
}

int cuda_status(nbx_pme* p, cudaError_t e)
{
    return e == cudaSuccess ? NBX_OK : pme_error(p, NBX_ERR_CUDA, cudaGetErrorString(e));
}

size_t real_points(const nbx_pme* p)
{
    return (size_t)p->d.n[0] * p->d.n[1] * p->d.n[2];
}

size_t complex_points(const nbx_pme* p)
{
    return (size_t)p->d.n[0] * p->d.n[1] * (p->d.n[2] / 2 + 1);
}

cudaError_t launch_spread(nbx_pme* p, int natoms, const float* d_x, const float* d_q, float* grid)
{
    cudaError_t e = cudaMemsetAsync(grid, 0, sizeof(float) * real_points(p), p->stream);
    if (e != cudaSuccess || natoms == 0)
    {
        return e;
    }
    const int  blocks = (int)((4LL * natoms + 255) / 256);
    const bool vec    = p->d.n[2] % 4 == 0 && (reinterpret_cast<uintptr_t>(grid) & 15) == 0;
    if (vec)
    {
        k_pme_spread<true><<<blocks, 256, 0, p->stream>>>(p->d, natoms, d_x, d_q, grid);
    }
    else
    {
        k_pme_spread<false><<<blocks, 256, 0, p->stream>>>(p->d, natoms, d_x, d_q, grid);
    }
    return cudaGetLastError();
}

cudaError_t launch_solve(nbx_pme* p, float2* cgrid, double* d_energy, double* d_virial)
{
    const double vol     = (double)p->box[0] * p->box[1] * p->box[2];
    const int    nc      = (int)complex_points(p);
    const int    cap     = (d_energy || d_virial) ? kSolveEnergyBlocksPerSm * p->num_sms : kSolveMaxBlocks;
    const int    nblocks = std::max(1, std::min((nc + kSolveThreads - 1) / kSolveThreads, cap));
    // factor = pi^2 / beta^2 (pme_solve.cpp:341,602), in float like `real`
    const float  factor  = (float)(M_PI * M_PI) / (p->beta * p->beta);
    if (p->lj)
    {
        // by = 3 V B_y / (pi sqrt(pi) beta^3) (pme_solve.cpp:664)
        const float by_pref = (float)(3.0 * vol / (M_PI * std::sqrt(M_PI) * (double)p->beta * p->beta * p->beta));
        k_pme_solve_lj<<<nblocks, kSolveThreads, 0, p->stream>>>(p->d, cgrid, p->bsp, factor, by_pref, p->sums,
                                                                 p->done, d_energy, d_virial);
        return cudaGetLastError();
    }
    // elfac = ONE_4PI_EPS0 / epsilon_r (pme_solve.cpp:354)
    const float elfac = (float)nbx::one_4pi_eps0() / p->epsilon_r;
    const float pivol = (float)M_PI * (float)vol;
    k_pme_solve<<<nblocks, kSolveThreads, 0, p->stream>>>(p->d, cgrid, p->bsp, elfac, factor, pivol, p->sums,
                                                          p->done, d_energy, d_virial);
    return cudaGetLastError();
}

// The fused x pass + Coulomb solve: one block per (ky, z-tile), the solve's partials sized for
// kSolveMaxBlocks blocks.
int x_solve_blocks(const nbx_pme* p)
{
    const int nzc = p->d.n[2] / 2 + 1;
    return p->d.n[1] * ((nzc + nbx::kFftTile - 1) / nbx::kFftTile);
}

bool fused_x_solve(const nbx_pme* p)
{
    return !p->lj && p->d.n[0] > 1 && x_solve_blocks(p) <= kSolveMaxBlocks && p->fused_smem_ok;
}

cudaError_t launch_x_solve(nbx_pme* p, double* d_energy, double* d_virial)
{
    const double vol    = (double)p->box[0] * p->box[1] * p->box[2];
    const float  factor = (float)(M_PI * M_PI) / (p->beta * p->beta);
    const float  elfac  = (float)nbx::one_4pi_eps0() / p->epsilon_r;
    const float  pivol  = (float)M_PI * (float)vol;
    const int    nzc    = p->d.n[2] / 2 + 1;
    const int    ntiles = (nzc + nbx::kFftTile - 1) / nbx::kFftTile;
    const size_t smem   = nbx::fft_tiled_smem(p->d.n[0]);
    const bool   energy = d_energy || d_virial;
    auto         go     = [&](auto kn) {
        constexpr int kN = decltype(kn)::value;
        if (energy)
        {
            k_pme_fft_x_solve<true, kN><<<x_solve_blocks(p), kSolveThreads, smem, p->stream>>>(
                    p->fft.ax[0], p->d, p->cgrid, p->bsp, elfac, factor, pivol, ntiles, p->sums, p->done, d_energy,
                    d_virial);
        }
        else
        {
            k_pme_fft_x_solve<false, kN><<<x_solve_blocks(p), kSolveThreads, smem, p->stream>>>(
                    p->fft.ax[0], p->d, p->cgrid, p->bsp, elfac, factor, pivol, ntiles, p->sums, p->done, nullptr,
                    nullptr);
        }
    };
    switch (p->d.n[0])
    {
#define NBX_FFT_CASE(L)                                                                                                \
    case L: go(std::integral_constant<int, L>{}); break;
        NBX_FFT_FIXED_LENGTHS(NBX_FFT_CASE)
#undef NBX_FFT_CASE
        default: go(std::integral_constant<int, 0>{}); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_gather(nbx_pme* p, int natoms, const float* d_x, const float* d_q, const float* grid, float* d_f)
{
    if (natoms == 0)
    {
        return cudaSuccess;
    }
    k_pme_gather<<<(natoms + 127) / 128, 128, 0, p->stream>>>(p->d, natoms, d_x, d_q, grid, d_f);
    return cudaGetLastError();
}

bool atoms_ok(int natoms, const void* a, const void* b)
{
    return natoms >= 0 && (natoms == 0 || (a && b));
}

} // namespace

extern "C" {

float nbx_ewald_coefficient(float rcoulomb, float ewald_rtol)
{
    if (!(rcoulomb > 0.0f))
    {
        return 0.0f;
    }
    return nbx::calc_ewaldcoeff_q(rcoulomb, ewald_rtol > 0.0f ? ewald_rtol : 1e-5f);
}

int nbx_pme_grid_size(const float* box, float spacing, int* n)
{
    if (!box || !n || !(spacing > 0.0f))
    {
        return pme_error(nullptr, NBX_ERR_INVALID_INPUT, "null argument or non-positive spacing");
    }
    for (int k = 0; k < 3; k++)
    {
        if (!(box[k] > 0.0f))
        {
            return pme_error(nullptr, NBX_ERR_INVALID_INPUT, "box edges must be positive");
        }
        n[k] = fft_grid_size(box[k], spacing);
    }
    return NBX_OK;
}

const char* nbx_pme_last_error(const nbx_pme* p)
{
    return p ? p->err.c_str() : g_pme_error.c_str();
}

int nbx_pme_create(const float* box, const int* grid, float ewaldcoeff_q, float epsilon_r, int device, nbx_pme** out)
{
    if (!box || !grid || !out || !(ewaldcoeff_q > 0.0f))
    {
        return pme_error(nullptr, NBX_ERR_INVALID_INPUT, "null argument or non-positive Ewald coefficient");
    }
    *out = nullptr;
    for (int k = 0; k < 3; k++)
    {
        if (!(box[k] > 0.0f) || grid[k] < 2 * (kOrder - 1) || grid[k] > 4096)
        {
            return pme_error(nullptr, NBX_ERR_INVALID_INPUT,
                             "box edges must be positive and grid sizes in [6, 4096] (minimalPmeGridSize)");
        }
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    {
        cudaGetLastError();
        return pme_error(nullptr, NBX_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= ndev)
    {
        return pme_error(nullptr, NBX_ERR_INVALID_INPUT, "device index out of range");
    }
    cudaSetDevice(device);
    nbx_pme* p   = new nbx_pme();
    p->device    = device;
    p->beta      = ewaldcoeff_q;
    p->epsilon_r = epsilon_r > 0.0f ? epsilon_r : 1.0f;
    for (int k = 0; k < 3; k++)
    {
        p->box[k]   = box[k];
        p->d.n[k]   = grid[k];
        p->d.rec[k] = 1.0f / box[k];
    }
    cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    p->own_stream = e == cudaSuccess;
    if (e == cudaSuccess) e = cudaMalloc(&p->grid, sizeof(float) * real_points(p));
    if (e == cudaSuccess) e = cudaMalloc(&p->cgrid, sizeof(float2) * complex_points(p));
    if (e == cudaSuccess) e = cudaMalloc(&p->bsp, sizeof(float) * (grid[0] + grid[1] + grid[2]));
    if (e == cudaSuccess) e = cudaMalloc(&p->sums, sizeof(double) * 8 * kSolveMaxBlocks);
    if (e == cudaSuccess) e = cudaMalloc(&p->done, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(p->done, 0, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess)
    {
        std::vector<float> mod(grid[0] + grid[1] + grid[2]);
        bspline_moduli(grid[0], mod.data());
        bspline_moduli(grid[1], mod.data() + grid[0]);
        bspline_moduli(grid[2], mod.data() + grid[0] + grid[1]);
        e = cudaMemcpy(p->bsp, mod.data(), sizeof(float) * mod.size(), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess)
    {
        const std::string msg = cudaGetErrorString(e);
        nbx_pme_destroy(p);
        return pme_error(nullptr, NBX_ERR_OUT_OF_MEMORY, "PME allocation: " + msg);
    }
    const cudaError_t fe = nbx::fft_plan_create(&p->fft, grid);
    p->plan              = (fe == cudaSuccess);
    if (p->plan)
    {
        const size_t xs  = nbx::fft_tiled_smem(grid[0]);
        p->fused_smem_ok = xs <= 48 * 1024
                           || (cudaFuncSetAttribute(k_pme_fft_x_solve<true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)xs) == cudaSuccess
                               && cudaFuncSetAttribute(k_pme_fft_x_solve<false, 0>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xs) == cudaSuccess);
    }
    if (!p->plan)
    {
        nbx_pme_destroy(p);
        return pme_error(nullptr, fe == cudaErrorInvalidValue ? NBX_ERR_INVALID_INPUT : NBX_ERR_CUDA,
                         fe == cudaErrorInvalidValue
                                 ? "FFT grid size: every dimension must be at most 1024 with prime factors of at most 255"
                                 : std::string("FFT plan: ") + cudaGetErrorString(fe));
    }
    *out = p;
    return NBX_OK;
}

int nbx_pme_create_lj(const float* box, const int* grid, float ewaldcoeff_lj, int device, nbx_pme** out)
{
    const int rc = nbx_pme_create(box, grid, ewaldcoeff_lj, 1.0f, device, out);
    if (rc == NBX_OK)
    {
        (*out)->lj = 1;
    }
    return rc;
}

float nbx_ewald_coefficient_lj(float rvdw, float ewald_rtol_lj)
{
    // calc_ewaldcoeff_lj (ewald/ewald_utils.cpp:76-115): exp(-x^2)(1 + x^2 + x^4/2) = rtol, x = beta rc
    if (!(rvdw > 0.0f))
    {
        return 0.0f;
    }
    const float rtol = ewald_rtol_lj > 0.0f ? ewald_rtol_lj : 1e-3f;
    auto        f    = [rvdw](float beta) {
        const float x2 = (beta * rvdw) * (beta * rvdw);
        return std::exp(-x2) * (1.0f + x2 + x2 * x2 / 2.0f);
    };
    float beta = 5.0f;
    int   i    = 0;
    do
    {
        i++;
        beta *= 2.0f;
    } while (f(beta) > rtol);
    const int n    = i + 60;
    float     low  = 0.0f, high = beta;
    for (i = 0; i < n; i++)
    {
        beta = (low + high) / 2.0f;
        if (f(beta) > rtol)
        {
            low = beta;
        }
        else
        {
            high = beta;
        }
    }
    return beta;
}

int nbx_pme_destroy(nbx_pme* p)
{
    if (!p)
    {
        return NBX_OK;
    }
    cudaSetDevice(p->device);
    if (p->stream)
    {
        cudaStreamSynchronize(p->stream);
    }
    if (p->plan)
    {
        nbx::fft_plan_destroy(&p->fft);
    }
    cudaFree(p->grid);
    cudaFree(p->cgrid);
    cudaFree(p->bsp);
    cudaFree(p->sums);
    cudaFree(p->done);
    if (p->own_stream)
    {
        cudaStreamDestroy(p->stream);
    }
    delete p;
    return NBX_OK;
}

int nbx_pme_set_stream(nbx_pme* p, void* s)
{
    if (!p)
    {
        return pme_error(nullptr, NBX_ERR_INVALID_INPUT, "null handle");
    }
    if (static_cast<cudaStream_t>(s) == p->stream)
    {
        return NBX_OK;
    }
    cudaSetDevice(p->device);
    cudaStreamSynchronize(p->stream);
    if (p->own_stream)
    {
        cudaStreamDestroy(p->stream);
    }
    p->stream     = static_cast<cudaStream_t>(s);
    p->own_stream = false;
    return NBX_OK;
}

int nbx_pme_get_info(const nbx_pme* p, int* grid, float* ewaldcoeff_q)
{
    if (!p)
    {
        return pme_error(nullptr, NBX_ERR_INVALID_INPUT, "null handle");
    }
    for (int k = 0; k < 3 && grid; k++)
    {
        grid[k] = p->d.n[k];
    }
    if (ewaldcoeff_q)
    {
        *ewaldcoeff_q = p->beta;
    }
    return NBX_OK;
}

int nbx_pme_splines_device(nbx_pme* p, int natoms, const float* d_x, int* d_idx, float* d_theta, float* d_dtheta)
{
    if (!p || !atoms_ok(natoms, d_x, d_idx) || (natoms > 0 && (!d_theta || !d_dtheta)))
    {
        return pme_error(p, NBX_ERR_INVALID_INPUT, "null argument or negative atom count");
    }
    cudaSetDevice(p->device);
    if (natoms == 0)
    {
        return NBX_OK;
    }
    k_pme_splines<<<(natoms + 127) / 128, 128, 0, p->stream>>>(p->d, natoms, d_x, d_idx, d_theta, d_dtheta);
    return cuda_status(p, cudaGetLastError());
}

int nbx_pme_spread_device(nbx_pme* p, int natoms, const float* d_x, const float* d_q, float* d_grid)
{
    if (!p || !atoms_ok(natoms, d_x, d_q) || !d_grid)
    {
        return pme_error(p, NBX_ERR_INVALID_INPUT, "null argument or negative atom count");
    }
    cudaSetDevice(p->device);
    return cuda_status(p, launch_spread(p, natoms, d_x, d_q, d_grid));
}

int nbx_pme_solve_device(nbx_pme* p, void* d_cgrid, double* d_energy, double* d_virial)
{
    if (!p || !d_cgrid)
    {
        return pme_error(p, NBX_ERR_INVALID_INPUT, "null argument");
    }
    cudaSetDevice(p->device);
    return cuda_status(p, launch_solve(p, static_cast<float2*>(d_cgrid), d_energy, d_virial));
}

int nbx_pme_gather_device(nbx_pme* p, int natoms, const float* d_x, const float* d_q, const float* d_grid, float* d_f)
{
    if (!p || !atoms_ok(natoms, d_x, d_q) || !d_grid || (natoms > 0 && !d_f))
    {
        return pme_error(p, NBX_ERR_INVALID_INPUT, "null argument or negative atom count");
    }
    cudaSetDevice(p->device);
    return cuda_status(p, launch_gather(p, natoms, d_x, d_q, d_grid, d_f));
}

struct nbx_fft3d
{
    int           device = 0;
    nbx::FftPlan3 plan{};
};

int nbx_fft3d_create(const int* grid, int device, nbx_fft3d** out)
{
    if (!grid || !out)
    {
        return pme_error(nullptr, NBX_ERR_INVALID_INPUT, "null argument");
    }
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess)
    {
        return pme_error(nullptr, NBX_ERR_NO_DEVICE, "no CUDA device " + std::to_string(device));
    }
    auto*             f = new nbx_fft3d;
    f->device           = device;
    const cudaError_t e = nbx::fft_plan_create(&f->plan, grid);
    if (e != cudaSuccess)
    {
        nbx::fft_plan_destroy(&f->plan);
        delete f;
        return pme_error(nullptr, e == cudaErrorInvalidValue ? NBX_ERR_INVALID_INPUT : NBX_ERR_CUDA,
                         e == cudaErrorInvalidValue
                                 ? "FFT grid size: every dimension must be at most 1024 with prime factors of at most 255"
                                 : std::string("FFT plan: ") + cudaGetErrorString(e));
    }
    *out = f;
    return NBX_OK;
}

int nbx_fft3d_destroy(nbx_fft3d* f)
{
    if (f)
    {
        cudaSetDevice(f->device);
        nbx::fft_plan_destroy(&f->plan);
        delete f;
    }
    return NBX_OK;
}

int nbx_fft3d_execute_device(nbx_fft3d* f, int direction, float* d_real, void* d_cgrid, void* stream)
{
    if (!f || !d_real || !d_cgrid || (direction != 1 && direction != -1))
    {
        return pme_error(nullptr, NBX_ERR_INVALID_INPUT, "null argument or direction other than +1 / -1");
    }
    cudaSetDevice(f->device);
    const auto        s = static_cast<cudaStream_t>(stream);
    const cudaError_t e = direction > 0 ? nbx::fft_r2c(f->plan, d_real, static_cast<float2*>(d_cgrid), s)
                                        : nbx::fft_c2r(f->plan, static_cast<float2*>(d_cgrid), d_real, s);
    return e == cudaSuccess ? NBX_OK : pme_error(nullptr, NBX_ERR_CUDA, cudaGetErrorString(e));
}

int nbx_pme_fft_device(nbx_pme* p, int direction, float* d_real, void* d_cgrid)
{
    if (!p || !d_real || !d_cgrid || (direction != 1 && direction != -1))
    {
        return pme_error(p, NBX_ERR_INVALID_INPUT, "null argument or direction other than +1 / -1");
    }
    cudaSetDevice(p->device);
    const cudaError_t e = direction > 0 ? nbx::fft_r2c(p->fft, d_real, static_cast<float2*>(d_cgrid), p->stream)
                                        : nbx::fft_c2r(p->fft, static_cast<float2*>(d_cgrid), d_real, p->stream);
    return cuda_status(p, e);
}

int nbx_pme_compute_device(nbx_pme* p, int natoms, const float* d_x, const float* d_q, float* d_f, double* d_energy,
                           double* d_virial)
{
    if (!p || !atoms_ok(natoms, d_x, d_q) || (natoms > 0 && !d_f))
    {
        return pme_error(p, NBX_ERR_INVALID_INPUT, "null argument or negative atom count");
    }
    cudaSetDevice(p->device);
    cudaError_t e = launch_spread(p, natoms, d_x, d_q, p->grid);
    if (e != cudaSuccess)
    {
        return cuda_status(p, e);
    }
    if (fused_x_solve(p))
    {
        // z and y forward, then x forward + solve + x backward in one pass, then y and z backward
        e = nbx::fft_r2c_zy(p->fft, p->grid, p->cgrid, p->stream);
        if (e == cudaSuccess)
        {
            e = launch_x_solve(p, d_energy, d_virial);
        }
        if (e == cudaSuccess)
        {
            e = nbx::fft_c2r_yz(p->fft, p->cgrid, p->grid, p->stream);
        }
        if (e != cudaSuccess)
        {
            return cuda_status(p, e);
        }
        return cuda_status(p, launch_gather(p, natoms, d_x, d_q, p->grid, d_f));
    }
    e = nbx::fft_r2c(p->fft, p->grid, p->cgrid, p->stream);
    if (e != cudaSuccess)
    {
        return cuda_status(p, e);
    }
    e = launch_solve(p, p->cgrid, d_energy, d_virial);
    if (e != cudaSuccess)
    {
        return cuda_status(p, e);
    }
    e = nbx::fft_c2r(p->fft, p->cgrid, p->grid, p->stream);
    if (e != cudaSuccess)
    {
        return cuda_status(p, e);
    }
    return cuda_status(p, launch_gather(p, natoms, d_x, d_q, p->grid, d_f));
}

int nbx_pme_synchronize(nbx_pme* p)
{
    if (!p)
    {
        return pme_error(nullptr, NBX_ERR_INVALID_INPUT, "null handle");
    }
    cudaSetDevice(p->device);
    return cuda_status(p, cudaStreamSynchronize(p->stream));
}

} // extern "C"
