// 3D real <-> half-complex FFT of the PME grids (plan, axis passes); the line transform is in
// nbx_fft.cuh.  Real grid [n0][n1][n2] (z fastest), half-complex [n0][n1][n2/2 + 1], unnormalised,
// exp(-2 pi i ...) forward and exp(+2 pi i ...) backward, as the reference's FFT wrapper
// (src/gromacs/fft/fft.h: gmx_fft_3d_real) and cuFFT's R2C / C2R define them.
#include "nbx_fft.cuh"

#include <cmath>
#include <vector>

namespace nbx
{
namespace
{

constexpr int kZWarps = 8;  // line pairs per block of the z passes

size_t z_smem(int n)
{
    return sizeof(float2) * ((size_t)n + (size_t)kZWarps * 2 * n);
}

size_t strided_smem(int n)
{
    return fft_tiled_smem(n);
}

int z_blocks(int nlines)
{
    return std::max(1, ((nlines + 1) / 2 + kZWarps - 1) / kZWarps);
}

__device__ __forceinline__ void load_roots(float2* W, const FftAxis& ax)
{
    for (int k = threadIdx.x; k < ax.n; k += blockDim.x)
    {
        W[k] = ax.roots[k];
    }
    __syncthreads();
}

// z forward: lines 2p and 2p + 1 of the real grid as one complex line a + i b, transformed, then
// A_k = (Z_k + conj Z_{n-k}) / 2 and B_k = (Z_k - conj Z_{n-k}) / 2i for k = 0 .. n/2.
template<int kN>
__global__ void __launch_bounds__(kZWarps * 32) k_fft_z_r2c(FftAxis ax, const float* __restrict__ real,
                                                            float2* __restrict__ cplx, int nlines)
{
    extern __shared__ float2 fsm[];
    float2*   W    = fsm;
    const int n    = kN > 0 ? kN : ax.n;
    const int nzc  = n / 2 + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2*   a    = fsm + n + warp * 2 * n;
    float2*   b    = a + n;
    load_roots(W, ax);
    const int npairs = (nlines + 1) / 2;
    for (int pr = blockIdx.x * kZWarps + warp; pr < npairs; pr += gridDim.x * kZWarps)
    {
        const int  la = 2 * pr, lb = 2 * pr + 1;
        const bool hb = lb < nlines;
        for (int i = lane; i < n; i += 32)
        {
            a[i] = make_float2(real[(size_t)la * n + i], hb ? real[(size_t)lb * n + i] : 0.0f);
        }
        __syncwarp();
        const float2* z = fft_line_any<kN, false>(a, 1, b, 1, W, ax, lane) ? b : a;
        for (int k = lane; k < nzc; k += 32)
        {
            const float2 zk = z[k];
            const float2 zn = z[k == 0 ? 0 : n - k];
            cplx[(size_t)la * nzc + k] = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
            if (hb)
            {
                cplx[(size_t)lb * nzc + k] = make_float2(0.5f * (zk.y + zn.y), 0.5f * (zn.x - zk.x));
            }
        }
        __syncwarp();
    }
}

// z backward: Z = A + i B over the full line (A_{n-k} = conj A_k), transformed back; the real and
// imaginary parts are lines 2p and 2p + 1 of the real grid.  The imaginary parts of A_0 and B_0
// (and of A_{n/2}, B_{n/2} for even n) are dropped, as a complex-to-real transform that assumes a
// Hermitian line does.
template<int kN>
__global__ void __launch_bounds__(kZWarps * 32) k_fft_z_c2r(FftAxis ax, const float2* __restrict__ cplx,
                                                            float* __restrict__ real, int nlines)
{
    extern __shared__ float2 fsm[];
    float2*   W    = fsm;
    const int n    = kN > 0 ? kN : ax.n;
    const int nzc  = n / 2 + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2*   a    = fsm + n + warp * 2 * n;
    float2*   b    = a + n;
    load_roots(W, ax);
    const int npairs = (nlines + 1) / 2;
    for (int pr = blockIdx.x * kZWarps + warp; pr < npairs; pr += gridDim.x * kZWarps)
    {
        const int  la = 2 * pr, lb = 2 * pr + 1;
        const bool hb = lb < nlines;
        for (int k = lane; k < n; k += 32)
        {
            const bool lo = k < nzc;
            const int  kk = lo ? k : n - k;
            float2     A  = cplx[(size_t)la * nzc + kk];
            float2     B  = hb ? cplx[(size_t)lb * nzc + kk] : make_float2(0.0f, 0.0f);
            if (!lo)
            {
                A.y = -A.y;
                B.y = -B.y;
            }
            else if (kk == 0 || 2 * kk == n)
            {
                // a Hermitian line has real values here: their imaginary parts are ignored
                A.y = 0.0f;
                B.y = 0.0f;
            }
            a[k] = make_float2(A.x - B.y, A.y + B.x);
        }
        __syncwarp();
        const float2* z = fft_line_any<kN, true>(a, 1, b, 1, W, ax, lane) ? b : a;
        for (int i = lane; i < n; i += 32)
        {
            const float2 v             = z[i];
            real[(size_t)la * n + i] = v.x;
            if (hb)
            {
                real[(size_t)lb * n + i] = v.y;
            }
        }
        __syncwarp();
    }
}

// Lines along y or x of the half-complex grid: block (outer index o, tile t) loads the kFftTile
// z-frequencies t*T .. t*T + T-1 of all n points of the line (rows of T consecutive elements:
// coalesced), warp c transforms column c, the tile is written back.
template<bool kInv, int kN>
__global__ void __launch_bounds__(kFftTile * 32) k_fft_strided(FftAxis ax, float2* __restrict__ data, int elem_stride,
                                                               int outer_stride, int ntiles, int nzc)
{
    extern __shared__ float2 fsm[];
    float2*   W    = fsm;
    const int n    = kN > 0 ? kN : ax.n;
    float2*   tile = fsm + n;                        // [n][T + 1]
    float2*   scr  = tile + (size_t)n * (kFftTile + 1);  // [T][n]
    const int o    = blockIdx.x / ntiles;
    const int t    = blockIdx.x - o * ntiles;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t base = (size_t)o * outer_stride + (size_t)t * kFftTile;
    const int    cols = min(kFftTile, nzc - t * kFftTile);
    for (int k = threadIdx.x; k < n; k += blockDim.x)
    {
        W[k] = ax.roots[k];
    }
    for (int idx = threadIdx.x; idx < n * kFftTile; idx += blockDim.x)
    {
        const int i = idx / kFftTile, c = idx - i * kFftTile;
        tile[i * (kFftTile + 1) + c] = c < cols ? data[base + (size_t)i * elem_stride + c] : make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    if (warp < cols)
    {
        float2* col = tile + warp;
        float2* s   = scr + (size_t)warp * n;
        if (fft_line_any<kN, kInv>(col, kFftTile + 1, s, 1, W, ax, lane))
        {
            for (int i = lane; i < n; i += 32)
            {
                col[i * (kFftTile + 1)] = s[i];
            }
        }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * kFftTile; idx += blockDim.x)
    {
        const int i = idx / kFftTile, c = idx - i * kFftTile;
        if (c < cols)
        {
            data[base + (size_t)i * elem_stride + c] = tile[i * (kFftTile + 1) + c];
        }
    }
}


// strided pass over axis 0 (x) or 1 (y)
template<bool kInv, int kN>
void strided_launch(const FftPlan3& p, int axis, float2* cplx, cudaStream_t s)
{
    const int nzc    = p.n[2] / 2 + 1;
    const int ntiles = (nzc + kFftTile - 1) / kFftTile;
    const int elem   = axis == 1 ? nzc : p.n[1] * nzc;
    const int outer  = axis == 1 ? p.n[1] * nzc : nzc;
    const int nouter = axis == 1 ? p.n[0] : p.n[1];
    const FftAxis& ax = p.ax[axis];
    k_fft_strided<kInv, kN><<<nouter * ntiles, kFftTile * 32, strided_smem(ax.n), s>>>(ax, cplx, elem, outer, ntiles,
                                                                                       nzc);
}

template<bool kInv>
cudaError_t strided_pass(const FftPlan3& p, int axis, float2* cplx, cudaStream_t s)
{
    switch (p.n[axis])
    {
#define NBX_FFT_CASE(L)                                                                                                \
    case L: strided_launch<kInv, L>(p, axis, cplx, s); break;
        NBX_FFT_FIXED_LENGTHS(NBX_FFT_CASE)
#undef NBX_FFT_CASE
        default: strided_launch<kInv, 0>(p, axis, cplx, s); break;
    }
    return cudaGetLastError();
}

template<int kN>
void z_launch(bool inv, const FftPlan3& p, const float* real_in, float* real_out, float2* cplx, cudaStream_t s)
{
    const int nlines = p.n[0] * p.n[1];
    if (!inv)
    {
        k_fft_z_r2c<kN><<<z_blocks(nlines), kZWarps * 32, z_smem(p.n[2]), s>>>(p.ax[2], real_in, cplx, nlines);
    }
    else
    {
        k_fft_z_c2r<kN><<<z_blocks(nlines), kZWarps * 32, z_smem(p.n[2]), s>>>(p.ax[2], cplx, real_out, nlines);
    }
}

cudaError_t z_pass(bool inv, const FftPlan3& p, const float* real_in, float* real_out, float2* cplx, cudaStream_t s)
{
    switch (p.n[2])
    {
#define NBX_FFT_CASE(L)                                                                                                \
    case L: z_launch<L>(inv, p, real_in, real_out, cplx, s); break;
        NBX_FFT_FIXED_LENGTHS(NBX_FFT_CASE)
#undef NBX_FFT_CASE
        default: z_launch<0>(inv, p, real_in, real_out, cplx, s); break;
    }
    return cudaGetLastError();
}

bool factorize(int n, FftAxis& ax)
{
    ax.n    = n;
    ax.nfac = 0;
    ax.facs = 0;
    int  m  = n;
    auto add = [&ax](int r) {
        ax.facs |= (unsigned long long)r << (8 * ax.nfac);
        ax.nfac++;
    };
    while (m % 4 == 0 && ax.nfac < kFftMaxFactors)
    {
        add(4);
        m /= 4;
    }
    for (int p = 2; p <= 255 && m > 1; p++)
    {
        while (m % p == 0 && ax.nfac < kFftMaxFactors)
        {
            add(p);
            m /= p;
        }
    }
    if (m != 1)
    {
        return false;
    }
    for (auto& wd : ax.stw)
    {
        wd = 0;
    }
    int Ns = 1;
    for (int st = 0; st < ax.nfac; st++)
    {
        const int R  = (int)((ax.facs >> (8 * st)) & 255u);
        const int mm = n / R;
        const int ts = mm / Ns;
        const unsigned long long word = (unsigned)R | ((unsigned)mm << 8) | ((unsigned)ts << 20);
        ax.stw[st / 2] |= word << (32 * (st & 1));
        Ns *= R;
    }
    return true;
}

} // namespace

cudaError_t fft_plan_create(FftPlan3* p, const int n[3])
{
    size_t total = 0;
    for (int d = 0; d < 3; d++)
    {
        if (n[d] < 1 || n[d] > kFftMaxLen || !factorize(n[d], p->ax[d]))
        {
            return cudaErrorInvalidValue;
        }
        p->n[d] = n[d];
        total += (size_t)n[d];
    }
    std::vector<float2> roots(total);
    size_t              off = 0;
    for (int d = 0; d < 3; d++)
    {
        for (int k = 0; k < n[d]; k++)
        {
            const double ang = -2.0 * 3.14159265358979323846 * (double)k / (double)n[d];
            roots[off + k]   = make_float2((float)std::cos(ang), (float)std::sin(ang));
        }
        off += (size_t)n[d];
    }
    cudaError_t e = cudaMalloc(&p->roots, sizeof(float2) * total);
    if (e == cudaSuccess)
    {
        e = cudaMemcpy(p->roots, roots.data(), sizeof(float2) * total, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess)
    {
        return e;
    }
    off = 0;
    for (int d = 0; d < 3; d++)
    {
        p->ax[d].roots = p->roots + off;
        off += (size_t)n[d];
    }
    // shared memory beyond 48 KB for long lines (set once here, not on the launch path)
    const size_t zmax = z_smem(n[2]);
    const size_t smax = std::max(strided_smem(n[0]), strided_smem(n[1]));
    if (e == cudaSuccess && zmax > 48 * 1024)
    {
        e = cudaFuncSetAttribute(k_fft_z_r2c<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zmax);
        if (e == cudaSuccess)
        {
            e = cudaFuncSetAttribute(k_fft_z_c2r<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zmax);
        }
    }
    if (e == cudaSuccess && smax > 48 * 1024)
    {
        e = cudaFuncSetAttribute(k_fft_strided<false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smax);
        if (e == cudaSuccess)
        {
            e = cudaFuncSetAttribute(k_fft_strided<true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smax);
        }
    }
    return e;
}

void fft_plan_destroy(FftPlan3* p)
{
    cudaFree(p->roots);
    p->roots = nullptr;
}

cudaError_t fft_r2c_zy(const FftPlan3& p, const float* real, float2* cplx, cudaStream_t s)
{
    cudaError_t e = z_pass(false, p, real, nullptr, cplx, s);
    if (e == cudaSuccess && p.n[1] > 1)
    {
        e = strided_pass<false>(p, 1, cplx, s);
    }
    return e;
}

cudaError_t fft_r2c(const FftPlan3& p, const float* real, float2* cplx, cudaStream_t s)
{
    cudaError_t e = fft_r2c_zy(p, real, cplx, s);
    if (e == cudaSuccess && p.n[0] > 1)
    {
        e = strided_pass<false>(p, 0, cplx, s);
    }
    return e;
}

cudaError_t fft_c2r_yz(const FftPlan3& p, float2* cplx, float* real, cudaStream_t s)
{
    cudaError_t e = cudaSuccess;
    if (p.n[1] > 1)
    {
        e = strided_pass<true>(p, 1, cplx, s);
    }
    if (e != cudaSuccess)
    {
        return e;
    }
    return z_pass(true, p, nullptr, real, cplx, s);
}

cudaError_t fft_c2r(const FftPlan3& p, float2* cplx, float* real, cudaStream_t s)
{
    cudaError_t e = cudaSuccess;
    if (p.n[0] > 1)
    {
        e = strided_pass<true>(p, 0, cplx, s);
    }
    return e == cudaSuccess ? fft_c2r_yz(p, cplx, real, s) : e;
}

} // namespace nbx
