// Warp-cooperative mixed-radix FFT of one complex line in shared memory, and the plan of a 3D
// real <-> half-complex transform built from it (the PME grids).
//
// The reference transforms its PME grids through a library FFT (fftpack / FFTW / MKL on the CPU,
// cuFFT on the GPU: src/gromacs/fft/fft.h, src/gromacs/ewald/pme_gpu_3dfft.cu:90-93), unnormalised
// in both directions, real grid [nx][ny][nz] (z fastest) <-> half-complex [nx][ny][nz/2 + 1].
// Here the transform is written out: each line of length n is done by one warp with Stockham
// auto-sort stages (radices 4, 2, 3, 5 as butterflies, any other prime up to 255 as a direct DFT;
// the stage of radix R with span Ns takes input
// j + r n / R and writes (j / Ns) Ns R + j % Ns + r Ns, so the result is in natural order after the
// last stage), twiddles from a table of the n roots exp(-2 pi i k / n) computed on the host in
// double.  Axis passes: along z two real lines form one complex line (a + i b) and are separated
// after the transform; along y and x a block loads a tile of 8 consecutive z-frequencies (coalesced
// rows) and each warp transforms one column.
#pragma once

#include <cuda_runtime.h>

namespace nbx
{

constexpr int kFftMaxFactors = 8;  // stages per axis (8-bit radices in one 64-bit word)
constexpr int kFftMaxLen     = 1024;  // per axis
constexpr int kFftTile       = 8;     // columns (z-frequencies) per block of the strided passes

// One axis of a plan: length, radices in stage order (8 bits each, stage 0 lowest: at most 8 stages
// for lengths up to 1024), device table of the n roots.
struct FftAxis
{
    int                n;
    int                nfac;
    unsigned long long facs;
    // stage words, two per element (stage s in bits 32 (s & 1) of stw[s / 2]): radix R (bits 0-7),
    // butterflies m = n / R (bits 8-19), root step ts = n / (Ns R) (bits 20-31)
    unsigned long long stw[kFftMaxFactors / 2];
    const float2*      roots;  // exp(-2 pi i k / n), k = 0 .. n-1 (device)
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// Root k of n from the shared-memory table; the inverse transform takes the conjugates.
template<bool kInv>
__device__ __forceinline__ float2 fft_root(const float2* W, int k)
{
    const float2 w = W[k];
    return kInv ? make_float2(w.x, -w.y) : w;
}

// In-register R-point DFT, V_q = sum_r v_r w^{q r}, w = exp(-+ 2 pi i / R); W the n-root table with
// n divisible by R (w^k = W[(k mod R) n / R]).
template<int R, bool kInv>
__device__ __forceinline__ void fft_small(float2 (&v)[R], const float2* W, int n)
{
    if (R == 2)
    {
        const float2 a = v[0], b = v[1];
        v[0]           = make_float2(a.x + b.x, a.y + b.y);
        v[1]           = make_float2(a.x - b.x, a.y - b.y);
    }
    else if (R == 4)
    {
        // w = -i forward, +i inverse
        const float2 s02 = make_float2(v[0].x + v[2].x, v[0].y + v[2].y);
        const float2 d02 = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
        const float2 s13 = make_float2(v[1].x + v[3].x, v[1].y + v[3].y);
        const float2 d13 = make_float2(v[1].x - v[3].x, v[1].y - v[3].y);
        // -i d13 = (d13.y, -d13.x)
        const float2 jd = kInv ? make_float2(-d13.y, d13.x) : make_float2(d13.y, -d13.x);
        v[0]            = make_float2(s02.x + s13.x, s02.y + s13.y);
        v[2]            = make_float2(s02.x - s13.x, s02.y - s13.y);
        v[1]            = make_float2(d02.x + jd.x, d02.y + jd.y);
        v[3]            = make_float2(d02.x - jd.x, d02.y - jd.y);
    }
    else if (R == 3)
    {
        // w = -1/2 -+ i sqrt(3)/2
        const float  h  = 0.866025403784438647f;
        const float2 t1 = make_float2(v[1].x + v[2].x, v[1].y + v[2].y);
        const float2 t2 = make_float2(v[1].x - v[2].x, v[1].y - v[2].y);
        const float2 m  = make_float2(fmaf(-0.5f, t1.x, v[0].x), fmaf(-0.5f, t1.y, v[0].y));
        // (-+ i h) t2
        const float2 r = kInv ? make_float2(-h * t2.y, h * t2.x) : make_float2(h * t2.y, -h * t2.x);
        v[0]           = make_float2(v[0].x + t1.x, v[0].y + t1.y);
        v[1]           = make_float2(m.x + r.x, m.y + r.y);
        v[2]           = make_float2(m.x - r.x, m.y - r.y);
    }
    else if (R == 5)
    {
        // c_k = cos(2 pi k / 5), s_k = sin(2 pi k / 5); V_1,4 = a1 -+ i b1, V_2,3 = a2 -+ i b2 forward
        const float  c1 = 0.309016994374947424f, c2 = -0.809016994374947424f;
        const float  s1 = 0.951056516295153572f, s2 = 0.587785252292473129f;
        const float2 t1 = make_float2(v[1].x + v[4].x, v[1].y + v[4].y);
        const float2 t2 = make_float2(v[2].x + v[3].x, v[2].y + v[3].y);
        const float2 t3 = make_float2(v[1].x - v[4].x, v[1].y - v[4].y);
        const float2 t4 = make_float2(v[2].x - v[3].x, v[2].y - v[3].y);
        const float2 a1 = make_float2(fmaf(c2, t2.x, fmaf(c1, t1.x, v[0].x)), fmaf(c2, t2.y, fmaf(c1, t1.y, v[0].y)));
        const float2 a2 = make_float2(fmaf(c1, t2.x, fmaf(c2, t1.x, v[0].x)), fmaf(c1, t2.y, fmaf(c2, t1.y, v[0].y)));
        const float2 b1 = make_float2(fmaf(s2, t4.x, s1 * t3.x), fmaf(s2, t4.y, s1 * t3.y));
        const float2 b2 = make_float2(fmaf(-s1, t4.x, s2 * t3.x), fmaf(-s1, t4.y, s2 * t3.y));
        // -i b = (b.y, -b.x); +i b = (-b.y, b.x)
        const float sg = kInv ? -1.0f : 1.0f;
        v[0]           = make_float2(v[0].x + t1.x + t2.x, v[0].y + t1.y + t2.y);
        v[1]           = make_float2(fmaf(sg, b1.y, a1.x), fmaf(-sg, b1.x, a1.y));
        v[4]           = make_float2(fmaf(-sg, b1.y, a1.x), fmaf(sg, b1.x, a1.y));
        v[2]           = make_float2(fmaf(sg, b2.y, a2.x), fmaf(-sg, b2.x, a2.y));
        v[3]           = make_float2(fmaf(-sg, b2.y, a2.x), fmaf(sg, b2.x, a2.y));
    }
}

// The per-stage constants of a Stockham stage of radix R and span Ns over a line of n: m = n / R
// butterflies, root step ts = n / (Ns R) (exp(-2 pi i r jn / (Ns R)) = W[r jn ts]), and 1 / Ns for
// the quotient j / Ns = (int)((j + 1/2) / Ns), exact for j < 2^20 (no integer division per
// butterfly).
struct FftStage
{
    int   R, Ns, m, ts;
    float inv_ns;
};

__device__ __forceinline__ void stage_split(const FftStage& st, int j, int& jq, int& jn)
{
    jq = (int)(((float)j + 0.5f) * st.inv_ns);
    jn = j - jq * st.Ns;
}

// Butterfly j of a Stockham stage of radix R: src with element stride ss, dst with ds.
template<int R, bool kInv>
__device__ __forceinline__ void fft_butterfly(const float2* src, int ss, float2* dst, int ds, const float2* W, int n,
                                              const FftStage& st, int j)
{
    const int m = st.m, ts = st.ts, Ns = st.Ns;
    int       jq, jn;
    stage_split(st, j, jq, jn);
    float2    v[R];
#pragma unroll
    for (int r = 0; r < R; r++)
    {
        v[r] = src[(j + r * m) * ss];
    }
#pragma unroll
    for (int r = 1; r < R; r++)
    {
        v[r] = cmul(v[r], fft_root<kInv>(W, r * jn * ts));
    }
    fft_small<R, kInv>(v, W, n);
    const int d0 = jq * Ns * R + jn;
#pragma unroll
    for (int r = 0; r < R; r++)
    {
        dst[(d0 + r * Ns) * ds] = v[r];
    }
}

// Butterfly j of a stage of any radix R (7, 11, 13: rare grid factors) as a direct R-point DFT that
// reads its inputs again for every output: few registers, R^2 loads.
template<bool kInv>
__device__ __forceinline__ void fft_butterfly_any(const float2* src, int ss, float2* dst, int ds, const float2* W,
                                                  const FftStage& st, int j)
{
    const int R = st.R, m = st.m, ts = st.ts, Ns = st.Ns;
    int       jq, jn;
    stage_split(st, j, jq, jn);
    const int d0 = jq * Ns * R + jn;
#pragma unroll 1
    for (int q = 0; q < R; q++)
    {
        float2 acc = make_float2(0.0f, 0.0f);
        int    qr  = 0;  // (q r) mod R
#pragma unroll 1
        for (int r = 0; r < R; r++)
        {
            const float2 x = cmul(src[(j + r * m) * ss], fft_root<kInv>(W, r * jn * ts));
            const float2 w = fft_root<kInv>(W, qr * m);
            acc            = make_float2(fmaf(x.x, w.x, fmaf(-x.y, w.y, acc.x)), fmaf(x.x, w.y, fmaf(x.y, w.x, acc.y)));
            qr += q;
            qr -= (qr >= R) ? R : 0;
        }
        dst[(d0 + q * Ns) * ds] = acc;
    }
}

// One line of length ax.n by the calling warp: data in a (stride sa), scratch b (stride sb), both
// shared memory; W the root table in shared memory.  Returns true when the result is in b (an odd
// number of stages), false when it is in a.
template<bool kInv>
__device__ bool fft_line(float2* a, int sa, float2* b, int sb, const float2* W, const FftAxis& ax, int lane)
{
    const int n   = ax.n;
    int       Ns  = 1;
    bool      inb = false;
    for (int s = 0; s < ax.nfac; s++)
    {
        // the stage's constants from the plan (no integer division on the device)
        const unsigned long long q = (s < 2) ? ax.stw[0] : (s < 4) ? ax.stw[1] : (s < 6) ? ax.stw[2] : ax.stw[3];
        const unsigned           w = (unsigned)(q >> (32 * (s & 1)));
        FftStage                 st;
        st.R              = (int)(w & 255u);
        st.m              = (int)((w >> 8) & 4095u);
        st.ts             = (int)(w >> 20);
        st.Ns             = Ns;
        st.inv_ns         = __frcp_rn((float)Ns);
        const int     R   = st.R;
        const int     m   = st.m;
        const float2* src = inb ? b : a;
        float2*       dst = inb ? a : b;
        const int     ss = inb ? sb : sa, ds = inb ? sa : sb;
        switch (R)
        {
            case 2:
                for (int j = lane; j < m; j += 32) fft_butterfly<2, kInv>(src, ss, dst, ds, W, n, st, j);
                break;
            case 3:
                for (int j = lane; j < m; j += 32) fft_butterfly<3, kInv>(src, ss, dst, ds, W, n, st, j);
                break;
            case 4:
                for (int j = lane; j < m; j += 32) fft_butterfly<4, kInv>(src, ss, dst, ds, W, n, st, j);
                break;
            case 5:
                for (int j = lane; j < m; j += 32) fft_butterfly<5, kInv>(src, ss, dst, ds, W, n, st, j);
                break;
            default:
                for (int j = lane; j < m; j += 32) fft_butterfly_any<kInv>(src, ss, dst, ds, W, st, j);
                break;
        }
        __syncwarp();
        Ns *= R;
        inb = !inb;
    }
    return inb;
}

// ---- lines of a length known at compile time (the common PME grid lengths) ----
// The same Stockham stages with every stage constant (radix, span, butterfly count, root step)
// folded at compile time: the butterflies' index arithmetic reduces to shifts and multiplications by
// constants, and no stage table or radix switch is read.  Lengths whose factors are 2, 3, 4, 5 only.

// Radix of stage s of n in the plan's order (4s, then 2, 3, 5), 0 past the last stage.
__host__ __device__ constexpr int fft_factor_c(int n, int s)
{
    int m = n, k = 0;
    while (m % 4 == 0)
    {
        if (k == s)
        {
            return 4;
        }
        m /= 4;
        k++;
    }
    for (int p = 2; p <= 5; p++)
    {
        while (m % p == 0)
        {
            if (k == s)
            {
                return p;
            }
            m /= p;
            k++;
        }
    }
    return 0;
}

template<int R, bool kInv, int N, int Ns>
__device__ __forceinline__ void fft_butterfly_c(const float2* src, int ss, float2* dst, int ds, const float2* W, int j)
{
    constexpr int m  = N / R;
    constexpr int ts = m / Ns;
    const int     jq = j / Ns;  // constant divisor
    const int     jn = j - jq * Ns;
    float2        v[R];
#pragma unroll
    for (int r = 0; r < R; r++)
    {
        v[r] = src[(j + r * m) * ss];
    }
#pragma unroll
    for (int r = 1; r < R; r++)
    {
        v[r] = cmul(v[r], fft_root<kInv>(W, r * jn * ts));
    }
    fft_small<R, kInv>(v, W, N);
    const int d0 = jq * (Ns * R) + jn;
#pragma unroll
    for (int r = 0; r < R; r++)
    {
        dst[(d0 + r * Ns) * ds] = v[r];
    }
}

// Stages S, S+1, ... of a length-N line (data in a, scratch b); true when the result is in b.
template<int N, bool kInv, int S = 0, int Ns = 1>
__device__ __forceinline__ bool fft_line_c(float2* a, int sa, float2* b, int sb, const float2* W, int lane)
{
    constexpr int R = fft_factor_c(N, S);
    if constexpr (R == 0)
    {
        return false;
    }
    else
    {
        static_assert(R == 2 || R == 3 || R == 4 || R == 5, "compile-time lengths take radices 2, 3, 4, 5");
        constexpr int m = N / R;
        for (int j = lane; j < m; j += 32)
        {
            fft_butterfly_c<R, kInv, N, Ns>(a, sa, b, sb, W, j);
        }
        __syncwarp();
        return !fft_line_c<N, kInv, S + 1, Ns * R>(b, sb, a, sa, W, lane);
    }
}

// A line of length kN when kN > 0, else of the runtime length ax.n.
template<int kN, bool kInv>
__device__ __forceinline__ bool fft_line_any(float2* a, int sa, float2* b, int sb, const float2* W, const FftAxis& ax,
                                             int lane)
{
    if constexpr (kN > 0)
    {
        return fft_line_c<kN, kInv>(a, sa, b, sb, W, lane);
    }
    else
    {
        return fft_line<kInv>(a, sa, b, sb, W, ax, lane);
    }
}

// The lengths with a compile-time path (kernels are instantiated for each; others run the
// runtime-length path): the 288k-atom box's 120 and the MD benchmark's 192, and their neighbours.
#define NBX_FFT_FIXED_LENGTHS(X) X(96) X(120) X(128) X(144) X(160) X(192)

// The 3D plan: one axis per dimension (device root tables owned by the plan).
struct FftPlan3
{
    int     n[3] = { 0, 0, 0 };
    FftAxis ax[3]{};
    float2* roots = nullptr;  // all three tables, one allocation
};

// Host: factors each length (4s, then 2, 3, 5, then larger primes up to 255 as direct DFT stages)
// and uploads the root tables; returns cudaErrorInvalidValue for a length above kFftMaxLen or with
// a prime factor above 255.
cudaError_t fft_plan_create(FftPlan3* p, const int n[3]);
void        fft_plan_destroy(FftPlan3* p);
// real [n0][n1][n2] -> half-complex [n0][n1][n2/2 + 1] (unnormalised, exp(-2 pi i ...)).
cudaError_t fft_r2c(const FftPlan3& p, const float* real, float2* cplx, cudaStream_t s);
// half-complex -> real (unnormalised, exp(+2 pi i ...)); cplx is overwritten.
cudaError_t fft_c2r(const FftPlan3& p, float2* cplx, float* real, cudaStream_t s);
// The same without the x transforms (a caller that fuses its own x pass between them).
cudaError_t fft_r2c_zy(const FftPlan3& p, const float* real, float2* cplx, cudaStream_t s);
cudaError_t fft_c2r_yz(const FftPlan3& p, float2* cplx, float* real, cudaStream_t s);
// Dynamic shared memory of a tiled pass over lines of length n (roots, tile, per-warp scratch).
inline size_t fft_tiled_smem(int n)
{
    return sizeof(float2) * ((size_t)n + (size_t)n * (kFftTile + 1) + (size_t)kFftTile * n);
}

} // namespace nbx
