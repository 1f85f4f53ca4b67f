// Dynamic / rolling pair-list pruning on the GPU.
//
// Same masks as the reference's prune-only kernel
// (src/gromacs/nbnxm/cuda/nbnxm_cuda_kernel_pruneonly.cuh:104-279):
//  - fresh list: every set (j-cluster, i-cluster, warp-half) bit is re-tested;
//    it stays in the outer mask if any of its 8x4 atom pairs is within
//    rlistOuter, and is set in the inner mask (used by the force kernel) if
//    any pair is within rlistInner;
//  - rolling pass: only bits in (outer XOR inner) are re-tested and may be
//    added to the inner mask.
// Fresh pass: one block per list entry, its warps taking the entry's cj4 groups
// in turn; lane (ip, jj) holds the shifted i-atoms ip and ip + 4 of the 8
// i-clusters in registers and tests both against j-atom jj in packed FP32x2
// arithmetic; the in-range flags of a j-cluster's 8 i-clusters become per-lane
// bit masks, ORed over the warp with one reduction per j-cluster.
// Rolling pass: one warp per list entry; the few bits to re-test are numbered
// over the warp and each lane tests whole bits (32 atom pairs).  Compiled with
// --fmad=false; r^2 = fma(dz, dz, fma(dy, dy, dx dx)) is written out with
// explicit multiply-adds, so it rounds exactly like the CPU restatement.
#include "nbx_internal.cuh"

#include <algorithm>

namespace nbx
{
namespace
{

// warps per block: 4 for the rolling pass (a warp per list entry), 4 for the fresh pass (a block per
// list entry, every bit tested, compute-bound)
constexpr int kPruneWarpsRolling = 4;
constexpr int kPruneWarpsFresh   = 4;

// Packed FP32 arithmetic without contraction (this unit is compiled with --fmad=false, and the
// intrinsics round each operation): r^2 = (dx dx + dy dy) + dz dz exactly as the scalar form.
__device__ __forceinline__ float2 p_sub(float2 a, float2 b)
{
    unsigned long long ra = *reinterpret_cast<unsigned long long*>(&a);
    unsigned long long rb = *reinterpret_cast<unsigned long long*>(&b);
    unsigned long long rd;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    return *reinterpret_cast<float2*>(&rd);
}

// Fresh prune of one list entry: each warp of the block takes cj4 groups warp, warp + W, ... on its
// own (no block barrier).  Lane (ip, jj), ip = lane & 3 and jj = lane >> 2, holds the shifted i-atoms
// ip and ip + 4 of the entry's 8 i-clusters in registers as pairs {x_ip, x_ip+4}, ... and tests
// both against j-atom jj of a j-cluster in one packed operation, so both results belong to the same
// warp half (jj / 4) and the lane keeps their minimum.  The in-range flags of the 8 i-clusters are
// collected as per-lane bit masks, inner and outer, placed by warp half in one word and ORed over the
// warp with one reduction per j-cluster; j-clusters without bits are skipped.
template<int kPruneWarps>
__device__ void prune_entry_fresh(const Sci& s, const Cj4* cj4, unsigned* imask_outer, const float4* xq,
                                  const float* shiftvec, float outer2, float inner2)
{
    const int      lane = threadIdx.x & 31;
    const int      warp = threadIdx.x >> 5;
    const int      ip   = lane & 3;
    const int      jj   = lane >> 2;
    const unsigned full = 0xffffffffu;
    // the next group's record is loaded while the current one is tested
    Cj4 c4n{};
    if (s.cj4_start + warp < s.cj4_end)
    {
        c4n = cj4[s.cj4_start + warp];
    }
    const float sx = shiftvec[3 * s.shift], sy = shiftvec[3 * s.shift + 1], sz = shiftvec[3 * s.shift + 2];
    // the j-atoms of the entry's j-clusters are fetched into L2 by the whole block (thread t: group
    // t / 4, j-cluster t % 4), so that only each warp's first group waits for device memory
    for (int q = threadIdx.x; q < (s.cj4_end - s.cj4_start) * kJg; q += blockDim.x)
    {
        const int cj = cj4[s.cj4_start + q / kJg].cj[q % kJg];
        asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(xq + (size_t)cj * kCl)));
    }
    if (s.cj4_start + warp >= s.cj4_end)
    {
        return;
    }
    float2 xi[kNcl], yi[kNcl], zi[kNcl];
#pragma unroll
    for (int c = 0; c < kNcl; c++)
    {
        const float4 a = xq[s.sci * kSc + c * kCl + ip];
        const float4 b = xq[s.sci * kSc + c * kCl + ip + 4];
        xi[c]          = make_float2(a.x + sx, b.x + sx);
        yi[c]          = make_float2(a.y + sy, b.y + sy);
        zi[c]          = make_float2(a.z + sz, b.z + sz);
    }
    // this lane's flags go to bits 0-15 (half 0) or 16-31 (half 1) of the reduced word
    const int    hshift   = 16 * (jj >> 2);
    const float2 inner2x2 = make_float2(inner2, inner2), outer2x2 = make_float2(outer2, outer2);
    for (int j4 = s.cj4_start + warp; j4 < s.cj4_end; j4 += kPruneWarps)
    {
        const Cj4 c4 = c4n;
        if (j4 + kPruneWarps < s.cj4_end)
        {
            c4n = cj4[j4 + kPruneWarps];
        }
        // per half: the bits to test (all set bits), the outer mask kept so far, the inner mask
        const unsigned check[kSplit]  = { c4.imei[0].imask, c4.imei[1].imask };
        unsigned       full_m[kSplit] = { check[0], check[1] };
        unsigned       nw[kSplit]     = { 0u, 0u };
        const unsigned either         = check[0] | check[1];
        if (!either)
        {
            continue;
        }
        // the j-atoms of the group's j-clusters with bits to test, all loaded before any is tested
        // (one memory latency per group instead of one per j-cluster)
        float4 xj[kJg];
#pragma unroll
        for (int jm = 0; jm < kJg; jm++)
        {
            if ((either >> (jm * kNcl)) & 0xffu)
            {
                xj[jm] = xq[c4.cj[jm] * kCl + jj];
            }
        }
#pragma unroll
        for (int jm = 0; jm < kJg; jm++)
        {
            const unsigned sh  = jm * kNcl;
            const unsigned sel = (either >> sh) & 0xffu;
            if (!sel)
            {
                continue;
            }
            const float2 xjj = make_float2(xj[jm].x, xj[jm].x);
            const float2 yjj = make_float2(xj[jm].y, xj[jm].y);
            const float2 zjj = make_float2(xj[jm].z, xj[jm].z);
            // per lane: bit i set when one of this lane's two pairs with i-cluster i is in range,
            // shifted in from the top i-cluster down.  All 8 i-clusters are tested (no per-cluster
            // branch); the flag is the sign of r^2 - cutoff^2 for the smaller r^2 of the two (the
            // difference of two floats is negative exactly when the first is smaller), taken for
            // two i-clusters at once in packed arithmetic.  r^2 = fma(dz, dz, fma(dy, dy, dx dx)),
            // the contraction of the reference's norm2 in its prune kernel.
            unsigned fin = 0u, fout = 0u;
#pragma unroll
            for (int i = kNcl - 1; i >= 0; i -= 2)
            {
                float mm[2];
#pragma unroll
                for (int u = 0; u < 2; u++)
                {
                    const float2   dx = p_sub(xi[i - u], xjj);
                    const float2   dy = p_sub(yi[i - u], yjj);
                    const float2   dz = p_sub(zi[i - u], zjj);
                    const float2   r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
                    mm[u]             = __uint_as_float(min(__float_as_uint(r2.x), __float_as_uint(r2.y)));
                }
                const float2 m2   = make_float2(mm[0], mm[1]);
                const float2 din  = p_sub(m2, inner2x2);
                const float2 dout = p_sub(m2, outer2x2);
                fin               = __funnelshift_l(__float_as_uint(din.x), fin, 1);
                fin               = __funnelshift_l(__float_as_uint(din.y), fin, 1);
                fout              = __funnelshift_l(__float_as_uint(dout.x), fout, 1);
                fout              = __funnelshift_l(__float_as_uint(dout.y), fout, 1);
            }
            // any pair of the (i-cluster, half) within range: one OR over the lanes of
            // {inner half 0, outer half 0, inner half 1, outer half 1}, 8 bits each
            const unsigned w  = __reduce_or_sync(full, (fin | (fout << 8)) << hshift);
            const unsigned t0 = check[0] & (0xffu << sh), t1 = check[1] & (0xffu << sh);
            nw[0] |= ((w & 0xffu) << sh) & t0;
            nw[1] |= (((w >> 16) & 0xffu) << sh) & t1;
            full_m[0] &= ~(t0 & ~(((w >> 8) & 0xffu) << sh));
            full_m[1] &= ~(t1 & ~((w >> 24) << sh));
        }
        if (lane < kSplit)
        {
            imask_outer[2 * j4 + lane]                 = lane == 0 ? full_m[0] : full_m[1];
            const_cast<Cj4*>(cj4)[j4].imei[lane].imask = lane == 0 ? nw[0] : nw[1];
        }
    }
}

// Position of the k-th (from 0) set bit of m, which has more than k set bits: a binary search on
// the population counts of the lower halves of shrinking windows.
__device__ __forceinline__ int nth_set_bit(unsigned m, int k)
{
    int pos = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1)
    {
        const int c = __popc((m >> pos) & ((1u << w) - 1u));
        if (k >= c)
        {
            k -= c;
            pos += w;
        }
    }
    return pos;
}

// Per-warp shared memory of the rolling pass: the j-clusters of the 32 groups in hand and the
// inner-mask bits found in range, per half.
struct RollSmem
{
    int      cj[32][kJg];
    unsigned add[kSplit][32];
};

// The rolling prune of one list entry by one warp: only bits in (outer XOR inner) are tested, a few
// per group.  The lanes take the entry's groups 32 at a time (one record per lane), a warp scan of
// the per-lane bit counts numbers the bits, and lane l tests bits l, l + 32, ...: all 32 atom pairs
// of the bit's (i-cluster, j-cluster half), the i-atom pairs {a, a + 4} against each j-atom in
// packed FP32x2 arithmetic.  Bits with a pair within the inner radius are ORed into the inner masks
// through shared memory.  Each warp waits on three dependent loads: the entry, its records, the
// atoms.
__device__ void prune_entry_rolling(const Sci& s, const Cj4* cj4, const unsigned* imask_outer, const float4* xq,
                                    const float* shiftvec, float inner2, RollSmem& sm)
{
    const int      lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    const float sx = shiftvec[3 * s.shift], sy = shiftvec[3 * s.shift + 1], sz = shiftvec[3 * s.shift + 2];
    const float4* const xi = xq + (size_t)s.sci * kSc;
    for (int g0 = s.cj4_start; g0 < s.cj4_end; g0 += 32)
    {
        const int g  = g0 + lane;
        unsigned  m0 = 0u, m1 = 0u, c0 = 0u, c1 = 0u;
        if (g < s.cj4_end)
        {
            const Cj4   c = cj4[g];
            const uint2 o = reinterpret_cast<const uint2*>(imask_outer)[g];
            m0            = c.imei[0].imask;
            m1            = c.imei[1].imask;
            c0            = m0 ^ o.x;
            c1            = m1 ^ o.y;
#pragma unroll
            for (int jm = 0; jm < kJg; jm++)
            {
                sm.cj[lane][jm] = c.cj[jm];
            }
        }
        sm.add[0][lane] = 0u;
        sm.add[1][lane] = 0u;
        const int n0    = __popc(c0);
        const int n     = n0 + __popc(c1);
        int       incl  = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const int t = __shfl_up_sync(full, incl, o);
            if (lane >= o)
            {
                incl += t;
            }
        }
        const int total = __shfl_sync(full, incl, 31);
        __syncwarp();
        for (int t0 = 0; t0 < total; t0 += 32)
        {
            const int t = t0 + lane;
            // the lane holding bit t: the first lane whose inclusive count exceeds t
            int owner = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1)
            {
                if (__shfl_sync(full, incl, owner + step - 1) <= t)
                {
                    owner += step;
                }
            }
            const int      o_excl = __shfl_sync(full, incl - n, min(owner, 31));
            const int      o_n0   = __shfl_sync(full, n0, min(owner, 31));
            const unsigned o_c0   = __shfl_sync(full, c0, min(owner, 31));
            const unsigned o_c1   = __shfl_sync(full, c1, min(owner, 31));
            if (t >= total)
            {
                continue;
            }
            const int  k    = t - o_excl;
            const int  half = k < o_n0 ? 0 : 1;
            const int  bit  = half == 0 ? nth_set_bit(o_c0, k) : nth_set_bit(o_c1, k - o_n0);
            const int  cj   = sm.cj[owner][bit / kNcl];
            const int  ic   = bit % kNcl;
            float2     xa[kCl / 2], ya[kCl / 2], za[kCl / 2];
            float4     xb[kCl / kSplit];
#pragma unroll
            for (int a = 0; a < kCl / 2; a++)
            {
                const float4 p = xi[ic * kCl + a];
                const float4 q = xi[ic * kCl + a + kCl / 2];
                xa[a]          = make_float2(p.x + sx, q.x + sx);
                ya[a]          = make_float2(p.y + sy, q.y + sy);
                za[a]          = make_float2(p.z + sz, q.z + sz);
            }
#pragma unroll
            for (int b = 0; b < kCl / kSplit; b++)
            {
                xb[b] = xq[cj * kCl + half * (kCl / kSplit) + b];
            }
            unsigned m = 0xffffffffu;
#pragma unroll
            for (int b = 0; b < kCl / kSplit; b++)
            {
                const float2 xj = make_float2(xb[b].x, xb[b].x);
                const float2 yj = make_float2(xb[b].y, xb[b].y);
                const float2 zj = make_float2(xb[b].z, xb[b].z);
#pragma unroll
                for (int a = 0; a < kCl / 2; a++)
                {
                    const float2 dx = p_sub(xa[a], xj);
                    const float2 dy = p_sub(ya[a], yj);
                    const float2 dz = p_sub(za[a], zj);
                    const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
                    m = min(m, min(__float_as_uint(r2.x), __float_as_uint(r2.y)));
                }
            }
            // r^2 and the squared cut-off are non-negative floats: r^2 < c^2 exactly when the bit
            // pattern of r^2 is the smaller one
            if (m < __float_as_uint(inner2))
            {
                atomicOr(&sm.add[half][owner], 1u << bit);
            }
        }
        __syncwarp();
        if (g < s.cj4_end)
        {
            const unsigned a0 = sm.add[0][lane], a1 = sm.add[1][lane];
            if (a0 | a1)
            {
                Imei* const im = const_cast<Cj4*>(cj4)[g].imei;
                im[0].imask    = m0 | a0;
                im[1].imask    = m1 | a1;
            }
        }
        __syncwarp();
    }
}

// Fresh prune: a block per list entry, its warps over the entry's groups.  Rolling prune: a warp
// per list entry.
template<int kPruneWarps, bool kFresh>
__global__ void __launch_bounds__(32 * kPruneWarps, kFresh ? 4 : 6) k_prune(DeviceView v, int part, int nparts)
{
    __shared__ RollSmem rsm[kFresh ? 1 : kPruneWarps];
    const int           numSci = v.hdr->num_sci;
    if (v.hdr->status & (kStatusListOverflow | kStatusExclOverflow))
    {
        return;
    }
    if constexpr (kFresh)
    {
        // the next entry's record is loaded while the current entry is pruned
        Sci sn{};
        if (blockIdx.x < numSci)
        {
            sn = v.sci[blockIdx.x];
        }
        for (int e = blockIdx.x; e < numSci; e += gridDim.x)
        {
            const Sci s = sn;
            if (e + gridDim.x < numSci)
            {
                sn = v.sci[e + gridDim.x];
            }
            prune_entry_fresh<kPruneWarps>(s, v.cj4, v.imask_outer, v.xq, v.shiftvec, v.rlist2, v.rlist_inner2);
        }
    }
    else
    {
        // entries part, part + nparts, ...
        const int warp = threadIdx.x >> 5;
        for (int e = part + (blockIdx.x * kPruneWarps + warp) * nparts; e < numSci;
             e += gridDim.x * kPruneWarps * nparts)
        {
            prune_entry_rolling(v.sci[e], v.cj4, v.imask_outer, v.xq, v.shiftvec, v.rlist_inner2, rsm[warp]);
        }
    }
}

// The system of global entry e in a batch: a search of the entry prefix sums.
__device__ __forceinline__ int batch_system_of(const int* entry_prefix, int nsys, int e)
{
    int lo = 0, hi = nsys - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (entry_prefix[mid] <= e)
        {
            lo = mid;
        }
        else
        {
            hi = mid - 1;
        }
    }
    return lo;
}

// The same prune over a batch of systems: global entry index -> system by a
// search of the entry prefix sums; entries whose index within their system is
// part (mod nparts) are pruned.
template<int kPruneWarps, bool kFresh>
__global__ void __launch_bounds__(32 * kPruneWarps)
        k_batch_prune(const BatchSys* sys, const int* entry_prefix, int nsys, float outer2, float inner2, int part,
                      int nparts)
{
    __shared__ RollSmem rsm[kFresh ? 1 : kPruneWarps];
    const int           total = entry_prefix[nsys];
    if constexpr (kFresh)
    {
        for (int e = blockIdx.x; e < total; e += gridDim.x)
        {
            const int       k = batch_system_of(entry_prefix, nsys, e);
            const BatchSys& b = sys[k];
            prune_entry_fresh<kPruneWarps>(b.sci[e - entry_prefix[k]], b.cj4, b.imask_outer, b.xq, b.shiftvec,
                                           outer2, inner2);
        }
    }
    else
    {
        const int warp = threadIdx.x >> 5;
        for (int e = blockIdx.x * kPruneWarps + warp; e < total; e += gridDim.x * kPruneWarps)
        {
            const int k     = batch_system_of(entry_prefix, nsys, e);
            const int local = e - entry_prefix[k];
            if ((local % nparts) != part)
            {
                continue;
            }
            const BatchSys& b = sys[k];
            prune_entry_rolling(b.sci[local], b.cj4, b.imask_outer, b.xq, b.shiftvec, inner2, rsm[warp]);
        }
    }
}

// One wave of resident blocks of a prune kernel (SM count x blocks per SM at its register and
// shared-memory use), computed once: entries are spread over the blocks by the grid-stride loops,
// so a second partial wave would only add a tail.
template<auto kKernel, int kThreads>
int resident_grid()
{
    static int blocks = 0;
    if (blocks == 0)
    {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kKernel, kThreads, 0);
        blocks = std::max(sms, 1) * std::max(per_sm, 1);
    }
    return blocks;
}

} // namespace

cudaError_t launch_batch_prune(const BatchSys* sys, const int* entry_prefix, int nsys, float outer2, float inner2,
                               int fresh, int part, int nparts, cudaStream_t s)
{
    if (fresh)
    {
        constexpr auto kKernel = k_batch_prune<kPruneWarpsFresh, true>;
        kKernel<<<resident_grid<kKernel, 32 * kPruneWarpsFresh>(), 32 * kPruneWarpsFresh, 0, s>>>(
                sys, entry_prefix, nsys, outer2, inner2, part, 1);
    }
    else
    {
        constexpr auto kKernel = k_batch_prune<kPruneWarpsRolling, false>;
        kKernel<<<resident_grid<kKernel, 32 * kPruneWarpsRolling>(), 32 * kPruneWarpsRolling, 0, s>>>(
                sys, entry_prefix, nsys, outer2, inner2, part, nparts);
    }
    return cudaGetLastError();
}

cudaError_t launch_prune(const DeviceView& v, int fresh, int part, int nparts, cudaStream_t s)
{
    if (fresh)
    {
        constexpr auto kKernel = k_prune<kPruneWarpsFresh, true>;
        kKernel<<<resident_grid<kKernel, 32 * kPruneWarpsFresh>(), 32 * kPruneWarpsFresh, 0, s>>>(v, 0, 1);
    }
    else
    {
        constexpr auto kKernel = k_prune<kPruneWarpsRolling, false>;
        kKernel<<<resident_grid<kKernel, 32 * kPruneWarpsRolling>(), 32 * kPruneWarpsRolling, 0, s>>>(v, part,
                                                                                                      nparts);
    }
    return cudaGetLastError();
}

} // namespace nbx
