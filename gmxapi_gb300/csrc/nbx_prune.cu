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
// One block per list entry, its warps taking the entry's cj4 groups in turn.
// Fresh pass: lane (ii, jj) holds the shifted i-atom ii of the 8 i-clusters in
// registers and tests its pairs with j-atoms jj and jj + 4 (both warp halves)
// in packed FP32x2 arithmetic; the in-range flags of a j-cluster's 8 i-clusters
// become per-lane bit masks, ORed over the warp with one reduction per mask.
// Rolling pass: the few bits to re-test are visited one at a time with warp
// votes, the shifted i-atoms staged in shared memory.  Compiled with
// --fmad=false; r^2 = fma(dz, dz, fma(dy, dy, dx dx)) is written out with
// explicit multiply-adds, so it rounds exactly like the CPU restatement.
#include "nbx_internal.cuh"

#include <algorithm>

namespace nbx
{
namespace
{

// warps per list entry: 8 for the rolling pass (few bits per group to test, latency-bound on the
// group records), 4 for the fresh pass (every bit tested, compute-bound)
constexpr int kPruneWarpsRolling = 8;
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
// own (no block barrier).  Lane (ii, jj) holds the shifted i-atom ii of the entry's 8 i-clusters in
// registers as duplicated pairs {x, x}, ...; for every i-cluster with a bit in either half it tests
// the pairs (ii, jj) of half 0 and (ii, jj + 4) of half 1 in one packed operation against the
// j-cluster's {x_jj, x_jj+4} pair read from the cluster-packed coordinate records, collects the
// in-range results of all i-clusters of a j-cluster as per-lane bit masks and ORs them over the
// warp with one reduction per mask.
template<int kPruneWarps>
__device__ void prune_entry_fresh(const Sci& s, const Cj4* cj4, unsigned* imask_outer, const float4* xq,
                                  const float* xqp, const float* shiftvec, float outer2, float inner2)
{
    const int      lane = threadIdx.x & 31;
    const int      warp = threadIdx.x >> 5;
    const int      ii   = lane & 7;
    const int      jj   = lane >> 3;
    const unsigned full = 0xffffffffu;
    if (s.cj4_start + warp >= s.cj4_end)
    {
        return;
    }
    // the next group's record is loaded while the current one is tested
    Cj4 c4n = cj4[s.cj4_start + warp];
    const float  sx = shiftvec[3 * s.shift], sy = shiftvec[3 * s.shift + 1], sz = shiftvec[3 * s.shift + 2];
    // r^2 and the squared cut-offs are non-negative floats: r^2 < c^2 exactly when the difference
    // of their bit patterns is negative
    const unsigned inner_bits = __float_as_uint(inner2), outer_bits = __float_as_uint(outer2);
    float2       xi[kNcl], yi[kNcl], zi[kNcl];
#pragma unroll
    for (int c = 0; c < kNcl; c++)
    {
        const float4 x  = xq[s.sci * kSc + c * kCl + ii];
        const float  xs = x.x + sx, ys = x.y + sy, zs = x.z + sz;
        xi[c]           = make_float2(xs, xs);
        yi[c]           = make_float2(ys, ys);
        zi[c]           = make_float2(zs, zs);
    }
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
        // the {half 0, half 1} coordinate pairs of the group's j-clusters with bits to test, all
        // loaded before any is tested (one memory latency per group instead of one per j-cluster)
        float2 xj[kJg], yj[kJg], zj[kJg];
#pragma unroll
        for (int jm = 0; jm < kJg; jm++)
        {
            if ((either >> (jm * kNcl)) & 0xffu)
            {
                const float2* pj = reinterpret_cast<const float2*>(xqp + (size_t)c4.cj[jm] * kPackWords);
                xj[jm]           = pj[jj];
                yj[jm]           = pj[4 + jj];
                zj[jm]           = pj[8 + jj];
            }
        }
#pragma unroll
        for (int jm = 0; jm < kJg; jm++)
        {
            if (!((either >> (jm * kNcl)) & 0xffu))
            {
                continue;
            }
            // per lane: bit i set when this lane's pair of half 0 / half 1 with i-cluster i is in
            // range.  All 8 i-clusters are tested (no per-cluster branch); the in-range flag is the
            // sign of the bit-pattern difference r^2 - cutoff^2, shifted into the masks from the top
            // i-cluster down, one funnel shift per flag.  r^2 = fma(dz, dz, fma(dy, dy, dx dx)), the
            // contraction of the reference's norm2 in its prune kernel.
            unsigned in0 = 0u, in1 = 0u, out0 = 0u, out1 = 0u;
#pragma unroll
            for (int i = kNcl - 1; i >= 0; i--)
            {
                const float2 dx = p_sub(xi[i], xj[jm]);
                const float2 dy = p_sub(yi[i], yj[jm]);
                const float2 dz = p_sub(zi[i], zj[jm]);
                const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
                in0             = __funnelshift_l(__float_as_uint(r2.x) - inner_bits, in0, 1);
                in1             = __funnelshift_l(__float_as_uint(r2.y) - inner_bits, in1, 1);
                out0            = __funnelshift_l(__float_as_uint(r2.x) - outer_bits, out0, 1);
                out1            = __funnelshift_l(__float_as_uint(r2.y) - outer_bits, out1, 1);
            }
            // any pair of the (i-cluster, half) within range: OR over the lanes
            const unsigned sh = jm * kNcl;
            in0               = __reduce_or_sync(full, in0) << sh;
            in1               = __reduce_or_sync(full, in1) << sh;
            out0              = __reduce_or_sync(full, out0) << sh;
            out1              = __reduce_or_sync(full, out1) << sh;
            const unsigned t0 = check[0] & (0xffu << sh), t1 = check[1] & (0xffu << sh);
            nw[0] |= in0 & t0;
            nw[1] |= in1 & t1;
            full_m[0] &= ~(t0 & ~out0);
            full_m[1] &= ~(t1 & ~out1);
        }
        if (lane < kSplit)
        {
            imask_outer[2 * j4 + lane]                 = lane == 0 ? full_m[0] : full_m[1];
            const_cast<Cj4*>(cj4)[j4].imei[lane].imask = lane == 0 ? nw[0] : nw[1];
        }
    }
}

// The rolling prune of one list entry (block-cooperative): only bits in (outer XOR inner) are
// tested (few per group), per bit with warp votes.  The 64 shifted i-atoms are staged in shared
// memory once per entry; the j-atoms of the bits' halves and j-clusters are loaded up front per
// group.
template<int kPruneWarps>
__device__ void prune_entry_rolling(const Sci& s, const Cj4* cj4, const unsigned* imask_outer, const float4* xq,
                                    const float* shiftvec, float inner2, float4* xib)
{
    const int      lane = threadIdx.x & 31;
    const int      warp = threadIdx.x >> 5;
    const int      ii   = lane & 7;
    const int      jj   = lane >> 3;
    const unsigned full = 0xffffffffu;
    const float sx = shiftvec[3 * s.shift], sy = shiftvec[3 * s.shift + 1], sz = shiftvec[3 * s.shift + 2];
    __syncthreads();
    for (int k = threadIdx.x; k < kSc; k += blockDim.x)
    {
        const float4 x = xq[s.sci * kSc + k];
        xib[k]         = make_float4(x.x + sx, x.y + sy, x.z + sz, 0.0f);
    }
    __syncthreads();
    Cj4   c4n{};
    uint2 outn{};
    if (s.cj4_start + warp < s.cj4_end)
    {
        c4n  = cj4[s.cj4_start + warp];
        outn = reinterpret_cast<const uint2*>(imask_outer)[s.cj4_start + warp];
    }
    for (int j4 = s.cj4_start + warp; j4 < s.cj4_end; j4 += kPruneWarps)
    {
        const Cj4   c4  = c4n;
        const uint2 out = outn;
        if (j4 + kPruneWarps < s.cj4_end)
        {
            c4n  = cj4[j4 + kPruneWarps];
            outn = reinterpret_cast<const uint2*>(imask_outer)[j4 + kPruneWarps];
        }
        unsigned nw[kSplit], check[kSplit];
        nw[0]    = c4.imei[0].imask;
        nw[1]    = c4.imei[1].imask;
        check[0] = nw[0] ^ out.x;
        check[1] = nw[1] ^ out.y;
        if (!(check[0] | check[1]))
        {
            continue;
        }
        float4 xj[kSplit][kJg];
#pragma unroll
        for (int w = 0; w < kSplit; w++)
        {
#pragma unroll
            for (int jm = 0; jm < kJg; jm++)
            {
                if ((check[w] >> (jm * kNcl)) & 0xffu)
                {
                    xj[w][jm] = xq[c4.cj[jm] * kCl + w * (kCl / kSplit) + jj];
                }
            }
        }
#pragma unroll
        for (int w = 0; w < kSplit; w++)
        {
#pragma unroll
            for (int jm = 0; jm < kJg; jm++)
            {
                if (!((check[w] >> (jm * kNcl)) & 0xffu))
                {
                    continue;
                }
#pragma unroll
                for (int i = 0; i < kNcl; i++)
                {
                    const unsigned bit = 1u << (jm * kNcl + i);
                    if (check[w] & bit)
                    {
                        const float4 xi = xib[i * kCl + ii];
                        const float  dx = xi.x - xj[w][jm].x, dy = xi.y - xj[w][jm].y, dz = xi.z - xj[w][jm].z;
                        const float  r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                        if (__any_sync(full, r2 < inner2))
                        {
                            nw[w] |= bit;
                        }
                    }
                }
            }
        }
        if (lane < kSplit)
        {
            const_cast<Cj4*>(cj4)[j4].imei[lane].imask = lane == 0 ? nw[0] : nw[1];
        }
    }
}

// Fresh or rolling prune of one list entry (each kernel instantiates one of the two).
template<int kPruneWarps, bool kFresh>
__device__ __forceinline__ void prune_entry(const Sci& s, const Cj4* cj4, unsigned* imask_outer, const float4* xq,
                                            const float* xqp, const float* shiftvec, float outer2, float inner2,
                                            float4* xib)
{
    if constexpr (kFresh)
    {
        prune_entry_fresh<kPruneWarps>(s, cj4, imask_outer, xq, xqp, shiftvec, outer2, inner2);
    }
    else
    {
        prune_entry_rolling<kPruneWarps>(s, cj4, imask_outer, xq, shiftvec, inner2, xib);
    }
}

template<int kPruneWarps, bool kFresh>
__global__ void __launch_bounds__(32 * kPruneWarps) k_prune(DeviceView v, int part, int nparts)
{
    __shared__ float4 xib[kFresh ? 1 : kSc];  // the rolling pass's shifted i-atoms
    const int         numSci = v.hdr->num_sci;
    if (v.hdr->status & (kStatusListOverflow | kStatusExclOverflow))
    {
        return;
    }
    // entries part, part + nparts, ... (all entries for a fresh list)
    for (int e = part + blockIdx.x * nparts; e < numSci; e += gridDim.x * nparts)
    {
        prune_entry<kPruneWarps, kFresh>(v.sci[e], v.cj4, v.imask_outer, v.xq, v.xqp, v.shiftvec, v.rlist2,
                                         v.rlist_inner2, xib);
    }
}

// The same prune over a batch of systems: global entry index -> system by a
// search of the entry prefix sums; entries whose index within their system is
// part (mod nparts) are pruned.
template<int kPruneWarps, bool kFresh>
__global__ void __launch_bounds__(32 * kPruneWarps)
        k_batch_prune(const BatchSys* sys, const int* entry_prefix, int nsys, float outer2, float inner2, int part,
                      int nparts)
{
    __shared__ float4 xib[kFresh ? 1 : kSc];  // the rolling pass's shifted i-atoms
    const int         total = entry_prefix[nsys];
    for (int e = blockIdx.x; e < total; e += gridDim.x)
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
        const int local = e - entry_prefix[lo];
        if (!kFresh && (local % nparts) != part)
        {
            continue;
        }
        const BatchSys& b = sys[lo];
        prune_entry<kPruneWarps, kFresh>(b.sci[local], b.cj4, b.imask_outer, b.xq, b.xqp, b.shiftvec, outer2,
                                         inner2, xib);
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
