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
// One block per list entry, one warp per cj4 (lane = j-atom-in-half * 8 +
// i-atom, both halves at once in packed FP32x2 arithmetic), the 64 shifted
// i-atoms staged in shared memory, the any-pair tests of a j-cluster's
// i-clusters combined into per-lane bit masks and one warp OR reduction per
// mask.  Compiled with --fmad=false: r^2 rounds exactly like the CPU
// restatement.
#include "nbx_internal.cuh"

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

// Prunes one list entry (block-cooperative): the shifted i-atoms go to shared memory as duplicated
// pairs {x, x, y, y}, {z, z, -, -}; each warp takes cj4 groups of the entry.  Lane (ii, jj) tests,
// for every i-cluster with a bit to test in either half, the pairs (ii, jj) of half 0 and
// (ii, jj + 4) of half 1 with packed arithmetic, collects the in-range results of all i-clusters of
// a j-cluster as per-lane bit masks and ORs them over the warp with one reduction per mask.
template<int kPruneWarps>
__device__ void prune_entry(const Sci& s, const Cj4* cj4, unsigned* imask_outer, const float4* xq,
                            const float* shiftvec, float outer2, float inner2, int fresh, float4* xib)
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
        const float  xs = x.x + sx, ys = x.y + sy, zs = x.z + sz;
        xib[2 * k]     = make_float4(xs, xs, ys, ys);
        xib[2 * k + 1] = make_float4(zs, zs, 0.0f, 0.0f);
    }
    __syncthreads();
    // the next group's record and outer masks are loaded while the current one is tested
    Cj4   c4n{};
    uint2 outn{};
    if (s.cj4_start + warp < s.cj4_end)
    {
        c4n  = cj4[s.cj4_start + warp];
        outn = fresh ? uint2{} : reinterpret_cast<const uint2*>(imask_outer)[s.cj4_start + warp];
    }
    for (int j4 = s.cj4_start + warp; j4 < s.cj4_end; j4 += kPruneWarps)
    {
        const Cj4   c4  = c4n;
        const uint2 out = outn;
        if (j4 + kPruneWarps < s.cj4_end)
        {
            c4n  = cj4[j4 + kPruneWarps];
            outn = fresh ? uint2{} : reinterpret_cast<const uint2*>(imask_outer)[j4 + kPruneWarps];
        }
        // per half: the bits to test, the outer mask kept so far, the inner mask so far
        unsigned full_m[kSplit], check[kSplit], nw[kSplit];
#pragma unroll
        for (int w = 0; w < kSplit; w++)
        {
            if (fresh)
            {
                full_m[w] = c4.imei[w].imask;
                check[w]  = full_m[w];
                nw[w]     = 0u;
            }
            else
            {
                full_m[w] = w == 0 ? out.x : out.y;
                nw[w]     = c4.imei[w].imask;
                check[w]  = nw[w] ^ full_m[w];
            }
        }
        const unsigned either = check[0] | check[1];
        if (!either)
        {
            continue;
        }
#pragma unroll 1
        for (int jm = 0; jm < kJg; jm++)
        {
            const unsigned cu = (either >> (jm * kNcl)) & 0xffu;
            if (!cu)
            {
                continue;
            }
            const float4 xa = xq[c4.cj[jm] * kCl + jj];
            const float4 xb = xq[c4.cj[jm] * kCl + jj + 4];
            const float2 xj = make_float2(xa.x, xb.x), yj = make_float2(xa.y, xb.y), zj = make_float2(xa.z, xb.z);
            // per lane: bit c set when this lane's pair of half 0 / half 1 is in range
            unsigned in0 = 0u, in1 = 0u, out0 = 0u, out1 = 0u;
#pragma unroll
            for (int i = 0; i < kNcl; i++)
            {
                if (!(cu & (1u << i)))
                {
                    continue;
                }
                const float4 p0 = xib[2 * (i * kCl + ii)];
                const float4 p1 = xib[2 * (i * kCl + ii) + 1];
                const float2 dx = p_sub(make_float2(p0.x, p0.y), xj);
                const float2 dy = p_sub(make_float2(p0.z, p0.w), yj);
                const float2 dz = p_sub(make_float2(p1.x, p1.y), zj);
                const float2 r2 = __fadd2_rn(__fadd2_rn(__fmul2_rn(dx, dx), __fmul2_rn(dy, dy)), __fmul2_rn(dz, dz));
                in0 |= (r2.x < inner2) ? (1u << i) : 0u;
                in1 |= (r2.y < inner2) ? (1u << i) : 0u;
                if (fresh)
                {
                    out0 |= (r2.x < outer2) ? (1u << i) : 0u;
                    out1 |= (r2.y < outer2) ? (1u << i) : 0u;
                }
            }
            // any pair of the (i-cluster, half) within range: OR over the lanes
            const unsigned sh = jm * kNcl;
            in0               = __reduce_or_sync(full, in0) << sh;
            in1               = __reduce_or_sync(full, in1) << sh;
            const unsigned t0 = check[0] & (0xffu << sh), t1 = check[1] & (0xffu << sh);
            nw[0] |= in0 & t0;
            nw[1] |= in1 & t1;
            if (fresh)
            {
                out0 = __reduce_or_sync(full, out0) << sh;
                out1 = __reduce_or_sync(full, out1) << sh;
                full_m[0] &= ~(t0 & ~out0);
                full_m[1] &= ~(t1 & ~out1);
            }
        }
        if (lane < kSplit)
        {
            const int w = lane;
            if (fresh)
            {
                imask_outer[2 * j4 + w] = full_m[w];
            }
            const_cast<Cj4*>(cj4)[j4].imei[w].imask = nw[w];
        }
    }
}

template<int kPruneWarps>
__global__ void __launch_bounds__(32 * kPruneWarps) k_prune(DeviceView v, int fresh, int part, int nparts)
{
    __shared__ float4 xib[2 * kSc];
    const int         numSci = v.hdr->num_sci;
    if (v.hdr->status & (kStatusListOverflow | kStatusExclOverflow))
    {
        return;
    }
    // entries part, part + nparts, ... (all entries for a fresh list)
    for (int e = part + blockIdx.x * nparts; e < numSci; e += gridDim.x * nparts)
    {
        prune_entry<kPruneWarps>(v.sci[e], v.cj4, v.imask_outer, v.xq, v.shiftvec, v.rlist2, v.rlist_inner2, fresh,
                                 xib);
    }
}

// The same prune over a batch of systems: global entry index -> system by a
// search of the entry prefix sums; entries whose index within their system is
// part (mod nparts) are pruned.
template<int kPruneWarps>
__global__ void __launch_bounds__(32 * kPruneWarps)
        k_batch_prune(const BatchSys* sys, const int* entry_prefix, int nsys, float outer2, float inner2, int fresh,
                      int part, int nparts)
{
    __shared__ float4 xib[2 * kSc];
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
        if (!fresh && (local % nparts) != part)
        {
            continue;
        }
        const BatchSys& b = sys[lo];
        prune_entry<kPruneWarps>(b.sci[local], b.cj4, b.imask_outer, b.xq, b.shiftvec, outer2, inner2, fresh, xib);
    }
}

} // namespace

cudaError_t launch_batch_prune(const BatchSys* sys, const int* entry_prefix, int nsys, float outer2, float inner2,
                               int fresh, int part, int nparts, cudaStream_t s)
{
    if (fresh)
    {
        k_batch_prune<kPruneWarpsFresh><<<152 * 8, 32 * kPruneWarpsFresh, 0, s>>>(sys, entry_prefix, nsys, outer2,
                                                                                 inner2, fresh, part, 1);
    }
    else
    {
        k_batch_prune<kPruneWarpsRolling><<<152 * 8, 32 * kPruneWarpsRolling, 0, s>>>(sys, entry_prefix, nsys, outer2,
                                                                                     inner2, fresh, part, nparts);
    }
    return cudaGetLastError();
}

cudaError_t launch_prune(const DeviceView& v, int fresh, int part, int nparts, cudaStream_t s)
{
    if (fresh)
    {
        part   = 0;
        nparts = 1;
    }
    // enough blocks for ~8 per SM; entries beyond are picked up by the grid-stride loop
    if (fresh)
    {
        k_prune<kPruneWarpsFresh><<<152 * 8, 32 * kPruneWarpsFresh, 0, s>>>(v, fresh, part, nparts);
    }
    else
    {
        k_prune<kPruneWarpsRolling><<<152 * 8, 32 * kPruneWarpsRolling, 0, s>>>(v, fresh, part, nparts);
    }
    return cudaGetLastError();
}

} // namespace nbx
