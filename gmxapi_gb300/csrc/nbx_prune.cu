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
// i-atom), the 64 shifted i-atoms staged in shared memory.  Compiled with
// --fmad=false: r^2 rounds exactly like the CPU restatement.
#include "nbx_internal.cuh"

namespace nbx
{
namespace
{

// warps per list entry: 8 for the rolling pass (few bits per group to test, latency-bound on the
// group records), 4 for the fresh pass (every bit tested, compute-bound)
constexpr int kPruneWarpsRolling = 8;
constexpr int kPruneWarpsFresh   = 4;

// Prunes one list entry (block-cooperative): the shifted i-atoms go to shared
// memory, each warp takes cj4 groups of the entry.
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
        xib[k]         = make_float4(x.x + sx, x.y + sy, x.z + sz, 0.0f);
    }
    __syncthreads();
    // the next group's record and outer masks are loaded while the current one is tested
    Cj4  c4n{};
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
        for (int w = 0; w < kSplit; w++)
        {
            unsigned full_m, check, nw;
            if (fresh)
            {
                full_m = c4.imei[w].imask;
                check  = full_m;
                nw     = 0u;
            }
            else
            {
                full_m = w == 0 ? out.x : out.y;
                nw     = c4.imei[w].imask;
                check  = nw ^ full_m;
            }
            if (!check)
            {
                continue;
            }
            for (int jm = 0; jm < kJg; jm++)
            {
                if (!(check & (0xffu << (jm * kNcl))))
                {
                    continue;
                }
                const float4 xj = xq[c4.cj[jm] * kCl + w * (kCl / kSplit) + jj];
#pragma unroll
                for (int i = 0; i < kNcl; i++)
                {
                    const unsigned bit = 1u << (jm * kNcl + i);
                    if (check & bit)
                    {
                        const float4 xi = xib[i * kCl + ii];
                        const float  dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
                        const float  r2 = dx * dx + dy * dy + dz * dz;
                        if (fresh && !__any_sync(full, r2 < outer2))
                        {
                            full_m &= ~bit;
                        }
                        if (__any_sync(full, r2 < inner2))
                        {
                            nw |= bit;
                        }
                    }
                }
            }
            if (lane == 0)
            {
                if (fresh)
                {
                    imask_outer[2 * j4 + w] = full_m;
                }
                const_cast<Cj4*>(cj4)[j4].imei[w].imask = nw;
            }
        }
    }
}

template<int kPruneWarps>
__global__ void __launch_bounds__(32 * kPruneWarps) k_prune(DeviceView v, int fresh, int part, int nparts)
{
    __shared__ float4 xib[kSc];
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
    __shared__ float4 xib[kSc];
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
