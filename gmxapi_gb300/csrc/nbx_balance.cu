// GPU list balancing after a search: split long entries, then sort entries by size.
//
// Restates, on the device, what the reference does on the host for GPU lists:
//  - split_sci_entry (src/gromacs/nbnxm/pairlist.cpp:2077-2165), without the
//    progressive variant: an entry with more cluster pairs than the target is cut
//    into pieces of close to nsp_max pairs (pairs counted as the bits of
//    imei[0].imask), the last two pieces evened out;
//  - the target of get_nsubpair_target (pairlist.cpp:2485-2585): no splitting
//    when the grid has at least min_ci_balanced cells, else
//    max(36, round(pairs / min_ci_balanced)), here with the exact pair count of
//    the list instead of the geometric estimate;
//  - sort_sci (pairlist.cpp:3827-3873): a stable counting sort on the number of
//    cj4 groups, large entries first, sizes above twice the average sharing one
//    class (the class count is capped at 255 here).
// The cj4 array is untouched: only entry boundaries and order change, so the set
// of cluster pairs is the same.  The persistent force kernel takes entries from an
// atomic queue in list order, so large-first order and even piece sizes shorten
// the tail of the launch.
//
// Sequence (no host synchronisation): count pieces per entry -> exclusive scan ->
// write pieces -> sort into the final list, all sizes from the list header.
#include "nbx_internal.cuh"

namespace nbx
{
namespace
{

constexpr int kMinTarget    = 36;   // nsubpair_target_min, pairlist.cpp:2495
constexpr int kMaxSizeClass = 255;
constexpr int kSortThreads  = 1024;
constexpr int kSortWarps    = kSortThreads / 32;
constexpr int kSortBatch    = 8;  // entries per lane loaded at a time by the sort
constexpr int kScanBatch    = 8;  // piece counts per thread loaded at a time by the scan

__device__ __forceinline__ int balance_target(const ListHeader* hdr, int min_ci_balanced)
{
    const int ncells = hdr->num_cells;
    if (min_ci_balanced <= 0 || ncells >= min_ci_balanced || ncells == 0)
    {
        return 0;
    }
    const long long nsp = hdr->num_subpairs;
    const long long t   = (2 * nsp + min_ci_balanced) / (2 * (long long)min_ci_balanced);
    return t > kMinTarget ? (int)t : kMinTarget;
}

// Walks entry e's cj4 groups (their cluster-pair counts, the bits of imei[0].imask, written by
// the search) and returns its number of pieces; with kWrite the pieces are stored from out[0].
template<bool kWrite>
__device__ int split_entry(const unsigned char* __restrict__ grp_pairs, Sci e, int nsp_max, Sci* out)
{
    const int j4len = e.cj4_end - e.cj4_start;
    if (!(nsp_max > 0 && j4len > 1 && j4len * kNcl * kJg > nsp_max))
    {
        if (kWrite)
        {
            out[0] = e;
        }
        return 1;
    }
    int n   = 1;
    int nsp = 0, nsp_sci = 0, nsp_cj4_e = 0, nsp_cj4 = 0;
    int prev_start = e.cj4_start;  // start of the open piece
    int last_start = e.cj4_start, last_end = e.cj4_start;  // previous closed piece
    for (int j = e.cj4_start; j < e.cj4_end; j++)
    {
        const int nsp_cj4_p = nsp_cj4;
        nsp_cj4             = grp_pairs[j];
        if (nsp > 0 && nsp_max - nsp < nsp + nsp_cj4 - nsp_max)
        {
            if (kWrite)
            {
                Sci p       = e;
                p.cj4_start = prev_start;
                p.cj4_end   = j;
                out[n - 1]  = p;
            }
            last_start = prev_start;
            last_end   = j;
            prev_start = j;
            n++;
            nsp_sci   = nsp;
            nsp_cj4_e = nsp_cj4_p;
            nsp       = 0;
        }
        nsp += nsp_cj4;
    }
    if (kWrite)
    {
        Sci p       = e;
        p.cj4_start = prev_start;
        p.cj4_end   = e.cj4_end;
        out[n - 1]  = p;
        // even out the last two pieces by moving one cj4 group
        if (n >= 2 && nsp_sci - nsp_cj4_e >= nsp + nsp_cj4_e)
        {
            out[n - 2].cj4_end   = last_end - 1;
            out[n - 1].cj4_start = last_end - 1;
        }
    }
    (void)last_start;
    return n;
}

__global__ void k_balance_count(DeviceView v, int min_ci_balanced)
{
    const ListHeader* hdr = v.hdr;
    if (hdr->status & (kStatusListOverflow | kStatusExclOverflow | kStatusGridOverflow))
    {
        return;
    }
    const int nsp_max = balance_target(hdr, min_ci_balanced);
    const int nsci    = hdr->num_sci;
    const int e       = blockIdx.x * blockDim.x + threadIdx.x;
    if (e == 0)
    {
        v.hdr->nsp_max         = nsp_max;
        v.hdr->num_sci_unsplit = nsci;
    }
    if (e < nsci)
    {
        v.sci_pieces[e] = split_entry<false>(v.grp_pairs, v.sci[e], nsp_max, nullptr);
    }
}

// Exclusive scan of the piece counts in place (one block, each thread a contiguous run); the
// total goes to num_sci_split.
__global__ void __launch_bounds__(1024) k_balance_scan(DeviceView v)
{
    __shared__ int    warp_sums[32];
    const ListHeader* hdr = v.hdr;
    if (hdr->status & (kStatusListOverflow | kStatusExclOverflow | kStatusGridOverflow))
    {
        return;
    }
    const int n    = hdr->num_sci_unsplit;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int per  = (n + blockDim.x - 1) / blockDim.x;
    const int i0   = min(n, (int)threadIdx.x * per);
    const int i1   = min(n, i0 + per);
    int       own  = 0;
    for (int b = i0; b < i1; b += kScanBatch)
    {
        int val[kScanBatch];
#pragma unroll
        for (int u = 0; u < kScanBatch; u++)
        {
            val[u] = b + u < i1 ? v.sci_pieces[b + u] : 0;
        }
#pragma unroll
        for (int u = 0; u < kScanBatch; u++)
        {
            own += val[u];
        }
    }
    int inc = own;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o)
        {
            inc += t;
        }
    }
    if (lane == 31)
    {
        warp_sums[warp] = inc;
    }
    __syncthreads();
    if (warp == 0)
    {
        int w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o)
            {
                w += t;
            }
        }
        warp_sums[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    int run = (warp > 0 ? warp_sums[warp - 1] : 0) + inc - own;
    for (int b = i0; b < i1; b += kScanBatch)
    {
        int val[kScanBatch];
#pragma unroll
        for (int u = 0; u < kScanBatch; u++)
        {
            val[u] = b + u < i1 ? v.sci_pieces[b + u] : 0;
        }
#pragma unroll
        for (int u = 0; u < kScanBatch; u++)
        {
            if (b + u < i1)
            {
                v.sci_pieces[b + u] = run;
                run += val[u];
            }
        }
    }
    if (threadIdx.x == blockDim.x - 1)
    {
        v.hdr->num_sci_split = run;
    }
}

__global__ void k_balance_write(DeviceView v)
{
    const ListHeader* hdr = v.hdr;
    if (hdr->status & (kStatusListOverflow | kStatusExclOverflow | kStatusGridOverflow))
    {
        return;
    }
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < hdr->num_sci_unsplit)
    {
        split_entry<true>(v.grp_pairs, v.sci[e], hdr->nsp_max, v.sci_tmp + v.sci_pieces[e]);
    }
}

// Stable counting sort of sci_tmp into sci, size classes descending (one block).  Warp w owns the
// w-th contiguous chunk of the entries: a per-warp class histogram, then per class the offsets of
// the warps' runs (warps in order, classes descending), then each warp places its chunk in order,
// the rank among equal classes of a batch of 32 from __match_any_sync.
__global__ void __launch_bounds__(kSortThreads) k_sort_entries(DeviceView v)
{
    __shared__ int hist[kSortWarps][kMaxSizeClass + 1];  // counts, then each warp's first position
    ListHeader*    hdr = v.hdr;
    if (hdr->status & (kStatusListOverflow | kStatusExclOverflow | kStatusGridOverflow))
    {
        return;
    }
    const int n    = hdr->num_sci_split;
    const int ncj4 = hdr->num_cj4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (n == 0)
    {
        if (threadIdx.x == 0)
        {
            hdr->num_sci = 0;
        }
        return;
    }
    int m = (ncj4 > n) ? (int)((2LL * ncj4) / n) : 0;  // m = 0: one class, order kept
    m     = m > kMaxSizeClass ? kMaxSizeClass : m;
    for (int k = threadIdx.x; k < kSortWarps * (kMaxSizeClass + 1); k += blockDim.x)
    {
        (&hist[0][0])[k] = 0;
    }
    __syncthreads();
    const int chunk = (n + kSortWarps - 1) / kSortWarps;
    const int e0    = min(n, warp * chunk);
    const int e1    = min(n, e0 + chunk);
    // kSortBatch entries per lane loaded before any is counted or placed
    for (int b = e0; b < e1; b += 32 * kSortBatch)
    {
        int len[kSortBatch];
#pragma unroll
        for (int u = 0; u < kSortBatch; u++)
        {
            const int e = b + u * 32 + lane;
            len[u]      = e < e1 ? v.sci_tmp[e].cj4_end - v.sci_tmp[e].cj4_start : -1;
        }
#pragma unroll
        for (int u = 0; u < kSortBatch; u++)
        {
            if (len[u] >= 0)
            {
                atomicAdd(&hist[warp][len[u] < m ? len[u] : m], 1);
            }
        }
    }
    __syncthreads();
    if (warp == 0)
    {
        // per class: the warps' runs in warp order; classes from m down to 0
        int base = 0;
        for (int c0 = m; c0 >= 0; c0 -= 32)
        {
            const int c     = c0 - lane;
            int       total = 0;
            if (c >= 0)
            {
                for (int w = 0; w < kSortWarps; w++)
                {
                    const int h = hist[w][c];
                    hist[w][c]  = total;
                    total += h;
                }
            }
            int incl = total;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o)
                {
                    incl += t;
                }
            }
            const int start = base + incl - total;
            if (c >= 0)
            {
                for (int w = 0; w < kSortWarps; w++)
                {
                    hist[w][c] += start;
                }
            }
            base += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
    __syncthreads();
    for (int b = e0; b < e1; b += 32 * kSortBatch)
    {
        Sci sv[kSortBatch];
#pragma unroll
        for (int u = 0; u < kSortBatch; u++)
        {
            const int e = b + u * 32 + lane;
            sv[u]       = e < e1 ? v.sci_tmp[e] : Sci{ 0, 0, 0, -1 };
        }
#pragma unroll
        for (int u = 0; u < kSortBatch; u++)
        {
            const int      len   = sv[u].cj4_end - sv[u].cj4_start;
            const int      cls   = len < 0 ? -1 : (len < m ? len : m);
            const unsigned peers = __match_any_sync(0xffffffffu, cls);
            const unsigned lower = peers & ((1u << lane) - 1u);
            if (cls >= 0)
            {
                v.sci[hist[warp][cls] + __popc(lower)] = sv[u];
            }
            __syncwarp();
            if (cls >= 0 && lower == 0u)
            {
                hist[warp][cls] += __popc(peers);
            }
            __syncwarp();
        }
    }
    if (threadIdx.x == 0)
    {
        hdr->num_sci = n;
    }
}

} // namespace

cudaError_t launch_balance(const DeviceView& v, int min_ci_balanced, cudaStream_t s)
{
    const int tb     = 256;
    const int blocks = (v.sci_cap + tb - 1) / tb;
    k_balance_count<<<blocks, tb, 0, s>>>(v, min_ci_balanced);
    k_balance_scan<<<1, 1024, 0, s>>>(v);
    k_balance_write<<<blocks, tb, 0, s>>>(v);
    k_sort_entries<<<1, kSortThreads, 0, s>>>(v);
    return cudaGetLastError();
}

} // namespace nbx
