// Cell gridding on the GPU: the nbnxm GPU ("super-cluster") grid geometry.
//
// Follows src/gromacs/nbnxm/grid.cpp and gridset.cpp:
//   calcColumnIndices (grid.cpp:1173-1268)  -> k_wrap_column
//   setCellIndices    (grid.cpp:1287-1445)  -> k_column_scan, k_scatter
//   sortColumnsGpuGeometry + sort_atoms + fillCell (grid.cpp:292-427, 860-986, 1051-1164)
//                                           -> k_sort_fill
// The reference's pigeonhole sort (sort_atoms) keeps every run of occupied
// holes ordered on (coordinate, atom index) and the hole index is monotonic in
// the coordinate, so its result is the atoms ordered on (coordinate, index),
// reversed for a backwards sort.  Here that order comes from a bitonic sort
// (columns, z) and from rank computation inside a warp (32-atom y slabs and
// 16-atom x halves).  All coordinate arithmetic is plain IEEE single precision
// (this file is compiled with --fmad=false) so the grid, and therefore the
// pair list, is bit-identical to the reference's.
#include "nbx_internal.cuh"

#include <algorithm>

#include <cfloat>

namespace nbx
{
namespace
{

__device__ __forceinline__ void set_status(ListHeader* hdr, unsigned bits)
{
    atomicOr(&hdr->status, bits);
}

// put_atoms_in_box (pbcutil/pbc.cpp:1389-1450, rectangular branch), bounded
// to 127 box lengths; *k returns the number of box lengths added.
__device__ __forceinline__ float wrap_coord(float v, float L, ListHeader* hdr, int* k)
{
    *k = 0;
    if (!(v == v))
    {
        set_status(hdr, kStatusNaN);
        return 0.0f;
    }
    int it = 0;
    while (v < 0.0f && it < 128)
    {
        v += L;
        it++;
        (*k)++;
    }
    while (v >= L && it < 128)
    {
        v -= L;
        it++;
        (*k)--;
    }
    if (it >= 128)
    {
        set_status(hdr, kStatusWrapLimit);
        v  = 0.0f;
        *k = 0;
    }
    return v;
}

constexpr int kGridThreads   = 1024;
constexpr int kAtomsPerThread = 4;
constexpr int kMaxSmemCols    = 8192;  // column counters kept in shared memory up to this many columns

// Wrap into the box, column index, and each atom's slot within its column.
// Column counts are gathered per block in shared memory; each block then
// reserves one contiguous range per column it touches with a single global
// atomic, so a column sees one global atomic per block instead of one per atom.
__global__ void __launch_bounds__(kGridThreads) k_wrap_column(DeviceView v, float* x, int write_back)
{
    extern __shared__ int s_cnt[];  // [ncol]: counts, then the block's base slot per column
    const int  ncol     = v.g.ncol;
    const bool use_smem = ncol <= kMaxSmemCols;
    if (use_smem)
    {
        for (int c = threadIdx.x; c < ncol; c += blockDim.x)
        {
            s_cnt[c] = 0;
        }
        __syncthreads();
    }
    int col[kAtomsPerThread], rank[kAtomsPerThread];
#pragma unroll
    for (int k = 0; k < kAtomsPerThread; k++)
    {
        const int i = (blockIdx.x * kAtomsPerThread + k) * blockDim.x + threadIdx.x;
        col[k]      = -1;
        if (i >= v.n)
        {
            continue;
        }
        float    c[3];
        unsigned code = 0;
        for (int d = 0; d < 3; d++)
        {
            int kk;
            c[d]             = wrap_coord(x[3 * i + d], v.g.box[d], v.hdr, &kk);
            v.xin[3 * i + d] = c[d];
            code |= ((unsigned)(kk & 0xff)) << (8 * d);
            if (write_back)
            {
                x[3 * i + d] = c[d];
            }
        }
        v.image[i] = write_back ? 0 : (int)code;
        // lower corner is 0, so (x - lower) == x exactly
        int cx    = (int)__fmul_rn(c[0], v.g.ics[0]);
        int cy    = (int)__fmul_rn(c[1], v.g.ics[1]);
        cx        = min(cx, v.g.ncx - 1);
        cy        = min(cy, v.g.ncy - 1);
        col[k]    = cx * v.g.ncy + cy;
        v.col[i]  = col[k];
        if (use_smem)
        {
            rank[k] = atomicAdd(&s_cnt[col[k]], 1);
        }
        else
        {
            v.slot[i] = atomicAdd(&v.cxy_na[col[k]], 1);
        }
    }
    if (!use_smem)
    {
        return;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < ncol; c += blockDim.x)
    {
        const int cnt = s_cnt[c];
        if (cnt > 0)
        {
            s_cnt[c] = atomicAdd(&v.cxy_na[c], cnt);
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kAtomsPerThread; k++)
    {
        if (col[k] >= 0)
        {
            v.slot[(blockIdx.x * kAtomsPerThread + k) * blockDim.x + threadIdx.x] = s_cnt[col[k]] + rank[k];
        }
    }
}

// Cells per column and their prefix sum (grid.cpp:1300-1330), one block.
__global__ void k_column_scan(DeviceView v)
{
    __shared__ int warp_sums[32];
    const int      ncol     = v.g.ncol;
    const int      nthreads = blockDim.x;
    const int      per      = (ncol + nthreads - 1) / nthreads;
    const int      c0       = threadIdx.x * per;
    const int      c1       = min(ncol, c0 + per);
    int            local    = 0;
    for (int c = c0; c < c1; c++)
    {
        local += (v.cxy_na[c] + kSc - 1) / kSc;
    }
    // block exclusive scan of the per-thread sums
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int       incl = local;
    for (int o = 1; o < 32; o <<= 1)
    {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o)
        {
            incl += t;
        }
    }
    if (lane == 31)
    {
        warp_sums[warp] = incl;
    }
    __syncthreads();
    if (warp == 0)
    {
        int w = (lane < (nthreads >> 5)) ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1)
        {
            int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o)
            {
                w += t;
            }
        }
        warp_sums[lane] = w;  // inclusive
    }
    __syncthreads();
    int run = incl - local + (warp > 0 ? warp_sums[warp - 1] : 0);
    for (int c = c0; c < c1; c++)
    {
        v.cxy_ind[c] = run;
        run += (v.cxy_na[c] + kSc - 1) / kSc;
    }
    if (threadIdx.x == nthreads - 1)
    {
        v.cxy_ind[ncol] = run;
        if (run > v.g.cells_capacity)
        {
            set_status(v.hdr, kStatusGridOverflow);
            v.hdr->num_cells = 0;
        }
        else
        {
            v.hdr->num_cells = run;
        }
    }
}

__global__ void k_scatter(DeviceView v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n || v.hdr->num_cells == 0)
    {
        return;
    }
    v.atom_indices[v.cxy_ind[v.col[i]] * kSc + v.slot[i]] = i;
}

// Total order key on (coordinate, atom index), ascending; -0.0 equals +0.0.
__device__ __forceinline__ unsigned long long sort_key(float f, int a)
{
    unsigned u = __float_as_uint(f);
    if ((u << 1) == 0u)
    {
        u = 0u;
    }
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return ((unsigned long long)u << 32) | (unsigned)a;
}

// Block-wide bitonic sort of keys[0..P), P a power of two.
__device__ void bitonic_sort(unsigned long long* keys, int P)
{
    for (int k = 2; k <= P; k <<= 1)
    {
        for (int j = k >> 1; j > 0; j >>= 1)
        {
            for (int t = threadIdx.x; t < P; t += blockDim.x)
            {
                const int p = t ^ j;
                if (p > t)
                {
                    const unsigned long long a = keys[t], b = keys[p];
                    const bool up = ((t & k) == 0);
                    if ((a > b) == up)
                    {
                        keys[t] = b;
                        keys[p] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Block-wide bitonic sort of keys[0..P) in shared memory, P a power of two from 64 on: the stages
// whose partners are at most 32 apart run in registers, each warp holding 64-key segments two keys
// per lane (partners 2..32 apart by shuffles, 1 apart within the lane); the wider stages run in
// shared memory, one compare-exchange pair per thread, with a block barrier each.  Same network and
// result as bitonic_sort.
__device__ void bitonic_sort_smem(unsigned long long* keys, int P)
{
    const unsigned full   = 0xffffffffu;
    const int      lane   = threadIdx.x & 31;
    const int      warp   = threadIdx.x >> 5;
    const int      nwarps = blockDim.x >> 5;
    // the stages of merge sizes kfirst .. klast with partners at most 32 apart, per segment
    auto reg_phase = [&](int kfirst, int klast) {
        for (int seg = warp; seg < P / 64; seg += nwarps)
        {
            const int          p0 = seg * 64 + 2 * lane;
            unsigned long long e0 = keys[p0], e1 = keys[p0 + 1];
            for (int k = kfirst; k <= klast; k <<= 1)
            {
                // ascending where bit k of the position is clear (the same for p0 and p0 + 1)
                const bool up = (p0 & k) == 0;
                for (int j = min(k >> 1, 32); j >= 2; j >>= 1)
                {
                    const unsigned long long y0      = __shfl_xor_sync(full, e0, j >> 1);
                    const unsigned long long y1      = __shfl_xor_sync(full, e1, j >> 1);
                    const bool               takeMin = ((p0 & j) == 0) == up;
                    // keep the smaller key when takeMin, else the larger: take the partner's key
                    // when the comparison says so (keys are distinct)
                    e0 = ((e0 > y0) == takeMin) ? y0 : e0;
                    e1 = ((e1 > y1) == takeMin) ? y1 : e1;
                }
                if ((e0 > e1) == up)
                {
                    const unsigned long long t = e0;
                    e0                         = e1;
                    e1                         = t;
                }
            }
            keys[p0]     = e0;
            keys[p0 + 1] = e1;
        }
    };
    reg_phase(2, min(P, 64));
    __syncthreads();
    for (int k = 128; k <= P; k <<= 1)
    {
        for (int j = k >> 1; j >= 64; j >>= 1)
        {
            for (int q = threadIdx.x; q < P / 2; q += blockDim.x)
            {
                const int                i = ((q & ~(j - 1)) << 1) | (q & (j - 1));  // lower key of pair q
                const int                l = i | j;
                const unsigned long long a = keys[i], b = keys[l];
                if ((a > b) == ((i & k) == 0))
                {
                    keys[i] = b;
                    keys[l] = a;
                }
            }
            __syncthreads();
        }
        reg_phase(k, k);
        __syncthreads();
    }
}

// Rank of this lane's (coordinate, atom) among the first `cnt` lanes of its
// group of `gsize` lanes (ascending, or descending when `backwards`).
__device__ __forceinline__ int group_rank(float c, int a, int cnt, int gsize, bool backwards)
{
    const int lane  = threadIdx.x & 31;
    const int gbase = lane & ~(gsize - 1);
    int       rank  = 0;
    for (int m = 0; m < gsize; m++)
    {
        const float cm = __shfl_sync(0xffffffffu, c, gbase + m);
        const int   am = __shfl_sync(0xffffffffu, a, gbase + m);
        if (m < cnt && (gbase + m) != lane)
        {
            const bool before = backwards ? (cm > c || (cm == c && am > a))
                                          : (cm < c || (cm == c && am < a));
            rank += before ? 1 : 0;
        }
    }
    return rank;
}

constexpr int kSortThreads   = 1024;
constexpr int kSmemSortItems = 4096;

// One block per grid column: z sort, per-slab y and x sorts, fill (fillCell).
__global__ void __launch_bounds__(kSortThreads) k_sort_fill(DeviceView v, unsigned long long* scratch)
{
    __shared__ unsigned long long skeys[kSmemSortItems];
    __shared__ int                slab[kSortThreads / 32][32];
    const int                     cxy = blockIdx.x;
    if (v.hdr->num_cells == 0)
    {
        return;
    }
    const int n      = v.cxy_na[cxy];
    const int cell0  = v.cxy_ind[cxy];
    const int ncells = v.cxy_ind[cxy + 1] - cell0;
    const int base   = cell0 * kSc;
    if (ncells == 0)
    {
        return;
    }
    int P = 64;  // at least one 64-key segment of the shared-memory sort
    while (P < n)
    {
        P <<= 1;
    }
    unsigned long long* keys = (P <= kSmemSortItems) ? skeys : scratch + 2 * (size_t)base;
    for (int t = threadIdx.x; t < P; t += blockDim.x)
    {
        if (t < n)
        {
            const int a = v.atom_indices[base + t];
            keys[t]     = sort_key(v.xin[3 * a + 2], a);
        }
        else
        {
            keys[t] = ~0ull;
        }
    }
    __syncthreads();
    if (P <= kSmemSortItems)
    {
        bitonic_sort_smem(keys, P);
    }
    else
    {
        bitonic_sort(keys, P);
    }
    for (int t = threadIdx.x; t < ncells * kSc; t += blockDim.x)
    {
        v.atom_indices[base + t] = (t < n) ? (int)(unsigned)(keys[t] & 0xffffffffu) : -1;
    }
    __syncthreads();

    // Cell z bounds and cluster counts, from the z-sorted order (grid.cpp:1090-1108)
    for (int cz = threadIdx.x; cz < ncells; cz += blockDim.x)
    {
        const int numAtoms = min(kSc, n - cz * kSc);
        const int cell     = cell0 + cz;
        v.nclusters[cell]  = min(kNcl, (numAtoms + kCl - 1) / kCl);
        const int aLo      = v.atom_indices[base + cz * kSc];
        const int aHi      = v.atom_indices[base + cz * kSc + numAtoms - 1];
        v.bbcz[cell]       = make_float2(v.xin[3 * aLo + 2], v.xin[3 * aHi + 2]);
    }
    __syncthreads();

    // 32-atom slabs: y sort (backwards on odd slabs), then x sort per 16-atom half
    // (backwards on odd halves), then fill the four clusters.
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int sub_z = warp; sub_z < ncells * 2; sub_z += kSortThreads / 32)
    {
        const int off  = sub_z * 32;
        const int nz   = n - off;  // may be <= 0
        const bool real = lane < nz;
        int   a        = real ? v.atom_indices[base + off + lane] : -1;
        float yv       = real ? v.xin[3 * a + 1] : 0.0f;
        const int ryr  = group_rank(yv, a, nz, 32, (sub_z & 1) != 0);
        const int ry   = real ? ryr : lane;
        __syncwarp();
        slab[warp][ry] = a;
        __syncwarp();
        a              = slab[warp][lane];
        const int half = lane >> 4;
        const int ny   = min(16, n - (off + half * 16));
        const bool realy = (lane & 15) < ny;
        float xv       = realy ? v.xin[3 * a + 0] : 0.0f;
        const int rxr  = group_rank(xv, a, ny, 16, half != 0);
        const int rx   = realy ? rxr : (lane & 15);
        __syncwarp();
        slab[warp][half * 16 + rx] = a;
        __syncwarp();
        a               = slab[warp][lane];
        const int slot  = base + off + lane;
        const bool ra   = (off + lane) < n;
        float4 xq;
        if (ra)
        {
            xq = make_float4(v.xin[3 * a], v.xin[3 * a + 1], v.xin[3 * a + 2], v.q[a]);
            v.cells[a]  = slot;
            v.tgrid[slot] = v.type[a];
        }
        else
        {
            xq            = make_float4(kFarAway, kFarAway, kFarAway, 0.0f);
            v.tgrid[slot] = v.ntypes1 - 1;
            a             = -1;
        }
        v.atom_indices[slot] = a;
        v.xq[slot]           = xq;
        // cluster bounding boxes over the real atoms (calc_bounding_box_xxxx,
        // grid.cpp:582-607); a cluster of only fillers takes the filler position
        float lo[3] = { ra ? xq.x : FLT_MAX, ra ? xq.y : FLT_MAX, ra ? xq.z : FLT_MAX };
        float hi[3] = { ra ? xq.x : -FLT_MAX, ra ? xq.y : -FLT_MAX, ra ? xq.z : -FLT_MAX };
        for (int o = 1; o < kCl; o <<= 1)
        {
            for (int d = 0; d < 3; d++)
            {
                lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
                hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
            }
        }
        if ((lane & (kCl - 1)) == 0)
        {
            const int cluster_in_col = (off + lane) / kCl;
            const int cluster        = cell0 * kNcl + cluster_in_col;
            const int nx             = n - (off + lane);
            float4    blo, bhi;
            if (nx <= 0)
            {
                blo = make_float4(kFarAway, kFarAway, kFarAway, 0.0f);
                bhi = blo;
            }
            else
            {
                blo = make_float4(lo[0], lo[1], lo[2], 0.0f);
                bhi = make_float4(hi[0], hi[1], hi[2], 0.0f);
            }
            v.bb[2 * cluster]     = blo;
            v.bb[2 * cluster + 1] = bhi;
        }
    }
}

// nbnxn_atomdata_copy_x_to_nbat_x (atomdata.cpp:1018-1073), plus the box
// shift each atom received at the last search so that coordinates which left
// the box since then stay consistent with the grid and the list.
// atom_order 0: one thread per grid slot (coalesced xq, x gathered by atom index),
// for coordinates in device memory; 1: one thread per atom (coalesced x, xq written
// by slot), for coordinates read from host memory over the host link.
// clear: also zero what a force evaluation accumulates into (the grid-order forces,
// shift forces, energies, virial, the work queue and the reduction's completion
// counter), in place of separate memsets before the force kernel.
__global__ void k_convert_x(DeviceView v, const float* __restrict__ x, int clear, int atom_order)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (clear)
    {
        if (t < v.g.cells_capacity * kSc)
        {
            v.fnb[t] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        if (blockIdx.x == 0)
        {
            for (int k = threadIdx.x; k < kNShift * 3; k += blockDim.x)
            {
                v.fshift[k] = 0.0;
            }
            if (threadIdx.x < 2)
            {
                v.energy[threadIdx.x] = 0.0;
            }
            if (threadIdx.x < 9)
            {
                v.virial[threadIdx.x] = 0.0;
            }
            if (threadIdx.x == 0)
            {
                v.hdr->work_counter  = 0;
                v.hdr->work_counter2 = 0;
            }
        }
    }
    int a, k;
    if (atom_order)
    {
        a = t;
        if (a >= v.n)
        {
            return;
        }
        k = v.cells[a];
        if ((unsigned)k >= (unsigned)(v.g.cells_capacity * kSc))
        {
            return;
        }
    }
    else
    {
        k = t;
        if (k >= v.hdr->num_cells * kSc)
        {
            return;
        }
        a = v.atom_indices[k];
        if (a < 0)
        {
            return;
        }
    }
    const float4 old  = v.xq[k];
    const int    code = v.image[a];
    float        c[3];
    for (int d = 0; d < 3; d++)
    {
        const int s = (int)(signed char)((code >> (8 * d)) & 0xff);
        c[d]        = (s == 0) ? x[3 * a + d] : x[3 * a + d] + (float)s * v.g.box[d];
    }
    v.xq[k] = make_float4(c[0], c[1], c[2], old.w);
    // the cluster-packed copy (charges and types too: they may change between searches)
    write_packed_slot(v.xqp, k, c[0], c[1], c[2], old.w, v.tgrid[k]);
}

// After a search: the cluster-packed copy of every grid slot, fillers included (the coordinate
// conversion rewrites only the slots that hold atoms).
__global__ void k_pack_slots(DeviceView v)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= v.hdr->num_cells * kSc)
    {
        return;
    }
    const float4 x = v.xq[k];
    write_packed_slot(v.xqp, k, x.x, x.y, x.z, x.w, v.tgrid[k]);
}

} // namespace

// The fnb force buffer (cells_capacity*64 float4) doubles as the sort scratch
// for columns too long for shared memory: a column starting at slot `base`
// with n atoms needs next_pow2(n) < 2n keys at offset 2*base, which fits.
cudaError_t launch_grid(const DeviceView& v, float* d_x, int write_back, cudaStream_t s)
{
    cudaMemsetAsync(v.cxy_na, 0, sizeof(int) * (v.g.ncol + 1), s);
    const int tb = 256;
    const int per_block = kGridThreads * kAtomsPerThread;
    const size_t smem   = v.g.ncol <= kMaxSmemCols ? sizeof(int) * (size_t)v.g.ncol : 0;
    k_wrap_column<<<(v.n + per_block - 1) / per_block, kGridThreads, smem, s>>>(v, d_x, write_back);
    k_column_scan<<<1, 1024, 0, s>>>(v);
    k_scatter<<<(v.n + tb - 1) / tb, tb, 0, s>>>(v);
    k_sort_fill<<<v.g.ncol, kSortThreads, 0, s>>>(v, reinterpret_cast<unsigned long long*>(v.fnb));
    k_pack_slots<<<(v.g.cells_capacity * kSc + tb - 1) / tb, tb, 0, s>>>(v);
    return cudaGetLastError();
}

cudaError_t launch_convert_x(const DeviceView& v, const float* d_x, cudaStream_t s, bool clear, bool atom_order)
{
    const int tb      = 256;
    const int items   = atom_order ? v.n : v.g.cells_capacity * kSc;
    const int threads = clear ? std::max(items, v.g.cells_capacity * kSc) : items;
    k_convert_x<<<threads > 0 ? (threads + tb - 1) / tb : 1, tb, 0, s>>>(v, d_x, clear ? 1 : 0, atom_order ? 1 : 0);
    return cudaGetLastError();
}

} // namespace nbx
