// Cluster-pair search on the GPU into the nbnxm GPU list layout.
//
// Follows nbnxn_make_pairlist_part (src/gromacs/nbnxm/pairlist.cpp:3076-3582)
// for one grid with full periodicity and a rectangular box, with
// make_cluster_list_supersub (:1090-1244), get_cell_range (:286-309),
// boundingbox_only_distance2 (:2841-2878), setSelfAndNewtonExclusionsGpu
// (:880-904) and setExclusionsForIEntry for GPU lists (:1874-1972).
//
// Count pass: one warp per i-cell (super-cluster) walks the shifts in the
// reference's order with the same single-precision arithmetic (this file is
// compiled with --fmad=false).  For each shift the lanes find the z-ranges of
// cells of up to 32 candidate j-columns at once; the warp then takes the flat,
// increasing sequence of j-cells four at a time, lane (cell, j-cluster)
// testing its j-cluster's bounding box against the 8 i-clusters.  The j-clusters
// found are stored as per-cell records (index, 8-bit i-cluster mask) with one
// code per entry, and the cell's entry / cj4 counts are written.  After a
// prefix sum of the counts, the emit pass (one warp per list entry) turns the
// records into sci / cj4 entries at fixed offsets, with the outer masks and
// per-group pair counts, and sets the diagonal and topology exclusion masks.
#include "nbx_internal.cuh"

#include <cstddef>

namespace nbx
{
namespace
{

constexpr int kWarpsPerBlock  = 4;
constexpr int kMaxCj4PerEntry = 1024;  // per (i-cell, shift) entry; beyond it the list overflows

__device__ __forceinline__ void set_status(ListHeader* hdr, unsigned bits)
{
    atomicOr(&hdr->status, bits);
}

__device__ __forceinline__ float sq(float x)
{
    return x * x;
}

__device__ __forceinline__ int xyz2is(int x, int y, int z)
{
    return 5 * (3 * (z + 1) + y + 1) + x + 2;
}

// get_cell_range (pairlist.cpp:286-309), lower corner 0.
__device__ void get_cell_range(float b0, float b1, int numCells, float cellSize, float invCellSize, float d2,
                               float rlist, int* cf, int* cl)
{
    const float listRangeBBToCell2 = rlist * rlist;
    const float distanceInCells    = (b0 - 0.0f) * invCellSize;
    int         f                  = max((int)distanceInCells, 0);
    while (f > 0 && d2 + sq((b0 - 0.0f) - (float)(f - 1 + 1) * cellSize) < listRangeBBToCell2)
    {
        f--;
    }
    int l = min((int)((b1 - 0.0f) * invCellSize), numCells - 1);
    while (l < numCells - 1 && d2 + sq((float)(l + 1) * cellSize - (b1 - 0.0f)) < listRangeBBToCell2)
    {
        l++;
    }
    *cf = f;
    *cl = l;
}

// clusterBoundingBoxDistance2 (pairlist.cpp:351-372)
__device__ __forceinline__ float bb_dist2(const float4 ilo, const float4 ihi, const float4 jlo, const float4 jhi)
{
    float dl  = ilo.x - jhi.x;
    float dh  = jlo.x - ihi.x;
    float dm  = fmaxf(dl, dh);
    float dm0 = fmaxf(dm, 0.0f);
    float d2  = dm0 * dm0;
    dl        = ilo.y - jhi.y;
    dh        = jlo.y - ihi.y;
    dm        = fmaxf(dl, dh);
    dm0       = fmaxf(dm, 0.0f);
    d2        = d2 + dm0 * dm0;
    dl        = ilo.z - jhi.z;
    dh        = jlo.z - ihi.z;
    dm        = fmaxf(dl, dh);
    dm0       = fmaxf(dm, 0.0f);
    d2        = d2 + dm0 * dm0;
    return d2;
}

constexpr int kEmitStage = 512;  // j-lists up to this length are staged in shared memory for the
                                 // exclusion lookups

struct CountSmem
{
    float4 bbc_lo[kNcl], bbc_hi[kNcl];  // the i-cell's cluster bounding boxes
    float4 bbi_lo[kNcl], bbi_hi[kNcl];  // and shifted for the current entry
};

__global__ void __launch_bounds__(32 * kWarpsPerBlock, 8) k_search_count(DeviceView v)
{
    __shared__ CountSmem wsm[kWarpsPerBlock];
    const int           lane = threadIdx.x & 31;
    const int           wib  = threadIdx.x >> 5;
    CountSmem&          sm   = wsm[wib];
    const int           ci   = blockIdx.x * kWarpsPerBlock + wib;
    const int           numCells = v.hdr->num_cells;
    if (ci >= numCells)
    {
        return;
    }
    const unsigned full = 0xffffffffu;
    // column of this cell (next_ci, pairlist.cpp:2808-2836)
    int lo = 0, hi = v.g.ncol - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (v.cxy_ind[mid] <= ci)
        {
            lo = mid;
        }
        else
        {
            hi = mid - 1;
        }
    }
    const int   ci_xy = lo;
    const int   ci_x  = ci_xy / v.g.ncy;
    const int   ci_y  = ci_xy - ci_x * v.g.ncy;
    const float rlist = v.rlist, rlist2 = v.rlist2, rbb2 = v.rbb2;
    const float listRangeBBToJCell2 = rlist * rlist;
    const float* box  = v.g.box;
    const float2 bbcz_i = v.bbcz[ci];
    const int    ncl_i  = v.nclusters[ci];
    // the cell's i-cluster bounding boxes, shifted per entry below
    if (lane < kNcl)
    {
        sm.bbc_lo[lane] = v.bb[2 * (ci * kNcl + lane)];
        sm.bbc_hi[lane] = v.bb[2 * (ci * kNcl + lane) + 1];
    }
    int          shp_x  = (box[0] < rlist) ? 2 : 1;

    int            num_entries = 0, num_cj4 = 0;
    int            rec_n = 0;   // records of this cell so far
    unsigned       pairs = 0u;  // cluster pairs found by this lane
    int* const           rec_cj = v.rec_cj + (size_t)ci * v.rec_cap;
    unsigned char* const rec_m  = v.rec_m + (size_t)ci * v.rec_cap;

    const float d2cx = 0.0f;
    for (int tz = -1; tz <= 1; tz++)
    {
        const float shz = (float)tz * box[2];
        const float bz0 = bbcz_i.x + shz;
        const float bz1 = bbcz_i.y + shz;
        float       d2z;
        if (tz == 0)
        {
            d2z = 0.0f;
        }
        else if (tz < 0)
        {
            d2z = sq(bz1);
        }
        else
        {
            d2z = sq(bz0 - box[2]);
        }
        const float d2z_cx = d2z + d2cx;
        if (d2z_cx >= rlist2)
        {
            continue;
        }
        float bz1_frac = bz1 / (float)(v.cxy_ind[ci_xy + 1] - v.cxy_ind[ci_xy]);
        if (bz1_frac < 0.0f)
        {
            bz1_frac = 0.0f;
        }
        for (int ty = -1; ty <= 1; ty++)
        {
            const float shy = (float)ty * box[1] + (float)tz * 0.0f;
            const float by0 = 0.0f + (float)ci_y * v.g.cs[1] + shy;
            const float by1 = 0.0f + ((float)ci_y + 1.0f) * v.g.cs[1] + shy;
            int         cyf, cyl;
            get_cell_range(by0, by1, v.g.ncy, v.g.cs[1], v.g.ics[1], d2z_cx, rlist, &cyf, &cyl);
            if (cyf > cyl)
            {
                continue;
            }
            float d2z_cy = d2z;
            if (by1 < 0.0f)
            {
                d2z_cy = d2z_cy + sq(0.0f - by1);
            }
            else if (by0 > box[1])
            {
                d2z_cy = d2z_cy + sq(by0 - box[1]);
            }
            for (int tx = -shp_x; tx <= shp_x; tx++)
            {
                const int shift = xyz2is(tx, ty, tz);
                if (shift > kCentral)
                {
                    continue;  // c_pbcShiftBackward (pairlist.cpp:94)
                }
                const bool  excludeSubDiagonal = (shift == kCentral);
                const float shx = (float)tx * box[0] + (float)ty * 0.0f + (float)tz * 0.0f;
                const float bx0 = 0.0f + (float)ci_x * v.g.cs[0] + shx;
                const float bx1 = 0.0f + ((float)ci_x + 1.0f) * v.g.cs[0] + shx;
                int         cxf, cxl;
                get_cell_range(bx0, bx1, v.g.ncx, v.g.cs[0], v.g.ics[0], d2z_cy, rlist, &cxf, &cxl);
                if (cxf > cxl)
                {
                    continue;
                }
                if (excludeSubDiagonal && cxf < ci_x)
                {
                    cxf = ci_x;
                }
                // shifted i-cluster bounding boxes (set_icell_bb, pairlist.cpp:2260-2303)
                __syncwarp();
                if (lane < kNcl)
                {
                    const float4 l  = sm.bbc_lo[lane];
                    const float4 h  = sm.bbc_hi[lane];
                    sm.bbi_lo[lane] = make_float4(l.x + shx, l.y + shy, l.z + shz, 0.0f);
                    sm.bbi_hi[lane] = make_float4(h.x + shx, h.y + shy, h.z + shz, 0.0f);
                }
                __syncwarp();
                int nj = 0;  // j-clusters in this entry
                // The candidate j-columns (cx major, cy minor, the reference's visiting order), 32
                // at a time: each lane finds the z-range of cells of one column, a warp scan turns
                // the cell counts into offsets of one flat, increasing sequence of j-cells.
                const int ny   = cyl - cyf + 1;
                const int ncol = (cxl - cxf + 1) * ny;
                for (int c0 = 0; c0 < ncol; c0 += 32)
                {
                    int       first = 0, count = 0;
                    const int c     = c0 + lane;
                    if (c < ncol)
                    {
                        const int   cx      = cxf + c / ny;
                        const int   cy      = cyf + c % ny;
                        const float cx_real = (float)cx;
                        float       d2zx    = d2z;
                        if (0.0f + cx_real * v.g.cs[0] > bx1)
                        {
                            d2zx = d2zx + sq(0.0f + cx_real * v.g.cs[0] - bx1);
                        }
                        else if (0.0f + (cx_real + 1.0f) * v.g.cs[0] < bx0)
                        {
                            d2zx = d2zx + sq(0.0f + (cx_real + 1.0f) * v.g.cs[0] - bx0);
                        }
                        const int cyf_x = (cx == 0 && shift == kCentral && cyf < ci_y) ? ci_y : cyf;
                        const int columnStart = v.cxy_ind[cx * v.g.ncy + cy];
                        const int columnEnd   = v.cxy_ind[cx * v.g.ncy + cy + 1];
                        // the column's cell z-bounds into L1 ahead of the walks below
                        for (int c = columnStart; c < columnEnd; c += 16)
                        {
                            asm volatile("prefetch.global.L1 [%0];" ::"l"(__cvta_generic_to_global(v.bbcz + c)));
                        }
                        const float cy_real   = (float)cy;
                        float       d2zxy     = d2zx;
                        if (0.0f + cy_real * v.g.cs[1] > by1)
                        {
                            d2zxy = d2zxy + sq(0.0f + cy_real * v.g.cs[1] - by1);
                        }
                        else if (0.0f + (cy_real + 1.0f) * v.g.cs[1] < by0)
                        {
                            d2zxy = d2zxy + sq(0.0f + (cy_real + 1.0f) * v.g.cs[1] - by0);
                        }
                        if (cy >= cyf_x && columnStart < columnEnd && d2zxy < listRangeBBToJCell2)
                        {
                            int midCell = columnStart + (int)(bz1_frac * (float)(columnEnd - columnStart));
                            if (midCell >= columnEnd)
                            {
                                midCell = columnEnd - 1;
                            }
                            const float d2xy = d2zxy - d2z;
                            int         down = midCell;
                            while (down >= columnStart)
                            {
                                const float u = v.bbcz[down].y;
                                if (!(u >= bz0 || d2xy + sq(u - bz0) < rlist2))
                                {
                                    break;
                                }
                                down--;
                            }
                            int firstCell = down + 1;
                            int up        = midCell + 1;
                            while (up < columnEnd)
                            {
                                const float l = v.bbcz[up].x;
                                if (!(l <= bz1 || d2xy + sq(l - bz1) < rlist2))
                                {
                                    break;
                                }
                                up++;
                            }
                            const int lastCell = up - 1;
                            if (shift == kCentral && firstCell < ci)
                            {
                                firstCell = ci;
                            }
                            if (lastCell >= firstCell)
                            {
                                first = firstCell;
                                count = lastCell - firstCell + 1;
                            }
                        }
                    }
                    int incl = count;
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
                    // four j-cells per step: lane (kk, jc) tests j-cluster jc of j-cell k0 + kk
                    // against the 8 i-clusters (make_cluster_list_supersub for (ci, scj))
                    const int kk = lane >> 3;
                    const int jc = lane & 7;
                    // j-cell of this lane at flat index k0 + kk
                    auto locate = [&](int k0) {
                        int col = 0;
#pragma unroll
                        for (int q = 0; q < 4; q++)
                        {
                            // columns that end at or before flat index k0 + q
                            const int before = __popc(__ballot_sync(full, incl <= k0 + q));
                            col              = (kk == q) ? before : col;
                        }
                        col                = min(col, 31);
                        const int colFirst = __shfl_sync(full, first, col);
                        const int colIncl  = __shfl_sync(full, incl, col);
                        const int colCount = __shfl_sync(full, count, col);
                        return colFirst + (k0 + kk - (colIncl - colCount));
                    };
                    // the j-cluster's bounding box is read with the cell's cluster count (empty
                    // cluster slots hold far-away boxes, their results are discarded); the next
                    // four j-cells' boxes are loaded while the current ones are tested
                    int    scj_n  = locate(0);
                    int    ncl_n  = 0;
                    float4 jlo_n{}, jhi_n{};
                    if (kk < total)
                    {
                        ncl_n = v.nclusters[scj_n];
                        jlo_n = v.bb[2 * (scj_n * kNcl + jc)];
                        jhi_n = v.bb[2 * (scj_n * kNcl + jc) + 1];
                    }
                    for (int k0 = 0; k0 < total; k0 += 4)
                    {
                        const int    scj      = scj_n;
                        const bool   has_cell = k0 + kk < total;
                        const int    ncl_j    = ncl_n;
                        const float4 jlo = jlo_n, jhi = jhi_n;
                        if (k0 + 4 < total)
                        {
                            scj_n = locate(k0 + 4);
                            if (k0 + 4 + kk < total)
                            {
                                ncl_n = v.nclusters[scj_n];
                                jlo_n = v.bb[2 * (scj_n * kNcl + jc)];
                                jhi_n = v.bb[2 * (scj_n * kNcl + jc) + 1];
                            }
                            else
                            {
                                ncl_n = 0;
                            }
                        }
                        const bool diag  = has_cell && excludeSubDiagonal && (scj == ci);
                        const int  ci1   = diag ? jc + 1 : ncl_i;
                        unsigned   im8   = 0u;
                        float      d2one = 0.0f;
                        if (jc < ncl_j)
                        {
#pragma unroll
                            for (int i = 0; i < kNcl; i++)
                            {
                                const float d2 = bb_dist2(sm.bbi_lo[i], sm.bbi_hi[i], jlo, jhi);
                                if (i < ci1 && d2 < rlist2)
                                {
                                    im8 |= 1u << i;
                                    d2one = d2;
                                }
                            }
                        }
                        // a single cluster pair in range beyond the bounding-box-only distance:
                        // check its atom pairs (PRUNE_LIST_CPU_ONE), one flagged j-cluster at a time
                        unsigned flagged = __ballot_sync(full, __popc(im8) == 1 && d2one >= rbb2);
                        while (flagged)
                        {
                            const int src = __ffs(flagged) - 1;
                            flagged &= flagged - 1;
                            const int    s_scj = __shfl_sync(full, scj, src);
                            const int    s_cl  = __ffs(__shfl_sync(full, im8, src)) - 1;
                            const float4 xi    = v.xq[ci * kSc + s_cl * kCl + (lane & 7)];
                            const float  ix = xi.x + shx, iy = xi.y + shy, iz = xi.z + shz;
                            const int    csj = s_scj * kNcl + (src & 7);
                            bool         in  = false;
#pragma unroll
                            for (int h = 0; h < 2; h++)
                            {
                                const float4 xj = v.xq[csj * kCl + (lane >> 3) + 4 * h];
                                const float  dx = ix - xj.x, dy = iy - xj.y, dz = iz - xj.z;
                                const float  r2 = dx * dx + dy * dy + dz * dz;
                                in              = in || (r2 < rlist2);
                            }
                            if (!__any_sync(full, in) && lane == src)
                            {
                                im8 = 0u;
                            }
                        }
                        const unsigned nz = __ballot_sync(full, im8 != 0u);
                        if (im8 != 0u)
                        {
                            const int r = rec_n + nj + __popc(nz & ((1u << lane) - 1u));
                            if (r < v.rec_cap)
                            {
                                rec_cj[r] = scj * kNcl + jc;
                                rec_m[r]  = (unsigned char)im8;
                            }
                            pairs += __popc(im8);
                        }
                        nj += __popc(nz);
                    }
                }
                if (nj == 0)
                {
                    continue;  // closeIEntry drops empty entries
                }
                const int ncj4 = (nj + kJg - 1) / kJg;
                if (ncj4 > kMaxCj4PerEntry && lane == 0)
                {
                    set_status(v.hdr, kStatusEntryOverflow);
                }
                if (lane == 0)
                {
                    v.rec_ent[ci * kMaxEntriesPerCell + num_entries] = shift | (nj << 8);
                }
                num_entries++;
                num_cj4 += ncj4;
                rec_n += nj;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        pairs += __shfl_xor_sync(full, pairs, o);
    }
    if (lane == 0)
    {
        v.sci_count[ci] = num_entries;
        v.cj4_count[ci] = num_cj4;
        // cluster pairs of the list, the count that list balancing splits by
        if (pairs > 0u)
        {
            atomicAdd(&v.hdr->num_subpairs, (int)pairs);
        }
        if (rec_n > v.rec_cap)
        {
            atomicMax(&v.hdr->rec_need, rec_n);
            set_status(v.hdr, kStatusRecordOverflow);
        }
    }
}

constexpr int kScanBatch = 8;    // cell counts per thread loaded at a time by the prefix sum
constexpr int kExclStage = 256;  // topology exclusions of a cell's i-atoms staged in shared memory

struct EmitSmem
{
    unsigned      need[2 * kMaxCj4PerEntry / 32];  // per (cj4, half): exclusion mask needed
    int           diag_pos[kNcl];                   // list positions of the diagonal j-clusters
    int           jl[kEmitStage];                   // the entry's j-clusters (short entries)
    unsigned char jm[kEmitStage];                   // and their i-cluster masks
    int           ex_j[kExclStage];                 // excluded partner's grid slot (-1: itself)
    unsigned char ex_i[kExclStage];                 // the i-atom's slot within the cell
};

// Emit pass: one warp per list entry (the entries numbered by the prefix sum of the per-cell
// counts) turns its search records into the entry's sci record and cj4 groups.  The warp finds its
// cell by a 32-way search of the entry offsets and the entry's first record and group from the
// codes of the cell's earlier entries, then writes the cj4 groups (one per lane: four j-clusters,
// the i-cluster masks of both warp halves, exclusion index 0 = all interacting), the outer masks
// (the fresh list's masks until a prune refines them) and the group's cluster-pair count for
// balancing; then the exclusions: flag the (cj4, half) pairs that need a mask (self/Newton pairs of
// the diagonal j-clusters and topology exclusions), allocate the flagged masks all interacting,
// clear j <= i on the diagonal (setSelfAndNewtonExclusionsGpu) and the excluded atom pairs
// (setExclusionsForIEntry).
__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_search_emit(DeviceView v)
{
    __shared__ EmitSmem wsm[kWarpsPerBlock];
    const int           lane = threadIdx.x & 31;
    const int           wib  = threadIdx.x >> 5;
    EmitSmem&           sm   = wsm[wib];
    const int           e    = blockIdx.x * kWarpsPerBlock + wib;
    const unsigned      full = 0xffffffffu;
    if (e >= v.hdr->num_sci
        || (v.hdr->status & (kStatusListOverflow | kStatusRecordOverflow | kStatusEntryOverflow)))
    {
        return;
    }
    // the cell of entry e: the last cell whose first entry is at most e (cells without entries
    // share their successor's offset); the search window shrinks 32-fold per step
    int ci = 0;
    {
        int len = v.hdr->num_cells;
        while (len > 1)
        {
            const int  step = (len + 31) / 32;
            const int  c    = ci + lane * step;
            const bool le   = c < ci + len && v.sci_offset[c] <= e;
            const int  cnt  = __popc(__ballot_sync(full, le));
            const int  lo   = ci + (cnt - 1) * step;
            len             = min(step, ci + len - lo);
            ci              = lo;
        }
    }
    const int kent = e - v.sci_offset[ci];
    // this entry's code; the records and groups of the cell's earlier entries
    const int cl   = lane <= kent ? v.rec_ent[ci * kMaxEntriesPerCell + lane] : 0;
    int       rec0 = lane < kent ? cl >> 8 : 0;
    int       grp0 = (rec0 + kJg - 1) / kJg;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        rec0 += __shfl_xor_sync(full, rec0, o);
        grp0 += __shfl_xor_sync(full, grp0, o);
    }
    const int            code    = __shfl_sync(full, cl, kent);
    const int            sci_out = e;
    const int            cj4_out = v.cj4_offset[ci] + grp0;
    const int*           rec_cj  = v.rec_cj + (size_t)ci * v.rec_cap + rec0;
    const unsigned char* rec_m   = v.rec_m + (size_t)ci * v.rec_cap + rec0;
    // the topology exclusions of the cell's i-atoms as (i-slot, partner grid slot) pairs (when they
    // fit; else the entry walks the exclusion lists); both halves of the 64 i-atoms load together
    int nex = 0;
    {
        int iAtom[2], x0[2] = { 0, 0 }, x1[2] = { 0, 0 };
#pragma unroll
        for (int h = 0; h < 2; h++)
        {
            iAtom[h] = v.atom_indices[ci * kSc + h * 32 + lane];
        }
#pragma unroll
        for (int h = 0; h < 2; h++)
        {
            if (iAtom[h] >= 0)
            {
                x0[h] = v.excl_index[iAtom[h]];
                x1[h] = v.excl_index[iAtom[h] + 1];
            }
        }
#pragma unroll
        for (int h = 0; h < 2; h++)
        {
            const int cnt  = x1[h] - x0[h];
            int       incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const int t = __shfl_up_sync(full, incl, o);
                if (lane >= o)
                {
                    incl += t;
                }
            }
            const int tot = __shfl_sync(full, incl, 31);
            if (nex + tot <= kExclStage)
            {
                const int off = nex + incl - cnt;
                // the partners four at a time: their list entries, then their grid slots
                for (int x = x0[h]; x < x1[h]; x += 4)
                {
                    int jAtom[4];
#pragma unroll
                    for (int u = 0; u < 4; u++)
                    {
                        jAtom[u] = x + u < x1[h] ? v.excl_list[x + u] : -1;
                    }
#pragma unroll
                    for (int u = 0; u < 4; u++)
                    {
                        if (x + u < x1[h])
                        {
                            sm.ex_j[off + (x + u - x0[h])] = (jAtom[u] == iAtom[h]) ? -1 : v.cells[jAtom[u]];
                            sm.ex_i[off + (x + u - x0[h])] = (unsigned char)(h * 32 + lane);
                        }
                    }
                }
            }
            nex += tot;
        }
    }
    const bool ex_staged = nex <= kExclStage;
    {
        const int  shift = code & 0xff;
        const int  nj    = code >> 8;
        const int  ncj4  = (nj + kJg - 1) / kJg;
        const bool excludeSubDiagonal = (shift == kCentral);
        if (lane < kNcl)
        {
            sm.diag_pos[lane] = -1;
        }
        for (int w = lane; w < 2 * kMaxCj4PerEntry / 32; w += 32)
        {
            sm.need[w] = 0u;
        }
        // the j-list is sorted on cluster index; short lists go to shared memory (four records per
        // lane loaded at a time) for the group writes and the exclusion lookups
        const bool staged = nj <= kEmitStage;
        if (staged)
        {
            for (int p0 = 0; p0 < nj; p0 += 128)
            {
                int           c[4];
                unsigned char m[4];
#pragma unroll
                for (int u = 0; u < 4; u++)
                {
                    const int p = p0 + u * 32 + lane;
                    c[u]        = p < nj ? rec_cj[p] : 0;
                    m[u]        = p < nj ? rec_m[p] : 0;
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
                {
                    const int p = p0 + u * 32 + lane;
                    if (p < nj)
                    {
                        sm.jl[p] = c[u];
                        sm.jm[p] = m[u];
                    }
                }
            }
        }
        __syncwarp();
        const int*           jlist = staged ? sm.jl : rec_cj;
        const unsigned char* mlist = staged ? sm.jm : rec_m;
        for (int g = lane; g < ncj4; g += 32)
        {
            Cj4      c;
            unsigned im = 0u;
#pragma unroll
            for (int off = 0; off < kJg; off++)
            {
                const int p = g * kJg + off;
                c.cj[off]   = p < nj ? jlist[p] : 0;
                im |= p < nj ? (unsigned)mlist[p] << (off * kNcl) : 0u;
            }
            c.imei[0].imask    = im;
            c.imei[0].excl_ind = 0;
            c.imei[1]          = c.imei[0];
            v.cj4[cj4_out + g] = c;
            reinterpret_cast<uint2*>(v.imask_outer)[cj4_out + g] = make_uint2(im, im);
            v.grp_pairs[cj4_out + g] = (unsigned char)__popc(im);
        }
        // the diagonal j-clusters (the i-cell's own clusters, central shift)
        if (excludeSubDiagonal)
        {
            for (int p = lane; p < nj; p += 32)
            {
                const int cj = jlist[p];
                if ((cj >> 3) == ci)
                {
                    sm.diag_pos[cj & (kNcl - 1)] = p;
                    atomicOr(&sm.need[(2 * (p / kJg)) / 32], 3u << ((2 * (p / kJg)) % 32));
                }
            }
        }
        int basei = 0;  // first exclusion mask of this entry
        // the mask of a flagged (cj4, half) slot: masks are allocated to the flagged slots in order
        auto excl_of_slot = [&](int slot) {
            int x = basei;
            for (int w = 0; w < slot / 32; w++)
            {
                x += __popc(sm.need[w]);
            }
            return x + __popc(sm.need[slot / 32] & ((1u << (slot % 32)) - 1u));
        };
        __syncwarp();
        __threadfence_block();
        if (lane == 0)
        {
            Sci e;
            e.sci          = ci;
            e.shift        = shift;
            e.cj4_start    = cj4_out;
            e.cj4_end      = cj4_out + ncj4;
            v.sci[sci_out] = e;
        }
        // --- topology exclusions (setExclusionsForIEntry, GPU list) ---
        const int  cjFirst     = jlist[0];
        const int  cjLast      = jlist[nj - 1];
        const bool diagRemoved = excludeSubDiagonal;
        // pass A: flag (cj4, half) pairs that need an exclusion mask; pass B (rep 1): clear the bits
        for (int rep = 0; rep < 2; rep++)
        {
            // one excluded atom pair (i-slot i of the cell, partner at grid slot jIndex)
            auto exclude = [&](int i, int jIndex) {
                if (diagRemoved && jIndex <= ci * kSc + i)
                {
                    return;
                }
                const int jCluster = jIndex / kCl;
                if (jCluster < cjFirst || jCluster > cjLast)
                {
                    return;
                }
                int a = 0, b = nj - 1, index = -1;
                while (a <= b)
                {
                    const int m  = (a + b) >> 1;
                    const int cm = jlist[m];
                    if (cm == jCluster)
                    {
                        index = m;
                        break;
                    }
                    if (cm < jCluster)
                    {
                        a = m + 1;
                    }
                    else
                    {
                        b = m - 1;
                    }
                }
                const int iCluster = i / kCl;
                if (index < 0 || !((mlist[index] >> iCluster) & 1u))
                {
                    return;
                }
                const unsigned pairMask = 1u << ((index % kJg) * kNcl + iCluster);
                const int      innerI   = i & (kCl - 1);
                const int      innerJ   = jIndex & (kCl - 1);
                const int      jHalf    = innerJ / (kCl / kSplit);
                const int      slot     = 2 * (index / kJg) + jHalf;
                if (rep == 0)
                {
                    atomicOr(&sm.need[slot / 32], 1u << (slot % 32));
                }
                else
                {
                    const int ei = excl_of_slot(slot);
                    atomicAnd(&v.excl[ei].pair[(innerJ & (kCl / kSplit - 1)) * kCl + innerI], ~pairMask);
                }
            };
            if (ex_staged)
            {
                for (int t = lane; t < nex; t += 32)
                {
                    if (sm.ex_j[t] >= 0)
                    {
                        exclude(sm.ex_i[t], sm.ex_j[t]);
                    }
                }
            }
            else
            {
                for (int i = lane; i < kSc; i += 32)
                {
                    const int iAtom = v.atom_indices[ci * kSc + i];
                    if (iAtom < 0)
                    {
                        continue;
                    }
                    for (int x = v.excl_index[iAtom]; x < v.excl_index[iAtom + 1]; x++)
                    {
                        const int jAtom = v.excl_list[x];
                        if (jAtom != iAtom)
                        {
                            exclude(i, v.cells[jAtom]);
                        }
                    }
                }
            }
            if (rep == 0)
            {
                // allocate the flagged masks, all interacting
                __syncwarp();
                int nneed = 0;
                for (int w = 0; w < (2 * ncj4 + 31) / 32; w++)
                {
                    nneed += __popc(sm.need[w]);
                }
                if (lane == 0 && nneed > 0)
                {
                    basei = atomicAdd(&v.hdr->num_excl, nneed);
                }
                basei = __shfl_sync(full, basei, 0);
                if (basei + nneed > v.hdr->excl_capacity)
                {
                    if (lane == 0)
                    {
                        set_status(v.hdr, kStatusExclOverflow);
                    }
                    return;
                }
                int run = basei;
                for (int w = 0; w < (2 * ncj4 + 31) / 32; w++)
                {
                    unsigned bits = sm.need[w];
                    while (bits)
                    {
                        const int b = __ffs(bits) - 1;
                        bits &= bits - 1;
                        const int slot = w * 32 + b;
                        v.excl[run].pair[lane] = 0xffffffffu;
                        if (lane == 0)
                        {
                            v.cj4[cj4_out + slot / 2].imei[slot % 2].excl_ind = run;
                        }
                        run++;
                    }
                }
                __syncwarp();
                __threadfence_block();
                // self and Newton exclusions of the diagonal cluster pairs
                // (setSelfAndNewtonExclusionsGpu): clear j <= i
                for (int dj = 0; dj < kNcl; dj++)
                {
                    const int pos = sm.diag_pos[dj];
                    if (pos < 0)
                    {
                        continue;
                    }
                    const int off = pos % kJg;
                    // lane = (jIndexInPart, i): word jIndexInPart*8 + i
                    const int jip = lane >> 3, ii = lane & 7;
                    for (int part = 0; part < kSplit; part++)
                    {
                        const int jOffset = part * (kCl / kSplit);
                        if (ii >= jOffset + jip)
                        {
                            const int ei = excl_of_slot(2 * (pos / kJg) + part);
                            atomicAnd(&v.excl[ei].pair[jip * kCl + ii], ~(1u << (off * kNcl + dj)));
                        }
                    }
                }
                __syncwarp();
            }
        }
    }
}

// Exclusive prefix sums of the per-cell entry and cj4 counts, one block.
__global__ void k_scan_counts(DeviceView v)
{
    __shared__ int ws[2][32];
    const int      n        = v.hdr->num_cells;
    const int      nthreads = blockDim.x;
    const int      per      = (n + nthreads - 1) / nthreads;
    const int      c0       = threadIdx.x * per;
    const int      c1       = min(n, c0 + per);
    int            ls = 0, lc = 0;
    // kScanBatch cells per thread loaded at a time
    for (int b = c0; b < c1; b += kScanBatch)
    {
        int cs[kScanBatch], cc[kScanBatch];
#pragma unroll
        for (int u = 0; u < kScanBatch; u++)
        {
            cs[u] = b + u < c1 ? v.sci_count[b + u] : 0;
            cc[u] = b + u < c1 ? v.cj4_count[b + u] : 0;
        }
#pragma unroll
        for (int u = 0; u < kScanBatch; u++)
        {
            ls += cs[u];
            lc += cc[u];
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int       is = ls, ic = lc;
    for (int o = 1; o < 32; o <<= 1)
    {
        const int ts = __shfl_up_sync(0xffffffffu, is, o);
        const int tc = __shfl_up_sync(0xffffffffu, ic, o);
        if (lane >= o)
        {
            is += ts;
            ic += tc;
        }
    }
    if (lane == 31)
    {
        ws[0][warp] = is;
        ws[1][warp] = ic;
    }
    __syncthreads();
    if (warp == 0)
    {
        int a = (lane < (nthreads >> 5)) ? ws[0][lane] : 0;
        int b = (lane < (nthreads >> 5)) ? ws[1][lane] : 0;
        for (int o = 1; o < 32; o <<= 1)
        {
            const int ta = __shfl_up_sync(0xffffffffu, a, o);
            const int tb = __shfl_up_sync(0xffffffffu, b, o);
            if (lane >= o)
            {
                a += ta;
                b += tb;
            }
        }
        ws[0][lane] = a;
        ws[1][lane] = b;
    }
    __syncthreads();
    int rs = is - ls + (warp > 0 ? ws[0][warp - 1] : 0);
    int rc = ic - lc + (warp > 0 ? ws[1][warp - 1] : 0);
    for (int b = c0; b < c1; b += kScanBatch)
    {
        int cs[kScanBatch], cc[kScanBatch];
#pragma unroll
        for (int u = 0; u < kScanBatch; u++)
        {
            cs[u] = b + u < c1 ? v.sci_count[b + u] : 0;
            cc[u] = b + u < c1 ? v.cj4_count[b + u] : 0;
        }
#pragma unroll
        for (int u = 0; u < kScanBatch; u++)
        {
            if (b + u < c1)
            {
                v.sci_offset[b + u] = rs;
                v.cj4_offset[b + u] = rc;
                rs += cs[u];
                rc += cc[u];
            }
        }
    }
    if (threadIdx.x == nthreads - 1)
    {
        v.sci_offset[n] = rs;
        v.cj4_offset[n] = rc;
        v.hdr->num_sci  = rs;
        v.hdr->num_cj4  = rc;
        v.hdr->num_excl = 1;
        if (rs > v.hdr->sci_capacity || rc > v.hdr->cj4_capacity)
        {
            set_status(v.hdr, kStatusListOverflow);
        }
    }
}

} // namespace

// count (+ records) -> prefix sum | emit.  All sizes stay on the device; the host reads them
// between the two halves to check the list and record capacities.
cudaError_t launch_search_count(const DeviceView& v, cudaStream_t s)
{
    const int cap    = v.g.cells_capacity;
    const int blocks = (cap + kWarpsPerBlock - 1) / kWarpsPerBlock;
    // num_subpairs .. rec_need: accumulated by the count pass or set by balancing
    cudaMemsetAsync(&v.hdr->num_subpairs, 0,
                    offsetof(ListHeader, rec_need) + sizeof(int) - offsetof(ListHeader, num_subpairs), s);
    k_search_count<<<blocks, 32 * kWarpsPerBlock, 0, s>>>(v);
    k_scan_counts<<<1, 1024, 0, s>>>(v);
    return cudaGetLastError();
}

cudaError_t launch_search_write(const DeviceView& v, int num_entries, cudaStream_t s)
{
    if (num_entries > 0)
    {
        const int blocks = (num_entries + kWarpsPerBlock - 1) / kWarpsPerBlock;
        k_search_emit<<<blocks, 32 * kWarpsPerBlock, 0, s>>>(v);
    }
    return cudaGetLastError();
}

} // namespace nbx
