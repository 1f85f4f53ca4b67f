/*
 * CPU-layout path of the reference (TEST INFRASTRUCTURE ONLY): the 4-atom-cluster grid, the
 * simple (4x4) cluster pair list and a 4-wide cluster-pair kernel.
 *
 * This is the path the reference's CPU kernels consume, restated in plain C for two uses:
 * the checker of the CPU list builder (a list complete within rlist, its cluster pairs and
 * exclusion masks), and the timed CPU baseline of bench.py (the analogue of the reference's
 * SIMD 4xM kernel, written with portable GCC vector extensions, which map to NEON on the Grace
 * host and SSE here).  Nothing in the product (gmxapi_gb300/) links, loads or calls it.
 *
 * Reference files (paths relative to the GROMACS source root):
 *   grid.cpp:103-262 Grid::setDimensions (CPU geometry: cubic cells of 4 atoms),
 *   grid.cpp:1173-1268 calcColumnIndices, grid.cpp:1287-1445 setCellIndices,
 *   grid.cpp:988-1048 sortColumnsCpuGeometry, grid.cpp:783-854 sort_cluster_on_flag,
 *   grid.cpp:860-986 fillCell (bounding boxes of the cluster's atoms),
 *   pairlist.cpp:3076-3582 nbnxn_make_pairlist_part (the bSimple branches),
 *   pairlist.cpp:963-1078 makeClusterListSimple, pairlist.cpp:907-910 get_imask,
 *   pairlist.cpp:1367-1435 setExclusionsForIEntry (CPU), pairlist.cpp:2002-2067 sort_cj_excl /
 *   closeIEntry, pairlist.cpp:2841-2878 boundingbox_only_distance2,
 *   kernels_simd_4xm/kernel_outer.h + kernel_inner.h (one i-cluster of 4 atoms against a
 *   j-cluster of 4 atoms per step: 4 i-rows of 4-wide j vectors, f_j summed over the rows,
 *   f_i reduced per i-entry, Ewald analytically, exclusion masks per cluster pair, the
 *   Ewald correction of excluded pairs inside the cut-off, the self term on the diagonal).
 * The Ewald real-space function uses the same erfc expansion as the GPU kernels
 * (erfc(x) = t P(t) e^{-x^2}, t = 1 / (1 + 0.47 x)); e^{-x^2} by 2^y with y split into an integer
 * and a fraction and the degree-7 Taylor series of e^z on |z| <= ln2 / 2.  The reference's SIMD
 * kernels use their own rational approximations of the Ewald correction; the work per pair is
 * comparable.
 */
#include "nbnxm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define CPU_CL 4          /* c_nbnxnCpuIClusterSize */
#define CPU_NSHIFT 45
#define CPU_CENTRAL 22
#define CPU_FAR_AWAY (-1000000.0f)
#define MASK_ALL 0xffffu  /* NBNXN_INTERACTION_MASK_ALL for 4x4 */
#define MASK_DIAG 0x08ceu /* j > i within the cluster: bits i * 4 + j */

static const float c_min_rsq = 3.82e-07f; /* pairlist.h:146 */

typedef float v4f __attribute__((vector_size(16)));
typedef int   v4i __attribute__((vector_size(16)));

typedef struct
{
    int ci, shift, cj_start, cj_end;
} cpu_ci_t;

typedef struct
{
    int      cj;
    uint32_t excl;
} cpu_cj_t;

struct orc_cpu
{
    int          n;
    float        box[3];
    const float* x; /* in box, N*3 (caller's) */
    const float* q;
    const int*   type;
    int          ntypes;
    const float* nbfp; /* ntypes^2 {6C6, 12C12} */
    const int*   excl_index;
    const int*   excl_list;
    float        rc, rlist, beta, epsfac, cpot6, cpot12;
    float        shiftvec[CPU_NSHIFT * 3];
    int          geometric; /* nbfp follows the geometric rule: per-atom sqrt(6C6), sqrt(12C12) */
    float*       sqrt_c6;   /* per type */
    float*       sqrt_c12;
    /* grid */
    int    ncx, ncy, ncol, ncells;
    float  cs[2], ics[2];
    int*   cxy_na;
    int*   cxy_ind;
    int*   atom_indices; /* ncells * 4 */
    int*   cells;        /* n */
    float* xs;           /* per cluster 4 x, 4 y, 4 z, 4 q (SoA per cluster) */
    int*   ts;           /* per slot type (dummy = ntypes for fillers) */
    float* ljc;          /* per cluster 4 sqrt(6C6), then 4 sqrt(12C12) */
    float* bb;           /* per cluster lower xyz, upper xyz */
    float* bbcz;
    int*   flags;
    /* list */
    cpu_ci_t* ci;
    int       nci, cap_ci;
    cpu_cj_t* cj;
    int       ncj, cap_cj;
    /* outputs */
    float* f;            /* grid order, 3 per slot */
    double fshift[CPU_NSHIFT * 3];
    double vc, vlj;
};

static void* cmalloc(size_t n)
{
    void* p = calloc(1, n ? n : 1);
    if (!p)
    {
        abort();
    }
    return p;
}

orc_cpu* orc_cpu_create(int n, const float* x, const float* box, const float* q, const int* type, int ntypes,
                        const float* nbfp, const int* excl_index, const int* excl_list, float rc, float rlist,
                        float beta, float epsfac)
{
    orc_cpu* c = (orc_cpu*)cmalloc(sizeof(orc_cpu));
    c->n       = n;
    memcpy(c->box, box, sizeof(c->box));
    c->x          = x;
    c->q          = q;
    c->type       = type;
    c->ntypes     = ntypes;
    c->nbfp       = nbfp;
    c->excl_index = excl_index;
    c->excl_list  = excl_list;
    c->rc         = rc;
    c->rlist      = rlist;
    c->beta       = beta;
    c->epsfac     = epsfac;
    /* potential shift of LJ at rc (forcerec.cpp:787-816) */
    c->cpot6  = (float)(-1.0 / pow((double)rc, 6.0));
    c->cpot12 = (float)(-1.0 / pow((double)rc, 12.0));
    for (int s = 0, m = -1; m <= 1; m++)
    {
        for (int l = -1; l <= 1; l++)
        {
            for (int k = -2; k <= 2; k++, s++)
            {
                c->shiftvec[3 * s + 0] = k * box[0];
                c->shiftvec[3 * s + 1] = l * box[1];
                c->shiftvec[3 * s + 2] = m * box[2];
            }
        }
    }
    /* combination-rule detection (atomdata.cpp:440-520): geometric when every pair parameter is
     * the product of the diagonal ones' square roots */
    c->sqrt_c6   = (float*)cmalloc(sizeof(float) * (size_t)(ntypes + 1));
    c->sqrt_c12  = (float*)cmalloc(sizeof(float) * (size_t)(ntypes + 1));
    c->geometric = 1;
    for (int i = 0; i < ntypes; i++)
    {
        c->sqrt_c6[i]  = sqrtf(nbfp[2 * (i * ntypes + i)]);
        c->sqrt_c12[i] = sqrtf(nbfp[2 * (i * ntypes + i) + 1]);
    }
    for (int i = 0; i < ntypes && c->geometric; i++)
    {
        for (int j = 0; j < ntypes; j++)
        {
            const float g6  = c->sqrt_c6[i] * c->sqrt_c6[j];
            const float g12 = c->sqrt_c12[i] * c->sqrt_c12[j];
            const float p6 = nbfp[2 * (i * ntypes + j)], p12 = nbfp[2 * (i * ntypes + j) + 1];
            if (fabsf(g6 - p6) > 1e-6f * fabsf(p6) + 1e-30f || fabsf(g12 - p12) > 1e-6f * fabsf(p12) + 1e-30f)
            {
                c->geometric = 0;
                break;
            }
        }
    }
    return c;
}

static void free_grid(orc_cpu* c)
{
    free(c->cxy_na);
    free(c->cxy_ind);
    free(c->atom_indices);
    free(c->cells);
    free(c->xs);
    free(c->ts);
    free(c->ljc);
    free(c->bb);
    free(c->bbcz);
    free(c->flags);
    free(c->f);
    c->cxy_na = c->cxy_ind = c->atom_indices = c->cells = c->ts = c->flags = NULL;
    c->xs = c->ljc = c->bb = c->bbcz = c->f = NULL;
}

void orc_cpu_destroy(orc_cpu* c)
{
    if (!c)
    {
        return;
    }
    free_grid(c);
    free(c->ci);
    free(c->cj);
    free(c->sqrt_c6);
    free(c->sqrt_c12);
    free(c);
}

/* grid.cpp:292-427 sort_atoms: atoms ordered on (coordinate, atom index) */
static void sort_on(int dim, int* a, int n, const float* x)
{
    for (int i = 1; i < n; i++)
    {
        const int   ai = a[i];
        const float xi = x[ai * 3 + dim];
        int         k  = i - 1;
        while (k >= 0)
        {
            const int   ak = a[k];
            const float xk = x[ak * 3 + dim];
            if ((xi > xk) || (xi == xk && ai > ak))
            {
                break;
            }
            a[k + 1] = ak;
            k--;
        }
        a[k + 1] = ai;
    }
}

static int has_vdw(const orc_cpu* c, int t)
{
    for (int j = 0; j < c->ntypes; j++)
    {
        if (c->nbfp[2 * (t * c->ntypes + j)] != 0.0f || c->nbfp[2 * (t * c->ntypes + j) + 1] != 0.0f)
        {
            return 1;
        }
    }
    return 0;
}

void orc_cpu_grid(orc_cpu* c)
{
    free_grid(c);
    const int   n       = c->n;
    const float det     = c->box[0] * (c->box[1] * c->box[2]);
    const float density = (float)n / det;
    /* setDimensions, CPU geometry: cubic cells of max(4, 4) atoms */
    if (n > CPU_CL)
    {
        const float tlen = cbrtf((float)CPU_CL / density);
        c->ncx           = (int)(c->box[0] / tlen);
        c->ncy           = (int)(c->box[1] / tlen);
        c->ncx           = c->ncx < 1 ? 1 : c->ncx;
        c->ncy           = c->ncy < 1 ? 1 : c->ncy;
    }
    else
    {
        c->ncx = c->ncy = 1;
    }
    c->cs[0]   = c->box[0] / c->ncx;
    c->cs[1]   = c->box[1] / c->ncy;
    c->ics[0]  = 1 / c->cs[0];
    c->ics[1]  = 1 / c->cs[1];
    c->ncol    = c->ncx * c->ncy;
    int* col   = (int*)cmalloc(sizeof(int) * (size_t)(n + 1));
    c->cxy_na  = (int*)cmalloc(sizeof(int) * (size_t)(c->ncol + 1));
    c->cxy_ind = (int*)cmalloc(sizeof(int) * (size_t)(c->ncol + 2));
    for (int i = 0; i < n; i++)
    {
        int cx = (int)(c->x[i * 3 + 0] * c->ics[0]);
        int cy = (int)(c->x[i * 3 + 1] * c->ics[1]);
        cx     = cx < c->ncx - 1 ? cx : c->ncx - 1;
        cy     = cy < c->ncy - 1 ? cy : c->ncy - 1;
        col[i] = cx * c->ncy + cy;
        c->cxy_na[col[i]]++;
    }
    /* setCellIndices: cells (= clusters of 4) per column */
    for (int i = 0; i < c->ncol; i++)
    {
        c->cxy_ind[i + 1] = c->cxy_ind[i] + (c->cxy_na[i] + CPU_CL - 1) / CPU_CL;
    }
    c->ncells       = c->cxy_ind[c->ncol];
    const int npad  = c->ncells * CPU_CL;
    c->atom_indices = (int*)cmalloc(sizeof(int) * (size_t)(npad + 1));
    c->cells        = (int*)cmalloc(sizeof(int) * (size_t)(n + 1));
    c->xs           = (float*)cmalloc(sizeof(float) * (size_t)(c->ncells + 1) * 16);
    c->ts           = (int*)cmalloc(sizeof(int) * (size_t)(npad + 1));
    c->ljc          = (float*)cmalloc(sizeof(float) * (size_t)(c->ncells + 1) * 8);
    c->bb           = (float*)cmalloc(sizeof(float) * (size_t)(c->ncells + 1) * 6);
    c->bbcz         = (float*)cmalloc(sizeof(float) * (size_t)(c->ncells + 1) * 2);
    c->flags        = (int*)cmalloc(sizeof(int) * (size_t)(c->ncells + 1));
    c->f            = (float*)cmalloc(sizeof(float) * (size_t)(npad + 1) * 3);
    int* fill       = (int*)cmalloc(sizeof(int) * (size_t)(c->ncol + 1));
    for (int i = 0; i < n; i++)
    {
        c->atom_indices[c->cxy_ind[col[i]] * CPU_CL + fill[col[i]]++] = i;
    }
    free(fill);
    free(col);
    /* sortColumnsCpuGeometry: z-sort per column, cells of 4 consecutive atoms */
    for (int cxy = 0; cxy < c->ncol; cxy++)
    {
        const int na     = c->cxy_na[cxy];
        const int ncz    = c->cxy_ind[cxy + 1] - c->cxy_ind[cxy];
        const int offset = c->cxy_ind[cxy] * CPU_CL;
        sort_on(2, c->atom_indices + offset, na, c->x);
        for (int ind = na; ind < ncz * CPU_CL; ind++)
        {
            c->atom_indices[offset + ind] = -1;
        }
        for (int cz = 0; cz < ncz; cz++)
        {
            const int cell = c->cxy_ind[cxy] + cz;
            int*      a    = c->atom_indices + cell * CPU_CL;
            /* sort_cluster_on_flag: atoms with LJ first when at most half have LJ and the last of
             * them sits in the second half of the cluster */
            int sort1[CPU_CL], sort2[CPU_CL], n1 = 0, n2 = 0, last_lj = -1, haveq = 0;
            for (int k = 0; k < CPU_CL; k++)
            {
                if (a[k] < 0)
                {
                    continue;
                }
                haveq = haveq || c->q[a[k]] != 0.0f;
                if (has_vdw(c, c->type[a[k]]))
                {
                    sort1[n1++] = a[k];
                    last_lj     = k;
                }
                else
                {
                    sort2[n2++] = a[k];
                }
            }
            c->flags[cell] = (n1 > 0 ? 1 : 0) | (haveq ? 2 : 0);
            if (n1 > 0 && 2 * n1 <= CPU_CL && 2 * last_lj >= CPU_CL)
            {
                for (int k = 0; k < n1; k++)
                {
                    a[k] = sort1[k];
                }
                for (int k = 0; k < n2; k++)
                {
                    a[n1 + k] = sort2[k];
                }
            }
            /* fillCell: cells, coordinates (fillers far away), bounding box of the real atoms */
            float* xc    = c->xs + (size_t)cell * 16;
            float  lo[3] = { 0, 0, 0 }, hi[3] = { 0, 0, 0 };
            int    first = 1;
            for (int k = 0; k < CPU_CL; k++)
            {
                const int at = a[k];
                const int sl = cell * CPU_CL + k;
                if (at >= 0)
                {
                    c->cells[at] = sl;
                    for (int d = 0; d < 3; d++)
                    {
                        const float v = c->x[at * 3 + d];
                        xc[4 * d + k] = v;
                        lo[d]         = first || v < lo[d] ? v : lo[d];
                        hi[d]         = first || v > hi[d] ? v : hi[d];
                    }
                    first                    = 0;
                    xc[12 + k]               = c->q[at];
                    c->ts[sl]                = c->type[at];
                    c->ljc[cell * 8 + k]     = c->sqrt_c6[c->type[at]];
                    c->ljc[cell * 8 + 4 + k] = c->sqrt_c12[c->type[at]];
                }
                else
                {
                    for (int d = 0; d < 3; d++)
                    {
                        xc[4 * d + k] = CPU_FAR_AWAY;
                    }
                    xc[12 + k]               = 0.0f;
                    c->ts[sl]                = c->ntypes;
                    c->ljc[cell * 8 + k]     = 0.0f;
                    c->ljc[cell * 8 + 4 + k] = 0.0f;
                }
            }
            for (int d = 0; d < 3; d++)
            {
                c->bb[cell * 6 + d]     = lo[d];
                c->bb[cell * 6 + 3 + d] = hi[d];
            }
            c->bbcz[cell * 2]     = lo[2];
            c->bbcz[cell * 2 + 1] = hi[2];
        }
    }
}

void orc_cpu_set_x(orc_cpu* c, const float* x)
{
    for (int cell = 0; cell < c->ncells; cell++)
    {
        for (int k = 0; k < CPU_CL; k++)
        {
            const int at = c->atom_indices[cell * CPU_CL + k];
            if (at >= 0)
            {
                for (int d = 0; d < 3; d++)
                {
                    c->xs[(size_t)cell * 16 + 4 * d + k] = x[at * 3 + d];
                }
            }
        }
    }
}

static float bb_dist2(const float* bi, const float* bj)
{
    float d2 = 0;
    for (int d = 0; d < 3; d++)
    {
        const float dl  = bi[d] - bj[3 + d];
        const float dh  = bj[d] - bi[3 + d];
        const float dm  = dl > dh ? dl : dh;
        const float dm0 = dm > 0.0f ? dm : 0.0f;
        d2 += dm0 * dm0;
    }
    return d2;
}

/* pairlist.cpp:286-309 get_cell_range (lower corner 0) */
static void cell_range(float b0, float b1, int numCells, float cellSize, float invCellSize, float d2, float rlist,
                       int* cf, int* cl)
{
    const float r2 = rlist * rlist;
    *cf            = (int)(b0 * invCellSize);
    *cf            = *cf > 0 ? *cf : 0;
    while (*cf > 0)
    {
        const float t = b0 - (*cf - 1 + 1) * cellSize;
        if (!(d2 + t * t < r2))
        {
            break;
        }
        (*cf)--;
    }
    *cl = (int)(b1 * invCellSize);
    *cl = *cl < numCells - 1 ? *cl : numCells - 1;
    while (*cl < numCells - 1)
    {
        const float t = (*cl + 1) * cellSize - b1;
        if (!(d2 + t * t < r2))
        {
            break;
        }
        (*cl)++;
    }
}

static void push_cj(orc_cpu* c, int cj, uint32_t excl)
{
    if (c->ncj == c->cap_cj)
    {
        c->cap_cj = c->cap_cj ? 2 * c->cap_cj : 1024;
        c->cj     = (cpu_cj_t*)realloc(c->cj, sizeof(cpu_cj_t) * (size_t)c->cap_cj);
        if (!c->cj)
        {
            abort();
        }
    }
    c->cj[c->ncj].cj   = cj;
    c->cj[c->ncj].excl = excl;
    c->ncj++;
}

static int any_pair_in_range(const orc_cpu* c, const float* x_ci, int jc, float rlist2)
{
    const float* xj = c->xs + (size_t)jc * 16;
    int          in = 0;
    for (int i = 0; i < CPU_CL && !in; i++)
    {
        for (int j = 0; j < CPU_CL; j++)
        {
            const float dx = x_ci[i * 3] - xj[j], dy = x_ci[i * 3 + 1] - xj[4 + j], dz = x_ci[i * 3 + 2] - xj[8 + j];
            in             = in || (dx * dx + dy * dy + dz * dz < rlist2);
        }
    }
    return in;
}

/* makeClusterListSimple: the contiguous j-cluster range from the first to the last cluster in
 * range (bounding-box distance below rbb2, or below rlist2 with an atom pair within rlist) */
static void cluster_list_simple(orc_cpu* c, const float* bb_ci, const float* x_ci, int icluster, int jfirst,
                                int jlast, int excludeSubDiagonal, float rlist2, float rbb2)
{
    int in_range = 0;
    while (!in_range && jfirst <= jlast)
    {
        const float d2 = bb_dist2(bb_ci, c->bb + (size_t)jfirst * 6);
        in_range       = d2 < rbb2 || (d2 < rlist2 && any_pair_in_range(c, x_ci, jfirst, rlist2));
        if (!in_range)
        {
            jfirst++;
        }
    }
    if (!in_range)
    {
        return;
    }
    in_range = 0;
    while (!in_range && jlast > jfirst)
    {
        const float d2 = bb_dist2(bb_ci, c->bb + (size_t)jlast * 6);
        in_range       = d2 < rbb2 || (d2 < rlist2 && any_pair_in_range(c, x_ci, jlast, rlist2));
        if (!in_range)
        {
            jlast--;
        }
    }
    for (int jc = jfirst; jc <= jlast; jc++)
    {
        push_cj(c, jc, (excludeSubDiagonal && icluster == jc) ? MASK_DIAG : MASK_ALL);
    }
    c->ci[c->nci - 1].cj_end = c->ncj;
}

/* setExclusionsForIEntry (CPU list): clear the bits of topology exclusions; the j-list of an
 * entry is sorted on cluster index */
static void set_exclusions_cpu(orc_cpu* c, int diagRemoved)
{
    const cpu_ci_t* e = &c->ci[c->nci - 1];
    if (e->cj_end == e->cj_start)
    {
        return;
    }
    const int cjFirst = c->cj[e->cj_start].cj, cjLast = c->cj[e->cj_end - 1].cj;
    for (int i = 0; i < CPU_CL; i++)
    {
        const int iIndex = e->ci * CPU_CL + i;
        const int iAtom  = c->atom_indices[iIndex];
        if (iAtom < 0)
        {
            continue;
        }
        for (int k = c->excl_index[iAtom]; k < c->excl_index[iAtom + 1]; k++)
        {
            const int jAtom = c->excl_list[k];
            if (jAtom == iAtom)
            {
                continue;
            }
            const int jIndex = c->cells[jAtom];
            if (diagRemoved && jIndex <= iIndex)
            {
                continue;
            }
            const int jCluster = jIndex / CPU_CL;
            if (jCluster < cjFirst || jCluster > cjLast)
            {
                continue;
            }
            int lo = e->cj_start, hi = e->cj_end - 1, idx = -1;
            while (lo <= hi)
            {
                const int mid = (lo + hi) / 2;
                if (c->cj[mid].cj == jCluster)
                {
                    idx = mid;
                    break;
                }
                if (c->cj[mid].cj < jCluster)
                {
                    lo = mid + 1;
                }
                else
                {
                    hi = mid - 1;
                }
            }
            if (idx >= 0)
            {
                c->cj[idx].excl &= ~(1u << (i * CPU_CL + (jIndex - jCluster * CPU_CL)));
            }
        }
    }
}

/* closeIEntry (CPU list): entries with exclusions first (sort_cj_excl), empty entries removed */
static void close_entry(orc_cpu* c)
{
    cpu_ci_t* e   = &c->ci[c->nci - 1];
    const int len = e->cj_end - e->cj_start;
    if (len == 0)
    {
        c->nci--;
        return;
    }
    cpu_cj_t* cj   = c->cj + e->cj_start;
    int       nexc = 0;
    for (int j = 0; j < len; j++)
    {
        nexc += cj[j].excl != MASK_ALL;
    }
    if (!(nexc == 0 || (nexc == 1 && cj[0].excl != MASK_ALL)))
    {
        cpu_cj_t* tmp = (cpu_cj_t*)cmalloc(sizeof(cpu_cj_t) * (size_t)len);
        int       k   = 0;
        for (int j = 0; j < len; j++)
        {
            if (cj[j].excl != MASK_ALL)
            {
                tmp[k++] = cj[j];
            }
        }
        for (int j = 0; j < len; j++)
        {
            if (cj[j].excl == MASK_ALL)
            {
                tmp[k++] = cj[j];
            }
        }
        memcpy(cj, tmp, sizeof(cpu_cj_t) * (size_t)len);
        free(tmp);
    }
}

void orc_cpu_search(orc_cpu* c)
{
    c->nci = c->ncj = 0;
    const float rlist  = c->rlist;
    const float rlist2 = rlist * rlist;
    /* boundingbox_only_distance2, simple lists */
    float rbb2;
    {
        const float  bbx = (float)(0.5 * (c->cs[0] + c->cs[0]));
        const float  bby = (float)(0.5 * (c->cs[1] + c->cs[1]));
        const double r   = (double)rlist - 0.5 * (double)sqrtf(bbx * bbx + bby * bby);
        rbb2             = (float)(r > 0.0 ? r : 0.0);
        rbb2             = rbb2 * rbb2;
    }
    const float* box    = c->box;
    int          shp[3] = { 1, 1, 1 };
    if (box[0] < rlist)
    {
        shp[0] = 2;
    }
    for (int cxy = 0; cxy < c->ncol; cxy++)
    {
        const int ci_x = cxy / c->ncy, ci_y = cxy - ci_x * c->ncy;
        const int ncz  = c->cxy_ind[cxy + 1] - c->cxy_ind[cxy];
        for (int ci = c->cxy_ind[cxy]; ci < c->cxy_ind[cxy + 1]; ci++)
        {
            if (c->flags[ci] == 0)
            {
                continue;
            }
            const float* bbi = c->bb + (size_t)ci * 6;
            for (int tz = -shp[2]; tz <= shp[2]; tz++)
            {
                const float shz = (float)tz * box[2];
                const float bz0 = c->bbcz[ci * 2] + shz, bz1 = c->bbcz[ci * 2 + 1] + shz;
                float       d2z = 0.0f;
                if (tz < 0)
                {
                    d2z = bz1 * bz1;
                }
                else if (tz > 0)
                {
                    d2z = (bz0 - box[2]) * (bz0 - box[2]);
                }
                if (d2z >= rlist2)
                {
                    continue;
                }
                float bz1_frac = bz1 / (float)ncz;
                bz1_frac       = bz1_frac < 0 ? 0 : bz1_frac;
                for (int ty = -shp[1]; ty <= shp[1]; ty++)
                {
                    const float shy = (float)ty * box[1];
                    const float by0 = bbi[1] + shy, by1 = bbi[4] + shy;
                    int         cyf, cyl;
                    cell_range(by0, by1, c->ncy, c->cs[1], c->ics[1], d2z, rlist, &cyf, &cyl);
                    if (cyf > cyl)
                    {
                        continue;
                    }
                    float d2z_cy = d2z;
                    if (by1 < 0)
                    {
                        d2z_cy += by1 * by1;
                    }
                    else if (by0 > box[1])
                    {
                        d2z_cy += (by0 - box[1]) * (by0 - box[1]);
                    }
                    for (int tx = -shp[0]; tx <= shp[0]; tx++)
                    {
                        const int shift              = 5 * (3 * (tz + 1) + ty + 1) + tx + 2;
                        const int excludeSubDiagonal = (shift == CPU_CENTRAL);
                        if (shift > CPU_CENTRAL)
                        {
                            continue; /* c_pbcShiftBackward: half of the shifts */
                        }
                        const float shx = (float)tx * box[0];
                        const float bx0 = bbi[0] + shx, bx1 = bbi[3] + shx;
                        int         cxf, cxl;
                        cell_range(bx0, bx1, c->ncx, c->cs[0], c->ics[0], d2z_cy, rlist, &cxf, &cxl);
                        if (cxf > cxl)
                        {
                            continue;
                        }
                        if (c->nci == c->cap_ci)
                        {
                            c->cap_ci = c->cap_ci ? 2 * c->cap_ci : 1024;
                            c->ci     = (cpu_ci_t*)realloc(c->ci, sizeof(cpu_ci_t) * (size_t)c->cap_ci);
                            if (!c->ci)
                            {
                                abort();
                            }
                        }
                        cpu_ci_t* e = &c->ci[c->nci++];
                        e->ci       = ci;
                        e->shift    = shift;
                        e->cj_start = e->cj_end = c->ncj;
                        if (excludeSubDiagonal && cxf < ci_x)
                        {
                            cxf = ci_x;
                        }
                        /* shifted i bounding box and coordinates (set_icell_bb, icell_set_x) */
                        float bb_ci[6], x_ci[CPU_CL * 3];
                        bb_ci[0] = bbi[0] + shx;
                        bb_ci[1] = bbi[1] + shy;
                        bb_ci[2] = bbi[2] + shz;
                        bb_ci[3] = bbi[3] + shx;
                        bb_ci[4] = bbi[4] + shy;
                        bb_ci[5] = bbi[5] + shz;
                        for (int i = 0; i < CPU_CL; i++)
                        {
                            x_ci[i * 3 + 0] = c->xs[(size_t)ci * 16 + i] + shx;
                            x_ci[i * 3 + 1] = c->xs[(size_t)ci * 16 + 4 + i] + shy;
                            x_ci[i * 3 + 2] = c->xs[(size_t)ci * 16 + 8 + i] + shz;
                        }
                        for (int cx = cxf; cx <= cxl; cx++)
                        {
                            float d2zx = d2z;
                            if ((float)cx * c->cs[0] > bx1)
                            {
                                d2zx += ((float)cx * c->cs[0] - bx1) * ((float)cx * c->cs[0] - bx1);
                            }
                            else if (((float)cx + 1) * c->cs[0] < bx0)
                            {
                                d2zx += (((float)cx + 1) * c->cs[0] - bx0) * (((float)cx + 1) * c->cs[0] - bx0);
                            }
                            const int cyf_x = (cx == 0 && excludeSubDiagonal && cyf < ci_y) ? ci_y : cyf;
                            for (int cy = cyf_x; cy <= cyl; cy++)
                            {
                                const int colj   = cx * c->ncy + cy;
                                const int cstart = c->cxy_ind[colj], cend = c->cxy_ind[colj + 1];
                                float     d2zxy  = d2zx;
                                if ((float)cy * c->cs[1] > by1)
                                {
                                    d2zxy += ((float)cy * c->cs[1] - by1) * ((float)cy * c->cs[1] - by1);
                                }
                                else if (((float)cy + 1) * c->cs[1] < by0)
                                {
                                    d2zxy += (((float)cy + 1) * c->cs[1] - by0) * (((float)cy + 1) * c->cs[1] - by0);
                                }
                                if (!(cstart < cend && d2zxy < rlist2))
                                {
                                    continue;
                                }
                                int mid = cstart + (int)(bz1_frac * (float)(cend - cstart));
                                mid     = mid >= cend ? cend - 1 : mid;
                                const float d2xy = d2zxy - d2z;
                                int         down = mid;
                                while (down >= cstart
                                       && (c->bbcz[down * 2 + 1] >= bz0
                                           || d2xy + (c->bbcz[down * 2 + 1] - bz0) * (c->bbcz[down * 2 + 1] - bz0)
                                                      < rlist2))
                                {
                                    down--;
                                }
                                int first = down + 1;
                                int up    = mid + 1;
                                while (up < cend
                                       && (c->bbcz[up * 2] <= bz1
                                           || d2xy + (c->bbcz[up * 2] - bz1) * (c->bbcz[up * 2] - bz1) < rlist2))
                                {
                                    up++;
                                }
                                const int last = up - 1;
                                if (excludeSubDiagonal && first < ci)
                                {
                                    first = ci;
                                }
                                if (first <= last)
                                {
                                    cluster_list_simple(c, bb_ci, x_ci, ci, first, last, excludeSubDiagonal, rlist2,
                                                        rbb2);
                                }
                            }
                        }
                        set_exclusions_cpu(c, excludeSubDiagonal);
                        close_entry(c);
                    }
                }
            }
        }
    }
}

/* ---- the 4-wide cluster-pair kernel ---- */

static inline v4f vsel(v4i m, v4f a, v4f b)
{
    return (v4f)(((v4i)a & m) | ((v4i)b & ~m));
}

static inline v4f v4(float a)
{
    return (v4f){ a, a, a, a };
}

/* 2^y for y <= 0 (|y| < 126): y = n + f with n = round(y), e^(f ln 2) by its Taylor series */
static inline v4f vexp2_neg(v4f y)
{
    y            = vsel(y < v4(-125.0f), v4(-125.0f), y);
    const v4i n  = __builtin_convertvector(y - v4(0.5f), v4i); /* truncation = rounding for y <= 0 */
    const v4f nf = __builtin_convertvector(n, v4f);
    const v4f z  = (y - nf) * v4(0.69314718055994531f);
    v4f       p  = v4(1.0f / 5040.0f);
    p            = p * z + v4(1.0f / 720.0f);
    p            = p * z + v4(1.0f / 120.0f);
    p            = p * z + v4(1.0f / 24.0f);
    p            = p * z + v4(1.0f / 6.0f);
    p            = p * z + v4(0.5f);
    p            = p * z + v4(1.0f);
    p            = p * z + v4(1.0f);
    const v4i e  = (n + (v4i){ 127, 127, 127, 127 }) << 23;
    return p * (v4f)e;
}

static inline v4f vrsqrt(v4f x)
{
    v4f r;
    for (int l = 0; l < 4; l++)
    {
        r[l] = 1.0f / sqrtf(x[l]);
    }
    return r;
}

typedef struct
{
    const orc_cpu* c;
    int            e0, e1, energy;
    float*         f;
    double         fsh[CPU_NSHIFT * 3];
    double         vc, vlj;
} cpu_task;

static void kernel_range(cpu_task* t)
{
    const orc_cpu* c      = t->c;
    const float    rc2    = c->rc * c->rc;
    const float    beta   = c->beta;
    const float    pbeta  = 0.47f * beta;
    const float    b2l2   = beta * beta * 1.4426950408889634f;
    const float    c2b    = 1.1283791670955126f * beta;
    const float    epsfac = c->epsfac;
    const int      nt     = c->ntypes;
    const int      geom   = c->geometric;
    double         vc = 0.0, vlj = 0.0;
    float*         f = t->f;
    for (int e = t->e0; e < t->e1; e++)
    {
        const cpu_ci_t* ce = &c->ci[e];
        const int       ci = ce->ci;
        const float*    sv = c->shiftvec + 3 * ce->shift;
        const float*    xi = c->xs + (size_t)ci * 16;
        v4f             ix[CPU_CL], iy[CPU_CL], iz[CPU_CL], iq[CPU_CL], fix[CPU_CL], fiy[CPU_CL], fiz[CPU_CL];
        v4f             ic6[CPU_CL], ic12[CPU_CL];
        int             ti[CPU_CL];
        for (int i = 0; i < CPU_CL; i++)
        {
            ix[i]   = v4(xi[i] + sv[0]);
            iy[i]   = v4(xi[4 + i] + sv[1]);
            iz[i]   = v4(xi[8 + i] + sv[2]);
            iq[i]   = v4(xi[12 + i] * epsfac);
            ic6[i]  = v4(c->ljc[ci * 8 + i]);
            ic12[i] = v4(c->ljc[ci * 8 + 4 + i]);
            ti[i]   = c->ts[ci * CPU_CL + i];
            fix[i] = fiy[i] = fiz[i] = v4(0.0f);
        }
        v4f vctot = v4(0.0f), vljtot = v4(0.0f);
        for (int k = ce->cj_start; k < ce->cj_end; k++)
        {
            const int      cj   = c->cj[k].cj;
            const uint32_t excl = c->cj[k].excl;
            const float*   xj   = c->xs + (size_t)cj * 16;
            v4f            jx, jy, jz, jq, jc6, jc12;
            memcpy(&jx, xj, 16);
            memcpy(&jy, xj + 4, 16);
            memcpy(&jz, xj + 8, 16);
            memcpy(&jq, xj + 12, 16);
            memcpy(&jc6, c->ljc + cj * 8, 16);
            memcpy(&jc12, c->ljc + cj * 8 + 4, 16);
            const int diag = (ce->shift == CPU_CENTRAL && cj == ci);
            v4f       fjx = v4(0.0f), fjy = v4(0.0f), fjz = v4(0.0f);
            for (int i = 0; i < CPU_CL; i++)
            {
                const v4f dx   = ix[i] - jx, dy = iy[i] - jy, dz = iz[i] - jz;
                v4f       rsq  = dx * dx + dy * dy + dz * dz;
                const v4i wco  = rsq < v4(rc2);
                const v4i intm = -(v4i){ (int)((excl >> (i * 4 + 0)) & 1u), (int)((excl >> (i * 4 + 1)) & 1u),
                                         (int)((excl >> (i * 4 + 2)) & 1u), (int)((excl >> (i * 4 + 3)) & 1u) };
                /* the diagonal's lower triangle (with the self pair) is outside the pair set */
                const v4i selfm = diag ? (v4i){ 0 > i ? -1 : 0, 1 > i ? -1 : 0, 2 > i ? -1 : 0, 3 > i ? -1 : 0 }
                                       : (v4i){ -1, -1, -1, -1 };
                const v4i inr   = wco & selfm;
                rsq             = vsel(rsq < v4(c_min_rsq), v4(c_min_rsq), rsq);
                const v4f rinv  = vsel(inr, vrsqrt(rsq), v4(0.0f));
                const v4f rinv2 = rinv * rinv;
                const v4f rinv6 = vsel(intm, rinv2 * rinv2 * rinv2, v4(0.0f));
                v4f       c6, c12;
                if (geom)
                {
                    c6  = ic6[i] * jc6;
                    c12 = ic12[i] * jc12;
                }
                else
                {
                    for (int l = 0; l < 4; l++)
                    {
                        const int tj = c->ts[cj * CPU_CL + l];
                        c6[l]        = tj < nt && ti[i] < nt ? c->nbfp[2 * (ti[i] * nt + tj)] : 0.0f;
                        c12[l]       = tj < nt && ti[i] < nt ? c->nbfp[2 * (ti[i] * nt + tj) + 1] : 0.0f;
                    }
                }
                const v4f vdisp = c6 * rinv6, vrep = c12 * rinv6 * rinv6;
                /* Ewald: erfc(beta r) / r = t P(t) e^{-beta^2 r^2} / r */
                const v4f r    = rsq * rinv;
                const v4f t1   = v4(1.0f) / (v4(1.0f) + v4(pbeta) * r);
                v4f       p    = v4(1.128007565e-02f);
                p              = p * t1 + v4(3.713922575e-02f);
                p              = p * t1 + v4(-3.248904943e-01f);
                p              = p * t1 + v4(5.147097111e-01f);
                p              = p * t1 + v4(-7.699845731e-02f);
                p              = p * t1 + v4(3.232774734e-01f);
                p              = p * t1 + v4(2.490737736e-01f);
                p              = p * t1 + v4(2.664087117e-01f);
                const v4f expm = vexp2_neg(v4(-b2l2) * rsq);
                const v4f tpr  = t1 * p * rinv;
                /* excluded pairs inside the cut-off keep only the Ewald correction */
                const v4f fcr2 = vsel(intm, expm * (tpr + v4(c2b)), expm * (tpr + v4(c2b)) - rinv);
                const v4f qq   = iq[i] * jq;
                const v4f fs   = (qq * fcr2 + vrep - vdisp) * rinv2;
                fix[i] += fs * dx;
                fiy[i] += fs * dy;
                fiz[i] += fs * dz;
                fjx -= fs * dx;
                fjy -= fs * dy;
                fjz -= fs * dz;
                if (t->energy)
                {
                    const v4i cnt = inr & intm;
                    /* LJ with the potential shift; Coulomb erfc(beta r)/r, and for excluded pairs
                     * inside the cut-off -erf(beta r)/r = erfc(beta r)/r - 1/r */
                    const v4f vl = vsel(cnt, (vrep + v4(c->cpot12) * c12) * v4(1.0f / 12.0f)
                                                     - (vdisp + v4(c->cpot6) * c6) * v4(1.0f / 6.0f),
                                        v4(0.0f));
                    const v4f ve = vsel(cnt, qq * tpr * expm, vsel(inr, qq * (tpr * expm - rinv), v4(0.0f)));
                    vljtot += vl;
                    vctot += ve;
                }
            }
            float* fj = f + (size_t)cj * CPU_CL * 3;
            for (int l = 0; l < 4; l++)
            {
                fj[l * 3 + 0] += fjx[l];
                fj[l * 3 + 1] += fjy[l];
                fj[l * 3 + 2] += fjz[l];
            }
        }
        float sx = 0, sy = 0, sz = 0;
        for (int i = 0; i < CPU_CL; i++)
        {
            const float fx = fix[i][0] + fix[i][1] + fix[i][2] + fix[i][3];
            const float fy = fiy[i][0] + fiy[i][1] + fiy[i][2] + fiy[i][3];
            const float fz = fiz[i][0] + fiz[i][1] + fiz[i][2] + fiz[i][3];
            f[(ci * CPU_CL + i) * 3 + 0] += fx;
            f[(ci * CPU_CL + i) * 3 + 1] += fy;
            f[(ci * CPU_CL + i) * 3 + 2] += fz;
            sx += fx;
            sy += fy;
            sz += fz;
        }
        t->fsh[3 * ce->shift + 0] += sx;
        t->fsh[3 * ce->shift + 1] += sy;
        t->fsh[3 * ce->shift + 2] += sz;
        if (t->energy)
        {
            vc += (double)(vctot[0] + vctot[1] + vctot[2] + vctot[3]);
            vlj += (double)(vljtot[0] + vljtot[1] + vljtot[2] + vljtot[3]);
            /* the self term, once per i-cluster on its central diagonal entry */
            if (ce->shift == CPU_CENTRAL)
            {
                for (int k = ce->cj_start; k < ce->cj_end; k++)
                {
                    if (c->cj[k].cj == ci)
                    {
                        for (int i = 0; i < CPU_CL; i++)
                        {
                            vc -= (double)xi[12 + i] * (double)xi[12 + i] * (double)epsfac * (double)beta
                                  * 0.56418958354775628695;
                        }
                        break;
                    }
                }
            }
        }
    }
    t->vc  = vc;
    t->vlj = vlj;
}

static void* kernel_thread(void* arg)
{
    kernel_range((cpu_task*)arg);
    return NULL;
}

int orc_cpu_force(orc_cpu* c, int e0, int e1, int energy, int nthreads)
{
    e0              = e0 < 0 ? 0 : e0;
    e1              = e1 > c->nci ? c->nci : e1;
    nthreads        = nthreads < 1 ? 1 : nthreads;
    const size_t nf = (size_t)c->ncells * CPU_CL * 3;
    cpu_task*    tk = (cpu_task*)cmalloc(sizeof(cpu_task) * (size_t)nthreads);
    pthread_t*   th = (pthread_t*)cmalloc(sizeof(pthread_t) * (size_t)nthreads);
    /* split the entries by their j-cluster counts */
    long long total = 0;
    for (int e = e0; e < e1; e++)
    {
        total += c->ci[e].cj_end - c->ci[e].cj_start + 1;
    }
    memset(c->f, 0, sizeof(float) * nf);
    int       e   = e0;
    long long acc = 0;
    for (int t = 0; t < nthreads; t++)
    {
        tk[t].c              = c;
        tk[t].energy         = energy;
        tk[t].e0             = e;
        const long long goal = total * (t + 1) / nthreads;
        while (e < e1 && acc < goal)
        {
            acc += c->ci[e].cj_end - c->ci[e].cj_start + 1;
            e++;
        }
        tk[t].e1 = (t == nthreads - 1) ? e1 : e;
        tk[t].f  = t == 0 ? c->f : (float*)cmalloc(sizeof(float) * nf);
    }
    int started = 0, ok = 1;
    for (int t = 1; t < nthreads; t++, started++)
    {
        if (pthread_create(&th[t], NULL, kernel_thread, &tk[t]) != 0)
        {
            ok = 0;
            break;
        }
    }
    kernel_range(&tk[0]);
    for (int t = 1; t <= started; t++)
    {
        pthread_join(th[t], NULL);
    }
    c->vc = c->vlj = 0.0;
    memset(c->fshift, 0, sizeof(c->fshift));
    for (int t = 0; t < nthreads; t++)
    {
        if (t > 0 && ok)
        {
            for (size_t k = 0; k < nf; k++)
            {
                c->f[k] += tk[t].f[k];
            }
        }
        for (int k = 0; k < CPU_NSHIFT * 3; k++)
        {
            c->fshift[k] += tk[t].fsh[k];
        }
        c->vc += tk[t].vc;
        c->vlj += tk[t].vlj;
        if (t > 0)
        {
            free(tk[t].f);
        }
    }
    free(tk);
    free(th);
    return ok ? 0 : -1;
}

/* ---- outputs ---- */
void orc_cpu_sizes(const orc_cpu* c, int* s4)
{
    s4[0] = c->ncells;
    s4[1] = c->nci;
    s4[2] = c->ncj;
    s4[3] = c->geometric;
}

void orc_cpu_list(const orc_cpu* c, int* ci4, int* cj2)
{
    for (int e = 0; e < c->nci; e++)
    {
        ci4[4 * e + 0] = c->ci[e].ci;
        ci4[4 * e + 1] = c->ci[e].shift;
        ci4[4 * e + 2] = c->ci[e].cj_start;
        ci4[4 * e + 3] = c->ci[e].cj_end;
    }
    for (int k = 0; k < c->ncj; k++)
    {
        cj2[2 * k]     = c->cj[k].cj;
        cj2[2 * k + 1] = (int)c->cj[k].excl;
    }
}

void orc_cpu_grid_arrays(const orc_cpu* c, int* atom_indices, float* xs)
{
    memcpy(atom_indices, c->atom_indices, sizeof(int) * (size_t)c->ncells * CPU_CL);
    memcpy(xs, c->xs, sizeof(float) * (size_t)c->ncells * 16);
}

void orc_cpu_forces(const orc_cpu* c, float* f_out)
{
    for (int a = 0; a < c->n; a++)
    {
        const int s = c->cells[a];
        for (int d = 0; d < 3; d++)
        {
            f_out[a * 3 + d] = c->f[s * 3 + d];
        }
    }
}

void orc_cpu_energies(const orc_cpu* c, double* e2)
{
    e2[0] = c->vlj;
    e2[1] = c->vc;
}
