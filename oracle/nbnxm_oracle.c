/*
 * CPU oracle for the short-range nonbonded path -- TEST INFRASTRUCTURE ONLY.
 * See nbnxm_oracle.h.  Build with -ffp-contract=off (oracle/Makefile).
 *
 * Deliberate differences from the reference, none of which changes a result
 * that is compared:
 *  - one search "thread", so sci entries come out in cell order; the
 *    reference's OpenMP blocking and its GPU load-balancing split
 *    (pairlist.cpp split_sci_entry :2077-2165, sort_sci :3827) only permute
 *    or cut entries, so the list is the same as a sorted set of cluster pairs;
 *  - energies: the per-pair formulas of kernel_gpu_ref.cpp evaluated in
 *    double on the float pair geometry (float dx, dy, dz, charges and
 *    parameters) and summed in double.  In float, the reference's own
 *    per-pair rounding (e.g. the single rounded qq of every O-H pair of rigid
 *    water) puts its Coulomb total 1e-6..4e-6 away from the exact sum, above
 *    the 1e-6 energy bar the GPU kernel is held to;
 *  - the rolling prune covers entry indices part, part+nparts, ... up to the
 *    end of the list (the reference's (nsci-part)/nparts rounds down,
 *    cuda/nbnxm_cuda.cu:640, and can skip up to nparts-1 trailing entries).
 */
#include "nbnxm_oracle.h"

#include <float.h>
#include <pthread.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Geometry constants of the GPU list (pairlistparams.h:60-89, pairlist.h:146-171) */
#define CL 8           /* atoms per cluster, c_nbnxnGpuClusterSize */
#define NCL 8          /* clusters per super-cluster, c_gpuNumClusterPerCell */
#define SC 64          /* atoms per super-cluster (cell) */
#define JG 4           /* j-clusters per cj4, c_nbnxnGpuJgroupSize */
#define SPLIT 2        /* c_nbnxnGpuClusterpairSplit */
#define EXCLW 32       /* words per exclusion mask, c_nbnxnGpuExclSize */
#define NSHIFT 45      /* SHIFTS, pbcutil/ishift.h:40-47 */
#define CENTRAL 22
#define FAR_AWAY (-1000000.0f) /* atomdata.cpp:146 */
static const float c_minDist2 = 3.82e-07f; /* pairlist.h:146 c_nbnxnMinDistanceSquared */
static const double c_pi = 3.14159265358979323846;
static const double c_1_sqrtpi = 0.56418958354775628695; /* 1/sqrt(pi) */

static int xyz2is(int x, int y, int z) { return 5 * (3 * (z + 1) + y + 1) + x + 2; }

/* pairlist.h:202-221 nbnxn_im_ei_t / nbnxn_cj4_t */
typedef struct
{
    uint32_t imask;
    int      excl_ind;
} imei_t;

typedef struct
{
    int    cj[JG];
    imei_t imei[SPLIT];
} cj4_t;

typedef struct
{
    int sci, shift, cj4_start, cj4_end;
} sci_t;

typedef struct
{
    uint32_t pair[EXCLW];
} excl_t;

struct orc_ctx
{
    /* system */
    int n;
    float box[3];
    float* x; /* in box, N*3 */
    int*   image; /* N*3 box lengths added by the wrap */
    float* q;
    int* type;
    int ntypes;   /* real types */
    int numTypes; /* + dummy */
    float* nbfp;  /* numTypes^2 * 2 */
    int* excl_index;
    int* excl_list;
    /* interaction constants */
    int coulomb;
    float rc, rlist_outer, rlist_inner;
    float beta, epsfac, k_rf, c_rf, sh_ewald;
    float cpot_disp, cpot_rep;
    /* LJ modifier (0 potential shift, 1 force switch, 2 potential switch, 3 none) */
    int   vdw_mod;
    float rvdw_switch;
    float fsw_disp_c2, fsw_disp_c3, fsw_rep_c2, fsw_rep_c3;
    float psw_c3, psw_c4, psw_c5;
    float tab_scale;
    int tab_n;
    float* tabF;
    float* tabV;
    float shiftvec[NSHIFT * 3];
    /* grid */
    int ncx, ncy, ncol, ncells, nclusters_tot;
    float cs[2], ics[2];
    int* cxy_na;
    int* cxy_ind;
    int* nclusters;
    float* bbcz;
    float* bb;
    int* atom_indices;
    int* cells;
    float* xq;
    int* tgrid;
    /* list */
    sci_t* sci;
    int nsci, cap_sci;
    cj4_t* cj4;
    int ncj4, cap_cj4;
    excl_t* excl;
    int nexcl, cap_excl;
    uint32_t* imask_outer;
    float rbb2;
    /* outputs */
    float* fnb;
    /* shift forces summed in double (the reference's are `real`): the virial's shift part is a
     * difference of large sums in small boxes, whose float rounding would dominate the check */
    double fshift[NSHIFT * 3];
    double vc, vlj;
};

double orc_one_4pi_eps0(void)
{
    /* units.h:69-79 */
    const double eps0 = (8.8541878128e-12 * 1e-9 * 1e3) / (1.602176634e-19 * 1.602176634e-19 * 6.02214076e23);
    return 1.0 / (4.0 * c_pi * eps0);
}

/* ewald/ewald_utils.cpp:46-71, in single precision ("real") */
static float calc_ewaldcoeff_q(float rc, float rtol)
{
    float beta = 5, low, high;
    int   n, i = 0;
    do
    {
        i++;
        beta *= 2;
    } while (erfcf(beta * rc) > rtol);
    n    = i + 60;
    low  = 0;
    high = beta;
    for (i = 0; i < n; i++)
    {
        beta = (low + high) / 2;
        if (erfcf(beta * rc) > rtol)
        {
            low = beta;
        }
        else
        {
            high = beta;
        }
    }
    return beta;
}

/* tables/forcetable.cpp:304-318 spline3_table_scale */
static double spline3_table_scale(double third_deriv_max, double x_scale, double func_tol)
{
    const double deriv_tol = 1.19209290e-07F; /* GMX_FLOAT_EPS */
    double sc_deriv = sqrt(third_deriv_max / (6 * 4 * deriv_tol * x_scale)) * x_scale;
    if (func_tol < (double)1.19209290e-07F)
    {
        func_tol = (double)1.19209290e-07F;
    }
    double sc_func = cbrt(third_deriv_max / (6 * 12 * sqrt(3.0) * func_tol)) * x_scale;
    return sc_deriv > sc_func ? sc_deriv : sc_func;
}

static double v_q_ewald_lr(double beta, double r)
{
    /* forcetable.cpp:114-124 */
    if (r == 0)
    {
        return beta * 2 / sqrt(c_pi);
    }
    return erf(beta * r) / r;
}

/* tables/forcetable.cpp:144-298 generateEwaldCorrectionTables (F and V parts) */
static void make_ewald_table(int numPoints, double scale, float beta, float* table_f, float* table_v)
{
    const double dx      = 1 / scale;
    const float  tab_max = 3.40282346E+38F * 0.0001f;
    int          bOutOfRange = 0, i_inrange = numPoints;
    double       v_inrange = 0, dc = 0, dc_new, v_r0, v_r1, vi, a0, a1, a2dx, x_r0;
    for (int i = numPoints - 1; i >= 0; i--)
    {
        x_r0 = i * dx;
        v_r0 = v_q_ewald_lr(beta, x_r0);
        if (!bOutOfRange)
        {
            i_inrange = i;
            v_inrange = v_r0;
            vi        = v_r0;
        }
        else
        {
            vi = v_inrange - dc * (i - i_inrange) * dx;
        }
        table_v[i] = (float)vi;
        if (i == 0)
        {
            continue;
        }
        v_r1 = v_q_ewald_lr(beta, (i - 1) * dx);
        if (v_r1 != v_r1 || v_r1 < -tab_max || v_r1 > tab_max)
        {
            bOutOfRange = 1;
        }
        if (!bOutOfRange)
        {
            a2dx = (v_r0 + v_r1 - 2 * v_q_ewald_lr(beta, x_r0 - 0.5 * dx)) / (0.25 * dx);
            dc   = (v_r0 - v_r1) / dx + 0.5 * a2dx;
        }
        if (i == numPoints - 1)
        {
            table_f[i] = (float)(-dc);
        }
        else
        {
            table_f[i] += (float)(-0.5 * dc);
        }
        if (!bOutOfRange)
        {
            a0     = v_r0;
            a1     = dc;
            a2dx   = (a1 * dx + v_r1 - a0) * 2 / dx;
            dc_new = a1 - a2dx;
            if (dc_new != dc_new || dc_new < -tab_max || dc_new > tab_max)
            {
                bOutOfRange = 1;
            }
            else
            {
                dc = dc_new;
            }
        }
        table_f[i - 1] = (float)(-0.5 * dc);
    }
    table_f[0] *= 2;
}

static void* xmalloc(size_t n)
{
    void* p = malloc(n ? n : 1);
    if (!p)
    {
        abort();
    }
    return p;
}

orc_ctx* orc_create(int n, const float* x, const float* box, const float* q, const int* type,
                    int ntypes, const float* nbfp, const int* excl_index, const int* excl_list,
                    int coulomb, float rc, float rlist_outer, float rlist_inner,
                    float ewald_rtol, float epsilon_rf, int use_ewald_shift)
{
    orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
    c->n       = n;
    for (int d = 0; d < 3; d++)
    {
        c->box[d] = box[d];
    }
    c->x    = (float*)xmalloc(sizeof(float) * 3 * (size_t)n);
    c->image = (int*)calloc(3 * (size_t)n, sizeof(int));
    c->q    = (float*)xmalloc(sizeof(float) * (size_t)n);
    c->type = (int*)xmalloc(sizeof(int) * (size_t)n);
    memcpy(c->q, q, sizeof(float) * (size_t)n);
    memcpy(c->type, type, sizeof(int) * (size_t)n);
    orc_set_coordinates(c, x);

    /* atomdata.cpp:440-620: one extra, all-zero type for the fillers */
    c->ntypes   = ntypes;
    c->numTypes = ntypes + 1;
    c->nbfp     = (float*)calloc((size_t)c->numTypes * c->numTypes * 2, sizeof(float));
    for (int i = 0; i < ntypes; i++)
    {
        for (int j = 0; j < ntypes; j++)
        {
            c->nbfp[(i * c->numTypes + j) * 2]     = nbfp[(i * ntypes + j) * 2];
            c->nbfp[(i * c->numTypes + j) * 2 + 1] = nbfp[(i * ntypes + j) * 2 + 1];
        }
    }
    c->excl_index = (int*)xmalloc(sizeof(int) * (size_t)(n + 1));
    memcpy(c->excl_index, excl_index, sizeof(int) * (size_t)(n + 1));
    c->excl_list = (int*)xmalloc(sizeof(int) * (size_t)(excl_index[n] + 1));
    memcpy(c->excl_list, excl_list, sizeof(int) * (size_t)excl_index[n]);

    /* api/nblib/gmxsetup.cpp:226-284 setupInteractionConst */
    c->coulomb     = coulomb;
    c->rc          = rc;
    c->rlist_outer = rlist_outer;
    c->rlist_inner = rlist_inner;
    c->epsfac      = (float)orc_one_4pi_eps0(); /* epsilon_r = 1 */
    /* math/functions.h:372-388: power6 = square(power3), power12 = square(power6) */
    {
        const float p3  = rc * rc * rc;
        const float p6  = p3 * p3;
        const float p12 = p6 * p6;
        c->cpot_disp    = (float)(-1.0 / p6);
        c->cpot_rep     = (float)(-1.0 / p12);
    }
    /* mdlib/rf_util.cpp:54-66 calc_rffac with eps_r = 1 */
    float eps_rf = (coulomb == ORC_COULOMB_CUTOFF) ? 1.0f : epsilon_rf;
    if (eps_rf == 0)
    {
        c->k_rf = 1 / (2 * rc * rc * rc);
    }
    else
    {
        c->k_rf = (eps_rf - 1.0f) / (2 * eps_rf + 1.0f) / (rc * rc * rc);
    }
    c->c_rf = 1 / rc + c->k_rf * rc * rc;
    if (coulomb == ORC_COULOMB_EWALD)
    {
        c->beta = calc_ewaldcoeff_q(rc, ewald_rtol);
        /* nblib leaves sh_ewald at 0 (mdtypes/interaction_const.h:153) */
        c->sh_ewald = use_ewald_shift ? erfcf(c->beta * rc) / rc : 0.0f;
        /* forcetable.cpp:332-362 ewald_spline3_table_scale, forcerec.cpp:726-764 */
        double etol = 0.1 * erfcf(c->beta * rc);
        float  sc_q = (float)spline3_table_scale(1.0522, c->beta, etol);
        float  sc   = 0;
        if (sc_q > sc)
        {
            sc = sc_q;
        }
        c->tab_scale = sc;
        c->tab_n     = (int)(rc * sc) + 2;
        c->tabF      = (float*)calloc((size_t)c->tab_n, sizeof(float));
        c->tabV      = (float*)calloc((size_t)c->tab_n, sizeof(float));
        make_ewald_table(c->tab_n, (double)sc, c->beta, c->tabF, c->tabV);
    }
    /* pbcutil/pbc.cpp:1187-1202 calc_shifts for a rectangular box */
    for (int n_ = 0, m = -1; m <= 1; m++)
    {
        for (int l = -1; l <= 1; l++)
        {
            for (int k = -2; k <= 2; k++, n_++)
            {
                c->shiftvec[n_ * 3 + 0] = k * box[0];
                c->shiftvec[n_ * 3 + 1] = l * box[1];
                c->shiftvec[n_ * 3 + 2] = m * box[2];
            }
        }
    }
    return c;
}

/* The LJ modifier constants of init_interaction_const (mdlib/forcerec.cpp:853-872):
 * force_switch_constants (forcerec.cpp:787-801) for p = 6 and 12 and
 * potential_switch_constants (forcerec.cpp:803-816), in double, stored as float. */
void orc_set_vdw_modifier(orc_ctx* c, int mod, float rvdw_switch)
{
    const double rc = c->rc, rs = rvdw_switch, d = rc - rs;
    c->vdw_mod      = mod;
    c->rvdw_switch  = rvdw_switch;
    c->fsw_disp_c2 = c->fsw_disp_c3 = c->fsw_rep_c2 = c->fsw_rep_c3 = 0;
    c->psw_c3 = c->psw_c4 = c->psw_c5 = 0;
    if (mod == 0)
    {
        c->cpot_disp = (float)(-1.0 / pow(rc, 6.0));
        c->cpot_rep  = (float)(-1.0 / pow(rc, 12.0));
    }
    else if (mod == 1)
    {
        for (int k = 0; k < 2; k++)
        {
            const double p  = k == 0 ? 6.0 : 12.0;
            const double c2 = ((p + 1) * rs - (p + 4) * rc) / (pow(rc, p + 2) * d * d);
            const double c3 = -((p + 1) * rs - (p + 3) * rc) / (pow(rc, p + 2) * d * d * d);
            const double cp = -pow(rc, -p) + p * c2 / 3 * d * d * d + p * c3 / 4 * d * d * d * d;
            if (k == 0)
            {
                c->fsw_disp_c2 = (float)c2;
                c->fsw_disp_c3 = (float)c3;
                c->cpot_disp   = (float)cp;
            }
            else
            {
                c->fsw_rep_c2 = (float)c2;
                c->fsw_rep_c3 = (float)c3;
                c->cpot_rep   = (float)cp;
            }
        }
    }
    else
    {
        c->cpot_disp = c->cpot_rep = 0;
        if (mod == 2)
        {
            c->psw_c3 = (float)(-10 / (d * d * d));
            c->psw_c4 = (float)(15 / (d * d * d * d));
            c->psw_c5 = (float)(-6 / (d * d * d * d * d));
        }
    }
}

static void free_grid(orc_ctx* c)
{
    free(c->cxy_na);
    free(c->cxy_ind);
    free(c->nclusters);
    free(c->bbcz);
    free(c->bb);
    free(c->atom_indices);
    free(c->cells);
    free(c->xq);
    free(c->tgrid);
    free(c->fnb);
    c->cxy_na = c->cxy_ind = c->nclusters = c->atom_indices = c->cells = c->tgrid = NULL;
    c->bbcz = c->bb = c->xq = c->fnb = NULL;
}

void orc_destroy(orc_ctx* c)
{
    if (!c)
    {
        return;
    }
    free_grid(c);
    free(c->x);
    free(c->image);
    free(c->q);
    free(c->type);
    free(c->nbfp);
    free(c->excl_index);
    free(c->excl_list);
    free(c->tabF);
    free(c->tabV);
    free(c->sci);
    free(c->cj4);
    free(c->excl);
    free(c->imask_outer);
    free(c);
}

void orc_set_coordinates(orc_ctx* c, const float* x)
{
    /* pbcutil/pbc.cpp:1389-1450 put_atoms_in_box, rectangular branch; the
     * number of box lengths added is kept for orc_set_x */
    for (int i = 0; i < c->n; i++)
    {
        for (int d = 0; d < 3; d++)
        {
            float v = x[i * 3 + d];
            int   k = 0;
            while (v < 0)
            {
                v += c->box[d];
                k++;
            }
            while (v >= c->box[d])
            {
                v -= c->box[d];
                k--;
            }
            c->x[i * 3 + d]     = v;
            c->image[i * 3 + d] = k;
        }
    }
}

/* ---------------------------------------------------------------- gridding */

/* grid.cpp:292-427 sort_atoms.  The pigeonhole insertion keeps every run of
 * occupied holes ordered on (coordinate, atom index), and the hole index is a
 * monotonic function of the coordinate, so its output is exactly the atoms
 * ordered on (coordinate, atom index), reversed when Backwards is set.  An
 * insertion sort on that key reproduces it. */
static void sort_atoms(int dim, int backwards, int* a, int n, const float* x)
{
    for (int i = 1; i < n; i++)
    {
        int   ai = a[i];
        float xi = x[ai * 3 + dim];
        int   k  = i - 1;
        while (k >= 0)
        {
            int   ak = a[k];
            float xk = x[ak * 3 + dim];
            int   after;
            if (!backwards)
            {
                after = (xi > xk) || (xi == xk && ai > ak);
            }
            else
            {
                after = (xi < xk) || (xi == xk && ai < ak);
            }
            if (after)
            {
                break;
            }
            a[k + 1] = ak;
            k--;
        }
        a[k + 1] = ai;
    }
}

/* grid.cpp:860-986 fillCell for the XYZQ format with xxxx bounding boxes */
static void fill_cell(orc_ctx* c, int atomStart, int numAtoms)
{
    for (int k = 0; k < numAtoms; k++)
    {
        c->cells[c->atom_indices[atomStart + k]] = atomStart + k;
    }
    /* atomdata.cpp:134-250 copy_rvec_to_nbat_real, nbatXYZQ */
    int i = 0;
    for (; i < numAtoms; i++)
    {
        const int a = c->atom_indices[atomStart + i];
        for (int d = 0; d < 3; d++)
        {
            c->xq[(atomStart + i) * 4 + d] = c->x[a * 3 + d];
        }
    }
    for (; i < CL; i++)
    {
        for (int d = 0; d < 3; d++)
        {
            c->xq[(atomStart + i) * 4 + d] = FAR_AWAY;
        }
    }
    /* grid.cpp:582-607 calc_bounding_box_xxxx: the first coordinate is used
     * even when the cluster only holds fillers */
    const float* xs  = c->xq + (size_t)atomStart * 4;
    float        lo[3], hi[3];
    for (int d = 0; d < 3; d++)
    {
        lo[d] = hi[d] = xs[d];
    }
    for (int j = 1; j < numAtoms; j++)
    {
        for (int d = 0; d < 3; d++)
        {
            float v = xs[j * 4 + d];
            lo[d]   = v < lo[d] ? v : lo[d];
            hi[d]   = v > hi[d] ? v : hi[d];
        }
    }
    float* bb = c->bb + (size_t)(atomStart / CL) * 6;
    for (int d = 0; d < 3; d++)
    {
        bb[d]     = lo[d];
        bb[3 + d] = hi[d];
    }
}

void orc_grid(orc_ctx* c)
{
    free_grid(c);
    const int n = c->n;
    /* api/nblib/gmxcalculator.cpp:85-103: lower corner 0, density N/det(box) */
    const float det     = c->box[0] * (c->box[1] * c->box[2]);
    const float density = (float)n / det;
    /* grid.cpp:103-262 setDimensions, GPU geometry */
    if (n > SC)
    {
        float tlen = cbrtf((float)CL / density);
        float tx   = tlen * 2;
        float ty   = tlen * 2;
        c->ncx     = (int)(c->box[0] / tx);
        c->ncy     = (int)(c->box[1] / ty);
        c->ncx     = c->ncx < 1 ? 1 : c->ncx;
        c->ncy     = c->ncy < 1 ? 1 : c->ncy;
    }
    else
    {
        c->ncx = c->ncy = 1;
    }
    c->cs[0]  = c->box[0] / c->ncx;
    c->cs[1]  = c->box[1] / c->ncy;
    c->ics[0] = 1 / c->cs[0];
    c->ics[1] = 1 / c->cs[1];
    c->ncol   = c->ncx * c->ncy;

    /* grid.cpp:1173-1268 calcColumnIndices (home zone) */
    int* col   = (int*)xmalloc(sizeof(int) * (size_t)(n + 1));
    c->cxy_na  = (int*)calloc((size_t)c->ncol + 1, sizeof(int));
    c->cxy_ind = (int*)calloc((size_t)c->ncol + 2, sizeof(int));
    for (int i = 0; i < n; i++)
    {
        int cx = (int)((c->x[i * 3 + 0] - 0.0f) * c->ics[0]);
        int cy = (int)((c->x[i * 3 + 1] - 0.0f) * c->ics[1]);
        cx     = cx < c->ncx - 1 ? cx : c->ncx - 1;
        cy     = cy < c->ncy - 1 ? cy : c->ncy - 1;
        col[i] = cx * c->ncy + cy;
        c->cxy_na[col[i]]++;
    }
    /* grid.cpp:1287-1330 setCellIndices: cells per column */
    c->cxy_ind[0] = 0;
    for (int i = 0; i < c->ncol; i++)
    {
        int ncz           = (c->cxy_na[i] + SC - 1) / SC;
        c->cxy_ind[i + 1] = c->cxy_ind[i] + ncz;
    }
    c->ncells            = c->cxy_ind[c->ncol];
    const int npad       = c->ncells * SC;
    c->nclusters         = (int*)calloc((size_t)c->ncells + 1, sizeof(int));
    c->bbcz              = (float*)calloc((size_t)c->ncells * 2 + 2, sizeof(float));
    c->bb                = (float*)calloc((size_t)c->ncells * NCL * 6 + 6, sizeof(float));
    c->atom_indices      = (int*)xmalloc(sizeof(int) * (size_t)(npad + 1));
    c->cells             = (int*)xmalloc(sizeof(int) * (size_t)(n + 1));
    c->xq                = (float*)calloc((size_t)npad * 4 + 4, sizeof(float));
    c->tgrid             = (int*)xmalloc(sizeof(int) * (size_t)(npad + 1));
    c->fnb               = (float*)calloc((size_t)npad * 3 + 3, sizeof(float));
    int* fill            = (int*)calloc((size_t)c->ncol + 1, sizeof(int));
    /* first, unsorted fill in atom order (grid.cpp:1378-1385) */
    for (int i = 0; i < n; i++)
    {
        int cxy                                          = col[i];
        c->atom_indices[c->cxy_ind[cxy] * SC + fill[cxy]++] = i;
    }
    free(fill);
    free(col);

    /* grid.cpp:1051-1164 sortColumnsGpuGeometry */
    for (int cxy = 0; cxy < c->ncol; cxy++)
    {
        const int gridX            = cxy / c->ncy;
        const int gridY            = cxy - gridX * c->ncy;
        const int numAtomsInColumn = c->cxy_na[cxy];
        const int numCellsInColumn = c->cxy_ind[cxy + 1] - c->cxy_ind[cxy];
        const int atomOffset       = c->cxy_ind[cxy] * SC;
        (void)gridX;
        (void)gridY;
        sort_atoms(2, 0, c->atom_indices + atomOffset, numAtomsInColumn, c->x);
        for (int sub_z = 0; sub_z < numCellsInColumn * 2; sub_z++)
        {
            const int atomOffsetZ = atomOffset + sub_z * 32;
            int       numAtomsZ   = numAtomsInColumn - (atomOffsetZ - atomOffset);
            numAtomsZ             = numAtomsZ < 32 ? numAtomsZ : 32;
            if (sub_z % 2 == 0)
            {
                const int cz   = sub_z / 2;
                const int cell = c->cxy_ind[cxy] + cz;
                int numAtoms   = numAtomsInColumn - (atomOffsetZ - atomOffset);
                numAtoms       = numAtoms < SC ? numAtoms : SC;
                int ncl        = (numAtoms + CL - 1) / CL;
                c->nclusters[cell] = ncl < NCL ? ncl : NCL;
                c->bbcz[cell * 2 + 0] = c->x[c->atom_indices[atomOffsetZ] * 3 + 2];
                c->bbcz[cell * 2 + 1] = c->x[c->atom_indices[atomOffsetZ + numAtoms - 1] * 3 + 2];
            }
            if (numAtomsZ > 1)
            {
                sort_atoms(1, (sub_z & 1) != 0, c->atom_indices + atomOffsetZ, numAtomsZ, c->x);
            }
            for (int sub_y = 0; sub_y < 2; sub_y++)
            {
                const int atomOffsetY = atomOffsetZ + sub_y * 16;
                int       numAtomsY   = numAtomsInColumn - (atomOffsetY - atomOffset);
                numAtomsY             = numAtomsY < 16 ? numAtomsY : 16;
                /* grid.cpp:1133: the direction flag reduces to sub_y & 1 for
                 * both even (cz >= 0) and odd (cz == -1) sub_z */
                if (numAtomsY > 1)
                {
                    sort_atoms(0, (sub_y & 1) != 0, c->atom_indices + atomOffsetY, numAtomsY, c->x);
                }
                for (int sub_x = 0; sub_x < 2; sub_x++)
                {
                    const int atomOffsetX = atomOffsetY + sub_x * CL;
                    int       numAtomsX   = numAtomsInColumn - (atomOffsetX - atomOffset);
                    numAtomsX             = numAtomsX < CL ? numAtomsX : CL;
                    fill_cell(c, atomOffsetX, numAtomsX);
                }
            }
        }
        for (int ind = numAtomsInColumn; ind < numCellsInColumn * SC; ind++)
        {
            c->atom_indices[atomOffset + ind] = -1;
        }
    }
    c->nclusters_tot = 0;
    for (int i = 0; i < c->ncells; i++)
    {
        c->nclusters_tot += c->nclusters[i];
    }
    /* atomdata.cpp:723-836: types (fillers get the dummy type) and charges */
    for (int k = 0; k < npad; k++)
    {
        const int a       = c->atom_indices[k];
        c->tgrid[k]       = a >= 0 ? c->type[a] : c->numTypes - 1;
        c->xq[k * 4 + 3] = a >= 0 ? c->q[a] : 0.0f;
    }
}

void orc_set_x(orc_ctx* c, const float* x)
{
    /* atomdata.cpp:1018-1073 nbnxn_atomdata_copy_x_to_nbat_x: real atoms get
     * the coordinates as given plus the box shift of their last wrap (so a
     * continuous trajectory stays consistent with the grid), fillers keep
     * FAR_AWAY */
    const int npad = c->ncells * SC;
    for (int k = 0; k < npad; k++)
    {
        const int a = c->atom_indices[k];
        if (a >= 0)
        {
            for (int d = 0; d < 3; d++)
            {
                const int s      = c->image[a * 3 + d];
                c->xq[k * 4 + d] = (s == 0) ? x[a * 3 + d] : x[a * 3 + d] + (float)s * c->box[d];
            }
        }
    }
}

/* ------------------------------------------------------------ pair search */

static void push_sci(orc_ctx* c, sci_t e)
{
    if (c->nsci == c->cap_sci)
    {
        c->cap_sci = c->cap_sci ? 2 * c->cap_sci : 1024;
        c->sci     = (sci_t*)realloc(c->sci, sizeof(sci_t) * (size_t)c->cap_sci);
    }
    c->sci[c->nsci++] = e;
}

static void push_cj4(orc_ctx* c)
{
    if (c->ncj4 == c->cap_cj4)
    {
        c->cap_cj4 = c->cap_cj4 ? 2 * c->cap_cj4 : 4096;
        c->cj4     = (cj4_t*)realloc(c->cj4, sizeof(cj4_t) * (size_t)c->cap_cj4);
    }
    memset(&c->cj4[c->ncj4], 0, sizeof(cj4_t));
    c->ncj4++;
}

static int push_excl(orc_ctx* c)
{
    if (c->nexcl == c->cap_excl)
    {
        c->cap_excl = c->cap_excl ? 2 * c->cap_excl : 1024;
        c->excl     = (excl_t*)realloc(c->excl, sizeof(excl_t) * (size_t)c->cap_excl);
    }
    for (int k = 0; k < EXCLW; k++)
    {
        c->excl[c->nexcl].pair[k] = 0xffffffffu;
    }
    return c->nexcl++;
}

/* pairlist.cpp:853-868 get_exclusion_mask */
static excl_t* get_exclusion_mask(orc_ctx* c, int cj4, int warp)
{
    if (c->cj4[cj4].imei[warp].excl_ind == 0)
    {
        int e                     = push_excl(c);
        c->cj4[cj4].imei[warp].excl_ind = e;
    }
    return &c->excl[c->cj4[cj4].imei[warp].excl_ind];
}

/* pairlist.cpp:880-904 setSelfAndNewtonExclusionsGpu */
static void set_self_and_newton_exclusions(orc_ctx* c, int cj4Index, int jOffsetInGroup, int iClusterInCell)
{
    const int numJatomsPerPart = CL / SPLIT;
    for (int part = 0; part < SPLIT; part++)
    {
        const int jOffset = part * numJatomsPerPart;
        excl_t*   excl    = get_exclusion_mask(c, cj4Index, part);
        for (int jIndexInPart = 0; jIndexInPart < numJatomsPerPart; jIndexInPart++)
        {
            for (int i = jOffset + jIndexInPart; i < CL; i++)
            {
                excl->pair[jIndexInPart * CL + i] &= ~(1U << (jOffsetInGroup * NCL + iClusterInCell));
            }
        }
    }
}

/* pairlist.cpp:351-372 clusterBoundingBoxDistance2 (same rounding as the
 * xxxx SIMD4 variant :407-450 without contraction) */
static float bb_dist2(const float* bi, const float* bj)
{
    float d2 = 0;
    for (int d = 0; d < 3; d++)
    {
        float dl  = bi[d] - bj[3 + d];
        float dh  = bj[d] - bi[3 + d];
        float dm  = dl > dh ? dl : dh;
        float dm0 = dm > 0.0f ? dm : 0.0f;
        d2 += dm0 * dm0;
    }
    return d2;
}

typedef struct
{
    float bb_ci[NCL * 6]; /* shifted i bounding boxes */
    float x_ci[SC * 3];   /* shifted i coordinates */
    int   cj_ind;         /* j-cluster count, pairlist.cpp work->cj_ind */
} search_work;

/* pairlist.cpp:479-606 clusterpair_in_range: any atom pair within rlist */
static int clusterpair_in_range(const orc_ctx* c, const search_work* w, int si, int csj, float rlist2)
{
    for (int i = 0; i < CL; i++)
    {
        const float* xi = w->x_ci + (si * CL + i) * 3;
        for (int j = 0; j < CL; j++)
        {
            const float* xj = c->xq + (size_t)(csj * CL + j) * 4;
            float        dx = xi[0] - xj[0];
            float        dy = xi[1] - xj[1];
            float        dz = xi[2] - xj[2];
            float        d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < rlist2)
            {
                return 1;
            }
        }
    }
    return 0;
}

/* pairlist.cpp:1090-1244 make_cluster_list_supersub */
static void make_cluster_list_supersub(orc_ctx* c, search_work* w, int sci, int scj,
                                       int excludeSubDiagonal, float rlist2, float rbb2)
{
    float d2l[NCL];
    for (int subc = 0; subc < c->nclusters[scj]; subc++)
    {
        const int cj4_ind   = w->cj_ind / JG;
        const int cj_offset = w->cj_ind - cj4_ind * JG;
        const int cj        = scj * NCL + subc;
        const int ci1       = (excludeSubDiagonal && sci == scj) ? subc + 1 : c->nclusters[sci];
        int       npair = 0, ci_last = -1;
        uint32_t  imask = 0;
        for (int ci = 0; ci < NCL && ci < ci1; ci++)
        {
            d2l[ci] = bb_dist2(w->bb_ci + ci * 6, c->bb + (size_t)cj * 6);
            if (d2l[ci] < rlist2)
            {
                imask |= (1U << (cj_offset * NCL + ci));
                ci_last = ci;
                npair++;
            }
        }
        if (npair == 1 && d2l[ci_last] >= rbb2 && !clusterpair_in_range(c, w, ci_last, cj, rlist2))
        {
            imask &= ~(1U << (cj_offset * NCL + ci_last));
            npair--;
        }
        if (npair > 0)
        {
            if (cj4_ind == c->ncj4)
            {
                push_cj4(c);
            }
            cj4_t* e          = &c->cj4[cj4_ind];
            e->cj[cj_offset] = cj;
            if (excludeSubDiagonal && sci == scj)
            {
                set_self_and_newton_exclusions(c, cj4_ind, cj_offset, subc);
                e = &c->cj4[cj4_ind];
            }
            for (int s = 0; s < SPLIT; s++)
            {
                e->imei[s].imask |= imask;
            }
            w->cj_ind++;
            c->sci[c->nsci - 1].cj4_end = (w->cj_ind + JG - 1) / JG;
        }
    }
}

/* pairlist.cpp:286-309 get_cell_range (lower corner 0, no atom-group radius) */
static void get_cell_range(float b0, float b1, int numCells, float cellSize, float invCellSize,
                           float d2, float rlist, int* cf, int* cl)
{
    const float listRangeBBToCell2 = rlist * rlist;
    const float distanceInCells    = (b0 - 0.0f) * invCellSize;
    *cf                            = (int)distanceInCells;
    *cf                            = *cf > 0 ? *cf : 0;
    while (*cf > 0)
    {
        float t = (b0 - 0.0f) - (*cf - 1 + 1) * cellSize;
        if (!(d2 + t * t < listRangeBBToCell2))
        {
            break;
        }
        (*cf)--;
    }
    *cl = (int)((b1 - 0.0f) * invCellSize);
    *cl = *cl < numCells - 1 ? *cl : numCells - 1;
    while (*cl < numCells - 1)
    {
        float t = (*cl + 1) * cellSize - (b1 - 0.0f);
        if (!(d2 + t * t < listRangeBBToCell2))
        {
            break;
        }
        (*cl)++;
    }
}

/* pairlist.cpp:1874-1972 setExclusionsForIEntry, GPU list */
static void set_exclusions_for_ientry(orc_ctx* c, const search_work* w, int diagRemoved, const sci_t* e)
{
    if (e->cj4_end - e->cj4_start == 0)
    {
        return;
    }
    const int cjIndexStart = e->cj4_start * JG;
    const int cjIndexEnd   = w->cj_ind;
    const int cjFirst      = c->cj4[cjIndexStart / JG].cj[cjIndexStart % JG];
    const int cjLast       = c->cj4[(cjIndexEnd - 1) / JG].cj[(cjIndexEnd - 1) % JG];
    const int iSuperCluster = e->sci;
    for (int i = 0; i < SC; i++)
    {
        const int iIndex = iSuperCluster * SC + i;
        const int iAtom  = c->atom_indices[iIndex];
        if (iAtom < 0)
        {
            continue;
        }
        const int iCluster = i / CL;
        for (int k = c->excl_index[iAtom]; k < c->excl_index[iAtom + 1]; k++)
        {
            const int jAtom = c->excl_list[k];
            if (jAtom == iAtom)
            {
                continue;
            }
            const int jIndex = c->cells[jAtom];
            if (diagRemoved && jIndex <= iSuperCluster * SC + i)
            {
                continue;
            }
            const int jCluster = jIndex / CL;
            if (jCluster < cjFirst || jCluster > cjLast)
            {
                continue;
            }
            /* the j-list of one entry is sorted on cluster index */
            int index = -1;
            for (int idx = cjIndexStart; idx < cjIndexEnd; idx++)
            {
                if (c->cj4[idx / JG].cj[idx % JG] == jCluster)
                {
                    index = idx;
                    break;
                }
            }
            if (index < 0)
            {
                continue;
            }
            const uint32_t pairMask = 1U << ((index % JG) * NCL + iCluster);
            if (c->cj4[index / JG].imei[0].imask & pairMask)
            {
                const int innerI = i & (CL - 1);
                const int innerJ = jIndex & (CL - 1);
                const int jHalf  = innerJ / (CL / SPLIT);
                excl_t*   m      = get_exclusion_mask(c, index / JG, jHalf);
                m->pair[(innerJ & (CL / SPLIT - 1)) * CL + innerI] &= ~pairMask;
            }
        }
    }
}

void orc_search(orc_ctx* c)
{
    c->nsci  = 0;
    c->ncj4  = 0;
    c->nexcl = 0;
    push_excl(c); /* entry 0: no exclusions */
    search_work w;
    memset(&w, 0, sizeof(w));

    const float rlist  = c->rlist_outer;
    const float rlist2 = rlist * rlist;
    /* pairlist.cpp:2841-2878 boundingbox_only_distance2 (double intermediates) */
    {
        float  bbx  = (float)(0.5 * (c->cs[0] + c->cs[0]));
        float  bby  = (float)(0.5 * (c->cs[1] + c->cs[1]));
        bbx /= 2;
        bby /= 2;
        double r    = (double)rlist - 0.5 * (double)sqrtf(bbx * bbx + bby * bby);
        float  rbb2 = (float)(r > 0.0 ? r : 0.0);
        c->rbb2     = rbb2 * rbb2;
    }
    const float rbb2 = c->rbb2;
    const float listRangeBBToJCell2 = rlist * rlist;
    const float* box = c->box;
    /* pairlist.cpp:3213-3235 shift range (rectangular, PBC xyz, no DD) */
    int shp[3] = { 1, 1, 1 };
    if (box[0] < rlist)
    {
        shp[0] = 2;
    }
    w.cj_ind = 0;
    int ci_x = 0, ci_y = 0;
    for (int ci = 0; ci < c->ncells; ci++)
    {
        /* pairlist.cpp:2808-2836 next_ci */
        while (ci >= c->cxy_ind[ci_x * c->ncy + ci_y + 1])
        {
            ci_y++;
            if (ci_y == c->ncy)
            {
                ci_x++;
                ci_y = 0;
            }
        }
        const float d2cx  = 0;
        const int   ci_xy = ci_x * c->ncy + ci_y;
        for (int tz = -shp[2]; tz <= shp[2]; tz++)
        {
            const float shz = (float)tz * box[2];
            const float bz0 = c->bbcz[ci * 2 + 0] + shz;
            const float bz1 = c->bbcz[ci * 2 + 1] + shz;
            float       d2z;
            if (tz == 0)
            {
                d2z = 0;
            }
            else if (tz < 0)
            {
                d2z = bz1 * bz1;
            }
            else
            {
                float t = bz0 - box[2];
                d2z     = t * t;
            }
            const float d2z_cx = d2z + d2cx;
            if (d2z_cx >= rlist2)
            {
                continue;
            }
            float bz1_frac = bz1 / (float)(c->cxy_ind[ci_xy + 1] - c->cxy_ind[ci_xy]);
            if (bz1_frac < 0)
            {
                bz1_frac = 0;
            }
            for (int ty = -shp[1]; ty <= shp[1]; ty++)
            {
                const float shy = (float)ty * box[1] + (float)tz * 0.0f;
                const float by0 = 0.0f + (float)ci_y * c->cs[1] + shy;
                const float by1 = 0.0f + ((float)ci_y + 1) * c->cs[1] + shy;
                int         cyf, cyl;
                get_cell_range(by0, by1, c->ncy, c->cs[1], c->ics[1], d2z_cx, rlist, &cyf, &cyl);
                if (cyf > cyl)
                {
                    continue;
                }
                float d2z_cy = d2z;
                if (by1 < 0.0f)
                {
                    float t = 0.0f - by1;
                    d2z_cy += t * t;
                }
                else if (by0 > box[1])
                {
                    float t = by0 - box[1];
                    d2z_cy += t * t;
                }
                for (int tx = -shp[0]; tx <= shp[0]; tx++)
                {
                    const int shift              = xyz2is(tx, ty, tz);
                    const int excludeSubDiagonal = (shift == CENTRAL);
                    if (shift > CENTRAL)
                    {
                        continue; /* c_pbcShiftBackward */
                    }
                    const float shx = (float)tx * box[0] + (float)ty * 0.0f + (float)tz * 0.0f;
                    const float bx0 = 0.0f + (float)ci_x * c->cs[0] + shx;
                    const float bx1 = 0.0f + ((float)ci_x + 1) * c->cs[0] + shx;
                    int         cxf, cxl;
                    get_cell_range(bx0, bx1, c->ncx, c->cs[0], c->ics[0], d2z_cy, rlist, &cxf, &cxl);
                    if (cxf > cxl)
                    {
                        continue;
                    }
                    /* addNewIEntry (pairlist.cpp:1988-1998) */
                    sci_t e = { ci, shift, c->ncj4, c->ncj4 };
                    push_sci(c, e);
                    w.cj_ind = c->ncj4 * JG; /* sync_work */
                    if (excludeSubDiagonal && cxf < ci_x)
                    {
                        cxf = ci_x;
                    }
                    /* set_icell_bb / icell_set_x (pairlist.cpp:2260-2403) */
                    for (int k = 0; k < NCL; k++)
                    {
                        const float* b = c->bb + (size_t)(ci * NCL + k) * 6;
                        w.bb_ci[k * 6 + 0] = b[0] + shx;
                        w.bb_ci[k * 6 + 1] = b[1] + shy;
                        w.bb_ci[k * 6 + 2] = b[2] + shz;
                        w.bb_ci[k * 6 + 3] = b[3] + shx;
                        w.bb_ci[k * 6 + 4] = b[4] + shy;
                        w.bb_ci[k * 6 + 5] = b[5] + shz;
                    }
                    for (int k = 0; k < SC; k++)
                    {
                        const float* xa   = c->xq + (size_t)(ci * SC + k) * 4;
                        w.x_ci[k * 3 + 0] = xa[0] + shx;
                        w.x_ci[k * 3 + 1] = xa[1] + shy;
                        w.x_ci[k * 3 + 2] = xa[2] + shz;
                    }
                    for (int cx = cxf; cx <= cxl; cx++)
                    {
                        const float cx_real = (float)cx;
                        float       d2zx    = d2z;
                        if (0.0f + cx_real * c->cs[0] > bx1)
                        {
                            float t = 0.0f + cx_real * c->cs[0] - bx1;
                            d2zx += t * t;
                        }
                        else if (0.0f + (cx_real + 1) * c->cs[0] < bx0)
                        {
                            float t = 0.0f + (cx_real + 1) * c->cs[0] - bx0;
                            d2zx += t * t;
                        }
                        const int cyf_x = (cx == 0 && shift == CENTRAL && cyf < ci_y) ? ci_y : cyf;
                        for (int cy = cyf_x; cy <= cyl; cy++)
                        {
                            const int   columnStart = c->cxy_ind[cx * c->ncy + cy];
                            const int   columnEnd   = c->cxy_ind[cx * c->ncy + cy + 1];
                            const float cy_real     = (float)cy;
                            float       d2zxy       = d2zx;
                            if (0.0f + cy_real * c->cs[1] > by1)
                            {
                                float t = 0.0f + cy_real * c->cs[1] - by1;
                                d2zxy += t * t;
                            }
                            else if (0.0f + (cy_real + 1) * c->cs[1] < by0)
                            {
                                float t = 0.0f + (cy_real + 1) * c->cs[1] - by0;
                                d2zxy += t * t;
                            }
                            if (!(columnStart < columnEnd && d2zxy < listRangeBBToJCell2))
                            {
                                continue;
                            }
                            int midCell = columnStart
                                          + (int)(bz1_frac * (float)(columnEnd - columnStart));
                            if (midCell >= columnEnd)
                            {
                                midCell = columnEnd - 1;
                            }
                            const float d2xy = d2zxy - d2z;
                            int         down = midCell;
                            while (down >= columnStart)
                            {
                                float u = c->bbcz[down * 2 + 1];
                                float t = u - bz0;
                                if (!(u >= bz0 || d2xy + t * t < rlist2))
                                {
                                    break;
                                }
                                down--;
                            }
                            int firstCell = down + 1;
                            int up        = midCell + 1;
                            while (up < columnEnd)
                            {
                                float l = c->bbcz[up * 2 + 0];
                                float t = l - bz1;
                                if (!(l <= bz1 || d2xy + t * t < rlist2))
                                {
                                    break;
                                }
                                up++;
                            }
                            int lastCell = up - 1;
                            if (shift == CENTRAL && firstCell < ci)
                            {
                                firstCell = ci;
                            }
                            for (int scj = firstCell; scj <= lastCell; scj++)
                            {
                                make_cluster_list_supersub(c, &w, ci, scj, excludeSubDiagonal,
                                                           rlist2, rbb2);
                            }
                        }
                    }
                    set_exclusions_for_ientry(c, &w, excludeSubDiagonal, &c->sci[c->nsci - 1]);
                    /* closeIEntry (pairlist.cpp:2167-2193) */
                    sci_t* last = &c->sci[c->nsci - 1];
                    if (last->cj4_end - last->cj4_start > 0)
                    {
                        w.cj_ind = ((w.cj_ind + JG - 1) / JG) * JG;
                    }
                    else
                    {
                        c->nsci--;
                    }
                }
            }
        }
    }
    free(c->imask_outer);
    c->imask_outer = (uint32_t*)calloc((size_t)c->ncj4 * SPLIT + 2, sizeof(uint32_t));
    for (int j = 0; j < c->ncj4; j++)
    {
        for (int s = 0; s < SPLIT; s++)
        {
            c->imask_outer[j * SPLIT + s] = c->cj4[j].imei[s].imask;
        }
    }
}

/* ------------------------------------------------------------ balancing */

static int popcount32(uint32_t v)
{
    int n = 0;
    while (v)
    {
        v &= v - 1;
        n++;
    }
    return n;
}

/* Target cluster pairs per entry: get_nsubpair_target (pairlist.cpp:2485-2585), with the
 * exact number of cluster pairs of the list (bits of imei[0].imask) in place of the
 * geometric estimate; 0 = no splitting.  Integer rounding of nsp / min_ci_balanced. */
static int balance_target(const orc_ctx* c, int min_ci_balanced)
{
    if (min_ci_balanced <= 0 || c->ncells >= min_ci_balanced || c->ncells == 0)
    {
        return 0;
    }
    long long nsp = 0;
    for (int j = 0; j < c->ncj4; j++)
    {
        nsp += popcount32(c->cj4[j].imei[0].imask);
    }
    const long long t = (2 * nsp + min_ci_balanced) / (2 * (long long)min_ci_balanced);
    return t > 36 ? (int)t : 36;
}

/* split_sci_entry (pairlist.cpp:2077-2165) without progressive balancing: pieces of close to
 * nsp_max cluster pairs, the last two evened out.  Appends the pieces of e to out. */
static int split_entry(const orc_ctx* c, sci_t e, int nsp_max, sci_t* out)
{
    const int j4len = e.cj4_end - e.cj4_start;
    int       n     = 0;
    out[n++]        = e;
    if (!(nsp_max > 0 && j4len > 1 && j4len * NCL * JG > nsp_max))
    {
        return n;
    }
    int nsp = 0, nsp_sci = 0, nsp_cj4_e = 0, nsp_cj4 = 0;
    for (int j = e.cj4_start; j < e.cj4_end; j++)
    {
        const int nsp_cj4_p = nsp_cj4;
        nsp_cj4             = popcount32(c->cj4[j].imei[0].imask);
        if (nsp > 0 && nsp_max - nsp < nsp + nsp_cj4 - nsp_max)
        {
            out[n - 1].cj4_end = j;
            sci_t next         = e;
            next.cj4_start     = j;
            out[n++]           = next;
            nsp_sci            = nsp;
            nsp_cj4_e          = nsp_cj4_p;
            nsp                = 0;
        }
        nsp += nsp_cj4;
    }
    out[n - 1].cj4_end = e.cj4_end;
    if (n >= 2 && nsp_sci - nsp_cj4_e >= nsp + nsp_cj4_e)
    {
        out[n - 2].cj4_end--;
        out[n - 1].cj4_start--;
    }
    return n;
}

/* sort_sci (pairlist.cpp:3827-3873): stable counting sort on the number of cj4 groups,
 * large first, sizes above twice the average (capped at 255) sharing one class. */
static void sort_entries(orc_ctx* c)
{
    if (c->ncj4 <= c->nsci)
    {
        return;
    }
    int m = (int)((2LL * c->ncj4) / c->nsci);
    m     = m > 255 ? 255 : m;
    int*   count  = (int*)calloc((size_t)m + 2, sizeof(int));
    sci_t* sorted = (sci_t*)xmalloc(sizeof(sci_t) * (size_t)c->nsci);
    for (int e = 0; e < c->nsci; e++)
    {
        const int len = c->sci[e].cj4_end - c->sci[e].cj4_start;
        count[len < m ? len : m]++;
    }
    /* offsets: class m first */
    int off = 0;
    for (int i = m; i >= 0; i--)
    {
        const int k = count[i];
        count[i]    = off;
        off += k;
    }
    for (int e = 0; e < c->nsci; e++)
    {
        const int len      = c->sci[e].cj4_end - c->sci[e].cj4_start;
        sorted[count[len < m ? len : m]++] = c->sci[e];
    }
    memcpy(c->sci, sorted, sizeof(sci_t) * (size_t)c->nsci);
    free(sorted);
    free(count);
}

int orc_balance(orc_ctx* c, int min_ci_balanced)
{
    const int nsp_max = balance_target(c, min_ci_balanced);
    if (nsp_max > 0)
    {
        sci_t* out = (sci_t*)xmalloc(sizeof(sci_t) * ((size_t)c->ncj4 + (size_t)c->nsci + 1));
        int    n   = 0;
        for (int e = 0; e < c->nsci; e++)
        {
            n += split_entry(c, c->sci[e], nsp_max, out + n);
        }
        free(c->sci);
        c->sci     = out;
        c->nsci    = n;
        c->cap_sci = c->ncj4 + c->nsci + 1;
    }
    sort_entries(c);
    return nsp_max;
}

/* ------------------------------------------------------------------ prune */

/* r^2 of the prune kernel.  The reference's prune-only kernel computes norm2(rv)
 * (nbnxm_cuda_kernel_pruneonly.cuh:245) in a unit built with nvcc's default
 * multiply-add contraction; the restatement fixes one contraction order,
 * fma(dz, dz, fma(dy, dy, dx * dx)), which the GPU prune uses explicitly. */
static float pair_r2(const float* xi, const float* xj)
{
    float dx = xi[0] - xj[0];
    float dy = xi[1] - xj[1];
    float dz = xi[2] - xj[2];
    return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

/* cuda/nbnxm_cuda_kernel_pruneonly.cuh:104-279, one "warp" = (8 i-atoms) x
 * (4 j-atoms of half w) */
static void prune_entry(orc_ctx* c, int e, int fresh)
{
    const sci_t* s        = &c->sci[e];
    const float  outer2   = c->rlist_outer * c->rlist_outer;
    const float  inner2   = c->rlist_inner * c->rlist_inner;
    const float* sv       = c->shiftvec + s->shift * 3;
    float        xib[SC * 3];
    for (int k = 0; k < SC; k++)
    {
        const float* xa = c->xq + (size_t)(s->sci * SC + k) * 4;
        xib[k * 3 + 0]  = xa[0] + sv[0];
        xib[k * 3 + 1]  = xa[1] + sv[1];
        xib[k * 3 + 2]  = xa[2] + sv[2];
    }
    for (int j4 = s->cj4_start; j4 < s->cj4_end; j4++)
    {
        for (int widx = 0; widx < SPLIT; widx++)
        {
            uint32_t imaskFull, imaskCheck, imaskNew;
            if (fresh)
            {
                imaskFull  = c->cj4[j4].imei[widx].imask;
                imaskCheck = imaskFull;
                imaskNew   = 0;
            }
            else
            {
                imaskFull  = c->imask_outer[j4 * SPLIT + widx];
                imaskNew   = c->cj4[j4].imei[widx].imask;
                imaskCheck = imaskNew ^ imaskFull;
            }
            if (!imaskCheck)
            {
                continue;
            }
            for (int jm = 0; jm < JG; jm++)
            {
                const int cj = c->cj4[j4].cj[jm];
                for (int i = 0; i < NCL; i++)
                {
                    const uint32_t bit = 1U << (jm * NCL + i);
                    if (!(imaskCheck & bit))
                    {
                        continue;
                    }
                    int anyOuter = 0, anyInner = 0;
                    for (int jj = 0; jj < CL / SPLIT; jj++)
                    {
                        const float* xj = c->xq + (size_t)(cj * CL + widx * (CL / SPLIT) + jj) * 4;
                        for (int ii = 0; ii < CL; ii++)
                        {
                            float r2 = pair_r2(xib + (i * CL + ii) * 3, xj);
                            anyOuter |= (r2 < outer2);
                            anyInner |= (r2 < inner2);
                        }
                    }
                    if (fresh && !anyOuter)
                    {
                        imaskFull &= ~bit;
                    }
                    if (anyInner)
                    {
                        imaskNew |= bit;
                    }
                }
            }
            if (fresh)
            {
                c->imask_outer[j4 * SPLIT + widx] = imaskFull;
            }
            c->cj4[j4].imei[widx].imask = imaskNew;
        }
    }
}

void orc_prune(orc_ctx* c, int fresh, int part, int nparts)
{
    if (fresh)
    {
        for (int e = 0; e < c->nsci; e++)
        {
            prune_entry(c, e, 1);
        }
        return;
    }
    for (int e = part; e < c->nsci; e += nparts)
    {
        prune_entry(c, e, 0);
    }
}

/* ------------------------------------------------------------ force kernel */

static void force_range(orc_ctx* c, int e_begin, int e_end, int computeEnergy);

/* kernels_reference/kernel_gpu_ref.cpp:57-379 nbnxn_kernel_gpu_ref */
void orc_force(orc_ctx* c, int computeEnergy)
{
    force_range(c, 0, c->nsci, computeEnergy);
}

/* The same kernel over list entries [e0, e1) only (a bounded sample for timing). */
void orc_force_entries(orc_ctx* c, int e0, int e1, int computeEnergy)
{
    e0 = e0 < 0 ? 0 : e0;
    e1 = e1 > c->nsci ? c->nsci : e1;
    force_range(c, e0, e1, computeEnergy);
}

/* Kernel body over entries [e_begin, e_end) into the given force / shift-force buffers
 * (cleared here) and energies; the single-threaded entry points pass the context's own. */
static void force_range_into(const orc_ctx* c, int e_begin, int e_end, int computeEnergy, float* fnb, double* fsh,
                             double* vc_out, double* vlj_out)
{
    const int    npad   = c->ncells * SC;
    const int    bEwald = (c->coulomb == ORC_COULOMB_EWALD);
    const float  rcut2  = c->rc * c->rc;
    const float  rvdw2  = c->rc * c->rc;
    const int    ntype  = c->numTypes;
    const float  facel  = c->epsfac;
    const double epsfac_d = orc_one_4pi_eps0();
    const float* x      = c->xq;
    const int*   type   = c->tgrid;
    memset(fnb, 0, sizeof(float) * (size_t)npad * 3);
    memset(fsh, 0, sizeof(double) * NSHIFT * 3);
    double Vc = 0, Vvdw = 0;
    for (int e = e_begin; e < e_end; e++)
    {
        const sci_t* nbln = &c->sci[e];
        const int    ish3 = 3 * nbln->shift;
        const float  shX = c->shiftvec[ish3], shY = c->shiftvec[ish3 + 1], shZ = c->shiftvec[ish3 + 2];
        const int    sci  = nbln->sci;
        double       vctot = 0, Vvdwtot = 0;
        if (nbln->shift == CENTRAL && c->cj4[nbln->cj4_start].cj[0] == sci * NCL)
        {
            /* self interaction energy term, kernel_gpu_ref.cpp:154-178 */
            double qsum = 0;
            for (int im = 0; im < NCL; im++)
            {
                for (int ic = 0; ic < CL; ic++)
                {
                    const int   ia = (sci * NCL + im) * CL + ic;
                    const double iq = x[ia * 4 + 3];
                    qsum += iq * iq;
                }
            }
            if (!bEwald)
            {
                vctot += qsum * (-epsfac_d * 0.5 * (double)c->c_rf);
            }
            else
            {
                vctot += qsum * (-epsfac_d * (double)c->beta * c_1_sqrtpi);
            }
        }
        for (int cj4_ind = nbln->cj4_start; cj4_ind < nbln->cj4_end; cj4_ind++)
        {
            const cj4_t*  cj4 = &c->cj4[cj4_ind];
            const excl_t* excl[SPLIT] = { &c->excl[cj4->imei[0].excl_ind], &c->excl[cj4->imei[1].excl_ind] };
            for (int jm = 0; jm < JG; jm++)
            {
                const int cj = cj4->cj[jm];
                for (int im = 0; im < NCL; im++)
                {
                    const int bitpos = jm * NCL + im;
                    if (!(((cj4->imei[0].imask | cj4->imei[1].imask) >> bitpos) & 1))
                    {
                        continue;
                    }
                    const int ci = sci * NCL + im;
                    for (int ic = 0; ic < CL; ic++)
                    {
                        const int   ia  = ci * CL + ic;
                        const float ix  = shX + x[ia * 4 + 0];
                        const float iy  = shY + x[ia * 4 + 1];
                        const float iz  = shZ + x[ia * 4 + 2];
                        const float iq  = facel * x[ia * 4 + 3];
                        const float iq_raw = x[ia * 4 + 3];
                        const int   nti = ntype * 2 * type[ia];
                        float       fix = 0, fiy = 0, fiz = 0;
                        for (int jc = 0; jc < CL; jc++)
                        {
                            const int ja = cj * CL + jc;
                            if (nbln->shift == CENTRAL && ci == cj && ja <= ia)
                            {
                                continue;
                            }
                            const int half = jc / (CL / SPLIT);
                            if (!((cj4->imei[half].imask >> bitpos) & 1))
                            {
                                continue; /* pruned half: all its pairs are beyond rlistInner */
                            }
                            const float int_bit =
                                    (float)((excl[half]->pair[(jc & (CL / SPLIT - 1)) * CL + ic] >> bitpos) & 1);
                            const float jx = x[ja * 4 + 0], jy = x[ja * 4 + 1], jz = x[ja * 4 + 2];
                            const float dx = ix - jx, dy = iy - jy, dz = iz - jz;
                            float       rsq = dx * dx + dy * dy + dz * dz;
                            if (rsq >= rcut2)
                            {
                                continue;
                            }
                            rsq               = rsq > c_minDist2 ? rsq : c_minDist2;
                            const float rinv   = 1.0f / sqrtf(rsq);
                            const float rinvsq = rinv * rinv;
                            const float qq     = iq * x[ja * 4 + 3];
                            float       fscal;
                            if (!bEwald)
                            {
                                const float krsq = c->k_rf * rsq;
                                fscal            = qq * (int_bit * rinv - 2 * krsq) * rinvsq;
                            }
                            else
                            {
                                const float r     = rsq * rinv;
                                const float rt    = r * c->tab_scale;
                                const int   n0    = (int)rt;
                                const float eps   = rt - (float)n0;
                                const float fexcl = (1 - eps) * c->tabF[n0] + eps * c->tabF[n0 + 1];
                                fscal             = qq * (int_bit * rinvsq - fexcl) * rinv;
                            }
                            if (rsq < rvdw2)
                            {
                                const int   tj        = nti + 2 * type[ja];
                                const float c6        = c->nbfp[tj];
                                const float c12       = c->nbfp[tj + 1];
                                const float rinvsix   = int_bit * rinvsq * rinvsq * rinvsq;
                                const float Vvdw_disp = c6 * rinvsix;
                                const float Vvdw_rep  = c12 * rinvsix * rinvsix;
                                float       frLJ      = Vvdw_rep - Vvdw_disp;
                                double      rswd      = 0.0;
                                if (c->vdw_mod == 1 || c->vdw_mod == 2)
                                {
                                    /* kernel_ref_inner.h:168-200: switching from rvdw_switch */
                                    const float r   = rsq * rinv;
                                    float       rsw = r - c->rvdw_switch;
                                    rsw             = rsw >= 0 ? rsw : 0;
                                    rswd            = (double)rsw;
                                    if (c->vdw_mod == 1)
                                    {
                                        frLJ += -c6 * (c->fsw_disp_c2 + c->fsw_disp_c3 * rsw) * rsw * rsw * r
                                                + c12 * (c->fsw_rep_c2 + c->fsw_rep_c3 * rsw) * rsw * rsw * r;
                                    }
                                    else
                                    {
                                        const float VLJ = (Vvdw_rep + c12 * c->cpot_rep) / 12
                                                          - (Vvdw_disp + c6 * c->cpot_disp) / 6;
                                        const float sw  = 1 + (c->psw_c3 + (c->psw_c4 + c->psw_c5 * rsw) * rsw)
                                                                     * rsw * rsw * rsw;
                                        const float dsw = (3 * c->psw_c3 + (4 * c->psw_c4 + 5 * c->psw_c5 * rsw) * rsw)
                                                          * rsw * rsw;
                                        frLJ            = frLJ * sw - r * VLJ * dsw;
                                    }
                                }
                                fscal += frLJ * rinvsq;
                                if (computeEnergy)
                                {
                                    /* the energy formulas of kernel_gpu_ref.cpp:286-291,327-336,
                                     * evaluated in double on the float pair geometry */
                                    const double r2d  = (double)dx * dx + (double)dy * dy + (double)dz * dz;
                                    const double r2c  = r2d > (double)c_minDist2 ? r2d : (double)c_minDist2;
                                    const double rd   = sqrt(r2c);
                                    const double ib   = (double)int_bit;
                                    const double qqd  = epsfac_d * (double)iq_raw * (double)x[ja * 4 + 3];
                                    double       vc;
                                    if (!bEwald)
                                    {
                                        vc = qqd * (ib / rd + (double)c->k_rf * r2c - (double)c->c_rf);
                                    }
                                    else
                                    {
                                        vc = qqd * ((ib - erf((double)c->beta * rd)) / rd - ib * (double)c->sh_ewald);
                                    }
                                    const double ir6 = ib / (r2c * r2c * r2c);
                                    vctot += vc;
                                    double vlj = ((double)c12 * ir6 * ir6 + ib * (double)c12 * (double)c->cpot_rep) / 12
                                                 - ((double)c6 * ir6 + ib * (double)c6 * (double)c->cpot_disp) / 6;
                                    if (c->vdw_mod == 1)
                                    {
                                        /* the switch terms' energy, masked like VLJ (kernel_ref_inner.h:179-192) */
                                        const double s3 = rswd * rswd * rswd;
                                        vlj += ib * (-(double)c6 * (-(double)c->fsw_disp_c2 / 3 - (double)c->fsw_disp_c3 / 4 * rswd) * s3
                                                     + (double)c12 * (-(double)c->fsw_rep_c2 / 3 - (double)c->fsw_rep_c3 / 4 * rswd) * s3);
                                    }
                                    else if (c->vdw_mod == 2)
                                    {
                                        vlj *= 1 + ((double)c->psw_c3 + ((double)c->psw_c4 + (double)c->psw_c5 * rswd) * rswd)
                                                           * rswd * rswd * rswd;
                                    }
                                    Vvdwtot += vlj;
                                }
                            }
                            const float tx = fscal * dx, ty = fscal * dy, tz = fscal * dz;
                            fix = fix + tx;
                            fiy = fiy + ty;
                            fiz = fiz + tz;
                            fnb[ja * 3 + 0] -= tx;
                            fnb[ja * 3 + 1] -= ty;
                            fnb[ja * 3 + 2] -= tz;
                        }
                        fnb[ia * 3 + 0] += fix;
                        fnb[ia * 3 + 1] += fiy;
                        fnb[ia * 3 + 2] += fiz;
                        fsh[ish3 + 0] += fix;
                        fsh[ish3 + 1] += fiy;
                        fsh[ish3 + 2] += fiz;
                    }
                }
            }
        }
        Vc += vctot;
        Vvdw += Vvdwtot;
    }
    *vc_out  = computeEnergy ? Vc : 0;
    *vlj_out = computeEnergy ? Vvdw : 0;
}

static void force_range(orc_ctx* c, int e_begin, int e_end, int computeEnergy)
{
    force_range_into(c, e_begin, e_end, computeEnergy, c->fnb, c->fshift, &c->vc, &c->vlj);
}

/* The same kernel split over nthreads POSIX threads (contiguous entry ranges, private
 * force buffers summed afterwards): the reference's OpenMP-parallel CPU kernel layout
 * (nbnxm/kerneldispatch.cpp, one output buffer per thread reduced in
 * atomdata.cpp:1181-1228).  Used as the multi-core CPU timing baseline. */
typedef struct
{
    const orc_ctx* c;
    int            e0, e1, energy;
    float*         fnb;
    double         fsh[NSHIFT * 3];
    double         vc, vlj;
} mt_task;

static void* mt_run(void* arg)
{
    mt_task* t = (mt_task*)arg;
    force_range_into(t->c, t->e0, t->e1, t->energy, t->fnb, t->fsh, &t->vc, &t->vlj);
    return NULL;
}

int orc_force_entries_mt(orc_ctx* c, int e0, int e1, int computeEnergy, int nthreads)
{
    e0 = e0 < 0 ? 0 : e0;
    e1 = e1 > c->nsci ? c->nsci : e1;
    if (nthreads < 1)
    {
        nthreads = 1;
    }
    const size_t npad3 = (size_t)c->ncells * SC * 3;
    mt_task*     tasks = (mt_task*)calloc((size_t)nthreads, sizeof(mt_task));
    pthread_t*   tid   = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    int          ok    = tasks && tid;
    for (int t = 0; ok && t < nthreads; t++)
    {
        tasks[t].c      = c;
        tasks[t].e0     = e0 + (int)(((long long)(e1 - e0) * t) / nthreads);
        tasks[t].e1     = e0 + (int)(((long long)(e1 - e0) * (t + 1)) / nthreads);
        tasks[t].energy = computeEnergy;
        tasks[t].fnb    = (float*)malloc(sizeof(float) * npad3 + 4);
        ok              = tasks[t].fnb != NULL;
    }
    int started = 0;
    for (int t = 0; ok && t < nthreads; t++, started++)
    {
        if (pthread_create(&tid[t], NULL, mt_run, &tasks[t]) != 0)
        {
            ok = 0;
            break;
        }
    }
    for (int t = 0; t < started; t++)
    {
        pthread_join(tid[t], NULL);
    }
    if (ok)
    {
        memset(c->fnb, 0, sizeof(float) * npad3);
        memset(c->fshift, 0, sizeof(c->fshift));
        c->vc = c->vlj = 0;
        for (int t = 0; t < nthreads; t++)
        {
            for (size_t k = 0; k < npad3; k++)
            {
                c->fnb[k] += tasks[t].fnb[k];
            }
            for (int k = 0; k < NSHIFT * 3; k++)
            {
                c->fshift[k] += tasks[t].fsh[k];
            }
            c->vc += tasks[t].vc;
            c->vlj += tasks[t].vlj;
        }
    }
    for (int t = 0; tasks && t < nthreads; t++)
    {
        free(tasks[t].fnb);
    }
    free(tasks);
    free(tid);
    return ok ? 0 : -1;
}

/* atomdata.cpp:1181-1228 nbnxn_atomdata_add_nbat_f_to_f_part: f[a] = fnb[cell[a]] */
void orc_forces_original_order(const orc_ctx* c, float* f_out)
{
    for (int a = 0; a < c->n; a++)
    {
        const int k = c->cells[a];
        for (int d = 0; d < 3; d++)
        {
            f_out[a * 3 + d] = c->fnb[k * 3 + d];
        }
    }
}

/* mdlib/sim_util.cpp:157-176 calc_virial + mdlib/calcvir.cpp:103-145:
 * vir = -1/2 (sum_i x_i (x) f_i + sum_s shift_s (x) fshift_s) */
void orc_virial(const orc_ctx* c, const float* x, const float* f, double* vir9)
{
    double v[9] = { 0 };
    for (int i = 0; i < c->n; i++)
    {
        for (int a = 0; a < 3; a++)
        {
            for (int b = 0; b < 3; b++)
            {
                v[a * 3 + b] += (double)x[i * 3 + a] * (double)f[i * 3 + b];
            }
        }
    }
    for (int s = 0; s < NSHIFT; s++)
    {
        for (int a = 0; a < 3; a++)
        {
            for (int b = 0; b < 3; b++)
            {
                v[a * 3 + b] += (double)c->shiftvec[s * 3 + a] * c->fshift[s * 3 + b];
            }
        }
    }
    for (int k = 0; k < 9; k++)
    {
        vir9[k] = -0.5 * v[k];
    }
}

void orc_energies(const orc_ctx* c, double* e2)
{
    e2[0] = c->vlj;
    e2[1] = c->vc;
}

void orc_fshift(const orc_ctx* c, float* fshift135)
{
    for (int k = 0; k < NSHIFT * 3; k++)
    {
        fshift135[k] = (float)c->fshift[k];
    }
}

float orc_beta(const orc_ctx* c) { return c->beta; }
float orc_table_scale(const orc_ctx* c) { return c->tab_scale; }
int   orc_table_size(const orc_ctx* c) { return c->tab_n; }
void  orc_table(const orc_ctx* c, float* F, float* V)
{
    if (c->tab_n > 0)
    {
        memcpy(F, c->tabF, sizeof(float) * (size_t)c->tab_n);
        memcpy(V, c->tabV, sizeof(float) * (size_t)c->tab_n);
    }
}
float orc_epsfac(const orc_ctx* c) { return c->epsfac; }
float orc_rbb2(const orc_ctx* c) { return c->rbb2; }

void orc_grid_dims(const orc_ctx* c, int* dims6, float* cs4)
{
    dims6[0] = c->ncx;
    dims6[1] = c->ncy;
    dims6[2] = c->ncol;
    dims6[3] = c->ncells;
    dims6[4] = c->nclusters_tot;
    dims6[5] = c->ncells * SC;
    cs4[0]   = c->cs[0];
    cs4[1]   = c->cs[1];
    cs4[2]   = c->ics[0];
    cs4[3]   = c->ics[1];
}
const int*      orc_cxy_ind(const orc_ctx* c) { return c->cxy_ind; }
const int*      orc_num_clusters(const orc_ctx* c) { return c->nclusters; }
const int*      orc_atom_indices(const orc_ctx* c) { return c->atom_indices; }
const int*      orc_cells(const orc_ctx* c) { return c->cells; }
const float*    orc_xq(const orc_ctx* c) { return c->xq; }
const int*      orc_types_grid(const orc_ctx* c) { return c->tgrid; }
const float*    orc_bb(const orc_ctx* c) { return c->bb; }
const float*    orc_bbcz(const orc_ctx* c) { return c->bbcz; }
const float*    orc_fnb(const orc_ctx* c) { return c->fnb; }
void            orc_list_sizes(const orc_ctx* c, int* s3)
{
    s3[0] = c->nsci;
    s3[1] = c->ncj4;
    s3[2] = c->nexcl;
}
const int*      orc_sci(const orc_ctx* c) { return (const int*)c->sci; }
const int*      orc_cj4(const orc_ctx* c) { return (const int*)c->cj4; }
const uint32_t* orc_excl(const orc_ctx* c) { return (const uint32_t*)c->excl; }
const uint32_t* orc_imask_outer(const orc_ctx* c) { return c->imask_outer; }

/* -------------------------------------------------- FP64 all-pairs oracle */

static int is_excluded(const int* excl_index, const int* excl_list, int i, int j)
{
    for (int k = excl_index[i]; k < excl_index[i + 1]; k++)
    {
        if (excl_list[k] == j)
        {
            return 1;
        }
    }
    return 0;
}

void orc_fp64_allpairs(int n, const float* xin, const float* box, const float* q, const int* type,
                       int ntypes, const float* nbfp, const int* excl_index, const int* excl_list,
                       int coulomb, double rc, double beta, double epsfac, double k_rf,
                       double c_rf, int use_ewald_shift, const int* subset, int nsub,
                       double* f_out, double* e2, int vdw_mod, double rvdw_switch, double beta_lj)
{
    /* vdw_mod 4: LJ-PME real space with the geometric grid (kernel_ref_inner.h:204-252): the
     * potential-shift LJ plus, for every pair within rc (excluded ones included), the grid part
     * c6grid (1 - e^-b (1 + b + b^2/2)) / r^6, b = beta_lj^2 r^2, with its shift sh_lj_ewald
     * (forcerec.cpp:711-712) on interacting pairs, and the self term C6_ii beta_lj^6 / 12. */
    const double bl2 = beta_lj * beta_lj, bl6_6 = bl2 * bl2 * bl2 / 6.0;
    const double crc2 = bl2 * rc * rc;
    const double sh_lj_ewald = vdw_mod == 4 ? (exp(-crc2) * (1 + crc2 + 0.5 * crc2 * crc2) - 1) / pow(rc, 6) : 0.0;
    /* wrap into the box in double */
    double* x = (double*)xmalloc(sizeof(double) * 3 * (size_t)n);
    for (int i = 0; i < n; i++)
    {
        for (int d = 0; d < 3; d++)
        {
            double v = xin[i * 3 + d];
            v -= floor(v / box[d]) * box[d];
            if (v >= box[d])
            {
                v -= box[d];
            }
            x[i * 3 + d] = v;
        }
    }
    /* cell list with cells >= rc and an explicit-image 27-cell stencil */
    int nc[3];
    for (int d = 0; d < 3; d++)
    {
        nc[d] = (int)floor(box[d] / rc);
        nc[d] = nc[d] < 1 ? 1 : nc[d];
    }
    const int ncell = nc[0] * nc[1] * nc[2];
    int*      head  = (int*)xmalloc(sizeof(int) * (size_t)ncell);
    int*      next  = (int*)xmalloc(sizeof(int) * (size_t)n);
    for (int k = 0; k < ncell; k++)
    {
        head[k] = -1;
    }
    for (int i = n - 1; i >= 0; i--)
    {
        int cc[3];
        for (int d = 0; d < 3; d++)
        {
            cc[d] = (int)(x[i * 3 + d] / box[d] * nc[d]);
            cc[d] = cc[d] >= nc[d] ? nc[d] - 1 : cc[d];
        }
        const int k = (cc[0] * nc[1] + cc[1]) * nc[2] + cc[2];
        next[i]     = head[k];
        head[k]     = i;
    }
    const double rc2      = rc * rc;
    const double sh_ewald = (coulomb == ORC_COULOMB_EWALD && use_ewald_shift) ? erfc(beta * rc) / rc : 0.0;
    /* LJ modifier constants in double (forcerec.cpp:787-816), see orc_set_vdw_modifier */
    double cpot6 = -1.0 / pow(rc, 6), cpot12 = -1.0 / pow(rc, 12);
    double fc2[2] = { 0, 0 }, fc3[2] = { 0, 0 }, sw3 = 0, sw4 = 0, sw5 = 0;
    {
        const double dd = rc - rvdw_switch;
        if (vdw_mod == 1)
        {
            for (int k = 0; k < 2; k++)
            {
                const double p = k == 0 ? 6.0 : 12.0;
                fc2[k] = ((p + 1) * rvdw_switch - (p + 4) * rc) / (pow(rc, p + 2) * dd * dd);
                fc3[k] = -((p + 1) * rvdw_switch - (p + 3) * rc) / (pow(rc, p + 2) * dd * dd * dd);
                const double cp = -pow(rc, -p) + p * fc2[k] / 3 * dd * dd * dd + p * fc3[k] / 4 * dd * dd * dd * dd;
                if (k == 0)
                {
                    cpot6 = cp;
                }
                else
                {
                    cpot12 = cp;
                }
            }
        }
        else if (vdw_mod == 2 || vdw_mod == 3)
        {
            cpot6 = cpot12 = 0;
            if (vdw_mod == 2)
            {
                sw3 = -10 / (dd * dd * dd);
                sw4 = 15 / (dd * dd * dd * dd);
                sw5 = -6 / (dd * dd * dd * dd * dd);
            }
        }
    }
    double       vlj = 0, vc = 0;
    for (int s = 0; s < nsub; s++)
    {
        const int i = subset[s];
        int       cc[3];
        for (int d = 0; d < 3; d++)
        {
            cc[d] = (int)(x[i * 3 + d] / box[d] * nc[d]);
            cc[d] = cc[d] >= nc[d] ? nc[d] - 1 : cc[d];
        }
        double fi[3] = { 0, 0, 0 };
        for (int ox = -1; ox <= 1; ox++)
        {
            for (int oy = -1; oy <= 1; oy++)
            {
                for (int oz = -1; oz <= 1; oz++)
                {
                    int    o[3] = { ox, oy, oz }, nb[3];
                    double img[3];
                    for (int d = 0; d < 3; d++)
                    {
                        int t  = cc[d] + o[d];
                        int w  = (int)floor((double)t / nc[d]);
                        nb[d]  = t - w * nc[d];
                        img[d] = w * box[d];
                    }
                    /* with cells >= rc, the 27 (cell, image) combinations
                     * are distinct also for 1 or 2 cells per dimension */
                    const int k = (nb[0] * nc[1] + nb[1]) * nc[2] + nb[2];
                    for (int j = head[k]; j >= 0; j = next[j])
                    {
                        double dr[3];
                        for (int d = 0; d < 3; d++)
                        {
                            dr[d] = x[i * 3 + d] - (x[j * 3 + d] + img[d]);
                        }
                        const double r2 = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
                        if (r2 >= rc2 || (j == i && r2 == 0.0))
                        {
                            continue;
                        }
                        /* a periodic self image interacts normally (the
                         * reference skips self exclusions, pairlist.cpp:1912) */
                        const int    excl = (j != i) && is_excluded(excl_index, excl_list, i, j);
                        const double r    = sqrt(r2);
                        const double qq   = epsfac * (double)q[i] * (double)q[j];
                        double       fscal = 0, v_c = 0, v_lj = 0;
                        if (coulomb == ORC_COULOMB_EWALD)
                        {
                            const double br  = beta * r;
                            const double g   = 2.0 * beta / sqrt(c_pi) * exp(-br * br);
                            if (!excl)
                            {
                                v_c   = qq * (erfc(br) / r - sh_ewald);
                                fscal = qq * (erfc(br) / r + g) / r2;
                            }
                            else
                            {
                                v_c   = -qq * erf(br) / r;
                                fscal = qq * (-erf(br) / r + g) / r2;
                            }
                        }
                        else
                        {
                            if (!excl)
                            {
                                v_c   = qq * (1.0 / r + k_rf * r2 - c_rf);
                                fscal = qq * (1.0 / (r * r2) - 2 * k_rf);
                            }
                            else
                            {
                                v_c   = qq * (k_rf * r2 - c_rf);
                                fscal = qq * (-2 * k_rf);
                            }
                        }
                        if (vdw_mod == 4)
                        {
                            /* the grid part, geometric: sqrt(6 C6_ii) sqrt(6 C6_jj) / 6 (float factors) */
                            const double c6g = (double)(sqrtf(nbfp[(type[i] * ntypes + type[i]) * 2])
                                                        * sqrtf(nbfp[(type[j] * ntypes + type[j]) * 2]))
                                               / 6.0;
                            const double ir6  = 1.0 / (r2 * r2 * r2);
                            const double b    = bl2 * r2;
                            const double em   = exp(-b);
                            const double poly = 1.0 + b + 0.5 * b * b;
                            fscal += 6.0 * c6g * (ir6 - em * (ir6 * poly + bl6_6)) / r2;
                            vlj += 0.5 * c6g * (ir6 * (1.0 - em * poly) + (excl ? 0.0 : sh_lj_ewald));
                        }
                        if (!excl)
                        {
                            const double c6   = nbfp[(type[i] * ntypes + type[j]) * 2] / 6.0;
                            const double c12  = nbfp[(type[i] * ntypes + type[j]) * 2 + 1] / 12.0;
                            const double ir6  = 1.0 / (r2 * r2 * r2);
                            v_lj              = c12 * (ir6 * ir6 + cpot12) - c6 * (ir6 + cpot6);
                            double       frlj = 12 * c12 * ir6 * ir6 - 6 * c6 * ir6; /* F r */
                            const double rsw  = r - rvdw_switch > 0 ? r - rvdw_switch : 0;
                            if (vdw_mod == 1)
                            {
                                /* 6C6 = 6 c6, 12C12 = 12 c12 in the switch terms */
                                frlj += (-6 * c6 * (fc2[0] + fc3[0] * rsw) + 12 * c12 * (fc2[1] + fc3[1] * rsw)) * rsw * rsw * r;
                                v_lj += (-6 * c6 * (-fc2[0] / 3 - fc3[0] / 4 * rsw)
                                         + 12 * c12 * (-fc2[1] / 3 - fc3[1] / 4 * rsw)) * rsw * rsw * rsw;
                            }
                            else if (vdw_mod == 2)
                            {
                                const double sw  = 1 + (sw3 + (sw4 + sw5 * rsw) * rsw) * rsw * rsw * rsw;
                                const double dsw = (3 * sw3 + (4 * sw4 + 5 * sw5 * rsw) * rsw) * rsw * rsw;
                                frlj             = frlj * sw - r * v_lj * dsw;
                                v_lj *= sw;
                            }
                            fscal += frlj / r2;
                        }
                        for (int d = 0; d < 3; d++)
                        {
                            fi[d] += fscal * dr[d];
                        }
                        vlj += 0.5 * v_lj;
                        vc += 0.5 * v_c;
                    }
                }
            }
        }
        for (int d = 0; d < 3; d++)
        {
            f_out[s * 3 + d] = fi[d];
        }
        if (vdw_mod == 4)
        {
            vlj += 0.5 * (double)nbfp[(type[i] * ntypes + type[i]) * 2] / 6.0 * bl6_6;
        }
        if (coulomb == ORC_COULOMB_EWALD)
        {
            vc -= epsfac * beta / sqrt(c_pi) * (double)q[i] * (double)q[i];
        }
        else
        {
            vc -= 0.5 * epsfac * c_rf * (double)q[i] * (double)q[i];
        }
    }
    if (e2)
    {
        e2[0] = vlj;
        e2[1] = vc;
    }
    free(x);
    free(head);
    free(next);
}
