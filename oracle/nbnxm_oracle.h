/*
 * CPU oracle for the short-range nonbonded path (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain-C restatement of the GROMACS 2021 nbnxm algorithm for the
 * GPU ("8x8x8" super-cluster) list layout, used only by tests/, smoke() and
 * the CPU-baseline leg of bench.py as the CHECKER of the CUDA path.  Nothing
 * in the product (gmxapi_gb300/) links, loads or calls it.
 *
 * Each function cites the reference source it follows (paths relative to the
 * GROMACS source root).  Pinning: forces are checked against the reference's
 * own golden vectors (api/nblib/tests/refdata/NBlibTest_{Argon,SpcMethanol}ForcesAreCorrect.xml) and against an FP64
 * all-pairs sum written independently here.
 *
 * Floating-point contract: build with -ffp-contract=off so that every float
 * operation rounds exactly as the reference built with -ffp-contract=off.
 */
#ifndef NBNXM_ORACLE_H
#define NBNXM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Coulomb flavours, matching nblib::CoulombType (api/nblib/kerneloptions.h:75-81) */
#define ORC_COULOMB_EWALD 0   /* nblib Pme: Ewald real space */
#define ORC_COULOMB_CUTOFF 1  /* nblib Cutoff: reaction field with eps_rf = 1 */
#define ORC_COULOMB_RF 2      /* nblib ReactionField */

typedef struct orc_ctx orc_ctx;

/* System + interaction setup.  x is wrapped into the rectangular box like
 * SimulationState does (api/nblib/simulationstate.cpp:88).  nbfp holds
 * ntypes*ntypes pairs {6*C6, 12*C12} (api/nblib/gmxsetup.cpp:143-166). */
orc_ctx* orc_create(int n, const float* x, const float* box, const float* q, const int* type,
                    int ntypes, const float* nbfp, const int* excl_index, const int* excl_list,
                    int coulomb, float rc, float rlist_outer, float rlist_inner,
                    float ewald_rtol, float epsilon_rf, int use_ewald_shift);
void orc_destroy(orc_ctx* c);
/* LJ modifier (0 potential shift (default), 1 force switch, 2 potential switch, 3 none)
 * with its constants, mdlib/forcerec.cpp:787-872. */
void orc_set_vdw_modifier(orc_ctx* c, int mod, float rvdw_switch);

/* Replace the (in-box) coordinates used for gridding and for orc_set_x. */
void orc_set_coordinates(orc_ctx* c, const float* x);

/* Gridding: grid.cpp Grid::setDimensions / calcColumnIndices / setCellIndices /
 * sortColumnsGpuGeometry / fillCell. */
void orc_grid(orc_ctx* c);
/* Pair search into the GPU layout: pairlist.cpp nbnxn_make_pairlist_part. */
void orc_search(orc_ctx* c);
/* GPU list balancing after a search: split_sci_entry (pairlist.cpp:2077-2165) with the
 * target of get_nsubpair_target (pairlist.cpp:2485-2585; exact pair count), then
 * sort_sci (pairlist.cpp:3827-3873).  min_ci_balanced = 44 x SM count in the reference
 * (cuda/nbnxm_cuda_data_mgmt.cu:93,545-548).  Returns the split target (0: none). */
int orc_balance(orc_ctx* c, int min_ci_balanced);
/* Copy coordinates (original order) into grid order without re-gridding:
 * atomdata.cpp nbnxn_atomdata_copy_x_to_nbat_x. */
void orc_set_x(orc_ctx* c, const float* x);
/* Prune: restates the rolling prune of cuda/nbnxm_cuda_kernel_pruneonly.cuh.
 * fresh=1: prune all entries from the search masks (outer and inner).
 * fresh=0: re-check entry indices i with i % nparts == part. */
void orc_prune(orc_ctx* c, int fresh, int part, int nparts);
/* Force kernel: kernels_reference/kernel_gpu_ref.cpp nbnxn_kernel_gpu_ref. */
void orc_force(orc_ctx* c, int compute_energy);
/* The force kernel over list entries [e0, e1) only (bounded timing samples). */
void orc_force_entries(orc_ctx* c, int e0, int e1, int compute_energy);

/* The same over nthreads threads (private force buffers, summed); 0 on success. */
int orc_force_entries_mt(orc_ctx* c, int e0, int e1, int compute_energy, int nthreads);

/* Outputs */
void orc_forces_original_order(const orc_ctx* c, float* f_out); /* N*3 */
void orc_virial(const orc_ctx* c, const float* x, const float* f, double* vir9);
void orc_energies(const orc_ctx* c, double* e2); /* {Vlj, Vcoul} */
void orc_fshift(const orc_ctx* c, float* fshift135);

/* Setup values */
float orc_beta(const orc_ctx* c);
float orc_table_scale(const orc_ctx* c);
int orc_table_size(const orc_ctx* c);
void orc_table(const orc_ctx* c, float* F, float* V);
float orc_epsfac(const orc_ctx* c);
float orc_rbb2(const orc_ctx* c);

/* Grid / list accessors */
void orc_grid_dims(const orc_ctx* c, int* dims6, float* cs4); /* ncx,ncy,ncol,ncells,nclusters_total,natoms_padded */
const int* orc_cxy_ind(const orc_ctx* c);
const int* orc_num_clusters(const orc_ctx* c);
const int* orc_atom_indices(const orc_ctx* c);
const int* orc_cells(const orc_ctx* c);
const float* orc_xq(const orc_ctx* c);
const int* orc_types_grid(const orc_ctx* c);
const float* orc_bb(const orc_ctx* c);   /* 6 floats per cluster: lower xyz, upper xyz */
const float* orc_bbcz(const orc_ctx* c); /* 2 floats per cell */
void orc_list_sizes(const orc_ctx* c, int* sizes3); /* nsci, ncj4, nexcl */
const int* orc_sci(const orc_ctx* c);     /* 4 ints per entry: sci, shift, cj4_start, cj4_end */
const int* orc_cj4(const orc_ctx* c);     /* 8 ints per cj4: cj[4], imask0, excl0, imask1, excl1 */
const uint32_t* orc_excl(const orc_ctx* c); /* 32 words per entry */
const uint32_t* orc_imask_outer(const orc_ctx* c); /* 2 words per cj4 (after fresh prune) */
const float* orc_fnb(const orc_ctx* c);  /* grid-order forces, 3 per padded atom */

/* Independent FP64 all-pairs oracle: explicit periodic images within rc,
 * analytic erfc, potential-shift LJ, exclusions with the Ewald exclusion
 * correction, Ewald self term.  Forces on atoms subset[0..nsub) from all
 * atoms.  Energies {Vlj, Vcoul} are totals only when nsub == n (and subset
 * is 0..n-1); set e2 to NULL otherwise. */
void orc_fp64_allpairs(int n, const float* x, const float* box, const float* q, const int* type,
                       int ntypes, const float* nbfp, const int* excl_index, const int* excl_list,
                       int coulomb, double rc, double beta, double epsfac, double k_rf,
                       double c_rf, int use_ewald_shift, const int* subset, int nsub,
                       double* f_out, double* e2, int vdw_mod, double rvdw_switch, double beta_lj);

/* nblib's 1/(4 pi eps0) in kJ mol^-1 nm e^-2 (src/gromacs/math/units.h:79) */
double orc_one_4pi_eps0(void);

/* ---- CPU layout (nbnxm_cpu_oracle.c): 4-atom clusters, the simple 4x4 list, a 4-wide kernel ----
 * Ewald real space with potential-shift LJ; x must stay valid for the lifetime of the context
 * (in box), nbfp holds ntypes^2 {6C6, 12C12}. */
typedef struct orc_cpu orc_cpu;
orc_cpu* orc_cpu_create(int n, const float* x, const float* box, const float* q, const int* type, int ntypes,
                        const float* nbfp, const int* excl_index, const int* excl_list, float rc, float rlist,
                        float beta, float epsfac);
void orc_cpu_destroy(orc_cpu* c);
/* grid.cpp setDimensions / calcColumnIndices / setCellIndices / sortColumnsCpuGeometry */
void orc_cpu_grid(orc_cpu* c);
/* pairlist.cpp nbnxn_make_pairlist_part with makeClusterListSimple */
void orc_cpu_search(orc_cpu* c);
/* new coordinates (atom order, same box images) into the grid layout without re-gridding */
void orc_cpu_set_x(orc_cpu* c, const float* x);
/* the cluster-pair kernel over list entries [e0, e1) on nthreads POSIX threads; 0 on success */
int  orc_cpu_force(orc_cpu* c, int e0, int e1, int energy, int nthreads);
void orc_cpu_sizes(const orc_cpu* c, int* s4); /* clusters, list entries, j entries, geometric rule */
void orc_cpu_list(const orc_cpu* c, int* ci4, int* cj2); /* {ci, shift, cj_start, cj_end}, {cj, excl} */
void orc_cpu_grid_arrays(const orc_cpu* c, int* atom_indices, float* xs); /* 4 per cluster; 16 per cluster */
void orc_cpu_forces(const orc_cpu* c, float* f_out); /* N*3, atom order */
void orc_cpu_energies(const orc_cpu* c, double* e2); /* {Vlj, Vcoul} */

#ifdef __cplusplus
}
#endif

#endif
