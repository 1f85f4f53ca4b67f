/*
 * nbnxm_gb300 -- C ABI of the GB300 (sm_103a) short-range nonbonded engine.
 *
 * This is the drop-in boundary for the GROMACS nbnxm path that nblib's
 * ForceCalculator drives:
 *   cell gridding -> cluster-pair search (GPU 8x8x8 layout) -> rolling
 *   prune -> cluster-pair LJ + Ewald real-space force / energy / virial.
 * Plain pointers and sizes only; no C++ or torch types.  Every call returns
 * an nbx_status; nbx_last_error() describes the last failure of a handle.
 *
 * Coordinate / force arrays are float[3*N] in the caller's atom order.
 * Energies are double[2] = {LJ, Coulomb} in kJ/mol; the virial is
 * double[9] (row-major 3x3, kJ/mol), both reduced in FP64 on the GPU.
 */
#ifndef NBNXM_GB300_H
#define NBNXM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum
{
    NBX_OK                = 0,
    NBX_ERR_INVALID_INPUT = 1, /* bad sizes/options, NaN coordinates, non-positive box */
    NBX_ERR_OUT_OF_MEMORY = 2,
    NBX_ERR_LIST_OVERFLOW = 3, /* a list or grid capacity was exceeded (the call is retried internally once) */
    NBX_ERR_CUDA          = 4, /* a CUDA runtime error; see nbx_last_error */
    NBX_ERR_TIMEOUT       = 5, /* a bounded device-side wait gave up */
    NBX_ERR_NO_DEVICE     = 6,
    NBX_ERR_STATE         = 7  /* call order: e.g. compute before the first search */
} nbx_status;

/* Coulomb interaction, same values as nblib::CoulombType (api/nblib/kerneloptions.h:75-81) */
typedef enum
{
    NBX_COULOMB_EWALD  = 0, /* nblib Pme: Ewald real space, beta from ewald_rtol */
    NBX_COULOMB_CUTOFF = 1, /* nblib Cutoff: reaction field with eps_rf = 1 */
    NBX_COULOMB_RF     = 2  /* nblib ReactionField with epsilon_rf */
} nbx_coulomb;

/* The system, as nblib's SimulationState + Topology hold it
 * (api/nblib/simulationstate.h, api/nblib/topology.h:72-98). */
typedef struct
{
    int          num_atoms;
    const float* x;          /* [3N] initial coordinates; wrapped into the box like SimulationState */
    const float* q;          /* [N] charges (e) */
    const int*   type;       /* [N] particle type index in [0, num_types) */
    int          num_types;
    const float* nbfp;       /* [num_types^2 * 2] {6*C6, 12*C12} per type pair (api/nblib/gmxsetup.cpp:143-166) */
    const int*   excl_index; /* [N+1] CSR offsets of the exclusion lists (gmx::ListOfLists) */
    const int*   excl_list;  /* [excl_index[N]] excluded atoms (self entries allowed, ignored) */
    float        box[3];     /* rectangular box edges (nm); triclinic boxes are rejected like nblib */
} nbx_system_desc;

/* Kernel options, nblib::NBKernelOptions plus the list parameters of
 * PairlistParams (src/gromacs/nbnxm/pairlistparams.h:115-141). */
typedef struct
{
    int   coulomb;          /* nbx_coulomb */
    float rcoulomb;         /* interaction cut-off, also rvdw (nm) */
    float rlist;            /* outer pair-list radius (nm), >= rcoulomb */
    float rlist_inner;      /* inner radius after dynamic pruning (nm); <= 0: = rlist */
    float ewald_rtol;       /* erfc(beta*rc) = ewald_rtol; 0 -> 1e-5 like nblib */
    float epsilon_rf;       /* reaction-field dielectric for NBX_COULOMB_RF */
    int   use_ewald_shift;  /* 1: shift the Ewald potential to 0 at rc (mdrun); 0: nblib (no shift) */
    int   nstlist;          /* steps between searches for nbx_md_step_device (>= 1) */
    int   nstlist_prune;    /* dynamic pruning interval (0 = off); rolling over nstlist_prune/2 parts */
    int   compute_energy;   /* default energy/virial flag for nbx_compute */
    int   vdw_modifier;     /* nbx_vdw_modifier (0 = potential shift, nblib's only choice) */
    float rvdw_switch;      /* switching distance for the switch modifiers (nm), < rcoulomb */
    float ewald_rtol_lj;    /* LJ-PME: the LJ Ewald coefficient from rtol (<= 0: 1e-3, the mdp default) */
} nbx_options;

/* LJ interaction modifiers (mdp vdw-modifier; interaction_const_t::vdw_modifier,
 * mdlib/forcerec.cpp:853-872).  Batches and the adjoint take the potential shift only. */
typedef enum
{
    NBX_VDW_POTSHIFT    = 0, /* potential shifted to zero at rc, force unchanged */
    NBX_VDW_FORCESWITCH = 1, /* force switched to zero between rvdw_switch and rc */
    NBX_VDW_POTSWITCH   = 2, /* potential switched to zero between rvdw_switch and rc */
    NBX_VDW_NONE        = 3, /* plain cut-off */
    NBX_VDW_LJPME       = 4  /* LJ-PME real space (vdwtype PME, geometric grid) with the potential shift:
                                the grid part c6grid (1 - e^-b (1 + b + b^2/2)) / r^6, b = beta_lj^2 r^2, is
                                subtracted (kernel_ref_inner.h:204-252); the reciprocal part is
                                nbx_pme_create_lj */
} nbx_vdw_modifier;

typedef struct nbx_handle nbx_handle;

/* Fills opts with nblib's defaults: Ewald, rc = rlist = 1.0, rtol 1e-5, no dynamic pruning. */
void nbx_default_options(nbx_options* opts);

/* Replaces nblib::ForceCalculator::ForceCalculator (api/nblib/forcecalculator.cpp:52-55 ->
 * GmxSetupDirector::setupGmxForceCalculator, api/nblib/gmxsetup.cpp:306-325): copies the
 * topology to the GPU, sets up the interaction constants, grids the atoms and builds the list. */
int nbx_create(const nbx_system_desc* sys, const nbx_options* opts, int device, nbx_handle** out);
int nbx_destroy(nbx_handle* h);
/* Text of the last error on h (or of the last failed nbx_create when h is NULL). */
const char* nbx_last_error(const nbx_handle* h);

/* Replaces ForceCalculator::updatePairList (api/nblib/forcecalculator.cpp:62-67 ->
 * GmxForceCalculator::setParticlesOnGrid, gmxcalculator.cpp:85-103) and, unlike the
 * reference, also rebuilds the pair list and atom data (which the reference leaves stale).
 * x: host [3N]. */
int nbx_update_pairlist(nbx_handle* h, const float* x);

/* Replaces ForceCalculator::compute (api/nblib/forcecalculator.cpp:57-60 ->
 * GmxForceCalculator::compute, gmxcalculator.cpp:70-83): convertCoordinates ->
 * nonbonded kernel -> atomdata_add_nbat_f_to_f.  Host arrays; forces are overwritten.
 * energies (double[2]) and virial (double[9]) may be NULL.  An array in pinned host memory mapped
 * into the device's address space (cudaMallocHost, cudaHostAlloc, cudaHostRegister) is read or
 * written by the kernels in place; other host memory is staged through device buffers. */
int nbx_compute(nbx_handle* h, const float* x, float* f, double* energies, double* virial);

/* ---- device-resident interface (pointers into device memory, asynchronous on the handle's stream) ---- */
/* Work queued on the previous stream is waited for, except when the new stream is capturing a CUDA
 * graph (then the capturing code orders the streams). */
int nbx_set_stream(nbx_handle* h, void* cuda_stream);
void* nbx_get_stream(nbx_handle* h);
/* nbnxn_put_on_grid + constructPairlist (src/gromacs/nbnxm/nbnxm.cpp:58-74, pairlist.cpp:4247-4262),
 * followed by the first prune when dynamic pruning is on (cuda/nbnxm_cuda.cu:510-517). */
int nbx_search_device(nbx_handle* h, const float* d_x);
/* Rolling prune of part `part` of nstlist_prune/2 parts, or a full prune of a fresh list for part < 0
 * (nbnxm_cuda_kernel_pruneonly.cuh; dispatch prunekerneldispatch.cpp:99-113). */
int nbx_prune_device(nbx_handle* h, int part);
/* convertCoordinates + kernel + reduction, into device buffers.  d_energies double[2],
 * d_virial double[9] may be NULL (then no energy/virial work is done). */
int nbx_compute_device(nbx_handle* h, const float* d_x, float* d_f, double* d_energies, double* d_virial);
/* One MD-style step with the reference's schedule: search when step % nstlist == 0, else a
 * rolling prune on even list ages (pairlistsets.h:106-114), then compute. */
int nbx_md_step_device(nbx_handle* h, long long step, const float* d_x, float* d_f, double* d_energies,
                       double* d_virial);
int nbx_synchronize(nbx_handle* h);
/* nbx_md_step_device with host arrays (x in, f / energies / virial out, inside the call; mapped
 * pinned arrays are used in place as in nbx_compute, except x on search steps, which is copied). */
int nbx_md_step(nbx_handle* h, long long step, const float* x, float* f, double* energies, double* virial);

/* ---- layout export, for parity checks against the nbnxm layout ---- */
/* sizes[8] = {num_atoms, ncx, ncy, num_cells, num_sci, num_cj4, num_excl, padded_atoms} */
int nbx_get_sizes(nbx_handle* h, int* sizes);
/* Grid: atom_indices[padded] (grid slot -> atom or -1), cells[N] (atom -> slot),
 * cxy_ind[ncx*ncy+1], num_clusters[num_cells], bb[num_cells*8*6] (lower xyz, upper xyz),
 * bbcz[num_cells*2], xq[padded*4].  Any pointer may be NULL. */
int nbx_get_grid(nbx_handle* h, int* atom_indices, int* cells, int* cxy_ind, int* num_clusters, float* bb,
                 float* bbcz, float* xq);
/* Pair list in the nbnxm GPU layout (pairlist.h:174-223): sci[4*num_sci] = {sci, shift, cj4_start,
 * cj4_end}; cj4[8*num_cj4] = {cj[4], imask0, excl_ind0, imask1, excl_ind1}; excl[32*num_excl];
 * imask_outer[2*num_cj4] (the rlist-pruned masks kept for rolling pruning).  Any pointer may be NULL. */
int nbx_get_pairlist(nbx_handle* h, int* sci, int* cj4, uint32_t* excl, uint32_t* imask_outer);
/* Per-pass counters of the last compute: pairs[0] = computed cluster pairs x 64 (all set imask bits),
 * pairs[1] = pairs inside the cut-off. */
int nbx_get_pair_counts(nbx_handle* h, long long* pairs);

/* ---- measurement helpers ---- */
/* enable != 0: record CUDA events around every force-kernel launch on the handle's stream. */
int nbx_set_timing(nbx_handle* h, int enable);
/* Since the last reset: force_ms = summed force-kernel event time, counts[0] = force-kernel launches,
 * counts[1] = all kernels this handle launched.  reset != 0 clears the counters after reading. */
int nbx_get_timings(nbx_handle* h, double* force_ms, long long* counts, int reset);
/* Summed device time (ms, CUDA events on the handle's stream, recorded while timing is on) and
 * event-pair counts per phase: [0] force kernel, [1] gridding (wrap, column scan, scatter, sort),
 * [2] search count pass, [3] search write pass, [4] prune (fresh or rolling).  ms and counts
 * are double[5] / long long[5] (either may be NULL); reset = 1 clears them. */
int nbx_get_phase_timings(nbx_handle* h, double* ms, long long* counts, int reset);
/* Force-kernel shape (no counterpart in the reference; the autotuner's tile and staging
 * axes).  tile 0: one atom pair per lane, a warp instruction covers 8 i-atoms x 4 j-atoms
 * (scalar FP32); tile 1 (default): two pairs per lane, 8 x 8 atoms per warp instruction
 * (packed FP32x2 arithmetic; potential-shift or plain cut-off LJ -- the switch modifiers and
 * LJ-PME always run tile 0).  stage_depth: j-cluster stage buffers per warp of tile 1, 2
 * (default) or 3 (two groups' copies in flight).  blocks_per_sm: resident 256-thread blocks per
 * SM of tile 1, 2 (default; up to 128 registers a thread) or 3 (80 registers).  Results agree
 * to rounding between shapes. */
int nbx_set_force_kernel(nbx_handle* h, int tile, int stage_depth, int blocks_per_sm);
int nbx_get_force_kernel(const nbx_handle* h, int* tile, int* stage_depth, int* blocks_per_sm);
/* Failure-detection test hook (no counterpart in the reference): with enable = 1 the force
 * kernel's shared-memory stage barriers wait for bytes that never arrive, so their bounded
 * (1 s) waits give up and the next nbx_compute / nbx_synchronize returns NBX_ERR_TIMEOUT; the
 * context stays usable.  Keep 0 outside that test. */
int nbx_set_wait_test(nbx_handle* h, int enable);
/* GPU list balancing (pairlist.cpp split_sci_entry / sort_sci): entries are split when the grid
 * has fewer than entries_per_sm x SMs cells (default 44, the reference's factor; 0 = never
 * split; entries are always sorted large-first).  Takes effect at the next search. */
/* The options the handle was created with. */
int nbx_get_options(const nbx_handle* h, nbx_options* out);
/* 1: nbx_compute_device / nbx_md_step_device ADD the nonbonded forces to d_f (mdrun's
 * nbnxn_gpu_add_nbat_f_to_f_kernel with accumulateForce, nbnxm_buffer_ops_kernels.cuh:134),
 * e.g. after bonded or PME forces; 0 (default): they overwrite d_f.  The host-array calls
 * (nbx_compute, nbx_md_step) always overwrite. */
int nbx_set_force_accumulate(nbx_handle* h, int enable);
int nbx_get_force_accumulate(const nbx_handle* h, int* enabled);
int nbx_set_list_balance(nbx_handle* h, int entries_per_sm);
/* out[4] = {min_ci_balanced, split target in cluster pairs (0: none), entries before
 * splitting, entries after} of the current list. */
int nbx_get_list_balance(nbx_handle* h, int* out);
/* Runs an FP32 FMA throughput probe on the device and returns the measured TFLOP/s
 * (2 flops per FMA); used as the FP32 roofline denominator. */
int nbx_measure_fp32_peak(int device, double* tflops);

/* ---- adjoint (differentiable forces) ---- */
/* No counterpart in the reference.  Given upstream gradients d_gF = dL/dF ([3N] float, atom
 * order) and d_gE = dL/dE for {LJ, Coulomb} energies ([2] double, NULL = zero), all in device
 * memory, recomputes every pair term of the current list at the coordinates d_x and writes
 * dL/dx ([3N] float: the Hessian-vector product with d_gF plus the energy terms), dL/dq ([N]
 * float) and dL/d(nbfp) ([num_types^2 * 2] double: gradients of the {6*C6, 12*C12} entries as the
 * list uses them, FP64 sums; entry (a, b) gets the pairs whose i-cluster atom has type a).
 * Any output may be NULL.  At most 15 particle types.  Runs on the handle's stream. */
int nbx_backward_device(nbx_handle* h, const float* d_x, const float* d_gF, const double* d_gE, float* d_gx,
                        float* d_gq, double* d_gnbfp);
/* Replaces the charges ([N], atom order) and/or the nbfp matrix ([num_types^2 * 2]), both in device
 * memory (either may be NULL); the list is kept.  The self energy then follows the new charges. */
int nbx_set_parameters_device(nbx_handle* h, const float* d_q, const float* d_nbfp);
/* The Lorentz-Berthelot type table and its adjoint, one kernel each on `stream` (device memory, no
 * handle): table[(i * ntypes + j) * 2 + {0, 1}] = {6 C6, 12 C12} with sigma_ij = (sigma_i +
 * sigma_j) / 2, epsilon_ij = sqrt(epsilon_i epsilon_j), C6 = 4 epsilon_ij sigma_ij^6, C12 = C6
 * sigma_ij^6 (nblib's combination, api/nblib/gmxsetup.cpp:143-166), all double; the backward pass
 * turns d L / d table into d L / d sigma and d L / d epsilon.  1 <= ntypes <= 64. */
int nbx_lb_table_device(const double* d_sigma, const double* d_epsilon, int ntypes, double* d_table, void* stream);
int nbx_lb_table_backward_device(const double* d_sigma, const double* d_epsilon, int ntypes, const double* d_gtable,
                                 double* d_gsigma, double* d_gepsilon, void* stream);
/* The force-matching loss sum_k (F_k - F_target_k)^2 over n3 float components, summed in FP64 into
 * d_loss (overwritten), and its gradient 2 (F - F_target) into d_gF, in one pass on `stream` (device
 * memory, no handle).  No counterpart in the reference (it computes forces, not fits); the batched
 * force matcher runs the same kernel inside its step. */
int nbx_match_loss_device(const float* d_f, const float* d_ftarget, long long n3, float* d_gF, double* d_loss,
                          void* stream);

/* ---- free-energy perturbation of some atoms (the perturbed-pair kernel) ---- */
/* Replaces the free-energy path of the nonbonded step: nb_free_energy_kernel
 * (src/gromacs/gmxlib/nonbonded/nb_free_energy.cpp:200-850) as dispatched from
 * kerneldispatch.cpp:458-567.  Perturbed atoms interpolate between state A (the topology's
 * charge and type) and state B with lambda_coul / lambda_vdw, with Beutler soft-core
 * (sc-r-power 6).  Ewald or reaction-field Coulomb; potential-shift or plain LJ cut-off. */
typedef struct
{
    int          num_perturbed;
    const int*   perturbed;    /* [P] atom indices */
    const float* qB;           /* [P] state-B charges */
    const int*   typeB;        /* [P] state-B types (< num_types) */
    float        lambda_coul;  /* initial lambdas, in [0, 1] */
    float        lambda_vdw;
    float        alpha_vdw;    /* sc-alpha for LJ and Coulomb (0: no soft-core) */
    float        alpha_coul;
    int          lambda_power; /* sc-power: 1 or 2 */
    float        sigma6_def;   /* sc-sigma^6 for pairs without C6 or C12 */
    float        sigma6_min;   /* lower bound of sigma^6 */
} nbx_fep_desc;

/* Masks the perturbed atoms out of the cluster path and computes every pair with a perturbed
 * atom in the perturbed-pair kernel from then on (energies include its lambda-weighted terms).
 * Needs box edges >= 2 rlist.  The next call must search (nbx_search_device, nbx_update_pairlist
 * or the search step of nbx_md_step_device). */
int nbx_fep_enable(nbx_handle* h, const nbx_fep_desc* desc);
int nbx_fep_set_lambda(nbx_handle* h, float lambda_coul, float lambda_vdw);
/* out[4] = {V_Coulomb, V_LJ, dV/dlambda_Coulomb, dV/dlambda_LJ} of the perturbed pairs (with their
 * self terms) from the last evaluation with energies; synchronises the handle's stream. */
int nbx_fep_get_energies(nbx_handle* h, double* out);
/* The same four FP64 values in device memory (valid after the evaluation on the handle's stream). */
const double* nbx_fep_energies_device(nbx_handle* h);
/* Back to the plain topology (the next call must search again). */
int nbx_fep_disable(nbx_handle* h);

/* ---- batched ensembles ---- */
/* Many independent systems (uneven sizes, shared types / nbfp / options) evaluated together:
 * per-system grids and lists, one persistent force launch over all list entries, per-system
 * FP64 energies and virials.  Coordinates and forces are one concatenated [3 * sum N] array in
 * system order; energies are double[2 * num_systems], virials double[9 * num_systems]. */
typedef struct nbx_batch nbx_batch;
int nbx_batch_create(int num_systems, const nbx_system_desc* systems, const nbx_options* opts, int device,
                     nbx_batch** out);
int nbx_batch_destroy(nbx_batch* b);
const char* nbx_batch_last_error(const nbx_batch* b);
/* offsets[num_systems+1]: atom offsets of the systems in the concatenated arrays (may be NULL) */
int nbx_batch_atoms(nbx_batch* b, long long* total_atoms, int* offsets);
int nbx_batch_set_stream(nbx_batch* b, void* cuda_stream);
/* Search every system (grid + list + first prune), like nbx_search_device per system. */
int nbx_batch_search_device(nbx_batch* b, const float* d_x);
/* Rolling prune of part `part` over all systems in one launch (part < 0: full prune of fresh lists). */
int nbx_batch_prune_device(nbx_batch* b, int part);
/* One batched force / energy / virial evaluation (six launches, or one CUDA graph launch). */
int nbx_batch_compute_device(nbx_batch* b, const float* d_x, float* d_f, double* d_energies, double* d_virial);
/* Scheduled step (search every nstlist steps, batched rolling prune, batched compute). */
int nbx_batch_md_step_device(nbx_batch* b, long long step, const float* d_x, float* d_f, double* d_energies,
                             double* d_virial);
/* The same step as num_systems sequential single-system nbx_md_step_device calls (comparison path). */
int nbx_batch_sequential_md_step_device(nbx_batch* b, long long step, const float* d_x, float* d_f,
                                        double* d_energies, double* d_virial);
/* Tuning knobs: CUDA-graph capture of the batched compute (default on), force-kernel launch shape
 * variant (0: 256x2, 1: 128x4, 2: 512x1, 3: 64x8 threads x blocks per SM) and the rolling-prune
 * interval with its inner radius (takes effect at the next search). */
int nbx_batch_set_graph(nbx_batch* b, int enable);
int nbx_batch_set_kernel_variant(nbx_batch* b, int variant);
/* The batched force kernel's tile and j-stage depth (as nbx_set_force_kernel; no counterpart in
 * the reference): tile 1 (default) two atom pairs per lane in packed FP32x2 arithmetic, tile 0
 * one pair per lane; stage_depth 2 (default) or 3.  The launch shape stays the kernel variant's.
 * The batched autotuner (gmxapi_gb300/batch.py) chooses among tile x depth x shape x prune
 * interval. */
int nbx_batch_set_force_kernel(nbx_batch* b, int tile, int stage_depth);
int nbx_batch_set_prune(nbx_batch* b, int nstlist_prune, float rlist_inner);
/* Batched adjoint (no counterpart in the reference).  d_q: all systems' charges, concatenated atom
 * order; d_nbfp: the shared {6 C6, 12 C12} table ([num_types^2 * 2]); either may be NULL.  Once
 * charges are set this way every system's self energy follows them. */
int nbx_batch_set_parameters_device(nbx_batch* b, const float* d_q, const float* d_nbfp);
/* dL/dx, dL/dq (concatenated atom order, float) and dL/dnbfp summed over all systems
 * ([num_types^2 * 2] double) for upstream d_gF ([3N] float) and d_gE ([2 * num_systems] double
 * {LJ, Coulomb} per system, NULL = 0); outputs may be NULL.  At most 15 particle types. */
int nbx_batch_backward_device(nbx_batch* b, const float* d_x, const float* d_gF, const double* d_gE, float* d_gx,
                              float* d_gq, double* d_gnbfp);
/* One force-matching gradient step over the batch, on the current pair lists: parameters (d_q,
 * d_nbfp as above) -> forces, energies, virials -> loss = sum |F - F_target|^2 (FP64, d_loss[1])
 * -> adjoint -> dL/dq ([N] float) and dL/dnbfp ([num_types^2 * 2] double).  Captured into one
 * CUDA graph (re-captured when an argument pointer changes) unless graphs are switched off.  The
 * type table is written to the copy the batched kernels read (the first system's); the other
 * systems' copies follow only nbx_batch_set_parameters_device. */
int nbx_batch_force_match_device(nbx_batch* b, const float* d_x, const float* d_q, const float* d_nbfp,
                                 const float* d_ftarget, double* d_loss, float* d_gq, double* d_gnbfp, double* d_e,
                                 double* d_vir);

/* ---- allocation-free force evaluation ---- */
/* Inputs of nbx_compute_noalloc: the atom data and pair list in the layouts that
 * nbx_get_grid / nbx_get_pairlist export, all in device memory. */
typedef struct
{
    int             num_atoms;  /* N */
    int             num_slots;  /* grid slots (padded atoms) in xq / types; at most 65536 */
    int             num_sci;    /* list entries */
    const float*    xq;         /* [4*num_slots] x, y, z, q per grid slot (fillers: far away, q = 0); 16-byte aligned */
    const int*      types;      /* [num_slots] type per slot; fillers carry num_types (the all-zero type); 16-byte aligned */
    int             num_types;  /* real types; nbfp has (num_types+1)^2 pairs */
    const float*    nbfp;       /* [(num_types+1)^2 * 2] {6*C6, 12*C12}, zero row/column for the filler type */
    const int*      cells;      /* [N] grid slot of each atom */
    const int*      sci;        /* [4*num_sci] */
    const int*      cj4;        /* [8*num_cj4] */
    const uint32_t* excl;       /* [32*num_excl] */
    const int*      excl_index; /* [N+1], needed when energies or the virial are requested */
    const int*      excl_list;
    float           box[3];
    int             coulomb;    /* nbx_coulomb */
    float           rcoulomb, rlist, ewald_rtol, epsilon_rf;
    int             use_ewald_shift;
} nbx_noalloc_args;

/* No counterpart in the reference: an extra entry point for callers that may not
 * allocate device memory -- an engine that owns every device allocation through
 * its own pool, or code that runs while allocation is forbidden.  It runs the
 * same force / energy / virial kernels as nbx_compute_device on a pair list the
 * caller already holds, and allocates nothing: its scratch (grid-order force
 * accumulator, FP64 sums, work-queue header) is one file-scope device array
 * sized for at most 65536 grid slots, which every GPU that loads the library
 * keeps until exit.  The first call on a device looks up that array's device
 * address (cudaGetSymbolAddress) with the device current, so make the first
 * call before any stream capture.  All calls share the array: calls that
 * overlap on the GPU (different streams, or different threads) race and must
 * be serialised by the caller.  Returns NBX_ERR_LIST_OVERFLOW when num_slots
 * exceeds the maximum and NBX_ERR_INVALID_INPUT when num_atoms > num_slots or
 * num_slots is not a multiple of 64; every cells[i] must be below num_slots.
 * f: [3N] output in atom order; energies (double[2]) and virial (double[9]) may
 * be NULL.  Asynchronous on cuda_stream: a failure on the device (a bounded
 * wait that gave up) cannot be returned by this call, so it turns every output
 * value of the call into NaN and leaves its code for nbx_noalloc_status. */
int nbx_compute_noalloc(const nbx_noalloc_args* args, float* d_f, double* d_energies, double* d_virial,
                        void* cuda_stream);
/* No counterpart in the reference: the device status of the last nbx_compute_noalloc on the
 * current device, read after synchronising cuda_stream (allocates nothing): NBX_OK,
 * NBX_ERR_TIMEOUT (a bounded device-side wait gave up; the outputs are NaN) or
 * NBX_ERR_LIST_OVERFLOW.  The next nbx_compute_noalloc clears it. */
int nbx_noalloc_status(void* cuda_stream);
/* Failure-detection test hook (no counterpart in the reference), the allocation-free analogue
 * of nbx_set_wait_test: with enable = 1 the stage barriers of later nbx_compute_noalloc calls
 * wait for bytes that never arrive, so their bounded (1 s) waits give up.  Keep 0 outside
 * that test. */
int nbx_noalloc_set_wait_test(int enable);

/* ---- smooth PME, reciprocal space (the long-range half of the Ewald sum) ---- */
/* Rectangular boxes, pme_order 4, one GPU, charges only (no LJ-PME, no free-energy
 * grids).  The real-space half is nbx_compute* with coulomb = NBX_COULOMB_EWALD and
 * the same Ewald coefficient.  Device layouts: real grid [nx][ny][nz] floats (z
 * fastest); half-complex grid [nx][ny][nz/2+1] of {re, im} float pairs. */
typedef struct nbx_pme nbx_pme;

/* Replaces calc_ewaldcoeff_q (src/gromacs/ewald/ewald_utils.h:68): the Ewald
 * coefficient beta with erfc(beta rc) = ewald_rtol (<= 0 means 1e-5); 0 for rc <= 0. */
float nbx_ewald_coefficient(float rcoulomb, float ewald_rtol);

/* Replaces calcFftGrid (src/gromacs/fft/calcgrid.h:46) with minGridPointsPerDim =
 * 2 (pme_order - 1): grid sizes n[3] for box edges box[3] and the largest spacing. */
int nbx_pme_grid_size(const float* box, float spacing, int* n);

/* Replaces gmx_pme_init (src/gromacs/ewald/pme.h:140): box[3] edges (nm), grid[3]
 * sizes (6..4096 each), the Ewald coefficient, epsilon_r (<= 0 means 1). */
int nbx_pme_create(const float* box, const int* grid, float ewaldcoeff_q, float epsilon_r, int device, nbx_pme** out);
/* The Lennard-Jones (dispersion) grid of LJ-PME with the geometric combination rule: the same
 * handle and calls, with the per-atom coefficients sqrt(C6_ii) in place of the charges (the
 * reference's sqrt_c6A, mdlib/mdatoms.cpp:444) and solve_pme_lj_yzx (pme_solve.cpp:588-915);
 * energies and virials are the dispersion energy and virial. */
int nbx_pme_create_lj(const float* box, const int* grid, float ewaldcoeff_lj, int device, nbx_pme** out);
/* Replaces calc_ewaldcoeff_lj (src/gromacs/ewald/ewald_utils.h): beta with
 * exp(-x^2)(1 + x^2 + x^4/2) = ewald_rtol_lj, x = beta rvdw (<= 0 means 1e-3). */
float nbx_ewald_coefficient_lj(float rvdw, float ewald_rtol_lj);
/* Replaces gmx_pme_destroy (src/gromacs/ewald/pme.h:168). */
int         nbx_pme_destroy(nbx_pme* p);
const char* nbx_pme_last_error(const nbx_pme* p);
int         nbx_pme_set_stream(nbx_pme* p, void* cuda_stream);
int         nbx_pme_synchronize(nbx_pme* p);
/* grid[3] sizes and the Ewald coefficient (either may be NULL). */
int nbx_pme_get_info(const nbx_pme* p, int* grid, float* ewaldcoeff_q);

/* Replaces gmx_pme_do (src/gromacs/ewald/pme.h:181) for the Coulomb grid: spreads the
 * charges d_q[N] at d_x[3N] (device, atom order, any image within two box lengths of
 * the unit cell), solves, and ADDS the reciprocal-space forces to d_f[3N].  d_energy
 * (double[1]) and d_virial (double[9]) may be NULL; when either is given the solve
 * sums the energy and virial (FP64).  Asynchronous on the handle's stream. */
int nbx_pme_compute_device(nbx_pme* p, int natoms, const float* d_x, const float* d_q, float* d_f, double* d_energy,
                           double* d_virial);

/* The stages of nbx_pme_compute_device one at a time, as the reference's PME tests
 * drive them (src/gromacs/ewald/tests/pmetestcommon.h: pmePerformSplineAndSpread,
 * pmePerformSolve, pmePerformGather):
 *  splines: gridline indices d_idx[N][3], weights d_theta[3][N][4], derivatives d_dtheta[3][N][4];
 *  spread:  overwrites the real grid d_grid with the spread charges;
 *  solve:   scales the half-complex grid d_cgrid in place, optional energy / virial;
 *  gather:  adds the forces interpolated from the real grid d_grid to d_f. */
int nbx_pme_splines_device(nbx_pme* p, int natoms, const float* d_x, int* d_idx, float* d_theta, float* d_dtheta);
int nbx_pme_spread_device(nbx_pme* p, int natoms, const float* d_x, const float* d_q, float* d_grid);
int nbx_pme_solve_device(nbx_pme* p, void* d_cgrid, double* d_energy, double* d_virial);
int nbx_pme_gather_device(nbx_pme* p, int natoms, const float* d_x, const float* d_q, const float* d_grid, float* d_f);
/* The 3D transform of the handle's grid between the stages (see nbx_fft3d_execute_device). */
int nbx_pme_fft_device(nbx_pme* p, int direction, float* d_real, void* d_cgrid);

/* ---- the 3D real <-> half-complex FFT on its own (hand-written, no FFT library) ---- */
typedef struct nbx_fft3d nbx_fft3d;
/* Replaces gmx_parallel_3dfft_init (src/gromacs/fft/parallel_3dfft.h) on one rank for real data:
 * grid[3] = {nx, ny, nz}, each in [1, 1024] with prime factors of at most 255 (NBX_ERR_INVALID_INPUT
 * otherwise; PME grids from nbx_pme_grid_size always qualify). */
int nbx_fft3d_create(const int* grid, int device, nbx_fft3d** out);
int nbx_fft3d_destroy(nbx_fft3d* f);
/* Replaces gmx_parallel_3dfft_execute: direction +1 real d_real[nx][ny][nz] -> half-complex
 * d_cgrid[nx][ny][nz/2+1] (float2, exp(-2 pi i ...)); -1 d_cgrid -> d_real (exp(+2 pi i ...),
 * d_cgrid overwritten; the imaginary parts of the kz = 0 and, for even nz, kz = nz/2 planes are
 * taken as a Hermitian spectrum's, i.e. dropped).  Unnormalised both ways, as the reference's.  On
 * `stream`; device memory. */
int nbx_fft3d_execute_device(nbx_fft3d* f, int direction, float* d_real, void* d_cgrid, void* stream);

/* ---- GPU-resident MD steps: leap-frog and the step loop ---- */
typedef struct nbx_leapfrog nbx_leapfrog;

/* Replaces nblib::LeapFrog::LeapFrog (api/nblib/integrator.h:71): inverse masses inv_mass[N]
 * (host, finite, >= 0) and the rectangular box edges box[3]. */
int         nbx_leapfrog_create(int num_atoms, const float* inv_mass, const float* box, int device,
                                nbx_leapfrog** out);
int         nbx_leapfrog_destroy(nbx_leapfrog* p);
const char* nbx_leapfrog_last_error(const nbx_leapfrog* p);
int         nbx_leapfrog_set_stream(nbx_leapfrog* p, void* cuda_stream);
/* Replaces nblib::LeapFrog::integrate (api/nblib/integrator.h:84): v += f dt / m; x += v dt;
 * put_atoms_in_box.  Host arrays [3N], updated in place. */
int nbx_leapfrog_integrate(nbx_leapfrog* p, float dt, float* x, float* v, const float* f);
/* The same on device arrays, asynchronous on the handle's stream; d_ekin (double[1], may be
 * NULL) receives 0.5 (KE(t - dt/2) + KE(t + dt/2)), summed in FP64. */
int nbx_leapfrog_integrate_device(nbx_leapfrog* p, float dt, float* d_x, float* d_v, const float* d_f,
                                  double* d_ekin);

/* num_steps GPU-resident MD steps from first_step (mdrun's do_force + update, sim_util.cpp):
 * nonbonded forces with the handle's search / rolling-prune schedule (nbx_md_step_device)
 * written to d_f (overwriting, whatever nbx_set_force_accumulate says), PME forces added when
 * pme is not NULL (charges d_q[N]), leap-frog update of d_x / d_v;
 * atoms are put in the box only on the update before a search step.  All on h's stream.
 * Every nstcalcenergy steps (counted from first_step) a row of d_energies receives
 * {E_LJ, E_Coulomb real space, E_Coulomb reciprocal, E_kin} (FP64; E_kin as in
 * nbx_leapfrog_integrate_device); d_energies may be NULL. */
int nbx_md_run_device(nbx_handle* h, nbx_pme* pme, nbx_leapfrog* lf, long long first_step, int num_steps, float dt,
                      float* d_x, float* d_v, float* d_f, const float* d_q, int nstcalcenergy, double* d_energies);

#ifdef __cplusplus
}
#endif

#endif /* NBNXM_GB300_H */
