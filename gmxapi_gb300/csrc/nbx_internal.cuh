// Internal declarations shared by the nbnxm_gb300 translation units.
#pragma once

#include <cmath>

#include <cstdint>
#include <cuda_runtime.h>

namespace nbx
{

// Cluster geometry of the GPU pair list (src/gromacs/nbnxm/pairlistparams.h:60-89,
// pairlist.h:146-171): 8-atom clusters, 8 clusters (2x2x2) per 64-atom cell,
// j-clusters in groups of 4, each 8x8 cluster pair split in two warp halves.
constexpr int kCl       = 8;
constexpr int kNcl      = 8;
constexpr int kSc       = 64;
constexpr int kJg       = 4;
constexpr int kSplit    = 2;
constexpr int kExclW    = 32;
constexpr int kNShift   = 45;
constexpr int kCentral  = 22;
constexpr float kFarAway = -1000000.0f;         // atomdata.cpp:146
constexpr float kMinDist2 = 3.82e-07f;          // pairlist.h:146
constexpr int kErfcTerms = 8;                    // degree-7 polynomial in t

// erfc(x) = t P(t) exp(-x^2) with t = 1 / (1 + kErfcP x): P interpolates erfc(x) exp(x^2) / t at
// the 8 Chebyshev nodes of t in [1 / (1 + kErfcP kErfcXMax), 1] (x in [0, kErfcXMax]), written as
// monomial coefficients in t (float32 of the double-precision fit; relative error of the
// expansion <= 1.6e-7 on [0, 4]).  The substitution makes erfc(x) exp(x^2), which decays like
// 1/x, smooth enough for degree 7.  tests/test_oracle.py recomputes the fit and checks these.
constexpr float kErfcP    = 0.47f;
constexpr float kErfcXMax = 4.0f;  // beta * rc <= 4, i.e. ewald_rtol >= erfc(4) = 1.5e-8
__device__ __forceinline__ float erfc_poly(float t)
{
    float p = 1.128007565e-02f;
    p       = fmaf(p, t, 3.713922575e-02f);
    p       = fmaf(p, t, -3.248904943e-01f);
    p       = fmaf(p, t, 5.147097111e-01f);
    p       = fmaf(p, t, -7.699845731e-02f);
    p       = fmaf(p, t, 3.232774734e-01f);
    p       = fmaf(p, t, 2.490737736e-01f);
    return fmaf(p, t, 2.664087117e-01f);
}

// sqrt(pi)/2 erf(x)/x for w = x^2 <= 1, from its Maclaurin series sum_n (-w)^n / (n! (2n+1)):
// 1 - w/3 in FP64 and the tail w^2 sum_{n>=2} in float (terms n <= 13; the first dropped term is
// 1.1e-13 at w = 1).  The tail is at most 0.1 of the result, so its float rounding stays below
// 1e-8 relative, and the FP64 part is three operations (FP64 issues at a small fraction of the
// FP32 rate).  wd is w in FP64; the float tail uses w rounded to float.
__device__ __forceinline__ double erf_over_x_series(double wd)
{
    const float w = (float)wd;
    float       r = 5.94779391e-12f;  // 1/(13! 27)
    r             = fmaf(r, -w, 8.35070277e-11f);
    r             = fmaf(r, -w, 1.08922216e-09f);
    r             = fmaf(r, -w, 1.31225333e-08f);
    r             = fmaf(r, -w, 1.45038527e-07f);
    r             = fmaf(r, -w, 1.45891693e-06f);
    r             = fmaf(r, -w, 1.32275136e-05f);
    r             = fmaf(r, -w, 1.06837608e-04f);
    r             = fmaf(r, -w, 7.57575734e-04f);
    r             = fmaf(r, -w, 4.62962966e-03f);
    r             = fmaf(r, -w, 2.38095243e-02f);
    r             = fmaf(r, -w, 1.00000001e-01f);  // 1/(2! 5)
    return fma(wd, -1.0 / 3.0, 1.0) + (double)(w * w * r);
}

// Device status word bits (nbx_status values are derived from these on the host).
enum StatusBits : unsigned
{
    kStatusNaN            = 1u << 0,
    kStatusListOverflow   = 1u << 1,
    kStatusGridOverflow   = 1u << 2,
    kStatusWrapLimit      = 1u << 3,
    kStatusTimeout        = 1u << 4,
    kStatusExclOverflow   = 1u << 5,
    // a cell found more j-clusters than its search-record capacity (the host grows the records and
    // counts again; never an error)
    kStatusRecordOverflow = 1u << 6,
    // an entry with more than the per-entry cj4 limit of the search (an error)
    kStatusEntryOverflow  = 1u << 7,
};

// Entries one i-cell can have: one per shift of the half shell, at most 23 (5 x 3 x 3 shifts when the
// box is shorter than rlist along x, of which 22 backward and the central one).
constexpr int kMaxEntriesPerCell = 24;

struct Sci
{
    int sci, shift, cj4_start, cj4_end;
};

struct Imei
{
    unsigned imask;
    int      excl_ind;
};

struct Cj4
{
    int  cj[kJg];
    Imei imei[kSplit];
};

struct Excl
{
    unsigned pair[kExclW];
};

// Sizes written by device kernels, read back only when needed.
struct ListHeader
{
    int num_cells;       // cells in the current grid
    int num_sci;         // entries in the list
    int num_cj4;
    int num_excl;        // exclusion masks in use (entry 0 = all interacting)
    int sci_capacity;
    int cj4_capacity;
    int excl_capacity;
    int num_clusters;    // non-empty clusters
    unsigned status;     // StatusBits
    int work_counter;    // persistent-kernel work queue head
    int work_counter2;
    int num_subpairs;    // cluster pairs of the searched list (bits of imei[0].imask)
    int nsp_max;         // split target of the last balancing (0: no split)
    int num_sci_unsplit; // entries before splitting
    int num_sci_split;   // entries after splitting (scan result)
    int rec_need;        // largest number of j-cluster records one cell produced in the count pass
};

// Grid dimensions, fixed for a handle (box and atom count do not change).
struct GridDims
{
    int   ncx, ncy, ncol;
    float cs[2], ics[2];
    float box[3];
    int   cells_capacity;  // N/64 + ncol (grid.cpp:206-214)
};

// Everything the device kernels need, passed by value.
struct DeviceView
{
    int        n;
    GridDims   g;
    // topology (original order)
    const float* q;
    const int*   type;
    const int*   excl_index;
    const int*   excl_list;
    int          ntypes1;  // types + dummy
    const float2* nbfp;    // ntypes1^2 {6C6, 12C12}
    // grid
    float*  xin;           // [3N] wrapped coordinates
    int*    col;           // [N] column of each atom
    int*    slot;          // [N] position of each atom within its column (before the column sort)
    int*    image;         // [N] box shifts applied by the wrap, 3 signed bytes (x, y, z)
    int*    cxy_na;        // [ncol]
    int*    cxy_ind;       // [ncol+1]
    int*    atom_indices;  // [cap*64]
    int*    cells;         // [N]
    float4* xq;            // [cap*64]
    int*    tgrid;         // [cap*64]
    // the same atoms cluster-packed for the packed force kernel: per cluster of 8 atoms one
    // 160-byte record x[8], y[8], z[8], q[8], type[8] (int bits) with atom a at position
    // 2 (a & 3) + (a >> 2), so atoms a and a + 4 are adjacent
    float*  xqp;           // [cap*64*5]
    float4* bb;            // [cap*8*2] lower, upper
    float2* bbcz;          // [cap]
    int*    nclusters;     // [cap]
    // list
    Sci*      sci;
    Sci*      sci_tmp;      // [sci_cap] split entries before the size sort
    int*      sci_pieces;   // [sci_cap + 1] pieces per searched entry, then their offsets
    Cj4*      cj4;
    Excl*     excl;
    unsigned* imask_outer;  // [2*cj4_cap]
    int       sci_cap, cj4_cap, excl_cap;
    int*      sci_count;    // [cap] entries per cell (search count pass)
    int*      cj4_count;    // [cap] cj4 per cell
    int*      sci_offset;   // [cap+1]
    int*      cj4_offset;   // [cap+1]
    // search records, written by the count pass and turned into the list by the emit pass: per cell
    // up to rec_cap j-clusters (index, 8-bit i-cluster mask) in list order and up to
    // kMaxEntriesPerCell entry codes (shift | j-clusters << 8)
    int*           rec_cj;     // [cap * rec_cap]
    unsigned char* rec_m;      // [cap * rec_cap]
    int*           rec_ent;    // [cap * kMaxEntriesPerCell]
    int            rec_cap;
    unsigned char* grp_pairs;  // [cj4_cap] cluster pairs (bits of imei[0].imask) per cj4 group
    // outputs
    float4*  fnb;           // [cap*64] grid-order forces
    double*  energy;        // [2] {LJ, Coulomb}
    double*  fshift;        // [45*3]
    double*  virial;        // [9]
    ListHeader* hdr;
    // interaction constants
    float rc2, rlist, rlist2, rbb2, rlist_inner2;
    float beta, epsfac, k_rf, c_rf, sh_ewald, cpot6, cpot12;
    // LJ modifier (nbx_vdw_modifier) and its constants (mdlib/forcerec.cpp:787-816):
    // force switch F/p = r^-(p+1) + c2 r^2 + c3 r^3 for p = 6 (disp) and 12 (rep);
    // potential switch sw = 1 + c3 rsw^3 + c4 rsw^4 + c5 rsw^5
    unsigned wait_test_bytes;  // 0; > 0 only in the failure-detection test of the bounded stage waits
    int   vdw_mod;
    float rvdw_switch;
    float fsw_disp_c2, fsw_disp_c3, fsw_rep_c2, fsw_rep_c3;
    float psw_c3, psw_c4, psw_c5;
    int   coulomb;
    float shiftvec[kNShift * 3];
    double self_energy;     // Ewald / RF self term, constant for the system
    int    self_on_device;  // 1: k_excl_energy adds the self term from the charges instead
    double epsfac_d;        // 1/(4 pi eps0) in double for the energy sums
    // erfc(x) = t * P(t) * exp(-x^2), t = 1/(1 + kErfcP x) (erfc_poly), valid for beta*rc <= kErfcXMax
    float erfc_p;
    // derived per-pair constants (set_pair_constants), read straight from the
    // kernel parameters inside the pair loop
    float pbeta;    // erfc_p * beta
    float beta2l2;  // beta^2 log2(e)
    float c2b;      // 2 beta / sqrt(pi)
    float k_rf2;    // 2 k_rf
    // LJ-PME real space (vdw_mod NBX_VDW_LJPME): beta_lj^2, beta_lj^6 / 6, the grid potential's
    // shift at rc (forcerec.cpp:711-712) and the LJ self energy sum_i C6_ii beta^6 / 12
    float  lje_coeff2, lje_coeff6_6, sh_lj_ewald;
    double self_energy_lj;
    // 1: k_reduce_f adds the nonbonded forces to the caller's buffer
    // (nbnxn_gpu_add_nbat_f_to_f_kernel<accumulateForce = true>); 0: overwrites it
    int accumulate_f;
    // > 0: the energy flavours of k_force also compute the excluded-pair and self energies, as
    // this many work items of kExclChunkAtoms atoms interleaved with the list entries
    int excl_chunks;
    // force kernel tile: 1 = packed core (two pairs per lane, FP32x2 arithmetic; potential-shift
    // or plain cut-off LJ), 0 = scalar core (one pair per lane); j-stage buffers per warp (2, 3)
    int pair_core;
    int stage_depth;
    int force_blocks;  // resident blocks of 256 threads per SM for the packed kernel (2, 3)
};

// The system of batch entry e: the last system whose entry prefix sum is <= e.
__device__ __forceinline__ int find_system(const int* prefix, int nsys, int e)
{
    int lo = 0, hi = nsys - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= e)
        {
            lo = mid;
        }
        else
        {
            hi = mid - 1;
        }
    }
    return lo;
}

// Cluster-packed record of 8 atoms (kPackWords 32-bit words, 160 B): x[8], y[8], z[8], q[8],
// and the type as a byte offset into a row of 16-byte type-pair entries (type * 16), atom a at
// position 2 (a & 3) + (a >> 2) of each, so that atoms a and a + 4 (the two warp halves' j-atoms
// of one lane) are adjacent.
constexpr int kPackWords = 40;

// Writes slot k's coordinates, charge and type into the cluster-packed records (DeviceView::xqp).
__device__ __forceinline__ void write_packed_slot(float* xqp, int k, float x, float y, float z, float q, int type)
{
    float* pc = xqp + (size_t)(k >> 3) * kPackWords + 2 * (k & 3) + ((k >> 2) & 1);
    pc[0]     = x;
    pc[8]     = y;
    pc[16]    = z;
    pc[24]    = q;
    pc[32]    = __int_as_float(type * 16);
}

// One system of a batch, as the batched kernels see it (device table).
// LJ modifier constants for cut-off rc (interaction_const setup, forcerec.cpp:787-872).
inline void set_lj_modifier(DeviceView& v, int mod, float rc, float rsw)
{
    v.vdw_mod     = mod;
    v.rvdw_switch = rsw;
    v.fsw_disp_c2 = v.fsw_disp_c3 = v.fsw_rep_c2 = v.fsw_rep_c3 = 0.0f;
    v.psw_c3 = v.psw_c4 = v.psw_c5 = 0.0f;
    const double r = rc, s = rsw;
    if (mod == 0)
    {
        v.cpot6  = (float)(-1.0 / std::pow(r, 6.0));
        v.cpot12 = (float)(-1.0 / std::pow(r, 12.0));
    }
    else if (mod == 1)
    {
        auto fsw = [&](double p, float* c2, float* c3, float* cpot) {
            const double d  = r - s;
            const double k2 = ((p + 1) * s - (p + 4) * r) / (std::pow(r, p + 2) * d * d);
            const double k3 = -((p + 1) * s - (p + 3) * r) / (std::pow(r, p + 2) * d * d * d);
            *c2             = (float)k2;
            *c3             = (float)k3;
            *cpot           = (float)(-std::pow(r, -p) + p * k2 / 3 * d * d * d + p * k3 / 4 * d * d * d * d);
        };
        fsw(6.0, &v.fsw_disp_c2, &v.fsw_disp_c3, &v.cpot6);
        fsw(12.0, &v.fsw_rep_c2, &v.fsw_rep_c3, &v.cpot12);
    }
    else
    {
        v.cpot6 = v.cpot12 = 0.0f;
        if (mod == 2)
        {
            const double d = r - s;
            v.psw_c3       = (float)(-10.0 / (d * d * d));
            v.psw_c4       = (float)(15.0 / (d * d * d * d));
            v.psw_c5       = (float)(-6.0 / (d * d * d * d * d));
        }
    }
}

// Fills the derived pair constants of a view whose beta / erfc fit / k_rf are set.
inline void set_pair_constants(DeviceView& v)
{
    v.pbeta   = v.erfc_p * v.beta;
    v.beta2l2 = v.beta * v.beta * 1.4426950408889634f;
    v.c2b     = 1.1283791670955126f * v.beta;
    v.k_rf2   = 2.0f * v.k_rf;
}

struct BatchSys
{
    const float4*     xq;
    const int*        tgrid;
    const float*      xqp;        // cluster-packed records (DeviceView::xqp)
    float4*           fnb;
    const Sci*        sci;
    const Cj4*        cj4;
    const Excl*       excl;
    unsigned*         imask_outer;
    const int*        cells;
    const int*        atom_indices;
    const int*        image;
    const ListHeader* hdr;
    const int*        excl_index;
    const int*        excl_list;
    const float4*     gnb;        // adjoint: upstream force gradients in grid order
    float4*           dnb;        // adjoint: accumulated dL/dx, dL/dq in grid order
    float*            q;          // charges, atom order
    int               n;          // atoms
    int               atom_base;  // offset in the concatenated coordinate / force arrays
    int               self_on_device;  // 1: the self energy comes from the current charges
    int               pad1;
    double            self_energy;
    float             box[3];
    float             shiftvec[kNShift * 3];
};

// Dynamic shared memory beyond the 48 KB default needs a per-kernel opt-in; the attribute is a
// property of the kernel in the current device's context.  total_bytes (dynamic + static) decides
// whether the opt-in is needed; the largest dynamic size set so far is remembered per kernel and
// device (setting it again is harmless, so concurrent first calls need no lock).
template<auto kKernel>
cudaError_t smem_optin(size_t total_bytes, size_t dynamic_bytes)
{
    if (total_bytes <= 48 * 1024)
    {
        return cudaSuccess;
    }
    static int done[64] = { 0 };
    int        dev      = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    {
        return cudaFuncSetAttribute(kKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dynamic_bytes);
    }
    if (done[dev] >= (int)dynamic_bytes)
    {
        return cudaSuccess;
    }
    const cudaError_t e = cudaFuncSetAttribute(kKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)dynamic_bytes);
    if (e == cudaSuccess)
    {
        done[dev] = (int)dynamic_bytes;
    }
    return e;
}

// ---- host set-up helpers (nbx_api.cu) ----
double one_4pi_eps0();
float  calc_ewaldcoeff_q(float rc, float rtol);

// ---- launchers (one translation unit each) ----
// Free-energy (perturbed) pairs: what the perturbed-pair kernel needs besides the DeviceView.
// The perturbed atoms are masked out of the cluster path (charge 0, all-zero LJ type), so every
// pair with a perturbed atom is computed here, once.
struct FepView
{
    int                  np;     // perturbed atoms
    const int*           plist;  // [np] original indices
    const unsigned char* pert;   // [N] 1 for perturbed atoms
    const float*         qA;     // [N] state-A charges (unscaled)
    const float*         qB;     // [N] state-B charges (= qA for unperturbed atoms)
    const int*           tA;     // [N] state-A types
    const int*           tB;     // [N] state-B types (= tA for unperturbed atoms)
    // lambda factors per state {A, B} (nb_free_energy.cpp:356-388)
    float lfc[2], lfv[2], lfac_c[2], dlfac_c[2], lfac_v[2], dlfac_v[2];
    float alpha_c, alpha_v, sigma6_def, sigma6_min;
    int   soft;  // soft-core on (alpha_c or alpha_v non-zero)
    double* sums;  // [4]: V_Coulomb, V_LJ, dV/dlambda_Coulomb, dV/dlambda_LJ of the perturbed pairs
};

cudaError_t launch_fep(const DeviceView& v, const FepView& fp, bool energy, cudaStream_t s);
cudaError_t launch_grid(const DeviceView& v, float* d_x, int write_back, cudaStream_t s);
// clear: also zero the force-evaluation accumulators (grid forces, shift forces, energies,
// virial, work queue) for the next launch_force / launch_reduce_f; atom_order: read x in atom
// order (x in host memory read over the host link)
cudaError_t launch_convert_x(const DeviceView& v, const float* d_x, cudaStream_t s, bool clear = false,
                             bool atom_order = false);
cudaError_t launch_search(const DeviceView& v, cudaStream_t s);
cudaError_t launch_prune(const DeviceView& v, int fresh, int part, int nparts, cudaStream_t s);
cudaError_t launch_force(const DeviceView& v, bool energy, cudaStream_t s, int num_sms, cudaEvent_t ev0 = nullptr,
                         cudaEvent_t ev1 = nullptr);
// the packed-core force kernel (v.pair_core 1; potential-shift or plain cut-off LJ), with the
// v.stage_depth j-stage buffers and v.force_blocks blocks per SM
cudaError_t launch_force_x2(const DeviceView& v, bool energy, cudaStream_t s, int num_sms, int* counter);
// forces to atom order (+ virial); with d_e / d_vir the last block also finishes the energies
// and virial (the accumulators must have been cleared by launch_convert_x(clear))
// (stage: write the forces through shared memory as contiguous floats, for f in host memory)
cudaError_t launch_reduce_f(const DeviceView& v, float* d_f, double* d_e, double* d_vir, cudaStream_t s,
                            bool stage = false);
cudaError_t launch_pair_count(const DeviceView& v, unsigned long long* d_out, cudaStream_t s);
cudaError_t measure_fp32_peak(double* tflops);
cudaError_t launch_batch_prune(const BatchSys* sys, const int* entry_prefix, int nsys, float outer2, float inner2,
                               int fresh, int part, int nparts, cudaStream_t s);
int         adjoint_max_types1();
cudaError_t optin_batch_force_smem();
// d_x: coordinates converted into xq by the preparation kernel (nullptr: xq is current)
cudaError_t launch_backward(const DeviceView& v, const float* d_x, const float* d_gF, const double* d_gE,
                            float4* gnb, float4* dnb, double* d_gnbfp, int* counter, float* d_gx, float* d_gq,
                            double* d_gnbfp_out, int num_sms, cudaStream_t s);
cudaError_t launch_set_parameters(const DeviceView& v, const float* d_q, const float* d_nbfp, cudaStream_t s);
cudaError_t launch_lb_table(const double* sig, const double* eps, int nt, double* table, cudaStream_t s);
cudaError_t launch_lb_table_backward(const double* sig, const double* eps, int nt, const double* gtable,
                                     double* gsig, double* geps, cudaStream_t s);
cudaError_t launch_compact_gnbfp(const double* padded, double* out, int nt, cudaStream_t s);
cudaError_t launch_batch_backward(const DeviceView& cv, const BatchSys* sys, const int* prefix, int nsys,
                                  int max_slots, int max_atoms, const float* d_gF, const double* d_gE,
                                  double* d_gnbfp, int* counter, float* d_gx, float* d_gq, int num_sms, cudaStream_t s);
cudaError_t launch_batch_convert(const BatchSys* sys, int nsys, int max_slots, const float* d_x, cudaStream_t s);
cudaError_t launch_batch_set_q(const BatchSys* sys, int nsys, int max_slots, const float* d_q, cudaStream_t s);
cudaError_t launch_match_loss(const float* d_f, const float* d_ft, size_t n3, float* d_gF, double* d_loss,
                              int num_sms, cudaStream_t s);
cudaError_t launch_batch_prefix(const BatchSys* sys, int nsys, int* prefix, unsigned* status, cudaStream_t s);
// The batched force kernel with the packed pair core: launch shape 0..3 as the one-pair-per-lane
// kernel's (256 x 2, 128 x 4, 512 x 1, 64 x 8 threads x blocks per SM), stage_depth 2 or 3.
cudaError_t launch_batch_force_x2(const DeviceView& cv, const BatchSys* sys, const int* prefix, int nsys, int* counter,
                                  double* energies, double* fshift, int shape, int stage_depth, bool energy,
                                  int num_sms, cudaStream_t s);
cudaError_t optin_batch_force_x2_smem();
cudaError_t launch_batch_compute(const DeviceView& cv, const BatchSys* sys, const int* prefix, int nsys,
                                 int max_slots, int max_atoms, const float* d_x, float* d_f, double* sums,
                                 size_t sums_bytes, int* counter, double* d_e, double* d_vir, int variant,
                                 int num_sms, cudaStream_t s);

// Bounded spin limit for device-side waits (iterations); a wait that runs out
// sets kStatusTimeout and returns instead of hanging.
constexpr long long kSpinLimit = 1LL << 24;

} // namespace nbx
