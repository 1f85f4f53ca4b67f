// Host side of nbnxm_gb300: handle, device memory, set-up constants and the C ABI.
//
// Set-up mirrors nblib's GmxSetupDirector (api/nblib/gmxsetup.cpp:226-325):
// interaction constants (Ewald beta by bisection, ewald/ewald_utils.cpp:46-71;
// RF constants, mdlib/rf_util.cpp:54-66; potential shifts), the nbfp matrix
// with one extra all-zero type (nbnxm/atomdata.cpp:440-620), the grid
// dimensions (nbnxm/grid.cpp:103-262) and the shift vectors
// (pbcutil/pbc.cpp:1187-1202).  Host arithmetic here is compiled with
// -ffp-contract=off so these constants round exactly like the reference's.
#include "../../include/nbnxm_gb300.h"
#include "nbx_internal.cuh"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <algorithm>
#include <vector>

namespace nbx
{
cudaError_t launch_search_count(const DeviceView& v, cudaStream_t s);
cudaError_t launch_search_write(const DeviceView& v, int num_entries, cudaStream_t s);
cudaError_t launch_balance(const DeviceView& v, int min_ci_balanced, cudaStream_t s);
} // namespace nbx

using namespace nbx;

struct nbx_handle
{
    int          device   = 0;
    int          num_sms  = 152;
    cudaStream_t stream   = nullptr;
    bool         own_stream = false;
    nbx_options  opts{};
    int          n        = 0;
    int          ntypes   = 0;
    DeviceView   v{};
    std::string  err;
    bool         have_list = false;
    long long    list_step = 0;   // step of the last search (nbx_md_step_device)
    int          prune_part = 0;  // next rolling-prune part
    int          nparts     = 1;
    bool         use_prune  = false;
    int          min_ci_balanced = 0;  // list balancing threshold (44 x SMs like the reference)
    std::vector<void*> allocations;
    // device buffers for the host-array interface
    float*  d_x = nullptr;
    float*  d_f = nullptr;
    double* d_out = nullptr;  // energies[2] + virial[9]
    unsigned long long* d_count = nullptr;
    ListHeader* h_hdr = nullptr;  // pinned copy for reading sizes
    double*     h_out = nullptr;  // pinned copy of the energies and virial (11 doubles)
    double*     d_hout = nullptr; // h_out's device address when the device can write it directly
    bool        x_host = false;   // this call's coordinates / forces are host memory used in place
    bool        f_host = false;
    // adjoint scratch, allocated on the first backward call
    float4* d_gnb   = nullptr;
    float4* d_dnb   = nullptr;
    double* d_gnbfp = nullptr;
    int*    d_adj_counter = nullptr;
    // timing / launch accounting
    bool        timing = false;
    std::vector<cudaEvent_t> ev_pool;
    struct PendingEvents
    {
        cudaEvent_t a, b;
        int         phase;
    };
    std::vector<PendingEvents> ev_pending;
    // summed event times and counts per phase (nbx_phase: force, grid, search count, search write, prune)
    double      phase_ms[5]    = { 0, 0, 0, 0, 0 };
    long long   phase_count[5] = { 0, 0, 0, 0, 0 };
    long long   force_launches = 0;
    long long   launches = 0;
    // free-energy perturbation (nbx_fep_*): the perturbed atoms leave the cluster path
    bool           fep_on       = false;
    FepView        fep{};
    float*         d_fep_q      = nullptr;  // [2N]: state A | state B charges
    int*           d_fep_t      = nullptr;  // [2N]: state A | state B types
    int*           d_fep_list   = nullptr;  // [N] perturbed atoms
    unsigned char* d_fep_pert   = nullptr;  // [N]
    double*        d_fep_sums   = nullptr;  // [4]
    double         self_energy_all = 0.0;    // the self energy with every atom, restored on disable
    int            fep_power       = 1;
};

namespace nbx
{

double one_4pi_eps0()
{
    // src/gromacs/math/units.h:69-79
    const double eps0 = (8.8541878128e-12 * 1e-9 * 1e3) / (1.602176634e-19 * 1.602176634e-19 * 6.02214076e23);
    return 1.0 / (4.0 * 3.14159265358979323846 * eps0);
}

// ewald/ewald_utils.cpp:46-71 in single precision
float calc_ewaldcoeff_q(float rc, float rtol)
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


} // namespace nbx

namespace
{

thread_local std::string g_create_error;

int set_error(nbx_handle* h, int code, const std::string& msg)
{
    if (h)
    {
        h->err = msg;
    }
    else
    {
        g_create_error = msg;
    }
    return code;
}

int cuda_check(nbx_handle* h, cudaError_t e, const char* where)
{
    if (e == cudaSuccess)
    {
        return NBX_OK;
    }
    if (e == cudaErrorMemoryAllocation)
    {
        return set_error(h, NBX_ERR_OUT_OF_MEMORY, std::string(where) + ": out of device memory");
    }
    return set_error(h, NBX_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

template<typename T>
cudaError_t dalloc(nbx_handle* h, T** p, size_t count)
{
    void*       q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess)
    {
        h->allocations.push_back(q);
        *p = static_cast<T*>(q);
    }
    return e;
}

void dfree(nbx_handle* h, void* p)
{
    for (auto it = h->allocations.begin(); it != h->allocations.end(); ++it)
    {
        if (*it == p)
        {
            cudaFree(p);
            h->allocations.erase(it);
            return;
        }
    }
}

int status_to_error(nbx_handle* h, unsigned st)
{
    if (st & kStatusNaN)
    {
        return set_error(h, NBX_ERR_INVALID_INPUT, "coordinates contain NaN");
    }
    if (st & kStatusWrapLimit)
    {
        return set_error(h, NBX_ERR_INVALID_INPUT, "a coordinate is more than 127 box lengths outside the box");
    }
    if (st & (kStatusListOverflow | kStatusExclOverflow | kStatusGridOverflow | kStatusEntryOverflow
              | kStatusRecordOverflow))
    {
        return set_error(h, NBX_ERR_LIST_OVERFLOW, "pair list or grid capacity exceeded");
    }
    if (st & kStatusTimeout)
    {
        return set_error(h, NBX_ERR_TIMEOUT, "a device-side wait timed out");
    }
    return NBX_OK;
}

int read_header(nbx_handle* h)
{
    cudaError_t e = cudaMemcpyAsync(h->h_hdr, h->v.hdr, sizeof(ListHeader), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess)
    {
        e = cudaStreamSynchronize(h->stream);
    }
    return cuda_check(h, e, "read list header");
}

// (Re)allocates the list arrays to hold num_sci / num_cj4 entries with headroom.
int ensure_list_capacity(nbx_handle* h, int num_sci, int num_cj4)
{
    DeviceView& v    = h->v;
    const int   need_cj4 = num_cj4 + num_cj4 / 4 + 256;
    // balancing splits entries into at most one piece per cj4 group
    const int   need_sci = num_sci + num_sci / 4 + 64 + need_cj4;
    if (v.sci && v.sci_cap >= num_sci + num_cj4 && v.cj4_cap >= num_cj4)
    {
        return NBX_OK;
    }
    dfree(h, v.sci);
    dfree(h, v.sci_tmp);
    dfree(h, v.sci_pieces);
    dfree(h, v.cj4);
    dfree(h, v.excl);
    dfree(h, v.imask_outer);
    dfree(h, v.grp_pairs);
    v.sci = nullptr;
    v.sci_tmp = nullptr;
    v.sci_pieces = nullptr;
    v.cj4 = nullptr;
    v.excl = nullptr;
    v.imask_outer = nullptr;
    v.grp_pairs   = nullptr;
    v.sci_cap  = need_sci;
    v.cj4_cap  = need_cj4;
    v.excl_cap = 2 * need_cj4 + 1;  // at most one mask per cj4 half
    cudaError_t e = dalloc(h, &v.sci, v.sci_cap);
    if (e == cudaSuccess) e = dalloc(h, &v.sci_tmp, v.sci_cap);
    if (e == cudaSuccess) e = dalloc(h, &v.sci_pieces, (size_t)v.sci_cap + 1);
    if (e == cudaSuccess) e = dalloc(h, &v.cj4, v.cj4_cap);
    if (e == cudaSuccess) e = dalloc(h, &v.excl, v.excl_cap);
    if (e == cudaSuccess) e = dalloc(h, &v.imask_outer, 2 * (size_t)v.cj4_cap);
    if (e == cudaSuccess) e = dalloc(h, &v.grp_pairs, (size_t)v.cj4_cap);
    if (e != cudaSuccess)
    {
        return cuda_check(h, e, "list allocation");
    }
    // exclusion entry 0: all pairs interacting
    e = cudaMemsetAsync(v.excl, 0xff, sizeof(Excl), h->stream);
    ListHeader caps{};
    caps.sci_capacity  = v.sci_cap;
    caps.cj4_capacity  = v.cj4_cap;
    caps.excl_capacity = v.excl_cap;
    if (e == cudaSuccess)
    {
        e = cudaMemcpyAsync(&v.hdr->sci_capacity, &caps.sci_capacity, 3 * sizeof(int), cudaMemcpyHostToDevice,
                            h->stream);
    }
    if (e == cudaSuccess)
    {
        e = cudaStreamSynchronize(h->stream);
    }
    return cuda_check(h, e, "list capacity");
}

cudaEvent_t take_event(nbx_handle* h)
{
    cudaEvent_t ev;
    if (!h->ev_pool.empty())
    {
        ev = h->ev_pool.back();
        h->ev_pool.pop_back();
    }
    else
    {
        cudaEventCreate(&ev);
    }
    return ev;
}

// Events around a group of launches on the handle's stream when timing is on.
struct PhaseTimer
{
    nbx_handle* h;
    int         phase;
    cudaEvent_t a = nullptr, b = nullptr;
    PhaseTimer(nbx_handle* hh, int ph) : h(hh), phase(ph)
    {
        if (h->timing)
        {
            a = take_event(h);
            b = take_event(h);
            cudaEventRecord(a, h->stream);
        }
    }
    void stop()
    {
        if (a)
        {
            cudaEventRecord(b, h->stream);
            h->ev_pending.push_back({ a, b, phase });
            a = nullptr;
        }
    }
    ~PhaseTimer() { stop(); }
};

// Search records per cell allocated up front (a water cell at rlist 1 nm finds about 150 j-clusters);
// a cell that finds more makes the host grow them and count again.
constexpr int kInitialRecordsPerCell = 512;

// (Re)allocates the per-cell search records (j-cluster index and i-cluster mask) for per_cell
// records in every cell of the grid.
cudaError_t alloc_search_records(nbx_handle* h, int per_cell)
{
    DeviceView& v = h->v;
    dfree(h, v.rec_cj);
    dfree(h, v.rec_m);
    v.rec_cj  = nullptr;
    v.rec_m   = nullptr;
    v.rec_cap = per_cell;
    const size_t n = (size_t)v.g.cells_capacity * per_cell;
    cudaError_t  e = dalloc(h, &v.rec_cj, n);
    if (e == cudaSuccess) e = dalloc(h, &v.rec_m, n);
    return e;
}

// Grid + count (and the prefix sum of the counts) of a search, without host synchronisation.
cudaError_t search_launch_count(nbx_handle* h, float* d_x, int write_back)
{
    DeviceView& v = h->v;
    cudaError_t e = cudaMemsetAsync(&v.hdr->status, 0, sizeof(unsigned), h->stream);
    {
        PhaseTimer t(h, 1);
        if (e == cudaSuccess) e = launch_grid(v, d_x, write_back, h->stream);
    }
    {
        PhaseTimer t(h, 2);
        if (e == cudaSuccess) e = launch_search_count(v, h->stream);
    }
    h->launches += 7;  // 5 grid kernels, count, scan
    return e;
}

// With the count pass's list header on the host (h_hdr): its status, the record regrowth (counting
// again, synchronously) and the list capacity; then the write pass, balancing and the fresh prune,
// without host synchronisation.
int search_launch_write(nbx_handle* h)
{
    DeviceView& v  = h->v;
    unsigned    st = h->h_hdr->status & ~(unsigned)(kStatusListOverflow | kStatusRecordOverflow);
    int         rc = status_to_error(h, st);
    if (rc != NBX_OK)
    {
        return rc;
    }
    cudaError_t e = cudaSuccess;
    if (h->h_hdr->status & kStatusRecordOverflow)
    {
        // a cell found more j-clusters than its records hold: grow them and count again
        const int need = h->h_hdr->rec_need;
        e = alloc_search_records(h, need + need / 4 + 64);
        if (e == cudaSuccess) e = cudaMemsetAsync(&v.hdr->status, 0, sizeof(unsigned), h->stream);
        if (e == cudaSuccess) e = launch_search_count(v, h->stream);
        h->launches += 2;
        if ((rc = cuda_check(h, e, "search count")) != NBX_OK || (rc = read_header(h)) != NBX_OK)
        {
            return rc;
        }
        st = h->h_hdr->status & ~(unsigned)kStatusListOverflow;
        if ((rc = status_to_error(h, st)) != NBX_OK)
        {
            return rc;
        }
    }
    if ((rc = ensure_list_capacity(h, h->h_hdr->num_sci, h->h_hdr->num_cj4)) != NBX_OK)
    {
        return rc;
    }
    // counts are unchanged; clear the overflow flag the count pass may have set
    e = cudaMemsetAsync(&v.hdr->status, 0, sizeof(unsigned), h->stream);
    {
        PhaseTimer t(h, 3);
        if (e == cudaSuccess) e = launch_search_write(v, h->h_hdr->num_sci, h->stream);
        // split long entries and order them large-first (the GPU list's load balancing)
        if (e == cudaSuccess) e = launch_balance(v, h->min_ci_balanced, h->stream);
    }
    if (e == cudaSuccess && h->use_prune)
    {
        PhaseTimer t(h, 4);
        e = launch_prune(v, 1, 0, 1, h->stream);
    }
    h->launches += 5 + (h->use_prune ? 1 : 0);  // emit, 4 balancing kernels, prune
    return cuda_check(h, e, "search write");
}

// With the write pass's list header on the host: its status; the list is in place.
int search_finish(nbx_handle* h)
{
    const int rc = status_to_error(h, h->h_hdr->status);
    if (rc != NBX_OK)
    {
        return rc;
    }
    h->have_list  = true;
    h->prune_part = 0;
    return NBX_OK;
}

// Grid + count, size the list, write, prune: the synchronous search.
int search_sync(nbx_handle* h, float* d_x, int write_back)
{
    int rc = cuda_check(h, search_launch_count(h, d_x, write_back), "grid/search count");
    if (rc == NBX_OK) rc = read_header(h);
    if (rc == NBX_OK) rc = search_launch_write(h);
    if (rc == NBX_OK) rc = read_header(h);
    return rc == NBX_OK ? search_finish(h) : rc;
}

// Accumulates the finished event pairs into their phases.
void collect_timings(nbx_handle* h, bool wait)
{
    std::vector<nbx_handle::PendingEvents> keep;
    for (auto& p : h->ev_pending)
    {
        if (wait)
        {
            cudaEventSynchronize(p.b);
        }
        if (cudaEventQuery(p.b) == cudaSuccess)
        {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, p.a, p.b);
            h->phase_ms[p.phase] += ms;
            h->phase_count[p.phase] += 1;
            h->ev_pool.push_back(p.a);
            h->ev_pool.push_back(p.b);
        }
        else
        {
            keep.push_back(p);
        }
    }
    cudaGetLastError();
    h->ev_pending.swap(keep);
}

int compute_async(nbx_handle* h, const float* d_x, float* d_f, double* d_e, double* d_vir)
{
    DeviceView& v      = h->v;
    const bool  energy = (d_e != nullptr) || (d_vir != nullptr);
    cudaError_t e      = launch_convert_x(v, d_x, h->stream, true, h->x_host);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (h->timing)
    {
        e0 = take_event(h);
        e1 = take_event(h);
    }
    // the events bracket the force kernel alone
    if (e == cudaSuccess) e = launch_force(v, energy, h->stream, h->num_sms, e0, e1);
    if (e == cudaSuccess && h->fep_on) e = launch_fep(v, h->fep, energy, h->stream);
    if (h->timing)
    {
        h->ev_pending.push_back({ e0, e1, 0 });
        if (h->ev_pending.size() > 256)
        {
            collect_timings(h, false);
        }
    }
    if (e == cudaSuccess) e = launch_reduce_f(v, d_f, d_e, d_vir, h->stream, h->f_host);
    h->force_launches += 1;
    h->launches += 3 + (v.vdw_mod == NBX_VDW_LJPME && energy ? 1 : 0) + (h->fep_on ? 1 : 0);
    return cuda_check(h, e, "compute");
}

// The device address of a host array the GPU can access directly (pinned memory mapped
// into the device's address space, e.g. cudaHostAlloc / cudaMallocHost under unified
// addressing), or nullptr: then the array is staged by copies.  Kernels then read the
// coordinates from and write the forces to host memory over the host link, overlapping
// the transfer with the kernels that use it.
void* mapped_device_ptr(const void* p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer) ? a.devicePointer : nullptr;
}

bool valid_box(const float* box)
{
    for (int d = 0; d < 3; d++)
    {
        if (!(box[d] > 0.0f) || !std::isfinite(box[d]))
        {
            return false;
        }
    }
    return true;
}

} // namespace

namespace
{

// lambda factors of nb_free_energy.cpp:356-388 (sc-r-power 6)
void set_fep_lambda(FepView& f, float lam_c, float lam_v, int power)
{
    const float lfc[2] = { 1.0f - lam_c, lam_c }, lfv[2] = { 1.0f - lam_v, lam_v }, dlf[2] = { -1.0f, 1.0f };
    for (int i = 0; i < 2; i++)
    {
        f.lfc[i]     = lfc[i];
        f.lfv[i]     = lfv[i];
        f.lfac_c[i]  = power == 2 ? (1 - lfc[i]) * (1 - lfc[i]) : (1 - lfc[i]);
        f.dlfac_c[i] = dlf[i] * power / 6.0f * (power == 2 ? (1 - lfc[i]) : 1.0f);
        f.lfac_v[i]  = power == 2 ? (1 - lfv[i]) * (1 - lfv[i]) : (1 - lfv[i]);
        f.dlfac_v[i] = dlf[i] * power / 6.0f * (power == 2 ? (1 - lfv[i]) : 1.0f);
    }
}

double self_energy_of(const DeviceView& v, const std::vector<float>& q)
{
    double qsq = 0.0;
    for (float c : q)
    {
        qsq += (double)c * (double)c;
    }
    return v.coulomb == NBX_COULOMB_EWALD ? -v.epsfac_d * (double)v.beta * 0.56418958354775628695 * qsq
                                          : -v.epsfac_d * 0.5 * (double)v.c_rf * qsq;
}

int fep_restore(nbx_handle* h)
{
    DeviceView& v = h->v;
    const int   n = h->n;
    cudaError_t e = cudaMemcpyAsync(const_cast<float*>(v.q), h->d_fep_q, sizeof(float) * n, cudaMemcpyDeviceToDevice,
                                    h->stream);
    if (e == cudaSuccess)
    {
        e = cudaMemcpyAsync(const_cast<int*>(v.type), h->d_fep_t, sizeof(int) * n, cudaMemcpyDeviceToDevice,
                            h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    v.self_energy = h->self_energy_all;
    h->fep_on     = false;
    h->have_list  = false;
    return cuda_check(h, e, "free-energy restore");
}

} // namespace

extern "C" {

void nbx_default_options(nbx_options* o)
{
    std::memset(o, 0, sizeof(*o));
    o->coulomb         = NBX_COULOMB_EWALD;
    o->rcoulomb        = 1.0f;
    o->rlist           = 1.0f;
    o->rlist_inner     = 0.0f;
    o->ewald_rtol      = 1e-5f;
    o->epsilon_rf      = 1.0f;
    o->use_ewald_shift = 0;
    o->nstlist         = 10;
    o->nstlist_prune   = 0;
    o->compute_energy  = 0;
    o->vdw_modifier    = NBX_VDW_POTSHIFT;
    o->rvdw_switch     = 0.0f;
    o->ewald_rtol_lj   = 1e-3f;
}

const char* nbx_last_error(const nbx_handle* h)
{
    return h ? h->err.c_str() : g_create_error.c_str();
}

int nbx_create(const nbx_system_desc* sys, const nbx_options* opts_in, int device, nbx_handle** out)
{
    if (!sys || !out)
    {
        return set_error(nullptr, NBX_ERR_INVALID_INPUT, "null argument");
    }
    *out = nullptr;
    nbx_options opts;
    if (opts_in)
    {
        opts = *opts_in;
    }
    else
    {
        nbx_default_options(&opts);
    }
    const int n = sys->num_atoms;
    if (n <= 0 || !sys->x || !sys->q || !sys->type || !sys->nbfp || !sys->excl_index || sys->num_types <= 0)
    {
        return set_error(nullptr, NBX_ERR_INVALID_INPUT, "empty system or missing arrays");
    }
    if (!valid_box(sys->box))
    {
        return set_error(nullptr, NBX_ERR_INVALID_INPUT, "box edges must be positive and finite");
    }
    if (!(opts.rcoulomb > 0.0f) || !(opts.rlist >= opts.rcoulomb))
    {
        return set_error(nullptr, NBX_ERR_INVALID_INPUT, "need 0 < rcoulomb <= rlist");
    }
    if (opts.coulomb < 0 || opts.coulomb > 2)
    {
        return set_error(nullptr, NBX_ERR_INVALID_INPUT, "unknown Coulomb type");
    }
    if (opts.vdw_modifier < 0 || opts.vdw_modifier > NBX_VDW_LJPME)
    {
        return set_error(nullptr, NBX_ERR_INVALID_INPUT, "unknown LJ modifier");
    }
    if ((opts.vdw_modifier == NBX_VDW_FORCESWITCH || opts.vdw_modifier == NBX_VDW_POTSWITCH)
        && !(opts.rvdw_switch >= 0.0f && opts.rvdw_switch < opts.rcoulomb))
    {
        return set_error(nullptr, NBX_ERR_INVALID_INPUT, "the switch modifiers need 0 <= rvdw_switch < rc");
    }
    if (sys->num_types + 1 > 48)
    {
        return set_error(nullptr, NBX_ERR_INVALID_INPUT, "at most 47 particle types");
    }
    if (opts.coulomb == NBX_COULOMB_EWALD
        && (double)calc_ewaldcoeff_q(opts.rcoulomb, opts.ewald_rtol > 0.0f ? opts.ewald_rtol : 1e-5f)
                           * (double)opts.rcoulomb
                   > (double)kErfcXMax)
    {
        return set_error(nullptr, NBX_ERR_INVALID_INPUT,
                         "ewald_rtol below erfc(4) = 1.5e-8 is not supported (beta * rc must be <= 4)");
    }
    for (int i = 0; i < 3 * n; i++)
    {
        if (!std::isfinite(sys->x[i]))
        {
            return set_error(nullptr, NBX_ERR_INVALID_INPUT, "input coordinates have at least one NaN");
        }
    }
    for (int i = 0; i < n; i++)
    {
        if (sys->type[i] < 0 || sys->type[i] >= sys->num_types)
        {
            return set_error(nullptr, NBX_ERR_INVALID_INPUT, "particle type out of range");
        }
    }
    if (sys->excl_index[0] != 0)
    {
        return set_error(nullptr, NBX_ERR_INVALID_INPUT, "exclusion offsets must start at 0");
    }
    for (int i = 0; i < n; i++)
    {
        if (sys->excl_index[i + 1] < sys->excl_index[i])
        {
            return set_error(nullptr, NBX_ERR_INVALID_INPUT, "exclusion offsets must be non-decreasing");
        }
        for (int k = sys->excl_index[i]; k < sys->excl_index[i + 1]; k++)
        {
            if (sys->excl_list[k] < 0 || sys->excl_list[k] >= n)
            {
                return set_error(nullptr, NBX_ERR_INVALID_INPUT, "excluded atom index out of range");
            }
        }
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    {
        cudaGetLastError();
        return set_error(nullptr, NBX_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= ndev)
    {
        return set_error(nullptr, NBX_ERR_INVALID_INPUT, "device index out of range");
    }

    nbx_handle* h = new nbx_handle();
    h->device     = device;
    h->opts       = opts;
    h->n          = n;
    h->ntypes     = sys->num_types;
    cudaSetDevice(device);
    cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device);
    // gpu_min_ci_balanced (cuda/nbnxm_cuda_data_mgmt.cu:93,545-548): 44 entries per SM
    h->min_ci_balanced = 44 * h->num_sms;
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    h->own_stream = true;
    DeviceView& v = h->v;
    v.n           = n;

    // ---- interaction constants (gmxsetup.cpp:226-284) ----
    const float rc = opts.rcoulomb;
    v.coulomb      = opts.coulomb;
    v.rc2          = rc * rc;
    v.rlist        = opts.rlist;
    v.rlist2       = opts.rlist * opts.rlist;
    const float rin = (opts.rlist_inner > 0.0f) ? opts.rlist_inner : opts.rlist;
    v.rlist_inner2 = rin * rin;
    v.epsfac       = (float)one_4pi_eps0();
    v.epsfac_d     = one_4pi_eps0();
    set_lj_modifier(v, opts.vdw_modifier, rc, opts.rvdw_switch);
    if (opts.vdw_modifier == NBX_VDW_LJPME)
    {
        // LJ-PME real space: the potential-shift constants of the plain part plus the grid terms
        // (forcerec.cpp:703-716, kernel_ref_outer.h:182-189); the self energy of the grid part
        // sum_i 0.5 (6 C6_ii) / 6 beta^6 / 6 (kernel_ref_outer.h:307-313)
        set_lj_modifier(v, NBX_VDW_POTSHIFT, rc, 0.0f);
        v.vdw_mod         = NBX_VDW_LJPME;
        const float bl    = nbx_ewald_coefficient_lj(rc, opts.ewald_rtol_lj);
        const float crc2  = (bl * rc) * (bl * rc);
        v.lje_coeff2      = bl * bl;
        v.lje_coeff6_6    = v.lje_coeff2 * v.lje_coeff2 * v.lje_coeff2 / 6.0f;
        v.sh_lj_ewald     = (std::exp(-crc2) * (1 + crc2 + 0.5f * crc2 * crc2) - 1) / (rc * rc * rc * rc * rc * rc);
        double self_lj    = 0.0;
        const int nt      = sys->num_types;
        for (int i = 0; i < n; i++)
        {
            const int t = sys->type[i];
            self_lj += 0.5 * (double)sys->nbfp[2 * (t * nt + t)] / 6.0 * (double)v.lje_coeff6_6;
        }
        v.self_energy_lj = self_lj;
    }
    const float eps_rf = (opts.coulomb == NBX_COULOMB_CUTOFF) ? 1.0f : opts.epsilon_rf;
    v.k_rf = (eps_rf == 0) ? 1 / (2 * rc * rc * rc) : (eps_rf - 1.0f) / (2 * eps_rf + 1.0f) / (rc * rc * rc);
    v.c_rf = 1 / rc + v.k_rf * rc * rc;
    double qsq = 0.0;
    for (int i = 0; i < n; i++)
    {
        qsq += (double)sys->q[i] * (double)sys->q[i];
    }
    if (opts.coulomb == NBX_COULOMB_EWALD)
    {
        const float rtol = opts.ewald_rtol > 0.0f ? opts.ewald_rtol : 1e-5f;
        v.beta           = calc_ewaldcoeff_q(rc, rtol);
        v.sh_ewald       = opts.use_ewald_shift ? erfcf(v.beta * rc) / rc : 0.0f;
        // Ewald self energy, kernel_gpu_ref.cpp:154-178
        v.self_energy = -v.epsfac_d * (double)v.beta * 0.56418958354775628695 * qsq;
        v.erfc_p = kErfcP;
    }
    else
    {
        v.beta        = 0.0f;
        v.sh_ewald    = 0.0f;
        v.self_energy = -v.epsfac_d * 0.5 * (double)v.c_rf * qsq;
    }
    set_pair_constants(v);
    v.pair_core    = 1;
    v.stage_depth  = 2;
    v.force_blocks = 2;
    // ---- shift vectors (pbc.cpp:1187-1202), rectangular box ----
    for (int s = 0, m = -1; m <= 1; m++)
    {
        for (int l = -1; l <= 1; l++)
        {
            for (int k = -2; k <= 2; k++, s++)
            {
                v.shiftvec[3 * s + 0] = k * sys->box[0];
                v.shiftvec[3 * s + 1] = l * sys->box[1];
                v.shiftvec[3 * s + 2] = m * sys->box[2];
            }
        }
    }
    // ---- grid dimensions (grid.cpp:103-262, GPU geometry; gmxcalculator.cpp:97) ----
    GridDims& g = v.g;
    for (int d = 0; d < 3; d++)
    {
        g.box[d] = sys->box[d];
    }
    const float det     = sys->box[0] * (sys->box[1] * sys->box[2]);
    const float density = (float)n / det;
    if (n > kSc)
    {
        const float tlen = cbrtf((float)kCl / density);
        g.ncx            = std::max(1, (int)(sys->box[0] / (tlen * 2)));
        g.ncy            = std::max(1, (int)(sys->box[1] / (tlen * 2)));
    }
    else
    {
        g.ncx = g.ncy = 1;
    }
    g.cs[0]          = sys->box[0] / g.ncx;
    g.cs[1]          = sys->box[1] / g.ncy;
    g.ics[0]         = 1 / g.cs[0];
    g.ics[1]         = 1 / g.cs[1];
    g.ncol           = g.ncx * g.ncy;
    g.cells_capacity = n / kSc + g.ncol;
    // ---- bounding-box-only distance (pairlist.cpp:2841-2878) ----
    {
        float  bbx = (float)(0.5 * (g.cs[0] + g.cs[0]));
        float  bby = (float)(0.5 * (g.cs[1] + g.cs[1]));
        bbx /= 2;
        bby /= 2;
        double r    = (double)opts.rlist - 0.5 * (double)sqrtf(bbx * bbx + bby * bby);
        float  rbb  = (float)(r > 0.0 ? r : 0.0);
        v.rbb2      = rbb * rbb;
    }
    // ---- nbfp with the dummy type (atomdata.cpp:498-530) ----
    const int         nt1 = sys->num_types + 1;
    v.ntypes1         = nt1;
    std::vector<float2> nbfp((size_t)nt1 * nt1, make_float2(0.0f, 0.0f));
    for (int i = 0; i < sys->num_types; i++)
    {
        for (int j = 0; j < sys->num_types; j++)
        {
            nbfp[i * nt1 + j] = make_float2(sys->nbfp[(i * sys->num_types + j) * 2],
                                            sys->nbfp[(i * sys->num_types + j) * 2 + 1]);
        }
    }

    // ---- device memory ----
    const size_t npad = (size_t)g.cells_capacity * kSc;
    const int    nexcl = sys->excl_index[n];
    float*  q = nullptr;
    int*    t = nullptr;
    int*    ei = nullptr;
    int*    el = nullptr;
    float2* nb = nullptr;
    if (e == cudaSuccess) e = dalloc(h, &q, n);
    if (e == cudaSuccess) e = dalloc(h, &t, n);
    if (e == cudaSuccess) e = dalloc(h, &ei, n + 1);
    if (e == cudaSuccess) e = dalloc(h, &el, nexcl + 1);
    if (e == cudaSuccess) e = dalloc(h, &nb, (size_t)nt1 * nt1);
    if (e == cudaSuccess) e = dalloc(h, &v.xin, 3 * (size_t)n);
    if (e == cudaSuccess) e = dalloc(h, &v.col, n);
    if (e == cudaSuccess) e = dalloc(h, &v.slot, n);
    if (e == cudaSuccess) e = dalloc(h, &v.image, n);
    if (e == cudaSuccess) e = dalloc(h, &v.cxy_na, g.ncol + 1);
    if (e == cudaSuccess) e = dalloc(h, &v.cxy_ind, g.ncol + 2);
    if (e == cudaSuccess) e = dalloc(h, &v.atom_indices, npad);
    if (e == cudaSuccess) e = dalloc(h, &v.cells, n);
    if (e == cudaSuccess) e = dalloc(h, &v.xq, npad);
    if (e == cudaSuccess) e = dalloc(h, &v.tgrid, npad);
    if (e == cudaSuccess) e = dalloc(h, &v.xqp, 5 * npad);
    if (e == cudaSuccess) e = dalloc(h, &v.bb, (size_t)g.cells_capacity * kNcl * 2);
    if (e == cudaSuccess) e = dalloc(h, &v.bbcz, g.cells_capacity);
    if (e == cudaSuccess) e = dalloc(h, &v.nclusters, g.cells_capacity);
    if (e == cudaSuccess) e = dalloc(h, &v.sci_count, g.cells_capacity + 1);
    if (e == cudaSuccess) e = dalloc(h, &v.cj4_count, g.cells_capacity + 1);
    if (e == cudaSuccess) e = dalloc(h, &v.sci_offset, g.cells_capacity + 1);
    if (e == cudaSuccess) e = dalloc(h, &v.cj4_offset, g.cells_capacity + 1);
    if (e == cudaSuccess) e = dalloc(h, &v.rec_ent, (size_t)g.cells_capacity * kMaxEntriesPerCell);
    if (e == cudaSuccess) e = alloc_search_records(h, kInitialRecordsPerCell);
    if (e == cudaSuccess) e = dalloc(h, &v.fnb, npad);
    if (e == cudaSuccess) e = dalloc(h, &v.energy, 2);
    if (e == cudaSuccess) e = dalloc(h, &v.fshift, kNShift * 3);
    if (e == cudaSuccess) e = dalloc(h, &v.virial, 9);
    if (e == cudaSuccess) e = dalloc(h, &v.hdr, 1);
    if (e == cudaSuccess) e = dalloc(h, &h->d_x, 3 * (size_t)n);
    if (e == cudaSuccess) e = dalloc(h, &h->d_f, 3 * (size_t)n);
    if (e == cudaSuccess) e = dalloc(h, &h->d_out, 11);
    if (e == cudaSuccess) e = dalloc(h, &h->d_count, 1);
    if (e == cudaSuccess) e = cudaMallocHost(&h->h_hdr, sizeof(ListHeader));
    if (e == cudaSuccess) e = cudaMallocHost(&h->h_out, 11 * sizeof(double));
    if (e == cudaSuccess) h->d_hout = static_cast<double*>(mapped_device_ptr(h->h_out));
    if (e == cudaSuccess) e = cudaMemcpyAsync(q, sys->q, sizeof(float) * n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t, sys->type, sizeof(int) * n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ei, sys->excl_index, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && nexcl > 0) e = cudaMemcpyAsync(el, sys->excl_list, sizeof(int) * nexcl, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(nb, nbfp.data(), sizeof(float2) * nbfp.size(), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(v.hdr, 0, sizeof(ListHeader), h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->d_x, sys->x, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    v.q          = q;
    v.type       = t;
    v.excl_index = ei;
    v.excl_list  = el;
    v.nbfp       = nb;
    int rc_ = cuda_check(h, e, "nbx_create");
    if (rc_ == NBX_OK)
    {
        h->use_prune = opts.nstlist_prune > 0;
        h->nparts    = h->use_prune ? std::max(1, opts.nstlist_prune / 2) : 1;
        // SimulationState wraps the coordinates once (simulationstate.cpp:88), then the list is built
        rc_ = search_sync(h, h->d_x, 0);
    }
    if (rc_ != NBX_OK)
    {
        g_create_error = h->err;
        nbx_destroy(h);
        return rc_;
    }
    *out = h;
    return NBX_OK;
}

int nbx_destroy(nbx_handle* h)
{
    if (!h)
    {
        return NBX_OK;
    }
    cudaSetDevice(h->device);
    if (h->stream)
    {
        cudaStreamSynchronize(h->stream);
    }
    for (void* p : h->allocations)
    {
        cudaFree(p);
    }
    if (h->h_hdr)
    {
        cudaFreeHost(h->h_hdr);
        cudaFreeHost(h->h_out);
    }
    for (auto& p : h->ev_pending)
    {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (auto ev : h->ev_pool)
    {
        cudaEventDestroy(ev);
    }
    if (h->own_stream && h->stream)
    {
        cudaStreamDestroy(h->stream);
    }
    delete h;
    return NBX_OK;
}

int nbx_set_stream(nbx_handle* h, void* s)
{
    if (!h)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (static_cast<cudaStream_t>(s) == h->stream)
    {
        return NBX_OK;
    }
    cudaSetDevice(h->device);
    // work queued on the previous stream finishes before the new one is used -- unless the new
    // stream is being captured into a CUDA graph, where a host synchronisation is not allowed and
    // the capturing code orders the streams itself (a capture starts after the work before it)
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(static_cast<cudaStream_t>(s), &capture) != cudaSuccess)
    {
        cudaGetLastError();
        capture = cudaStreamCaptureStatusNone;
    }
    if (capture == cudaStreamCaptureStatusNone)
    {
        cudaStreamSynchronize(h->stream);
    }
    if (h->own_stream)
    {
        cudaStreamDestroy(h->stream);
    }
    h->stream     = static_cast<cudaStream_t>(s);
    h->own_stream = false;
    return NBX_OK;
}

void* nbx_get_stream(nbx_handle* h)
{
    return h ? static_cast<void*>(h->stream) : nullptr;
}

int nbx_update_pairlist(nbx_handle* h, const float* x)
{
    if (!h || !x)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(h->device);
    cudaError_t e = cudaMemcpyAsync(h->d_x, x, sizeof(float) * 3 * h->n, cudaMemcpyHostToDevice, h->stream);
    int         rc = cuda_check(h, e, "nbx_update_pairlist");
    return rc != NBX_OK ? rc : search_sync(h, h->d_x, 0);
}

int nbx_compute(nbx_handle* h, const float* x, float* f, double* energies, double* virial)
{
    if (!h || !x || !f)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (!h->have_list)
    {
        return set_error(h, NBX_ERR_STATE, "no pair list");
    }
    cudaSetDevice(h->device);
    const size_t bytes = sizeof(float) * 3 * h->n;
    // mapped pinned arrays are read / written by the kernels in place; others are copied
    const float* d_x = static_cast<const float*>(mapped_device_ptr(x));
    float*       d_f = static_cast<float*>(mapped_device_ptr(f));
    if (!d_x)
    {
        const int rc = cuda_check(h, cudaMemcpyAsync(h->d_x, x, bytes, cudaMemcpyHostToDevice, h->stream),
                                  "nbx_compute H2D");
        if (rc != NBX_OK)
        {
            return rc;
        }
        d_x = h->d_x;
    }
    // host arrays: forces are overwritten (GmxForceCalculator::compute), whatever nbx_set_force_accumulate says
    const int accumulate = h->v.accumulate_f;
    h->v.accumulate_f    = 0;
    h->x_host = d_x != h->d_x;
    h->f_host = d_f != nullptr;
    int rc = compute_async(h, d_x, d_f ? d_f : h->d_f, energies ? h->d_out : nullptr, virial ? h->d_out + 2 : nullptr);
    h->v.accumulate_f = accumulate;
    h->x_host = h->f_host = false;
    if (rc != NBX_OK)
    {
        return rc;
    }
    cudaError_t e = d_f ? cudaSuccess : cudaMemcpyAsync(f, h->d_f, bytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && (energies || virial))
    {
        e = cudaMemcpyAsync(h->h_out, h->d_out, 11 * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->h_hdr, h->v.hdr, sizeof(ListHeader), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if ((rc = cuda_check(h, e, "nbx_compute D2H")) != NBX_OK)
    {
        return rc;
    }
    if (energies)
    {
        energies[0] = h->h_out[0];
        energies[1] = h->h_out[1];
    }
    if (virial)
    {
        std::memcpy(virial, h->h_out + 2, 9 * sizeof(double));
    }
    return status_to_error(h, h->h_hdr->status);
}

int nbx_search_device(nbx_handle* h, const float* d_x)
{
    if (!h || !d_x)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(h->device);
    return search_sync(h, const_cast<float*>(d_x), 0);
}

int nbx_prune_device(nbx_handle* h, int part)
{
    if (!h)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (!h->have_list)
    {
        return set_error(h, NBX_ERR_STATE, "no pair list");
    }
    cudaSetDevice(h->device);
    PhaseTimer  t(h, 4);
    cudaError_t e = (part < 0) ? launch_prune(h->v, 1, 0, 1, h->stream)
                               : launch_prune(h->v, 0, part % h->nparts, h->nparts, h->stream);
    t.stop();
    h->launches += 1;
    return cuda_check(h, e, "nbx_prune_device");
}

int nbx_compute_device(nbx_handle* h, const float* d_x, float* d_f, double* d_e, double* d_vir)
{
    if (!h || !d_x || !d_f)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (!h->have_list)
    {
        return set_error(h, NBX_ERR_STATE, "no pair list");
    }
    cudaSetDevice(h->device);
    return compute_async(h, d_x, d_f, d_e, d_vir);
}

int nbx_md_step_device(nbx_handle* h, long long step, const float* d_x, float* d_f, double* d_e, double* d_vir)
{
    if (!h || !d_x || !d_f)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(h->device);
    const int nstlist = std::max(1, h->opts.nstlist);
    int       rc      = NBX_OK;
    if (!h->have_list || step % nstlist == 0)
    {
        // the search grids the atoms put in the box (mdlib/sim_util.cpp:1316); their
        // box shifts are kept for the coordinate conversion until the next search
        rc = search_sync(h, const_cast<float*>(d_x), 0);
        h->list_step = step;
        if (rc != NBX_OK)
        {
            return rc;
        }
    }
    else if (h->use_prune)
    {
        // isDynamicPruningStepGpu (pairlistsets.h:106-114): every second list age, rolling parts
        const long long age = step - h->list_step;
        if (age > 0 && age % 2 == 0)
        {
            PhaseTimer  t(h, 4);
            cudaError_t e = launch_prune(h->v, 0, h->prune_part, h->nparts, h->stream);
            t.stop();
            h->prune_part = (h->prune_part + 1) % h->nparts;
            h->launches += 1;
            if ((rc = cuda_check(h, e, "rolling prune")) != NBX_OK)
            {
                return rc;
            }
        }
    }
    return compute_async(h, d_x, d_f, d_e, d_vir);
}

int nbx_md_step(nbx_handle* h, long long step, const float* x, float* f, double* energies, double* virial)
{
    if (!h || !x || !f)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(h->device);
    const size_t bytes = sizeof(float) * 3 * h->n;
    // mapped pinned arrays are read / written by the kernels in place, except the
    // coordinates of a search step (the gridding passes read them several times)
    const bool   search = !h->have_list || step % std::max(1, h->opts.nstlist) == 0;
    const float* d_x    = search ? nullptr : static_cast<const float*>(mapped_device_ptr(x));
    float*       d_f    = static_cast<float*>(mapped_device_ptr(f));
    if (!d_x)
    {
        const int rc = cuda_check(h, cudaMemcpyAsync(h->d_x, x, bytes, cudaMemcpyHostToDevice, h->stream),
                                  "nbx_md_step H2D");
        if (rc != NBX_OK)
        {
            return rc;
        }
        d_x = h->d_x;
    }
    const int accumulate = h->v.accumulate_f;  // host arrays: forces are overwritten
    h->v.accumulate_f    = 0;
    // energies and virial: written by the finishing kernel into the pinned h_out when the
    // device can address it, else copied there
    double* d_out = h->d_hout ? h->d_hout : h->d_out;
    h->x_host     = d_x != h->d_x;
    h->f_host     = d_f != nullptr;
    int     rc    = nbx_md_step_device(h, step, d_x, d_f ? d_f : h->d_f, energies ? d_out : nullptr,
                                       virial ? d_out + 2 : nullptr);
    h->v.accumulate_f = accumulate;
    h->x_host = h->f_host = false;
    if (rc != NBX_OK)
    {
        return rc;
    }
    cudaError_t e = d_f ? cudaSuccess : cudaMemcpyAsync(f, h->d_f, bytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && (energies || virial) && !h->d_hout)
    {
        e = cudaMemcpyAsync(h->h_out, h->d_out, 11 * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if ((rc = cuda_check(h, e, "nbx_md_step D2H")) != NBX_OK)
    {
        return rc;
    }
    if (energies)
    {
        energies[0] = h->h_out[0];
        energies[1] = h->h_out[1];
    }
    if (virial)
    {
        std::memcpy(virial, h->h_out + 2, 9 * sizeof(double));
    }
    return NBX_OK;
}

int nbx_backward_device(nbx_handle* h, const float* d_x, const float* d_gF, const double* d_gE, float* d_gx,
                        float* d_gq, double* d_gnbfp)
{
    if (!h || !d_x || !d_gF)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (!h->have_list)
    {
        return set_error(h, NBX_ERR_STATE, "no pair list");
    }
    if (h->fep_on)
    {
        return set_error(h, NBX_ERR_INVALID_INPUT, "the adjoint does not cover perturbed atoms");
    }
    if (h->v.ntypes1 > adjoint_max_types1())
    {
        return set_error(h, NBX_ERR_INVALID_INPUT, "the adjoint supports at most 15 particle types");
    }
    if (h->v.vdw_mod == NBX_VDW_FORCESWITCH || h->v.vdw_mod == NBX_VDW_POTSWITCH || h->v.vdw_mod == NBX_VDW_LJPME)
    {
        return set_error(h, NBX_ERR_INVALID_INPUT, "the adjoint takes the potential-shift or plain LJ cut-off");
    }
    cudaSetDevice(h->device);
    DeviceView& v = h->v;
    cudaError_t e = cudaSuccess;
    if (!h->d_gnb)
    {
        const size_t slots = (size_t)v.g.cells_capacity * kSc;
        e = dalloc(h, &h->d_gnb, slots);
        if (e == cudaSuccess) e = dalloc(h, &h->d_dnb, slots);
        if (e == cudaSuccess) e = dalloc(h, &h->d_gnbfp, 2 * (size_t)v.ntypes1 * v.ntypes1);
        if (e == cudaSuccess) e = dalloc(h, &h->d_adj_counter, 1);
        if (e != cudaSuccess)
        {
            return cuda_check(h, e, "adjoint allocation");
        }
    }
    // the coordinate conversion is part of the preparation kernel
    // (the type-pair gradients are copied out by the finishing kernel)
    e = launch_backward(v, d_x, d_gF, d_gE, h->d_gnb, h->d_dnb, h->d_gnbfp, h->d_adj_counter, d_gx, d_gq, d_gnbfp,
                        h->num_sms, h->stream);
    h->launches += 3;
    return cuda_check(h, e, "nbx_backward_device");
}

int nbx_set_parameters_device(nbx_handle* h, const float* d_q, const float* d_nbfp)
{
    if (!h)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (h->fep_on)
    {
        return set_error(h, NBX_ERR_INVALID_INPUT, "parameters cannot change while perturbed atoms are set");
    }
    cudaSetDevice(h->device);
    if (d_q)
    {
        // the self energy now comes from the charges on the device
        h->v.self_on_device = 1;
        h->v.self_energy    = 0.0;
    }
    cudaError_t e = launch_set_parameters(h->v, d_q, d_nbfp, h->stream);
    h->launches += (d_q ? 1 : 0) + (d_nbfp ? 1 : 0);
    return cuda_check(h, e, "nbx_set_parameters_device");
}

int nbx_lb_table_device(const double* d_sigma, const double* d_epsilon, int ntypes, double* d_table, void* stream)
{
    if (!d_sigma || !d_epsilon || !d_table || ntypes < 1 || ntypes > 64)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    const cudaError_t e = launch_lb_table(d_sigma, d_epsilon, ntypes, d_table, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? NBX_OK : NBX_ERR_CUDA;
}

int nbx_lb_table_backward_device(const double* d_sigma, const double* d_epsilon, int ntypes, const double* d_gtable,
                                 double* d_gsigma, double* d_gepsilon, void* stream)
{
    if (!d_sigma || !d_epsilon || !d_gtable || !d_gsigma || !d_gepsilon || ntypes < 1 || ntypes > 64)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    const cudaError_t e = launch_lb_table_backward(d_sigma, d_epsilon, ntypes, d_gtable, d_gsigma, d_gepsilon,
                                                   static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? NBX_OK : NBX_ERR_CUDA;
}

int nbx_match_loss_device(const float* d_f, const float* d_ftarget, long long n3, float* d_gF, double* d_loss,
                          void* stream)
{
    if (!d_f || !d_ftarget || !d_gF || !d_loss || n3 < 0)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    {
        return NBX_ERR_CUDA;
    }
    const cudaError_t e = launch_match_loss(d_f, d_ftarget, (size_t)n3, d_gF, d_loss, sms, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? NBX_OK : NBX_ERR_CUDA;
}

int nbx_set_force_kernel(nbx_handle* h, int tile, int stage_depth, int blocks_per_sm)
{
    if (!h || tile < 0 || tile > 1 || stage_depth < 2 || stage_depth > 3 || blocks_per_sm < 2 || blocks_per_sm > 3)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    h->v.pair_core    = tile;
    h->v.stage_depth  = stage_depth;
    h->v.force_blocks = blocks_per_sm;
    return NBX_OK;
}

int nbx_get_force_kernel(const nbx_handle* h, int* tile, int* stage_depth, int* blocks_per_sm)
{
    if (!h || !tile || !stage_depth || !blocks_per_sm)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    *tile          = h->v.pair_core;
    *stage_depth   = h->v.stage_depth;
    *blocks_per_sm = h->v.force_blocks;
    return NBX_OK;
}

int nbx_set_wait_test(nbx_handle* h, int enable)
{
    if (!h)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    h->v.wait_test_bytes = enable ? 16u : 0u;
    return NBX_OK;
}

int nbx_fep_enable(nbx_handle* h, const nbx_fep_desc* d)
{
    if (!h || !d || d->num_perturbed < 0 || d->num_perturbed > h->n
        || (d->num_perturbed > 0 && (!d->perturbed || !d->qB || !d->typeB)))
    {
        return h ? set_error(h, NBX_ERR_INVALID_INPUT, "null argument or bad perturbed-atom count")
                 : NBX_ERR_INVALID_INPUT;
    }
    DeviceView& v = h->v;
    if (d->lambda_power != 1 && d->lambda_power != 2)
    {
        return set_error(h, NBX_ERR_INVALID_INPUT, "sc-power must be 1 or 2");
    }
    if (!(d->alpha_vdw >= 0.0f) || !(d->alpha_coul >= 0.0f) || !(d->sigma6_def > 0.0f) || !(d->sigma6_min > 0.0f))
    {
        return set_error(h, NBX_ERR_INVALID_INPUT, "soft-core alpha must be >= 0 and sigma^6 > 0");
    }
    if (v.vdw_mod != NBX_VDW_POTSHIFT && v.vdw_mod != NBX_VDW_NONE)
    {
        return set_error(h, NBX_ERR_INVALID_INPUT, "perturbed atoms take the potential-shift or plain LJ cut-off");
    }
    for (int k = 0; k < 3; k++)
    {
        if (v.g.box[k] < 2.0f * v.rlist)
        {
            return set_error(h, NBX_ERR_INVALID_INPUT, "perturbed atoms need box edges of at least 2 rlist");
        }
    }
    const int          n  = h->n;
    const int          nt = v.ntypes1 - 1;
    std::vector<char>  seen(n, 0);
    for (int k = 0; k < d->num_perturbed; k++)
    {
        const int a = d->perturbed[k];
        if (a < 0 || a >= n || seen[a] || d->typeB[k] < 0 || d->typeB[k] >= nt || !std::isfinite(d->qB[k]))
        {
            return set_error(h, NBX_ERR_INVALID_INPUT, "perturbed atoms: bad or repeated index, type or charge");
        }
        seen[a] = 1;
    }
    cudaSetDevice(h->device);
    if (h->fep_on)
    {
        int rc = fep_restore(h);
        if (rc != NBX_OK)
        {
            return rc;
        }
    }
    cudaError_t e = cudaSuccess;
    if (!h->d_fep_q)
    {
        e = dalloc(h, &h->d_fep_q, 2 * (size_t)n);
        if (e == cudaSuccess) e = dalloc(h, &h->d_fep_t, 2 * (size_t)n);
        if (e == cudaSuccess) e = dalloc(h, &h->d_fep_list, (size_t)n);
        if (e == cudaSuccess) e = dalloc(h, &h->d_fep_pert, (size_t)n);
        if (e == cudaSuccess) e = dalloc(h, &h->d_fep_sums, 4);
        if (e != cudaSuccess)
        {
            return set_error(h, NBX_ERR_OUT_OF_MEMORY, "free-energy buffers");
        }
    }
    // state A = the topology's charges and types (on the device)
    std::vector<float> q(2 * (size_t)n);
    std::vector<int>   t(2 * (size_t)n);
    e = cudaMemcpyAsync(q.data(), v.q, sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t.data(), v.type, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess)
    {
        return cuda_check(h, e, "free-energy setup");
    }
    std::copy(q.begin(), q.begin() + n, q.begin() + n);
    std::copy(t.begin(), t.begin() + n, t.begin() + n);
    std::vector<unsigned char> pert(n, 0);
    std::vector<float>         qm(q.begin(), q.begin() + n);
    std::vector<int>           tm(t.begin(), t.begin() + n);
    for (int k = 0; k < d->num_perturbed; k++)
    {
        const int a = d->perturbed[k];
        q[n + a]    = d->qB[k];
        t[n + a]    = d->typeB[k];
        pert[a]     = 1;
        qm[a]       = 0.0f;  // masked out of the cluster path (atomdata_mask_fep)
        tm[a]       = nt;    // the all-zero type
    }
    h->self_energy_all = self_energy_of(v, std::vector<float>(q.begin(), q.begin() + n));
    e = cudaMemcpyAsync(h->d_fep_q, q.data(), sizeof(float) * 2 * n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->d_fep_t, t.data(), sizeof(int) * 2 * n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && d->num_perturbed > 0)
    {
        e = cudaMemcpyAsync(h->d_fep_list, d->perturbed, sizeof(int) * d->num_perturbed, cudaMemcpyHostToDevice,
                            h->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->d_fep_pert, pert.data(), n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
    {
        e = cudaMemcpyAsync(const_cast<float*>(v.q), qm.data(), sizeof(float) * n, cudaMemcpyHostToDevice, h->stream);
    }
    if (e == cudaSuccess)
    {
        e = cudaMemcpyAsync(const_cast<int*>(v.type), tm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, h->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess)
    {
        return cuda_check(h, e, "free-energy setup");
    }
    FepView& f     = h->fep;
    f.np           = d->num_perturbed;
    f.plist        = h->d_fep_list;
    f.pert         = h->d_fep_pert;
    f.qA           = h->d_fep_q;
    f.qB           = h->d_fep_q + n;
    f.tA           = h->d_fep_t;
    f.tB           = h->d_fep_t + n;
    f.alpha_c      = d->alpha_coul;
    f.alpha_v      = d->alpha_vdw;
    f.sigma6_def   = d->sigma6_def;
    f.sigma6_min   = d->sigma6_min;
    f.soft         = (d->alpha_coul != 0.0f || d->alpha_vdw != 0.0f) ? 1 : 0;
    f.sums         = h->d_fep_sums;
    h->fep_power   = d->lambda_power;
    set_fep_lambda(f, d->lambda_coul, d->lambda_vdw, d->lambda_power);
    v.self_energy  = self_energy_of(v, qm);
    h->fep_on      = true;
    h->have_list   = false;  // the next search fills the masked charges and types into the grid
    return NBX_OK;
}

int nbx_fep_set_lambda(nbx_handle* h, float lambda_coul, float lambda_vdw)
{
    if (!h)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (!h->fep_on)
    {
        return set_error(h, NBX_ERR_STATE, "no perturbed atoms set");
    }
    if (!(lambda_coul >= 0.0f && lambda_coul <= 1.0f && lambda_vdw >= 0.0f && lambda_vdw <= 1.0f))
    {
        return set_error(h, NBX_ERR_INVALID_INPUT, "lambda must lie in [0, 1]");
    }
    set_fep_lambda(h->fep, lambda_coul, lambda_vdw, h->fep_power);
    return NBX_OK;
}

int nbx_fep_get_energies(nbx_handle* h, double* out)
{
    if (!h || !out)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (!h->fep_on)
    {
        return set_error(h, NBX_ERR_STATE, "no perturbed atoms set");
    }
    cudaSetDevice(h->device);
    cudaError_t e = cudaMemcpyAsync(out, h->d_fep_sums, sizeof(double) * 4, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return cuda_check(h, e, "free-energy energies");
}

const double* nbx_fep_energies_device(nbx_handle* h)
{
    return (h && h->fep_on) ? h->d_fep_sums : nullptr;
}

int nbx_fep_disable(nbx_handle* h)
{
    if (!h)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (!h->fep_on)
    {
        return NBX_OK;
    }
    cudaSetDevice(h->device);
    return fep_restore(h);
}

int nbx_get_options(const nbx_handle* h, nbx_options* out)
{
    if (!h || !out)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    *out = h->opts;
    return NBX_OK;
}

int nbx_set_force_accumulate(nbx_handle* h, int enable)
{
    if (!h)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    h->v.accumulate_f = enable ? 1 : 0;
    return NBX_OK;
}

int nbx_get_force_accumulate(const nbx_handle* h, int* enabled)
{
    if (!h || !enabled)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    *enabled = h->v.accumulate_f;
    return NBX_OK;
}

int nbx_set_list_balance(nbx_handle* h, int entries_per_sm)
{
    if (!h || entries_per_sm < 0)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    h->min_ci_balanced = entries_per_sm * h->num_sms;
    return NBX_OK;
}

int nbx_get_list_balance(nbx_handle* h, int* out)
{
    if (!h || !out)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (!h->have_list)
    {
        return set_error(h, NBX_ERR_STATE, "no pair list");
    }
    cudaSetDevice(h->device);
    int rc = read_header(h);
    if (rc != NBX_OK)
    {
        return rc;
    }
    out[0] = h->min_ci_balanced;
    out[1] = h->h_hdr->nsp_max;
    out[2] = h->h_hdr->num_sci_unsplit;
    out[3] = h->h_hdr->num_sci;
    return NBX_OK;
}

int nbx_set_timing(nbx_handle* h, int enable)
{
    if (!h)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    h->timing = enable != 0;
    return NBX_OK;
}

int nbx_get_timings(nbx_handle* h, double* force_ms, long long* counts, int reset)
{
    if (!h)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(h->device);
    collect_timings(h, true);
    if (force_ms)
    {
        *force_ms = h->phase_ms[0];
    }
    if (counts)
    {
        counts[0] = h->force_launches;
        counts[1] = h->launches;
    }
    if (reset)
    {
        for (int k = 0; k < 5; k++)
        {
            h->phase_ms[k]    = 0.0;
            h->phase_count[k] = 0;
        }
        h->force_launches = 0;
        h->launches       = 0;
    }
    return NBX_OK;
}

int nbx_get_phase_timings(nbx_handle* h, double* ms, long long* counts, int reset)
{
    if (!h)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(h->device);
    collect_timings(h, true);
    for (int k = 0; k < 5; k++)
    {
        if (ms)
        {
            ms[k] = h->phase_ms[k];
        }
        if (counts)
        {
            counts[k] = h->phase_count[k];
        }
        if (reset)
        {
            h->phase_ms[k]    = 0.0;
            h->phase_count[k] = 0;
        }
    }
    return NBX_OK;
}

int nbx_synchronize(nbx_handle* h)
{
    if (!h)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(h->device);
    int rc = read_header(h);
    return rc != NBX_OK ? rc : status_to_error(h, h->h_hdr->status);
}

int nbx_get_sizes(nbx_handle* h, int* sizes)
{
    if (!h || !sizes)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(h->device);
    int rc = read_header(h);
    if (rc != NBX_OK)
    {
        return rc;
    }
    sizes[0] = h->n;
    sizes[1] = h->v.g.ncx;
    sizes[2] = h->v.g.ncy;
    sizes[3] = h->h_hdr->num_cells;
    sizes[4] = h->h_hdr->num_sci;
    sizes[5] = h->h_hdr->num_cj4;
    sizes[6] = h->h_hdr->num_excl;
    sizes[7] = h->h_hdr->num_cells * kSc;
    return NBX_OK;
}

int nbx_get_grid(nbx_handle* h, int* atom_indices, int* cells, int* cxy_ind, int* num_clusters, float* bb,
                 float* bbcz, float* xq)
{
    int sizes[8];
    int rc = nbx_get_sizes(h, sizes);
    if (rc != NBX_OK)
    {
        return rc;
    }
    const int   nc = sizes[3];
    cudaStream_t s = h->stream;
    cudaError_t e  = cudaSuccess;
    if (atom_indices) e = cudaMemcpyAsync(atom_indices, h->v.atom_indices, sizeof(int) * nc * kSc, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && cells) e = cudaMemcpyAsync(cells, h->v.cells, sizeof(int) * h->n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && cxy_ind) e = cudaMemcpyAsync(cxy_ind, h->v.cxy_ind, sizeof(int) * (h->v.g.ncol + 1), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && num_clusters) e = cudaMemcpyAsync(num_clusters, h->v.nclusters, sizeof(int) * nc, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && bbcz) e = cudaMemcpyAsync(bbcz, h->v.bbcz, sizeof(float2) * nc, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && xq) e = cudaMemcpyAsync(xq, h->v.xq, sizeof(float4) * nc * kSc, cudaMemcpyDeviceToHost, s);
    std::vector<float4> tmp;
    if (e == cudaSuccess && bb)
    {
        tmp.resize((size_t)nc * kNcl * 2);
        e = cudaMemcpyAsync(tmp.data(), h->v.bb, sizeof(float4) * tmp.size(), cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && bb)
    {
        for (size_t c = 0; c < (size_t)nc * kNcl; c++)
        {
            bb[6 * c + 0] = tmp[2 * c].x;
            bb[6 * c + 1] = tmp[2 * c].y;
            bb[6 * c + 2] = tmp[2 * c].z;
            bb[6 * c + 3] = tmp[2 * c + 1].x;
            bb[6 * c + 4] = tmp[2 * c + 1].y;
            bb[6 * c + 5] = tmp[2 * c + 1].z;
        }
    }
    return cuda_check(h, e, "nbx_get_grid");
}

int nbx_get_pairlist(nbx_handle* h, int* sci, int* cj4, uint32_t* excl, uint32_t* imask_outer)
{
    int sizes[8];
    int rc = nbx_get_sizes(h, sizes);
    if (rc != NBX_OK)
    {
        return rc;
    }
    cudaStream_t s = h->stream;
    cudaError_t  e = cudaSuccess;
    if (sci) e = cudaMemcpyAsync(sci, h->v.sci, sizeof(Sci) * sizes[4], cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && cj4) e = cudaMemcpyAsync(cj4, h->v.cj4, sizeof(Cj4) * sizes[5], cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && excl) e = cudaMemcpyAsync(excl, h->v.excl, sizeof(Excl) * sizes[6], cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && imask_outer) e = cudaMemcpyAsync(imask_outer, h->v.imask_outer, sizeof(unsigned) * 2 * sizes[5], cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return cuda_check(h, e, "nbx_get_pairlist");
}

int nbx_get_pair_counts(nbx_handle* h, long long* pairs)
{
    if (!h || !pairs)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(h->device);
    unsigned long long c = 0;
    cudaError_t        e = launch_pair_count(h->v, h->d_count, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&c, h->d_count, sizeof(c), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    pairs[0] = (long long)c;
    pairs[1] = -1;
    return cuda_check(h, e, "nbx_get_pair_counts");
}

int nbx_measure_fp32_peak(int device, double* tflops)
{
    if (!tflops)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(device);
    cudaError_t e = measure_fp32_peak(tflops);
    return e == cudaSuccess ? NBX_OK : NBX_ERR_CUDA;
}


} // extern "C"

// ----------------------------------------------------------------- batches

struct nbx_batch
{
    int                      device     = 0;
    int                      num_sms    = 152;
    cudaStream_t             stream     = nullptr;
    bool                     own_stream = false;
    std::vector<nbx_handle*> sys;
    std::vector<int>         offsets;  // atom offsets, size nsys+1
    nbx_options              opts{};
    std::string              err;
    DeviceView               cv{};     // interaction constants shared by all systems
    BatchSys*                d_table  = nullptr;
    BatchSys*                h_table  = nullptr;  // pinned
    int*                     d_prefix = nullptr;
    unsigned*                d_status = nullptr;
    double*                  d_sums   = nullptr;
    size_t                   sums_bytes = 0;
    int*                     d_counter  = nullptr;
    int                      max_slots  = 0;
    int                      max_atoms  = 0;
    bool                     have_list  = false;
    long long                list_step  = 0;
    int                      prune_part = 0;
    int                      nparts     = 1;
    bool                     use_prune  = false;
    int                      variant    = 0;  // launch shape of the batched force kernel (0..3)
    int                      tile       = 1;  // 1: packed pair core, 0: one pair per lane
    int                      depth      = 2;  // j-stage buffers per warp of the packed core
    bool                     use_graph  = true;
    cudaGraphExec_t          graph      = nullptr;
    cudaStream_t             capture_stream = nullptr;  // private: capture is not allowed on legacy streams
    const void*              graph_key[4] = { nullptr, nullptr, nullptr, nullptr };
    std::vector<cudaStream_t> search_streams;  // the systems' searches run concurrently on these
    // adjoint / force matching
    double*                  d_gnbfp_pad = nullptr;  // (nt+1)^2 * 2 FP64 type-pair sums
    int*                     d_adj_counter = nullptr;
    float*                   d_fm_f = nullptr;       // forces of the force-matching step, 3N
    float*                   d_fm_g = nullptr;       // dL/dF, 3N
    bool                     charges_on_device = false;
    cudaGraphExec_t          fm_graph = nullptr;
    const void*              fm_key[9] = { nullptr };
};

namespace
{
thread_local std::string g_batch_error;

// The force-kernel choice passed to launch_batch_compute: launch shape in bits 0-1, the packed
// core in bit 2, three stage buffers in bit 3.
int batch_variant_code(const nbx_batch* b)
{
    return b->variant | (b->tile ? 4 : 0) | (b->tile && b->depth == 3 ? 8 : 0);
}

int batch_error(nbx_batch* b, int code, const std::string& msg)
{
    if (b)
    {
        b->err = msg;
    }
    else
    {
        g_batch_error = msg;
    }
    return code;
}

void drop_graph(nbx_batch* b)
{
    if (b->graph)
    {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    for (auto& k : b->graph_key)
    {
        k = nullptr;
    }
}

// Rebuilds the device table of per-system pointers (they change when a list grows) and the
// entry prefix sums; called after every search.
int batch_refresh(nbx_batch* b)
{
    const int nsys = (int)b->sys.size();
    for (int i = 0; i < nsys; i++)
    {
        const DeviceView& v = b->sys[i]->v;
        BatchSys&         t = b->h_table[i];
        t.xq                = v.xq;
        t.tgrid             = v.tgrid;
        t.xqp               = v.xqp;
        t.fnb               = v.fnb;
        t.sci               = v.sci;
        t.cj4               = v.cj4;
        t.excl              = v.excl;
        t.imask_outer       = v.imask_outer;
        t.cells             = v.cells;
        t.atom_indices      = v.atom_indices;
        t.image             = v.image;
        t.hdr               = v.hdr;
        t.excl_index        = v.excl_index;
        t.excl_list         = v.excl_list;
        t.n                 = v.n;
        t.atom_base         = b->offsets[i];
        t.self_energy       = v.self_energy;
        t.self_on_device    = v.self_on_device;
        t.gnb               = b->sys[i]->d_gnb;
        t.dnb               = b->sys[i]->d_dnb;
        t.q                 = const_cast<float*>(v.q);
        for (int d = 0; d < 3; d++)
        {
            t.box[d] = v.g.box[d];
        }
        std::memcpy(t.shiftvec, v.shiftvec, sizeof(t.shiftvec));
    }
    cudaError_t e = cudaMemcpyAsync(b->d_table, b->h_table, sizeof(BatchSys) * nsys, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = launch_batch_prefix(b->d_table, nsys, b->d_prefix, b->d_status, b->stream);
    unsigned st = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, b->d_status, sizeof(st), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess)
    {
        return batch_error(b, NBX_ERR_CUDA, std::string("batch refresh: ") + cudaGetErrorString(e));
    }
    if (st & (kStatusListOverflow | kStatusExclOverflow | kStatusGridOverflow))
    {
        return batch_error(b, NBX_ERR_LIST_OVERFLOW, "a system's pair list or grid overflowed");
    }
    return NBX_OK;
}

constexpr int kSearchStreams = 8;

// The systems' searches, spread over kSearchStreams streams so that the small grid, search, balance
// and prune launches of different systems run concurrently, in two rounds: every system's grid +
// count, one host synchronisation for all their list headers, every system's write + balancing +
// fresh prune, one more synchronisation (a system whose records overflow counts again synchronously
// in between).  The batch's stream is synchronised first (the coordinates come from it) and the
// systems use it again afterwards.
int batch_search(nbx_batch* b, const float* d_x)
{
    const size_t nsys = b->sys.size();
    cudaError_t  e    = cudaStreamSynchronize(b->stream);
    while (e == cudaSuccess && b->search_streams.size() < (size_t)kSearchStreams)
    {
        cudaStream_t s = nullptr;
        e              = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e == cudaSuccess)
        {
            b->search_streams.push_back(s);
        }
    }
    if (e != cudaSuccess)
    {
        return batch_error(b, NBX_ERR_CUDA, cudaGetErrorString(e));
    }
    for (size_t i = 0; i < nsys; i++)
    {
        b->sys[i]->stream = b->search_streams[i % kSearchStreams];
    }
    auto sync_all = [&]() {
        cudaError_t r = cudaSuccess;
        for (cudaStream_t s : b->search_streams)
        {
            const cudaError_t q = cudaStreamSynchronize(s);
            r                   = r == cudaSuccess ? q : r;
        }
        return r;
    };
    auto restore = [&]() {
        sync_all();
        for (nbx_handle* h : b->sys)
        {
            h->stream = b->stream;
        }
    };
    auto fail = [&](size_t i, int rc) {
        restore();
        return batch_error(b, rc, "system " + std::to_string(i) + ": " + b->sys[i]->err);
    };
    auto headers = [&](size_t i) {
        nbx_handle* h = b->sys[i];
        return cuda_check(h, cudaMemcpyAsync(h->h_hdr, h->v.hdr, sizeof(ListHeader), cudaMemcpyDeviceToHost,
                                             h->stream),
                          "read list header");
    };
    for (size_t i = 0; i < nsys; i++)
    {
        nbx_handle* h  = b->sys[i];
        int         rc = cuda_check(h, search_launch_count(h, const_cast<float*>(d_x) + 3 * (size_t)b->offsets[i], 0),
                                    "grid/search count");
        if (rc == NBX_OK) rc = headers(i);
        if (rc != NBX_OK)
        {
            return fail(i, rc);
        }
    }
    if ((e = sync_all()) != cudaSuccess)
    {
        restore();
        return batch_error(b, NBX_ERR_CUDA, cudaGetErrorString(e));
    }
    for (size_t i = 0; i < nsys; i++)
    {
        int rc = search_launch_write(b->sys[i]);
        if (rc == NBX_OK) rc = headers(i);
        if (rc != NBX_OK)
        {
            return fail(i, rc);
        }
    }
    e = sync_all();
    restore();
    if (e != cudaSuccess)
    {
        return batch_error(b, NBX_ERR_CUDA, cudaGetErrorString(e));
    }
    for (size_t i = 0; i < nsys; i++)
    {
        const int rc = search_finish(b->sys[i]);
        if (rc != NBX_OK)
        {
            return batch_error(b, rc, "system " + std::to_string(i) + ": " + b->sys[i]->err);
        }
    }
    b->have_list  = true;
    b->prune_part = 0;
    return batch_refresh(b);
}

int batch_compute(nbx_batch* b, const float* d_x, float* d_f, double* d_e, double* d_vir)
{
    const int nsys = (int)b->sys.size();
    auto      run  = [&](cudaStream_t s) {
        return launch_batch_compute(b->cv, b->d_table, b->d_prefix, nsys, b->max_slots, b->max_atoms, d_x, d_f,
                                    b->d_sums, b->sums_bytes, b->d_counter, d_e, d_vir, batch_variant_code(b), b->num_sms, s);
    };
    if (!b->use_graph)
    {
        cudaError_t e = run(b->stream);
        return e == cudaSuccess ? NBX_OK : batch_error(b, NBX_ERR_CUDA, cudaGetErrorString(e));
    }
    const void* key[4] = { d_x, d_f, d_e, d_vir };
    if (!b->graph || std::memcmp(key, b->graph_key, sizeof(key)) != 0)
    {
        drop_graph(b);
        cudaGraph_t g = nullptr;
        // capture records without executing, so a private stream works for any caller stream
        cudaError_t e = cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess)
        {
            cudaError_t e2 = run(b->capture_stream);
            e              = cudaStreamEndCapture(b->capture_stream, &g);
            if (e2 != cudaSuccess)
            {
                e = e2;
            }
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
        if (g)
        {
            cudaGraphDestroy(g);
        }
        if (e != cudaSuccess)
        {
            drop_graph(b);
            return batch_error(b, NBX_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        }
        std::memcpy(b->graph_key, key, sizeof(key));
    }
    cudaError_t e = cudaGraphLaunch(b->graph, b->stream);
    return e == cudaSuccess ? NBX_OK : batch_error(b, NBX_ERR_CUDA, cudaGetErrorString(e));
}
// Adjoint scratch of every system and of the batch (first use), then the table.
int batch_ensure_adjoint(nbx_batch* b)
{
    if (b->d_gnbfp_pad)
    {
        return NBX_OK;
    }
    if (b->cv.ntypes1 > adjoint_max_types1())
    {
        return batch_error(b, NBX_ERR_INVALID_INPUT, "the adjoint supports at most 15 particle types");
    }
    cudaError_t e = cudaSuccess;
    for (nbx_handle* h : b->sys)
    {
        if (!h->d_gnb)
        {
            const size_t slots = (size_t)h->v.g.cells_capacity * kSc;
            e = dalloc(h, &h->d_gnb, slots);
            if (e == cudaSuccess) e = dalloc(h, &h->d_dnb, slots);
            if (e == cudaSuccess) e = dalloc(h, &h->d_gnbfp, 2 * (size_t)h->v.ntypes1 * h->v.ntypes1);
            if (e == cudaSuccess) e = dalloc(h, &h->d_adj_counter, 1);
            if (e != cudaSuccess)
            {
                return batch_error(b, NBX_ERR_OUT_OF_MEMORY, "adjoint allocation");
            }
        }
    }
    const size_t n3 = 3 * (size_t)b->offsets.back();
    e = cudaMalloc(&b->d_gnbfp_pad, sizeof(double) * 2 * b->cv.ntypes1 * b->cv.ntypes1);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_adj_counter, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_fm_f, sizeof(float) * n3);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_fm_g, sizeof(float) * n3);
    if (e != cudaSuccess)
    {
        return batch_error(b, NBX_ERR_OUT_OF_MEMORY, "adjoint allocation");
    }
    return b->have_list ? batch_refresh(b) : NBX_OK;
}

// From now on every system's self energy follows the charges on the device.
int batch_charges_on_device(nbx_batch* b)
{
    if (b->charges_on_device)
    {
        return NBX_OK;
    }
    for (nbx_handle* h : b->sys)
    {
        h->v.self_on_device = 1;
        h->v.self_energy    = 0.0;
    }
    b->charges_on_device = true;
    drop_graph(b);  // the table changes
    return b->have_list ? batch_refresh(b) : NBX_OK;
}

cudaError_t batch_backward_launch(nbx_batch* b, const float* d_gF, const double* d_gE, float* d_gx, float* d_gq,
                                  double* d_gnbfp, cudaStream_t s)
{
    const int   nsys = (int)b->sys.size();
    cudaError_t e    = launch_batch_backward(b->cv, b->d_table, b->d_prefix, nsys, b->max_slots, b->max_atoms, d_gF,
                                             d_gE, b->d_gnbfp_pad, b->d_adj_counter, d_gx, d_gq, b->num_sms, s);
    if (e == cudaSuccess && d_gnbfp)
    {
        e = launch_compact_gnbfp(b->d_gnbfp_pad, d_gnbfp, b->cv.ntypes1 - 1, s);
    }
    return e;
}

} // namespace

extern "C" {

int nbx_batch_set_parameters_device(nbx_batch* b, const float* d_q, const float* d_nbfp)
{
    if (!b)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(b->device);
    if (d_q)
    {
        int rc = batch_charges_on_device(b);
        if (rc != NBX_OK)
        {
            return rc;
        }
    }
    cudaError_t e = cudaSuccess;
    for (size_t i = 0; d_nbfp && i < b->sys.size() && e == cudaSuccess; i++)
    {
        // every system's copy of the shared type table (the batched kernels read the first)
        e = launch_set_parameters(b->sys[i]->v, nullptr, d_nbfp, b->stream);
    }
    if (e == cudaSuccess && d_q)
    {
        e = launch_batch_set_q(b->d_table, (int)b->sys.size(), b->max_slots, d_q, b->stream);
    }
    return e == cudaSuccess ? NBX_OK : batch_error(b, NBX_ERR_CUDA, cudaGetErrorString(e));
}

int nbx_batch_backward_device(nbx_batch* b, const float* d_x, const float* d_gF, const double* d_gE, float* d_gx,
                              float* d_gq, double* d_gnbfp)
{
    if (!b || !d_x || !d_gF)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (!b->have_list)
    {
        return batch_error(b, NBX_ERR_STATE, "no pair lists");
    }
    cudaSetDevice(b->device);
    int rc = batch_ensure_adjoint(b);
    if (rc != NBX_OK)
    {
        return rc;
    }
    // coordinates into the grid layout (the kernel also clears the force buffers)
    cudaError_t e = launch_batch_convert(b->d_table, (int)b->sys.size(), b->max_slots, d_x, b->stream);
    if (e == cudaSuccess) e = batch_backward_launch(b, d_gF, d_gE, d_gx, d_gq, d_gnbfp, b->stream);
    return e == cudaSuccess ? NBX_OK : batch_error(b, NBX_ERR_CUDA, cudaGetErrorString(e));
}

int nbx_batch_force_match_device(nbx_batch* b, const float* d_x, const float* d_q, const float* d_nbfp,
                                 const float* d_ftarget, double* d_loss, float* d_gq, double* d_gnbfp, double* d_e,
                                 double* d_vir)
{
    if (!b || !d_x || !d_q || !d_nbfp || !d_ftarget || !d_loss)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (!b->have_list)
    {
        return batch_error(b, NBX_ERR_STATE, "no pair lists");
    }
    cudaSetDevice(b->device);
    int rc = batch_ensure_adjoint(b);
    if (rc == NBX_OK) rc = batch_charges_on_device(b);
    if (rc != NBX_OK)
    {
        return rc;
    }
    const int    nsys = (int)b->sys.size();
    const size_t n3   = 3 * (size_t)b->offsets.back();
    auto         run  = [&](cudaStream_t s) {
        cudaError_t e = launch_set_parameters(b->sys[0]->v, nullptr, d_nbfp, s);
        if (e == cudaSuccess) e = launch_batch_set_q(b->d_table, nsys, b->max_slots, d_q, s);
        if (e == cudaSuccess)
            e = launch_batch_compute(b->cv, b->d_table, b->d_prefix, nsys, b->max_slots, b->max_atoms, d_x,
                                     b->d_fm_f, b->d_sums, b->sums_bytes, b->d_counter, d_e, d_vir, batch_variant_code(b),
                                     b->num_sms, s);
        if (e == cudaSuccess) e = launch_match_loss(b->d_fm_f, d_ftarget, n3, b->d_fm_g, d_loss, b->num_sms, s);
        if (e == cudaSuccess) e = batch_backward_launch(b, b->d_fm_g, nullptr, nullptr, d_gq, d_gnbfp, s);
        return e;
    };
    if (!b->use_graph)
    {
        cudaError_t e = run(b->stream);
        return e == cudaSuccess ? NBX_OK : batch_error(b, NBX_ERR_CUDA, cudaGetErrorString(e));
    }
    const void* key[9] = { d_x, d_q, d_nbfp, d_ftarget, d_loss, d_gq, d_gnbfp, d_e, d_vir };
    if (!b->fm_graph || std::memcmp(key, b->fm_key, sizeof(key)) != 0)
    {
        if (b->fm_graph)
        {
            cudaGraphExecDestroy(b->fm_graph);
            b->fm_graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess)
        {
            cudaError_t e2 = run(b->capture_stream);
            e              = cudaStreamEndCapture(b->capture_stream, &g);
            if (e2 != cudaSuccess)
            {
                e = e2;
            }
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->fm_graph, g, 0);
        if (g)
        {
            cudaGraphDestroy(g);
        }
        if (e != cudaSuccess)
        {
            if (b->fm_graph)
            {
                cudaGraphExecDestroy(b->fm_graph);
            }
            b->fm_graph = nullptr;
            return batch_error(b, NBX_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        }
        std::memcpy(b->fm_key, key, sizeof(key));
    }
    cudaError_t e = cudaGraphLaunch(b->fm_graph, b->stream);
    return e == cudaSuccess ? NBX_OK : batch_error(b, NBX_ERR_CUDA, cudaGetErrorString(e));
}

const char* nbx_batch_last_error(const nbx_batch* b)
{
    return b ? b->err.c_str() : g_batch_error.c_str();
}

int nbx_batch_create(int num_systems, const nbx_system_desc* systems, const nbx_options* opts, int device,
                     nbx_batch** out)
{
    if (num_systems <= 0 || !systems || !out)
    {
        return batch_error(nullptr, NBX_ERR_INVALID_INPUT, "need at least one system");
    }
    *out = nullptr;
    if (opts && (opts->vdw_modifier == NBX_VDW_FORCESWITCH || opts->vdw_modifier == NBX_VDW_POTSWITCH
                 || opts->vdw_modifier == NBX_VDW_LJPME))
    {
        return batch_error(nullptr, NBX_ERR_INVALID_INPUT, "batches take the potential-shift or plain LJ cut-off");
    }
    for (int i = 1; i < num_systems; i++)
    {
        const nbx_system_desc& a = systems[0];
        const nbx_system_desc& c = systems[i];
        if (c.num_types != a.num_types
            || std::memcmp(c.nbfp, a.nbfp, sizeof(float) * 2 * (size_t)a.num_types * a.num_types) != 0)
        {
            return batch_error(nullptr, NBX_ERR_INVALID_INPUT, "all systems of a batch share types and nbfp");
        }
    }
    nbx_batch* b = new nbx_batch();
    b->device    = device;
    cudaSetDevice(device);
    cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, device);
    optin_batch_force_smem();
    optin_batch_force_x2_smem();
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
    b->own_stream = true;
    if (opts)
    {
        b->opts = *opts;
    }
    else
    {
        nbx_default_options(&b->opts);
    }
    b->offsets.push_back(0);
    for (int i = 0; i < num_systems && e == cudaSuccess; i++)
    {
        nbx_handle* h  = nullptr;
        int         rc = nbx_create(&systems[i], &b->opts, device, &h);
        if (rc != NBX_OK)
        {
            std::string msg = "system " + std::to_string(i) + ": " + nbx_last_error(nullptr);
            nbx_batch_destroy(b);
            return batch_error(nullptr, rc, msg);
        }
        nbx_set_stream(h, b->stream);
        b->sys.push_back(h);
        b->offsets.push_back(b->offsets.back() + systems[i].num_atoms);
        b->max_slots = std::max(b->max_slots, h->v.g.cells_capacity * kSc);
        b->max_atoms = std::max(b->max_atoms, h->n);
    }
    b->cv        = b->sys[0]->v;
    b->use_prune = b->opts.nstlist_prune > 0;
    b->nparts    = b->use_prune ? std::max(1, b->opts.nstlist_prune / 2) : 1;
    const size_t nsys = (size_t)num_systems;
    b->sums_bytes     = sizeof(double) * (2 + kNShift * 3 + 9) * nsys + 64;
    if (e == cudaSuccess) e = cudaMalloc(&b->d_table, sizeof(BatchSys) * nsys);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_table, sizeof(BatchSys) * nsys);
    // entry prefix sums, then the exclusion work items' prefix sums (k_batch_prefix)
    if (e == cudaSuccess) e = cudaMalloc(&b->d_prefix, sizeof(int) * 2 * (nsys + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_status, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_sums, b->sums_bytes);
    if (e != cudaSuccess)
    {
        nbx_batch_destroy(b);
        return batch_error(nullptr, NBX_ERR_OUT_OF_MEMORY, "batch allocation");
    }
    // the work counter sits after the FP64 sums, inside the region cleared each step
    b->d_counter = reinterpret_cast<int*>(reinterpret_cast<char*>(b->d_sums) + b->sums_bytes - 64);
    int rc       = batch_refresh(b);
    if (rc != NBX_OK)
    {
        std::string msg = b->err;
        nbx_batch_destroy(b);
        return batch_error(nullptr, rc, msg);
    }
    b->have_list = true;
    *out         = b;
    return NBX_OK;
}

int nbx_batch_destroy(nbx_batch* b)
{
    if (!b)
    {
        return NBX_OK;
    }
    cudaSetDevice(b->device);
    if (b->stream)
    {
        cudaStreamSynchronize(b->stream);
    }
    for (cudaStream_t s : b->search_streams)
    {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    drop_graph(b);
    if (b->fm_graph)
    {
        cudaGraphExecDestroy(b->fm_graph);
    }
    cudaFree(b->d_gnbfp_pad);
    cudaFree(b->d_adj_counter);
    cudaFree(b->d_fm_f);
    cudaFree(b->d_fm_g);
    for (nbx_handle* h : b->sys)
    {
        nbx_destroy(h);
    }
    cudaFree(b->d_table);
    cudaFreeHost(b->h_table);
    cudaFree(b->d_prefix);
    cudaFree(b->d_status);
    cudaFree(b->d_sums);
    if (b->own_stream && b->stream)
    {
        cudaStreamDestroy(b->stream);
    }
    if (b->capture_stream)
    {
        cudaStreamDestroy(b->capture_stream);
    }
    delete b;
    return NBX_OK;
}

int nbx_batch_atoms(nbx_batch* b, long long* total, int* offsets)
{
    if (!b)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (total)
    {
        *total = b->offsets.back();
    }
    if (offsets)
    {
        std::memcpy(offsets, b->offsets.data(), sizeof(int) * b->offsets.size());
    }
    return NBX_OK;
}

int nbx_batch_set_stream(nbx_batch* b, void* s)
{
    if (!b)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (static_cast<cudaStream_t>(s) == b->stream)
    {
        return NBX_OK;
    }
    cudaSetDevice(b->device);
    // work queued on the previous stream finishes before the new one is used (not while the new
    // stream is capturing a CUDA graph); the batch's own graphs were captured on a private stream
    // and are launched on whichever is current
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(static_cast<cudaStream_t>(s), &capture) != cudaSuccess)
    {
        cudaGetLastError();
        capture = cudaStreamCaptureStatusNone;
    }
    if (capture == cudaStreamCaptureStatusNone)
    {
        cudaStreamSynchronize(b->stream);
    }
    if (b->own_stream)
    {
        cudaStreamDestroy(b->stream);
    }
    b->stream     = static_cast<cudaStream_t>(s);
    b->own_stream = false;
    for (nbx_handle* h : b->sys)
    {
        h->stream = b->stream;
    }
    return NBX_OK;
}

int nbx_batch_search_device(nbx_batch* b, const float* d_x)
{
    if (!b || !d_x)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(b->device);
    return batch_search(b, d_x);
}

int nbx_batch_prune_device(nbx_batch* b, int part)
{
    if (!b)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(b->device);
    const float outer2 = b->cv.rlist2, inner2 = b->cv.rlist_inner2;
    cudaError_t e = (part < 0) ? launch_batch_prune(b->d_table, b->d_prefix, (int)b->sys.size(), outer2, inner2, 1, 0,
                                                    1, b->stream)
                               : launch_batch_prune(b->d_table, b->d_prefix, (int)b->sys.size(), outer2, inner2, 0,
                                                    part % b->nparts, b->nparts, b->stream);
    return e == cudaSuccess ? NBX_OK : batch_error(b, NBX_ERR_CUDA, cudaGetErrorString(e));
}

int nbx_batch_compute_device(nbx_batch* b, const float* d_x, float* d_f, double* d_e, double* d_vir)
{
    if (!b || !d_x || !d_f)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(b->device);
    return batch_compute(b, d_x, d_f, d_e, d_vir);
}

int nbx_batch_md_step_device(nbx_batch* b, long long step, const float* d_x, float* d_f, double* d_e,
                             double* d_vir)
{
    if (!b || !d_x || !d_f)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(b->device);
    const int nstlist = std::max(1, b->opts.nstlist);
    int       rc      = NBX_OK;
    if (!b->have_list || step % nstlist == 0)
    {
        if ((rc = batch_search(b, d_x)) != NBX_OK)
        {
            return rc;
        }
        b->list_step = step;
    }
    else if (b->use_prune)
    {
        const long long age = step - b->list_step;
        if (age > 0 && age % 2 == 0)
        {
            rc            = nbx_batch_prune_device(b, b->prune_part);
            b->prune_part = (b->prune_part + 1) % b->nparts;
            if (rc != NBX_OK)
            {
                return rc;
            }
        }
    }
    return batch_compute(b, d_x, d_f, d_e, d_vir);
}

int nbx_batch_sequential_md_step_device(nbx_batch* b, long long step, const float* d_x, float* d_f, double* d_e,
                                        double* d_vir)
{
    if (!b || !d_x || !d_f)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    cudaSetDevice(b->device);
    for (size_t i = 0; i < b->sys.size(); i++)
    {
        const size_t o  = 3 * (size_t)b->offsets[i];
        int          rc = nbx_md_step_device(b->sys[i], step, d_x + o, d_f + o, d_e ? d_e + 2 * i : nullptr,
                                             d_vir ? d_vir + 9 * i : nullptr);
        if (rc != NBX_OK)
        {
            return batch_error(b, rc, "system " + std::to_string(i) + ": " + b->sys[i]->err);
        }
    }
    return NBX_OK;
}

int nbx_batch_set_graph(nbx_batch* b, int enable)
{
    if (!b)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    b->use_graph = enable != 0;
    drop_graph(b);
    return NBX_OK;
}

int nbx_batch_set_kernel_variant(nbx_batch* b, int variant)
{
    if (!b || variant < 0 || variant > 3)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    b->variant = variant;
    drop_graph(b);
    return NBX_OK;
}

int nbx_batch_set_force_kernel(nbx_batch* b, int tile, int stage_depth)
{
    if (!b || tile < 0 || tile > 1 || stage_depth < 2 || stage_depth > 3)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    b->tile  = tile;
    b->depth = stage_depth;
    drop_graph(b);
    return NBX_OK;
}

int nbx_batch_set_prune(nbx_batch* b, int nstlist_prune, float rlist_inner)
{
    if (!b || nstlist_prune < 0 || (nstlist_prune > 0 && !(rlist_inner >= b->opts.rcoulomb)))
    {
        return NBX_ERR_INVALID_INPUT;
    }
    b->opts.nstlist_prune = nstlist_prune;
    b->opts.rlist_inner   = rlist_inner;
    b->use_prune          = nstlist_prune > 0;
    b->nparts             = b->use_prune ? std::max(1, nstlist_prune / 2) : 1;
    const float rin       = (b->use_prune && rlist_inner > 0.0f) ? rlist_inner : b->opts.rlist;
    b->cv.rlist_inner2    = rin * rin;
    for (nbx_handle* h : b->sys)
    {
        h->opts.nstlist_prune = nstlist_prune;
        h->opts.rlist_inner   = rlist_inner;
        h->use_prune          = b->use_prune;
        h->nparts             = b->nparts;
        h->v.rlist_inner2     = rin * rin;
    }
    b->have_list = false;  // the next step searches and prunes with the new settings
    return NBX_OK;
}

} // extern "C"
