// Batched evaluation of many independent systems of uneven size.
//
// Each system keeps its own grid and pair list (built by the single-system
// search); one step for the whole batch is six launches, independent of the
// number of systems: clearing the sums, coordinate conversion, FP64 exclusion
// energies (one wave of warps over 128-atom items of all systems), one
// persistent force kernel over the concatenated entry space of all systems
// (an entry finds its system by searching the entry prefix sums), the force
// gather + virial, and the per-system energy / virial finish.  The sequence
// has no host synchronisation and is captured in a CUDA graph by the host.
// Per-system energies, shift forces and virials are reduced in FP64.
#include "nbx_internal.cuh"
#include "nbx_pair_core.cuh"

namespace nbx
{
namespace
{

// Entry prefix sums over the systems' lists (after every search), prefix[0..nsys], and the
// prefix sums of their exclusion work items (kExclChunkAtoms atoms each),
// prefix[nsys + 1 .. 2 nsys + 1]; systems whose list or grid overflowed contribute neither
// and are flagged.
__global__ void k_batch_prefix(const BatchSys* sys, int nsys, int* prefix, unsigned* status)
{
    if (threadIdx.x != 0)
    {
        return;
    }
    int*     chunk_prefix = prefix + nsys + 1;
    int      run = 0, run_c = 0;
    unsigned st  = 0;
    for (int s = 0; s < nsys; s++)
    {
        prefix[s]          = run;
        chunk_prefix[s]    = run_c;
        const ListHeader* h = sys[s].hdr;
        if (h->status & (kStatusListOverflow | kStatusExclOverflow | kStatusGridOverflow))
        {
            st |= h->status;
            continue;
        }
        run += h->num_sci;
        run_c += (sys[s].n + kExclChunkAtoms - 1) / kExclChunkAtoms;
    }
    prefix[nsys]       = run;
    chunk_prefix[nsys] = run_c;
    *status            = st;
}

// nbnxn_atomdata_copy_x_to_nbat_x for all systems (blockIdx.y = system); also
// clears the grid-order force accumulators, so no per-system memset is needed.
__global__ void k_batch_convert(const BatchSys* __restrict__ sys, const float* __restrict__ x)
{
    const BatchSys& b = sys[blockIdx.y];
    const int       k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= b.hdr->num_cells * kSc)
    {
        return;
    }
    b.fnb[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int a = b.atom_indices[k];
    if (a >= 0)
    {
        const float* xa   = x + 3 * (size_t)(b.atom_base + a);
        const float4 old  = b.xq[k];
        const int    code = b.image[a];
        float        c[3];
        for (int d = 0; d < 3; d++)
        {
            const int s = (int)(signed char)((code >> (8 * d)) & 0xff);
            c[d]        = (s == 0) ? xa[d] : xa[d] + (float)s * b.box[d];
        }
        const_cast<float4*>(b.xq)[k] = make_float4(c[0], c[1], c[2], old.w);
        write_packed_slot(const_cast<float*>(b.xqp), k, c[0], c[1], c[2], old.w, b.tgrid[k]);
    }
}


// Excluded-pair Coulomb energies and self terms in FP64 for all systems: one warp per work
// item of kExclChunkAtoms atoms (the item prefix sums of k_batch_prefix), one wave of blocks,
// one FP64 atomic per item into its system's energy.
__global__ void __launch_bounds__(256) k_batch_excl_energy(DeviceView cv, const BatchSys* __restrict__ sys,
                                                           const int* __restrict__ prefix, int nsys,
                                                           double* energies)
{
    const int* chunk_prefix = prefix + nsys + 1;
    const int  total        = chunk_prefix[nsys];
    const int  lane         = threadIdx.x & 31;
    const int  nwarps       = (gridDim.x * blockDim.x) >> 5;
    const double beta2      = (double)cv.beta * (double)cv.beta;
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < total; c += nwarps)
    {
        const int       cs = find_system(chunk_prefix, nsys, c);
        const BatchSys& b  = sys[cs];
        const int       a0 = (c - chunk_prefix[cs]) * kExclChunkAtoms;
        double          acc = 0.0, acc_s = 0.0, acc_lj = 0.0;
        for (int i = a0 + lane; i < min(b.n, a0 + kExclChunkAtoms); i += 32)
        {
            excl_atom(cv, b, i, false, beta2, acc, acc_s, acc_lj);
        }
        acc += acc_s * (-(double)cv.beta * 1.1283791670955125739);
        for (int o = 16; o > 0; o >>= 1)
        {
            acc += __shfl_xor_sync(0xffffffffu, acc, o);
        }
        if (lane == 0 && acc != 0.0)
        {
            atomicAdd(&energies[2 * cs + 1], acc * cv.epsfac_d);
        }
    }
}

// The force kernel over all systems' entries; energies flushed per entry into
// the entry's system slots.
template<bool kEnergy, bool kEwald, int kThreads, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
        k_batch_force(DeviceView cv, const BatchSys* __restrict__ sys, const int* __restrict__ prefix, int nsys,
                      int* work_counter, double* energies, double* fshift)
{
    extern __shared__ float4 nbfp_s[];
    const int nt1 = cv.ntypes1;
    for (int k = threadIdx.x; k < nt1 * nt1; k += blockDim.x)
    {
        const float2 p = cv.nbfp[k];
        nbfp_s[k] = make_float4(p.x, p.y, p.y * cv.cpot12 * (1.0f / 12.0f) - p.x * cv.cpot6 * (1.0f / 6.0f), 0.0f);
    }
    __syncthreads();
    const unsigned full    = 0xffffffffu;
    const int      lane    = threadIdx.x & 31;
    const int      ii      = lane & 7;
    const int      jj      = lane >> 3;
    const int      total   = prefix[nsys];
    const float    rc2     = cv.rc2;
    const float    beta    = cv.beta;
    const float    pbeta   = cv.pbeta;
    const float    beta2l2 = cv.beta2l2;  // beta^2 * log2(e)
    const float    c2b     = cv.c2b;      // 2 beta / sqrt(pi)
    const float    k_rf2   = cv.k_rf2;
    // per-warp double-buffered j stage (bulk copies), after the type table
    JStage js = stage_carve(nbfp_s, nt1 * nt1, threadIdx.x >> 5, blockDim.x >> 5);
    stage_init(js, lane);
    for (;;)
    {
        int e = 0;
        if (lane == 0)
        {
            e = atomicAdd(work_counter, 1);
        }
        e = __shfl_sync(full, e, 0);
        if (e >= total)
        {
            break;
        }
        const int       sidx = find_system(prefix, nsys, e);
        const BatchSys& b    = sys[sidx];
        const Sci       s    = b.sci[e - prefix[sidx]];
        const SysPtrs   p    = { b.xq, b.tgrid, b.fnb, b.cj4, b.excl, b.shiftvec, fshift + (size_t)kNShift * 3 * sidx };
        double          elj = 0.0, eel = 0.0;
        if (!process_entry<kEnergy, kEwald>(cv, p, s, nbfp_s, js, nt1, lane, ii, jj, rc2, pbeta, beta2l2, c2b, k_rf2,
                                            elj, eel))
        {
            stage_timeout(js, const_cast<unsigned*>(&b.hdr->status), lane);
            break;
        }
        if (kEnergy)
        {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
            {
                elj += __shfl_xor_sync(full, elj, o);
                eel += __shfl_xor_sync(full, eel, o);
            }
            if (lane == 0)
            {
                atomicAdd(&energies[2 * sidx], elj);
                atomicAdd(&energies[2 * sidx + 1], eel * cv.epsfac_d);
            }
        }
    }
}

constexpr int kBatchReduceAtoms = 8;

// f (concatenated, atom order) and per-system sum x (x) f, float partials reduced in FP64.
__global__ void k_batch_reduce(const BatchSys* __restrict__ sys, float* __restrict__ f, double* virial,
                               int do_virial)
{
    const BatchSys& b = sys[blockIdx.y];
    float           w[9];
#pragma unroll
    for (int k = 0; k < 9; k++)
    {
        w[k] = 0.0f;
    }
    const int a0 = blockIdx.x * blockDim.x * kBatchReduceAtoms + threadIdx.x;
#pragma unroll
    for (int r = 0; r < kBatchReduceAtoms; r++)
    {
        const int a = a0 + r * blockDim.x;
        if (a < b.n)
        {
            const int    k  = b.cells[a];
            const float4 fa = b.fnb[k];
            float*       fo = f + 3 * (size_t)(b.atom_base + a);
            fo[0]           = fa.x;
            fo[1]           = fa.y;
            fo[2]           = fa.z;
            if (do_virial)
            {
                const float4 xa    = b.xq[k];
                const float  xv[3] = { xa.x, xa.y, xa.z };
                const float  fv[3] = { fa.x, fa.y, fa.z };
#pragma unroll
                for (int p = 0; p < 3; p++)
                {
#pragma unroll
                    for (int q = 0; q < 3; q++)
                    {
                        w[p * 3 + q] = fmaf(xv[p], fv[q], w[p * 3 + q]);
                    }
                }
            }
        }
    }
    if (!do_virial)
    {
        return;
    }
    __shared__ double ws[9][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // the warp's sum in float (FP64 runs at a small fraction of the FP32 rate here), the warps'
    // partials in FP64
#pragma unroll
    for (int k = 0; k < 9; k++)
    {
        float t = w[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            t += __shfl_xor_sync(0xffffffffu, t, o);
        }
        if (lane == 0)
        {
            ws[k][warp] = (double)t;
        }
    }
    __syncthreads();
    if (threadIdx.x < 9)
    {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++)
        {
            t += ws[threadIdx.x][k];
        }
        if (t != 0.0)
        {
            atomicAdd(&virial[9 * blockIdx.y + threadIdx.x], t);
        }
    }
}

// Per-system energies (+ self term) and virial = -1/2 (sum x (x) f + sum shift (x) fshift).
__global__ void k_batch_finish(const BatchSys* __restrict__ sys, int nsys, const double* energies,
                               const double* fshift, const double* virial, double* d_e, double* d_vir)
{
    const int s = blockIdx.x;
    const int t = threadIdx.x;
    if (s >= nsys)
    {
        return;
    }
    if (d_e && t < 2)
    {
        d_e[2 * s + t] = energies[2 * s + t] + (t == 1 ? sys[s].self_energy : 0.0);
    }
    if (d_vir && t < 9)
    {
        const int p = t / 3, q = t % 3;
        double    acc = virial[9 * s + t];
        for (int sh = 0; sh < kNShift; sh++)
        {
            acc += (double)sys[s].shiftvec[3 * sh + p] * fshift[(size_t)kNShift * 3 * s + 3 * sh + q];
        }
        d_vir[9 * s + t] = -0.5 * acc;
    }
}

template<bool kE, bool kW, int kT, int kM>
void launch_batch_force_t(const DeviceView& cv, const BatchSys* sys, const int* prefix, int nsys, int* ctr,
                          double* en, double* fs, int num_sms, cudaStream_t s)
{
    const size_t smem = sizeof(float4) * (size_t)cv.ntypes1 * cv.ntypes1 + (size_t)(kT / 32) * kStageSmemPerWarp;
    k_batch_force<kE, kW, kT, kM><<<num_sms * kM, kT, smem, s>>>(cv, sys, prefix, nsys, ctr, en, fs);
}

template<bool kE, bool kW, int kT, int kM>
cudaError_t optin_batch_t()
{
    // the type table (up to 48^2 entries) and the per-warp stages may pass 48 KB
    return cudaFuncSetAttribute(k_batch_force<kE, kW, kT, kM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(float4) * 48 * 48 + (kT / 32) * kStageSmemPerWarp));
}

template<bool kE, bool kW>
cudaError_t optin_batch_variants()
{
    cudaError_t e = optin_batch_t<kE, kW, 256, 2>();
    if (e == cudaSuccess) e = optin_batch_t<kE, kW, 128, 4>();
    if (e == cudaSuccess) e = optin_batch_t<kE, kW, 512, 1>();
    if (e == cudaSuccess) e = optin_batch_t<kE, kW, 64, 8>();
    return e;
}

template<bool kE, bool kW>
void launch_batch_force_variant(int variant, const DeviceView& cv, const BatchSys* sys, const int* prefix, int nsys,
                                int* ctr, double* en, double* fs, int num_sms, cudaStream_t s)
{
    switch (variant)
    {
        case 1: launch_batch_force_t<kE, kW, 128, 4>(cv, sys, prefix, nsys, ctr, en, fs, num_sms, s); break;
        case 2: launch_batch_force_t<kE, kW, 512, 1>(cv, sys, prefix, nsys, ctr, en, fs, num_sms, s); break;
        case 3: launch_batch_force_t<kE, kW, 64, 8>(cv, sys, prefix, nsys, ctr, en, fs, num_sms, s); break;
        default: launch_batch_force_t<kE, kW, 256, 2>(cv, sys, prefix, nsys, ctr, en, fs, num_sms, s); break;
    }
}

} // namespace

cudaError_t launch_batch_prefix(const BatchSys* sys, int nsys, int* prefix, unsigned* status, cudaStream_t s)
{
    k_batch_prefix<<<1, 32, 0, s>>>(sys, nsys, prefix, status);
    return cudaGetLastError();
}

// One batched step: sums (energies | fshift | virial partials | work counter)
cudaError_t launch_batch_convert(const BatchSys* sys, int nsys, int max_slots, const float* d_x, cudaStream_t s)
{
    const int tb = 256;
    k_batch_convert<<<dim3((max_slots + tb - 1) / tb, nsys), tb, 0, s>>>(sys, d_x);
    return cudaGetLastError();
}

// cleared with one memset, then the five kernels.
cudaError_t launch_batch_compute(const DeviceView& cv, const BatchSys* sys, const int* prefix, int nsys,
                                 int max_slots, int max_atoms, const float* d_x, float* d_f, double* sums,
                                 size_t sums_bytes, int* counter, double* d_e, double* d_vir, int variant,
                                 int num_sms, cudaStream_t s)
{
    const bool energy  = (d_e != nullptr) || (d_vir != nullptr);
    double*    en      = sums;
    double*    fs      = sums + 2 * (size_t)nsys;
    double*    vir     = fs + (size_t)kNShift * 3 * nsys;
    cudaError_t e      = cudaMemsetAsync(sums, 0, sums_bytes, s);
    const int  tb      = 256;
    dim3       gconv((max_slots + tb - 1) / tb, nsys);
    k_batch_convert<<<gconv, tb, 0, s>>>(sys, d_x);
    if (energy)
    {
        k_batch_excl_energy<<<num_sms * 8, 256, 0, s>>>(cv, sys, prefix, nsys, en);
    }
    const bool ewald = (cv.coulomb == 0);
    if (variant & 4)
    {
        // the packed pair core: launch shape in bits 0-1, three stage buffers in bit 3
        const cudaError_t ex = launch_batch_force_x2(cv, sys, prefix, nsys, counter, en, fs, variant & 3,
                                                     (variant & 8) ? 3 : 2, energy, num_sms, s);
        if (e == cudaSuccess)
        {
            e = ex;
        }
    }
    else if (energy)
    {
        if (ewald)
            launch_batch_force_variant<true, true>(variant, cv, sys, prefix, nsys, counter, en, fs, num_sms, s);
        else
            launch_batch_force_variant<true, false>(variant, cv, sys, prefix, nsys, counter, en, fs, num_sms, s);
    }
    else
    {
        if (ewald)
            launch_batch_force_variant<false, true>(variant, cv, sys, prefix, nsys, counter, en, fs, num_sms, s);
        else
            launch_batch_force_variant<false, false>(variant, cv, sys, prefix, nsys, counter, en, fs, num_sms, s);
    }
    dim3 gred((max_atoms + tb * kBatchReduceAtoms - 1) / (tb * kBatchReduceAtoms), nsys);
    k_batch_reduce<<<gred, tb, 0, s>>>(sys, d_f, vir, d_vir ? 1 : 0);
    if (energy)
    {
        k_batch_finish<<<nsys, 32, 0, s>>>(sys, nsys, en, fs, vir, d_e, d_vir);
    }
    return e == cudaSuccess ? cudaGetLastError() : e;
}

// Raises the dynamic shared-memory limit of every batched force kernel (host set-up
// before any launch or capture; the 512-thread shape with many types needs > 48 KB).
cudaError_t optin_batch_force_smem()
{
    cudaError_t e = optin_batch_variants<true, true>();
    if (e == cudaSuccess) e = optin_batch_variants<true, false>();
    if (e == cudaSuccess) e = optin_batch_variants<false, true>();
    if (e == cudaSuccess) e = optin_batch_variants<false, false>();
    return e;
}

} // namespace nbx
