// Cluster-pair LJ + Ewald real-space (or reaction-field) force / energy kernel with the packed
// pair core (nbx_pair_x2.cuh): two atom pairs per lane in FP32x2 arithmetic.
//
// Physics of the reference's GPU-layout kernels
// (src/gromacs/nbnxm/kernels_reference/kernel_gpu_ref.cpp:57-379), potential-shift or plain
// cut-off LJ; the switch modifiers and LJ-PME run the one-pair-per-lane kernel (nbx_force.cu).
// The launch, work queue, excluded-pair energy items and FP64 energy sums are those of that
// kernel; the shapes (j-stage buffers per warp, blocks per SM) are template parameters chosen at
// run time (nbx_set_force_kernel, the batched autotuner).
#include "../../include/nbnxm_gb300.h"
#include "nbx_internal.cuh"
#include "nbx_pair_x2.cuh"

namespace nbx
{
namespace
{

constexpr int kForceThreads = 256;

// The same force / energy evaluation with the packed pair core (nbx_pair_x2.cuh): potential-shift
// or plain cut-off LJ with Ewald or reaction-field Coulomb.  kDepth: j-stage buffers per warp.
template<bool kEnergy, int kCoul, int kDepth, int kBlocks>
__global__ void __launch_bounds__(kForceThreads, kBlocks) k_force_x2(DeviceView v, int* work_counter)
{
    // {-6*C6, 12*C12, LJ energy shift of the pair, 0} per type pair
    extern __shared__ float4 smem_x2[];
    float4*   nbfp_s = smem_x2;
    const int nt1    = v.ntypes1;
    for (int k = threadIdx.x; k < nt1 * nt1; k += blockDim.x)
    {
        const float2 p = v.nbfp[k];
        // (12C12 cpot12)/12 - (6C6 cpot6)/6 (kernel_gpu_ref.cpp:327-336)
        nbfp_s[k] = make_float4(-p.x, p.y, p.y * v.cpot12 * (1.0f / 12.0f) - p.x * v.cpot6 * (1.0f / 6.0f), 0.0f);
    }
    __syncthreads();
    if (v.hdr->status & (kStatusListOverflow | kStatusExclOverflow | kStatusGridOverflow))
    {
        return;
    }
    const unsigned   full = 0xffffffffu;
    const int        lane = threadIdx.x & 31;
    const int        numSci = v.hdr->num_sci;
    JStageP<kDepth>  js;
    WarpSmemX2       w;
    carve_x2<kDepth>(smem_x2 + nt1 * nt1, threadIdx.x >> 5, js, w);
    stage_init_x2(js, lane);
    PairConstsX2 k;
    k.rc2      = v.rc2;
    k.pbeta    = v.pbeta;
    k.nbeta2l2 = -v.beta2l2;
    k.c2b      = v.c2b;
    k.k_rf2    = v.k_rf2;
    k.nk_rf2   = -v.k_rf2;
    k.sh_ewald = v.sh_ewald;
    k.k_rf     = v.k_rf;
    k.c_rf     = v.c_rf;
    k.epsfac   = v.epsfac;
    const SysPtrsX2 p = { v.xq, v.tgrid, v.xqp, v.fnb, v.cj4, v.excl, v.shiftvec, v.fshift };

    __shared__ double e_acc_s[2][kForceThreads];
    double&           e_lj_acc = e_acc_s[0][threadIdx.x];
    double&           e_el_acc = e_acc_s[1][threadIdx.x];
    e_lj_acc                   = 0.0;
    e_el_acc                   = 0.0;
    const int numChunks = kEnergy ? v.excl_chunks : 0;
    for (;;)
    {
        int t = 0;
        if (lane == 0)
        {
            t = atomicAdd(work_counter, 1);
        }
        t = __shfl_sync(full, t, 0);
        if (t >= numSci + numChunks)
        {
            break;
        }
        int e;
        if (item_is_chunk(t, numSci, numChunks, e))
        {
            if (kEnergy)
            {
                const double beta2  = (double)v.beta * (double)v.beta;
                double       excl_s = 0.0;
                for (int i = e * kExclChunkAtoms + lane; i < min(v.n, (e + 1) * kExclChunkAtoms); i += 32)
                {
                    double dummy_lj = 0.0;
                    excl_atom(v, v, i, false, beta2, e_el_acc, excl_s, dummy_lj);
                }
                e_el_acc = fma(excl_s, -(double)v.beta * 1.1283791670955125739, e_el_acc);
            }
            continue;
        }
        if (!process_entry_x2<kEnergy, kCoul, kDepth>(k, p, v.sci[e], reinterpret_cast<const char*>(nbfp_s), js, w,
                                                        nt1, lane, v.wait_test_bytes, e_lj_acc, e_el_acc))
        {
            stage_timeout_x2(js, &v.hdr->status, lane);
            break;
        }
    }
    if (kEnergy)
    {
        double elj = e_lj_acc, eel = e_el_acc;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            elj += __shfl_xor_sync(full, elj, o);
            eel += __shfl_xor_sync(full, eel, o);
        }
        if (lane == 0)
        {
            atomicAdd(&v.energy[0], elj);
            atomicAdd(&v.energy[1], eel * v.epsfac_d);
        }
    }
}

template<bool kEnergy, int kCoul, int kDepth, int kBlocks>
cudaError_t launch_x2(const DeviceView& v, cudaStream_t s, int num_sms, int* counter)
{
    const size_t smem = sizeof(float4) * ((size_t)v.ntypes1 * v.ntypes1
                                          + (size_t)(kForceThreads / 32) * warp_smem_f4_x2<kDepth>());
    cudaError_t e = smem_optin<k_force_x2<kEnergy, kCoul, kDepth, kBlocks>>(
            smem + sizeof(double) * 2 * kForceThreads, smem);
    if (e != cudaSuccess)
    {
        return e;
    }
    k_force_x2<kEnergy, kCoul, kDepth, kBlocks><<<num_sms * kBlocks, kForceThreads, smem, s>>>(v, counter);
    return cudaGetLastError();
}

// Coulomb flavour of the packed core: 0 reaction field, 1 Ewald, 2 Ewald with the potential shift
// (energies only; forces do not depend on the shift)
int coulomb_flavour(const DeviceView& v, bool energy)
{
    if (v.coulomb != 0)
    {
        return 0;
    }
    return (energy && v.sh_ewald != 0.0f) ? 2 : 1;
}

} // namespace

cudaError_t launch_force_x2(const DeviceView& v, bool energy, cudaStream_t s, int num_sms, int* counter)
{
    using Launch = cudaError_t (*)(const DeviceView&, cudaStream_t, int, int*);
    // [blocks 2, 3][depth 2, 3][energy][coulomb flavour]
    static const Launch table[2][2][2][3] = {
        { { { launch_x2<false, 0, 2, 2>, launch_x2<false, 1, 2, 2>, launch_x2<false, 1, 2, 2> },
            { launch_x2<true, 0, 2, 2>, launch_x2<true, 1, 2, 2>, launch_x2<true, 2, 2, 2> } },
          { { launch_x2<false, 0, 3, 2>, launch_x2<false, 1, 3, 2>, launch_x2<false, 1, 3, 2> },
            { launch_x2<true, 0, 3, 2>, launch_x2<true, 1, 3, 2>, launch_x2<true, 2, 3, 2> } } },
        { { { launch_x2<false, 0, 2, 3>, launch_x2<false, 1, 2, 3>, launch_x2<false, 1, 2, 3> },
            { launch_x2<true, 0, 2, 3>, launch_x2<true, 1, 2, 3>, launch_x2<true, 2, 2, 3> } },
          { { launch_x2<false, 0, 3, 3>, launch_x2<false, 1, 3, 3>, launch_x2<false, 1, 3, 3> },
            { launch_x2<true, 0, 3, 3>, launch_x2<true, 1, 3, 3>, launch_x2<true, 2, 3, 3> } } },
    };
    return table[v.force_blocks == 3 ? 1 : 0][v.stage_depth == 3 ? 1 : 0][energy ? 1 : 0][coulomb_flavour(v, energy)](
            v, s, num_sms, counter);
}

} // namespace nbx
