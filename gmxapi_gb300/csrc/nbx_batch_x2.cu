// Batched force kernel with the packed pair core (nbx_pair_x2.cuh): the persistent launch over
// the concatenated list entries of all systems of a batch (an entry finds its system by a binary
// search of the entry prefix sums), two atom pairs per lane in FP32x2 arithmetic.  The shapes
// (threads x blocks per SM, j-stage buffers per warp) are what the batched autotuner chooses
// among, together with the one-pair-per-lane kernel of nbx_batch.cu.
#include "nbx_internal.cuh"
#include "nbx_pair_x2.cuh"

namespace nbx
{
namespace
{

template<bool kEnergy, int kCoul, int kThreads, int kMinBlocks, int kDepth>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
        k_batch_force_x2(DeviceView cv, const BatchSys* __restrict__ sys, const int* __restrict__ prefix, int nsys,
                         int* work_counter, double* energies, double* fshift)
{
    // {-6*C6, 12*C12, LJ energy shift of the pair, 0} per type pair (kernel_gpu_ref.cpp:327-336)
    extern __shared__ float4 smem_bx2[];
    float4*   nbfp_s = smem_bx2;
    const int nt1    = cv.ntypes1;
    for (int k = threadIdx.x; k < nt1 * nt1; k += blockDim.x)
    {
        const float2 p = cv.nbfp[k];
        nbfp_s[k] = make_float4(-p.x, p.y, p.y * cv.cpot12 * (1.0f / 12.0f) - p.x * cv.cpot6 * (1.0f / 6.0f), 0.0f);
    }
    __syncthreads();
    const unsigned  full  = 0xffffffffu;
    const int       lane  = threadIdx.x & 31;
    const int       total = prefix[nsys];
    JStageP<kDepth> js;
    WarpSmemX2      w;
    carve_x2<kDepth>(smem_bx2 + nt1 * nt1, threadIdx.x >> 5, js, w);
    stage_init_x2(js, lane);
    PairConstsX2 k;
    k.rc2      = cv.rc2;
    k.pbeta    = cv.pbeta;
    k.nbeta2l2 = -cv.beta2l2;
    k.c2b      = cv.c2b;
    k.k_rf2    = cv.k_rf2;
    k.nk_rf2   = -cv.k_rf2;
    k.sh_ewald = cv.sh_ewald;
    k.k_rf     = cv.k_rf;
    k.c_rf     = cv.c_rf;
    k.epsfac   = cv.epsfac;
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
        const SysPtrsX2 p    = { b.xq, b.tgrid, b.xqp, b.fnb, b.cj4, b.excl, b.shiftvec,
                                 fshift + (size_t)kNShift * 3 * sidx };
        double          elj = 0.0, eel = 0.0;
        if (!process_entry_x2<kEnergy, kCoul, kDepth>(k, p, s, reinterpret_cast<const char*>(nbfp_s), js, w, nt1,
                                                       lane, cv.wait_test_bytes, elj, eel))
        {
            stage_timeout_x2(js, const_cast<unsigned*>(&b.hdr->status), lane);
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

constexpr size_t kMaxTableF4 = 48 * 48;  // the largest type table the kernels accept

template<int kThreads, int kDepth>
size_t batch_x2_smem(int nt1)
{
    return sizeof(float4) * ((size_t)nt1 * nt1 + (size_t)(kThreads / 32) * warp_smem_f4_x2<kDepth>());
}

template<bool kE, int kW, int kT, int kM, int kD>
cudaError_t launch_t(const DeviceView& cv, const BatchSys* sys, const int* prefix, int nsys, int* ctr, double* en,
                     double* fs, int num_sms, cudaStream_t s)
{
    k_batch_force_x2<kE, kW, kT, kM, kD><<<num_sms * kM, kT, batch_x2_smem<kT, kD>(cv.ntypes1), s>>>(
            cv, sys, prefix, nsys, ctr, en, fs);
    return cudaGetLastError();
}

template<bool kE, int kW, int kT, int kM, int kD>
cudaError_t optin_t()
{
    const size_t smem = sizeof(float4) * (kMaxTableF4 + (size_t)(kT / 32) * warp_smem_f4_x2<kD>());
    return cudaFuncSetAttribute(k_batch_force_x2<kE, kW, kT, kM, kD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
}

template<bool kE, int kW, int kD>
cudaError_t launch_shape(int shape, const DeviceView& cv, const BatchSys* sys, const int* prefix, int nsys, int* ctr,
                         double* en, double* fs, int num_sms, cudaStream_t s)
{
    switch (shape)
    {
        case 1: return launch_t<kE, kW, 128, 4, kD>(cv, sys, prefix, nsys, ctr, en, fs, num_sms, s);
        case 2: return launch_t<kE, kW, 512, 1, kD>(cv, sys, prefix, nsys, ctr, en, fs, num_sms, s);
        case 3: return launch_t<kE, kW, 64, 8, kD>(cv, sys, prefix, nsys, ctr, en, fs, num_sms, s);
        default: return launch_t<kE, kW, 256, 2, kD>(cv, sys, prefix, nsys, ctr, en, fs, num_sms, s);
    }
}

template<bool kE, int kW, int kD>
cudaError_t optin_shapes()
{
    cudaError_t e = optin_t<kE, kW, 256, 2, kD>();
    if (e == cudaSuccess) e = optin_t<kE, kW, 128, 4, kD>();
    if (e == cudaSuccess) e = optin_t<kE, kW, 512, 1, kD>();
    if (e == cudaSuccess) e = optin_t<kE, kW, 64, 8, kD>();
    return e;
}

} // namespace

cudaError_t launch_batch_force_x2(const DeviceView& cv, const BatchSys* sys, const int* prefix, int nsys, int* counter,
                                  double* energies, double* fshift, int shape, int stage_depth, bool energy,
                                  int num_sms, cudaStream_t s)
{
    using Launch = cudaError_t (*)(int, const DeviceView&, const BatchSys*, const int*, int, int*, double*, double*,
                                   int, cudaStream_t);
    // [depth 2, 3][energy][coulomb: 0 reaction field, 1 Ewald, 2 Ewald with the potential shift]
    static const Launch table[2][2][3] = {
        { { launch_shape<false, 0, 2>, launch_shape<false, 1, 2>, launch_shape<false, 1, 2> },
          { launch_shape<true, 0, 2>, launch_shape<true, 1, 2>, launch_shape<true, 2, 2> } },
        { { launch_shape<false, 0, 3>, launch_shape<false, 1, 3>, launch_shape<false, 1, 3> },
          { launch_shape<true, 0, 3>, launch_shape<true, 1, 3>, launch_shape<true, 2, 3> } },
    };
    const int coul = cv.coulomb != 0 ? 0 : (energy && cv.sh_ewald != 0.0f ? 2 : 1);
    return table[stage_depth == 3 ? 1 : 0][energy ? 1 : 0][coul](shape, cv, sys, prefix, nsys, counter, energies,
                                                                   fshift, num_sms, s);
}

// Raises the dynamic shared-memory limit of every packed batched force kernel (host set-up before
// any launch or capture).
cudaError_t optin_batch_force_x2_smem()
{
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = optin_shapes<true, 0, 2>();
    if (e == cudaSuccess) e = optin_shapes<true, 1, 2>();
    if (e == cudaSuccess) e = optin_shapes<true, 2, 2>();
    if (e == cudaSuccess) e = optin_shapes<false, 0, 2>();
    if (e == cudaSuccess) e = optin_shapes<false, 1, 2>();
    if (e == cudaSuccess) e = optin_shapes<true, 0, 3>();
    if (e == cudaSuccess) e = optin_shapes<true, 1, 3>();
    if (e == cudaSuccess) e = optin_shapes<true, 2, 3>();
    if (e == cudaSuccess) e = optin_shapes<false, 0, 3>();
    if (e == cudaSuccess) e = optin_shapes<false, 1, 3>();
    return e;
}

} // namespace nbx
