// Cluster-pair LJ + Ewald real-space (or reaction-field) force / energy kernel.
//
// Physics of the reference's GPU-layout kernels
// (src/gromacs/nbnxm/kernels_reference/kernel_gpu_ref.cpp:57-379 and
// cuda/nbnxm_cuda_kernel.cuh:148-649): for every set bit of the pair-list
// mask, the 8x8 atom pairs of an i-cluster / j-cluster within rc interact with
//   LJ      6*C6, 12*C12 from nbfp, potential-shifted energies,
//   Ewald   qq*erfc(beta r)/r (exclusions within rc: -qq*erf(beta r)/r),
//   RF      qq*(1/r + k_rf r^2 - c_rf),
// and the forces on j are the negated forces on i (half list).
//
// This file holds the one-pair-per-lane kernel (k_force: the switch modifiers, LJ-PME and the
// autotuner's tile 0), the force reduction, the allocation-free entry and the launch dispatch; the
// default kernel for potential-shift and plain cut-off LJ is the packed two-pairs-per-lane core of
// nbx_force_x2.cu / nbx_pair_x2.cuh, which shares the work queue, the exclusion work items and the
// reduction below.
//
// GB300 design (not the reference's 8x8-thread blocks):
//  - persistent warps take list entries from an atomic work queue;
//  - one warp owns one entry: lane = (j-atom of the half, 0..3) * 8 + i-atom;
//    the 64 shifted i-atoms (x, y, z, q*epsfac, type row) live in registers,
//    so i-data is loaded once per entry instead of once per pair;
//  - the per-(i-cluster, j-cluster) mask test is warp-uniform, the per-pair
//    cut-off / exclusion / self test is a multiply mask (no divergence);
//  - erfc(beta r) = t P(t) exp(-beta^2 r^2) with t = 1/(1 + p beta r) and a
//    degree-7 polynomial P interpolated at set-up for this beta and rc
//    (relative error ~1e-7 on [0, beta rc]); the exponential is shared with
//    the force;
//  - cj4 halves without an exclusion mask take a path with no exclusion or
//    self-pair logic; energies are accumulated with compensated sums of
//    q_i (q_j h(r)) (no single rounded q_i q_j per type pair, whose error
//    would be systematic) and reduced in FP64; the Coulomb energies of
//    excluded pairs and the self terms are summed in FP64 (rigid molecules
//    repeat the same pair geometry, so their float rounding would not average
//    out) by work items of 128 atoms interleaved with the list entries in the
//    same queue (k_excl_energy, a separate kernel, only for LJ-PME);
//  - a force evaluation is three launches: k_convert_x (clears the
//    accumulators), k_force or k_force_x2, k_reduce_f (its last block writes
//    the energies and the virial);
//  - j forces are reduced over the 8 i-lanes with shuffles and added with one
//    vector red.global.add.v4.f32 per j-atom; i forces stay in registers
//    until the entry ends; shift forces and energies are reduced in FP64.
#include "../../include/nbnxm_gb300.h"
#include "nbx_internal.cuh"
#include "nbx_pair_core.cuh"

#include <algorithm>
#include <mutex>

namespace nbx
{
namespace
{

constexpr int kForceThreads   = 256;
constexpr int kForceMinBlocks = 2;
constexpr int kMaxTypes1      = 48;  // types + dummy held in shared memory (36 KB)
constexpr int kStageBytes     = kStageSmemPerWarp;  // per warp: double-buffered j stage and barriers

constexpr int kExclThreads      = 256;
constexpr int kExclBlocksPerSm = 4;

template<bool kEnergy, bool kEwald, int kLj = 0>
__global__ void __launch_bounds__(kForceThreads, kForceMinBlocks) k_force(DeviceView v, int* work_counter)
{
    // {6*C6, 12*C12, LJ energy shift of the pair, LJ-PME grid 6*C6 (geometric)} per type pair
    extern __shared__ float4 nbfp_s[];
    const int nt1 = v.ntypes1;
    for (int k = threadIdx.x; k < nt1 * nt1; k += blockDim.x)
    {
        const float2 p = v.nbfp[k];
        // LJ-PME grid: sqrt(6 C6_ii) sqrt(6 C6_jj), the reference's nbfp_comb product (geometric rule)
        float c6grid = 0.0f;
        if (kLj == 3)
        {
            const int ti = k / nt1, tj = k % nt1;
            c6grid       = sqrtf(v.nbfp[ti * nt1 + ti].x) * sqrtf(v.nbfp[tj * nt1 + tj].x);
        }
        // (12C12 cpot12)/12 - (6C6 cpot6)/6 (kernel_gpu_ref.cpp:327-336)
        nbfp_s[k] = make_float4(p.x, p.y, p.y * v.cpot12 * (1.0f / 12.0f) - p.x * v.cpot6 * (1.0f / 6.0f), c6grid);
    }
    __syncthreads();
    if (v.hdr->status & (kStatusListOverflow | kStatusExclOverflow | kStatusGridOverflow))
    {
        return;
    }
    const unsigned full    = 0xffffffffu;
    const int      lane    = threadIdx.x & 31;
    const int      ii      = lane & 7;   // i-atom within the i-cluster
    const int      jj      = lane >> 3;  // j-atom within the warp half
    const int      numSci  = v.hdr->num_sci;
    // per-warp double-buffered j stage (bulk copies), after the type table
    JStage js = stage_carve(nbfp_s, nt1 * nt1, threadIdx.x >> 5, blockDim.x >> 5);
    stage_init(js, lane);
    const float    rc2     = v.rc2;
    const float    beta    = v.beta;
    const float    pbeta   = v.pbeta;
    const float    beta2l2 = v.beta2l2;  // beta^2 * log2(e)
    const float    c2b     = v.c2b;      // 2 beta / sqrt(pi)
    const float    k_rf2   = v.k_rf2;

    // per-lane FP64 energy sums, in shared memory: they change once per entry, and registers
    // are what the pair loop is short of
    __shared__ double e_acc_s[2][kForceThreads];
    double&           e_lj_acc = e_acc_s[0][threadIdx.x];
    double&           e_el_acc = e_acc_s[1][threadIdx.x];
    e_lj_acc                   = 0.0;
    e_el_acc                   = 0.0;
    // excluded-pair and self energies as work items of this queue (LJ-PME keeps its own kernel)
    const int numChunks = (kEnergy && kLj != 3) ? v.excl_chunks : 0;
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
            if (kEnergy && kLj != 3)
            {
                const double beta2  = (double)v.beta * (double)v.beta;
                double       excl_s = 0.0;  // Ewald series sums of this item
                for (int i = e * kExclChunkAtoms + lane; i < min(v.n, (e + 1) * kExclChunkAtoms); i += 32)
                {
                    double dummy_lj = 0.0;
                    excl_atom(v, v, i, false, beta2, e_el_acc, excl_s, dummy_lj);
                }
                e_el_acc = fma(excl_s, -(double)v.beta * 1.1283791670955125739, e_el_acc);
            }
            continue;
        }
        const Sci     s = v.sci[e];
        const SysPtrs p = { v.xq, v.tgrid, v.fnb, v.cj4, v.excl, v.shiftvec, v.fshift };
        if (!process_entry<kEnergy, kEwald, kLj>(v, p, s, nbfp_s, js, nt1, lane, ii, jj, rc2, pbeta, beta2l2, c2b,
                                                 k_rf2, e_lj_acc, e_el_acc))
        {
            stage_timeout(js, &v.hdr->status, lane);
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

__global__ void __launch_bounds__(kExclThreads) k_excl_energy(DeviceView v)
{
    double    acc    = 0.0;
    double    acc_lj = 0.0;  // LJ-PME: the grid part of excluded pairs
    double    acc_s  = 0.0;  // Ewald: sum of q_i q_j S(beta^2 r^2) over excluded pairs
    const bool ljpme = v.vdw_mod == NBX_VDW_LJPME;
    const double beta2 = (double)v.beta * (double)v.beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.n; i += gridDim.x * blockDim.x)
    {
        excl_atom(v, v, i, ljpme, beta2, acc, acc_s, acc_lj);
    }
    acc += acc_s * (-(double)v.beta * 1.1283791670955125739);
    // warp, then block sums: one atomic per block and sum (a few hundred blocks), not one per
    // warp, because same-address FP64 atomics serialise in L2
    __shared__ double part[2][kExclThreads / 32];
    for (int o = 16; o > 0; o >>= 1)
    {
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
        acc_lj += __shfl_xor_sync(0xffffffffu, acc_lj, o);
    }
    if ((threadIdx.x & 31) == 0)
    {
        part[0][threadIdx.x >> 5] = acc;
        part[1][threadIdx.x >> 5] = acc_lj;
    }
    __syncthreads();
    if (threadIdx.x < 2)
    {
        double t = 0.0;
        for (int w = 0; w < kExclThreads / 32; w++)
        {
            t += part[threadIdx.x][w];
        }
        if (t != 0.0)
        {
            if (threadIdx.x == 0)
            {
                atomicAdd(&v.energy[1], t * v.epsfac_d);
            }
            else
            {
                atomicAdd(&v.energy[0], t);
            }
        }
    }
}

int excl_blocks(int n, int num_sms)
{
    return std::max(1, std::min((n + kExclThreads - 1) / kExclThreads, kExclBlocksPerSm * num_sms));
}

// energies += self terms; virial = -1/2 (sum x (x) f + sum shift (x) fshift)
// (mdlib/sim_util.cpp:157-176, calcvir.cpp:103-145).  Threads t < 9 of one block; the sums are
// read past L1 (other blocks of the calling kernel added to them).
__device__ __forceinline__ void finish_sums(const DeviceView& v, double* d_energies, double* d_virial, int t)
{
    if (d_energies && t < 2)
    {
        d_energies[t] = __ldcg(&v.energy[t]) + (t == 1 ? v.self_energy : v.self_energy_lj);
    }
    if (d_virial && t < 9)
    {
        const int p = t / 3, q = t % 3;
        double    s = __ldcg(&v.virial[t]);
        for (int sh = 0; sh < kNShift; sh++)
        {
            s += (double)v.shiftvec[3 * sh + p] * __ldcg(&v.fshift[3 * sh + q]);
        }
        d_virial[t] = -0.5 * s;
    }
}

// f[a] = fnb[cells[a]] (atomdata.cpp:1181-1228) and sum_k x_k (x) f_k: each
// thread gathers kReduceAtoms atoms and sums their x (x) f in float, the
// partial sums are reduced in FP64.
constexpr int kReduceAtoms   = 4;
constexpr int kReduceThreads = 256;

__global__ void __launch_bounds__(kReduceThreads)
        k_reduce_f(DeviceView v, float* __restrict__ f, int do_virial, double* d_energies, double* d_virial, int stage)
{
    float w[9];
#pragma unroll
    for (int k = 0; k < 9; k++)
    {
        w[k] = 0.0f;
    }
    // all gathers first, then the stores: stores through f may alias the loads, so loads
    // written after a store would wait for it
    const int a0 = (blockIdx.x * kReduceThreads) * kReduceAtoms + threadIdx.x;
    int       ks[kReduceAtoms];
#pragma unroll
    for (int r = 0; r < kReduceAtoms; r++)
    {
        const int a = a0 + r * kReduceThreads;
        ks[r]       = a < v.n ? v.cells[a] : -1;
    }
    float4 fa[kReduceAtoms], xa[kReduceAtoms];
#pragma unroll
    for (int r = 0; r < kReduceAtoms; r++)
    {
        if (ks[r] >= 0)
        {
            fa[r] = v.fnb[ks[r]];
            if (do_virial)
            {
                xa[r] = v.xq[ks[r]];
            }
        }
    }
    if (do_virial)
    {
        // the virial of the nonbonded forces only (before any accumulation into f)
#pragma unroll
        for (int r = 0; r < kReduceAtoms; r++)
        {
            if (ks[r] >= 0)
            {
                const float xv[3] = { xa[r].x, xa[r].y, xa[r].z };
                const float fv[3] = { fa[r].x, fa[r].y, fa[r].z };
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
    if (stage)
    {
        // the block's forces through shared memory, written as contiguous floats: whole
        // sectors when f is host memory written over the host link
        __shared__ float sf[3 * kReduceThreads * kReduceAtoms];
#pragma unroll
        for (int r = 0; r < kReduceAtoms; r++)
        {
            if (ks[r] >= 0)
            {
                const int j   = threadIdx.x + r * kReduceThreads;
                sf[3 * j]     = fa[r].x;
                sf[3 * j + 1] = fa[r].y;
                sf[3 * j + 2] = fa[r].z;
            }
        }
        __syncthreads();
        const int base  = blockIdx.x * kReduceThreads * kReduceAtoms;
        const int count = 3 * min(kReduceThreads * kReduceAtoms, v.n - base);
        float*    fb    = f + 3 * (size_t)base;
        for (int i = threadIdx.x; i < count; i += kReduceThreads)
        {
            fb[i] = v.accumulate_f ? fb[i] + sf[i] : sf[i];
        }
    }
    else
    {
        if (v.accumulate_f)
        {
            float old[kReduceAtoms][3];
#pragma unroll
            for (int r = 0; r < kReduceAtoms; r++)
            {
                if (ks[r] >= 0)
                {
                    const int a = a0 + r * kReduceThreads;
                    old[r][0]   = f[3 * a];
                    old[r][1]   = f[3 * a + 1];
                    old[r][2]   = f[3 * a + 2];
                }
            }
#pragma unroll
            for (int r = 0; r < kReduceAtoms; r++)
            {
                fa[r].x += old[r][0];
                fa[r].y += old[r][1];
                fa[r].z += old[r][2];
            }
        }
#pragma unroll
        for (int r = 0; r < kReduceAtoms; r++)
        {
            if (ks[r] >= 0)
            {
                const int a  = a0 + r * kReduceThreads;
                f[3 * a]     = fa[r].x;
                f[3 * a + 1] = fa[r].y;
                f[3 * a + 2] = fa[r].z;
            }
        }
    }
    if (do_virial)
    {
        __shared__ double ws[9][32];
        const int         lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        // the warp's 128 atoms summed in float (FP64 arithmetic runs at a small fraction of the
        // FP32 rate on this GPU: 9 x 5 FP64 shuffle levels per warp cost several microseconds),
        // the warps' partials in FP64
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
            atomicAdd(&v.virial[threadIdx.x], t);
            __threadfence();
        }
    }
    if (!d_energies && !d_virial)
    {
        return;
    }
    // the last block to finish writes the energies and the virial (no separate launch)
    __shared__ int last;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        last = atomicAdd(reinterpret_cast<unsigned*>(&v.hdr->work_counter2), 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last)
    {
        __threadfence();
        // the shift-force part of the virial, sum_s shift_s (x) fshift_s: one warp per component
        // (8 warps, component 8 on warp 0), the 45 shifts over the lanes, a shuffle reduction
        __shared__ double sv[9];
        if (d_virial)
        {
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            for (int c = warp; c < 9; c += kReduceThreads / 32)
            {
                double t = 0.0;
                for (int sh = lane; sh < kNShift; sh += 32)
                {
                    t += (double)v.shiftvec[3 * sh + c / 3] * __ldcg(&v.fshift[3 * sh + c % 3]);
                }
                for (int o = 16; o > 0; o >>= 1)
                {
                    t += __shfl_xor_sync(0xffffffffu, t, o);
                }
                if (lane == 0)
                {
                    sv[c] = t + __ldcg(&v.virial[c]);
                }
            }
        }
        __syncthreads();
        if (d_energies && threadIdx.x < 2)
        {
            d_energies[threadIdx.x] = __ldcg(&v.energy[threadIdx.x])
                                      + (threadIdx.x == 1 ? v.self_energy : v.self_energy_lj);
        }
        if (d_virial && threadIdx.x < 9)
        {
            d_virial[threadIdx.x] = -0.5 * sv[threadIdx.x];
        }
    }
}

// energies += self term; virial = -1/2 (sum x (x) f + sum shift (x) fshift)
// (mdlib/sim_util.cpp:157-176, calcvir.cpp:103-145).
__global__ void k_finish(DeviceView v, double* d_energies, double* d_virial)
{
    finish_sums(v, d_energies, d_virial, threadIdx.x);
}

__global__ void k_pair_count(DeviceView v, unsigned long long* out)
{
    const int          j   = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long cnt = 0;
    if (j < v.hdr->num_cj4)
    {
        cnt = 32ull * (__popc(v.cj4[j].imei[0].imask) + __popc(v.cj4[j].imei[1].imask));
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0)
    {
        atomicAdd(out, cnt);
    }
}

__global__ void k_noalloc_init(ListHeader* hdr, int num_sci, int num_cells)
{
    hdr->num_sci      = num_sci;
    hdr->num_cells    = num_cells;
    hdr->status       = 0u;
    hdr->work_counter = 0;
}

__global__ void k_fma_probe(float* out, int iters)
{
    float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
    float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; i++)
    {
#pragma unroll
        for (int k = 0; k < 16; k++)
        {
            a0 = fmaf(a0, m, c);
            a1 = fmaf(a1, m, c);
            a2 = fmaf(a2, m, c);
            a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c);
            a5 = fmaf(a5, m, c);
            a6 = fmaf(a6, m, c);
            a7 = fmaf(a7, m, c);
        }
    }
    const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 12345.678f)
    {
        out[0] = s;
    }
}

template<bool kEnergy, bool kEwald, int kLj>
void launch_k_force(const DeviceView& v, int blocks, size_t smem, cudaStream_t s, int* counter)
{
    if (smem_optin<k_force<kEnergy, kEwald, kLj>>(smem + sizeof(double) * 2 * kForceThreads, smem) != cudaSuccess)
    {
        return;  // the launch error is reported by cudaGetLastError
    }
    k_force<kEnergy, kEwald, kLj><<<blocks, kForceThreads, smem, s>>>(v, counter);
}

// Marks the outputs of an allocation-free evaluation whose device status word is non-zero (a
// bounded stage wait gave up, or a capacity check failed): every force component, the energies
// and the virial become NaN, so a failed evaluation cannot pass for a correct one.
__global__ void k_noalloc_check(const ListHeader* hdr, float* f, int n3, double* d_energies, double* d_virial)
{
    if (__ldcg(&hdr->status) == 0u)
    {
        return;
    }
    const float nan = __int_as_float(0x7fc00000);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x)
    {
        f[i] = nan;
    }
    if (blockIdx.x == 0 && threadIdx.x < 9)
    {
        const double dnan = __longlong_as_double(0x7ff8000000000000ll);
        if (d_energies && threadIdx.x < 2)
        {
            d_energies[threadIdx.x] = dnan;
        }
        if (d_virial)
        {
            d_virial[threadIdx.x] = dnan;
        }
    }
}

} // namespace

cudaError_t launch_force(const DeviceView& v, bool energy, cudaStream_t s, int num_sms, cudaEvent_t ev0,
                         cudaEvent_t ev1)
{
    if (v.ntypes1 > kMaxTypes1)
    {
        return cudaErrorInvalidValue;
    }
    // the accumulators (grid forces, shift forces, energies, work queue) were cleared by the
    // coordinate conversion of this evaluation (launch_convert_x with clear)
    int* counter = &v.hdr->work_counter;
    const int    blocks = num_sms * kForceMinBlocks;
    const size_t smem   = sizeof(float4) * (size_t)v.ntypes1 * v.ntypes1 + kStageBytes * (kForceThreads / 32);
    const bool   ewald  = (v.coulomb == 0);
    // the energy flavours take the excluded-pair and self energies as work items, except LJ-PME
    // (its excluded pairs need the FP64 grid term: a separate kernel)
    DeviceView kv = v;
    kv.excl_chunks = 0;
    if (energy && v.vdw_mod == NBX_VDW_LJPME)
    {
        k_excl_energy<<<excl_blocks(v.n, num_sms), kExclThreads, 0, s>>>(v);
    }
    else if (energy)
    {
        kv.excl_chunks = (v.n + kExclChunkAtoms - 1) / kExclChunkAtoms;
    }
    if (ev0)
    {
        cudaEventRecord(ev0, s);
    }
    // the switch modifiers have their own instantiations; shift and plain cut-off share one
    const int lj = (v.vdw_mod == NBX_VDW_FORCESWITCH) ? 1
                   : (v.vdw_mod == NBX_VDW_POTSWITCH) ? 2
                   : (v.vdw_mod == NBX_VDW_LJPME)     ? 3
                                                       : 0;
    if (lj == 0 && v.pair_core == 1)
    {
        // the packed core (potential shift or plain cut-off)
        launch_force_x2(kv, energy, s, num_sms, counter);
        if (ev1)
        {
            cudaEventRecord(ev1, s);
        }
        return cudaGetLastError();
    }
    using Launch = void (*)(const DeviceView&, int, size_t, cudaStream_t, int*);
    // [lj][energy][ewald]
    static const Launch table[4][2][2] = {
        { { launch_k_force<false, false, 0>, launch_k_force<false, true, 0> },
          { launch_k_force<true, false, 0>, launch_k_force<true, true, 0> } },
        { { launch_k_force<false, false, 1>, launch_k_force<false, true, 1> },
          { launch_k_force<true, false, 1>, launch_k_force<true, true, 1> } },
        { { launch_k_force<false, false, 2>, launch_k_force<false, true, 2> },
          { launch_k_force<true, false, 2>, launch_k_force<true, true, 2> } },
        { { launch_k_force<false, false, 3>, launch_k_force<false, true, 3> },
          { launch_k_force<true, false, 3>, launch_k_force<true, true, 3> } },
    };
    table[lj][energy ? 1 : 0][ewald ? 1 : 0](kv, blocks, smem, s, counter);
    if (ev1)
    {
        cudaEventRecord(ev1, s);
    }
    return cudaGetLastError();
}

cudaError_t launch_reduce_f(const DeviceView& v, float* d_f, double* d_e, double* d_vir, cudaStream_t s, bool stage)
{
    const int per_block = kReduceThreads * kReduceAtoms;
    k_reduce_f<<<(v.n + per_block - 1) / per_block, kReduceThreads, 0, s>>>(v, d_f, d_vir ? 1 : 0, d_e, d_vir,
                                                                           stage ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_pair_count(const DeviceView& v, unsigned long long* d_out, cudaStream_t s)
{
    cudaMemsetAsync(d_out, 0, sizeof(unsigned long long), s);
    k_pair_count<<<(v.cj4_cap + 255) / 256, 256, 0, s>>>(v, d_out);
    return cudaGetLastError();
}

cudaError_t measure_fp32_peak(double* tflops)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float* out = nullptr;
    if (cudaMalloc(&out, sizeof(float)) != cudaSuccess)
    {
        return cudaErrorMemoryAllocation;
    }
    const int blocks = sms * 8, threads = 256, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma_probe<<<blocks, threads>>>(out, 64);  // warm-up
    cudaEventRecord(e0);
    k_fma_probe<<<blocks, threads>>>(out, iters);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float       ms  = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
    *tflops            = flops / (ms * 1e-3) / 1e12;
    return err;
}


// ---------------------------------------------------------------------------
// Allocation-free force evaluation (nbx_compute_noalloc).
//
// The scratch this evaluation needs -- the grid-order force accumulator, the
// FP64 energy / shift-force / virial sums and the work-queue header -- lives
// in one file-scope device array, so the entry point calls no cudaMalloc,
// cudaFree or allocating library routine.  That array is a host-side stand-in
// in host code; its device address is fetched once per device with
// cudaGetSymbolAddress (see noalloc_scratch_address).  Every call shares it.
constexpr int    kNoAllocMaxSlots  = 65536;  // grid slots (padded atoms): 1 MiB of float4
constexpr size_t kNoAllocFnbBytes  = sizeof(float4) * (size_t)kNoAllocMaxSlots;
constexpr size_t kNoAllocSumsBytes = sizeof(double) * (2 + kNShift * 3 + 9);
constexpr size_t kNoAllocBytes     = kNoAllocFnbBytes + 256 + kNoAllocSumsBytes + 256 + sizeof(ListHeader);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace
{
constexpr int kMaxDevices = 64;
std::mutex    g_noalloc_mutex;
// failure-detection test hook (nbx_noalloc_set_wait_test): bytes the stage barriers wait for in vain
unsigned      g_noalloc_wait_test = 0u;
void*         g_noalloc_addr[kMaxDevices] = { nullptr };

// Device address of the scratch array on the current device (set-up on the
// first call per device).
cudaError_t noalloc_scratch_address(unsigned char** out)
{
    int         dev = 0;
    cudaError_t e   = cudaGetDevice(&dev);
    if (e != cudaSuccess)
    {
        return e;
    }
    if (dev < 0 || dev >= kMaxDevices)
    {
        return cudaErrorInvalidDevice;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev])
    {
        void* ptr = nullptr;
        e         = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess)
        {
            return e;
        }
        g_noalloc_addr[dev] = ptr;
    }
    *out = static_cast<unsigned char*>(g_noalloc_addr[dev]);
    return cudaSuccess;
}
} // namespace

} // namespace nbx

extern "C" int nbx_compute_noalloc(const nbx_noalloc_args* a, float* d_f, double* d_energies, double* d_virial,
                                   void* stream)
{
    using namespace nbx;
    if (!a || !d_f || !a->xq || !a->types || !a->nbfp || !a->cells || !a->sci || !a->cj4 || !a->excl)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    // the grid holds every atom, in whole 64-slot cells
    if (a->num_atoms <= 0 || a->num_slots <= 0 || a->num_sci < 0 || a->num_types <= 0
        || a->num_types + 1 > kMaxTypes1 || a->num_atoms > a->num_slots || a->num_slots % kSc != 0)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (a->num_slots > kNoAllocMaxSlots)
    {
        return NBX_ERR_LIST_OVERFLOW;  // the fixed scratch holds kNoAllocMaxSlots grid slots
    }
    const bool energy = (d_energies != nullptr) || (d_virial != nullptr);
    if (energy && (!a->excl_index || !a->excl_list))
    {
        return NBX_ERR_INVALID_INPUT;
    }
    if (!(a->rcoulomb > 0.0f) || !(a->rlist >= a->rcoulomb) || a->coulomb < 0 || a->coulomb > 2)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    // the force kernel copies j-clusters with bulk copies: 16-byte aligned sources
    if ((reinterpret_cast<uintptr_t>(a->xq) & 15u) != 0 || (reinterpret_cast<uintptr_t>(a->types) & 15u) != 0)
    {
        return NBX_ERR_INVALID_INPUT;
    }
    unsigned char* base = nullptr;
    if (noalloc_scratch_address(&base) != cudaSuccess)
    {
        return NBX_ERR_CUDA;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    DeviceView v{};
    v.n          = a->num_atoms;
    v.q          = nullptr;
    v.type       = nullptr;
    v.excl_index = a->excl_index;
    v.excl_list  = a->excl_list;
    v.ntypes1    = a->num_types + 1;
    v.nbfp       = reinterpret_cast<const float2*>(a->nbfp);
    v.xq         = const_cast<float4*>(reinterpret_cast<const float4*>(a->xq));
    v.tgrid      = const_cast<int*>(a->types);
    v.cells      = const_cast<int*>(a->cells);
    v.sci        = const_cast<Sci*>(reinterpret_cast<const Sci*>(a->sci));
    v.cj4        = const_cast<Cj4*>(reinterpret_cast<const Cj4*>(a->cj4));
    v.excl       = const_cast<Excl*>(reinterpret_cast<const Excl*>(a->excl));
    v.fnb        = reinterpret_cast<float4*>(base);
    double* sums = reinterpret_cast<double*>(base + kNoAllocFnbBytes + 256);
    v.energy     = sums;
    v.fshift     = sums + 2;
    v.virial     = sums + 2 + kNShift * 3;
    v.hdr        = reinterpret_cast<ListHeader*>(base + kNoAllocFnbBytes + 256 + kNoAllocSumsBytes + 256);
    v.wait_test_bytes = g_noalloc_wait_test;
    for (int d = 0; d < 3; d++)
    {
        v.g.box[d] = a->box[d];
    }
    v.g.cells_capacity = a->num_slots / kSc;
    // interaction constants, as in nbx_create (api/nblib/gmxsetup.cpp:226-284)
    const float rc = a->rcoulomb;
    v.coulomb      = a->coulomb;
    v.rc2          = rc * rc;
    v.rlist        = a->rlist;
    v.rlist2       = a->rlist * a->rlist;
    v.epsfac       = (float)one_4pi_eps0();
    v.epsfac_d     = one_4pi_eps0();
    set_lj_modifier(v, NBX_VDW_POTSHIFT, rc, 0.0f);
    const float eps_rf = (a->coulomb == NBX_COULOMB_CUTOFF) ? 1.0f : a->epsilon_rf;
    v.k_rf = (eps_rf == 0) ? 1 / (2 * rc * rc * rc) : (eps_rf - 1.0f) / (2 * eps_rf + 1.0f) / (rc * rc * rc);
    v.c_rf = 1 / rc + v.k_rf * rc * rc;
    if (a->coulomb == NBX_COULOMB_EWALD)
    {
        v.beta     = calc_ewaldcoeff_q(rc, a->ewald_rtol > 0.0f ? a->ewald_rtol : 1e-5f);
        v.sh_ewald = a->use_ewald_shift ? erfcf(v.beta * rc) / rc : 0.0f;
        if ((double)v.beta * (double)rc > (double)kErfcXMax)
        {
            return NBX_ERR_INVALID_INPUT;
        }
        v.erfc_p = kErfcP;
    }
    set_pair_constants(v);
    v.self_energy    = 0.0;
    v.self_on_device = 1;
    for (int sh = 0, m = -1; m <= 1; m++)
    {
        for (int l = -1; l <= 1; l++)
        {
            for (int k = -2; k <= 2; k++, sh++)
            {
                v.shiftvec[3 * sh + 0] = k * a->box[0];
                v.shiftvec[3 * sh + 1] = l * a->box[1];
                v.shiftvec[3 * sh + 2] = m * a->box[2];
            }
        }
    }
    // the array keeps the previous call's contents: clear what must start at zero
    k_noalloc_init<<<1, 1, 0, s>>>(v.hdr, a->num_sci, a->num_slots / kSc);
    cudaError_t e = cudaMemsetAsync(v.fnb, 0, sizeof(float4) * (size_t)a->num_slots, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(sums, 0, kNoAllocSumsBytes, s);
    int num_sms = 0, dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
    {
        const int    blocks = num_sms * kForceMinBlocks;
        const size_t smem   = sizeof(float4) * (size_t)v.ntypes1 * v.ntypes1 + kStageBytes * (kForceThreads / 32);
        int*         ctr    = &v.hdr->work_counter;
        if (energy)
        {
            k_excl_energy<<<excl_blocks(v.n, num_sms), kExclThreads, 0, s>>>(v);
            if (v.coulomb == 0)
            {
                launch_k_force<true, true, 0>(v, blocks, smem, s, ctr);
            }
            else
            {
                launch_k_force<true, false, 0>(v, blocks, smem, s, ctr);
            }
        }
        else if (v.coulomb == 0)
        {
            launch_k_force<false, true, 0>(v, blocks, smem, s, ctr);
        }
        else
        {
            launch_k_force<false, false, 0>(v, blocks, smem, s, ctr);
        }
        k_reduce_f<<<(v.n + kReduceThreads * kReduceAtoms - 1) / (kReduceThreads * kReduceAtoms), kReduceThreads, 0, s>>>(
                v, d_f, d_virial ? 1 : 0, nullptr, nullptr, 0);
        if (energy)
        {
            k_finish<<<1, 32, 0, s>>>(v, d_energies, d_virial);
        }
        k_noalloc_check<<<std::min(num_sms, (3 * v.n + 255) / 256), 256, 0, s>>>(v.hdr, d_f, 3 * v.n, d_energies,
                                                                                 d_virial);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? NBX_OK : NBX_ERR_CUDA;
}

extern "C" int nbx_noalloc_status(void* stream)
{
    using namespace nbx;
    unsigned char* base = nullptr;
    if (noalloc_scratch_address(&base) != cudaSuccess)
    {
        return NBX_ERR_CUDA;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the status word sits in the scratch array's header; a synchronous read into a host
    // variable (pageable: no pinned buffer is allocated)
    const ListHeader* hdr = reinterpret_cast<const ListHeader*>(base + kNoAllocFnbBytes + 256 + kNoAllocSumsBytes + 256);
    unsigned          st  = 0u;
    cudaError_t       e   = cudaStreamSynchronize(s);
    if (e == cudaSuccess)
    {
        e = cudaMemcpy(&st, &hdr->status, sizeof(unsigned), cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess)
    {
        return NBX_ERR_CUDA;
    }
    if (st & (kStatusListOverflow | kStatusExclOverflow | kStatusGridOverflow))
    {
        return NBX_ERR_LIST_OVERFLOW;
    }
    if (st & kStatusTimeout)
    {
        return NBX_ERR_TIMEOUT;
    }
    return st ? NBX_ERR_INVALID_INPUT : NBX_OK;
}

extern "C" int nbx_noalloc_set_wait_test(int enable)
{
    nbx::g_noalloc_wait_test = enable ? 16u : 0u;
    return NBX_OK;
}
