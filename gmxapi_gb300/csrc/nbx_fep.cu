// Free-energy (perturbed) nonbonded pairs on the GPU.
//
// Restates nb_free_energy_kernel (src/gromacs/gmxlib/nonbonded/nb_free_energy.cpp:200-850) for
// the pairs with at least one perturbed atom: lambda-weighted state A / B Coulomb (Ewald real
// space or reaction field) and Lennard-Jones (potential shift or plain cut-off), Beutler soft-core
// with sc-r-power 6 and sc-power 1 or 2, dV/dlambda for Coulomb and LJ, excluded pairs (reaction
// field terms, Ewald reciprocal-space subtraction) and the perturbed atoms' self terms.
//
// The reference runs this on the CPU over a separate perturbed-pair list built by the search.
// Here the perturbed atoms are masked out of the cluster path (charge 0, all-zero LJ type; their
// self terms leave the handle's self energy) and one block per perturbed atom finds its partners
// in the grid cells within rlist of it (minimum image: the box is at least 2 rlist), computes
// each pair once (a pair of two perturbed atoms by the lower index) and adds the forces to the
// grid-order force buffer before the reduction, the i-forces per periodic shift to the shift
// forces (so the virial follows), energies and dV/dlambda in FP64.
#include "nbx_internal.cuh"

#include <cuda_runtime.h>

namespace nbx
{
namespace
{

constexpr int kFepWarps   = 8;
constexpr int kFepMaxExcl = 64;  // exclusions of one perturbed atom kept in shared memory

struct FepAcc
{
    float vc, vv, dc, dv;
};

__device__ __forceinline__ void red_v4(float4* addr, float x, float y, float z)
{
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(x), "f"(y), "f"(z), "f"(0.0f));
}

__device__ __forceinline__ int shift_index(int sx, int sy, int sz)
{
    return ((sz + 1) * 3 + (sy + 1)) * 5 + (sx + 2);
}

// erf(beta r)/r and -(d/dr)(erf(beta r)/r)/r, the reciprocal-space part the kernel subtracts
__device__ __forceinline__ void ewald_lr(const DeviceView& v, float rsq, float* v_lr, float* f_lr)
{
    if (rsq > 0.0f)
    {
        const float rinv = rsqrtf(rsq);
        const float r    = rsq * rinv;
        const float br   = v.beta * r;
        *v_lr            = erff(br) * rinv;
        *f_lr            = (*v_lr - v.c2b * expf(-br * br)) * rinv * rinv;
    }
    else
    {
        *v_lr = v.c2b;  // the r -> 0 limit 2 beta / sqrt(pi)
        *f_lr = 0.0f;
    }
}

// An included pair, both states (nb_free_energy.cpp:455-645).  Returns F/r (times dx: force on i).
template<bool kEwald>
__device__ float fep_pair(const DeviceView& v, const FepView& fp, float rsq, const float qq[2], const float2 nb[2],
                          FepAcc& acc)
{
    const float rinv = rsq > 0.0f ? rsqrtf(rsq) : 0.0f;
    const float r    = rsq * rinv;
    float       rpm2, rp, a_v = 0.0f, a_c = 0.0f;
    if (fp.soft)
    {
        rpm2 = rsq * rsq;
        rp   = rpm2 * rsq;
        // soft-core only when one end state has no repulsion (:502-509)
        const bool both = nb[0].y > 0.0f && nb[1].y > 0.0f;
        a_v             = both ? 0.0f : fp.alpha_v;
        a_c             = both ? 0.0f : fp.alpha_c;
    }
    else
    {
        rpm2 = rinv * rinv;
        rp   = 1.0f;
    }
    float Fscal = 0.0f;
#pragma unroll
    for (int s = 0; s < 2; s++)
    {
        const float c6 = nb[s].x, c12 = nb[s].y;
        if (qq[s] == 0.0f && c6 == 0.0f && c12 == 0.0f)
        {
            continue;
        }
        float sig6 = 0.0f, rpinvC = 1.0f, rpinvV = 1.0f, rinvC = rinv, rC = r, rinvV = rinv, rV = r;
        if (fp.soft)
        {
            sig6   = (c6 > 0.0f && c12 > 0.0f) ? fmaxf(0.5f * c12 / c6, fp.sigma6_min) : fp.sigma6_def;
            rpinvC = 1.0f / (a_c * fp.lfac_c[s] * sig6 + rp);
            rC     = rsqrtf(cbrtf(rpinvC));  // (1 / rpinvC)^(1/6)
            rinvC  = 1.0f / rC;
            rpinvV = 1.0f / (a_v * fp.lfac_v[s] * sig6 + rp);
            rV     = rsqrtf(cbrtf(rpinvV));
            rinvV  = 1.0f / rV;
        }
        float Vc = 0.0f, FC = 0.0f, Vv = 0.0f, FV = 0.0f;
        if (qq[s] != 0.0f && (kEwald ? rsq < v.rc2 : rC * rC < v.rc2))
        {
            if (kEwald)
            {
                Vc = qq[s] * (rinvC - v.sh_ewald);
                FC = qq[s] * rinvC;
            }
            else
            {
                Vc = qq[s] * (rinvC + v.k_rf * rC * rC - v.c_rf);
                FC = qq[s] * (rinvC - 2.0f * v.k_rf * rC * rC);
            }
        }
        if ((c6 != 0.0f || c12 != 0.0f) && rV * rV < v.rc2)
        {
            float rinv6;
            if (fp.soft)
            {
                rinv6 = rpinvV;
            }
            else
            {
                const float r2i = rinvV * rinvV;
                rinv6           = r2i * r2i * r2i;
            }
            const float v6  = c6 * rinv6;
            const float v12 = c12 * rinv6 * rinv6;
            Vv              = (v12 + c12 * v.cpot12) * (1.0f / 12.0f) - (v6 + c6 * v.cpot6) * (1.0f / 6.0f);
            FV              = v12 - v6;
        }
        FC *= rpinvC;
        FV *= rpinvV;
        const float dlf = s == 0 ? -1.0f : 1.0f;
        acc.vc += fp.lfc[s] * Vc;
        acc.vv += fp.lfv[s] * Vv;
        Fscal += (fp.lfc[s] * FC + fp.lfv[s] * FV) * rpm2;
        acc.dc += Vc * dlf + (fp.soft ? fp.lfc[s] * a_c * fp.dlfac_c[s] * FC * sig6 : 0.0f);
        acc.dv += Vv * dlf + (fp.soft ? fp.lfv[s] * a_v * fp.dlfac_v[s] * FV * sig6 : 0.0f);
    }
    if (kEwald)
    {
        // the reciprocal-space part, subtracted on r for pairs within rc (:669-723)
        float v_lr, f_lr;
        ewald_lr(v, rsq, &v_lr, &f_lr);
#pragma unroll
        for (int s = 0; s < 2; s++)
        {
            const float dlf = s == 0 ? -1.0f : 1.0f;
            acc.vc -= fp.lfc[s] * qq[s] * v_lr;
            Fscal -= fp.lfc[s] * qq[s] * f_lr;
            acc.dc -= dlf * qq[s] * v_lr;
        }
    }
    return Fscal;
}

// An excluded pair within rc: reaction-field terms or the Ewald reciprocal-space subtraction.
template<bool kEwald>
__device__ float fep_excluded(const DeviceView& v, const FepView& fp, float rsq, const float qq[2], FepAcc& acc)
{
    float Fscal = 0.0f;
    if (kEwald)
    {
        float v_lr, f_lr;
        ewald_lr(v, rsq, &v_lr, &f_lr);
#pragma unroll
        for (int s = 0; s < 2; s++)
        {
            const float dlf = s == 0 ? -1.0f : 1.0f;
            acc.vc -= fp.lfc[s] * qq[s] * v_lr;
            Fscal -= fp.lfc[s] * qq[s] * f_lr;
            acc.dc -= dlf * qq[s] * v_lr;
        }
    }
    else
    {
        const float VV = v.k_rf * rsq - v.c_rf;
        const float FF = -2.0f * v.k_rf;
#pragma unroll
        for (int s = 0; s < 2; s++)
        {
            const float dlf = s == 0 ? -1.0f : 1.0f;
            acc.vc += fp.lfc[s] * qq[s] * VV;
            Fscal += fp.lfc[s] * qq[s] * FF;
            acc.dc += dlf * qq[s] * VV;
        }
    }
    return Fscal;
}

__device__ __forceinline__ bool excluded_from(int aj, const int* exl, int nex, const int* excl_list, int e0, int e1)
{
    for (int k = 0; k < nex; k++)
    {
        if (exl[k] == aj)
        {
            return true;
        }
    }
    for (int k = e0 + nex; k < e1; k++)  // beyond the shared-memory copy
    {
        if (excl_list[k] == aj)
        {
            return true;
        }
    }
    return false;
}

// minimum-image separation of i from j (grid positions) and the shift index of i's image
__device__ __forceinline__ int min_image(const DeviceView& v, float4 xi, float4 xj, float* d)
{
    const float L[3]  = { v.g.box[0], v.g.box[1], v.g.box[2] };
    const float xv[3] = { xi.x - xj.x, xi.y - xj.y, xi.z - xj.z };
    int         n[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        const float t = rintf(xv[k] / L[k]);
        n[k]          = (int)t;
        d[k]          = xv[k] - t * L[k];
    }
    // i's image is x_i - n L; shifts outside the table (coordinates far from the box) get no
    // shift-force entry
    if (n[0] < -2 || n[0] > 2 || n[1] < -1 || n[1] > 1 || n[2] < -1 || n[2] > 1)
    {
        return -1;
    }
    return shift_index(-n[0], -n[1], -n[2]);
}

// One block per perturbed atom.  Its warps take the grid columns within rlist in turn; in a
// column the lanes test 32 cells' z ranges (bbcz, periodic) at once and the warp then walks the
// 64 slots of each cell in range (2 per lane).  The i-force is added once per warp, the shift
// forces and energies once per block.
template<bool kEwald>
__global__ void __launch_bounds__(kFepWarps * 32) k_fep(DeviceView v, FepView fp, int energy)
{
    __shared__ float  fsh[kNShift * 3];
    __shared__ int    exl[kFepMaxExcl];
    __shared__ double esum[kFepWarps][4];
    const int         lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (int k = threadIdx.x; k < kNShift * 3; k += blockDim.x)
    {
        fsh[k] = 0.0f;
    }
    const int    ai  = fp.plist[blockIdx.x];
    const int    si  = v.cells[ai];
    const float4 xi  = v.xq[si];
    const float  qAi = v.epsfac * fp.qA[ai], qBi = v.epsfac * fp.qB[ai];
    const int    tAi = fp.tA[ai], tBi = fp.tB[ai];
    const int    e0 = v.excl_index[ai], e1 = v.excl_index[ai + 1];
    const int    nex = min(e1 - e0, kFepMaxExcl);
    for (int k = threadIdx.x; k < nex; k += blockDim.x)
    {
        exl[k] = v.excl_list[e0 + k];
    }
    __syncthreads();
    FepAcc acc{ 0.0f, 0.0f, 0.0f, 0.0f };
    float  fi[3] = { 0.0f, 0.0f, 0.0f };

    // one pair: j at grid slot `slot`, atom aj, not excluded, not the atom itself
    auto pair = [&](int slot, int aj) {
        float       d[3];
        const int   sh  = min_image(v, xi, v.xq[slot], d);
        const float rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (rsq >= v.rc2)
        {
            return;
        }
        const int    tAj   = fp.tA[aj], tBj = fp.tB[aj];
        const float  qq[2] = { qAi * fp.qA[aj], qBi * fp.qB[aj] };
        const float2 nb[2] = { v.nbfp[tAi * v.ntypes1 + tAj], v.nbfp[tBi * v.ntypes1 + tBj] };
        const float  F     = fep_pair<kEwald>(v, fp, rsq, qq, nb, acc);
        const float  tx = F * d[0], ty = F * d[1], tz = F * d[2];
        fi[0] += tx;
        fi[1] += ty;
        fi[2] += tz;
        red_v4(&v.fnb[slot], -tx, -ty, -tz);
        if (energy && sh >= 0)
        {
            atomicAdd(&fsh[3 * sh + 0], tx);
            atomicAdd(&fsh[3 * sh + 1], ty);
            atomicAdd(&fsh[3 * sh + 2], tz);
        }
    };

    // grid columns within rlist of the atom (periodic; every column once when the range wraps)
    const float rl  = v.rlist;
    const int   ncx = v.g.ncx, ncy = v.g.ncy;
    int         cx0 = (int)floorf((xi.x - rl) * v.g.ics[0]);
    int         nxc = (int)floorf((xi.x + rl) * v.g.ics[0]) - cx0 + 1;
    int         cy0 = (int)floorf((xi.y - rl) * v.g.ics[1]);
    int         nyc = (int)floorf((xi.y + rl) * v.g.ics[1]) - cy0 + 1;
    if (nxc >= ncx)
    {
        cx0 = 0;
        nxc = ncx;
    }
    if (nyc >= ncy)
    {
        cy0 = 0;
        nyc = ncy;
    }
    const float Lz = v.g.box[2];
    for (int c = wib; c < nxc * nyc; c += kFepWarps)
    {
        const int cx   = ((cx0 + c / nyc) % ncx + ncx) % ncx;
        const int cy   = ((cy0 + c % nyc) % ncy + ncy) % ncy;
        const int col  = cx * ncy + cy;
        const int c0   = v.cxy_ind[col], c1 = v.cxy_ind[col + 1];
        for (int cb = c0; cb < c1; cb += 32)
        {
            bool near = false;
            if (cb + lane < c1)
            {
                const float2 z = v.bbcz[cb + lane];
                for (int k = -1; k <= 1; k++)
                {
                    near |= (z.y + k * Lz >= xi.z - rl) && (z.x + k * Lz <= xi.z + rl);
                }
            }
            unsigned todo = __ballot_sync(0xffffffffu, near);
            while (todo)
            {
                const int cell = cb + __ffs(todo) - 1;
                todo &= todo - 1;
                for (int k = lane; k < kSc; k += 32)
                {
                    const int slot = cell * kSc + k;
                    const int aj   = v.atom_indices[slot];
                    if (aj < 0 || aj == ai || (fp.pert[aj] && aj < ai)
                        || excluded_from(aj, exl, nex, v.excl_list, e0, e1))
                    {
                        continue;
                    }
                    pair(slot, aj);
                }
            }
        }
    }
    // excluded pairs within rc, and the self pair (warp 0)
    if (wib == 0)
    {
        for (int k = e0 + lane; k < e1; k += 32)
        {
            const int aj = v.excl_list[k];
            if (aj < 0 || aj >= v.n || aj == ai || (fp.pert[aj] && aj < ai))
            {
                continue;
            }
            const int   sj = v.cells[aj];
            float       d[3];
            const int   sh  = min_image(v, xi, v.xq[sj], d);
            const float rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (rsq >= v.rc2)
            {
                continue;
            }
            const float qq[2] = { qAi * fp.qA[aj], qBi * fp.qB[aj] };
            const float F     = fep_excluded<kEwald>(v, fp, rsq, qq, acc);
            const float tx = F * d[0], ty = F * d[1], tz = F * d[2];
            fi[0] += tx;
            fi[1] += ty;
            fi[2] += tz;
            red_v4(&v.fnb[sj], -tx, -ty, -tz);
            if (energy && sh >= 0)
            {
                atomicAdd(&fsh[3 * sh + 0], tx);
                atomicAdd(&fsh[3 * sh + 1], ty);
                atomicAdd(&fsh[3 * sh + 2], tz);
            }
        }
        // half of the r = 0 excluded term (nb_free_energy.cpp:696-706)
        if (lane == 0)
        {
            const float vself  = kEwald ? v.c2b : v.c_rf;
            const float qqs[2] = { qAi * fp.qA[ai], qBi * fp.qB[ai] };
#pragma unroll
            for (int s = 0; s < 2; s++)
            {
                const float dlf = s == 0 ? -1.0f : 1.0f;
                acc.vc -= 0.5f * fp.lfc[s] * qqs[s] * vself;
                acc.dc -= 0.5f * dlf * qqs[s] * vself;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        for (int o = 16; o > 0; o >>= 1)
        {
            fi[k] += __shfl_xor_sync(0xffffffffu, fi[k], o);
        }
    }
    if (lane == 0 && (fi[0] != 0.0f || fi[1] != 0.0f || fi[2] != 0.0f))
    {
        red_v4(&v.fnb[si], fi[0], fi[1], fi[2]);
    }
    if (!energy)
    {
        return;
    }
    double e[4] = { acc.vc, acc.vv, acc.dc, acc.dv };
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
        for (int o = 16; o > 0; o >>= 1)
        {
            e[k] += __shfl_xor_sync(0xffffffffu, e[k], o);
        }
        if (lane == 0)
        {
            esum[wib][k] = e[k];
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kNShift * 3; k += blockDim.x)
    {
        if (fsh[k] != 0.0f)
        {
            atomicAdd(&v.fshift[k], (double)fsh[k]);
        }
    }
    if (threadIdx.x < 4)
    {
        double t = 0.0;
        for (int w = 0; w < kFepWarps; w++)
        {
            t += esum[w][threadIdx.x];
        }
        atomicAdd(&fp.sums[threadIdx.x], t);
        if (threadIdx.x < 2)
        {
            atomicAdd(&v.energy[1 - threadIdx.x], t);  // V_Coulomb -> energy[1], V_LJ -> energy[0]
        }
    }
}

} // namespace

cudaError_t launch_fep(const DeviceView& v, const FepView& fp, bool energy, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(fp.sums, 0, sizeof(double) * 4, s);
    if (e != cudaSuccess || fp.np == 0)
    {
        return e;
    }
    if (v.coulomb == 0)
    {
        k_fep<true><<<fp.np, kFepWarps * 32, 0, s>>>(v, fp, energy ? 1 : 0);
    }
    else
    {
        k_fep<false><<<fp.np, kFepWarps * 32, 0, s>>>(v, fp, energy ? 1 : 0);
    }
    return cudaGetLastError();
}

} // namespace nbx
