// Adjoint of the cluster-pair force / energy kernel.
//
// There is no counterpart in the reference (it only computes forces).  Given
// upstream gradients G_i = dL/dF_i on the forces and gE = dL/dE on the LJ and
// Coulomb energies, one pass over the same pair list recomputes every pair
// term (nothing from the forward pass is stored) and accumulates
//   dL/dx  (a Hessian-vector product with G, plus -gE times the forces),
//   dL/dq  per atom,
//   dL/d(6 C6), dL/d(12 C12) per type pair (FP64 sums).
// For a pair with r = x_i - x_j (+ shift), s = r^2, force on i f = phi(s) r and
// g = G_i - G_j:
//   dL/dr = phi g + (2 phi'(s) (g.r) - gE_lj phi_lj - gE_c qq psi) r,
// with phi = phi_lj + qq psi, phi_lj = (12C12 r^-12 - 6C6 r^-6) / r^2 and, for
// Ewald, psi = erfc(br)/r^3 + (2b/sqrt(pi)) e^{-b^2 r^2}/r^2 (minus 1/r^3 for an
// excluded pair), whose derivative is psi' = -(1.5 psi + (2b/sqrt(pi)) b^2
// e^{-b^2 r^2}) / r^2 for normal and excluded pairs alike.
//
// Layout: as the forward kernel (persistent warps, one list entry per warp,
// lane = j-atom-of-half * 8 + i-atom); the entry's shifted i-atoms and their
// upstream gradients are staged in shared memory, the per-lane i accumulators
// (dx, dy, dz, dq per i-cluster) stay in registers; j accumulators are reduced
// over the 8 i-lanes and added with one vector red per j-atom.  Type-pair
// gradients go to a warp-private shared table and are flushed to FP64 global
// sums after every entry.
#include "nbx_internal.cuh"
#include "nbx_pair_core.cuh"

#include <algorithm>

namespace nbx
{
namespace
{

constexpr int kAdjThreads    = 256;
constexpr int kAdjBlocksPerSm = 2;  // 16 warps per SM (128 registers a thread, no spills)
constexpr int kAdjWarps      = kAdjThreads / 32;
constexpr int kAdjMaxTypes1  = 16;
// Up to this many types (+ the dummy type) every warp keeps one type-pair gradient table per
// i-atom lane index (8 replicas): the lanes that add into one table in the same instruction then
// share their i-atom, so two of them hit the same entry only when their j-atoms have the same type.
constexpr int kAdjRepTypes1  = 10;
constexpr int kAdjReplicas   = kCl;

// Type-pair gradient tables of one warp: replicas x (nt1^2 + 1) float2, each replica planar (its
// nt1^2 + 1 dc6 sums, then its nt1^2 + 1 dc12 sums; the +1 staggers the replicas over the
// shared-memory banks).
__host__ __device__ __forceinline__ int adj_table_replicas(int nt1)
{
    return nt1 <= kAdjRepTypes1 ? kAdjReplicas : 1;
}
__host__ __device__ __forceinline__ int adj_table_stride(int nt1)
{
    return nt1 * nt1 + 1;
}

struct AdjConsts
{
    float gE_lj, gE_c;  // upstream energy gradients
};

// The per-system arrays one list entry of the adjoint touches.
struct AdjPtrs
{
    const float4* xq;
    const int*    tgrid;
    const Cj4*    cj4;
    const Excl*   excl;
    const float*  shiftvec;
    const float4* gnb;
    float4*       dnb;
};

// One atom pair (i-atom ii of i-cluster c, the lane's j-atom): recomputes the pair terms, adds
// the i-side gradients to the lane's accumulator slot acc[(c * 8 + ii) * 4 + jj] (shared memory,
// one slot per lane and i-atom: no conflicts), the j-side ones to dj*, and the type-pair gradient
// to the lane's table.
template<bool kEwald, bool kExcl>
__device__ __forceinline__ void adj_pair(const DeviceView& v, const float2* __restrict__ nbfp_s, float2* ttab,
                                         const float4* __restrict__ xis, const float4* __restrict__ gis, float4* acc,
                                         int c, const float4 xj, const float4 gj, int tj, unsigned wj, bool diag_cj,
                                         int h, int ii, int jj, const AdjConsts& k, float pbeta, float beta2l2,
                                         float c2b, float b2c2b, float& djx, float& djy, float& djz, float& djq)
{
    const int    nt1 = v.ntypes1;
    const float4 xi  = xis[c * kCl + ii];
    const float4 gi  = gis[c * kCl + ii];
    const int    ti  = __float_as_int(gi.w);
    const float  dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    float        r2 = dx * dx + dy * dy + dz * dz;
    bool         in_range;
    float        int_bit;
    if (kExcl)
    {
        // the diagonal cluster pair counts j > i only
        const bool self_lower = diag_cj && (c == (int)(wj >> 24)) && (h * (kCl / kSplit) + jj <= ii);
        in_range              = (r2 < v.rc2) && !self_lower;
        int_bit               = (wj & (1u << c)) ? 1.0f : 0.0f;
    }
    else
    {
        in_range = r2 < v.rc2;
        int_bit  = 1.0f;
    }
    r2                   = fmaxf(r2, kMinDist2);
    float       rinv     = rsqrtf(r2);
    rinv                 = rinv * (1.5f - 0.5f * r2 * rinv * rinv);
    const float  rinv2   = rinv * rinv;
    const float2 lj      = nbfp_s[ti * nt1 + tj];
    float        rinv6   = rinv2 * rinv2 * rinv2;
    if (kExcl)
    {
        rinv6 *= int_bit;
    }
    const float vrep    = lj.y * rinv6 * rinv6;
    const float vdisp   = lj.x * rinv6;
    const float phi_lj  = (vrep - vdisp) * rinv2;
    const float dphi_lj = (4.0f * vdisp - 7.0f * vrep) * rinv2 * rinv2;
    float       psi, dpsi, hq;  // Coulomb phi / qq, its s-derivative, energy / qq
    if (kEwald)
    {
        const float r    = r2 * rinv;
        const float t    = fast_rcp(fmaf(pbeta, r, 1.0f));
        const float poly = erfc_poly(t);
        const float expm = fast_ex2(-beta2l2 * r2);
        const float tp   = t * poly;
        psi              = expm * fmaf(tp, rinv, c2b) * rinv2;
        hq               = tp * expm * rinv - int_bit * v.sh_ewald;
        if (kExcl)
        {
            psi -= (1.0f - int_bit) * rinv * rinv2;
            hq -= (1.0f - int_bit) * rinv;
        }
        dpsi = -(1.5f * psi + b2c2b * expm) * rinv2;
    }
    else
    {
        const float r3 = rinv * rinv2;
        psi            = int_bit * r3 - 2.0f * v.k_rf;
        dpsi           = -1.5f * int_bit * r3 * rinv2;
        hq             = int_bit * rinv + v.k_rf * r2 - v.c_rf;
    }
    const float qq   = v.epsfac * xi.w * xj.w;
    const float phi  = fmaf(qq, psi, phi_lj);
    const float dphi = fmaf(qq, dpsi, dphi_lj);
    const float gx = gi.x - gj.x, gy = gi.y - gj.y, gz = gi.z - gj.z;
    const float gr   = gx * dx + gy * dy + gz * dz;
    const float coef = 2.0f * dphi * gr - fmaf(k.gE_c * qq, psi, k.gE_lj * phi_lj);
    float       ux   = fmaf(phi, gx, coef * dx);
    float       uy   = fmaf(phi, gy, coef * dy);
    float       uz   = fmaf(phi, gz, coef * dz);
    float       wq   = v.epsfac * fmaf(psi, gr, k.gE_c * hq);
    ux               = in_range ? ux : 0.0f;
    uy               = in_range ? uy : 0.0f;
    uz               = in_range ? uz : 0.0f;
    wq               = in_range ? wq : 0.0f;
    float4* const ai = &acc[(c * kCl + ii) * 4 + jj];
    float4        av = *ai;
    av.x += ux;
    av.y += uy;
    av.z += uz;
    av.w = fmaf(wq, xj.w, av.w);
    *ai  = av;
    djx -= ux;
    djy -= uy;
    djz -= uz;
    djq = fmaf(wq, xi.w, djq);
    // dL/d(6C6), dL/d(12C12) of this type pair
    if (in_range && int_bit != 0.0f)
    {
        const float dc12 = fmaf(gr * rinv6, rinv6 * rinv2, k.gE_lj * (rinv6 * rinv6 + v.cpot12) * (1.0f / 12.0f));
        const float dc6  = -fmaf(gr * rinv6, rinv2, k.gE_lj * (rinv6 + v.cpot6) * (1.0f / 6.0f));
        // planar replica: the dc6 sums, then (one table stride on) the dc12 sums, so that a warp's
        // 32 atomics spread over all banks instead of the even ones of interleaved pairs
        float* const slot = reinterpret_cast<float*>(ttab) + ti * nt1 + tj;
        atomicAdd(slot, dc6);
        atomicAdd(slot + adj_table_stride(nt1), dc12);
    }
}

// One warp half's j-clusters of a cj4 group: per j-cluster with set bits, the set i-clusters are
// visited two at a time (two independent pair computations in one basic block), the j-side sums
// reduced over the 8 i-lanes and added with one vector red per j-atom.
template<bool kEwald, bool kExcl>
__device__ __forceinline__ void adj_half(const DeviceView& v, const float4* __restrict__ jx,
                                         const float4* __restrict__ jg, const float2* __restrict__ nbfp_s,
                                         float2* ttab, const float4* __restrict__ xis, const float4* __restrict__ gis,
                                         float4* acc, float4* dnb, const int cj_lane, unsigned im, unsigned wexcl,
                                         int h, int sci, bool central, int ii, int jj, const AdjConsts& k,
                                         float pbeta, float beta2l2, float c2b, float b2c2b)
{
    const unsigned full = 0xffffffffu;
#pragma unroll 1
    for (int jm = 0; jm < kJg; jm++)
    {
        unsigned   rem = (im >> (jm * kNcl)) & 0xffu;
        const int  cj  = __shfl_sync(full, cj_lane, jm);
        if (!rem)
        {
            continue;
        }
        const int    aj = cj * kCl + h * (kCl / kSplit) + jj;
        // the cj4 group's 32 j-atoms are staged in shared memory (slot jm * 8 + atom)
        const int    sj = jm * kCl + h * (kCl / kSplit) + jj;
        const float4 xj = jx[sj];
        const float4 gj = jg[sj];
        const int    tj = __float_as_int(gj.w);
        // exclusion bits of this j-cluster's i-clusters; bits 24.. carry the diagonal i-cluster
        const bool     diag_cj = kExcl && central && (cj >= sci * kNcl) && (cj < sci * kNcl + kNcl);
        const unsigned wj      = kExcl ? (((wexcl >> (jm * kNcl)) & 0xffu) | ((unsigned)(cj - sci * kNcl) << 24)) : 0u;
        float          djx = 0.0f, djy = 0.0f, djz = 0.0f, djq = 0.0f;
        while (rem)
        {
            const int ca = __ffs(rem) - 1;
            rem &= rem - 1;
            if (rem)
            {
                const int cb = __ffs(rem) - 1;
                rem &= rem - 1;
                adj_pair<kEwald, kExcl>(v, nbfp_s, ttab, xis, gis, acc, ca, xj, gj, tj, wj, diag_cj, h, ii, jj, k,
                                        pbeta, beta2l2, c2b, b2c2b, djx, djy, djz, djq);
                adj_pair<kEwald, kExcl>(v, nbfp_s, ttab, xis, gis, acc, cb, xj, gj, tj, wj, diag_cj, h, ii, jj, k,
                                        pbeta, beta2l2, c2b, b2c2b, djx, djy, djz, djq);
            }
            else
            {
                adj_pair<kEwald, kExcl>(v, nbfp_s, ttab, xis, gis, acc, ca, xj, gj, tj, wj, diag_cj, h, ii, jj, k,
                                        pbeta, beta2l2, c2b, b2c2b, djx, djy, djz, djq);
            }
        }
#pragma unroll
        for (int o = 1; o < kCl; o <<= 1)
        {
            djx += __shfl_xor_sync(full, djx, o);
            djy += __shfl_xor_sync(full, djy, o);
            djz += __shfl_xor_sync(full, djz, o);
            djq += __shfl_xor_sync(full, djq, o);
        }
        if (ii == 0)
        {
            red_add_v4(&dnb[aj], djx, djy, djz, djq);
        }
    }
}

// One list entry: its 64 shifted i-atoms and their upstream gradients go to the
// warp's shared-memory slots, all cj4 groups are processed, then the i-side sums
// and the entry's type-pair table are flushed (vector reds / FP64 atomics).
template<bool kEwald>
__device__ __forceinline__ void adj_entry(const DeviceView& v, const AdjPtrs& p, const Sci& s,
                                          const float2* __restrict__ nbfp_s, float2* ttab, float4* xis, float4* gis,
                                          float4* jx, float4* jg, float4* acc, int lane, const AdjConsts& k,
                                          float pbeta, float beta2l2, float c2b, float b2c2b, double* gnbfp)
{
    const unsigned full    = 0xffffffffu;
    const int      ii      = lane & 7;
    const int      jj      = lane >> 3;
    const int      nt1     = v.ntypes1;
    const float    sx = p.shiftvec[3 * s.shift], sy = p.shiftvec[3 * s.shift + 1], sz = p.shiftvec[3 * s.shift + 2];
    const bool     central = (s.shift == kCentral);
    const int      reps    = adj_table_replicas(nt1);
    const int      tstride = adj_table_stride(nt1);
    float2* const  ttab_lane = ttab + (reps > 1 ? ii : 0) * tstride;
    __syncwarp();
    for (int m = lane; m < kSc; m += 32)
    {
        const int    a = s.sci * kSc + m;
        const float4 x = p.xq[a];
        const float4 g = p.gnb[a];
        xis[m]         = make_float4(x.x + sx, x.y + sy, x.z + sz, x.w);
        gis[m]         = make_float4(g.x, g.y, g.z, __int_as_float(p.tgrid[a]));
    }
    for (int m = lane; m < kSc * 4; m += 32)
    {
        acc[m] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    __syncwarp();
    // software pipeline over the cj4 groups, as in the force kernel: the next group's
    // record is loaded when a group starts, its 32 j-atoms after the group's first half
    int4   rec_ime{};
    int    rec_cj = 0;
    float4 xr{}, gr{};
    if (s.cj4_start < s.cj4_end)
    {
        rec_ime     = *reinterpret_cast<const int4*>(&p.cj4[s.cj4_start].imei[0]);
        rec_cj      = (lane < kJg) ? p.cj4[s.cj4_start].cj[lane] : 0;
        const int a = __shfl_sync(full, rec_cj, lane >> 3) * kCl + (lane & (kCl - 1));
        xr          = p.xq[a];
        gr          = p.gnb[a];
        gr.w        = __int_as_float(p.tgrid[a]);
    }
    for (int j4 = s.cj4_start; j4 < s.cj4_end; j4++)
    {
        const int4 ime     = rec_ime;
        const int  cj_lane = rec_cj;
        __syncwarp();
        jx[lane] = xr;
        jg[lane] = gr;
        __syncwarp();
        const bool more = j4 + 1 < s.cj4_end;
        if (more)
        {
            rec_ime = *reinterpret_cast<const int4*>(&p.cj4[j4 + 1].imei[0]);
            rec_cj  = (lane < kJg) ? p.cj4[j4 + 1].cj[lane] : 0;
        }
#pragma unroll 1
        for (int h = 0; h < kSplit; h++)
        {
            if (h == 1 && more)
            {
                const int a = __shfl_sync(full, rec_cj, lane >> 3) * kCl + (lane & (kCl - 1));
                xr          = p.xq[a];
                gr          = p.gnb[a];
                gr.w        = __int_as_float(p.tgrid[a]);
            }
            const unsigned im  = (h == 0) ? (unsigned)ime.x : (unsigned)ime.z;
            const int      exi = (h == 0) ? ime.y : ime.w;
            if (!im)
            {
                continue;
            }
            if (exi == 0)
            {
                adj_half<kEwald, false>(v, jx, jg, nbfp_s, ttab_lane, xis, gis, acc, p.dnb, cj_lane, im, 0u, h, s.sci,
                                        central, ii, jj, k, pbeta, beta2l2, c2b, b2c2b);
            }
            else
            {
                const unsigned wexcl = p.excl[exi].pair[lane];
                adj_half<kEwald, true>(v, jx, jg, nbfp_s, ttab_lane, xis, gis, acc, p.dnb, cj_lane, im, wexcl, h,
                                       s.sci, central, ii, jj, k, pbeta, beta2l2, c2b, b2c2b);
            }
        }
    }
    // the i-side sums: the 4 lane slots of every i-atom, one vector red per atom
    __syncwarp();
    for (int m = lane; m < kSc; m += 32)
    {
        const float4 a0 = acc[m * 4], a1 = acc[m * 4 + 1], a2 = acc[m * 4 + 2], a3 = acc[m * 4 + 3];
        red_add_v4(&p.dnb[s.sci * kSc + m], (a0.x + a1.x) + (a2.x + a3.x), (a0.y + a1.y) + (a2.y + a3.y),
                   (a0.z + a1.z) + (a2.z + a3.z), (a0.w + a1.w) + (a2.w + a3.w));
    }
    // flush the type-pair gradients of this entry into the block's FP64 sums (shared memory;
    // added to the global sums once per block at the end).  The replicas are summed in float
    // first: one conversion and one FP64 add per element, where FP64 runs at a small fraction of
    // the FP32 rate (a conversion and an add per replica kept the FP64 pipe 37 % busy).
    __syncwarp();
    for (int m = lane; m < nt1 * nt1; m += 32)
    {
        float tx = 0.0f, ty = 0.0f;
        for (int r = 0; r < reps; r++)
        {
            // replica r: dc6 sums at 2 r stride + m, dc12 sums one stride on (planar)
            float* const t = reinterpret_cast<float*>(ttab) + 2 * r * tstride + m;
            tx += t[0];
            ty += t[tstride];
            t[0]       = 0.0f;
            t[tstride] = 0.0f;
        }
        if (tx != 0.0f || ty != 0.0f)
        {
            atomicAdd(&gnbfp[2 * m], (double)tx);
            atomicAdd(&gnbfp[2 * m + 1], (double)ty);
        }
    }
    __syncwarp();
}

// Shared set-up of the adjoint kernels: the type table and zeroed per-warp tables.
__device__ __forceinline__ void adj_setup(const DeviceView& v, float2* nbfp_s, float2* ttab_all, double* gsum_s)
{
    const int nt1 = v.ntypes1;
    for (int m = threadIdx.x; m < nt1 * nt1; m += blockDim.x)
    {
        nbfp_s[m]         = v.nbfp[m];
        gsum_s[2 * m]     = 0.0;
        gsum_s[2 * m + 1] = 0.0;
    }
    const int ntab = kAdjWarps * adj_table_replicas(nt1) * adj_table_stride(nt1);
    for (int m = threadIdx.x; m < ntab; m += blockDim.x)
    {
        ttab_all[m] = make_float2(0.0f, 0.0f);
    }
    __syncthreads();
}

// The block's FP64 type-pair gradient sums into the global ones (one atomic per non-zero element
// and block instead of one per element and list entry).
__device__ __forceinline__ void adj_flush(const double* gsum_s, double* gnbfp, int n)
{
    __syncthreads();
    for (int m = threadIdx.x; m < n; m += blockDim.x)
    {
        if (gsum_s[m] != 0.0)
        {
            atomicAdd(&gnbfp[m], gsum_s[m]);
        }
    }
}

template<bool kEwald>
__global__ void __launch_bounds__(kAdjThreads, kAdjBlocksPerSm)
        k_backward(DeviceView v, const float4* __restrict__ gnb, float4* dnb, double* gnbfp, int* work_counter,
                   const double* __restrict__ gE)
{
    AdjConsts k{ 0.0f, 0.0f };
    if (gE)
    {
        k.gE_lj = (float)gE[0];
        k.gE_c  = (float)gE[1];
    }
    __shared__ float2 nbfp_s[kAdjMaxTypes1 * kAdjMaxTypes1];
    __shared__ double gsum_s[2 * kAdjMaxTypes1 * kAdjMaxTypes1];
    // dynamic: per warp the i-side accumulators (64 i-atoms x 4 lane slots), then the type-pair
    // gradient tables (kAdjWarps x replicas x stride)
    extern __shared__ float4 adj_dyn[];
    float4* const acc_w  = adj_dyn + (threadIdx.x >> 5) * (kSc * 4);
    float2* const ttab_s = reinterpret_cast<float2*>(adj_dyn + kAdjWarps * kSc * 4);
    __shared__ float4 xis_s[kAdjWarps][kSc];
    __shared__ float4 gis_s[kAdjWarps][kSc];
    __shared__ float4 jx_s[kAdjWarps][32];
    __shared__ float4 jg_s[kAdjWarps][32];
    adj_setup(v, nbfp_s, ttab_s, gsum_s);
    float2* const ttab_w = ttab_s + (threadIdx.x >> 5) * adj_table_replicas(v.ntypes1) * adj_table_stride(v.ntypes1);
    if (v.hdr->status & (kStatusListOverflow | kStatusExclOverflow | kStatusGridOverflow))
    {
        return;
    }
    const int     warp   = threadIdx.x >> 5;
    const int     lane   = threadIdx.x & 31;
    const int     numSci = v.hdr->num_sci;
    const float   b2c2b  = v.beta * v.beta * v.c2b;
    const AdjPtrs p      = { v.xq, v.tgrid, v.cj4, v.excl, v.shiftvec, gnb, dnb };
    for (;;)
    {
        int e = 0;
        if (lane == 0)
        {
            e = atomicAdd(work_counter, 1);
        }
        e = __shfl_sync(0xffffffffu, e, 0);
        if (e >= numSci)
        {
            break;
        }
        adj_entry<kEwald>(v, p, v.sci[e], nbfp_s, ttab_w, xis_s[warp], gis_s[warp], jx_s[warp], jg_s[warp],
                          acc_w, lane, k, v.pbeta,
                          v.beta2l2, v.c2b, b2c2b, gsum_s);
    }
    adj_flush(gsum_s, gnbfp, 2 * v.ntypes1 * v.ntypes1);
}

__device__ __forceinline__ int adj_find_system(const int* prefix, int nsys, int e)
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

// The adjoint over all systems of a batch (shared type table and type-pair
// gradient sums; per-system upstream energy gradients gE[2 s], gE[2 s + 1]).
template<bool kEwald>
__global__ void __launch_bounds__(kAdjThreads, kAdjBlocksPerSm)
        k_batch_backward(DeviceView cv, const BatchSys* __restrict__ sys, const int* __restrict__ prefix, int nsys,
                         double* gnbfp, int* work_counter, const double* __restrict__ gE)
{
    __shared__ float2 nbfp_s[kAdjMaxTypes1 * kAdjMaxTypes1];
    __shared__ double gsum_s[2 * kAdjMaxTypes1 * kAdjMaxTypes1];
    // dynamic: per warp the i-side accumulators (64 i-atoms x 4 lane slots), then the type-pair
    // gradient tables (kAdjWarps x replicas x stride)
    extern __shared__ float4 adj_dyn[];
    float4* const acc_w  = adj_dyn + (threadIdx.x >> 5) * (kSc * 4);
    float2* const ttab_s = reinterpret_cast<float2*>(adj_dyn + kAdjWarps * kSc * 4);
    __shared__ float4 xis_s[kAdjWarps][kSc];
    __shared__ float4 gis_s[kAdjWarps][kSc];
    __shared__ float4 jx_s[kAdjWarps][32];
    __shared__ float4 jg_s[kAdjWarps][32];
    adj_setup(cv, nbfp_s, ttab_s, gsum_s);
    float2* const ttab_w =
            ttab_s + (threadIdx.x >> 5) * adj_table_replicas(cv.ntypes1) * adj_table_stride(cv.ntypes1);
    const int   warp  = threadIdx.x >> 5;
    const int   lane  = threadIdx.x & 31;
    const int   total = prefix[nsys];
    const float b2c2b = cv.beta * cv.beta * cv.c2b;
    for (;;)
    {
        int e = 0;
        if (lane == 0)
        {
            e = atomicAdd(work_counter, 1);
        }
        e = __shfl_sync(0xffffffffu, e, 0);
        if (e >= total)
        {
            break;
        }
        const int       sidx = adj_find_system(prefix, nsys, e);
        const BatchSys& b    = sys[sidx];
        AdjConsts       k{ 0.0f, 0.0f };
        if (gE)
        {
            k.gE_lj = (float)gE[2 * sidx];
            k.gE_c  = (float)gE[2 * sidx + 1];
        }
        const AdjPtrs p = { b.xq, b.tgrid, b.cj4, b.excl, b.shiftvec, b.gnb, b.dnb };
        adj_entry<kEwald>(cv, p, b.sci[e - prefix[sidx]], nbfp_s, ttab_w, xis_s[warp], gis_s[warp],
                          jx_s[warp], jg_s[warp], acc_w, lane, k,
                          cv.pbeta, cv.beta2l2, cv.c2b, b2c2b, gsum_s);
    }
    adj_flush(gsum_s, gnbfp, 2 * cv.ntypes1 * cv.ntypes1);
}

// Batched upstream gradients to grid order (blockIdx.y = system), outputs cleared.
__global__ void k_batch_adj_prepare(const BatchSys* __restrict__ sys, const float* __restrict__ gF, int* counter,
                                    double* gnbfp, int n_gnbfp)
{
    // block (0, 0) also clears the work queue and the FP64 type-pair gradient table
    if (blockIdx.x == 0 && blockIdx.y == 0)
    {
        for (int i = threadIdx.x; i < n_gnbfp; i += blockDim.x)
        {
            gnbfp[i] = 0.0;
        }
        if (threadIdx.x == 0)
        {
            *counter = 0;
        }
    }
    const BatchSys& b = sys[blockIdx.y];
    const int       k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= b.hdr->num_cells * kSc)
    {
        return;
    }
    const int     a = b.atom_indices[k];
    const float*  g = gF + 3 * (size_t)(b.atom_base + (a >= 0 ? a : 0));
    const_cast<float4*>(b.gnb)[k] = (a >= 0) ? make_float4(g[0], g[1], g[2], 0.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    b.dnb[k]                      = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// Batched atom-order outputs (blockIdx.y = system), dL/dq with the self-energy term.
__global__ void k_batch_adj_finish(DeviceView cv, const BatchSys* __restrict__ sys, const double* __restrict__ gE,
                                   float* gx, float* gq)
{
    const BatchSys& b = sys[blockIdx.y];
    const int       a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= b.n)
    {
        return;
    }
    const int    k = b.cells[a];
    const float4 d = b.dnb[k];
    const size_t o = (size_t)b.atom_base + a;
    if (gx)
    {
        gx[3 * o]     = d.x;
        gx[3 * o + 1] = d.y;
        gx[3 * o + 2] = d.z;
    }
    if (gq)
    {
        const float q    = b.xq[k].w;
        const float self = (cv.coulomb == 0) ? -2.0f * cv.epsfac * cv.beta * 0.5641895835477563f * q
                                             : -cv.epsfac * cv.c_rf * q;
        gq[o]            = gE ? d.w + (float)gE[2 * blockIdx.y + 1] * self : d.w;
    }
}

// Charges of all systems (concatenated atom order) into xq.w and each system's q.
__global__ void k_batch_set_q(const BatchSys* __restrict__ sys, const float* __restrict__ q)
{
    const BatchSys& b = sys[blockIdx.y];
    const int       k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= b.hdr->num_cells * kSc)
    {
        return;
    }
    const int a = b.atom_indices[k];
    if (a >= 0)
    {
        const float qa                  = q[(size_t)b.atom_base + a];
        const_cast<float4*>(b.xq)[k].w  = qa;
        b.q[a]                          = qa;
    }
}

// Loss sum |F - F_target|^2 (FP64) and its gradient 2 (F - F_target) per coordinate.
__global__ void k_match_loss(const float* __restrict__ f, const float* __restrict__ ft, size_t n3, float* gF,
                             double* loss)
{
    double acc = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (size_t)gridDim.x * blockDim.x)
    {
        const float d = f[i] - ft[i];
        gF[i]         = 2.0f * d;
        acc += (double)d * (double)d;
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    }
    if ((threadIdx.x & 31) == 0 && acc != 0.0)
    {
        atomicAdd(loss, acc);
    }
}

// Upstream force gradients to grid order; clears the output accumulators.
// Per grid slot: the coordinates of this evaluation into xq (as k_convert_x, with the box shifts of
// the last search) when x is given, the upstream force gradient in grid order, a cleared dL/dx
// accumulator; block 0 also clears the work queue and the FP64 type-pair gradient table (in place
// of separate memsets).
__global__ void k_adj_prepare(DeviceView v, const float* __restrict__ x, const float* __restrict__ gF, float4* gnb,
                              float4* dnb, int* counter, double* gnbfp, int n_gnbfp)
{
    if (blockIdx.x == 0)
    {
        for (int i = threadIdx.x; i < n_gnbfp; i += blockDim.x)
        {
            gnbfp[i] = 0.0;
        }
        if (threadIdx.x == 0)
        {
            *counter = 0;
        }
    }
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= v.hdr->num_cells * kSc)
    {
        return;
    }
    const int a = v.atom_indices[k];
    if (x && a >= 0)
    {
        const float4 old  = v.xq[k];
        const int    code = v.image[a];
        float        c[3];
        for (int d = 0; d < 3; d++)
        {
            const int sh = (int)(signed char)((code >> (8 * d)) & 0xff);
            c[d]         = (sh == 0) ? x[3 * a + d] : x[3 * a + d] + (float)sh * v.g.box[d];
        }
        v.xq[k] = make_float4(c[0], c[1], c[2], old.w);
    }
    gnb[k] = (a >= 0) ? make_float4(gF[3 * a], gF[3 * a + 1], gF[3 * a + 2], 0.0f) : make_float4(0, 0, 0, 0);
    dnb[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// Atom-order outputs; dL/dq also gets the self-energy term.  Block 0 also copies the type-pair
// gradients out of the padded (nt+1)^2 table into the caller's nt^2 one when gout is given (the
// adjoint kernel has finished: no separate launch).
__global__ void k_adj_finish(DeviceView v, const float4* __restrict__ dnb, const double* __restrict__ gE, float* gx,
                             float* gq, const double* __restrict__ gpad, double* gout)
{
    if (gout && blockIdx.x == 0)
    {
        const int nt = v.ntypes1 - 1;
        for (int m = threadIdx.x; m < nt * nt; m += blockDim.x)
        {
            const int i = m / nt, j = m % nt;
            gout[2 * m]     = gpad[2 * (i * (nt + 1) + j)];
            gout[2 * m + 1] = gpad[2 * (i * (nt + 1) + j) + 1];
        }
    }
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= v.n)
    {
        return;
    }
    const int    k = v.cells[a];
    const float4 d = dnb[k];
    if (gx)
    {
        gx[3 * a]     = d.x;
        gx[3 * a + 1] = d.y;
        gx[3 * a + 2] = d.z;
    }
    if (gq)
    {
        const float q    = v.xq[k].w;
        // d/dq of -epsfac beta/sqrt(pi) q^2 (Ewald) or -epsfac c_rf q^2 / 2 (RF)
        const float self = (v.coulomb == 0) ? -2.0f * v.epsfac * v.beta * 0.5641895835477563f * q
                                            : -v.epsfac * v.c_rf * q;
        gq[a]            = gE ? d.w + (float)gE[1] * self : d.w;
    }
}

// Lorentz-Berthelot type table {6 C6, 12 C12} from per-type sigma and epsilon (one block):
// sigma_ij = (sigma_i + sigma_j) / 2, epsilon_ij = sqrt(epsilon_i epsilon_j), C6 = 4 eps s^6,
// C12 = 4 eps s^12 (the combination nblib applies, api/nblib/gmxsetup.cpp:143-166).
__global__ void k_lb_table(const double* __restrict__ sig, const double* __restrict__ eps, int nt, double* table)
{
    for (int m = threadIdx.x; m < nt * nt; m += blockDim.x)
    {
        const int    i = m / nt, j = m - (m / nt) * nt;
        const double s  = 0.5 * (sig[i] + sig[j]);
        const double e  = sqrt(eps[i] * eps[j]);
        const double s2 = s * s;
        const double s6 = s2 * s2 * s2;
        const double c6 = 4.0 * e * s6;
        table[2 * m]     = 6.0 * c6;
        table[2 * m + 1] = 12.0 * (c6 * s6);
    }
}

// Its adjoint: d L / d sigma_k and d L / d epsilon_k from d L / d table (one block; every type's
// sums run over its row and column in a fixed order).  d epsilon_ij / d epsilon_i is written
// epsilon_j / (2 epsilon_ij), as the derivative of the square root of the product.
__global__ void k_lb_table_backward(const double* __restrict__ sig, const double* __restrict__ eps, int nt,
                                    const double* __restrict__ gt, double* gsig, double* geps)
{
    extern __shared__ double lbs[];  // [2][nt * nt]: d L / d sigma_ij, d L / d epsilon_ij
    double* gs = lbs;
    double* ge = lbs + nt * nt;
    for (int m = threadIdx.x; m < nt * nt; m += blockDim.x)
    {
        const int    i = m / nt, j = m - (m / nt) * nt;
        const double s  = 0.5 * (sig[i] + sig[j]);
        const double e  = sqrt(eps[i] * eps[j]);
        const double s2 = s * s;
        const double s5 = s2 * s2 * s;
        const double s6 = s5 * s;
        const double g6 = gt[2 * m], g12 = gt[2 * m + 1];
        // 6 C6 = 24 e s^6, 12 C12 = 48 e s^12
        gs[m] = g6 * 144.0 * e * s5 + g12 * 576.0 * e * s5 * s6;
        ge[m] = g6 * 24.0 * s6 + g12 * 48.0 * s6 * s6;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nt; k += blockDim.x)
    {
        double as = 0.0, ae = 0.0;
        for (int j = 0; j < nt; j++)
        {
            const double eij = sqrt(eps[k] * eps[j]);
            // row k (sigma_k, epsilon_k as the first index) and column k (as the second)
            as += 0.5 * gs[k * nt + j] + 0.5 * gs[j * nt + k];
            ae += (ge[k * nt + j] + ge[j * nt + k]) * (eps[j] / (2.0 * eij));
        }
        gsig[k] = as;
        geps[k] = ae;
    }
}

} // namespace

int adjoint_max_types1()
{
    return kAdjMaxTypes1;
}

cudaError_t launch_lb_table(const double* sig, const double* eps, int nt, double* table, cudaStream_t s)
{
    k_lb_table<<<1, 256, 0, s>>>(sig, eps, nt, table);
    return cudaGetLastError();
}

cudaError_t launch_lb_table_backward(const double* sig, const double* eps, int nt, const double* gtable,
                                     double* gsig, double* geps, cudaStream_t s)
{
    k_lb_table_backward<<<1, 256, 2 * sizeof(double) * nt * nt, s>>>(sig, eps, nt, gtable, gsig, geps);
    return cudaGetLastError();
}

namespace
{

// Dynamic shared memory of the adjoint kernels: the warps' i-side accumulators and type-pair tables.
size_t adj_table_bytes(int nt1)
{
    return sizeof(float4) * (size_t)kAdjWarps * kSc * 4
           + sizeof(float2) * (size_t)kAdjWarps * adj_table_replicas(nt1) * adj_table_stride(nt1);
}

// Opts an adjoint kernel in to its static + dynamic shared memory beyond 48 KB.
template<auto kKernel>
cudaError_t adj_optin(size_t dynamic_bytes)
{
    cudaFuncAttributes a{};
    cudaError_t        e = cudaFuncGetAttributes(&a, kKernel);
    if (e != cudaSuccess)
    {
        return e;
    }
    return smem_optin<kKernel>(a.sharedSizeBytes + dynamic_bytes, dynamic_bytes);
}

} // namespace

cudaError_t launch_backward(const DeviceView& v, const float* d_x, const float* d_gF, const double* d_gE,
                            float4* gnb, float4* dnb, double* d_gnbfp, int* counter, float* d_gx, float* d_gq,
                            double* d_gnbfp_out, int num_sms, cudaStream_t s)
{
    const int tb    = 256;
    const int slots = v.g.cells_capacity * kSc;
    k_adj_prepare<<<(slots + tb - 1) / tb, tb, 0, s>>>(v, d_x, d_gF, gnb, dnb, counter, d_gnbfp,
                                                       2 * v.ntypes1 * v.ntypes1);
    const size_t dyn = adj_table_bytes(v.ntypes1);
    cudaError_t  e   = cudaSuccess;
    if (v.coulomb == 0)
    {
        e = adj_optin<k_backward<true>>(dyn);
        k_backward<true><<<num_sms * kAdjBlocksPerSm, kAdjThreads, dyn, s>>>(v, gnb, dnb, d_gnbfp, counter, d_gE);
    }
    else
    {
        e = adj_optin<k_backward<false>>(dyn);
        k_backward<false><<<num_sms * kAdjBlocksPerSm, kAdjThreads, dyn, s>>>(v, gnb, dnb, d_gnbfp, counter, d_gE);
    }
    if (e != cudaSuccess)
    {
        return e;
    }
    k_adj_finish<<<std::max(1, (v.n + tb - 1) / tb), tb, 0, s>>>(v, dnb, d_gE, d_gx, d_gq, d_gnbfp, d_gnbfp_out);
    return cudaGetLastError();
}

cudaError_t launch_batch_backward(const DeviceView& cv, const BatchSys* sys, const int* prefix, int nsys,
                                  int max_slots, int max_atoms, const float* d_gF, const double* d_gE,
                                  double* d_gnbfp, int* counter, float* d_gx, float* d_gq, int num_sms, cudaStream_t s)
{
    const int tb = 256;
    k_batch_adj_prepare<<<dim3((max_slots + tb - 1) / tb, nsys), tb, 0, s>>>(sys, d_gF, counter, d_gnbfp,
                                                                             2 * cv.ntypes1 * cv.ntypes1);
    const size_t dyn = adj_table_bytes(cv.ntypes1);
    cudaError_t  e   = cudaSuccess;
    if (cv.coulomb == 0)
    {
        e = adj_optin<k_batch_backward<true>>(dyn);
        k_batch_backward<true><<<num_sms * kAdjBlocksPerSm, kAdjThreads, dyn, s>>>(cv, sys, prefix, nsys, d_gnbfp, counter, d_gE);
    }
    else
    {
        e = adj_optin<k_batch_backward<false>>(dyn);
        k_batch_backward<false><<<num_sms * kAdjBlocksPerSm, kAdjThreads, dyn, s>>>(cv, sys, prefix, nsys, d_gnbfp, counter, d_gE);
    }
    if (e != cudaSuccess)
    {
        return e;
    }
    k_batch_adj_finish<<<dim3((max_atoms + tb - 1) / tb, nsys), tb, 0, s>>>(cv, sys, d_gE, d_gx, d_gq);
    return cudaGetLastError();
}

cudaError_t launch_batch_set_q(const BatchSys* sys, int nsys, int max_slots, const float* d_q, cudaStream_t s)
{
    const int tb = 256;
    k_batch_set_q<<<dim3((max_slots + tb - 1) / tb, nsys), tb, 0, s>>>(sys, d_q);
    return cudaGetLastError();
}

cudaError_t launch_match_loss(const float* d_f, const float* d_ft, size_t n3, float* d_gF, double* d_loss,
                              int num_sms, cudaStream_t s)
{
    cudaMemsetAsync(d_loss, 0, sizeof(double), s);
    k_match_loss<<<num_sms * 4, 256, 0, s>>>(d_f, d_ft, n3, d_gF, d_loss);
    return cudaGetLastError();
}

cudaError_t launch_set_nbfp(const DeviceView& v, const float* d_nbfp, cudaStream_t s)
{
    return launch_set_parameters(v, nullptr, d_nbfp, s);
}

// Charges and LJ parameters for force matching: q (atom order) into xq.w and the
// nbfp table (with the all-zero filler type); the self energy follows the charges.
__global__ void k_set_q(DeviceView v, const float* __restrict__ q)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= v.hdr->num_cells * kSc)
    {
        return;
    }
    const int a = v.atom_indices[k];
    if (a >= 0)
    {
        v.xq[k].w = q[a];
    }
}

__global__ void k_set_nbfp(float2* nbfp, const float* __restrict__ src, int nt)
{
    const int m   = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt1 = nt + 1;
    if (m >= nt1 * nt1)
    {
        return;
    }
    const int i = m / nt1, j = m % nt1;
    nbfp[m]     = (i < nt && j < nt) ? make_float2(src[2 * (i * nt + j)], src[2 * (i * nt + j) + 1])
                                     : make_float2(0.0f, 0.0f);
}

__global__ void k_compact_gnbfp(const double* padded, double* out, int nt)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nt * nt)
    {
        return;
    }
    const int i = m / nt, j = m % nt;
    out[2 * m]     = padded[2 * (i * (nt + 1) + j)];
    out[2 * m + 1] = padded[2 * (i * (nt + 1) + j) + 1];
}

cudaError_t launch_compact_gnbfp(const double* padded, double* out, int nt, cudaStream_t s)
{
    k_compact_gnbfp<<<(nt * nt + 255) / 256, 256, 0, s>>>(padded, out, nt);
    return cudaGetLastError();
}

cudaError_t launch_set_parameters(const DeviceView& v, const float* d_q, const float* d_nbfp, cudaStream_t s)
{
    const int tb = 256;
    if (d_q)
    {
        cudaMemcpyAsync(const_cast<float*>(v.q), d_q, sizeof(float) * v.n, cudaMemcpyDeviceToDevice, s);
        k_set_q<<<(v.g.cells_capacity * kSc + tb - 1) / tb, tb, 0, s>>>(v, d_q);
    }
    if (d_nbfp)
    {
        const int nt = v.ntypes1 - 1;
        k_set_nbfp<<<(v.ntypes1 * v.ntypes1 + tb - 1) / tb, tb, 0, s>>>(const_cast<float2*>(v.nbfp), d_nbfp, nt);
    }
    return cudaGetLastError();
}

} // namespace nbx
