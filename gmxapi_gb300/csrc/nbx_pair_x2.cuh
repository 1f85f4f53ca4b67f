// Packed FP32x2 pair core: each lane computes two atom pairs with one instruction stream.
//
// Physics of the reference's GPU-layout kernels
// (src/gromacs/nbnxm/kernels_reference/kernel_gpu_ref.cpp:57-379), as in nbx_pair_core.cuh; the
// difference is the lane mapping and the arithmetic width.  The force kernel is bound by
// instruction issue, not by the FP32 pipe: Blackwell's packed instructions (FFMA2 / FMUL2 /
// FADD2, two FP32 lanes of work per issue slot) let one issue slot feed the FMA pipe for two
// cycles.  Lane (ii, jj) = (lane & 7, lane >> 3) computes, for an i-cluster / j-cluster pair,
// the pairs (i-atom ii, j-atom jj) and (ii, jj + 4): one from each warp half of the j-cluster, so
// one packed pass covers the whole 8x8 cluster pair.  The j-atoms come from a cluster-packed
// copy of the atom data (x[8], y[8], z[8], q[8], type[8] per cluster with atoms a and a + 4
// adjacent, written by the coordinate conversion), so each j operand is one 8-byte shared-memory
// load;
// the i-atoms sit in the warp's shared memory as duplicated pairs {x, x, y, y}, {z, z, q, q}.
// One bulk copy per j-cluster brings its record (coordinates, charges and types, 160 B).
// A cluster pair is computed when either half's mask bit is set; pairs of a half whose bit is
// clear are masked exactly like pairs beyond the cut-off, so the result is the reference's.
#pragma once

#include "nbx_pair_core.cuh"

namespace nbx
{

// ---- packed FP32 arithmetic ----
__device__ __forceinline__ float2 f2(float a)
{
    return make_float2(a, a);
}
__device__ __forceinline__ float2 add2(float2 a, float2 b)
{
    return __fadd2_rn(a, b);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b)
{
    return __fmul2_rn(a, b);
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c)
{
    return __ffma2_rn(a, b, c);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    unsigned long long ra = *reinterpret_cast<unsigned long long*>(&a);
    unsigned long long rb = *reinterpret_cast<unsigned long long*>(&b);
    unsigned long long rd;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    return *reinterpret_cast<float2*>(&rd);
}
// The erfc expansion polynomial of erfc_poly (nbx_internal.cuh), same coefficients, evaluated by
// Estrin's scheme: (c0 + c1 t) + (c2 + c3 t) t^2 + ((c4 + c5 t) + (c6 + c7 t) t^2) t^4 -- a
// dependency depth of 4 instead of Horner's 7, for two more multiplications (the pair loop is
// bound by dependent-instruction latency).
__device__ __forceinline__ float2 erfc_poly2(float2 t)
{
    const float2 t2 = mul2(t, t);
    const float2 a  = fma2(f2(2.490737736e-01f), t, f2(2.664087117e-01f));
    const float2 b  = fma2(f2(-7.699845731e-02f), t, f2(3.232774734e-01f));
    const float2 c  = fma2(f2(-3.248904943e-01f), t, f2(5.147097111e-01f));
    const float2 d  = fma2(f2(1.128007565e-02f), t, f2(3.713922575e-02f));
    const float2 t4 = mul2(t2, t2);
    const float2 lo = fma2(b, t2, a);
    const float2 hi = fma2(d, t2, c);
    return fma2(hi, t4, lo);
}

// Position of atom a (0..7) of a cluster in the packed layout: a and a + 4 adjacent.
__host__ __device__ __forceinline__ int pack_pos(int a)
{
    return 2 * (a & 3) + (a >> 2);
}

// A warp's j stage with kDepth buffers: each holds one cj4 group's four packed j-cluster records
// (4 x 40 words).  uses counts the groups staged so far (buffer uses % kDepth, barrier parity
// (uses / kDepth) & 1).
template<int kDepth>
struct JStageP
{
    float*              x;    // [kDepth][4 * kPackWords]
    unsigned long long* bar;  // [kDepth]
    unsigned            uses;
};

// Per warp, in float4 units: stage x and types, barriers (one float4 holds two), and one record
// of 7 float4 per i-atom (i-cluster c, atom ii): {x, x, y, y}, {z, z, q, q}, the i-force partials
// of the four lanes (ii, jj), and the atom's type-table row offset in bytes.  One base address per
// i-cluster reaches all of them (records of 112 B: the 8 atoms of a cluster fall in distinct banks).
constexpr int kIRecF4 = 7;
template<int kDepth>
__host__ __device__ constexpr int warp_smem_f4_x2()
{
    return kDepth * kPackWords + (kDepth + 1) / 2 + kSc * kIRecF4;
}

struct WarpSmemX2
{
    float4* irec;  // [64][7]
};

template<int kDepth>
__device__ __forceinline__ void carve_x2(float4* base, int warp, JStageP<kDepth>& js, WarpSmemX2& w)
{
    float4* p = base + warp * warp_smem_f4_x2<kDepth>();
    js.x      = reinterpret_cast<float*>(p);
    js.bar    = reinterpret_cast<unsigned long long*>(p + kDepth * kPackWords);
    w.irec    = p + kDepth * kPackWords + (kDepth + 1) / 2;
    js.uses   = 0;
}

template<int kDepth>
__device__ __forceinline__ void stage_init_x2(JStageP<kDepth>& js, int lane)
{
    if (lane == 0)
    {
#pragma unroll
        for (int b = 0; b < kDepth; b++)
        {
            mbar_init(&js.bar[b], 1);
        }
        fence_mbar_init();
    }
    js.uses = 0;
    __syncwarp();
}

// Lanes 0-3 (after __syncwarp), each holding one j-cluster index cj of a cj4 group, copy the
// group's packed records (160 B per cluster) into buffer b.
template<int kDepth>
__device__ __forceinline__ void stage_issue_x2(const JStageP<kDepth>& js, int b, int lane, int cj, const float* xqp,
                                               unsigned extra_tx)
{
    fence_proxy_async();
    if (lane == 0)
    {
        mbar_expect_tx(&js.bar[b], kJg * kPackWords * 4 + extra_tx);
    }
    bulk_g2s(js.x + (b * kJg + lane) * kPackWords, xqp + (size_t)cj * kPackWords, kPackWords * 4, &js.bar[b]);
}

template<int kDepth>
__device__ __forceinline__ bool stage_wait_x2(const JStageP<kDepth>& js, int b, unsigned parity)
{
    if (__all_sync(0xffffffffu, mbar_try_wait(&js.bar[b], parity)))
    {
        return true;
    }
    const unsigned long long t0 = global_ns();
    for (;;)
    {
        const bool done = mbar_try_wait(&js.bar[b], parity);
        if (__all_sync(0xffffffffu, done))
        {
            return true;
        }
        const bool late = __shfl_sync(0xffffffffu, global_ns() - t0 > kStageWaitNs, 0);
        if (late)
        {
            return false;
        }
    }
}

// After a wait gave up: flag the timeout and give every buffer's copies a bounded chance to land.
template<int kDepth>
__device__ __forceinline__ void stage_timeout_x2(const JStageP<kDepth>& js, unsigned* status, int lane)
{
    if (lane == 0)
    {
        atomicOr(status, (unsigned)kStatusTimeout);
    }
#pragma unroll
    for (int k = 0; k < kDepth; k++)
    {
        const unsigned u = js.uses + k;
        stage_wait_x2(js, u % kDepth, (u / kDepth) & 1);
    }
}

// The per-system arrays one list entry touches (packed layouts for the j side).
struct SysPtrsX2
{
    const float4* xq;      // i side: grid-order {x, y, z, q}
    const int*    tgrid;   // i side: type per slot
    const float*  xqp;     // j side: cluster-packed records (coordinates, charges, types)
    float4*       fnb;
    const Cj4*    cj4;
    const Excl*   excl;
    const float*  shiftvec;
    double*       fshift;
};

// Constants of the pair loop, read once per entry.
struct PairConstsX2
{
    float rc2, pbeta, nbeta2l2, c2b, k_rf2, nk_rf2, sh_ewald, k_rf, c_rf, epsfac;
};

// The geometry of one packed step: i-cluster c's atom ii (record rec in shared memory) against
// the lane's two j-atoms.  in: the pair is inside the cut-off and its half's mask bit is set (and,
// on the diagonal, j > i); kExcl: int = the pair's exclusion bit as 0 / 1.
struct GeomX2
{
    float4* rec;
    float2  qi;               // {q_i, q_i}
    float2  dx, dy, dz, r2;
    bool    inA, inB;
    float   intA, intB;
};

__device__ __forceinline__ void pair_geom_x2(const PairConstsX2& k, float4* __restrict__ rec, const float2 xj,
                                             const float2 yj, const float2 zj, bool okA, bool okB, float intA,
                                             float intB, GeomX2& g)
{
    const float4 i0 = rec[0];  // {x, x, y, y}
    const float4 i1 = rec[1];  // {z, z, q, q}
    g.rec           = rec;
    g.qi            = make_float2(i1.z, i1.w);
    g.dx            = sub2(make_float2(i0.x, i0.y), xj);
    g.dy            = sub2(make_float2(i0.z, i0.w), yj);
    g.dz            = sub2(make_float2(i1.x, i1.y), zj);
    g.r2            = fma2(g.dz, g.dz, fma2(g.dy, g.dy, mul2(g.dx, g.dx)));
    g.inA           = okA && (g.r2.x < k.rc2);
    g.inB           = okB && (g.r2.y < k.rc2);
    g.intA          = intA;
    g.intB          = intB;
}

// The forces and energies of one packed step whose geometry is g; the lane's i-force partial for
// atom (c, ii) is read, updated and written back in shared memory.
template<bool kEnergy, int kCoul, bool kExcl>
__device__ __forceinline__ void pair_phys_x2(const PairConstsX2& k, const char* __restrict__ nbfp_b, const GeomX2& g,
                                             int jj, const float2 qje, const int2 tjb, float2& fjx, float2& fjy,
                                             float2& fjz, float2& ejel, float2& ejlj)
{
    float4* const rec  = g.rec;
    const int     ti   = __float_as_int(rec[6].x);  // type-table row, bytes
    const float2  dx = g.dx, dy = g.dy, dz = g.dz;
    const bool    inA = g.inA, inB = g.inB;
    const float   intA = g.intA, intB = g.intB;
    float2        r2   = make_float2(fmaxf(g.r2.x, kMinDist2), fmaxf(g.r2.y, kMinDist2));
    float2        rinv = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
    if (kEnergy)
    {
        // one Newton step: rsqrt.approx -> ~correctly rounded, unbiased for the energy sums;
        // y (1.5 - (r^2 / 2) y^2) with -r^2 / 2 formed beside the rsqrt
        const float2 r2h = mul2(r2, f2(-0.5f));
        rinv             = mul2(rinv, fma2(r2h, mul2(rinv, rinv), f2(1.5f)));
    }
    // pairs outside the cut-off (or of a pruned half, or the diagonal's lower triangle) get
    // 1/r = 0: every force term below carries 1/r^2 and vanishes
    rinv               = make_float2(inA ? rinv.x : 0.0f, inB ? rinv.y : 0.0f);
    const float2 rinv2 = mul2(rinv, rinv);
    // {-6 C6, 12 C12, LJ shift, -} per type pair, in scalar form (the two halves' parameters
    // come from two table rows)
    const float4 lA    = *reinterpret_cast<const float4*>(nbfp_b + ti + tjb.x);
    const float4 lB    = *reinterpret_cast<const float4*>(nbfp_b + ti + tjb.y);
    float2       rinv6 = mul2(mul2(rinv2, rinv2), rinv2);
    if (kExcl)
    {
        rinv6 = mul2(rinv6, make_float2(intA, intB));
    }
    const float2 nvdisp = make_float2(lA.x * rinv6.x, lB.x * rinv6.y);
    const float2 flj    = make_float2(fmaf(lA.y * rinv6.x, rinv6.x, nvdisp.x),
                                      fmaf(lB.y * rinv6.y, rinv6.y, nvdisp.y));  // F r^2: vrep - vdisp
    const float2 qq     = mul2(g.qi, qje);
    float2       fcr2;  // Coulomb F r^2 / (q_i q_j)
    float2       hel;   // Coulomb energy / (q_i q_j epsfac), before masking
    if (kCoul >= 1)
    {
        // erfc(beta r) = t P(t) exp(-beta^2 r^2), t = 1/(1 + p beta r)
        const float2 r    = mul2(r2, rinv);
        const float2 tt   = fma2(f2(k.pbeta), r, f2(1.0f));
        const float2 t    = make_float2(fast_rcp(tt.x), fast_rcp(tt.y));
        const float2 poly = erfc_poly2(t);
        const float2 earg = mul2(f2(k.nbeta2l2), r2);
        const float2 expm = make_float2(fast_ex2(earg.x), fast_ex2(earg.y));
        const float2 tpr  = mul2(mul2(t, poly), rinv);  // erfc(beta r) / r = tpr * expm
        fcr2              = mul2(expm, add2(tpr, f2(k.c2b)));
        if (kExcl)
        {
            // excluded pairs keep only the Ewald correction: drop the plain 1/r
            fcr2 = fma2(make_float2(intA - 1.0f, intB - 1.0f), rinv, fcr2);
        }
        if (kEnergy)
        {
            // with the Ewald potential modifier the shift counts for pairs in range; without it the
            // term vanishes outside the cut-off by itself (1/r = 0)
            hel = (kCoul == 2) ? fma2(tpr, expm, make_float2(inA ? -k.sh_ewald : 0.0f, inB ? -k.sh_ewald : 0.0f))
                               : mul2(tpr, expm);
        }
    }
    else
    {
        fcr2 = kExcl ? fma2(f2(k.nk_rf2), r2, mul2(rinv, make_float2(intA, intB))) : fma2(f2(k.nk_rf2), r2, rinv);
        if (kEnergy)
        {
            // 1/r + k_rf r^2 - c_rf for pairs in range, 0 outside
            hel = fma2(f2(k.k_rf), r2, sub2(rinv, f2(k.c_rf)));
            hel = make_float2(inA ? hel.x : 0.0f, inB ? hel.y : 0.0f);
        }
    }
    const float2 fscal = mul2(fma2(qq, fcr2, flj), rinv2);
    if (kEnergy)
    {
        // Only pairs inside the cut-off that are not excluded count.  Outside the cut-off 1/r = 0
        // already zeroes every r-dependent term, so only the constant shifts need the mask; an
        // excluded pair inside the cut-off (int 0) has 1/r^6 = 0 (LJ) but its Ewald term must go.
        const bool cA = kExcl ? (inA && intA != 0.0f) : inA;
        const bool cB = kExcl ? (inB && intB != 0.0f) : inB;
        // LJ energy: vrep/12 - vdisp/6 + shift = (flj - vdisp)/12 + shift
        const float2 vlj = fma2(add2(flj, nvdisp), f2(1.0f / 12.0f), make_float2(cA ? lA.z : 0.0f, cB ? lB.z : 0.0f));
        ejlj             = add2(ejlj, vlj);
        if (kExcl)
        {
            hel = make_float2(cA ? hel.x : 0.0f, cB ? hel.y : 0.0f);
        }
        ejel = fma2(g.qi, hel, ejel);
    }
    float4 fi = rec[2 + jj];
    fi.x      = fmaf(fscal.y, dx.y, fmaf(fscal.x, dx.x, fi.x));
    fi.y      = fmaf(fscal.y, dy.y, fmaf(fscal.x, dy.x, fi.y));
    fi.z      = fmaf(fscal.y, dz.y, fmaf(fscal.x, dz.x, fi.z));
    rec[2 + jj] = fi;
    // j forces with the sign of the i forces; negated once per j-cluster
    fjx = fma2(fscal, dx, fjx);
    fjy = fma2(fscal, dy, fjy);
    fjz = fma2(fscal, dz, fjz);
}

// The half-mask, diagonal and exclusion bits of i-cluster c of the current j-cluster.
template<bool kExcl>
__device__ __forceinline__ void pair_bits_x2(int c, unsigned mA, unsigned mB, unsigned xA, unsigned xB, bool diag_j,
                                             int sci, int cj, int ii, int jj, bool& okA, bool& okB, float& intA,
                                             float& intB)
{
    okA = (mA >> c) & 1u;
    okB = (mB >> c) & 1u;
    if (kExcl)
    {
        // the diagonal cluster pair counts j > i only (kernel_gpu_ref.cpp:242)
        const bool diag = diag_j && (sci * kNcl + c == cj);
        okA             = okA && !(diag && jj <= ii);
        okB             = okB && !(diag && jj + 4 <= ii);
        intA            = ((xA >> c) & 1u) ? 1.0f : 0.0f;
        intB            = ((xB >> c) & 1u) ? 1.0f : 0.0f;
    }
    else
    {
        intA = intB = 1.0f;
    }
}

// Takes set i-clusters off `rem` until one has a pair inside the cut-off (any lane) and returns its
// geometry; false when `rem` runs out.  Steps with every pair beyond the cut-off (about one in
// eight on a list pruned to rlist_inner 0.95 nm at rc 0.9 nm) contribute exact zeros, so they are
// left out after the cheap geometry part.  kSame: both halves' masks equal rem.
template<bool kExcl, bool kSame>
__device__ __forceinline__ bool next_step_x2(const PairConstsX2& k, float4* __restrict__ lane_rec, unsigned& rem,
                                             unsigned mA, unsigned mB, unsigned xA, unsigned xB, bool central,
                                             int sci, int cj, int ii, int jj, const float2 xj, const float2 yj,
                                             const float2 zj, GeomX2& g)
{
#pragma unroll 1
    while (rem)
    {
        const int c = __ffs(rem) - 1;
        rem &= rem - 1;
        bool  okA = true, okB = true;
        float intA = 1.0f, intB = 1.0f;
        if (!kSame)
        {
            pair_bits_x2<kExcl>(c, mA, mB, xA, xB, central, sci, cj, ii, jj, okA, okB, intA, intB);
        }
        pair_geom_x2(k, lane_rec + c * (kCl * kIRecF4), xj, yj, zj, okA, okB, intA, intB, g);
        if (__any_sync(0xffffffffu, g.inA || g.inB))
        {
            return true;
        }
    }
    return false;
}

// The set i-clusters `rem` of one j-cluster, the ones with pairs inside the cut-off visited two at
// a time so that two independent pair computations share a basic block.
template<bool kEnergy, int kCoul, bool kExcl, bool kSame>
__device__ __forceinline__ void jcluster_x2(const PairConstsX2& k, const char* __restrict__ nbfp_b,
                                            float4* __restrict__ lane_rec, unsigned rem, unsigned mA, unsigned mB,
                                            unsigned xA, unsigned xB, bool central, int sci, int cj, int ii, int jj,
                                            const float2 xj, const float2 yj, const float2 zj, const float2 qje,
                                            const int2 tjb, float2& fjx, float2& fjy, float2& fjz, float2& ejel,
                                            float2& ejlj)
{
#pragma unroll 1
    for (;;)
    {
        GeomX2 ga;
        if (!next_step_x2<kExcl, kSame>(k, lane_rec, rem, mA, mB, xA, xB, central, sci, cj, ii, jj, xj, yj, zj, ga))
        {
            break;
        }
        GeomX2 gb;
        if (!next_step_x2<kExcl, kSame>(k, lane_rec, rem, mA, mB, xA, xB, central, sci, cj, ii, jj, xj, yj, zj, gb))
        {
            pair_phys_x2<kEnergy, kCoul, kExcl>(k, nbfp_b, ga, jj, qje, tjb, fjx, fjy, fjz, ejel, ejlj);
            break;
        }
        pair_phys_x2<kEnergy, kCoul, kExcl>(k, nbfp_b, ga, jj, qje, tjb, fjx, fjy, fjz, ejel, ejlj);
        pair_phys_x2<kEnergy, kCoul, kExcl>(k, nbfp_b, gb, jj, qje, tjb, fjx, fjy, fjz, ejel, ejlj);
    }
}

// All set cluster pairs of one cj4 group.  m0 / m1: the group's half masks; wA / wB: the
// lane's exclusion words of the two halves (all ones without exclusions).
template<bool kEnergy, int kCoul, bool kExcl>
__device__ __forceinline__ void group_x2(const PairConstsX2& k, const SysPtrsX2& p, const char* __restrict__ nbfp_b,
                                         const float* __restrict__ jx,
                                         float4* __restrict__ lane_rec, int cj_lane, unsigned m0, unsigned m1,
                                         unsigned wA, unsigned wB, int sci, bool central, int ii, int jj,
                                         float& acc_el, float& cmp_el, float& acc_lj, float& cmp_lj)
{
    const unsigned full = 0xffffffffu;
    const unsigned u    = m0 | m1;
#pragma unroll 1
    for (int jm = 0; jm < kJg; jm++)
    {
        unsigned  rem = (u >> (jm * kNcl)) & 0xffu;
        const int cj  = __shfl_sync(full, cj_lane, jm);
        if (!rem)
        {
            continue;
        }
        const float* xs   = jx + jm * kPackWords + 2 * jj;
        const float2 xj   = *reinterpret_cast<const float2*>(xs);
        const float2 yj   = *reinterpret_cast<const float2*>(xs + 8);
        const float2 zj   = *reinterpret_cast<const float2*>(xs + 16);
        const float2 qj   = *reinterpret_cast<const float2*>(xs + 24);
        const int2   tjb  = *reinterpret_cast<const int2*>(xs + 32);  // type-pair row offsets, bytes
        const float2 qje  = mul2(qj, f2(k.epsfac));
        const unsigned mA = m0 >> (jm * kNcl), mB = m1 >> (jm * kNcl);
        const unsigned xA = wA >> (jm * kNcl), xB = wB >> (jm * kNcl);
        float2 fjx = f2(0.0f), fjy = f2(0.0f), fjz = f2(0.0f);
        float2 ejel = f2(0.0f), ejlj = f2(0.0f);
        if (!kExcl && ((mA ^ mB) & 0xffu) == 0)
        {
            // both halves set for every i-cluster of this j-cluster (the common case)
            jcluster_x2<kEnergy, kCoul, false, true>(k, nbfp_b, lane_rec, rem, mA, mB, xA, xB, central, sci, cj, ii,
                                                     jj, xj, yj, zj, qje, tjb, fjx, fjy, fjz, ejel, ejlj);
        }
        else
        {
            jcluster_x2<kEnergy, kCoul, kExcl, false>(k, nbfp_b, lane_rec, rem, mA, mB, xA, xB, central, sci, cj, ii,
                                                      jj, xj, yj, zj, qje, tjb, fjx, fjy, fjz, ejel, ejlj);
        }
        if (kEnergy)
        {
            kahan_add(acc_el, cmp_el, qj.x * ejel.x);
            kahan_add(acc_el, cmp_el, qj.y * ejel.y);
            kahan_add(acc_lj, cmp_lj, ejlj.x + ejlj.y);
        }
        // j forces: sum over the 8 i-lanes, reduce-scatter on the first level so that lanes
        // ii < 4 end with the half-0 atom (jj) and lanes ii >= 4 with the half-1 atom (jj + 4)
        const bool hi = (ii & 4) != 0;
        float      kx = hi ? fjx.y : fjx.x, ky = hi ? fjy.y : fjy.x, kz = hi ? fjz.y : fjz.x;
        const float sx = hi ? fjx.x : fjx.y, sy = hi ? fjy.x : fjy.y, sz = hi ? fjz.x : fjz.y;
        kx += __shfl_xor_sync(full, sx, 4);
        ky += __shfl_xor_sync(full, sy, 4);
        kz += __shfl_xor_sync(full, sz, 4);
#pragma unroll
        for (int o = 2; o > 0; o >>= 1)
        {
            kx += __shfl_xor_sync(full, kx, o);
            ky += __shfl_xor_sync(full, ky, o);
            kz += __shfl_xor_sync(full, kz, o);
        }
        if ((ii & 3) == 0)
        {
            red_add_v4(&p.fnb[cj * kCl + jj + (hi ? 4 : 0)], -kx, -ky, -kz);
        }
    }
}

// The lane's exclusion words of a cj4 group's two halves (excl[0] is the all-interacting mask).
__device__ __forceinline__ uint2 excl_words(const SysPtrsX2& p, const int4 ime, int lane)
{
    if ((ime.y | ime.w) == 0)
    {
        return make_uint2(~0u, ~0u);
    }
    return make_uint2(p.excl[ime.y].pair[lane], p.excl[ime.w].pair[lane]);
}

// One list entry with the packed core; energies added to e_lj_acc / e_el_acc (per lane, FP64).
template<bool kEnergy, int kCoul, int kDepth>
__device__ __forceinline__ bool process_entry_x2(const PairConstsX2& k, const SysPtrsX2& p, const Sci& s,
                                                 const char* __restrict__ nbfp_b, JStageP<kDepth>& js,
                                                 const WarpSmemX2& w, int nt1, int lane, unsigned wait_test_bytes,
                                                 double& e_lj_acc, double& e_el_acc)
{
    const unsigned full = 0xffffffffu;
    const int      ii = lane & 7, jj = lane >> 3;
    const float    shx = p.shiftvec[3 * s.shift], shy = p.shiftvec[3 * s.shift + 1], shz = p.shiftvec[3 * s.shift + 2];
    const bool     central = (s.shift == kCentral);
    // the 64 shifted i-atoms into the warp's shared memory as duplicated pairs
    __syncwarp();
#pragma unroll
    for (int r = 0; r < 2; r++)
    {
        const int    a = lane + 32 * r;
        const float4 x = p.xq[s.sci * kSc + a];
        const float  xs = x.x + shx, ys = x.y + shy, zs = x.z + shz;
        float4*      ra = w.irec + a * kIRecF4;
        ra[0]           = make_float4(xs, xs, ys, ys);
        ra[1]           = make_float4(zs, zs, x.w, x.w);
        ra[6].x         = __int_as_float(p.tgrid[s.sci * kSc + a] * nt1 * (int)sizeof(float4));
    }
    float4* const lane_rec = w.irec + ii * kIRecF4;
#pragma unroll
    for (int c = 0; c < kNcl; c++)
    {
        lane_rec[c * kCl * kIRecF4 + 2 + jj] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    __syncwarp();
    float acc_el = 0.0f, cmp_el = 0.0f, acc_lj = 0.0f, cmp_lj = 0.0f;
    // pipeline over the cj4 groups: kDepth - 1 groups' copies in flight ahead of the one computed
    // (with each group's record and, where it has exclusion masks, the lane's exclusion words,
    // so their load latency is hidden behind the groups computed before)
    int4  rec_ime[kDepth - 1];
    int   rec_cj[kDepth - 1];
    uint2 rec_w[kDepth - 1];
    int   issued = s.cj4_start;
#pragma unroll
    for (int d = 0; d < kDepth - 1; d++)
    {
        if (issued < s.cj4_end)
        {
            rec_ime[d] = *reinterpret_cast<const int4*>(&p.cj4[issued].imei[0]);
            rec_cj[d]  = (lane < kJg) ? p.cj4[issued].cj[lane] : 0;
            rec_w[d]   = excl_words(p, rec_ime[d], lane);
            __syncwarp();
            if (lane < kJg)
            {
                stage_issue_x2(js, (js.uses + d) % kDepth, lane, rec_cj[d], p.xqp, wait_test_bytes);
            }
            issued++;
        }
    }
    for (int j4 = s.cj4_start; j4 < s.cj4_end; j4++)
    {
        const int4     ime     = rec_ime[0];
        const int      cj_lane = rec_cj[0];
        const uint2    wAB     = rec_w[0];
#pragma unroll
        for (int d = 0; d + 1 < kDepth - 1; d++)
        {
            rec_ime[d] = rec_ime[d + 1];
            rec_cj[d]  = rec_cj[d + 1];
            rec_w[d]   = rec_w[d + 1];
        }
        const int      b      = js.uses % kDepth;
        const unsigned parity = (js.uses / kDepth) & 1;
        if (issued < s.cj4_end)
        {
            rec_ime[kDepth - 2] = *reinterpret_cast<const int4*>(&p.cj4[issued].imei[0]);
            rec_cj[kDepth - 2]  = (lane < kJg) ? p.cj4[issued].cj[lane] : 0;
            rec_w[kDepth - 2]   = excl_words(p, rec_ime[kDepth - 2], lane);
            __syncwarp();  // the buffer's last readers (the group before this one) are done
            if (lane < kJg)
            {
                stage_issue_x2(js, (js.uses + kDepth - 1) % kDepth, lane, rec_cj[kDepth - 2], p.xqp,
                               wait_test_bytes);
            }
            issued++;
        }
        if (!stage_wait_x2(js, b, parity))
        {
            return false;
        }
        js.uses++;
        const unsigned m0 = (unsigned)ime.x, m1 = (unsigned)ime.z;
        if (!(m0 | m1))
        {
            continue;
        }
        const float* jx = js.x + b * kJg * kPackWords;
        if ((ime.y | ime.w) == 0)
        {
            group_x2<kEnergy, kCoul, false>(k, p, nbfp_b, jx, lane_rec, cj_lane, m0, m1, ~0u, ~0u, s.sci, central,
                                             ii, jj, acc_el, cmp_el, acc_lj, cmp_lj);
        }
        else
        {
            group_x2<kEnergy, kCoul, true>(k, p, nbfp_b, jx, lane_rec, cj_lane, m0, m1, wAB.x, wAB.y, s.sci,
                                            central, ii, jj, acc_el, cmp_el, acc_lj, cmp_lj);
        }
    }
    // i forces: reduce over the 4 j-lanes of each i-atom
    float sfx = 0.0f, sfy = 0.0f, sfz = 0.0f;
#pragma unroll
    for (int c = 0; c < kNcl; c++)
    {
        const float4 fi = lane_rec[c * kCl * kIRecF4 + 2 + jj];
        float        fx = fi.x, fy = fi.y, fz = fi.z;
        fx += __shfl_xor_sync(full, fx, 8);
        fy += __shfl_xor_sync(full, fy, 8);
        fz += __shfl_xor_sync(full, fz, 8);
        fx += __shfl_xor_sync(full, fx, 16);
        fy += __shfl_xor_sync(full, fy, 16);
        fz += __shfl_xor_sync(full, fz, 16);
        if (jj == 0)
        {
            red_add_v4(&p.fnb[(s.sci * kNcl + c) * kCl + ii], fx, fy, fz);
            sfx += fx;
            sfy += fy;
            sfz += fz;
        }
    }
    if (kEnergy)
    {
        e_el_acc += (double)acc_el - (double)cmp_el;
        e_lj_acc += (double)acc_lj - (double)cmp_lj;
    }
    if (!central)
    {
#pragma unroll
        for (int o = 1; o < kCl; o <<= 1)
        {
            sfx += __shfl_xor_sync(full, sfx, o);
            sfy += __shfl_xor_sync(full, sfy, o);
            sfz += __shfl_xor_sync(full, sfz, o);
        }
        if (lane == 0)
        {
            atomicAdd(&p.fshift[3 * s.shift + 0], (double)sfx);
            atomicAdd(&p.fshift[3 * s.shift + 1], (double)sfy);
            atomicAdd(&p.fshift[3 * s.shift + 2], (double)sfz);
        }
    }
    return true;
}

} // namespace nbx
