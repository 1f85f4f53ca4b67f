// Pair-interaction core shared by the single-system and batched force kernels.
//
// Physics of the reference's GPU-layout kernels
// (src/gromacs/nbnxm/kernels_reference/kernel_gpu_ref.cpp:57-379): every set
// bit of the list mask is an 8x8 i-cluster / j-cluster block of atom pairs;
// pairs within rc interact with potential-shifted LJ from nbfp and Ewald real
// space (or reaction field), exclusions keep only the Ewald correction, and
// the force on j is the negated force on i (half list).
#pragma once

#include "nbx_internal.cuh"

namespace nbx
{

// The per-system arrays one list entry touches.
struct SysPtrs
{
    const float4* xq;
    const int*    tgrid;
    float4*       fnb;
    const Cj4*    cj4;
    const Excl*   excl;
    const float*  shiftvec;
    double*       fshift;
};

__device__ __forceinline__ float fast_rcp(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float fast_ex2(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Vector reduction into a buffer this kernel never reads back, so no memory clobber:
// loads may be scheduled across it.
__device__ __forceinline__ void red_add_v4(float4* addr, float x, float y, float z, float w = 0.0f)
{
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(x), "f"(y), "f"(z), "f"(w));
}

// ---- bulk asynchronous copies (TMA engine) into a warp's shared-memory stage ----
constexpr int                kStageTx       = kJg * kCl * (16 + 4);  // bytes per cj4 group: 32 xq + 32 types
constexpr unsigned long long kStageWaitNs   = 1000000000ull;         // a stage wait gives up after 1 s

__device__ __forceinline__ unsigned smem_u32(const void* p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* m, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* m, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* m, unsigned parity)
{
    unsigned ok;
    asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(smem_u32(m)), "r"(parity)
            : "memory");
    return ok != 0;
}
// global -> shared bulk copy completing on mbarrier m (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* m)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(m))
                 : "memory");
}

// A warp's double-buffered j stage: two copies of one cj4 group's 32 j-atoms
// (xq, types) and their two barriers; `uses` counts the groups staged so far
// (buffer uses & 1, barrier parity (uses >> 1) & 1).
struct JStage
{
    float4*             x;     // [2][32]
    int*                t;     // [2][32]
    unsigned long long* bar;   // [2]
    unsigned            uses;
};

// Lanes 0-3 of the warp (after __syncwarp), each holding one j-cluster index cj of a
// cj4 group, start the group's bulk copies into buffer b: one warp instruction per
// array copies all four clusters (128 B of xq and 32 B of types each).  Lane 0 arms
// the barrier with the group's byte count.
__device__ __forceinline__ void stage_issue(const JStage& js, int b, int lane, int cj, const float4* xq,
                                            const int* tgrid, unsigned extra_tx = 0)
{
    fence_proxy_async();  // earlier shared reads of the buffer before the async writes
    if (lane == 0)
    {
        // extra_tx > 0 (a failure-detection test only) arms the barrier for bytes that never
        // arrive, so the bounded wait runs out
        mbar_expect_tx(&js.bar[b], kStageTx + extra_tx);
    }
    bulk_g2s(js.x + b * 32 + lane * kCl, xq + (size_t)cj * kCl, kCl * 16, &js.bar[b]);
    bulk_g2s(js.t + b * 32 + lane * kCl, tgrid + (size_t)cj * kCl, kCl * 4, &js.bar[b]);
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded, warp-uniform wait for buffer b (1 s of wall time); false when the copies
// did not land.
__device__ __forceinline__ bool stage_wait(const JStage& js, int b, unsigned parity)
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
        // lane 0's clock decides, so every lane leaves together
        const bool late = __shfl_sync(0xffffffffu, global_ns() - t0 > kStageWaitNs, 0);
        if (late)
        {
            return false;
        }
    }
}

// Per-warp barrier set-up (lane 0), once per kernel.
__device__ __forceinline__ void stage_init(JStage& js, int lane)
{
    if (lane == 0)
    {
        mbar_init(&js.bar[0], 1);
        mbar_init(&js.bar[1], 1);
        fence_mbar_init();
    }
    js.uses = 0;
    __syncwarp();
}

// Compensated (Kahan) accumulation: sum + c carries ~2x float precision.
__device__ __forceinline__ void kahan_add(float& sum, float& c, float v)
{
    const float y = v - c;
    const float t = sum + y;
    c             = (t - sum) - y;
    sum           = t;
}

// Per-warp state of one list entry.
struct EntryState
{
    float xi[kNcl], yi[kNcl], zi[kNcl], qi[kNcl];
    int   ti[kNcl];
    float fix[kNcl], fiy[kNcl], fiz[kNcl];
    float acc_el, cmp_el;              // sum q_i (q_j h_ij), compensated
    float acc_lj, cmp_lj;
};

// All pair interactions of one (cj4, warp half).  kExcl: this half has an
// exclusion mask (diagonal cluster pair or topology exclusions).  The loop
// over the 4 j-clusters stays rolled and only the loop over the 8 i-clusters
// (register-resident i-data) is unrolled, which keeps the kernel inside the
// instruction cache.
template<bool kEnergy, bool kEwald, bool kExcl, int kLj = 0>
__device__ __forceinline__ void process_half(const DeviceView& v, const SysPtrs& p, const float4* __restrict__ nbfp_s,
                                             const float4* __restrict__ jx, const int* __restrict__ jt,
                                             EntryState& st, const int cj_lane, unsigned im, unsigned wexcl,
                                             int h, int sci, bool central, int ii, int jj, float rc2, float pbeta,
                                             float beta2l2, float c2b, float k_rf2)
{
    const unsigned full = 0xffffffffu;
#pragma unroll 1
    for (int jm = 0; jm < kJg; jm++)
    {
        const unsigned imj = (im >> (jm * kNcl)) & 0xffu;
        const int      cj  = __shfl_sync(full, cj_lane, jm);
        if (!imj)
        {
            continue;
        }
        const int    aj  = cj * kCl + h * (kCl / kSplit) + jj;
        // the cj4 group's 32 j-atoms are staged in shared memory (slot jm * 8 + atom)
        const float4 xj  = jx[jm * kCl + h * (kCl / kSplit) + jj];
        const int    tj  = jt[jm * kCl + h * (kCl / kSplit) + jj];
        const float  qje = xj.w * v.epsfac;
        const unsigned wj = wexcl >> (jm * kNcl);
        float        fjx = 0.0f, fjy = 0.0f, fjz = 0.0f;
        // energies of this j-atom's (up to 8) pairs: plain float partial sums, folded
        // into the compensated per-lane totals once per j-cluster
        float        ej_el = 0.0f, ej_lj = 0.0f;
#pragma unroll
        for (int c = 0; c < kNcl; c++)
        {
            if (!(imj & (1u << c)))
            {
                continue;
            }
            const float dx = st.xi[c] - xj.x;
            const float dy = st.yi[c] - xj.y;
            const float dz = st.zi[c] - xj.z;
            float       r2 = dx * dx + dy * dy + dz * dz;
            float       mask, int_bit;
            if (kExcl)
            {
                // the diagonal cluster pair counts j > i only (kernel_gpu_ref.cpp:242)
                const bool self_lower = central && (sci * kNcl + c == cj) && (h * (kCl / kSplit) + jj <= ii);
                mask    = (r2 < rc2 && !self_lower) ? 1.0f : 0.0f;
                int_bit = (wj & (1u << c)) ? 1.0f : 0.0f;
            }
            else
            {
                mask    = (r2 < rc2) ? 1.0f : 0.0f;
                int_bit = 1.0f;
            }
            const bool in_range = kExcl ? (mask != 0.0f) : (r2 < rc2);
            r2         = fmaxf(r2, kMinDist2);
            float rinv = rsqrtf(r2);
            if (kEnergy)
            {
                // one Newton step: rsqrt.approx -> ~correctly rounded, unbiased for the energy sums
                rinv = rinv * (1.5f - 0.5f * r2 * rinv * rinv);
            }
            const float  rinv2 = rinv * rinv;
            float4       lj;
            if (kEnergy || kLj == 3)
            {
                lj = nbfp_s[st.ti[c] + tj];
            }
            else
            {
                const float2 l2 = *reinterpret_cast<const float2*>(&nbfp_s[st.ti[c] + tj]);
                lj              = make_float4(l2.x, l2.y, 0.0f, 0.0f);
            }
            float       rinv6    = rinv2 * rinv2 * rinv2;
            const float rinv6_nm = rinv6;  // LJ-PME: the grid part also acts on excluded pairs
            if (kExcl)
            {
                rinv6 *= int_bit;
            }
            // everything below is F r^2 until the one multiply by rinv2
            const float c12r6 = lj.y * rinv6;
            const float vdisp = lj.x * rinv6;
            float       flj   = fmaf(c12r6, rinv6, -vdisp);  // vrep - vdisp, vrep = 12 C12 / r^12
            // LJ energy: vrep/12 - vdisp/6 + (shift constant of this type pair) = (flj - vdisp)/12 + shift
            float vlj = (kEnergy || kLj == 2) ? fmaf(flj - vdisp, 1.0f / 12.0f, lj.z) : 0.0f;
            if (kLj == 3)
            {
                // LJ-PME, geometric grid c6grid = lj.w (kernel_ref_inner.h:204-252): subtract the grid
                // part c6grid (1 - e^-b (1 + b + b^2/2)) / r^6, b = beta_lj^2 r^2, from F r and V
                const float cr2  = v.lje_coeff2 * r2;
                const float expm = fast_ex2(-1.4426950408889634f * cr2);
                const float poly = fmaf(0.5f * cr2, cr2, 1.0f + cr2);
                flj              = fmaf(lj.w, rinv6_nm - expm * fmaf(rinv6_nm, poly, v.lje_coeff6_6), flj);
                if (kEnergy)
                {
                    // the grid potential's shift only for pairs that interact
                    vlj = fmaf(lj.w * (1.0f / 6.0f), fmaf(rinv6_nm, 1.0f - expm * poly, int_bit * v.sh_lj_ewald),
                               vlj);
                }
            }
            else if (kLj != 0)
            {
                // force / potential switch from rvdw_switch to rc (kernel_ref_inner.h:168-200)
                const float r   = r2 * rinv;
                const float rsw = fmaxf(r - v.rvdw_switch, 0.0f);
                const float rs2 = rsw * rsw;
                if (kLj == 1)
                {
                    // F r += (-6C6 (c2 + c3 rsw) + 12C12 (c2' + c3' rsw)) rsw^2 r; the energy gains
                    // the integral terms (-c2/3 - c3/4 rsw) rsw^3 of each
                    flj = fmaf((lj.y * fmaf(v.fsw_rep_c3, rsw, v.fsw_rep_c2)
                                - lj.x * fmaf(v.fsw_disp_c3, rsw, v.fsw_disp_c2))
                                       * rs2,
                               r, flj);
                    if (kEnergy)
                    {
                        const float erep  = fmaf(v.fsw_rep_c3 * -0.25f, rsw, v.fsw_rep_c2 * (-1.0f / 3.0f));
                        const float edisp = fmaf(v.fsw_disp_c3 * -0.25f, rsw, v.fsw_disp_c2 * (-1.0f / 3.0f));
                        vlj = fmaf(lj.y * erep - lj.x * edisp, rs2 * rsw, vlj);
                    }
                }
                else
                {
                    // sw = 1 + c3 rsw^3 + c4 rsw^4 + c5 rsw^5; F r = F r sw - r V dsw, V *= sw
                    const float sw  = fmaf(fmaf(fmaf(v.psw_c5, rsw, v.psw_c4), rsw, v.psw_c3), rs2 * rsw, 1.0f);
                    const float dsw = fmaf(fmaf(5.0f * v.psw_c5, rsw, 4.0f * v.psw_c4), rsw, 3.0f * v.psw_c3) * rs2;
                    flj             = fmaf(flj, sw, -r * vlj * dsw);
                    vlj *= sw;
                }
            }
            const float qq    = st.qi[c] * qje;
            float       fcr2;                                 // Coulomb F r^2 / (q_i q_j)
            float       h_el = 0.0f;  // q_i q_j h_el is the pair's Coulomb energy / epsfac
            if (kEwald)
            {
                // erfc(beta r) = t P(t) exp(-beta^2 r^2), t = 1/(1 + p beta r)
                const float r    = r2 * rinv;
                const float t    = fast_rcp(fmaf(pbeta, r, 1.0f));
                const float poly = erfc_poly(t);
                const float expm = fast_ex2(-beta2l2 * r2);
                const float tpr  = t * poly * rinv;  // erfc(beta r) / r = tpr * expm
                // -(d/dr)(erfc(beta r)/r) r = expm (erfc/r-part + 2 beta/sqrt(pi)); exclusions drop 1/r
                fcr2 = expm * (tpr + c2b);
                if (kExcl)
                {
                    fcr2 -= (1.0f - int_bit) * rinv;
                }
                if (kEnergy)
                {
                    h_el = fmaf(tpr, expm, -v.sh_ewald);
                }
            }
            else
            {
                fcr2 = kExcl ? fmaf(-k_rf2, r2, rinv * int_bit) : fmaf(-k_rf2, r2, rinv);
                if (kEnergy)
                {
                    h_el = (rinv - v.c_rf) + v.k_rf * r2;
                }
            }
            float fscal = fmaf(qq, fcr2, flj) * rinv2;
            fscal       = in_range ? fscal : 0.0f;
            if (kEnergy)
            {
                const bool counted = kExcl ? (in_range && int_bit != 0.0f) : in_range;
                // q_i h_ij here; q_j multiplies the j-cluster's sum
                ej_el = fmaf(st.qi[c], counted ? h_el : 0.0f, ej_el);
                ej_lj += counted ? vlj : 0.0f;
            }
            st.fix[c] = fmaf(fscal, dx, st.fix[c]);
            st.fiy[c] = fmaf(fscal, dy, st.fiy[c]);
            st.fiz[c] = fmaf(fscal, dz, st.fiz[c]);
            fjx       = fmaf(-fscal, dx, fjx);
            fjy       = fmaf(-fscal, dy, fjy);
            fjz       = fmaf(-fscal, dz, fjz);
        }
        if (kEnergy)
        {
            kahan_add(st.acc_el, st.cmp_el, xj.w * ej_el);
            kahan_add(st.acc_lj, st.cmp_lj, ej_lj);
        }
        // reduce the j force over the 8 i-lanes, one vector red per j-atom
#pragma unroll
        for (int o = 1; o < kCl; o <<= 1)
        {
            fjx += __shfl_xor_sync(full, fjx, o);
            fjy += __shfl_xor_sync(full, fjy, o);
            fjz += __shfl_xor_sync(full, fjz, o);
        }
        if (ii == 0)
        {
            red_add_v4(&p.fnb[aj], fjx, fjy, fjz);
        }
    }
}

// One list entry: load the 64 shifted i-atoms, all its cj4 groups, then the
// i-force, shift-force and energy reductions.  The entry's energies are added
// to e_lj_acc / e_el_acc (per lane, FP64).
// kLj: 0 potential shift or plain cut-off, 1 force switch, 2 potential switch, 3 LJ-PME (grid part).
template<bool kEnergy, bool kEwald, int kLj = 0>
__device__ __forceinline__ bool process_entry(const DeviceView& v, const SysPtrs& p, const Sci& s,
                                              const float4* __restrict__ nbfp_s, JStage& js, int nt1, int lane,
                                              int ii, int jj, float rc2, float pbeta, float beta2l2, float c2b,
                                              float k_rf2, double& e_lj_acc, double& e_el_acc)
{
    const unsigned full = 0xffffffffu;
    const float shx = p.shiftvec[3 * s.shift], shy = p.shiftvec[3 * s.shift + 1], shz = p.shiftvec[3 * s.shift + 2];
    const bool  central = (s.shift == kCentral);
    EntryState  st;
#pragma unroll
    for (int c = 0; c < kNcl; c++)
    {
        const int    ai = (s.sci * kNcl + c) * kCl + ii;
        const float4 x  = p.xq[ai];
        st.xi[c]        = x.x + shx;
        st.yi[c]        = x.y + shy;
        st.zi[c]        = x.z + shz;
        st.qi[c]        = x.w;
        st.ti[c]        = p.tgrid[ai] * nt1;
        st.fix[c] = st.fiy[c] = st.fiz[c] = 0.0f;
    }
    st.acc_el = st.cmp_el = 0.0f;
    st.acc_lj = st.cmp_lj = 0.0f;
    // Pipeline over the cj4 groups: the 32 j-atoms of group k+1 are copied by the TMA
    // engine into the other stage buffer while group k is computed; the masks and
    // j-cluster indices of k+1 are loaded into registers ahead as well.
    int4           rec_ime{};
    int            rec_cj = 0;
    if (s.cj4_start < s.cj4_end)
    {
        rec_ime = *reinterpret_cast<const int4*>(&p.cj4[s.cj4_start].imei[0]);
        rec_cj  = (lane < kJg) ? p.cj4[s.cj4_start].cj[lane] : 0;
        __syncwarp();
        if (lane < kJg)
        {
            stage_issue(js, js.uses & 1, lane, rec_cj, p.xq, p.tgrid, v.wait_test_bytes);
        }
    }
    for (int j4 = s.cj4_start; j4 < s.cj4_end; j4++)
    {
        const int4     ime     = rec_ime;
        const int      cj_lane = rec_cj;
        const int      b       = js.uses & 1;
        const unsigned parity  = (js.uses >> 1) & 1;
        const bool     more    = j4 + 1 < s.cj4_end;
        if (more)
        {
            rec_ime = *reinterpret_cast<const int4*>(&p.cj4[j4 + 1].imei[0]);
            rec_cj  = (lane < kJg) ? p.cj4[j4 + 1].cj[lane] : 0;
            __syncwarp();  // the other buffer's last readers (group k-1) are done
            if (lane < kJg)
            {
                stage_issue(js, b ^ 1, lane, rec_cj, p.xq, p.tgrid, v.wait_test_bytes);
            }
        }
        if (!stage_wait(js, b, parity))
        {
            return false;
        }
        js.uses++;
        const float4* jx = js.x + b * 32;
        const int*    jt = js.t + b * 32;
#pragma unroll 1
        for (int h = 0; h < kSplit; h++)
        {
            const unsigned im  = (h == 0) ? (unsigned)ime.x : (unsigned)ime.z;
            const int      exi = (h == 0) ? ime.y : ime.w;
            if (!im)
            {
                continue;
            }
            if (exi == 0)
            {
                process_half<kEnergy, kEwald, false, kLj>(v, p, nbfp_s, jx, jt, st, cj_lane, im, 0u, h, s.sci, central,
                                                     ii, jj, rc2, pbeta, beta2l2, c2b, k_rf2);
            }
            else
            {
                const unsigned wexcl = p.excl[exi].pair[lane];
                process_half<kEnergy, kEwald, true, kLj>(v, p, nbfp_s, jx, jt, st, cj_lane, im, wexcl, h, s.sci,
                                                    central, ii, jj, rc2, pbeta, beta2l2, c2b, k_rf2);
            }
        }
    }
    // i forces: reduce over the 4 j-lanes of each i-atom
    float sfx = 0.0f, sfy = 0.0f, sfz = 0.0f;
#pragma unroll
    for (int c = 0; c < kNcl; c++)
    {
        float fx = st.fix[c], fy = st.fiy[c], fz = st.fiz[c];
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
        e_el_acc += (double)st.acc_el - (double)st.cmp_el;
        e_lj_acc += (double)st.acc_lj - (double)st.cmp_lj;
    }
    if (!central)
    {
        // shift forces for the virial (the central shift vector is zero)
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

// Per-warp j stage in a kernel's dynamic shared memory, after a table of `table_f4`
// float4: [nwarps][64] float4 of xq, [nwarps][64] int of types, [nwarps][2] barriers.
__device__ __forceinline__ JStage stage_carve(float4* smem, int table_f4, int warp, int nwarps)
{
    float4* base = smem + table_f4;
    JStage  js;
    js.x   = base + warp * 64;
    js.t   = reinterpret_cast<int*>(base + nwarps * 64) + warp * 64;
    js.bar = reinterpret_cast<unsigned long long*>(reinterpret_cast<int*>(base + nwarps * 64) + nwarps * 64) + warp * 2;
    js.uses = 0;
    return js;
}
constexpr int kStageSmemPerWarp = 64 * 16 + 64 * 4 + 2 * 8;

// After a stage wait gave up: flag the timeout, give the copies in flight a bounded
// second chance to land, then the warp leaves the kernel.
__device__ __forceinline__ void stage_timeout(const JStage& js, unsigned* status, int lane)
{
    if (lane == 0)
    {
        atomicOr(status, (unsigned)kStatusTimeout);
    }
    const unsigned u = js.uses;
    stage_wait(js, u & 1, (u >> 1) & 1);
    stage_wait(js, (u + 1) & 1, ((u + 1) >> 1) & 1);
}

// Box edges of a system: the single-system view keeps them in its grid geometry.
__device__ __forceinline__ float sys_box(const DeviceView& v, int d)
{
    return v.g.box[d];
}
__device__ __forceinline__ float sys_box(const BatchSys& b, int d)
{
    return b.box[d];
}

// Coulomb energy of the excluded pairs within rc, summed in FP64 (Ewald: the
// series of erf(x)/x with its tail in float, erf_over_x_series), from the exclusion
// lists: every excluded pair i < j and every periodic image of it with
// r^2 < rc^2 in the pair kernel's float arithmetic, i.e. exactly the
// excluded pairs the list-based kernel sees (the half list holds each image
// pair once).  Ewald: -q_i q_j erf(beta r)/r; RF: q_i q_j (k_rf r^2 - c_rf)
// (kernel_gpu_ref.cpp:259-291 with int_bit = 0).  Energies only.

constexpr int kExclChunkAtoms = 128;  // atoms per exclusion work item of the force kernels (4 per lane)

// The excluded pairs (j > i) and the self term of atom i of system b (a DeviceView or a
// BatchSys: coordinates, cells, exclusion lists, shift vectors, box): Coulomb terms into acc
// (scaled by epsfac by the caller), the Ewald series sums into acc_s (scaled by
// -beta 2/sqrt(pi) by the caller), the LJ-PME grid part into acc_lj (single systems only).
// The interaction constants come from v.
template<class Sys>
__device__ __forceinline__ void excl_atom(const DeviceView& v, const Sys& b, int i, bool ljpme, double beta2,
                                          double& acc, double& acc_s, double& acc_lj)
{
    const float4 xi  = b.xq[b.cells[i]];
    const double qi  = (double)xi.w;
    const int    nt1 = v.ntypes1;
    const float  sci = ljpme ? sqrtf(v.nbfp[v.type[i] * (nt1 + 1)].x) : 0.0f;
    if (b.self_on_device)
    {
        // self term, kernel_gpu_ref.cpp:154-178 (acc is scaled by epsfac by the caller)
        acc += (double)xi.w * (double)xi.w
               * (v.coulomb == 0 ? -(double)v.beta * 0.56418958354775628695 : -0.5 * (double)v.c_rf);
    }
    const int    nx  = (sys_box(b, 0) < v.rlist) ? 2 : 1;
    // a box edge of at least 2 rc leaves one image within rc in that dimension: the nearest
    // (same shift-vector arithmetic as the full image loop, so the same float results)
    const float  rc  = sqrtf(v.rc2);
    for (int k = b.excl_index[i]; k < b.excl_index[i + 1]; k++)
    {
        const int j = b.excl_list[k];
        if (j <= i)
        {
            continue;
        }
        const float4 xj  = b.xq[b.cells[j]];
        int          lo[3], hi[3];
        const float  xd[3] = { xj.x - xi.x, xj.y - xi.y, xj.z - xi.z };
        for (int d = 0; d < 3; d++)
        {
            const int lim = d == 0 ? nx : 1;
            if (sys_box(b, d) >= 2.0f * rc)
            {
                const int t = min(max((int)rintf(xd[d] / sys_box(b, d)), -lim), lim);
                lo[d] = hi[d] = t;
            }
            else
            {
                lo[d] = -lim;
                hi[d] = lim;
            }
        }
        for (int tz = lo[2]; tz <= hi[2]; tz++)
        {
            for (int ty = lo[1]; ty <= hi[1]; ty++)
            {
                for (int tx = lo[0]; tx <= hi[0]; tx++)
                {
                    const int   s  = 5 * (3 * (tz + 1) + ty + 1) + tx + 2;
                    const float dx = (xi.x + b.shiftvec[3 * s]) - xj.x;
                    const float dy = (xi.y + b.shiftvec[3 * s + 1]) - xj.y;
                    const float dz = (xi.z + b.shiftvec[3 * s + 2]) - xj.z;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    if (!(r2 < v.rc2))
                    {
                        continue;
                    }
                    const double qq  = qi * (double)xj.w;
                    // r^2 in FP64 from the float differences, only where the series is not used
                    auto r2_fp64 = [&]() {
                        return fmax((double)dx * dx + (double)dy * dy + (double)dz * dz, (double)kMinDist2);
                    };
                    if (v.coulomb == 0)
                    {
                        // -erf(beta r)/r = -beta 2/sqrt(pi) S(beta^2 r^2); excluded pairs are
                        // short (beta r <= 1), so S comes from its series (the factor is
                        // applied once per thread by the caller).  w from the float r^2: its rounding
                        // differs from pair to pair and averages out in the sum.
                        const double w = beta2 * (double)r2;
                        if (w <= 1.0)
                        {
                            acc_s = fma(qq, erf_over_x_series(w), acc_s);
                        }
                        else
                        {
                            const double rd = sqrt(r2_fp64());
                            acc -= qq * erf((double)v.beta * rd) / rd;
                        }
                    }
                    else
                    {
                        acc += qq * ((double)v.k_rf * r2_fp64() - (double)v.c_rf);
                    }
                    if (ljpme)
                    {
                        // c6grid / 6 r^-6 (1 - e^-b (1 + b + b^2/2)), b = beta_lj^2 r^2
                        const int    tj     = v.type[j];
                        const double c6grid = (double)(sci * sqrtf(v.nbfp[tj * (nt1 + 1)].x));
                        const double r2d    = r2_fp64();
                        const double b      = (double)v.lje_coeff2 * r2d;
                        const double ir6    = 1.0 / (r2d * r2d * r2d);
                        acc_lj += c6grid / 6.0 * ir6 * (1.0 - exp(-b) * (1.0 + b + 0.5 * b * b));
                    }
                }
            }
        }
    }
}

// Work item t of k_force's queue: list entries E and exclusion chunks C interleaved, one chunk
// after every E / C entries (the chunks' FP64 and gather work then overlaps other warps' pair
// work instead of running as a separate launch); idx is the entry or the chunk.
__device__ __forceinline__ bool item_is_chunk(int t, int E, int C, int& idx)
{
    if (C == 0)
    {
        idx = t;
        return false;
    }
    const int s = E / C;
    if (s >= 1)
    {
        const int q = t / (s + 1), r = t - q * (s + 1);
        if (q < C)
        {
            idx = (r == s) ? q : q * s + r;
            return r == s;
        }
        idx = C * s + (t - C * (s + 1));
        return false;
    }
    if (t < 2 * E)
    {
        idx = t >> 1;
        return (t & 1) != 0;
    }
    idx = E + (t - 2 * E);
    return true;
}

} // namespace nbx
