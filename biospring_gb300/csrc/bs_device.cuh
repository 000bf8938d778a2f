// bs_device.cuh -- device functions shared by the single-system and the batched kernels:
// order-preserving float codes, own reciprocal and square-root refinements, the reference's
// cell coordinate and exact pair test, compensated energy sums, and the per-particle force and
// integration routine of one step.
#pragma once

#include <cfloat>
#include <climits>

#include "bs_kernels.cuh"

namespace bsg
{
namespace
{


__device__ __forceinline__ int status_of(const Ctl *c) { return *(volatile const int *)&c->status; }

// Programmatic dependent launch: lets the next kernel of the stream begin launching now, then waits
// until the previous kernel has completed and its writes are visible. The launch of the next
// kernel thus overlaps this one; both instructions are no-ops for a kernel launched without the
// programmatic-serialization attribute. Every kernel of the rebuild and step chains calls it first.
__device__ __forceinline__ void pdl_enter()
{
#if BS_PDL
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}

__device__ __forceinline__ unsigned int f2ord(float f)
{
    const unsigned int b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned int u)
{
    const unsigned int b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    return __uint_as_float(b);
}

// 1/x: hardware approximation refined by one Newton-Raphson step for f(r) = 1/r - x,
// r1 = r0 + r0 (1 - x r0); about one unit in the last place for normal x.
__device__ __forceinline__ float recip_nr(float x)
{
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return fmaf(r, fmaf(-x, r, 1.0f), r);
}

// 1/x for the LJ pair body: the refined reciprocal, or (BS_LJ_RCP_REFINE 0) the hardware
// approximation alone.
__device__ __forceinline__ float recip_lj(float x)
{
#if BS_LJ_RCP_REFINE
    return recip_nr(x);
#else
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#endif
}

// 1/sqrt(x): hardware approximation refined by one Newton-Raphson step for
// f(r) = 1/r^2 - x, r1 = r0 (3 - x r0^2) / 2.
__device__ __forceinline__ float rsqrt_nr(float x)
{
    float r;
    asm("rsqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r * fmaf(-0.5f * x, r * r, 1.5f);
}

// Reference cell coordinate along one axis: (size_t)((x - min) / radius), clamped (nsearch.hpp:282-289).
__device__ __forceinline__ int ref_cell_coord(float x, double mn, float radius, int ncell)
{
    const double t = __ddiv_rn(__dsub_rn(static_cast<double>(x), mn), static_cast<double>(radius));
    unsigned long long c = static_cast<unsigned long long>(t);
    const unsigned long long lim = static_cast<unsigned long long>(ncell - 1);
    return static_cast<int>(c < lim ? c : lim);
}

// Search grid over the box [mn, mx] with cell edge `edge`: ncells = ceil(len / edge) + 1 per
// axis in FP64 (nsearch.hpp:351-354), minimum corner as double. Returns the total cell count as a
// double (it can exceed the int range; the per-axis counts saturate at 1e9).
__device__ __forceinline__ double grid_dims(const float (&mn)[3], const float (&mx)[3], float edge, double (&gmin)[3],
                                            int (&nc)[3])
{
    const double r = static_cast<double>(edge);
    double cells = 1.0;
    for (int k = 0; k < 3; ++k)
    {
        const double len = __dsub_rn(static_cast<double>(mx[k]), static_cast<double>(mn[k]));
        const double c = ceil(__ddiv_rn(len, r)) + 1.0;
        cells *= c;
        nc[k] = c < 1.0e9 ? static_cast<int>(c) : 1000000000;
        gmin[k] = static_cast<double>(mn[k]);
    }
    return cells;
}

// Exact reference test of one candidate pair for one cutoff: the grid filter compares the FP64
// distance of the float coordinates (nsearch.hpp:230, measure.hpp:163-169); the force routine
// then compares the float-rounded FP64 norm of the float difference vector (Particle.cpp:222-224,
// Vector3f.cpp:9-12, measure.hpp:188-196). Only pairs inside the guard band come here.
__device__ __noinline__ bool exact_pair_test(float4 pi, float4 pj, float cutoff, bool nonzero)
{
    const double ax = __dsub_rn(static_cast<double>(pi.x), static_cast<double>(pj.x));
    const double ay = __dsub_rn(static_cast<double>(pi.y), static_cast<double>(pj.y));
    const double az = __dsub_rn(static_cast<double>(pi.z), static_cast<double>(pj.z));
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay)), __dmul_rn(az, az));
    if (!(__dsqrt_rn(s) < static_cast<double>(cutoff)))
        return false;
    const double fx = static_cast<double>(__fsub_rn(pj.x, pi.x));
    const double fy = static_cast<double>(__fsub_rn(pj.y, pi.y));
    const double fz = static_cast<double>(__fsub_rn(pj.z, pi.z));
    double nrm = 0.0;
    if (!(fabs(fx) < 1e-40 && fabs(fy) < 1e-40 && fabs(fz) < 1e-40))
        nrm = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(fx, fx), __dmul_rn(fy, fy)), __dmul_rn(fz, fz)));
    const float d = __double2float_rn(nrm);
    if (!(d < cutoff))
        return false;
    if (nonzero && !(d != 0.0f))
        return false;
    return true;
}

// Classifies a pair for one term. Outside the band [lo2, hi2) the FP32 squared distance decides
// (its error is far below the band); inside it, and for (near-)coincident particles, the exact
// reference test decides.
__device__ __forceinline__ bool pair_in(float r2, float lo2, float hi2, float4 pi, float4 pj, float cutoff,
                                        bool nonzero)
{
    if (r2 >= hi2)
        return false;
    if (r2 < lo2 && r2 > 1e-20f)
        return true;
    return exact_pair_test(pi, pj, cutoff, nonzero);
}

// Knuth's TwoSum: s = fl(a + b) and s + err == a + b exactly (round-to-nearest, no contraction).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &err)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (hi, lo) += (h2, l2) in float-float (double-single) arithmetic: about 44 significant bits.
__device__ __forceinline__ void ff_add(float &hi, float &lo, float h2, float l2)
{
    float s, e;
    two_sum(hi, h2, s, e);
    e = __fadd_rn(e, __fadd_rn(lo, l2));
    two_sum(s, e, hi, lo);
}

// Deterministic reduction of NE per-thread float partials over the grid, in three levels:
// block -> group of kEnergyGroup consecutive blocks -> grid. Warp sums are FP32 trees; above the
// warp every sum is float-float (compensated, about 44 significant bits). The last block of a
// group to finish sums the group's block partials, and the last group to finish sums the group
// partials and writes the totals as double. Every sum runs in a fixed order (lane = block or
// group index, a fixed shuffle tree), so the result does not depend on which block finishes
// last. The group level keeps the serial tail short: the final block reads a few hundred
// partials instead of one per block of the grid. The result carries the accuracy of an FP64
// reduction without the FP64 pipe, which runs at a small fraction of the FP32 rate on this part.
//
// blk_d holds [blk_cap][16] floats of block partials ((hi, lo) per energy), then
// [energy_groups(blk_cap)][16] floats of group partials, then one counter per group; the
// counters and *done start at zero and are reset by the block that completes them.
// (hi, lo) of lane `lane` summed over the warp in a fixed tree; the total lands in lane 0.
__device__ __forceinline__ void warp_ff_sum(float &hi, float &lo)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        const float h2 = __shfl_down_sync(0xffffffffu, hi, o);
        const float l2 = __shfl_down_sync(0xffffffffu, lo, o);
        ff_add(hi, lo, h2, l2);
    }
}

template <int NE, int BLOCK>
__device__ __forceinline__ bool reduce_energies(const float (&e)[NE], double *blk_d, int blk_cap, unsigned int *done,
                                                double *dst)
{
    static_assert(NE <= 8, "16 floats per partial");
    float *blk = reinterpret_cast<float *>(blk_d);
    float *grp = blk + static_cast<size_t>(blk_cap) * 16;
    const int ngrp = energy_groups(gridDim.x);
    unsigned int *grp_cnt = reinterpret_cast<unsigned int *>(grp + static_cast<size_t>(energy_groups(blk_cap)) * 16);
    __shared__ float shh[NE][BLOCK / 32], shl[NE][BLOCK / 32];
    __shared__ bool am_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NE; ++k)
    {
        // 32 terms: a plain FP32 tree keeps ~1e-7 relative; compensation starts above the warp
        float v = e[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0)
        {
            shh[k][warp] = v;
            shl[k][warp] = 0.0f;
        }
    }
    __syncthreads();
    if (threadIdx.x < NE)
    {
        float hi = 0.0f, lo = 0.0f;
        for (int w = 0; w < BLOCK / 32; ++w)
            ff_add(hi, lo, shh[threadIdx.x][w], shl[threadIdx.x][w]);
        blk[static_cast<size_t>(blockIdx.x) * 16 + 2 * threadIdx.x] = hi;
        blk[static_cast<size_t>(blockIdx.x) * 16 + 2 * threadIdx.x + 1] = lo;
    }
    // ---- group level: the last block of the group sums its kEnergyGroup block partials ----
    const int g = blockIdx.x / kEnergyGroup;
    const int g0 = g * kEnergyGroup;
    const int gsize = min(kEnergyGroup, static_cast<int>(gridDim.x) - g0);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0)
        am_last = atomicAdd(&grp_cnt[g], 1u) == static_cast<unsigned int>(gsize - 1);
    __syncthreads();
    if (!am_last)
        return false;
    __threadfence();
    for (int k = warp; k < NE; k += BLOCK / 32)
    {
        float hi = 0.0f, lo = 0.0f;
        if (lane < gsize)
        {
            const float2 v = __ldcg(reinterpret_cast<const float2 *>(blk + static_cast<size_t>(g0 + lane) * 16 + 2 * k));
            hi = v.x;
            lo = v.y;
        }
        warp_ff_sum(hi, lo);
        if (lane == 0)
        {
            grp[static_cast<size_t>(g) * 16 + 2 * k] = hi;
            grp[static_cast<size_t>(g) * 16 + 2 * k + 1] = lo;
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0)
    {
        grp_cnt[g] = 0u;
        am_last = atomicAdd(done, 1u) == static_cast<unsigned int>(ngrp - 1);
    }
    __syncthreads();
    if (!am_last)
        return false;
    __threadfence();
    // ---- grid level: lane l sums groups l, l + 32, ... in order, then a fixed warp tree ----
    for (int k = warp; k < NE; k += BLOCK / 32)
    {
        float hi = 0.0f, lo = 0.0f;
        for (int q = lane; q < ngrp; q += 32)
        {
            const float2 v = __ldcg(reinterpret_cast<const float2 *>(grp + static_cast<size_t>(q) * 16 + 2 * k));
            ff_add(hi, lo, v.x, v.y);
        }
        warp_ff_sum(hi, lo);
        if (lane == 0)
            dst[k] = static_cast<double>(hi) + static_cast<double>(lo);
    }
    __syncthreads();
    if (threadIdx.x == 0)
        *done = 0u;
    return true;
}

// Springs of slot s handled by lane t of T (Spring.cpp:20-34, spring.hpp:17-29). Returns the
// force before the unit conversion and scale, and the weighted energy before the scale.
template <int T>
__device__ __forceinline__ void spring_forces(const Params &p, int s, int t, float4 pi,
                                              const float4 *__restrict__ pos, float &fx, float &fy, float &fz,
                                              float &e)
{
    const int deg = p.se_deg[s];
    if (t >= deg)
        return;
    const size_t stride = static_cast<size_t>(p.npad);
    // software-pipelined: the next entry and its partner position are loaded before this one is used
    size_t at = static_cast<size_t>(t) * stride + s;
    unsigned int cn = __ldg(&p.se_col[at]);
    float kn = __ldg(&p.se_k[at]), rn = __ldg(&p.se_r0[at]);
    float4 pn = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!(cn & kEntryInactive))
        pn = __ldg(&pos[cn & kSlotMask]);
    for (int k = t; k < deg; k += T)
    {
        const unsigned int c = cn;
        const float kk = kn, r0 = rn;
        const float4 pj = pn;
        if (k + T < deg)
        {
            at += static_cast<size_t>(T) * stride;
            cn = __ldg(&p.se_col[at]);
            kn = __ldg(&p.se_k[at]);
            rn = __ldg(&p.se_r0[at]);
            if (!(cn & kEntryInactive))
                pn = __ldg(&pos[cn & kSlotMask]);
        }
        if (c & kEntryInactive)
            continue;
        const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float inv = r2 > 0.0f ? rsqrt_nr(r2) : 0.0f;
        const float len = r2 * inv;
        const float dv = len - r0;
        const float w = (c & kEntryStatic) ? 1.0f : 0.5f;
        e = fmaf(w * 0.5f * kk, dv * dv, e);
        const float fod = kk * dv * inv;
        fx = fmaf(dx, fod, fx);
        fy = fmaf(dy, fod, fy);
        fz = fmaf(dz, fod, fz);
    }
}

// Steric pairs of slot s handled by lane t of T (Particle.cpp:368-429, steric.hpp:27-156).
// KIND 0: list 0 in 16-bit mode (partner = slot + offset, dynamic partners, half the pair
// energy); KIND 1: list 0 in 32-bit mode; KIND 2: list 3 (static partners, full energy).
// The loop is software-pipelined: entries are loaded two iterations ahead of use and
// positions (and the LJ factor of the partner) one iteration ahead.
template <int SM, int T, int KIND>
__device__ __forceinline__ void steric_forces(const Params &p, int s, int t, float4 pi, float fhi_i,
                                              const float4 *__restrict__ pos, const float *__restrict__ fhi,
                                              float &fx, float &fy, float &fz, float &e)
{
    const PairList &L = p.pl[KIND == 2 ? kListStericStatic : 0];
    const int cnt = L.cnt[s];
    if (t >= cnt)
        return;
    const size_t row = static_cast<size_t>(s) * L.cap;
    const short *__restrict__ idx16 = reinterpret_cast<const short *>(L.idx) + row;
    const unsigned int *__restrict__ idx32 = L.idx + row;
    auto entry = [&](int k) -> int {
        if (KIND == 0)
            return s + static_cast<int>(__ldg(idx16 + k));
        return static_cast<int>(__ldg(idx32 + k) & kSlotMask);
    };
    const float lo2 = p.lo2_s, hi2 = p.hi2_s;
    const float w = KIND == 2 ? 1.0f : 0.5f;
    constexpr bool LJ = SM != BS_STERIC_LINEAR;
    int jn = entry(t);
    int jn2 = t + T < cnt ? entry(t + T) : 0;
    float4 pn = __ldg(&pos[jn]);
    float hn = LJ ? __ldg(&fhi[jn]) : 0.0f;
    for (int k = t; k < cnt; k += T)
    {
        const float4 pj = pn;
        const float hj = hn;
        jn = jn2;
        if (k + 2 * T < cnt)
            jn2 = entry(k + 2 * T);
        if (k + T < cnt)
        {
            pn = __ldg(&pos[jn]);
            if (LJ)
                hn = __ldg(&fhi[jn]);
        }
        const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (SM == BS_STERIC_LINEAR)
        {
            // Few listed pairs overlap: the branches skip the square root and division of the rest.
            if (r2 >= hi2)
                continue;
            if (!(r2 < lo2 && r2 > 1e-20f) && !exact_pair_test(pi, pj, p.c_steric, false))
                continue;
            // steric.hpp:37-59: E = (d - (ri + rj))^2 / 2 when overlapping, |F| = |d - (ri + rj)|.
            // d - (ri + rj) cancels near contact, so d is the correctly rounded square root here.
            const float d = sqrtf(r2);
            const float inv = d > 0.0f ? 1.0f / d : 0.0f;
            const float dv = d - (pi.w + pj.w);
            if (dv > 0.0f)
                continue;
            e = fmaf(w * 0.5f, dv * dv, e);
            const float fod = dv * inv; // -|dv| / d
            fx = fmaf(dx, fod, fx);
            fy = fmaf(dy, fod, fy);
            fz = fmaf(dz, fod, fz);
        }
        else
        {
            // Most listed pairs are inside the cutoff: the body is branch-free and a rejected
            // entry adds exact zeros (selects, not products, so an infinite or NaN term of a
            // rejected pair cannot leak in). Only entries inside the guard band, or
            // (near-)coincident, branch to the exact reference test.
            bool ok = r2 < lo2 && r2 > 1e-20f;
            if (!ok && r2 < hi2)
                ok = exact_pair_test(pi, pj, p.c_steric, false);
            ok = ok && !(r2 < 0.01f); // d < 0.1 A: the LJ forms give zero (steric.hpp:71-72)
            const float inv2 = recip_nr(r2);
            const float i6 = inv2 * inv2 * inv2;
            const float t6 = pi.w * pj.w * i6;
            float fod, de;
            if (SM == BS_STERIC_LJ_12_6_AMBER)
            {
                const float t12 = fhi_i * hj * i6 * i6;
                de = t12 - 2.0f * t6;
                fod = 12.0f * (t6 - t12) * inv2;
            }
            else if (SM == BS_STERIC_LJ_8_6_LEWITT)
            {
                const float t8 = fhi_i * hj * i6 * inv2;
                de = 3.0f * t8 - 4.0f * t6;
                fod = 24.0f * (t6 - t8) * inv2;
            }
            else
            {
                const float t8 = fhi_i * hj * i6 * inv2;
                de = t8 - t6;
                fod = (6.0f * t6 - 8.0f * t8) * inv2;
            }
            e = fmaf(w, ok ? de : 0.0f, e);
            fod = ok ? fod : 0.0f;
            fx = fmaf(dx, fod, fx);
            fy = fmaf(dy, fod, fy);
            fz = fmaf(dz, fod, fz);
        }
    }
}

// The LJ pair body of steric_forces: adds the pair's weighted energy to e and returns the force
// over distance (both zero for a rejected pair). ok says whether the pair is in the cutoff.
template <int SM>
__device__ __forceinline__ float lj_pair(float r2, bool ok, float pw, float fhi_i, float4 pj, float hj, float w,
                                         float &e)
{
    const float inv2 = recip_lj(r2);
    const float i6 = inv2 * inv2 * inv2;
    const float t6 = pw * pj.w * i6;
    float fod, de;
    if (SM == BS_STERIC_LJ_12_6_AMBER)
    {
        const float t12 = fhi_i * hj * i6 * i6;
        de = t12 - 2.0f * t6;
        fod = 12.0f * (t6 - t12) * inv2;
    }
    else if (SM == BS_STERIC_LJ_8_6_LEWITT)
    {
        const float t8 = fhi_i * hj * i6 * inv2;
        de = 3.0f * t8 - 4.0f * t6;
        fod = 24.0f * (t6 - t8) * inv2;
    }
    else
    {
        const float t8 = fhi_i * hj * i6 * inv2;
        de = t8 - t6;
        fod = (6.0f * t6 - 8.0f * t8) * inv2;
    }
    e = fmaf(w, ok ? de : 0.0f, e);
    return ok ? fod : 0.0f;
}

// Steric pairs of slot s with its dynamic partners (list 0), lane t of T, in passes of kGatherU
// consecutive entries per lane: lane t takes entries [base + U t, base + U t + U) with one vector
// load of the row (U offsets of 16 bits, or U slots), then issues the U partners' position and LJ
// factor loads together before any of them is used, so U gathers are in flight per lane and a
// warp waits for one round trip per U pairs instead of one per pair. Entries past the row's end
// read the slot past the particles (far from all of them) and fail the distance test. Rows start on 16-byte boundaries (capacities are
// multiples of 8 entries), so the vector loads are aligned and never leave the row's capacity.
template <int SM, int T, bool PL16, bool UF = false>
__device__ __forceinline__ void steric_forces_batched(const Params &p, int s, int t, float4 pi, float fhi_i,
                                                      const float4 *__restrict__ pos, const float *__restrict__ fhi,
                                                      float &fx, float &fy, float &fz, float &e, int cnt_in = -1,
                                                      uint2 w16_in = make_uint2(0u, 0u))
{
    constexpr int U = kGatherU;
    static_assert(U == 4, "one 8-byte (16-bit mode) or 16-byte (32-bit mode) load per pass");
    const PairList &L = p.pl[0];
    // cnt_in >= 0: the caller has already read the row's count and (16-bit rows) the lane's first
    // four entries
    const int cnt = cnt_in >= 0 ? cnt_in : L.cnt[s];
    const size_t row = static_cast<size_t>(s) * L.cap;
    const float lo2 = p.lo2_s, hi2 = p.hi2_s;
    constexpr bool LJ = SM != BS_STERIC_LINEAR;
    // BS_GATHER 3: the next pass's entries are loaded before this pass's partners, so the entry
    // load of a pass overlaps the previous pass instead of preceding its partner loads.
    uint2 w16n = w16_in;
    uint4 w32n = make_uint4(0u, 0u, 0u, 0u);
    if (BS_GATHER == 3 && U * t < cnt && !(PL16 && cnt_in >= 0))
    {
        if (PL16)
            w16n = __ldg(reinterpret_cast<const uint2 *>(reinterpret_cast<const short *>(L.idx) + row + U * t));
        else
            w32n = __ldg(reinterpret_cast<const uint4 *>(L.idx + row + U * t));
    }
    for (int base = (BS_GATHER == 2 ? t : U * t); base < cnt; base += U * T)
    {
        int j[U];
        if (BS_GATHER == 3)
        {
            const uint2 w16 = w16n;
            const uint4 w32 = w32n;
            if (base + U * T < cnt)
            {
                if (PL16)
                    w16n = __ldg(reinterpret_cast<const uint2 *>(reinterpret_cast<const short *>(L.idx) + row + base + U * T));
                else
                    w32n = __ldg(reinterpret_cast<const uint4 *>(L.idx + row + base + U * T));
            }
            if (PL16)
            {
                j[0] = s + static_cast<int>(static_cast<short>(w16.x & 0xffffu));
                j[1] = s + (static_cast<int>(w16.x) >> 16);
                j[2] = s + static_cast<int>(static_cast<short>(w16.y & 0xffffu));
                j[3] = s + (static_cast<int>(w16.y) >> 16);
            }
            else
            {
                j[0] = static_cast<int>(w32.x & kSlotMask);
                j[1] = static_cast<int>(w32.y & kSlotMask);
                j[2] = static_cast<int>(w32.z & kSlotMask);
                j[3] = static_cast<int>(w32.w & kSlotMask);
            }
        }
        else if (BS_GATHER == 2)
        {
            // interleaved: entries base + T u, so at each u the T lanes of the particle read
            // consecutive entries (neighbouring partner slots, often one cache line)
#pragma unroll
            for (int u = 0; u < U; ++u)
            {
                const int k = min(base + T * u, cnt - 1);
                if (PL16)
                    j[u] = s + static_cast<int>(__ldg(reinterpret_cast<const short *>(L.idx) + row + k));
                else
                    j[u] = static_cast<int>(__ldg(L.idx + row + k) & kSlotMask);
            }
        }
        else if (PL16)
        {
            const uint2 w = __ldg(reinterpret_cast<const uint2 *>(reinterpret_cast<const short *>(L.idx) + row + base));
            j[0] = s + static_cast<int>(static_cast<short>(w.x & 0xffffu));
            j[1] = s + (static_cast<int>(w.x) >> 16);
            j[2] = s + static_cast<int>(static_cast<short>(w.y & 0xffffu));
            j[3] = s + (static_cast<int>(w.y) >> 16);
        }
        else
        {
            const uint4 w = __ldg(reinterpret_cast<const uint4 *>(L.idx + row + base));
            j[0] = static_cast<int>(w.x & kSlotMask);
            j[1] = static_cast<int>(w.y & kSlotMask);
            j[2] = static_cast<int>(w.z & kSlotMask);
            j[3] = static_cast<int>(w.w & kSlotMask);
        }
        float4 pj[U];
        float hj[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
        {
            // past the row: a stale entry; the slot past the particles (far from every particle)
            // is read instead, and its squared distance (infinite) rejects it below
            if ((BS_GATHER == 2 ? base + T * u : base + u) >= cnt)
                j[u] = p.npad;
            pj[u] = __ldg(&pos[j[u]]);
            hj[u] = LJ ? (UF ? p.lj_F : __ldg(&fhi[j[u]])) : 0.0f; // one LJ type: no factor to gather
        }
        unsigned int band = 0u; // LJ pairs of this pass within the guard band (BS_LJ_BAND_AFTER)
#pragma unroll
        for (int u = 0; u < U; ++u)
        {
            const float dx = pj[u].x - pi.x, dy = pj[u].y - pi.y, dz = pj[u].z - pi.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (SM == BS_STERIC_LINEAR)
            {
                if (!(r2 < hi2))
                    continue;
                if (!(r2 < lo2 && r2 > 1e-20f) && !exact_pair_test(pi, pj[u], p.c_steric, false))
                    continue;
                const float d = sqrtf(r2);
                const float inv = d > 0.0f ? 1.0f / d : 0.0f;
                const float dv = d - (pi.w + pj[u].w);
                if (dv > 0.0f)
                    continue;
                e = fmaf(0.25f, dv * dv, e); // half the pair energy: weight 0.5 times E = dv^2 / 2
                const float fod = dv * inv;
                fx = fmaf(dx, fod, fx);
                fy = fmaf(dy, fod, fy);
                fz = fmaf(dz, fod, fz);
            }
            else
            {
                // The FP32 squared distance decides outside the guard band [lo2, hi2); inside it
                // (a few pairs per ten million) the exact test decides, either at once or
                // (BS_LJ_BAND_AFTER) after the pass, which keeps the branch out of the pair body
                // but the pass's partner data live longer. (Near-)coincident pairs need no exact
                // test: below 0.1 A the LJ forms give zero (steric.hpp:71-72).
#if BS_LJ_BAND_AFTER
                const bool ok = r2 < lo2 && r2 >= 0.01f;
                band |= (r2 >= lo2 && r2 < hi2) ? 1u << u : 0u;
#else
                bool ok = r2 < lo2;
                if (!ok && r2 < hi2)
                    ok = exact_pair_test(pi, pj[u], p.c_steric, false);
                ok = ok && r2 >= 0.01f;
#endif
                const float fod = lj_pair<SM>(r2, ok, pi.w, fhi_i, pj[u], hj[u], 0.5f, e);
                fx = fmaf(dx, fod, fx);
                fy = fmaf(dy, fod, fy);
                fz = fmaf(dz, fod, fz);
            }
        }
        if (BS_LJ_BAND_AFTER && SM != BS_STERIC_LINEAR && band)
        {
#pragma unroll
            for (int u = 0; u < U; ++u)
            {
                if (!((band >> u) & 1u) || !exact_pair_test(pi, pj[u], p.c_steric, false))
                    continue;
                const float dx = pj[u].x - pi.x, dy = pj[u].y - pi.y, dz = pj[u].z - pi.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                const float fod = lj_pair<SM>(r2, true, pi.w, fhi_i, pj[u], hj[u], 0.5f, e);
                fx = fmaf(dx, fod, fx);
                fy = fmaf(dy, fod, fy);
                fz = fmaf(dz, fod, fz);
            }
        }
    }
}

// Springs of slot s, lane t of T, in passes of kGatherU entries per lane (entries t + T u of the
// ELL row, the same entries in the same order as spring_forces): the U entries' columns are read
// first, then the U partner positions together.
template <int T>
__device__ __forceinline__ void spring_forces_batched(const Params &p, int s, int t, float4 pi,
                                                      const float4 *__restrict__ pos, float &fx, float &fy, float &fz,
                                                      float &e)
{
    constexpr int U = kGatherU;
    const int deg = p.se_deg[s];
    const size_t stride = static_cast<size_t>(p.npad);
    for (int k0 = t; k0 < deg; k0 += T * U)
    {
        unsigned int c[U];
        float kk[U], r0[U];
        float4 pj[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
        {
            const int k = k0 + u * T;
            c[u] = kEntryInactive;
            kk[u] = 0.0f;
            r0[u] = 0.0f;
            if (k < deg)
            {
                const size_t at = static_cast<size_t>(k) * stride + s;
                c[u] = __ldg(&p.se_col[at]);
                kk[u] = __ldg(&p.se_k[at]);
                r0[u] = __ldg(&p.se_r0[at]);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            pj[u] = (c[u] & kEntryInactive) ? pi : __ldg(&pos[c[u] & kSlotMask]);
#pragma unroll
        for (int u = 0; u < U; ++u)
        {
            if (c[u] & kEntryInactive)
                continue;
            const float dx = pj[u].x - pi.x, dy = pj[u].y - pi.y, dz = pj[u].z - pi.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            const float inv = r2 > 0.0f ? rsqrt_nr(r2) : 0.0f;
            const float len = r2 * inv;
            const float dv = len - r0[u];
            const float w = (c[u] & kEntryStatic) ? 1.0f : 0.5f;
            e = fmaf(w * 0.5f * kk[u], dv * dv, e);
            const float fod = kk[u] * dv * inv;
            fx = fmaf(dx, fod, fx);
            fy = fmaf(dy, fod, fy);
            fz = fmaf(dz, fod, fz);
        }
    }
}

// Coulomb pairs of a charged slot, lane t of T (Particle.cpp:191-253, electrostatic.hpp:16-49).
// With the distance-dependent dielectric eps = D r, E = K q q / (D r^2) and F = -dE/dr.
template <int T>
__device__ __forceinline__ void coulomb_forces(const Params &p, int s, int t, float4 pi, float qi,
                                               const float4 *__restrict__ pos, const float *__restrict__ chg,
                                               float &fx, float &fy, float &fz, float &e)
{
    const PairList &L = p.pl[1];
    const int cnt = L.cnt[s];
    const unsigned int *__restrict__ row = L.idx + static_cast<size_t>(s) * L.cap;
    const bool dist = p.dielectric_mode == BS_DIELECTRIC_DISTANCE;
    if (t >= cnt)
        return;
    // software-pipelined like the steric loop: entries two ahead, partner data one ahead
    unsigned int jn = __ldg(row + t);
    unsigned int jn2 = t + T < cnt ? __ldg(row + t + T) : 0u;
    float4 pn = __ldg(&pos[jn & kSlotMask]);
    float qn = __ldg(&chg[jn & kSlotMask]);
    for (int k = t; k < cnt; k += T)
    {
        const unsigned int j = jn;
        const float4 pj = pn;
        const float qj = qn;
        jn = jn2;
        if (k + 2 * T < cnt)
            jn2 = __ldg(row + k + 2 * T);
        if (k + T < cnt)
        {
            pn = __ldg(&pos[jn & kSlotMask]);
            qn = __ldg(&chg[jn & kSlotMask]);
        }
        const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (!pair_in(r2, p.lo2_c, p.hi2_c, pi, pj, p.c_coulomb, true))
            continue;
        if (r2 < 1e-6f) // d < 0.001 A gives zero (electrostatic.hpp:18-19)
            continue;
        const float inv = rsqrt_nr(r2);
        const float qq = qi * qj;
        const float w = (j & kEntryStatic) ? 1.0f : 0.5f;
        float tq = qq * inv;
        float fod;
        if (dist)
        {
            tq *= inv;
            fod = -2.0f * tq * inv * inv;
        }
        else
            fod = -tq * inv * inv;
        e = fmaf(w, tq, e);
        fx = fmaf(dx, fod, fx);
        fy = fmaf(dy, fod, fy);
        fz = fmaf(dz, fod, fz);
    }
}

// Hydrophobic pairs, lane t of T (Particle.cpp:269-330, hydrophobic.hpp:20-39).
template <int T>
__device__ __forceinline__ void hydro_forces(const Params &p, int s, int t, float4 pi, float hi,
                                             const float4 *__restrict__ pos, const float *__restrict__ hyd,
                                             float &fx, float &fy, float &fz, float &e)
{
    const PairList &L = p.pl[2];
    const int cnt = L.cnt[s];
    const unsigned int *__restrict__ row = L.idx + static_cast<size_t>(s) * L.cap;
    for (int k = t; k < cnt; k += T)
    {
        const unsigned int j = __ldg(row + k);
        const float4 pj = __ldg(&pos[j & kSlotMask]);
        const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (!pair_in(r2, p.lo2_h, p.hi2_h, pi, pj, p.c_hydro, true))
            continue;
        const float inv = rsqrt_nr(r2);
        const float d = r2 * inv;
        const float x = hi * __ldg(&hyd[j & kSlotMask]) * expf(-d);
        const float w = (j & kEntryStatic) ? 1.0f : 0.5f;
        e = fmaf(-w, x, e);
        const float fod = x * inv;
        fx = fmaf(dx, fod, fx);
        fy = fmaf(dy, fod, fy);
        fz = fmaf(dz, fod, fz);
    }
}

// Force of the probe on one dynamic particle at pi and the particle's share of the pair energies
// (Particle::addStericProbeForce / addElectrostaticProbeForce, Particle.cpp:434-465): no cutoff,
// the full pair energy counts (the reference adds it to the totals once per particle). The same
// pair kernels as the list terms, with the probe's own steric factors.
template <int SM>
__device__ __forceinline__ void probe_pair(const Params &p, const float4 &prb, float4 pi, float fhi_i, float qi,
                                           float &fx, float &fy, float &fz, float &es, float &ec)
{
    const float dx = prb.x - pi.x, dy = prb.y - pi.y, dz = prb.z - pi.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (p.probe_steric)
    {
        float fod = 0.0f;
        if (SM == BS_STERIC_LINEAR)
        {
            const float d = sqrtf(r2);
            const float dv = d - (p.probe_P + pi.w);
            if (dv <= 0.0f)
            {
                es = fmaf(0.5f * p.steric_scale, dv * dv, es);
                fod = d > 0.0f ? dv / d : 0.0f;
            }
        }
        else if (r2 >= 0.01f)
        {
            const float inv2 = recip_nr(r2);
            const float i6 = inv2 * inv2 * inv2;
            const float t6 = p.probe_P * pi.w * i6;
            if (SM == BS_STERIC_LJ_12_6_AMBER)
            {
                const float t12 = p.probe_F * fhi_i * i6 * i6;
                es = fmaf(p.steric_scale, t12 - 2.0f * t6, es);
                fod = 12.0f * (t6 - t12) * inv2;
            }
            else if (SM == BS_STERIC_LJ_8_6_LEWITT)
            {
                const float t8 = p.probe_F * fhi_i * i6 * inv2;
                es = fmaf(p.steric_scale, 3.0f * t8 - 4.0f * t6, es);
                fod = 24.0f * (t6 - t8) * inv2;
            }
            else
            {
                const float t8 = p.probe_F * fhi_i * i6 * inv2;
                es = fmaf(p.steric_scale, t8 - t6, es);
                fod = (6.0f * t6 - 8.0f * t8) * inv2;
            }
        }
        const float k = fod * p.k_spring_f * p.steric_scale;
        fx = fmaf(dx, k, fx);
        fy = fmaf(dy, k, fy);
        fz = fmaf(dz, k, fz);
    }
    if (p.probe_elec && r2 >= 1e-6f) // d < 0.001 A gives zero (electrostatic.hpp:18-19)
    {
        const float inv = rsqrt_nr(r2);
        float tq = p.probe_q * qi * inv;
        float fod;
        if (p.dielectric_mode == BS_DIELECTRIC_DISTANCE)
        {
            tq *= inv;
            fod = -2.0f * tq * inv * inv;
        }
        else
            fod = -tq * inv * inv;
        ec = fmaf(tq, p.k_elec_e, ec);
        const float k = fod * p.k_elec_f;
        fx = fmaf(dx, k, fx);
        fy = fmaf(dy, k, fy);
        fz = fmaf(dz, k, fz);
    }
}

// Cell of field grid g holding the particle at pi, or -1 when the particle is outside the grid's
// box (GridCoordinatesSystem::is_out_of_grid, GridCoordinatesSystem.hpp:206-218). The index along
// an axis is trunc((x - origin) / cell size) evaluated in double (GridCoordinatesSystem.hpp:85-94);
// the float estimate decides unless it lies within its error bound of an integer, where the
// double expression is evaluated.
__device__ __forceinline__ int field_cell(const Params &p, int g, const float4 &pi)
{
    const float x[3] = {pi.x, pi.y, pi.z};
    int idx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        if (!(x[a] >= p.fg_lo[g][a] && x[a] <= p.fg_hi[g][a]))
            return -1;
        const float t = (x[a] - p.fg_of[g][a]) * p.fg_ih[g][a];
        int c;
        if (fabsf(t - rintf(t)) < 1e-3f + 4e-7f * fabsf(t))
            c = static_cast<int>(__ddiv_rn(__dsub_rn(static_cast<double>(x[a]), p.fg_o[g][a]), p.fg_h[g][a]));
        else
            c = static_cast<int>(t);
        idx[a] = min(max(c, 0), p.fg_n[g][a] - 1);
    }
    return (idx[0] * p.fg_n[g][1] + idx[1]) * p.fg_n[g][2] + idx[2];
}

// Field-grid forces of one dynamic particle (SpringNetwork.cpp:110-118): the potential map's
// force q v s and energy s * field_energy(scalar, q) (Particle.cpp:161-189,
// electrostatic_field.hpp:16-23), and the density map's force b v s' (Particle.cpp:136-159),
// with the reference's float products and double unit steps.
__device__ __forceinline__ void field_forces(const Params &p, const float4 &pi, float q, float bur, float &fx,
                                             float &fy, float &fz, float &e_elec)
{
    if (p.fg_on[0])
    {
        const int c = field_cell(p, 0, pi);
        if (c >= 0)
        {
            const float4 v = p.fgrid[0][c];
            const float gs = p.fg_scale[0];
            fx += __fmul_rn(__fmul_rn(v.y, q), gs);
            fy += __fmul_rn(__fmul_rn(v.z, q), gs);
            fz += __fmul_rn(__fmul_rn(v.w, q), gs);
            float en = __fmul_rn(v.x, q);
            en = __double2float_rn(__dmul_rn(static_cast<double>(en), 1.3806504E-23));
            en = __double2float_rn(__dmul_rn(static_cast<double>(en), 1.0E-3));
            en = __double2float_rn(__dmul_rn(static_cast<double>(en), 6.02214169E23));
            e_elec += __fmul_rn(gs, en);
        }
    }
    if (p.fg_on[1])
    {
        const int c = field_cell(p, 1, pi);
        if (c >= 0)
        {
            const float4 v = p.fgrid[1][c];
            const float gs = p.fg_scale[1];
            fx += __fmul_rn(__fmul_rn(v.y, bur), gs);
            fy += __fmul_rn(__fmul_rn(v.z, bur), gs);
            fz += __fmul_rn(__fmul_rn(v.w, bur), gs);
        }
    }
}

// IMPALA for the double membrane with tube curvatures (imp.hpp:29-159, ForceField.cpp:62-85):
// each membrane m, at signed offset o (upper +, lower -) with tube radius R = 1 / |curvature|
// (1e6 A when flat) around an axis along y at z = o - sign R, sees the particle at depth d: its
// z when flat, else its distance from the axis folded to the membrane's frame. The membrane adds
// (-S T + A_lip S) C(|d - o|) to the energy and the opposite of that term's derivative along the
// direction from the axis (z when flat) to the force.
__device__ __forceinline__ void imp_double_membrane(const Params &p, const float4 &pi, float S, float T, float &fx,
                                                    float &fz, float &e)
{
    const float gg = -S * T + kAlip * S;
#pragma unroll
    for (int m = 0; m < 2; ++m)
    {
        const float off = p.imp_off[m], c = p.imp_curv[m];
        const float R = c == 0.0f ? 1000000.0f : fabsf(1.0f / c);
        const float sg = c > 0.0f ? 1.0f : (c < 0.0f ? -1.0f : 0.0f);
        const float axis = off - sg * R;
        const float rx = pi.x, rz = pi.z - axis;
        const float rn = sqrtf(rx * rx + rz * rz);
        const float depth = sg == 0.0f ? pi.z : (pi.z > axis ? sg * rn : -sg * rn) + off - R;
        const float u = depth - off;
        const float ex = expf(p.imp_alpha * (fabsf(u) - p.imp_z0));
        e = fmaf(p.imp_scale * gg, 0.5f - 1.0f / (1.0f + ex), e);
        // dC/du = alpha sign(u) e / (1 + e)^2, written without overflow
        float dcz = u != 0.0f ? p.imp_alpha / (ex + 2.0f + 1.0f / ex) : 0.0f;
        if (u < 0.0f)
            dcz = -dcz;
        if (!isfinite(dcz))
            dcz = 0.0f;
        float dx = 0.0f, dz = 1.0f;
        if (sg != 0.0f)
        {
            dx = rn > 1e-40f ? rx / rn : 0.0f;
            dz = rn > 1e-40f ? rz / rn : 0.0f;
        }
        const float f = p.imp_scale * (gg * dcz * p.k_imp_f);
        fx -= f * dx;
        fz -= f * dz;
    }
}

// Sum over the T consecutive lanes of a particle group (result in every lane of the group).
template <int T> __device__ __forceinline__ float group_sum(float v)
{
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One particle of one step (or of one force evaluation), lane t of the T consecutive lanes that
// share slot s: each lane takes every T-th entry of the particle's spring row and pair lists, the
// group sums its partial forces with shuffles, and the group's first lane adds the per-particle
// terms and integrates (reading buffer sb, writing sb ^ 1). Slots at or beyond `send` are
// inactive. Every lane of the warp must call it (shuffles). Adds the particle's energies to
// eacc (spring, steric, Coulomb, hydrophobic, IMPALA, kinetic) and returns the status bits it
// raised (ST_NONFINITE, ST_STALE). SINGLE selects the single-system form: field-grid forces and
// Coulomb rows walked by the whole warp. The batched kernel leaves both out (fewer live registers
// under its 64-register budget: with them its spills grew and its step slowed by 7%); it walks
// Coulomb rows with the particle's own lanes (the same pairs, summed in another order).
template <int MODE, int SM, int T, bool SINGLE = true, bool LEAN = false>
__device__ __forceinline__ int particle_step(const Params &p, const int s, const int t, const int send,
                                             const int sb, const int lb, const bool ext_on, float (&eacc)[6])
{
    const float4 *__restrict__ pos = p.pos[sb];
    const bool lead = t == 0;
    int pend = 0;

    // energies: spring, steric, coulomb, hydrophobic, imp, kinetic
    float e[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float fx = 0.f, fy = 0.f, fz = 0.f;
    unsigned int fi = PF_STATIC;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    // BS_HOIST: the lean single-system step reads the steric row's count and the lane's first
    // entries with the particle itself, so the row's first partner loads wait for one round trip
    // fewer (the entries lie inside the row's capacity whatever the count)
    constexpr bool kHoist = BS_HOIST && LEAN && SINGLE;
    int cnt0 = -1;
    uint2 w0 = make_uint2(0u, 0u);
    float fhi_i = 0.0f;
    if (s < send)
    {
        pi = pos[s];
        fi = p.flags[lb][s];
        fhi_i = p.fhi[lb][s];
        if (kHoist && p.steric_on && p.lj_uniform && p.pl16)
        {
            const PairList &L = p.pl[0];
            cnt0 = L.cnt[s];
            if (kGatherU * t < L.cap)
                w0 = __ldg(reinterpret_cast<const uint2 *>(reinterpret_cast<const short *>(L.idx) +
                                                         static_cast<size_t>(s) * L.cap + kGatherU * t));
        }
    }
    const bool active = s < send && !(fi & PF_STATIC);
    if (active)
    {
        if (p.steric_on)
        {
            float sx = 0.f, sy = 0.f, sz = 0.f, es = 0.f;
            if (LEAN && p.lj_uniform && p.pl16)
                steric_forces_batched<SM, T, true, true>(p, s, t, pi, fhi_i, pos, p.fhi[lb], sx, sy, sz, es, cnt0, w0);
            else if ((SINGLE && BS_GATHER) || (!SINGLE && BS_GATHER_BATCH))
            {
                if (p.pl16)
                    steric_forces_batched<SM, T, true>(p, s, t, pi, fhi_i, pos, p.fhi[lb], sx, sy, sz, es);
                else
                    steric_forces_batched<SM, T, false>(p, s, t, pi, fhi_i, pos, p.fhi[lb], sx, sy, sz, es);
            }
            else if (p.pl16)
                steric_forces<SM, T, 0>(p, s, t, pi, fhi_i, pos, p.fhi[lb], sx, sy, sz, es);
            else
                steric_forces<SM, T, 1>(p, s, t, pi, fhi_i, pos, p.fhi[lb], sx, sy, sz, es);
            // the static-partner list exists only when some particle is static
            if (p.pl[kListStericStatic].on && p.pl[kListStericStatic].cnt[s] > 0)
                steric_forces<SM, T, 2>(p, s, t, pi, fhi_i, pos, p.fhi[lb], sx, sy, sz, es);
            const float kf = p.k_spring_f * p.steric_scale;
            fx = fmaf(sx, kf, fx);
            fy = fmaf(sy, kf, fy);
            fz = fmaf(sz, kf, fz);
            e[1] = es * p.steric_scale;
        }
        // springs after the steric pairs: no spring sums are live across the steric loop
        if (p.spring_on)
        {
            float sx = 0.f, sy = 0.f, sz = 0.f, es = 0.f;
            if ((SINGLE && BS_GATHER) || (!SINGLE && BS_GATHER_BATCH))
                spring_forces_batched<T>(p, s, t, pi, pos, sx, sy, sz, es);
            else
                spring_forces<T>(p, s, t, pi, pos, sx, sy, sz, es);
            const float kf = p.k_spring_f * p.spring_scale;
            fx = fmaf(sx, kf, fx);
            fy = fmaf(sy, kf, fy);
            fz = fmaf(sz, kf, fz);
            e[0] = es * p.spring_scale;
        }
        if ((!SINGLE || !BS_COUL_WARP) && p.coulomb_on && (fi & PF_CHARGED))
        {
            float sx = 0.f, sy = 0.f, sz = 0.f, es = 0.f;
            coulomb_forces<T>(p, s, t, pi, p.chg[lb][s], pos, p.chg[lb], sx, sy, sz, es);
            fx = fmaf(sx, p.k_elec_f, fx);
            fy = fmaf(sy, p.k_elec_f, fy);
            fz = fmaf(sz, p.k_elec_f, fz);
            e[2] = es * p.k_elec_e;
        }
        if (!LEAN && p.hydro_on && (fi & PF_HYDROPHOBIC))
        {
            float sx = 0.f, sy = 0.f, sz = 0.f, es = 0.f;
            hydro_forces<T>(p, s, t, pi, p.hyd[lb][s], pos, p.hyd[lb], sx, sy, sz, es);
            const float kf = p.k_spring_f * p.hydro_scale;
            fx = fmaf(sx, kf, fx);
            fy = fmaf(sy, kf, fy);
            fz = fmaf(sz, kf, fz);
            e[3] = es * p.k_hydro_e * p.hydro_scale;
        }
    }
    if (T > 1)
    {
        // every lane of the warp takes part in the group reductions
        fx = group_sum<T>(fx);
        fy = group_sum<T>(fy);
        fz = group_sum<T>(fz);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            e[k] = group_sum<T>(e[k]);
        if (!lead)
        {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                e[k] = 0.f;
        }
    }
    // Coulomb pairs, a warp at a time: few particles are charged, so instead of a particle's own
    // T lanes, all 32 lanes of the warp walk the row of each charged particle of the warp in turn
    // (coalesced entries, one or two per lane), and the lead lane of that particle takes the sum.
    if (SINGLE && BS_COUL_WARP && p.coulomb_on)
    {
        const int lane = static_cast<int>(threadIdx.x & 31);
        unsigned todo = __ballot_sync(0xffffffffu, lead && active && (fi & PF_CHARGED));
        while (todo)
        {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const int sc = __shfl_sync(0xffffffffu, s, src);
            const float4 pc = make_float4(__shfl_sync(0xffffffffu, pi.x, src), __shfl_sync(0xffffffffu, pi.y, src),
                                          __shfl_sync(0xffffffffu, pi.z, src), __shfl_sync(0xffffffffu, pi.w, src));
            float cx = 0.f, cy = 0.f, cz = 0.f, ce = 0.f;
            coulomb_forces<32>(p, sc, lane, pc, p.chg[lb][sc], pos, p.chg[lb], cx, cy, cz, ce);
            cx = group_sum<32>(cx);
            cy = group_sum<32>(cy);
            cz = group_sum<32>(cz);
            ce = group_sum<32>(ce);
            if (lane == src)
            {
                fx = fmaf(cx, p.k_elec_f, fx);
                fy = fmaf(cy, p.k_elec_f, fy);
                fz = fmaf(cz, p.k_elec_f, fz);
                e[2] = ce * p.k_elec_e;
            }
        }
    }
    if (lead && s < send)
    {
        if (!active)
        {
            if (MODE == MODE_STEP)
            {
                p.pos[sb ^ 1][s] = pi;
                p.vel[sb ^ 1][s] = p.vel[sb][s];
                if (!LEAN && p.pos_lo[0])
                    p.pos_lo[sb ^ 1][s] = p.pos_lo[sb][s];
            }
            else
                p.force_out[p.perm[lb][s]] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (!LEAN && p.probe_on)
                p.probe_f[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        else
        {
            const float4 v = p.vel[sb][s];
            // ---- field grids (SpringNetwork.cpp:110-118) ----
            if (SINGLE && !LEAN && (p.fg_on[0] || p.fg_on[1]))
                field_forces(p, pi, p.chg[lb][s], p.fg_on[1] ? p.bur[lb][s] : 0.0f, fx, fy, fz, e[2]);
            // ---- viscosity (Particle.cpp:80-84) ----
            if (p.visc_on)
            {
                fx -= v.x * p.visc;
                fy -= v.y * p.visc;
                fz -= v.z * p.visc;
            }
            const float4 ip = p.iprm[lb][s];
            // ---- IMPALA, flat membrane (imp.hpp:29-159, ForceField.cpp:62-88) ----
            if (p.imp_on && p.imp_double)
                imp_double_membrane(p, pi, ip.y, ip.z, fx, fz, e[4]);
            else if (p.imp_on)
            {
                const float ex = expf(p.imp_alpha * (fabsf(pi.z) - p.imp_z0));
                const float cz = 0.5f - 1.0f / (1.0f + ex);
                const float gg = -ip.y * ip.z + kAlip * ip.y;
                e[4] = p.imp_scale * gg * cz;
                // dC/dz = alpha sign(z) e / (1 + e)^2, written without overflow
                float dcz = pi.z != 0.0f ? p.imp_alpha / (ex + 2.0f + 1.0f / ex) : 0.0f;
                if (pi.z < 0.0f)
                    dcz = -dcz;
                if (!isfinite(dcz))
                    dcz = 0.0f;
                fz -= p.imp_scale * (gg * dcz * p.k_imp_f);
            }
            // ---- external force (SpringNetwork::setForce, SpringNetwork.cpp:438-442) ----
            if (ext_on)
            {
                float *xf = p.ext + 3 * static_cast<size_t>(p.perm[lb][s]);
                const float ex = xf[0], ey = xf[1], ez = xf[2];
                fx += ex;
                fy += ey;
                fz += ez;
                if (MODE == MODE_STEP && (ex != 0.f || ey != 0.f || ez != 0.f))
                {
                    xf[0] = 0.f;
                    xf[1] = 0.f;
                    xf[2] = 0.f;
                }
            }
            // ---- probe (SpringNetwork.cpp:156-182), after every other term ----
            if (!LEAN && p.probe_on)
            {
                const float4 prb = p.ctl->probe_pos;
                float px = 0.f, py = 0.f, pz = 0.f;
                probe_pair<SM>(p, prb, pi, p.fhi[lb][s], p.chg[lb][s], px, py, pz, e[1], e[2]);
                fx += px;
                fy += py;
                fz += pz;
                p.probe_f[s] = make_float4(-px, -py, -pz, 0.f);
            }
            if (MODE == MODE_FORCES)
            {
                p.force_out[p.perm[lb][s]] = make_float4(fx, fy, fz, 0.f);
            }
            else if (!LEAN && (fi & PF_RIGID))
            {
                // a rigid particle's force goes to its body (RigidBody.cpp:567-580); the body
                // kernel moves the particle, and its kinetic energy counts as zero
                p.rforce[s] = make_float4(fx, fy, fz, 0.f);
            }
            else
            {
                // ---- semi-implicit Euler (Particle.cpp:109-128), no fused multiply-adds ----
                const float m = ip.x;
                float vx = v.x, vy = v.y, vz = v.z;
                if (m > 0.0f)
                {
                    vx = __fadd_rn(vx, __fmul_rn(__fdiv_rn(fx, m), p.dt));
                    vy = __fadd_rn(vy, __fmul_rn(__fdiv_rn(fy, m), p.dt));
                    vz = __fadd_rn(vz, __fmul_rn(__fdiv_rn(fz, m), p.dt));
                }
                const float v2 = vx * vx + vy * vy + vz * vz;
                e[5] = 0.5f * m * v2 * p.k_kin;
                float nx, ny, nz;
                if (!LEAN && p.pos_lo[0])
                {
                    // x += v dt in float-float: the increment's rounding error and the carried
                    // remainder are kept, so increments below half an ulp of x are not lost
                    const float4 lo = p.pos_lo[sb][s];
                    float ex, ey, ez;
                    two_sum(pi.x, __fmul_rn(vx, p.dt), nx, ex);
                    two_sum(pi.y, __fmul_rn(vy, p.dt), ny, ey);
                    two_sum(pi.z, __fmul_rn(vz, p.dt), nz, ez);
                    two_sum(nx, __fadd_rn(ex, lo.x), nx, ex);
                    two_sum(ny, __fadd_rn(ey, lo.y), ny, ey);
                    two_sum(nz, __fadd_rn(ez, lo.z), nz, ez);
                    p.pos_lo[sb ^ 1][s] = make_float4(ex, ey, ez, 0.f);
                }
                else
                {
                    nx = __fadd_rn(pi.x, __fmul_rn(vx, p.dt));
                    ny = __fadd_rn(pi.y, __fmul_rn(vy, p.dt));
                    nz = __fadd_rn(pi.z, __fmul_rn(vz, p.dt));
                }
                p.pos[sb ^ 1][s] = make_float4(nx, ny, nz, pi.w);
                p.vel[sb ^ 1][s] = make_float4(vx, vy, vz, 0.f);
                if (!isfinite(nx) || !isfinite(ny) || !isfinite(nz))
                    pend |= ST_NONFINITE;
                const float4 b = p.pos_build[s];
                const float ddx = nx - b.x, ddy = ny - b.y, ddz = nz - b.z;
                if (ddx * ddx + ddy * ddy + ddz * ddz > p.half_skin2)
                    pend |= ST_STALE;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k)
        eacc[k] += e[k];
    return pend;
}

} // namespace
} // namespace bsg
