// bs_kernels.cu -- sm_103a kernels of BioSpring's per-step force-and-integrate loop.
//
// Data layout (all in HBM, structure of arrays, particles in cell-sorted order):
//   pos[2]   float4 (x, y, z, charge)       double-buffered: a step reads one, writes the other
//   vel[2]   float4 (vx, vy, vz, 0)
//   jprm[2]  float4 (steric a, steric b, hydrophobicity, flag bits)  re-laid out at each rebuild
//   perm[2]  sorted slot -> caller id;  inv: caller id -> sorted slot
//   se_*     springs of each slot, ELL column-major [k * npad + slot] (coalesced per warp)
//   pl       nonbonded pair list, ELL column-major [k * npad + slot], rebuilt every K steps
//
// Rebuild (every K steps, or when a particle drifted more than skin/2):
//   k_bbox -> k_cell_count -> k_cell_scan -> k_cell_place -> k_cell_sort -> k_reorder
//   -> k_spring_ell -> k_pairlist
// Step: k_step, one thread per particle, gathers its springs and nonbonded pairs (no atomics
// on forces, so results are deterministic) and integrates in the same pass.
//
// Reference behaviour reproduced (paths inside the BioSpring project):
//   cell grid and cell id           src/nsearch.hpp:277-293, 342-390 (FP64, same formula)
//   pair filters                    src/nsearch.hpp:230 (FP64 distance) and src/spn/Particle.cpp:
//                                   213-224 (spring exclusion, float distance < cutoff, != 0),
//                                   :209 (static neighbour: full energy, no force on it)
//   force expressions               src/forcefield/energy/{spring,steric,electrostatic,hydrophobic,imp}.hpp
//   viscosity and Euler step        src/spn/Particle.cpp:80-84, 109-128
//   non-finite position check       src/spn/SpringNetwork.cpp:222-229 (status bit, no abort)

#include <cfloat>
#include <climits>

#include "bs_kernels.cuh"

namespace bsg
{

namespace
{

constexpr uint32_t kColMask = 0x3fffffffu;
constexpr uint32_t kColStatic = 0x80000000u;   // partner is static: the pair's full energy is ours
constexpr uint32_t kColInactive = 0x40000000u; // spring between two rigid particles: excluded, no force

__device__ __forceinline__ int status_of(const Ctl *c) { return *(volatile const int *)&c->status; }

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

// Reference cell coordinate along one axis: (size_t)((x - min) / radius), clamped (nsearch.hpp:282-289).
__device__ __forceinline__ int ref_cell_coord(float x, double mn, float radius, int ncell)
{
    const double t = __ddiv_rn(__dsub_rn(static_cast<double>(x), mn), static_cast<double>(radius));
    unsigned long long c = static_cast<unsigned long long>(t);
    const unsigned long long lim = static_cast<unsigned long long>(ncell - 1);
    return static_cast<int>(c < lim ? c : lim);
}

// Exact reference test of one candidate pair for one cutoff: the grid filter compares the FP64
// distance of the float coordinates (nsearch.hpp:230, measure.hpp:163-169); the force routine
// then compares the float-rounded FP64 norm of the float difference vector (Particle.cpp:222-224,
// Vector3f.cpp:9-12, measure.hpp:188-196). Only pairs inside the guard band come here.
__device__ __noinline__ bool exact_pair_test(float4 pi, float4 pj, float cutoff, bool nonzero, float *dist)
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
    *dist = d;
    return true;
}

// Classifies a pair for one term. Outside the band [lo2, hi2) the FP32 squared distance decides
// (its error is far below the band); inside it, and for (near-)coincident particles, the exact
// reference test decides. Returns true if the pair interacts and sets d.
__device__ __forceinline__ bool pair_in(float r2, float lo2, float hi2, float4 pi, float4 pj, float cutoff, bool nonzero,
                                        float *d)
{
    if (r2 >= hi2)
        return false;
    if (r2 < lo2 && r2 > 1e-20f)
    {
        *d = sqrtf(r2);
        return true;
    }
    return exact_pair_test(pi, pj, cutoff, nonzero, d);
}

// Steric force module and pair energy (energy/steric.hpp:27-156, scale applied by the caller).
// a, b are the per-particle factors: Amber/Lewitt sqrt(eps), sqrt(radius); Zacharias eps, radius;
// linear: b = radius.
template <int SM>
__device__ __forceinline__ void steric_pair(float d, float inv_d, float ai, float bi, float aj, float bj, float kf,
                                            float &fm, float &e)
{
    if (SM == BS_STERIC_LINEAR)
    {
        const float dv = d - (bi + bj);
        if (dv > 0.0f)
        {
            fm = 0.0f;
            e = 0.0f;
        }
        else
        {
            e = 0.5f * dv * dv;
            fm = -fabsf(dv) * kf;
        }
    }
    else
    {
        if (d < 0.1f)
        {
            fm = 0.0f;
            e = 0.0f;
            return;
        }
        const float eij = ai * aj;
        const float sr = (bi * bj) * inv_d;
        const float s2 = sr * sr;
        const float s6 = s2 * s2 * s2;
        if (SM == BS_STERIC_LJ_12_6_AMBER)
        {
            const float s12 = s6 * s6;
            e = eij * (s12 - 2.0f * s6);
            fm = 12.0f * eij * inv_d * (s6 - s12) * kf;
        }
        else if (SM == BS_STERIC_LJ_8_6_LEWITT)
        {
            const float s8 = s6 * s2;
            e = eij * (3.0f * s8 - 4.0f * s6);
            fm = 24.0f * eij * inv_d * (s6 - s8) * kf;
        }
        else
        {
            const float s8 = s6 * s2;
            e = eij * (s8 - s6);
            fm = eij * inv_d * (6.0f * s6 - 8.0f * s8) * kf;
        }
    }
}

// Coulomb force module and energy (energy/electrostatic.hpp:16-49); with the distance-dependent
// dielectric eps = D r the energy is K q q / (D r^2) and the module is -dE/dr.
__device__ __forceinline__ void coulomb_pair(const Params &p, float d, float inv_d, float qq, float &fm, float &e)
{
    if (d < 0.001f)
    {
        fm = 0.0f;
        e = 0.0f;
        return;
    }
    const float invD = 1.0f / p.dielectric;
    if (p.dielectric_mode == BS_DIELECTRIC_DISTANCE)
    {
        const float t = qq * inv_d * inv_d * invD;
        e = p.k_elec_e * t;
        fm = -2.0f * p.k_elec_f * t * inv_d;
    }
    else
    {
        const float t = qq * inv_d * invD;
        e = p.k_elec_e * t;
        fm = -p.k_elec_f * t * inv_d;
    }
    e *= p.coulomb_scale;
    fm *= p.coulomb_scale;
}

// Block-wide FP64 reduction of NE per-thread float partials into the block's slot of
// blk_energy; the last block to finish sums every block's partials in block order.
template <int NE, int BLOCK>
__device__ __forceinline__ bool reduce_energies(const float (&e)[NE], double *blk, Ctl *ctl, unsigned int *done,
                                                double *dst, bool accumulate_first)
{
    __shared__ double sh[NE][BLOCK / 32];
    __shared__ bool am_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NE; ++k)
    {
        double v = static_cast<double>(e[k]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0)
            sh[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < NE)
    {
        double v = 0.0;
        for (int w = 0; w < BLOCK / 32; ++w)
            v += sh[threadIdx.x][w];
        blk[static_cast<size_t>(blockIdx.x) * 8 + threadIdx.x] = v;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0)
        am_last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!am_last)
        return false;
    __threadfence();
    // Last block: fixed-order sum over blocks.
    for (int k = 0; k < NE; ++k)
    {
        double v = 0.0;
        for (unsigned int b = threadIdx.x; b < gridDim.x; b += BLOCK)
            v += __ldcg(&blk[static_cast<size_t>(b) * 8 + k]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
        __syncthreads();
        if (lane == 0)
            sh[0][warp] = v;
        __syncthreads();
        if (threadIdx.x == 0)
        {
            double t = 0.0;
            for (int w = 0; w < BLOCK / 32; ++w)
                t += sh[0][w];
            if (accumulate_first && k == 0)
                dst[k] += t;
            else
                dst[k] = t;
        }
    }
    if (threadIdx.x == 0)
        *done = 0u;
    return true;
}

// ------------------------------------------------------------------------------------------
// Rebuild kernels
// ------------------------------------------------------------------------------------------

__global__ void __launch_bounds__(kBboxBlock) k_bbox(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const float4 *pos = p.pos[ctl->sbuf];
    float mn0 = FLT_MAX, mn1 = FLT_MAX, mn2 = FLT_MAX, mx0 = -FLT_MAX, mx1 = -FLT_MAX, mx2 = -FLT_MAX;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += gridDim.x * blockDim.x)
    {
        const float4 q = pos[i];
        mn0 = fminf(mn0, q.x);
        mn1 = fminf(mn1, q.y);
        mn2 = fminf(mn2, q.z);
        mx0 = fmaxf(mx0, q.x);
        mx1 = fmaxf(mx1, q.y);
        mx2 = fmaxf(mx2, q.z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        mn0 = fminf(mn0, __shfl_down_sync(0xffffffffu, mn0, o));
        mn1 = fminf(mn1, __shfl_down_sync(0xffffffffu, mn1, o));
        mn2 = fminf(mn2, __shfl_down_sync(0xffffffffu, mn2, o));
        mx0 = fmaxf(mx0, __shfl_down_sync(0xffffffffu, mx0, o));
        mx1 = fmaxf(mx1, __shfl_down_sync(0xffffffffu, mx1, o));
        mx2 = fmaxf(mx2, __shfl_down_sync(0xffffffffu, mx2, o));
    }
    unsigned int *enc = ctl->bbox_enc;
    if ((threadIdx.x & 31) == 0)
    {
        atomicMin(&enc[0], f2ord(mn0));
        atomicMin(&enc[1], f2ord(mn1));
        atomicMin(&enc[2], f2ord(mn2));
        atomicMax(&enc[3], f2ord(mx0));
        atomicMax(&enc[4], f2ord(mx1));
        atomicMax(&enc[5], f2ord(mx2));
    }
    __threadfence();
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0)
        last = atomicAdd(&ctl->done_bbox, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last || threadIdx.x != 0)
        return;
    __threadfence();
    float mn[3], mx[3];
    for (int k = 0; k < 3; ++k)
    {
        mn[k] = ord2f(atomicAdd(&enc[k], 0u));
        mx[k] = ord2f(atomicAdd(&enc[3 + k], 0u));
        enc[k] = 0xffffffffu; // reset for the next rebuild
        enc[3 + k] = 0u;
    }
    // Grid dimensions, reference formula ncells = ceil(len / radius) + 1 (nsearch.hpp:351-354).
    const double r = static_cast<double>(p.list_radius);
    double cells = 1.0;
    int nc[3];
    for (int k = 0; k < 3; ++k)
    {
        const double len = __dsub_rn(static_cast<double>(mx[k]), static_cast<double>(mn[k]));
        const double c = ceil(__ddiv_rn(len, r)) + 1.0;
        cells *= c;
        nc[k] = c < 1.0e9 ? static_cast<int>(c) : 1000000000;
        ctl->gmin[k] = static_cast<double>(mn[k]);
    }
    ctl->gradius = p.list_radius;
    ctl->gnx = nc[0];
    ctl->gny = nc[1];
    ctl->gnz = nc[2];
    if (!(cells <= static_cast<double>(p.cell_cap)))
    {
        ctl->ncells_needed = cells < 2.0e9 ? static_cast<int>(cells) : INT_MAX;
        atomicOr(&ctl->status, ST_CELL_CAPACITY);
    }
    atomicAnd(&ctl->status, ~ST_STALE);
    ctl->done_bbox = 0u;
}

__global__ void __launch_bounds__(kBuildBlock) k_cell_count(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n)
        return;
    const float4 q = p.pos[ctl->sbuf][i];
    const float r = ctl->gradius;
    const int nx = ctl->gnx, ny = ctl->gny, nz = ctl->gnz;
    const int cx = ref_cell_coord(q.x, ctl->gmin[0], r, nx);
    const int cy = ref_cell_coord(q.y, ctl->gmin[1], r, ny);
    const int cz = ref_cell_coord(q.z, ctl->gmin[2], r, nz);
    const int c = cx + cy * nx + cz * nx * ny;
    p.cell_of[i] = c;
    atomicAdd(&p.cell_cnt[c], 1);
}

// Single-block exclusive scan of the cell counts; also primes the fill cursors and
// clears the counts for the next rebuild.
__global__ void __launch_bounds__(1024) k_cell_scan(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int nc = ctl->gnx * ctl->gny * ctl->gnz;
    const int per = (nc + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per, b1 = min(nc, b0 + per);
    int sum = 0;
    for (int c = b0; c < b1; ++c)
        sum += p.cell_cnt[c];
    __shared__ int sh[1024];
    sh[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1)
    {
        const int v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += v;
        __syncthreads();
    }
    int run = sh[threadIdx.x] - sum;
    for (int c = b0; c < b1; ++c)
    {
        const int k = p.cell_cnt[c];
        p.cell_start[c] = run;
        p.cell_fill[c] = run;
        p.cell_cnt[c] = 0;
        run += k;
    }
    if (threadIdx.x == blockDim.x - 1)
        p.cell_start[nc] = run;
}

__global__ void __launch_bounds__(kBuildBlock) k_cell_place(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n)
        return;
    const int slot = atomicAdd(&p.cell_fill[p.cell_of[i]], 1);
    p.tmp_perm[slot] = p.perm[ctl->lbuf][i];
}

// One warp per cell: orders the cell's particles by caller id (the reference appends them to
// a cell in index order, nsearch.hpp:376-389), which makes the layout deterministic.
__global__ void __launch_bounds__(kBuildBlock) k_cell_sort(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int nc = ctl->gnx * ctl->gny * ctl->gnz;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    int *out = p.perm[ctl->lbuf ^ 1];
    for (int c = warp; c < nc; c += nwarps)
    {
        const int s0 = p.cell_start[c], s1 = p.cell_start[c + 1];
        const int len = s1 - s0;
        for (int e = lane; e < len; e += 32)
        {
            const int id = p.tmp_perm[s0 + e];
            int rank = 0;
            for (int f = 0; f < len; ++f)
                rank += p.tmp_perm[s0 + f] < id;
            out[s0 + rank] = id;
            p.cell_of[s0 + rank] = c;
        }
    }
}

// Moves the state into the new layout, records build positions and the new inverse permutation,
// then (last block) makes the new layout current.
__global__ void __launch_bounds__(kBuildBlock) k_reorder(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int sb = ctl->sbuf, lb = ctl->lbuf;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < p.n)
    {
        const int id = p.perm[lb ^ 1][i];
        const int old = p.inv[id];
        const float4 q = p.pos[sb][old];
        p.pos[sb ^ 1][i] = q;
        p.vel[sb ^ 1][i] = p.vel[sb][old];
        p.jprm[lb ^ 1][i] = p.jprm[lb][old];
        p.iprm[lb ^ 1][i] = p.iprm[lb][old];
        p.pos_build[i] = q;
        p.inv[id] = i;
    }
    __threadfence();
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0)
        last = atomicAdd(&ctl->done_reorder, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last && threadIdx.x == 0)
    {
        ctl->sbuf = sb ^ 1;
        ctl->lbuf = lb ^ 1;
        ctl->done_reorder = 0u;
    }
}

// Springs of every slot in the new layout, partners as slots (ELL, column-major).
__global__ void __launch_bounds__(kBuildBlock) k_spring_ell(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.npad)
        return;
    if (s >= p.n)
    {
        p.se_deg[s] = 0;
        return;
    }
    const int id = p.perm[ctl->lbuf][s];
    const int r0 = p.sp_row[id], r1 = p.sp_row[id + 1];
    for (int e = r0; e < r1; ++e)
    {
        const uint32_t c = static_cast<uint32_t>(p.sp_col[e]);
        const uint32_t slot = static_cast<uint32_t>(p.inv[c & kColMask]);
        const size_t at = static_cast<size_t>(e - r0) * p.npad + s;
        p.se_col[at] = static_cast<int>(slot | (c & ~kColMask));
        p.se_k[at] = p.sp_k[e];
        p.se_r0[at] = p.sp_r0[e];
    }
    p.se_deg[s] = r1 - r0;
}

// Pair list of every dynamic slot: all slots within the list radius (cutoff + skin) found in
// the 27 neighbouring cells, minus the slot itself and, when springs are enabled, its spring
// partners (Particle.cpp:213-218). Entries come out in increasing slot order.
__global__ void __launch_bounds__(kBuildBlock) k_pairlist(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.npad)
        return;
    if (s >= p.n)
    {
        p.pl_cnt[s] = 0;
        return;
    }
    const int sb = ctl->sbuf, lb = ctl->lbuf;
    const float4 *pos = p.pos[sb];
    const float4 *jp = p.jprm[lb];
    const uint32_t fi = __float_as_uint(jp[s].w);
    if (fi & PF_STATIC)
    {
        p.pl_cnt[s] = 0;
        return;
    }
    const float4 pi = pos[s];
    const int nx = ctl->gnx, ny = ctl->gny, nz = ctl->gnz;
    const int c = p.cell_of[s];
    const int cx = c % nx, cy = (c / nx) % ny, cz = c / (nx * ny);
    const int deg = p.se_deg[s];
    int cnt = 0;
    const bool need_flags = !p.steric_on;
    for (int dz = -1; dz <= 1; ++dz)
    {
        const int z = cz + dz;
        if (z < 0 || z >= nz)
            continue;
        for (int dy = -1; dy <= 1; ++dy)
        {
            const int y = cy + dy;
            if (y < 0 || y >= ny)
                continue;
            const int xa = max(cx - 1, 0), xb = min(cx + 1, nx - 1);
            const int base = (z * ny + y) * nx;
            const int j0 = p.cell_start[base + xa], j1 = p.cell_start[base + xb + 1];
            for (int j = j0; j < j1; ++j)
            {
                if (j == s)
                    continue;
                const float4 pj = pos[j];
                const float dx = pj.x - pi.x, dy2 = pj.y - pi.y, dz2 = pj.z - pi.z;
                const float r2 = dx * dx + dy2 * dy2 + dz2 * dz2;
                if (!(r2 < p.list_r2))
                    continue;
                if (need_flags)
                {
                    const uint32_t fj = __float_as_uint(jp[j].w);
                    const bool cc = p.coulomb_on && (fi & PF_CHARGED) && (fj & PF_CHARGED);
                    const bool hh = p.hydro_on && (fi & PF_HYDROPHOBIC) && (fj & PF_HYDROPHOBIC);
                    if (!cc && !hh)
                        continue;
                }
                if (p.spring_on)
                {
                    bool bonded = false;
                    for (int k = 0; k < deg; ++k)
                        if ((static_cast<uint32_t>(p.se_col[static_cast<size_t>(k) * p.npad + s]) & kColMask) ==
                            static_cast<uint32_t>(j))
                        {
                            bonded = true;
                            break;
                        }
                    if (bonded)
                        continue;
                }
                if (cnt < p.pl_cap)
                    p.pl[static_cast<size_t>(cnt) * p.npad + s] = j;
                ++cnt;
            }
        }
    }
    if (cnt > p.pl_cap)
    {
        atomicOr(&ctl->status, ST_PAIR_CAPACITY);
        atomicMax(&ctl->max_row, cnt);
        cnt = p.pl_cap;
    }
    p.pl_cnt[s] = cnt;
}

// ------------------------------------------------------------------------------------------
// Step kernel
// ------------------------------------------------------------------------------------------

template <int MODE, int SM>
__global__ void __launch_bounds__(kStepBlock) k_step(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) != 0)
        return;
    const int sb = ctl->sbuf, lb = ctl->lbuf;
    const float4 *__restrict__ pos = p.pos[sb];
    const float4 *__restrict__ jp = p.jprm[lb];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;

    // energies: spring, steric, coulomb, hydrophobic, imp, kinetic
    float e[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};

    if (s < p.n)
    {
        const float4 pi = pos[s];
        const float4 ai = jp[s];
        const uint32_t fi = __float_as_uint(ai.w);
        const int id = p.perm[lb][s];
        if (fi & PF_STATIC)
        {
            if (MODE == MODE_STEP)
            {
                p.pos[sb ^ 1][s] = pi;
                p.vel[sb ^ 1][s] = p.vel[sb][s];
            }
            else
                p.force_out[id] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        else
        {
            float fx = 0.f, fy = 0.f, fz = 0.f;
            // ---- springs (Spring.cpp:20-34) ----
            if (p.spring_on)
            {
                const int deg = p.se_deg[s];
                for (int k = 0; k < deg; ++k)
                {
                    const size_t at = static_cast<size_t>(k) * p.npad + s;
                    const uint32_t c = static_cast<uint32_t>(__ldg(&p.se_col[at]));
                    if (c & kColInactive)
                        continue;
                    const float4 pj = pos[c & kColMask];
                    const float kk = __ldg(&p.se_k[at]), r0 = __ldg(&p.se_r0[at]);
                    const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
                    const float len = sqrtf(dx * dx + dy * dy + dz * dz);
                    const float dv = len - r0;
                    const float w = (c & kColStatic) ? 1.0f : 0.5f;
                    e[0] += w * (0.5f * kk * dv * dv);
                    const float fm = kk * dv * p.k_spring_f;
                    const float inv = len > 1e-40f ? 1.0f / len : 0.0f;
                    fx += dx * inv * fm;
                    fy += dy * inv * fm;
                    fz += dz * inv * fm;
                }
                e[0] *= p.spring_scale;
                fx *= p.spring_scale;
                fy *= p.spring_scale;
                fz *= p.spring_scale;
            }
            // ---- nonbonded pairs (Particle.cpp:191-253, 269-330, 368-429) ----
            {
                float sfx = 0.f, sfy = 0.f, sfz = 0.f, es = 0.f;
                float cfx = 0.f, cfy = 0.f, cfz = 0.f, ec = 0.f;
                float hfx = 0.f, hfy = 0.f, hfz = 0.f, eh = 0.f;
                const int cnt = p.pl_cnt[s];
                const bool qi_on = p.coulomb_on && (fi & PF_CHARGED);
                const bool hi_on = p.hydro_on && (fi & PF_HYDROPHOBIC);
                for (int k = 0; k < cnt; ++k)
                {
                    const int j = __ldg(&p.pl[static_cast<size_t>(k) * p.npad + s]);
                    const float4 pj = pos[j];
                    const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 >= p.r2_any)
                        continue;
                    const float4 aj = jp[j];
                    const uint32_t fj = __float_as_uint(aj.w);
                    const float w = (fj & PF_STATIC) ? 1.0f : 0.5f;
                    float d;
                    if (p.steric_on && pair_in(r2, p.lo2_s, p.hi2_s, pi, pj, p.c_steric, false, &d))
                    {
                        const float inv_d = d > 1e-40f ? 1.0f / d : 0.0f;
                        float fm, pe;
                        steric_pair<SM>(d, inv_d, ai.x, ai.y, aj.x, aj.y, p.k_spring_f, fm, pe);
                        es += w * pe;
                        sfx += dx * inv_d * fm;
                        sfy += dy * inv_d * fm;
                        sfz += dz * inv_d * fm;
                    }
                    if (qi_on && pj.w != 0.0f && pair_in(r2, p.lo2_c, p.hi2_c, pi, pj, p.c_coulomb, true, &d))
                    {
                        const float inv_d = 1.0f / d;
                        float fm, pe;
                        coulomb_pair(p, d, inv_d, pi.w * pj.w, fm, pe);
                        ec += w * pe;
                        cfx += dx * inv_d * fm;
                        cfy += dy * inv_d * fm;
                        cfz += dz * inv_d * fm;
                    }
                    if (hi_on && aj.z != 0.0f && pair_in(r2, p.lo2_h, p.hi2_h, pi, pj, p.c_hydro, true, &d))
                    {
                        const float inv_d = 1.0f / d;
                        const float x = ai.z * aj.z * expf(-d);
                        const float pe = -x * p.k_hydro_e * p.hydro_scale;
                        const float fm = x * p.k_spring_f * p.hydro_scale;
                        eh += w * pe;
                        hfx += dx * inv_d * fm;
                        hfy += dy * inv_d * fm;
                        hfz += dz * inv_d * fm;
                    }
                }
                e[1] = es * p.steric_scale;
                e[2] = ec;
                e[3] = eh;
                fx += sfx * p.steric_scale + cfx + hfx;
                fy += sfy * p.steric_scale + cfy + hfy;
                fz += sfz * p.steric_scale + cfz + hfz;
            }
            const float4 v = p.vel[sb][s];
            // ---- viscosity (Particle.cpp:80-84) ----
            if (p.visc_on)
            {
                fx -= v.x * p.visc;
                fy -= v.y * p.visc;
                fz -= v.z * p.visc;
            }
            const float4 ip = p.iprm[lb][s];
            // ---- IMPALA, flat membrane (imp.hpp:29-159, ForceField.cpp:62-88) ----
            if (p.imp_on)
            {
                const float ex = expf(p.imp_alpha * (fabsf(pi.z) - p.imp_z0));
                const float cz = 0.5f - 1.0f / (1.0f + ex);
                const float g = -ip.y * ip.z + kAlip * ip.y;
                e[4] = p.imp_scale * g * cz;
                // dC/dz = alpha sign(z) e / (1 + e)^2, written without overflow
                float dcz = pi.z != 0.0f ? p.imp_alpha / (ex + 2.0f + 1.0f / ex) : 0.0f;
                if (pi.z < 0.0f)
                    dcz = -dcz;
                if (!isfinite(dcz))
                    dcz = 0.0f;
                fz -= p.imp_scale * (g * dcz * p.k_imp_f);
            }
            // ---- external force (SpringNetwork::setForce, SpringNetwork.cpp:438-442) ----
            if (ctl->ext_pending)
            {
                const float4 xf = p.ext[id];
                fx += xf.x;
                fy += xf.y;
                fz += xf.z;
                if (MODE == MODE_STEP && (xf.x != 0.f || xf.y != 0.f || xf.z != 0.f))
                    p.ext[id] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            if (MODE == MODE_FORCES)
            {
                p.force_out[id] = make_float4(fx, fy, fz, 0.f);
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
                const float nx = __fadd_rn(pi.x, __fmul_rn(vx, p.dt));
                const float ny = __fadd_rn(pi.y, __fmul_rn(vy, p.dt));
                const float nz = __fadd_rn(pi.z, __fmul_rn(vz, p.dt));
                p.pos[sb ^ 1][s] = make_float4(nx, ny, nz, pi.w);
                p.vel[sb ^ 1][s] = make_float4(vx, vy, vz, 0.f);
                if (!isfinite(nx) || !isfinite(ny) || !isfinite(nz))
                    atomicOr(&ctl->status_pending, ST_NONFINITE);
                const float4 b = p.pos_build[s];
                const float ddx = nx - b.x, ddy = ny - b.y, ddz = nz - b.z;
                if (ddx * ddx + ddy * ddy + ddz * ddz > p.half_skin2)
                    atomicOr(&ctl->status_pending, ST_STALE);
            }
        }
    }
    if (reduce_energies<6, kStepBlock>(e, p.blk_energy, ctl, &ctl->done_step, ctl->energies, false))
    {
        if (threadIdx.x == 0)
        {
            // energies[] order: kinetic, spring, steric, electrostatic, imp, hydrophobic
            const double sp = ctl->energies[0], st = ctl->energies[1], co = ctl->energies[2],
                         hy = ctl->energies[3], im = ctl->energies[4], ki = ctl->energies[5];
            ctl->energies[BS_ENERGY_KINETIC] = ki;
            ctl->energies[BS_ENERGY_SPRING] = sp;
            ctl->energies[BS_ENERGY_STERIC] = st;
            ctl->energies[BS_ENERGY_ELECTROSTATIC] = co;
            ctl->energies[BS_ENERGY_IMP] = im;
            ctl->energies[BS_ENERGY_HYDROPHOBIC] = hy;
            if (MODE == MODE_STEP)
            {
                ctl->sbuf = sb ^ 1;
                ctl->steps += 1;
                ctl->ext_pending = 0;
            }
            // Raised bits take effect for the following kernels only, so every block of this
            // launch saw the same status at entry.
            const int pend = atomicExch(&ctl->status_pending, 0);
            if (pend)
                atomicOr(&ctl->status, pend);
        }
    }
}

// ------------------------------------------------------------------------------------------
// Host-facing helpers
// ------------------------------------------------------------------------------------------

// Writes positions (what = 0), velocities (1) or forces of the last force-only evaluation (2)
// in caller order as float[3n].
__global__ void k_unsort(Params p, int what, float *out)
{
    const Ctl *ctl = p.ctl;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n)
        return;
    if (what == 2)
    {
        const float4 f = p.force_out[s];
        out[3 * s] = f.x;
        out[3 * s + 1] = f.y;
        out[3 * s + 2] = f.z;
        return;
    }
    const int id = p.perm[ctl->lbuf][s];
    const float4 q = what == 0 ? p.pos[ctl->sbuf][s] : p.vel[ctl->sbuf][s];
    out[3 * id] = q.x;
    out[3 * id + 1] = q.y;
    out[3 * id + 2] = q.z;
}

// Overwrites positions and/or velocities from caller-order float[3n] arrays (nullable).
__global__ void k_set_state(Params p, const float *xyz, const float *vel)
{
    const Ctl *ctl = p.ctl;
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= p.n)
        return;
    const int s = p.inv[id];
    if (xyz)
    {
        float4 q = p.pos[ctl->sbuf][s];
        q.x = xyz[3 * id];
        q.y = xyz[3 * id + 1];
        q.z = xyz[3 * id + 2];
        p.pos[ctl->sbuf][s] = q;
    }
    if (vel)
        p.vel[ctl->sbuf][s] = make_float4(vel[3 * id], vel[3 * id + 1], vel[3 * id + 2], 0.f);
}

// Reference cell id of each particle for a grid of edge (cutoff + skin) over the bounding box of
// all particles (nsearch.hpp:277-293, 342-390); -1 for particles without `need_flag`. One block.
__global__ void __launch_bounds__(1024) k_diag_cells(Params p, float cutoff, float skin, uint32_t need_flag,
                                                     long long *out)
{
    const Ctl *ctl = p.ctl;
    const float4 *pos = p.pos[ctl->sbuf];
    const float4 *jp = p.jprm[ctl->lbuf];
    __shared__ float smin[3][32], smax[3][32];
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = threadIdx.x; i < p.n; i += blockDim.x)
    {
        const float4 q = pos[i];
        mn[0] = fminf(mn[0], q.x);
        mn[1] = fminf(mn[1], q.y);
        mn[2] = fminf(mn[2], q.z);
        mx[0] = fmaxf(mx[0], q.x);
        mx[1] = fmaxf(mx[1], q.y);
        mx[2] = fmaxf(mx[2], q.z);
    }
    for (int k = 0; k < 3; ++k)
        for (int o = 16; o > 0; o >>= 1)
        {
            mn[k] = fminf(mn[k], __shfl_down_sync(0xffffffffu, mn[k], o));
            mx[k] = fmaxf(mx[k], __shfl_down_sync(0xffffffffu, mx[k], o));
        }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 3; ++k)
        {
            smin[k][warp] = mn[k];
            smax[k][warp] = mx[k];
        }
    __syncthreads();
    float bmn[3], bmx[3];
    for (int k = 0; k < 3; ++k)
    {
        bmn[k] = smin[k][0];
        bmx[k] = smax[k][0];
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w)
        {
            bmn[k] = fminf(bmn[k], smin[k][w]);
            bmx[k] = fmaxf(bmx[k], smax[k][w]);
        }
    }
    const float radius = cutoff + skin;
    int nc[3];
    for (int k = 0; k < 3; ++k)
    {
        const double len = __dsub_rn(static_cast<double>(bmx[k]), static_cast<double>(bmn[k]));
        nc[k] = static_cast<int>(ceil(__ddiv_rn(len, static_cast<double>(radius))) + 1.0);
    }
    for (int s = threadIdx.x; s < p.n; s += blockDim.x)
    {
        const int id = p.perm[ctl->lbuf][s];
        const uint32_t f = __float_as_uint(jp[s].w);
        if (need_flag && !(f & need_flag))
        {
            out[id] = -1;
            continue;
        }
        const float4 q = pos[s];
        const long long cx = ref_cell_coord(q.x, static_cast<double>(bmn[0]), radius, nc[0]);
        const long long cy = ref_cell_coord(q.y, static_cast<double>(bmn[1]), radius, nc[1]);
        const long long cz = ref_cell_coord(q.z, static_cast<double>(bmn[2]), radius, nc[2]);
        out[id] = cx + cy * nc[0] + cz * static_cast<long long>(nc[0]) * nc[1];
    }
}

// Emits the unique interacting pairs of one term, using the step kernel's classification,
// as caller ids (min, max). Pairs of two dynamic particles are emitted once, from the lower id.
__global__ void __launch_bounds__(kStepBlock) k_diag_pairs(Params p, int term, long long *out,
                                                           unsigned long long *count, unsigned long long cap)
{
    const Ctl *ctl = p.ctl;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n)
        return;
    const float4 *pos = p.pos[ctl->sbuf];
    const float4 *jp = p.jprm[ctl->lbuf];
    const uint32_t fi = __float_as_uint(jp[s].w);
    if (fi & PF_STATIC)
        return;
    if (term == BS_TERM_STERIC && !p.steric_on)
        return;
    if (term == BS_TERM_COULOMB && !(p.coulomb_on && (fi & PF_CHARGED)))
        return;
    if (term == BS_TERM_HYDROPHOBIC && !(p.hydro_on && (fi & PF_HYDROPHOBIC)))
        return;
    const float4 pi = pos[s];
    const int idi = p.perm[ctl->lbuf][s];
    const int cnt = p.pl_cnt[s];
    for (int k = 0; k < cnt; ++k)
    {
        const int j = p.pl[static_cast<size_t>(k) * p.npad + s];
        const float4 pj = pos[j];
        const uint32_t fj = __float_as_uint(jp[j].w);
        const int idj = p.perm[ctl->lbuf][j];
        if (!(fj & PF_STATIC) && idj < idi)
            continue;
        const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        float d;
        bool in;
        if (term == BS_TERM_STERIC)
            in = pair_in(r2, p.lo2_s, p.hi2_s, pi, pj, p.c_steric, false, &d);
        else if (term == BS_TERM_COULOMB)
            in = (fj & PF_CHARGED) && pair_in(r2, p.lo2_c, p.hi2_c, pi, pj, p.c_coulomb, true, &d);
        else
            in = (fj & PF_HYDROPHOBIC) && pair_in(r2, p.lo2_h, p.hi2_h, pi, pj, p.c_hydro, true, &d);
        if (!in)
            continue;
        const unsigned long long at = atomicAdd(count, 1ull);
        if (at < cap)
        {
            out[2 * at] = min(idi, idj);
            out[2 * at + 1] = max(idi, idj);
        }
    }
}

} // namespace

int launch_rebuild(const Params &p, cudaStream_t st)
{
    const int nb = (p.n + kBuildBlock - 1) / kBuildBlock;
    const int nbp = (p.npad + kBuildBlock - 1) / kBuildBlock;
    int bb = (p.n + kBboxBlock - 1) / kBboxBlock;
    bb = bb > 304 ? 304 : (bb < 1 ? 1 : bb);
    k_bbox<<<bb, kBboxBlock, 0, st>>>(p);
    k_cell_count<<<nb, kBuildBlock, 0, st>>>(p);
    k_cell_scan<<<1, 1024, 0, st>>>(p);
    k_cell_place<<<nb, kBuildBlock, 0, st>>>(p);
    k_cell_sort<<<1216, kBuildBlock, 0, st>>>(p);
    k_reorder<<<nb, kBuildBlock, 0, st>>>(p);
    k_spring_ell<<<nbp, kBuildBlock, 0, st>>>(p);
    k_pairlist<<<nbp, kBuildBlock, 0, st>>>(p);
    return 8;
}

int launch_step(const Params &p, int mode, cudaStream_t st)
{
    const int nb = (p.n + kStepBlock - 1) / kStepBlock;
#define BS_STEP_CASE(SMV)                                                                                              \
    case SMV:                                                                                                          \
        if (mode == MODE_STEP)                                                                                         \
            k_step<MODE_STEP, SMV><<<nb, kStepBlock, 0, st>>>(p);                                                      \
        else                                                                                                           \
            k_step<MODE_FORCES, SMV><<<nb, kStepBlock, 0, st>>>(p);                                                    \
        break;
    switch (p.steric_mode)
    {
        BS_STEP_CASE(BS_STERIC_LINEAR)
        BS_STEP_CASE(BS_STERIC_LJ_12_6_AMBER)
        BS_STEP_CASE(BS_STERIC_LJ_8_6_LEWITT)
        BS_STEP_CASE(BS_STERIC_LJ_8_6_ZACHARIAS)
    default:
        break;
    }
#undef BS_STEP_CASE
    return 1;
}

int launch_unsort(const Params &p, int what, float *out3, cudaStream_t st)
{
    k_unsort<<<(p.n + 255) / 256, 256, 0, st>>>(p, what, out3);
    return 1;
}

int launch_set_positions(const Params &p, const float *xyz, const float *vel, cudaStream_t st)
{
    k_set_state<<<(p.n + 255) / 256, 256, 0, st>>>(p, xyz, vel);
    return 1;
}

int launch_diag_cells(const Params &p, float cutoff, float skin, uint32_t need_flag, long long *out, cudaStream_t st)
{
    k_diag_cells<<<1, 1024, 0, st>>>(p, cutoff, skin, need_flag, out);
    return 1;
}

int launch_diag_pairs(const Params &p, int term, long long *out, unsigned long long *count, unsigned long long cap,
                      cudaStream_t st)
{
    k_diag_pairs<<<(p.n + kStepBlock - 1) / kStepBlock, kStepBlock, 0, st>>>(p, term, out, count, cap);
    return 1;
}

} // namespace bsg
