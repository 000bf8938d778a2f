// bs_kernels.cu -- sm_103a kernels of BioSpring's per-step force-and-integrate loop.
//
// Data layout (all in HBM, structure of arrays, particles in cell-sorted order):
//   pos[2]    float4 (x, y, z, P)   double-buffered: a step reads one and writes the other
//   vel[2]    float4 (vx, vy, vz, 0)
//   fhi/chg/hyd/flags/iprm[2]       per-particle parameters, re-laid out at every rebuild
//   perm[2]   sorted slot -> caller id;  inv: caller id -> sorted slot
//   se_*      springs of each slot, ELL column-major [k * npad + slot] (coalesced per warp),
//             rows ascending by partner slot
//   pl[t]     typed nonbonded pair lists (steric dynamic / static partners, Coulomb,
//             hydrophobic), row-major [slot * cap + k], entries ascending, rebuilt every K steps
//             from the cell grid; the steric row holds 16-bit slot offsets when they fit
//
// Steric factors: the pair parameters of the LJ forms factor per particle,
// eps_ij r_ij^m = (a_i b_i^m)(a_j b_j^m) with eps_ij = a_i a_j and r_ij = b_i b_j
// (Amber/Lewitt: a = sqrt(eps), b = sqrt(r), CombinationRules.hpp:18-31; Zacharias: a = eps,
// b = r), so P = a b^6 and fhi = a b^12 (Amber) or a b^8 (Lewitt, Zacharias); the LJ path
// then needs only 1/r^2 (no square root, no division).
//
// Rebuild (every K steps, or when a particle drifted more than skin/2):
//   k_bbox -> k_cell_count -> k_cell_scan -> k_cell_place -> k_cell_sort -> k_reorder
//   -> k_spring_ell -> k_pairlist
// Step: k_step, T consecutive lanes per particle, gathers its springs and nonbonded pairs (no
// atomics on forces, so results are deterministic) and integrates in the same pass.
//
// Reference behaviour reproduced (paths inside the BioSpring project):
//   cell grid and cell id           src/nsearch.hpp:277-293, 342-390 (FP64, same formula; the
//                                   search grid uses edge (cutoff + skin) / kGridDiv, the
//                                   diagnostic grid of bs_get_cells the reference edge)
//   pair filters                    src/nsearch.hpp:230 (FP64 distance) and src/spn/Particle.cpp:
//                                   213-224 (spring exclusion, float distance < cutoff, != 0),
//                                   :209 (static neighbour: full energy, no force on it)
//   force expressions               src/forcefield/energy/{spring,steric,electrostatic,hydrophobic,imp}.hpp
//   viscosity and Euler step        src/spn/Particle.cpp:80-84, 109-128
//   non-finite position check       src/spn/SpringNetwork.cpp:222-229 (status bit, no abort)

#include "bs_device.cuh"

namespace bsg
{

namespace
{

// ------------------------------------------------------------------------------------------
// Rebuild kernels
// ------------------------------------------------------------------------------------------

__global__ void __launch_bounds__(kBboxBlock) k_bbox(Params p)
{
    pdl_enter();
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const float4 *pos = p.pos[ctl->sbuf];
    float v[6] = {FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX}; // min x,y,z and -max x,y,z
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += gridDim.x * blockDim.x)
    {
        const float4 q = pos[i];
        v[0] = fminf(v[0], q.x);
        v[1] = fminf(v[1], q.y);
        v[2] = fminf(v[2], q.z);
        v[3] = fminf(v[3], -q.x);
        v[4] = fminf(v[4], -q.y);
        v[5] = fminf(v[5], -q.z);
    }
    __shared__ float sh[6][kBboxBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 6; ++k)
    {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v[k] = fminf(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
        if (lane == 0)
            sh[k][warp] = v[k];
    }
    __syncthreads();
    unsigned int *enc = ctl->bbox_enc;
    if (threadIdx.x < 6)
    {
        float m = sh[threadIdx.x][0];
        for (int w = 1; w < kBboxBlock / 32; ++w)
            m = fminf(m, sh[threadIdx.x][w]);
        if (threadIdx.x < 3)
            atomicMin(&enc[threadIdx.x], f2ord(m));
        else
            atomicMax(&enc[threadIdx.x], f2ord(-m));
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
    // the cell-block list build uses cells of a kGridDiv-th of the list radius, the warp-per-particle
    // build (sparse systems) cells of the list radius
    const float edge = p.list_radius / static_cast<float>(p.pl_sparse ? kSparseDiv : kGridDiv);
    int nc[3];
    double gmin[3];
    const double cells = grid_dims(mn, mx, edge, gmin, nc);
    for (int k = 0; k < 3; ++k)
        ctl->gmin[k] = gmin[k];
    ctl->gradius = edge;
    ctl->gnx = nc[0];
    ctl->gny = nc[1];
    ctl->gnz = nc[2];
    if (!(cells <= static_cast<double>(p.cell_cap)))
    {
        ctl->ncells_needed = cells < 2.0e9 ? static_cast<int>(cells) : INT_MAX;
        atomicOr(&ctl->status, ST_CELL_CAPACITY);
    }
    if (status_of(ctl) & ST_STALE)
        ctl->stale_events += 1;
    atomicAnd(&ctl->status, ~ST_STALE);
    ctl->done_bbox = 0u;
}

__global__ void __launch_bounds__(kBuildBlock) k_cell_count(Params p)
{
    pdl_enter();
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

// Exclusive scan of the cell counts in three passes over tiles of kScanTile cells, so that grids
// of millions of (mostly empty) cells cost a few microseconds. Pass 1: each block scans one tile
// (4 consecutive cells per thread) and writes the in-tile prefixes and the tile's total.
__global__ void __launch_bounds__(1024) k_scan_tiles(Params p)
{
    pdl_enter();
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int nc = ctl->gnx * ctl->gny * ctl->gnz;
    const int base = blockIdx.x * kScanTile;
    if (base >= nc)
        return;
    const int c0 = base + 4 * threadIdx.x;
    int v[4], sum = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        v[k] = c0 + k < nc ? p.cell_cnt[c0 + k] : 0;
        sum += v[k];
    }
    __shared__ int sh_warp[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o)
            inc += t;
    }
    if (lane == 31)
        sh_warp[warp] = inc;
    __syncthreads();
    if (warp == 0)
    {
        int w = sh_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o)
                w += t;
        }
        sh_warp[lane] = w; // inclusive over warps
    }
    __syncthreads();
    int run = inc - sum + (warp > 0 ? sh_warp[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        if (c0 + k < nc)
            p.cell_start[c0 + k] = run;
        run += v[k];
    }
    if (threadIdx.x == blockDim.x - 1)
        p.tile_sum[blockIdx.x] = sh_warp[31];
}

// Pass 2 (one block): exclusive scan of the tile totals, in place; writes the grand total after
// the last cell.
__global__ void __launch_bounds__(1024) k_scan_top(Params p)
{
    pdl_enter();
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int nc = ctl->gnx * ctl->gny * ctl->gnz;
    const int nt = (nc + kScanTile - 1) / kScanTile;
    const int per = (nt + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per, b1 = min(nt, b0 + per);
    int sum = 0;
    for (int t = b0; t < b1; ++t)
        sum += p.tile_sum[t];
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
    for (int t = b0; t < b1; ++t)
    {
        const int k = p.tile_sum[t];
        p.tile_sum[t] = run;
        run += k;
    }
    if (threadIdx.x == blockDim.x - 1)
        p.cell_start[nc] = run;
}

// Pass 3: adds each tile's offset, primes the fill cursors and clears the counts for the next
// rebuild.
__global__ void __launch_bounds__(1024) k_scan_add(Params p)
{
    pdl_enter();
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int nc = ctl->gnx * ctl->gny * ctl->gnz;
    const int base = blockIdx.x * kScanTile;
    if (base >= nc)
        return;
    const int off = p.tile_sum[blockIdx.x];
    const int c0 = base + 4 * threadIdx.x;
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        const int c = c0 + k;
        if (c < nc)
        {
            const int st = p.cell_start[c] + off;
            p.cell_start[c] = st;
            p.cell_fill[c] = st;
            p.cell_cnt[c] = 0;
        }
    }
}

__global__ void __launch_bounds__(kBuildBlock) k_cell_place(Params p)
{
    pdl_enter();
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n)
        return;
    const int slot = atomicAdd(&p.cell_fill[p.cell_of[i]], 1);
    const int id = p.perm[ctl->lbuf][i];
    // the order key of k_cell_sort: x coordinate, then caller id
    p.tmp_key[slot] = (static_cast<unsigned long long>(f2ord(p.pos[ctl->sbuf][i].x)) << 32) |
                      static_cast<unsigned int>(id);
}

// One warp per cell: orders the cell's particles by x coordinate, ties by caller id, which makes
// the layout deterministic and every x-run of cells one x-sorted sequence (the pair-list build
// bounds its candidates in a run by binary search). Cells are filled in any order by
// k_cell_place; the reference appends to a cell in index order (nsearch.hpp:376-389), an order
// no result here depends on.
__global__ void __launch_bounds__(kBuildBlock) k_cell_sort(Params p)
{
    pdl_enter();
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int nc = ctl->gnx * ctl->gny * ctl->gnz;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    int *out = p.perm[ctl->lbuf ^ 1];
    const unsigned long long *__restrict__ key = p.tmp_key;
    for (int c = warp; c < nc; c += nwarps)
    {
        const int s0 = p.cell_start[c], s1 = p.cell_start[c + 1];
        const int len = s1 - s0;
        if (len <= 64)
        {
            // up to two keys per lane, ranked against every key of the cell by shuffles
            const unsigned long long k0 = lane < len ? key[s0 + lane] : ~0ull;
            const unsigned long long k1 = lane + 32 < len ? key[s0 + 32 + lane] : ~0ull;
            int r0 = 0, r1 = 0;
            for (int f = 0; f < len; ++f)
            {
                const unsigned long long kf = __shfl_sync(0xffffffffu, f < 32 ? k0 : k1, f & 31);
                r0 += kf < k0;
                r1 += kf < k1;
            }
            if (lane < len)
            {
                out[s0 + r0] = static_cast<int>(k0 & 0xffffffffu);
                p.cell_of[s0 + r0] = c;
            }
            if (lane + 32 < len)
            {
                out[s0 + r1] = static_cast<int>(k1 & 0xffffffffu);
                p.cell_of[s0 + r1] = c;
            }
            continue;
        }
        for (int e = lane; e < len; e += 32)
        {
            const unsigned long long ke = key[s0 + e];
            int rank = 0;
            for (int f = 0; f < len; ++f)
                rank += key[s0 + f] < ke;
            out[s0 + rank] = static_cast<int>(ke & 0xffffffffu);
            p.cell_of[s0 + rank] = c;
        }
    }
}

// Moves the state into the new layout, records build positions and the new inverse permutation,
// then (last block) makes the new layout current.
__global__ void __launch_bounds__(kBuildBlock) k_reorder(Params p)
{
    pdl_enter();
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
        if (p.pos_lo[0])
            p.pos_lo[sb ^ 1][i] = p.pos_lo[sb][old];
        p.fhi[lb ^ 1][i] = p.fhi[lb][old];
        p.chg[lb ^ 1][i] = p.chg[lb][old];
        p.hyd[lb ^ 1][i] = p.hyd[lb][old];
        if (p.bur[0])
            p.bur[lb ^ 1][i] = p.bur[lb][old];
        p.flags[lb ^ 1][i] = p.flags[lb][old];
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

// Springs of every slot in the new layout, partners as slots (ELL, column-major). ell_lanes
// consecutive threads share a slot and take every ell_lanes-th spring of its caller-order row,
// so the row is read with contiguous loads and the partner lookups of a slot overlap; with one
// lane per slot, the threads of a warp store each column contiguously.
__global__ void __launch_bounds__(kBuildBlock) k_spring_ell(Params p)
{
    pdl_enter();
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const long long g = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int L = p.ell_lanes;
    const int s = static_cast<int>(g / L), t = static_cast<int>(g % L);
    if (s >= p.npad)
        return;
    if (s >= p.n)
    {
        if (t == 0)
            p.se_deg[s] = 0;
        return;
    }
    const int id = p.perm[ctl->lbuf][s];
    const int r0 = p.sp_row[id], r1 = p.sp_row[id + 1];
    const size_t stride = static_cast<size_t>(p.npad);
    for (int e = r0 + t; e < r1; e += L)
    {
        const unsigned int c = p.sp_col[e];
        const unsigned int slot = static_cast<unsigned int>(p.inv[c & kSlotMask]);
        const size_t dst = static_cast<size_t>(e - r0) * stride + s;
        p.se_col[dst] = slot | (c & ~kSlotMask);
        p.se_k[dst] = p.sp_k[e];
        p.se_r0[dst] = p.sp_r0[e];
        if (p.se_sid)
            p.se_sid[dst] = p.sp_sid[e];
    }
    if (t == 0)
        p.se_deg[s] = r1 - r0;
}

// Typed pair lists from the cell grid: steric (every pair within its cutoff + skin, dynamic and
// static partners apart), Coulomb (both charged) and hydrophobic (both hydrophobic), minus the
// slot itself and, when springs are enabled, its spring partners (Particle.cpp:213-218).
//
// The grid edge is (cutoff + skin) / kGridDiv, so a particle's neighbours lie within kGridDiv
// cells in each direction: in (2 kGridDiv + 1)^2 x-runs of cells, each a contiguous range of
// slots. A block owns a group of kGridDiv^3 cells (grid-stride over the groups) and stages in
// shared memory the x-runs that cover the group's neighbourhood, (3 kGridDiv)^2 rows of
// 3 kGridDiv cells; its kPlWarps warps share the group's home particles. Cells are x-sorted and
// a cell's index grows with x, so every staged row is one x-sorted sequence: for one home particle
// at a time, lane r bounds the home's run r by binary search to the x-interval the list radius
// allows at that run's y/z distance. With kGridDiv > 1 the bounded runs are walked as one packed
// sequence (every window full but the last), else run by run; 32 candidates per pass, one per
// lane. Accepted candidates are found with one ballot and appended to the home particle's
// row-major row at consecutive positions (coalesced stores); the home particle's state stays in
// registers and lanes never diverge. Rows come out in ascending slot order (runs ascend in z, then
// y; slots ascend within a run). Bonded partners are excluded without touching memory in the
// windows: the home's spring partners sit in registers (two per lane), each lane maps its partners
// once to their positions in the candidate sequence (runs are contiguous slot ranges), and a
// window's excluded lanes come from one OR-reduction over the warp. A group whose neighbourhood exceeds the stage reads whole rows from global memory. In
// 16-bit mode the steric row holds partner-minus-slot offsets.
template <bool PL16>
__global__ void __launch_bounds__(kPlWarps * 32, kPlMinBlocks) k_pairlist(Params p)
{
    pdl_enter();
    constexpr int kD = kGridDiv;        // neighbours lie within kD cells
    constexpr int kG = kGridDiv;        // a block's group is kG^3 cells
    constexpr int kSpan = 2 * kD + 1;   // a home particle's runs per dimension (y, z)
    constexpr int kRuns = kSpan * kSpan;
    constexpr int kRowsD = kG + 2 * kD; // staged rows per dimension (y, z)
    constexpr int kRows = kRowsD * kRowsD;
    constexpr int kStageUnroll = 4;
    static_assert(kRuns <= 32, "one lane per x-run");
    __shared__ int sh_row[kRows][3];     // first slot, end slot, offset in the stage
    __shared__ int sh_home[kG * kG][3];  // the group's home x-runs: first slot, end slot, first home
#if BS_PL_PACK
    __shared__ int sh_cr[kPlWarps][2 * kRuns]; // per warp: the non-empty runs' stage index and first k
#endif
    __shared__ float4 sh_pos[kPlStage];
    __shared__ int sh_slot[kPlStage];
    __shared__ unsigned char sh_flag[kPlStage];
    __shared__ int blocked, staged, n_home, n_stage;
    Ctl *ctl = p.ctl;
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0)
        blocked = (status_of(ctl) & kRebuildBlocking) != 0;
    __syncthreads();
    if (blocked)
        return;
    const int nx = ctl->gnx, ny = ctl->gny, nz = ctl->gnz;
    const int ngx = (nx + kG - 1) / kG, ngy = (ny + kG - 1) / kG, ngz = (nz + kG - 1) / kG;
    const int ngroups = ngx * ngy * ngz;
    const int sb = ctl->sbuf, lb = ctl->lbuf;
    const float4 *__restrict__ pos = p.pos[sb];
    const unsigned int *__restrict__ fl = p.flags[lb];
    const float r2_0 = p.pl[0].r2, r2_1 = p.pl[1].r2, r2_2 = p.pl[2].r2;
    const float edge = ctl->gradius;
    const float gy = static_cast<float>(ctl->gmin[1]), gz = static_cast<float>(ctl->gmin[2]);
    constexpr float kRowMargin = 1e-2f; // A: covers the FP32 rounding of the cell bounds
    const bool l0 = p.pl[0].on, l1 = p.pl[1].on, l2 = p.pl[2].on, l3 = p.pl[3].on;
    const int cap0 = p.pl[0].cap, cap1 = p.pl[1].cap, cap2 = p.pl[2].cap, cap3 = p.pl[3].cap;
    const size_t stride = static_cast<size_t>(p.npad);
    const unsigned int below = (1u << lane) - 1u;
    for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x)
    {
        const int gx0 = grp % ngx * kG, gy0 = grp / ngx % ngy * kG, gz0 = grp / (ngx * ngy) * kG;
        const int xa = max(gx0 - kD, 0), xb = min(gx0 + kG - 1 + kD, nx - 1), hxb = min(gx0 + kG - 1, nx - 1);
        __syncthreads(); // the previous group's stage and tables are no longer read
        for (int t = threadIdx.x; t < kRows + kG * kG; t += blockDim.x)
        {
            int j0 = 0, j1 = 0;
            if (t < kRows)
            {
                const int y = gy0 - kD + t % kRowsD, z = gz0 - kD + t / kRowsD;
                if (y >= 0 && y < ny && z >= 0 && z < nz)
                {
                    const int base = (z * ny + y) * nx;
                    j0 = p.cell_start[base + xa];
                    j1 = p.cell_start[base + xb + 1];
                }
                sh_row[t][0] = j0;
                sh_row[t][1] = j1;
            }
            else
            {
                const int u = t - kRows;
                const int y = gy0 + u % kG, z = gz0 + u / kG;
                if (y < ny && z < nz)
                {
                    const int base = (z * ny + y) * nx;
                    j0 = p.cell_start[base + gx0];
                    j1 = p.cell_start[base + hxb + 1];
                }
                sh_home[u][0] = j0;
                sh_home[u][1] = j1;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0)
        {
            int tot = 0, nh = 0, lo = INT_MAX, hi = INT_MIN, hmin = INT_MAX, hmax = INT_MIN;
            for (int u = 0; u < kG * kG; ++u)
            {
                sh_home[u][2] = nh;
                const int len = sh_home[u][1] - sh_home[u][0];
                nh += len;
                if (len > 0)
                {
                    hmin = min(hmin, sh_home[u][0]);
                    hmax = max(hmax, sh_home[u][1]);
                }
            }
            for (int r = 0; r < kRows; ++r)
            {
                sh_row[r][2] = tot;
                const int len = sh_row[r][1] - sh_row[r][0];
                tot += len;
                if (len > 0)
                {
                    lo = min(lo, sh_row[r][0]);
                    hi = max(hi, sh_row[r][1]);
                }
            }
            n_home = nh;
            n_stage = tot;
            staged = tot <= kPlStage;
            // every candidate offset of this group fits 16 bits, or the list goes 32-bit
            if (PL16 && nh > 0 && (hi - 1 - hmin > 32767 || lo - (hmax - 1) < -32768))
                atomicOr(&ctl->status, ST_WIDE);
        }
        __syncthreads();
        const int nh = n_home;
        if (nh == 0)
            continue;
        // the candidates of the group's rows are read by every warp of the block: stage them,
        // kStageUnroll loads in flight per thread
        if (staged)
            for (int k0 = threadIdx.x; k0 < n_stage; k0 += kStageUnroll * blockDim.x)
            {
                float4 v[kStageUnroll];
                unsigned int f[kStageUnroll];
                int sl[kStageUnroll];
#pragma unroll
                for (int u = 0; u < kStageUnroll; ++u)
                {
                    const int k = k0 + u * static_cast<int>(blockDim.x);
                    sl[u] = -1;
                    if (k < n_stage)
                    {
                        int a = 0, b = kRows - 1; // the last row whose offset is <= k
                        while (a < b)
                        {
                            const int m = (a + b + 1) >> 1;
                            if (sh_row[m][2] <= k)
                                a = m;
                            else
                                b = m - 1;
                        }
                        sl[u] = sh_row[a][0] + (k - sh_row[a][2]);
                        v[u] = pos[sl[u]];
                        f[u] = fl[sl[u]];
                    }
                }
#pragma unroll
                for (int u = 0; u < kStageUnroll; ++u)
                    if (sl[u] >= 0)
                    {
                        const int k = k0 + u * static_cast<int>(blockDim.x);
                        sh_pos[k] = v[u];
                        sh_slot[k] = sl[u];
                        sh_flag[k] = static_cast<unsigned char>(f[u]);
                    }
            }
        __syncthreads();
        for (int hh = wid; hh < nh; hh += kPlWarps)
        {
            int hu = 0;
            while (hu + 1 < kG * kG && sh_home[hu + 1][2] <= hh)
                ++hu;
            const int i = sh_home[hu][0] + (hh - sh_home[hu][2]);
            const int hy = hu % kG, hz = hu / kG; // the home's cell in the group (y, z)
            const unsigned int fi = fl[i];
            const bool dyn = !(fi & PF_STATIC);
            const bool on0 = dyn && l0;
            const bool on1 = dyn && l1 && ((fi & PF_CHARGED) || p.coul_all);
            const bool on2 = dyn && l2 && (fi & PF_HYDROPHOBIC);
            const bool need_fj = l3 || on1 || on2;
            float r2max = on0 ? r2_0 : 0.0f;
            if (on1)
                r2max = fmaxf(r2max, r2_1);
            if (on2)
                r2max = fmaxf(r2max, r2_2);
            int cnt0 = 0, cnt1 = 0, cnt2 = 0, cnt3 = 0;
            if (on0 || on1 || on2)
            {
                const float4 pi = pos[i];
                // spring partners of i in registers: lane m holds partners m and m + 32 (slots, -1
                // for none); a home with more than 64 compares every candidate with its ELL row
                const int deg = p.spring_on ? p.se_deg[i] : 0;
                const bool small = deg <= 64;
                const int ps0 = small && lane < deg
                                    ? static_cast<int>(p.se_col[static_cast<size_t>(lane) * stride + i] & kSlotMask)
                                    : -1;
                const int ps1 = small && lane + 32 < deg
                                    ? static_cast<int>(p.se_col[static_cast<size_t>(lane + 32) * stride + i] & kSlotMask)
                                    : -1;
                // the lanes whose candidate is a spring partner: partner positions t in [0, 32)
                // relative to the window's first candidate, OR-ed over the warp
                auto partner_mask = [&](const int t0, const int t1) {
                    unsigned int b = t0 >= 0 && t0 < 32 ? 1u << t0 : 0u;
                    if (t1 >= 0 && t1 < 32)
                        b |= 1u << t1;
                    return __reduce_or_sync(0xffffffffu, b);
                };
                short *row0s = reinterpret_cast<short *>(p.pl[0].idx) + static_cast<size_t>(i) * cap0;
                unsigned int *row0 = p.pl[0].idx + static_cast<size_t>(i) * cap0;
                unsigned int *row1 = p.pl[1].idx + static_cast<size_t>(i) * cap1;
                unsigned int *row2 = p.pl[2].idx + static_cast<size_t>(i) * cap2;
                unsigned int *row3 = p.pl[3].idx + static_cast<size_t>(i) * cap3;
                // One window of up to 32 candidates, one per lane; bonded marks the lanes whose
                // candidate is a spring partner.
                auto window = [&](const int j, const bool jv, const float4 pj, const unsigned int fj,
                                  const unsigned int bonded) {
                    const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    bool in = jv && r2 < r2max && j != i && !((bonded >> lane) & 1u);
                    if (!small)
                        for (int k = 0; k < deg; ++k)
                            in = in && static_cast<int>(p.se_col[static_cast<size_t>(k) * stride + i] & kSlotMask) != j;
                    const bool st = (fj & PF_STATIC) != 0;
                    if (on0)
                    {
                        const bool a0 = in && !st && r2 < r2_0;
                        const unsigned int m0 = __ballot_sync(0xffffffffu, a0);
                        if (a0)
                        {
                            const int at = cnt0 + __popc(m0 & below);
                            if (at < cap0)
                            {
                                if (PL16)
                                    row0s[at] = static_cast<short>(j - i);
                                else
                                    row0[at] = static_cast<unsigned int>(j);
                            }
                        }
                        cnt0 += __popc(m0);
                        if (l3)
                        {
                            const bool a3 = in && st && r2 < r2_0;
                            const unsigned int m3 = __ballot_sync(0xffffffffu, a3);
                            if (a3 && cnt3 + __popc(m3 & below) < cap3)
                                row3[cnt3 + __popc(m3 & below)] = static_cast<unsigned int>(j) | kEntryStatic;
                            cnt3 += __popc(m3);
                        }
                    }
                    if (on1)
                    {
                        const bool a1 = in && ((fj & PF_CHARGED) || p.coul_all) && r2 < r2_1;
                        const unsigned int m1 = __ballot_sync(0xffffffffu, a1);
                        if (a1 && cnt1 + __popc(m1 & below) < cap1)
                            row1[cnt1 + __popc(m1 & below)] = static_cast<unsigned int>(j) | (st ? kEntryStatic : 0u);
                        cnt1 += __popc(m1);
                    }
                    if (on2)
                    {
                        const bool a2 = in && (fj & PF_HYDROPHOBIC) && r2 < r2_2;
                        const unsigned int m2 = __ballot_sync(0xffffffffu, a2);
                        if (a2 && cnt2 + __popc(m2 & below) < cap2)
                            row2[cnt2 + __popc(m2 & below)] = static_cast<unsigned int>(j) | (st ? kEntryStatic : 0u);
                        cnt2 += __popc(m2);
                    }
                };
                if (staged)
                {
                    // lane r bounds the home's run r (cell offsets -kD + r % kSpan in y and
                    // -kD + r / kSpan in z; cell bounds widened by kRowMargin, the grid's outer
                    // cells unbounded) by binary search. Every candidate inside the bounds is still
                    // tested exactly; those outside are farther than the radius.
                    int lo_r = 0, cnt_r = 0;
                    if (lane < kRuns)
                    {
                        const int a = lane % kSpan, b = lane / kSpan;
                        const int row = (hz + b) * kRowsD + (hy + a);
                        const int len = sh_row[row][1] - sh_row[row][0], o = sh_row[row][2];
                        if (len > 0)
                        {
                            const int ry = gy0 + hy + a - kD, rz = gz0 + hz + b - kD;
                            const float y0 = ry == 0 ? -FLT_MAX : gy + ry * edge - kRowMargin;
                            const float y1 = ry == ny - 1 ? FLT_MAX : gy + (ry + 1) * edge + kRowMargin;
                            const float z0 = rz == 0 ? -FLT_MAX : gz + rz * edge - kRowMargin;
                            const float z1 = rz == nz - 1 ? FLT_MAX : gz + (rz + 1) * edge + kRowMargin;
                            const float dy = fmaxf(0.0f, fmaxf(y0 - pi.y, pi.y - y1));
                            const float dz = fmaxf(0.0f, fmaxf(z0 - pi.z, pi.z - z1));
                            const float d2 = dy * dy + dz * dz;
                            if (d2 < r2max)
                            {
                                const float hx = sqrtf(r2max - d2) * 1.0001f + kRowMargin;
                                const float xa_ = pi.x - hx, xb_ = pi.x + hx;
                                int u0 = 0, v0 = len;
                                while (u0 < v0)
                                {
                                    const int m = (u0 + v0) >> 1;
                                    if (sh_pos[o + m].x < xa_)
                                        u0 = m + 1;
                                    else
                                        v0 = m;
                                }
                                int u1 = u0, v1 = len;
                                while (u1 < v1)
                                {
                                    const int m = (u1 + v1) >> 1;
                                    if (sh_pos[o + m].x <= xb_)
                                        u1 = m + 1;
                                    else
                                        v1 = m;
                                }
                                lo_r = o + u0;
                                cnt_r = u1 - u0;
                            }
                        }
                    }
#if BS_PL_PACK
                    // The bounded runs, empty ones dropped, are walked as one sequence of
                    // candidates (k = 0 .. total-1, in run order, hence ascending slots) so that
                    // every window but the last is full. Lane c holds the c-th non-empty run: its
                    // first stage index and its first k; a lane finds the run of its k from the run
                    // starts inside its window.
                    const unsigned int ne = __ballot_sync(0xffffffffu, cnt_r > 0);
                    int incl = cnt_r;
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1)
                    {
                        const int v = __shfl_up_sync(0xffffffffu, incl, d);
                        if (lane >= d)
                            incl += v;
                    }
                    const int total = __shfl_sync(0xffffffffu, incl, 31);
                    const int nr = __popc(ne);
                    int *cr = sh_cr[wid];
                    if (cnt_r > 0)
                    {
                        const int c = __popc(ne & below);
                        cr[2 * c] = lo_r;
                        cr[2 * c + 1] = incl - cnt_r;
                    }
                    __syncwarp();
                    const int lo_c = lane < nr ? cr[2 * lane] : 0;
                    const int pre_c = lane < nr ? cr[2 * lane + 1] : total;
                    const int nxt = __shfl_down_sync(0xffffffffu, pre_c, 1);
                    const int end_c = lane + 1 < nr ? nxt : total;
                    // each spring partner's index in the candidate sequence (-1: not a candidate):
                    // the last run whose first slot is <= the partner's, by a binary search over
                    // the lanes' runs; runs are contiguous slot ranges
                    int pk0 = -1, pk1 = -1;
                    if (deg > 0 && small && total > 0)
                    {
                        const int s_c = lane < nr ? sh_slot[lo_c] : INT_MAX;
                        const int n_c = end_c - pre_c;
                        auto locate = [&](const int ps) {
                            int at = 0;
#pragma unroll
                            for (int step = 16; step > 0; step >>= 1)
                            {
                                const int v = __shfl_sync(0xffffffffu, s_c, (at + step) & 31);
                                if (at + step < nr && v <= ps)
                                    at += step;
                            }
                            const int s0 = __shfl_sync(0xffffffffu, s_c, at);
                            const int n0 = __shfl_sync(0xffffffffu, n_c, at);
                            const int k0 = __shfl_sync(0xffffffffu, pre_c, at);
                            return ps >= s0 && ps < s0 + n0 ? k0 + (ps - s0) : -1;
                        };
                        pk0 = locate(ps0);
                        if (deg > 32)
                            pk1 = locate(ps1);
                    }
                    for (int wb = 0; wb < total; wb += 32)
                    {
                        const int k = wb + lane;
                        const int r0 = __popc(__ballot_sync(0xffffffffu, lane < nr && end_c <= wb));
                        const int t = pre_c - wb;
                        const unsigned int starts =
                            __reduce_or_sync(0xffffffffu, (lane < nr && t > 0 && t < 32) ? (1u << t) : 0u);
                        const int rk = min(r0 + __popc(starts & ((2u << lane) - 1u)), nr - 1);
                        const int lo = __shfl_sync(0xffffffffu, lo_c, rk);
                        const int pre = __shfl_sync(0xffffffffu, pre_c, rk);
                        const bool jv = k < total;
                        const int qc = jv ? lo + (k - pre) : lo;
                        const unsigned int bonded =
                            deg > 0 && small ? partner_mask(pk0 < 0 ? -1 : pk0 - wb, pk1 < 0 ? -1 : pk1 - wb) : 0u;
                        window(sh_slot[qc], jv, sh_pos[qc], sh_flag[qc], bonded);
                    }
#else
                    for (int r = 0; r < kRuns; ++r)
                    {
                        const int lo = __shfl_sync(0xffffffffu, lo_r, r);
                        const int cn = __shfl_sync(0xffffffffu, cnt_r, r);
                        for (int jb = 0; jb < cn; jb += 32)
                        {
                            const bool jv = jb + lane < cn;
                            const int qc = lo + (jv ? jb + lane : cn - 1);
                            const int j0 = __shfl_sync(0xffffffffu, sh_slot[qc], 0);
                            const unsigned int bonded =
                                deg > 0 && small ? partner_mask(ps0 < 0 ? -1 : ps0 - j0, ps1 < 0 ? -1 : ps1 - j0) : 0u;
                            window(sh_slot[qc], jv, sh_pos[qc], sh_flag[qc], bonded & (jv ? ~0u : 0u));
                        }
                    }
#endif
                }
                else
                    for (int r = 0; r < kRuns; ++r)
                    {
                        const int row = (hz + r / kSpan) * kRowsD + (hy + r % kSpan);
                        const int j0 = sh_row[row][0], j1 = sh_row[row][1];
                        for (int jb = j0; jb < j1; jb += 32)
                        {
                            const int j = jb + lane;
                            const bool jv = j < j1;
                            const int jc = jv ? j : j1 - 1;
                            const unsigned int bonded =
                                deg > 0 && small ? partner_mask(ps0 < 0 ? -1 : ps0 - jb, ps1 < 0 ? -1 : ps1 - jb) : 0u;
                            window(jc, jv, pos[jc], need_fj ? fl[jc] : 0u, bonded);
                        }
                    }
            }
            if (lane == 0)
            {
                const int cnts[kLists] = {cnt0, cnt1, cnt2, cnt3};
#pragma unroll
                for (int q = 0; q < kLists; ++q)
                {
                    int k = cnts[q];
                    if (k > p.pl[q].cap)
                    {
                        atomicOr(&ctl->status, ST_PAIR_CAPACITY);
                        atomicMax(&ctl->max_row[q], k);
                        k = p.pl[q].cap;
                    }
                    p.pl[q].cnt[i] = k;
                }
            }
        }
    }
}

// One step (or one force evaluation) for every particle. T consecutive lanes share a particle:
// each takes every T-th entry of the particle's spring row and pair lists, the group sums its
// partial forces with shuffles, and the group's first lane adds the per-particle terms and
// integrates. T > 1 gives the latency-bound gather loops T times more independent loads in
// flight than one thread per particle would.
template <int MODE, int SM, int T, bool LEAN>
__global__ void __launch_bounds__(kStepKernelBlock, kStepMinBlocks) k_step(Params p)
{
    pdl_enter();
    Ctl *ctl = p.ctl;
    if (status_of(ctl) != 0)
        return;
    const int sb = ctl->sbuf, lb = ctl->lbuf;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    float e[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const int pend = particle_step<MODE, SM, T, true, LEAN>(p, g / T, g % T, p.n, sb, lb, ctl->ext_pending != 0, e);
    if (pend)
        atomicOr(&ctl->status_pending, pend);
    if (reduce_energies<6, kStepKernelBlock>(e, p.blk_energy, p.blk_cap, &ctl->done_step, ctl->energies))
    {
        if (threadIdx.x == 0)
        {
            // energies[] were written in e[] order: spring, steric, coulomb, hydrophobic, imp, kinetic
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

// The probe's own step, after the step kernel (SpringNetwork.cpp:156-182): the sum of the
// particles' reactions (float-float, fixed order), viscosity from its velocity, the Euler step
// (Particle.cpp:109-128) and its kinetic energy, added to the step's total. One block.
__global__ void __launch_bounds__(1024) k_probe(Params p)
{
    pdl_enter();
    Ctl *ctl = p.ctl;
    const long long steps = *(volatile const long long *)&ctl->steps;
    if (steps == ctl->probe_steps)
        return; // the step kernel did not run
    float acc[3][2] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (int s = threadIdx.x; s < p.n; s += blockDim.x)
    {
        const float4 f = p.probe_f[s];
        ff_add(acc[0][0], acc[0][1], f.x, 0.f);
        ff_add(acc[1][0], acc[1][1], f.y, 0.f);
        ff_add(acc[2][0], acc[2][1], f.z, 0.f);
    }
    __shared__ float sh[3][2][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        float hi = acc[k][0], lo = acc[k][1];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            const float h2 = __shfl_down_sync(0xffffffffu, hi, o);
            const float l2 = __shfl_down_sync(0xffffffffu, lo, o);
            ff_add(hi, lo, h2, l2);
        }
        if (lane == 0)
        {
            sh[k][0][warp] = hi;
            sh[k][1][warp] = lo;
        }
    }
    __syncthreads();
    if (threadIdx.x != 0)
        return;
    float F[3];
    for (int k = 0; k < 3; ++k)
    {
        float hi = 0.f, lo = 0.f;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w)
            ff_add(hi, lo, sh[k][0][w], sh[k][1][w]);
        F[k] = __fadd_rn(hi, lo);
    }
    float4 v = ctl->probe_vel, x = ctl->probe_pos;
    if (p.visc_on)
    {
        F[0] = __fsub_rn(F[0], __fmul_rn(v.x, p.visc));
        F[1] = __fsub_rn(F[1], __fmul_rn(v.y, p.visc));
        F[2] = __fsub_rn(F[2], __fmul_rn(v.z, p.visc));
    }
    const float m = p.probe_mass;
    if (m > 0.0f)
    {
        v.x = __fadd_rn(v.x, __fmul_rn(__fdiv_rn(F[0], m), p.dt));
        v.y = __fadd_rn(v.y, __fmul_rn(__fdiv_rn(F[1], m), p.dt));
        v.z = __fadd_rn(v.z, __fmul_rn(__fdiv_rn(F[2], m), p.dt));
    }
    const double vx = v.x, vy = v.y, vz = v.z;
    const float vit = static_cast<float>(sqrt(__dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz))));
    const float ke = 0.5f * m * (vit * vit) * p.k_kin;
    x.x = __fadd_rn(x.x, __fmul_rn(v.x, p.dt));
    x.y = __fadd_rn(x.y, __fmul_rn(v.y, p.dt));
    x.z = __fadd_rn(x.z, __fmul_rn(v.z, p.dt));
    ctl->probe_pos = x;
    ctl->probe_vel = v;
    ctl->energies[BS_ENERGY_KINETIC] += static_cast<double>(ke);
    ctl->probe_steps = steps;
}

// ------------------------------------------------------------------------------------------
// Host-facing helpers
// ------------------------------------------------------------------------------------------

// Writes positions (what = 0), velocities (1), forces of the last force-only evaluation (2) or
// the positions' rounding remainders (3, precise_positions) in caller order as float[3n].
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
    float4 q;
    if (what == 3)
        q = p.pos_lo[0] ? p.pos_lo[ctl->sbuf][s] : make_float4(0.f, 0.f, 0.f, 0.f);
    else
        q = what == 0 ? p.pos[ctl->sbuf][s] : p.vel[ctl->sbuf][s];
    out[3 * id] = q.x;
    out[3 * id + 1] = q.y;
    out[3 * id + 2] = q.z;
}

// Overwrites positions and/or velocities from caller-order float[3n] arrays (nullable); new
// positions get the rounding remainders `lo` (float[3n], nullable: zero).
__global__ void k_set_state(Params p, const float *xyz, const float *vel, const float *lo)
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
        if (p.pos_lo[0])
            p.pos_lo[ctl->sbuf][s] = lo ? make_float4(lo[3 * id], lo[3 * id + 1], lo[3 * id + 2], 0.f)
                                        : make_float4(0.f, 0.f, 0.f, 0.f);
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
    const unsigned int *fl = p.flags[ctl->lbuf];
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
        if (need_flag && !(fl[s] & need_flag))
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
    const unsigned int fi = p.flags[ctl->lbuf][s];
    if (fi & PF_STATIC)
        return;
    if (!p.pl[term].on)
        return;
    const float4 pi = pos[s];
    const int idi = p.perm[ctl->lbuf][s];
    float lo2 = p.lo2_s, hi2 = p.hi2_s, cut = p.c_steric;
    if (term == BS_TERM_COULOMB)
    {
        lo2 = p.lo2_c;
        hi2 = p.hi2_c;
        cut = p.c_coulomb;
    }
    else if (term == BS_TERM_HYDROPHOBIC)
    {
        lo2 = p.lo2_h;
        hi2 = p.hi2_h;
        cut = p.c_hydro;
    }
    // the steric term has two lists: dynamic partners (0) and static partners (3)
    for (int pass = 0; pass < 2; ++pass)
    {
    const int li = pass == 0 ? term : kListStericStatic;
    if (pass == 1 && term != BS_TERM_STERIC)
        break;
    const PairList &L = p.pl[li];
    const int cnt = L.cnt[s];
    for (int k = 0; k < cnt; ++k)
    {
        unsigned int e;
        const size_t pos_in_row = static_cast<size_t>(s) * L.cap + k;
        if (li == 0 && p.pl16)
            e = static_cast<unsigned int>(s + reinterpret_cast<const short *>(L.idx)[pos_in_row]);
        else
            e = L.idx[pos_in_row];
        const int j = static_cast<int>(e & kSlotMask);
        const float4 pj = pos[j];
        const int idj = p.perm[ctl->lbuf][j];
        const bool j_static = (p.flags[ctl->lbuf][j] & PF_STATIC) != 0;
        if (!j_static && idj < idi)
            continue;
        const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (!pair_in(r2, lo2, hi2, pi, pj, cut, term != BS_TERM_STERIC))
            continue;
        const unsigned long long at = atomicAdd(count, 1ull);
        if (at < cap)
        {
            out[2 * at] = min(idi, idj);
            out[2 * at + 1] = max(idi, idj);
        }
    }
    }
}

} // namespace

// Launches a kernel of the rebuild or step chain; with BS_PDL set, with programmatic stream
// serialisation, so that it may start launching while its predecessor runs (it waits in pdl_enter).
template <typename... KArgs, typename... Args>
static void launch_plain(void (*kern)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                         Args &&...args)
{
    kern<<<grid, block, smem, st>>>(std::forward<Args>(args)...);
}

template <typename... KArgs, typename... Args>
static void launch_chain(void (*kern)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                         Args &&...args)
{
#if BS_PDL
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
#else
    kern<<<grid, block, smem, st>>>(std::forward<Args>(args)...);
#endif
}

#if BS_PDL_STEP
#define BS_STEP_LAUNCH launch_chain
#else
#define BS_STEP_LAUNCH launch_plain
#endif

int launch_rebuild(const Params &p, cudaStream_t st)
{
    const int nb = (p.n + kBuildBlock - 1) / kBuildBlock;
    int bb = (p.n + kBboxBlock - 1) / kBboxBlock;
    bb = bb > 304 ? 304 : (bb < 1 ? 1 : bb);
    int launched = 0;
    if (p.nsys > 0)
        launched += launch_batch_grid(p, st);
    else
    {
        const int tiles = p.cell_cap / kScanTile + 1;
        launch_chain(k_bbox, bb, kBboxBlock, 0, st, p);
        launch_chain(k_cell_count, nb, kBuildBlock, 0, st, p);
        launch_chain(k_scan_tiles, tiles, 1024, 0, st, p);
        launch_chain(k_scan_top, 1, 1024, 0, st, p);
        launch_chain(k_scan_add, tiles, 1024, 0, st, p);
        launched += 5;
    }
    launch_chain(k_cell_place, nb, kBuildBlock, 0, st, p);
    launch_chain(k_cell_sort, 1216, kBuildBlock, 0, st, p);
    launch_chain(k_reorder, nb, kBuildBlock, 0, st, p);
    launch_chain(k_spring_ell,
                 static_cast<unsigned>((static_cast<long long>(p.npad) * p.ell_lanes + kBuildBlock - 1) / kBuildBlock),
                 kBuildBlock, 0, st, p);
    launched += 4;
    if (p.nsys > 0 || p.pl_sparse)
        return launched + launch_batch_pairlist(p, st);
    // one block per group of kGridDiv^3 cells (the grid's size is only known on the device: cover
    // the capacity; blocks past the last group return at once, and the kernel strides over groups)
    const int plb = p.cell_cap / (kGridDiv * kGridDiv * kGridDiv) + 1;
    if (p.pl16)
        launch_chain(k_pairlist<true>, plb, kPlWarps * 32, 0, st, p);
    else
        launch_chain(k_pairlist<false>, plb, kPlWarps * 32, 0, st, p);
    return launched + 1;
}

// The lean step kernel leaves out, at compile time, the terms most systems do not use (pairwise
// hydrophobic forces, field grids, the probe, rigid bodies, float-float positions): fewer live
// registers, so the common kernel runs without register spills.
static bool lean_step(const Params &p)
{
    return BS_LEAN && !(p.hydro_on || p.fg_on[0] || p.fg_on[1] || p.probe_on || p.nbody > 0 || p.pos_lo[0]);
}

template <int MODE, int SM>
static void launch_step_lanes(const Params &p, cudaStream_t st)
{
    const long long threads_per = p.step_lanes;
    const int nb = static_cast<int>((static_cast<long long>(p.n) * threads_per + kStepKernelBlock - 1) / kStepKernelBlock);
    const bool lean = lean_step(p);
    switch (p.step_lanes)
    {
    case 2:
        BS_STEP_LAUNCH(k_step<MODE, SM, 2, false>, nb, kStepKernelBlock, 0, st, p);
        break;
    case 8:
        if (lean)
            BS_STEP_LAUNCH(k_step<MODE, SM, 8, true>, nb, kStepKernelBlock, 0, st, p);
        else
            BS_STEP_LAUNCH(k_step<MODE, SM, 8, false>, nb, kStepKernelBlock, 0, st, p);
        break;
    case 16:
        if (lean)
            BS_STEP_LAUNCH(k_step<MODE, SM, 16, true>, nb, kStepKernelBlock, 0, st, p);
        else
            BS_STEP_LAUNCH(k_step<MODE, SM, 16, false>, nb, kStepKernelBlock, 0, st, p);
        break;
    default:
        if (lean)
            BS_STEP_LAUNCH(k_step<MODE, SM, 4, true>, nb, kStepKernelBlock, 0, st, p);
        else
            BS_STEP_LAUNCH(k_step<MODE, SM, 4, false>, nb, kStepKernelBlock, 0, st, p);
        break;
    }
}

// Burying of every particle into the current layout (bs_set_burying), from caller order.
__global__ void k_set_burying(Params p, const float *b)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id < p.n)
        p.bur[p.ctl->lbuf][p.inv[id]] = b[id];
}

int launch_set_burying(const Params &p, const float *b, cudaStream_t st)
{
    k_set_burying<<<(p.n + 255) / 256, 256, 0, st>>>(p, b);
    return 1;
}

// New charges into the current layout (bs_set_charges): the value and the charged flag that
// decides Coulomb list membership (the caller forces a list rebuild before the next step).
__global__ void k_set_charges(Params p, const float *q)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id < p.n)
    {
        const int lb = p.ctl->lbuf, slot = p.inv[id];
        p.chg[lb][slot] = q[id];
        const unsigned int f = p.flags[lb][slot] & ~static_cast<unsigned int>(PF_CHARGED);
        p.flags[lb][slot] = q[id] != 0.0f ? (f | PF_CHARGED) : f;
    }
}

int launch_set_charges(const Params &p, const float *q, cudaStream_t st)
{
    k_set_charges<<<(p.n + 255) / 256, 256, 0, st>>>(p, q);
    return 1;
}

// Adds one particle's external force for the next step and marks it pending (bs_set_force).
__global__ void k_ext_add(Params p, long long i, float fx, float fy, float fz)
{
    p.ext[3 * i] += fx;
    p.ext[3 * i + 1] += fy;
    p.ext[3 * i + 2] += fz;
    p.ctl->ext_pending = 1;
}

int launch_ext_add(const Params &p, long long i, float fx, float fy, float fz, cudaStream_t st)
{
    k_ext_add<<<1, 1, 0, st>>>(p, i, fx, fy, fz);
    return 1;
}

// Frame recorder, after a step (and the bodies and the probe): a frame is due when the step
// count is a multiple of frame_every and its ring slot does not already hold it (a step that did
// not run leaves the count, so the frame is not written twice). k_frame_open marks the slot as
// being written; k_frame writes the positions in caller order straight into the mapped host ring
// (one thread per particle, coalesced), and its last block writes the header after a system-wide
// fence, so a reader that sees the header's sequence number sees the whole frame.
__device__ __forceinline__ bool frame_due(const Params &p, long long &seq, int &slot)
{
    const long long st = *(volatile const long long *)&p.ctl->steps;
    if (st <= 0 || st % p.frame_every != 0)
        return false;
    seq = st / p.frame_every;
    slot = static_cast<int>(seq % p.frame_cap);
    return *(volatile const long long *)&p.frame_hdr[slot].seq != seq;
}

__global__ void k_frame_open(Params p)
{
    pdl_enter();
    long long seq;
    int slot;
    if (!frame_due(p, seq, slot))
        return;
    *(volatile long long *)&p.frame_hdr[slot].seq = -1;
    __threadfence_system();
}

__global__ void __launch_bounds__(256) k_frame(Params p)
{
    pdl_enter();
    long long seq;
    int slot;
    // the header of this slot is -1 while the frame is written: the decision is the same in every
    // block, because only the last block of this launch changes it
    const long long st = *(volatile const long long *)&p.ctl->steps;
    if (st <= 0 || st % p.frame_every != 0)
        return;
    seq = st / p.frame_every;
    slot = static_cast<int>(seq % p.frame_cap);
    if (*(volatile const long long *)&p.frame_hdr[slot].seq != -1)
        return;
    Ctl *ctl = p.ctl;
    const float4 *pos = p.pos[ctl->sbuf];
    float *dst = p.frame_xyz + static_cast<size_t>(slot) * 3 * static_cast<size_t>(p.n);
    for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < p.n; id += gridDim.x * blockDim.x)
    {
        const float4 q = pos[p.inv[id]];
        dst[3 * static_cast<size_t>(id)] = q.x;
        dst[3 * static_cast<size_t>(id) + 1] = q.y;
        dst[3 * static_cast<size_t>(id) + 2] = q.z;
    }
    __threadfence_system();
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0)
        last = atomicAdd(&ctl->done_frame, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last || threadIdx.x != 0)
        return;
    __threadfence_system();
    FrameHeader *h = p.frame_hdr + slot;
    h->step = st;
    for (int k = 0; k < 6; ++k)
        h->energies[k] = ctl->energies[k];
    __threadfence_system();
    *(volatile long long *)&h->seq = seq;
    ctl->done_frame = 0u;
}

int launch_step(const Params &p, int mode, cudaStream_t st)
{
    int launched = launch_step_only(p, mode, st);
    if (mode == MODE_STEP && p.nbody > 0)
        launched += launch_rigid(p, st); // after the step kernel, on the same stream
    if (mode == MODE_STEP && p.probe_on)
    {
        BS_STEP_LAUNCH(k_probe, 1, 1024, 0, st, p);
        launched += 1;
    }
    if (mode == MODE_STEP && p.frame_every > 0)
    {
        BS_STEP_LAUNCH(k_frame_open, 1, 1, 0, st, p);
        BS_STEP_LAUNCH(k_frame, std::min((p.n + 255) / 256, 608), 256, 0, st, p);
        launched += 2;
    }
    return launched;
}

int launch_step_only(const Params &p, int mode, cudaStream_t st)
{
#define BS_STEP_CASE(SMV)                                                                                              \
    case SMV:                                                                                                          \
        if (mode == MODE_STEP)                                                                                         \
            launch_step_lanes<MODE_STEP, SMV>(p, st);                                                                  \
        else                                                                                                           \
            launch_step_lanes<MODE_FORCES, SMV>(p, st);                                                                \
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

int launch_set_positions(const Params &p, const float *xyz, const float *vel, cudaStream_t st, const float *lo)
{
    k_set_state<<<(p.n + 255) / 256, 256, 0, st>>>(p, xyz, vel, lo);
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
