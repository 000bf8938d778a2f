// bs_batch.cu -- batched ensembles: many independent spring networks in one handle.
//
// Layout. The systems' particles are concatenated; every system keeps a fixed, contiguous range
// of slots in every layout, because its cells are numbered after the previous system's cells, so
// the counting sort by cell reorders particles only inside their system. Each system has its own
// search grid (bounding box of its own particles, the single-system formula). Spring partners and
// pair-list partners are always in the same system.
//
// Rebuild: k_batch_bbox (one block per system, then the last block numbers the cells of all
// systems) -> k_batch_cell_count -> k_batch_cell_scan (one block per system) -> the
// single-system place / sort / reorder / spring kernels -> k_batch_pairlist (one warp per home
// particle: systems are sparse, a cell holds a few particles).
//
// Step: k_batch_run, a persistent kernel launched with thread-block clusters. A cluster owns a
// list of whole systems (a host-side longest-processing-time assignment) and runs each of them
// for the period's steps before moving to the next, with one cluster barrier per step; no other
// synchronisation is needed because systems are independent. A system's state stays in L2
// (and L1) across its steps. The per-particle work is the single-system routine
// (particle_step), so a system follows the same arithmetic as when it is stepped alone.
//
// Lists go stale per system: a step whose end positions drift more than half the list skin
// records its index in stale_at[b]; the system stops after that step and resumes after the next
// rebuild. At the end of a launch every system's state is put in the buffer the launch's nominal
// step count implies, so the next rebuild sees one consistent buffer index.

#include <cooperative_groups.h>

#include "bs_device.cuh"

namespace bsg
{
namespace
{

namespace cg = cooperative_groups;

// the batched list build loads a warp's next home while it lists the current one
#ifndef BS_BPL_PREFETCH
#define BS_BPL_PREFETCH 1
#endif
constexpr int kBatchBboxBlock = 256;
constexpr int kBatchPlWarps = 8;
constexpr int kMaxSysCells = 1 << 26; // a system spread wider than this falls back to one cell

// One block per system: bounding box of the system's particles and its grid; the last block to
// finish numbers the cells of all systems and publishes the total as a 1-D grid (gnx = total)
// for the shared place / sort kernels.
__global__ void __launch_bounds__(kBatchBboxBlock) k_batch_bbox(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int b = blockIdx.x;
    const int n0 = p.sys_start[b], n1 = p.sys_start[b + 1];
    const float4 *pos = p.pos[ctl->sbuf];
    float v[6] = {FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX}; // min x,y,z and -max x,y,z
    for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x)
    {
        const float4 q = pos[i];
        v[0] = fminf(v[0], q.x);
        v[1] = fminf(v[1], q.y);
        v[2] = fminf(v[2], q.z);
        v[3] = fminf(v[3], -q.x);
        v[4] = fminf(v[4], -q.y);
        v[5] = fminf(v[5], -q.z);
    }
    __shared__ float sh[6][kBatchBboxBlock / 32];
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
    if (threadIdx.x == 0)
    {
        float mn[3], mx[3];
        bool ok = n1 > n0;
        for (int k = 0; k < 3; ++k)
        {
            float a = sh[k][0], c = sh[3 + k][0];
            for (int w = 1; w < kBatchBboxBlock / 32; ++w)
            {
                a = fminf(a, sh[k][w]);
                c = fminf(c, sh[3 + k][w]);
            }
            mn[k] = a;
            mx[k] = -c;
            ok = ok && isfinite(mn[k]) && isfinite(mx[k]) && mn[k] <= mx[k];
        }
        SysGrid g;
        g.radius = p.list_radius / static_cast<float>(kSparseDiv);
        int nc[3] = {1, 1, 1};
        double gmin[3] = {0.0, 0.0, 0.0};
        double cells = ok ? grid_dims(mn, mx, g.radius, gmin, nc) : 1.0;
        if (!(cells <= static_cast<double>(kMaxSysCells)))
        {
            // one cell holds the whole system: the neighbour walk sees every particle, which
            // gives the same pairs (every candidate is tested against the list radius)
            nc[0] = nc[1] = nc[2] = 1;
            cells = 1.0;
        }
        for (int k = 0; k < 3; ++k)
            g.gmin[k] = gmin[k];
        g.nx = nc[0];
        g.ny = nc[1];
        g.nz = nc[2];
        g.cells = static_cast<int>(cells);
        p.sys_grid[b] = g;
        p.stale_at[b] = LLONG_MAX; // a fresh list
        p.sys_status[b] &= ~ST_STALE;
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
    long long total = 0;
    for (int s = 0; s < p.nsys; ++s)
    {
        p.sys_cells[s] = static_cast<int>(total < INT_MAX ? total : INT_MAX);
        total += __ldcg(&p.sys_grid[s].cells);
    }
    p.sys_cells[p.nsys] = static_cast<int>(total < INT_MAX ? total : INT_MAX);
    if (total > static_cast<long long>(p.cell_cap))
    {
        ctl->ncells_needed = static_cast<int>(total < INT_MAX ? total : INT_MAX);
        atomicOr(&ctl->status, ST_CELL_CAPACITY);
    }
    ctl->gnx = static_cast<int>(total < p.cell_cap ? total : p.cell_cap);
    ctl->gny = 1;
    ctl->gnz = 1;
    atomicAnd(&ctl->status, ~ST_STALE);
    ctl->done_bbox = 0u;
}

__global__ void __launch_bounds__(kBuildBlock) k_batch_cell_count(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n)
        return;
    const int b = p.sys_of[i];
    const SysGrid &g = p.sys_grid[b];
    const float4 q = p.pos[ctl->sbuf][i];
    const int cx = ref_cell_coord(q.x, g.gmin[0], g.radius, g.nx);
    const int cy = ref_cell_coord(q.y, g.gmin[1], g.radius, g.ny);
    const int cz = ref_cell_coord(q.z, g.gmin[2], g.radius, g.nz);
    const int c = p.sys_cells[b] + cx + cy * g.nx + cz * g.nx * g.ny;
    p.cell_of[i] = c;
    atomicAdd(&p.cell_cnt[c], 1);
}

// One block per system: exclusive scan of the system's cell counts, offset by the system's first
// slot; primes the fill cursors and clears the counts for the next rebuild.
__global__ void __launch_bounds__(1024) k_batch_cell_scan(Params p)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int b = blockIdx.x;
    const int c0 = p.sys_cells[b], c1 = p.sys_cells[b + 1];
    const int nc = c1 - c0;
    const int per = (nc + blockDim.x - 1) / blockDim.x;
    const int b0 = c0 + threadIdx.x * per, b1 = min(c1, b0 + per);
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
    int run = p.sys_start[b] + sh[threadIdx.x] - sum;
    for (int c = b0; c < b1; ++c)
    {
        const int k = p.cell_cnt[c];
        p.cell_start[c] = run;
        p.cell_fill[c] = run;
        p.cell_cnt[c] = 0;
        run += k;
    }
    if (threadIdx.x == 0)
        p.cell_start[c1] = p.sys_start[b + 1];
}

// Typed pair lists, one warp per home particle: the rules of the cell-block build (every pair
// within the list radius of its term, the slot itself and spring partners excluded, static
// partners of the steric term apart); the warp walks the (2 kSparseDiv + 1)^2 contiguous x-runs of
// the neighbour cells packed into one sequence of full 32-candidate windows, and a ballot appends
// the accepted ones to the row in run order and ascending slot order within a run. Spring partners
// sit in registers, are located once in the candidate sequence and are excluded by a per-window
// lane mask. Used for batched ensembles (BATCH: each system's own grid) and for
// sparse single systems (a few particles per cell or fewer), where one block per group of cells
// would mostly schedule empty blocks.
template <bool PL16, bool BATCH>
__global__ void __launch_bounds__(kBatchPlWarps * 32) k_batch_pairlist(Params p)
{
    constexpr int kSpan = 2 * kSparseDiv + 1;
    static_assert(kSpan * kSpan <= 32, "one lane per x-run");
    __shared__ int sh_cr[kBatchPlWarps][2 * kSpan * kSpan]; // per warp: the non-empty runs' first slot and first k
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sb = ctl->sbuf, lb = ctl->lbuf;
    const float4 *__restrict__ pos = p.pos[sb];
    const unsigned int *__restrict__ fl = p.flags[lb];
    const float r2_0 = p.pl[0].r2, r2_1 = p.pl[1].r2, r2_2 = p.pl[2].r2;
    const bool l0 = p.pl[0].on, l1 = p.pl[1].on, l2 = p.pl[2].on, l3 = p.pl[3].on;
    const int cap0 = p.pl[0].cap, cap1 = p.pl[1].cap, cap2 = p.pl[2].cap, cap3 = p.pl[3].cap;
    const size_t stride = static_cast<size_t>(p.npad);
    const unsigned int below = (1u << lane) - 1u;
    // Each warp lists homes i, i + istride, ...; the next home's own data (flags, position, cell,
    // system, spring degree) are loaded while the warp lists the current one, so a home's set-up
    // starts one dependent round trip later in its chain.
    const int istride = static_cast<int>(gridDim.x) * kBatchPlWarps;
    int i = static_cast<int>(blockIdx.x) * kBatchPlWarps + wid;
    unsigned int fi_n = 0u;
    float4 pi_n = make_float4(0.f, 0.f, 0.f, 0.f);
    int cell_n = 0, sys_n = 0, deg_n = 0;
    auto fetch = [&](int h) {
        if (h < p.n)
        {
            fi_n = fl[h];
            pi_n = pos[h];
            cell_n = p.cell_of[h];
            if (BATCH)
                sys_n = p.sys_of[h];
            deg_n = p.spring_on ? p.se_deg[h] : 0;
        }
    };
    if (BS_BPL_PREFETCH)
        fetch(i);
    for (; i < p.n; i += istride)
    {
        if (!BS_BPL_PREFETCH)
            fetch(i);
        const unsigned int fi = fi_n;
        const float4 pi = pi_n;
        const int cell_i = cell_n, sys_i = sys_n, deg = deg_n;
        if (BS_BPL_PREFETCH)
            fetch(i + istride);
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
        bool wide = false;
        if (on0 || on1 || on2)
        {
            int cbase = 0, nx = ctl->gnx, ny = ctl->gny, nz = ctl->gnz;
            if (BATCH)
            {
                const int b = sys_i;
                cbase = p.sys_cells[b];
                nx = p.sys_grid[b].nx;
                ny = p.sys_grid[b].ny;
                nz = p.sys_grid[b].nz;
            }
            const int lc = cell_i - cbase;
            const int cx = lc % nx, cy = (lc / nx) % ny, cz = lc / (nx * ny);
            // spring partners of i in registers: lane m holds partners m and m + 32 (slots, -1 for
            // none); a home with more than 64 compares every candidate with its ELL row
            const bool small = deg <= 64;
            const int ps0 = small && lane < deg ? static_cast<int>(p.se_col[static_cast<size_t>(lane) * stride + i] & kSlotMask) : -1;
            const int ps1 =
                small && lane + 32 < deg ? static_cast<int>(p.se_col[static_cast<size_t>(lane + 32) * stride + i] & kSlotMask) : -1;
            short *row0s = reinterpret_cast<short *>(p.pl[0].idx) + static_cast<size_t>(i) * cap0;
            unsigned int *row0 = p.pl[0].idx + static_cast<size_t>(i) * cap0;
            unsigned int *row1 = p.pl[1].idx + static_cast<size_t>(i) * cap1;
            unsigned int *row2 = p.pl[2].idx + static_cast<size_t>(i) * cap2;
            unsigned int *row3 = p.pl[3].idx + static_cast<size_t>(i) * cap3;
            // lane r < kSpan^2 holds run r (cell offsets -kSparseDiv + r % kSpan in y and
            // -kSparseDiv + r / kSpan in z): the contiguous slots of its 2 kSparseDiv + 1 cells in x
            int lo_r = 0, cnt_r = 0;
            if (lane < kSpan * kSpan)
            {
                const int y = cy + lane % kSpan - kSparseDiv;
                const int z = cz + lane / kSpan - kSparseDiv;
                if (y >= 0 && y < ny && z >= 0 && z < nz)
                {
                    const int rowc = cbase + (z * ny + y) * nx;
                    lo_r = p.cell_start[rowc + max(cx - kSparseDiv, 0)];
                    cnt_r = p.cell_start[rowc + min(cx + kSparseDiv, nx - 1) + 1] - lo_r;
                }
            }
            // The runs are walked as one sequence of candidates (k = 0 .. total-1, in run order,
            // hence ascending slots within each run and rows in the order of the run-by-run walk),
            // so that every window but the last is full. Lane c holds the c-th non-empty run: its
            // first slot and its first k.
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
            __syncwarp();
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
            // each spring partner's index in the candidate sequence (-1: not a candidate): the
            // last run whose first slot is <= the partner's, by a binary search over the lanes'
            // runs (runs are contiguous slot ranges)
            int pk0 = -1, pk1 = -1;
            if (deg > 0 && small && total > 0)
            {
                const int s_c = lane < nr ? lo_c : INT_MAX;
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
                const int rr = __popc(__ballot_sync(0xffffffffu, lane < nr && end_c <= wb));
                const int t = pre_c - wb;
                const unsigned int starts =
                    __reduce_or_sync(0xffffffffu, (lane < nr && t > 0 && t < 32) ? (1u << t) : 0u);
                const int rk = min(rr + __popc(starts & ((2u << lane) - 1u)), nr - 1);
                const int lo = __shfl_sync(0xffffffffu, lo_c, rk);
                const int pre = __shfl_sync(0xffffffffu, pre_c, rk);
                const bool jv = k < total;
                const int j = jv ? lo + (k - pre) : lo;
                // the lanes whose candidate is a spring partner, OR-ed over the warp
                unsigned int bonded = 0u;
                if (deg > 0 && small)
                {
                    const int t0 = pk0 < 0 ? -1 : pk0 - wb, t1 = pk1 < 0 ? -1 : pk1 - wb;
                    unsigned int bb = t0 >= 0 && t0 < 32 ? 1u << t0 : 0u;
                    if (t1 >= 0 && t1 < 32)
                        bb |= 1u << t1;
                    bonded = __reduce_or_sync(0xffffffffu, bb);
                }
                const float4 pj = pos[j];
                const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                bool in = jv && r2 < r2max && j != i && !((bonded >> lane) & 1u);
                if (!small)
                    for (int q = 0; q < deg; ++q)
                        in = in && static_cast<int>(p.se_col[static_cast<size_t>(q) * stride + i] & kSlotMask) != j;
                const unsigned int fj = need_fj ? fl[j] : 0u;
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
                            {
                                const int off = j - i;
                                wide = wide || off < -32768 || off > 32767;
                                row0s[at] = static_cast<short>(off);
                            }
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
            }
        }
        if (PL16 && __any_sync(0xffffffffu, wide) && lane == 0)
            atomicOr(&ctl->status, ST_WIDE);
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

// Block sum of NE per-thread energies: FP32 warp trees, float-float over the warps. Thread k < NE
// writes (hi, lo) of energy k to out[2k], out[2k + 1].
template <int NE>
__device__ __forceinline__ void block_energy_partial(const float (&e)[NE], float *out)
{
    __shared__ float shh[NE][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NE; ++k)
    {
        float v = e[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0)
            shh[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < NE)
    {
        float hi = 0.0f, lo = 0.0f;
        for (int w = 0; w < nwarps; ++w)
            ff_add(hi, lo, shh[threadIdx.x][w], 0.0f);
        out[2 * threadIdx.x] = hi;
        out[2 * threadIdx.x + 1] = lo;
    }
    __syncthreads();
}

// The persistent step kernel of a batched ensemble (see the top of the file). `chunk` is the
// nominal number of steps of this launch: every live system runs until it has completed
// ctl->nominal + chunk steps, unless its list goes stale first. chunk = 0 only lets systems that
// fell behind catch up.
template <int SM, int T, bool LEAN>
__global__ void __launch_bounds__(kBatchMaxBlock, 2) k_batch_run(Params p, int chunk)
{
    cg::cluster_group cl = cg::this_cluster();
    const int rank = static_cast<int>(cl.block_rank());
    const int csize = static_cast<int>(cl.num_blocks());
    const int cid = static_cast<int>(blockIdx.x) / csize;
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return; // uniform: the status does not change while this kernel runs
    const int sb0 = ctl->sbuf, lb = ctl->lbuf;
    const long long upto = ctl->nominal + chunk;
    const int out_parity = chunk & 1;
    const int stride = csize * static_cast<int>(blockDim.x);
    const int me = rank * static_cast<int>(blockDim.x) + static_cast<int>(threadIdx.x);
    for (int q = p.cl_start[cid]; q < p.cl_start[cid + 1]; ++q)
    {
        const int b = p.cl_sys[q];
        const int n0 = p.sys_start[b], n1 = p.sys_start[b + 1];
        const long long done = p.sys_steps[b];
        const bool dead = (p.sys_status[b] & ST_NONFINITE) != 0;
        // stale_at[b] < done: the list went stale before this launch (no rebuild since)
        long long stale = p.stale_at[b];
        // every thread of the cluster has read this system's control words before any of them
        // can write them (a step records staleness and non-finite positions)
        cl.sync();
        int k = 0;
        float e[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const int span = (n1 - n0) * T;
        // Loop condition: every thread of the cluster evaluates the same values, because a step
        // only records its own index in stale_at, which is >= done + k for steps not yet waited
        // for at the barrier.
        while (!dead && stale >= done + k && done + k < upto)
        {
            const int sb = sb0 ^ (k & 1);
#pragma unroll
            for (int j = 0; j < 6; ++j)
                e[j] = 0.f;
            int pend = 0;
            for (int g0 = 0; g0 < span; g0 += stride)
            {
                const int g = g0 + me;
                pend |= particle_step<MODE_STEP, SM, T, false, LEAN>(p, n0 + g / T, g % T, n1, sb, lb, false, e);
            }
            if (pend)
            {
                atomicMin(&p.stale_at[b], done + k); // the end positions of step done + k left the skin
                if (pend & ST_NONFINITE)
                    atomicOr(&p.sys_status[b], ST_NONFINITE);
            }
            ++k;
            cl.sync();
            stale = atomicAdd(reinterpret_cast<unsigned long long *>(&p.stale_at[b]), 0ull);
        }
        if (k == 0)
            continue;
        float *part = p.sys_part + (static_cast<size_t>(b) * kMaxCluster + rank) * 16;
        block_energy_partial<6>(e, part);
        if ((k & 1) != out_parity)
        {
            // bring the state into the buffer the launch's nominal step count implies
            const int from = sb0 ^ (k & 1), to = sb0 ^ out_parity;
            for (int s = n0 + me; s < n1; s += stride)
            {
                p.pos[to][s] = p.pos[from][s];
                p.vel[to][s] = p.vel[from][s];
                if (p.pos_lo[0])
                    p.pos_lo[to][s] = p.pos_lo[from][s];
            }
        }
        cl.sync();
        if (rank == 0 && threadIdx.x < 6)
        {
            float hi = 0.0f, lo = 0.0f;
            for (int r = 0; r < csize; ++r)
            {
                const float *pr = p.sys_part + (static_cast<size_t>(b) * kMaxCluster + r) * 16;
                ff_add(hi, lo, __ldcg(pr + 2 * threadIdx.x), __ldcg(pr + 2 * threadIdx.x + 1));
            }
            // e[] order: spring, steric, Coulomb, hydrophobic, IMPALA, kinetic
            const int slot[6] = {BS_ENERGY_SPRING, BS_ENERGY_STERIC, BS_ENERGY_ELECTROSTATIC, BS_ENERGY_HYDROPHOBIC,
                                 BS_ENERGY_IMP, BS_ENERGY_KINETIC};
            p.sys_energy[static_cast<size_t>(b) * 8 + slot[threadIdx.x]] = static_cast<double>(hi) + static_cast<double>(lo);
        }
        if (rank == 0 && threadIdx.x == 0)
            p.sys_steps[b] = done + k;
    }
}

// After a launch of k_batch_run: advances the nominal step count and the buffer index, counts
// systems that fell behind or died, and sums the systems' energies (system order, FP64).
__global__ void __launch_bounds__(256) k_batch_finish(Params p, int chunk)
{
    Ctl *ctl = p.ctl;
    if (status_of(ctl) & kRebuildBlocking)
        return;
    __shared__ int sh_lag, sh_dead;
    if (threadIdx.x == 0)
    {
        sh_lag = 0;
        sh_dead = 0;
    }
    __syncthreads();
    const long long nominal = ctl->nominal + chunk;
    int lag = 0, dead = 0;
    for (int b = threadIdx.x; b < p.nsys; b += blockDim.x)
    {
        if (p.sys_status[b] & ST_NONFINITE)
            ++dead;
        else if (p.sys_steps[b] < nominal)
            ++lag;
    }
    atomicAdd(&sh_lag, lag);
    atomicAdd(&sh_dead, dead);
    __syncthreads();
    if (threadIdx.x < BS_NUM_ENERGIES)
    {
        double s = 0.0;
        for (int b = 0; b < p.nsys; ++b)
            s += p.sys_energy[static_cast<size_t>(b) * 8 + threadIdx.x];
        ctl->energies[threadIdx.x] = s;
    }
    if (threadIdx.x == 0)
    {
        ctl->nominal = nominal;
        ctl->steps = nominal;
        ctl->sbuf ^= chunk & 1;
        ctl->lagging = sh_lag;
        ctl->dead = sh_dead;
        if (sh_dead)
            atomicOr(&ctl->status, ST_NONFINITE);
    }
}

} // namespace

int launch_batch_grid(const Params &p, cudaStream_t st)
{
    k_batch_bbox<<<p.nsys, kBatchBboxBlock, 0, st>>>(p);
    k_batch_cell_count<<<(p.n + kBuildBlock - 1) / kBuildBlock, kBuildBlock, 0, st>>>(p);
    k_batch_cell_scan<<<p.nsys, 1024, 0, st>>>(p);
    return 3;
}

int launch_batch_pairlist(const Params &p, cudaStream_t st)
{
    const long long warps = p.n;
    long long blocks = (warps + kBatchPlWarps - 1) / kBatchPlWarps;
    if (blocks > 152 * 64)
        blocks = 152 * 64;
    if (blocks < 1)
        blocks = 1;
    if (p.nsys > 0)
    {
        if (p.pl16)
            k_batch_pairlist<true, true><<<static_cast<int>(blocks), kBatchPlWarps * 32, 0, st>>>(p);
        else
            k_batch_pairlist<false, true><<<static_cast<int>(blocks), kBatchPlWarps * 32, 0, st>>>(p);
    }
    else if (p.pl16)
        k_batch_pairlist<true, false><<<static_cast<int>(blocks), kBatchPlWarps * 32, 0, st>>>(p);
    else
        k_batch_pairlist<false, false><<<static_cast<int>(blocks), kBatchPlWarps * 32, 0, st>>>(p);
    return 1;
}

template <int SM, int T> static const void *batch_run_fn(bool lean)
{
    return lean ? reinterpret_cast<const void *>(&k_batch_run<SM, T, true>)
                : reinterpret_cast<const void *>(&k_batch_run<SM, T, false>);
}

// The lean instance (no pairwise hydrophobic term, no float-float positions; ensembles have no
// rigid bodies, probe or field grids) keeps fewer registers live under the kernel's 64.
const void *batch_run_kernel(int steric_mode, int lanes, bool lean)
{
#define BS_RUN_CASE(SMV)                                                                                               \
    case SMV:                                                                                                          \
        switch (lanes)                                                                                                 \
        {                                                                                                              \
        case 1:                                                                                                        \
            return batch_run_fn<SMV, 1>(lean);                                                                             \
        case 2:                                                                                                        \
            return batch_run_fn<SMV, 2>(lean);                                                                             \
        case 8:                                                                                                        \
            return batch_run_fn<SMV, 8>(lean);                                                                             \
        default:                                                                                                       \
            return batch_run_fn<SMV, 4>(lean);                                                                             \
        }
    switch (steric_mode)
    {
        BS_RUN_CASE(BS_STERIC_LINEAR)
        BS_RUN_CASE(BS_STERIC_LJ_12_6_AMBER)
        BS_RUN_CASE(BS_STERIC_LJ_8_6_LEWITT)
        BS_RUN_CASE(BS_STERIC_LJ_8_6_ZACHARIAS)
    default:
        return nullptr;
    }
#undef BS_RUN_CASE
}

cudaError_t launch_batch_run(const Params &p, const BatchShape &shape, int chunk, cudaStream_t st)
{
    const void *fn = batch_run_kernel(p.steric_mode, shape.lanes, BS_LEAN && !p.hydro_on && !p.pos_lo[0]);
    if (!fn)
        return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(p.ncl * shape.cluster), 1, 1);
    cfg.blockDim = dim3(static_cast<unsigned>(shape.block), 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(shape.cluster);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void *args[] = {const_cast<Params *>(&p), &chunk};
    return cudaLaunchKernelExC(&cfg, fn, args);
}

int launch_batch_finish(const Params &p, int chunk, cudaStream_t st)
{
    k_batch_finish<<<1, 256, 0, st>>>(p, chunk);
    return 1;
}

cudaError_t batch_max_clusters(const Params &p, const BatchShape &shape, int *out)
{
    const void *fn = batch_run_kernel(p.steric_mode, shape.lanes, BS_LEAN && !p.hydro_on && !p.pos_lo[0]);
    if (!fn)
        return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(shape.cluster), 1, 1);
    cfg.blockDim = dim3(static_cast<unsigned>(shape.block), 1, 1);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(shape.cluster);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaOccupancyMaxActiveClusters(out, fn, &cfg);
}

} // namespace bsg
