// bs_capi.cu -- host side of the C ABI (include/biospring_gb300.h): handle, device buffers,
// CUDA-graph step schedule, error reporting. No torch types, no allocation on the step path.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_set>
#include <vector>

#include "../../include/biospring_gb300.h"
#include "bs_field.h"
#include "bs_nc.h"
#include "bs_kernels.cuh"

using namespace bsg;

namespace
{

thread_local std::string g_last_error;

struct DeviceBuffers
{
    std::vector<void *> owned;
    template <typename T> cudaError_t alloc(T **ptr, size_t count)
    {
        void *p = nullptr;
        const cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess)
        {
            owned.push_back(p);
            *ptr = static_cast<T *>(p);
        }
        return e;
    }
    void free_all()
    {
        for (void *p : owned)
            cudaFree(p);
        owned.clear();
    }
};

} // namespace

struct bs_sim
{
    std::string err;
    cudaStream_t stream = nullptr;
    // host copies (caller order)
    int64_t n = 0;
    std::vector<float> xyz, vel, mass, charge, radius, eps, hydro, sasa, transfer;
    std::vector<uint8_t> is_static, rigid;
    std::vector<int32_t> sp_i, sp_j;
    std::vector<float> sp_r0, sp_k;
    std::unordered_set<uint64_t> sp_seen;
    std::vector<std::vector<int32_t>> bodies;
    // field grids given with bs_set_field_grid (else read from the configured path at set-up)
    struct FieldHost
    {
        bool set = false;
        int shape[3] = {0, 0, 0};
        double origin[3] = {0.0, 0.0, 0.0}, spacing[3] = {1.0, 1.0, 1.0};
        std::vector<float> scalar;
        std::vector<float> cells; // 4 per cell after set-up: scalar, force vector
    } field[2];
    std::vector<float> burying; // caller order; empty: 1 for every particle
    // frame recorder: page-locked host ring the device writes (mapped), next sequence to read
    float *frame_xyz_h = nullptr;
    FrameHeader *frame_hdr_h = nullptr;
    long long frame_next = 1;
    bs_config cfg{};
    bool have_cfg = false;
    bool ready = false;
    // device side
    DeviceBuffers dev;
    Params p{};
    Ctl *ctl_host = nullptr; // pinned mirror
    float *staging = nullptr; // device float[3n]
    float *ext_stage = nullptr; // pinned float[3n]: external forces from pageable caller memory
    int *one_host = nullptr;    // pinned constant 1 (source of the ext_pending flag)
    long long ctl_read_at = -1; // launch count when ctl_host was last read (all work finished)
    int step_blocks = 0;
    // schedule
    bool list_valid = false;
    int since_rebuild = 0;
    long long steps_done = 0;
    long long target = 0; // steps requested since setup
    cudaGraphExec_t period_graph = nullptr;
    int period_kernels = 0;
    long long launches = 0;
    // growable buffers (pair lists, grid arrays), freed on regrowth
    unsigned int *pl_idx[kLists] = {nullptr, nullptr, nullptr, nullptr};
    int *cell_buf[4] = {nullptr, nullptr, nullptr, nullptr};
    // batched ensembles: caller's partition into systems (empty: one system)
    std::vector<int64_t> sys_off;
    BatchShape shape{256, 4, 1};
    int *cl_start_d = nullptr;
    int *cl_sys_d = nullptr;
    // adjoint: directed spring ids of the caller-order CSR, scratch, and the captured run
    std::vector<unsigned int> csr_sid;
    std::vector<int> csr_pos; // CSR position of each spring's two directed entries
    unsigned int *sp_sid_d = nullptr;
    DeviceBuffers adj_dev;
    int adj_ck_cap = 0, adj_seg_cap = 0;
    float *adj_ck_xyz = nullptr, *adj_ck_vel = nullptr, *adj_ck_lo = nullptr;
    float4 *adj_seg = nullptr, *adj_seg_lo = nullptr, *adj_lx = nullptr, *adj_lv = nullptr, *adj_nu[2] = {nullptr, nullptr};
    float4 *adj_cx = nullptr, *adj_cv = nullptr, *adj_target = nullptr;
    float *adj_gk = nullptr, *adj_gr0 = nullptr, *adj_ok = nullptr, *adj_or0 = nullptr;
    double *adj_blk = nullptr, *adj_loss = nullptr;
    unsigned int *adj_done = nullptr;
    cudaGraphExec_t adj_graph = nullptr;
    int adj_key[4] = {0, 0, 0, 0};
    // double membrane: upper offset, lower offset, upper and lower tube curvatures (bs_set_membrane)
    float memb[4] = {0.f, 0.f, 0.f, 0.f};
    float *adj_gq = nullptr; // dL/dq per caller id
    long long adj_kernels = 0;
    // diagnostics scratch
    long long *diag_out = nullptr;
    unsigned long long *diag_count = nullptr;
    size_t diag_cap = 0;
};

namespace
{

int fail(bs_sim *s, int code, const std::string &msg)
{
    if (s)
        s->err = msg;
    g_last_error = msg;
    return code;
}

int cuda_fail(bs_sim *s, cudaError_t e, const char *what)
{
    return fail(s, BS_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define BS_CUDA(call)                                                                                                  \
    do                                                                                                                 \
    {                                                                                                                  \
        const cudaError_t e_ = (call);                                                                                 \
        if (e_ != cudaSuccess)                                                                                         \
            return cuda_fail(s, e_, #call);                                                                            \
    } while (0)

void destroy_graph(bs_sim *s)
{
    if (s->period_graph)
    {
        cudaGraphExecDestroy(s->period_graph);
        s->period_graph = nullptr;
    }
    if (s->adj_graph)
    {
        cudaGraphExecDestroy(s->adj_graph);
        s->adj_graph = nullptr;
    }
}

void free_growable(bs_sim *s);

void free_frames(bs_sim *s)
{
    if (s->frame_xyz_h)
        cudaFreeHost(s->frame_xyz_h);
    if (s->frame_hdr_h)
        cudaFreeHost(s->frame_hdr_h);
    s->frame_xyz_h = nullptr;
    s->frame_hdr_h = nullptr;
    s->p.frame_every = 0;
    s->p.frame_cap = 0;
    s->p.frame_xyz = nullptr;
    s->p.frame_hdr = nullptr;
}

void release_device(bs_sim *s)
{
    destroy_graph(s);
    if (s->stream)
        cudaStreamSynchronize(s->stream);
    free_frames(s);
    free_growable(s);
    s->dev.free_all();
    s->adj_dev.free_all();
    s->adj_gq = nullptr;
    s->adj_ck_cap = 0;
    s->adj_seg_cap = 0;
    s->sp_sid_d = nullptr;
    s->diag_out = nullptr;
    s->diag_count = nullptr;
    s->diag_cap = 0;
    s->staging = nullptr;
    s->cl_start_d = nullptr;
    s->cl_sys_d = nullptr;
    if (s->ctl_host)
    {
        cudaFreeHost(s->ctl_host);
        s->ctl_host = nullptr;
    }
    if (s->ext_stage)
    {
        cudaFreeHost(s->ext_stage);
        s->ext_stage = nullptr;
    }
    if (s->one_host)
    {
        cudaFreeHost(s->one_host);
        s->one_host = nullptr;
    }
    s->ctl_read_at = -1;
    s->ready = false;
}

// Guard band on r^2 around a cutoff c: c (1 -+ 2^-19), squared. The FP32 squared distance of a
// pair is within ~6 * 2^-24 (relative) of the exact one and the reference's float-rounded distance
// within 2^-23 on the square, so outside the band (+-2^-18 on r^2, about ten times wider) the FP32
// value classifies the pair exactly; inside it the FP64 reference test decides.
float band_lo2(double c) { return static_cast<float>((c * (1.0 - 1.0 / 524288.0)) * (c * (1.0 - 1.0 / 524288.0))); }
float band_hi2(double c) { return static_cast<float>((c * (1.0 + 1.0 / 524288.0)) * (c * (1.0 + 1.0 / 524288.0))); }

// Reads the control block back (synchronises the handle's stream).
int read_ctl(bs_sim *s)
{
    BS_CUDA(cudaMemcpyAsync(s->ctl_host, s->p.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s->stream));
    BS_CUDA(cudaStreamSynchronize(s->stream));
    s->ctl_read_at = s->launches;
    return BS_OK;
}

int clear_status(bs_sim *s, int bits)
{
    s->ctl_host->status &= ~bits;
    BS_CUDA(cudaMemcpyAsync(&s->p.ctl->status, &s->ctl_host->status, sizeof(int), cudaMemcpyHostToDevice, s->stream));
    return BS_OK;
}

// Frees the growable buffers (pair lists and grid arrays).
void free_growable(bs_sim *s)
{
    for (int t = 0; t < kLists; ++t)
    {
        if (s->pl_idx[t])
            cudaFree(s->pl_idx[t]);
        s->pl_idx[t] = nullptr;
    }
    for (int k = 0; k < 4; ++k)
    {
        if (s->cell_buf[k])
            cudaFree(s->cell_buf[k]);
        s->cell_buf[k] = nullptr;
    }
}

// (Re)allocates the three pair lists and the cell arrays for the given capacities. The stream
// is idle when this runs (callers synchronise first), so the old buffers can be released.
int alloc_lists(bs_sim *s, const int caps[kLists], int cell_cap)
{
    Params &p = s->p;
    BS_CUDA(cudaStreamSynchronize(s->stream));
    free_growable(s);
    for (int t = 0; t < kLists; ++t)
    {
        // a multiple of 8 entries, so every row starts on a 16-byte boundary (vector loads of the
        // step kernel read 4 entries at a time)
        const int cap = p.pl[t].on ? (std::max(caps[t], 1) + 7) / 8 * 8 : 8;
        BS_CUDA(cudaMalloc(reinterpret_cast<void **>(&s->pl_idx[t]),
                           static_cast<size_t>(p.npad) * cap * sizeof(unsigned int)));
        p.pl[t].idx = s->pl_idx[t];
        p.pl[t].cap = cap;
    }
    for (int k = 0; k < 3; ++k)
        BS_CUDA(cudaMalloc(reinterpret_cast<void **>(&s->cell_buf[k]), (static_cast<size_t>(cell_cap) + 1) * sizeof(int)));
    BS_CUDA(cudaMemsetAsync(s->cell_buf[0], 0, (static_cast<size_t>(cell_cap) + 1) * sizeof(int), s->stream));
    BS_CUDA(cudaMalloc(reinterpret_cast<void **>(&s->cell_buf[3]),
                       (static_cast<size_t>(cell_cap) / kScanTile + 2) * sizeof(int)));
    p.cell_cnt = s->cell_buf[0];
    p.cell_start = s->cell_buf[1];
    p.cell_fill = s->cell_buf[2];
    p.tile_sum = s->cell_buf[3];
    p.cell_cap = cell_cap;
    destroy_graph(s);
    return BS_OK;
}

int current_caps(const bs_sim *s, int caps[kLists])
{
    for (int t = 0; t < kLists; ++t)
        caps[t] = s->p.pl[t].cap;
    return 0;
}

// Runs a rebuild now and repairs capacity overflows until the list is valid.
int rebuild_now(bs_sim *s)
{
    for (int attempt = 0; attempt < 8; ++attempt)
    {
        s->launches += launch_rebuild(s->p, s->stream);
        BS_CUDA(cudaGetLastError());
        int rc = read_ctl(s);
        if (rc)
            return rc;
        const int st = s->ctl_host->status;
        if (st & ST_NONFINITE)
            return fail(s, BS_E_NONFINITE, "non-finite particle position");
        if (st & ST_CELL_CAPACITY)
        {
            const long long need = s->ctl_host->ncells_needed;
            if (need > (1ll << 28))
                return fail(s, BS_E_CAPACITY, "search grid needs more than 2^28 cells (particles spread too far)");
            int caps[kLists];
            current_caps(s, caps);
            rc = alloc_lists(s, caps, static_cast<int>(need + need / 2 + 64));
            if (rc)
                return rc;
            rc = clear_status(s, ST_CELL_CAPACITY);
            if (rc)
                return rc;
            continue;
        }
        if (st & ST_WIDE)
        {
            // a neighbour offset left the 16-bit range: switch the steric list to 32-bit entries
            s->p.pl16 = 0;
            destroy_graph(s);
            rc = clear_status(s, ST_WIDE | ST_PAIR_CAPACITY);
            if (rc)
                return rc;
            continue;
        }
        if (st & ST_PAIR_CAPACITY)
        {
            int caps[kLists];
            current_caps(s, caps);
            for (int t = 0; t < kLists; ++t)
            {
                const int need = s->ctl_host->max_row[t];
                if (need > caps[t])
                    caps[t] = need + need / 8 + 8;
                if (static_cast<double>(caps[t]) * s->p.npad > 2.0e9)
                    return fail(s, BS_E_CAPACITY, "pair list would exceed 2^31 entries");
            }
            rc = alloc_lists(s, caps, s->p.cell_cap);
            if (rc)
                return rc;
            rc = clear_status(s, ST_PAIR_CAPACITY);
            if (rc)
                return rc;
            continue;
        }
        s->list_valid = true;
        s->since_rebuild = 0;
        return BS_OK;
    }
    return fail(s, BS_E_CAPACITY, "pair list or grid did not fit after repeated growth");
}

int capture_period_graph(bs_sim *s)
{
    destroy_graph(s);
    const int K = std::max(1, s->cfg.rebuild_every);
    cudaGraph_t g = nullptr;
    BS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int kernels = launch_rebuild(s->p, s->stream);
    for (int k = 0; k < K; ++k)
        kernels += launch_step(s->p, MODE_STEP, s->stream);
    BS_CUDA(cudaStreamEndCapture(s->stream, &g));
    const cudaError_t e = cudaGraphInstantiate(&s->period_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
        return cuda_fail(s, e, "cudaGraphInstantiate");
    s->period_kernels = kernels;
    return BS_OK;
}

// Assigns whole systems to the clusters of the persistent batched kernel: as many clusters as
// can be resident at once for the current shape, systems in decreasing order of work each given
// to the least-loaded cluster (longest-processing-time rule). Work of a system: its particles plus
// its directed spring entries.
int assign_clusters(bs_sim *s)
{
    Params &p = s->p;
    int maxc = 0;
    BS_CUDA(batch_max_clusters(p, s->shape, &maxc));
    if (maxc < 1)
        return fail(s, BS_E_ARG, "batch shape does not fit on the device (block " + std::to_string(s->shape.block) +
                                     ", cluster " + std::to_string(s->shape.cluster) + ")");
    const int nsys = p.nsys;
    const int ncl = std::max(1, std::min(maxc, nsys));
    std::vector<long long> cost(nsys, 0);
    std::vector<int> deg(s->n, 0);
    for (size_t t = 0; t < s->sp_i.size(); ++t)
    {
        deg[s->sp_i[t]]++;
        deg[s->sp_j[t]]++;
    }
    for (int b = 0; b < nsys; ++b)
        for (int64_t i = s->sys_off[b]; i < s->sys_off[b + 1]; ++i)
            cost[b] += 1 + deg[i];
    std::vector<int> order(nsys);
    for (int b = 0; b < nsys; ++b)
        order[b] = b;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<long long> load(ncl, 0);
    std::vector<std::vector<int>> lists(ncl);
    for (int b : order)
    {
        int best = 0;
        for (int c = 1; c < ncl; ++c)
            if (load[c] < load[best])
                best = c;
        load[best] += cost[b];
        lists[best].push_back(b);
    }
    std::vector<int> start(ncl + 1, 0), sys;
    for (int c = 0; c < ncl; ++c)
    {
        start[c + 1] = start[c] + static_cast<int>(lists[c].size());
        sys.insert(sys.end(), lists[c].begin(), lists[c].end());
    }
    BS_CUDA(cudaMemcpyAsync(s->cl_start_d, start.data(), sizeof(int) * (ncl + 1), cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(s->cl_sys_d, sys.data(), sizeof(int) * nsys, cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaStreamSynchronize(s->stream));
    p.ncl = ncl;
    destroy_graph(s);
    return BS_OK;
}

// One period of a batched ensemble: rebuild, then the persistent kernel for K nominal steps.
int capture_batch_graph(bs_sim *s)
{
    destroy_graph(s);
    const int K = std::max(1, s->cfg.rebuild_every);
    cudaGraph_t g = nullptr;
    BS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int kernels = launch_rebuild(s->p, s->stream);
    const cudaError_t le = launch_batch_run(s->p, s->shape, K, s->stream);
    kernels += 1 + launch_batch_finish(s->p, K, s->stream);
    const cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
    if (le != cudaSuccess)
    {
        if (g)
            cudaGraphDestroy(g);
        return cuda_fail(s, le, "batched step launch");
    }
    if (ce != cudaSuccess)
        return cuda_fail(s, ce, "cudaStreamEndCapture");
    const cudaError_t e = cudaGraphInstantiate(&s->period_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
        return cuda_fail(s, e, "cudaGraphInstantiate");
    s->period_kernels = kernels;
    return BS_OK;
}

// Enqueues `count` nominal steps of a batched ensemble on the rebuild schedule of the single-system
// path; `catchup` first lets systems that stopped on a stale list reach the nominal count.
int enqueue_batch(bs_sim *s, long long count, bool catchup)
{
    const int K = std::max(1, s->cfg.rebuild_every);
    if (catchup)
    {
        s->launches += launch_rebuild(s->p, s->stream);
        BS_CUDA(launch_batch_run(s->p, s->shape, 0, s->stream));
        s->launches += 1 + launch_batch_finish(s->p, 0, s->stream);
        s->list_valid = true;
    }
    long long remaining = count;
    while (remaining > 0)
    {
        if (!s->list_valid || s->since_rebuild >= K)
        {
            if (remaining >= K)
            {
                if (!s->period_graph)
                {
                    const int rc = capture_batch_graph(s);
                    if (rc)
                        return rc;
                }
                BS_CUDA(cudaGraphLaunch(s->period_graph, s->stream));
                s->launches += s->period_kernels;
                s->list_valid = true;
                s->since_rebuild = K;
                remaining -= K;
                continue;
            }
            s->launches += launch_rebuild(s->p, s->stream);
            s->list_valid = true;
            s->since_rebuild = 0;
        }
        const int chunk = static_cast<int>(std::min<long long>(remaining, K - s->since_rebuild));
        BS_CUDA(launch_batch_run(s->p, s->shape, chunk, s->stream));
        s->launches += 1 + launch_batch_finish(s->p, chunk, s->stream);
        s->since_rebuild += chunk;
        remaining -= chunk;
    }
    BS_CUDA(cudaGetLastError());
    return BS_OK;
}

// The double membrane into the step parameters (flat when every value is zero).
void apply_membrane(bs_sim *s)
{
    Params &p = s->p;
    p.imp_off[0] = s->memb[0];
    p.imp_off[1] = -s->memb[1];
    p.imp_curv[0] = s->memb[2];
    p.imp_curv[1] = s->memb[3];
    p.imp_double = (s->memb[0] != 0.f || s->memb[1] != 0.f || s->memb[2] != 0.f || s->memb[3] != 0.f) ? 1 : 0;
}

} // namespace

extern "C" {

int bs_default_config(bs_config *c)
{
    if (!c)
        return fail(nullptr, BS_E_ARG, "bs_default_config: null config");
    std::memset(c, 0, sizeof(*c));
    // configuration::defaultConfiguration() (Configuration.hpp:153-234)
    c->nbsteps = -1;
    c->timestep = 0.01;
    c->neighborskin = 0.0;
    c->steric_enable = 0;
    c->steric_gridscale = 1.0;
    c->steric_cutoff = 1.0;
    c->steric_mode = BS_STERIC_LINEAR;
    c->spring_enable = 0;
    c->spring_scale = 1.0;
    c->hydrophobicity_enable = 0;
    c->hydrophobicity_cutoff = 15.0;
    c->hydrophobicity_scale = 1.0;
    c->coulomb_enable = 0;
    c->coulomb_cutoff = 16.0;
    c->coulomb_scale = 1.0;
    c->coulomb_dielectric = 1.0;
    c->viscosity_enable = 0;
    c->viscosity_value = 1.0;
    c->rigidbody_enable = 0;
    c->impala_enable = 0;
    c->impala_scale = 1.0;
    // device-path knobs
    c->dielectric_mode = BS_DIELECTRIC_CONSTANT;
    c->impala_z0 = 15.75;
    c->impala_alpha = 1.99;
    c->rebuild_every = 10;
    c->list_skin = 1.0;
    c->probe_x = c->probe_y = c->probe_z = 1.0;
    c->probe_mass = 1.0;
    c->probe_epsilon = 1.0;
    c->probe_radius = 1.0;
    c->probe_charge = 0.0;
    c->potentialgrid_scale = 1.0;
    c->densitygrid_scale = 1.0;
    return BS_OK;
}

int bs_create(bs_sim **out)
{
    if (!out)
        return fail(nullptr, BS_E_ARG, "bs_create: null output");
    auto *s = new bs_sim();
    const cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess)
    {
        const int rc = cuda_fail(nullptr, e, "cudaStreamCreate");
        delete s;
        return rc;
    }
    bs_default_config(&s->cfg);
    *out = s;
    return BS_OK;
}

int bs_destroy(bs_sim *s)
{
    if (!s)
        return BS_OK;
    if (s->stream)
        cudaStreamSynchronize(s->stream);
    release_device(s);
    if (s->stream)
        cudaStreamDestroy(s->stream);
    delete s;
    return BS_OK;
}

int bs_upload_particles(bs_sim *s, int64_t n, const float *xyz, const float *vel, const float *mass,
                        const float *charge, const float *radius, const float *epsilon, const float *hydrophobicity,
                        const float *sasa, const float *transfer, const uint8_t *is_static)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->sp_i.empty())
        return fail(s, BS_E_STATE, "SpringNetwork::addParticle: particles must be added before springs");
    if (n < 0 || n > (1ll << 29) || (n > 0 && !xyz))
        return fail(s, BS_E_ARG, "bs_upload_particles: bad particle count or null coordinates");
    auto put = [&](std::vector<float> &v, const float *src, int64_t per, float def) {
        const size_t off = v.size();
        v.resize(off + static_cast<size_t>(n * per), def);
        if (src)
            std::memcpy(v.data() + off, src, sizeof(float) * n * per);
    };
    put(s->xyz, xyz, 3, 0.0f);
    put(s->vel, vel, 3, 0.0f);
    put(s->mass, mass, 1, 1.0f);
    put(s->charge, charge, 1, 0.0f);
    put(s->radius, radius, 1, 1.0f);
    put(s->eps, epsilon, 1, 0.0f);
    put(s->hydro, hydrophobicity, 1, 0.0f);
    put(s->sasa, sasa, 1, 0.0f);
    put(s->transfer, transfer, 1, 0.0f);
    const size_t off = s->is_static.size();
    s->is_static.resize(off + n, 0);
    if (is_static)
        for (int64_t i = 0; i < n; ++i)
            s->is_static[off + i] = is_static[i] ? 1 : 0;
    s->n += n;
    s->rigid.assign(s->n, 0);
    s->ready = false;
    return BS_OK;
}

int bs_upload_springs(bs_sim *s, int64_t ns, const int32_t *ij, const float *equilibrium, const float *stiffness)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (ns < 0 || (ns > 0 && (!ij || !equilibrium || !stiffness)))
        return fail(s, BS_E_ARG, "bs_upload_springs: bad arguments");
    for (int64_t t = 0; t < ns; ++t)
    {
        const int64_t a = ij[2 * t], b = ij[2 * t + 1];
        if (a < 0 || b < 0 || a >= s->n || b >= s->n)
            return fail(s, BS_E_ARG, "SpringNetwork::addSpring: particle index out of range");
        if (a == b)
            return fail(s, BS_E_ARG, "SpringNetwork::addSpring: a spring requires two distinct particles");
    }
    for (int64_t t = 0; t < ns; ++t)
    {
        const uint32_t a = static_cast<uint32_t>(ij[2 * t]), b = static_cast<uint32_t>(ij[2 * t + 1]);
        const uint64_t key = (static_cast<uint64_t>(std::min(a, b)) << 32) | std::max(a, b);
        if (!s->sp_seen.insert(key).second)
            continue; // already bonded: SpringNetwork::addSpring ignores it
        s->sp_i.push_back(static_cast<int32_t>(a));
        s->sp_j.push_back(static_cast<int32_t>(b));
        s->sp_r0.push_back(equilibrium[t]);
        s->sp_k.push_back(stiffness[t]);
    }
    s->ready = false;
    return BS_OK;
}

int bs_set_rigid_bodies(bs_sim *s, int32_t nb, const int32_t *offsets, const int32_t *ids)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (nb < 0 || (nb > 0 && (!offsets || !ids)))
        return fail(s, BS_E_ARG, "bs_set_rigid_bodies: bad arguments");
    std::vector<std::vector<int32_t>> bodies(nb);
    std::vector<uint8_t> seen(s->n, 0);
    for (int32_t b = 0; b < nb; ++b)
    {
        if (offsets[b + 1] <= offsets[b])
            return fail(s, BS_E_ARG, "bs_set_rigid_bodies: every body needs at least one particle");
        for (int32_t t = offsets[b]; t < offsets[b + 1]; ++t)
        {
            const int32_t id = ids[t];
            if (id < 0 || id >= s->n)
                return fail(s, BS_E_ARG, "bs_set_rigid_bodies: particle id out of range");
            if (seen[id])
                return fail(s, BS_E_ARG, "bs_set_rigid_bodies: a particle belongs to two bodies");
            if (s->is_static[id])
                return fail(s, BS_E_ARG, "bs_set_rigid_bodies: a static particle cannot belong to a rigid body");
            seen[id] = 1;
            bodies[b].push_back(id);
        }
    }
    s->bodies = bodies;
    s->ready = false;
    return BS_OK;
}

int bs_load_nc(bs_sim *s, const char *path, int64_t *n_particles, int64_t *n_springs)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!path)
        return fail(s, BS_E_ARG, "bs_load_nc: null path");
    bsg::NcTopology t;
    std::string msg;
    if (!bsg::read_topology_nc(path, t, msg))
        return fail(s, BS_E_ARG, "NetCDFReader: " + msg);
    auto opt = [](const std::vector<float> &v) { return v.empty() ? nullptr : v.data(); };
    int rc = bs_upload_particles(s, t.n, t.xyz.data(), nullptr, t.mass.data(), t.charge.data(), t.radius.data(),
                                 t.epsilon.data(), opt(t.hydrophobicity), opt(t.sasa), opt(t.transfer),
                                 t.is_static.data());
    if (rc)
        return rc;
    const int64_t m = static_cast<int64_t>(t.r0.size());
    rc = bs_upload_springs(s, m, t.ij.data(), t.r0.data(), t.k.data());
    if (rc)
        return rc;
    if (n_particles)
        *n_particles = t.n;
    if (n_springs)
        *n_springs = m;
    return BS_OK;
}

int bs_set_frames(bs_sim *s, int32_t every, int32_t capacity)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "bs_set_frames: call bs_setup first");
    if (s->p.nsys > 0)
        return fail(s, BS_E_STATE, "bs_set_frames: frames are recorded for single systems");
    if (every < 0 || (every > 0 && capacity < 1))
        return fail(s, BS_E_ARG, "bs_set_frames: every >= 0 and capacity >= 1 are required");
    int rc = bs_synchronize(s); // no queued step may still write the old ring
    if (rc)
        return rc;
    destroy_graph(s);
    free_frames(s);
    if (every == 0)
        return BS_OK;
    const size_t n3 = 3 * static_cast<size_t>(s->n);
    BS_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&s->frame_xyz_h), sizeof(float) * n3 * capacity,
                          cudaHostAllocMapped));
    BS_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&s->frame_hdr_h), sizeof(FrameHeader) * capacity,
                          cudaHostAllocMapped));
    for (int32_t k = 0; k < capacity; ++k)
    {
        s->frame_hdr_h[k].seq = -2; // never a sequence number, nor "being written"
        s->frame_hdr_h[k].step = 0;
    }
    Params &p = s->p;
    BS_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void **>(&p.frame_xyz), s->frame_xyz_h, 0));
    BS_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void **>(&p.frame_hdr), s->frame_hdr_h, 0));
    p.frame_every = every;
    p.frame_cap = capacity;
    s->frame_next = s->steps_done / every + 1; // the first frame still to come
    return BS_OK;
}

int bs_read_frames(bs_sim *s, int32_t max, int64_t *steps, float *xyz, double *energies, int32_t *count,
                   int64_t *dropped)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!count || max < 0)
        return fail(s, BS_E_ARG, "bs_read_frames: bad arguments");
    *count = 0;
    if (dropped)
        *dropped = 0;
    if (s->p.frame_every == 0)
        return fail(s, BS_E_STATE, "bs_read_frames: no frames are recorded (bs_set_frames)");
    const size_t n3 = 3 * static_cast<size_t>(s->n);
    const int cap = s->p.frame_cap;
    int32_t got = 0;
    int64_t lost = 0;
    while (got < max)
    {
        const long long want = s->frame_next;
        FrameHeader *h = s->frame_hdr_h + want % cap;
        // a sequence lock: the device sets seq to -1 before it rewrites a slot and to the frame's
        // number after the frame is complete
        const long long seq1 = __atomic_load_n(&h->seq, __ATOMIC_ACQUIRE);
        if (seq1 == want)
        {
            const long long st = h->step;
            double e[6];
            for (int k = 0; k < 6; ++k)
                e[k] = h->energies[k];
            if (xyz)
                std::memcpy(xyz + static_cast<size_t>(got) * n3, s->frame_xyz_h + static_cast<size_t>(want % cap) * n3,
                            sizeof(float) * n3);
            std::atomic_thread_fence(std::memory_order_acquire);
            if (__atomic_load_n(&h->seq, __ATOMIC_RELAXED) != seq1)
            {
                ++lost; // overwritten while it was copied
                ++s->frame_next;
                continue;
            }
            if (steps)
                steps[got] = st;
            if (energies)
                for (int k = 0; k < 6; ++k)
                    energies[static_cast<size_t>(got) * 6 + k] = e[k];
            ++got;
            ++s->frame_next;
        }
        else if (seq1 > want)
        {
            ++lost; // the ring went round before this frame was read
            ++s->frame_next;
        }
        else
            break; // not written yet (or being written)
    }
    *count = got;
    if (dropped)
        *dropped = lost;
    return BS_OK;
}

int bs_set_field_grid(bs_sim *s, int32_t which, const int32_t shape[3], const double origin[3],
                      const double spacing[3], const float *scalar)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if ((which != BS_GRID_POTENTIAL && which != BS_GRID_DENSITY) || !shape || !origin || !spacing || !scalar)
        return fail(s, BS_E_ARG, "bs_set_field_grid: bad arguments");
    size_t cells = 1;
    for (int a = 0; a < 3; ++a)
    {
        if (shape[a] < 1 || !(spacing[a] > 0.0) || !std::isfinite(spacing[a]) || !std::isfinite(origin[a]))
            return fail(s, BS_E_ARG, "bs_set_field_grid: shape >= 1, spacing > 0 and a finite origin are required");
        cells *= static_cast<size_t>(shape[a]);
    }
    // the reference re-derives the shape from the box (GridCoordinatesSystem.hpp:180-191)
    const long counts[3] = {shape[0], shape[1], shape[2]};
    int derived[3];
    bsg::field_shape(counts, origin, spacing, derived);
    if (derived[0] != shape[0] || derived[1] != shape[1] || derived[2] != shape[2])
        return fail(s, BS_E_ARG, "bs_set_field_grid: the box origin + shape * spacing rounds to another shape");
    auto &f = s->field[which];
    f.set = true;
    for (int a = 0; a < 3; ++a)
    {
        f.shape[a] = shape[a];
        f.origin[a] = origin[a];
        f.spacing[a] = spacing[a];
    }
    f.scalar.assign(scalar, scalar + cells);
    s->ready = false;
    return BS_OK;
}

int bs_get_field_grid(bs_sim *s, int32_t which, int32_t shape[3], float *out)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if ((which != BS_GRID_POTENTIAL && which != BS_GRID_DENSITY) || !shape)
        return fail(s, BS_E_ARG, "bs_get_field_grid: bad arguments");
    if (!s->ready || s->field[which].cells.empty())
        return fail(s, BS_E_STATE, "bs_get_field_grid: no such grid in the current set-up");
    for (int a = 0; a < 3; ++a)
        shape[a] = s->field[which].shape[a];
    if (out)
        std::memcpy(out, s->field[which].cells.data(), sizeof(float) * s->field[which].cells.size());
    return BS_OK;
}

int bs_set_membrane(bs_sim *s, float upper_offset, float lower_offset, float upper_curvature,
                    float lower_curvature)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!std::isfinite(upper_offset) || !std::isfinite(lower_offset) || !std::isfinite(upper_curvature) ||
        !std::isfinite(lower_curvature))
        return fail(s, BS_E_ARG, "bs_set_membrane: offsets and curvatures must be finite");
    BS_CUDA(cudaStreamSynchronize(s->stream)); // no step in flight uses the old parameters
    s->memb[0] = upper_offset;
    s->memb[1] = lower_offset;
    s->memb[2] = upper_curvature;
    s->memb[3] = lower_curvature;
    apply_membrane(s);
    destroy_graph(s); // the captured periods hold the old parameters
    return BS_OK;
}

int bs_set_burying(bs_sim *s, const float *burying)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!burying)
        return fail(s, BS_E_ARG, "bs_set_burying: null argument");
    s->burying.assign(burying, burying + s->n);
    if (s->ready && s->p.bur[0])
    {
        // into the current layout, in stream order
        BS_CUDA(cudaStreamSynchronize(s->stream));
        BS_CUDA(cudaMemcpyAsync(s->staging, burying, sizeof(float) * s->n, cudaMemcpyHostToDevice, s->stream));
        s->launches += launch_set_burying(s->p, s->staging, s->stream);
        BS_CUDA(cudaStreamSynchronize(s->stream));
    }
    return BS_OK;
}

int bs_set_charges(bs_sim *s, const float *charge)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!charge)
        return fail(s, BS_E_ARG, "bs_set_charges: null argument");
    for (int64_t i = 0; i < s->n; ++i)
        if (!std::isfinite(charge[i]))
            return fail(s, BS_E_ARG, "bs_set_charges: charges must be finite");
    s->charge.assign(charge, charge + s->n);
    if (s->ready)
    {
        // into the current layout, in stream order; Coulomb list membership follows the new
        // charges from the next rebuild on, which the next step forces
        BS_CUDA(cudaStreamSynchronize(s->stream));
        BS_CUDA(cudaMemcpyAsync(s->staging, charge, sizeof(float) * s->n, cudaMemcpyHostToDevice, s->stream));
        s->launches += launch_set_charges(s->p, s->staging, s->stream);
        BS_CUDA(cudaStreamSynchronize(s->stream));
        s->list_valid = false;
    }
    return BS_OK;
}

int bs_setup(bs_sim *s, const bs_config *cfg)
{
    if (!s || !cfg)
        return fail(s, BS_E_ARG, "bs_setup: null argument");
    const bs_config &c = *cfg;
    // Validation as in SpringNetwork::_setupSteric/_setupElectrostatic/_setupHydrophobic
    // (SpringNetwork.cpp:663-737) and NeighborSearchBase (nsearch.hpp:61-68).
    if (c.steric_enable && c.steric_cutoff < 1e-6)
        return fail(s, BS_E_ARG, "Steric cutoff must be > 0");
    if (c.coulomb_enable && c.coulomb_cutoff < 1e-6)
        return fail(s, BS_E_ARG, "Electrostatic cutoff must be > 0");
    if (c.hydrophobicity_enable && c.hydrophobicity_cutoff < 1e-6)
        return fail(s, BS_E_ARG, "Hydrophobic cutoff must be > 0");
    if (c.steric_enable && s->n == 0)
        return fail(s, BS_E_ARG, "the particle list is empty");
    if (c.steric_mode < BS_STERIC_LINEAR || c.steric_mode > BS_STERIC_LJ_8_6_ZACHARIAS)
        return fail(s, BS_E_ARG, "steric.mode: invalid choice");
    if (c.dielectric_mode != BS_DIELECTRIC_CONSTANT && c.dielectric_mode != BS_DIELECTRIC_DISTANCE)
        return fail(s, BS_E_ARG, "cuda.dielectricmode: invalid choice");
    if (c.rebuild_every < 1)
        return fail(s, BS_E_ARG, "cuda.rebuildevery must be >= 1");
    if (!(c.list_skin >= 0.0))
        return fail(s, BS_E_ARG, "cuda.listskin must be >= 0");
    if (s->n == 0)
        return fail(s, BS_E_ARG, "bs_setup: no particles");
    const bool batch = !s->sys_off.empty();
    int max_sys = static_cast<int>(s->n);
    if (batch)
    {
        if (s->sys_off.back() != s->n)
            return fail(s, BS_E_ARG, "bs_set_systems: the offsets must end at the particle count");
        if (!s->bodies.empty())
            return fail(s, BS_E_ARG, "rigid bodies are not available for batched ensembles");
        if (c.probe_enable)
            return fail(s, BS_E_ARG, "the probe is not available for batched ensembles");
        if (c.potentialgrid_enable || c.densitygrid_enable)
            return fail(s, BS_E_ARG, "field grids are not available for batched ensembles");
        std::vector<int> sys_of_id(s->n);
        max_sys = 0;
        for (size_t b = 0; b + 1 < s->sys_off.size(); ++b)
        {
            max_sys = std::max(max_sys, static_cast<int>(s->sys_off[b + 1] - s->sys_off[b]));
            for (int64_t i = s->sys_off[b]; i < s->sys_off[b + 1]; ++i)
                sys_of_id[i] = static_cast<int>(b);
        }
        for (size_t t = 0; t < s->sp_i.size(); ++t)
            if (sys_of_id[s->sp_i[t]] != sys_of_id[s->sp_j[t]])
                return fail(s, BS_E_ARG, "a spring joins particles of two systems of the batch");
    }

    release_device(s);
    s->cfg = c;
    s->have_cfg = true;
    const int64_t n = s->n;
    Params &p = s->p;
    p = Params{};
    p.n = static_cast<int>(n);
    p.npad = static_cast<int>((n + 31) / 32 * 32);
    const int npad = p.npad;

    // ---- rigid bodies (RigidBodiesManager::InitRigidBodies, RigidBodiesManager.cpp:11-43):
    // members are rigid only when rigidbody.enable is set ----
    const bool bodies_on = c.rigidbody_enable && !s->bodies.empty();
    s->rigid.assign(n, 0);
    if (bodies_on)
        for (const auto &body : s->bodies)
            for (int32_t id : body)
                s->rigid[id] = 1;

    // ---- spring CSR in caller order (both directions) ----
    std::vector<int> deg(n, 0);
    for (size_t t = 0; t < s->sp_i.size(); ++t)
    {
        deg[s->sp_i[t]]++;
        deg[s->sp_j[t]]++;
    }
    std::vector<int> row(n + 1, 0);
    for (int64_t i = 0; i < n; ++i)
        row[i + 1] = row[i] + deg[i];
    const int nnz = row[n];
    std::vector<unsigned int> col(std::max(nnz, 1));
    std::vector<float> kk(std::max(nnz, 1)), rr(std::max(nnz, 1));
    std::vector<int> fillp(row.begin(), row.end() - 1);
    s->csr_sid.assign(std::max(nnz, 1), 0u);
    s->csr_pos.assign(2 * s->sp_i.size(), 0);
    auto partner_code = [&](int a, int b) {
        uint32_t code = static_cast<uint32_t>(b);
        if (s->is_static[b])
            code |= kEntryStatic;
        if (s->rigid[a] && s->rigid[b])
            code |= kEntryInactive;
        return code;
    };
    for (size_t t = 0; t < s->sp_i.size(); ++t)
    {
        const int a = s->sp_i[t], b = s->sp_j[t];
        int e = fillp[a]++;
        col[e] = partner_code(a, b);
        kk[e] = s->sp_k[t];
        rr[e] = s->sp_r0[t];
        s->csr_sid[e] = static_cast<unsigned int>(2 * t);
        s->csr_pos[2 * t] = e;
        e = fillp[b]++;
        col[e] = partner_code(b, a);
        kk[e] = s->sp_k[t];
        rr[e] = s->sp_r0[t];
        s->csr_sid[e] = static_cast<unsigned int>(2 * t + 1);
        s->csr_pos[2 * t + 1] = e;
    }
    int maxdeg = 1;
    for (int64_t i = 0; i < n; ++i)
        maxdeg = std::max(maxdeg, deg[i]);
    p.sp_maxdeg = maxdeg;
    // Spring-table rebuild: kBuildLanes threads per slot overlap a slot's partner lookups, but
    // their column-major stores do not coalesce, which only L2 absorbs; a table well beyond L2
    // (large batches) is rebuilt one thread per slot, with each column stored contiguously.
    const double ell_bytes = static_cast<double>(npad) * maxdeg * 12.0;
    p.ell_lanes = ell_bytes > 48.0e6 ? 1 : kBuildLanes;

    // ---- per-particle packed parameters ----
    // Steric factors: eps_ij r_ij^m = (a_i b_i^m)(a_j b_j^m) with eps_ij = a_i a_j, r_ij = b_i b_j
    // (CombinationRules.hpp:18-31); P = a b^6 rides in pos.w, fhi = a b^12 (Amber) or a b^8.
    std::vector<float4> pos0(npad), vel0(npad), iprm0(npad);
    std::vector<float> fhi0(npad, 0.f), chg0(npad, 0.f), hyd0(npad, 0.f);
    std::vector<unsigned int> flags0(npad, PF_STATIC);
    for (int64_t i = 0; i < n; ++i)
    {
        double P = s->radius[i], F = 0.0;
        const double eps = s->eps[i], rad = s->radius[i];
        if (c.steric_mode == BS_STERIC_LJ_12_6_AMBER || c.steric_mode == BS_STERIC_LJ_8_6_LEWITT)
        {
            // a = sqrt(eps), b = sqrt(r): P = a b^6 = sqrt(eps) r^3, fhi = a b^12 or a b^8
            P = std::sqrt(eps) * rad * rad * rad;
            F = std::sqrt(eps) * std::pow(rad, c.steric_mode == BS_STERIC_LJ_12_6_AMBER ? 6 : 4);
        }
        else if (c.steric_mode == BS_STERIC_LJ_8_6_ZACHARIAS)
        {
            P = eps * std::pow(rad, 6);
            F = eps * std::pow(rad, 8);
        }
        pos0[i] = make_float4(s->xyz[3 * i], s->xyz[3 * i + 1], s->xyz[3 * i + 2], static_cast<float>(P));
        vel0[i] = make_float4(s->vel[3 * i], s->vel[3 * i + 1], s->vel[3 * i + 2], 0.f);
        fhi0[i] = static_cast<float>(F);
        chg0[i] = s->charge[i];
        hyd0[i] = s->hydro[i];
        unsigned int flags = 0;
        if (s->is_static[i])
            flags |= PF_STATIC;
        if (s->charge[i] != 0.0f)
            flags |= PF_CHARGED;
        if (s->hydro[i] != 0.0f)
            flags |= PF_HYDROPHOBIC;
        if (s->rigid[i])
            flags |= PF_RIGID;
        flags0[i] = flags;
        iprm0[i] = make_float4(s->mass[i], s->sasa[i], s->transfer[i], 0.f);
    }
    p.lj_uniform = n > 0 ? 1 : 0;
    for (int64_t i = 1; i < n && p.lj_uniform; ++i)
        if (fhi0[i] != fhi0[0])
            p.lj_uniform = 0;
    p.lj_F = n > 0 ? fhi0[0] : 0.0f;
    std::vector<int> perm0(npad, 0), inv0(n);
    for (int64_t i = 0; i < n; ++i)
    {
        perm0[i] = static_cast<int>(i);
        inv0[i] = static_cast<int>(i);
    }

    // ---- device allocation ----
    for (int b = 0; b < 2; ++b)
    {
        // one slot past the particles (a position far from everything, LJ factor zero), read by
        // the step kernel for list entries past a row's end (no per-pair test of the row end)
        BS_CUDA(s->dev.alloc(&p.pos[b], npad + 32));
        BS_CUDA(s->dev.alloc(&p.vel[b], npad));
        BS_CUDA(s->dev.alloc(&p.fhi[b], npad + 32));
        BS_CUDA(cudaMemsetAsync(p.fhi[b] + npad, 0, sizeof(float) * 32, s->stream));
        BS_CUDA(s->dev.alloc(&p.chg[b], npad));
        BS_CUDA(s->dev.alloc(&p.hyd[b], npad));
        BS_CUDA(s->dev.alloc(&p.flags[b], npad));
        BS_CUDA(s->dev.alloc(&p.iprm[b], npad));
        BS_CUDA(s->dev.alloc(&p.perm[b], npad));
    }
    BS_CUDA(s->dev.alloc(&p.inv, n));
    BS_CUDA(s->dev.alloc(&p.pos_build, npad));
    if (c.precise_positions)
        for (int b = 0; b < 2; ++b)
        {
            BS_CUDA(s->dev.alloc(&p.pos_lo[b], npad));
            BS_CUDA(cudaMemsetAsync(p.pos_lo[b], 0, sizeof(float4) * npad, s->stream));
        }
    BS_CUDA(s->dev.alloc(&p.ext, 3 * static_cast<size_t>(n)));
    BS_CUDA(s->dev.alloc(&p.force_out, n));
    int *d_row;
    unsigned int *d_col;
    float *d_k, *d_r0;
    BS_CUDA(s->dev.alloc(&d_row, n + 1));
    BS_CUDA(s->dev.alloc(&d_col, std::max(nnz, 1)));
    BS_CUDA(s->dev.alloc(&d_k, std::max(nnz, 1)));
    BS_CUDA(s->dev.alloc(&d_r0, std::max(nnz, 1)));
    p.sp_row = d_row;
    p.sp_col = d_col;
    p.sp_k = d_k;
    p.sp_r0 = d_r0;
    BS_CUDA(s->dev.alloc(&p.se_col, static_cast<size_t>(npad) * maxdeg));
    BS_CUDA(s->dev.alloc(&p.se_k, static_cast<size_t>(npad) * maxdeg));
    BS_CUDA(s->dev.alloc(&p.se_r0, static_cast<size_t>(npad) * maxdeg));
    BS_CUDA(s->dev.alloc(&p.se_deg, npad));
    for (int t = 0; t < kLists; ++t)
        BS_CUDA(s->dev.alloc(&p.pl[t].cnt, npad));
    BS_CUDA(s->dev.alloc(&p.cell_of, npad));
    BS_CUDA(s->dev.alloc(&p.tmp_key, npad));
    s->step_blocks = static_cast<int>((static_cast<long long>(p.n) * 16 + kStepBlock - 1) / kStepBlock);
    p.blk_cap = s->step_blocks;
    BS_CUDA(s->dev.alloc(&p.blk_energy, energy_scratch_doubles(s->step_blocks)));
    BS_CUDA(cudaMemsetAsync(p.blk_energy, 0, sizeof(double) * energy_scratch_doubles(s->step_blocks), s->stream));
    BS_CUDA(s->dev.alloc(&p.ctl, 1));
    BS_CUDA(s->dev.alloc(&s->staging, 3 * static_cast<size_t>(n)));
    BS_CUDA(cudaMallocHost(reinterpret_cast<void **>(&s->ctl_host), sizeof(Ctl)));
    BS_CUDA(cudaMallocHost(reinterpret_cast<void **>(&s->ext_stage), sizeof(float) * 3 * n));
    BS_CUDA(cudaMallocHost(reinterpret_cast<void **>(&s->one_host), sizeof(int)));
    *s->one_host = 1;

    // ---- pair lists: which terms, radii, first capacities from the density ----
    const double skin = c.list_skin;
    bool any_static = false;
    for (int64_t i = 0; i < n; ++i)
        any_static = any_static || s->is_static[i];
    const double cut[kLists] = {c.steric_cutoff, c.coulomb_cutoff, c.hydrophobicity_cutoff, c.steric_cutoff};
    const int on[kLists] = {c.steric_enable != 0, c.coulomb_enable != 0, c.hydrophobicity_enable != 0,
                            c.steric_enable != 0 && any_static};
    double list_radius = 1e-3;
    p.pl16 = 1;
    for (int t = 0; t < kLists; ++t)
    {
        p.pl[t].on = on[t];
        const double R = static_cast<float>(cut[t]) + skin;
        p.pl[t].r2 = static_cast<float>(R * R * (1.0 + 1e-5));
        if (on[t])
            list_radius = std::max(list_radius, R);
    }
    if (!(on[0] || on[1] || on[2] || on[3]))
        list_radius = 1.0e4; // no nonbonded term: a grid of a few cells keeps the rebuild trivial
    p.list_radius = static_cast<float>(list_radius);
    // grid cells and density from the bounding box of each system (one system unless batched)
    const int nsys = batch ? static_cast<int>(s->sys_off.size() - 1) : 1;
    // cells of the list radius (warp-per-particle build, batches) and of a kGridDiv-th of it
    // (cell-block build)
    double cells1 = 0.0, cells_div = 0.0, density = 0.0;
    for (int b = 0; b < nsys; ++b)
    {
        const int64_t i0 = batch ? s->sys_off[b] : 0, i1 = batch ? s->sys_off[b + 1] : n;
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int64_t i = i0; i < i1; ++i)
            for (int k = 0; k < 3; ++k)
            {
                lo[k] = std::min(lo[k], static_cast<double>(s->xyz[3 * i + k]));
                hi[k] = std::max(hi[k], static_cast<double>(s->xyz[3 * i + k]));
            }
        double c1 = 1.0, cd = 1.0, volume = 1.0;
        for (int k = 0; k < 3; ++k)
        {
            c1 *= std::ceil((hi[k] - lo[k]) / (list_radius / kSparseDiv)) + 3.0;
            cd *= std::ceil((hi[k] - lo[k]) / (list_radius / kGridDiv)) + 3.0;
            volume *= std::max(hi[k] - lo[k], 1.0);
        }
        cells1 += c1;
        cells_div += cd;
        density = std::max(density, static_cast<double>(i1 - i0) / volume);
    }
    // fewer than ~8 particles per cell of the list radius: one warp per particle builds the lists
    // faster than one block per (mostly empty) group of cells
    p.pl_sparse = static_cast<double>(n) < 8.0 * cells1 ? 1 : 0;
    const double cells = batch || p.pl_sparse ? cells1 : cells_div;
    const int cell_cap = static_cast<int>(std::min(2.0 * cells + 1024.0, 2.0e8));
    // first capacity: 1.5x the mean count expected in the list sphere, at least 32
    int caps[kLists];
    for (int t = 0; t < kLists; ++t)
    {
        const double R = static_cast<float>(cut[t]) + skin;
        const double expect = density * 4.18879 * R * R * R;
        caps[t] = static_cast<int>(std::min(std::max(1.5 * expect + 16.0, 32.0), 4096.0));
    }
    if (batch && max_sys > 32768)
        p.pl16 = 0; // offsets inside a system would not fit 16 bits
    int rc = alloc_lists(s, caps, cell_cap);
    if (rc)
        return rc;
    if (batch)
    {
        p.nsys = nsys;
        std::vector<int> start(nsys + 1), of(npad, 0);
        for (int b = 0; b <= nsys; ++b)
            start[b] = static_cast<int>(s->sys_off[b]);
        for (int b = 0; b < nsys; ++b)
            for (int i = start[b]; i < start[b + 1]; ++i)
                of[i] = b;
        int *d_start, *d_of;
        BS_CUDA(s->dev.alloc(&d_start, nsys + 1));
        BS_CUDA(s->dev.alloc(&d_of, npad));
        p.sys_start = d_start;
        p.sys_of = d_of;
        BS_CUDA(s->dev.alloc(&p.sys_grid, nsys));
        BS_CUDA(s->dev.alloc(&p.sys_cells, nsys + 1));
        BS_CUDA(s->dev.alloc(&p.sys_status, nsys));
        BS_CUDA(s->dev.alloc(&p.sys_steps, nsys));
        BS_CUDA(s->dev.alloc(&p.stale_at, nsys));
        BS_CUDA(s->dev.alloc(&p.sys_energy, static_cast<size_t>(nsys) * 8));
        BS_CUDA(s->dev.alloc(&p.sys_part, static_cast<size_t>(nsys) * kMaxCluster * 16));
        BS_CUDA(s->dev.alloc(&s->cl_start_d, nsys + 1));
        BS_CUDA(s->dev.alloc(&s->cl_sys_d, nsys));
        p.cl_start = s->cl_start_d;
        p.cl_sys = s->cl_sys_d;
        BS_CUDA(cudaMemcpyAsync(d_start, start.data(), sizeof(int) * (nsys + 1), cudaMemcpyHostToDevice, s->stream));
        BS_CUDA(cudaMemcpyAsync(d_of, of.data(), sizeof(int) * npad, cudaMemcpyHostToDevice, s->stream));
        BS_CUDA(cudaMemsetAsync(p.sys_status, 0, sizeof(int) * nsys, s->stream));
        BS_CUDA(cudaMemsetAsync(p.sys_steps, 0, sizeof(long long) * nsys, s->stream));
        BS_CUDA(cudaMemsetAsync(p.sys_energy, 0, sizeof(double) * nsys * 8, s->stream));
        BS_CUDA(cudaMemsetAsync(p.stale_at, 0x7f, sizeof(long long) * nsys, s->stream));
    }

    // ---- uploads ----
    BS_CUDA(cudaMemcpyAsync(p.pos[0], pos0.data(), sizeof(float4) * npad, cudaMemcpyHostToDevice, s->stream));
    {
        static const float4 far_slot = make_float4(1.0e30f, 1.0e30f, 1.0e30f, 0.0f);
        for (int b = 0; b < 2; ++b)
            BS_CUDA(cudaMemcpyAsync(p.pos[b] + npad, &far_slot, sizeof(float4), cudaMemcpyHostToDevice, s->stream));
    }
    BS_CUDA(cudaMemcpyAsync(p.vel[0], vel0.data(), sizeof(float4) * npad, cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(p.fhi[0], fhi0.data(), sizeof(float) * npad, cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(p.chg[0], chg0.data(), sizeof(float) * npad, cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(p.hyd[0], hyd0.data(), sizeof(float) * npad, cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(p.flags[0], flags0.data(), sizeof(unsigned int) * npad, cudaMemcpyHostToDevice,
                            s->stream));
    BS_CUDA(cudaMemcpyAsync(p.iprm[0], iprm0.data(), sizeof(float4) * npad, cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(p.perm[0], perm0.data(), sizeof(int) * npad, cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(p.inv, inv0.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(d_row, row.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(d_col, col.data(), sizeof(int) * std::max(nnz, 1), cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(d_k, kk.data(), sizeof(float) * std::max(nnz, 1), cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(d_r0, rr.data(), sizeof(float) * std::max(nnz, 1), cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemsetAsync(p.ext, 0, sizeof(float) * 3 * n, s->stream));
    BS_CUDA(cudaMemsetAsync(p.force_out, 0, sizeof(float4) * n, s->stream));
    // ---- field grids (SpringNetwork::_setupElectrostatic / _setupDensityGrid,
    // SpringNetwork.cpp:712-747): the potential map acts when coulomb.enable is set too ----
    for (int g = 0; g < 2; ++g)
    {
        auto &f = s->field[g];
        f.cells.clear();
        const bool on = g == 0 ? (c.potentialgrid_enable && c.coulomb_enable) : c.densitygrid_enable != 0;
        if (!on)
            continue;
        if (!f.set)
        {
            const char *path = g == 0 ? c.potentialgrid_path : c.densitygrid_path;
            std::string msg;
            std::vector<float> v;
            int sh[3];
            if (!path[0])
                return fail(s, BS_E_ARG, std::string(g == 0 ? "potentialgrid" : "densitygrid") +
                                             ".enable: no grid (give a path or call bs_set_field_grid)");
            if (!bsg::read_dx(path, sh, f.origin, f.spacing, &v, msg))
                return fail(s, BS_E_ARG, msg);
            for (int a = 0; a < 3; ++a)
                f.shape[a] = sh[a];
            f.scalar = v;
        }
        const size_t ncell = f.scalar.size();
        f.cells.resize(4 * ncell);
        bsg::field_cells(f.shape, f.spacing, f.scalar.data(), f.cells.data());
        float4 *d = nullptr;
        BS_CUDA(s->dev.alloc(&d, std::max<size_t>(ncell, 1)));
        BS_CUDA(cudaMemcpyAsync(d, f.cells.data(), sizeof(float) * 4 * ncell, cudaMemcpyHostToDevice, s->stream));
        p.fgrid[g] = d;
        p.fg_on[g] = 1;
        p.fg_scale[g] = static_cast<float>(g == 0 ? c.potentialgrid_scale : c.densitygrid_scale);
        for (int a = 0; a < 3; ++a)
        {
            p.fg_n[g][a] = f.shape[a];
            p.fg_o[g][a] = f.origin[a];
            p.fg_h[g][a] = f.spacing[a];
            p.fg_of[g][a] = static_cast<float>(f.origin[a]);
            p.fg_ih[g][a] = static_cast<float>(1.0 / f.spacing[a]);
            // in-grid test min <= x <= max - 1e-6 in double (GridCoordinatesSystem.hpp:206-218), for a
            // float x: the smallest float >= min and the largest float <= max - 1e-6
            const double lo = f.origin[a];
            const double hi = (f.origin[a] + static_cast<double>(f.shape[a]) * f.spacing[a]) - 1e-6;
            float flo = static_cast<float>(lo), fhi = static_cast<float>(hi);
            if (static_cast<double>(flo) < lo)
                flo = std::nextafter(flo, INFINITY);
            if (static_cast<double>(fhi) > hi)
                fhi = std::nextafter(fhi, -INFINITY);
            p.fg_lo[g][a] = flo;
            p.fg_hi[g][a] = fhi;
        }
        if (g == 1)
        {
            std::vector<float> b0(npad, 1.0f);
            if (!s->burying.empty())
                std::copy(s->burying.begin(), s->burying.end(), b0.begin());
            for (int b = 0; b < 2; ++b)
                BS_CUDA(s->dev.alloc(&p.bur[b], npad));
            BS_CUDA(cudaMemcpyAsync(p.bur[0], b0.data(), sizeof(float) * npad, cudaMemcpyHostToDevice, s->stream));
            BS_CUDA(cudaStreamSynchronize(s->stream)); // b0 is a local
        }
    }
    std::memset(s->ctl_host, 0, sizeof(Ctl));
    for (int k = 0; k < 3; ++k)
    {
        s->ctl_host->bbox_enc[k] = 0xffffffffu;
        s->ctl_host->bbox_enc[3 + k] = 0u;
    }
    // ---- probe (SpringNetwork::_setupProbe, SpringNetwork.cpp:749-766): steric factors as a
    // particle's, state in the control block ----
    if (c.probe_enable)
    {
        const double eps = static_cast<float>(c.probe_epsilon), rad = static_cast<float>(c.probe_radius);
        double P = rad, F = 0.0;
        if (c.steric_mode == BS_STERIC_LJ_12_6_AMBER || c.steric_mode == BS_STERIC_LJ_8_6_LEWITT)
        {
            P = std::sqrt(eps) * rad * rad * rad;
            F = std::sqrt(eps) * std::pow(rad, c.steric_mode == BS_STERIC_LJ_12_6_AMBER ? 6 : 4);
        }
        else if (c.steric_mode == BS_STERIC_LJ_8_6_ZACHARIAS)
        {
            P = eps * std::pow(rad, 6);
            F = eps * std::pow(rad, 8);
        }
        p.probe_on = 1;
        p.probe_steric = c.probe_steric != 0;
        p.probe_elec = c.probe_electrostatic != 0;
        p.probe_P = static_cast<float>(P);
        p.probe_F = static_cast<float>(F);
        p.probe_q = static_cast<float>(c.probe_charge);
        p.probe_mass = static_cast<float>(c.probe_mass);
        BS_CUDA(s->dev.alloc(&p.probe_f, npad));
        BS_CUDA(cudaMemsetAsync(p.probe_f, 0, sizeof(float4) * npad, s->stream));
        s->ctl_host->probe_pos = make_float4(static_cast<float>(c.probe_x), static_cast<float>(c.probe_y),
                                             static_cast<float>(c.probe_z), 0.f);
    }
    BS_CUDA(cudaMemcpyAsync(p.ctl, s->ctl_host, sizeof(Ctl), cudaMemcpyHostToDevice, s->stream));

    // ---- rigid-body state (RigidBody.cpp:57-123): total mass (FP64 sum), mass-weighted
    // barycentre and member offsets in float, sphere inertia 2/5 M (radius 1) ----
    if (bodies_on)
    {
        const int nb = static_cast<int>(s->bodies.size());
        std::vector<BodyState> bs(nb);
        std::vector<int> start(nb + 1, 0), ids;
        std::vector<float4> p0;
        for (int b = 0; b < nb; ++b)
        {
            const auto &mem = s->bodies[b];
            double m = 0.0;
            for (int32_t i : mem)
                m += s->mass[i];
            float bx = 0.f, by = 0.f, bz = 0.f;
            double tm = 0.0;
            for (int32_t i : mem)
            {
                bx = bx + s->xyz[3 * i] * s->mass[i];
                by = by + s->xyz[3 * i + 1] * s->mass[i];
                bz = bz + s->xyz[3 * i + 2] * s->mass[i];
                tm = tm + s->mass[i];
            }
            const float inv_tm = static_cast<float>(1.0 / tm);
            bx = bx * inv_tm;
            by = by * inv_tm;
            bz = bz * inv_tm;
            BodyState st{};
            st.pos = make_float4(bx, by, bz, 0.f);
            st.vel = make_float4(0.f, 0.f, 0.f, 0.f);
            st.L = make_float4(0.f, 0.f, 0.f, 0.f);
            st.q = make_float4(0.f, 0.f, 0.f, 1.f);
            st.mass = m;
            st.ibodyinv = 1.0 / ((2.0 / 5.0) * m * 1.0 * 1.0);
            bs[b] = st;
            for (int32_t i : mem)
            {
                ids.push_back(i);
                p0.push_back(make_float4(s->xyz[3 * i] - bx, s->xyz[3 * i + 1] - by, s->xyz[3 * i + 2] - bz, 0.f));
            }
            start[b + 1] = static_cast<int>(ids.size());
        }
        int *d_start, *d_ids;
        float4 *d_p0;
        BS_CUDA(s->dev.alloc(&p.body, nb));
        BS_CUDA(s->dev.alloc(&d_start, nb + 1));
        BS_CUDA(s->dev.alloc(&d_ids, ids.size()));
        BS_CUDA(s->dev.alloc(&d_p0, p0.size()));
        BS_CUDA(s->dev.alloc(&p.rforce, npad));
        BS_CUDA(cudaMemcpyAsync(p.body, bs.data(), sizeof(BodyState) * nb, cudaMemcpyHostToDevice, s->stream));
        BS_CUDA(cudaMemcpyAsync(d_start, start.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, s->stream));
        BS_CUDA(cudaMemcpyAsync(d_ids, ids.data(), sizeof(int) * ids.size(), cudaMemcpyHostToDevice, s->stream));
        BS_CUDA(cudaMemcpyAsync(d_p0, p0.data(), sizeof(float4) * p0.size(), cudaMemcpyHostToDevice, s->stream));
        BS_CUDA(cudaMemsetAsync(p.rforce, 0, sizeof(float4) * npad, s->stream));
        p.body_start = d_start;
        p.body_ids = d_ids;
        p.body_p0 = d_p0;
        p.nbody = nb;
    }

    // ---- step parameters ----
    p.dt = static_cast<float>(c.timestep);
    p.spring_on = c.spring_enable != 0;
    p.steric_on = c.steric_enable != 0;
    p.coulomb_on = c.coulomb_enable != 0;
    p.hydro_on = c.hydrophobicity_enable != 0;
    p.imp_on = c.impala_enable != 0;
    p.visc_on = c.viscosity_enable != 0;
    p.steric_mode = c.steric_mode;
    // lanes per particle: the fewest of 4, 8, 16 that still give the GPU some 64-80k threads
    // (measured: 4 lanes from 20k particles, 8 from 8k, 16 below); BS_STEP_LANES overrides
    p.step_lanes = n >= 20000 ? 4 : (n >= 8000 ? 8 : 16);
    if (const char *env = std::getenv("BS_STEP_LANES"))
    {
        const int v = std::atoi(env);
        if (v == 2 || v == 4 || v == 8 || v == 16)
            p.step_lanes = v;
    }
    p.dielectric_mode = c.dielectric_mode;
    p.c_steric = static_cast<float>(c.steric_cutoff);
    p.c_coulomb = static_cast<float>(c.coulomb_cutoff);
    p.c_hydro = static_cast<float>(c.hydrophobicity_cutoff);
    p.lo2_s = band_lo2(p.c_steric);
    p.hi2_s = band_hi2(p.c_steric);
    p.lo2_c = band_lo2(p.c_coulomb);
    p.hi2_c = band_hi2(p.c_coulomb);
    p.lo2_h = band_lo2(p.c_hydro);
    p.hi2_h = band_hi2(p.c_hydro);
    const double hs = 0.5 * c.list_skin * (1.0 - 1e-5);
    p.half_skin2 = static_cast<float>(hs * hs);
    p.spring_scale = static_cast<float>(c.spring_scale);
    p.steric_scale = static_cast<float>(c.steric_gridscale);
    p.coulomb_scale = static_cast<float>(c.coulomb_scale);
    p.hydro_scale = static_cast<float>(c.hydrophobicity_scale);
    p.imp_scale = static_cast<float>(c.impala_scale);
    p.visc = static_cast<float>(c.viscosity_value);
    p.imp_z0 = static_cast<float>(c.impala_z0);
    p.imp_alpha = static_cast<float>(c.impala_alpha);
    apply_membrane(s);
    const double D = static_cast<float>(c.coulomb_dielectric);
    const double cs = static_cast<float>(c.coulomb_scale);
    p.k_spring_f = static_cast<float>(kSpringForceConvert);
    p.k_elec_e = static_cast<float>(kCoulombEnergyPerA * cs / D);
    p.k_elec_f = static_cast<float>(kElecForceConvert / (4.0 * kPi) * cs / D);
    p.k_kin = static_cast<float>(kKineticConvert);
    p.k_imp_f = static_cast<float>(kImpForceConvert);
    p.k_hydro_e = static_cast<float>(kAvogadro * 1.0E-3);

    s->ready = true;
    s->steps_done = 0;
    s->target = 0;
    s->list_valid = false;
    if (batch)
    {
        rc = assign_clusters(s);
        if (rc)
        {
            s->ready = false;
            return rc;
        }
    }
    rc = rebuild_now(s);
    if (rc)
    {
        s->ready = false;
        return rc;
    }
    return BS_OK;
}

// Enqueues `count` steps following the rebuild schedule (a rebuild every K steps, or when
// the list is invalid); aligned periods go out as one captured graph.
static int enqueue_steps(bs_sim *s, long long count)
{
    const int K = std::max(1, s->cfg.rebuild_every);
    long long remaining = count;
    while (remaining > 0)
    {
        if (!s->list_valid || s->since_rebuild >= K)
        {
            if (remaining >= K)
            {
                if (!s->period_graph)
                {
                    const int rc = capture_period_graph(s);
                    if (rc)
                        return rc;
                }
                BS_CUDA(cudaGraphLaunch(s->period_graph, s->stream));
                s->launches += s->period_kernels;
                s->list_valid = true;
                s->since_rebuild = K;
                remaining -= K;
                continue;
            }
            s->launches += launch_rebuild(s->p, s->stream);
            s->list_valid = true;
            s->since_rebuild = 0;
        }
        const long long chunk = std::min<long long>(remaining, K - s->since_rebuild);
        for (long long k = 0; k < chunk; ++k)
            s->launches += launch_step(s->p, MODE_STEP, s->stream);
        s->since_rebuild += static_cast<int>(chunk);
        remaining -= chunk;
    }
    BS_CUDA(cudaGetLastError());
    return BS_OK;
}

int bs_step_async(bs_sim *s, int32_t nsteps)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "bs_step: call bs_setup first");
    if (nsteps < 0)
        return fail(s, BS_E_ARG, "bs_step: negative step count");
    s->target += nsteps;
    int rc = BS_OK;
    if (s->p.nsys > 0)
        return enqueue_batch(s, nsteps, false);
    return enqueue_steps(s, nsteps);
}

// Completes the queued work of a batched ensemble: repairs capacity overflows, lets systems
// stopped by a stale list catch up, and reports the first system with a non-finite position.
static int synchronize_batch(bs_sim *s)
{
    for (int round = 0; round < 64; ++round)
    {
        int rc = read_ctl(s);
        if (rc)
            return rc;
        const Ctl &h = *s->ctl_host;
        s->steps_done = h.nominal;
        if (h.status & ST_NONFINITE)
        {
            std::vector<int> st(s->p.nsys);
            BS_CUDA(cudaMemcpy(st.data(), s->p.sys_status, sizeof(int) * st.size(), cudaMemcpyDeviceToHost));
            int first = -1;
            for (size_t b = 0; b < st.size() && first < 0; ++b)
                if (st[b] & ST_NONFINITE)
                    first = static_cast<int>(b);
            return fail(s, BS_E_NONFINITE,
                        "Found non-finite position in system " + std::to_string(first) + " of the batch");
        }
        if (h.status & (ST_CELL_CAPACITY | ST_PAIR_CAPACITY | ST_WIDE))
        {
            rc = rebuild_now(s);
            if (rc)
                return rc;
            continue;
        }
        if (h.nominal < s->target)
        {
            rc = enqueue_batch(s, s->target - h.nominal, false);
            if (rc)
                return rc;
            continue;
        }
        if (h.lagging > 0)
        {
            rc = enqueue_batch(s, 0, true);
            if (rc)
                return rc;
            continue;
        }
        return BS_OK;
    }
    return fail(s, BS_E_STATE, "bs_synchronize: the batch could not complete the requested steps");
}

int bs_synchronize(bs_sim *s)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    if (s->p.nsys > 0)
        return synchronize_batch(s);
    for (int round = 0; round < 64; ++round)
    {
        int rc = read_ctl(s);
        if (rc)
            return rc;
        const Ctl &h = *s->ctl_host;
        s->steps_done = h.steps;
        if (h.status & ST_NONFINITE)
            return fail(s, BS_E_NONFINITE, "Found non-finite position (a particle position became NaN or infinite)");
        if (h.status & (ST_CELL_CAPACITY | ST_PAIR_CAPACITY | ST_WIDE))
        {
            rc = rebuild_now(s); // grows the lists and rebuilds
            if (rc)
                return rc;
        }
        else if (h.status & ST_STALE)
            s->list_valid = false; // the next rebuild clears the bit
        if (s->steps_done >= s->target)
            return BS_OK;
        rc = enqueue_steps(s, s->target - s->steps_done);
        if (rc)
            return rc;
    }
    return fail(s, BS_E_STATE, "bs_synchronize: could not complete the requested steps");
}

int bs_step(bs_sim *s, int32_t nsteps)
{
    const int rc = bs_step_async(s, nsteps);
    return rc ? rc : bs_synchronize(s);
}

int bs_get_step_count(bs_sim *s, int64_t *steps)
{
    if (!s || !steps)
        return fail(s, BS_E_ARG, "bs_get_step_count: null argument");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    const int rc = read_ctl(s);
    if (rc)
        return rc;
    *steps = s->ctl_host->steps;
    return BS_OK;
}

int bs_get_stream(bs_sim *s, void **stream)
{
    if (!s || !stream)
        return fail(s, BS_E_ARG, "bs_get_stream: null argument");
    *stream = static_cast<void *>(s->stream);
    return BS_OK;
}

int bs_launch_phase(bs_sim *s, int32_t phase)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    if (phase == 0)
    {
        s->launches += launch_rebuild(s->p, s->stream);
        s->list_valid = true;
        s->since_rebuild = 0;
    }
    else if (phase == 1)
    {
        s->launches += launch_step(s->p, MODE_STEP, s->stream);
        s->target += 1;
        s->since_rebuild += 1;
    }
    else
        return fail(s, BS_E_ARG, "bs_launch_phase: phase must be 0 or 1");
    BS_CUDA(cudaGetLastError());
    return BS_OK;
}

static int set_external_forces(bs_sim *s, const float *f, bool wait);

int bs_set_external_forces(bs_sim *s, const float *f)
{
    return set_external_forces(s, f, true);
}

int bs_set_external_forces_async(bs_sim *s, const float *f)
{
    return set_external_forces(s, f, false);
}

static int set_external_forces(bs_sim *s, const float *f, bool wait)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    if (s->p.nsys > 0)
        return fail(s, BS_E_STATE, "external forces are not available for batched ensembles");
    if (!f)
        return fail(s, BS_E_ARG, "bs_set_external_forces: null forces");
    // Copied in stream order after the enqueued steps: straight from the caller's buffer when it
    // is page-locked, else through the handle's pinned staging buffer. With wait (or a pageable
    // buffer) the call returns when the copy is done, so the caller may reuse f.
    const size_t bytes = sizeof(float) * 3 * static_cast<size_t>(s->n);
    cudaPointerAttributes attr{};
    const bool pinned = cudaPointerGetAttributes(&attr, f) == cudaSuccess && attr.type == cudaMemoryTypeHost;
    if (!pinned)
    {
        cudaGetLastError(); // clear a pageable-pointer query error, if any
        BS_CUDA(cudaStreamSynchronize(s->stream)); // the staging buffer may still feed an earlier copy
        std::memcpy(s->ext_stage, f, bytes);
    }
    BS_CUDA(cudaMemcpyAsync(s->p.ext, pinned ? f : s->ext_stage, bytes, cudaMemcpyHostToDevice, s->stream));
    BS_CUDA(cudaMemcpyAsync(&s->p.ctl->ext_pending, s->one_host, sizeof(int), cudaMemcpyHostToDevice, s->stream));
    if (wait || !pinned)
        BS_CUDA(cudaStreamSynchronize(s->stream));
    return BS_OK;
}

// Completes steps enqueued with bs_step_async before the state is read or replaced.
static int settle(bs_sim *s)
{
    return s->target > s->steps_done ? bs_synchronize(s) : BS_OK;
}

int bs_compute_forces(bs_sim *s)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "bs_compute_forces: call bs_setup first");
    int rc = settle(s);
    if (rc)
        return rc;
    if (!s->list_valid || (s->ctl_host->status & ST_STALE))
    {
        rc = rebuild_now(s);
        if (rc)
            return rc;
    }
    s->launches += launch_step(s->p, MODE_FORCES, s->stream);
    BS_CUDA(cudaGetLastError());
    rc = read_ctl(s);
    if (rc)
        return rc;
    if (s->ctl_host->status & ~ST_STALE)
        return fail(s, BS_E_STATE, "bs_compute_forces: device status not clean");
    return BS_OK;
}

static int get_vec(bs_sim *s, int what, float *out)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    if (!out)
        return fail(s, BS_E_ARG, "null output");
    const int rc = settle(s);
    if (rc)
        return rc;
    s->launches += launch_unsort(s->p, what, s->staging, s->stream);
    BS_CUDA(cudaGetLastError());
    BS_CUDA(cudaMemcpyAsync(out, s->staging, sizeof(float) * 3 * s->n, cudaMemcpyDeviceToHost, s->stream));
    BS_CUDA(cudaStreamSynchronize(s->stream));
    return BS_OK;
}

int bs_get_positions(bs_sim *s, float *xyz) { return get_vec(s, 0, xyz); }
int bs_get_velocities(bs_sim *s, float *v) { return get_vec(s, 1, v); }
int bs_get_forces(bs_sim *s, float *f) { return get_vec(s, 2, f); }

static int set_state(bs_sim *s, const float *xyz, const float *vel)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    const float *src = xyz ? xyz : vel;
    if (!src)
        return fail(s, BS_E_ARG, "null input");
    const int rc = settle(s);
    if (rc)
        return rc;
    BS_CUDA(cudaMemcpyAsync(s->staging, src, sizeof(float) * 3 * s->n, cudaMemcpyHostToDevice, s->stream));
    s->launches += launch_set_positions(s->p, xyz ? s->staging : nullptr, xyz ? nullptr : s->staging, s->stream);
    BS_CUDA(cudaGetLastError());
    BS_CUDA(cudaStreamSynchronize(s->stream));
    if (xyz)
        s->list_valid = false;
    return BS_OK;
}

int bs_set_positions(bs_sim *s, const float *xyz) { return set_state(s, xyz, nullptr); }
int bs_set_velocities(bs_sim *s, const float *vel) { return set_state(s, nullptr, vel); }

int bs_set_force(bs_sim *s, int64_t i, const float f[3])
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    if (s->p.nsys > 0)
        return fail(s, BS_E_STATE, "external forces are not available for batched ensembles");
    if (i < 0 || i >= s->n || !f)
        return fail(s, BS_E_ARG, "bs_set_force: particle index out of range");
    // added on the device in stream order: applies to the next step (after any enqueued ones)
    s->launches += launch_ext_add(s->p, i, f[0], f[1], f[2], s->stream);
    BS_CUDA(cudaGetLastError());
    return BS_OK;
}

int bs_get_energies(bs_sim *s, double out[BS_NUM_ENERGIES])
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    const int rc = settle(s);
    if (rc)
        return rc;
    // the energies change only in kernels: if none was launched since the last full read of the
    // control block (which waited for all enqueued work), its copy is current
    if (s->ctl_read_at != s->launches)
    {
        BS_CUDA(cudaMemcpyAsync(s->ctl_host->energies, s->p.ctl->energies, sizeof(double) * BS_NUM_ENERGIES,
                                cudaMemcpyDeviceToHost, s->stream));
        BS_CUDA(cudaStreamSynchronize(s->stream));
    }
    for (int k = 0; k < BS_NUM_ENERGIES; ++k)
        out[k] = s->ctl_host->energies[k];
    return BS_OK;
}

int bs_get_pairs(bs_sim *s, int32_t term, int64_t *out, int64_t cap, int64_t *n_out)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    if (term < BS_TERM_STERIC || term > BS_TERM_HYDROPHOBIC || cap < 0 || !n_out || (cap > 0 && !out))
        return fail(s, BS_E_ARG, "bs_get_pairs: bad arguments");
    if (s->p.nsys > 0)
        return fail(s, BS_E_STATE, "pair and cell diagnostics are for single systems");
    {
        const int rc = settle(s);
        if (rc)
            return rc;
    }
    if (!s->list_valid || (s->ctl_host->status & ST_STALE))
    {
        const int rc = rebuild_now(s);
        if (rc)
            return rc;
    }
    // Diagnostic scratch, sized on demand (diagnostics are not on the step path).
    const size_t want = static_cast<size_t>(std::max<int64_t>(cap, 1));
    if (s->diag_cap < want)
    {
        BS_CUDA(s->dev.alloc(&s->diag_out, 2 * want));
        s->diag_cap = want;
    }
    if (!s->diag_count)
        BS_CUDA(s->dev.alloc(&s->diag_count, 1));
    BS_CUDA(cudaMemsetAsync(s->diag_count, 0, sizeof(unsigned long long), s->stream));
    s->launches += launch_diag_pairs(s->p, term, s->diag_out, s->diag_count, static_cast<unsigned long long>(cap),
                                     s->stream);
    BS_CUDA(cudaGetLastError());
    unsigned long long count = 0;
    BS_CUDA(cudaMemcpyAsync(&count, s->diag_count, sizeof(count), cudaMemcpyDeviceToHost, s->stream));
    BS_CUDA(cudaStreamSynchronize(s->stream));
    const int64_t w = std::min<int64_t>(static_cast<int64_t>(count), cap);
    if (w > 0)
    {
        BS_CUDA(cudaMemcpy(out, s->diag_out, sizeof(int64_t) * 2 * w, cudaMemcpyDeviceToHost));
        // sort by (i, j): the device emits in slot order
        std::vector<std::pair<int64_t, int64_t>> v(w);
        for (int64_t t = 0; t < w; ++t)
            v[t] = {out[2 * t], out[2 * t + 1]};
        std::sort(v.begin(), v.end());
        for (int64_t t = 0; t < w; ++t)
        {
            out[2 * t] = v[t].first;
            out[2 * t + 1] = v[t].second;
        }
    }
    *n_out = static_cast<int64_t>(count);
    return BS_OK;
}

int bs_get_cells(bs_sim *s, int32_t term, int64_t *out)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    if (term < BS_TERM_STERIC || term > BS_TERM_HYDROPHOBIC || !out)
        return fail(s, BS_E_ARG, "bs_get_cells: bad arguments");
    if (s->p.nsys > 0)
        return fail(s, BS_E_STATE, "pair and cell diagnostics are for single systems");
    {
        const int rc = settle(s);
        if (rc)
            return rc;
    }
    const bs_config &c = s->cfg;
    float cutoff = static_cast<float>(c.steric_cutoff);
    uint32_t need = 0;
    bool on = c.steric_enable != 0;
    if (term == BS_TERM_COULOMB)
    {
        cutoff = static_cast<float>(c.coulomb_cutoff);
        need = PF_CHARGED;
        on = c.coulomb_enable != 0;
    }
    else if (term == BS_TERM_HYDROPHOBIC)
    {
        cutoff = static_cast<float>(c.hydrophobicity_cutoff);
        need = PF_HYDROPHOBIC;
        on = c.hydrophobicity_enable != 0;
    }
    if (!on)
    {
        for (int64_t i = 0; i < s->n; ++i)
            out[i] = -1;
        return BS_OK;
    }
    long long *d_out = nullptr;
    if (s->diag_cap < static_cast<size_t>(s->n))
    {
        BS_CUDA(s->dev.alloc(&s->diag_out, 2 * static_cast<size_t>(s->n)));
        s->diag_cap = static_cast<size_t>(s->n);
    }
    d_out = s->diag_out;
    s->launches += launch_diag_cells(s->p, cutoff, static_cast<float>(c.neighborskin), need, d_out, s->stream);
    BS_CUDA(cudaGetLastError());
    BS_CUDA(cudaMemcpyAsync(out, d_out, sizeof(int64_t) * s->n, cudaMemcpyDeviceToHost, s->stream));
    BS_CUDA(cudaStreamSynchronize(s->stream));
    return BS_OK;
}

int bs_set_systems(bs_sim *s, int32_t nsys, const int64_t *offsets)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (nsys < 0 || (nsys > 0 && !offsets))
        return fail(s, BS_E_ARG, "bs_set_systems: bad arguments");
    if (nsys == 0)
    {
        s->sys_off.clear();
        s->ready = false;
        return BS_OK;
    }
    if (offsets[0] != 0)
        return fail(s, BS_E_ARG, "bs_set_systems: the first offset must be 0");
    for (int32_t b = 0; b < nsys; ++b)
        if (offsets[b + 1] <= offsets[b])
            return fail(s, BS_E_ARG, "bs_set_systems: every system needs at least one particle");
    s->sys_off.assign(offsets, offsets + nsys + 1);
    s->ready = false;
    return BS_OK;
}

int bs_set_batch_shape(bs_sim *s, int32_t block, int32_t lanes, int32_t cluster)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!(block == 128 || block == 256 || block == 512) || !(lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8) ||
        !(cluster == 1 || cluster == 2 || cluster == 4 || cluster == 8))
        return fail(s, BS_E_ARG, "bs_set_batch_shape: block in {128, 256, 512}, lanes in {1, 2, 4, 8}, cluster in {1, 2, 4, 8}");
    const BatchShape old = s->shape;
    s->shape = BatchShape{block, lanes, cluster};
    if (s->ready && s->p.nsys > 0)
    {
        int rc = bs_synchronize(s);
        if (rc == BS_OK)
            rc = assign_clusters(s);
        if (rc)
        {
            s->shape = old;
            return rc;
        }
    }
    return BS_OK;
}

int bs_get_batch_shape(bs_sim *s, int32_t shape[3])
{
    if (!s || !shape)
        return fail(s, BS_E_ARG, "bs_get_batch_shape: null argument");
    shape[0] = s->shape.block;
    shape[1] = s->shape.lanes;
    shape[2] = s->shape.cluster;
    return BS_OK;
}

int bs_batch_autotune(bs_sim *s, int32_t shape[3])
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready || s->p.nsys == 0)
        return fail(s, BS_E_STATE, "bs_batch_autotune: set up a batched ensemble first");
    int rc = bs_synchronize(s);
    if (rc)
        return rc;
    if (!s->list_valid)
    {
        rc = rebuild_now(s);
        if (rc)
            return rc;
    }
    Params &p = s->p;
    const size_t np = static_cast<size_t>(p.npad), ns = static_cast<size_t>(p.nsys);
    // Trials step the real state; it is saved here and put back after every trial.
    DeviceBuffers save;
    float4 *sv[4];
    long long *s_steps, *s_stale;
    int *s_status;
    double *s_energy;
    for (int k = 0; k < 4; ++k)
        BS_CUDA(save.alloc(&sv[k], np));
    BS_CUDA(save.alloc(&s_steps, ns));
    BS_CUDA(save.alloc(&s_stale, ns));
    BS_CUDA(save.alloc(&s_status, ns));
    BS_CUDA(save.alloc(&s_energy, ns * 8));
    float4 *live[4] = {p.pos[0], p.pos[1], p.vel[0], p.vel[1]};
    auto copy_all = [&](bool to_save) -> cudaError_t {
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < 4 && e == cudaSuccess; ++k)
            e = cudaMemcpyAsync(to_save ? sv[k] : live[k], to_save ? live[k] : sv[k], sizeof(float4) * np,
                                cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(to_save ? s_steps : p.sys_steps, to_save ? p.sys_steps : s_steps, sizeof(long long) * ns,
                                cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(to_save ? s_stale : p.stale_at, to_save ? p.stale_at : s_stale, sizeof(long long) * ns,
                                cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(to_save ? s_status : p.sys_status, to_save ? p.sys_status : s_status, sizeof(int) * ns,
                                cudaMemcpyDeviceToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(to_save ? s_energy : p.sys_energy, to_save ? p.sys_energy : s_energy,
                                sizeof(double) * ns * 8, cudaMemcpyDeviceToDevice, s->stream);
        return e;
    };
    cudaError_t e = copy_all(true);
    if (e != cudaSuccess)
    {
        save.free_all();
        return cuda_fail(s, e, "bs_batch_autotune: saving the state");
    }
    cudaEvent_t ev[2];
    cudaEventCreate(&ev[0]);
    cudaEventCreate(&ev[1]);
    const int K = std::max(1, s->cfg.rebuild_every);
    const BatchShape old = s->shape;
    BatchShape best = old;
    float best_ms = 1e30f;
    const int blocks[3] = {128, 256, 512}, lanes[3] = {2, 4, 8}, clusters[4] = {1, 2, 4, 8};
    for (int cb : clusters)
        for (int bb : blocks)
            for (int lb : lanes)
            {
                s->shape = BatchShape{bb, lb, cb};
                if (assign_clusters(s) != BS_OK)
                    continue;
                float ms = 1e30f;
                for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep)
                {
                    e = cudaEventRecord(ev[0], s->stream);
                    if (e == cudaSuccess)
                        e = launch_batch_run(p, s->shape, K, s->stream);
                    if (e == cudaSuccess)
                        e = cudaEventRecord(ev[1], s->stream);
                    if (e == cudaSuccess)
                        e = cudaEventSynchronize(ev[1]);
                    float t = 0.f;
                    if (e == cudaSuccess)
                        e = cudaEventElapsedTime(&t, ev[0], ev[1]);
                    if (e == cudaSuccess)
                        e = copy_all(false);
                    ms = std::min(ms, t);
                }
                if (e != cudaSuccess)
                    break;
                if (ms < best_ms)
                {
                    best_ms = ms;
                    best = s->shape;
                }
            }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    if (e == cudaSuccess)
        e = copy_all(false);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s->stream);
    save.free_all();
    s->ctl_read_at = -1; // the trial runs were not counted as launches
    if (e != cudaSuccess)
        return cuda_fail(s, e, "bs_batch_autotune: trial run");
    s->shape = best;
    rc = assign_clusters(s);
    if (rc)
        return rc;
    if (shape)
    {
        shape[0] = best.block;
        shape[1] = best.lanes;
        shape[2] = best.cluster;
    }
    return BS_OK;
}

int bs_get_system_energies(bs_sim *s, double *out)
{
    if (!s || !out)
        return fail(s, BS_E_ARG, "bs_get_system_energies: null argument");
    if (!s->ready || s->p.nsys == 0)
        return fail(s, BS_E_STATE, "bs_get_system_energies: set up a batched ensemble first");
    int rc = bs_synchronize(s);
    if (rc)
        return rc;
    const int nsys = s->p.nsys;
    std::vector<double> e(static_cast<size_t>(nsys) * 8);
    BS_CUDA(cudaMemcpy(e.data(), s->p.sys_energy, sizeof(double) * e.size(), cudaMemcpyDeviceToHost));
    for (int b = 0; b < nsys; ++b)
        for (int k = 0; k < BS_NUM_ENERGIES; ++k)
            out[static_cast<size_t>(b) * BS_NUM_ENERGIES + k] = e[static_cast<size_t>(b) * 8 + k];
    return BS_OK;
}

int bs_get_probe(bs_sim *s, float state[6])
{
    if (!s || !state)
        return fail(s, BS_E_ARG, "bs_get_probe: null argument");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    int rc = bs_synchronize(s);
    if (rc == BS_OK)
        rc = read_ctl(s);
    if (rc)
        return rc;
    const Ctl &h = *s->ctl_host;
    const float v[6] = {h.probe_pos.x, h.probe_pos.y, h.probe_pos.z, h.probe_vel.x, h.probe_vel.y, h.probe_vel.z};
    for (int k = 0; k < 6; ++k)
        state[k] = s->p.probe_on ? v[k] : 0.0f;
    return BS_OK;
}

int bs_get_spring_count(bs_sim *s, int64_t *count)
{
    if (!s || !count)
        return fail(s, BS_E_ARG, "bs_get_spring_count: null argument");
    *count = static_cast<int64_t>(s->sp_i.size());
    return BS_OK;
}

int bs_set_spring_parameters(bs_sim *s, const float *stiffness, const float *equilibrium)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    int rc = bs_synchronize(s);
    if (rc)
        return rc;
    const size_t ns = s->sp_i.size();
    if (ns == 0)
        return BS_OK;
    for (size_t t = 0; t < ns; ++t)
    {
        if (stiffness)
            s->sp_k[t] = stiffness[t];
        if (equilibrium)
            s->sp_r0[t] = equilibrium[t];
    }
    const size_t nnz = 2 * ns;
    std::vector<float> kk(nnz), rr(nnz);
    for (size_t t = 0; t < ns; ++t)
        for (int e = 0; e < 2; ++e)
        {
            kk[s->csr_pos[2 * t + e]] = s->sp_k[t];
            rr[s->csr_pos[2 * t + e]] = s->sp_r0[t];
        }
    BS_CUDA(cudaMemcpyAsync(const_cast<float *>(s->p.sp_k), kk.data(), sizeof(float) * nnz, cudaMemcpyHostToDevice,
                            s->stream));
    BS_CUDA(cudaMemcpyAsync(const_cast<float *>(s->p.sp_r0), rr.data(), sizeof(float) * nnz, cudaMemcpyHostToDevice,
                            s->stream));
    BS_CUDA(cudaStreamSynchronize(s->stream));
    s->list_valid = false; // the next rebuild copies them into the sorted spring table
    return BS_OK;
}

// Records the whole adjoint run (forward with checkpoints, then the backward sweep with
// recomputation from each checkpoint) on the handle's stream.
// keep_all: the positions of every step of every interval are kept from the first forward pass
// (they fit the memory budget), so the backward pass restores each interval's layout with one
// rebuild from its checkpoint and recomputes no step; otherwise only the last interval's are kept
// and each earlier interval is recomputed from its checkpoint.
static int record_adjoint(bs_sim *s, int nsteps, int K, bool charges, bool keep_all)
{
    Params &p = s->p;
    const int S = (nsteps + K - 1) / K;
    const size_t n3 = 3 * static_cast<size_t>(s->n), np = static_cast<size_t>(p.npad);
    auto seg_len = [&](int seg) { return std::min(K, nsteps - seg * K); };
    float4 *lo_seg = p.pos_lo[0] ? s->adj_seg_lo : nullptr;
    BS_CUDA(cudaMemsetAsync(s->adj_gk, 0, sizeof(float) * 2 * std::max<size_t>(s->sp_i.size(), 1), s->stream));
    BS_CUDA(cudaMemsetAsync(s->adj_gr0, 0, sizeof(float) * 2 * std::max<size_t>(s->sp_i.size(), 1), s->stream));
    if (charges)
        BS_CUDA(cudaMemsetAsync(s->adj_gq, 0, sizeof(float) * s->n, s->stream));
    // forward: a checkpoint (caller order) and a rebuild at the start of every interval; the
    // positions of the last interval are kept as they are produced
    for (int seg = 0; seg < S; ++seg)
    {
        s->launches += launch_unsort(p, 0, s->adj_ck_xyz + seg * n3, s->stream);
        s->launches += launch_unsort(p, 1, s->adj_ck_vel + seg * n3, s->stream);
        if (p.pos_lo[0])
            s->launches += launch_unsort(p, 3, s->adj_ck_lo + seg * n3, s->stream);
        s->launches += launch_rebuild(p, s->stream);
        for (int k = 0; k < seg_len(seg); ++k)
        {
            if (keep_all || seg == S - 1)
            {
                const size_t at = (keep_all ? static_cast<size_t>(seg) * K + k : static_cast<size_t>(k)) * np;
                s->launches += launch_adj_save(p, s->adj_seg + at, lo_seg ? lo_seg + at : nullptr, s->stream);
            }
            s->launches += launch_step(p, MODE_STEP, s->stream);
        }
    }
    AdjState a{nullptr, nullptr, s->adj_lx, s->adj_lv, s->adj_nu[0], s->adj_nu[1], s->adj_gk, s->adj_gr0,
               charges ? s->adj_gq : nullptr};
    s->launches += launch_adj_init(p, a, s->adj_target, s->adj_blk, s->adj_done, s->adj_loss, s->stream);
    int cur = 0;
    for (int seg = S - 1; seg >= 0; --seg)
    {
        const int len = seg_len(seg);
        if (seg != S - 1)
        {
            a.nu_in = s->adj_nu[cur];
            s->launches += launch_adj_permute(p, a, s->adj_cx, s->adj_cv, 0, s->stream);
            s->launches += launch_set_positions(p, s->adj_ck_xyz + seg * n3, s->adj_ck_vel + seg * n3, s->stream,
                                                p.pos_lo[0] ? s->adj_ck_lo + seg * n3 : nullptr);
            s->launches += launch_rebuild(p, s->stream);
            for (int k = 0; !keep_all && k < len; ++k)
            {
                s->launches += launch_adj_save(p, s->adj_seg + k * np, lo_seg ? lo_seg + k * np : nullptr,
                                               s->stream);
                if (k < len - 1)
                    s->launches += launch_step(p, MODE_STEP, s->stream);
            }
            s->launches += launch_adj_permute(p, a, s->adj_cx, s->adj_cv, 1, s->stream);
        }
        for (int k = len - 1; k >= 0; --k)
        {
            const size_t at = (keep_all ? static_cast<size_t>(seg) * K + k : static_cast<size_t>(k)) * np;
            a.x = s->adj_seg + at;
            a.xlo = lo_seg ? lo_seg + at : nullptr;
            a.nu_in = s->adj_nu[cur];
            a.nu_out = s->adj_nu[cur ^ 1];
            s->launches += launch_adj_step(p, a, s->stream);
            cur ^= 1;
        }
    }
    s->launches += launch_adj_combine(static_cast<int>(s->sp_i.size()), s->adj_gk, s->adj_gr0, s->adj_ok, s->adj_or0,
                                      s->stream);
    // the state goes back to the start
    s->launches += launch_set_positions(p, s->adj_ck_xyz, s->adj_ck_vel, s->stream,
                                        p.pos_lo[0] ? s->adj_ck_lo : nullptr);
    return BS_OK;
}

int bs_adjoint(bs_sim *s, int32_t nsteps, int32_t checkpoint, const float *target, double *loss, float *dL_dk,
               float *dL_dr0, float *dL_dq)
{
    if (!s)
        return fail(nullptr, BS_E_ARG, "null handle");
    if (!s->ready)
        return fail(s, BS_E_STATE, "call bs_setup first");
    if (s->p.nsys > 0)
        return fail(s, BS_E_STATE, "bs_adjoint: not available for batched ensembles");
    if (nsteps < 1 || checkpoint < 1 || !target || !loss)
        return fail(s, BS_E_ARG, "bs_adjoint: nsteps >= 1, checkpoint >= 1, target and loss are required");
    if (!s->sp_i.empty() && (!dL_dk || !dL_dr0))
        return fail(s, BS_E_ARG, "bs_adjoint: dL_dk and dL_dr0 are required");
    const bs_config &c = s->cfg;
    if (c.hydrophobicity_enable || c.impala_enable)
        return fail(s, BS_E_ARG, "bs_adjoint: differentiates springs, linear steric, Coulomb and viscosity; "
                                 "disable hydrophobicity and impala");
    if (c.steric_enable && c.steric_mode != BS_STERIC_LINEAR)
        return fail(s, BS_E_ARG, "bs_adjoint: only the linear steric mode is differentiated");
    if (s->p.nbody > 0 || s->p.probe_on)
        return fail(s, BS_E_ARG, "bs_adjoint: rigid bodies and the probe are not differentiated");
    if (s->p.fg_on[0] || s->p.fg_on[1])
        return fail(s, BS_E_ARG, "bs_adjoint: field-grid forces are not differentiated");
    int rc = bs_synchronize(s); // ends with a fresh read of the control block
    if (rc)
        return rc;
    if (s->ctl_host->ext_pending)
        return fail(s, BS_E_STATE, "bs_adjoint: an external force is pending; step or clear it first");
    Params &p = s->p;
    // charge gradients need every pair of a charged particle, so the adjoint's list builds (and a
    // regrowth on the way) list the Coulomb partners of every dynamic particle; the flag goes
    // back when the call returns (the next step rebuilds the lists)
    const bool charges = dL_dq != nullptr;
    struct CoulAll
    {
        Params &p;
        int old;
        ~CoulAll() { p.coul_all = old; }
    } coul_all_guard{p, p.coul_all};
    p.coul_all = charges && c.coulomb_enable ? 1 : 0;
    if (charges && !s->adj_gq)
        BS_CUDA(s->adj_dev.alloc(&s->adj_gq, static_cast<size_t>(s->n)));
    const int K = std::min(checkpoint, nsteps);
    const int S = (nsteps + K - 1) / K;
    const size_t n3 = 3 * static_cast<size_t>(s->n), np = static_cast<size_t>(p.npad);
    const size_t ns = s->sp_i.size();
    // Positions of every step kept when they take at most a quarter of the free device memory
    // (10,000 particles x 200 steps: 32 MB, twice that with precise positions).
    bool keep_all = false;
    {
        size_t free_b = 0, total_b = 0;
        BS_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const double per_step = static_cast<double>(np) * sizeof(float4) * (p.pos_lo[0] ? 2.0 : 1.0);
        const double held = static_cast<double>(s->adj_seg_cap) * per_step;
        keep_all = static_cast<double>(nsteps) * per_step <= 0.25 * (static_cast<double>(free_b) + held);
    }
    const int seg_cap = keep_all ? nsteps : K;
    // directed spring ids in the sorted spring table (filled by every rebuild from now on)
    if (!p.se_sid)
    {
        unsigned int *d_sid = nullptr, *e_sid = nullptr;
        BS_CUDA(s->adj_dev.alloc(&d_sid, s->csr_sid.size()));
        BS_CUDA(s->adj_dev.alloc(&e_sid, np * p.sp_maxdeg));
        BS_CUDA(cudaMemcpyAsync(d_sid, s->csr_sid.data(), sizeof(unsigned int) * s->csr_sid.size(),
                                cudaMemcpyHostToDevice, s->stream));
        p.sp_sid = d_sid;
        p.se_sid = e_sid;
        s->sp_sid_d = d_sid;
        destroy_graph(s);
    }
    if (S > s->adj_ck_cap || seg_cap > s->adj_seg_cap || !s->adj_lx)
    {
        destroy_graph(s);
        // (buffers of a smaller earlier run stay allocated until the handle is set up again)
        s->adj_ck_cap = std::max(S, s->adj_ck_cap);
        s->adj_seg_cap = std::max(seg_cap, s->adj_seg_cap);
        BS_CUDA(s->dev.alloc(&s->adj_ck_xyz, s->adj_ck_cap * n3));
        BS_CUDA(s->dev.alloc(&s->adj_ck_vel, s->adj_ck_cap * n3));
        BS_CUDA(s->dev.alloc(&s->adj_ck_lo, s->adj_ck_cap * n3));
        BS_CUDA(s->dev.alloc(&s->adj_seg, s->adj_seg_cap * np));
        if (p.pos_lo[0])
            BS_CUDA(s->dev.alloc(&s->adj_seg_lo, s->adj_seg_cap * np));
        BS_CUDA(s->dev.alloc(&s->adj_lx, np));
        BS_CUDA(s->dev.alloc(&s->adj_lv, np));
        BS_CUDA(s->dev.alloc(&s->adj_nu[0], np));
        BS_CUDA(s->dev.alloc(&s->adj_nu[1], np));
        BS_CUDA(s->dev.alloc(&s->adj_cx, np));
        BS_CUDA(s->dev.alloc(&s->adj_cv, np));
        BS_CUDA(s->dev.alloc(&s->adj_target, np));
        BS_CUDA(s->dev.alloc(&s->adj_gk, 2 * std::max<size_t>(ns, 1)));
        BS_CUDA(s->dev.alloc(&s->adj_gr0, 2 * std::max<size_t>(ns, 1)));
        BS_CUDA(s->dev.alloc(&s->adj_ok, std::max<size_t>(ns, 1)));
        BS_CUDA(s->dev.alloc(&s->adj_or0, std::max<size_t>(ns, 1)));
        BS_CUDA(s->dev.alloc(&s->adj_blk, (np + 255) / 256));
        BS_CUDA(s->dev.alloc(&s->adj_loss, 1));
        BS_CUDA(s->dev.alloc(&s->adj_done, 1));
        BS_CUDA(cudaMemsetAsync(s->adj_done, 0, sizeof(unsigned int), s->stream));
    }
    // the target, caller order
    {
        std::vector<float4> tg(np, make_float4(0.f, 0.f, 0.f, 0.f));
        for (int64_t i = 0; i < s->n; ++i)
            tg[i] = make_float4(target[3 * i], target[3 * i + 1], target[3 * i + 2], 0.f);
        BS_CUDA(cudaMemcpyAsync(s->adj_target, tg.data(), sizeof(float4) * np, cudaMemcpyHostToDevice, s->stream));
        BS_CUDA(cudaStreamSynchronize(s->stream));
    }
    rc = read_ctl(s);
    if (rc)
        return rc;
    const Ctl saved = *s->ctl_host;
    for (int attempt = 0; attempt < 4; ++attempt)
    {
        if (!s->adj_graph || s->adj_key[0] != nsteps || s->adj_key[1] != K || s->adj_key[2] != (charges ? 1 : 0) ||
            s->adj_key[3] != (keep_all ? 1 : 0))
        {
            if (s->adj_graph)
            {
                cudaGraphExecDestroy(s->adj_graph);
                s->adj_graph = nullptr;
            }
            cudaGraph_t g = nullptr;
            BS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            const long long before = s->launches;
            // the adjoint's forward runs record no frames
            const int frame_every = s->p.frame_every;
            s->p.frame_every = 0;
            rc = record_adjoint(s, nsteps, K, charges, keep_all);
            s->p.frame_every = frame_every;
            const cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
            if (rc)
            {
                if (g)
                    cudaGraphDestroy(g);
                return rc;
            }
            if (ce != cudaSuccess)
                return cuda_fail(s, ce, "bs_adjoint: capture");
            const cudaError_t ie = cudaGraphInstantiate(&s->adj_graph, g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess)
                return cuda_fail(s, ie, "bs_adjoint: cudaGraphInstantiate");
            s->adj_key[0] = nsteps;
            s->adj_key[1] = K;
            s->adj_key[2] = charges ? 1 : 0;
            s->adj_key[3] = keep_all ? 1 : 0;
            s->adj_kernels = s->launches - before;
            s->launches = before;
        }
        BS_CUDA(cudaGraphLaunch(s->adj_graph, s->stream));
        s->launches += s->adj_kernels;
        s->list_valid = false;
        rc = read_ctl(s);
        if (rc)
            return rc;
        const Ctl &h = *s->ctl_host;
        if (h.status & ST_NONFINITE)
            return fail(s, BS_E_NONFINITE, "bs_adjoint: a position became non-finite");
        if ((h.status & ST_STALE) || h.stale_events != saved.stale_events)
        {
            // put the counters back before reporting
            s->ctl_host->status &= ~ST_STALE;
            s->ctl_host->stale_events = saved.stale_events;
            s->ctl_host->steps = saved.steps;
            for (int k = 0; k < 8; ++k)
                s->ctl_host->energies[k] = saved.energies[k];
            BS_CUDA(cudaMemcpy(s->p.ctl, s->ctl_host, sizeof(Ctl), cudaMemcpyHostToDevice));
            return fail(s, BS_E_CAPACITY, "bs_adjoint: a particle moved more than half the list skin within a "
                                          "checkpoint interval; raise cuda.listskin or shorten the interval");
        }
        if (h.status & (ST_CELL_CAPACITY | ST_PAIR_CAPACITY | ST_WIDE))
        {
            // a list or the grid overflowed at one of the rebuilds: grow it (this rebuilds from the
            // restored start state) and run again
            rc = rebuild_now(s);
            if (rc)
                return rc;
            continue;
        }
        // step count and energies as before the call
        s->ctl_host->steps = saved.steps;
        for (int k = 0; k < 8; ++k)
            s->ctl_host->energies[k] = saved.energies[k];
        BS_CUDA(cudaMemcpy(s->p.ctl, s->ctl_host, sizeof(Ctl), cudaMemcpyHostToDevice));
        BS_CUDA(cudaMemcpy(loss, s->adj_loss, sizeof(double), cudaMemcpyDeviceToHost));
        if (ns)
        {
            BS_CUDA(cudaMemcpy(dL_dk, s->adj_ok, sizeof(float) * ns, cudaMemcpyDeviceToHost));
            BS_CUDA(cudaMemcpy(dL_dr0, s->adj_or0, sizeof(float) * ns, cudaMemcpyDeviceToHost));
        }
        if (charges)
        {
            if (c.coulomb_enable)
                BS_CUDA(cudaMemcpy(dL_dq, s->adj_gq, sizeof(float) * s->n, cudaMemcpyDeviceToHost));
            else
                std::memset(dL_dq, 0, sizeof(float) * s->n);
        }
        return BS_OK;
    }
    return fail(s, BS_E_CAPACITY, "bs_adjoint: lists did not fit after repeated growth");
}

int bs_get_launch_count(bs_sim *s, int64_t *count)
{
    if (!s || !count)
        return fail(s, BS_E_ARG, "bs_get_launch_count: null argument");
    *count = s->launches;
    return BS_OK;
}

int bs_last_error(bs_sim *s, char *buf, size_t len)
{
    if (!buf || len == 0)
        return BS_E_ARG;
    const std::string &m = s ? s->err : g_last_error;
    std::snprintf(buf, len, "%s", m.c_str());
    return BS_OK;
}

} // extern "C"
