// bs_kernels.cuh -- kernel declarations of the GB300 step engine.
#pragma once

#include "bs_common.cuh"

namespace bsg
{

constexpr int kStepBlock = 128; // adjoint and diagnostic kernels
#ifndef BS_STEP_BLOCK
#define BS_STEP_BLOCK 256
#endif
#ifndef BS_STEP_MIN_BLOCKS
#define BS_STEP_MIN_BLOCKS (1024 / BS_STEP_BLOCK)
#endif
// threads per block of the step kernel, and the resident blocks per SM it is compiled for
// (1024 resident threads: at most 64 registers)
constexpr int kStepKernelBlock = BS_STEP_BLOCK;
constexpr int kStepMinBlocks = BS_STEP_MIN_BLOCKS;
constexpr int kBuildBlock = 128;
constexpr int kBuildLanes = 8;    // threads per slot of the spring-table rebuild when the table fits L2
constexpr int kBboxBlock = 256;
constexpr int kMaxEnergyBlocks = 1 << 16;

// status bits that stop a rebuild; a stale list is what a rebuild repairs
constexpr int kRebuildBlocking = ST_NONFINITE | ST_PAIR_CAPACITY | ST_CELL_CAPACITY | ST_WIDE;
// Programmatic dependent launch in the rebuild chain (its eleven kernels overlap their launches:
// 351 -> 344 us at 100k). BS_PDL_STEP extends it to the step kernels, which made the graph-replayed
// 100k step slower (120 -> 130 us), so it is off.
// Coulomb rows walked by the whole warp, one charged particle at a time, instead of by the
// particle's own lanes (100k step after an L2 flush: 112.0 -> 110.8 us; warm: unchanged).
#ifndef BS_COUL_WARP
#define BS_COUL_WARP 1
#endif
#ifndef BS_PDL
#define BS_PDL 1
#endif
// Gathers in flight per lane in the step kernel's spring and steric loops: kGatherU entries are
// read per pass and their partners loaded together (0: the entry-by-entry software-pipelined
// loops). BS_GATHER_BATCH selects it for the persistent ensemble kernel (512 Calpha networks of
// degree 19: 2.19e9 -> 2.96e9 particle-steps/s); both forms sum the same entries in the same order.
#ifndef BS_GATHER
#define BS_GATHER 3
#endif
#ifndef BS_GATHER_BATCH
#define BS_GATHER_BATCH 1
#endif
constexpr int kGatherU = 4;
// the LJ pair body refines the hardware reciprocal by one Newton step (0: the approximation alone)
#ifndef BS_LJ_RCP_REFINE
#define BS_LJ_RCP_REFINE 1
#endif
#ifndef BS_LJ_BAND_AFTER
#define BS_LJ_BAND_AFTER 0
#endif
#ifndef BS_HOIST
#define BS_HOIST 1
#endif
// the lean step kernel (BS_LEAN 0: always the full one)
#ifndef BS_LEAN
#define BS_LEAN 1
#endif
#ifndef BS_PDL_STEP
#define BS_PDL_STEP 0
#endif
// Cell-block list build on cells of half the list radius, in groups of 2 x 2 x 2 cells per block,
// the bounded runs packed into full windows and spring partners excluded by lane masks: 323
// candidates tested per particle instead of 505 at 100k (rebuild 355 -> 310 us).
#ifndef BS_GRID_DIV
#define BS_GRID_DIV 2
#endif
// the cell-block list build walks the bounded runs as one packed sequence when there are many
#ifndef BS_PL_PACK
#define BS_PL_PACK (BS_GRID_DIV > 1)
#endif
#ifndef BS_PL_WARPS
#define BS_PL_WARPS 8
#endif
#ifndef BS_PL_STAGE
#define BS_PL_STAGE 2048
#endif
constexpr int kGridDiv = BS_GRID_DIV; // cell-block list build: cells per list radius (stencil of +-kGridDiv cells)
constexpr int kSparseDiv = 1;         // warp-per-particle list build (sparse systems, batches): cells of the radius
constexpr int kPlWarps = BS_PL_WARPS; // warps per block (one cell) in the pair-list build
constexpr int kPlStage = BS_PL_STAGE; // candidate positions staged in shared memory per block
constexpr int kPlMinBlocks = 4;       // resident list-build blocks per SM (the stage allows 4)
constexpr int kPlBatch = 16;         // home particles per warp
constexpr int kPlBatchesPerCell = 4; // warps per cell (a cell with more than 64 particles loops)
constexpr int kScanTile = 4096;      // cells per block of the cell-count scan (4 per thread)

enum StepMode
{
    MODE_STEP = 0,   // forces + Euler step (SpringNetwork::computeStep)
    MODE_FORCES = 1, // forces and energies only (SpringNetwork::computeForces)
};

// Launchers (all asynchronous on `stream`); each returns the number of kernels launched.
int launch_rebuild(const Params &p, cudaStream_t stream);
int launch_step(const Params &p, int mode, cudaStream_t stream);      // step kernel, then the bodies
int launch_step_only(const Params &p, int mode, cudaStream_t stream); // the step kernel alone
int launch_rigid(const Params &p, cudaStream_t stream);               // bs_rigid.cu
int launch_ext_add(const Params &p, long long i, float fx, float fy, float fz, cudaStream_t stream);
int launch_set_burying(const Params &p, const float *burying, cudaStream_t stream);
int launch_set_charges(const Params &p, const float *q, cudaStream_t st);
int launch_unsort(const Params &p, int what, float *out3, cudaStream_t stream);
int launch_diag_cells(const Params &p, float cutoff, float skin, uint32_t need_flag, long long *out,
                      cudaStream_t stream);
int launch_diag_pairs(const Params &p, int term, long long *out, unsigned long long *count,
                      unsigned long long cap, cudaStream_t stream);
int launch_set_positions(const Params &p, const float *xyz, const float *vel, cudaStream_t stream,
                         const float *lo = nullptr);

// Discrete adjoint (bs_adjoint.cu).
struct AdjState
{
    const float4 *x;   // positions at the start of the step being reversed (sorted layout)
    const float4 *xlo; // their rounding remainders (precise_positions), else null
    float4 *lx;      // dL/dx
    float4 *lv;      // dL/dv
    float4 *nu_in;   // b (lambda_v + dt lambda_x) of the later step
    float4 *nu_out;  // the same for the step being reversed
    float *gk;       // per directed spring entry: dL/dk, dL/dr0 partial sums
    float *gr0;
    float *gq;       // dL/dq per caller id (null: no charge gradients)
};
int launch_adj_step(const Params &p, const AdjState &a, cudaStream_t stream);
int launch_adj_init(const Params &p, const AdjState &a, const float4 *target, double *blk, unsigned int *done,
                    double *loss, cudaStream_t stream);
int launch_adj_permute(const Params &p, const AdjState &a, float4 *cx, float4 *cv, int dir, cudaStream_t stream);
int launch_adj_save(const Params &p, float4 *dst, float4 *dst_lo, cudaStream_t stream);
int launch_adj_combine(int nsp, const float *gk, const float *gr0, float *ok, float *or0, cudaStream_t stream);

// Batched ensembles (bs_batch.cu).
constexpr int kBatchMaxBlock = 512; // largest block of the persistent step kernel
struct BatchShape
{
    int block;   // threads per block
    int lanes;   // threads per particle (1, 2, 4, 8)
    int cluster; // blocks per cluster (1, 2, 4, 8)
};
int launch_batch_grid(const Params &p, cudaStream_t stream);
int launch_batch_pairlist(const Params &p, cudaStream_t stream);
cudaError_t launch_batch_run(const Params &p, const BatchShape &shape, int chunk, cudaStream_t stream);
int launch_batch_finish(const Params &p, int chunk, cudaStream_t stream);
cudaError_t batch_max_clusters(const Params &p, const BatchShape &shape, int *out);

} // namespace bsg
