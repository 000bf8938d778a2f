// bs_common.cuh -- shared device definitions of the GB300 step engine.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/biospring_gb300.h"

namespace bsg
{

// ---- unit constants (values of src/forcefield/constants.hpp:36-118) -------------------
constexpr double kElectronChargeC = 1.60217653E-19;
constexpr double kAngstromToMeter = 1.0E-10;
constexpr double kMeterToAngstrom = 1.0E10;
constexpr double kDaltonToKg = 1.66054E-27;
constexpr double kFsToS = 1.0E-15;
constexpr double kSToFs = 1.0E15;
constexpr double kPi = 3.1415927;
constexpr double kVacuumPermittivity = 8.854187817E-12;
constexpr double kAvogadro = 6.02214169E23;
constexpr double kCoulombK = 1.0 / (4.0 * kPi * kVacuumPermittivity);
constexpr double kNewtonToDaAFs2 = kMeterToAngstrom * (1.0 / kDaltonToKg) * kFsToS * kFsToS;
// force conversions: molar kJ/mol/A -> Da.A.fs^-2, and the Coulomb one
constexpr double kSpringForceConvert = 1.0E3 / kAvogadro * kMeterToAngstrom * kNewtonToDaAFs2;
constexpr double kImpForceConvert = kSpringForceConvert;
constexpr double kElecForceConvert = kNewtonToDaAFs2 * (kElectronChargeC * kElectronChargeC) /
                                     (kVacuumPermittivity * kAngstromToMeter * kAngstromToMeter);
constexpr double kKineticConvert = (kAngstromToMeter * kSToFs) * (kAngstromToMeter * kSToFs) * kAvogadro *
                                   kDaltonToKg * 1.0E-3;
// Coulomb energy of two unit charges at 1 A with dielectric 1, in kJ/mol
constexpr double kCoulombEnergyPerA = kCoulombK * kElectronChargeC * kElectronChargeC / kAngstromToMeter * kAvogadro * 1.0E-3;
constexpr float kAlip = -0.018f;

// ---- status bits (device -> host) ------------------------------------------------------
enum : int
{
    ST_NONFINITE = 1,       // a position became non-finite
    ST_PAIR_CAPACITY = 2,   // a pair-list row overflowed
    ST_CELL_CAPACITY = 4,   // the search grid needs more cells than allocated
    ST_STALE = 8,           // a particle drifted more than half the list skin: rebuild needed
    ST_WIDE = 16,           // a neighbour offset does not fit the 16-bit steric list
};

// particle flag bits
enum : uint32_t
{
    PF_STATIC = 1u,
    PF_CHARGED = 2u,
    PF_HYDROPHOBIC = 4u,
    PF_RIGID = 8u,
};

// list entry bits: the low 30 bits are a slot
constexpr uint32_t kSlotMask = 0x3fffffffu;
constexpr uint32_t kEntryStatic = 0x80000000u;   // the partner is static: the pair's full energy is ours
constexpr uint32_t kEntryInactive = 0x40000000u; // spring between two rigid particles: no force

constexpr int kTerms = 3; // nonbonded terms: steric, Coulomb, hydrophobic
// Pair lists: 0 = steric, dynamic partners (16-bit slot offsets when they fit), 1 = Coulomb,
// 2 = hydrophobic, 3 = steric, static partners (full pair energy, rare)
constexpr int kLists = 4;
constexpr int kListStericStatic = 3;

// Step energies are reduced block -> group of kEnergyGroup blocks -> grid; the scratch holds
// 16 floats per block partial and per group partial, then one counter per group.
constexpr int kEnergyGroup = 32;
__host__ __device__ constexpr int energy_groups(int blocks) { return (blocks + kEnergyGroup - 1) / kEnergyGroup; }
__host__ __device__ constexpr size_t energy_scratch_doubles(int blocks)
{
    return static_cast<size_t>(blocks + energy_groups(blocks)) * 8 + (energy_groups(blocks) + 1) / 2;
}

// Device control block: one per simulation handle, in device memory.
struct Ctl
{
    int status;
    int sbuf;                 // index of the buffer holding the current positions/velocities
    int lbuf;                 // index of the buffer holding the current particle layout
    unsigned int done_step;   // last-block counters
    unsigned int done_bbox;
    unsigned int done_reorder;
    long long steps;          // completed steps since setup
    int max_row[kLists];      // largest row of each pair list seen at the last build
    int ncells_needed;
    // search grid of the current layout (reference formula, nsearch.hpp:342-354)
    double gmin[3];
    float gradius;
    int gnx, gny, gnz;
    unsigned int bbox_enc[6];  // order-preserving codes of min xyz, max xyz (reset after use)
    int status_pending;        // bits raised during a step, merged into status by its last block
    int ext_pending;           // an external force waits in Params::ext
    double energies[8];        // BS_ENERGY_* of the last evaluation
    // batched ensembles
    long long nominal;         // steps every system should have completed after the queued work
    int lagging;               // live systems behind `nominal` (stopped early by a stale list)
    int dead;                  // systems with a non-finite position
    int stale_events;          // rebuilds that found a stale list (counted, never reset)
    long long rigid_steps;     // value of `steps` for which the rigid bodies last moved
    unsigned int done_rigid;   // last-block counter of the body kernel
    // probe particle (SpringNetwork.cpp:749-766)
    float4 probe_pos;
    float4 probe_vel;
    long long probe_steps;     // value of `steps` for which the probe last moved
    unsigned int done_frame;   // last-block counter of the frame kernel
};

// Header of a recorded frame in the host ring: the frame's sequence number (step / every; -1
// while it is being written), its step and the energies of that step (BS_ENERGY_* order).
struct FrameHeader
{
    long long seq;
    long long step;
    double energies[6];
};

// State of one rigid body (RigidBody.h): position, velocity, angular momentum, orientation
// (x, y, z, w), total mass and the inverse of its diagonal inertia.
struct BodyState
{
    float4 pos;
    float4 vel;
    float4 L;
    float4 q;
    double mass;
    double ibodyinv;
};

// Search grid of one system of a batched ensemble (same formula as the single-system grid).
struct SysGrid
{
    double gmin[3];
    float radius;
    int nx, ny, nz;
    int cells;
};

// One typed pair list, row-major [slot * cap + k]: entries = slot | kEntryStatic, or for
// list 0 in 16-bit mode, (short)(partner slot - slot).
struct PairList
{
    unsigned int *idx;
    int *cnt;                 // [npad]
    int cap;
    float r2;                 // squared list radius (cutoff + skin), slightly inflated
    int on;
};

// Step parameters passed by value to the kernels.
struct Params
{
    int n;                    // particles
    int npad;                 // n rounded up to a multiple of 32 (ELL row stride)
    // double-buffered sorted state: positions/velocities flip every step (Ctl::sbuf), the
    // per-particle parameters flip at every rebuild (Ctl::lbuf)
    float4 *pos[2];           // x, y, z, steric factor P (F6 for LJ modes, radius for linear)
    float4 *vel[2];           // vx, vy, vz, 0
    float4 *pos_lo[2];        // rounding remainders of x, y, z (precise_positions), else null
    float *fhi[2];            // second steric factor (F12 Amber, F8 Lewitt/Zacharias)
    float *chg[2];            // charge
    float *hyd[2];            // hydrophobicity
    unsigned int *flags[2];   // PF_* bits
    float4 *iprm[2];          // mass, sasa, transfer, 0
    int *perm[2];             // sorted slot -> caller id
    int *inv;                 // caller id -> sorted slot (current layout)
    float4 *pos_build;        // positions at the last pair-list build (sorted)
    // per-particle data in caller order
    float *ext;               // external force for the next step, float[3n] by caller id
    float4 *force_out;        // forces of a force-only evaluation
    // springs: caller-order CSR (static topology), partner | kEntryStatic | kEntryInactive
    const int *sp_row;        // [n+1]
    const unsigned int *sp_col;
    const float *sp_k;
    const float *sp_r0;
    int sp_maxdeg;
    int ell_lanes;            // threads per slot of the spring-table rebuild (1 or kBuildLanes)
    // springs: sorted-space ELL, column-major [k * npad + slot], each row ascending by partner slot
    unsigned int *se_col;
    float *se_k;
    float *se_r0;
    int *se_deg;              // [npad]
    // spring ids of the directed entries (2 * spring + end), for the adjoint; null when unused
    const unsigned int *sp_sid; // caller-order CSR
    unsigned int *se_sid;       // sorted-space ELL
    // nonbonded pair lists
    PairList pl[kLists];
    int pl16;                 // list 0 holds 16-bit offsets
    int lj_uniform;           // every particle has the same second steric factor, lj_F (one LJ type):
    float lj_F;               // the step kernel then reads no per-partner factor
    // search grid
    int *cell_of;             // [npad] cell of each sorted slot (new layout)
    int *cell_cnt;            // [cell_cap + 1]
    int *cell_start;          // [cell_cap + 1]
    int *cell_fill;           // [cell_cap]
    unsigned long long *tmp_key; // [npad] cell-sort key of each placed particle (x bits, caller id)
    int cell_cap;
    int *tile_sum;            // [cell_cap / kScanTile + 2] per-tile totals of the cell scan
    int pl_sparse;            // build the pair lists one warp per particle (few particles per cell)
    int coul_all;             // list Coulomb partners of every dynamic particle, charged or not (charge gradients)
    // energies: per-block partials
    double *blk_energy;       // block and group partials of the step energies, group counters
    int blk_cap;              // block partials it holds (the step kernel's largest grid)
    Ctl *ctl;
    // configuration
    float dt;
    int spring_on, steric_on, coulomb_on, hydro_on, imp_on, visc_on;
    int steric_mode, dielectric_mode;
    int step_lanes;           // threads per particle in the step kernel (1, 2, 4 or 8)
    float c_steric, c_coulomb, c_hydro;               // cutoffs
    float lo2_s, hi2_s, lo2_c, hi2_c, lo2_h, hi2_h;   // guard bands on r^2
    float list_radius;        // grid edge: largest cutoff + skin
    float half_skin2;         // (skin/2)^2, slightly deflated
    float spring_scale, steric_scale, coulomb_scale, hydro_scale, imp_scale;
    float visc;
    float imp_z0, imp_alpha;
    int imp_double;           // the double membrane (any offset or tube curvature set)
    float imp_off[2];         // signed offsets of the upper (+) and lower (-) membranes
    float imp_curv[2];        // their tube curvatures (1/A; 0 flat)
    float k_spring_f;         // (float) kSpringForceConvert
    float k_elec_e;           // kCoulombEnergyPerA / dielectric
    float k_elec_f;           // kElecForceConvert / (4 pi dielectric)
    float k_kin;              // kKineticConvert
    float k_imp_f;            // kImpForceConvert
    float k_hydro_e;          // N_A * 1e-3
    // batched ensembles (nsys = 0: one system). Every system keeps a fixed, contiguous range of
    // slots in every layout: its cells are numbered after the previous system's, so the sort by
    // cell never mixes systems, and its pair lists and springs stay inside the range.
    int nsys;
    const int *sys_start;     // [nsys + 1] slot ranges
    const int *sys_of;        // [npad] system of each slot (0 for padding)
    SysGrid *sys_grid;        // [nsys]
    int *sys_cells;           // [nsys + 1] first global cell of each system
    int *sys_status;          // [nsys] ST_NONFINITE / ST_STALE raised by the system
    long long *sys_steps;     // [nsys] steps completed by each system
    long long *stale_at;      // [nsys] first step whose end positions left the list skin
    double *sys_energy;       // [nsys * 8] BS_ENERGY_* of each system's last step
    float *sys_part;          // [nsys * kMaxCluster * 16] per-block energy partials (hi, lo)
    const int *cl_start;      // [ncl + 1] systems of each cluster of the persistent kernel
    const int *cl_sys;        // [nsys]
    int ncl;
    // rigid bodies (nbody = 0: none)
    int nbody;
    BodyState *body;          // [nbody]
    const int *body_start;    // [nbody + 1] member ranges
    const int *body_ids;      // caller ids of the members, in the caller's order per body
    const float4 *body_p0;    // member position relative to the barycentre at set-up
    float4 *rforce;           // [npad] total force on each rigid particle in the current step
    // probe (probe_on = 0: none): its steric factors (P, F as the particles'), charge and mass,
    // and the reaction of every slot on it in the current step
    int probe_on, probe_steric, probe_elec;
    float probe_P, probe_F, probe_q, probe_mass;
    float4 *probe_f;          // [npad]
    // field grids, 0 = electrostatic potential (on charges), 1 = density (on burying); cells in
    // OpenDX order (scalar, force vector). A float x lies in the grid along an axis iff
    // fg_lo <= x <= fg_hi, the float translation of the reference's double bounds test.
    const float4 *fgrid[2];
    int fg_on[2];
    int fg_n[2][3];
    double fg_o[2][3], fg_h[2][3];  // origin and cell size, as the reference holds them
    float fg_lo[2][3], fg_hi[2][3];
    float fg_of[2][3], fg_ih[2][3]; // origin and 1 / cell size in float, for the fast cell index
    float fg_scale[2];              // potentialgrid.scale (force and energy), densitygrid.scale
    float *bur[2];                  // per-particle burying, layout lb
    // frame recorder (frame_every = 0: off): every frame_every steps the positions, in caller
    // order, and the energies go to a ring of frame_cap frames in page-locked host memory that the
    // device writes directly (mapped); headers are written last
    int frame_every, frame_cap;
    float *frame_xyz;               // [frame_cap][3n], device view of the host ring
    FrameHeader *frame_hdr;         // [frame_cap]
};

constexpr int kMaxCluster = 16;

} // namespace bsg
