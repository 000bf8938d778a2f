/*
 * biospring_gb300.h -- C ABI of the GB300 (sm_103a) implementation of BioSpring's
 * per-step force-and-integrate loop.
 *
 * The reference engine is the C++ class biospring::spn::SpringNetwork
 * (src/spn/SpringNetwork.h). A CUDA backend plugs into it the same way the
 * OpenCL backend does (src/opencl/SpringNetworkOpenCL.h:84-182): a subclass that
 * overrides the step virtuals and forwards them to these entry points.
 *
 * Conventions
 *   - Every entry point returns an int status: BS_OK (0) or one of BS_E_*.
 *     Nothing aborts the process; bs_last_error() gives a one-line reason.
 *   - Arrays are plain host pointers, structure-of-arrays, in the caller's
 *     particle order (the reference's particle index). They are copied on call.
 *   - Positions, velocities and forces are float[3*n] (x0,y0,z0,x1,...).
 *   - Units are the reference's: Angstrom, femtosecond, Dalton, kJ/mol,
 *     forces in Da.A.fs^-2 (src/forcefield/constants.hpp:88-118).
 *   - A handle is not thread-safe; several handles may coexist. Each handle owns
 *     one CUDA stream on the current device.
 */
#ifndef BIOSPRING_GB300_H
#define BIOSPRING_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------ */
#define BS_OK 0
#define BS_E_ARG 1        /* invalid argument (reference: std::invalid_argument / out_of_range) */
#define BS_E_CUDA 2       /* a CUDA runtime call failed */
#define BS_E_NONFINITE 3  /* non-finite position (reference: logging::die, SpringNetwork.cpp:222-229) */
#define BS_E_CAPACITY 4   /* a device list overflowed and could not be regrown */
#define BS_E_TIMEOUT 5    /* a bounded device-side wait gave up */
#define BS_E_STATE 6      /* call made in the wrong order (e.g. step before setup) */

/* ---- steric modes (steric.mode, src/configuration/Setting.hpp:269-273) ---------- */
#define BS_STERIC_LINEAR 0            /* "linear" */
#define BS_STERIC_LJ_12_6_AMBER 1     /* "lennard-jones-12-6Amber" */
#define BS_STERIC_LJ_8_6_LEWITT 2     /* "lennard-jones-8-6Lewitt" */
#define BS_STERIC_LJ_8_6_ZACHARIAS 3  /* "lennard-jones-8-6Zacharias" */

/* ---- dielectric modes (extension; the reference only has a constant) ------------ */
#define BS_DIELECTRIC_CONSTANT 0  /* eps = coulomb.dielectric (energy/electrostatic.hpp:16-49) */
#define BS_DIELECTRIC_DISTANCE 1  /* eps = coulomb.dielectric * r  (no counterpart in the reference) */

/* ---- nonbonded terms, for the pair/cell diagnostics ---------------------------- */
#define BS_TERM_STERIC 0
#define BS_TERM_COULOMB 1
#define BS_TERM_HYDROPHOBIC 2

/* ---- energies, order of bs_get_energies() -------------------------------------- */
#define BS_ENERGY_KINETIC 0
#define BS_ENERGY_SPRING 1
#define BS_ENERGY_STERIC 2
#define BS_ENERGY_ELECTROSTATIC 3
#define BS_ENERGY_IMP 4
#define BS_ENERGY_HYDROPHOBIC 5
#define BS_NUM_ENERGIES 6

/*
 * Run parameters: a plain mirror of the .msp groups the step reads
 * (src/configuration/Configuration.hpp:18-151, defaults at :153-234), plus a
 * few device-path knobs grouped last. bs_default_config() fills it exactly
 * like defaultConfiguration() (Configuration.hpp:153).
 */
typedef struct bs_config {
    /* simulation.* */
    int32_t nbsteps;
    double timestep;        /* fs */
    double neighborskin;    /* A; reference cell-list skin (nsearch.hpp:185-190) */
    /* spring.* */
    int32_t spring_enable;
    double spring_scale;
    /* steric.* */
    int32_t steric_enable;
    double steric_gridscale;
    double steric_cutoff;
    int32_t steric_mode;    /* BS_STERIC_* */
    /* coulomb.* */
    int32_t coulomb_enable;
    double coulomb_scale;
    double coulomb_cutoff;
    double coulomb_dielectric;
    /* hydrophobicity.* */
    int32_t hydrophobicity_enable;
    double hydrophobicity_scale;
    double hydrophobicity_cutoff;
    /* impala.* */
    int32_t impala_enable;
    double impala_scale;
    /* viscosity.* */
    int32_t viscosity_enable;
    double viscosity_value; /* Da/fs */
    /* rigidbody.enable */
    int32_t rigidbody_enable;
    /* --- device-path knobs (new .msp group "cuda.*"; no reference counterpart) --- */
    int32_t dielectric_mode;  /* BS_DIELECTRIC_* */
    double impala_z0;         /* membrane half-thickness, reference hard-codes 15.75 (imp.hpp:13-15) */
    double impala_alpha;      /* reference hard-codes 1.99 */
    int32_t rebuild_every;    /* rebuild the device pair list every K steps (>= 1) */
    double list_skin;         /* A; extra radius of the device pair list; drift > skin/2 forces a rebuild */
    int32_t precise_positions; /* carry each position's rounding remainder (float-float x += v dt);
                                  off (0) reproduces the reference's FP32 update */
    /* probe.* (Configuration.hpp:186-195): one extra interactive particle that every dynamic
       particle feels without cutoff (SpringNetwork.cpp:156-182) */
    int32_t probe_enable;
    int32_t probe_electrostatic; /* probe.enableelectrostatic */
    int32_t probe_steric;        /* probe.enablesteric */
    double probe_x, probe_y, probe_z;
    double probe_mass, probe_epsilon, probe_radius, probe_charge;
    /* potentialgrid.* and densitygrid.* (GridSetting, Setting.hpp:192-222): forces read from a
       scalar map on a regular grid (SpringNetwork.cpp:110-118, Particle.cpp:136-189). The
       potential map acts on charges when coulomb.enable is set too; the density map acts on
       every dynamic particle through its burying. A path is read at bs_setup unless a grid was
       given with bs_set_field_grid. */
    int32_t potentialgrid_enable;
    int32_t densitygrid_enable;
    double potentialgrid_scale;
    double densitygrid_scale;
    char potentialgrid_path[512];
    char densitygrid_path[512];
} bs_config;

typedef struct bs_sim bs_sim;

/* Fills *cfg like configuration::defaultConfiguration() (Configuration.hpp:153-234)
 * and sets the device knobs to dielectric_mode=constant, impala_z0=15.75,
 * impala_alpha=1.99, rebuild_every=10, list_skin=1.0. */
int bs_default_config(bs_config *cfg);

/* Parses .msp text ("group.param = value" lines, '#' comments) on top of *cfg.
 * Unknown or duplicated parameters are rejected, as in
 * SafeConfigurationReader::read (src/configuration/SafeConfigurationReader.cpp:11-40).
 * err (nullable) receives a one-line message on failure. */
int bs_config_parse_msp(const char *text, bs_config *cfg, char *err, size_t err_len);

/* Creates an empty simulation on the current CUDA device
 * (replaces SpringNetwork::SpringNetwork(), SpringNetwork.h:103). */
int bs_create(bs_sim **out);

/* Frees every device and host resource of the handle (SpringNetwork::~SpringNetwork). */
int bs_destroy(bs_sim *sim);

/* Copies n particles in (replaces SpringNetwork::addParticle, SpringNetwork.cpp:498-527,
 * called n times in index order). Nullable arrays take the ParticleProperty defaults
 * (src/spn/ParticleProperty.h:20-24): vel 0, mass 1, charge 0, radius 1, epsilon 0,
 * hydrophobicity 0, sasa 0, transfer 0, is_static 0. A particle is charged iff
 * charge != 0 and hydrophobic iff hydrophobicity != 0 (ParticleProperty.cpp). */
int bs_upload_particles(bs_sim *sim, int64_t n, const float *xyz, const float *vel,
                        const float *mass, const float *charge, const float *radius,
                        const float *epsilon, const float *hydrophobicity,
                        const float *sasa, const float *transfer, const uint8_t *is_static);

/* Adds s springs (replaces s calls of SpringNetwork::addSpring(id1, id2, equilibrium,
 * stiffness), SpringNetwork.cpp:452-486): out-of-range ids and id1 == id2 are
 * BS_E_ARG; a spring between an already-bonded pair is ignored. Springs also
 * exclude their pair from every nonbonded term when spring.enable is set
 * (Particle.cpp:213-218). ij is int32[2*s]. */
int bs_upload_springs(bs_sim *sim, int64_t s, const int32_t *ij, const float *equilibrium,
                      const float *stiffness);

/* Declares rigid bodies: body b owns ids[offsets[b] .. offsets[b+1]-1].
 * Replaces RigidBodiesManager::InitRigidBodies (RigidBodiesManager.cpp:11-43);
 * springs whose two ends are rigid stop acting (RigidBody.cpp:41-53).
 * Effective when rigidbody_enable is set. */
int bs_set_rigid_bodies(bs_sim *sim, int32_t nbodies, const int32_t *offsets, const int32_t *ids);

/* Frame recorder (no reference counterpart; replaces the step loop's trajectory and energy writes,
 * SpringNetwork.cpp:406, 768-779, which stop the run to copy particles): every `every` steps the
 * device writes the positions, in caller order, and the energies of that step into a ring of
 * `capacity` frames in page-locked host memory, without stopping the queued steps. every = 0
 * stops recording. Call after bs_setup (a new set-up stops it). */
int bs_set_frames(bs_sim *sim, int32_t every, int32_t capacity);

/* Takes up to max complete frames, oldest first, without waiting for the device: steps[max] (the
 * step of each frame), xyz[max * 3n] and energies[max * BS_NUM_ENERGIES] (each nullable). *count
 * receives the frames written; *dropped (nullable) the frames lost because the ring went round
 * before they were read. It may run on one other thread while the handle steps (a writer
 * draining the ring); bs_set_frames may not. */
int bs_read_frames(bs_sim *sim, int32_t max, int64_t *steps, float *xyz, double *energies, int32_t *count,
                   int64_t *dropped);

/* Reads a BioSpring topology from a NetCDF classic file (CDF-1, CDF-2 or CDF-5) and uploads it
 * as bs_upload_particles + bs_upload_springs would: coordinates, charges, radii, epsilon, mass (a
 * zero mass becomes 1), dynamicstate (0: static), and when present surfaceaccessibility,
 * hydrophobicityscale (IMPALA transfer energy) and hydrophobicity; then the springs (pairs,
 * springsequilibrium, springsstiffness). Replaces NetCDFReader::read (src/IO/NetCDFReader.cpp:
 * 67-203) with the same array checks and messages; NetCDF-4 (HDF5) files are BS_E_ARG.
 * n_particles and n_springs (nullable) receive the counts read. */
int bs_load_nc(bs_sim *sim, const char *path, int64_t *n_particles, int64_t *n_springs);

/* The same topology into caller arrays, without a handle: call with NULL arrays for the counts,
 * then with arrays of n_particles (xyz: 3 n), n_springs (ij: 2 m) entries. present (int32[3],
 * nullable) tells whether surfaceaccessibility, hydrophobicityscale and hydrophobicity were in the
 * file (absent arrays are left untouched). */
int bs_read_nc(const char *path, int64_t *n_particles, int64_t *n_springs, float *xyz, float *mass, float *charge,
               float *radius, float *epsilon, float *sasa, float *transfer, float *hydrophobicity,
               uint8_t *is_static, int32_t *ij, float *equilibrium, float *stiffness, int32_t *present, char *err,
               size_t err_len);

/* Field grids (PotentialGrid, src/grid/PotentialGrid.hpp): which = BS_GRID_POTENTIAL or
 * BS_GRID_DENSITY. A grid of shape[0] x shape[1] x shape[2] cells of size spacing (A) from
 * origin, scalar values in OpenDX order (scalar[(i * shape[1] + j) * shape[2] + k]). The library
 * derives each cell's force vector as PotentialGrid::compute_gradient does (PotentialGrid.cpp:
 * 20-59); a particle takes the cell holding it, and one outside the box gets no field force and
 * no field energy (Particle.cpp:136-189). Replaces reading the map at set-up
 * (SpringNetwork.cpp:717-747); call before bs_setup. */
#define BS_GRID_POTENTIAL 0
#define BS_GRID_DENSITY 1
int bs_set_field_grid(bs_sim *sim, int32_t which, const int32_t shape[3], const double origin[3],
                      const double spacing[3], const float *scalar);

/* Reads an OpenDX scalar map as OpenDXReader::read does (src/IO/OpenDXReader.cpp): the grid
 * shape the reference derives from the file's box, origin and spacing, then the values. With
 * scalar NULL only the header is read (shape, origin, spacing); otherwise scalar must hold
 * shape[0] * shape[1] * shape[2] floats. */
int bs_read_dx(const char *path, int32_t shape[3], double origin[3], double spacing[3], float *scalar,
               char *err, size_t err_len);

/* The grid after set-up: its shape and, when out is not NULL, 4 floats per cell in OpenDX order:
 * the scalar and the force vector (PotentialCell, PotentialGrid.hpp:12-16); out holds
 * 4 * shape[0] * shape[1] * shape[2] floats. */
int bs_get_field_grid(bs_sim *sim, int32_t which, int32_t shape[3], float *out);

/* Per-particle burying (ParticleProperty::setBurying, ParticleProperty.h:61; default 1), the
 * weight of the density-grid force, caller order. */
int bs_set_burying(bs_sim *sim, const float *burying);

/* The IMPALA double membrane (replaces ForceField::setImpDoubleMembraneUpperMembOffset,
 * ...LowerMembOffset, ...UpperMembTubeCurv, ...LowerMembTubeCurv, ForceField.h:100-110, which the
 * MDDriver interactor sets, CustomData.cpp:61-107): the upper membrane centred at
 * z = +upper_offset and the lower at z = -lower_offset (A), each bent into a tube along y of
 * curvature 1/A (0: flat; the sign says which side the tube's axis lies on), energies and forces
 * of energy/imp.hpp:29-159. All zero (the default) is the flat single membrane. Takes effect at
 * the next step or force evaluation; valid at any time after bs_create. */
int bs_set_membrane(bs_sim *sim, float upper_offset, float lower_offset, float upper_curvature,
                    float lower_curvature);

/* Replaces every particle's charge (ParticleProperty::setCharge, ParticleProperty.h:27, for the
 * whole array: float[n], caller order, finite), before or after bs_setup,
 * e.g. between steps of a charge fit driven by bs_adjoint's dL_dq. A particle whose charge becomes
 * zero leaves the Coulomb pair lists and one whose charge becomes non-zero joins them at the next
 * step, which rebuilds the lists. */
int bs_set_charges(bs_sim *sim, const float *charge);

/* Validates the configuration, uploads everything and builds the first cell list
 * and pair list (replaces SpringNetwork::setup, SpringNetwork.cpp:646-737).
 * Cutoffs below 1e-6 for an enabled term are BS_E_ARG (SpringNetwork.cpp:667-668). */
int bs_setup(bs_sim *sim, const bs_config *cfg);

/* Runs nsteps full steps (replaces nsteps calls of SpringNetwork::computeStep,
 * SpringNetwork.cpp:251-268). Energies of the last step are kept for
 * bs_get_energies. Returns BS_E_NONFINITE if a position became non-finite. */
int bs_step(bs_sim *sim, int32_t nsteps);

/* Enqueues nsteps steps on the handle's stream and returns without waiting (the steps run as
 * captured CUDA graphs). Status is checked by the next synchronising call. */
int bs_step_async(bs_sim *sim, int32_t nsteps);

/* Waits for enqueued work, checks the device status word and, if a particle drifted too far
 * for the pair list or a list overflowed, rebuilds and completes the remaining steps. Returns
 * BS_E_NONFINITE if a position became non-finite (SpringNetwork.cpp:222-229). */
int bs_synchronize(bs_sim *sim);

/* Number of steps the device has completed since bs_setup (synchronises). */
int bs_get_step_count(bs_sim *sim, int64_t *steps);

/* The CUDA stream (cudaStream_t) the handle launches on, for callers that order their own
 * work or record CUDA events around the step. */
int bs_get_stream(bs_sim *sim, void **stream);

/* Enqueues one phase without waiting, for profiling: phase 0 = pair-list rebuild (cell list,
 * counting sort, reorder, spring and pair lists), phase 1 = one step kernel. */
int bs_launch_phase(bs_sim *sim, int32_t phase);

/* Computes forces and energies at the current positions without integrating
 * (replaces idleRun() + computeForces(), SpringNetwork.cpp:244-249, 344-365).
 * The forces are then readable with bs_get_forces. */
int bs_compute_forces(bs_sim *sim);

/* Reads or overwrites per-particle state, in the caller's particle order
 * (Particle::getPosition / setPosition ...). Setting positions or velocities
 * invalidates the pair list, which is rebuilt before the next force evaluation. */
int bs_get_positions(bs_sim *sim, float *xyz);
int bs_get_velocities(bs_sim *sim, float *vel);
int bs_get_forces(bs_sim *sim, float *f);
int bs_set_positions(bs_sim *sim, const float *xyz);
int bs_set_velocities(bs_sim *sim, const float *vel);

/* Adds an external force to particle i for the next step only (replaces
 * SpringNetwork::setForce, SpringNetwork.cpp:438-442, the interactor path). */
int bs_set_force(bs_sim *sim, int64_t i, const float f[3]);

/* Sets the external force of every particle for the next step (float[3n], caller order);
 * the bulk form of bs_set_force used by interactive drivers every step. Returns when the copy is
 * done: the caller may reuse f at once. */
int bs_set_external_forces(bs_sim *sim, const float *f);

/* The same, enqueued on the handle's stream without waiting: f must be page-locked and must stay
 * unchanged until the next call that waits for the stream (bs_step, bs_synchronize, a getter);
 * an interactive driver alternates two buffers. A pageable f is copied as bs_set_external_forces
 * does. Saves the wait of a step's force upload. */
int bs_set_external_forces_async(bs_sim *sim, const float *f);

/* Probe position and velocity (float[6]: x, y, z, vx, vy, vz) after the last step; zeros when
 * probe.enable is off (replaces SpringNetwork::getProbeParticle, SpringNetwork.h:277). The probe
 * moves with bs_step; a force-only evaluation (bs_compute_forces) applies its force to the
 * particles but does not move it. */
int bs_get_probe(bs_sim *sim, float state[6]);

/* XTC trajectory frames, host code (no device involved). The reference writes XTC through its
 * vendored xdrfile library: src/IO/modern/XTCTrajectoryWriter.cpp:15-32 (write_xtc with the
 * coordinates in nm, an identity box, the frame counter as step and time, precision 1000;
 * selected at src/spn/SpringNetwork.cpp:768-779). bs_xtc_encode_frame writes one frame of
 * natoms coordinates (float[3 natoms], nm) into out (cap bytes) and its size into *len
 * (BS_E_CAPACITY, with *len set, when it does not fit); box is float[9] (NULL: identity).
 * bs_xtc_frame_bound gives a capacity that always fits. bs_xtc_decode_frame reads one frame of
 * natoms atoms from in, returning its step, time, box, coordinates, precision (0 for frames of at
 * most 9 atoms, stored uncompressed) and the bytes it used (each output nullable except xyz). */
int bs_xtc_frame_bound(int64_t natoms, size_t *bytes);
int bs_xtc_encode_frame(int64_t natoms, int32_t step, float time, const float box[9], const float *xyz,
                        float precision, uint8_t *out, size_t cap, size_t *len);
int bs_xtc_decode_frame(const uint8_t *in, size_t len, int64_t natoms, int32_t *step, float *time, float box[9],
                        float *xyz, float *precision, size_t *consumed);

/* Energies of the last step or force evaluation, BS_ENERGY_* order, in kJ/mol
 * (SpringNetwork::getKineticEnergy ... getHydrophobicEnergy, SpringNetwork.h:157-162).
 * They are reduced in FP64 on the device. */
int bs_get_energies(bs_sim *sim, double out[BS_NUM_ENERGIES]);

/* Diagnostics for the bit-exact checks.
 * bs_get_pairs: the unique interacting pairs (i < j, caller ids) of one nonbonded term
 * at the current positions, i.e. the pairs for which the reference calls the force
 * routine (Particle.cpp:191-253, 269-330, 368-429). Sorted by (i, j). If *n_out > cap
 * only cap pairs are written. out is int64[2*cap].
 * bs_get_cells: the reference cell id (nsearch.hpp:277-293) of every particle for the
 * grid of one term (cell edge = cutoff + neighborskin, bounding box of all particles),
 * computed on the device; -1 for particles not in that grid. */
int bs_get_pairs(bs_sim *sim, int32_t term, int64_t *out, int64_t cap, int64_t *n_out);
int bs_get_cells(bs_sim *sim, int32_t term, int64_t *out);

/* Number of kernels this handle launched so far (for launch accounting). */
int bs_get_launch_count(bs_sim *sim, int64_t *count);

/* Copies the last error message of the handle (or of the library when sim is NULL). */
int bs_last_error(bs_sim *sim, char *buf, size_t len);

/* ---- gradients (no counterpart in the reference) ----------------------------------
 *
 * Number of springs the handle holds (bs_upload_springs ignores repeated pairs); the spring
 * arrays below have this length, in upload order. */
int bs_get_spring_count(bs_sim *sim, int64_t *count);

/* Replaces every spring's stiffness and/or rest length (nullable arrays keep the current
 * values), e.g. between steps of a parameter fit. Takes effect at the next step. */
int bs_set_spring_parameters(bs_sim *sim, const float *stiffness, const float *equilibrium);

/* Loss L = (1/n) sum_i |x_i(nsteps) - target_i|^2 after nsteps steps from the current state, and
 * its gradient with respect to every spring's stiffness (dL_dk) and rest length (dL_dr0) and,
 * when dL_dq is not NULL, every particle's charge (float[n], caller order; zero without
 * coulomb.enable), by the discrete adjoint of the damped step with checkpoints every
 * `checkpoint` steps and recomputation in between (FP32 adjoint state). The steps run with a
 * rebuild at every checkpoint; the state, step count and energies are left as they were.
 * Differentiates springs, the linear steric mode, Coulomb (both dielectric modes) and viscosity:
 * hydrophobic and IMPALA terms are BS_E_ARG. Charge gradients of static particles are summed
 * with atomics (their order is not fixed). A particle that moves more than half the list skin
 * within one checkpoint interval gives BS_E_CAPACITY. target is float[3n]. */
int bs_adjoint(bs_sim *sim, int32_t nsteps, int32_t checkpoint, const float *target, double *loss,
               float *dL_dk, float *dL_dr0, float *dL_dq);

/* ---- batched ensembles ----------------------------------------------------------
 *
 * Many independent networks in one handle (no reference counterpart: the reference runs one
 * SpringNetwork per process). Upload the systems' particles concatenated with
 * bs_upload_particles, their springs with bs_upload_springs (indices into the concatenation;
 * a spring may not join two systems), then declare the partition before bs_setup:
 * system b owns particles [offsets[b], offsets[b+1]). All systems share one bs_config.
 * bs_step advances every system by nsteps with a persistent kernel in which a
 * thread-block cluster owns whole systems; bs_get_positions / bs_get_velocities /
 * bs_compute_forces work on the concatenation, bs_get_energies gives the sums over systems and
 * bs_get_system_energies each system's. External forces and the pair/cell diagnostics are for
 * single systems (BS_E_STATE); rigid bodies, the probe and field grids are BS_E_ARG at bs_setup. */
int bs_set_systems(bs_sim *sim, int32_t nsys, const int64_t *offsets);

/* Energies of every system of a batch after its last step: double[nsys * BS_NUM_ENERGIES]. */
int bs_get_system_energies(bs_sim *sim, double *out);

/* Launch shape of the persistent batched step kernel: threads per block (128, 256, 512),
 * threads per particle (1, 2, 4, 8) and blocks per cluster (1, 2, 4, 8). */
int bs_set_batch_shape(bs_sim *sim, int32_t block, int32_t lanes, int32_t cluster);
int bs_get_batch_shape(bs_sim *sim, int32_t shape[3]);

/* Times the persistent kernel for one period of the current state under every shape (the state is
 * restored after each trial), keeps the fastest and writes it to shape (nullable). */
int bs_batch_autotune(bs_sim *sim, int32_t shape[3]);

/* ---- nonbonded forces without allocation (no counterpart in the reference) ------
 *
 * Steric, Coulomb and hydrophobic forces and energies of at most
 * BS_NOALLOC_MAX_PARTICLES particles by direct summation over all pairs. Unlike the
 * rest of this API it takes DEVICE pointers the caller owns and allocates no memory:
 * its scratch is a fixed array inside the library. It is for callers whose device
 * memory is all managed by their own pool, or that evaluate forces inside a frame
 * budget where an allocation could stall or fail.
 *
 * Same pair rules as the handle's force evaluation with spring.enable = 0 (no pair is
 * excluded); spring, IMPALA, viscosity and rigid-body fields of *cfg are ignored.
 * d_radius is required when steric is on, d_epsilon too in the Lennard-Jones modes;
 * d_charge, d_hydrophobicity and d_is_static may be NULL (no charges, no hydrophobic
 * particles, all dynamic). Outputs: d_forces float[3n] (0 for static particles),
 * d_energies double[BS_NUM_ENERGIES] (steric, electrostatic and hydrophobic filled,
 * the rest 0). Asynchronous on `stream` (a cudaStream_t, NULL = default stream).
 *
 * n outside [1, BS_NOALLOC_MAX_PARTICLES] returns BS_E_ARG. The first call on a device
 * sets up the scratch (it loads the kernels onto that device) and should come before
 * any stream capture. The scratch address found then is kept for the life of the
 * process, so calls after a cudaDeviceReset of that device are not supported. All
 * calls on one device share the scratch: two calls in flight at once (other streams,
 * other threads) race; order them on one stream. err (nullable) receives a one-line
 * message on failure. */
#define BS_NOALLOC_MAX_PARTICLES 16384
int bs_nonbonded_forces_noalloc(const bs_config *cfg, int64_t n, const float *d_xyz,
                                const float *d_radius, const float *d_epsilon,
                                const float *d_charge, const float *d_hydrophobicity,
                                const uint8_t *d_is_static, float *d_forces, double *d_energies,
                                void *stream, char *err, size_t err_len);

#ifdef __cplusplus
}
#endif

#endif /* BIOSPRING_GB300_H */
