// ref_driver.cpp -- test infrastructure, not product code.
//
// A thin extern "C" driver around the UNMODIFIED reference engine
// (biospring::spn::SpringNetwork), compiled together with the reference's own
// sources by oracle/ref.mk into oracle/_ref/libbsref.so. It exists only to
// pin the CPU restatement (oracle/bs_oracle.cpp) and to generate the golden
// fixtures under tests/golden/. Nothing in the product links or loads it.
//
// Every call goes through the reference's public API:
//   addParticle / addSpring          src/spn/SpringNetwork.cpp:452-527
//   setup(Configuration)             src/spn/SpringNetwork.cpp:646-737
//   computeStep()                    src/spn/SpringNetwork.cpp:251-268
//   idleRun() + computeForces()      src/spn/SpringNetwork.cpp:244-249, 344-365
//   RigidBodiesManager::InitRigidBodies  src/rigidbody/RigidBodiesManager.cpp:11-43
// Pair sets are read by querying the reference's own neighbour grids
// (nsearch.hpp:214-234) and applying the filters the force routines apply
// (Particle.cpp:191-253, 269-330, 368-429). Cell ids come from a
// NeighborSearch built on the same particles (nsearch.hpp:277-293).

#include <chrono>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "configuration/Configuration.hpp"
#include "nsearch.hpp"
#include "rigidbody/RigidBodiesManager.h"
#include "spn/Particle.h"
#include "spn/SpringNetwork.h"

#include "../include/biospring_gb300.h"

namespace spn = biospring::spn;
namespace cfgns = biospring::configuration;

namespace
{

// Exposes the protected cell computation of the reference grid.
struct CellPeek : public biospring::nsearch::NeighborSearch<std::vector<spn::Particle>>
{
    using Base = biospring::nsearch::NeighborSearch<std::vector<spn::Particle>>;
    CellPeek(const std::vector<spn::Particle> & c, float cutoff, std::vector<size_t> inc, float skin)
        : Base(c, cutoff, std::move(inc), skin)
    {
    }
    CellPeek(const std::vector<spn::Particle> & c, float cutoff, float skin) : Base(c, cutoff, skin) {}
    size_t cell_of(const spn::Particle & p) const
    {
        return _compute_cell(biospring::concepts::locatable::get_position(p));
    }
};

struct RefSim
{
    spn::SpringNetwork sn;
    cfgns::Configuration conf;
    bool rigid = false;
    unsigned n = 0; // the caller's particles (the probe, when enabled, is appended after them)
};

cfgns::Configuration to_reference_config(const bs_config & c)
{
    cfgns::Configuration conf = cfgns::defaultConfiguration();
    conf.sim.nbsteps = c.nbsteps;
    conf.sim.timestep = c.timestep;
    conf.sim.neighborskin = c.neighborskin;
    conf.spring.enable = c.spring_enable != 0;
    conf.spring.scale = c.spring_scale;
    conf.steric.enable = c.steric_enable != 0;
    conf.steric.gridscale = c.steric_gridscale;
    conf.steric.cutoff = c.steric_cutoff;
    switch (c.steric_mode)
    {
    case BS_STERIC_LJ_12_6_AMBER: conf.steric.mode = "lennard-jones-12-6Amber"; break;
    case BS_STERIC_LJ_8_6_LEWITT: conf.steric.mode = "lennard-jones-8-6Lewitt"; break;
    case BS_STERIC_LJ_8_6_ZACHARIAS: conf.steric.mode = "lennard-jones-8-6Zacharias"; break;
    default: conf.steric.mode = "linear"; break;
    }
    conf.electrostatic.enable = c.coulomb_enable != 0;
    conf.electrostatic.scale = c.coulomb_scale;
    conf.electrostatic.cutoff = c.coulomb_cutoff;
    conf.electrostatic.dielectric = c.coulomb_dielectric;
    conf.hydrophobicity.enable = c.hydrophobicity_enable != 0;
    conf.hydrophobicity.scale = c.hydrophobicity_scale;
    conf.hydrophobicity.cutoff = c.hydrophobicity_cutoff;
    conf.imp.enable = c.impala_enable != 0;
    conf.imp.scale = c.impala_scale;
    conf.viscosity.enable = c.viscosity_enable != 0;
    conf.viscosity.value = c.viscosity_value;
    conf.rigidbody.enable = c.rigidbody_enable != 0;
    conf.probe.enable = c.probe_enable != 0;
    conf.probe.enableelectrostatic = c.probe_electrostatic != 0;
    conf.probe.enablesteric = c.probe_steric != 0;
    conf.probe.x = c.probe_x;
    conf.probe.y = c.probe_y;
    conf.probe.z = c.probe_z;
    conf.probe.mass = c.probe_mass;
    conf.probe.epsilon = c.probe_epsilon;
    conf.probe.radius = c.probe_radius;
    conf.probe.charge = c.probe_charge;
    conf.potentialgrid.enable = c.potentialgrid_enable != 0;
    conf.potentialgrid.scale = c.potentialgrid_scale;
    conf.potentialgrid.path = c.potentialgrid_path;
    conf.densitygrid.enable = c.densitygrid_enable != 0;
    conf.densitygrid.scale = c.densitygrid_scale;
    conf.densitygrid.path = c.densitygrid_path;
    return conf;
}

} // namespace

extern "C" {

void * bsref_create(const bs_config * cfg, int64_t n, const float * xyz, const float * vel, const float * mass,
                    const float * charge, const float * radius, const float * eps, const float * hydro,
                    const float * sasa, const float * transfer, const uint8_t * is_static, int64_t ns,
                    const int32_t * ij, const float * r0, const float * k)
{
    auto * h = new RefSim();
    h->n = static_cast<unsigned>(n);
    for (int64_t i = 0; i < n; ++i)
    {
        spn::Particle p;
        p.setPosition(Vector3f(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
        if (vel)
            p.setVelocity(Vector3f(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]));
        if (mass)
            p.setMass(mass[i]);
        if (charge)
            p.setCharge(charge[i]);
        if (radius)
            p.setRadius(radius[i]);
        if (eps)
            p.setEpsilon(eps[i]);
        if (hydro)
            p.setHydrophobicity(hydro[i]);
        if (sasa)
            p.setSolventAccessibilitySurface(sasa[i]);
        if (transfer)
            p.setTransferEnergyByAccessibleSurface(transfer[i]);
        if (is_static)
            p.setStatic(is_static[i] != 0);
        h->sn.addParticle(p);
    }
    for (int64_t s = 0; s < ns; ++s)
        h->sn.addSpring(static_cast<unsigned>(ij[2 * s]), static_cast<unsigned>(ij[2 * s + 1]), r0[s], k[s]);
    h->conf = to_reference_config(*cfg);
    h->sn.setup(h->conf);
    if (cfg->rigidbody_enable)
    {
        // As SpringNetwork::run() does (SpringNetwork.cpp:281-292): one body made of
        // every dynamic particle.
        biospring::rigidbody::RigidBodiesManager::InitRigidBodies(&h->sn, h->sn.getDynamicParticles());
        h->rigid = true;
    }
    return h;
}

// The double membrane and its tube curvatures on the reference's force field, as the MDDriver
// interactor sets them (src/interactor/mddriver/CustomData.cpp:61-107, ForceField.h:100-110).
void bsref_set_membrane(void * hp, float upper_offset, float lower_offset, float upper_curv, float lower_curv)
{
    auto * h = static_cast<RefSim *>(hp);
    biospring::forcefield::ForceField * ff = h->sn.getForceField();
    ff->setImpDoubleMembraneUpperMembOffset(upper_offset);
    ff->setImpDoubleMembraneLowerMembOffset(lower_offset);
    ff->setImpDoubleMembraneUpperMembTubeCurv(upper_curv);
    ff->setImpDoubleMembraneLowerMembTubeCurv(lower_curv);
}

// ParticleProperty::setBurying on every caller particle.
void bsref_set_burying(void * hp, const float * b)
{
    auto * h = static_cast<RefSim *>(hp);
    for (unsigned i = 0; i < h->n; ++i)
        h->sn.getParticle(i).setBurying(b[i]);
}

// The reference's grid (0 potential, 1 density) as read at set-up: shape and, when out is not
// NULL, 4 floats per cell (scalar, force vector) in OpenDX order.
void bsref_get_field_grid(void * hp, int32_t which, int32_t * shape, float * out)
{
    auto * h = static_cast<RefSim *>(hp);
    const biospring::grid::PotentialGrid & g = which == 0 ? h->sn.getPotentialGrid() : h->sn.getDensityGrid();
    for (int a = 0; a < 3; ++a)
        shape[a] = static_cast<int32_t>(g.shape()[a]);
    if (!out)
        return;
    size_t c = 0;
    for (size_t i = 0; i < g.shape()[0]; ++i)
        for (size_t j = 0; j < g.shape()[1]; ++j)
            for (size_t k = 0; k < g.shape()[2]; ++k, ++c)
            {
                const auto & cell = g.at(biospring::grid::discrete_coordinates(
                    {static_cast<int>(i), static_cast<int>(j), static_cast<int>(k)}));
                out[4 * c] = cell.scalar;
                out[4 * c + 1] = cell.vector.getX();
                out[4 * c + 2] = cell.vector.getY();
                out[4 * c + 3] = cell.vector.getZ();
            }
}

void bsref_destroy(void * hp)
{
    auto * h = static_cast<RefSim *>(hp);
    if (h->rigid)
        biospring::rigidbody::RigidBodiesManager::CleanRigidBodies();
    delete h;
}

int bsref_step(void * hp, int nsteps)
{
    auto * h = static_cast<RefSim *>(hp);
    for (int s = 0; s < nsteps; ++s)
        h->sn.computeStep();
    return 0;
}

double bsref_time_steps(void * hp, int nsteps)
{
    auto * h = static_cast<RefSim *>(hp);
    const auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < nsteps; ++s)
        h->sn.computeStep();
    const auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

// Forces of one evaluation at the current positions: every particle's force is
// cleared first (the reference clears dynamic forces at the end of each step,
// SpringNetwork.cpp:232), then idleRun() + computeForces().
int bsref_compute_forces(void * hp)
{
    auto * h = static_cast<RefSim *>(hp);
    for (unsigned i = 0; i < h->n; ++i)
        h->sn.getParticle(i).resetForce();
    h->sn.idleRun();
    h->sn.computeForces();
    return 0;
}

void bsref_get_positions(void * hp, float * out)
{
    auto * h = static_cast<RefSim *>(hp);
    for (unsigned i = 0; i < h->n; ++i)
    {
        const Vector3f v = h->sn.getParticle(i).getPosition();
        out[3 * i] = v.getX();
        out[3 * i + 1] = v.getY();
        out[3 * i + 2] = v.getZ();
    }
}

void bsref_get_velocities(void * hp, float * out)
{
    auto * h = static_cast<RefSim *>(hp);
    for (unsigned i = 0; i < h->n; ++i)
    {
        const Vector3f v = h->sn.getParticle(i).getVelocity();
        out[3 * i] = v.getX();
        out[3 * i + 1] = v.getY();
        out[3 * i + 2] = v.getZ();
    }
}

void bsref_get_forces(void * hp, float * out)
{
    auto * h = static_cast<RefSim *>(hp);
    for (unsigned i = 0; i < h->n; ++i)
    {
        const Vector3f v = h->sn.getParticle(i).getForce();
        out[3 * i] = v.getX();
        out[3 * i + 1] = v.getY();
        out[3 * i + 2] = v.getZ();
    }
}

// Positions are set, then setup() is run again so that the reference grids are
// rebuilt from the new coordinates (setup re-creates every NeighborSearch,
// SpringNetwork.cpp:663-737).
void bsref_set_positions(void * hp, const float * xyz)
{
    auto * h = static_cast<RefSim *>(hp);
    for (unsigned i = 0; i < h->n; ++i)
        h->sn.getParticle(i).setPosition(Vector3f(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
    h->sn.setup(h->conf);
}

// Probe position and velocity (the copy the reference keeps after the particles).
void bsref_get_probe(void * hp, float * out)
{
    auto * h = static_cast<RefSim *>(hp);
    for (int k = 0; k < 6; ++k)
        out[k] = 0.0f;
    if (!h->conf.probe.enable || h->sn.getNumberOfParticles() <= h->n)
        return;
    const auto & pr = h->sn.getProbeParticle();
    const Vector3f x = pr.getPosition(), v = pr.getVelocity();
    out[0] = x.getX();
    out[1] = x.getY();
    out[2] = x.getZ();
    out[3] = v.getX();
    out[4] = v.getY();
    out[5] = v.getZ();
}

void bsref_get_energies(void * hp, double * out)
{
    auto * h = static_cast<RefSim *>(hp);
    out[BS_ENERGY_KINETIC] = h->sn.getKineticEnergy();
    out[BS_ENERGY_SPRING] = h->sn.getSpringEnergy();
    out[BS_ENERGY_STERIC] = h->sn.getStericEnergy();
    out[BS_ENERGY_ELECTROSTATIC] = h->sn.getElectrostaticEnergy();
    out[BS_ENERGY_IMP] = h->sn.getIMPEnergy();
    out[BS_ENERGY_HYDROPHOBIC] = h->sn.getHydrophobicEnergy();
}

// Unique interacting pairs of one term, written as (min id, max id). The filters
// are those of the force routines, in their order (Particle.cpp:199-224 for
// Coulomb, :279-303 hydrophobic, :378-402 steric).
int64_t bsref_get_pairs(void * hp, int term, int64_t * out, int64_t cap)
{
    auto * h = static_cast<RefSim *>(hp);
    spn::SpringNetwork & sn = h->sn;
    const auto & ns = sn.getNeighborSearch();
    const biospring::nsearch::NeighborSearch<std::vector<spn::Particle>> * searcher = nullptr;
    float cutoff = 0.0f;
    if (term == BS_TERM_STERIC)
    {
        searcher = ns.steric.get();
        cutoff = sn.getStericCutoff();
    }
    else if (term == BS_TERM_COULOMB)
    {
        searcher = ns.electrostatic.get();
        cutoff = sn.getElectrostaticCutoff();
    }
    else
    {
        searcher = ns.hydrophobic.get();
        cutoff = sn.getHydrophobicCutoff();
    }
    if (!searcher)
        return 0;
    int64_t count = 0;
    for (const unsigned id : sn.getDynamicParticles())
    {
        const spn::Particle & pi = sn.getParticle(id);
        if (term == BS_TERM_COULOMB && !pi.isCharged())
            continue;
        if (term == BS_TERM_HYDROPHOBIC && !pi.isHydrophobic())
            continue;
        searcher->for_each_neighbor(pi, [&](size_t j) {
            if (sn.isProbeParticle(j))
                return;
            const spn::Particle & pj = sn.getParticle(static_cast<unsigned>(j));
            if (pj.isDynamic() && j < static_cast<size_t>(pi.getId()))
                return;
            if (sn.isSpringEnabled() && pi.isInSpringNeighbors(static_cast<unsigned>(pj.getId())))
                return;
            if (term == BS_TERM_STERIC && pj.getId() == pi.getId())
                return;
            const Vector3f f = pj.getPosition() - pi.getPosition();
            const float distance = f.norm();
            if (!(distance < cutoff))
                return;
            if (term != BS_TERM_STERIC && !(distance != 0.0))
                return;
            if (count < cap)
            {
                const int64_t a = pi.getId(), b = static_cast<int64_t>(j);
                out[2 * count] = a < b ? a : b;
                out[2 * count + 1] = a < b ? b : a;
            }
            ++count;
        });
    }
    return count;
}

// Reference cell id of every particle for the grid of one term; -1 when the
// particle is not in that grid (uncharged for Coulomb, non-hydrophobic for the
// hydrophobic term).
int bsref_get_cells(void * hp, int term, int64_t * out)
{
    auto * h = static_cast<RefSim *>(hp);
    spn::SpringNetwork & sn = h->sn;
    const auto & parts = sn.getParticles();
    const float skin = sn.getNeighborSkin();
    std::vector<size_t> inc;
    float cutoff = sn.getStericCutoff();
    if (term == BS_TERM_COULOMB)
    {
        cutoff = sn.getElectrostaticCutoff();
        for (size_t i = 0; i < parts.size(); ++i)
            if (parts[i].isCharged())
                inc.push_back(i);
    }
    else if (term == BS_TERM_HYDROPHOBIC)
    {
        cutoff = sn.getHydrophobicCutoff();
        for (size_t i = 0; i < parts.size(); ++i)
            if (parts[i].isHydrophobic())
                inc.push_back(i);
    }
    std::unique_ptr<CellPeek> peek;
    if (term == BS_TERM_STERIC)
        peek = std::make_unique<CellPeek>(parts, cutoff, skin);
    else
    {
        if (inc.empty())
        {
            for (size_t i = 0; i < parts.size(); ++i)
                out[i] = -1;
            return 0;
        }
        peek = std::make_unique<CellPeek>(parts, cutoff, inc, skin);
    }
    std::vector<char> member(parts.size(), term == BS_TERM_STERIC ? 1 : 0);
    for (size_t i : inc)
        member[i] = 1;
    for (size_t i = 0; i < parts.size(); ++i)
        out[i] = member[i] ? static_cast<int64_t>(peek->cell_of(parts[i])) : -1;
    return 0;
}

} // extern "C"
