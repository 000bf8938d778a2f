// SpringNetworkCUDA.cpp -- the SpringNetwork subclass that runs the step loop through the
// C ABI of include/biospring_gb300.h (see SpringNetworkCUDA.h).
//
// Build (beside the reference's sources, as the reference builds SpringNetworkOpenCL.cpp):
//   g++ -std=c++20 -O2 -fopenmp -DOPENMP_SUPPORT -I<reference>/src -I<reference>/src/spn
//       -I<generated version.h dir> -I<this repository>/include -c SpringNetworkCUDA.cpp
// and link with the reference's objects, libbiospring_gb300.so and -lcudart.

#include "SpringNetworkCUDA.h"

#include <cstring>
#include <stdexcept>
#include <string>

#include "logging.h"

namespace biospring
{
namespace spn
{

namespace
{

int steric_mode_of(const std::string & mode)
{
    // StericSetting's choices (src/configuration/Setting.hpp:260-275)
    if (mode == "linear")
        return BS_STERIC_LINEAR;
    if (mode == "lennard-jones-12-6Amber")
        return BS_STERIC_LJ_12_6_AMBER;
    if (mode == "lennard-jones-8-6Lewitt")
        return BS_STERIC_LJ_8_6_LEWITT;
    if (mode == "lennard-jones-8-6Zacharias")
        return BS_STERIC_LJ_8_6_ZACHARIAS;
    throw std::invalid_argument("unknown steric mode '" + mode + "'");
}

void copy_path(char (&dst)[512], const std::string & src)
{
    std::memset(dst, 0, sizeof dst);
    std::strncpy(dst, src.c_str(), sizeof dst - 1);
}

} // namespace

SpringNetworkCUDA::~SpringNetworkCUDA()
{
    if (_sim)
        bs_destroy(_sim);
}

void SpringNetworkCUDA::_check(int rc, const char * what) const
{
    if (rc == BS_OK)
        return;
    char msg[512] = {0};
    bs_last_error(_sim, msg, sizeof msg);
    const std::string text = std::string(what) + ": " + msg;
    if (rc == BS_E_NONFINITE)
        logging::die("%s", text.c_str()); // as SpringNetwork.cpp:222-229
    if (rc == BS_E_ARG)
        throw std::invalid_argument(msg); // the reference's set-up messages (SpringNetwork.cpp:667-668)
    throw std::runtime_error(text);
}

// The probe, when enabled, is the last host particle (SpringNetwork.cpp:749-766); the device
// keeps it apart (bs_config probe_*), so it is not uploaded as a particle.
int64_t SpringNetworkCUDA::_deviceParticles() const
{
    const int64_t n = static_cast<int64_t>(getNumberOfParticles());
    return isProbeEnabled() && n > 0 ? n - 1 : n;
}

void SpringNetworkCUDA::_fillConfig(bs_config & c) const
{
    bs_default_config(&c);
    c.nbsteps = _config.sim.nbsteps;
    c.timestep = _config.sim.timestep;
    c.neighborskin = _config.sim.neighborskin;
    c.spring_enable = _config.spring.enable;
    c.spring_scale = _config.spring.scale;
    c.steric_enable = _config.steric.enable;
    c.steric_gridscale = _config.steric.gridscale;
    c.steric_cutoff = _config.steric.cutoff;
    c.steric_mode = steric_mode_of(_config.steric.mode);
    c.coulomb_enable = _config.electrostatic.enable;
    c.coulomb_scale = _config.electrostatic.scale;
    c.coulomb_cutoff = _config.electrostatic.cutoff;
    c.coulomb_dielectric = _config.electrostatic.dielectric;
    c.hydrophobicity_enable = _config.hydrophobicity.enable;
    c.hydrophobicity_scale = _config.hydrophobicity.scale;
    c.hydrophobicity_cutoff = _config.hydrophobicity.cutoff;
    c.impala_enable = _config.imp.enable;
    c.impala_scale = _config.imp.scale;
    c.viscosity_enable = _config.viscosity.enable;
    c.viscosity_value = _config.viscosity.value;
    c.rigidbody_enable = _config.rigidbody.enable;
    c.probe_enable = _config.probe.enable;
    c.probe_electrostatic = _config.probe.enableelectrostatic;
    c.probe_steric = _config.probe.enablesteric;
    c.probe_x = _config.probe.x;
    c.probe_y = _config.probe.y;
    c.probe_z = _config.probe.z;
    c.probe_mass = _config.probe.mass;
    c.probe_epsilon = _config.probe.epsilon;
    c.probe_radius = _config.probe.radius;
    c.probe_charge = _config.probe.charge;
    c.potentialgrid_enable = _config.potentialgrid.enable;
    c.potentialgrid_scale = _config.potentialgrid.scale;
    copy_path(c.potentialgrid_path, _config.potentialgrid.path);
    c.densitygrid_enable = _config.densitygrid.enable;
    c.densitygrid_scale = _config.densitygrid.scale;
    copy_path(c.densitygrid_path, _config.densitygrid.path);
}

void SpringNetworkCUDA::_upload(int64_t n)
{
    std::vector<float> xyz(3 * n), vel(3 * n), mass(n), q(n), r(n), eps(n), h(n), sasa(n), tr(n);
    std::vector<uint8_t> st(n);
    for (int64_t i = 0; i < n; ++i)
    {
        const Particle & p = getParticle(static_cast<unsigned>(i));
        const Vector3f x = p.getPosition();
        const Vector3f v = p.getVelocity();
        xyz[3 * i] = x.getX();
        xyz[3 * i + 1] = x.getY();
        xyz[3 * i + 2] = x.getZ();
        vel[3 * i] = v.getX();
        vel[3 * i + 1] = v.getY();
        vel[3 * i + 2] = v.getZ();
        mass[i] = p.getMass();
        q[i] = p.getCharge();
        r[i] = p.getRadius();
        eps[i] = p.getEpsilon();
        h[i] = p.getHydrophobicity();
        sasa[i] = p.getSolventAccessibilitySurface();
        tr[i] = p.getTransferEnergyByAccessibleSurface();
        st[i] = p.isStatic() ? 1 : 0;
    }
    _check(bs_upload_particles(_sim, n, xyz.data(), vel.data(), mass.data(), q.data(), r.data(), eps.data(), h.data(),
                               sasa.data(), tr.data(), st.data()),
           "bs_upload_particles");
    const auto & springs = getSprings();
    std::vector<int32_t> ij(2 * springs.size());
    std::vector<float> r0(springs.size()), k(springs.size());
    for (size_t s = 0; s < springs.size(); ++s)
    {
        ij[2 * s] = springs[s].getParticle1().getId();
        ij[2 * s + 1] = springs[s].getParticle2().getId();
        r0[s] = springs[s].getEquilibrium();
        k[s] = springs[s].getStiffness();
    }
    _check(bs_upload_springs(_sim, static_cast<int64_t>(springs.size()), ij.data(), r0.data(), k.data()),
           "bs_upload_springs");
}

void SpringNetworkCUDA::_ensureDevice()
{
    if (_sim)
        return;
    const int64_t n = _deviceParticles();
    _check(bs_create(&_sim), "bs_create");
    _upload(n);
    if (isRigidBodyEnabled())
    {
        // SpringNetwork::run() makes every dynamic particle one body
        // (RigidBodiesManager::InitRigidBodies(this, getDynamicParticles()), SpringNetwork.cpp:282-285)
        std::vector<int32_t> ids;
        for (unsigned i : getDynamicParticles())
            if (static_cast<int64_t>(i) < n)
                ids.push_back(static_cast<int32_t>(i));
        const int32_t offsets[2] = {0, static_cast<int32_t>(ids.size())};
        _check(bs_set_rigid_bodies(_sim, 1, offsets, ids.data()), "bs_set_rigid_bodies");
    }
    bs_config c;
    _fillConfig(c);
    _check(bs_setup(_sim, &c), "bs_setup");
    // forces added on the host before the device state existed (setForce) act on the next step
    for (int64_t i = 0; i < n; ++i)
    {
        const Vector3f f = getParticle(static_cast<unsigned>(i)).getForce();
        if (f.getX() != 0.0f || f.getY() != 0.0f || f.getZ() != 0.0f)
        {
            const float ff[3] = {f.getX(), f.getY(), f.getZ()};
            _check(bs_set_force(_sim, i, ff), "bs_set_force");
        }
    }
    _hostDirty = false;
    _xyzValid = false;
}

void SpringNetworkCUDA::_pullEnergies()
{
    double e[BS_NUM_ENERGIES];
    _check(bs_get_energies(_sim, e), "bs_get_energies");
    _energies.kinetic = static_cast<float>(e[BS_ENERGY_KINETIC]);
    _energies.spring = static_cast<float>(e[BS_ENERGY_SPRING]);
    _energies.steric = static_cast<float>(e[BS_ENERGY_STERIC]);
    _energies.electrostatic = static_cast<float>(e[BS_ENERGY_ELECTROSTATIC]);
    _energies.imp = static_cast<float>(e[BS_ENERGY_IMP]);
    _energies.hydrophobic = static_cast<float>(e[BS_ENERGY_HYDROPHOBIC]);
}

void SpringNetworkCUDA::_pullPositions() const
{
    if (_xyzValid || !_sim)
        return;
    const int64_t n = _deviceParticles();
    _xyz.resize(3 * static_cast<size_t>(n));
    _check(bs_get_positions(_sim, _xyz.data()), "bs_get_positions");
    _xyzValid = true;
}

void SpringNetworkCUDA::syncHost()
{
    if (!_sim)
        return;
    const int64_t n = _deviceParticles();
    _pullPositions();
    std::vector<float> vel(3 * static_cast<size_t>(n));
    _check(bs_get_velocities(_sim, vel.data()), "bs_get_velocities");
    for (int64_t i = 0; i < n; ++i)
    {
        Particle & p = getParticle(static_cast<unsigned>(i));
        p.setPosition(Vector3f(_xyz[3 * i], _xyz[3 * i + 1], _xyz[3 * i + 2]));
        p.setVelocity(Vector3f(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]));
    }
    if (isProbeEnabled() && getNumberOfParticles() > 0)
    {
        float prb[6];
        _check(bs_get_probe(_sim, prb), "bs_get_probe");
        Particle & p = getParticle(getNumberOfParticles() - 1);
        p.setPosition(Vector3f(prb[0], prb[1], prb[2]));
        p.setVelocity(Vector3f(prb[3], prb[4], prb[5]));
    }
    _hostDirty = false;
}

// A trajectory writer writes when the iteration count is a multiple of its frequency
// (TrajectoryManager::write_step, src/IO/modern/TrajectoryManager.cpp:10-17).
bool SpringNetworkCUDA::_writeFrameDue() const
{
    const size_t it = static_cast<size_t>(getNbIterations());
    const auto due = [it](bool on, int freq) { return on && freq > 0 && it % static_cast<size_t>(freq) == 0; };
    return due(isPDBTrajectoryWriterEnabled(), getPDBTrajectoryWriterFreq()) ||
           due(isXTCTrajectoryWriterEnabled(), getXTCTrajectoryWriterFreq()) ||
           due(isCSVTrajectoryWriterEnabled(), getCSVTrajectoryWriterFreq());
}

void SpringNetworkCUDA::initRun()
{
    SpringNetwork::initRun();
    _ensureDevice();
}

void SpringNetworkCUDA::endRun()
{
    syncHost();
    SpringNetwork::endRun();
}

void SpringNetworkCUDA::idleRun()
{
    // writers read the host particles: bring them up to date on write frames only
    if (_sim && _hostDirty && _writeFrameDue())
        syncHost();
    SpringNetwork::idleRun();
}

void SpringNetworkCUDA::computeStep()
{
    _ensureDevice();
    idleRun();
    _check(bs_step(_sim, 1), "bs_step");
    _pullEnergies();
    _hostDirty = true;
    _xyzValid = false;
    if (isInsertionVectorEnabled())
    {
        syncHost();
        _updateInsertionVector();
    }
}

void SpringNetworkCUDA::computeForces()
{
    _ensureDevice();
    _check(bs_compute_forces(_sim), "bs_compute_forces");
    _pullEnergies();
    const int64_t n = _deviceParticles();
    std::vector<float> f(3 * static_cast<size_t>(n));
    _check(bs_get_forces(_sim, f.data()), "bs_get_forces");
    for (int64_t i = 0; i < n; ++i)
        getParticle(static_cast<unsigned>(i)).setForce(Vector3f(f[3 * i], f[3 * i + 1], f[3 * i + 2]));
}

void SpringNetworkCUDA::computeSpringForces() {}

void SpringNetworkCUDA::computeParticleForces() { computeForces(); }

void SpringNetworkCUDA::updateParticlePositions()
{
    throw std::logic_error("SpringNetworkCUDA integrates positions inside computeStep(); "
                           "updateParticlePositions() has no separate device form");
}

void SpringNetworkCUDA::getParticlePosition(unsigned i, float position[3]) const
{
    const int64_t n = _deviceParticles();
    if (!_sim || static_cast<int64_t>(i) >= n)
    {
        SpringNetwork::getParticlePosition(i, position); // before set-up, or the probe's host copy
        return;
    }
    _pullPositions();
    position[0] = _xyz[3 * static_cast<size_t>(i)];
    position[1] = _xyz[3 * static_cast<size_t>(i) + 1];
    position[2] = _xyz[3 * static_cast<size_t>(i) + 2];
}

void SpringNetworkCUDA::setForce(unsigned i, float force[3])
{
    if (!_sim)
    {
        SpringNetwork::setForce(i, force); // before set-up: on the host particle, as the reference
        return;
    }
    if (static_cast<int64_t>(i) >= _deviceParticles())
        throw std::out_of_range("SpringNetworkCUDA::setForce: particle index out of range");
    _check(bs_set_force(_sim, static_cast<int64_t>(i), force), "bs_set_force");
}

} // namespace spn
} // namespace biospring
