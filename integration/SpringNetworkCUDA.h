// SpringNetworkCUDA.h -- BioSpring's SpringNetwork with the per-step loop on one GB300.
//
// A drop-in subclass of biospring::spn::SpringNetwork (src/spn/SpringNetwork.h), the seam the
// reference's own OpenCL backend uses (src/opencl/SpringNetworkOpenCL.h:84-182). It overrides the
// step virtuals (SpringNetwork.h:303-308, 330-332, 395-397) and forwards them to the C ABI of
// include/biospring_gb300.h; topology loading, configuration parsing, trajectory writers and
// interactors stay the reference's code. The selection point is src/cli/biospring-cli.cpp:89-96,
// where a flag would create this class instead of SpringNetwork or SpringNetworkOpenCL.
//
// Behaviour the reference's callers rely on:
//  * computeStep() keeps the reference's order (SpringNetwork.cpp:251-268): idleRun() first
//    (interactors, writers, energy reset, iteration count), then one device step (forces,
//    rigid bodies, Euler step), then the insertion vector on the host when it is enabled;
//  * the energy getters (getSpringEnergy(), ...) read _energies, written after every step and
//    every force evaluation;
//  * getParticles()/getParticle(i) are brought up to date lazily: before a trajectory writer
//    writes (idleRun on a write frame), on syncHost(), at endRun(), and after computeForces()
//    (forces); getParticlePosition(i) reads the device positions of the current step;
//  * setForce(i, f) adds an external force consumed by the next step (SpringNetwork.cpp:438-442);
//  * a non-finite position dies as SpringNetwork.cpp:222-229 does; a bad set-up throws
//    std::invalid_argument with the reference's message; other failures throw std::runtime_error.
//
// The device state is created on the first initRun(), computeStep() or computeForces() after
// setup(), from the host particles and springs and the configuration at that time.
#ifndef SPRINGNETWORKCUDA_H
#define SPRINGNETWORKCUDA_H

#include <vector>

#include "spn/SpringNetwork.h"

#include "biospring_gb300.h"

namespace biospring
{
namespace spn
{

class SpringNetworkCUDA : public SpringNetwork
{
  public:
    SpringNetworkCUDA() = default;
    ~SpringNetworkCUDA() override;

    void initRun() override;
    void endRun() override;
    void idleRun() override;

    void computeStep() override;
    // One device evaluation of every enabled term (springs included, SpringNetwork.cpp:244-249);
    // forces go to the host particles, energies to _energies.
    void computeForces() override;
    // Springs are evaluated with the other terms by computeParticleForces(): this is a no-op.
    void computeSpringForces() override;
    void computeParticleForces() override;
    // Positions are integrated inside computeStep(); called alone this throws std::logic_error.
    void updateParticlePositions() override;

    void getParticlePosition(unsigned i, float position[3]) const override;
    void setForce(unsigned i, float force[3]) override;

    // Copies the device positions, velocities (and the probe) into the host particles now.
    void syncHost();
    // The library handle (null before the device state exists).
    bs_sim * handle() const { return _sim; }

  private:
    void _ensureDevice();
    void _upload(int64_t n);
    void _fillConfig(bs_config & c) const;
    void _pullEnergies();
    void _pullPositions() const;
    bool _writeFrameDue() const;
    void _check(int rc, const char * what) const;
    int64_t _deviceParticles() const;

    bs_sim * _sim = nullptr;
    bool _hostDirty = false;            // the device has stepped since the host particles were synced
    mutable std::vector<float> _xyz;    // device positions of the current step, caller order
    mutable bool _xyzValid = false;
};

} // namespace spn
} // namespace biospring

#endif
