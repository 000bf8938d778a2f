// drive_springnetwork_cuda.cpp -- runs SpringNetworkCUDA beside the reference's SpringNetwork on
// the same small network and prints how far apart they are.
//
// Both are built with the reference's own API the way a BioSpring program builds them
// (addParticle, addSpring, setup(Configuration), computeStep); the CUDA one only differs by its
// class. Exit status 0 when the two agree (or when no CUDA device is present: the device
// subclass then reports the library's error as std::runtime_error, which is printed), 1 otherwise.

#include <cmath>
#include <cstdio>
#include <stdexcept>

#include "SpringNetworkCUDA.h"

using biospring::spn::Particle;
using biospring::spn::SpringNetwork;
using biospring::spn::SpringNetworkCUDA;

namespace
{

// A 6 x 6 x 6 lattice of 3.8 A spacing, slightly displaced, springs to lattice neighbours within
// 6 A, some particles charged, a few static.
void build(SpringNetwork & net)
{
    const int m = 6;
    int id = 0;
    for (int a = 0; a < m; ++a)
        for (int b = 0; b < m; ++b)
            for (int c = 0; c < m; ++c, ++id)
            {
                Particle p;
                const float jx = 0.3f * std::sin(1.7f * id), jy = 0.3f * std::cos(2.3f * id),
                            jz = 0.3f * std::sin(0.7f * id + 1.0f);
                p.setPosition(Vector3f(3.8f * a + jx, 3.8f * b + jy, 3.8f * c + jz));
                p.setMass(12.0f);
                p.setRadius(1.9f);
                p.setEpsilon(0.35f);
                if (id % 5 == 0)
                    p.setCharge(id % 10 == 0 ? 1.0f : -1.0f);
                p.setStatic(id % 37 == 0);
                net.addParticle(p);
            }
    const unsigned n = net.getNumberOfParticles();
    for (unsigned i = 0; i < n; ++i)
        for (unsigned j = i + 1; j < n; ++j)
        {
            const float d = Particle::distance(net.getParticle(i), net.getParticle(j));
            if (d < 6.0f)
                net.addSpring(i, j, d, 2.0f);
        }
}

biospring::configuration::Configuration config()
{
    auto c = biospring::configuration::defaultConfiguration();
    c.sim.nbsteps = 50;
    c.spring.enable = true;
    c.steric.enable = true;
    c.steric.cutoff = 9.0;
    c.steric.mode = std::string("lennard-jones-12-6Amber");
    c.electrostatic.enable = true;
    c.electrostatic.cutoff = 12.0;
    c.electrostatic.dielectric = 4.0;
    c.viscosity.enable = true;
    return c;
}

} // namespace

int main()
{
    SpringNetwork ref;
    SpringNetworkCUDA gpu;
    build(ref);
    build(gpu);
    ref.setup(config());
    gpu.setup(config());
    try
    {
        gpu.initRun();
    }
    catch (const std::runtime_error & e)
    {
        std::printf("device-unavailable: %s\n", e.what());
        return 0;
    }
    ref.initRun();
    float ext[3] = {0.002f, 0.0f, -0.001f};
    ref.setForce(7, ext);
    gpu.setForce(7, ext);
    for (int s = 0; s < 50; ++s)
    {
        ref.computeStep();
        gpu.computeStep();
    }
    gpu.syncHost();
    double dx = 0.0;
    for (unsigned i = 0; i < ref.getNumberOfParticles(); ++i)
    {
        float a[3], b[3];
        ref.getParticlePosition(i, a);
        gpu.getParticlePosition(i, b);
        for (int k = 0; k < 3; ++k)
            dx = std::fmax(dx, std::fabs(static_cast<double>(a[k]) - b[k]));
        const auto pa = ref.getParticle(i).getPosition(), pb = gpu.getParticle(i).getPosition();
        dx = std::fmax(dx, std::fabs(static_cast<double>(pa.getX()) - pb.getX()));
    }
    const double es = std::fabs(ref.getSpringEnergy() - gpu.getSpringEnergy()) / std::fmax(1e-30, std::fabs(ref.getSpringEnergy()));
    const double el = std::fabs(ref.getStericEnergy() - gpu.getStericEnergy()) / std::fmax(1e-30, std::fabs(ref.getStericEnergy()));
    const double ee = std::fabs(ref.getElectrostaticEnergy() - gpu.getElectrostaticEnergy()) /
                      std::fmax(1e-30, std::fabs(ref.getElectrostaticEnergy()));
    std::printf("compared: max |dx| %.3e A, energy rel spring %.2e steric %.2e electrostatic %.2e, iterations %d %d\n",
                dx, es, el, ee, ref.getNbIterations(), gpu.getNbIterations());
    ref.endRun();
    gpu.endRun();
    const bool ok = dx < 1e-4 && es < 1e-4 && el < 1e-4 && ee < 1e-4 && ref.getNbIterations() == gpu.getNbIterations();
    return ok ? 0 : 1;
}
